// In-process stand-in for the few MPI calls include/mfgpu_mpi.hpp makes, so
// its wire code runs without an MPI library.  One FakeWorld holds the
// ranks' mailboxes; each rank is a FakeComm pointing at it.  Calls never
// block: a test runs the ranks one after another -- senders before
// receivers, the non-root ranks of a collective before its root -- and a
// receive with no matching message returns MPI_ERR_OTHER.
#pragma once
#include <cstring>
#include <deque>
#include <vector>

typedef int MPI_Datatype;  // element size << 4 | kind
#define MPI_BYTE ((1 << 4) | 0)
#define MPI_INT ((4 << 4) | 1)
#define MPI_FLOAT ((4 << 4) | 2)
#define MPI_DOUBLE ((8 << 4) | 3)
#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)

struct MPI_Status
{
    int MPI_SOURCE, MPI_TAG, MPI_ERROR;
};
#define MPI_STATUS_IGNORE ((MPI_Status *) 0)

struct FakeMsg
{
    int src, tag;
    MPI_Datatype type;
    std::vector<char> bytes;
};
struct FakeWorld
{
    explicit FakeWorld(int n) : size(n), p2p(n), coll(n) {}
    int size;
    std::vector<std::deque<FakeMsg>> p2p, coll;  // per destination rank
    int fail_after = -1;                         // calls until MPI_ERR_OTHER (-1: never)
};
struct FakeComm
{
    FakeWorld *w;
    int rank;
};
typedef FakeComm *MPI_Comm;

namespace fake_mpi
{
inline size_t bytes(int count, MPI_Datatype t) { return (size_t) count * (size_t) (t >> 4); }
inline bool failing(MPI_Comm c) { return c->w->fail_after >= 0 && c->w->fail_after-- == 0; }
inline void push(std::deque<FakeMsg> &q, int src, int tag, MPI_Datatype t, const void *buf, int count)
{
    FakeMsg m{src, tag, t, std::vector<char>(bytes(count, t))};
    if (!m.bytes.empty()) std::memcpy(m.bytes.data(), buf, m.bytes.size());
    q.push_back(std::move(m));
}
// first message from src (any when MPI_ANY_SOURCE) with tag (any when
// MPI_ANY_TAG) and type t that fits count elements
inline int pop(std::deque<FakeMsg> &q, int src, int tag, MPI_Datatype t, void *buf, int count, MPI_Status *st)
{
    for (auto it = q.begin(); it != q.end(); ++it)
    {
        if ((src != MPI_ANY_SOURCE && it->src != src) || (tag != MPI_ANY_TAG && it->tag != tag)) continue;
        if (it->type != t || it->bytes.size() > bytes(count, t)) return MPI_ERR_OTHER;
        if (!it->bytes.empty()) std::memcpy(buf, it->bytes.data(), it->bytes.size());
        if (st) *st = MPI_Status{it->src, it->tag, MPI_SUCCESS};
        q.erase(it);
        return MPI_SUCCESS;
    }
    return MPI_ERR_OTHER;
}
}  // namespace fake_mpi

inline int MPI_Comm_rank(MPI_Comm c, int *r)
{
    *r = c->rank;
    return MPI_SUCCESS;
}
inline int MPI_Comm_size(MPI_Comm c, int *n)
{
    *n = c->w->size;
    return MPI_SUCCESS;
}
inline int MPI_Send(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm c)
{
    if (fake_mpi::failing(c) || dest < 0 || dest >= c->w->size) return MPI_ERR_OTHER;
    fake_mpi::push(c->w->p2p[dest], c->rank, tag, t, buf, count);
    return MPI_SUCCESS;
}
inline int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *st)
{
    if (fake_mpi::failing(c)) return MPI_ERR_OTHER;
    return fake_mpi::pop(c->w->p2p[c->rank], src, tag, t, buf, count, st);
}
inline int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm c)
{
    if (fake_mpi::failing(c)) return MPI_ERR_OTHER;
    if (c->rank != root) return fake_mpi::pop(c->w->coll[c->rank], root, 0, t, buf, count, nullptr);
    for (int r = 0; r < c->w->size; ++r)
        if (r != root) fake_mpi::push(c->w->coll[r], root, 0, t, buf, count);
    return MPI_SUCCESS;
}
inline int MPI_Gatherv(const void *sbuf, int scount, MPI_Datatype st, void *rbuf, const int *rcounts,
                       const int *displs, MPI_Datatype rt, int root, MPI_Comm c)
{
    if (fake_mpi::failing(c) || st != rt) return MPI_ERR_OTHER;
    if (c->rank != root)
    {
        fake_mpi::push(c->w->coll[root], c->rank, 0, st, sbuf, scount);
        return MPI_SUCCESS;
    }
    for (int r = 0; r < c->w->size; ++r)
    {
        char *dst = (char *) rbuf + fake_mpi::bytes(displs[r], rt);
        if (r == root)
        {
            if (scount > rcounts[r]) return MPI_ERR_OTHER;
            if (scount) std::memcpy(dst, sbuf, fake_mpi::bytes(scount, st));
        }
        else if (fake_mpi::pop(c->w->coll[root], r, 0, rt, dst, rcounts[r], nullptr) != MPI_SUCCESS)
            return MPI_ERR_OTHER;
    }
    return MPI_SUCCESS;
}
inline int MPI_Gather(const void *sbuf, int scount, MPI_Datatype st, void *rbuf, int rcount, MPI_Datatype rt,
                      int root, MPI_Comm c)
{
    std::vector<int> counts(c->w->size, rcount), displs(c->w->size);
    for (int r = 0; r < c->w->size; ++r) displs[r] = r * rcount;
    return MPI_Gatherv(sbuf, scount, st, rbuf, counts.data(), displs.data(), rt, root, c);
}
