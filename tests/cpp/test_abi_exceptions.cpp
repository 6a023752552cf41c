// Exceptions never cross the C ABI: every entry point catches them with
// the handler below, which maps each kind to a status code and leaves the
// exception's text in mfgpu_last_error().  No GPU needed.
#include <cstdio>
#include <cstring>
#include <new>
#include <stdexcept>
#include "mfgpu.h"

namespace mfgpu
{
mfgpu_status status_of_exception() noexcept;
}

template <class E> static int check(const E &e, mfgpu_status want, const char *text)
{
    mfgpu_status got = MFGPU_OK;
    try
    {
        throw e;
    }
    catch (...)
    {
        got = mfgpu::status_of_exception();
    }
    const char *msg = mfgpu_last_error();
    if (got != want || !msg || !std::strstr(msg, text))
    {
        std::printf("FAIL: status %d (want %d), message '%s' (want '%s')\n", (int) got, (int) want, msg ? msg : "",
                    text);
        return 1;
    }
    return 0;
}

int main()
{
    int bad = 0;
    bad += check(std::bad_alloc(), MFGPU_ENOMEM, "host exception");
    bad += check(std::invalid_argument("n_obs = -1"), MFGPU_EINVAL, "n_obs = -1");
    bad += check(std::out_of_range("vector index 7"), MFGPU_EINVAL, "vector index 7");
    bad += check(std::runtime_error("bad state"), MFGPU_ESTATE, "bad state");
    bad += check(42, MFGPU_ESTATE, "unknown exception");
    if (bad == 0) std::puts("ALL PASSED");
    return bad;
}
