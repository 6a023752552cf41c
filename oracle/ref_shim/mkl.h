/*
 * Project-written stand-in for the MKL allocator calls used by the mflib
 * hot-path sources (MKL_calloc/MKL_free, mkl_calloc/mkl_free, mkl_finalize).
 * TEST INFRASTRUCTURE ONLY (oracle/_ref build).
 */
#ifndef ORC_SHIM_MKL_H
#define ORC_SHIM_MKL_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
void *MKL_calloc(size_t num, size_t size, int alignment);
void MKL_free(void *p);
void *mkl_calloc(size_t num, size_t size, int alignment);
void mkl_free(void *p);
void mkl_finalize(void);
#ifdef __cplusplus
}
#endif
#endif
