/* Empty stand-in: src/matchedFilter.cpp includes <mkl_cblas.h> but calls no
 * CBLAS routine.  TEST INFRASTRUCTURE ONLY (oracle/_ref build). */
#ifndef ORC_SHIM_MKL_CBLAS_H
#define ORC_SHIM_MKL_CBLAS_H
#endif
