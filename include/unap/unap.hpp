/* UNAP C++ API for the GB300 library: base types and macros.
 *
 * The headers in this directory declare the classes of the reference's C++
 * API (namespace UNAP: src/base/unap.hpp, src/base/vectors/unapVector.hpp,
 * src/matrix/unapMatrix.hpp:9-373, the concrete solvers, preconditioners,
 * smoothers and agglomeration) with the same names, constructors and
 * virtual functions, so a C++ code written against UNAP compiles against
 * them unchanged.  Vectors and matrix arrays are host containers, as in the
 * reference; every numerical operation (SpMV, preconditioning, smoothing,
 * agglomeration, the solves) goes through the C ABI of libunap_cuda.so
 * (unap_cuda.h) to the GPU.  There is no CPU fallback: a failed call prints
 * the library's error and exits, as the reference's CHECK_POINTER does.
 *
 * Everything is inline, so `label` may be 32- or 64-bit (-DLABEL_INT64)
 * without a library of matching layout: labels are converted to the C ABI's
 * int at the boundary (a size beyond 2^31 - 1 is an error).  Scalars are
 * double (the reference's SCALAR_FLOAT64). */
#ifndef UNAP_HPP
#define UNAP_HPP

#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <iostream>
#include <typeinfo>

#include "../unap_cuda.h"

#if defined(SCALAR_FLOAT32)
#error "the GB300 library computes in double-precision scalars (SCALAR_FLOAT64)"
#endif

namespace UNAP
{
#if defined(LABEL_INT64)
typedef long int label;
#else
typedef int label;
#endif
typedef double scalar;

#define COUT std::cout
#define ENDL std::endl
#define EXIT exit(0)
#define ERROR_EXIT exit(1)

/* loop over [0, length) */
#define forAll(i, length) for (int i = 0; i < (length); i++)

#define SMALL (1.0e-37)
#define VSMALL (1.0e-128)
#define GREAT (1.0e+37)
#define VGREAT (1.0e+128)

#define CHECK_POINTER(ptr)                                                                 \
    if (!(ptr)) {                                                                          \
        COUT << "ERROR in " << __FILE__ << " " << __LINE__ << ": " << #ptr << " is NULL!" \
             << ENDL;                                                                      \
        ERROR_EXIT;                                                                        \
    }
#define DELETE_POINTER(ptr) \
    if (ptr) {              \
        delete[] ptr;       \
        ptr = NULL;         \
    }
#define DELETE_OBJECT_POINTER(ptr) \
    if (ptr) {                     \
        delete ptr;                \
        ptr = NULL;                \
    }
/* ptr = new copy of oldObj */
#define ALLOCATE_POINTER(ptr, oldObj, T) \
    {                                    \
        DELETE_OBJECT_POINTER(ptr)       \
        ptr = new T((oldObj).size());    \
        *ptr = (oldObj);                 \
    }
#define MAX(x, y) (((x) > (y)) ? (x) : (y))
#define MIN(x, y) (((x) < (y)) ? (x) : (y))

template <typename T>
T mag(T v)
{
    return v < T(0) ? -v : v;
}

namespace detail
{
/* a failed library call: print its error and exit (the reference exits on
 * errors it detects) */
inline void check(int rc, const char* what)
{
    if (rc != UNAP_CUDA_OK) {
        std::cerr << "UNAP (GB300): " << what << " failed: " << unap_cuda_last_error()
                  << std::endl;
        ERROR_EXIT;
    }
}

inline int to_int(long long v, const char* what)
{
    if (v < 0 || v > 2147483647LL) {
        std::cerr << "UNAP (GB300): " << what << " out of the 32-bit range of the C ABI"
                  << std::endl;
        ERROR_EXIT;
    }
    return (int)v;
}
}  // namespace detail

}  // namespace UNAP

#endif
