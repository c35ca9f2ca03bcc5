// Device helpers shared by the kernel files: read-only loads, fixed-tree
// block reductions, the SELL-32 row product and the reference's convergence
// test.
#pragma once

#include "kernels.hpp"

namespace unapgpu {

#define SMALL_D 1.0e-37   // SMALL, src/base/unap.hpp:88
#define VSMALL_D 1.0e-128 // VSMALL, src/base/unap.hpp:89

template <class T>
__device__ __forceinline__ T ldg(const T* p)
{
    return __ldg(p);
}

// true when the solver state says the kernel has nothing to do (done, or
// the BiCGStab half-step exit)
__device__ __forceinline__ bool gate_closed(const Gate& g)
{
    if (!g.st) return false;
    if ((g.mask & 1) && g.st->done) return true;
    if ((g.mask & 2) && g.st->early) return true;
    return false;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Fixed-tree block sum of K values; the result is valid in thread 0.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K])
{
    __shared__ double sm[K][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) sm[k][wid] = v[k];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double t = lane < nw ? sm[k][lane] : 0.0;
            v[k] = warp_sum(t);
        }
    }
    __syncthreads();
}

// Two-level deterministic reduction: block tree -> per-block partials -> the
// launch's last block (ticket) sums them in block order into launch slot
// r.slot; when r.fin asks for it, that block sums slots 0..nSlots-1 in order
// and calls fin(t) on one thread.
template <int K, class F>
__device__ __forceinline__ void reduce_launch(double (&v)[K], const RSpec& r, F&& fin)
{
    block_sum<K>(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) r.blockPart[blockIdx.x * K + k] = v[k];
    }
    __threadfence();
    __shared__ int amLast;
    if (threadIdx.x == 0) amLast = (atomicAdd(r.ticket, 1u) == gridDim.x - 1) ? 1 : 0;
    __syncthreads();
    if (!amLast) return;
    __threadfence();
    double s[K];
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
#pragma unroll
        for (int k = 0; k < K; ++k) s[k] += __ldcg(r.blockPart + b * K + k);
    }
    block_sum<K>(s);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) r.launchAcc[r.slot * K + k] = s[k];
        *r.ticket = 0u;
        if (r.fin != FIN_STORE && r.fin != FIN_NONE) {
            double t[K];
#pragma unroll
            for (int k = 0; k < K; ++k) t[k] = 0.0;
            for (int j = 0; j < r.nSlots; ++j) {
#pragma unroll
                for (int k = 0; k < K; ++k) t[k] += __ldcg(r.launchAcc + j * K + k);
            }
            fin(t);
        }
        __threadfence();
    }
}

// solverPerformance::checkConvergence, unapMatrixTest.cpp:3-31
__device__ __forceinline__ int check_conv(double fin, double init, double tol, double rel,
                                          int iter, int minIter)
{
    return ((fin < tol || (rel > SMALL_D && fin <= rel * init)) && iter >= minIter) ? 1 : 0;
}

// How a kernel reads the vector it multiplies: through the read-only path
// (only when nothing writes it during the launch), with plain loads (written
// earlier in the launch by this CTA), or from L2 (written earlier in the
// launch by other CTAs, after a grid-wide barrier).
enum XLoad : int { XL_NC = 0, XL_PLAIN = 1, XL_CG = 2 };

template <int XL, class T>
__device__ __forceinline__ T ldx(const T* p)
{
    if constexpr (XL == XL_NC)
        return __ldg(p);
    else if constexpr (XL == XL_CG)
        return __ldcg(p);
    else
        return *p;
}

// Matrix streams of large levels are read once per sweep: ST loads them with
// the streaming (evict-first) policy so the gathered vector stays in L2.
template <bool ST, class T>
__device__ __forceinline__ T lds(const T* p)
{
    if constexpr (ST)
        return __ldcs(p);
    else
        return __ldg(p);
}

// One row of y = A x in the reference's order (lduMatrixSpMV.cpp:83-92):
// Apsi = 0; += diag psi; then the row's faces in face order.
//
// Entries are processed in chunks of CK: all index/value loads of a chunk
// are issued, then all gathers, then the in-order accumulation, so a row of
// up to CK entries costs two dependent memory round trips.
//
// FM: each product-and-sum as one fused multiply-add (one rounding), for
// the mixed-precision solve's FP64 outer loop, where GB300's FP64 pipe and
// not the bytes bounds the SpMV; FM = false keeps the reference's separate
// roundings.
template <class T, int XL = XL_NC, bool ST = false, int CK = 8, bool FM = false>
__device__ __forceinline__ T row_apply(const Rows<T>& A, int r, const T* x)
{
    const int info = lds<ST>(A.rowInfo + r);
    const int len = info & 0xffff;
    const int base = ldg(A.sliceOff + (r >> 5)) + (r & 31);
    T acc = T(0);
    if constexpr (FM)
        acc = lds<ST>(A.diag + r) * ldx<XL>(x + r);
    else
        acc += lds<ST>(A.diag + r) * ldx<XL>(x + r);
    for (int j0 = 0; j0 < len; j0 += CK) {
        int c[CK];
        T v[CK], xv[CK];
#pragma unroll
        for (int k = 0; k < CK; ++k) {
            const int e = base + 32 * (j0 + k);
            c[k] = j0 + k < len ? lds<ST>(A.col + e) : r;
            v[k] = j0 + k < len ? lds<ST>(A.val + e) : T(0);
        }
#pragma unroll
        for (int k = 0; k < CK; ++k) xv[k] = ldx<XL>(x + c[k]);
#pragma unroll
        for (int k = 0; k < CK; ++k)
            if (j0 + k < len) {
                if constexpr (FM)
                    acc = fma(v[k], xv[k], acc);
                else
                    acc += v[k] * xv[k];
            }
    }
    return acc;
}

// Subtract a run of a row's entries from acc in entry order, j in [j0, j1):
// acc -= val[e] * x[col[e]], with the loads of each CK-entry chunk issued
// before the ordered subtractions.  x may be written concurrently by other
// wavefronts' rows (plain loads, not the read-only path).
template <class T, bool ST = false, int CK = 8>
__device__ __forceinline__ T row_subtract(const Rows<T>& A, const T* coef, int base, int j0,
                                          int j1, const T* x, T acc)
{
    for (int jc = j0; jc < j1; jc += CK) {
        int c[CK];
        T v[CK], xv[CK];
#pragma unroll
        for (int k = 0; k < CK; ++k) {
            const int e = base + 32 * (jc + k);
            const bool on = jc + k < j1;
            c[k] = on ? lds<ST>(A.col + e) : 0;
            v[k] = on ? lds<ST>(coef + e) : T(0);
        }
#pragma unroll
        for (int k = 0; k < CK; ++k) xv[k] = jc + k < j1 ? x[c[k]] : T(0);
#pragma unroll
        for (int k = 0; k < CK; ++k)
            if (jc + k < j1) acc -= v[k] * xv[k];
    }
    return acc;
}

// Row i of the AMG coarsest product x = Minv b (Minv column-major, b staged
// in sb as FP64): the columns in chunks of kDenseChunk, each chunk summed
// in ascending order from 0, the chunk sums added in chunk order from 0.
// dense_apply_kernel sums the chunks in separate threads; this one-thread
// form gives the same bits.  (kDenseChunk: kernels.hpp)
__device__ __forceinline__ double dense_row_chunked(const double* M, int n, int i,
                                                    const double* sb)
{
    double t = 0.0;
    for (int j0 = 0; j0 < n; j0 += kDenseChunk) {
        const int j1 = min(j0 + kDenseChunk, n);
        double p = 0.0;
#pragma unroll 16
        for (int j = j0; j < j1; ++j) p += __ldg(M + (size_t)j * n + i) * sb[j];
        t += p;
    }
    return t;
}

// --- finalize operations (run by one thread) -----------------------------

// do { ... } while (++nIter < maxIter && !checkConvergence(...)),
// PCG.cpp:167-180 / PBiCGStab.cpp:443-456 / MGSolve.cpp:161-176
__device__ __forceinline__ void iteration_end(KState* st)
{
    st->nIter++;
    if (!(st->nIter < st->maxIter)) {
        st->done = 1;
        return;
    }
    st->converged = check_conv(st->finalRes, st->initRes, st->tol, st->relTol, st->nIter,
                               st->minIter);
    if (st->converged) st->done = 1;
}

// rA0rA update at the top of a PBiCGStab iteration (PBiCGStab.cpp:155-243)
__device__ __forceinline__ void bicg_rr(KState* st, double rr)
{
    st->rA0rAold = st->rA0rA;
    st->rA0rA = rr;
    if (!(fabs(st->rA0rA) > SMALL_D)) {
        st->singular = 1;
        st->done = 1;
        return;
    }
    if (st->first) {
        st->useBeta = 0;
        st->first = 0;
    } else {
        st->useBeta = 1;
        st->beta = (st->rA0rA / st->rA0rAold) * (st->alpha / st->omega);
    }
}

// Solver-state update run once per reduction site with the site sums s[0..K).
__device__ __forceinline__ void apply_fin(KState* st, int fin, const double* s, int K)
{
    switch (fin) {
    case FIN_INIT_RES:
        st->initRes = sqrt(s[0]) + SMALL_D;
        st->finalRes = st->initRes;
        break;
    case FIN_RES_ONLY: st->finalRes = sqrt(s[0]) + SMALL_D; break;
    case FIN_TRUE_RES: st->trueRes = sqrt(s[0]) + SMALL_D; break;
    case FIN_PCG_WR: {
        st->wArAold = st->wArA;
        st->wArA = s[0];
        // checkSingularity(mag(wArA)), PCG.cpp:107-117
        if (!(fabs(st->wArA) > SMALL_D)) {
            st->singular = 1;
            st->done = 1;
            break;
        }
        if (st->first) {
            st->useBeta = 0;
            st->first = 0;
        } else {
            st->useBeta = 1;
            if (st->flexible && K > 1)
                st->beta = (-st->alpha * s[K > 1 ? 1 : 0]) / st->wArAold;
            else
                st->beta = st->wArA / st->wArAold;
        }
        break;
    }
    case FIN_PCG_ALPHA:
        st->wApA = s[0];
        st->alpha = st->wArA / st->wApA;
        break;
    case FIN_PCG_RES:
        st->finalRes = sqrt(s[0]) + SMALL_D;
        iteration_end(st);
        break;
    case FIN_MG_RES:
        st->finalRes = sqrt(s[0]) + SMALL_D;
        iteration_end(st);
        break;
    case FIN_BICG_INIT:
        // initial residual; s[1] = rA0.rA of the first iteration
        st->initRes = sqrt(s[0]) + SMALL_D;
        st->finalRes = st->initRes;
        st->rA0rA = 0.0;
        bicg_rr(st, s[K > 1 ? 1 : 0]);
        break;
    case FIN_BICG_ALPHA: st->alpha = st->rA0rA / s[0]; break;
    case FIN_BICG_S:
        st->finalRes = sqrt(s[0]) + SMALL_D;
        // PBiCGStab.cpp:298-349: converged on ||s|| -> x += alpha y,
        // nIterations()++, return.  `early` gates the rest of the iteration.
        if (check_conv(st->finalRes, st->initRes, st->tol, st->relTol, st->nIter + 1,
                       st->minIter)) {
            st->converged = 1;
            st->early = 1;
            st->nIter++;
        } else {
            st->converged = 0;
        }
        break;
    case FIN_BICG_OMEGA:
        st->tAtA = s[0];
        st->tAsA = s[K > 1 ? 1 : 0];
        st->omega = st->tAsA / st->tAtA;
        break;
    case FIN_BICG_RES:
        if (st->early) {  // half-step exit finished: x += alpha y is done
            st->done = 1;
            break;
        }
        // ||r|| and the loop test; s[1] = rA0.r is the next iteration's
        // rA0rA (PBiCGStab.cpp:155-196), tested for singularity only when the
        // loop continues
        st->finalRes = sqrt(s[0]) + SMALL_D;
        iteration_end(st);
        if (!st->done) bicg_rr(st, s[K > 1 ? 1 : 0]);
        break;
    default: break;
    }
}

}  // namespace unapgpu
