// Single-CTA Krylov solves: one thread block runs a whole PCG or PBiCGStab
// solve (PCG.cpp:35-183, PBiCGStab.cpp:45-459) on a small LDU system held in
// global memory (L2-resident), with __syncthreads between vector steps and
// wavefront-by-wavefront DIC/DILU sweeps.  One launch solves a batch: block
// b takes system b.  Used for the MGSolver's coarsest level
// (solveCoarsestLevel.cpp:10-55: PCG+DIC or PBiCGStab+DILU, relTol 1e-2,
// maxIter 100, x0 = 0) and for small systems of a batch.
//
// Rows are computed with the same per-row formulas as the multi-block
// kernels, so SpMV and preconditioner applications are bit-identical to
// them; dot products use the fixed block reduction tree.
#include "device_common.cuh"
#include "small_solve.hpp"

namespace unapgpu {

namespace {

__device__ double blk_dot(int n, const double* a, const double* b)
{
    __shared__ double out;
    double v[1] = {0.0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) v[0] += a[i] * b[i];
    block_sum<1>(v);
    if (threadIdx.x == 0) out = v[0];
    __syncthreads();
    return out;
}

__device__ void blk_spmv(const Rows<double>& A, const double* x, double* y)
{
    for (int i = threadIdx.x; i < A.n; i += blockDim.x) y[i] = row_apply<double, XL_PLAIN>(A, i, x);
    __syncthreads();
}

// w = M^-1 r (unapMatrixPrecond.cpp, lduDiagPrecond.cpp:44-73,
// lduDICPrecond.cpp:45-77, lduDILUPrecond.cpp:46-86)
__device__ void blk_precond(const SmallSystem& S, const double* r, double* w)
{
    const Rows<double>& A = S.A;
    const int n = A.n;
    if (S.precond == 0 || S.precond == 1) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) w[i] = S.precond ? S.rD[i] * r[i] : r[i];
        __syncthreads();
        return;
    }
    const double* coef = S.precond == 3 ? A.val : A.valT;
    for (int k = 0; k < S.nWave; ++k) {
        for (int i = S.waveStart[k] + threadIdx.x; i < S.waveStart[k + 1]; i += blockDim.x) {
            const int info = A.rowInfo[i];
            const int nLow = info >> 16;
            const int base = A.sliceOff[i >> 5] + (i & 31);
            const double rd = S.rD[i];
            double acc = rd * r[i];
            for (int j = 0; j < nLow; ++j) {
                const int e = base + 32 * j;
                acc -= rd * coef[e] * w[A.col[e]];
            }
            w[i] = acc;
        }
        __syncthreads();
    }
    for (int k = S.nWave - 1; k >= 0; --k) {
        for (int i = S.waveStart[k] + threadIdx.x; i < S.waveStart[k + 1]; i += blockDim.x) {
            const int info = A.rowInfo[i];
            const int len = info & 0xffff;
            const int nLow = info >> 16;
            const int base = A.sliceOff[i >> 5] + (i & 31);
            const double rd = S.rD[i];
            double acc = w[i];
            for (int j = len - 1; j >= nLow; --j) {
                const int e = base + 32 * j;
                acc -= rd * A.val[e] * w[A.col[e]];
            }
            w[i] = acc;
        }
        __syncthreads();
    }
}

__device__ void small_pcg(const SmallSystem& S, SmallResult& R)
{
    const int n = S.A.n;
    double* x = S.x;
    double* p = S.work;
    double* w = S.work + n;
    double* r = S.work + 2 * n;
    blk_spmv(S.A, x, w);
    for (int i = threadIdx.x; i < n; i += blockDim.x) r[i] = S.b[i] - w[i];
    __syncthreads();
    R.initRes = sqrt(blk_dot(n, r, r)) + SMALL_D;
    R.finalRes = R.initRes;
    double wArA = 1.0e37, wArAold;
    for (;;) {
        wArAold = wArA;
        blk_precond(S, r, w);
        wArA = blk_dot(n, w, r);
        if (!(fabs(wArA) > SMALL_D)) {
            R.singular = 1;
            break;
        }
        const bool first = R.nIter == 0;
        const double beta = first ? 0.0 : wArA / wArAold;
        for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = first ? w[i] : w[i] + beta * p[i];
        __syncthreads();
        blk_spmv(S.A, p, w);
        const double wApA = blk_dot(n, w, p);
        const double alpha = wArA / wApA;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            x[i] += alpha * p[i];
            r[i] -= alpha * w[i];
        }
        __syncthreads();
        R.finalRes = sqrt(blk_dot(n, r, r)) + SMALL_D;
        if (!(++R.nIter < S.maxIter)) break;
        R.converged = check_conv(R.finalRes, R.initRes, S.tol, S.relTol, R.nIter, S.minIter);
        if (R.converged) break;
    }
}

__device__ void small_bicgstab(const SmallSystem& S, SmallResult& R)
{
    const int n = S.A.n;
    double* x = S.x;
    double* p = S.work;
    double* y = S.work + n;
    double* r = S.work + 2 * n;
    double* r0 = S.work + 3 * n;
    double* Ay = S.work + 4 * n;
    double* s = S.work + 5 * n;
    double* z = S.work + 6 * n;
    double* t = S.work + 7 * n;
    blk_spmv(S.A, x, y);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        r[i] = S.b[i] - y[i];
        r0[i] = r[i];
    }
    __syncthreads();
    R.initRes = sqrt(blk_dot(n, r, r)) + SMALL_D;
    R.finalRes = R.initRes;
    double rA0rA = 0, alpha = 0, omega = 0;
    for (;;) {
        const double rA0rAold = rA0rA;
        rA0rA = blk_dot(n, r0, r);
        if (!(fabs(rA0rA) > SMALL_D)) {
            R.singular = 1;
            break;
        }
        if (R.nIter == 0) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = r[i];
        } else {
            const double beta = (rA0rA / rA0rAold) * (alpha / omega);
            for (int i = threadIdx.x; i < n; i += blockDim.x)
                p[i] = r[i] + beta * (p[i] - omega * Ay[i]);
        }
        __syncthreads();
        blk_precond(S, p, y);
        blk_spmv(S.A, y, Ay);
        alpha = rA0rA / blk_dot(n, r0, Ay);
        for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = r[i] - alpha * Ay[i];
        __syncthreads();
        R.finalRes = sqrt(blk_dot(n, s, s)) + SMALL_D;
        if (check_conv(R.finalRes, R.initRes, S.tol, S.relTol, R.nIter + 1, S.minIter)) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] += alpha * y[i];
            __syncthreads();
            R.converged = 1;
            R.nIter++;
            return;
        }
        blk_precond(S, s, z);
        blk_spmv(S.A, z, t);
        const double tAtA = blk_dot(n, t, t);
        omega = blk_dot(n, t, s);
        omega /= tAtA;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            x[i] += alpha * y[i] + omega * z[i];
            r[i] = s[i] - omega * t[i];
        }
        __syncthreads();
        R.finalRes = sqrt(blk_dot(n, r, r)) + SMALL_D;
        if (!(++R.nIter < S.maxIter)) break;
        R.converged = check_conv(R.finalRes, R.initRes, S.tol, S.relTol, R.nIter, S.minIter);
        if (R.converged) break;
    }
}

template <int NT>
__global__ void __launch_bounds__(NT) small_krylov_kernel(const SmallSystem* systems,
                                                          const KState* gate)
{
    if (gate && gate->done) return;
    const SmallSystem S = systems[blockIdx.x];
    SmallResult R{};
    if (S.zeroX) {
        for (int i = threadIdx.x; i < S.A.n; i += blockDim.x) S.x[i] = 0.0;
        __syncthreads();
    }
    if (S.method == 1)
        small_bicgstab(S, R);
    else
        small_pcg(S, R);
    if (threadIdx.x == 0 && S.result) *S.result = R;
}

}  // namespace

void launch_small_krylov(cudaStream_t s, const SmallSystem* d_systems, int count,
                         const KState* gate, int threads)
{
    if (count <= 0) return;
    if (!capturing()) count_launches(1);
    switch (threads) {
    case 128: small_krylov_kernel<128><<<count, 128, 0, s>>>(d_systems, gate); break;
    case 256: small_krylov_kernel<256><<<count, 256, 0, s>>>(d_systems, gate); break;
    case 1024: small_krylov_kernel<1024><<<count, 1024, 0, s>>>(d_systems, gate); break;
    default: small_krylov_kernel<512><<<count, 512, 0, s>>>(d_systems, gate); break;
    }
}

}  // namespace unapgpu
