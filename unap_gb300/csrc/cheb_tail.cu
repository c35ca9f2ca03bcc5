// The coarse end of a Chebyshev V-cycle in one thread-block-cluster launch
// (see cheby.hpp).  From the first tail level down to the coarsest and back,
// every step of the per-step V-cycle — Chebyshev steps, residual,
// restriction fused with the next level's first step, the coarsest dense
// product, prolongation — runs as a pass of the cluster's threads over the
// level's rows, separated by cluster barriers (barrier.cluster
// arrive.release / wait.acquire) instead of kernel launches.  Each row's
// arithmetic is the per-step kernels' (cheb_step_kernel, residual_kernel,
// restrict_cheb_zero_kernel, prolong_to_kernel, dense_apply_kernel's chunk
// order), so the V-cycle's bits are the same either way.  Vectors live in
// global memory; those written in the launch are read from L2
// (ld.global.cg).
#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "cheby.hpp"
#include "device_common.cuh"

namespace unapgpu {

namespace {

std::atomic<int> g_chebTailRows{0};

__device__ __forceinline__ void ct_sync()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

template <class T>
__device__ __forceinline__ T ldc(const T* p)
{
    return __ldcg(p);
}

// one Chebyshev step over the level's rows (cheb_step_kernel's formulas)
template <class T>
__device__ void ct_cheb(const ChebTailLevel<T>& L, int g, int stride, const T* xin, T* xout, T c1,
                        T c2, int first)
{
    const Rows<T>& A = L.A;
    for (int r = g; r < A.n; r += stride) {
        const T acc = row_apply<T, XL_CG>(A, r, xin);
        const T d = __ldg(A.diag + r);
        const T bb = ldc(L.b + r);
        const T rD = T(1) / d;
        T wi;
        if (first)
            wi = rD * (bb - acc) * c1;
        else
            wi = c1 * ldc(L.w + r) + c2 * rD * (bb - acc);
        L.w[r] = wi;
        xout[r] = ldc(xin + r) + wi;
    }
}

template <class T, int C>
__global__ void __launch_bounds__(512) cheb_tail_kernel(ChebTailArgs<T> a, Gate g)
{
    if (gate_closed(g)) return;
    const int rank = C == 1 ? 0 : (int)(blockIdx.x % C);
    const int gt = rank * (int)blockDim.x + (int)threadIdx.x;
    const int stride = C * (int)blockDim.x;
    const int deg = a.deg;
    // down: levels first .. coarsest - 1 (level 0 of the args is the first
    // tail level, its b, first iterate and w set by the restriction before
    // the launch)
    for (int l = 0; l < a.nLev; ++l) {
        const ChebTailLevel<T>& L = a.lev[l];
        for (int j = 1; j < deg; ++j) {
            ct_cheb(L, gt, stride, L.cb[(j - 1) & 1], L.cb[j & 1], L.d1[j], L.d2[j], 0);
            ct_sync();
        }
        // residual r = b - A x into the w / r buffer (residual_kernel)
        for (int r = gt; r < L.A.n; r += stride) {
            const T ax = row_apply<T, XL_CG>(L.A, r, L.x);
            L.w[r] = ldc(L.b + r) - ax;
        }
        ct_sync();
        if (l + 1 < a.nLev) {
            // restriction fused with the next level's first step
            // (restrict_cheb_zero_kernel)
            const ChebTailLevel<T>& N = a.lev[l + 1];
            for (int c = gt; c < N.A.n; c += stride) {
                T acc = T(0);
                const int k1 = N.childStart[c + 1];
                for (int k = N.childStart[c]; k < k1; ++k) acc += ldc(L.w + N.child[k]);
                N.b[c] = acc;
                const T rD = T(1) / __ldg(N.A.diag + c);
                const T wi = rD * acc * N.Rth;
                N.w[c] = wi;
                N.cb[0][c] = wi;
            }
        } else {
            // restriction into the coarsest level (restrict_kernel)
            for (int c = gt; c < a.nc; c += stride) {
                T acc = T(0);
                const int k1 = a.cChildStart[c + 1];
                for (int k = a.cChildStart[c]; k < k1; ++k) acc += ldc(L.w + a.cChild[k]);
                a.cb[c] = acc;
            }
        }
        ct_sync();
    }
    // coarsest: x = Minv b in FP64, dense_row_chunked's order: the (row,
    // chunk) partial sums first, then each row adds its chunks in order
    {
        const int n = a.nc;
        const int nChunks = (n + kDenseChunk - 1) / kDenseChunk;
        for (int p = gt; p < n * nChunks; p += stride) {
            const int i = p % n, q = p / n;
            const int j0 = q * kDenseChunk, j1 = min(j0 + kDenseChunk, n);
            double s = 0.0;
            for (int j = j0; j < j1; ++j)
                s += __ldg(a.Minv + (size_t)j * n + i) * (double)ldc(a.cb + j);
            a.part[p] = s;
        }
        ct_sync();
        for (int i = gt; i < n; i += stride) {
            double t = 0.0;
            for (int q = 0; q < nChunks; ++q) t += __ldcg(a.part + (size_t)q * n + i);
            a.cx[i] = (T)t;
        }
        ct_sync();
    }
    // up: coarsest - 1 .. first
    for (int l = a.nLev - 1; l >= 0; --l) {
        const ChebTailLevel<T>& L = a.lev[l];
        const T* coarseX = l + 1 < a.nLev ? a.lev[l + 1].x : a.cx;
        const int* cmap = l + 1 < a.nLev ? a.lev[l + 1].cmap : a.cCmap;
        // prolongation into the buffer the post-smoothing chain starts from
        T* prev = L.post;
        for (int r = gt; r < L.A.n; r += stride)
            prev[r] = ldc(L.x + r) + ldc(coarseX + cmap[r]);
        ct_sync();
        for (int j = 0; j < deg; ++j) {
            T* out = L.cb[j & 1];
            ct_cheb(L, gt, stride, prev, out, j == 0 ? L.Rth : L.d1[j], j == 0 ? T(0) : L.d2[j],
                    j == 0 ? 1 : 0);
            ct_sync();
            prev = out;
        }
    }
}

template <class T, int C>
void ct_launch(const Exec& ex, const ChebTailArgs<T>& a, Gate g, int threads)
{
    static std::mutex m;
    static std::vector<int> done;
    int dev = 0;
    UNAP_CK(cudaGetDevice(&dev));
    {
        // (set already by cheby_tail_cluster() at setup on the first device)
        std::lock_guard<std::mutex> lk(m);
        if (std::find(done.begin(), done.end(), dev) == done.end()) {
            if (C > 8 && !capturing())
                UNAP_CK(cudaFuncSetAttribute(cheb_tail_kernel<T, C>,
                                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
            done.push_back(dev);
        }
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.stream = ex.s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    UNAP_CK(cudaLaunchKernelEx(&cfg, cheb_tail_kernel<T, C>, a, g));
}

}  // namespace

int set_cheby_tail_rows(int rows) { return g_chebTailRows.exchange(std::max(rows, 0)); }
int cheby_tail_rows() { return g_chebTailRows.load(); }

int cheby_tail_cluster()
{
    static std::atomic<int> cached{-1};
    int c = cached.load();
    if (c >= 0) return c;
    c = 0;
    for (int C : {16, 8}) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(C);
        cfg.blockDim = dim3(512);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = C;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        cudaError_t e;
        if (C == 16) {
            // both precisions' attributes here, at hierarchy setup, outside
            // any stream capture
            cudaFuncSetAttribute(cheb_tail_kernel<float, 16>,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            cudaFuncSetAttribute(cheb_tail_kernel<double, 16>,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            e = cudaOccupancyMaxActiveClusters(&n, cheb_tail_kernel<float, 16>, &cfg);
        } else {
            e = cudaOccupancyMaxActiveClusters(&n, cheb_tail_kernel<float, 8>, &cfg);
        }
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            continue;
        }
        if (n >= 1) {
            c = C;
            break;
        }
    }
    cached = c;
    return c;
}

template <class T>
void launch_cheb_tail(const Exec& ex, const ChebTailArgs<T>& a, Gate g)
{
    if (a.nLev < 1 || a.nLev > kChebTailMaxLevels)
        throw std::invalid_argument("Chebyshev tail: 1 to 8 levels above the coarsest");
    if (!capturing()) count_launches(1);
    if (cheby_tail_cluster() == 16)
        ct_launch<T, 16>(ex, a, g, 512);
    else
        ct_launch<T, 8>(ex, a, g, 512);
}

template void launch_cheb_tail<float>(const Exec&, const ChebTailArgs<float>&, Gate);
template void launch_cheb_tail<double>(const Exec&, const ChebTailArgs<double>&, Gate);

}  // namespace unapgpu
