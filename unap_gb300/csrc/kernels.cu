// sm_103a kernels of the UNAP solve path.  Everything here is bandwidth- or
// latency-bound sparse work (no tensor-core shapes): SELL-32 row gathers with
// coalesced index/value loads, wavefront-scheduled triangular sweeps, and
// vector updates with fused warp-shuffle reductions.
//
// Reductions are deterministic and launch-free: each block reduces with a
// fixed shuffle tree, the last block of a launch (ticket counter) sums the
// block partials in a fixed order into a per-launch slot, and the last launch
// of a site sums its slots and runs a finalize step on the solver state
// (alpha, beta, residual norm, convergence test) in device memory.
//
// The library is compiled with --fmad=false so that every product and sum
// rounds separately, as the reference's loops do on the CPU.
#include <atomic>
#include <cmath>

#include "device_common.cuh"

namespace unapgpu {

static std::atomic<long long> g_launches{0};
static thread_local bool g_capturing = false;
void count_launches(long long k) { g_launches += k; }
long long launch_count() { return g_launches.load(); }
void set_capturing(bool on) { g_capturing = on; }
bool capturing() { return g_capturing; }
static inline void tick()
{
    if (!g_capturing) g_launches++;
}

// Finalize of a reduction site (the state logic is shared with the
// persistent step executor, see apply_fin in device_common.cuh).
template <int K>
__device__ void finalize(const RSpec& r, const double (&s)[K])
{
    apply_fin(r.st, r.fin, s, K);
}

// Two-level deterministic reduction + finalize.
template <int K>
__device__ __forceinline__ void reduce_and_finalize(double (&v)[K], const RSpec& r)
{
    reduce_launch<K>(v, r, [&](const double (&t)[K]) { finalize<K>(r, t); });
}

// --------------------------------------------------------------------------
// SELL-32 row helpers
// --------------------------------------------------------------------------
template <class T, int CK, bool FM>
__global__ void __launch_bounds__(kBlock) spmv_kernel(Rows<T> A, const T* __restrict__ x,
                                                      T* __restrict__ y, const T* dotWith,
                                                      RSpec red, Gate g)
{
    if (gate_closed(g)) return;
    double v[1] = {0.0};
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += gridDim.x * blockDim.x) {
        T a = row_apply<T, XL_NC, true, CK, FM>(A, r, x);
        y[r] = a;
        if (dotWith) {
            if constexpr (FM)
                v[0] = fma((double)a, (double)dotWith[r], v[0]);
            else
                v[0] += (double)a * (double)dotWith[r];
        }
    }
    if (red.blockPart) reduce_and_finalize<1>(v, red);
}

template <class T>
void k_spmv(const Exec& ex, const Rows<T>& A, const T* x, T* y, const T* dotWith, RSpec red,
            Gate g, bool fused)
{
    if (A.n <= 0) return;
    const T* dw = red.blockPart ? dotWith : nullptr;
    const dim3 grid = ex.rowGrid(A.n, red);
    tick();
    if (fused) {
        if (A.wide)
            spmv_kernel<T, 16, true><<<grid, kBlock, 0, ex.s>>>(A, x, y, dw, red, g);
        else
            spmv_kernel<T, 8, true><<<grid, kBlock, 0, ex.s>>>(A, x, y, dw, red, g);
    } else {
        if (A.wide)
            spmv_kernel<T, 16, false><<<grid, kBlock, 0, ex.s>>>(A, x, y, dw, red, g);
        else
            spmv_kernel<T, 8, false><<<grid, kBlock, 0, ex.s>>>(A, x, y, dw, red, g);
    }
}

template <class T, int CK>
__global__ void __launch_bounds__(kBlock) residual_kernel(Rows<T> A, const T* __restrict__ x,
                                                          const T* __restrict__ b,
                                                          T* __restrict__ r, RSpec red, Gate g)
{
    if (gate_closed(g)) return;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
        T a = row_apply<T, XL_NC, true, CK>(A, i, x);
        T ri = lds<true>(b + i) - a;
        r[i] = ri;
        v[0] += (double)ri * (double)ri;
    }
    if (red.blockPart) reduce_and_finalize<1>(v, red);
}

template <class T>
void k_residual(const Exec& ex, const Rows<T>& A, const T* x, const T* b, T* r, RSpec red, Gate g)
{
    if (A.n <= 0) return;
    if (A.wide)
        tick(), residual_kernel<T, 16><<<ex.rowGrid(A.n, red), kBlock, 0, ex.s>>>(A, x, b, r, red, g);
    else
        tick(), residual_kernel<T, 8><<<ex.rowGrid(A.n, red), kBlock, 0, ex.s>>>(A, x, b, r, red, g);
}

// --------------------------------------------------------------------------
// Gauss-Seidel (lduGaussSeidelSmoother.cpp:40-79) on one wavefront.
// x_c = (b_c - sum_low val x_l - sum_up val x_u) / D_c, lower-side faces
// first, each side in ascending face order, exactly the reference's
// bPrime accumulation followed by the owner-face loop.
// --------------------------------------------------------------------------
template <class T, int CK>
__global__ void __launch_bounds__(kBlock) gs_kernel(Rows<T> A, T* x, const T* __restrict__ b,
                                                    int r0, int r1, int skipUpper, Gate g)
{
    // Programmatic dependent launch: the next wavefront's kernel may begin
    // launching now.  Before griddepcontrol.wait a kernel reads only the
    // matrix, which no kernel writes; b (the previous kernel may have just
    // written it: a restriction, a conversion), x and the solver state are
    // read after it, when the previous kernel's writes are visible.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    int r = r0 + blockIdx.x * blockDim.x + threadIdx.x;
    int info = 0, base = 0;
    T d = T(1), bb = T(0);
    int c[CK];
    T v[CK];
    if (r < r1) {
        info = lds<true>(A.rowInfo + r);
        base = ldg(A.sliceOff + (r >> 5)) + (r & 31);
        d = lds<true>(A.diag + r);
        const int len = info & 0xffff;
#pragma unroll
        for (int k = 0; k < CK; ++k) {
            const int e = base + 32 * k;
            c[k] = k < len ? lds<true>(A.col + e) : 0;
            v[k] = k < len ? lds<true>(A.val + e) : T(0);
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (gate_closed(g)) return;
    if (r < r1) {
        bb = __ldcg(b + r);
        const int jEnd = skipUpper ? (info >> 16) : (info & 0xffff);
        T xv[CK];
#pragma unroll
        for (int k = 0; k < CK; ++k) xv[k] = k < jEnd ? x[c[k]] : T(0);
        T acc = bb;
#pragma unroll
        for (int k = 0; k < CK; ++k)
            if (k < jEnd) acc -= v[k] * xv[k];
        if (jEnd > CK) acc = row_subtract<T, true, CK>(A, A.val, base, CK, jEnd, x, acc);
        x[r] = acc / d;
    }
    for (r += gridDim.x * blockDim.x; r < r1; r += gridDim.x * blockDim.x) {
        const int info2 = lds<true>(A.rowInfo + r);
        const int len = info2 & 0xffff;
        const int nLow = info2 >> 16;
        const int base2 = ldg(A.sliceOff + (r >> 5)) + (r & 31);
        T acc = lds<true>(b + r);
        acc = row_subtract<T, true, CK>(A, A.val, base2, 0, nLow, x, acc);
        if (!skipUpper) acc = row_subtract<T, true, CK>(A, A.val, base2, nLow, len, x, acc);
        x[r] = acc / lds<true>(A.diag + r);
    }
}

static std::atomic<int> g_pdl{1};
static thread_local int g_pdlThread = -1;  // this thread's override (-1: none)
int set_wave_pdl(int on) { return g_pdl.exchange(on ? 1 : 0); }
int set_thread_wave_pdl(int mode)
{
    const int old = g_pdlThread;
    g_pdlThread = mode;
    return old;
}
bool wave_pdl() { return g_pdlThread >= 0 ? g_pdlThread != 0 : g_pdl.load() != 0; }
static std::atomic<int> g_rowGrid{1};
int set_wave_grid(int oneRowPerThread) { return g_rowGrid.exchange(oneRowPerThread ? 1 : 0); }

// one wavefront launch, with programmatic dependent launch when enabled
template <class T, int CK>
static void launch_gs(const Exec& ex, const Rows<T>& A, T* x, const T* b, int r0, int r1,
                      int skipUpper, Gate g)
{
    cudaLaunchConfig_t cfg = {};
    // one row per thread (every row's matrix data is loaded before the
    // dependency wait), or a grid-stride loop over at most maxBlocks CTAs;
    // wavefronts of up to 100,000 rows go out in CTAs of one warp, spread
    // over eight times as many SMs (latency-bound, as gs_sweep_packed)
    const int threads = g_rowGrid.load() && r1 - r0 <= 100000 ? 32 : kBlock;
    const long long need = div_up(r1 - r0, threads);
    cfg.gridDim = dim3((unsigned)(g_rowGrid.load() ? std::max(1LL, need) : ex.grid(r1 - r0)));
    cfg.blockDim = dim3(threads);
    cfg.stream = ex.s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = wave_pdl() ? 1 : 0;
    tick();
    UNAP_CK(cudaLaunchKernelEx(&cfg, gs_kernel<T, CK>, A, x, b, r0, r1, skipUpper, g));
}

template <class T>
void k_gs_rows(const Exec& ex, const Rows<T>& A, T* x, const T* b, int r0, int r1, bool skipUpper,
               Gate g)
{
    if (r1 <= r0) return;
    if (A.wide)
        launch_gs<T, 16>(ex, A, x, b, r0, r1, skipUpper ? 1 : 0, g);
    else
        launch_gs<T, 8>(ex, A, x, b, r0, r1, skipUpper ? 1 : 0, g);
}

template <class T>
void gs_sweep(const Exec& ex, const Level& L, const Rows<T>& A, T* x, const T* b, bool backward,
              bool xIsZero, Gate g)
{
    const int W = L.nWave;
    for (int k = 0; k < W; ++k) {
        int w = backward ? W - 1 - k : k;
        k_gs_rows<T>(ex, A, x, b, L.waveStart[w], L.waveStart[w + 1], xIsZero && !backward, g);
    }
}

// --------------------------------------------------------------------------
// DIC / DILU
// --------------------------------------------------------------------------

// lduDICPrecond::calcReciprocalD (lduDICPrecond.cpp:15-42) and the DILU
// variant (lduDILUPrecond.cpp:15-43) on one wavefront:
// dfac_c = D_c - sum over lower-side faces (asc) of (c1 c2) / dfac_l
__global__ void __launch_bounds__(kBlock) factor_kernel(Rows<double> A, const double* c1,
                                                        const double* c2, double* dfac, int r0,
                                                        int r1)
{
    for (int r = r0 + blockIdx.x * blockDim.x + threadIdx.x; r < r1;
         r += gridDim.x * blockDim.x) {
        const int info = ldg(A.rowInfo + r);
        const int nLow = info >> 16;
        const int base = ldg(A.sliceOff + (r >> 5)) + (r & 31);
        double d = ldg(A.diag + r);
        for (int j = 0; j < nLow; ++j) {
            const int e = base + 32 * j;
            d -= ldg(c1 + e) * ldg(c2 + e) / dfac[ldg(A.col + e)];
        }
        dfac[r] = d;
    }
}

__global__ void recip_kernel(int n, const double* __restrict__ d, double* __restrict__ rD)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        rD[i] = 1.0 / d[i];
}

void dic_factor(const Exec& ex, const Level& L, bool dilu, double* dfac, double* rD)
{
    Rows<double> A = rows64(L);
    // DIC: upper * upper; DILU: upper * lower.  On the lower side of a row the
    // face's upper coefficient is valT and its lower coefficient is val.
    const double* c1 = A.valT;
    const double* c2 = dilu ? A.val : A.valT;
    for (int w = 0; w < L.nWave; ++w) {
        int r0 = L.waveStart[w], r1 = L.waveStart[w + 1];
        if (r1 > r0) tick(), factor_kernel<<<ex.grid(r1 - r0), kBlock, 0, ex.s>>>(A, c1, c2, dfac, r0, r1);
    }
    if (L.n) tick(), recip_kernel<<<ex.grid(L.n), kBlock, 0, ex.s>>>(L.n, dfac, rD);
}

// forward sweep (lduDICPrecond.cpp:63-71; DILU in losort order,
// lduDILUPrecond.cpp:70-80): w_c = rD_c r_c - sum_low (rD_c coef) w_l
template <int CK>
__global__ void __launch_bounds__(kBlock) dic_fwd_kernel(Rows<double> A, const double* coef,
                                                         const double* __restrict__ rD,
                                                         const double* rr, double* w, int r0,
                                                         int r1, Gate g)
{
    // Programmatic dependent launch: the next wavefront's kernel may launch
    // now.  Before griddepcontrol.wait this kernel reads only the matrix and
    // rD (written at factorisation); r, w and the solver state after it.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int r = r0 + blockIdx.x * blockDim.x + threadIdx.x;
    int nLow = 0, base = 0;
    double rd = 0.0;
    int c[CK];
    double v[CK];
    if (r < r1) {
        nLow = ldg(A.rowInfo + r) >> 16;
        base = ldg(A.sliceOff + (r >> 5)) + (r & 31);
        rd = ldg(rD + r);
#pragma unroll
        for (int k = 0; k < CK; ++k) {
            const int e = base + 32 * k;
            c[k] = k < nLow ? ldg(A.col + e) : r;
            v[k] = k < nLow ? ldg(coef + e) : 0.0;
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (gate_closed(g) || r >= r1) return;
    // lduDICPrecond.cpp:65-71: w = rD r, then w_u -= (rD_u coef) w_l in face order
    double acc = rd * rr[r];
#pragma unroll
    for (int k = 0; k < CK; ++k)
        if (k < nLow) acc -= rd * v[k] * w[c[k]];
    for (int j = CK; j < nLow; ++j) {
        const int e = base + 32 * j;
        acc -= rd * ldg(coef + e) * w[ldg(A.col + e)];
    }
    w[r] = acc;
}

// backward sweep (lduDICPrecond.cpp:73-76): faces in reverse order,
// w_c -= (rD_c upper) w_u; sums w.r for the PCG/PBiCGStab dot product
__global__ void __launch_bounds__(kBlock) dic_bwd_kernel(Rows<double> A,
                                                         const double* __restrict__ rD,
                                                         const double* rr, double* w, int r0,
                                                         int r1, RSpec red, Gate g)
{
    // programmatic dependent launch: launch the next wavefront now, wait for
    // this one's inputs before reading anything the chain writes
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (gate_closed(g)) return;
    double v[1] = {0.0};
    for (int r = r0 + blockIdx.x * blockDim.x + threadIdx.x; r < r1;
         r += gridDim.x * blockDim.x) {
        const int info = ldg(A.rowInfo + r);
        const int len = info & 0xffff;
        const int nLow = info >> 16;
        const int base = ldg(A.sliceOff + (r >> 5)) + (r & 31);
        const double rd = ldg(rD + r);
        double acc = w[r];
        for (int j = len - 1; j >= nLow; --j) {
            const int e = base + 32 * j;
            acc -= rd * ldg(A.val + e) * w[ldg(A.col + e)];
        }
        w[r] = acc;
        v[0] += acc * rr[r];
    }
    if (red.blockPart) reduce_and_finalize<1>(v, red);
}

// wavefronts of up to this many rows launch one-warp CTAs (spread over more
// SMs, as for the Gauss-Seidel wavefronts)
constexpr int kDicSmallRows = 100000;

void dic_apply(const Exec& ex, const Level& L, bool dilu, const double* rD, const double* r,
               double* w, const RedPool* pool, int site, KState* st, int fin, Gate g)
{
    Rows<double> A = rows64(L);
    const double* coef = dilu ? A.val : A.valT;  // DIC uses upper on the lower side
    const int W = L.nWave;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.stream = ex.s;
    cfg.attrs = at;
    cfg.numAttrs = wave_pdl() ? 1 : 0;
    for (int k = 0; k < W; ++k) {
        const int r0 = L.waveStart[k], r1 = L.waveStart[k + 1];
        if (r1 <= r0) continue;
        const int threads = (r1 - r0) <= kDicSmallRows ? 32 : kBlock;
        cfg.gridDim = dim3((unsigned)div_up(r1 - r0, threads));
        cfg.blockDim = dim3((unsigned)threads);
        tick();
        UNAP_CK(cudaLaunchKernelEx(&cfg, dic_fwd_kernel<4>, A, coef, rD, r, w, r0, r1, g));
    }
    // backward: one launch slot per non-empty wavefront
    int nonEmpty = 0;
    for (int k = 0; k < W; ++k) nonEmpty += L.waveStart[k + 1] > L.waveStart[k];
    int slot = 0;
    for (int k = W - 1; k >= 0; --k) {
        const int r0 = L.waveStart[k], r1 = L.waveStart[k + 1];
        if (r1 <= r0) continue;
        RSpec red;
        if (pool) red = pool->site(site, st, slot == nonEmpty - 1 ? fin : FIN_STORE, slot, nonEmpty);
        const int threads = (r1 - r0) <= kDicSmallRows ? 32 : kBlock;
        int grid = div_up(r1 - r0, threads);
        if (red.blockPart && grid > red.maxBlocks) grid = red.maxBlocks;
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3((unsigned)threads);
        tick();
        UNAP_CK(cudaLaunchKernelEx(&cfg, dic_bwd_kernel, A, rD, r, w, r0, r1, red, g));
        ++slot;
    }
}

__global__ void __launch_bounds__(kBlock) diag_apply_kernel(int n, const double* __restrict__ rD,
                                                            const double* __restrict__ r,
                                                            double* __restrict__ w, RSpec red,
                                                            Gate g)
{
    if (gate_closed(g)) return;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double wi = rD ? rD[i] * r[i] : r[i];
        w[i] = wi;
        v[0] += wi * r[i];
    }
    if (red.blockPart) reduce_and_finalize<1>(v, red);
}

void diag_apply(const Exec& ex, int n, const double* rD, const double* r, double* w, RSpec red,
                Gate g)
{
    if (n <= 0) return;
    tick(), diag_apply_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, rD, r, w, red, g);
}

// --------------------------------------------------------------------------
// PCG vector kernels (PCG.cpp:119-151)
// --------------------------------------------------------------------------
// FM: fused multiply-adds (see row_apply), for the mixed solve's outer loop
template <bool FM>
__device__ __forceinline__ double mad(double a, double b, double c)
{
    if constexpr (FM)
        return fma(a, b, c);
    else
        return c + a * b;
}

template <bool FM>
__global__ void __launch_bounds__(kBlock) pcg_direction_kernel(int n, const double* __restrict__ w,
                                                               double* __restrict__ p,
                                                               const KState* st, Gate g)
{
    if (gate_closed(g)) return;
    const bool useBeta = st->useBeta;
    const double beta = st->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        p[i] = useBeta ? mad<FM>(beta, p[i], w[i]) : w[i];
}

void k_pcg_direction(const Exec& ex, int n, const double* w, double* p, const KState* st, Gate g,
                     bool fused)
{
    if (n <= 0) return;
    tick();
    if (fused)
        pcg_direction_kernel<true><<<ex.grid(n), kBlock, 0, ex.s>>>(n, w, p, st, g);
    else
        pcg_direction_kernel<false><<<ex.grid(n), kBlock, 0, ex.s>>>(n, w, p, st, g);
}

template <bool FM>
__global__ void __launch_bounds__(kBlock) pcg_update_kernel(int n, double* __restrict__ x,
                                                            double* __restrict__ r,
                                                            const double* __restrict__ p,
                                                            const double* __restrict__ q,
                                                            RSpec red, Gate g)
{
    if (gate_closed(g)) return;
    const double alpha = red.st->alpha;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] = mad<FM>(alpha, p[i], x[i]);
        double ri = mad<FM>(-alpha, q[i], r[i]);
        r[i] = ri;
        v[0] = mad<FM>(ri, ri, v[0]);
    }
    reduce_and_finalize<1>(v, red);
}

void k_pcg_update(const Exec& ex, int n, double* x, double* r, const double* p, const double* q,
                  RSpec red, Gate g, bool fused)
{
    if (n <= 0) return;
    tick();
    if (fused)
        pcg_update_kernel<true><<<ex.grid(n), kBlock, 0, ex.s>>>(n, x, r, p, q, red, g);
    else
        pcg_update_kernel<false><<<ex.grid(n), kBlock, 0, ex.s>>>(n, x, r, p, q, red, g);
}

template <bool FM>
__global__ void __launch_bounds__(kBlock) dot2_kernel(int n, const double* __restrict__ a,
                                                      const double* __restrict__ b,
                                                      const double* __restrict__ c,
                                                      const double* __restrict__ d, RSpec red,
                                                      Gate g)
{
    if (gate_closed(g)) return;
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        v[0] = mad<FM>(a[i], b[i], v[0]);
        if (c) v[1] = mad<FM>(c[i], d[i], v[1]);
    }
    reduce_and_finalize<2>(v, red);
}

void k_dot2(const Exec& ex, int n, const double* a, const double* b, const double* c,
            const double* d, RSpec red, Gate g, bool fused)
{
    tick();
    if (fused)
        dot2_kernel<true><<<ex.grid(n > 0 ? n : 1), kBlock, 0, ex.s>>>(n, a, b, c, d, red, g);
    else
        dot2_kernel<false><<<ex.grid(n > 0 ? n : 1), kBlock, 0, ex.s>>>(n, a, b, c, d, red, g);
}

// --------------------------------------------------------------------------
// PBiCGStab vector kernels (PBiCGStab.cpp:83-396, x86 branches)
// --------------------------------------------------------------------------

// r = b - Ax, r0 = r; sums r.r and r0.r
__global__ void __launch_bounds__(kBlock) bicg_init_kernel(int n, const double* __restrict__ b,
                                                           const double* __restrict__ Ax,
                                                           double* __restrict__ r,
                                                           double* __restrict__ r0, RSpec red)
{
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double ri = b[i] - Ax[i];
        r[i] = ri;
        r0[i] = ri;
        v[0] += ri * ri;
        v[1] += ri * ri;
    }
    reduce_and_finalize<2>(v, red);
}

void k_bicg_init(const Exec& ex, int n, const double* b, const double* Ax, double* r, double* r0,
                 RSpec red)
{
    tick(), bicg_init_kernel<<<ex.grid(n > 0 ? n : 1), kBlock, 0, ex.s>>>(n, b, Ax, r, r0, red);
}

// p = r (first) or p = r + beta (p - omega Ay)
__global__ void __launch_bounds__(kBlock) bicg_direction_kernel(int n,
                                                                const double* __restrict__ r,
                                                                const double* __restrict__ Ay,
                                                                double* __restrict__ p,
                                                                const KState* st, Gate g)
{
    if (gate_closed(g)) return;
    const bool useBeta = st->useBeta;
    const double beta = st->beta, omega = st->omega;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        p[i] = useBeta ? r[i] + beta * (p[i] - omega * Ay[i]) : r[i];
}

void k_bicg_direction(const Exec& ex, int n, const double* r, const double* Ay, double* p,
                      const KState* st, Gate g)
{
    if (n <= 0) return;
    tick(), bicg_direction_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, r, Ay, p, st, g);
}

// s = r - alpha Ay; sums s.s
__global__ void __launch_bounds__(kBlock) bicg_s_kernel(int n, const double* __restrict__ r,
                                                        const double* __restrict__ Ay,
                                                        double* __restrict__ s, RSpec red, Gate g)
{
    if (gate_closed(g)) return;
    const double alpha = red.st->alpha;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double si = r[i] - alpha * Ay[i];
        s[i] = si;
        v[0] += si * si;
    }
    reduce_and_finalize<1>(v, red);
}

void k_bicg_s(const Exec& ex, int n, const double* r, const double* Ay, double* s, RSpec red,
              Gate g)
{
    tick(), bicg_s_kernel<<<ex.grid(n > 0 ? n : 1), kBlock, 0, ex.s>>>(n, r, Ay, s, red, g);
}

// early exit: x += alpha y; else x += alpha y + omega z, r = s - omega t;
// sums r.r and r0.r (the next iteration's rA0rA)
__global__ void __launch_bounds__(kBlock) bicg_update_kernel(int n, double* __restrict__ x,
                                                             double* __restrict__ r,
                                                             const double* __restrict__ y,
                                                             const double* __restrict__ z,
                                                             const double* __restrict__ s,
                                                             const double* __restrict__ t,
                                                             const double* __restrict__ r0,
                                                             RSpec red, Gate g)
{
    if (gate_closed(g)) return;
    KState* st = red.st;
    const double alpha = st->alpha, omega = st->omega;
    double v[2] = {0.0, 0.0};
    if (st->early) {
        // PBiCGStab.cpp:310-349: x += alpha y and return (the iteration
        // count was advanced by the ||s|| finalize; the finalize of this
        // launch's reduction, run after every block has updated x, sets done)
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            x[i] += alpha * y[i];
    } else {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
             i += gridDim.x * blockDim.x) {
            x[i] += alpha * y[i] + omega * z[i];
            double ri = s[i] - omega * t[i];
            r[i] = ri;
            v[0] += ri * ri;
            v[1] += r0[i] * ri;
        }
    }
    reduce_and_finalize<2>(v, red);
}

void k_bicg_update(const Exec& ex, int n, double* x, double* r, const double* y, const double* z,
                   const double* s, const double* t, const double* r0, RSpec red, Gate g)
{
    tick(), bicg_update_kernel<<<ex.grid(n > 0 ? n : 1), kBlock, 0, ex.s>>>(n, x, r, y, z, s, t, r0, red,
                                                                    g);
}

// --------------------------------------------------------------------------
// permutations, transfers, dense coarsest solve, helpers
// --------------------------------------------------------------------------
template <class T>
__global__ void to_internal_kernel(int n, const int* __restrict__ perm, const T* __restrict__ in,
                                   T* __restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = in[perm[i]];
}

template <class T>
__global__ void to_reference_kernel(int n, const int* __restrict__ perm,
                                    const T* __restrict__ in, T* __restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[perm[i]] = in[i];
}

template <class T>
void k_to_internal(const Exec& ex, int n, const int* perm, const T* in, T* out)
{
    if (n > 0) tick(), to_internal_kernel<T><<<ex.grid(n), kBlock, 0, ex.s>>>(n, perm, in, out);
}

template <class T>
void k_to_reference(const Exec& ex, int n, const int* perm, const T* in, T* out)
{
    if (n > 0) tick(), to_reference_kernel<T><<<ex.grid(n), kBlock, 0, ex.s>>>(n, perm, in, out);
}

// restrictField (unapMatrix.hpp:378-407) in gather form: children ascending
template <class T>
__global__ void restrict_kernel(int nc, const int* __restrict__ cs, const int* __restrict__ ch,
                                const T* __restrict__ fine, T* __restrict__ coarse, Gate g)
{
    if (gate_closed(g)) return;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        T s = T(0);
        for (int k = cs[c]; k < cs[c + 1]; ++k) s += fine[ch[k]];
        coarse[c] = s;
    }
}

template <class T>
void k_restrict(const Exec& ex, int nCoarse, const int* childStart, const int* child,
                const T* fine, T* coarse, Gate g)
{
    if (nCoarse > 0)
        tick(), restrict_kernel<T><<<ex.grid(nCoarse), kBlock, 0, ex.s>>>(nCoarse, childStart, child, fine,
                                                                  coarse, g);
}

template <class T>
__global__ void prolong_add_kernel(int nf, const int* __restrict__ cmap,
                                   const T* __restrict__ coarse, T* __restrict__ fine, Gate g)
{
    if (gate_closed(g)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += gridDim.x * blockDim.x)
        fine[i] += coarse[cmap[i]];
}

template <class T>
void k_prolong_add(const Exec& ex, int nFine, const int* cmap, const T* coarse, T* fine, Gate g)
{
    if (nFine > 0)
        tick(), prolong_add_kernel<T><<<ex.grid(nFine), kBlock, 0, ex.s>>>(nFine, cmap, coarse, fine, g);
}

// Coarsest level of the AMG V-cycle: x = Minv b with the dense FP64 inverse
// (column-major; column j holds Minv[.][j] with rows in the level's internal
// order), accumulated in FP64.  Each row is summed in chunks of kDenseChunk
// columns (dense_row_chunked's order): a CTA takes 32 consecutive rows, and
// warp q of it the chunks q, q + nWarps, ... of those rows (a warp reads 32
// consecutive rows of one column per step); the chunk sums meet in shared
// memory and the first warp adds them in chunk order.  The dependency chain
// of a row is 64 + n / 64 additions instead of n.  gather (optional) maps
// column j to its entry of b.
template <class T>
__global__ void dense_apply_kernel(int n, const double* __restrict__ M, const T* __restrict__ b,
                                   const int* __restrict__ gather, T* __restrict__ x, Gate g)
{
    if (gate_closed(g)) return;
    extern __shared__ double sm[];
    double* sb = sm;  // b, n entries
    const int nChunks = (n + kDenseChunk - 1) / kDenseChunk;
    double* part = sm + n;  // [chunk][32 rows]
    for (int j = threadIdx.x; j < n; j += blockDim.x) sb[j] = (double)b[gather ? gather[j] : j];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int i = blockIdx.x * 32 + lane;
    for (int q = w; q < nChunks; q += nw) {
        double p = 0.0;
        if (i < n) {
            const int j0 = q * kDenseChunk, j1 = min(j0 + kDenseChunk, n);
#pragma unroll 16
            for (int j = j0; j < j1; ++j) p += ldg(M + (size_t)j * n + i) * sb[j];
        }
        part[q * 32 + lane] = p;
    }
    __syncthreads();
    if (w == 0 && i < n) {
        double t = 0.0;
        for (int q = 0; q < nChunks; ++q) t += part[q * 32 + lane];
        x[i] = (T)t;
    }
}

template <class T>
void k_dense_apply(const Exec& ex, int n, const double* MinvColMajor, const T* b, const int* gather,
                   T* x, Gate g)
{
    if (n <= 0) return;
    const int nChunks = (n + kDenseChunk - 1) / kDenseChunk;
    const int threads = 32 * std::min(nChunks, 32);
    const size_t smem = (size_t)(n + 32 * nChunks) * sizeof(double);
    if (smem > 48 * 1024)  // coarsest levels above 4,096 cells (the limit is 8,192)
        UNAP_CK(cudaFuncSetAttribute(dense_apply_kernel<T>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    tick(), dense_apply_kernel<T><<<div_up(n, 32), threads, smem, ex.s>>>(n, MinvColMajor, b,
                                                                          gather, x, g);
}

template <class T>
__global__ void fill_kernel(long long n, T* x, T v)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        x[i] = v;
}

template <class T>
void k_fill(const Exec& ex, long long n, T* x, T v)
{
    if (n > 0) tick(), fill_kernel<T><<<ex.grid(n), kBlock, 0, ex.s>>>(n, x, v);
}

__global__ void d2f_kernel(int n, const double* __restrict__ in, float* __restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

__global__ void f2d_kernel(int n, const float* __restrict__ in, double* __restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

void k_d2f(const Exec& ex, int n, const double* in, float* out)
{
    if (n > 0) tick(), d2f_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, in, out);
}

void k_f2d(const Exec& ex, int n, const float* in, double* out)
{
    if (n > 0) tick(), f2d_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, in, out);
}

void k_axpy_f2d(const Exec& ex, int n, const float* in, double* out) { k_f2d(ex, n, in, out); }

// scalingFactor.cpp:35-64: sums source.field and Acf.field, then a Jacobi
// step field += (source - Acf)/D
template <class T>
__global__ void __launch_bounds__(kBlock) scaling_kernel(int n, const T* __restrict__ src,
                                                         const T* __restrict__ Acf, T* field,
                                                         const T* __restrict__ D, RSpec red,
                                                         Gate g)
{
    if (gate_closed(g)) return;
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        T f = field[i];
        v[0] += (double)(src[i] * f);
        v[1] += (double)(Acf[i] * f);
        field[i] = f + (src[i] - Acf[i]) / D[i];
    }
    reduce_and_finalize<2>(v, red);
}

template <class T>
void k_scaling_sums(const Exec& ex, int n, const T* source, const T* Acf, T* field, const T* D,
                    RSpec red, Gate g)
{
    tick(), scaling_kernel<T><<<ex.grid(n > 0 ? n : 1), kBlock, 0, ex.s>>>(n, source, Acf, field, D, red,
                                                                   g);
}

template <class T>
__global__ void axpby_kernel(int n, T a, const T* __restrict__ x, T b, T* __restrict__ y, Gate g)
{
    if (gate_closed(g)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] = a * x[i] + b * y[i];
}

template <class T>
void k_axpby(const Exec& ex, int n, T a, const T* x, T b, T* y, Gate g)
{
    if (n > 0) tick(), axpby_kernel<T><<<ex.grid(n), kBlock, 0, ex.s>>>(n, a, x, b, y, g);
}

// --------------------------------------------------------------------------
Rows<double> rows64(const Level& L)
{
    Rows<double> A;
    A.n = L.n;
    A.sliceOff = L.d_sliceOff.p;
    A.rowInfo = L.d_rowInfo.p;
    A.col = L.d_col.p;
    A.val = L.d_val.p;
    A.valT = L.symm ? L.d_val.p : L.d_valT.p;
    A.diag = L.d_diag.p;
    A.wide = 2.0 * L.nf > 8.5 * L.n ? 1 : 0;
    return A;
}

Rows<float> rows32(const Level& L)
{
    Rows<float> A;
    A.n = L.n;
    A.sliceOff = L.d_sliceOff.p;
    A.rowInfo = L.d_rowInfo.p;
    A.col = L.d_col.p;
    A.val = L.d_val32.p;
    A.valT = L.d_val32.p;
    A.diag = L.d_diag32.p;
    A.wide = 2.0 * L.nf > 8.5 * L.n ? 1 : 0;
    return A;
}

void make_fp32(Level& L, cudaStream_t s)
{
    if (L.d_val32.p) return;
    Exec ex;
    ex.s = s;
    ex.maxBlocks = device_max_blocks();
    L.d_val32.alloc((size_t)L.nEntries);
    L.d_diag32.alloc((size_t)L.n);
    if (L.nEntries) tick(), d2f_kernel<<<ex.grid(L.nEntries), kBlock, 0, s>>>((int)L.nEntries, L.d_val.p, L.d_val32.p);
    if (L.n) tick(), d2f_kernel<<<ex.grid(L.n), kBlock, 0, s>>>(L.n, L.d_diag.p, L.d_diag32.p);
    UNAP_CK(cudaGetLastError());
}

void RedPool::init(int sites, int blocks, int launches, cudaStream_t s)
{
    nSites = sites;
    maxBlocks = blocks;
    maxLaunch = launches;
    blockPart.alloc((size_t)sites * blocks * kRedK);
    launchAcc.alloc((size_t)sites * launches * kRedK);
    tickets.alloc((size_t)sites);
    tickets.zero(s);
}

RSpec RedPool::site(int i, KState* st, int fin, int slot, int nSlots) const
{
    RSpec r;
    r.blockPart = blockPart.p + (size_t)i * maxBlocks * kRedK;
    r.launchAcc = launchAcc.p + (size_t)i * maxLaunch * kRedK;
    r.ticket = tickets.p + i;
    r.slot = slot;
    r.nSlots = nSlots;
    r.fin = fin;
    r.st = st;
    r.maxBlocks = maxBlocks;
    return r;
}

int device_max_blocks()
{
    static int cached = 0;
    if (!cached) {
        int dev = 0, sms = 0, perSm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&perSm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
        if (sms <= 0) sms = 152;
        if (perSm <= 0) perSm = 2048;
        cached = sms * (perSm / kBlock);
    }
    return cached;
}

// --------------------------------------------------------------------------
// explicit instantiations
// --------------------------------------------------------------------------
#define INST(T)                                                                                   \
    template void k_spmv<T>(const Exec&, const Rows<T>&, const T*, T*, const T*, RSpec, Gate,      \
                            bool);                                                               \
    template void k_residual<T>(const Exec&, const Rows<T>&, const T*, const T*, T*, RSpec, Gate); \
    template void k_gs_rows<T>(const Exec&, const Rows<T>&, T*, const T*, int, int, bool, Gate);   \
    template void gs_sweep<T>(const Exec&, const Level&, const Rows<T>&, T*, const T*, bool, bool, \
                              Gate);                                                              \
    template void k_to_internal<T>(const Exec&, int, const int*, const T*, T*);                   \
    template void k_to_reference<T>(const Exec&, int, const int*, const T*, T*);                  \
    template void k_restrict<T>(const Exec&, int, const int*, const int*, const T*, T*, Gate);    \
    template void k_prolong_add<T>(const Exec&, int, const int*, const T*, T*, Gate);             \
    template void k_dense_apply<T>(const Exec&, int, const double*, const T*, const int*, T*, Gate);          \
    template void k_fill<T>(const Exec&, long long, T*, T);                                        \
    template void k_scaling_sums<T>(const Exec&, int, const T*, const T*, T*, const T*, RSpec,    \
                                    Gate);                                                        \
    template void k_axpby<T>(const Exec&, int, T, const T*, T, T*, Gate);

INST(double)
INST(float)
template void k_fill<int>(const Exec&, long long, int*, int);

}  // namespace unapgpu
