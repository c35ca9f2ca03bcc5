// Chebyshev smoothing and the diagonal-PCG eigenvalue estimate on the device
// (see cheby.hpp).
#include <atomic>
#include <cmath>
#include <vector>

#include "cheby.hpp"
#include "device_common.cuh"

namespace unapgpu {

namespace {

void tick()
{
    if (!capturing()) count_launches(1);
}

std::atomic<int> g_smallRows{100000};
// 0: 16 entries on long-row levels below kChunk8Rows rows, else 8.  Large
// FP32 levels are bandwidth-bound and the 8-entry form holds six CTAs per
// SM instead of four (256^3 hierarchy, level 1: 163 vs 179 us per step);
// small ones are latency-bound and want one round trip per row.
std::atomic<int> g_chunk{0};
constexpr int kChunk8Rows = 1 << 20;

// ---- eigenDiagPCG::diagPCGLoops (eigenDiagPCG.cpp:48-238) ----------------
__global__ void __launch_bounds__(kBlock) eig_wr_kernel(int n, const double* __restrict__ rD,
                                                        const double* __restrict__ rA,
                                                        double* __restrict__ wA, EigState* es,
                                                        int it, RSpec red)
{
    if (es->broken) return;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double w = rD[i] * rA[i];
        wA[i] = w;
        v[0] += w * rA[i];
    }
    reduce_launch<1>(v, red, [&](const double (&t)[1]) {
        es->wArAold = es->wArA;
        es->wArA = t[0];
        if (fabs(es->wArA) < VSMALL_D) {
            es->broken = 1;
        } else if (it == 0) {
            es->betas[0] = 0.0;
        } else {
            es->beta = es->wArA / es->wArAold;
            es->betas[it] = es->beta;
        }
    });
}

__global__ void eig_p_kernel(int n, const double* __restrict__ wA, double* __restrict__ pA,
                             const EigState* es, int it)
{
    if (es->broken) return;
    const double beta = es->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        pA[i] = it == 0 ? wA[i] : wA[i] + beta * pA[i];
}

__global__ void __launch_bounds__(kBlock) eig_alpha_kernel(Rows<double> A,
                                                           const double* __restrict__ pA,
                                                           double* __restrict__ wA, EigState* es,
                                                           int it, RSpec red)
{
    if (es->broken) return;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
        double w = row_apply<double>(A, i, pA);
        wA[i] = w;
        v[0] += w * pA[i];
    }
    reduce_launch<1>(v, red, [&](const double (&t)[1]) {
        es->wApA = t[0];
        es->alpha = es->wArA / es->wApA;
        es->alphas[it] = es->alpha;
    });
}

__global__ void eig_update_kernel(int n, double* __restrict__ x, double* __restrict__ rA,
                                  const double* __restrict__ pA, const double* __restrict__ wA,
                                  const EigState* es)
{
    if (es->broken) return;
    const double alpha = es->alpha;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += alpha * pA[i];
        rA[i] -= alpha * wA[i];
    }
}

// Lanczos tridiagonal + Sturm-sequence bisection to 1e-5 (k = 1), over the
// iterations the diagonal PCG completed
__global__ void eig_sturm_kernel(EigState* es, int nMax)
{
    int nP = 0;
    while (nP < nMax && nP < 16 && es->alphas[nP] != 0.0) ++nP;
    if (nP < 2) {
        es->maxEig = nP == 1 ? 1.0 / es->alphas[0] : 1.0;
        return;
    }
    double T[16][16];
    for (int i = 0; i < nP; ++i)
        for (int j = 0; j < nP; ++j) T[i][j] = 0;
    for (int i = 0; i < nP; ++i) {
        if (i == 0)
            T[i][i] = 1.0 / es->alphas[i];
        else
            T[i][i] = 1.0 / es->alphas[i] + es->betas[i] / es->alphas[i - 1];
        if (i < nP - 1) T[i][i + 1] = sqrt(es->betas[i + 1]) / es->alphas[i];
        if (i > 0) T[i][i - 1] = T[i - 1][i];
    }
    double xBegin = 0.0, xEnd = 0.0;
    for (int i = 0; i < nP; ++i) {
        double Tr = (i == nP - 1) ? 0 : T[i][i + 1];
        double Tl = (i == 0) ? 0 : T[i][i - 1];
        double lambMax = T[i][i] + fabs(Tr) + fabs(Tl);
        double lambMin = T[i][i] - fabs(Tr) - fabs(Tl);
        xBegin = (xBegin >= lambMin) ? lambMin : xBegin;
        xEnd = (xEnd <= lambMax) ? lambMax : xEnd;
    }
    double p[16];
    double xn = 0.0;
    int guard = 0;
    do {
        xn = (xBegin + xEnd) * 0.5;
        int s = 0;
        p[0] = xn - T[0][0];
        if (p[0] < 0) s = 1;
        p[1] = (xn - T[1][1]) * p[0] - T[0][1] * T[0][1];
        if (p[1] * p[0] < 0) s++;
        for (int k = 2; k < nP; ++k) {
            p[k] = (xn - T[k][k]) * p[k - 1] - T[k - 1][k] * T[k - 1][k] * p[k - 2];
            if (p[k] * p[k - 1] < 0) s++;
        }
        if (s >= 1)
            xBegin = xn;
        else
            xEnd = xn;
    } while ((xEnd - xBegin) >= 0.00001 && ++guard < 4096);
    es->maxEig = xn;
}

// splitmix64 (Steele, Lea and Flood, 2014): the eigenvalue start vector
__host__ __device__ inline double eig_start_value(long long c)
{
    unsigned long long z = (unsigned long long)c + 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

__global__ void eig_start_kernel(int n, const int* __restrict__ perm, double* __restrict__ b)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        b[i] = eig_start_value(perm ? perm[i] : i);
}

// ---- Chebyshev steps ------------------------------------------------------
__global__ void recip_kernel(int n, const double* __restrict__ d, double* __restrict__ r)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        r[i] = 1.0 / d[i];
}

// FP32 steps with 8-entry chunks fit 40 registers: six CTAs per SM (48
// warps) keep more row loads in flight than the 16-entry form's four
template <class T, int CK>
__global__ void __launch_bounds__(kBlock, (CK == 8 && sizeof(T) == 4) ? 6 : 1)
    cheb_step_kernel(Rows<T> A, const T* xin, T* xout,
                                                           const T* __restrict__ b, T* w, T c1,
                                                           T c2, int first, Gate g)
{
    // the next step's kernel may launch now; before the wait this kernel
    // reads only the matrix, which no kernel writes (b may have just been
    // written by the previous kernel, a restriction: it is read after the
    // wait, with x and w)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    int len = 0, base = 0;
    T d = T(1), bb = T(0);
    int c[CK];
    T v[CK];
    if (r < A.n) {
        len = lds<true>(A.rowInfo + r) & 0xffff;
        base = ldg(A.sliceOff + (r >> 5)) + (r & 31);
        d = lds<true>(A.diag + r);
#pragma unroll
        for (int k = 0; k < CK; ++k) {
            const int e = base + 32 * k;
            c[k] = k < len ? lds<true>(A.col + e) : r;
            v[k] = k < len ? lds<true>(A.val + e) : T(0);
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (gate_closed(g) || r >= A.n) return;
    bb = __ldcg(b + r);
    // A x in the reference's order: 0, + diag x, then the row's faces
    const T xr = xin[r];
    T xv[CK];
#pragma unroll
    for (int k = 0; k < CK; ++k) xv[k] = xin[c[k]];
    T acc = T(0);
    acc += d * xr;
#pragma unroll
    for (int k = 0; k < CK; ++k)
        if (k < len) acc += v[k] * xv[k];
    for (int j0 = CK; j0 < len; j0 += CK) {
#pragma unroll
        for (int k = 0; k < CK; ++k) {
            const int e = base + 32 * (j0 + k);
            c[k] = j0 + k < len ? lds<true>(A.col + e) : r;
            v[k] = j0 + k < len ? lds<true>(A.val + e) : T(0);
        }
#pragma unroll
        for (int k = 0; k < CK; ++k) xv[k] = xin[c[k]];
#pragma unroll
        for (int k = 0; k < CK; ++k)
            if (j0 + k < len) acc += v[k] * xv[k];
    }
    const T rD = T(1) / d;
    T wi;
    if (first)
        wi = rD * (bb - acc) * c1;
    else
        wi = c1 * w[r] + c2 * rD * (bb - acc);
    w[r] = wi;
    xout[r] = xr + wi;
}

template <class T>
__global__ void cheb_zero_kernel(int n, const T* __restrict__ diag, T* __restrict__ b,
                                 const double* __restrict__ r64, T* __restrict__ x,
                                 T* __restrict__ w, T Rth, Gate g)
{
    if (gate_closed(g)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        T bi;
        if (r64) {
            bi = (T)r64[i];
            b[i] = bi;
        } else {
            bi = b[i];
        }
        const T rD = T(1) / diag[i];
        const T wi = rD * bi * Rth;
        w[i] = wi;
        x[i] = wi;
    }
}

template <class T>
__global__ void restrict_cheb_zero_kernel(int nC, const int* __restrict__ cs,
                                          const int* __restrict__ ch, const T* __restrict__ fine,
                                          T* __restrict__ coarse, const T* __restrict__ diagC,
                                          T* __restrict__ xC, T* __restrict__ wC, T Rth, Gate g)
{
    if (gate_closed(g)) return;
    for (int C = blockIdx.x * blockDim.x + threadIdx.x; C < nC; C += gridDim.x * blockDim.x) {
        T acc = T(0);
        const int k1 = cs[C + 1];
        for (int k = cs[C]; k < k1; ++k) acc += fine[ch[k]];
        coarse[C] = acc;
        const T rD = T(1) / diagC[C];
        const T wi = rD * acc * Rth;
        wC[C] = wi;
        xC[C] = wi;
    }
}

template <class T>
__global__ void prolong_to_kernel(int n, const int* __restrict__ cmap, const T* __restrict__ coarse,
                                  const T* __restrict__ xin, T* __restrict__ xout, Gate g)
{
    if (gate_closed(g)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        xout[i] = xin[i] + coarse[cmap[i]];
}

}  // namespace

int set_cheby_small_rows(int rows) { return g_smallRows.exchange(rows); }

int set_cheby_chunk(int entries)
{
    if (entries != 0 && entries != 8 && entries != 16)
        throw std::invalid_argument("Chebyshev chunk must be 0, 8 or 16 entries");
    return g_chunk.exchange(entries);
}

void eig_diag_pcg(const Exec& ex, const Rows<double>& A, const double* rD, double* x,
                  const double* b, double* rA, double* wA, double* pA, EigState* es,
                  const RSpec& wr, const RSpec& al, int nIt)
{
    const int n = A.n;
    k_residual<double>(ex, A, x, b, rA, RSpec{}, Gate{});  // rA = b - A x
    for (int it = 0; it < nIt; ++it) {
        tick();
        eig_wr_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, rD, rA, wA, es, it, wr);
        tick();
        eig_p_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, wA, pA, es, it);
        tick();
        eig_alpha_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(A, pA, wA, es, it, al);
        tick();
        eig_update_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, x, rA, pA, wA, es);
    }
    UNAP_CK(cudaGetLastError());
}

void k_eig_sturm(const Exec& ex, EigState* es, int nMax)
{
    tick();
    eig_sturm_kernel<<<1, 1, 0, ex.s>>>(es, nMax);
    UNAP_CK(cudaGetLastError());
}

void k_eig_start(const Exec& ex, int n, const int* perm, double* b)
{
    if (n <= 0) return;
    tick();
    eig_start_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, perm, b);
    UNAP_CK(cudaGetLastError());
}

void k_reciprocal(const Exec& ex, int n, const double* d, double* r)
{
    if (n <= 0) return;
    tick();
    recip_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, d, r);
    UNAP_CK(cudaGetLastError());
}

void cheby_coeffs(double lam, double ratio, int deg, double* Rtheta, double* d1, double* d2)
{
    const double maxEig = lam * 1.1;
    const double minEig = lam / ratio;
    const double delta = 2.0 / (maxEig - minEig);
    const double theta = 0.5 * (maxEig + minEig);
    const double s1 = theta * delta;
    double rhok = 1.0 / s1;
    *Rtheta = 1.0 / theta;
    d1[0] = d2[0] = 0.0;
    for (int k = 1; k < deg; ++k) {
        const double rhokp1 = 1.0 / (2.0 * s1 - rhok);
        d1[k] = rhokp1 * rhok;
        d2[k] = 2.0 * rhokp1 * delta;
        rhok = rhokp1;
    }
}

template <class T>
void k_cheb_step(const Exec& ex, const Rows<T>& A, const T* xin, T* xout, const T* b, T* w, T c1,
                 T c2, int first, Gate g)
{
    if (A.n <= 0) return;
    const int threads = A.n <= g_smallRows.load() ? 32 : kBlock;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)div_up(A.n, threads));
    cfg.blockDim = dim3((unsigned)threads);
    cfg.stream = ex.s;
    cfg.attrs = at;
    cfg.numAttrs = wave_pdl() ? 1 : 0;
    tick();
    const int ck = g_chunk.load();
    if (ck == 16 || (ck == 0 && A.wide && (sizeof(T) == 8 || A.n < kChunk8Rows)))
        UNAP_CK(cudaLaunchKernelEx(&cfg, cheb_step_kernel<T, 16>, A, xin, xout, b, w, c1, c2,
                                   first, g));
    else
        UNAP_CK(cudaLaunchKernelEx(&cfg, cheb_step_kernel<T, 8>, A, xin, xout, b, w, c1, c2,
                                   first, g));
}

template <class T>
void k_cheb_zero(const Exec& ex, int n, const T* diag, T* b, const double* r64, T* x, T* w, T Rth,
                 Gate g)
{
    if (n <= 0) return;
    tick();
    cheb_zero_kernel<T><<<div_up(n, kBlock), kBlock, 0, ex.s>>>(n, diag, b, r64, x, w, Rth, g);
    UNAP_CK(cudaGetLastError());
}

template <class T>
void k_restrict_cheb_zero(const Exec& ex, int nC, const int* childStart, const int* child,
                          const T* fine, T* coarse, const T* diagC, T* xC, T* wC, T Rth, Gate g)
{
    if (nC <= 0) return;
    const int threads = nC <= g_smallRows.load() ? 32 : kBlock;
    tick();
    restrict_cheb_zero_kernel<T><<<div_up(nC, threads), threads, 0, ex.s>>>(
        nC, childStart, child, fine, coarse, diagC, xC, wC, Rth, g);
    UNAP_CK(cudaGetLastError());
}

template <class T>
void k_prolong_add_to(const Exec& ex, int n, const int* cmap, const T* coarse, const T* xin,
                      T* xout, Gate g)
{
    if (n <= 0) return;
    const int threads = n <= g_smallRows.load() ? 32 : kBlock;
    tick();
    prolong_to_kernel<T><<<div_up(n, threads), threads, 0, ex.s>>>(n, cmap, coarse, xin, xout, g);
    UNAP_CK(cudaGetLastError());
}

#define UNAP_CHEB_INST(T)                                                                          \
    template void k_cheb_step<T>(const Exec&, const Rows<T>&, const T*, T*, const T*, T*, T, T,   \
                                 int, Gate);                                                       \
    template void k_cheb_zero<T>(const Exec&, int, const T*, T*, const double*, T*, T*, T, Gate); \
    template void k_restrict_cheb_zero<T>(const Exec&, int, const int*, const int*, const T*, T*, \
                                          const T*, T*, T*, T, Gate);                              \
    template void k_prolong_add_to<T>(const Exec&, int, const int*, const T*, const T*, T*, Gate);
UNAP_CHEB_INST(float)
UNAP_CHEB_INST(double)
#undef UNAP_CHEB_INST

}  // namespace unapgpu
