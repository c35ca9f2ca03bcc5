// Whole Krylov solves in one launch: a team of C CTAs (C = 1, or a
// thread-block cluster of 2 .. 16 CTAs) runs a complete PCG or PBiCGStab
// solve (PCG.cpp:35-183, PBiCGStab.cpp:45-459) on a small LDU system held in
// global memory (L2-resident), with a team barrier between vector steps and
// wavefront-by-wavefront DIC/DILU sweeps.  One launch solves a batch: team t
// takes system t.  Used for the MGSolver's coarsest level
// (solveCoarsestLevel.cpp:10-55: PCG+DIC or PBiCGStab+DILU, relTol 1e-2,
// maxIter 100, x0 = 0), for small systems of a batch and for single small
// solves.
//
// Thread g of the team (rank * blockDim + threadIdx) takes rows g, g + C
// blockDim, ...  With C = 1 the barrier is __syncthreads and vectors are
// read with plain loads; with C > 1 it is the cluster barrier
// (barrier.cluster arrive.release / wait.acquire) and vectors written during
// the launch are read from L2 (ld.global.cg), so every CTA of the cluster
// sees the other CTAs' rows after the barrier.
//
// Rows are computed with the same per-row formulas as the multi-block
// kernels, so SpMV and preconditioner applications are bit-identical to
// them.  A dot product is the fixed block tree of each CTA; with C > 1 the
// C block sums are exchanged through distributed shared memory and added in
// rank order, identically in every CTA, so every CTA takes the same
// branches.
#include "device_common.cuh"
#include "small_solve.hpp"

namespace unapgpu {

namespace {

__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// load a double from the shared memory of CTA `rank` of this cluster
__device__ __forceinline__ double ld_dsmem(const double* p, unsigned rank)
{
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    unsigned ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(ra) : "memory");
    return v;
}

template <int C>
struct Team {
    int g;       // first row of this thread
    int stride;  // rows between this thread's rows
    int flip;    // DSMEM buffer of the next dot product
    __device__ Team()
        : g((C == 1 ? 0 : (int)(blockIdx.x % C)) * (int)blockDim.x + (int)threadIdx.x),
          stride(C * (int)blockDim.x), flip(0)
    {
    }
    __device__ __forceinline__ void sync() const
    {
        if constexpr (C == 1)
            __syncthreads();
        else
            cluster_sync_all();
    }
};

// a vector written earlier in this launch (by this thread, this CTA or,
// with C > 1, another CTA of the cluster)
template <int C>
__device__ __forceinline__ double ldv(const double* p)
{
    if constexpr (C == 1)
        return *p;
    else
        return __ldcg(p);
}

template <int C>
__device__ double team_dot(Team<C>& T, int n, const double* a, const double* b)
{
    __shared__ double part[2];
    __shared__ double out;
    double v[1] = {0.0};
    for (int i = T.g; i < n; i += T.stride) v[0] += ldv<C>(a + i) * ldv<C>(b + i);
    block_sum<1>(v);
    if constexpr (C == 1) {
        if (threadIdx.x == 0) out = v[0];
        __syncthreads();
        return out;
    } else {
        // block sums -> this CTA's DSMEM slot; after the cluster barrier
        // warp 0 of every CTA adds the C slots with the same tree.  The two
        // slots alternate: a slot is rewritten two dot products later, after
        // the next dot product's barrier, which every reader of it has
        // passed.
        const int f = T.flip;
        T.flip ^= 1;
        if (threadIdx.x == 0) part[f] = v[0];
        cluster_sync_all();
        if (threadIdx.x < 32) {
            double s = threadIdx.x < C ? ld_dsmem(&part[f], threadIdx.x) : 0.0;
            s = warp_sum(s);
            if (threadIdx.x == 0) out = s;
        }
        __syncthreads();
        return out;
    }
}

template <int C>
__device__ void team_spmv(const Team<C>& T, const Rows<double>& A, const double* x, double* y)
{
    constexpr int XL = C == 1 ? XL_PLAIN : XL_CG;
    for (int i = T.g; i < A.n; i += T.stride) y[i] = row_apply<double, XL>(A, i, x);
    T.sync();
}

// Row data of a DIC/DILU sweep that does not depend on the sweep's previous
// wavefronts: the row's reciprocal, its starting value (r forward, w
// backward) and its first kPre entries (forward: lower entries in order;
// backward: upper entries from the last).  A thread loads them for its row
// of the next wavefront while it computes the current one, so a wavefront
// costs one dependent round trip (the gather of finished neighbours) and a
// barrier.
constexpr int kPre = 4;

struct RowPre {
    int i;       // row, -1: none
    int lo, hi;  // entries [lo, hi) of the row
    int base;
    double rd, a0;
    int c[kPre];
    double v[kPre];
};

template <int C, bool FWD>
__device__ __forceinline__ void sweep_pre(const SmallSystem& S, const double* coef,
                                          const double* src, int i, RowPre& P)
{
    P.i = i;
    if (i < 0) return;
    const Rows<double>& A = S.A;
    const int info = A.rowInfo[i];
    const int len = info & 0xffff, nLow = info >> 16;
    P.base = A.sliceOff[i >> 5] + (i & 31);
    P.rd = S.rD[i];
    P.a0 = ldv<C>(src + i);
    P.lo = FWD ? 0 : nLow;
    P.hi = FWD ? nLow : len;
#pragma unroll
    for (int k = 0; k < kPre; ++k) {
        const int j = FWD ? P.lo + k : P.hi - 1 - k;
        const bool on = k < P.hi - P.lo;
        const int e = P.base + 32 * j;
        P.c[k] = on ? A.col[e] : i;
        P.v[k] = on ? coef[e] : 0.0;
    }
}

// lduDICPrecond.cpp:57-76 / lduDILUPrecond.cpp:60-85 for one row, in the
// reference's order: forward acc = rD r, then acc -= rD coef w[l] over the
// lower entries in face order; backward acc = w, then acc -= rD upper w[u]
// over the upper entries from the last
template <int C, bool FWD>
__device__ __forceinline__ double sweep_row(const SmallSystem& S, const double* coef,
                                            const RowPre& P, const double* w)
{
    double acc = FWD ? P.rd * P.a0 : P.a0;
    const int cnt = P.hi - P.lo;
    double xv[kPre];
#pragma unroll
    for (int k = 0; k < kPre; ++k) xv[k] = k < cnt ? ldv<C>(w + P.c[k]) : 0.0;
#pragma unroll
    for (int k = 0; k < kPre; ++k)
        if (k < cnt) acc -= P.rd * P.v[k] * xv[k];
    for (int k = kPre; k < cnt; ++k) {
        const int j = FWD ? P.lo + k : P.hi - 1 - k;
        const int e = P.base + 32 * j;
        acc -= P.rd * coef[e] * ldv<C>(w + S.A.col[e]);
    }
    return acc;
}

// one sweep over the wavefronts (forward: 0 .. nWave-1, backward: reverse)
template <int C, bool FWD>
__device__ __noinline__ void team_sweep(const Team<C>& T, const SmallSystem& S, const double* coef,
                           const double* src, double* w)
{
    const int nW = S.nWave;
    if (nW <= 0) return;
    // wavefront q of the sweep is wavefront FWD ? q : nW-1-q of the matrix
    auto lo = [&](int q) { return S.waveStart[FWD ? q : nW - 1 - q]; };
    auto hi = [&](int q) { return S.waveStart[FWD ? q + 1 : nW - q]; };
    int r0 = lo(0), r1 = hi(0);
    RowPre cur;
    sweep_pre<C, FWD>(S, coef, src, r0 + T.g < r1 ? r0 + T.g : -1, cur);
    for (int q = 0; q < nW; ++q) {
        int n0 = 0, n1 = 0;
        if (q + 1 < nW) {
            n0 = lo(q + 1);
            n1 = hi(q + 1);
        }
        RowPre nxt;
        sweep_pre<C, FWD>(S, coef, src, n0 + T.g < n1 ? n0 + T.g : -1, nxt);
        if (cur.i >= 0) w[cur.i] = sweep_row<C, FWD>(S, coef, cur, w);
        for (int i = r0 + T.g + T.stride; i < r1; i += T.stride) {
            RowPre more;
            sweep_pre<C, FWD>(S, coef, src, i, more);
            w[i] = sweep_row<C, FWD>(S, coef, more, w);
        }
        T.sync();
        cur = nxt;
        r0 = n0;
        r1 = n1;
    }
}

// w = M^-1 r (unapMatrixPrecond.cpp, lduDiagPrecond.cpp:44-73,
// lduDICPrecond.cpp:45-77, lduDILUPrecond.cpp:46-86)
template <int C>
__device__ void team_precond(const Team<C>& T, const SmallSystem& S, const double* r, double* w)
{
    const Rows<double>& A = S.A;
    const int n = A.n;
    if (S.precond == 0 || S.precond == 1) {
        for (int i = T.g; i < n; i += T.stride)
            w[i] = S.precond ? S.rD[i] * ldv<C>(r + i) : ldv<C>(r + i);
        T.sync();
        return;
    }
    team_sweep<C, true>(T, S, S.precond == 3 ? A.val : A.valT, r, w);
    team_sweep<C, false>(T, S, A.val, w, w);
}

template <int C>
__device__ void team_pcg(Team<C>& T, const SmallSystem& S, SmallResult& R)
{
    const int n = S.A.n;
    double* x = S.x;
    double* p = S.work;
    double* w = S.work + n;
    double* r = S.work + 2 * n;
    team_spmv(T, S.A, x, w);
    for (int i = T.g; i < n; i += T.stride) r[i] = ldv<C>(S.b + i) - ldv<C>(w + i);
    T.sync();
    R.initRes = sqrt(team_dot(T, n, r, r)) + SMALL_D;
    R.finalRes = R.initRes;
    double wArA = 1.0e37, wArAold;
    for (;;) {
        wArAold = wArA;
        team_precond(T, S, r, w);
        wArA = team_dot(T, n, w, r);
        if (!(fabs(wArA) > SMALL_D)) {
            R.singular = 1;
            break;
        }
        const bool first = R.nIter == 0;
        const double beta = first ? 0.0 : wArA / wArAold;
        for (int i = T.g; i < n; i += T.stride)
            p[i] = first ? ldv<C>(w + i) : ldv<C>(w + i) + beta * ldv<C>(p + i);
        T.sync();
        team_spmv(T, S.A, p, w);
        const double wApA = team_dot(T, n, w, p);
        const double alpha = wArA / wApA;
        for (int i = T.g; i < n; i += T.stride) {
            x[i] = ldv<C>(x + i) + alpha * ldv<C>(p + i);
            r[i] = ldv<C>(r + i) - alpha * ldv<C>(w + i);
        }
        T.sync();
        R.finalRes = sqrt(team_dot(T, n, r, r)) + SMALL_D;
        if (!(++R.nIter < S.maxIter)) break;
        R.converged = check_conv(R.finalRes, R.initRes, S.tol, S.relTol, R.nIter, S.minIter);
        if (R.converged) break;
    }
}

template <int C>
__device__ void team_bicgstab(Team<C>& T, const SmallSystem& S, SmallResult& R)
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
    team_spmv(T, S.A, x, y);
    for (int i = T.g; i < n; i += T.stride) {
        const double ri = ldv<C>(S.b + i) - ldv<C>(y + i);
        r[i] = ri;
        r0[i] = ri;
    }
    T.sync();
    R.initRes = sqrt(team_dot(T, n, r, r)) + SMALL_D;
    R.finalRes = R.initRes;
    double rA0rA = 0, alpha = 0, omega = 0;
    for (;;) {
        const double rA0rAold = rA0rA;
        rA0rA = team_dot(T, n, r0, r);
        if (!(fabs(rA0rA) > SMALL_D)) {
            R.singular = 1;
            break;
        }
        if (R.nIter == 0) {
            for (int i = T.g; i < n; i += T.stride) p[i] = ldv<C>(r + i);
        } else {
            const double beta = (rA0rA / rA0rAold) * (alpha / omega);
            for (int i = T.g; i < n; i += T.stride)
                p[i] = ldv<C>(r + i) + beta * (ldv<C>(p + i) - omega * ldv<C>(Ay + i));
        }
        T.sync();
        team_precond(T, S, p, y);
        team_spmv(T, S.A, y, Ay);
        alpha = rA0rA / team_dot(T, n, r0, Ay);
        for (int i = T.g; i < n; i += T.stride) s[i] = ldv<C>(r + i) - alpha * ldv<C>(Ay + i);
        T.sync();
        R.finalRes = sqrt(team_dot(T, n, s, s)) + SMALL_D;
        if (check_conv(R.finalRes, R.initRes, S.tol, S.relTol, R.nIter + 1, S.minIter)) {
            for (int i = T.g; i < n; i += T.stride) x[i] = ldv<C>(x + i) + alpha * ldv<C>(y + i);
            T.sync();
            R.converged = 1;
            R.nIter++;
            return;
        }
        team_precond(T, S, s, z);
        team_spmv(T, S.A, z, t);
        const double tAtA = team_dot(T, n, t, t);
        omega = team_dot(T, n, t, s);
        omega /= tAtA;
        for (int i = T.g; i < n; i += T.stride) {
            x[i] = ldv<C>(x + i) + (alpha * ldv<C>(y + i) + omega * ldv<C>(z + i));
            r[i] = ldv<C>(s + i) - omega * ldv<C>(t + i);
        }
        T.sync();
        R.finalRes = sqrt(team_dot(T, n, r, r)) + SMALL_D;
        if (!(++R.nIter < S.maxIter)) break;
        R.converged = check_conv(R.finalRes, R.initRes, S.tol, S.relTol, R.nIter, S.minIter);
        if (R.converged) break;
    }
}

template <int NT, int C>
__global__ void __launch_bounds__(NT) small_krylov_kernel(const SmallSystem* systems,
                                                          const KState* gate)
{
    // every CTA of a team reads the same gate and takes the same branches
    if (gate && gate->done) return;
    // the system's descriptor in shared memory: its fields are read where
    // they are used instead of held in registers across the solve
    __shared__ SmallSystem sS;
    if (threadIdx.x == 0) sS = systems[blockIdx.x / C];
    __syncthreads();
    const SmallSystem& S = sS;
    Team<C> T;
    SmallResult R{};
    if (S.zeroX) {
        for (int i = T.g; i < S.A.n; i += T.stride) S.x[i] = 0.0;
        T.sync();
    }
    if (S.method == 1)
        team_bicgstab(T, S, R);
    else
        team_pcg(T, S, R);
    if (blockIdx.x % C == 0 && threadIdx.x == 0 && S.result) *S.result = R;
    // no CTA leaves while another may still read its DSMEM slots
    if constexpr (C > 1) cluster_sync_all();
}

template <int NT, int C>
cudaLaunchConfig_t team_config(cudaStream_t s, int count, cudaLaunchAttribute* at)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(count * C));
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cfg;
}

template <int NT, int C>
void launch_team(cudaStream_t s, const SmallSystem* d, int count, const KState* gate)
{
    if constexpr (C == 1) {
        small_krylov_kernel<NT, 1><<<count, NT, 0, s>>>(d, gate);
    } else {
        if constexpr (C > 8)
            UNAP_CK(cudaFuncSetAttribute(small_krylov_kernel<NT, C>,
                                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        cudaLaunchAttribute at[1];
        cudaLaunchConfig_t cfg = team_config<NT, C>(s, count, at);
        UNAP_CK(cudaLaunchKernelEx(&cfg, small_krylov_kernel<NT, C>, d, gate));
    }
}

template <int NT, int C>
int team_capacity()
{
    if constexpr (C == 1) {
        int dev = 0, sms = 0, per = 0;
        UNAP_CK(cudaGetDevice(&dev));
        UNAP_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        UNAP_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, small_krylov_kernel<NT, 1>, NT,
                                                              0));
        return sms * per;
    } else {
        if constexpr (C > 8)
            UNAP_CK(cudaFuncSetAttribute(small_krylov_kernel<NT, C>,
                                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        cudaLaunchAttribute at[1];
        cudaLaunchConfig_t cfg = team_config<NT, C>(nullptr, 1, at);
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, small_krylov_kernel<NT, C>, &cfg) != cudaSuccess) {
            (void)cudaGetLastError();
            return 0;
        }
        return n;
    }
}

template <int C>
void launch_c(cudaStream_t s, const SmallSystem* d, int count, const KState* gate, int threads)
{
    switch (threads) {
    case 128: launch_team<128, C>(s, d, count, gate); break;
    case 256: launch_team<256, C>(s, d, count, gate); break;
    case 1024: launch_team<1024, C>(s, d, count, gate); break;
    default: launch_team<512, C>(s, d, count, gate); break;
    }
}

template <int C>
int capacity_c(int threads)
{
    switch (threads) {
    case 128: return team_capacity<128, C>();
    case 256: return team_capacity<256, C>();
    case 1024: return team_capacity<1024, C>();
    default: return team_capacity<512, C>();
    }
}

}  // namespace

bool small_team_size_ok(int threads, int cluster)
{
    const bool t = threads == 128 || threads == 256 || threads == 512 || threads == 1024;
    const bool c = cluster == 1 || cluster == 2 || cluster == 4 || cluster == 8 || cluster == 16;
    return t && c;
}

void launch_small_krylov(cudaStream_t s, const SmallSystem* d_systems, int count,
                         const KState* gate, int threads, int cluster)
{
    if (count <= 0) return;
    if (!small_team_size_ok(threads, cluster))
        throw std::invalid_argument("small Krylov launch: threads must be 128, 256, 512 or "
                                    "1024 and the cluster 1, 2, 4, 8 or 16 CTAs");
    if (!capturing()) count_launches(1);
    switch (cluster) {
    case 2: launch_c<2>(s, d_systems, count, gate, threads); break;
    case 4: launch_c<4>(s, d_systems, count, gate, threads); break;
    case 8: launch_c<8>(s, d_systems, count, gate, threads); break;
    case 16: launch_c<16>(s, d_systems, count, gate, threads); break;
    default: launch_c<1>(s, d_systems, count, gate, threads); break;
    }
}

int small_team_capacity(int threads, int cluster)
{
    if (!small_team_size_ok(threads, cluster)) return 0;
    switch (cluster) {
    case 2: return capacity_c<2>(threads);
    case 4: return capacity_c<4>(threads);
    case 8: return capacity_c<8>(threads);
    case 16: return capacity_c<16>(threads);
    default: return capacity_c<1>(threads);
    }
}

}  // namespace unapgpu
