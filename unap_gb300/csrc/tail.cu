// Coarse-level V-cycle tail in one cluster launch (see tail.hpp).
//
// Memory rules inside the launch.  x of every tail level is in shared memory
// (own slices stored locally, other CTAs' slices read with
// ld.shared::cluster); the cluster barrier's arrive.release / wait.acquire
// orders those accesses between wavefronts.  Residuals and right-hand sides
// are in global memory: data another CTA wrote in this launch is read with
// ld.global.cg (L2) after a cluster barrier.  Matrix data is read-only for
// the whole launch (ld.global.nc).
//
#include <algorithm>
#include <atomic>
#include <mutex>

#include "device_common.cuh"
#include "tail.hpp"

namespace unapgpu {

namespace {

// per V-cycle precision (0 FP64, 1 FP32), measured on the 256^3 log-normal
// hierarchy: FP32 per-wavefront launches of the row-packed sweep (with
// programmatic dependent launch) beat the cluster tail on every level, so it
// is off; FP64 launches are slower and the tail still wins from ~100k rows
std::atomic<int> g_packedSweeps{1};

std::atomic<long long> g_tailRows[2] = {{1ll << 21}, {8192}};
std::atomic<long long> g_singleRows[2] = {{8192}, {8192}};

constexpr int kStaticSmem =
    kTailMaxWaves * 4 + kTailMaxCluster * 4 + kTailMaxLevels * (int)sizeof(TailLevel) + 64;

__device__ __forceinline__ unsigned cluster_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Barrier of every thread of every CTA of the cluster, ordering shared and
// global memory at cluster scope (hardware barrier, no spinning).
__device__ __forceinline__ void cluster_barrier()
{
    asm volatile(
        "barrier.cluster.arrive.release.aligned;\n\t"
        "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// generic address of the same shared-memory location in CTA `rank` of the
// cluster (distributed shared memory)
__device__ __forceinline__ void* cluster_map(void* p, unsigned rank)
{
    unsigned long long r;
    asm volatile("mapa.u64 %0, %1, %2;" : "=l"(r) : "l"(p), "r"(rank));
    return (void*)r;
}

struct Ctx {
    unsigned rank, C, cm1, lc;  // cluster rank, size, size - 1, log2(size)
    int warp, lane, nw;
    unsigned char* const* rx;   // every rank's x area (distributed shared memory)
};

// byte offset of element i of a cluster-distributed vector at xOffB
template <int ESZ>
__device__ __forceinline__ unsigned dist_off(const Ctx& c, unsigned xOffB, int i)
{
    return xOffB + (unsigned)((((i >> (5 + c.lc)) << 5) | (i & 31)) * ESZ);
}

// Where a read of a tail vector goes: a cluster-distributed vector (32-row
// slice s on rank s mod C), a first-CTA vector read by the first CTA itself,
// or a first-CTA vector read by any CTA.
enum XAt : int { XA_DIST = 0, XA_LOCAL = 1, XA_FIRST = 2 };

// xs is this CTA's x area: the kernel's extern shared array itself, so that
// local reads compile to shared-memory loads
template <class T, int AT>
__device__ __forceinline__ T xget(const Ctx& c, const unsigned char* xs, unsigned xOffB, int i)
{
    if constexpr (AT == XA_DIST) {
        const unsigned owner = ((unsigned)i >> 5) & c.cm1;
        return *(const T*)(c.rx[owner] + dist_off<sizeof(T)>(c, xOffB, i));
    } else if constexpr (AT == XA_LOCAL) {
        return ((const T*)(xs + xOffB))[i];
    } else {
        return ((const T*)(c.rx[0] + xOffB))[i];
    }
}

// this CTA's own element i
template <class T, bool DIST>
__device__ __forceinline__ T& xmine(const Ctx& c, unsigned char* xs, unsigned xOffB, int i)
{
    if constexpr (DIST)
        return *(T*)(xs + dist_off<sizeof(T)>(c, xOffB, i));
    else
        return ((T*)(xs + xOffB))[i];
}

// ---- work units: 32 rows a warp handles together ---------------------------
// cluster-distributed: unit u = slice u (rows 32u .. 32u+31), warps of CTA q
// take the slices s == q (mod C); first-CTA: unit u = rows r0 + 32u ...
template <bool DIST>
__device__ __forceinline__ bool unit_first(const Ctx& c, int r0, int r1, int& u)
{
    if (r1 <= r0) return false;
    if constexpr (DIST) {
        const int s0 = r0 >> 5, s1 = (r1 - 1) >> 5;
        u = s0 + (int)((c.rank - (unsigned)s0) & c.cm1) + c.warp * (int)c.C;
        return u <= s1;
    } else {
        u = c.warp;
        return r0 + 32 * u < r1;
    }
}

template <bool DIST>
__device__ __forceinline__ bool unit_next(const Ctx& c, int r0, int r1, int& u)
{
    if constexpr (DIST) {
        u += c.nw * (int)c.C;
        return u <= ((r1 - 1) >> 5);
    } else {
        u += c.nw;
        return r0 + 32 * u < r1;
    }
}

template <bool DIST>
__device__ __forceinline__ int unit_row(const Ctx& c, int r0, int r1, int u)
{
    const int r = DIST ? (u << 5) + c.lane : r0 + 32 * u + c.lane;
    return (r >= r0 && r < r1) ? r : -1;
}

template <bool DIST>
__device__ __forceinline__ void level_barrier()
{
    if constexpr (DIST)
        cluster_barrier();
    else
        __syncthreads();
}

// ---- a row's data in registers (row-packed records) ------------------------
template <class T>
struct Pk;
template <>
struct Pk<float> {
    static constexpr int EPR = 2;  // entries per 16-byte record
    __device__ static __forceinline__ void entry(const int4& q, int h, int& col, float& v)
    {
        col = h ? q.z : q.x;
        v = __int_as_float(h ? q.w : q.y);
    }
};
template <>
struct Pk<double> {
    static constexpr int EPR = 1;
    __device__ static __forceinline__ void entry(const int4& q, int, int& col, double& v)
    {
        col = q.x;
        v = __hiloint2double(q.w, q.z);
    }
};

// KW entries (KW / EPR records) are held; later entries are read when the
// row is computed
template <class T, int KW>
struct Row {
    static constexpr int R = KW / Pk<T>::EPR;
    int r, info, start;
    T b, d;
    int4 rec[R];
};

__device__ __forceinline__ void fetch_meta(const TailLevel& L, int r, int& start, int& info)
{
    if (r >= 0) {
        const int2 m = ldg(L.pmeta + r);
        start = m.x;
        info = m.y;
    }
}

template <class T, int KW>
__device__ __forceinline__ void fetch_row(const TailLevel& L, Row<T, KW>& q)
{
    if (q.r < 0) return;
    constexpr int EPR = Pk<T>::EPR;
    const int len = q.info & 0xffff;
    q.b = __ldcg((const T*)L.b + q.r);
    q.d = ldg((const T*)L.diag + q.r);
    const int4* rec = L.prec + q.start;
#pragma unroll
    for (int k = 0; k < Row<T, KW>::R; ++k)
        if (k * EPR < len) q.rec[k] = ldg(rec + k);
}

// x_r = (b_r - sum_{j < jEnd} val_j x_col_j) / d_r in entry order
// (gs_kernel's arithmetic)
template <class T, int KW, bool DIST>
__device__ __forceinline__ void gs_row(const TailLevel& L, const Ctx& c, unsigned char* xs,
                                       unsigned xOffB, const Row<T, KW>& q, bool skipUpper)
{
    constexpr int EPR = Pk<T>::EPR;
    constexpr int AT = DIST ? XA_DIST : XA_LOCAL;
    const int jEnd = skipUpper ? (q.info >> 16) : (q.info & 0xffff);
    T acc = q.b;
#pragma unroll
    for (int k = 0; k < Row<T, KW>::R; ++k) {
#pragma unroll
        for (int h = 0; h < EPR; ++h) {
            if (k * EPR + h < jEnd) {
                int col;
                T v;
                Pk<T>::entry(q.rec[k], h, col, v);
                acc -= v * xget<T, AT>(c, xs, xOffB, col);
            }
        }
    }
    for (int j = KW; j < jEnd; ++j) {
        int col;
        T v;
        Pk<T>::entry(ldg(L.prec + q.start + j / EPR), j % EPR, col, v);
        acc -= v * xget<T, AT>(c, xs, xOffB, col);
    }
    xmine<T, DIST>(c, xs, xOffB, q.r) = acc / q.d;
}

// A Gauss-Seidel sweep over the level's wavefronts (forward or backward),
// one barrier after each wavefront.  A warp's first unit of the next
// wavefront is loaded into registers before the barrier (its position and
// length one wavefront earlier still); further units of a wavefront are
// loaded when reached.  Not inlined: each instance gets its own register
// allocation.
template <class T, int KW, bool DIST>
__device__ __noinline__ void tail_sweep(const TailLevel& L, const int* W, Ctx c, bool backward,
                                        bool skipUpper)
{
    extern __shared__ __align__(16) unsigned char dyn[];
    const unsigned xOffB = (unsigned)(L.xOff * (int)sizeof(T));
    const int nW = L.nWave;
    auto wv = [&](int wi) { return backward ? nW - 1 - wi : wi; };
    // row of this lane in the warp's first unit of wave index wi (-1: none)
    auto first_row = [&](int wi) {
        if (wi >= nW) return -1;
        const int w = wv(wi);
        int u;
        return unit_first<DIST>(c, W[w], W[w + 1], u) ? unit_row<DIST>(c, W[w], W[w + 1], u) : -1;
    };
    Row<T, KW> q;
    q.r = first_row(0);
    fetch_meta(L, q.r, q.start, q.info);
    fetch_row<T, KW>(L, q);
    int r1 = first_row(1), start1 = 0, info1 = 0;
    fetch_meta(L, r1, start1, info1);
    for (int wi = 0; wi < nW; ++wi) {
        const int w = wv(wi);
        const int r0 = W[w], rEnd = W[w + 1];
        int u;
        if (unit_first<DIST>(c, r0, rEnd, u)) {
            if (q.r >= 0) gs_row<T, KW, DIST>(L, c, dyn, xOffB, q, skipUpper);
            while (unit_next<DIST>(c, r0, rEnd, u)) {
                q.r = unit_row<DIST>(c, r0, rEnd, u);
                fetch_meta(L, q.r, q.start, q.info);
                fetch_row<T, KW>(L, q);
                if (q.r >= 0) gs_row<T, KW, DIST>(L, c, dyn, xOffB, q, skipUpper);
            }
        }
        // the next wavefront's first unit, then the position of the one after
        q.r = r1;
        q.start = start1;
        q.info = info1;
        fetch_row<T, KW>(L, q);
        r1 = first_row(wi + 2);
        fetch_meta(L, r1, start1, info1);
        level_barrier<DIST>();
    }
}

// rows [0, n) by units, no pipelining
template <bool DIST, class F>
__device__ __forceinline__ void for_units(const Ctx& c, int n, F&& f)
{
    int u;
    if (!unit_first<DIST>(c, 0, n, u)) return;
    do {
        const int r = unit_row<DIST>(c, 0, n, u);
        if (r >= 0) f(r);
    } while (unit_next<DIST>(c, 0, n, u));
}

template <class T, bool DIST>
__device__ __noinline__ void tail_residual(const TailLevel& L, Ctx c)
{
    extern __shared__ __align__(16) unsigned char dyn[];
    constexpr int EPR = Pk<T>::EPR;
    constexpr int AT = DIST ? XA_DIST : XA_LOCAL;
    const unsigned xOffB = (unsigned)(L.xOff * (int)sizeof(T));
    for_units<DIST>(c, L.n, [&](int i) {
        const int2 m = ldg(L.pmeta + i);
        const int len = m.y & 0xffff;
        const T bi = __ldcg((const T*)L.b + i);
        T acc = T(0);
        acc += ldg((const T*)L.diag + i) * xget<T, AT>(c, dyn, xOffB, i);
        for (int j0 = 0; j0 < len; j0 += 8) {
            int4 rc[8 / EPR];
#pragma unroll
            for (int k = 0; k < 8 / EPR; ++k)
                if (j0 + k * EPR < len) rc[k] = ldg(L.prec + m.x + j0 / EPR + k);
#pragma unroll
            for (int k = 0; k < 8 / EPR; ++k) {
#pragma unroll
                for (int h = 0; h < EPR; ++h) {
                    if (j0 + k * EPR + h < len) {
                        int col;
                        T v;
                        Pk<T>::entry(rc[k], h, col, v);
                        acc += v * xget<T, AT>(c, dyn, xOffB, col);
                    }
                }
            }
        }
        ((T*)L.r)[i] = bi - acc;
    });
}

template <class T, int KW, bool DIST>
__device__ void level_down(const TailArgs& a, const TailLevel& L, const int* W, const Ctx& c)
{
    extern __shared__ __align__(16) unsigned char dyn[];
    if (DIST || c.rank == 0) {
        if (a.nPre > 0) {
            for (int sw = 0; sw < a.nPre; ++sw) tail_sweep<T, KW, DIST>(L, W, c, false, sw == 0);
        } else {
            const unsigned xOffB = (unsigned)(L.xOff * (int)sizeof(T));
            for_units<DIST>(c, L.n, [&](int r) { xmine<T, DIST>(c, dyn, xOffB, r) = T(0); });
            level_barrier<DIST>();
        }
        tail_residual<T, DIST>(L, c);
    }
    cluster_barrier();
}

// b' = R r: each coarse cell sums its children's residuals in ascending
// order (restrict_kernel), run by the CTAs that own the coarser level
template <class T, bool NEXT_DIST>
__device__ void restrict_stage(const TailLevel& F, T* bNext, const Ctx& c)
{
    if (NEXT_DIST || c.rank == 0) {
        const T* r = (const T*)F.r;
        for_units<NEXT_DIST>(c, F.nNext, [&](int cc) {
            T acc = T(0);
            const int k0 = ldg(F.childStart + cc), k1 = ldg(F.childStart + cc + 1);
            for (int k = k0; k < k1; ++k) acc += __ldcg(r + ldg(F.child + k));
            bNext[cc] = acc;
        });
    }
    cluster_barrier();
}

// x_c = Minv b_c in FP64, in dense_row_chunked's order (as
// dense_apply_kernel); x_c is cluster-distributed, each warp computes one
// 32-row slice
template <class T>
__device__ __noinline__ void coarsest_stage(const TailArgs& a, double* sb, Ctx c)
{
    extern __shared__ __align__(16) unsigned char dyn[];
    const T* b = (const T*)a.bc;
    for (int j = (int)threadIdx.x; j < a.nc; j += (int)blockDim.x) sb[j] = (double)__ldcg(b + j);
    __syncthreads();
    const unsigned xOffB = (unsigned)(a.xcOff * (int)sizeof(T));
    for_units<true>(c, a.nc, [&](int i) {
        xmine<T, true>(c, dyn, xOffB, i) = (T)dense_row_chunked(a.Minv, a.nc, i, sb);
    });
    cluster_barrier();
}

// x += P e (prolong_add_kernel), then nPost backward sweeps
template <class T, int KW, bool DIST, bool NEXT_DIST>
__device__ void level_up(const TailArgs& a, const TailLevel& L, int nextOff, const int* W,
                         const Ctx& c)
{
    extern __shared__ __align__(16) unsigned char dyn[];
    if (DIST || c.rank == 0) {
        const unsigned xOffB = (unsigned)(L.xOff * (int)sizeof(T));
        const unsigned nOffB = (unsigned)(nextOff * (int)sizeof(T));
        for_units<DIST>(c, L.n, [&](int i) {
            T& xi = xmine<T, DIST>(c, dyn, xOffB, i);
            constexpr int AT = NEXT_DIST ? XA_DIST : (DIST ? XA_FIRST : XA_LOCAL);
            xi = xi + xget<T, AT>(c, dyn, nOffB, ldg(L.cmap + i));
        });
        level_barrier<DIST>();
        for (int sw = 0; sw < a.nPost; ++sw) tail_sweep<T, KW, DIST>(L, W, c, true, false);
    }
    cluster_barrier();
}

template <class T>
__global__ void __launch_bounds__(kTailThreads, 1)
    tail_vcycle_kernel(const __grid_constant__ TailArgs a)
{
    constexpr int KW = sizeof(T) == 4 ? 24 : 8;
    extern __shared__ __align__(16) unsigned char dyn[];
    __shared__ int ws[kTailMaxWaves];
    __shared__ unsigned char* rx[kTailMaxCluster];
    // level descriptors in shared memory: indexing the kernel parameter with
    // a run-time level index would turn every field access into a generic
    // load of parameter memory on the critical path
    __shared__ TailLevel sl[kTailMaxLevels];
    if (gate_closed(a.g)) return;  // the same answer in every CTA
    Ctx c;
    c.rank = cluster_rank();
    c.C = gridDim.x;  // one cluster per launch
    c.cm1 = c.C - 1;
    c.lc = 31 - __clz((int)c.C);
    c.warp = (int)(threadIdx.x >> 5);
    c.lane = (int)(threadIdx.x & 31);
    c.nw = (int)(blockDim.x >> 5);
    c.rx = rx;
    double* sb = (double*)(dyn + (((size_t)a.xElems * sizeof(T) + 15) & ~(size_t)15));
    if (threadIdx.x < c.C) rx[threadIdx.x] = (unsigned char*)cluster_map(dyn, threadIdx.x);
    for (int i = (int)threadIdx.x; i < a.nWaveTotal; i += (int)blockDim.x) ws[i] = ldg(a.waves + i);
    if ((int)threadIdx.x < a.nLv) sl[threadIdx.x] = a.lv[threadIdx.x];
    // every CTA of the cluster is running before any shared memory is read
    // across CTAs
    cluster_barrier();
    for (int k = 0; k < a.nLv; ++k) {
        const TailLevel& L = sl[k];
        if (L.single)
            level_down<T, KW, false>(a, L, ws + L.waveOff, c);
        else
            level_down<T, KW, true>(a, L, ws + L.waveOff, c);
        const bool last = k + 1 == a.nLv;
        T* bNext = (T*)(last ? a.bc : sl[k + 1].b);
        if (last || !sl[k + 1].single)
            restrict_stage<T, true>(L, bNext, c);
        else
            restrict_stage<T, false>(L, bNext, c);
    }
    coarsest_stage<T>(a, sb, c);
    for (int k = a.nLv - 1; k >= 0; --k) {
        const TailLevel& L = sl[k];
        const bool last = k + 1 == a.nLv;
        const int nextOff = last ? a.xcOff : sl[k + 1].xOff;
        const bool nextDist = last || !sl[k + 1].single;
        const int* W = ws + L.waveOff;
        if (L.single) {
            if (nextDist)
                level_up<T, KW, false, true>(a, L, nextOff, W, c);
            else
                level_up<T, KW, false, false>(a, L, nextOff, W, c);
        } else {
            if (nextDist)
                level_up<T, KW, true, true>(a, L, nextOff, W, c);
            else
                level_up<T, KW, true, false>(a, L, nextOff, W, c);
        }
    }
    // x of the first tail level back to global for the finer levels
    {
        const TailLevel& L = sl[0];
        const unsigned xOffB = (unsigned)(L.xOff * (int)sizeof(T));
        T* out = (T*)a.xOut;
        if (L.single) {
            if (c.rank == 0)
                for_units<false>(c, L.n, [&](int i) { out[i] = xmine<T, false>(c, dyn, xOffB, i); });
        } else {
            for_units<true>(c, L.n, [&](int i) { out[i] = xmine<T, true>(c, dyn, xOffB, i); });
        }
    }
    // no CTA leaves while another may still read its shared memory
    cluster_barrier();
}

cudaLaunchConfig_t tail_config(int C, size_t smem, cudaStream_t s, cudaLaunchAttribute* at)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)C);
    cfg.blockDim = dim3(kTailThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cfg;
}

struct TailDevice {
    bool known = false;
    int cluster = 0;
    size_t smem = 0;
};

TailDevice& tail_device()
{
    static std::mutex mu;
    static TailDevice dev[64];
    int d = 0;
    UNAP_CK(cudaGetDevice(&d));
    if (d < 0 || d >= 64) throw std::invalid_argument("device index out of range");
    std::lock_guard<std::mutex> lk(mu);
    TailDevice& t = dev[d];
    if (t.known) return t;
    int optin = 0;
    UNAP_CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, d));
    const size_t smem = optin > kStaticSmem + 1024 ? (size_t)(optin - kStaticSmem - 1024) : 0;
    const void* fns[2] = {(const void*)tail_vcycle_kernel<float>,
                          (const void*)tail_vcycle_kernel<double>};
    for (const void* f : fns) {
        UNAP_CK(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        // clusters above 8 CTAs are not portable; a device that refuses
        // keeps the portable sizes
        if (cudaFuncSetAttribute(f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
            cudaSuccess)
            cudaGetLastError();
    }
    int best = 0;
    for (int C : {16, 8, 4, 2}) {
        bool ok = true;
        for (const void* f : fns) {
            cudaLaunchAttribute at[1];
            cudaLaunchConfig_t cfg = tail_config(C, smem, 0, at);
            int clusters = 0;
            if (cudaOccupancyMaxActiveClusters(&clusters, f, &cfg) != cudaSuccess || clusters < 1) {
                cudaGetLastError();
                ok = false;
            }
        }
        if (ok) {
            best = C;
            break;
        }
    }
    t.cluster = best;
    t.smem = smem;
    t.known = true;
    return t;
}

}  // namespace

int tail_cluster_size() { return tail_device().cluster; }
size_t tail_smem_bytes() { return tail_device().smem; }

long long tail_x_elems(const std::vector<int>& sizes, int C, long long singleRows)
{
    long long e = 0;
    for (size_t k = 0; k < sizes.size(); ++k) {
        const long long n = sizes[k];
        const bool coarsest = k + 1 == sizes.size();
        if (!coarsest && n <= singleRows) {
            e += n;
        } else {
            const long long slices = (n + 31) / 32;
            e += (slices + C - 1) / C * 32;
        }
    }
    return e;
}

void set_tail_rows(int precision, long long tailRows, long long singleRows, long long* oldTail,
                   long long* oldSingle)
{
    if (precision != 0 && precision != 1) throw std::invalid_argument("precision must be 0 or 1");
    const long long t = g_tailRows[precision].exchange(tailRows < 0 ? 0 : tailRows);
    const long long s = g_singleRows[precision].exchange(singleRows < 0 ? 0 : singleRows);
    if (oldTail) *oldTail = t;
    if (oldSingle) *oldSingle = s;
}

int set_packed_sweeps(int mode) { return g_packedSweeps.exchange(mode < 0 || mode > 3 ? 1 : mode); }
int packed_sweeps() { return g_packedSweeps.load(); }

long long tail_rows(int precision) { return g_tailRows[precision ? 1 : 0].load(); }
long long single_rows(int precision) { return g_singleRows[precision ? 1 : 0].load(); }

template <class T>
void launch_tail_vcycle(const TailArgs& a, int C, cudaStream_t s)
{
    const size_t smem = (((size_t)a.xElems * sizeof(T) + 15) & ~(size_t)15) +
                        (size_t)a.nc * sizeof(double);
    if (a.nLv < 1 || a.nLv > kTailMaxLevels || a.nWaveTotal > kTailMaxWaves || a.nc < 1 ||
        a.nc > kTailMaxCoarsest || C < 1 || C > kTailMaxCluster || (C & (C - 1)) ||
        smem > tail_smem_bytes())
        throw std::invalid_argument("tail V-cycle: levels, wavefronts, cluster or memory out of range");
    cudaLaunchAttribute at[1];
    cudaLaunchConfig_t cfg = tail_config(C, smem, s, at);
    if (!capturing()) count_launches(1);
    UNAP_CK(cudaLaunchKernelEx(&cfg, tail_vcycle_kernel<T>, a));
}

template void launch_tail_vcycle<float>(const TailArgs&, int, cudaStream_t);
template void launch_tail_vcycle<double>(const TailArgs&, int, cudaStream_t);

namespace {

template <class T>
__global__ void pack_rows_kernel(Rows<T> A, const int* __restrict__ start, int2* __restrict__ meta,
                                 int4* __restrict__ rec)
{
    constexpr int EPR = Pk<T>::EPR;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += gridDim.x * blockDim.x) {
        const int info = A.rowInfo[r];
        const int len = info & 0xffff;
        const int base = A.sliceOff[r >> 5] + (r & 31);
        const int s = start[r];
        meta[r] = make_int2(s, info);
        for (int j = 0; j < len; j += EPR) {
            int4 q;
            if constexpr (EPR == 2) {
                const bool two = j + 1 < len;
                q.x = A.col[base + 32 * j];
                q.y = __float_as_int((float)A.val[base + 32 * j]);
                q.z = two ? A.col[base + 32 * (j + 1)] : r;
                q.w = two ? __float_as_int((float)A.val[base + 32 * (j + 1)]) : 0;
            } else {
                const double v = (double)A.val[base + 32 * j];
                q.x = A.col[base + 32 * j];
                q.y = 0;
                q.z = __double2loint(v);
                q.w = __double2hiint(v);
            }
            rec[s + j / EPR] = q;
        }
    }
}

}  // namespace

template <class T>
void pack_rows(const Rows<T>& A, PackedRows& out, cudaStream_t s)
{
    constexpr int EPR = Pk<T>::EPR;
    const int n = A.n;
    std::vector<int> info((size_t)n), start((size_t)n);
    if (n) UNAP_CK(cudaMemcpyAsync(info.data(), A.rowInfo, sizeof(int) * (size_t)n,
                                   cudaMemcpyDeviceToHost, s));
    UNAP_CK(cudaStreamSynchronize(s));
    long long total = 0;
    for (int r = 0; r < n; ++r) {
        start[(size_t)r] = (int)total;
        total += ((info[(size_t)r] & 0xffff) + EPR - 1) / EPR;
        if (total > 0x7fffffffLL) throw std::invalid_argument("level too large to pack");
    }
    DevArray<int> dStart;
    dStart.upload(start, s);
    out.meta.alloc((size_t)n);
    out.rec.alloc((size_t)std::max(total, 1LL));
    if (n) {
        const int grid = std::min(div_up(n, 256), 4096);
        pack_rows_kernel<T><<<grid, 256, 0, s>>>(A, dStart.p, out.meta.p, out.rec.p);
        UNAP_CK(cudaGetLastError());
    }
    UNAP_CK(cudaStreamSynchronize(s));
}

namespace {

template <class T, int KW>
__global__ void __launch_bounds__(kBlock) gs_packed_kernel(const int2* __restrict__ meta,
                                                           const int4* __restrict__ rec,
                                                           const T* __restrict__ diag, T* x,
                                                           const T* __restrict__ b, int r0, int r1,
                                                           int skipUpper, Gate g)
{
    constexpr int EPR = Pk<T>::EPR;
    constexpr int R = KW / EPR;
    // the next wavefront's kernel may launch now; before the wait this
    // kernel reads only the matrix, which no kernel writes (b may have just
    // been written by the previous kernel: it is read after the wait)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int r = r0 + blockIdx.x * blockDim.x + threadIdx.x;
    int start = 0, info = 0;
    T d = T(1), bb = T(0);
    int4 q[R];
    if (r < r1) {
        const int2 m = ldg(meta + r);
        start = m.x;
        info = m.y;
        d = ldg(diag + r);
        const int len = info & 0xffff;
#pragma unroll
        for (int k = 0; k < R; ++k)
            if (k * EPR < len) q[k] = ldg(rec + start + k);
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (gate_closed(g) || r >= r1) return;
    bb = __ldcg(b + r);
    const int jEnd = skipUpper ? (info >> 16) : (info & 0xffff);
    T xv[KW];
#pragma unroll
    for (int k = 0; k < R; ++k) {
#pragma unroll
        for (int h = 0; h < EPR; ++h) {
            int col;
            T v;
            Pk<T>::entry(q[k], h, col, v);
            xv[k * EPR + h] = k * EPR + h < jEnd ? x[col] : T(0);
        }
    }
    T acc = bb;
#pragma unroll
    for (int k = 0; k < R; ++k) {
#pragma unroll
        for (int h = 0; h < EPR; ++h) {
            if (k * EPR + h < jEnd) {
                int col;
                T v;
                Pk<T>::entry(q[k], h, col, v);
                acc -= v * xv[k * EPR + h];
            }
        }
    }
    for (int j = KW; j < jEnd; ++j) {
        int col;
        T v;
        Pk<T>::entry(ldg(rec + start + j / EPR), j % EPR, col, v);
        acc -= v * x[col];
    }
    x[r] = acc / d;
}

}  // namespace

constexpr int kSmallWaveRows = 100000;

template <class T>
void gs_sweep_packed(const Exec& ex, const Level& L, const PackedRows& P, const T* diag, T* x,
                     const T* b, bool backward, bool xIsZero, bool wide, Gate g)
{
    const bool narrow = !wide;
    const int W = L.nWave;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    for (int k = 0; k < W; ++k) {
        const int w = backward ? W - 1 - k : k;
        const int r0 = L.waveStart[(size_t)w], r1 = L.waveStart[(size_t)w + 1];
        if (r1 <= r0) continue;
        // a wavefront of up to kSmallWaveRows rows in CTAs of one warp is
        // spread over eight times as many SMs as with 256 threads: each SM
        // then carries fewer rows' loads and gathers, so the latency-bound
        // wavefront ends sooner (256^3 FP32 V-cycle 10.14 ms with 256,
        // 9.38 ms with 64, 9.27 ms with 32 threads per CTA)
        const int threads = (r1 - r0) <= kSmallWaveRows ? 32 : kBlock;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)div_up(r1 - r0, threads));
        cfg.blockDim = dim3(threads);
        cfg.stream = ex.s;
        cfg.attrs = at;
        cfg.numAttrs = wave_pdl() ? 1 : 0;
        if (!capturing()) count_launches(1);
        const int skip = (xIsZero && !backward) ? 1 : 0;
        if (narrow)
            UNAP_CK(cudaLaunchKernelEx(&cfg, gs_packed_kernel<T, sizeof(T) == 4 ? 16 : 8>, P.meta.p,
                                       P.rec.p, diag, x, b, r0, r1, skip, g));
        else
            UNAP_CK(cudaLaunchKernelEx(&cfg, gs_packed_kernel<T, sizeof(T) == 4 ? 24 : 12>,
                                       P.meta.p, P.rec.p, diag, x, b, r0, r1, skip, g));
    }
}

template void gs_sweep_packed<float>(const Exec&, const Level&, const PackedRows&, const float*,
                                     float*, const float*, bool, bool, bool, Gate);
template void gs_sweep_packed<double>(const Exec&, const Level&, const PackedRows&, const double*,
                                      double*, const double*, bool, bool, bool, Gate);

template void pack_rows<float>(const Rows<float>&, PackedRows&, cudaStream_t);
template void pack_rows<double>(const Rows<double>&, PackedRows&, cudaStream_t);

}  // namespace unapgpu
