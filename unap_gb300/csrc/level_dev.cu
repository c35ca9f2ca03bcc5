// Device construction of a Level: the same internal order, SELL-32 layout
// and face-entry maps as the host construction in level.cpp, computed by
// kernels on the matrix's stream.  Bit-for-bit the same Level, so every
// kernel, reduction and solve downstream gives the same bits whichever side
// built it; the host build stays the specification and the fallback for
// shapes the device build declines (listed at build_level_device).
//
// Steps (n cells, F faces; all integer work, HBM-bound):
//   1. check the faces (in range, l < u, l non-decreasing) and count each
//      cell's lower-side faces (upperAddr == c) and upper-side faces;
//   2. ownStart from the sorted lowerAddr (run boundaries), loStart by an
//      exclusive scan of the counts, losort by an atomic bucket fill and an
//      insertion sort of each bucket by face index (stable like the host's
//      counting sort);
//   3. forward wavefront of every cell, level-synchronously (Kahn): a cell
//      joins wavefront d + 1 when its last lower neighbour was in wavefront
//      d, which is the host's 1 + max over lower neighbours;
//   4. the host's BFS visit rank, reproduced exactly: per BFS level every
//      frontier cell claims each unvisited neighbour with the key
//      (frontier position, adjacency index) by atomicMin, and the winners
//      are ranked in key order -- the order a FIFO queue discovers them in
//      (components start at their smallest cell, as the host's seed loop
//      does; runs of isolated cells are ranked in one scan);
//   5. cells in key order, then a stable multisplit by wavefront (one warp
//      per chunk of 4096 cells, ranks within a warp by __match_any_sync);
//   6. row lengths, slice widths, sliceOff (64-bit scan, overflow checked),
//      column indices and face-entry maps, one thread per row, and the
//      FP64 values scattered to their entries.
#include <algorithm>
#include <atomic>
#include <climits>

#include "unap_internal.hpp"

namespace unapgpu {

namespace {

constexpr int kThreads = 256;
constexpr int kScanThreads = 1024;
constexpr int kScanTile = 2 * kScanThreads;
constexpr int kMaxWaves = 4096;        // longer wavefront chains: host build
constexpr int kMaxComponents = 64;     // more connected components: host build
constexpr int kMaxBucket = 1024;       // longer lower-face lists: host build
constexpr int kSplitChunk = 4096;      // cells per warp in the wavefront multisplit

int grid_for(long long n, int threads = kThreads)
{
    long long b = (n + threads - 1) / threads;
    return (int)std::max(1LL, std::min(b, 1LL << 30));
}

template <class T>
using Scratch = StreamScratch<T>;

// ------------------------------------------------------------------ scans

template <class T>
__device__ T warp_inclusive_scan(T v)
{
    const int lane = threadIdx.x & 31;
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    return v;
}

// exclusive scan of one value per thread over the block; *total gets the sum
template <class T>
__device__ T block_exclusive_scan(T v, T* total)
{
    __shared__ T ws[33];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T inc = warp_inclusive_scan(v);
    if (lane == 31) ws[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        T s = lane < nw ? ws[lane] : T(0);
        T si = warp_inclusive_scan(s);
        ws[lane] = si - s;
        if (lane == 31) ws[32] = si;
    }
    __syncthreads();
    T r = ws[wid] + inc - v;
    *total = ws[32];
    __syncthreads();
    return r;
}

template <class TI, class TO>
__global__ void __launch_bounds__(kScanThreads) k_tile_sums(const TI* in, long long n, TO* sums)
{
    const long long base = (long long)blockIdx.x * kScanTile + 2 * threadIdx.x;
    TO a = (base < n ? (TO)in[base] : TO(0)) + (base + 1 < n ? (TO)in[base + 1] : TO(0));
    TO tot;
    block_exclusive_scan(a, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <class TO>
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(TO* sums, int nb)
{
    TO carry = 0;
    for (int b0 = 0; b0 < nb; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        TO v = i < nb ? sums[i] : TO(0);
        TO tot;
        TO ex = block_exclusive_scan(v, &tot);
        if (i < nb) sums[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

// out[i] = sum of in[0..i), out[n] = total; in == out is allowed
template <class TI, class TO>
__global__ void __launch_bounds__(kScanThreads)
    k_tile_apply(const TI* in, long long n, const TO* sums, TO* out)
{
    const long long base = (long long)blockIdx.x * kScanTile + 2 * threadIdx.x;
    TO a0 = base < n ? (TO)in[base] : TO(0);
    TO a1 = base + 1 < n ? (TO)in[base + 1] : TO(0);
    TO tot;
    TO ex = block_exclusive_scan(TO(a0 + a1), &tot) + sums[blockIdx.x];
    if (base < n) out[base] = ex;
    if (base + 1 < n) out[base + 1] = ex + a0;
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = sums[gridDim.x];
}

// exclusive scan of n values into n + 1 (out[n] = total)
template <class TI, class TO>
void exclusive_scan(const TI* in, TO* out, long long n, cudaStream_t s)
{
    if (n <= 0) {
        UNAP_CK(cudaMemsetAsync(out, 0, sizeof(TO), s));
        return;
    }
    const long long nb = (n + kScanTile - 1) / kScanTile;
    Scratch<TO> sums((size_t)nb + 1, s);
    k_tile_sums<TI, TO><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, sums.p);
    k_scan_sums<TO><<<1, kScanThreads, 0, s>>>(sums.p, (int)nb);
    k_tile_apply<TI, TO><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, sums.p, out);
    UNAP_CK(cudaGetLastError());
}

// ------------------------------------------------------- faces and buckets

// bad |= 1: address out of range or not oriented, 2: lowerAddr decreasing
__global__ void k_check_count(const int* __restrict__ l, const int* __restrict__ u, int nf, int n,
                              int* lowCnt, int* bad, int* maxLow)
{
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf;
         f += (long long)gridDim.x * blockDim.x) {
        const int a = l[f], b = u[f];
        if (a < 0 || a >= n || b < 0 || b >= n || a >= b) {
            atomicOr(bad, 1);
            continue;
        }
        if (f && l[f - 1] > a) atomicOr(bad, 2);
        const int c = atomicAdd(&lowCnt[b], 1);
        if (c + 1 > kMaxBucket) atomicMax(maxLow, c + 1);
    }
}

// ownStart[c] = first face with lowerAddr >= c (lowerAddr sorted)
__global__ void k_own_start(const int* __restrict__ l, int nf, int n, int* ownStart)
{
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f <= nf;
         f += (long long)gridDim.x * blockDim.x) {
        const int lo = f == 0 ? -1 : l[f - 1];
        const int hi = f == nf ? n : l[f];
        for (int c = lo + 1; c <= hi; ++c) ownStart[c] = (int)f;
    }
}

__global__ void k_bucket_fill(const int* __restrict__ u, int nf, int* cursor, int* list)
{
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf;
         f += (long long)gridDim.x * blockDim.x)
        list[atomicAdd(&cursor[u[f]], 1)] = (int)f;
}

__global__ void k_bucket_sort(const int* __restrict__ start, int n, int* list)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const int a = start[c], e = start[c + 1];
        for (int i = a + 1; i < e; ++i) {
            const int v = list[i];
            int j = i - 1;
            while (j >= a && list[j] > v) {
                list[j + 1] = list[j];
                --j;
            }
            list[j + 1] = v;
        }
    }
}

// ---------------------------------------------------------------- waves

__global__ void k_wave_init(const int* __restrict__ loStart, int n, int* indeg, int* wave,
                            int* front, int* cnt)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const int d = loStart[c + 1] - loStart[c];
        indeg[c] = d;
        if (d == 0) {
            wave[c] = 0;
            front[atomicAdd(cnt, 1)] = (int)c;
        }
    }
}

__global__ void k_wave_step(const int* __restrict__ front, int m, const int* __restrict__ ownStart,
                            const int* __restrict__ u, int* indeg, int* wave, int d, int* next,
                            int* cnt)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < m;
         p += (long long)gridDim.x * blockDim.x) {
        const int v = front[p];
        for (int f = ownStart[v]; f < ownStart[v + 1]; ++f) {
            const int w = u[f];
            if (atomicSub(&indeg[w], 1) == 1) {
                wave[w] = d + 1;
                next[atomicAdd(cnt, 1)] = w;
            }
        }
    }
}

// ------------------------------------------------------------------ BFS

struct Adj {
    const int* loStart;
    const int* loList;
    const int* ownStart;
    const int* l;
    const int* u;
    __device__ int low(int v) const { return loStart[v + 1] - loStart[v]; }
    __device__ int deg(int v) const { return low(v) + ownStart[v + 1] - ownStart[v]; }
    // neighbour j of v in the host BFS's visiting order: cells behind the
    // lower-side faces (losort order), then behind the upper-side faces
    __device__ int nbr(int v, int j, int lowN) const
    {
        return j < lowN ? l[loList[loStart[v] + j]] : u[ownStart[v] + (j - lowN)];
    }
};

__device__ __forceinline__ unsigned long long claim_key(long long p, int j)
{
    return ((unsigned long long)p << 32) | (unsigned)j;
}

__global__ void k_bfs_claim(Adj A, const int* __restrict__ F, int m, const int* rank,
                            unsigned long long* disc)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < m;
         p += (long long)gridDim.x * blockDim.x) {
        const int v = F[p], lowN = A.low(v), dg = A.deg(v);
        for (int j = 0; j < dg; ++j) {
            const int w = A.nbr(v, j, lowN);
            if (rank[w] < 0) atomicMin(&disc[w], claim_key(p, j));
        }
    }
}

__global__ void k_bfs_count(Adj A, const int* __restrict__ F, int m, const int* rank,
                            const unsigned long long* disc, int* won)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < m;
         p += (long long)gridDim.x * blockDim.x) {
        const int v = F[p], lowN = A.low(v), dg = A.deg(v);
        int c = 0;
        for (int j = 0; j < dg; ++j) {
            const int w = A.nbr(v, j, lowN);
            c += (rank[w] < 0 && disc[w] == claim_key(p, j));
        }
        won[p] = c;
    }
}

// A winner alone writes rank[w]; any other thread reading it concurrently
// sees -1 or a rank, and in both cases its own key differs from disc[w].
__global__ void k_bfs_assign(Adj A, const int* __restrict__ F, int m, const int* __restrict__ off,
                             int rankBase, int* rank, const unsigned long long* disc, int* next)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < m;
         p += (long long)gridDim.x * blockDim.x) {
        const int v = F[p], lowN = A.low(v), dg = A.deg(v);
        int t = off[p];
        for (int j = 0; j < dg; ++j) {
            const int w = A.nbr(v, j, lowN);
            if (rank[w] < 0 && disc[w] == claim_key(p, j)) {
                rank[w] = rankBase + t;
                next[t] = w;
                ++t;
            }
        }
    }
}

// smallest cell >= from that is unvisited (with needNbr != 0: and has at
// least one neighbour), atomically minimised into *best
__global__ void k_first_unvisited(Adj A, int from, int n, const int* rank, int needNbr, int* best)
{
    for (long long c = from + blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        if (rank[c] >= 0) continue;
        if (needNbr && A.deg((int)c) == 0) continue;
        atomicMin(best, (int)c);
        return;  // later cells of this thread are larger
    }
}

__global__ void k_unvisited_flags(int from, int to, const int* rank, int* flag)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < to - from;
         i += (long long)gridDim.x * blockDim.x)
        flag[i] = rank[from + i] < 0;
}

__global__ void k_rank_run(int from, int to, const int* flag, const int* ex, int base, int* rank)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < to - from;
         i += (long long)gridDim.x * blockDim.x)
        if (flag[i]) rank[from + i] = base + ex[i];
}

__global__ void k_set(int* p, int v) { *p = v; }

// -------------------------------------------------------- order and split

__global__ void k_scatter_by_rank(const int* __restrict__ rank, int n, int* byKey)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x)
        if (rank[c] >= 0 && rank[c] < n) byKey[rank[c]] = (int)c;
}

__global__ void k_key_slots(const int* __restrict__ key, int n, int* slot, int* dup)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x)
        if (atomicCAS(&slot[key[c]], -1, (int)c) != -1) atomicOr(dup, 1);
}

__global__ void k_slot_flags(const int* __restrict__ slot, long long K, int* flag)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < K;
         i += (long long)gridDim.x * blockDim.x)
        flag[i] = slot[i] >= 0;
}

__global__ void k_slot_compact(const int* __restrict__ slot, long long K, const int* __restrict__ ex,
                               int* byKey)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < K;
         i += (long long)gridDim.x * blockDim.x)
        if (slot[i] >= 0) byKey[ex[i]] = slot[i];
}

// Stable multisplit of byKey by wavefront.  cnt holds one row of nWave
// counters per chunk, touched only by that chunk's warp; __syncwarp orders a
// leader's update before the next batch reads it.
template <bool kPlace>
__global__ void k_split(const int* __restrict__ byKey, const int* __restrict__ wave, int n,
                        int nWave, int* cnt, const int* __restrict__ waveStart, int* perm)
{
    const int lane = threadIdx.x & 31;
    const long long chunk = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long r0 = chunk * kSplitChunk;
    if (r0 >= n) return;
    int* row = cnt + chunk * nWave;
    const long long r1 = min((long long)n, r0 + (long long)kSplitChunk);
    for (long long b = r0; b < r1; b += 32) {
        const long long r = b + lane;
        const bool ok = r < r1;
        const int c = ok ? byKey[r] : -1;
        const int w = ok ? wave[c] : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, w);
        const bool leader = lane == __ffs(peers) - 1;
        const int before = row[ok ? w : 0];
        if (kPlace && ok)
            perm[waveStart[w] + before + __popc(peers & ((1u << lane) - 1u))] = c;
        __syncwarp();
        if (ok && leader) row[w] = before + __popc(peers);
        __syncwarp();
    }
}

// per wavefront: chunk counts -> chunk offsets within the wavefront
__global__ void k_split_scan(int* cnt, long long nChunks, int nWave, int* total)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nWave) return;
    int run = 0;
    for (long long k = 0; k < nChunks; ++k) {
        const int t = cnt[k * nWave + w];
        cnt[k * nWave + w] = run;
        run += t;
    }
    total[w] = run;
}

// Rows of a level without wavefronts, reordered inside every window of
// kLenWindow internal rows by decreasing row length (stable), so that
// SELL-32 slices hold rows of similar length: one CTA per window.
constexpr int kLenWindow = 256;

__global__ void __launch_bounds__(kLenWindow) k_window_by_length(Adj adj, int n, int* perm)
{
    __shared__ int cell[kLenWindow], len[kLenWindow];
    const int w0 = blockIdx.x * kLenWindow;
    const int m = min(kLenWindow, n - w0);
    const int t = threadIdx.x;
    if (t < m) {
        cell[t] = perm[w0 + t];
        len[t] = adj.deg(cell[t]);
    }
    __syncthreads();
    int rank = 0;
    if (t < m)
        for (int j = 0; j < m; ++j) rank += (len[j] > len[t]) || (len[j] == len[t] && j < t);
    if (t < m) perm[w0 + rank] = cell[t];
}

__global__ void k_iperm(const int* __restrict__ perm, int n, int* iperm)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        iperm[perm[i]] = (int)i;
}

// ----------------------------------------------------------------- SELL

__global__ void k_rows(const int* __restrict__ perm, int n, const int* __restrict__ loStart,
                       const int* __restrict__ ownStart, int* rowInfo, int* rowLen, int* tooLong)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = perm[i];
        const int lo = loStart[c + 1] - loStart[c];
        const int len = lo + ownStart[c + 1] - ownStart[c];
        if (len > 0xffff) atomicOr(tooLong, 1);
        rowLen[i] = len;
        rowInfo[i] = len | (lo << 16);
    }
}

__global__ void k_slice_width(const int* __restrict__ rowLen, int n, int nSlices,
                              long long* sliceEnt, int* maxLen)
{
    for (long long sl = blockIdx.x * (long long)blockDim.x + threadIdx.x; sl < nSlices;
         sl += (long long)gridDim.x * blockDim.x) {
        int w = 0;
        const long long r1 = min((long long)n, sl * 32 + 32);
        for (long long r = sl * 32; r < r1; ++r) w = max(w, rowLen[r]);
        sliceEnt[sl] = 32LL * w;
        atomicMax(maxLen, w);
    }
}

__global__ void k_slice_off32(const long long* __restrict__ off64, int nSlices, int* off32)
{
    for (long long sl = blockIdx.x * (long long)blockDim.x + threadIdx.x; sl <= nSlices;
         sl += (long long)gridDim.x * blockDim.x)
        off32[sl] = (int)off64[sl];
}

// one thread per row (including the padding rows of the last slice)
__global__ void k_fill(const int* __restrict__ perm, const int* __restrict__ iperm, int n,
                       int nSlices, const int* __restrict__ sliceOff,
                       const int* __restrict__ loStart, const int* __restrict__ loList,
                       const int* __restrict__ ownStart, const int* __restrict__ l,
                       const int* __restrict__ u, int* col, int* entLo, int* entUp)
{
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < 32LL * nSlices;
         r += (long long)gridDim.x * blockDim.x) {
        const long long sl = r >> 5;
        const long long base = sliceOff[sl] + (r & 31);
        const int width = (sliceOff[sl + 1] - sliceOff[sl]) >> 5;
        int j = 0;
        if (r < n) {
            const int c = perm[r];
            int a = loStart[c], ae = loStart[c + 1];
            int b = ownStart[c], be = ownStart[c + 1];
            while (a < ae || b < be) {
                const bool takeLow = b >= be || (a < ae && loList[a] < b);
                const long long e = base + 32LL * j;
                if (takeLow) {
                    const int f = loList[a++];
                    col[e] = iperm[l[f]];
                    entLo[f] = (int)e;
                } else {
                    const int f = b++;
                    col[e] = iperm[u[f]];
                    entUp[f] = (int)e;
                }
                ++j;
            }
        }
        // padding entries point at the row itself (0 past the last row)
        for (; j < width; ++j) col[base + 32LL * j] = r < n ? (int)r : 0;
    }
}

__global__ void k_values(const int* __restrict__ entLo, const int* __restrict__ entUp, int nf,
                         const double* __restrict__ lower, const double* __restrict__ upper,
                         double* val, double* valT)
{
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf;
         f += (long long)gridDim.x * blockDim.x) {
        val[entLo[f]] = lower[f];
        val[entUp[f]] = upper[f];
        if (valT) {
            valT[entLo[f]] = upper[f];
            valT[entUp[f]] = lower[f];
        }
    }
}

__global__ void k_diag(const int* __restrict__ perm, int n, const double* __restrict__ diagRef,
                       double* diag)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        diag[i] = diagRef[perm[i]];
}

template <class T>
void to_host(std::vector<T>& h, const T* d, size_t n, cudaStream_t s)
{
    h.resize(n);
    if (n) UNAP_CK(cudaMemcpyAsync(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost, s));
}

// a few device ints read back (pageable: no pinned allocation, which would
// synchronize the device)
struct Readback {
    int h[16] = {};
    cudaStream_t s;
    explicit Readback(cudaStream_t st) : s(st) {}
    int get(const int* d, int slot = 0)
    {
        UNAP_CK(cudaMemcpyAsync(h + slot, d, sizeof(int), cudaMemcpyDeviceToHost, s));
        UNAP_CK(cudaStreamSynchronize(s));
        return h[slot];
    }
};

std::atomic<long long> g_deviceMinCells{32768};

}  // namespace

void device_exclusive_scan(const int* in, int* out, long long n, cudaStream_t s)
{
    exclusive_scan(in, out, n, s);
}

long long set_device_setup_min_cells(long long minCells)
{
    return g_deviceMinCells.exchange(minCells);
}

long long device_setup_min_cells() { return g_deviceMinCells.load(); }

// Returns nullptr (nothing built) when the matrix is not oriented and
// owner-sorted, has a cell with more than kMaxBucket lower-side faces, more
// than kMaxWaves wavefronts or kMaxComponents connected components, or a
// locality key that repeats; build_level then builds it on the host.
std::unique_ptr<Level> build_level_device(const HostLdu& A, const std::vector<int>* key,
                                          cudaStream_t s, bool wavefronts)
{
    const int n = A.n, nf = A.nf;
    if (n <= 0) return nullptr;
    int minKey = 0, maxKey = -1;
    const bool haveKey = key && (int)key->size() == n;
    if (haveKey) {
        minKey = INT_MAX;
        for (int k : *key) minKey = std::min(minKey, k), maxKey = std::max(maxKey, k);
        if (minKey < 0) return nullptr;  // the host build reports it
    }
    Readback rb(s);
    const int g = grid_for(std::max(n, nf) + 1);

    Scratch<int> dl((size_t)nf, s), du((size_t)nf, s);
    if (nf) {
        UNAP_CK(cudaMemcpyAsync(dl.p, A.l.data(), sizeof(int) * (size_t)nf, cudaMemcpyHostToDevice, s));
        UNAP_CK(cudaMemcpyAsync(du.p, A.u.data(), sizeof(int) * (size_t)nf, cudaMemcpyHostToDevice, s));
    }
    // 1-2: checks, counts, ownStart, loStart, losort
    Scratch<int> flags(4, s);
    Scratch<int> loStart((size_t)n + 1, s), ownStart((size_t)n + 1, s), loList((size_t)nf, s);
    UNAP_CK(cudaMemsetAsync(flags.p, 0, 4 * sizeof(int), s));
    UNAP_CK(cudaMemsetAsync(loStart.p, 0, sizeof(int) * ((size_t)n + 1), s));
    if (nf) k_check_count<<<g, kThreads, 0, s>>>(dl.p, du.p, nf, n, loStart.p, flags.p, flags.p + 1);
    UNAP_CK(cudaGetLastError());
    UNAP_CK(cudaMemcpyAsync(rb.h, flags.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    UNAP_CK(cudaStreamSynchronize(s));
    if (rb.h[0] != 0 || rb.h[1] != 0) return nullptr;
    exclusive_scan(loStart.p, loStart.p, n, s);
    k_own_start<<<g, kThreads, 0, s>>>(dl.p, nf, n, ownStart.p);
    {
        Scratch<int> cursor((size_t)n, s);
        UNAP_CK(cudaMemcpyAsync(cursor.p, loStart.p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s));
        if (nf) k_bucket_fill<<<g, kThreads, 0, s>>>(du.p, nf, cursor.p, loList.p);
    }
    k_bucket_sort<<<grid_for(n), kThreads, 0, s>>>(loStart.p, n, loList.p);
    UNAP_CK(cudaGetLastError());
    Adj adj{loStart.p, loList.p, ownStart.p, dl.p, du.p};

    // 3: forward wavefronts
    Scratch<int> wave((size_t)n, s), indeg((size_t)n, s), fa((size_t)n, s), fb((size_t)n, s);
    int nWave = 0;
    if (!wavefronts) {
        // one range: every row in locality order
        UNAP_CK(cudaMemsetAsync(wave.p, 0, sizeof(int) * (size_t)n, s));
        nWave = 1;
    } else {
        UNAP_CK(cudaMemsetAsync(flags.p, 0, sizeof(int), s));
        k_wave_init<<<grid_for(n), kThreads, 0, s>>>(loStart.p, n, indeg.p, wave.p, fa.p, flags.p);
        int m = rb.get(flags.p);
        int* F = fa.p;
        int* G = fb.p;
        while (m > 0) {
            if (++nWave > kMaxWaves) return nullptr;
            UNAP_CK(cudaMemsetAsync(flags.p, 0, sizeof(int), s));
            k_wave_step<<<grid_for(m), kThreads, 0, s>>>(F, m, ownStart.p, du.p, indeg.p, wave.p,
                                                         nWave - 1, G, flags.p);
            m = rb.get(flags.p);
            std::swap(F, G);
        }
    }

    // 4-5: locality order, then stable by wavefront
    Scratch<int> byKey((size_t)n, s);
    if (haveKey) {
        const long long K = (long long)maxKey + 1;
        Scratch<int> slot((size_t)K, s), kd((size_t)n, s), fl((size_t)K + 1, s);
        UNAP_CK(cudaMemcpyAsync(kd.p, key->data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, s));
        UNAP_CK(cudaMemsetAsync(slot.p, 0xff, sizeof(int) * (size_t)K, s));
        UNAP_CK(cudaMemsetAsync(flags.p, 0, sizeof(int), s));
        k_key_slots<<<grid_for(n), kThreads, 0, s>>>(kd.p, n, slot.p, flags.p);
        if (rb.get(flags.p) != 0) return nullptr;  // repeated keys: the host's stable sort
        k_slot_flags<<<grid_for(K), kThreads, 0, s>>>(slot.p, K, fl.p);
        exclusive_scan(fl.p, fl.p, K, s);
        k_slot_compact<<<grid_for(K), kThreads, 0, s>>>(slot.p, K, fl.p, byKey.p);
    } else {
        // BFS visit rank (reuses indeg as rank, fa/fb as frontiers)
        int* rank = indeg.p;
        Scratch<unsigned long long> disc((size_t)n, s);
        Scratch<int> won((size_t)n + 1, s);
        UNAP_CK(cudaMemsetAsync(rank, 0xff, sizeof(int) * (size_t)n, s));
        UNAP_CK(cudaMemsetAsync(disc.p, 0xff, sizeof(unsigned long long) * (size_t)n, s));
        int nextRank = 0, from = 0, comps = 0;
        while (nextRank < n) {
            k_set<<<1, 1, 0, s>>>(flags.p, n);
            k_first_unvisited<<<grid_for(n - from), kThreads, 0, s>>>(adj, from, n, rank, 0, flags.p);
            const int seed = rb.get(flags.p);
            if (seed >= n) return nullptr;  // cannot happen while nextRank < n
            k_set<<<1, 1, 0, s>>>(flags.p, n);
            k_first_unvisited<<<grid_for(n - seed), kThreads, 0, s>>>(adj, seed, n, rank, 1, flags.p);
            const int m1 = rb.get(flags.p);
            if (m1 > seed) {
                // cells [seed, m1) that are unvisited have no neighbour: one
                // component each, ranked in index order
                const int len = m1 - seed;
                k_unvisited_flags<<<grid_for(len), kThreads, 0, s>>>(seed, m1, rank, won.p);
                Scratch<int> ex((size_t)len + 1, s);
                exclusive_scan(won.p, ex.p, len, s);
                k_rank_run<<<grid_for(len), kThreads, 0, s>>>(seed, m1, won.p, ex.p, nextRank, rank);
                const int t = rb.get(ex.p + len);
                if (t > n - nextRank) return nullptr;
                nextRank += t;
                from = m1;
                continue;
            }
            if (++comps > kMaxComponents) return nullptr;
            k_set<<<1, 1, 0, s>>>(rank + seed, nextRank);
            k_set<<<1, 1, 0, s>>>(fa.p, seed);
            ++nextRank;
            int* F = fa.p;
            int* G = fb.p;
            int m = 1;
            for (;;) {
                k_bfs_claim<<<grid_for(m), kThreads, 0, s>>>(adj, F, m, rank, disc.p);
                k_bfs_count<<<grid_for(m), kThreads, 0, s>>>(adj, F, m, rank, disc.p, won.p);
                exclusive_scan(won.p, won.p, m, s);
                const int t = rb.get(won.p + m);
                if (t == 0) break;
                if (t > n - nextRank) return nullptr;  // cannot happen: each cell is won once
                k_bfs_assign<<<grid_for(m), kThreads, 0, s>>>(adj, F, m, won.p, nextRank, rank,
                                                              disc.p, G);
                nextRank += t;
                m = t;
                std::swap(F, G);
            }
            UNAP_CK(cudaGetLastError());
            from = seed + 1;
        }
        k_scatter_by_rank<<<grid_for(n), kThreads, 0, s>>>(rank, n, byKey.p);
    }
    UNAP_CK(cudaGetLastError());

    auto L = std::make_unique<Level>();
    L->n = n;
    L->nf = nf;
    L->symm = A.symm;
    L->sweepable = wavefronts;
    L->nWave = nWave;
    L->d_perm.alloc((size_t)n);
    L->d_iperm.alloc((size_t)n);
    Scratch<int> ws((size_t)nWave + 1, s);
    {
        const long long nChunks = (n + kSplitChunk - 1) / kSplitChunk;
        Scratch<int> cnt((size_t)(nChunks * nWave), s), tot((size_t)nWave, s);
        UNAP_CK(cudaMemsetAsync(cnt.p, 0, sizeof(int) * (size_t)(nChunks * nWave), s));
        const int warpsGrid = (int)((nChunks * 32 + kThreads - 1) / kThreads);
        k_split<false><<<warpsGrid, kThreads, 0, s>>>(byKey.p, wave.p, n, nWave, cnt.p, nullptr, nullptr);
        k_split_scan<<<grid_for(nWave), kThreads, 0, s>>>(cnt.p, nChunks, nWave, tot.p);
        exclusive_scan(tot.p, ws.p, nWave, s);
        k_split<true><<<warpsGrid, kThreads, 0, s>>>(byKey.p, wave.p, n, nWave, cnt.p, ws.p, L->d_perm.p);
    }
    if (!wavefronts)
        k_window_by_length<<<(n + kLenWindow - 1) / kLenWindow, kLenWindow, 0, s>>>(adj, n,
                                                                                L->d_perm.p);
    k_iperm<<<grid_for(n), kThreads, 0, s>>>(L->d_perm.p, n, L->d_iperm.p);
    Scratch<int> locRank((size_t)n, s);
    k_iperm<<<grid_for(n), kThreads, 0, s>>>(byKey.p, n, locRank.p);
    UNAP_CK(cudaGetLastError());

    // 6: SELL-32
    L->nSlices = (n + 31) / 32;
    const int nSlices = L->nSlices;
    Scratch<int> rowLen((size_t)n, s);
    L->d_rowInfo.alloc((size_t)n);
    UNAP_CK(cudaMemsetAsync(flags.p, 0, 4 * sizeof(int), s));
    k_rows<<<grid_for(n), kThreads, 0, s>>>(L->d_perm.p, n, loStart.p, ownStart.p, L->d_rowInfo.p,
                                           rowLen.p, flags.p);
    Scratch<long long> sliceEnt((size_t)nSlices + 1, s);
    k_slice_width<<<grid_for(nSlices), kThreads, 0, s>>>(rowLen.p, n, nSlices, sliceEnt.p, flags.p + 1);
    exclusive_scan(sliceEnt.p, sliceEnt.p, nSlices, s);
    long long total = 0;
    UNAP_CK(cudaMemcpyAsync(rb.h, flags.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    UNAP_CK(cudaMemcpyAsync(&total, sliceEnt.p + nSlices, sizeof(long long), cudaMemcpyDeviceToHost, s));
    UNAP_CK(cudaStreamSynchronize(s));
    if (rb.h[0]) throw std::invalid_argument("row with more than 65535 faces");
    if (total > 0x7fffffffLL) throw std::invalid_argument("matrix too large for int32 SELL offsets");
    L->maxRowLen = rb.h[1];
    L->nEntries = total;
    L->d_sliceOff.alloc((size_t)nSlices + 1);
    k_slice_off32<<<grid_for(nSlices + 1), kThreads, 0, s>>>(sliceEnt.p, nSlices, L->d_sliceOff.p);
    L->d_col.alloc((size_t)total);
    Scratch<int> entLo((size_t)nf, s), entUp((size_t)nf, s);
    k_fill<<<grid_for(32LL * nSlices), kThreads, 0, s>>>(
        L->d_perm.p, L->d_iperm.p, n, nSlices, L->d_sliceOff.p, loStart.p, loList.p, ownStart.p,
        dl.p, du.p, L->d_col.p, entLo.p, entUp.p);
    UNAP_CK(cudaGetLastError());

    // FP64 values
    {
        Scratch<double> up((size_t)nf, s), lo(A.symm ? 0 : (size_t)nf, s), dg((size_t)n, s);
        if (nf)
            UNAP_CK(cudaMemcpyAsync(up.p, A.upper.data(), sizeof(double) * (size_t)nf,
                                    cudaMemcpyHostToDevice, s));
        if (!A.symm && nf)
            UNAP_CK(cudaMemcpyAsync(lo.p, A.lower.data(), sizeof(double) * (size_t)nf,
                                    cudaMemcpyHostToDevice, s));
        UNAP_CK(cudaMemcpyAsync(dg.p, A.diag.data(), sizeof(double) * (size_t)n,
                                cudaMemcpyHostToDevice, s));
        L->d_val.alloc((size_t)total);
        L->d_val.zero(s);
        if (!A.symm) {
            L->d_valT.alloc((size_t)total);
            L->d_valT.zero(s);
        }
        if (nf)
            k_values<<<grid_for(nf), kThreads, 0, s>>>(entLo.p, entUp.p, nf, A.symm ? up.p : lo.p,
                                                       up.p, L->d_val.p, A.symm ? nullptr : L->d_valT.p);
        L->d_diag.alloc((size_t)n);
        k_diag<<<grid_for(n), kThreads, 0, s>>>(L->d_perm.p, n, dg.p, L->d_diag.p);
        UNAP_CK(cudaGetLastError());
    }

    // host copies the rest of the library reads
    to_host(L->perm, L->d_perm.p, (size_t)n, s);
    to_host(L->iperm, L->d_iperm.p, (size_t)n, s);
    to_host(L->locRank, locRank.p, (size_t)n, s);
    to_host(L->waveStart, ws.p, (size_t)nWave + 1, s);
    to_host(L->entLo, entLo.p, (size_t)nf, s);
    to_host(L->entUp, entUp.p, (size_t)nf, s);
    UNAP_CK(cudaStreamSynchronize(s));
    return L;
}

}  // namespace unapgpu
