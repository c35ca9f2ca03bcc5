// Internal declarations of the GB300 UNAP library (not part of the C ABI).
//
// Device data model, one `Level` per LDU matrix of a hierarchy:
//
//  * Cells are renumbered into an internal order that is level-major with
//    respect to the forward dependency DAG of the matrix in its own
//    numbering (cell c depends on every lower neighbour l < c, i.e. on every
//    face f with upperAddr[f] == c).  Each wavefront is a contiguous internal
//    range, so the forward sweeps of DIC/DILU/Gauss-Seidel walk the
//    wavefronts in order and the backward sweeps walk them in reverse, with
//    exactly the reference's cell-order dependencies.  Within a wavefront
//    cells follow a locality key (BFS order on the finest level, inherited
//    through the aggregates on coarse levels) so neighbour gathers hit L2.
//  * Off-diagonal entries are stored as sliced ELLPACK with slices of 32 rows
//    (SELL-32): entry j of row r lives at sliceOff[r/32] + 32*j + r%32, so a
//    warp loads 32 consecutive column indices and values.  A row's entries
//    are its faces in ascending face order; for owner-sorted matrices that is
//    [faces with upperAddr == c][faces with lowerAddr == c], the split point
//    being nLow.  Per-row summation order therefore equals the reference's
//    face loops (lduMatrixSpMV.cpp:83-92, lduGaussSeidelSmoother.cpp:53-78,
//    lduDICPrecond.cpp:63-76), which makes those kernels bit-identical to it.
//  * val[e] is the matrix entry A[row][col] (lower[f] on the lower side,
//    upper[f] on the upper side); valT[e] is the transposed coefficient
//    (upper[f] on the lower side), needed by DIC/DILU on asymmetric storage.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <memory>
#include <mutex>
#include <shared_mutex>
#include <stdexcept>
#include <string>
#include <vector>

namespace unapgpu {

struct CudaError : std::runtime_error {
    explicit CudaError(const std::string& m) : std::runtime_error(m) {}
};

#define UNAP_CK(call)                                                                     \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            throw ::unapgpu::CudaError(std::string(#call) + ": " + cudaGetErrorString(e_) + \
                                       " at " + __FILE__ + ":" + std::to_string(__LINE__)); \
    } while (0)

void set_last_error(const std::string& msg);
const char* last_error();

// Stream captures (thread-local mode) run in several host threads at once,
// e.g. one per served request.  Device and pinned allocations and frees
// synchronize the device, which would break a capture in progress, so they
// take this gate exclusively while captures hold it shared.  Nothing may
// allocate inside a capture section.
std::shared_mutex& capture_gate();
bool& thread_in_capture();
struct AllocGate {
    std::unique_lock<std::shared_mutex> lk;
    AllocGate() : lk(capture_gate(), std::defer_lock)
    {
        if (thread_in_capture()) throw std::logic_error("device allocation inside a stream capture");
        lk.lock();
    }
};
struct CaptureGate {
    std::shared_lock<std::shared_mutex> lk;
    CaptureGate() : lk(capture_gate()) { thread_in_capture() = true; }
    ~CaptureGate() { thread_in_capture() = false; }
};
inline cudaError_t gated_malloc(void** p, size_t bytes)
{
    AllocGate g;
    return cudaMalloc(p, bytes);
}
inline cudaError_t gated_free(void* p)
{
    AllocGate g;
    return cudaFree(p);
}
inline cudaError_t gated_malloc_host(void** p, size_t bytes)
{
    AllocGate g;
    return cudaMallocHost(p, bytes);
}
inline cudaError_t gated_free_host(void* p)
{
    AllocGate g;
    return cudaFreeHost(p);
}

// Stream-ordered allocation scope.  While a thread holds one, the DevArrays
// it allocates come from the device's memory pool in the order of the
// scope's stream (cudaMallocAsync) and return to the pool in that order when
// released (cudaFreeAsync): no device-wide synchronization and no allocation
// gate, so concurrent solves on other streams keep running.  Everything
// that touches those arrays must run on the scope's stream (the server's
// slot workers: one stream each).  The pool keeps freed memory for reuse
// instead of returning it to the driver at each synchronization.
cudaStream_t& thread_alloc_stream();
void keep_pool_memory();
struct StreamAllocScope {
    cudaStream_t prev;
    explicit StreamAllocScope(cudaStream_t s) : prev(thread_alloc_stream())
    {
        keep_pool_memory();
        thread_alloc_stream() = s;
    }
    ~StreamAllocScope() { thread_alloc_stream() = prev; }
    StreamAllocScope(const StreamAllocScope&) = delete;
    StreamAllocScope& operator=(const StreamAllocScope&) = delete;
};

// Calls on caller-owned device vectors run on the matrix's own
// (non-blocking) stream; this orders that stream after all work the caller
// issued before the call to the legacy default stream or any blocking
// stream (e.g. the fill of an initial guess), so the call reads its inputs
// as the caller left them.
void order_after_default_stream(cudaStream_t s);

// Small pinned host blocks (solver state read back every iteration) from a
// process-wide free list: cudaFreeHost would synchronize the device.
void* pinned_block_alloc(size_t bytes);
void pinned_block_free(void* p);

template <class T>
struct DevArray {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t as = nullptr;  // allocation stream of a stream-ordered array
    bool async = false;
    DevArray() = default;
    explicit DevArray(size_t count) { alloc(count); }
    DevArray(const DevArray&) = delete;
    DevArray& operator=(const DevArray&) = delete;
    DevArray(DevArray&& o) noexcept : p(o.p), n(o.n), as(o.as), async(o.async)
    {
        o.p = nullptr;
        o.n = 0;
        o.async = false;
    }
    DevArray& operator=(DevArray&& o) noexcept
    {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            as = o.as;
            async = o.async;
            o.p = nullptr;
            o.n = 0;
            o.async = false;
        }
        return *this;
    }
    ~DevArray() { release(); }
    void alloc(size_t count)
    {
        release();
        n = count;
        if (!count) return;
        cudaStream_t s = thread_alloc_stream();
        if (s) {
            if (thread_in_capture())
                throw std::logic_error("device allocation inside a stream capture");
            UNAP_CK(cudaMallocAsync((void**)&p, count * sizeof(T), s));
            as = s;
            async = true;
        } else {
            UNAP_CK(gated_malloc((void**)&p, count * sizeof(T)));
        }
    }
    void release()
    {
        if (p) {
            if (async)
                cudaFreeAsync(p, as);
            else
                gated_free(p);
        }
        p = nullptr;
        n = 0;
        async = false;
    }
    // stream 0 means the array's own stream for a stream-ordered array
    cudaStream_t on(cudaStream_t s) const { return (!s && async) ? as : s; }
    void upload(const T* h, size_t count, cudaStream_t s = 0)
    {
        if (count != n) alloc(count);
        if (count)
            UNAP_CK(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, on(s)));
    }
    void upload(const std::vector<T>& h, cudaStream_t s = 0) { upload(h.data(), h.size(), s); }
    void zero(cudaStream_t s = 0)
    {
        if (n) UNAP_CK(cudaMemsetAsync(p, 0, n * sizeof(T), on(s)));
    }
    size_t bytes() const { return n * sizeof(T); }
};

// Stream-ordered scratch (cudaMallocAsync), freed on its stream when it
// goes out of scope; for the setup kernels that must not synchronize the
// device while other streams are solving.
template <class T>
struct StreamScratch {
    T* p = nullptr;
    cudaStream_t s = 0;
    StreamScratch(size_t count, cudaStream_t st) : s(st)
    {
        if (count) UNAP_CK(cudaMallocAsync((void**)&p, count * sizeof(T), s));
    }
    StreamScratch(const StreamScratch&) = delete;
    StreamScratch& operator=(const StreamScratch&) = delete;
    ~StreamScratch()
    {
        if (p) cudaFreeAsync(p, s);
    }
};

// Host copy of one LDU matrix in the reference's layout.
struct HostLdu {
    int n = 0, nf = 0;
    bool symm = true;
    std::vector<int> l, u;
    std::vector<double> lower, diag, upper;  // lower empty when symm
    bool oriented = true;     // lowerAddr[f] < upperAddr[f] for every face
    bool ownerSorted = true;  // lowerAddr non-decreasing
    const double* lowerPtr() const { return symm ? upper.data() : lower.data(); }
    void validate();
};

// Per-matrix topology on the device (shared by FP64 and FP32 values).
struct Level {
    int n = 0, nf = 0;
    bool symm = true;
    bool sweepable = true;   // oriented && ownerSorted: DIC/DILU/GS allowed
    int nWave = 0;           // number of forward wavefronts
    std::vector<int> waveStart;  // nWave+1, internal row ranges
    std::vector<int> perm;       // internal -> reference cell
    std::vector<int> iperm;      // reference cell -> internal
    // reference cell -> rank in the locality order (the key order, or the
    // BFS order of the finest level): internal order within a wavefront,
    // and the whole internal order of a level built without wavefronts
    std::vector<int> locRank;
    int nSlices = 0;
    long long nEntries = 0;      // padded SELL storage
    int maxRowLen = 0;
    DevArray<int> d_perm, d_iperm;
    DevArray<int> d_sliceOff, d_rowInfo, d_col;
    // FP64 values
    DevArray<double> d_val, d_valT, d_diag;
    // FP32 values (mixed precision); filled on demand
    DevArray<float> d_val32, d_diag32;
    // SELL positions of each face's two entries (row u: lower side, row l:
    // upper side), kept to refresh coefficients without rebuilding topology
    std::vector<int> entLo, entUp;
    int version = 0;  // process-unique, renewed on every coefficient update
    size_t deviceBytes() const;
};

// Replace the FP64 coefficients of a Level (same addressing and symmetry).
void update_level_values(Level& L, const HostLdu& A, cudaStream_t s);

// Build the internal order, the SELL-32 structure and upload FP64 values.
// `key` (optional, size n) gives the locality order inside a wavefront;
// when empty a BFS order of the matrix graph is used.  `identityOrder`
// keeps the reference numbering (used for the dense coarsest level).
// wavefronts == false puts every row in one range in locality order (for
// levels that are never swept: SpMV-shaped smoothing only); such a level is
// marked not sweepable.
std::unique_ptr<Level> build_level(const HostLdu& A, const std::vector<int>* key,
                                   bool identityOrder, cudaStream_t s, bool wavefronts = true);
void make_fp32(Level& L, cudaStream_t s);
// The same Level built by kernels on stream s (level_dev.cu); nullptr when
// the matrix has a shape the device build leaves to the host.
std::unique_ptr<Level> build_level_device(const HostLdu& A, const std::vector<int>* key,
                                          cudaStream_t s, bool wavefronts = true);
// Levels of at least this many cells are built on the device (< 0: none).
long long set_device_setup_min_cells(long long minCells);
long long device_setup_min_cells();
// out[i] = in[0] + ... + in[i-1] for i <= n (n + 1 outputs), on stream s
void device_exclusive_scan(const int* in, int* out, long long n, cudaStream_t s);
// COO (1-based rows and columns) or CSR (0-based row pointer and columns)
// to LDU on the device, bit-identical to the host form; false when it
// declines (a column with too many lower entries) and nothing was done.
bool coo_to_ldu_device(const double* val, const int* rowsOrPtr, const int* cols, int n, int size,
                       bool symm, bool csr, cudaStream_t s, HostLdu& out);

// Solver state shared by the device kernels of one solve (device memory).
// Every kernel of an iteration first checks `done` (and `early` where the
// BiCGStab half-step exit applies) and returns at once when set, so a host
// can enqueue or graph-launch iterations ahead of the convergence test.
struct KState {
    double wArA, wArAold, wApA, alpha, beta, omega;
    double rA0rA, rA0rAold, tAtA, tAsA, zq;
    double initRes, finalRes, trueRes;
    double tol, relTol;
    int nIter, maxIter, minIter, converged, singular, done;
    int first;    // the next direction update starts a (re)start
    int useBeta;  // direction update uses beta (0: p = z)
    int early;    // BiCGStab converged on ||s|| inside the iteration
    int flexible; // PCG: Polak-Ribiere beta
    int status;   // 0 ok, otherwise an error code
    int pad;
};

// Finalize operations run by the last block of a reducing kernel.
enum Fin : int {
    FIN_NONE = 0,
    FIN_STORE,        // launch sums only (a later launch finalizes)
    FIN_INIT_RES,     // initRes = finalRes = sqrt(sum0) + SMALL
    FIN_PCG_WR,       // wArA (+ zq) -> singularity test, beta
    FIN_PCG_ALPHA,    // wApA -> alpha
    FIN_PCG_RES,      // finalRes, iteration count, convergence
    FIN_BICG_INIT,    // initRes from sum0; sum1 = first rA0rA
    FIN_BICG_ALPHA,   // rA0.AyA -> alpha
    FIN_BICG_S,       // ||s|| -> early-exit test
    FIN_BICG_OMEGA,   // tAtA, tA.sA -> omega
    FIN_BICG_RES,     // ||r||, rA0.r -> iteration count, convergence
    FIN_RES_ONLY,     // finalRes = sqrt(sum0) + SMALL (no iteration logic)
    FIN_MG_RES,       // MGSolver: finalRes, iteration count, convergence
    FIN_TRUE_RES,     // trueRes = sqrt(sum0) + SMALL
};

// One reduction site: per-block partials, per-launch sums, one ticket.
struct RSpec {
    double* blockPart = nullptr;  // >= gridDim.x * K
    double* launchAcc = nullptr;  // >= nSlots * K
    unsigned* ticket = nullptr;
    int slot = 0;    // this launch's index into launchAcc
    int nSlots = 1;  // launches to combine when finalizing
    int fin = FIN_NONE;
    KState* st = nullptr;
    int maxBlocks = 0;  // blockPart holds partials of at most this many CTAs
};

// Gate: skip the kernel when st->done (mask 1) or st->early (mask 2) is set.
struct Gate {
    const KState* st = nullptr;
    int mask = 0;
};

// Device workspace for the reduction sites of one solver.
struct RedPool {
    DevArray<double> blockPart;  // nSites * maxBlocks * 4
    DevArray<double> launchAcc;  // nSites * maxLaunch * 4
    DevArray<unsigned> tickets;  // nSites
    int nSites = 0, maxBlocks = 0, maxLaunch = 0;
    void init(int sites, int blocks, int launches, cudaStream_t s);
    RSpec site(int i, KState* st, int fin, int slot = 0, int nSlots = 1) const;
};

constexpr int kBlock = 256;
constexpr int kRedK = 4;  // max values reduced together

inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

// Launch context: stream and the grid cap (blocks) for grid-stride kernels.
struct Exec {
    cudaStream_t s = 0;
    int maxBlocks = 1216;
    int grid(long long n) const
    {
        int g = div_up(n, kBlock);
        return g < 1 ? 1 : (g > maxBlocks ? maxBlocks : g);
    }
    // one row per thread; a reducing launch stays within its reduction
    // site's partial buffer
    int rowGrid(long long n, const RSpec& red) const
    {
        int g = div_up(n, kBlock);
        if (g < 1) g = 1;
        if (red.blockPart && g > red.maxBlocks) g = red.maxBlocks;
        return g;
    }
};

int device_max_blocks();  // SMs * resident 256-thread blocks

// Count of kernel launches issued by this library (graph launches add their
// kernel-node count; launches recorded into a graph capture are not counted).
void count_launches(long long k);
long long launch_count();
void set_capturing(bool on);
bool capturing();

}  // namespace unapgpu
