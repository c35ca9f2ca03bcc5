// Coarse-level tail of the AMG V-cycle in one thread-block-cluster launch.
//
// Below a few hundred thousand rows a Gauss-Seidel wavefront holds too few
// rows to fill the GPU, and one kernel launch per wavefront costs more than
// the wavefront's work.  The tail kernel runs every level from a chosen level
// down to the dense coarsest solve and back up (pre-smoothing, residual,
// restriction, coarsest product, prolongation, post-smoothing) inside ONE
// launch of a single cluster of CTAs (16 where the GPU schedules it, else 8,
// 4, 2):
//
//  * the iterate x of every tail level lives in shared memory: 32-row slices
//    round-robin over the cluster's CTAs (slice s on CTA s mod C), read
//    across CTAs through distributed shared memory; levels of at most
//    `singleRows` rows live in, and run on, the first CTA alone;
//  * wavefronts are separated by the cluster's hardware barrier
//    (barrier.cluster arrive.release / wait.acquire), or by the block
//    barrier on a first-CTA-only level;
//  * the matrix data of a thread's next row (row info, entries, diagonal,
//    right-hand side) is loaded into registers before the barrier that
//    precedes it, so only shared-memory reads of x remain after it.
//
// Every row keeps the per-step kernels' arithmetic order, so the V-cycle
// result is bit-identical to them.
#pragma once

#include "kernels.hpp"

namespace unapgpu {

constexpr int kTailMaxLevels = 24;
constexpr int kTailThreads = 256;
constexpr int kTailMaxWaves = 4096;  // wave starts of all tail levels, staged in shared memory
constexpr int kTailMaxCoarsest = 4096;
constexpr int kTailMaxCluster = 16;
constexpr int kTailPackRows = 1 << 24;  // levels up to this size get a row-packed copy

// One smoothed level of the tail (pointers to T = float or double data).
struct TailLevel {
    int n = 0, nWave = 0, waveOff = 0, single = 0;
    int nNext = 0;                 // cells of the next coarser level
    int xOff = 0;                  // this level's x in each CTA's shared x area (elements)
    const int* sliceOff = nullptr;
    const int* rowInfo = nullptr;
    const int* col = nullptr;
    const void* val = nullptr;
    const void* diag = nullptr;
    void* b = nullptr;             // global (L2-resident)
    void* r = nullptr;             // global residual, read by the restriction
    const int* childStart = nullptr;  // restriction into the next level
    const int* child = nullptr;
    const int* cmap = nullptr;        // prolongation from the next level (size n)
    // row-packed copy of the matrix (see PackedRows)
    const int2* pmeta = nullptr;
    const int4* prec = nullptr;
};

// Row-packed copy of a level for the tail kernel: a row's entries are
// contiguous 16-byte records, in the row's entry order (the SELL-32 order),
// so a thread loads its whole row with a few vector loads.  FP32: two
// entries per record {col, value bits, col, value bits}; FP64: one entry per
// record {col, 0, value low word, value high word}.  meta[r] = {first record
// of row r, row info (len | nLow << 16)}.
struct PackedRows {
    DevArray<int2> meta;
    DevArray<int4> rec;
    size_t bytes() const { return meta.bytes() + rec.bytes(); }
};
template <class T>
void pack_rows(const Rows<T>& A, PackedRows& out, cudaStream_t s);

// Gauss-Seidel sweep of a level, one launch per wavefront like gs_sweep,
// reading the row-packed copy: a thread loads its row's first 24 (FP32) or
// 12 (FP64) entries as 16-byte records before the dependency wait of the
// programmatic dependent launch, so after it only the x gathers remain.
// Same arithmetic and results as gs_sweep.
// AMG V-cycle sweeps on levels with long rows: 1 (default) gs_sweep_packed
// with the register window chosen by the level's mean row length (16 / 8
// entries below 12.5 entries per row, 24 / 12 above); 2 always 16 / 8; 3
// always 24 / 12; 0 the SELL-32 kernel.  Returns the previous value.
int set_packed_sweeps(int mode);
int packed_sweeps();

template <class T>
void gs_sweep_packed(const Exec& ex, const Level& L, const PackedRows& P, const T* diag, T* x,
                     const T* b, bool backward, bool xIsZero, bool wide, Gate g);

struct TailArgs {
    TailLevel lv[kTailMaxLevels];
    int nLv = 0, nPre = 2, nPost = 2;
    int nc = 0;                    // coarsest cells (dense FP64 inverse)
    int xcOff = 0;                 // coarsest x in the shared x area (cluster-distributed)
    int xElems = 0;                // shared x area per CTA (elements)
    const double* Minv = nullptr;  // column-major nc x nc
    void* bc = nullptr;
    void* xOut = nullptr;          // x of the first tail level, written back to global
    const int* waves = nullptr;    // wave starts of the tail levels, concatenated
    int nWaveTotal = 0;
    Gate g;
};

// Largest cluster size the device schedules for the tail kernel (0: none).
int tail_cluster_size();
// Bytes of dynamic shared memory a tail CTA may use.
size_t tail_smem_bytes();

// Shared x area (elements per CTA) of a tail over levels of the given sizes
// (the coarsest last); singleRows as in set_tail_rows.
long long tail_x_elems(const std::vector<int>& sizes, int clusterSize, long long singleRows);

// Tail thresholds (process-wide, per V-cycle precision: 0 FP64, 1 FP32):
// levels with at most `tailRows` rows run in the tail kernel (0 disables it)
// as far as their x fits in shared memory; tail levels with at most
// `singleRows` rows run on one CTA.  Returns the previous values through the
// pointers.
void set_tail_rows(int precision, long long tailRows, long long singleRows, long long* oldTail,
                   long long* oldSingle);
long long tail_rows(int precision);
long long single_rows(int precision);

template <class T>
void launch_tail_vcycle(const TailArgs& a, int clusterSize, cudaStream_t s);

}  // namespace unapgpu
