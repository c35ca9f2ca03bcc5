// Agglomeration AMG on the device: hierarchy, V-cycle, AMG-PCG.
#pragma once

#include <memory>
#include <vector>

#include "cheby.hpp"
#include "engine.hpp"
#include "tail.hpp"

namespace unapgpu {

// One coarse level produced by the host agglomeration (reference numbering).
struct CoarseHost {
    HostLdu A;
    std::vector<int> restrictAddr;  // finer cells -> this level's cells
    std::vector<int> faceRestrict;  // finer faces -> coarse face, or -(cell+1)
};

std::vector<int> pairwise_pass(const HostLdu& A, const std::vector<double>& w, int& nCoarse);
void coarse_addressing(const HostLdu& fine, const std::vector<int>& map, int nCoarse,
                       CoarseHost& out);
void coarse_coefficients(const HostLdu& fine, CoarseHost& c);
// stopRule 0: the reference's rule (keep a level while it has >= nCoarsest
// cells); stopRule 1: agglomerate until the coarsest has <= nCoarsest cells.
// Levels of at least device_setup_min_cells() cells are agglomerated by
// kernels on stream s (aggl_dev.cu), with the same result.
std::vector<CoarseHost> agglomerate_levels(const HostLdu& fine, const std::vector<double>& weights,
                                           int nCoarsest, int maxLevels, int stopRule,
                                           cudaStream_t s = 0);
bool agglomerate_level_device(const HostLdu& A, const std::vector<double>& w, CoarseHost& out,
                              std::vector<double>& cw, int& nCoarse, cudaStream_t s);
std::vector<double> mg_face_weights(const HostLdu& A);

struct AmgParams {
    int nCoarsest = 1000;
    int maxLevels = 50;
    int nPre = 2, nPost = 2;
    int precision = 0;  // 0 FP64 V-cycle, 1 FP32 V-cycle (coarsest solve FP64)
    int smoother = 0;     // 0 Gauss-Seidel, 1 Chebyshev on levels >= chebyFrom
    int chebyDegree = 3;  // Chebyshev steps before and after the coarse correction
    int chebyFrom = 0;    // first Chebyshev level (Gauss-Seidel above it)
    double eigRatio = 30; // interval [lam / eigRatio, 1.1 lam]; <= 0: the reference's 1.5
};

// Device hierarchy for AMG as a fixed, symmetric PCG preconditioner:
//   level k < L: x = 0; nPre forward GS sweeps; r = b - A x; b' = R r;
//                e = V(k+1, b'); x += P e; nPost backward GS sweeps
//   level L:     x = Minv b (dense FP64 inverse, rows summed in column order)
// R sums the aggregate's cells in ascending cell order, P injects.
// With the Chebyshev smoother a level k >= chebyFrom replaces the sweeps by
// chebyDegree Chebyshev steps from x = 0 before, and from x after, the
// coarse correction (cheby.hpp), over [lam_k / eigRatio, 1.1 lam_k] with
// lam_k the reference's diagonal-PCG estimate of the level's largest
// eigenvalue of D^-1 A taken once at setup (FP64, from x = 0 and the
// splitmix64 start vector); the same polynomial on both sides keeps the
// preconditioner symmetric.  A level's first step from x = 0 is fused into
// the restriction that produces its right-hand side.
class AmgHierarchy {
public:
    AmgHierarchy(Matrix& A, const AmgParams& p);
    int nLevels() const { return (int)lv.size(); }
    std::vector<int> levelCells() const;
    std::vector<int> levelWavefronts() const;
    // z = M^-1 r, internal order of the finest level
    void vcycle(const Exec& ex, const double* r, double* z, Gate g);
    // mean V-cycle time over `reps` runs on internal vectors (ms[0]), then
    // per level from one run with events around every level (ms[1 + k]:
    // level k's own steps; a level running in the cluster tail holds the
    // whole tail's time and the levels below it 0); returns levels written
    int profile(cudaStream_t s, int reps, double* ms, int maxOut);
    // mean time of one smoothing launch group on level k (< the coarsest)
    // in the V-cycle's precision, over `reps` runs after one warm-up, on
    // scratch vectors: a Chebyshev step (one launch) on Chebyshev levels, a
    // forward Gauss-Seidel sweep (one launch per wavefront) otherwise.
    // *bytes = its algorithmic bytes, *launches = launches per run.
    double profileSmoother(cudaStream_t s, int k, int reps, double* bytes, int* launches);
    // the same V-cycle as a step program (mega.hpp); lv[0] is the finest
    void appendVcycle(std::vector<Step>& out, std::vector<LevelRows>& lv, const double* r,
                      double* z);
    AmgParams params;
    double setupSeconds = 0;
    // host wall time of the setup phases, seconds: face weights and
    // agglomeration, coarse level builds and transfer maps, coarsest
    // inverse, vectors and FP32 copies, row packing, eigenvalue estimates
    double setupPhase[6] = {0, 0, 0, 0, 0, 0};
    size_t deviceBytes() const;

    struct Lv {
        const Level* L = nullptr;        // device structure (level 0: the matrix's)
        std::unique_ptr<Level> own;
        int n = 0;
        DevArray<int> childStart, child;  // restriction into this level (k >= 1)
        DevArray<int> cmap;               // prolongation from this level (k >= 1)
        DevArray<double> x, b, r;
        DevArray<float> xf, bf, rf;
        DevArray<double> t;  // second Chebyshev iterate (FP64 V-cycle)
        DevArray<float> tf;  // second Chebyshev iterate (FP32 V-cycle)
        PackedRows pack;  // row-packed copy for the cluster tail (coarse levels)
        double lam = 0;   // Chebyshev: eigenvalue estimate and coefficients
        double Rth = 0, d1[kChebyMaxDegree] = {}, d2[kChebyMaxDegree] = {};
    };
    std::vector<Lv> lv;
    DevArray<double> Minv;  // coarsest dense inverse, column-major
    const int* denseGather = nullptr;  // b index of each Minv column (null: identity)
    int nc = 0;
    DevArray<int> dWaves;       // wave starts of every level, concatenated
    std::vector<int> waveOff;   // level k's first entry in dWaves (size levels + 1)
    // first level of the V-cycle that runs in the cluster tail kernel under
    // the current thresholds and shared-memory capacity for elements of
    // elemBytes bytes (nLevels() - 1: no tail)
    int tailFirst(size_t elemBytes) const;
    // level k (< the coarsest) is smoothed by Chebyshev steps
    bool isCheby(int k) const
    {
        return params.smoother == 1 && k >= params.chebyFrom && k < nLevels() - 1;
    }
    std::vector<double> eigenvalues() const;

private:
    void setupCheby(cudaStream_t s);
    template <class T>
    T* Tmp(int k);
    // the buffer holding step j of a level's pre- (or post-) smoothing chain,
    // chosen so that the last step lands in X(k)
    template <class T>
    T* chebBuf(int k, int j);
    Matrix& A;
    template <class T>
    void vcycle_level(const Exec& ex, int k, Gate g);
    template <class T>
    void launch_tail(const Exec& ex, int t, Gate g);
    template <class T>
    void sweep(const Exec& ex, int k, const Level& Lk, const Rows<T>& Rk, T* x, const T* b,
               bool backward, bool xIsZero, Gate g);
    int curTail = -1;
    // first level of the Chebyshev cluster tail (launch_cheb_tail), -1: none
    int chebTail = -1;
    DevArray<double> chebTailPart;  // its coarsest chunk sums
    template <class T>
    ChebTailArgs<T> chebTailArgs(int k);
    std::vector<cudaEvent_t>* profIn = nullptr;   // per-level events (profiling)
    std::vector<cudaEvent_t>* profOut = nullptr;
    template <class T>
    void append_level(std::vector<Step>& out, int k, int tableBase);
    template <class T>
    T* X(int k);
    template <class T>
    T* B(int k);
    template <class T>
    T* R(int k);
};

class AmgPrecond : public Precond {
public:
    explicit AmgPrecond(AmgHierarchy& h) : H(h) {}
    void apply(const Exec& ex, const double* r, double* w, const RedPool*, int, KState*, int,
               Gate g) override
    {
        H.vcycle(ex, r, w, g);
    }
    bool appendSteps(std::vector<Step>& out, std::vector<LevelRows>& lv, const double* r,
                     double* w, int, bool* dotFused) override
    {
        H.appendVcycle(out, lv, r, w);
        *dotFused = false;
        return true;
    }
    AmgHierarchy& H;
};

}  // namespace unapgpu
