// Batched solves of many LDU systems (batch.cu).
#pragma once

#include <map>
#include <vector>

#include "engine.hpp"
#include "small_solve.hpp"

namespace unapgpu {

// Systems of at most team_solve_cells() cells (default below) are solved by
// one fused launch, a team of CTAs per system (small_solve.cu).
constexpr int kTeamSolveCells = 65536;
int team_solve_cells();
int set_team_solve_cells(int cells);  // returns the previous value; 0 turns it off

struct BatchItem {
    Matrix* A = nullptr;
    int method = 0;   // 0 PCG, 1 PBiCGStab
    int precond = 0;  // 0 none, 1 Diag, 2 DIC, 3 DILU
    double tol = 0.0, relTol = 1e-6;
    int maxIter = 1000, minIter = 0;
    double* x = nullptr;        // device, caller's order (initial guess in, solution out)
    const double* b = nullptr;  // device, caller's order
};

class BatchSolver {
public:
    explicit BatchSolver(cudaStream_t s);
    ~BatchSolver();
    std::vector<SolveStats> solve(const std::vector<BatchItem>& items);
    TeamShape lastShape{0, 0};  // shape of the last fused launch
    int lastLargeMode = -1;     // systems above the whole-solve size: 1 one
                                // group launch, 0 one after another, -1 none

    // drop the cached preconditioner diagonals of a matrix that is going away
    void forget(const Matrix* A);

private:
    struct Key {
        const Matrix* A;
        int precond;
        bool operator<(const Key& o) const
        {
            return A < o.A || (A == o.A && precond < o.precond);
        }
    };
    struct Fac {
        int version = -1;
        DevArray<double> rD;
    };
    cudaStream_t stream;
    std::map<Key, Fac> factors;       // preconditioner diagonals per matrix
    DevArray<double> ws;              // internal-order x, b and work vectors
    DevArray<SmallSystem> dSys;
    DevArray<SmallResult> results;
    std::vector<DevArray<int>> waveDev;
    DevArray<unsigned char> dIn, dOut;  // gather / scatter job lists
    const double* factor(Matrix& A, int precond);
    // the systems idx in one whole-solve launch (largeGroup: systems above
    // the whole-solve size, clusters of 16 only); *tunedMs = the chosen
    // shape's capped trial time (timed now or cached with the shape), left
    // as it is for a forced shape
    void solveSmall(const std::vector<BatchItem>& items, const std::vector<int>& idx,
                    std::vector<SolveStats>& out, bool largeGroup = false,
                    float* tunedMs = nullptr);
    SolveStats solveOne(const BatchItem& it, int maxIter);
    double timeSequential(const std::vector<BatchItem>& items, const std::vector<int>& idx);
};

// Shape of a fused launch of m systems (device array d_systems, largest
// nMax cells): the autotuner's choice for the pair (nMax rounded up to a
// power of two, m in classes 1 / 2-4 / 5-16 / 17-64 / more).  The first
// launch of a pair times every launchable shape (CTA size 128 .. 1024 x
// cluster 1 .. 16 CTAs) on these systems with the iterations capped, the
// initial guesses restored after each trial, and caches the fastest.
TeamShape tuned_team_shape(cudaStream_t s, const SmallSystem* d_systems, int m, int nMax,
                           bool largeGroup = false, float* bestMs = nullptr);
// the cached shape of a pair ({0, 0}: not tuned yet)
TeamShape cached_team_shape(int nMax, int m, bool largeGroup = false);
// systems above the whole-solve size in a batch: 1 one group launch, 0 one
// after another, -1 not measured yet for this pair
int cached_large_mode(int nMax, int m);
// every later launch uses this shape instead of the tuner's (threads 0:
// back to the tuner)
void force_team_shape(int threads, int cluster);

}  // namespace unapgpu
