// The reference's MGSolver (V-cycle iteration) on the device.
#pragma once

#include <memory>
#include <vector>

#include "amg.hpp"
#include "cheby.hpp"
#include "small_solve.hpp"

namespace unapgpu {

struct MgParams {
    int nCoarsest = 50;   // lduAgglomeration.cpp:11
    int maxLevels = 50;   // lduAgglomeration.cpp:10
    int smoother = 1;     // 1 Gauss-Seidel, 2 Chebyshev
    int nPre = 0, nPost = 2, nFinest = 2;  // MG.cpp:3-19
    int scaleCorr = -1;   // -1: A.symm() (MG.cpp:13)
    double tol = 0.0, relTol = 1e-6;
    int maxIter = 1000, minIter = 0;
};

// MGSolver::solve (MGSolve.cpp:17-187) with Vcycle (Vcycle.cpp:27-332),
// scalingFactor (scalingFactor.cpp:11-65) and solveCoarsestLevel
// (solveCoarsestLevel.cpp:10-55).  Hierarchy: the reference's agglomeration
// and stop rule.  Every vector operation keeps the reference's per-row
// order; reductions (norms, scaling sums, the eigenvalue estimate's dot
// products) use fixed device trees.
class MgSolver {
public:
    MgSolver(Matrix& A, const std::vector<double>& weights, const MgParams& p);
    ~MgSolver();
    MgParams params;
    SolveStats solveDevice(double* x_ref, const double* b_ref);
    SolveStats solveHost(double* x, const double* b);
    // MGSolver::initSmoothers (MG.cpp:55-63): Chebyshev smoothers estimate
    // their eigenvalue again on their next call
    void initSmoothers();
    int nCoarseLevels() const { return (int)lv.size() - 1; }
    std::vector<int> levelCells() const;

private:
    struct Lv {
        const Level* L = nullptr;
        std::unique_ptr<Level> own;
        int n = 0;
        DevArray<int> childStart, child, cmap;  // transfer into this level (k >= 1)
        DevArray<double> corr, src, acf, pre, rD, w, p;
        DevArray<double> dfac, pfac;  // coarsest DIC/DILU factor
    };
    Matrix& A;
    std::vector<Lv> lv;  // lv[0] finest, lv[k] coarse level k-1 of the reference
    bool scale;
    Exec ex;
    DevArray<double> x, b, Apsi, fc, fr;
    DevArray<double> sfs;          // scaling factors of one V-cycle
    DevArray<EigState> eig;        // one per smoother slot
    std::vector<int> chebyFirst;   // host: slot not yet estimated
    DevArray<SmallSystem> coarseSys;
    DevArray<double> coarseWork;
    DevArray<int> waveDev;
    KState* d_st = nullptr;
    KState* h_st = nullptr;
    RedPool pool;
    cudaEvent_t ev0, ev1;
    void smooth(int slot, int k, double* xk, const double* bk, int nSweeps);
    void scaling(int k, double* field, const double* source, double* Acf, int sfSlot);
    void vcycle();
    void chebyshev(int slot, int k, double* xk, const double* bk, int nSweeps);
    void eigen_estimate(int slot, int k, double* xk, const double* bk);
};

}  // namespace unapgpu
