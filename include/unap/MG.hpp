/* UNAP::MGSolver (src/solvers/MG/MG.hpp, MG.cpp:3-63, MGSolve.cpp:17-187,
 * Vcycle.cpp:11-332, scalingFactor.cpp:11-65, solveCoarsestLevel.cpp:10-55):
 * the multigrid V-cycle iteration, run on the GPU over the hierarchy that
 * the lduAgglomeration's last agglomerate() call defines (same weights,
 * coarsest size and level limit), with the smoothers' kind (every level
 * Gauss-Seidel, or every level Chebyshev).  Defaults: 0 pre-, 2 post- and
 * 2 finest sweeps, correction scaling when the matrix is symmetric.  The
 * device solver is kept between solves and rebuilt when the matrix or the
 * hierarchy changes; initSmoothers() restarts the Chebyshev estimates. */
#ifndef MG_HPP
#define MG_HPP

#include "chebySmoother.hpp"
#include "lduAgglomeration.hpp"
#include "lduGaussSeidelSmoother.hpp"

namespace UNAP
{

class MGSolver : public matrix::solver
{
protected:
    const matrix& finestMatrix_;
    bool cacheAgglomeration_;
    label nPreSweeps_;
    label nPostSweeps_;
    label nFinestSweeps_;
    bool scaleCorrection_;
    matrix::agglomeration& agglomeration_;
    const PtrList<matrix::smoother>& smoothers_;
    mutable long int mg_;
    mutable long int mgMatrix_;
    mutable const void* mgWeights_;

    int smoother_kind_() const
    {
        int kind = 0;
        forAll(i, smoothers_.size())
        {
            const matrix::smoother* s = smoothers_.get(i);
            if (!s) continue;
            const int k = dynamic_cast<const lduGaussSeidelSmoother*>(s) ? 1
                          : dynamic_cast<const chebySmoother*>(s)        ? 2
                                                                         : -1;
            if (k < 0 || (kind && k != kind)) {
                std::cerr << "UNAP (GB300): MGSolver runs one smoother kind on every level "
                             "(lduGaussSeidelSmoother or chebySmoother)"
                          << std::endl;
                ERROR_EXIT;
            }
            kind = k;
        }
        if (!kind) {
            std::cerr << "UNAP (GB300): MGSolver has no smoother" << std::endl;
            ERROR_EXIT;
        }
        return kind;
    }

    void release_() const
    {
        if (mg_) unap_cuda_mg_destroy(mg_);
        mg_ = 0;
    }

public:
    MGSolver(const matrix& A, matrix::agglomeration& agglomerator,
             const PtrList<matrix::smoother>& smoothers)
        : finestMatrix_(A), cacheAgglomeration_(false), nPreSweeps_(0), nPostSweeps_(2),
          nFinestSweeps_(2), scaleCorrection_(A.symm()), agglomeration_(agglomerator),
          smoothers_(smoothers), mg_(0), mgMatrix_(0), mgWeights_(NULL)
    {
    }
    MGSolver(const MGSolver&) = delete;
    MGSolver& operator=(const MGSolver&) = delete;
    virtual ~MGSolver() { release_(); }

    virtual matrix::solverPerformance solve(scalarField& x, const matrix& A,
                                            const scalarField& b) const
    {
        const lduMatrix* L = dynamic_cast<const lduMatrix*>(&A);
        const lduAgglomeration* G = dynamic_cast<const lduAgglomeration*>(&agglomeration_);
        if (!L || !G || &G->finestMatrix() != L) {
            std::cerr << "UNAP (GB300): MGSolver solves the lduMatrix its lduAgglomeration "
                         "was built on"
                      << std::endl;
            ERROR_EXIT;
        }
        if (!G->agglomerated()) {
            std::cerr << "UNAP (GB300): call agglomerate(weights) before MGSolver::solve"
                      << std::endl;
            ERROR_EXIT;
        }
        if (x.size() != L->size() || b.size() != L->size()) {
            std::cerr << "UNAP (GB300): x and b must have nCells entries" << std::endl;
            ERROR_EXIT;
        }
        const long int h = L->deviceHandle();
        const int kind = smoother_kind_();
        if (mg_ && (mgMatrix_ != h || mgWeights_ != G->weights().values())) release_();
        if (!mg_) {
            detail::check(
                unap_cuda_mg_create(&mg_, h, G->weights().values(), kind,
                                    detail::to_int(G->nCellsInCoarsestLevel(), "nCoarsest"),
                                    detail::to_int(G->maxLevels(), "maxLevels"),
                                    detail::to_int(nPreSweeps_, "nPreSweeps"),
                                    detail::to_int(nPostSweeps_, "nPostSweeps"),
                                    detail::to_int(nFinestSweeps_, "nFinestSweeps"),
                                    scaleCorrection_ ? 1 : 0, tolerance_, relTol_,
                                    detail::to_int(maxIter_, "maxIter"),
                                    detail::to_int(minIter_, "minIter")),
                "MGSolver");
            mgMatrix_ = h;
            mgWeights_ = G->weights().values();
        } else {
            detail::check(unap_cuda_mg_set(mg_, detail::to_int(nPreSweeps_, "nPreSweeps"),
                                           detail::to_int(nPostSweeps_, "nPostSweeps"),
                                           detail::to_int(nFinestSweeps_, "nFinestSweeps"),
                                           scaleCorrection_ ? 1 : 0, tolerance_, relTol_,
                                           detail::to_int(maxIter_, "maxIter"),
                                           detail::to_int(minIter_, "minIter")),
                          "MGSolver");
        }
        unap_cuda_stats st;
        detail::check(unap_cuda_mg_solve_host(mg_, x.values(), b.values(), &st), "MGSolver::solve");
        if (ifPrint_)
            COUT << "MGSolver: " << st.nIterations << " V-cycles, residual " << st.initialResidual
                 << " -> " << st.finalResidual << ENDL;
        return matrix::solverPerformance(st.initialResidual, st.finalResidual, st.nIterations,
                                         st.converged != 0, st.singular != 0);
    }

    void SET_nPreSweeps(const label n) { nPreSweeps_ = n; }
    void SET_nPostSweeps(const label n) { nPostSweeps_ = n; }
    void SET_nFinestSweeps(const label n) { nFinestSweeps_ = n; }
    void SET_cacheAgglomeration(bool c) { cacheAgglomeration_ = c; }
    void SET_scaleCorrection(bool s) { scaleCorrection_ = s; }

    /* MG.cpp:55-63: the smoothers start over (Chebyshev estimates again) */
    void initSmoothers()
    {
        forAll(i, smoothers_.size())
        {
            if (smoothers_.get(i)) smoothers_[i].init();
        }
        release_();
    }

    matrix::agglomeration& agglomeration() { return agglomeration_; }
};

}  // namespace UNAP

#endif
