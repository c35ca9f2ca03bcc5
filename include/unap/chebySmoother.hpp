/* UNAP::chebySmoother (src/smoothers/chebySmoother/chebySmoother.cpp:13-149,
 * defaults chebySmoother.hpp:41-53): the first smooth() after construction
 * or init() estimates the largest eigenvalue of D^-1 A with 10
 * diagonal-PCG iterations (eigenDiagPCG.cpp:11-361), which change x, and
 * returns; later calls run nSweeps Chebyshev steps over
 * [maxEig / 1.5, 1.1 maxEig].  All of it on the GPU. */
#ifndef CHEBYSMOOTHER_HPP
#define CHEBYSMOOTHER_HPP

#include "lduMatrix.hpp"

namespace UNAP
{

class chebySmoother : public matrix::smoother
{
private:
    label nDiagPCGs_;
    mutable scalar maxEigPCG_;
    mutable bool eigFirstTimeComputed_;
    scalar eigRatioCheby_;
    scalar boostFactorCheby_;
    scalar eigRatioCoarest_;
    label preSmoothUsing_;

public:
    chebySmoother()
        : nDiagPCGs_(10), maxEigPCG_(0.0), eigFirstTimeComputed_(true), eigRatioCheby_(1.5),
          boostFactorCheby_(1.1), eigRatioCoarest_(1.0), preSmoothUsing_(0)
    {
    }
    virtual ~chebySmoother() {}

    virtual void smooth(scalarField& x, const matrix& A, const scalarField& b,
                        const label nSweeps) const
    {
        const lduMatrix* L = dynamic_cast<const lduMatrix*>(&A);
        if (!L) {
            std::cerr << "UNAP (GB300): chebySmoother smooths lduMatrix systems" << std::endl;
            ERROR_EXIT;
        }
        smooth(x, *L, b, nSweeps);
    }

    void smooth(scalarField& x, const lduMatrix& A, const scalarField& b,
                const label nSweeps) const
    {
        int estimated = eigFirstTimeComputed_ ? 0 : 1;
        detail::check(unap_cuda_cheby_smooth_host(A.deviceHandle(), x.values(), b.values(),
                                                  detail::to_int(nSweeps, "nSweeps"),
                                                  &maxEigPCG_, &estimated),
                      "chebySmoother::smooth");
        eigFirstTimeComputed_ = estimated == 0;
    }

    virtual void init() const { eigFirstTimeComputed_ = true; }

    /* the eigenvalue estimate (0 before the first call); no counterpart in
     * the reference */
    scalar maxEigenValue() const { return maxEigPCG_; }
};

}  // namespace UNAP

#endif
