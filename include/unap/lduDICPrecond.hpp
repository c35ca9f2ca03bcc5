/* UNAP::lduDICPrecond (src/preconditioners/lduPreconditioners/lduDIC/lduDICPrecond.cpp:15-77):
 * the incomplete-Cholesky diagonal and its forward and backward sweeps, computed on the GPU for the matrix it was built on. */
#ifndef LDUDICPRECOND_HPP
#define LDUDICPRECOND_HPP

#include "lduMatrix.hpp"

namespace UNAP
{

class lduDICPrecond : public matrix::preconditioner
{
private:
    mutable scalarField rD_;
    const lduMatrix* APtr_;

public:
    static const int deviceType = 2;

    explicit lduDICPrecond(const lduMatrix& A) : APtr_(&A) {}
    virtual ~lduDICPrecond() {}

    static void calcReciprocalD(scalarField& rD, const lduMatrix& A)
    {
        rD.SET_size(A.size());
        detail::check(unap_cuda_precond_rD(A.deviceHandle(), deviceType, rD.values()),
                      "lduDICPrecond::calcReciprocalD");
    }

    virtual void precondition(scalarField& w, const scalarField& r) const
    {
        detail::check(unap_cuda_precondition_host(APtr_->deviceHandle(), deviceType, r.values(),
                                                  w.values()),
                      "lduDICPrecond::precondition");
    }

    virtual const scalarField& rD() const
    {
        calcReciprocalD(rD_, *APtr_);
        return rD_;
    }

    /* the matrix this preconditioner belongs to */
    const lduMatrix& matrixRef() const { return *APtr_; }
};

}  // namespace UNAP

#endif
