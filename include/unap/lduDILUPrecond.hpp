/* UNAP::lduDILUPrecond (src/preconditioners/lduPreconditioners/lduDILU/lduDILUPrecond.cpp:15-86):
 * the incomplete-LU diagonal, the forward sweep in losort order and the backward sweep, computed on the GPU for the matrix it was built on. */
#ifndef LDUDILUPRECOND_HPP
#define LDUDILUPRECOND_HPP

#include "lduMatrix.hpp"

namespace UNAP
{

class lduDILUPrecond : public matrix::preconditioner
{
private:
    mutable scalarField rD_;
    const lduMatrix* APtr_;

public:
    static const int deviceType = 3;

    explicit lduDILUPrecond(const lduMatrix& A) : APtr_(&A) {}
    virtual ~lduDILUPrecond() {}

    static void calcReciprocalD(scalarField& rD, const lduMatrix& A)
    {
        rD.SET_size(A.size());
        detail::check(unap_cuda_precond_rD(A.deviceHandle(), deviceType, rD.values()),
                      "lduDILUPrecond::calcReciprocalD");
    }

    virtual void precondition(scalarField& w, const scalarField& r) const
    {
        detail::check(unap_cuda_precondition_host(APtr_->deviceHandle(), deviceType, r.values(),
                                                  w.values()),
                      "lduDILUPrecond::precondition");
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
