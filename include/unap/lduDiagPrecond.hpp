/* UNAP::lduDiagPrecond (src/preconditioners/lduPreconditioners/lduDiagonal/lduDiagPrecond.cpp:13-73):
 * rD = 1 / diag, w = rD r, computed on the GPU for the matrix it was built on. */
#ifndef LDUDIAGPRECOND_HPP
#define LDUDIAGPRECOND_HPP

#include "lduMatrix.hpp"

namespace UNAP
{

class lduDiagPrecond : public matrix::preconditioner
{
private:
    mutable scalarField rD_;
    const lduMatrix* APtr_;

public:
    static const int deviceType = 1;

    explicit lduDiagPrecond(const lduMatrix& A) : APtr_(&A) {}
    virtual ~lduDiagPrecond() {}

    static void calcReciprocalD(scalarField& rD, const lduMatrix& A)
    {
        rD.SET_size(A.size());
        detail::check(unap_cuda_precond_rD(A.deviceHandle(), deviceType, rD.values()),
                      "lduDiagPrecond::calcReciprocalD");
    }

    virtual void precondition(scalarField& w, const scalarField& r) const
    {
        detail::check(unap_cuda_precondition_host(APtr_->deviceHandle(), deviceType, r.values(),
                                                  w.values()),
                      "lduDiagPrecond::precondition");
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
