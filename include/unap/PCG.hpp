/* UNAP::PCG (src/solvers/PCG/PCG.cpp:35-183): preconditioned conjugate
 * gradients on the GPU.
 * The solver keeps a non-owning pointer to its preconditioner, as the
 * reference does; its default is the identity. */
#ifndef PCG_HPP
#define PCG_HPP

#include "unapDevicePrecond.hpp"

namespace UNAP
{

class PCG : public matrix::solver
{
private:
    bool deletePrecondPtr_;
    matrix::preconditioner* precondPtr_;

public:
    PCG() : deletePrecondPtr_(true), precondPtr_(new matrix::preconditioner) {}

    explicit PCG(matrix::preconditioner& precond)
        : deletePrecondPtr_(false), precondPtr_(&precond)
    {
    }

    PCG(const PCG&) = delete;
    PCG& operator=(const PCG&) = delete;

    virtual ~PCG()
    {
        if (deletePrecondPtr_) delete precondPtr_;
        precondPtr_ = NULL;
    }

    virtual matrix::solverPerformance solve(scalarField& x, const matrix& A,
                                            const scalarField& b) const
    {
        return detail::run_krylov(0, "PCG", precondPtr_, x, A, b, tolerance_, relTol_,
                                  maxIter_, minIter_, ifPrint_);
    }

    void SET_preconditioner(matrix::preconditioner& precond)
    {
        if (deletePrecondPtr_) delete precondPtr_;
        deletePrecondPtr_ = false;
        precondPtr_ = &precond;
    }
};

}  // namespace UNAP

#endif
