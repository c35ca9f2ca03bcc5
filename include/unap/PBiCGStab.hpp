/* UNAP::PBiCGStab (src/solvers/PBiCGStab/PBiCGStab.cpp:45-459): preconditioned
 * BiCGStab on the GPU.
 * The solver keeps a non-owning pointer to its preconditioner, as the
 * reference does; its default is the identity. */
#ifndef PBICGSTAB_HPP
#define PBICGSTAB_HPP

#include "unapDevicePrecond.hpp"

namespace UNAP
{

class PBiCGStab : public matrix::solver
{
private:
    bool deletePrecondPtr_;
    matrix::preconditioner* precondPtr_;

public:
    PBiCGStab() : deletePrecondPtr_(true), precondPtr_(new matrix::preconditioner) {}

    explicit PBiCGStab(matrix::preconditioner& precond)
        : deletePrecondPtr_(false), precondPtr_(&precond)
    {
    }

    PBiCGStab(const PBiCGStab&) = delete;
    PBiCGStab& operator=(const PBiCGStab&) = delete;

    virtual ~PBiCGStab()
    {
        if (deletePrecondPtr_) delete precondPtr_;
        precondPtr_ = NULL;
    }

    virtual matrix::solverPerformance solve(scalarField& x, const matrix& A,
                                            const scalarField& b) const
    {
        return detail::run_krylov(1, "PBiCGStab", precondPtr_, x, A, b, tolerance_, relTol_,
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
