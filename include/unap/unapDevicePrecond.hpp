/* Which preconditioner a Krylov solve runs on the GPU (no counterpart in the
 * reference, whose solvers call precondition() on the host every
 * iteration): the identity base class, lduDiagPrecond, lduDICPrecond or
 * lduDILUPrecond, built on the matrix being solved.  Any other
 * preconditioner would need a host call per iteration, which this library
 * does not make: it is an error. */
#ifndef UNAPDEVICEPRECOND_HPP
#define UNAPDEVICEPRECOND_HPP

#include <typeinfo>

#include "lduDICPrecond.hpp"
#include "lduDILUPrecond.hpp"
#include "lduDiagPrecond.hpp"

namespace UNAP
{
namespace detail
{

template <class P>
inline int device_type_of(const matrix::preconditioner* p, const lduMatrix& A)
{
    const P* q = dynamic_cast<const P*>(p);
    if (!q) return -1;
    if (&q->matrixRef() != &A) {
        std::cerr << "UNAP (GB300): the preconditioner must be built on the matrix being solved"
                  << std::endl;
        ERROR_EXIT;
    }
    return P::deviceType;
}

inline int precond_code(const matrix::preconditioner* p, const lduMatrix& A)
{
    if (!p || typeid(*p) == typeid(matrix::preconditioner)) return 0;
    int t = device_type_of<lduDiagPrecond>(p, A);
    if (t < 0) t = device_type_of<lduDICPrecond>(p, A);
    if (t < 0) t = device_type_of<lduDILUPrecond>(p, A);
    if (t < 0) {
        std::cerr << "UNAP (GB300): preconditioner " << typeid(*p).name()
                  << " has no GPU form (lduDiagPrecond, lduDICPrecond or lduDILUPrecond)"
                  << std::endl;
        ERROR_EXIT;
    }
    return t;
}

inline const lduMatrix& as_ldu(const matrix& A, const char* who)
{
    const lduMatrix* L = dynamic_cast<const lduMatrix*>(&A);
    if (!L) {
        std::cerr << "UNAP (GB300): " << who << " solves lduMatrix systems" << std::endl;
        ERROR_EXIT;
    }
    return *L;
}

inline void check_sizes(const lduMatrix& A, const scalarField& x, const scalarField& b)
{
    if (x.size() != A.size() || b.size() != A.size()) {
        std::cerr << "UNAP (GB300): x and b must have nCells entries" << std::endl;
        ERROR_EXIT;
    }
}

inline matrix::solverPerformance run_krylov(int method, const char* who,
                                            const matrix::preconditioner* p, scalarField& x,
                                            const matrix& A, const scalarField& b, scalar tol,
                                            scalar relTol, label maxIter, label minIter,
                                            bool print)
{
    const lduMatrix& L = as_ldu(A, who);
    check_sizes(L, x, b);
    const int pc = precond_code(p, L);
    unap_cuda_stats st;
    check(unap_cuda_krylov_solve_host(L.deviceHandle(), method, pc, tol, relTol,
                                      to_int(maxIter, "maxIter"), to_int(minIter, "minIter"),
                                      x.values(), b.values(), &st),
          who);
    if (print)
        COUT << who << ": " << st.nIterations << " iterations, residual " << st.initialResidual
             << " -> " << st.finalResidual << ENDL;
    return matrix::solverPerformance(st.initialResidual, st.finalResidual, st.nIterations,
                                     st.converged != 0, st.singular != 0);
}

}  // namespace detail
}  // namespace UNAP

#endif
