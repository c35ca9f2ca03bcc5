/* UNAP::lduGaussSeidelSmoother
 * (src/smoothers/lduSmoothers/lduGaussSeidelSmoother/lduGaussSeidelSmoother.cpp:3-80):
 * forward Gauss-Seidel sweeps in cell order, run on the GPU as wavefronts
 * that keep the reference's dependencies (same results). */
#ifndef LDUGAUSSSEIDELSMOOTHER_HPP
#define LDUGAUSSSEIDELSMOOTHER_HPP

#include "lduMatrix.hpp"

namespace UNAP
{

class lduGaussSeidelSmoother : public matrix::smoother
{
public:
    lduGaussSeidelSmoother() {}
    virtual ~lduGaussSeidelSmoother() {}

    virtual void smooth(scalarField& x, const matrix& A, const scalarField& b,
                        const label nSweeps) const
    {
        const lduMatrix* L = dynamic_cast<const lduMatrix*>(&A);
        if (!L) {
            std::cerr << "UNAP (GB300): lduGaussSeidelSmoother smooths lduMatrix systems"
                      << std::endl;
            ERROR_EXIT;
        }
        smooth(x, *L, b, nSweeps);
    }

    void smooth(scalarField& x, const lduMatrix& A, const scalarField& b,
                const label nSweeps) const
    {
        detail::check(unap_cuda_gauss_seidel_host(A.deviceHandle(), x.values(), b.values(),
                                                  detail::to_int(nSweeps, "nSweeps"), 0),
                      "lduGaussSeidelSmoother::smooth");
    }

    virtual void init() const {}
};

}  // namespace UNAP

#endif
