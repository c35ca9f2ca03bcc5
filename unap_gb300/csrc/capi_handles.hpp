// Objects behind the opaque `long int` handles of the C ABI.
#pragma once

#include <memory>

#include "engine.hpp"

namespace unapgpu {

// Matrix handle.  The reference's handle API creates the topology first
// (contruct_sw_matrix__) and fills coefficients later
// (fill_sw_matrix_coefficients__), so the device build is deferred until
// coefficients exist.
struct MatHandle {
    static constexpr unsigned kMagic = 0x554e4150u;  // "UNAP"
    unsigned magic = kMagic;
    HostLdu pending;
    bool hasValues = false;
    std::unique_ptr<Matrix> M;
    DevArray<double> s1, s2;  // scratch for single-kernel entry points
    Matrix& get();
    int n() const;
    void setValues(const double* diag, const double* upper, const double* lower);
    void ensureScratch()
    {
        size_t n_ = (size_t)get().n();
        if (s1.n != n_) s1.alloc(n_);
        if (s2.n != n_) s2.alloc(n_);
    }
    ~MatHandle() { magic = 0; }
};

// PBiCGStab solver handle (contruct_solver_pbicgstab__ and setters,
// fortranInterface.cpp:925-1060).  Defaults of matrix::solver
// (unapMatrixSolver.cpp:3-10): maxIter 1000, minIter 0, relTol 1e-6, tol 0.
struct BicgHandle {
    static constexpr unsigned kMagic = 0x42494347u;  // "BICG"
    unsigned magic = kMagic;
    int maxIter = 1000, minIter = 0;
    double tol = 0.0, relTol = 1e-6;
    int precondType = 0;  // identity until set_precond
    MatHandle* precondMat = nullptr;
    std::unique_ptr<Precond> P;
    const Matrix* precondFor = nullptr;
    int precondVersion = -1;
    ~BicgHandle() { magic = 0; }
};

MatHandle* mat_from(long int h);
HostLdu host_from_arrays(int n, int nf, const int* l, const int* u, const double* lower,
                         const double* diag, const double* upper);

}  // namespace unapgpu
