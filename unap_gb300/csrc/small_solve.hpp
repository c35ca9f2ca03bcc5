// Single-CTA Krylov solves (small_solve.cu).
#pragma once

#include "kernels.hpp"

namespace unapgpu {

constexpr int kSmallBlock = 512;

struct SmallResult {
    int nIter, converged, singular, pad;
    double initRes, finalRes;
};

struct SmallSystem {
    Rows<double> A;             // internal order, SELL rows
    const int* waveStart;       // device, nWave + 1
    int nWave;
    const double* rD;           // 1/D (Diag) or factored reciprocal (DIC/DILU)
    int method;                 // 0 PCG, 1 PBiCGStab
    int precond;                // 0 none, 1 Diag, 2 DIC, 3 DILU
    double tol, relTol;
    int maxIter, minIter;
    int zeroX;                  // start from x = 0
    double* x;
    const double* b;
    double* work;               // 8 n doubles
    SmallResult* result;        // may be null
};

// One block of `threads` (128, 256, 512 or 1024) per system; skipped when
// gate->done is set.
void launch_small_krylov(cudaStream_t s, const SmallSystem* d_systems, int count,
                         const KState* gate, int threads = kSmallBlock);

}  // namespace unapgpu
