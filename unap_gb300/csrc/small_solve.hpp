// Single-CTA Krylov solves (small_solve.cu).
#pragma once

#include "kernels.hpp"

namespace unapgpu {

constexpr int kSmallBlock = 512;

// Launch shape of a fused solve: CTA size and CTAs per system.
struct TeamShape {
    int threads = kSmallBlock;
    int cluster = 1;
};

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

// A team of `cluster` CTAs (1, 2, 4, 8 or 16; a thread-block cluster when
// above 1) of `threads` threads (128, 256, 512 or 1024) per system; skipped
// when gate->done is set.
void launch_small_krylov(cudaStream_t s, const SmallSystem* d_systems, int count,
                         const KState* gate, int threads = kSmallBlock, int cluster = 1);

bool small_team_size_ok(int threads, int cluster);

// Teams of this shape resident at once on the current device (0: the shape
// cannot be launched there).
int small_team_capacity(int threads, int cluster);

}  // namespace unapgpu
