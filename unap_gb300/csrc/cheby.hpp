// Chebyshev smoothing (chebySmoother.cpp:44-148) and its largest-eigenvalue
// estimate (eigenDiagPCG.cpp:11-361) on the device, shared by the
// reference MGSolver (mg.cu) and the AMG V-cycle (amg.cu).
//
// A Chebyshev step is SpMV-shaped: every row reads the previous iterate of
// its neighbours and nothing else of the step, so a level is one launch per
// step (no wavefronts), with the iterate double-buffered.  Per row, in the
// reference's arithmetic order (A x as lduMatrix::spMV sums it, rD = 1/diag):
//   first step from x = 0:  w = rD b Rtheta;              x = w
//   first step from x:      w = rD (b - A x) Rtheta;      x = x + w
//   step j >= 1:            w = d1_j w + d2_j rD (b - A x); x = x + w
#pragma once

#include "kernels.hpp"

namespace unapgpu {

constexpr int kChebyMaxDegree = 16;

// Eigenvalue estimate state of one smoother (eigenDiagPCG.cpp:48-238:
// diagonal-PCG iterations recording alpha and beta).
struct EigState {
    double wArA, wArAold, wApA, alpha, beta;
    int broken, pad;
    double alphas[16], betas[16];
    double maxEig;
};

// eigenDiagPCG::diagPCGLoops: nIt (<= 16) diagonal-PCG iterations on
// (x, b), x updated in place.  es must hold wArA = GREAT and zeros on entry;
// a breakdown (|wArA| < VSMALL) sets es->broken and leaves the remaining
// alphas 0.  rA, wA, pA: n-vector scratch; wr and al: two reduction sites.
void eig_diag_pcg(const Exec& ex, const Rows<double>& A, const double* rD, double* x,
                  const double* b, double* rA, double* wA, double* pA, EigState* es,
                  const RSpec& wr, const RSpec& al, int nIt);

// eigenDiagPCG::computeMaxEig (eigenDiagPCG.cpp:242-361) on one device
// thread: es->maxEig = the largest eigenvalue of the Lanczos tridiagonal of
// the iterations done (nonzero alphas, at most nMax <= 16) by Sturm-sequence
// bisection to a band of 1e-5; 1 / alpha_0 after one iteration, 1 after none.
void k_eig_sturm(const Exec& ex, EigState* es, int nMax);

// Start vector of the AMG levels' eigenvalue estimate: cell c (reference
// numbering of its level) gets a uniform value in [-1, 1) from splitmix64.
void k_eig_start(const Exec& ex, int n, const int* perm, double* b);

// r[i] = 1 / d[i] (lduDiagPrecond.cpp:13-41)
void k_reciprocal(const Exec& ex, int n, const double* d, double* r);

// chebySmoother.cpp:62-108 for the interval [lam / ratio, 1.1 lam]:
// Rtheta of the first step and (d1[j], d2[j]) of steps j = 1 .. deg - 1.
void cheby_coeffs(double lam, double ratio, int deg, double* Rtheta, double* d1, double* d2);

// One Chebyshev step on every row of A: first != 0 is the first step from a
// nonzero x (c1 = Rtheta), else a later step (c1 = d1, c2 = d2).  xin and
// xout are distinct.  Launched with programmatic dependent launch when
// wave_pdl() is on: the kernel loads its rows' matrix data and b before it
// waits for the previous kernel.
template <class T>
void k_cheb_step(const Exec& ex, const Rows<T>& A, const T* xin, T* xout, const T* b, T* w, T c1,
                 T c2, int first, Gate g);
// First step from x = 0: w = x = rD b Rtheta.  With r64 != null (FP32
// levels entered from FP64) b is first set to (float)r64.
template <class T>
void k_cheb_zero(const Exec& ex, int n, const T* diag, T* b, const double* r64, T* x, T* w, T Rth,
                 Gate g);
// Restriction into a Chebyshev level fused with that level's first step:
// coarse[C] = sum of the children (ascending), then w = x = rD coarse Rtheta.
template <class T>
void k_restrict_cheb_zero(const Exec& ex, int nC, const int* childStart, const int* child,
                          const T* fine, T* coarse, const T* diagC, T* xC, T* wC, T Rth, Gate g);
// Out-of-place prolongation: xout[i] = xin[i] + coarse[cmap[i]].
template <class T>
void k_prolong_add_to(const Exec& ex, int n, const int* cmap, const T* coarse, const T* xin,
                      T* xout, Gate g);

// ---- the coarse end of a Chebyshev V-cycle in one cluster launch --------
constexpr int kChebTailMaxLevels = 8;

// one tail level: its matrix, the restriction into it (children of each
// cell, ascending), the prolongation out of it (cmap: finer row -> cell),
// its vectors (x, b, w = the residual buffer, the two buffers of the step
// chain: step j writes cb[j & 1], the post-smoothing chain starting from
// `post`) and Chebyshev coefficients
template <class T>
struct ChebTailLevel {
    Rows<T> A;
    const int* childStart;
    const int* child;
    const int* cmap;
    T* x;
    T* b;
    T* w;
    T* cb[2];
    T* post;
    T Rth;
    T d1[kChebyMaxDegree];
    T d2[kChebyMaxDegree];
};

template <class T>
struct ChebTailArgs {
    ChebTailLevel<T> lev[kChebTailMaxLevels];  // first tail level .. coarsest - 1
    int nLev;
    int deg;
    int nc;                   // coarsest level
    const int* cChildStart;   // restriction into it
    const int* cChild;
    const int* cCmap;         // prolongation out of it
    T* cb;
    T* cx;
    const double* Minv;       // dense inverse, column-major
    double* part;             // nc x ceil(nc / 64) chunk sums (scratch)
};

// One launch of a thread-block cluster (16 CTAs of 512 threads, else 8)
// runs the V-cycle from a.lev[0] (its b, first iterate and w already set by
// the fused restriction) down to the coarsest and back, bit-identical to the
// per-step kernels.
template <class T>
void launch_cheb_tail(const Exec& ex, const ChebTailArgs<T>& a, Gate g);
// Chebyshev V-cycles run their levels of at most `rows` rows (and every
// level below them) in the tail launch; 0 turns it off.  Returns the
// previous value; applies to hierarchies built afterwards.
int set_cheby_tail_rows(int rows);
int cheby_tail_rows();
// cluster size the tail launches with on this device (0: none schedulable)
int cheby_tail_cluster();

// Rows per level below which Chebyshev-step launches use one-warp CTAs
// (spread over more SMs); returns the previous value.
int set_cheby_small_rows(int rows);
// Entries of a row loaded per dependent round trip by the Chebyshev step: 0
// (default) 16 on levels averaging more than 8 entries per row, except FP32
// levels of a million rows or more (8: more CTAs per SM), else 8; 8 or 16
// on every level.  Returns the previous value.
int set_cheby_chunk(int entries);

}  // namespace unapgpu
