/*
 * unap_oracle -- CPU restatement of UNAP's solve hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker for the CUDA library, and
 * the "port" CPU baseline that bench.py times beside it.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU legs load it.  The product
 * (unap_gb300/) never links, loads or calls it.
 *
 * Every function restates a reference function (file:line given at each
 * definition) in plain C with the reference's exact loop orders, so that
 * a kernel that keeps the same per-row summation order is bit-identical to
 * it.  Functions marked NEW have no counterpart in the reference (AMG as a
 * PCG preconditioner, backward Gauss-Seidel, dense coarsest solve, FP32
 * V-cycle); their semantics are defined here and in the CUDA library alike.
 *
 * Conventions: 0-based int32 addressing, FP64 values, `symm` != 0 means the
 * lower coefficients are the upper ones (the reference's lowerPtr_ ==
 * upperPtr_, lduMatrix.hpp:210-220) and `lower` may be NULL.
 */
#ifndef UNAP_ORACLE_H
#define UNAP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- matrix kernels -------------------------------------------------- */
void orc_spmv(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
              const double* up, int symm, const double* x, double* y);
void orc_losort(int n, int nf, const int* l, const int* u, int* losort, int* ownerStart,
                int* losortStart);
void orc_precond(int type, int n, int nf, const int* l, const int* u, const double* lo,
                 const double* d, const double* up, int symm, const double* r, double* w,
                 double* rD);
void orc_gs(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
            const double* up, int symm, double* x, const double* b, int nSweeps);
void orc_gs_bwd(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
                const double* up, int symm, double* x, const double* b, int nSweeps);
double orc_eigen(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
                 const double* up, int symm, double* x, const double* b, int nDiagPCGs);
void orc_cheby(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
               const double* up, int symm, double* x, const double* b, int nSweeps, int nCalls);

/* ---- Krylov solvers -------------------------------------------------- */
void orc_pcg(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
             const double* up, int symm, int precond, double tol, double relTol, int maxIter,
             int minIter, double* x, const double* b, int* nIter, double* initRes,
             double* finalRes, int* converged, int* singular);
void orc_pbicgstab(int n, int nf, const int* l, const int* u, const double* lo,
                   const double* d, const double* up, int symm, int precond, double tol,
                   double relTol, int maxIter, int minIter, double* x, const double* b,
                   int* nIter, double* initRes, double* finalRes, int* converged,
                   int* singular);

/* ---- agglomeration hierarchy ----------------------------------------- */
/* stopRule 0: the reference's rule (keep a level while it has >= nCoarsest
 * cells).  stopRule 1 (NEW): keep agglomerating while the coarsest kept level
 * has more than nCoarsest cells, so the coarsest ends <= nCoarsest. */
void* orc_hier_create(int n, int nf, const int* l, const int* u, const double* lo,
                      const double* d, const double* up, int symm, const double* weights,
                      int nCoarsest, int maxLevels, int stopRule);
int orc_hier_nlevels(void* h);
int orc_hier_ncells(void* h, int level);
int orc_hier_nfaces(void* h, int level);
void orc_hier_addressing(void* h, int level, int* restrictAddr, int* faceRestrict,
                         int* coarseLower, int* coarseUpper);
void orc_hier_coeffs(void* h, int level, double* diag, double* upper, double* lower);
void orc_hier_destroy(void* h);
void orc_mg_weights(int nf, const double* up, double* weights);

/* ---- MGSolver (reference V-cycle iteration) -------------------------- */
void orc_mg(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
            const double* up, int symm, const double* weights, int nCoarsest, int maxLevels,
            int smootherType, int nPre, int nPost, int nFinest, int scaleCorr, double tol,
            double relTol, int maxIter, int minIter, double* x, const double* b, int* nIter,
            double* initRes, double* finalRes, int* converged, int* nLevels);

/* ---- NEW: AMG as a fixed symmetric PCG preconditioner ---------------- */
typedef struct {
    int nCoarsest;     /* coarsest level has at most this many cells (stopRule 1) */
    int maxLevels;     /* reference default 50 */
    int nPre, nPost;   /* forward GS sweeps before, backward GS sweeps after */
    int precision;     /* 0: FP64 V-cycle, 1: FP32 V-cycle (coarsest solve FP64) */
    int flexible;      /* 1: Polak-Ribiere beta (flexible PCG) */
    double tol, relTol;
    int maxIter, minIter;
    /* smoother 0: Gauss-Seidel (nPre forward / nPost backward sweeps);
     * smoother 1: Chebyshev of degree chebyDegree before and after the
     * coarse correction on levels >= chebyFrom (Gauss-Seidel below), over
     * [lambda / eigRatio, 1.1 lambda] (chebySmoother.cpp:44-148) with lambda
     * the level's diagonal-PCG estimate (eigenDiagPCG.cpp:11-361) taken once
     * at setup from x = 0 and the start vector orc_eig_start.  eigRatio <= 0
     * means the reference's 1.5. */
    int smoother, chebyDegree, chebyFrom;
    double eigRatio;
} orc_amg_params;

void* orc_amg_create(int n, int nf, const int* l, const int* u, const double* d,
                     const double* up, const orc_amg_params* p);
int orc_amg_nlevels(void* h);
int orc_amg_ncells(void* h, int level);
/* one V-cycle application z = M^-1 r (level 0 = the input matrix) */
void orc_amg_vcycle(void* h, const double* r, double* z);
/* AMG-PCG solve; returns the recurrence residual like PCG.cpp and the true
 * residual ||b - A x|| computed afterwards. */
void orc_amg_pcg(void* h, double* x, const double* b, int* nIter, double* initRes,
                 double* finalRes, double* trueRes, int* converged);
/* dense inverse of the coarsest matrix, row-major n x n (FP64) */
void orc_amg_coarse_inverse(void* h, double* inv);
void orc_amg_destroy(void* h);
void orc_amg_set_max_iter(void* h, int maxIter);
/* per-level largest-eigenvalue estimates of D^-1 A used by the Chebyshev
 * smoother (levels 0..nLevels-2; 0 where the level uses Gauss-Seidel);
 * set_eigs replaces them (a test feeds the device's estimates back so the
 * two V-cycles can be compared bit for bit) */
void orc_amg_eigs(void* h, double* lam);
void orc_amg_set_eigs(void* h, const double* lam);
/* the AMG levels' Chebyshev chain of `degree` steps on one matrix (FP64),
 * in place on x: fromZero 1 starts from x = 0 (x's input ignored) */
void orc_cheby_chain(int n, int nf, const int* l, const int* u, const double* lo,
                     const double* d, const double* up, int symm, double lam, double ratio,
                     int degree, double* x, const double* b, int fromZero);
/* start vector of the eigenvalue estimate: value of cell c (reference
 * numbering of its level), uniform in [-1, 1) from splitmix64(c) */
double orc_eig_start(long long c);

/* Cholesky-based inverse of a dense SPD matrix (row-major), as used for the
 * coarsest level.  Returns 0 on success, -1 when not positive definite. */
int orc_dense_spd_inverse(int n, const double* A, double* inv);

#ifdef __cplusplus
}
#endif

#endif
