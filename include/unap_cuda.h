/*
 * unap_cuda.h -- C ABI of the GB300 UNAP solve library (libunap_cuda.so).
 *
 * Part 1 re-exports the reference's Fortran-callable interface with the same
 * symbol names, argument order and meaning, so a Fortran/C caller of
 * UNAP's src/tools/cInterface/fortranInterface.h relinks against this library
 * unchanged.  Conventions kept from the reference:
 *   - every argument is passed by pointer; labels are 32-bit `int`
 *     (the C header fortranInterface.h:8-102 uses int*);
 *   - handles are C pointers stored in a `long int` the caller owns;
 *   - one-shot solves (pcgsolversolve_, pbicgstabsolversolve_,
 *     mgsolversolve_) copy x/b in and out and DELETE the matrix handle they
 *     were given (fortranInterface.cpp:267,345,463);
 *   - preconditioner codes 1 Diag, 2 DIC, 3 DILU, anything else none;
 *     smoother codes 1 Gauss-Seidel, 2 Chebyshev;
 *   - a matrix is symmetric iff the `lower` and `upper` pointers are equal.
 * Differences, all documented at the declaration:
 *   - ldumatrixcreat_ builds an asymmetric matrix from separate lower/upper
 *     arrays (the reference overwrites upper with lower,
 *     fortranInterface.cpp:51-58);
 *   - errors do not exit(): the solve reports num_iterations = -1 and
 *     final_res_norm = NaN and the message is kept for unap_cuda_last_error().
 *   - processor interfaces (MPI halos) are accepted and ignored: one GPU is
 *     one rank, and the reference ignores interfaces on a single rank
 *     (lduMatrix.cpp:488-503, PARRUN false).
 *
 * Part 2 adds unap_cuda_* entry points that have no counterpart in the
 * reference: device-pointer solves and kernels, AMG-PCG in FP64 and mixed
 * precision, batched and served solves.  They return 0 on success and a
 * negative code on error.  A call on device vectors runs after all work the
 * caller issued before it to the legacy default stream (or any blocking
 * stream), e.g. the fill of an initial guess, and returns when its results
 * are in place.
 */
#ifndef UNAP_CUDA_H
#define UNAP_CUDA_H

#ifdef __cplusplus
extern "C" {
#endif

/* ===================================================================== */
/* Part 1: the reference's Fortran-convention interface                  */
/* ===================================================================== */

/* fortranInterface.h:8-18 / fortranInterface.cpp:31-71.
 * 0-based addresses; faces should be oriented lowerAddr < upperAddr and sorted
 * by owner for DIC/DILU/Gauss-Seidel (SpMV accepts any order). */
void ldumatrixcreat_(long int* APtrPtr, int* nCells, int* upperSize, int* lowerAddr,
                     int* upperAddr, double* lower, double* diag, double* upper);

/* fortranInterface.h:20-29 / fortranInterface.cpp:74-120.  1-based COO rows
 * and columns, rows sorted; the structure must be symmetric.  symm != 0 means
 * the values are symmetric. */
void coo2ldumatrixcreat_(long int* APtrPtr, const double* dataPtr, const int* rowsPtr,
                         const int* columnPtr, const int* nCells, const int* size,
                         const int* symm);

/* fortranInterface.h:32-41 / fortranInterface.cpp:123-146.  Compressed rows
 * with sorted columns; like the reference (which calls csr2ldu on the
 * caller's arrays directly) the row pointer and columns are used as given. */
void csr2ldumatrixcreat_(long int* APtrPtr, const double* dataPtr, const int* compRowsPtr,
                         const int* columnPtr, const int* nCells, const int* size,
                         const int* symm);

/* fortranInterface.h:44-52 / fortranInterface.cpp:149-197.  Accepted and
 * ignored on one GPU (single-rank semantics of the reference). */
void matrixinterfacescreat_(long int* APtrPtr, const int* nNeiProcs, const int* destRank,
                            const int* locPosition, const int* faceCells, const double* data);

/* fortranInterface.h:55-68 / fortranInterface.cpp:200-268.  Deletes *APtrPtr. */
void pcgsolversolve_(double* x, long int* APtrPtr, double* b, int* nCells, int* precond,
                     double* tol, double* relTol, int* maxIter, int* minIter,
                     int* num_iterations, double* final_res_norm);

/* fortranInterface.h:71-84 / fortranInterface.cpp:271-346.  Deletes *APtrPtr. */
void pbicgstabsolversolve_(double* x, long int* APtrPtr, double* b, int* nCells, int* precond,
                           double* tol, double* relTol, int* maxIter, int* minIter,
                           int* num_iterations, double* final_res_norm);

/* fortranInterface.h:87-102 / fortranInterface.cpp:349-464.  aggl 1 weights
 * |upper|/||upper||, 2 faceAreaPtr; smoother 1 GS, 2 Cheby; the reference's
 * MGSolver defaults with nPreSweeps 0.  Deletes *APtrPtr. */
void mgsolversolve_(double* x, long int* APtrPtr, double* b, int* nCells, int* aggl,
                    int* smoother, double* tol, double* relTol, int* maxIter, int* minIter,
                    int* num_iterations, double* final_res_norm, double* faceAreaPtr);

/* Handle API, fortranInterface.hpp:173-331 / fortranInterface.cpp:537-1102.
 * contruct_solver_mg__ builds the hierarchy at once (maxLevels, coarsest
 * threshold as given); *AgglPtr receives a value identifying it (the
 * hierarchy is owned by the MG handle).  sw_solve_mg__ resets the Chebyshev
 * eigenvalue estimates (initSmoothers) before every solve, as the
 * reference does; the hierarchy is rebuilt when the matrix coefficients
 * changed since it was made. */
void contruct_solver_mg__(long int* mgPtrPtr, long int* APtrPtr, long int* AgglPtr,
                          const double* weightsPtr, const int* smootherTypePtr,
                          const int* maxLevelsPtr, const int* nCellsCoarsestPtr);
void sw_solver_mg_set_maxiter__(long int* solverPtrPtr, const int* maxIterPtr);
void sw_solver_mg_set_miniter__(long int* solverPtrPtr, const int* minIterPtr);
void sw_solver_mg_set_tol__(long int* solverPtrPtr, const double* tolPtr);
void sw_solver_mg_set_reltol__(long int* solverPtrPtr, const double* reltolPtr);
void sw_solver_mg_set_npresweeps__(long int* solverPtrPtr, const int* numPtr);
void sw_solver_mg_set_npostsweeps__(long int* solverPtrPtr, const int* numPtr);
void sw_solver_mg_set_nfinestsweeps__(long int* solverPtrPtr, const int* numPtr);
void sw_solve_mg__(long int* mgPtrPtr, long int* APtrPtr, double* xPtr, double* bPtr,
                   double* res_normPtr);
void sw_solver_destroy_mg__(long int* solverPtrPtr);

/* Handle API (PBiCGStab and matrices) */
void contruct_sw_matrix__(long int* APtrPtr, const int* nCellsPtr, const int* rowsPtr,
                          const int* colsPtr, const int* sizePtr);
void contruct_sw_matrix_interfaces__(long int* APtrPtr, const int* nNeiProcsPtr,
                                     const int* destRankPtr, const int* offDiagRowsPtr,
                                     const int* offDiagStartsPtr);
void fill_sw_matrix_coefficients__(long int* APtrPtr, const double* diagPtr,
                                   const double* upperPtr, const double* lowerPtr);
void fill_sw_matrix_interfaces_coefficients__(long int* APtrPtr, const int* offDiagStartsPtr,
                                              const double* offDiagCoeffs);
void contruct_solver_pbicgstab__(long int* solverPtrPtr);
void sw_solver_pbicgstab_set_maxiter__(long int* solverPtrPtr, const int* maxIterPtr);
void sw_solver_pbicgstab_set_miniter__(long int* solverPtrPtr, const int* minIterPtr);
void sw_solver_pbicgstab_set_tol__(long int* solverPtrPtr, const double* tolPtr);
void sw_solver_pbicgstab_set_reltol__(long int* solverPtrPtr, const double* reltolPtr);
void sw_solver_pbicgstab_set_precond__(long int* solverPtrPtr, long int* APtrPtr,
                                       const int* precondTypePtr);
void sw_solve_pbicgstab__(long int* solverPtrPtr, long int* APtrPtr, double* xPtr,
                          double* bPtr, double* res_normPtr);
void sw_matrix_destroy__(long int* APtrPtr);
void sw_solver_destroy_pbicgstab__(long int* solverPtrPtr);

/* COO / face reordering (fortranInterface.hpp:110-145, defined in
 * fortranInterface.cpp:467-534 over matrixConversion.cpp:38-222), 1-based
 * row and column indices on entry, 0-based on return.  reordercoo_ groups
 * the entries by row and orders each row by column, moving the values with
 * them (it shifts to 0-based only when row[0] != 0, as the reference does);
 * reorderuface__ does the same to the indices alone and returns each
 * entry's new position in newOrder (0-based); reorderlface__ groups them by
 * column, stable in input order, with newOrder likewise; reordervalue__
 * moves val[i] to val[newOrder[i]].  Input the reference leaves undefined
 * (an index out of range, a repeated (row, column) pair, a newOrder that is
 * not a permutation) leaves the arrays unchanged and prints the error. */
void reordercoo_(double* val, int* row, int* col, int* nCellsPtr, int* sizePtr);
void reorderuface__(int* row, int* col, int* nCellsPtr, int* sizePtr, int* newOrder);
void reorderlface__(int* row, int* col, int* nCellsPtr, int* sizePtr, int* newOrder);
void reordervalue__(double* val, int* newOrder, int* sizePtr);

/* ===================================================================== */
/* Part 2: GB300 entry points (no counterpart in the reference)          */
/* ===================================================================== */

typedef struct {
    int nIterations;
    int converged;
    int singular;
    int status; /* 0 ok */
    double initialResidual;
    double finalResidual;
    double trueResidual; /* ||b - A x|| + 1e-37 when computed, else -1 */
    double seconds;      /* device time of the solve */
    double algorithmicBytes; /* DRAM bytes the solve must move (persistent
                              * executor; 0 otherwise), for roofline use */
} unap_cuda_stats;

#define UNAP_CUDA_OK 0
#define UNAP_CUDA_EINVAL (-1)
#define UNAP_CUDA_ECUDA (-2)
#define UNAP_CUDA_ENOMEM (-3)
#define UNAP_CUDA_EINTERNAL (-4)

/* text of the last error on this thread */
const char* unap_cuda_last_error(void);
/* library version string */
const char* unap_cuda_version(void);

/* Matrix from host LDU arrays (copied).  lower == NULL or lower == upper
 * makes it symmetric.  *handle receives an opaque handle. */
int unap_cuda_matrix_create(long int* handle, int nCells, int nFaces, const int* lowerAddr,
                            const int* upperAddr, const double* lower, const double* diag,
                            const double* upper);
int unap_cuda_matrix_destroy(long int handle);
/* Replace a matrix's coefficients, keeping its addressing and its symmetry
 * (lower NULL or == upper for a symmetric matrix). */
int unap_cuda_matrix_set_values(long int handle, const double* diag, const double* upper,
                                const double* lower);
/* Sizes and host copy of a handle's LDU arrays (any handle from Part 1 or
 * Part 2; no GPU work).  lower receives upper's values when symmetric. */
int unap_cuda_matrix_size(long int handle, int* nCells, int* nFaces, int* symm);
int unap_cuda_matrix_get_ldu(long int handle, int* lowerAddr, int* upperAddr, double* lower,
                             double* diag, double* upper);
/* structure facts: forward wavefronts, padded SELL entries, device bytes */
int unap_cuda_matrix_info(long int handle, int* nWavefronts, long long* nEntries,
                          long long* deviceBytes);

/* Internal cell order of a matrix: *nWavefronts forward wavefronts;
 * perm[i] (nCells entries) is the cell stored at internal row i and
 * waveStart (nWavefronts + 1 entries) the wavefront boundaries.  Builds the
 * matrix on the device if it is not built yet.  No reference counterpart. */
int unap_cuda_matrix_layout(long int handle, int* nWavefronts, int* perm, int* waveStart);
/* Matrices (and AMG levels) of at least minCells cells build their device
 * structure (internal order, SELL-32 layout, values) with kernels instead
 * of host loops; minCells < 0 builds every one on the host.  Both give the
 * same structure bit for bit.  Default 32768; the previous value is
 * returned through the (nullable) pointer.  No reference counterpart. */
int unap_cuda_set_device_setup(long long minCells, long long* oldMinCells);

/* Kernels on device vectors in the caller's cell order (FP64). */
int unap_cuda_spmv(long int handle, const double* x, double* y);
/* y = A x like unap_cuda_spmv, for callers that cannot allocate device memory
 * at call time (a time-stepping code that reserved its whole device-memory
 * budget up front, or a host thread that must not take the CUDA allocator's
 * locks).  No counterpart in the reference.  It calls no cudaMalloc/cudaFree:
 * its scratch is a static device array of 2 x 1,048,576 doubles (16 MiB,
 * held by every GPU that loads the library until exit), so matrices above
 * 1,048,576 cells are rejected (UNAP_CUDA_EINVAL).  The handle must already
 * be built on the device.  The call runs on the device the matrix was built
 * on (whichever device is current) and is synchronous: it returns when its
 * kernels have finished, so it must not be called while a stream capture is
 * active on the calling thread.  Its first call on a device looks up the
 * array's device address.  All calls share the array: calls whose work
 * overlaps on the GPU race; calls on one stream are safe. */
int unap_cuda_spmv_noalloc(long int handle, const double* x, double* y);
/* w = M^-1 r, precond 1 Diag, 2 DIC, 3 DILU */
int unap_cuda_precondition(long int handle, int precond, const double* r, double* w);

/* The same calls on HOST vectors in the caller's cell order: each copies its
 * vectors to the device, runs the kernels there and copies the result back
 * (the layer under the C++ class API, include/unap/).  No counterpart in the
 * reference, which works on host vectors throughout. */
int unap_cuda_spmv_host(long int handle, const double* x, double* y);
int unap_cuda_precondition_host(long int handle, int precond, const double* r, double* w);
/* rD of lduDiagPrecond (1), lduDICPrecond (2) or lduDILUPrecond (3) in cell
 * order (lduDiagPrecond.cpp:13-41, lduDICPrecond.cpp:15-42,
 * lduDILUPrecond.cpp:15-43), computed on the device */
int unap_cuda_precond_rD(long int handle, int precond, double* rD);
int unap_cuda_gauss_seidel_host(long int handle, double* x, const double* b, int nSweeps,
                                int backward);
/* chebySmoother::smooth (chebySmoother.cpp:13-149) with its state held by
 * the caller: while *estimated is 0 the call estimates the largest
 * eigenvalue with 10 diagonal-PCG iterations on (x, b), leaving x as they
 * change it, stores it in *maxEig and sets *estimated; later calls run
 * nSweeps (<= 16) Chebyshev steps over [maxEig / 1.5, 1.1 maxEig]. */
int unap_cuda_cheby_smooth_host(long int handle, double* x, const double* b, int nSweeps,
                                double* maxEig, int* estimated);
int unap_cuda_krylov_solve_host(long int handle, int method, int precond, double tol,
                                double relTol, int maxIter, int minIter, double* x,
                                const double* b, unap_cuda_stats* stats);

/* 0-based forms of the reordering calls above (matrixConversion.cpp:38-222);
 * they return UNAP_CUDA_EINVAL on the inputs listed there. */
int unap_cuda_reorder_coo(double* val, int* row, int* col, int nCells, int size);
int unap_cuda_reorder_uface(int* row, int* col, int nCells, int size, int* newOrder);
int unap_cuda_reorder_lface(int* row, int* col, int nCells, int size, int* newOrder);
int unap_cuda_reorder_value(double* val, const int* newOrder, int size);

/* Pairwise agglomeration of a matrix (lduAgglomeration::agglomerate,
 * lduAgglomerate.cpp:4-271 with lduAgglomerationAddressing.cpp:8-178 and
 * lduAgglomerateMatrix.cpp:3-131): face weights as given (the C++ API's
 * agglomerate(weights)), levels kept while they have at least
 * nCellsInCoarsestLevel cells, at most maxLevels.  _level copies level k's
 * arrays (any pointer may be NULL): restrictAddr (finer cells -> cells of
 * level k), faceRestrict (finer faces -> coarse face or -(cell + 1)), and
 * the level's LDU matrix. */
int unap_cuda_agglomeration_create(long int* aggl, long int matrix, const double* weights,
                                   int nCellsInCoarsestLevel, int maxLevels);
int unap_cuda_agglomeration_size(long int aggl, int* nLevels);
int unap_cuda_agglomeration_level(long int aggl, int level, int* nCells, int* nFaces, int* symm,
                                  int* restrictAddr, int* faceRestrict, int* lowerAddr,
                                  int* upperAddr, double* diag, double* upper, double* lower);
int unap_cuda_agglomeration_destroy(long int aggl);
/* nSweeps Gauss-Seidel sweeps in place on x; backward != 0 sweeps in reverse
 * cell order (no reference counterpart) */
int unap_cuda_gauss_seidel(long int handle, double* x, const double* b, int nSweeps,
                           int backward);

/* PCG (method 0) or PBiCGStab (method 1) with an LDU preconditioner
 * (precond 0 none, 1 Diag, 2 DIC, 3 DILU; other codes return
 * UNAP_CUDA_EINVAL, unlike the Fortran-convention calls, which fall back to
 * none as the reference does) on device vectors; x holds the initial guess
 * on entry. */
int unap_cuda_krylov_solve(long int handle, int method, int precond, double tol, double relTol,
                           int maxIter, int minIter, double* x, const double* b,
                           unap_cuda_stats* stats);

/* ---- AMG-preconditioned PCG (no counterpart in the reference: its
 * MGPrecond, src/preconditioners/MGPreconditioner/MGPreconditioner.cpp:35-42,
 * is an empty stub).  The hierarchy is the reference's pairwise
 * agglomeration (weights |upper|/||upper||, fortranInterface.cpp:383-395),
 * continued until the coarsest level has at most nCoarsest cells; the
 * V-cycle is x = 0, nPreSweeps forward Gauss-Seidel sweeps, restriction of
 * b - A x, recursion, injection, nPostSweeps backward sweeps; the coarsest
 * level is solved with a dense FP64 Cholesky-based inverse.  precision 1
 * runs the whole V-cycle in FP32 inside the FP64 PCG (true residual, dot
 * products, norms and the coarsest product stay FP64).
 *
 * smoother 1 smooths the levels from chebyFrom down (Gauss-Seidel above)
 * with the reference's Chebyshev iteration (chebySmoother.cpp:44-148) of
 * degree chebyDegree before and after the coarse correction, over
 * [lambda / eigRatio, 1.1 lambda]; lambda is the reference's
 * diagonal-PCG + Lanczos estimate (eigenDiagPCG.cpp:11-361) of each level's
 * largest eigenvalue of D^-1 A, taken once at setup from x = 0 (the
 * reference's smoother estimates on its first call and leaves x changed by
 * it, which a fixed PCG preconditioner cannot do).  eigRatio <= 0 selects
 * the reference's 1.5. */
typedef struct {
    int nCoarsest;   /* default 1000 */
    int maxLevels;   /* default 50 */
    int nPreSweeps;  /* default 2 (Gauss-Seidel levels) */
    int nPostSweeps; /* default 2 (Gauss-Seidel levels) */
    int precision;   /* 0 FP64 V-cycle, 1 FP32 V-cycle */
    int flexible;    /* 1: Polak-Ribiere beta (default 1 when precision 1) */
    double tol;      /* default 0 */
    double relTol;   /* default 1e-10 */
    int maxIter;     /* default 500 */
    int minIter;     /* default 0 */
    int smoother;    /* 0 Gauss-Seidel (default), 1 Chebyshev */
    int chebyDegree; /* default 3 (1..16) */
    int chebyFrom;   /* first Chebyshev level, default 0 (all) */
    double eigRatio; /* default 30 */
    int fusedOuter;  /* 1 (default): with an FP32 V-cycle, the outer PCG's
                        SpMV, dots and updates use fused multiply-adds (half
                        the FP64 instructions; GB300's FP64 pipe bounds them);
                        0: the reference's separate roundings */
} unap_cuda_amg_params;

void unap_cuda_amg_default_params(unap_cuda_amg_params* p);
/* builds the hierarchy of an existing matrix handle (the matrix must outlive
 * the AMG handle) */
int unap_cuda_amg_create(long int* amg, long int matrix, const unap_cuda_amg_params* p);
/* Size (cells, faces) and internal cell order of AMG level `level` (0 =
 * the matrix), the order as unap_cuda_matrix_layout gives it. */
int unap_cuda_amg_level_layout(long int amg, int level, int* nCells, long long* nFaces,
                               int* nWavefronts, int* perm, int* waveStart);
/* nLevels including the finest; cells[k] for k < min(nLevels, maxOut) */
int unap_cuda_amg_info(long int amg, int* nLevels, int* cells, int* wavefronts, int maxOut,
                       double* setupSeconds, long long* deviceBytes);
/* one V-cycle z = M^-1 r on device vectors in the caller's cell order */
int unap_cuda_amg_vcycle(long int amg, const double* r, double* z);
/* V-cycle timing on the handle's stream: one V-cycle is captured as a CUDA
 * graph (as inside a solve) with an event node around every level; ms[0] =
 * mean of `reps` graph launches; ms[1 + k] = level k's own steps in the last
 * launch (a level that starts the cluster tail holds the whole tail's time,
 * the levels below it 0).  *written = entries filled.  No counterpart in the
 * reference. */
int unap_cuda_amg_profile_vcycle(long int amg, int reps, double* ms, int maxOut, int* written);
/* Mean device time (CUDA events on the handle's stream) of one smoothing
 * launch group on AMG level `level` (not the coarsest), in the V-cycle's
 * precision, on scratch vectors: one Chebyshev step on a Chebyshev level,
 * one forward Gauss-Seidel sweep (a launch per wavefront) otherwise.
 * *bytes = its algorithmic DRAM bytes, *launches = kernel launches per
 * group.  No counterpart in the reference. */
int unap_cuda_amg_profile_smoother(long int amg, int level, int reps, double* ms, double* bytes,
                                   int* launches);
/* The Chebyshev smoother's eigenvalue estimate of every level but the
 * coarsest (0 on Gauss-Seidel levels): lam[k] for k < min(nLevels - 1,
 * maxOut); *written = entries filled.  No counterpart in the reference. */
int unap_cuda_amg_eigenvalues(long int amg, double* lam, int maxOut, int* written);
/* Host wall time of the hierarchy's setup phases, seconds[0..5]: face
 * weights and agglomeration; coarse level builds and transfer maps; the
 * coarsest inverse; level vectors and FP32 copies; row packing; eigenvalue
 * estimates.  No counterpart in the reference. */
int unap_cuda_amg_setup_phases(long int amg, double* seconds);
/* AMG-PCG on device vectors (x holds the initial guess) */
int unap_cuda_amg_solve(long int amg, double* x, const double* b, unap_cuda_stats* stats);
/* AMG-PCG on host vectors: copies b and x in, solves, copies x out */
int unap_cuda_amg_solve_host(long int amg, double* x, const double* b, unap_cuda_stats* stats);
int unap_cuda_amg_destroy(long int amg);

/* ---- MGSolver on device vectors (MGSolve.cpp:17-187).  weights NULL means
 * |upper|/||upper||; negative nCoarsest/maxLevels/nPre/nPost/nFinest keep the
 * reference defaults (50, 50, 0, 2, 2); scaleCorr -1 means "if symmetric". */
int unap_cuda_mg_create(long int* mg, long int matrix, const double* weights, int smoother,
                        int nCoarsest, int maxLevels, int nPre, int nPost, int nFinest,
                        int scaleCorr, double tol, double relTol, int maxIter, int minIter);
/* number of coarse levels; cells[k] for k <= nCoarseLevels (k = 0 finest) */
int unap_cuda_mg_levels(long int mg, int* nCoarseLevels, int* cells, int maxOut);
int unap_cuda_mg_solve(long int mg, double* x, const double* b, unap_cuda_stats* stats);
/* the same on host vectors (copied to the device and back) */
int unap_cuda_mg_solve_host(long int mg, double* x, const double* b, unap_cuda_stats* stats);
/* MGSolver setters after creation (MG.cpp:22-53): nPre/nPost/nFinest
 * sweeps, correction scaling (0/1), tol, relTol, maxIter, minIter */
int unap_cuda_mg_set(long int mg, int nPre, int nPost, int nFinest, int scaleCorr, double tol,
                     double relTol, int maxIter, int minIter);
int unap_cuda_mg_destroy(long int mg);

/* ---- Batched solves of many systems of uneven size.  Systems of at most
 * 65,536 cells (unap_cuda_set_team_solve_cells) are solved together in one
 * launch: a team of CTAs per system (one CTA, or a thread-block cluster of
 * 2 to 16) runs that system's whole PCG / PBiCGStab solve; larger ones run
 * one after another with the per-system driver.  The launch shape (CTA size
 * x CTAs per system) is chosen by the autotuner: the first batch of each
 * (size class, count class) times every launchable shape.  x and b are
 * device pointers in each system's cell order. */
typedef struct {
    long int matrix; /* handle from unap_cuda_matrix_create / ldumatrixcreat_ */
    int method;      /* 0 PCG, 1 PBiCGStab */
    int precond;     /* 0 none, 1 Diag, 2 DIC, 3 DILU */
    double tol, relTol;
    int maxIter, minIter;
    double* x;
    const double* b;
} unap_cuda_batch_item;

int unap_cuda_batch_create(long int* batch);
int unap_cuda_batch_solve(long int batch, int count, const unap_cuda_batch_item* items,
                          unap_cuda_stats* stats, int* ctaThreads);
int unap_cuda_batch_destroy(long int batch);
/* launch shape of the batch's last fused launch: CTA size, CTAs per system */
int unap_cuda_batch_last_shape(long int batch, int* ctaThreads, int* clusterCtas);
/* How the last batch solved its systems above the whole-solve size: 1 all
 * in one group launch (thread-block clusters of 16 CTAs), 0 one after
 * another with the per-step driver, -1 it had none.  The autotuner times
 * both (iterations capped) for the first batch of each (size class, count
 * class) and keeps the faster. */
int unap_cuda_batch_large_mode(long int batch, int* mode);
/* Systems of at most `cells` cells with an LDU preconditioner (none, Diag,
 * DIC, DILU) are solved by one whole-solve launch, in batches and by
 * unap_cuda_krylov_solve / pcgsolversolve_ / pbicgstabsolversolve_ alike
 * (default 65,536; 0 turns it off).  Returns the previous value; it applies
 * to solvers created afterwards. */
int unap_cuda_set_team_solve_cells(int cells);
/* the autotuner's cached shape for `systems` systems of up to `cells`
 * cells ({0, 0}: not tuned yet) */
int unap_cuda_team_shape(int cells, int systems, int* ctaThreads, int* clusterCtas);
/* every later whole-solve launch uses this shape (CTA size 128, 256, 512 or
 * 1024; cluster 1, 2, 4, 8 or 16 CTAs) instead of the autotuner's; a shape
 * the device cannot schedule is an error.  ctaThreads = 0 returns to the
 * autotuner. */
int unap_cuda_force_team_shape(int ctaThreads, int clusterCtas);

/* ---- Continuous-batching solve server.  Requests carry their own matrix
 * (host arrays, copied) and right-hand side; method 0 mixed AMG-PCG, 1 FP64
 * AMG-PCG (both with the Chebyshev degree-3 V-cycle on every level,
 * eigRatio 30), 2 PCG+DIC, 3 PBiCGStab+DILU.  A request is admitted when a slot
 * is free and its device-memory estimate fits what the solves in flight
 * leave of memoryBudget (0: 80% of free memory); maxSlots large solves run
 * on their own streams so their work overlaps on the GPU; PCG/PBiCGStab
 * requests of at most smallCells cells are collected and solved together
 * in one fused launch.  wait() blocks until the request is done, copies x
 * (host) and reports timings measured from submission; a request is
 * collected once (a second wait on its id returns UNAP_CUDA_EINVAL). */
typedef struct {
    int status;     /* 0 ok */
    int batched;    /* solved in a fused small-system launch */
    int nIterations;
    int converged;
    double initialResidual, finalResidual;
    double queueSeconds, setupSeconds, solveSeconds, latencySeconds;
} unap_cuda_request_info;

int unap_cuda_server_create(long int* server, long long memoryBudget, int maxSlots,
                            int smallCells);
int unap_cuda_server_submit(long int server, int nCells, int nFaces, const int* lowerAddr,
                            const int* upperAddr, const double* lower, const double* diag,
                            const double* upper, const double* b, int method, double relTol,
                            int maxIter, long long* id);
int unap_cuda_server_wait(long int server, long long id, double* x, unap_cuda_request_info* info);
int unap_cuda_server_destroy(long int server);
/* server slots replay each Krylov iteration from a CUDA graph (1, the
 * default) or launch its kernels one by one (0); applies to requests started
 * afterwards; returns the previous setting */
int unap_cuda_set_server_graphs(int on);
/* PCG/PBiCGStab requests of up to `cells` cells that a server slot solves
 * (those above the batch lane's size) run as one whole-solve launch on a
 * thread-block cluster (default 0: none, every slot request runs per-step
 * launches, which serve the mixed stream faster); returns the previous
 * value */
int unap_cuda_set_server_team_cells(int cells);
/* AMG requests of the server: coarsest level target (default 200 cells)
 * and the Chebyshev interval [lambda / eigRatio, 1.1 lambda] (default 30),
 * for requests started afterwards */
int unap_cuda_set_server_amg(int nCoarsest, double eigRatio);

int unap_cuda_device_synchronize(void);

/* Kernel timings on the matrix's own stream with CUDA events (the GB300
 * counterpart of the reference's swTimer hooks, src/tools/timers/swTimer.cpp).
 * Average milliseconds over `reps` after one warm-up, in internal order:
 * ms[0] SpMV, ms[1] DIC apply (forward + backward sweeps), ms[2] DILU apply,
 * ms[3] forward Gauss-Seidel sweep, ms[4] backward Gauss-Seidel sweep,
 * ms[5] FP32 SpMV, ms[6] FP32 forward Gauss-Seidel sweep, ms[7] residual. */
int unap_cuda_profile_kernels(long int handle, int reps, double* ms);

/* Kernel launches issued by this library since it was loaded (a CUDA-graph
 * launch counts its kernel nodes). */
long long unap_cuda_launch_count(void);

/* Executor of PCG solves created after the call: 0 (default) launches one
 * kernel per step, one iteration captured as a CUDA graph; 1 runs the whole
 * solve as one persistent cooperative launch that executes a compiled step
 * program.  Both give the same iterates up to dot-product summation order.
 * Returns the previous setting.  No counterpart in the reference. */
int unap_cuda_set_executor(int persistent);

/* How host threads of this process wait for the GPU (synchronizations,
 * read-backs) on the current device: 0 the CUDA default, 1 spin, 2 yield,
 * 3 block on an OS primitive (frees the core for other host threads, e.g.
 * a server's slot workers).  Call before the device's context is created
 * (the first CUDA call of the process on that device). */
int unap_cuda_set_host_wait(int mode);

/* Per-wavefront Gauss-Seidel launches use programmatic dependent launch:
 * the next wavefront's kernel starts launching while the previous one runs
 * and loads its rows' matrix data before it waits for it (1, default); 0
 * launches them one after the other.  Results are identical.  Returns the
 * previous setting.  No counterpart in the reference. */
int unap_cuda_set_wave_pdl(int on);

/* Grid of the per-wavefront Gauss-Seidel launches: 1 (default) one CTA per
 * 256 rows of the wavefront, so every row's matrix data is loaded before the
 * dependency wait; 0 a grid-stride loop over at most (SMs x 8) CTAs.
 * Results are identical.  Returns the previous setting.  No counterpart in
 * the reference. */
int unap_cuda_set_wave_grid(int oneRowPerThread);

/* AMG V-cycle Gauss-Seidel sweeps on levels whose rows average more than 8
 * entries read a row-packed copy of the level (a row's entries as 16-byte
 * records, loaded before the dependency wait): mode 1 (default) holds the
 * first 16 (FP32) / 8 (FP64) entries in registers on levels averaging under
 * 12.5 entries per row and 24 / 12 above; mode 2 always 16 / 8, mode 3
 * always 24 / 12; mode 0 reads the SELL-32 storage.  Results are
 * identical.  Returns the previous setting.  No counterpart in the
 * reference. */
int unap_cuda_set_packed_sweeps(int mode);

/* Chebyshev-step launches (AMG V-cycle with smoother 1) on levels of at
 * most `rows` rows use one-warp CTAs, spread over more SMs than 256-thread
 * CTAs would be (default 100000).  Results are identical.  Returns the
 * previous setting.  No counterpart in the reference. */
int unap_cuda_set_cheby_small_rows(int rows);
/* Matrices created afterwards (any C ABI call that builds one) get
 * wavefront ranges for DIC/DILU/Gauss-Seidel sweeps (1, default), or only a
 * locality order (0): cheaper to build and faster for SpMV gathers, but
 * only SpMV-shaped work runs on them -- SpMV, Krylov solves without a
 * preconditioner or with Diag, AMG-PCG with Chebyshev from level 0; the
 * sweeps return UNAP_CUDA_EINVAL.  Returns the previous setting.  No
 * counterpart in the reference. */
int unap_cuda_set_matrix_wavefronts(int on);
/* Entries of a row the Chebyshev step loads per dependent round trip: 0
 * (default) 16 on levels averaging more than 8 entries per row, except FP32
 * levels of 2^20 rows or more, and 8 elsewhere; or 8 / 16 everywhere (fewer
 * registers and more resident warps against one round trip per row).  Results are identical.  Returns the
 * previous setting, or UNAP_CUDA_EINVAL for another value.  No counterpart
 * in the reference. */
int unap_cuda_set_cheby_chunk(int entries);
/* Chebyshev V-cycles run their coarse levels of at most `rows` rows (and
 * every level below them, at most 8 above the coarsest) in one
 * thread-block-cluster launch instead of a launch per step (0: never).
 * Results are identical.  Returns the previous value; applies to AMG
 * handles created afterwards.  No counterpart in the reference. */
int unap_cuda_set_cheby_tail_rows(int rows);

/* Coarse-level tail of the AMG V-cycle (per-step executor), set for the FP64
 * (precision 0) or FP32 (precision 1) V-cycle: every level with at most
 * tailRows rows whose iterate fits in the cluster's shared memory, down to
 * the dense coarsest solve and back, runs in one launch of a single
 * thread-block cluster, wavefronts separated by the cluster barrier; tail
 * levels with at most singleRows rows run on the cluster's first CTA alone.
 * tailRows = 0 launches one kernel per wavefront on every level.  The
 * V-cycle result is bit-identical either way.  Defaults: FP64 2097152 and
 * 8192, FP32 8192 and 8192; the previous values are returned through the
 * (nullable) pointers.  Applies to V-cycles launched after the call, CUDA
 * graphs captured before keep their launches.  No counterpart in the
 * reference. */
int unap_cuda_set_tail_rows(int precision, long long tailRows, long long singleRows,
                            long long* oldTailRows, long long* oldSingleRows);

/* Cluster size (CTAs) the tail kernel launches with on the current device,
 * 0 when the device schedules no cluster of 2 or more 1024-thread CTAs. */
int unap_cuda_tail_cluster_size(int* clusterSize);

/* Failure-detection self-test of the persistent executor's bounded waits:
 * one CTA sleeps (bounded) past a deliberately tiny barrier-wait bound, the
 * other CTAs give up, the launch ends and reports the timeout
 * (*timedOut = 1); a second launch with the normal bound then completes
 * (*recovered = 1).  Nothing faults and nothing waits without a bound. */
int unap_cuda_selftest_barrier_timeout(int* timedOut, int* recovered);

/* ---- Text dumps in the reference's on-disk formats (host only; no GPU
 * work).  Fields are read like the reference reader (lines split at '\n',
 * fields at white space, reals by atof, integers by atoi): the values are
 * bit-identical to its.  Printers write "<name>_0.txt" (the reference's
 * "<name>_<rank>.txt" on a single rank) with "%.15e" reals, byte-identical
 * to its printers.  The reference reader aborts the process on a malformed
 * file; these return UNAP_CUDA_EINVAL with its message instead. */

/* constructLDUMatrixFromOpenFOAM (tools/readData/readFromOpenFOAM/
 * readFromOpenFOAM.cpp:9-139): header "nCells: N nnz: M symm: s", N diagonal
 * lines "i i diag", then "l u upper [lower]" per face.  *handle receives a
 * matrix handle like ldumatrixcreat_'s (built on the device on first use);
 * unap_cuda_matrix_size / unap_cuda_matrix_get_ldu return its arrays. */
int unap_cuda_read_ldu_matrix(const char* fileName, long int* handle);
/* constructVectorFromOpenFOAM (readFromOpenFOAM.cpp:142-204): header
 * "nCells: N", then one value per line; N must equal n. */
int unap_cuda_read_vector(const char* fileName, long long n, double* v);
/* constructLDUInterfacesFromOpenFOAM (readFromOpenFOAM.cpp:207-322): header
 * with nNeiProcs in field 2 and the total face count in field 5, then per
 * neighbour "processor: <rank> size: <m>" and m lines "faceCell coeff".
 * Sizes are always returned; each non-NULL array is filled (neighbour and
 * size hold nNeiProcs entries, faceCells and coeffs nFaces).  Coefficients
 * are stored negated, as the reference's patches keep them.  Call once with
 * NULL arrays to size them. */
int unap_cuda_read_interfaces(const char* fileName, int* nNeiProcs, long long* nFaces,
                              int* neighbour, int* size, int* faceCells, double* coeffs);
/* printLDUMatrix (tools/printData/printUNAP/printUNAP.cpp:8-58) */
int unap_cuda_print_ldu_matrix(long int handle, const char* name);
/* printVector (printUNAP.hpp:27-42) */
int unap_cuda_print_vector(const char* name, long long n, const double* v);
/* printInterfaces (printUNAP.cpp:61-87), from the arrays
 * unap_cuda_read_interfaces returns.  Its header line carries only
 * nNeiProcs, so like the reference's, its output is not a file the reader
 * accepts. */
int unap_cuda_print_interfaces(const char* name, int nNeiProcs, const int* neighbour,
                               const int* size, const int* faceCells, const double* coeffs);

#ifdef __cplusplus
}
#endif

#endif /* UNAP_CUDA_H */
