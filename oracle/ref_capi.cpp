/*
 * Flat C entry points over the reference UNAP library (oracle/_ref).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is compiled together with the
 * reference's own x86 sources, read in place, by oracle/Makefile into
 * oracle/_ref/libunap_ref.so.  The pytest suite loads that library through
 * ctypes to pin the C restatement (oracle/unap_oracle.c) against the real
 * reference code and to generate the golden fixtures under tests/golden.
 * Nothing in the product links or loads it.
 *
 * All functions take 0-based int32 addressing and FP64 values and convert to
 * the reference's label/scalar types (built with -DLABEL_INT64
 * -DSCALAR_FLOAT64, the working flag set of SConstruct:13,52).
 */
#include <vector>
#include <cstring>

#include "unap.hpp"
#include "lduMatrix.hpp"
#include "PCG.hpp"
#include "PBiCGStab.hpp"
#include "MG.hpp"
#include "lduDiagPrecond.hpp"
#include "lduDICPrecond.hpp"
#include "lduDILUPrecond.hpp"
#include "lduGaussSeidelSmoother.hpp"
#include "chebySmoother.hpp"
#include "lduAgglomeration.hpp"
#include "eigenDiagPCG.hpp"
#include "matrixConversion.hpp"
#include "readFromOpenFOAM.hpp"
#include "printUNAP.hpp"

using namespace UNAP;

namespace {

struct RefMatrix {
    labelField lowerAddr, upperAddr;
    scalarField lower, diag, upper;
    lduMatrix* A;

    RefMatrix(int n, int nf, const int* l, const int* u, const double* lo,
              const double* d, const double* up, int symm)
        : lowerAddr(nf), upperAddr(nf), lower(symm ? 0 : nf), diag(n), upper(nf), A(nullptr)
    {
        for (int f = 0; f < nf; ++f) {
            lowerAddr[f] = l[f];
            upperAddr[f] = u[f];
            upper[f] = up[f];
            if (!symm) lower[f] = lo[f];
        }
        for (int c = 0; c < n; ++c) diag[c] = d[c];
        // lduMatrix.cpp:54-61: symmetric iff the same scalarField is passed twice
        if (symm)
            A = new lduMatrix(n, lowerAddr, upperAddr, upper, diag, upper);
        else
            A = new lduMatrix(n, lowerAddr, upperAddr, lower, diag, upper);
    }
    ~RefMatrix() { delete A; }
};

void copyIn(scalarField& f, const double* v, int n)
{
    for (int i = 0; i < n; ++i) f[i] = v[i];
}

void copyOut(double* v, const scalarField& f, int n)
{
    for (int i = 0; i < n; ++i) v[i] = f[i];
}

matrix::preconditioner* makePrecond(int type, const lduMatrix& A)
{
    // fortranInterface.cpp:227-238 numbering: 1 Diag, 2 DIC, 3 DILU
    if (type == 1) return new lduDiagPrecond(A);
    if (type == 2) return new lduDICPrecond(A);
    if (type == 3) return new lduDILUPrecond(A);
    return new matrix::preconditioner();
}

}  // namespace

extern "C" {

void ref_spmv(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
              const double* up, int symm, const double* x, double* y)
{
    RefMatrix M(n, nf, l, u, lo, d, up, symm);
    scalarField xs(n), ys(n);
    copyIn(xs, x, n);
    M.A->spMV(ys, xs);
    copyOut(y, ys, n);
}

void ref_losort(int n, int nf, const int* l, const int* u, int* losort, int* ownerStart,
                int* losortStart)
{
    std::vector<double> zero(nf, 0.0), dz(n, 1.0);
    RefMatrix M(n, nf, l, u, zero.data(), dz.data(), zero.data(), 1);
    const labelField& ls = M.A->losortAddr();
    const labelField& os = M.A->ownerStartAddr();
    const labelField& lss = M.A->losortStartAddr();
    for (int f = 0; f < nf; ++f) losort[f] = (int)ls[f];
    for (int c = 0; c <= n; ++c) {
        ownerStart[c] = (int)os[c];
        losortStart[c] = (int)lss[c];
    }
}

void ref_precond(int type, int n, int nf, const int* l, const int* u, const double* lo,
                 const double* d, const double* up, int symm, const double* r, double* w,
                 double* rD)
{
    RefMatrix M(n, nf, l, u, lo, d, up, symm);
    matrix::preconditioner* P = makePrecond(type, *M.A);
    scalarField rs(n), ws(n);
    copyIn(rs, r, n);
    P->precondition(ws, rs);
    copyOut(w, ws, n);
    if (rD && type >= 1 && type <= 3) copyOut(rD, P->rD(), n);
    delete P;
}

void ref_gs(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
            const double* up, int symm, double* x, const double* b, int nSweeps)
{
    RefMatrix M(n, nf, l, u, lo, d, up, symm);
    scalarField xs(n), bs(n);
    copyIn(xs, x, n);
    copyIn(bs, b, n);
    lduGaussSeidelSmoother gs;
    gs.smooth(xs, *M.A, bs, nSweeps);
    copyOut(x, xs, n);
}

/* nCalls consecutive smooth() calls on the same smoother object: the first
 * one only estimates the eigenvalue (chebySmoother.cpp:22-42). */
void ref_cheby(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
               const double* up, int symm, double* x, const double* b, int nSweeps, int nCalls)
{
    RefMatrix M(n, nf, l, u, lo, d, up, symm);
    scalarField xs(n), bs(n);
    copyIn(xs, x, n);
    copyIn(bs, b, n);
    chebySmoother cs;
    for (int k = 0; k < nCalls; ++k) cs.smooth(xs, *M.A, bs, nSweeps);
    copyOut(x, xs, n);
}

double ref_eigen(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
                 const double* up, int symm, double* x, const double* b, int nDiagPCGs)
{
    RefMatrix M(n, nf, l, u, lo, d, up, symm);
    scalarField xs(n), bs(n);
    copyIn(xs, x, n);
    copyIn(bs, b, n);
    lduDiagPrecond P(*M.A);
    eigenDiagPCG e(*M.A, xs, bs, P, nDiagPCGs);
    copyOut(x, xs, n);
    return e.maxEigenValue();
}

static void finishPerf(const matrix::solverPerformance& perf, int* nIter, double* initRes,
                       double* finalRes, int* converged, int* singular)
{
    if (nIter) *nIter = (int)perf.nIterations();
    if (initRes) *initRes = perf.initialResidual();
    if (finalRes) *finalRes = perf.finalResidual();
    if (converged) *converged = perf.converged() ? 1 : 0;
    if (singular) *singular = perf.singular() ? 1 : 0;
}

void ref_pcg(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
             const double* up, int symm, int precond, double tol, double relTol, int maxIter,
             int minIter, double* x, const double* b, int* nIter, double* initRes,
             double* finalRes, int* converged, int* singular)
{
    RefMatrix M(n, nf, l, u, lo, d, up, symm);
    matrix::preconditioner* P = makePrecond(precond, *M.A);
    PCG solver(*P);
    solver.SET_tolerance(tol);
    solver.SET_relTol(relTol);
    solver.SET_maxIter(maxIter);
    solver.SET_minIter(minIter);
    scalarField xs(n), bs(n);
    copyIn(xs, x, n);
    copyIn(bs, b, n);
    matrix::solverPerformance perf = solver.solve(xs, *M.A, bs);
    copyOut(x, xs, n);
    finishPerf(perf, nIter, initRes, finalRes, converged, singular);
    delete P;
}

void ref_pbicgstab(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
                   const double* up, int symm, int precond, double tol, double relTol,
                   int maxIter, int minIter, double* x, const double* b, int* nIter,
                   double* initRes, double* finalRes, int* converged, int* singular)
{
    RefMatrix M(n, nf, l, u, lo, d, up, symm);
    matrix::preconditioner* P = makePrecond(precond, *M.A);
    PBiCGStab solver(*P);
    solver.SET_tolerance(tol);
    solver.SET_relTol(relTol);
    solver.SET_maxIter(maxIter);
    solver.SET_minIter(minIter);
    scalarField xs(n), bs(n);
    copyIn(xs, x, n);
    copyIn(bs, b, n);
    matrix::solverPerformance perf = solver.solve(xs, *M.A, bs);
    copyOut(x, xs, n);
    finishPerf(perf, nIter, initRes, finalRes, converged, singular);
    delete P;
}

/* ---- agglomeration hierarchy ------------------------------------------- */

struct RefAggl {
    RefMatrix* M;
    lduAgglomeration* agg;
};

void* ref_aggl_create(int n, int nf, const int* l, const int* u, const double* lo,
                      const double* d, const double* up, int symm, const double* weights,
                      int nCoarsest, int maxLevels)
{
    RefAggl* h = new RefAggl;
    h->M = new RefMatrix(n, nf, l, u, lo, d, up, symm);
    h->agg = new lduAgglomeration(*h->M->A);
    if (maxLevels > 0) h->agg->SET_maxLevels(maxLevels);
    if (nCoarsest > 0) h->agg->SET_nCellsInCoarsestLevel(nCoarsest);
    scalarField w(nf);
    copyIn(w, weights, nf);
    h->agg->agglomerate(w);
    return h;
}

int ref_aggl_nlevels(void* hv) { return (int)((RefAggl*)hv)->agg->size(); }

int ref_aggl_ncells(void* hv, int level)
{
    return (int)((RefAggl*)hv)->agg->coarseMatrixLevels(level).size();
}

int ref_aggl_nfaces(void* hv, int level)
{
    return (int)((RefAggl*)hv)->agg->coarseMatrixLevels(level).upperAddr().size();
}

/* restrictAddressing(level) maps the cells of fine level `level` (0 = the
 * input matrix) to coarse level `level`; faceRestrict likewise for faces. */
void ref_aggl_addressing(void* hv, int level, int* restrictAddr, int* faceRestrict,
                         int* coarseLower, int* coarseUpper)
{
    RefAggl* h = (RefAggl*)hv;
    const labelField& ra = h->agg->restrictAddressing(level);
    const labelField& fa = h->agg->faceRestrictAddressing(level);
    const lduMatrix& C = h->agg->coarseMatrixLevels(level);
    for (label i = 0; i < ra.size(); ++i) restrictAddr[i] = (int)ra[i];
    for (label i = 0; i < fa.size(); ++i) faceRestrict[i] = (int)fa[i];
    for (label i = 0; i < C.lowerAddr().size(); ++i) {
        coarseLower[i] = (int)C.lowerAddr()[i];
        coarseUpper[i] = (int)C.upperAddr()[i];
    }
}

/* Runs agglomerateMatrix for every level (as MGSolve.cpp:108-111 does) and
 * returns the coarse coefficients of one level. */
void ref_aggl_coeffs(void* hv, int level, double* diag, double* upper, double* lower)
{
    RefAggl* h = (RefAggl*)hv;
    for (int k = 0; k <= level; ++k) {
        // agglomerateMatrix is private on lduAgglomeration, public on the base.
        matrix::agglomeration& base = *h->agg;
        base.agglomerateMatrix(k);
    }
    const lduMatrix& C = h->agg->coarseMatrixLevels(level);
    copyOut(diag, C.diag(), (int)C.size());
    int nfc = (int)C.upperAddr().size();
    copyOut(upper, C.upper(), nfc);
    if (lower) copyOut(lower, C.lower(), nfc);
}

void ref_aggl_destroy(void* hv)
{
    RefAggl* h = (RefAggl*)hv;
    delete h->agg;
    delete h->M;
    delete h;
}

/* MGSolver::solve with the reference's defaults unless overridden
 * (negative arguments keep the default of MG.cpp:3-19). smoother: 1 GS, 2 Cheby. */
void ref_mg(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
            const double* up, int symm, const double* weights, int nCoarsest, int maxLevels,
            int smootherType, int nPre, int nPost, int nFinest, int scaleCorr, double tol,
            double relTol, int maxIter, int minIter, double* x, const double* b, int* nIter,
            double* initRes, double* finalRes, int* converged, int* nLevels)
{
    RefMatrix M(n, nf, l, u, lo, d, up, symm);
    lduAgglomeration agg(*M.A);
    if (maxLevels > 0) agg.SET_maxLevels(maxLevels);
    if (nCoarsest > 0) agg.SET_nCellsInCoarsestLevel(nCoarsest);
    scalarField w(nf);
    copyIn(w, weights, nf);
    agg.agglomerate(w);
    if (nLevels) *nLevels = (int)agg.size();

    PtrList<matrix::smoother> sm(agg.size());
    for (label i = 0; i < agg.size(); ++i) {
        if (smootherType == 2)
            sm.setLevel(i, *new chebySmoother);
        else
            sm.setLevel(i, *new lduGaussSeidelSmoother);
    }
    MGSolver mg(*M.A, agg, sm);
    mg.SET_tolerance(tol);
    mg.SET_relTol(relTol);
    mg.SET_maxIter(maxIter);
    mg.SET_minIter(minIter);
    if (nPre >= 0) mg.SET_nPreSweeps(nPre);
    if (nPost >= 0) mg.SET_nPostSweeps(nPost);
    if (nFinest >= 0) mg.SET_nFinestSweeps(nFinest);
    if (scaleCorr >= 0) mg.SET_scaleCorrection(scaleCorr != 0);

    scalarField xs(n), bs(n);
    copyIn(xs, x, n);
    copyIn(bs, b, n);
    matrix::solverPerformance perf = mg.solve(xs, *M.A, bs);
    copyOut(x, xs, n);
    finishPerf(perf, nIter, initRes, finalRes, converged, nullptr);
}

/* coo2ldu (matrixConversion/coo2ldu.cpp:3-113) on 0-based sorted COO input. */
void* ref_coo2ldu(const double* val, const int* row, const int* col, int n, int nnz, int symm)
{
    std::vector<label> r(row, row + nnz), c(col, col + nnz);
    lduMatrix& A = coo2ldu(val, r.data(), c.data(), n, nnz, symm != 0);
    return &A;
}

int ref_ldu_nfaces(void* Av) { return (int)((lduMatrix*)Av)->upperAddr().size(); }

void ref_ldu_get(void* Av, int* l, int* u, double* lower, double* diag, double* upper)
{
    lduMatrix& A = *(lduMatrix*)Av;
    int nf = (int)A.upperAddr().size();
    for (int f = 0; f < nf; ++f) {
        l[f] = (int)A.lowerAddr()[f];
        u[f] = (int)A.upperAddr()[f];
        upper[f] = A.upper()[f];
        lower[f] = A.lower()[f];
    }
    for (label c = 0; c < A.size(); ++c) diag[c] = A.diag()[c];
}

void ref_ldu_destroy(void* Av) { delete (lduMatrix*)Av; }

/* ---- text dumps: the reference reader and printers, unchanged ---- */

void* ref_read_ldu(const char* path)
{
    lduMatrix* A = new lduMatrix;
    constructLDUMatrixFromOpenFOAM(*A, path);
    return A;
}

int ref_ldu_ncells(void* Av) { return (int)((lduMatrix*)Av)->size(); }
int ref_ldu_symm(void* Av) { return ((lduMatrix*)Av)->symm() ? 1 : 0; }

void ref_read_vector(const char* path, int n, double* out)
{
    scalarField b(n);
    constructVectorFromOpenFOAM(b, path);
    for (int i = 0; i < n; ++i) out[i] = b[i];
}

void ref_print_ldu(void* Av, const char* name) { printLDUMatrix(*(lduMatrix*)Av, name); }

void ref_print_vector(const char* name, int n, const double* v)
{
    scalarField b(n);
    for (int i = 0; i < n; ++i) b[i] = v[i];
    printVector(b, name);
}

/* reads an interfaces file into a matrix (sizes via the first call with
 * NULL arrays), copies its patches out and prints them back with
 * printInterfaces when name != NULL */
int ref_read_interfaces(const char* path, int* nNei, int* nFaces, int* neighbour, int* size,
                        int* faceCells, double* coeffs, const char* name)
{
    lduMatrix A;
    constructLDUInterfacesFromOpenFOAM(A, path);
    const interfaces& I = A.matrixInterfaces();
    int np = (int)I.size(), k = 0;
    for (int i = 0; i < np; ++i) {
        patch& P = I.patchList(i);
        if (neighbour) neighbour[i] = (int)P.neighbProcNo();
        if (size) size[i] = (int)P.size();
        for (label f = 0; f < P.size(); ++f, ++k) {
            if (faceCells) faceCells[k] = (int)P.faceCells()[f];
            if (coeffs) coeffs[k] = P.patchCoeffs(f);
        }
    }
    *nNei = np;
    *nFaces = k;
    if (name) printInterfaces(A, name);
    return 0;
}

/* matrixConversion.cpp:38-222, 0-based: the reference's reorderings on
 * label copies of the caller's int arrays */
void ref_reorder_coo(double* val, int* row, int* col, int n, int size)
{
    std::vector<label> r(row, row + size), c(col, col + size);
    reorderCOO(val, r.data(), c.data(), n, size);
    for (int i = 0; i < size; ++i) {
        row[i] = (int)r[(size_t)i];
        col[i] = (int)c[(size_t)i];
    }
}

void ref_reorder_faces(int byColumn, int* row, int* col, int n, int size, int* newOrder)
{
    std::vector<label> r(row, row + size), c(col, col + size), o((size_t)size);
    if (byColumn)
        reorderLFace(r.data(), c.data(), n, size, o.data());
    else
        reorderUFace(r.data(), c.data(), n, size, o.data());
    for (int i = 0; i < size; ++i) {
        row[i] = (int)r[(size_t)i];
        col[i] = (int)c[(size_t)i];
        newOrder[i] = (int)o[(size_t)i];
    }
}

void ref_reorder_value(double* val, const int* newOrder, int size)
{
    std::vector<label> o(newOrder, newOrder + size);
    reorderValue(val, o.data(), size);
}

}  // extern "C"
