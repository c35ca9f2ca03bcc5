/*
 * unap_oracle.c -- CPU restatement of UNAP's solve hot path (see
 * unap_oracle.h).  TEST INFRASTRUCTURE ONLY: the checker for the CUDA
 * library and the "port" CPU baseline; never part of the product.
 *
 * Parity is pinned two ways by the test suite: against the reference library
 * itself compiled in place (oracle/_ref, where the reference tree exists) and
 * against golden fixtures generated from it (tests/golden/).
 *
 * Built with -ffp-contract=off so that no multiply-add is fused on any host.
 */
#include "unap_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define SMALL_ 1.0e-37   /* src/base/unap.hpp:88 */
#define VSMALL_ 1.0e-128 /* src/base/unap.hpp:89 */
#define GREAT_ 1.0e+37   /* src/base/unap.hpp:92 */

static void* xcalloc(size_t n, size_t s)
{
    void* p = calloc(n ? n : 1, s);
    if (!p) abort();
    return p;
}

/* ------------------------------------------------------------------------
 * Matrix view with lazily built addressing
 * --------------------------------------------------------------------- */
typedef struct {
    int n, nf, symm;
    const int *l, *u;
    const double *lower, *diag, *upper;
    int* ownerStart; /* n+1 */
    int* losort;     /* nf */
} omat;

static omat mat_view(int n, int nf, const int* l, const int* u, const double* lo,
                     const double* d, const double* up, int symm)
{
    omat m;
    m.n = n;
    m.nf = nf;
    m.symm = symm;
    m.l = l;
    m.u = u;
    m.upper = up;
    m.lower = symm ? up : lo;
    m.diag = d;
    m.ownerStart = NULL;
    m.losort = NULL;
    return m;
}

static void mat_free_addr(omat* m)
{
    free(m->ownerStart);
    free(m->losort);
    m->ownerStart = NULL;
    m->losort = NULL;
}

/* lduMatrix::calcOwnerStart, lduMatrix.cpp:269-296 */
static void calc_owner_start(int n, int nf, const int* own, int* ownStart)
{
    for (int i = 0; i <= n; ++i) ownStart[i] = nf;
    ownStart[0] = 0;
    int nOwnStart = 0;
    int i = 1;
    for (int f = 0; f < nf; ++f) {
        int curOwn = own[f];
        if (curOwn > nOwnStart) {
            while (i <= curOwn) ownStart[i++] = f;
            nOwnStart = curOwn;
        }
    }
}

/* lduMatrix::calcLosort, lduMatrix.cpp:310-367: faces ordered by neighbour,
 * stable in face order. */
static void calc_losort(int n, int nf, const int* nbr, int* losort)
{
    int* cnt = (int*)xcalloc((size_t)n + 1, sizeof(int));
    for (int f = 0; f < nf; ++f) cnt[nbr[f] + 1]++;
    for (int c = 0; c < n; ++c) cnt[c + 1] += cnt[c];
    for (int f = 0; f < nf; ++f) losort[cnt[nbr[f]]++] = f;
    free(cnt);
}

/* lduMatrix::calcLosortStart, lduMatrix.cpp:381-414.  Restated with its
 * quirk: cells above the largest neighbour index keep start 0. */
static void calc_losort_start(int n, int nf, const int* nbr, const int* lsrt, int* lsrtStart)
{
    for (int i = 0; i <= n; ++i) lsrtStart[i] = 0;
    int nLsrtStart = 0;
    int i = 0;
    for (int f = 0; f < nf; ++f) {
        int curNbr = nbr[lsrt[f]];
        if (curNbr > nLsrtStart) {
            while (i <= curNbr) lsrtStart[i++] = f;
            nLsrtStart = curNbr;
        }
    }
    lsrtStart[n] = nf;
}

static const int* mat_owner_start(omat* m)
{
    if (!m->ownerStart) {
        m->ownerStart = (int*)xcalloc((size_t)m->n + 1, sizeof(int));
        calc_owner_start(m->n, m->nf, m->l, m->ownerStart);
    }
    return m->ownerStart;
}

static const int* mat_losort(omat* m)
{
    if (!m->losort) {
        m->losort = (int*)xcalloc((size_t)m->nf, sizeof(int));
        calc_losort(m->n, m->nf, m->u, m->losort);
    }
    return m->losort;
}

void orc_losort(int n, int nf, const int* l, const int* u, int* losort, int* ownerStart,
                int* losortStart)
{
    calc_losort(n, nf, u, losort);
    calc_owner_start(n, nf, l, ownerStart);
    calc_losort_start(n, nf, u, losort, losortStart);
}

/* ------------------------------------------------------------------------
 * Vector helpers: sequential sums starting from 0 like the reference
 * --------------------------------------------------------------------- */

/* dot(), unapVectorOperations.cpp:6-34 */
static double vdot(int n, const double* a, const double* b)
{
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* solver::normFactor = SumSqrt + SMALL, unapMatrixSolver.cpp:12-16 and
 * Vector::SumSqr/SumSqrt, unapVector.hpp:459-485 */
static double norm_factor(int n, const double* r)
{
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += r[i] * r[i];
    return sqrt(s) + SMALL_;
}

/* ------------------------------------------------------------------------
 * SpMV: lduMatrix::spMV, lduMatrixSpMV.cpp:16-98 (x86 branch :83-92)
 * --------------------------------------------------------------------- */
static void mat_spmv(const omat* m, const double* x, double* y)
{
    for (int c = 0; c < m->n; ++c) y[c] = 0.0;
    for (int c = 0; c < m->n; ++c) y[c] += m->diag[c] * x[c];
    for (int f = 0; f < m->nf; ++f) {
        y[m->u[f]] += m->lower[f] * x[m->l[f]];
        y[m->l[f]] += m->upper[f] * x[m->u[f]];
    }
}

void orc_spmv(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
              const double* up, int symm, const double* x, double* y)
{
    omat m = mat_view(n, nf, l, u, lo, d, up, symm);
    mat_spmv(&m, x, y);
}

/* ------------------------------------------------------------------------
 * Preconditioners
 * --------------------------------------------------------------------- */

/* lduDiagPrecond ctor, lduDiagPrecond.cpp:13-41 */
static void diag_rD(const omat* m, double* rD)
{
    for (int c = 0; c < m->n; ++c) rD[c] = 1.0 / m->diag[c];
}

/* lduDICPrecond::calcReciprocalD, lduDICPrecond.cpp:15-42 */
static void dic_rD(const omat* m, double* rD)
{
    for (int c = 0; c < m->n; ++c) rD[c] = m->diag[c];
    for (int f = 0; f < m->nf; ++f)
        rD[m->u[f]] -= m->upper[f] * m->upper[f] / rD[m->l[f]];
    for (int c = 0; c < m->n; ++c) rD[c] = 1.0 / rD[c];
}

/* lduDILUPrecond::calcReciprocalD, lduDILUPrecond.cpp:15-43 */
static void dilu_rD(const omat* m, double* rD)
{
    for (int c = 0; c < m->n; ++c) rD[c] = m->diag[c];
    for (int f = 0; f < m->nf; ++f)
        rD[m->u[f]] -= m->upper[f] * m->lower[f] / rD[m->l[f]];
    for (int c = 0; c < m->n; ++c) rD[c] = 1.0 / rD[c];
}

/* lduDICPrecond::precondition, lduDICPrecond.cpp:45-77 */
static void dic_apply(const omat* m, const double* rD, const double* r, double* w)
{
    const int* u = m->u;
    const int* l = m->l;
    const double* up = m->upper;
    for (int c = 0; c < m->n; ++c) w[c] = rD[c] * r[c];
    for (int f = 0; f < m->nf; ++f) w[u[f]] -= rD[u[f]] * up[f] * w[l[f]];
    for (int f = m->nf - 1; f >= 0; --f) w[l[f]] -= rD[l[f]] * up[f] * w[u[f]];
}

/* lduDILUPrecond::precondition, lduDILUPrecond.cpp:46-86 */
static void dilu_apply(omat* m, const double* rD, const double* r, double* w)
{
    const int* u = m->u;
    const int* l = m->l;
    const int* ls = mat_losort(m);
    for (int c = 0; c < m->n; ++c) w[c] = rD[c] * r[c];
    for (int i = 0; i < m->nf; ++i) {
        int f = ls[i];
        w[u[f]] -= rD[u[f]] * m->lower[f] * w[l[f]];
    }
    for (int f = m->nf - 1; f >= 0; --f) w[l[f]] -= rD[l[f]] * m->upper[f] * w[u[f]];
}

typedef struct {
    int type; /* 0 none, 1 diag, 2 DIC, 3 DILU */
    double* rD;
} oprec;

static oprec prec_make(int type, const omat* m)
{
    oprec p;
    p.type = (type >= 1 && type <= 3) ? type : 0;
    p.rD = NULL;
    if (p.type) {
        p.rD = (double*)xcalloc((size_t)m->n, sizeof(double));
        if (p.type == 1) diag_rD(m, p.rD);
        if (p.type == 2) dic_rD(m, p.rD);
        if (p.type == 3) dilu_rD(m, p.rD);
    }
    return p;
}

static void prec_apply(const oprec* p, omat* m, const double* r, double* w)
{
    switch (p->type) {
    case 1:
        for (int c = 0; c < m->n; ++c) w[c] = p->rD[c] * r[c]; /* lduDiagPrecond.cpp:44-73 */
        break;
    case 2: dic_apply(m, p->rD, r, w); break;
    case 3: dilu_apply(m, p->rD, r, w); break;
    default: /* identity, unapMatrixPrecond.cpp:4-17 */
        for (int c = 0; c < m->n; ++c) w[c] = r[c];
    }
}

void orc_precond(int type, int n, int nf, const int* l, const int* u, const double* lo,
                 const double* d, const double* up, int symm, const double* r, double* w,
                 double* rD)
{
    omat m = mat_view(n, nf, l, u, lo, d, up, symm);
    oprec p = prec_make(type, &m);
    prec_apply(&p, &m, r, w);
    if (rD && p.rD) memcpy(rD, p.rD, sizeof(double) * (size_t)n);
    free(p.rD);
    mat_free_addr(&m);
}

/* ------------------------------------------------------------------------
 * Gauss-Seidel: lduGaussSeidelSmoother::smooth, lduGaussSeidelSmoother.cpp:3-80
 * --------------------------------------------------------------------- */
static void gs_forward(omat* m, double* x, const double* b, int nSweeps)
{
    const int* os = mat_owner_start(m);
    double* bPrime = (double*)xcalloc((size_t)m->n, sizeof(double));
    for (int sweep = 0; sweep < nSweeps; ++sweep) {
        for (int c = 0; c < m->n; ++c) bPrime[c] = b[c] - 0.0; /* b - interfaces (none) */
        int fEnd = os[0];
        for (int c = 0; c < m->n; ++c) {
            int fStart = fEnd;
            fEnd = os[c + 1];
            double curX = bPrime[c];
            for (int f = fStart; f < fEnd; ++f) curX -= m->upper[f] * x[m->u[f]];
            curX /= m->diag[c];
            for (int f = fStart; f < fEnd; ++f) bPrime[m->u[f]] -= m->lower[f] * curX;
            x[c] = curX;
        }
    }
    free(bPrime);
}

/* NEW (no reference counterpart; the reference sweeps forward only).
 * Backward sweep in reverse cell order with the same per-row formula as the
 * forward sweep: x_c = (b_c - sum_{faces f with u_f = c, ascending f}
 * lower_f x_{l_f} - sum_{faces f with l_f = c, ascending f} upper_f x_{u_f})
 * / D_c, where the upper neighbours already hold this sweep's values. */
static void gs_backward(omat* m, double* x, const double* b, int nSweeps)
{
    const int* os = mat_owner_start(m);
    const int* ls = mat_losort(m);
    int* lstart = (int*)xcalloc((size_t)m->n + 1, sizeof(int));
    for (int i = 0; i < m->nf; ++i) lstart[m->u[ls[i]] + 1]++;
    for (int c = 0; c < m->n; ++c) lstart[c + 1] += lstart[c];
    for (int sweep = 0; sweep < nSweeps; ++sweep) {
        for (int c = m->n - 1; c >= 0; --c) {
            double acc = b[c];
            for (int i = lstart[c]; i < lstart[c + 1]; ++i) {
                int f = ls[i];
                acc -= m->lower[f] * x[m->l[f]];
            }
            for (int f = os[c]; f < os[c + 1]; ++f) acc -= m->upper[f] * x[m->u[f]];
            x[c] = acc / m->diag[c];
        }
    }
    free(lstart);
}

void orc_gs(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
            const double* up, int symm, double* x, const double* b, int nSweeps)
{
    omat m = mat_view(n, nf, l, u, lo, d, up, symm);
    gs_forward(&m, x, b, nSweeps);
    mat_free_addr(&m);
}

void orc_gs_bwd(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
                const double* up, int symm, double* x, const double* b, int nSweeps)
{
    omat m = mat_view(n, nf, l, u, lo, d, up, symm);
    gs_backward(&m, x, b, nSweeps);
    mat_free_addr(&m);
}

/* ------------------------------------------------------------------------
 * Eigenvalue estimate: eigenDiagPCG.cpp:11-361
 * --------------------------------------------------------------------- */

/* diagPCGLoops, eigenDiagPCG.cpp:48-238 (mutates x) */
static void diag_pcg_loops(const omat* m, double* x, const double* b, const double* rD,
                           int nDiagPCGs, double* alphas, double* betas)
{
    int n = m->n;
    double* pA = (double*)xcalloc((size_t)n, sizeof(double));
    double* wA = (double*)xcalloc((size_t)n, sizeof(double));
    double* rA = (double*)xcalloc((size_t)n, sizeof(double));
    double wArA = GREAT_, wArAold;
    mat_spmv(m, x, wA);
    for (int c = 0; c < n; ++c) rA[c] = b[c] - wA[c];
    for (int it = 0; it < nDiagPCGs; ++it) {
        wArAold = wArA;
        wArA = 0.0;
        for (int c = 0; c < n; ++c) {
            wA[c] = rD[c] * rA[c];
            wArA += wA[c] * rA[c];
        }
        if (fabs(wArA) < VSMALL_) break;
        if (it == 0) {
            betas[it] = 0.0;
            for (int c = 0; c < n; ++c) pA[c] = wA[c];
        } else {
            double beta = wArA / wArAold;
            betas[it] = beta;
            for (int c = 0; c < n; ++c) pA[c] = wA[c] + beta * pA[c];
        }
        mat_spmv(m, pA, wA);
        double wApA = 0.0;
        for (int c = 0; c < n; ++c) wApA += wA[c] * pA[c];
        double alpha = wArA / wApA;
        alphas[it] = alpha;
        for (int c = 0; c < n; ++c) {
            x[c] += alpha * pA[c];
            rA[c] -= alpha * wA[c];
        }
    }
    free(pA);
    free(wA);
    free(rA);
}

/* computeMaxEig + computeValueForMatrix + determineEigRange + h14Sturm,
 * eigenDiagPCG.cpp:242-361 (tridiagonal Lanczos matrix, Sturm bisection).
 *
 * One departure, where the diagonal PCG stops early (wArA below VSMALL:
 * a one-cell system, a two-cell convection-diffusion system): the
 * reference still builds the tridiagonal matrix from all nDiagPCGs
 * iterations, the missing alphas are 0 and the matrix holds infinities;
 * its bisection then returns an artefact of them (0.99999237 for one cell)
 * or never ends (the two-cell case).  Here, as in the CUDA path, the
 * matrix stops at the first iteration that did not run (one row: 1 /
 * alpha_0; none: 1) and the bisection at 4096 halvings.  Whenever the
 * diagonal PCG runs all its iterations the result is the reference's, bit
 * for bit. */
static double compute_max_eig(const double* alphas, const double* betas, int nP)
{
    {
        int ran = 0;
        while (ran < nP && alphas[ran] != 0.0) ++ran;
        nP = ran;
    }
    if (nP < 2) return nP == 1 ? 1.0 / alphas[0] : 1.0;
    double* T = (double*)xcalloc((size_t)nP * (size_t)nP, sizeof(double));
#define T_(i, j) T[(size_t)(i) * (size_t)nP + (size_t)(j)]
    for (int i = 0; i < nP; ++i) {
        if (i == 0)
            T_(i, i) = 1.0 / alphas[i];
        else
            T_(i, i) = 1.0 / alphas[i] + betas[i] / alphas[i - 1];
        if (i < nP - 1) T_(i, i + 1) = sqrt(betas[i + 1]) / alphas[i];
        if (i > 0) T_(i, i - 1) = T_(i - 1, i);
    }
    double xBegin = 0.0, xEnd = 0.0, lambMax, lambMin;
    for (int i = 0; i < nP; ++i) {
        double Tr = (i == nP - 1) ? 0 : T_(i, i + 1);
        double Tl = (i == 0) ? 0 : T_(i, i - 1);
        lambMax = T_(i, i) + fabs(Tr) + fabs(Tl);
        lambMin = T_(i, i) - fabs(Tr) - fabs(Tl);
        xBegin = (xBegin >= lambMin) ? lambMin : xBegin;
        xEnd = (xEnd <= lambMax) ? lambMax : xEnd;
    }
    double* p = (double*)xcalloc((size_t)nP, sizeof(double));
    double xn;
    int halvings = 0;
    do {
        xn = (xBegin + xEnd) * 0.5;
        int s = 0;
        p[0] = xn - T_(0, 0);
        if (p[0] < 0) s = 1;
        p[1] = (xn - T_(1, 1)) * p[0] - pow(T_(0, 1), 2);
        if (p[1] * p[0] < 0) s++;
        for (int k = 2; k < nP; ++k) {
            p[k] = (xn - T_(k, k)) * p[k - 1] - pow(T_(k - 1, k), 2) * p[k - 2];
            if (p[k] * p[k - 1] < 0) s++;
        }
        if (s >= 1)
            xBegin = xn;
        else
            xEnd = xn;
    } while ((xEnd - xBegin) >= 0.00001 && ++halvings < 4096);
#undef T_
    free(p);
    free(T);
    return xn;
}

static double eigen_estimate(const omat* m, double* x, const double* b, int nDiagPCGs)
{
    double* rD = (double*)xcalloc((size_t)m->n, sizeof(double));
    double* al = (double*)xcalloc((size_t)nDiagPCGs, sizeof(double));
    double* be = (double*)xcalloc((size_t)nDiagPCGs, sizeof(double));
    diag_rD(m, rD);
    diag_pcg_loops(m, x, b, rD, nDiagPCGs, al, be);
    double e = compute_max_eig(al, be, nDiagPCGs);
    free(rD);
    free(al);
    free(be);
    return e;
}

double orc_eigen(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
                 const double* up, int symm, double* x, const double* b, int nDiagPCGs)
{
    omat m = mat_view(n, nf, l, u, lo, d, up, symm);
    return eigen_estimate(&m, x, b, nDiagPCGs);
}

/* ------------------------------------------------------------------------
 * Chebyshev smoother: chebySmoother.cpp:13-149, defaults chebySmoother.hpp:41-53
 * --------------------------------------------------------------------- */
typedef struct {
    int firstTime;
    double maxEigPCG;
} ocheby;

static void cheby_smooth(ocheby* cs, const omat* m, double* x, const double* b, int nSweeps)
{
    int n = m->n;
    if (cs->firstTime) {
        cs->maxEigPCG = eigen_estimate(m, x, b, 10);
        cs->firstTime = 0;
        return;
    }
    double* rD = (double*)xcalloc((size_t)n, sizeof(double));
    double* p = (double*)xcalloc((size_t)n, sizeof(double));
    double* w = (double*)xcalloc((size_t)n, sizeof(double));
    diag_rD(m, rD);
    double maxEig = cs->maxEigPCG * 1.1;
    double minEig = cs->maxEigPCG / 1.5;
    double delta = 2.0 / (maxEig - minEig);
    double theta = 0.5 * (maxEig + minEig);
    double s1 = theta * delta;
    double rhok = 1.0 / s1;
    mat_spmv(m, x, w);
    double Rtheta = 1.0 / theta;
    for (int c = 0; c < n; ++c) {
        w[c] = rD[c] * (b[c] - w[c]) * Rtheta;
        x[c] += w[c];
    }
    for (int sweep = 1; sweep < nSweeps; ++sweep) {
        double rhokp1 = 1.0 / (2.0 * s1 - rhok);
        double dtemp1 = rhokp1 * rhok;
        double dtemp2 = 2.0 * rhokp1 * delta;
        rhok = rhokp1;
        mat_spmv(m, x, p);
        for (int c = 0; c < n; ++c) {
            w[c] = dtemp1 * w[c] + dtemp2 * rD[c] * (b[c] - p[c]);
            x[c] += w[c];
        }
    }
    free(rD);
    free(p);
    free(w);
}

void orc_cheby(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
               const double* up, int symm, double* x, const double* b, int nSweeps, int nCalls)
{
    omat m = mat_view(n, nf, l, u, lo, d, up, symm);
    ocheby cs = {1, 0.0};
    for (int k = 0; k < nCalls; ++k) cheby_smooth(&cs, &m, x, b, nSweeps);
}

/* ------------------------------------------------------------------------
 * solverPerformance::checkConvergence, unapMatrixTest.cpp:3-31
 * --------------------------------------------------------------------- */
static int check_conv(double finalRes, double initRes, double tol, double relTol, int iter,
                      int minIter)
{
    return ((finalRes < tol || (relTol > SMALL_ && finalRes <= relTol * initRes)) &&
            iter >= minIter);
}

/* ------------------------------------------------------------------------
 * PCG::solve, PCG.cpp:35-183
 * --------------------------------------------------------------------- */
typedef void (*precond_fn)(void* ctx, const double* r, double* w);

typedef struct {
    int nIter, converged, singular;
    double initRes, finalRes;
} operf;

static operf pcg_core(const omat* A, precond_fn pf, void* pctx, double tol, double relTol,
                      int maxIter, int minIter, double* x, const double* b)
{
    int n = A->n;
    operf perf = {0, 0, 0, 0.0, 0.0};
    double* pA = (double*)xcalloc((size_t)n, sizeof(double));
    double* wA = (double*)xcalloc((size_t)n, sizeof(double));
    double* rA = (double*)xcalloc((size_t)n, sizeof(double));
    double wArA = GREAT_, wArAold;
    mat_spmv(A, x, wA);
    for (int c = 0; c < n; ++c) rA[c] = b[c] - wA[c];
    perf.initRes = norm_factor(n, rA);
    perf.finalRes = perf.initRes;
    do {
        wArAold = wArA;
        pf(pctx, rA, wA);
        wArA = vdot(n, wA, rA);
        perf.singular = !(fabs(wArA) > SMALL_); /* checkSingularity, unapMatrixTest.cpp:82-97 */
        if (perf.singular) break;
        if (perf.nIter == 0) {
            for (int c = 0; c < n; ++c) pA[c] = wA[c];
        } else {
            double beta = wArA / wArAold;
            for (int c = 0; c < n; ++c) pA[c] = wA[c] + beta * pA[c];
        }
        mat_spmv(A, pA, wA);
        double wApA = vdot(n, wA, pA);
        double alpha = wArA / wApA;
        for (int c = 0; c < n; ++c) {
            x[c] += alpha * pA[c];
            rA[c] -= alpha * wA[c];
        }
        perf.finalRes = norm_factor(n, rA);
    } while (++perf.nIter < maxIter &&
             !(perf.converged = check_conv(perf.finalRes, perf.initRes, tol, relTol,
                                           perf.nIter, minIter)));
    free(pA);
    free(wA);
    free(rA);
    return perf;
}

typedef struct {
    oprec* p;
    omat* m;
} prec_ctx;

static void prec_cb(void* ctx, const double* r, double* w)
{
    prec_ctx* c = (prec_ctx*)ctx;
    prec_apply(c->p, c->m, r, w);
}

static void put_perf(const operf* p, int* nIter, double* initRes, double* finalRes,
                     int* converged, int* singular)
{
    if (nIter) *nIter = p->nIter;
    if (initRes) *initRes = p->initRes;
    if (finalRes) *finalRes = p->finalRes;
    if (converged) *converged = p->converged;
    if (singular) *singular = p->singular;
}

void orc_pcg(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
             const double* up, int symm, int precond, double tol, double relTol, int maxIter,
             int minIter, double* x, const double* b, int* nIter, double* initRes,
             double* finalRes, int* converged, int* singular)
{
    omat m = mat_view(n, nf, l, u, lo, d, up, symm);
    oprec p = prec_make(precond, &m);
    prec_ctx ctx = {&p, &m};
    operf perf = pcg_core(&m, prec_cb, &ctx, tol, relTol, maxIter, minIter, x, b);
    put_perf(&perf, nIter, initRes, finalRes, converged, singular);
    free(p.rD);
    mat_free_addr(&m);
}

/* ------------------------------------------------------------------------
 * PBiCGStab::solve, PBiCGStab.cpp:45-459 (x86 branches)
 * --------------------------------------------------------------------- */
static operf pbicgstab_core(omat* A, oprec* P, double tol, double relTol, int maxIter,
                            int minIter, double* x, const double* b)
{
    int n = A->n;
    operf perf = {0, 0, 0, 0.0, 0.0};
    double* pA = (double*)xcalloc((size_t)n, sizeof(double));
    double* yA = (double*)xcalloc((size_t)n, sizeof(double));
    double* rA = (double*)xcalloc((size_t)n, sizeof(double));
    double* rA0 = (double*)xcalloc((size_t)n, sizeof(double));
    double* AyA = (double*)xcalloc((size_t)n, sizeof(double));
    double* sA = (double*)xcalloc((size_t)n, sizeof(double));
    double* zA = (double*)xcalloc((size_t)n, sizeof(double));
    double* tA = (double*)xcalloc((size_t)n, sizeof(double));
    mat_spmv(A, x, yA);
    for (int c = 0; c < n; ++c) {
        rA[c] = b[c] - yA[c];
        rA0[c] = rA[c];
    }
    perf.initRes = norm_factor(n, rA);
    perf.finalRes = perf.initRes;
    double rA0rA = 0, alpha = 0, omega = 0;
    do {
        double rA0rAold = rA0rA;
        rA0rA = vdot(n, rA0, rA);
        perf.singular = !(fabs(rA0rA) > SMALL_);
        if (perf.singular) break;
        if (perf.nIter == 0) {
            for (int c = 0; c < n; ++c) pA[c] = rA[c];
        } else {
            double beta = (rA0rA / rA0rAold) * (alpha / omega);
            for (int c = 0; c < n; ++c) pA[c] = rA[c] + beta * (pA[c] - omega * AyA[c]);
        }
        prec_apply(P, A, pA, yA);
        mat_spmv(A, yA, AyA);
        double rA0AyA = vdot(n, rA0, AyA);
        alpha = rA0rA / rA0AyA;
        for (int c = 0; c < n; ++c) sA[c] = rA[c] - alpha * AyA[c];
        perf.finalRes = norm_factor(n, sA);
        if ((perf.converged = check_conv(perf.finalRes, perf.initRes, tol, relTol,
                                         perf.nIter + 1, minIter))) {
            for (int c = 0; c < n; ++c) x[c] += alpha * yA[c];
            perf.nIter++;
            goto done;
        }
        prec_apply(P, A, sA, zA);
        mat_spmv(A, zA, tA);
        double tAtA = 0.0;
        for (int c = 0; c < n; ++c) tAtA += tA[c] * tA[c]; /* Vector::SumSqr */
        omega = vdot(n, tA, sA);
        omega /= tAtA;
        for (int c = 0; c < n; ++c) {
            x[c] += alpha * yA[c] + omega * zA[c];
            rA[c] = sA[c] - omega * tA[c];
        }
        perf.finalRes = norm_factor(n, rA);
    } while (++perf.nIter < maxIter &&
             !(perf.converged = check_conv(perf.finalRes, perf.initRes, tol, relTol,
                                           perf.nIter, minIter)));
done:
    free(pA);
    free(yA);
    free(rA);
    free(rA0);
    free(AyA);
    free(sA);
    free(zA);
    free(tA);
    return perf;
}

void orc_pbicgstab(int n, int nf, const int* l, const int* u, const double* lo,
                   const double* d, const double* up, int symm, int precond, double tol,
                   double relTol, int maxIter, int minIter, double* x, const double* b,
                   int* nIter, double* initRes, double* finalRes, int* converged,
                   int* singular)
{
    omat m = mat_view(n, nf, l, u, lo, d, up, symm);
    oprec p = prec_make(precond, &m);
    operf perf = pbicgstab_core(&m, &p, tol, relTol, maxIter, minIter, x, b);
    put_perf(&perf, nIter, initRes, finalRes, converged, singular);
    free(p.rD);
    mat_free_addr(&m);
}

/* ------------------------------------------------------------------------
 * Agglomeration hierarchy: lduAgglomerate.cpp, lduAgglomerationAddressing.cpp,
 * lduAgglomerateMatrix.cpp, lduAgglomeration.cpp
 * --------------------------------------------------------------------- */
typedef struct {
    int n, nf;
    int *l, *u;           /* coarse addressing (owned) */
    double *diag, *upper, *lower; /* lower == upper when symm */
    int* restrictAddr;    /* size of the finer level's cells */
    int* faceRestrict;    /* size of the finer level's faces */
    omat m;               /* view for kernels */
} olevel;

typedef struct {
    omat fine;
    int symm;
    int nLevels;
    olevel* lv; /* coarse levels 0..nLevels-1 */
} ohier;

/* pairwise lduAgglomeration::agglomerate, lduAgglomerate.cpp:94-271
 * (forward_ is always true: lduAgglomeration.cpp:3) */
static int* pairwise_agglomerate(int nFine, int nf, const int* l, const int* u,
                                 const double* w, int* nCoarseOut)
{
    int* off = (int*)xcalloc((size_t)nFine + 1, sizeof(int));
    int* cellFaces = (int*)xcalloc(2 * (size_t)nf, sizeof(int));
    int* cnt = (int*)xcalloc((size_t)nFine, sizeof(int));
    for (int f = 0; f < nf; ++f) cnt[u[f]]++;
    for (int f = 0; f < nf; ++f) cnt[l[f]]++;
    for (int c = 0; c < nFine; ++c) off[c + 1] = off[c] + cnt[c];
    memset(cnt, 0, sizeof(int) * (size_t)nFine);
    /* upper side first, then lower side (lduAgglomerate.cpp:53-71) */
    for (int f = 0; f < nf; ++f) cellFaces[off[u[f]] + cnt[u[f]]++] = f;
    for (int f = 0; f < nf; ++f) cellFaces[off[l[f]] + cnt[l[f]]++] = f;
    free(cnt);

    int* map = (int*)malloc(sizeof(int) * (size_t)(nFine ? nFine : 1));
    for (int c = 0; c < nFine; ++c) map[c] = -1;
    int nCoarse = 0;
    for (int c = 0; c < nFine; ++c) {
        if (map[c] >= 0) continue;
        int match = -1;
        double maxW = SMALL_;
        for (int k = off[c]; k < off[c + 1]; ++k) {
            int f = cellFaces[k];
            if (map[u[f]] < 0 && map[l[f]] < 0 && w[f] > maxW) {
                match = f;
                maxW = w[f];
            }
        }
        if (match >= 0) {
            map[u[match]] = nCoarse;
            map[l[match]] = nCoarse;
            nCoarse++;
        } else {
            int cmatch = -1;
            double cmax = SMALL_;
            for (int k = off[c]; k < off[c + 1]; ++k) {
                int f = cellFaces[k];
                if (w[f] > cmax) {
                    cmatch = f;
                    cmax = w[f];
                }
            }
            if (cmatch >= 0) {
                int a = map[u[cmatch]], b2 = map[l[cmatch]];
                map[c] = a > b2 ? a : b2;
            }
        }
    }
    for (int c = 0; c < nFine; ++c)
        if (map[c] < 0) map[c] = nCoarse++;
    free(off);
    free(cellFaces);
    *nCoarseOut = nCoarse;
    return map;
}

/* agglomerateLduAddressing, lduAgglomerationAddressing.cpp:8-178 (serial part) */
static void agglomerate_addressing(int nFineFaces, const int* l, const int* u,
                                   const int* restrictMap, int nCoarse, olevel* cl)
{
    int* faceRestrict = (int*)xcalloc((size_t)nFineFaces, sizeof(int));
    int* ccCount = (int*)xcalloc((size_t)nCoarse, sizeof(int));
    int* ccCap = (int*)xcalloc((size_t)nCoarse, sizeof(int));
    int** ccFaces = (int**)xcalloc((size_t)nCoarse, sizeof(int*));
    int* initNei = (int*)xcalloc((size_t)nFineFaces, sizeof(int));
    int nCoarseFaces = 0;
    for (int f = 0; f < nFineFaces; ++f) {
        int rmU = restrictMap[u[f]];
        int rmL = restrictMap[l[f]];
        if (rmU == rmL) {
            faceRestrict[f] = -(rmU + 1);
            continue;
        }
        int cOwn = rmU, cNei = rmL;
        if (rmU > rmL) {
            cOwn = rmL;
            cNei = rmU;
        }
        int found = 0;
        for (int i = 0; i < ccCount[cOwn]; ++i) {
            if (initNei[ccFaces[cOwn][i]] == cNei) {
                found = 1;
                faceRestrict[f] = ccFaces[cOwn][i];
                break;
            }
        }
        if (!found) {
            if (ccCount[cOwn] == ccCap[cOwn]) {
                ccCap[cOwn] = ccCap[cOwn] ? 2 * ccCap[cOwn] : 8;
                ccFaces[cOwn] = (int*)realloc(ccFaces[cOwn], sizeof(int) * (size_t)ccCap[cOwn]);
                if (!ccFaces[cOwn]) abort();
            }
            ccFaces[cOwn][ccCount[cOwn]++] = nCoarseFaces;
            initNei[nCoarseFaces] = cNei;
            faceRestrict[f] = nCoarseFaces;
            nCoarseFaces++;
        }
    }
    int* cOwner = (int*)xcalloc((size_t)nCoarseFaces, sizeof(int));
    int* cNeigh = (int*)xcalloc((size_t)nCoarseFaces, sizeof(int));
    int* cMap = (int*)xcalloc((size_t)nCoarseFaces, sizeof(int));
    int k = 0;
    for (int c = 0; c < nCoarse; ++c) {
        for (int i = 0; i < ccCount[c]; ++i) {
            cOwner[k] = c;
            cNeigh[k] = initNei[ccFaces[c][i]];
            cMap[ccFaces[c][i]] = k;
            k++;
        }
        free(ccFaces[c]);
    }
    for (int f = 0; f < nFineFaces; ++f)
        if (faceRestrict[f] >= 0) faceRestrict[f] = cMap[faceRestrict[f]];
    free(ccCount);
    free(ccCap);
    free(ccFaces);
    free(initNei);
    free(cMap);
    cl->n = nCoarse;
    cl->nf = nCoarseFaces;
    cl->l = cOwner;
    cl->u = cNeigh;
    cl->faceRestrict = faceRestrict;
}

/* restrictField, unapMatrix.hpp:378-407 */
static void restrict_field(int nFine, const int* map, const double* ff, int nCoarse, double* cf)
{
    for (int c = 0; c < nCoarse; ++c) cf[c] = 0;
    for (int i = 0; i < nFine; ++i) cf[map[i]] += ff[i];
}

/* agglomerateMatrix, lduAgglomerateMatrix.cpp:3-104 */
static void agglomerate_matrix(const omat* fine, olevel* cl, int symm)
{
    cl->diag = (double*)xcalloc((size_t)cl->n, sizeof(double));
    cl->upper = (double*)xcalloc((size_t)cl->nf, sizeof(double));
    restrict_field(fine->n, cl->restrictAddr, fine->diag, cl->n, cl->diag);
    if (!symm) {
        cl->lower = (double*)xcalloc((size_t)cl->nf, sizeof(double));
        for (int f = 0; f < fine->nf; ++f) {
            int cf = cl->faceRestrict[f];
            if (cf >= 0) {
                if (cl->l[cf] == cl->restrictAddr[fine->l[f]]) {
                    cl->upper[cf] += fine->upper[f];
                    cl->lower[cf] += fine->lower[f];
                } else if (cl->u[cf] == cl->restrictAddr[fine->l[f]]) {
                    cl->upper[cf] += fine->lower[f];
                    cl->lower[cf] += fine->upper[f];
                } else {
                    abort(); /* inconsistent addressing: the reference exits */
                }
            } else {
                cl->diag[-1 - cf] += fine->upper[f] + fine->lower[f];
            }
        }
    } else {
        cl->lower = cl->upper;
        for (int f = 0; f < fine->nf; ++f) {
            int cf = cl->faceRestrict[f];
            if (cf >= 0)
                cl->upper[cf] += fine->upper[f];
            else
                cl->diag[-1 - cf] += 2 * fine->upper[f];
        }
    }
    cl->m = mat_view(cl->n, cl->nf, cl->l, cl->u, cl->lower, cl->diag, cl->upper, symm);
}

/* lduAgglomeration::agglomerate(weights), lduAgglomerate.cpp:4-91 and
 * continueAgglomerating, lduAgglomeration.cpp:26-43 */
static ohier* hier_build(omat fine, const double* weights, int nCoarsest, int maxLevels,
                         int stopRule)
{
    ohier* h = (ohier*)xcalloc(1, sizeof(ohier));
    h->fine = fine;
    h->symm = fine.symm;
    if (maxLevels <= 0) maxLevels = 50;
    if (nCoarsest <= 0) nCoarsest = 50;
    h->lv = (olevel*)xcalloc((size_t)maxLevels, sizeof(olevel));
    const double* w = weights;
    double* wOwned = NULL;
    int nCreated = 0;
    while (nCreated < maxLevels - 1) {
        const omat* fm = nCreated == 0 ? &h->fine : &h->lv[nCreated - 1].m;
        if (stopRule == 1 && fm->n <= nCoarsest) break;
        int nCoarse = -1;
        int* map = pairwise_agglomerate(fm->n, fm->nf, fm->l, fm->u, w, &nCoarse);
        int keep = stopRule == 1 ? (nCoarse < fm->n) : (nCoarse >= nCoarsest);
        if (!keep) {
            free(map);
            break;
        }
        olevel* cl = &h->lv[nCreated];
        cl->restrictAddr = map;
        agglomerate_addressing(fm->nf, fm->l, fm->u, map, nCoarse, cl);
        agglomerate_matrix(fm, cl, h->symm);
        /* restrictFaceField of the weights, unapMatrix.hpp:441-475 */
        double* cw = (double*)xcalloc((size_t)cl->nf, sizeof(double));
        for (int f = 0; f < fm->nf; ++f)
            if (cl->faceRestrict[f] >= 0) cw[cl->faceRestrict[f]] += w[f];
        free(wOwned);
        wOwned = cw;
        w = cw;
        nCreated++;
    }
    free(wOwned);
    h->nLevels = nCreated;
    return h;
}

static void hier_free(ohier* h)
{
    if (!h) return;
    for (int k = 0; k < h->nLevels; ++k) {
        olevel* cl = &h->lv[k];
        free(cl->l);
        free(cl->u);
        free(cl->diag);
        if (cl->lower != cl->upper) free(cl->lower);
        free(cl->upper);
        free(cl->restrictAddr);
        free(cl->faceRestrict);
        mat_free_addr(&cl->m);
    }
    mat_free_addr(&h->fine);
    free(h->lv);
    free(h);
}

void* orc_hier_create(int n, int nf, const int* l, const int* u, const double* lo,
                      const double* d, const double* up, int symm, const double* weights,
                      int nCoarsest, int maxLevels, int stopRule)
{
    return hier_build(mat_view(n, nf, l, u, lo, d, up, symm), weights, nCoarsest, maxLevels,
                      stopRule);
}

int orc_hier_nlevels(void* hv) { return ((ohier*)hv)->nLevels; }
int orc_hier_ncells(void* hv, int level) { return ((ohier*)hv)->lv[level].n; }
int orc_hier_nfaces(void* hv, int level) { return ((ohier*)hv)->lv[level].nf; }

void orc_hier_addressing(void* hv, int level, int* restrictAddr, int* faceRestrict,
                         int* coarseLower, int* coarseUpper)
{
    ohier* h = (ohier*)hv;
    olevel* cl = &h->lv[level];
    const omat* fm = level == 0 ? &h->fine : &h->lv[level - 1].m;
    memcpy(restrictAddr, cl->restrictAddr, sizeof(int) * (size_t)fm->n);
    memcpy(faceRestrict, cl->faceRestrict, sizeof(int) * (size_t)fm->nf);
    memcpy(coarseLower, cl->l, sizeof(int) * (size_t)cl->nf);
    memcpy(coarseUpper, cl->u, sizeof(int) * (size_t)cl->nf);
}

void orc_hier_coeffs(void* hv, int level, double* diag, double* upper, double* lower)
{
    olevel* cl = &((ohier*)hv)->lv[level];
    memcpy(diag, cl->diag, sizeof(double) * (size_t)cl->n);
    memcpy(upper, cl->upper, sizeof(double) * (size_t)cl->nf);
    if (lower) memcpy(lower, cl->lower, sizeof(double) * (size_t)cl->nf);
}

void orc_hier_destroy(void* hv) { hier_free((ohier*)hv); }

/* Face weights of mgsolversolve_ agglType 1, fortranInterface.cpp:383-395:
 * |upper| / sqrt(sum upper^2). */
void orc_mg_weights(int nf, const double* up, double* weights)
{
    double s = 0.0;
    for (int f = 0; f < nf; ++f) s += up[f] * up[f];
    double avg = sqrt(s);
    for (int f = 0; f < nf; ++f) weights[f] = fabs(up[f]) / avg;
}

/* ------------------------------------------------------------------------
 * MGSolver: MG.cpp, MGSolve.cpp, Vcycle.cpp, scalingFactor.cpp,
 * solveCoarsestLevel.cpp
 * --------------------------------------------------------------------- */
typedef struct {
    ohier* h;
    int smootherType; /* 1 GS, 2 Cheby */
    ocheby* cheby;    /* one per smoother slot (finest + coarse 0..L-1) */
    int nPre, nPost, nFinest, scaleCorr;
} omg;

static const omat* mg_level_mat(omg* g, int lv) { return &g->h->lv[lv].m; }

static void mg_smooth(omg* g, int slot, omat* m, double* x, const double* b, int nSweeps)
{
    if (g->smootherType == 2)
        cheby_smooth(&g->cheby[slot], m, x, b, nSweeps);
    else
        gs_forward(m, x, b, nSweeps);
}

/* scalingFactor.cpp:11-65 */
static double scaling_factor(const omat* A, double* Acf, double* field, const double* source)
{
    mat_spmv(A, field, Acf);
    double s0 = 0.0, s1 = 0.0;
    for (int i = 0; i < A->n; ++i) {
        s0 += source[i] * field[i];
        s1 += Acf[i] * field[i];
        field[i] += (source[i] - Acf[i]) / A->diag[i];
    }
    return s0 / (s1 + SMALL_);
}

static void prolong_field(int nFine, const int* map, const double* cf, double* ff)
{
    for (int i = 0; i < nFine; ++i) ff[i] = cf[map[i]];
}

/* solveCoarsestLevel.cpp:10-55 */
static void mg_solve_coarsest(omg* g, double* corr, const double* src)
{
    int L = g->h->nLevels - 1;
    omat* m = &g->h->lv[L].m;
    for (int c = 0; c < m->n; ++c) corr[c] = 0;
    if (m->symm) {
        oprec p = prec_make(2, m);
        prec_ctx ctx = {&p, m};
        pcg_core(m, prec_cb, &ctx, 0.0, 1.0e-2, 100, 0, corr, src);
        free(p.rD);
    } else {
        oprec p = prec_make(3, m);
        pbicgstab_core(m, &p, 0.0, 1.0e-2, 100, 0, corr, src);
        free(p.rD);
    }
}

/* MGSolver::Vcycle, Vcycle.cpp:27-332 */
static void mg_vcycle(omg* g, double* psi, const double* source, double* Apsi,
                      double* finestCorrection, double* finestResidual, double** corr,
                      double** src)
{
    ohier* h = g->h;
    int L = h->nLevels - 1;
    if (L >= 0) restrict_field(h->fine.n, h->lv[0].restrictAddr, finestResidual, h->lv[0].n, src[0]);
    for (int lv = 0; lv < L; ++lv) {
        omat* A = &h->lv[lv].m;
        int n = A->n;
        if (g->nPre) {
            for (int c = 0; c < n; ++c) corr[lv][c] = 0.0;
            mg_smooth(g, lv + 1, A, corr[lv], src[lv], g->nPre + lv);
            double* ACf = (double*)xcalloc((size_t)n, sizeof(double));
            if (g->scaleCorr && lv < L - 1) {
                double sf = scaling_factor(A, ACf, corr[lv], src[lv]);
                for (int c = 0; c < n; ++c) corr[lv][c] *= sf;
            }
            mat_spmv(A, corr[lv], ACf);
            for (int c = 0; c < n; ++c) src[lv][c] -= ACf[c];
            free(ACf);
        }
        restrict_field(n, h->lv[lv + 1].restrictAddr, src[lv], h->lv[lv + 1].n, src[lv + 1]);
    }
    if (L >= 0) mg_solve_coarsest(g, corr[L], src[L]);
    for (int lv = L - 1; lv >= 0; --lv) {
        omat* A = &h->lv[lv].m;
        int n = A->n;
        double* pre = (double*)xcalloc((size_t)n, sizeof(double));
        if (g->nPre) memcpy(pre, corr[lv], sizeof(double) * (size_t)n);
        prolong_field(n, h->lv[lv + 1].restrictAddr, corr[lv + 1], corr[lv]);
        if (g->scaleCorr && lv < L - 1) {
            double* ACf = (double*)xcalloc((size_t)n, sizeof(double));
            double sf = scaling_factor(A, ACf, corr[lv], src[lv]);
            for (int c = 0; c < n; ++c) corr[lv][c] *= sf;
            free(ACf);
        }
        if (g->nPre)
            for (int c = 0; c < n; ++c) corr[lv][c] += pre[c];
        free(pre);
        mg_smooth(g, lv + 1, A, corr[lv], src[lv], g->nPost + lv);
    }
    int nF = h->fine.n;
    if (L >= 0) prolong_field(nF, h->lv[0].restrictAddr, corr[0], finestCorrection);
    if (g->scaleCorr) {
        double fsf = scaling_factor(&h->fine, Apsi, finestCorrection, finestResidual);
        for (int i = 0; i < nF; ++i) psi[i] += fsf * finestCorrection[i];
    } else {
        for (int i = 0; i < nF; ++i) psi[i] += finestCorrection[i];
    }
    mg_smooth(g, 0, &h->fine, psi, source, g->nFinest);
}

/* MGSolver::solve, MGSolve.cpp:17-187 */
static operf mg_solve(omg* g, double tol, double relTol, int maxIter, int minIter, double* x,
                      const double* b)
{
    ohier* h = g->h;
    int n = h->fine.n;
    operf perf = {0, 0, 0, 0.0, 0.0};
    double* Apsi = (double*)xcalloc((size_t)n, sizeof(double));
    double* fc = (double*)xcalloc((size_t)n, sizeof(double));
    double* fr = (double*)xcalloc((size_t)n, sizeof(double));
    mat_spmv(&h->fine, x, Apsi);
    for (int c = 0; c < n; ++c) fr[c] = b[c] - Apsi[c];
    perf.initRes = norm_factor(n, fr);
    perf.finalRes = perf.initRes;
    if (!check_conv(perf.finalRes, perf.initRes, tol, relTol, perf.nIter, minIter)) {
        int nl = h->nLevels;
        double** corr = (double**)xcalloc((size_t)(nl ? nl : 1), sizeof(double*));
        double** src = (double**)xcalloc((size_t)(nl ? nl : 1), sizeof(double*));
        for (int k = 0; k < nl; ++k) {
            corr[k] = (double*)xcalloc((size_t)h->lv[k].n, sizeof(double));
            src[k] = (double*)xcalloc((size_t)h->lv[k].n, sizeof(double));
        }
        do {
            mg_vcycle(g, x, b, Apsi, fc, fr, corr, src);
            mat_spmv(&h->fine, x, Apsi);
            for (int c = 0; c < n; ++c) fr[c] = b[c] - Apsi[c];
            perf.finalRes = norm_factor(n, fr);
        } while (++perf.nIter < maxIter &&
                 !(perf.converged = check_conv(perf.finalRes, perf.initRes, tol, relTol,
                                               perf.nIter, minIter)));
        for (int k = 0; k < nl; ++k) {
            free(corr[k]);
            free(src[k]);
        }
        free(corr);
        free(src);
    } else {
        perf.converged = 1;
    }
    free(Apsi);
    free(fc);
    free(fr);
    return perf;
}

void orc_mg(int n, int nf, const int* l, const int* u, const double* lo, const double* d,
            const double* up, int symm, const double* weights, int nCoarsest, int maxLevels,
            int smootherType, int nPre, int nPost, int nFinest, int scaleCorr, double tol,
            double relTol, int maxIter, int minIter, double* x, const double* b, int* nIter,
            double* initRes, double* finalRes, int* converged, int* nLevels)
{
    omg g;
    g.h = hier_build(mat_view(n, nf, l, u, lo, d, up, symm), weights, nCoarsest, maxLevels, 0);
    g.smootherType = smootherType == 2 ? 2 : 1;
    g.nPre = nPre >= 0 ? nPre : 0;
    g.nPost = nPost >= 0 ? nPost : 2;
    g.nFinest = nFinest >= 0 ? nFinest : 2;
    g.scaleCorr = scaleCorr >= 0 ? (scaleCorr != 0) : (symm != 0); /* MG.cpp:3-19 */
    int slots = g.h->nLevels ? g.h->nLevels : 1;
    g.cheby = (ocheby*)xcalloc((size_t)slots, sizeof(ocheby));
    for (int i = 0; i < slots; ++i) g.cheby[i].firstTime = 1;
    operf perf = mg_solve(&g, tol, relTol, maxIter, minIter, x, b);
    put_perf(&perf, nIter, initRes, finalRes, converged, NULL);
    if (nLevels) *nLevels = g.h->nLevels;
    (void)mg_level_mat;
    free(g.cheby);
    hier_free(g.h);
}

/* ------------------------------------------------------------------------
 * NEW: dense SPD inverse for the coarsest level.
 * Cholesky A = L L^T (column by column), L^-1 by forward substitution, then
 * A^-1 = L^-T L^-1 with every sum taken in ascending index order.
 * --------------------------------------------------------------------- */
int orc_dense_spd_inverse(int n, const double* A, double* inv)
{
    double* L = (double*)xcalloc((size_t)n * (size_t)n, sizeof(double));
    double* Li = (double*)xcalloc((size_t)n * (size_t)n, sizeof(double));
#define IX(i, j) ((size_t)(i) * (size_t)n + (size_t)(j))
    int ok = 0;
    for (int j = 0; j < n && ok == 0; ++j) {
        double s = A[IX(j, j)];
        for (int k = 0; k < j; ++k) s -= L[IX(j, k)] * L[IX(j, k)];
        if (!(s > 0.0)) {
            ok = -1;
            break;
        }
        double djj = sqrt(s);
        L[IX(j, j)] = djj;
        for (int i = j + 1; i < n; ++i) {
            double t = A[IX(i, j)];
            for (int k = 0; k < j; ++k) t -= L[IX(i, k)] * L[IX(j, k)];
            L[IX(i, j)] = t / djj;
        }
    }
    if (ok == 0) {
        for (int j = 0; j < n; ++j) {
            Li[IX(j, j)] = 1.0 / L[IX(j, j)];
            for (int i = j + 1; i < n; ++i) {
                double t = 0.0;
                for (int k = j; k < i; ++k) t += L[IX(i, k)] * Li[IX(k, j)];
                Li[IX(i, j)] = -t / L[IX(i, i)];
            }
        }
        for (int i = 0; i < n; ++i) {
            for (int j = 0; j <= i; ++j) {
                double t = 0.0;
                for (int k = i; k < n; ++k) t += Li[IX(k, i)] * Li[IX(k, j)];
                inv[IX(i, j)] = t;
                inv[IX(j, i)] = t;
            }
        }
    }
#undef IX
    free(L);
    free(Li);
    return ok;
}

/* ------------------------------------------------------------------------
 * NEW: AMG as a fixed symmetric PCG preconditioner.
 *
 * V-cycle on levels 0..L (0 = input matrix, k >= 1 = coarse level k-1 of the
 * reference agglomeration):
 *   level k < L:  x = 0; nPre forward GS sweeps; r = b - A x (reference SpMV
 *                 order); b' = restrict(r); e = V(k+1, b'); x += prolong(e);
 *                 nPost backward GS sweeps.
 *   level L:      x = Ainv b, Ainv the dense inverse above; each row is
 *                 summed in chunks of ORC_DENSE_CHUNK columns, each chunk in
 *                 ascending order from 0, the chunk sums added in order from
 *                 0 (orc_dense_row).
 * precision 1 runs every level matrix, vector and sweep in FP32 (values
 * rounded from FP64), with the coarsest product in FP64.
 *
 * smoother 1 replaces the sweeps of levels k >= chebyFrom by the reference's
 * Chebyshev iteration (chebySmoother.cpp:44-148) of degree chebyDegree
 * before and after the coarse correction:
 *   from x = 0:   w = rD b Rtheta;  x = w
 *   from x != 0:  w = rD (b - A x) Rtheta;  x += w
 *   step j >= 1:  w = d1_j w + d2_j rD (b - A x);  x += w
 * rD = 1 / diag, A x in the reference SpMV order, the coefficients from the
 * level's eigenvalue estimate lambda as in chebySmoother.cpp:62-108 with
 * [lambda / eigRatio, 1.1 lambda].  lambda is estimated once at setup by
 * the reference's diagonal-PCG + Lanczos + Sturm bisection
 * (eigenDiagPCG.cpp:11-361) from x = 0 and b = orc_eig_start, on the FP64
 * level matrix; the same polynomial before and after keeps the V-cycle
 * symmetric, so it stays a fixed PCG preconditioner (the reference's first
 * call, which only estimates and leaves x changed, would not be).  FP32
 * levels use rD = 1.0f / diag32 and the coefficients rounded to float.
 * --------------------------------------------------------------------- */
typedef struct {
    int n, nf;
    const int *l, *u;
    float *diag, *upper; /* FP32 copies (symmetric) */
    int* ownerStart;
    int* losort;
    int* lstart;
} fmat;

typedef struct {
    ohier* h;
    orc_amg_params p;
    double* lam;       /* per smoothed level: eigenvalue estimate (Chebyshev) */
    int nLv;           /* total levels incl. fine */
    const omat** A;    /* per level FP64 view */
    fmat* F;           /* per level FP32 copy (precision 1) */
    double* Ainv;      /* coarsest dense inverse */
    int nc;
    double **x, **b, **r; /* FP64 work per level */
    float **xf, **bf, **rf;
} oamg;

static void fmat_build(fmat* f, const omat* m)
{
    f->n = m->n;
    f->nf = m->nf;
    f->l = m->l;
    f->u = m->u;
    f->diag = (float*)xcalloc((size_t)m->n, sizeof(float));
    f->upper = (float*)xcalloc((size_t)m->nf, sizeof(float));
    for (int c = 0; c < m->n; ++c) f->diag[c] = (float)m->diag[c];
    for (int k = 0; k < m->nf; ++k) f->upper[k] = (float)m->upper[k];
    f->ownerStart = (int*)xcalloc((size_t)m->n + 1, sizeof(int));
    calc_owner_start(m->n, m->nf, m->l, f->ownerStart);
    f->losort = (int*)xcalloc((size_t)m->nf, sizeof(int));
    calc_losort(m->n, m->nf, m->u, f->losort);
    f->lstart = (int*)xcalloc((size_t)m->n + 1, sizeof(int));
    for (int i = 0; i < m->nf; ++i) f->lstart[m->u[f->losort[i]] + 1]++;
    for (int c = 0; c < m->n; ++c) f->lstart[c + 1] += f->lstart[c];
}

static void fmat_free(fmat* f)
{
    free(f->diag);
    free(f->upper);
    free(f->ownerStart);
    free(f->losort);
    free(f->lstart);
}

/* FP32 forms of gs_forward / gs_backward / mat_spmv with identical orders */
static void fgs_sweep(const fmat* m, float* x, const float* b, int backward)
{
    for (int k = 0; k < m->n; ++k) {
        int c = backward ? m->n - 1 - k : k;
        float acc = b[c];
        for (int i = m->lstart[c]; i < m->lstart[c + 1]; ++i) {
            int f = m->losort[i];
            acc -= m->upper[f] * x[m->l[f]];
        }
        for (int f = m->ownerStart[c]; f < m->ownerStart[c + 1]; ++f)
            acc -= m->upper[f] * x[m->u[f]];
        x[c] = acc / m->diag[c];
    }
}

static void fspmv(const fmat* m, const float* x, float* y)
{
    for (int c = 0; c < m->n; ++c) y[c] = 0.0f;
    for (int c = 0; c < m->n; ++c) y[c] += m->diag[c] * x[c];
    for (int f = 0; f < m->nf; ++f) {
        y[m->u[f]] += m->upper[f] * x[m->l[f]];
        y[m->l[f]] += m->upper[f] * x[m->u[f]];
    }
}

static const int* amg_restrict_map(oamg* g, int k) { return g->h->lv[k].restrictAddr; }

/* splitmix64 (Steele, Lea, Flood 2014), the start vector's hash */
double orc_eig_start(long long c)
{
    unsigned long long z = (unsigned long long)c + 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

/* Chebyshev coefficients, chebySmoother.cpp:62-108: Rtheta for the first
 * step and (d1, d2) of steps 1..deg-1 */
static void amg_cheb_coeffs(double lam, double ratio, int deg, double* Rtheta, double* d1,
                            double* d2)
{
    double maxEig = lam * 1.1;
    double minEig = lam / ratio;
    double delta = 2.0 / (maxEig - minEig);
    double theta = 0.5 * (maxEig + minEig);
    double s1 = theta * delta;
    double rhok = 1.0 / s1;
    *Rtheta = 1.0 / theta;
    for (int k = 1; k < deg; ++k) {
        double rhokp1 = 1.0 / (2.0 * s1 - rhok);
        d1[k] = rhokp1 * rhok;
        d2[k] = 2.0 * rhokp1 * delta;
        rhok = rhokp1;
    }
}

#define AMG_MAX_DEGREE 16

static int amg_is_cheby(const oamg* g, int k)
{
    return g->p.smoother == 1 && k >= g->p.chebyFrom;
}

static double amg_ratio(const oamg* g) { return g->p.eigRatio > 0 ? g->p.eigRatio : 1.5; }

/* eigenDiagPCG.cpp:11-361 from x = 0, b = orc_eig_start: a breakdown
 * (|wArA| < VSMALL) ends the Lanczos matrix at the iterations done */
static double amg_level_eig(const omat* m)
{
    int n = m->n;
    double* x = (double*)xcalloc((size_t)n, sizeof(double));
    double* b = (double*)xcalloc((size_t)n, sizeof(double));
    double* rD = (double*)xcalloc((size_t)n, sizeof(double));
    double al[10] = {0}, be[10] = {0};
    for (int c = 0; c < n; ++c) b[c] = orc_eig_start(c);
    diag_rD(m, rD);
    diag_pcg_loops(m, x, b, rD, 10, al, be);
    int nP = 0;
    while (nP < 10 && al[nP] != 0.0) ++nP;
    double lam = nP >= 2 ? compute_max_eig(al, be, nP) : (nP == 1 ? 1.0 / al[0] : 1.0);
    free(x);
    free(b);
    free(rD);
    return lam;
}

/* the Chebyshev chain of one level in FP64 (w: n-vector scratch) */
static void cheb_chain64(const omat* A, double lam, double ratio, int deg, double* x,
                         const double* b, double* w, int fromZero)
{
    int n = A->n;
    double Rth, d1[AMG_MAX_DEGREE], d2[AMG_MAX_DEGREE];
    amg_cheb_coeffs(lam, ratio, deg, &Rth, d1, d2);
    double* p = (double*)xcalloc((size_t)n, sizeof(double));
    if (fromZero) {
        for (int c = 0; c < n; ++c) {
            double rD = 1.0 / A->diag[c];
            double wi = rD * b[c] * Rth;
            w[c] = wi;
            x[c] = wi;
        }
    } else {
        mat_spmv(A, x, p);
        for (int c = 0; c < n; ++c) {
            double rD = 1.0 / A->diag[c];
            double wi = rD * (b[c] - p[c]) * Rth;
            w[c] = wi;
            x[c] = x[c] + wi;
        }
    }
    for (int j = 1; j < deg; ++j) {
        mat_spmv(A, x, p);
        for (int c = 0; c < n; ++c) {
            double rD = 1.0 / A->diag[c];
            double wi = d1[j] * w[c] + d2[j] * rD * (b[c] - p[c]);
            w[c] = wi;
            x[c] = x[c] + wi;
        }
    }
    free(p);
}

static void amg_cheby64(oamg* g, int k, double* x, const double* b, int fromZero)
{
    cheb_chain64(g->A[k], g->lam[k], amg_ratio(g), g->p.chebyDegree, x, b, g->r[k], fromZero);
}

void orc_cheby_chain(int n, int nf, const int* l, const int* u, const double* lo,
                     const double* d, const double* up, int symm, double lam, double ratio,
                     int degree, double* x, const double* b, int fromZero)
{
    omat m = mat_view(n, nf, l, u, lo, d, up, symm);
    double* w = (double*)xcalloc((size_t)n, sizeof(double));
    if (degree < 1 || degree > AMG_MAX_DEGREE) degree = 3;
    cheb_chain64(&m, lam, ratio, degree, x, b, w, fromZero);
    free(w);
}

static void fspmv(const fmat* m, const float* x, float* y);

static void amg_cheby32(oamg* g, int k, float* x, const float* b, int fromZero)
{
    const fmat* A = &g->F[k];
    int n = A->n, deg = g->p.chebyDegree;
    double Rth, d1[AMG_MAX_DEGREE], d2[AMG_MAX_DEGREE];
    amg_cheb_coeffs(g->lam[k], amg_ratio(g), deg, &Rth, d1, d2);
    const float Rf = (float)Rth;
    float* w = g->rf[k];
    float* p = (float*)xcalloc((size_t)n, sizeof(float));
    if (fromZero) {
        for (int c = 0; c < n; ++c) {
            float rD = 1.0f / A->diag[c];
            float wi = rD * b[c] * Rf;
            w[c] = wi;
            x[c] = wi;
        }
    } else {
        fspmv(A, x, p);
        for (int c = 0; c < n; ++c) {
            float rD = 1.0f / A->diag[c];
            float wi = rD * (b[c] - p[c]) * Rf;
            w[c] = wi;
            x[c] = x[c] + wi;
        }
    }
    for (int j = 1; j < deg; ++j) {
        const float d1f = (float)d1[j], d2f = (float)d2[j];
        fspmv(A, x, p);
        for (int c = 0; c < n; ++c) {
            float rD = 1.0f / A->diag[c];
            float wi = d1f * w[c] + d2f * rD * (b[c] - p[c]);
            w[c] = wi;
            x[c] = x[c] + wi;
        }
    }
    free(p);
}

/* Row i of the coarsest product: the columns in chunks of ORC_DENSE_CHUNK,
 * each chunk summed in ascending order from 0, then the chunk sums added in
 * chunk order from 0.  (A chunked sum keeps the dependency chain short on
 * the GPU, where chunks are summed by separate threads.) */
#define ORC_DENSE_CHUNK 64
static double orc_dense_row(const double* Ainv, int n, int i, const double* b)
{
    double t = 0.0;
    for (int j0 = 0; j0 < n; j0 += ORC_DENSE_CHUNK) {
        const int j1 = j0 + ORC_DENSE_CHUNK < n ? j0 + ORC_DENSE_CHUNK : n;
        double p = 0.0;
        for (int j = j0; j < j1; ++j) p += Ainv[(size_t)i * (size_t)n + (size_t)j] * b[j];
        t += p;
    }
    return t;
}

static void amg_vcycle64(oamg* g, int k)
{
    int L = g->nLv - 1;
    double* x = g->x[k];
    const double* b = g->b[k];
    if (k == L) {
        int n = g->nc;
        for (int i = 0; i < n; ++i) x[i] = orc_dense_row(g->Ainv, n, i, b);
        return;
    }
    omat* A = (omat*)g->A[k];
    int n = A->n;
    const int cheb = amg_is_cheby(g, k);
    if (cheb) {
        amg_cheby64(g, k, x, b, 1);
    } else {
        for (int c = 0; c < n; ++c) x[c] = 0.0;
        if (g->p.nPre > 0) gs_forward(A, x, b, g->p.nPre);
    }
    mat_spmv(A, x, g->r[k]);
    for (int c = 0; c < n; ++c) g->r[k][c] = b[c] - g->r[k][c];
    restrict_field(n, amg_restrict_map(g, k), g->r[k], g->A[k + 1]->n, g->b[k + 1]);
    amg_vcycle64(g, k + 1);
    const int* map = amg_restrict_map(g, k);
    for (int c = 0; c < n; ++c) x[c] += g->x[k + 1][map[c]];
    if (cheb)
        amg_cheby64(g, k, x, b, 0);
    else if (g->p.nPost > 0)
        gs_backward(A, x, b, g->p.nPost);
}

static void amg_vcycle32(oamg* g, int k)
{
    int L = g->nLv - 1;
    float* x = g->xf[k];
    const float* b = g->bf[k];
    if (k == L) {
        int n = g->nc;
        double* bd = (double*)xcalloc((size_t)n, sizeof(double));
        for (int j = 0; j < n; ++j) bd[j] = (double)b[j];
        for (int i = 0; i < n; ++i) x[i] = (float)orc_dense_row(g->Ainv, n, i, bd);
        free(bd);
        return;
    }
    const fmat* A = &g->F[k];
    int n = A->n;
    const int cheb = amg_is_cheby(g, k);
    if (cheb) {
        amg_cheby32(g, k, x, b, 1);
    } else {
        for (int c = 0; c < n; ++c) x[c] = 0.0f;
        for (int s = 0; s < g->p.nPre; ++s) fgs_sweep(A, x, b, 0);
    }
    float* r = g->rf[k];
    fspmv(A, x, r);
    for (int c = 0; c < n; ++c) r[c] = b[c] - r[c];
    const int* map = amg_restrict_map(g, k);
    int nC = g->A[k + 1]->n;
    float* bc = g->bf[k + 1];
    for (int c = 0; c < nC; ++c) bc[c] = 0.0f;
    for (int i = 0; i < n; ++i) bc[map[i]] += r[i];
    amg_vcycle32(g, k + 1);
    for (int c = 0; c < n; ++c) x[c] += g->xf[k + 1][map[c]];
    if (cheb)
        amg_cheby32(g, k, x, b, 0);
    else
        for (int s = 0; s < g->p.nPost; ++s) fgs_sweep(A, x, b, 1);
}

void* orc_amg_create(int n, int nf, const int* l, const int* u, const double* d,
                     const double* up, const orc_amg_params* p)
{
    oamg* g = (oamg*)xcalloc(1, sizeof(oamg));
    g->p = *p;
    double* w = (double*)xcalloc((size_t)nf, sizeof(double));
    orc_mg_weights(nf, up, w);
    g->h = hier_build(mat_view(n, nf, l, u, NULL, d, up, 1), w,
                      p->nCoarsest > 0 ? p->nCoarsest : 1000, p->maxLevels > 0 ? p->maxLevels : 50,
                      1);
    free(w);
    g->nLv = g->h->nLevels + 1;
    g->A = (const omat**)xcalloc((size_t)g->nLv, sizeof(omat*));
    g->A[0] = &g->h->fine;
    for (int k = 1; k < g->nLv; ++k) g->A[k] = &g->h->lv[k - 1].m;
    const omat* C = g->A[g->nLv - 1];
    g->nc = C->n;
    double* dense = (double*)xcalloc((size_t)g->nc * (size_t)g->nc, sizeof(double));
    for (int c = 0; c < C->n; ++c) dense[(size_t)c * (size_t)C->n + (size_t)c] = C->diag[c];
    for (int f = 0; f < C->nf; ++f) {
        dense[(size_t)C->l[f] * (size_t)C->n + (size_t)C->u[f]] += C->upper[f];
        dense[(size_t)C->u[f] * (size_t)C->n + (size_t)C->l[f]] += C->lower[f];
    }
    g->Ainv = (double*)xcalloc((size_t)g->nc * (size_t)g->nc, sizeof(double));
    orc_dense_spd_inverse(g->nc, dense, g->Ainv);
    free(dense);
    g->x = (double**)xcalloc((size_t)g->nLv, sizeof(double*));
    g->b = (double**)xcalloc((size_t)g->nLv, sizeof(double*));
    g->r = (double**)xcalloc((size_t)g->nLv, sizeof(double*));
    g->xf = (float**)xcalloc((size_t)g->nLv, sizeof(float*));
    g->bf = (float**)xcalloc((size_t)g->nLv, sizeof(float*));
    g->rf = (float**)xcalloc((size_t)g->nLv, sizeof(float*));
    for (int k = 0; k < g->nLv; ++k) {
        int nk = g->A[k]->n;
        g->x[k] = (double*)xcalloc((size_t)nk, sizeof(double));
        g->b[k] = (double*)xcalloc((size_t)nk, sizeof(double));
        g->r[k] = (double*)xcalloc((size_t)nk, sizeof(double));
        if (p->precision == 1) {
            g->xf[k] = (float*)xcalloc((size_t)nk, sizeof(float));
            g->bf[k] = (float*)xcalloc((size_t)nk, sizeof(float));
            g->rf[k] = (float*)xcalloc((size_t)nk, sizeof(float));
        }
    }
    if (p->precision == 1) {
        g->F = (fmat*)xcalloc((size_t)g->nLv, sizeof(fmat));
        for (int k = 0; k < g->nLv - 1; ++k) fmat_build(&g->F[k], g->A[k]);
    }
    g->lam = (double*)xcalloc((size_t)g->nLv, sizeof(double));
    if (g->p.smoother == 1) {
        if (g->p.chebyDegree < 1 || g->p.chebyDegree > AMG_MAX_DEGREE) g->p.chebyDegree = 3;
        for (int k = 0; k < g->nLv - 1; ++k)
            if (amg_is_cheby(g, k)) g->lam[k] = amg_level_eig(g->A[k]);
    }
    return g;
}

void orc_amg_eigs(void* hv, double* lam)
{
    oamg* g = (oamg*)hv;
    for (int k = 0; k < g->nLv - 1; ++k) lam[k] = g->lam[k];
}

void orc_amg_set_eigs(void* hv, const double* lam)
{
    oamg* g = (oamg*)hv;
    for (int k = 0; k < g->nLv - 1; ++k) g->lam[k] = lam[k];
}

int orc_amg_nlevels(void* hv) { return ((oamg*)hv)->nLv; }
int orc_amg_ncells(void* hv, int level) { return ((oamg*)hv)->A[level]->n; }

void orc_amg_coarse_inverse(void* hv, double* inv)
{
    oamg* g = (oamg*)hv;
    memcpy(inv, g->Ainv, sizeof(double) * (size_t)g->nc * (size_t)g->nc);
}

void orc_amg_vcycle(void* hv, const double* r, double* z)
{
    oamg* g = (oamg*)hv;
    int n = g->A[0]->n;
    if (g->p.precision == 1) {
        for (int c = 0; c < n; ++c) g->bf[0][c] = (float)r[c];
        amg_vcycle32(g, 0);
        for (int c = 0; c < n; ++c) z[c] = (double)g->xf[0][c];
    } else {
        memcpy(g->b[0], r, sizeof(double) * (size_t)n);
        amg_vcycle64(g, 0);
        memcpy(z, g->x[0], sizeof(double) * (size_t)n);
    }
}

static void amg_prec_cb(void* ctx, const double* r, double* w) { orc_amg_vcycle(ctx, r, w); }

/* PCG.cpp:35-183 with the V-cycle as preconditioner.  flexible: beta =
 * z_k.(r_k - r_{k-1}) / z_{k-1}.r_{k-1}, using r_{k-1} = r_k + alpha q. */
/* Bench helper (reference arm): the iteration cap of later solves. */
void orc_amg_set_max_iter(void* hv, int maxIter)
{
    ((oamg*)hv)->p.maxIter = maxIter;
}

void orc_amg_pcg(void* hv, double* x, const double* b, int* nIter, double* initRes,
                 double* finalRes, double* trueRes, int* converged)
{
    oamg* g = (oamg*)hv;
    const omat* A = g->A[0];
    int n = A->n;
    const orc_amg_params* p = &g->p;
    double* pA = (double*)xcalloc((size_t)n, sizeof(double));
    double* wA = (double*)xcalloc((size_t)n, sizeof(double));
    double* zA = (double*)xcalloc((size_t)n, sizeof(double));
    double* rA = (double*)xcalloc((size_t)n, sizeof(double));
    operf perf = {0, 0, 0, 0.0, 0.0};
    double wArA = GREAT_, wArAold, alpha = 0.0;
    int first = 1;
    mat_spmv(A, x, wA);
    for (int c = 0; c < n; ++c) rA[c] = b[c] - wA[c];
    perf.initRes = norm_factor(n, rA);
    perf.finalRes = perf.initRes;
    for (;;) {
        do {
            wArAold = wArA;
            amg_prec_cb(g, rA, zA);
            wArA = vdot(n, zA, rA);
            if (!(fabs(wArA) > SMALL_)) {
                perf.singular = 1;
                break;
            }
            if (first) {
                for (int c = 0; c < n; ++c) pA[c] = zA[c];
                first = 0;
            } else {
                double beta;
                if (p->flexible) {
                    double zq = vdot(n, zA, wA);
                    beta = (-alpha * zq) / wArAold;
                } else {
                    beta = wArA / wArAold;
                }
                for (int c = 0; c < n; ++c) pA[c] = zA[c] + beta * pA[c];
            }
            mat_spmv(A, pA, wA);
            double wApA = vdot(n, wA, pA);
            alpha = wArA / wApA;
            for (int c = 0; c < n; ++c) {
                x[c] += alpha * pA[c];
                rA[c] -= alpha * wA[c];
            }
            perf.finalRes = norm_factor(n, rA);
        } while (++perf.nIter < p->maxIter &&
                 !(perf.converged = check_conv(perf.finalRes, perf.initRes, p->tol, p->relTol,
                                               perf.nIter, p->minIter)));
        /* true residual; restart from it if the recurrence drifted */
        mat_spmv(A, x, wA);
        for (int c = 0; c < n; ++c) wA[c] = b[c] - wA[c];
        double tr = norm_factor(n, wA);
        if (trueRes) *trueRes = tr;
        if (perf.singular || !perf.converged || perf.nIter >= p->maxIter ||
            check_conv(tr, perf.initRes, p->tol, p->relTol, perf.nIter, p->minIter))
            break;
        memcpy(rA, wA, sizeof(double) * (size_t)n);
        perf.finalRes = tr;
        perf.converged = 0;
        first = 1;
        wArA = GREAT_;
    }
    if (nIter) *nIter = perf.nIter;
    if (initRes) *initRes = perf.initRes;
    if (finalRes) *finalRes = perf.finalRes;
    if (converged) *converged = perf.converged;
    free(pA);
    free(wA);
    free(zA);
    free(rA);
}

void orc_amg_destroy(void* hv)
{
    oamg* g = (oamg*)hv;
    if (!g) return;
    for (int k = 0; k < g->nLv; ++k) {
        free(g->x[k]);
        free(g->b[k]);
        free(g->r[k]);
        free(g->xf[k]);
        free(g->bf[k]);
        free(g->rf[k]);
    }
    if (g->F) {
        for (int k = 0; k < g->nLv - 1; ++k) fmat_free(&g->F[k]);
        free(g->F);
    }
    free(g->x);
    free(g->b);
    free(g->r);
    free(g->xf);
    free(g->bf);
    free(g->rf);
    free(g->Ainv);
    free(g->lam);
    free((void*)g->A);
    hier_free(g->h);
    free(g);
}
