// Persistent cooperative "step program" executor for whole Krylov solves.
//
// The host compiles one Krylov iteration (with its preconditioner, e.g. a
// full AMG V-cycle) into a list of Steps; a single cooperative launch runs
// the list repeatedly until the solver state says done.  Steps on large
// levels run on every CTA, separated by a grid barrier; consecutive steps on
// small levels form a segment that CTA 0 runs alone with block barriers,
// followed by one grid barrier.  Reductions write per-block partials that
// every CTA sums in block order after the barrier, so all CTAs hold the same
// scalars (alpha, beta, residual norm, convergence) without a host round
// trip.  Grid barriers spin with an iteration bound and report a timeout in
// MegaStatus instead of hanging.
#pragma once

#include <vector>

#include "kernels.hpp"

namespace unapgpu {

enum StepOp : int {
    ST_GS = 1,        // Gauss-Seidel rows [r0, r1) of level lvl; f0 = skipUpper
    ST_RESID,         // r = b - A x over level lvl (c = r, a = x, b = b)
    ST_RESTRICT,      // coarse[C] = sum children (a = fine, c = coarse, i0 = start, i1 = child)
    ST_PROLONG_ADD,   // fine[i] += coarse[cmap[i]] (a = coarse, c = fine, i0 = cmap)
    ST_DENSE,         // x = Minv b (e = Minv column-major, a = b, c = x), n = r1
    ST_FILL0,         // c[0:n] = 0
    ST_D2F,           // (float)c = (double)a
    ST_F2D,           // (double)c = (float)a
    ST_DIC_FWD,       // rows [r0,r1): w = rD r - sum_low rD coef w  (a = r, c = w, e = rD, d = coef)
    ST_DIC_BWD,       // rows [r0,r1): w -= sum_up rD val w (c = w, e = rD); partial red += w.r (a = r)
    ST_DIAG,          // w = rD r (or w = r when e == null); partial red += w.r
    ST_SPMV_DOT,      // q = A p (lvl); partial red += q.p   (a = p, c = q)
    ST_DOT2,          // partial red += a.b (and red+1 += c.d when c != null)
    ST_PCG_DIR,       // p = useBeta ? z + beta p : z   (a = z, c = p)
    ST_PCG_UPD,       // x += alpha p; r -= alpha q; partial red += r.r (c = x, d = r, a = p, b = q)
    ST_SCALAR,        // finalize: f0 = operation (Fin), reads partial slots red..red+1
                      // summed over r1 blocks (r1 < 0: every block of the grid)
    ST_RESID_NORM,    // r = b - A x; partial red += r.r (FP64, lvl)
    ST_COPY,          // c = a (double)
    ST_SLEEP,         // CTA 0 thread 0 sleeps f0 microseconds (bounded; barrier self-test)
    ST_CHEB,          // Chebyshev step on level lvl (cheby.hpp): a = x in, c = x out,
                      // b = b, d = w; f0 = first step from x; k1, k2 coefficients
    ST_CHEB0,         // first Chebyshev step from x = 0: c = x, d = w, b = b (first set
                      // to (float) e when e != null); k1 = Rtheta; diag of level lvl
    ST_RESTRICT_CHEB0,// ST_RESTRICT fused with the coarse level's ST_CHEB0: d = x,
                      // e = w of the coarse level lvl; k1 = its Rtheta
    ST_PROLONG_TO,    // c[i] = b[i] + a[i0[i]] (out-of-place prolongation)
};

struct Step {
    int op = 0;
    int prec = 0;    // 0 double, 1 float
    int single = 0;  // 1: CTA 0 runs it inside a block segment
    int lvl = 0;
    int r0 = 0, r1 = 0;
    int f0 = 0;      // op flag (skipUpper / finalize code)
    int red = -1;    // partial slot
    const void* a = nullptr;
    const void* b = nullptr;
    void* c = nullptr;
    const void* d = nullptr;
    const void* e = nullptr;
    const int* i0 = nullptr;
    const int* i1 = nullptr;
    double k1 = 0, k2 = 0;  // Chebyshev coefficients
    double bytes = 0;  // algorithmic DRAM bytes of the step (host bookkeeping)
};

// Algorithmic bytes of a row range of a Gauss-Seidel / residual pass: per
// cell b, x read, x write, diag; per face one value and two int32 addresses
// (each LDU array touched once).  FP32 rows: 16 B/cell + 12 B/face; FP64:
// 32 B/cell + 16 B/face.  A wavefront of `rows` of an n-row level carries
// rows/n of the level's nf faces.
inline double sweep_bytes(int rows, int n, int nf, bool fp32)
{
    const double cb = fp32 ? 16.0 : 32.0, fb = fp32 ? 12.0 : 16.0;
    return rows * cb + (n > 0 ? (double)rows / n * nf * fb : 0.0);
}

// Algorithmic bytes of a Chebyshev step over a level: per cell diag, b, x
// gathered once, x write, w write and (after the first step) w read; per
// face one value and two int32 addresses.
inline double cheb_bytes(int n, int nf, bool fp32, bool readW)
{
    const double e = fp32 ? 4.0 : 8.0;
    return n * e * (readW ? 6.0 : 5.0) + (double)nf * (fp32 ? 12.0 : 16.0);
}

struct LevelRows {
    Rows<double> r64;
    Rows<float> r32;
};

struct MegaStatus {
    unsigned count, gen;  // grid barrier
    int timeout;          // a barrier wait hit its bound
    int pad;
};

struct MegaArgs {
    const Step* steps = nullptr;
    int nSteps = 0;
    int nInit = 0;             // steps [0, nInit) run once before the iterations
    const LevelRows* levels = nullptr;
    KState* st = nullptr;
    MegaStatus* status = nullptr;
    double* partials = nullptr;  // [nSlots][gridDim]
    int nSlots = 0;
    int maxLoops = 0;            // iteration bound of this launch
    int skipInit = 0;            // start with the iteration steps
    unsigned spinLimit = 0;      // barrier wait bound (polls of ~32 ns)
};

class MegaRunner {
public:
    MegaRunner();
    ~MegaRunner();
    // program: steps[0, nInit) once, then steps[nInit, end) per iteration
    void setProgram(const std::vector<Step>& steps, int nInit, const std::vector<LevelRows>& lv,
                    int nSlots, cudaStream_t s);
    // runs until st->done (or maxLoops iterations); returns false on a
    // barrier timeout
    bool run(KState* d_st, int maxLoops, cudaStream_t s, bool skipInit = false,
             unsigned spinLimit = 0);
    int gridBlocks() const { return blocks; }
    int threads() const;

private:
    DevArray<Step> d_steps;
    DevArray<LevelRows> d_levels;
    DevArray<double> d_partials;
    DevArray<MegaStatus> d_status;
    MegaStatus* h_status = nullptr;
    int nSteps = 0, nInit = 0, nSlots = 0, blocks = 0;
};

// Rows of a level are small enough for the single-CTA segments.
bool mega_single_level(int nRows);

}  // namespace unapgpu
