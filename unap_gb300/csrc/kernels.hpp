// Launch wrappers for the sm_103a kernels (implemented in kernels.cu).
// All vectors are in a level's internal (wavefront-major) order.
#pragma once

#include "unap_internal.hpp"

namespace unapgpu {

template <class T>
struct Rows {
    int n = 0;
    const int* sliceOff = nullptr;
    const int* rowInfo = nullptr;
    const int* col = nullptr;
    const T* val = nullptr;   // A[row][col]
    const T* valT = nullptr;  // transposed coefficient (== val when symmetric)
    const T* diag = nullptr;
    int wide = 0;  // rows average more than 8 entries: 16-entry load chunks
};

Rows<double> rows64(const Level& L);
Rows<float> rows32(const Level& L);

// columns per chunk of the AMG coarsest product's row sums (each chunk
// summed in order, then the chunk sums in order)
constexpr int kDenseChunk = 64;

// y = A x; with a reduction spec, also sums y.dotWith (dotWith may be x).
// fused: products and sums as fused multiply-adds (the mixed solve's outer
// loop); otherwise the reference's separate roundings.
template <class T>
void k_spmv(const Exec& ex, const Rows<T>& A, const T* x, T* y, const T* dotWith, RSpec red,
            Gate g, bool fused = false);

// r = b - A x; with a reduction spec, sums r.r (sum0)
template <class T>
void k_residual(const Exec& ex, const Rows<T>& A, const T* x, const T* b, T* r, RSpec red,
                Gate g);

// One Gauss-Seidel pass over rows [r0, r1) (one wavefront), in place on x.
// skipUpper: x is known to be zero above this row (first forward sweep).
template <class T>
void k_gs_rows(const Exec& ex, const Rows<T>& A, T* x, const T* b, int r0, int r1, bool skipUpper,
               Gate g);

// Whole forward / backward Gauss-Seidel sweeps over all wavefronts.
template <class T>
void gs_sweep(const Exec& ex, const Level& L, const Rows<T>& A, T* x, const T* b, bool backward,
              bool xIsZero, Gate g);

// DIC (dilu=false) or DILU factorisation: rD = 1 / factored diagonal.
void dic_factor(const Exec& ex, const Level& L, bool dilu, double* dfac, double* rD);

// w = M^-1 r for M = DIC/DILU with rD; with a reduction spec, sums w.r over
// all wavefronts (backward sweep launches) and finalizes on the last one.
void dic_apply(const Exec& ex, const Level& L, bool dilu, const double* rD, const double* r,
               double* w, const RedPool* pool, int site, KState* st, int fin, Gate g);

// w = rD * r (Diag) or w = r (rD == nullptr); sums w.r.
void diag_apply(const Exec& ex, int n, const double* rD, const double* r, double* w, RSpec red,
                Gate g);

// PCG pieces (fused: fused multiply-adds, as for k_spmv).
// p = useBeta ? w + beta p : w
void k_pcg_direction(const Exec& ex, int n, const double* w, double* p, const KState* st, Gate g,
                     bool fused = false);
// x += alpha p, r -= alpha q; sums r.r
void k_pcg_update(const Exec& ex, int n, double* x, double* r, const double* p, const double* q,
                  RSpec red, Gate g, bool fused = false);
// sums a.b (and c.d when c != nullptr)
void k_dot2(const Exec& ex, int n, const double* a, const double* b, const double* c,
            const double* d, RSpec red, Gate g, bool fused = false);

// PBiCGStab pieces (PBiCGStab.cpp:155-456)
void k_bicg_init(const Exec& ex, int n, const double* b, const double* Ax, double* r, double* r0,
                 RSpec red);
void k_bicg_direction(const Exec& ex, int n, const double* r, const double* Ay, double* p,
                      const KState* st, Gate g);
void k_bicg_s(const Exec& ex, int n, const double* r, const double* Ay, double* s, RSpec red,
              Gate g);
void k_bicg_update(const Exec& ex, int n, double* x, double* r, const double* y, const double* z,
                   const double* s, const double* t, const double* r0, RSpec red, Gate g);

// permutation between reference and internal order:
// to_internal: out[i] = in[perm[i]];  to_reference: out[perm[i]] = in[i]
template <class T>
void k_to_internal(const Exec& ex, int n, const int* perm, const T* in, T* out);
template <class T>
void k_to_reference(const Exec& ex, int n, const int* perm, const T* in, T* out);

// AMG transfer: coarse[C] = sum over children (ascending) of fine[child]
template <class T>
void k_restrict(const Exec& ex, int nCoarse, const int* childStart, const int* child,
                const T* fine, T* coarse, Gate g);
// fine[i] += coarse[cmap[i]]
template <class T>
void k_prolong_add(const Exec& ex, int nFine, const int* cmap, const T* coarse, T* fine, Gate g);
// x = Minv b with Minv column-major n x n FP64, each row summed over ascending columns
template <class T>
void k_dense_apply(const Exec& ex, int n, const double* MinvColMajor, const T* b, const int* gather,
                   T* x, Gate g);

// elementwise helpers
template <class T>
void k_fill(const Exec& ex, long long n, T* x, T v);
void k_d2f(const Exec& ex, int n, const double* in, float* out);
void k_f2d(const Exec& ex, int n, const float* in, double* out);
void k_axpy_f2d(const Exec& ex, int n, const float* in, double* out);  // out = (double)in

// MGSolver pieces (scalingFactor.cpp, Vcycle.cpp)
// field scaling: sum0 = source.field, sum1 = Acf.field, then
// field += (source - Acf) / D;  finalize stores sf in st->beta (FIN_STORE + host)
template <class T>
void k_scaling_sums(const Exec& ex, int n, const T* source, const T* Acf, T* field, const T* D,
                    RSpec red, Gate g);
template <class T>
void k_axpby(const Exec& ex, int n, T a, const T* x, T b, T* y, Gate g);  // y = a x + b y

// Wavefront Gauss-Seidel launches use programmatic dependent launch (the
// next wavefront's kernel launches while the previous one runs and loads its
// matrix data before waiting); 0 turns it off.  Returns the previous value.
int set_wave_pdl(int on);
// this host thread's setting, over the process-wide one: 0 off, 1 on, -1
// follow the process-wide one; returns the previous override
int set_thread_wave_pdl(int mode);
bool wave_pdl();
// Wavefront Gauss-Seidel grids: 1 (default) one row per thread, 0 a
// grid-stride loop over at most SMs x 8 CTAs.  Returns the previous value.
int set_wave_grid(int oneRowPerThread);

}  // namespace unapgpu
