// Host-array entry points of the C ABI (declared in include/unap_cuda.h):
// the matrix-level calls on host vectors in the caller's cell order, the
// reference's COO/face reordering calls, and the agglomeration handle.  They
// are the layer under the C++ class API (include/unap/*.hpp): every call
// copies its vectors to the device, runs the kernels there and copies the
// result back; nothing is computed on the host except integer reordering of
// caller arrays.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <vector>

#include "amg.hpp"
#include "capi_handles.hpp"
#include "cheby.hpp"
#include "../../include/unap_cuda.h"

using namespace unapgpu;

namespace {

// an inner entry point failed: its status and message are passed on as is
struct Status {
    int rc;
};

void call(int rc)
{
    if (rc != UNAP_CUDA_OK) throw Status{rc};
}

template <class F>
int guarded(F&& f)
{
    try {
        f();
        return UNAP_CUDA_OK;
    } catch (const Status& s) {
        return s.rc;
    } catch (const CudaError& e) {
        set_last_error(e.what());
        return UNAP_CUDA_ECUDA;
    } catch (const std::bad_alloc&) {
        set_last_error("out of host memory");
        return UNAP_CUDA_ENOMEM;
    } catch (const std::invalid_argument& e) {
        set_last_error(e.what());
        return UNAP_CUDA_EINVAL;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return UNAP_CUDA_EINTERNAL;
    }
}

// Device copies of host vectors (reference cell order) for one call.
struct Staged {
    Matrix& A;
    size_t n;
    DevArray<double> a, b;
    explicit Staged(MatHandle* h) : A(h->get()), n((size_t)A.n()), a(n), b(n) {}
    void in(DevArray<double>& d, const double* host)
    {
        if (!host) throw std::invalid_argument("null vector");
        UNAP_CK(cudaMemcpyAsync(d.p, host, n * sizeof(double), cudaMemcpyHostToDevice, A.stream));
    }
    void out(double* host, const DevArray<double>& d)
    {
        if (!host) throw std::invalid_argument("null vector");
        UNAP_CK(cudaMemcpyAsync(host, d.p, n * sizeof(double), cudaMemcpyDeviceToHost, A.stream));
        UNAP_CK(cudaStreamSynchronize(A.stream));
    }
};

void put_stats(const SolveStats& s, unap_cuda_stats* o)
{
    if (!o) return;
    o->nIterations = s.nIter;
    o->converged = s.converged;
    o->singular = s.singular;
    o->status = s.status;
    o->initialResidual = s.initRes;
    o->finalResidual = s.finalRes;
    o->trueResidual = s.trueRes;
    o->seconds = s.seconds;
    o->algorithmicBytes = s.bytes;
}

// ---- reordering (matrixConversion.cpp:38-222), 0-based -----------------

void check_entries(const int* row, const int* col, int n, int size)
{
    if (n < 0 || size < 0) throw std::invalid_argument("negative size");
    if (size && (!row || !col)) throw std::invalid_argument("null index array");
    for (int i = 0; i < size; ++i)
        if (row[i] < 0 || row[i] >= n || col[i] < 0 || col[i] >= n)
            throw std::invalid_argument("entry index out of range");
}

// Position of every entry after grouping by row (rows in ascending order)
// and ordering each row by column: the row's start plus the number of
// entries of the row with a smaller column.  A repeated (row, column) pair
// would give two entries one position (the reference leaves that
// undefined): rejected.
std::vector<int> row_major_positions(const int* row, const int* col, int n, int size)
{
    check_entries(row, col, n, size);
    std::vector<int> start((size_t)n + 1, 0);
    for (int i = 0; i < size; ++i) start[(size_t)row[i] + 1]++;
    for (int c = 0; c < n; ++c) start[(size_t)c + 1] += start[(size_t)c];
    // the entries of each row, in input order
    std::vector<int> fill(start.begin(), start.end() - 1), members((size_t)size);
    for (int i = 0; i < size; ++i) members[(size_t)fill[(size_t)row[i]]++] = i;
    std::vector<int> pos((size_t)size);
    for (int r = 0; r < n; ++r) {
        const int b = start[(size_t)r], e = start[(size_t)r + 1];
        for (int p = b; p < e; ++p) {
            const int i = members[(size_t)p];
            int rank = 0;
            for (int q = b; q < e; ++q) {
                const int j = members[(size_t)q];
                if (col[i] > col[j]) ++rank;
                else if (col[i] == col[j] && i != j)
                    throw std::invalid_argument("repeated (row, column) entry");
            }
            pos[(size_t)i] = b + rank;
        }
    }
    return pos;
}

void reorder_coo0(double* val, int* row, int* col, int n, int size)
{
    std::vector<int> pos = row_major_positions(row, col, n, size);
    std::vector<int> r2((size_t)size), c2((size_t)size);
    std::vector<double> v2((size_t)size);
    for (int i = 0; i < size; ++i) {
        const size_t p = (size_t)pos[(size_t)i];
        r2[p] = row[i];
        c2[p] = col[i];
        v2[p] = val[i];
    }
    std::copy(r2.begin(), r2.end(), row);
    std::copy(c2.begin(), c2.end(), col);
    std::copy(v2.begin(), v2.end(), val);
}

void reorder_uface0(int* row, int* col, int n, int size, int* newOrder)
{
    std::vector<int> pos = row_major_positions(row, col, n, size);
    std::vector<int> r2((size_t)size), c2((size_t)size);
    for (int i = 0; i < size; ++i) {
        const size_t p = (size_t)pos[(size_t)i];
        newOrder[i] = (int)p;
        r2[p] = row[i];
        c2[p] = col[i];
    }
    std::copy(r2.begin(), r2.end(), row);
    std::copy(c2.begin(), c2.end(), col);
}

// stable grouping by column (matrixConversion.cpp:180-222)
void reorder_lface0(int* row, int* col, int n, int size, int* newOrder)
{
    check_entries(row, col, n, size);
    std::vector<int> start((size_t)n + 1, 0);
    for (int i = 0; i < size; ++i) start[(size_t)col[i] + 1]++;
    for (int c = 0; c < n; ++c) start[(size_t)c + 1] += start[(size_t)c];
    std::vector<int> r2((size_t)size), c2((size_t)size);
    for (int i = 0; i < size; ++i) {
        const int p = start[(size_t)col[i]]++;
        newOrder[i] = p;
        r2[(size_t)p] = row[i];
        c2[(size_t)p] = col[i];
    }
    std::copy(r2.begin(), r2.end(), row);
    std::copy(c2.begin(), c2.end(), col);
}

// val[newOrder[i]] = old val[i] (matrixConversion.cpp:101-112); newOrder
// must be a permutation of 0 .. size-1
void reorder_value0(double* val, const int* newOrder, int size)
{
    if (size < 0) throw std::invalid_argument("negative size");
    std::vector<char> seen((size_t)size, 0);
    for (int i = 0; i < size; ++i) {
        if (newOrder[i] < 0 || newOrder[i] >= size || seen[(size_t)newOrder[i]])
            throw std::invalid_argument("newOrder is not a permutation");
        seen[(size_t)newOrder[i]] = 1;
    }
    std::vector<double> old(val, val + size);
    for (int i = 0; i < size; ++i) val[newOrder[i]] = old[(size_t)i];
}

// ---- agglomeration handle (lduAgglomeration.cpp, lduAgglomerate.cpp) ----

struct AgglHandle {
    static constexpr unsigned kMagic = 0x41474c31u;  // "AGL1"
    unsigned magic = kMagic;
    int nFine = 0, nfFine = 0;
    std::vector<CoarseHost> levels;
    ~AgglHandle() { magic = 0; }
};

AgglHandle* aggl_from(long int h)
{
    AgglHandle* a = reinterpret_cast<AgglHandle*>(h);
    if (!a || a->magic != AgglHandle::kMagic)
        throw std::invalid_argument("invalid agglomeration handle");
    return a;
}

}  // namespace

extern "C" {

int unap_cuda_matrix_set_values(long int handle, const double* diag, const double* upper,
                                const double* lower)
{
    return guarded([&] {
        if (!diag || !upper) throw std::invalid_argument("null coefficient array");
        mat_from(handle)->setValues(diag, upper, lower);
    });
}

int unap_cuda_spmv_host(long int handle, const double* x, double* y)
{
    return guarded([&] {
        Staged S(mat_from(handle));
        S.in(S.a, x);
        call(unap_cuda_spmv(handle, S.a.p, S.b.p));
        S.out(y, S.b);
    });
}

int unap_cuda_precondition_host(long int handle, int precond, const double* r, double* w)
{
    return guarded([&] {
        Staged S(mat_from(handle));
        S.in(S.a, r);
        call(unap_cuda_precondition(handle, precond, S.a.p, S.b.p));
        S.out(w, S.b);
    });
}

int unap_cuda_precond_rD(long int handle, int precond, double* rD)
{
    return guarded([&] {
        MatHandle* h = mat_from(handle);
        Matrix& A = h->get();
        const int n = A.n();
        if (!rD) throw std::invalid_argument("null rD");
        if (precond == 1) {
            // lduDiagPrecond.cpp:13-41
            for (int c = 0; c < n; ++c) rD[c] = 1.0 / A.host.diag[(size_t)c];
            return;
        }
        if (precond != 2 && precond != 3) throw std::invalid_argument("precond must be 1, 2 or 3");
        if (!A.L->sweepable)
            throw std::invalid_argument("DIC/DILU need faces oriented lowerAddr < upperAddr and sorted by owner");
        Exec ex{A.stream, device_max_blocks()};
        DevArray<double> dfac((size_t)n), ri((size_t)n), ro((size_t)n);
        dic_factor(ex, *A.L, precond == 3, dfac.p, ri.p);
        k_to_reference<double>(ex, n, A.L->d_perm.p, ri.p, ro.p);
        UNAP_CK(cudaMemcpyAsync(rD, ro.p, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost,
                                A.stream));
        UNAP_CK(cudaStreamSynchronize(A.stream));
    });
}

int unap_cuda_gauss_seidel_host(long int handle, double* x, const double* b, int nSweeps,
                                int backward)
{
    return guarded([&] {
        Staged S(mat_from(handle));
        S.in(S.a, x);
        S.in(S.b, b);
        call(unap_cuda_gauss_seidel(handle, S.a.p, S.b.p, nSweeps, backward));
        S.out(x, S.a);
    });
}

int unap_cuda_cheby_smooth_host(long int handle, double* x, const double* b, int nSweeps,
                                double* maxEig, int* estimated)
{
    return guarded([&] {
        if (!maxEig || !estimated) throw std::invalid_argument("null smoother state");
        MatHandle* h = mat_from(handle);
        Matrix& A = h->get();
        const int n = A.n();
        Exec ex{A.stream, device_max_blocks()};
        Staged S(h);
        S.in(S.a, x);
        S.in(S.b, b);
        DevArray<double> xi((size_t)n), bi((size_t)n), t((size_t)n), w((size_t)n);
        k_to_internal<double>(ex, n, A.L->d_perm.p, S.a.p, xi.p);
        k_to_internal<double>(ex, n, A.L->d_perm.p, S.b.p, bi.p);
        const Rows<double> R = rows64(*A.L);
        double* out = xi.p;
        if (!*estimated) {
            // chebySmoother.cpp:22-42: the first call estimates the largest
            // eigenvalue with 10 diagonal-PCG iterations on (x, b), leaving
            // x as those iterations change it
            DevArray<double> rD((size_t)n), pA((size_t)n);
            DevArray<EigState> es(1);
            RedPool pool;
            pool.init(2, ex.maxBlocks, 1, A.stream);
            k_reciprocal(ex, n, R.diag, rD.p);
            EigState st{};
            st.wArA = 1.0e37;  // GREAT, eigenDiagPCG.cpp:75
            UNAP_CK(cudaMemcpyAsync(es.p, &st, sizeof st, cudaMemcpyHostToDevice, A.stream));
            eig_diag_pcg(ex, R, rD.p, xi.p, bi.p, t.p, w.p, pA.p, es.p,
                         pool.site(0, nullptr, FIN_RES_ONLY), pool.site(1, nullptr, FIN_RES_ONLY),
                         10);
            k_eig_sturm(ex, es.p, 10);
            UNAP_CK(cudaMemcpyAsync(&st, es.p, sizeof st, cudaMemcpyDeviceToHost, A.stream));
            UNAP_CK(cudaStreamSynchronize(A.stream));
            *maxEig = st.maxEig;
            *estimated = 1;
        } else if (nSweeps > 0) {
            // chebySmoother.cpp:44-148 on [maxEig / 1.5, 1.1 maxEig]
            if (nSweeps > kChebyMaxDegree) throw std::invalid_argument("at most 16 sweeps");
            double Rth, d1[kChebyMaxDegree], d2[kChebyMaxDegree];
            cheby_coeffs(*maxEig, 1.5, nSweeps, &Rth, d1, d2);
            double* in = xi.p;
            double* o = t.p;
            for (int j = 0; j < nSweeps; ++j) {
                k_cheb_step<double>(ex, R, in, o, bi.p, w.p, j == 0 ? Rth : d1[j],
                                    j == 0 ? 0.0 : d2[j], j == 0 ? 1 : 0, Gate{});
                std::swap(in, o);
            }
            out = in;
        }
        k_to_reference<double>(ex, n, A.L->d_perm.p, out, S.a.p);
        S.out(x, S.a);
    });
}

int unap_cuda_krylov_solve_host(long int handle, int method, int precond, double tol,
                                double relTol, int maxIter, int minIter, double* x,
                                const double* b, unap_cuda_stats* stats)
{
    return guarded([&] {
        Staged S(mat_from(handle));
        S.in(S.a, x);
        S.in(S.b, b);
        call(unap_cuda_krylov_solve(handle, method, precond, tol, relTol, maxIter, minIter, S.a.p,
                                    S.b.p, stats));
        S.out(x, S.a);
    });
}

// ---- reordering ------------------------------------------------------------

int unap_cuda_reorder_coo(double* val, int* row, int* col, int nCells, int size)
{
    return guarded([&] { reorder_coo0(val, row, col, nCells, size); });
}

int unap_cuda_reorder_uface(int* row, int* col, int nCells, int size, int* newOrder)
{
    return guarded([&] { reorder_uface0(row, col, nCells, size, newOrder); });
}

int unap_cuda_reorder_lface(int* row, int* col, int nCells, int size, int* newOrder)
{
    return guarded([&] { reorder_lface0(row, col, nCells, size, newOrder); });
}

int unap_cuda_reorder_value(double* val, const int* newOrder, int size)
{
    return guarded([&] { reorder_value0(val, newOrder, size); });
}

// Fortran convention (fortranInterface.cpp:467-534): 1-based row and column
// indices.  reordercoo_ shifts them to 0-based only when the first row
// index is not 0, as the reference does; the face calls always shift.
void reordercoo_(double* val, int* row, int* col, int* nCellsPtr, int* sizePtr)
{
    const int size = *sizePtr;
    if (size > 0 && row[0] != 0)
        for (int i = 0; i < size; ++i) {
            row[i] -= 1;
            col[i] -= 1;
        }
    if (unap_cuda_reorder_coo(val, row, col, *nCellsPtr, size))
        std::fprintf(stderr, "unap_cuda: reordercoo_ failed: %s\n", last_error());
}

void reorderuface__(int* row, int* col, int* nCellsPtr, int* sizePtr, int* newOrder)
{
    for (int i = 0; i < *sizePtr; ++i) {
        row[i] -= 1;
        col[i] -= 1;
    }
    if (unap_cuda_reorder_uface(row, col, *nCellsPtr, *sizePtr, newOrder))
        std::fprintf(stderr, "unap_cuda: reorderuface__ failed: %s\n", last_error());
}

void reorderlface__(int* row, int* col, int* nCellsPtr, int* sizePtr, int* newOrder)
{
    for (int i = 0; i < *sizePtr; ++i) {
        row[i] -= 1;
        col[i] -= 1;
    }
    if (unap_cuda_reorder_lface(row, col, *nCellsPtr, *sizePtr, newOrder))
        std::fprintf(stderr, "unap_cuda: reorderlface__ failed: %s\n", last_error());
}

void reordervalue__(double* val, int* newOrder, int* sizePtr)
{
    if (unap_cuda_reorder_value(val, newOrder, *sizePtr))
        std::fprintf(stderr, "unap_cuda: reordervalue__ failed: %s\n", last_error());
}

// ---- agglomeration ------------------------------------------------------------

int unap_cuda_agglomeration_create(long int* aggl, long int matrix, const double* weights,
                                   int nCellsInCoarsestLevel, int maxLevels)
{
    return guarded([&] {
        if (!aggl) throw std::invalid_argument("null handle pointer");
        MatHandle* m = mat_from(matrix);
        Matrix& A = m->get();
        if (!weights) throw std::invalid_argument("null weights");
        if (maxLevels < 1) throw std::invalid_argument("maxLevels must be >= 1");
        auto h = std::make_unique<AgglHandle>();
        h->nFine = A.host.n;
        h->nfFine = A.host.nf;
        std::vector<double> w(weights, weights + A.host.nf);
        h->levels = agglomerate_levels(A.host, w, nCellsInCoarsestLevel, maxLevels, 0, A.stream);
        *aggl = reinterpret_cast<long int>(h.release());
    });
}

int unap_cuda_agglomeration_size(long int aggl, int* nLevels)
{
    return guarded([&] {
        AgglHandle* h = aggl_from(aggl);
        if (nLevels) *nLevels = (int)h->levels.size();
    });
}

int unap_cuda_agglomeration_level(long int aggl, int level, int* nCells, int* nFaces, int* symm,
                                  int* restrictAddr, int* faceRestrict, int* lowerAddr,
                                  int* upperAddr, double* diag, double* upper, double* lower)
{
    return guarded([&] {
        AgglHandle* h = aggl_from(aggl);
        if (level < 0 || level >= (int)h->levels.size()) throw std::invalid_argument("no such level");
        const CoarseHost& c = h->levels[(size_t)level];
        const HostLdu& H = c.A;
        if (nCells) *nCells = H.n;
        if (nFaces) *nFaces = H.nf;
        if (symm) *symm = H.symm ? 1 : 0;
        auto cp = [](auto* dst, const auto& src) {
            if (dst) std::copy(src.begin(), src.end(), dst);
        };
        cp(restrictAddr, c.restrictAddr);
        cp(faceRestrict, c.faceRestrict);
        cp(lowerAddr, H.l);
        cp(upperAddr, H.u);
        cp(diag, H.diag);
        cp(upper, H.upper);
        if (lower) {
            if (H.symm)
                std::copy(H.upper.begin(), H.upper.end(), lower);
            else
                std::copy(H.lower.begin(), H.lower.end(), lower);
        }
    });
}

int unap_cuda_agglomeration_destroy(long int aggl)
{
    return guarded([&] { delete aggl_from(aggl); });
}

}  // extern "C"
