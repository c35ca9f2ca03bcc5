// extern "C" boundary of libunap_cuda.so (declared in include/unap_cuda.h).
// Every entry point catches C++ exceptions: the Fortran-convention calls
// report failure through num_iterations = -1 / res_norm = NaN, the
// unap_cuda_* calls return a negative status; the message is kept for
// unap_cuda_last_error().
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>

#include "capi_handles.hpp"
#include "../../include/unap_cuda.h"

using namespace unapgpu;

namespace unapgpu {

Matrix& MatHandle::get()
{
    if (!M) {
        if (!hasValues) throw std::invalid_argument("matrix coefficients were never filled");
        M = std::make_unique<Matrix>(std::move(pending), nullptr, matrix_wavefronts() != 0);
    }
    return *M;
}

int MatHandle::n() const { return M ? M->n() : pending.n; }

void MatHandle::setValues(const double* diag, const double* upper, const double* lower)
{
    if (M) {
        M->setValues(diag, upper, lower);
        return;
    }
    pending.diag.assign(diag, diag + pending.n);
    pending.upper.assign(upper, upper + pending.nf);
    pending.symm = (lower == nullptr || lower == upper);
    if (pending.symm)
        pending.lower.clear();
    else
        pending.lower.assign(lower, lower + pending.nf);
    hasValues = true;
}

MatHandle* mat_from(long int h)
{
    MatHandle* m = reinterpret_cast<MatHandle*>(h);
    if (!m || m->magic != MatHandle::kMagic) throw std::invalid_argument("invalid matrix handle");
    return m;
}

HostLdu host_from_arrays(int n, int nf, const int* l, const int* u, const double* lower,
                         const double* diag, const double* upper)
{
    if (n < 0 || nf < 0) throw std::invalid_argument("negative size");
    HostLdu h;
    h.n = n;
    h.nf = nf;
    h.l.assign(l, l + nf);
    h.u.assign(u, u + nf);
    h.diag.assign(diag, diag + n);
    h.upper.assign(upper, upper + nf);
    h.symm = (lower == nullptr || lower == upper);
    if (!h.symm) h.lower.assign(lower, lower + nf);
    return h;
}

}  // namespace unapgpu

namespace {

template <class F>
int guarded(F&& f)
{
    try {
        f();
        return UNAP_CUDA_OK;
    } catch (const CudaError& e) {
        set_last_error(e.what());
        return UNAP_CUDA_ECUDA;
    } catch (const std::bad_alloc& e) {
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

void report_failure(const char* where, int* nIter, double* res)
{
    std::fprintf(stderr, "unap_cuda: %s failed: %s\n", where, last_error());
    if (nIter) *nIter = -1;
    if (res) *res = std::numeric_limits<double>::quiet_NaN();
}

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

// coo2ldu (matrixConversion/coo2ldu.cpp:3-113) after reorderCOO
// (matrixConversion.cpp:38-98): 0-based, row-grouped COO of a structurally
// symmetric matrix -> owner-sorted LDU.  Upper faces come from the (row < col)
// entries in row-major order; the lower coefficient of face (c, r) is the
// (r, c) entry, grouped by owner c in order of appearance.  Input the
// reference leaves undefined is an error: rows out of order, a repeated
// entry, a column whose lower entries do not number its upper faces.  The
// device form (coo_dev.cu) gives the same arrays.
HostLdu coo_to_ldu(const double* val, const std::vector<int>& row0, const std::vector<int>& col0,
                   int n, int size, bool symm)
{
    // reorderCOO: within each row, entries ordered by column
    std::vector<int> cnt((size_t)n + 1, 0);
    for (int i = 0; i < size; ++i) {
        if (row0[(size_t)i] < 0 || row0[(size_t)i] >= n || col0[(size_t)i] < 0 || col0[(size_t)i] >= n)
            throw std::invalid_argument("COO entry out of range");
        cnt[(size_t)row0[(size_t)i] + 1]++;
    }
    for (int i = 1; i < size; ++i)
        if (row0[(size_t)i - 1] > row0[(size_t)i])
            throw std::invalid_argument("COO entries must be grouped by row in ascending row order");
    for (int c = 0; c < n; ++c) cnt[(size_t)c + 1] += cnt[(size_t)c];
    std::vector<int> rows((size_t)size), cols((size_t)size);
    std::vector<double> vals((size_t)size);
    for (int i = 0; i < size; ++i) {
        int r = row0[(size_t)i];
        int start = cnt[(size_t)r], len = cnt[(size_t)r + 1] - cnt[(size_t)r];
        int pos = 0;
        for (int k = 0; k < len; ++k) {
            int ck = col0[(size_t)(start + k)];
            if (col0[(size_t)i] > ck || (start + k < i && col0[(size_t)i] == ck)) pos++;
        }
        rows[(size_t)(start + pos)] = r;
        cols[(size_t)(start + pos)] = col0[(size_t)i];
        vals[(size_t)(start + pos)] = val[i];
    }
    HostLdu h;
    h.n = n;
    int nZeros = (size - n) / 2;
    h.diag.assign((size_t)n, 0.0);
    h.l.reserve((size_t)nZeros);
    h.u.reserve((size_t)nZeros);
    h.upper.reserve((size_t)nZeros);
    std::vector<int> lowerCol;
    std::vector<double> lowerVal;
    std::vector<int> upperNbrs((size_t)n, 0);
    for (int i = 0; i < size; ++i) {
        int r = rows[(size_t)i], c = cols[(size_t)i];
        if (i && rows[(size_t)i - 1] == r && cols[(size_t)i - 1] >= c)
            throw std::invalid_argument("COO matrix repeats an entry");
        if (r == c) {
            h.diag[(size_t)r] = vals[(size_t)i];
        } else if (c > r) {
            h.u.push_back(c);
            h.l.push_back(r);
            h.upper.push_back(vals[(size_t)i]);
            upperNbrs[(size_t)r]++;
        } else if (!symm) {
            lowerCol.push_back(c);
            lowerVal.push_back(vals[(size_t)i]);
        }
    }
    h.nf = (int)h.upper.size();
    if (h.nf != nZeros) throw std::invalid_argument("COO matrix is not structurally symmetric");
    h.symm = symm;
    if (!symm) {
        // sortData (matrixConversion.cpp:4-35): group lower values by owner
        if ((int)lowerVal.size() != h.nf)
            throw std::invalid_argument("COO matrix is not structurally symmetric");
        std::vector<int> off((size_t)n + 1, 0), c2((size_t)n, 0);
        for (int c = 0; c < n; ++c) off[(size_t)c + 1] = off[(size_t)c] + upperNbrs[(size_t)c];
        for (int o : lowerCol) c2[(size_t)o]++;
        for (int c = 0; c < n; ++c)
            if (c2[(size_t)c] != upperNbrs[(size_t)c])
                throw std::invalid_argument("COO matrix is not structurally symmetric");
        std::fill(c2.begin(), c2.end(), 0);
        h.lower.assign((size_t)h.nf, 0.0);
        for (size_t k = 0; k < lowerVal.size(); ++k) {
            int o = lowerCol[k];
            h.lower[(size_t)(off[(size_t)o] + c2[(size_t)o]++)] = lowerVal[k];
        }
    }
    return h;
}

}  // namespace

extern "C" {

const char* unap_cuda_last_error(void) { return last_error(); }
const char* unap_cuda_version(void) { return "unap_cuda 0.1 (sm_103a)"; }

int unap_cuda_device_synchronize(void)
{
    return guarded([] { UNAP_CK(cudaDeviceSynchronize()); });
}

/* ---------------- reference Fortran-convention interface ---------------- */

void ldumatrixcreat_(long int* APtrPtr, int* nCells, int* upperSize, int* lowerAddr,
                     int* upperAddr, double* lower, double* diag, double* upper)
{
    int rc = guarded([&] {
        auto* m = new MatHandle;
        m->pending = host_from_arrays(*nCells, *upperSize, lowerAddr, upperAddr,
                                      lower == upper ? nullptr : lower, diag, upper);
        m->hasValues = true;
        *APtrPtr = reinterpret_cast<long int>(m);
    });
    if (rc) {
        std::fprintf(stderr, "unap_cuda: ldumatrixcreat_ failed: %s\n", last_error());
        *APtrPtr = 0;
    }
}

void coo2ldumatrixcreat_(long int* APtrPtr, const double* dataPtr, const int* rowsPtr,
                         const int* columnPtr, const int* nCells, const int* size, const int* symm)
{
    int rc = guarded([&] {
        auto m = std::make_unique<MatHandle>();
        const long long minCells = device_setup_min_cells();
        if (!(minCells >= 0 && *nCells >= minCells &&
              coo_to_ldu_device(dataPtr, rowsPtr, columnPtr, *nCells, *size, *symm != 0, false,
                                0, m->pending))) {
            std::vector<int> r((size_t)*size), c((size_t)*size);
            for (int i = 0; i < *size; ++i) {
                r[(size_t)i] = rowsPtr[i] - 1;  // fortranInterface.cpp:90-95
                c[(size_t)i] = columnPtr[i] - 1;
            }
            m->pending = coo_to_ldu(dataPtr, r, c, *nCells, *size, *symm != 0);
        }
        m->hasValues = true;
        *APtrPtr = reinterpret_cast<long int>(m.release());
    });
    if (rc) {
        std::fprintf(stderr, "unap_cuda: coo2ldumatrixcreat_ failed: %s\n", last_error());
        *APtrPtr = 0;
    }
}

void csr2ldumatrixcreat_(long int* APtrPtr, const double* dataPtr, const int* compRowsPtr,
                         const int* columnPtr, const int* nCells, const int* size, const int* symm)
{
    int rc = guarded([&] {
        // csr2ldu (coo2ldu.cpp:116-148) expands the row pointer and calls
        // coo2ldu without re-sorting; indices are used as given (0-based)
        auto m = std::make_unique<MatHandle>();
        const long long minCells = device_setup_min_cells();
        if (!(minCells >= 0 && *nCells >= minCells &&
              coo_to_ldu_device(dataPtr, compRowsPtr, columnPtr, *nCells, *size, *symm != 0, true,
                                0, m->pending))) {
            if (compRowsPtr[0] != 0 || compRowsPtr[*nCells] != *size)
                throw std::invalid_argument("CSR row pointer is not a valid partition of the entries");
            std::vector<int> r((size_t)*size), c(columnPtr, columnPtr + *size);
            for (int i = 0; i < *nCells; ++i) {
                if (compRowsPtr[i + 1] < compRowsPtr[i])
                    throw std::invalid_argument("CSR row pointer is not a valid partition of the entries");
                for (int j = compRowsPtr[i]; j < compRowsPtr[i + 1]; ++j) r[(size_t)j] = i;
            }
            m->pending = coo_to_ldu(dataPtr, r, c, *nCells, *size, *symm != 0);
        }
        m->hasValues = true;
        *APtrPtr = reinterpret_cast<long int>(m.release());
    });
    if (rc) {
        std::fprintf(stderr, "unap_cuda: csr2ldumatrixcreat_ failed: %s\n", last_error());
        *APtrPtr = 0;
    }
}

void matrixinterfacescreat_(long int* APtrPtr, const int* nNeiProcs, const int*, const int*,
                            const int*, const double*)
{
    // one GPU is a single rank: the reference ignores interfaces when
    // PARRUN is false (lduMatrix.cpp:488-503)
    int rc = guarded([&] { mat_from(*APtrPtr); });
    if (rc) std::fprintf(stderr, "unap_cuda: matrixinterfacescreat_: %s\n", last_error());
    (void)nNeiProcs;
}

static void krylov_oneshot(Method m, const char* name, double* x, long int* APtrPtr, double* b,
                           int* nCells, int* precond, double* tol, double* relTol, int* maxIter,
                           int* minIter, int* num_iterations, double* final_res_norm)
{
    int rc = guarded([&] {
        MatHandle* h = mat_from(*APtrPtr);
        Matrix& A = h->get();
        if (*nCells != A.n()) throw std::invalid_argument("nCells does not match the matrix");
        auto P = make_ldu_precond(*precond, A);
        Krylov K(A, P.get(), m);
        K.tol = *tol;
        K.relTol = *relTol;
        K.maxIter = *maxIter;
        K.minIter = *minIter;
        SolveStats st = K.solveHost(x, b);
        *num_iterations = st.nIter;
        *final_res_norm = st.finalRes;
    });
    if (rc) report_failure(name, num_iterations, final_res_norm);
    // the one-shot call consumes the matrix (fortranInterface.cpp:266-267)
    try {
        delete mat_from(*APtrPtr);
    } catch (...) {
    }
}

void pcgsolversolve_(double* x, long int* APtrPtr, double* b, int* nCells, int* precond,
                     double* tol, double* relTol, int* maxIter, int* minIter, int* num_iterations,
                     double* final_res_norm)
{
    krylov_oneshot(Method::PCG, "pcgsolversolve_", x, APtrPtr, b, nCells, precond, tol, relTol,
                   maxIter, minIter, num_iterations, final_res_norm);
}

void pbicgstabsolversolve_(double* x, long int* APtrPtr, double* b, int* nCells, int* precond,
                           double* tol, double* relTol, int* maxIter, int* minIter,
                           int* num_iterations, double* final_res_norm)
{
    krylov_oneshot(Method::PBiCGStab, "pbicgstabsolversolve_", x, APtrPtr, b, nCells, precond,
                   tol, relTol, maxIter, minIter, num_iterations, final_res_norm);
}

/* handle API */

void contruct_sw_matrix__(long int* APtrPtr, const int* nCellsPtr, const int* rowsPtr,
                          const int* colsPtr, const int* sizePtr)
{
    int rc = guarded([&] {
        // fortranInterface.cpp:537-571: addresses taken as given, values 0
        auto* m = new MatHandle;
        int n = *nCellsPtr, nf = *sizePtr;
        m->pending.n = n;
        m->pending.nf = nf;
        m->pending.l.assign(rowsPtr, rowsPtr + nf);
        m->pending.u.assign(colsPtr, colsPtr + nf);
        m->pending.diag.assign((size_t)n, 0.0);
        m->pending.upper.assign((size_t)nf, 0.0);
        m->pending.symm = true;
        m->hasValues = false;
        *APtrPtr = reinterpret_cast<long int>(m);
    });
    if (rc) {
        std::fprintf(stderr, "unap_cuda: contruct_sw_matrix__ failed: %s\n", last_error());
        *APtrPtr = 0;
    }
}

void contruct_sw_matrix_interfaces__(long int* APtrPtr, const int*, const int*, const int*,
                                     const int*)
{
    int rc = guarded([&] { mat_from(*APtrPtr); });
    if (rc) std::fprintf(stderr, "unap_cuda: contruct_sw_matrix_interfaces__: %s\n", last_error());
}

void fill_sw_matrix_coefficients__(long int* APtrPtr, const double* diagPtr,
                                   const double* upperPtr, const double* lowerPtr)
{
    int rc = guarded([&] { mat_from(*APtrPtr)->setValues(diagPtr, upperPtr, lowerPtr); });
    if (rc) std::fprintf(stderr, "unap_cuda: fill_sw_matrix_coefficients__: %s\n", last_error());
}

void fill_sw_matrix_interfaces_coefficients__(long int* APtrPtr, const int*, const double*)
{
    int rc = guarded([&] { mat_from(*APtrPtr); });
    if (rc)
        std::fprintf(stderr, "unap_cuda: fill_sw_matrix_interfaces_coefficients__: %s\n",
                     last_error());
}

void contruct_solver_pbicgstab__(long int* solverPtrPtr)
{
    auto* s = new BicgHandle;
    *solverPtrPtr = reinterpret_cast<long int>(s);
}

static BicgHandle* bicg_from(long int* p)
{
    BicgHandle* s = reinterpret_cast<BicgHandle*>(*p);
    if (!s || s->magic != BicgHandle::kMagic) throw std::invalid_argument("invalid PBiCGStab handle");
    return s;
}

void sw_solver_pbicgstab_set_maxiter__(long int* p, const int* v)
{
    guarded([&] { bicg_from(p)->maxIter = *v; });
}
void sw_solver_pbicgstab_set_miniter__(long int* p, const int* v)
{
    guarded([&] { bicg_from(p)->minIter = *v; });
}
void sw_solver_pbicgstab_set_tol__(long int* p, const double* v)
{
    guarded([&] { bicg_from(p)->tol = *v; });
}
void sw_solver_pbicgstab_set_reltol__(long int* p, const double* v)
{
    guarded([&] { bicg_from(p)->relTol = *v; });
}

void sw_solver_pbicgstab_set_precond__(long int* solverPtrPtr, long int* APtrPtr,
                                       const int* precondTypePtr)
{
    int rc = guarded([&] {
        BicgHandle* s = bicg_from(solverPtrPtr);
        int t = *precondTypePtr;
        if (t < 1 || t > 3) {
            // fortranInterface.cpp:992-996 prints and keeps the old one
            std::fprintf(stderr,
                         "ERROR: preconditioner type is not recognized!\n"
                         "Valid option is: 1--diagonal, 2--DIC, 3--DILU\n");
            return;
        }
        s->precondType = t;
        s->precondMat = mat_from(*APtrPtr);
        s->P.reset();
    });
    if (rc) std::fprintf(stderr, "unap_cuda: sw_solver_pbicgstab_set_precond__: %s\n", last_error());
}

void sw_solve_pbicgstab__(long int* solverPtrPtr, long int* APtrPtr, double* xPtr, double* bPtr,
                          double* res_normPtr)
{
    int rc = guarded([&] {
        BicgHandle* s = bicg_from(solverPtrPtr);
        Matrix& A = mat_from(*APtrPtr)->get();
        // the preconditioner is (re)factored for the current coefficients
        if (!s->P || s->precondVersion != A.L->version || s->precondFor != &A) {
            s->P = make_ldu_precond(s->precondType, A);
            s->precondVersion = A.L->version;
            s->precondFor = &A;
        }
        Krylov K(A, s->P.get(), Method::PBiCGStab);
        K.tol = s->tol;
        K.relTol = s->relTol;
        K.maxIter = s->maxIter;
        K.minIter = s->minIter;
        SolveStats st = K.solveHost(xPtr, bPtr);
        *res_normPtr = st.finalRes;
    });
    if (rc) report_failure("sw_solve_pbicgstab__", nullptr, res_normPtr);
}

void sw_matrix_destroy__(long int* APtrPtr)
{
    guarded([&] {
        delete mat_from(*APtrPtr);
        *APtrPtr = 0;
    });
}

void sw_solver_destroy_pbicgstab__(long int* solverPtrPtr)
{
    guarded([&] {
        delete bicg_from(solverPtrPtr);
        *solverPtrPtr = 0;
    });
}

/* ---------------- GB300 entry points ---------------- */

int unap_cuda_matrix_create(long int* handle, int nCells, int nFaces, const int* lowerAddr,
                            const int* upperAddr, const double* lower, const double* diag,
                            const double* upper)
{
    return guarded([&] {
        if (!handle) throw std::invalid_argument("null handle pointer");
        auto m = std::make_unique<MatHandle>();
        m->pending = host_from_arrays(nCells, nFaces, lowerAddr, upperAddr, lower, diag, upper);
        m->hasValues = true;
        m->get();
        *handle = reinterpret_cast<long int>(m.release());
    });
}

int unap_cuda_matrix_destroy(long int handle)
{
    return guarded([&] { delete mat_from(handle); });
}

int unap_cuda_matrix_size(long int handle, int* nCells, int* nFaces, int* symm)
{
    return guarded([&] {
        MatHandle* h = mat_from(handle);
        const HostLdu& H = h->M ? h->M->host : h->pending;
        if (nCells) *nCells = H.n;
        if (nFaces) *nFaces = H.nf;
        if (symm) *symm = H.symm ? 1 : 0;
    });
}

int unap_cuda_matrix_get_ldu(long int handle, int* lowerAddr, int* upperAddr, double* lower,
                             double* diag, double* upper)
{
    return guarded([&] {
        MatHandle* h = mat_from(handle);
        const HostLdu& H = h->M ? h->M->host : h->pending;
        size_t nf = (size_t)H.nf, n = (size_t)H.n;
        if (lowerAddr) std::memcpy(lowerAddr, H.l.data(), nf * sizeof(int));
        if (upperAddr) std::memcpy(upperAddr, H.u.data(), nf * sizeof(int));
        if (upper) std::memcpy(upper, H.upper.data(), nf * sizeof(double));
        if (lower) std::memcpy(lower, H.lowerPtr(), nf * sizeof(double));
        if (diag) std::memcpy(diag, H.diag.data(), n * sizeof(double));
    });
}

int unap_cuda_set_device_setup(long long minCells, long long* oldMinCells)
{
    return guarded([&] {
        long long o = set_device_setup_min_cells(minCells);
        if (oldMinCells) *oldMinCells = o;
    });
}

int unap_cuda_matrix_layout(long int handle, int* nWavefronts, int* perm, int* waveStart)
{
    return guarded([&] {
        const Level& L = *mat_from(handle)->get().L;
        if (nWavefronts) *nWavefronts = L.nWave;
        if (perm) std::memcpy(perm, L.perm.data(), sizeof(int) * L.perm.size());
        if (waveStart) std::memcpy(waveStart, L.waveStart.data(), sizeof(int) * L.waveStart.size());
    });
}

int unap_cuda_matrix_info(long int handle, int* nWavefronts, long long* nEntries,
                          long long* deviceBytes)
{
    return guarded([&] {
        Matrix& A = mat_from(handle)->get();
        if (nWavefronts) *nWavefronts = A.L->nWave;
        if (nEntries) *nEntries = A.L->nEntries;
        if (deviceBytes) *deviceBytes = (long long)A.L->deviceBytes();
    });
}

int unap_cuda_spmv(long int handle, const double* x, double* y)
{
    return guarded([&] {
        MatHandle* h = mat_from(handle);
        Matrix& A = h->get();
        order_after_default_stream(A.stream);
        Exec ex{A.stream, device_max_blocks()};
        h->ensureScratch();
        k_to_internal<double>(ex, A.n(), A.L->d_perm.p, x, h->s1.p);
        k_spmv<double>(ex, rows64(*A.L), h->s1.p, h->s2.p, nullptr, RSpec{}, Gate{});
        k_to_reference<double>(ex, A.n(), A.L->d_perm.p, h->s2.p, y);
        UNAP_CK(cudaGetLastError());
        UNAP_CK(cudaStreamSynchronize(A.stream));
    });
}

int unap_cuda_precondition(long int handle, int precond, const double* r, double* w)
{
    return guarded([&] {
        MatHandle* h = mat_from(handle);
        Matrix& A = h->get();
        order_after_default_stream(A.stream);
        Exec ex{A.stream, device_max_blocks()};
        h->ensureScratch();
        auto P = make_ldu_precond(precond, A);
        k_to_internal<double>(ex, A.n(), A.L->d_perm.p, r, h->s1.p);
        P->apply(ex, h->s1.p, h->s2.p, nullptr, 0, nullptr, FIN_NONE, Gate{});
        k_to_reference<double>(ex, A.n(), A.L->d_perm.p, h->s2.p, w);
        UNAP_CK(cudaGetLastError());
        UNAP_CK(cudaStreamSynchronize(A.stream));
    });
}

int unap_cuda_gauss_seidel(long int handle, double* x, const double* b, int nSweeps, int backward)
{
    return guarded([&] {
        MatHandle* h = mat_from(handle);
        Matrix& A = h->get();
        order_after_default_stream(A.stream);
        if (!A.L->sweepable)
            throw std::invalid_argument(
                "Gauss-Seidel needs oriented, owner-sorted faces and a matrix built with "
                "wavefronts");
        Exec ex{A.stream, device_max_blocks()};
        h->ensureScratch();
        k_to_internal<double>(ex, A.n(), A.L->d_perm.p, x, h->s1.p);
        k_to_internal<double>(ex, A.n(), A.L->d_perm.p, b, h->s2.p);
        Rows<double> R = rows64(*A.L);
        for (int k = 0; k < nSweeps; ++k)
            gs_sweep<double>(ex, *A.L, R, h->s1.p, h->s2.p, backward != 0, false, Gate{});
        k_to_reference<double>(ex, A.n(), A.L->d_perm.p, h->s1.p, x);
        UNAP_CK(cudaGetLastError());
        UNAP_CK(cudaStreamSynchronize(A.stream));
    });
}

int unap_cuda_krylov_solve(long int handle, int method, int precond, double tol, double relTol,
                           int maxIter, int minIter, double* x, const double* b,
                           unap_cuda_stats* stats)
{
    return guarded([&] {
        Matrix& A = mat_from(handle)->get();
        if (method != 0 && method != 1)
            throw std::invalid_argument("method 0 (PCG) or 1 (PBiCGStab)");
        if (precond < 0 || precond > 3)
            throw std::invalid_argument("precond 0 (none), 1 (Diag), 2 (DIC) or 3 (DILU)");
        auto P = make_ldu_precond(precond, A);
        Krylov K(A, P.get(), method == 1 ? Method::PBiCGStab : Method::PCG);
        order_after_default_stream(A.stream);
        K.tol = tol;
        K.relTol = relTol;
        K.maxIter = maxIter;
        K.minIter = minIter;
        SolveStats st = K.solveDevice(x, b);
        put_stats(st, stats);
    });
}

}  // extern "C"

extern "C" int unap_cuda_profile_kernels(long int handle, int reps, double* ms)
{
    return guarded([&] {
        MatHandle* h = mat_from(handle);
        Matrix& A = h->get();
        if (reps < 1) throw std::invalid_argument("reps must be >= 1");
        Level& L = *A.L;
        Exec ex{A.stream, device_max_blocks()};
        const int n = A.n();
        DevArray<double> a((size_t)n), b((size_t)n), c((size_t)n);
        DevArray<float> af((size_t)n), bf((size_t)n);
        k_fill<double>(ex, n, a.p, 1.0);
        k_fill<double>(ex, n, b.p, 0.5);
        k_fill<float>(ex, n, af.p, 1.0f);
        k_fill<float>(ex, n, bf.p, 0.5f);
        make_fp32(L, A.stream);
        Rows<double> R = rows64(L);
        Rows<float> R32 = rows32(L);
        std::unique_ptr<Precond> dic, dilu;
        if (L.sweepable) {
            dic = make_ldu_precond(2, A);
            dilu = make_ldu_precond(3, A);
        }
        cudaEvent_t e0, e1;
        UNAP_CK(cudaEventCreate(&e0));
        UNAP_CK(cudaEventCreate(&e1));
        auto timeit = [&](auto&& fn) -> double {
            fn();
            UNAP_CK(cudaEventRecord(e0, ex.s));
            for (int k = 0; k < reps; ++k) fn();
            UNAP_CK(cudaEventRecord(e1, ex.s));
            UNAP_CK(cudaEventSynchronize(e1));
            float t = 0;
            UNAP_CK(cudaEventElapsedTime(&t, e0, e1));
            return (double)t / reps;
        };
        for (int i = 0; i < 8; ++i) ms[i] = -1.0;
        ms[0] = timeit([&] { k_spmv<double>(ex, R, a.p, b.p, nullptr, RSpec{}, Gate{}); });
        if (L.sweepable) {
            ms[1] = timeit([&] { dic->apply(ex, a.p, b.p, nullptr, 0, nullptr, FIN_NONE, Gate{}); });
            ms[2] = timeit([&] { dilu->apply(ex, a.p, b.p, nullptr, 0, nullptr, FIN_NONE, Gate{}); });
            ms[3] = timeit([&] { gs_sweep<double>(ex, L, R, b.p, a.p, false, false, Gate{}); });
            ms[4] = timeit([&] { gs_sweep<double>(ex, L, R, b.p, a.p, true, false, Gate{}); });
            ms[6] = timeit([&] { gs_sweep<float>(ex, L, R32, bf.p, af.p, false, false, Gate{}); });
        }
        ms[5] = timeit([&] { k_spmv<float>(ex, R32, af.p, bf.p, nullptr, RSpec{}, Gate{}); });
        ms[7] = timeit([&] { k_residual<double>(ex, R, a.p, b.p, c.p, RSpec{}, Gate{}); });
        UNAP_CK(cudaGetLastError());
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    });
}
