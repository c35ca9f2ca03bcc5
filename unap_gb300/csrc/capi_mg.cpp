// C ABI of the MGSolver (declared in include/unap_cuda.h).
#include <cstdio>
#include <limits>
#include <memory>

#include "capi_handles.hpp"
#include "mg.hpp"
#include "../../include/unap_cuda.h"

using namespace unapgpu;

namespace {

struct MgHandle {
    static constexpr unsigned kMagic = 0x4d475331u;  // "MGS1"
    unsigned magic = kMagic;
    Matrix* A = nullptr;
    std::vector<double> weights;
    MgParams p;
    std::unique_ptr<MgSolver> S;
    int builtVersion = -1;
    MgSolver& get()
    {
        // MGSolve.cpp:108-111 re-agglomerates the coarse coefficients on
        // every solve; the hierarchy here is rebuilt when the matrix
        // coefficients changed since it was made
        if (!S || builtVersion != A->L->version) {
            S = std::make_unique<MgSolver>(*A, weights, p);
            builtVersion = A->L->version;
        }
        return *S;
    }
    ~MgHandle() { magic = 0; }
};

MgHandle* mg_from(long int h)
{
    MgHandle* m = reinterpret_cast<MgHandle*>(h);
    if (!m || m->magic != MgHandle::kMagic) throw std::invalid_argument("invalid MG handle");
    return m;
}

template <class F>
int guarded(F&& f)
{
    try {
        f();
        return UNAP_CUDA_OK;
    } catch (const CudaError& e) {
        set_last_error(e.what());
        return UNAP_CUDA_ECUDA;
    } catch (const std::invalid_argument& e) {
        set_last_error(e.what());
        return UNAP_CUDA_EINVAL;
    } catch (const std::bad_alloc&) {
        set_last_error("out of host memory");
        return UNAP_CUDA_ENOMEM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return UNAP_CUDA_EINTERNAL;
    }
}

void fail(const char* where, int* nIter, double* res)
{
    std::fprintf(stderr, "unap_cuda: %s failed: %s\n", where, last_error());
    if (nIter) *nIter = -1;
    if (res) *res = std::numeric_limits<double>::quiet_NaN();
}

}  // namespace

namespace {

void mg_solve_device(MgHandle* h, double* x, const double* b, unap_cuda_stats* stats)
{
    MgSolver& S = h->get();
    S.params = h->p;
    SolveStats st = S.solveDevice(x, b);
    if (stats) {
        stats->nIterations = st.nIter;
        stats->converged = st.converged;
        stats->singular = st.singular;
        stats->status = st.status;
        stats->initialResidual = st.initRes;
        stats->finalResidual = st.finalRes;
        stats->trueResidual = -1;
        stats->seconds = st.seconds;
        stats->algorithmicBytes = st.bytes;
    }
}

}  // namespace

extern "C" {

void mgsolversolve_(double* x, long int* APtrPtr, double* b, int* nCells, int* aggl,
                    int* smoother, double* tol, double* relTol, int* maxIter, int* minIter,
                    int* num_iterations, double* final_res_norm, double* faceAreaPtr)
{
    int rc = guarded([&] {
        Matrix& A = mat_from(*APtrPtr)->get();
        if (*nCells != A.n()) throw std::invalid_argument("nCells does not match the matrix");
        std::vector<double> w;
        if (*aggl == 1)
            w = mg_face_weights(A.host);  // fortranInterface.cpp:383-395
        else if (*aggl == 2)
            w.assign(faceAreaPtr, faceAreaPtr + A.host.nf);
        else
            throw std::invalid_argument("agglomeration type must be 1 (coefficients) or 2 (face area)");
        if (*smoother != 1 && *smoother != 2)
            throw std::invalid_argument("smoother type must be 1 (Gauss-Seidel) or 2 (Chebyshev)");
        MgParams p;
        p.smoother = *smoother;
        p.tol = *tol;
        p.relTol = *relTol;
        p.maxIter = *maxIter;
        p.minIter = *minIter;
        p.nPre = 0;  // fortranInterface.cpp:434
        MgSolver S(A, w, p);
        SolveStats st = S.solveHost(x, b);
        *num_iterations = st.nIter;
        *final_res_norm = st.finalRes;
    });
    if (rc) fail("mgsolversolve_", num_iterations, final_res_norm);
    try {
        delete mat_from(*APtrPtr);  // fortranInterface.cpp:462-463
    } catch (...) {
    }
}

void contruct_solver_mg__(long int* mgPtrPtr, long int* APtrPtr, long int* AgglPtr,
                          const double* weightsPtr, const int* smootherTypePtr,
                          const int* maxLevelsPtr, const int* nCellsCoarsestPtr)
{
    int rc = guarded([&] {
        auto h = std::make_unique<MgHandle>();
        h->A = &mat_from(*APtrPtr)->get();
        h->weights.assign(weightsPtr, weightsPtr + h->A->host.nf);
        if (*smootherTypePtr != 1 && *smootherTypePtr != 2)
            throw std::invalid_argument("smoother type is not recognized (1 GaussSeidel, 2 Chebyshev)");
        h->p.smoother = *smootherTypePtr;
        h->p.maxLevels = *maxLevelsPtr;
        h->p.nCoarsest = *nCellsCoarsestPtr;
        h->get();
        *mgPtrPtr = reinterpret_cast<long int>(h.get());
        // the reference hands back its lduAgglomeration; here the hierarchy
        // belongs to the MG handle and this value only identifies it
        if (AgglPtr) *AgglPtr = reinterpret_cast<long int>(h.get());
        h.release();
    });
    if (rc) {
        std::fprintf(stderr, "unap_cuda: contruct_solver_mg__ failed: %s\n", last_error());
        *mgPtrPtr = 0;
    }
}

void sw_solver_mg_set_maxiter__(long int* p, const int* v) { guarded([&] { mg_from(*p)->p.maxIter = *v; }); }
void sw_solver_mg_set_miniter__(long int* p, const int* v) { guarded([&] { mg_from(*p)->p.minIter = *v; }); }
void sw_solver_mg_set_tol__(long int* p, const double* v) { guarded([&] { mg_from(*p)->p.tol = *v; }); }
void sw_solver_mg_set_reltol__(long int* p, const double* v) { guarded([&] { mg_from(*p)->p.relTol = *v; }); }
void sw_solver_mg_set_npresweeps__(long int* p, const int* v) { guarded([&] { mg_from(*p)->p.nPre = *v; }); }
void sw_solver_mg_set_npostsweeps__(long int* p, const int* v) { guarded([&] { mg_from(*p)->p.nPost = *v; }); }
void sw_solver_mg_set_nfinestsweeps__(long int* p, const int* v) { guarded([&] { mg_from(*p)->p.nFinest = *v; }); }

void sw_solve_mg__(long int* mgPtrPtr, long int* APtrPtr, double* xPtr, double* bPtr,
                   double* res_normPtr)
{
    int rc = guarded([&] {
        MgHandle* h = mg_from(*mgPtrPtr);
        Matrix& A = mat_from(*APtrPtr)->get();
        if (&A != h->A) throw std::invalid_argument("matrix handle differs from the one the solver was built on");
        MgSolver& S = h->get();
        S.params = h->p;
        S.initSmoothers();  // fortranInterface.cpp:877
        SolveStats st = S.solveHost(xPtr, bPtr);
        *res_normPtr = st.finalRes;
    });
    if (rc) fail("sw_solve_mg__", nullptr, res_normPtr);
}

void sw_solver_destroy_mg__(long int* solverPtrPtr)
{
    guarded([&] {
        delete mg_from(*solverPtrPtr);
        *solverPtrPtr = 0;
    });
}

int unap_cuda_mg_create(long int* mg, long int matrix, const double* weights, int smoother,
                        int nCoarsest, int maxLevels, int nPre, int nPost, int nFinest,
                        int scaleCorr, double tol, double relTol, int maxIter, int minIter)
{
    return guarded([&] {
        auto h = std::make_unique<MgHandle>();
        h->A = &mat_from(matrix)->get();
        if (weights)
            h->weights.assign(weights, weights + h->A->host.nf);
        else
            h->weights = mg_face_weights(h->A->host);
        h->p.smoother = smoother;
        if (nCoarsest > 0) h->p.nCoarsest = nCoarsest;
        if (maxLevels > 0) h->p.maxLevels = maxLevels;
        if (nPre >= 0) h->p.nPre = nPre;
        if (nPost >= 0) h->p.nPost = nPost;
        if (nFinest >= 0) h->p.nFinest = nFinest;
        h->p.scaleCorr = scaleCorr;
        h->p.tol = tol;
        h->p.relTol = relTol;
        h->p.maxIter = maxIter;
        h->p.minIter = minIter;
        h->get();
        *mg = reinterpret_cast<long int>(h.release());
    });
}

int unap_cuda_mg_levels(long int mg, int* nCoarseLevels, int* cells, int maxOut)
{
    return guarded([&] {
        MgSolver& S = mg_from(mg)->get();
        std::vector<int> c = S.levelCells();
        if (nCoarseLevels) *nCoarseLevels = (int)c.size() - 1;
        for (int k = 0; k < (int)c.size() && k < maxOut; ++k) cells[k] = c[(size_t)k];
    });
}

int unap_cuda_mg_solve(long int mg, double* x, const double* b, unap_cuda_stats* stats)
{
    return guarded([&] {
        MgHandle* h = mg_from(mg);
        order_after_default_stream(h->A->stream);
        mg_solve_device(h, x, b, stats);
    });
}

int unap_cuda_mg_solve_host(long int mg, double* x, const double* b, unap_cuda_stats* stats)
{
    return guarded([&] {
        MgHandle* h = mg_from(mg);
        if (!x || !b) throw std::invalid_argument("null vector");
        const size_t n = (size_t)h->A->n();
        DevArray<double> dx(n), db(n);
        UNAP_CK(cudaMemcpyAsync(dx.p, x, n * sizeof(double), cudaMemcpyHostToDevice, h->A->stream));
        UNAP_CK(cudaMemcpyAsync(db.p, b, n * sizeof(double), cudaMemcpyHostToDevice, h->A->stream));
        mg_solve_device(h, dx.p, db.p, stats);
        UNAP_CK(cudaMemcpyAsync(x, dx.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->A->stream));
        UNAP_CK(cudaStreamSynchronize(h->A->stream));
    });
}

int unap_cuda_mg_set(long int mg, int nPre, int nPost, int nFinest, int scaleCorr, double tol,
                     double relTol, int maxIter, int minIter)
{
    return guarded([&] {
        MgHandle* h = mg_from(mg);
        if (nPre < 0 || nPost < 0 || nFinest < 0 || maxIter < 0 || minIter < 0)
            throw std::invalid_argument("negative sweep or iteration count");
        h->p.nPre = nPre;
        h->p.nPost = nPost;
        h->p.nFinest = nFinest;
        h->p.scaleCorr = scaleCorr;
        h->p.tol = tol;
        h->p.relTol = relTol;
        h->p.maxIter = maxIter;
        h->p.minIter = minIter;
    });
}

int unap_cuda_mg_destroy(long int mg)
{
    return guarded([&] { delete mg_from(mg); });
}

}  // extern "C"
