// C ABI of batched solves (declared in include/unap_cuda.h).
#include <memory>

#include "batch.hpp"
#include "capi_handles.hpp"
#include "../../include/unap_cuda.h"

using namespace unapgpu;

namespace {

struct BatchHandle {
    static constexpr unsigned kMagic = 0x42415431u;  // "BAT1"
    unsigned magic = kMagic;
    cudaStream_t stream = nullptr;
    std::unique_ptr<BatchSolver> S;
    ~BatchHandle()
    {
        S.reset();
        if (stream) cudaStreamDestroy(stream);
        magic = 0;
    }
};

BatchHandle* batch_from(long int h)
{
    BatchHandle* b = reinterpret_cast<BatchHandle*>(h);
    if (!b || b->magic != BatchHandle::kMagic) throw std::invalid_argument("invalid batch handle");
    return b;
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

}  // namespace

extern "C" {

int unap_cuda_batch_create(long int* batch)
{
    return guarded([&] {
        auto h = std::make_unique<BatchHandle>();
        UNAP_CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->S = std::make_unique<BatchSolver>(h->stream);
        *batch = reinterpret_cast<long int>(h.release());
    });
}

int unap_cuda_batch_solve(long int batch, int count, const unap_cuda_batch_item* items,
                          unap_cuda_stats* stats, int* ctaThreads)
{
    return guarded([&] {
        BatchHandle* h = batch_from(batch);
        if (count < 0 || (count > 0 && !items))
            throw std::invalid_argument("batch: count >= 0 and an item array");
        std::vector<BatchItem> v((size_t)count);
        for (int i = 0; i < count; ++i) {
            const unap_cuda_batch_item& it = items[i];
            if (it.method != 0 && it.method != 1)
                throw std::invalid_argument("batch item: method 0 (PCG) or 1 (PBiCGStab)");
            if (it.precond < 0 || it.precond > 3)
                throw std::invalid_argument("batch item: precond 0 (none), 1 (Diag), 2 (DIC) or 3 "
                                            "(DILU)");
            BatchItem& b = v[(size_t)i];
            b.A = &mat_from(it.matrix)->get();
            b.method = it.method;
            b.precond = it.precond;
            b.tol = it.tol;
            b.relTol = it.relTol;
            b.maxIter = it.maxIter;
            b.minIter = it.minIter;
            b.x = it.x;
            b.b = it.b;
        }
        // the matrices' own streams finish their setup before the batch runs
        for (const BatchItem& b : v) UNAP_CK(cudaStreamSynchronize(b.A->stream));
        // and the caller's vectors, filled on the default stream, are ready
        order_after_default_stream(h->stream);
        std::vector<SolveStats> st = h->S->solve(v);
        for (int i = 0; i < count && stats; ++i) {
            stats[i].nIterations = st[(size_t)i].nIter;
            stats[i].converged = st[(size_t)i].converged;
            stats[i].singular = st[(size_t)i].singular;
            stats[i].status = st[(size_t)i].status;
            stats[i].initialResidual = st[(size_t)i].initRes;
            stats[i].finalResidual = st[(size_t)i].finalRes;
            stats[i].trueResidual = st[(size_t)i].trueRes;
            stats[i].seconds = st[(size_t)i].seconds;
            stats[i].algorithmicBytes = st[(size_t)i].bytes;
        }
        if (ctaThreads) *ctaThreads = h->S->lastShape.threads;
    });
}

int unap_cuda_batch_last_shape(long int batch, int* ctaThreads, int* clusterCtas)
{
    return guarded([&] {
        BatchHandle* h = batch_from(batch);
        if (ctaThreads) *ctaThreads = h->S->lastShape.threads;
        if (clusterCtas) *clusterCtas = h->S->lastShape.cluster;
    });
}

int unap_cuda_batch_large_mode(long int batch, int* mode)
{
    return guarded([&] {
        BatchHandle* h = batch_from(batch);
        if (mode) *mode = h->S->lastLargeMode;
    });
}

int unap_cuda_set_team_solve_cells(int cells) { return set_team_solve_cells(cells); }

int unap_cuda_force_team_shape(int ctaThreads, int clusterCtas)
{
    return guarded([&] { force_team_shape(ctaThreads, clusterCtas); });
}

int unap_cuda_team_shape(int cells, int systems, int* ctaThreads, int* clusterCtas)
{
    return guarded([&] {
        const TeamShape t = cached_team_shape(cells, systems);
        if (ctaThreads) *ctaThreads = t.threads;
        if (clusterCtas) *clusterCtas = t.cluster;
    });
}

int unap_cuda_batch_destroy(long int batch)
{
    return guarded([&] { delete batch_from(batch); });
}

}  // extern "C"
