// C ABI of the solve server (declared in include/unap_cuda.h).
#include <cstring>
#include <memory>

#include "capi_handles.hpp"
#include "server.hpp"
#include "../../include/unap_cuda.h"

using namespace unapgpu;

namespace {

struct ServerHandle {
    static constexpr unsigned kMagic = 0x53525631u;  // "SRV1"
    unsigned magic = kMagic;
    std::unique_ptr<Server> S;
    ~ServerHandle() { magic = 0; }
};

ServerHandle* server_from(long int h)
{
    ServerHandle* s = reinterpret_cast<ServerHandle*>(h);
    if (!s || s->magic != ServerHandle::kMagic) throw std::invalid_argument("invalid server handle");
    return s;
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

int unap_cuda_server_create(long int* server, long long memoryBudget, int maxSlots,
                            int smallCells)
{
    return guarded([&] {
        ServerParams p;
        p.memoryBudget = memoryBudget;
        if (maxSlots > 0) p.maxSlots = maxSlots;
        if (smallCells >= 0) p.smallCells = smallCells;
        auto h = std::make_unique<ServerHandle>();
        h->S = std::make_unique<Server>(p);
        *server = reinterpret_cast<long int>(h.release());
    });
}

int unap_cuda_server_submit(long int server, int nCells, int nFaces, const int* lowerAddr,
                            const int* upperAddr, const double* lower, const double* diag,
                            const double* upper, const double* b, int method, double relTol,
                            int maxIter, long long* id)
{
    return guarded([&] {
        ServerHandle* h = server_from(server);
        if (method < 0 || method > 3) throw std::invalid_argument("method must be 0..3");
        auto r = std::make_unique<ServeRequest>();
        r->A = host_from_arrays(nCells, nFaces, lowerAddr, upperAddr, lower, diag, upper);
        r->b.assign(b, b + nCells);
        r->method = method;
        r->relTol = relTol;
        r->maxIter = maxIter;
        *id = h->S->submit(std::move(r));
    });
}

int unap_cuda_server_wait(long int server, long long id, double* x,
                          unap_cuda_request_info* info)
{
    return guarded([&] {
        ServerHandle* h = server_from(server);
        std::unique_ptr<ServeRequest> r = h->S->wait(id);
        if (x && !r->x.empty()) std::memcpy(x, r->x.data(), r->x.size() * sizeof(double));
        if (info) {
            info->status = r->status;
            info->batched = r->batched ? 1 : 0;
            info->nIterations = r->st.nIter;
            info->converged = r->st.converged;
            info->initialResidual = r->st.initRes;
            info->finalResidual = r->st.finalRes;
            info->queueSeconds = r->tStart - r->tSubmit;
            info->setupSeconds = r->tSetup - r->tStart;
            info->solveSeconds = r->tEnd - r->tSetup;
            info->latencySeconds = r->tEnd - r->tSubmit;
        }
        if (r->status) throw std::runtime_error("request failed: " + r->error);
    });
}

int unap_cuda_server_destroy(long int server)
{
    return guarded([&] { delete server_from(server); });
}

int unap_cuda_set_server_graphs(int on) { return set_server_graphs(on); }

int unap_cuda_set_server_team_cells(int cells) { return set_server_team_cells(cells); }

int unap_cuda_set_server_amg(int nCoarsest, double eigRatio)
{
    return guarded([&] { set_server_amg(nCoarsest, eigRatio); });
}

}  // extern "C"
