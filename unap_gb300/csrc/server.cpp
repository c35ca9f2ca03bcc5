// Continuous-batching solve server (see server.hpp).
#include <algorithm>
#include <chrono>

#include "amg.hpp"
#include "server.hpp"

namespace unapgpu {

namespace {
std::atomic<int> g_serverGraphs{1};
std::atomic<int> g_serverTeamCells{0};
// AMG requests: coarsest level target.  200 rather than the headline's
// 1000: the coarsest dense inverse (one launch per column) is a large part
// of a small request's setup (400 requests of the serving stream: 39.6
// solves/s against 37.7 with 1000)
std::atomic<int> g_serverCoarsest{200};
std::atomic<int> g_serverEigRatio10{300};  // AMG requests: Chebyshev ratio x 10
}  // namespace

void set_server_amg(int nCoarsest, double eigRatio)
{
    if (nCoarsest < 2 || !(eigRatio > 1.0))
        throw std::invalid_argument("server AMG: nCoarsest >= 2 and eigRatio > 1");
    g_serverCoarsest = nCoarsest;
    g_serverEigRatio10 = (int)(eigRatio * 10.0 + 0.5);
}

int server_graphs() { return g_serverGraphs.load(); }
int set_server_graphs(int on) { return g_serverGraphs.exchange(on ? 1 : 0); }
int set_server_team_cells(int cells) { return g_serverTeamCells.exchange(std::max(cells, 0)); }


double now_seconds()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

namespace {

// device-memory estimate of one request (matrix structure, vectors, the AMG
// hierarchy and its FP32 copies, the dense coarsest inverse)
size_t estimate_bytes(const ServeRequest& r)
{
    const size_t n = (size_t)r.A.n, nf = (size_t)r.A.nf;
    size_t base = 24 * nf + 112 * n + (r.A.symm ? 0 : 16 * nf);
    if (r.method == SERVE_AMG_MIXED || r.method == SERVE_AMG_FP64) {
        base = 2 * base + 8ull * 1000 * 1000;
        if (r.method == SERVE_AMG_MIXED) base += 2 * 8 * nf + 16 * n;
    }
    return base;
}

}  // namespace

Server::Server(const ServerParams& p) : params(p)
{
    if (params.memoryBudget <= 0) {
        size_t freeB = 0, totalB = 0;
        UNAP_CK(cudaMemGetInfo(&freeB, &totalB));
        params.memoryBudget = (long long)(0.8 * (double)freeB);
    }
    if (params.maxSlots < 1) params.maxSlots = 1;
    int dev = 0;
    UNAP_CK(cudaGetDevice(&dev));
    for (int i = 0; i < params.maxSlots; ++i)
        workers.emplace_back([this, dev] {
            cudaSetDevice(dev);
            largeWorker();
        });
    batchThread = std::thread([this, dev] {
        cudaSetDevice(dev);
        batchWorker();
    });
}

Server::~Server()
{
    {
        std::lock_guard<std::mutex> lk(mu);
        stopping = true;
    }
    cv.notify_all();
    for (auto& t : workers) t.join();
    batchThread.join();
}

bool Server::admissible(const ServeRequest& r) const
{
    // a request larger than the whole budget runs alone
    if ((long long)r.bytes >= params.memoryBudget) return used.load() == 0;
    return (long long)(used.load() + r.bytes) <= params.memoryBudget;
}

long long Server::submit(std::unique_ptr<ServeRequest> r)
{
    r->A.validate();
    if ((int)r->b.size() != r->A.n) throw std::invalid_argument("rhs size differs from nCells");
    const bool amg = r->method == SERVE_AMG_MIXED || r->method == SERVE_AMG_FP64;
    if (amg && !r->A.symm) throw std::invalid_argument("AMG-PCG needs a symmetric matrix");
    r->id = nextId++;
    r->bytes = estimate_bytes(*r);
    r->batched = !amg && r->A.n <= params.smallCells;
    r->tSubmit = now_seconds();
    const long long id = r->id;
    {
        std::lock_guard<std::mutex> lk(mu);
        ServeRequest* raw = r.get();
        all[id] = std::move(r);
        (raw->batched ? pendingSmall : pendingLarge).push_back(raw);
    }
    cv.notify_all();
    return id;
}

std::unique_ptr<ServeRequest> Server::wait(long long id)
{
    std::unique_lock<std::mutex> lk(mu);
    if (all.find(id) == all.end()) throw std::invalid_argument("unknown request id");
    // looked up again after every wake-up: another thread waiting on the
    // same id may have collected the request meanwhile
    doneCv.wait(lk, [&] {
        auto j = all.find(id);
        return j == all.end() || j->second->done;
    });
    auto it = all.find(id);
    if (it == all.end()) throw std::invalid_argument("request already collected");
    std::unique_ptr<ServeRequest> out = std::move(it->second);
    all.erase(it);
    return out;
}

void Server::finish(ServeRequest* r)
{
    r->tEnd = now_seconds();
    {
        // the budget is released under the lock: a worker between its
        // admission check (false) and its wait holds the lock, so the
        // release and the notification below cannot fall in that window
        std::lock_guard<std::mutex> lk(mu);
        r->done = true;
        used -= r->bytes;
    }
    doneCv.notify_all();
    cv.notify_all();
}

void Server::largeWorker()
{
    cudaStream_t s = nullptr;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    // every device array of this slot's requests comes from the memory pool
    // in this stream's order: a slot's setup never synchronizes the device
    // (and so never waits for the other slots' solves)
    StreamAllocScope scope(s);
    // Programmatic dependent launch off in the slots: a dependent kernel's
    // CTAs launched early wait on SMs the other slots' kernels could use
    // (8 concurrent PCG+DIC solves of 373k cells: 36.7 solves/s without it,
    // 22.1 with it)
    set_thread_wave_pdl(0);
    for (;;) {
        ServeRequest* r = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] {
                return stopping || (!pendingLarge.empty() && admissible(*pendingLarge.front()));
            });
            if (pendingLarge.empty() || !admissible(*pendingLarge.front())) {
                if (stopping) break;
                continue;
            }
            r = pendingLarge.front();
            pendingLarge.pop_front();
            used += r->bytes;
        }
        r->tStart = now_seconds();
        try {
            // AMG requests smooth every level by Chebyshev steps: their
            // matrix needs no wavefronts (cheaper setup, local gathers)
            const bool amgReq = r->method == SERVE_AMG_MIXED || r->method == SERVE_AMG_FP64;
            Matrix A(std::move(r->A), s, !amgReq);
            const size_t n = (size_t)A.n();
            DevArray<double> dx(n), db(n);
            db.upload(r->b, s);
            dx.zero(s);
            std::unique_ptr<AmgHierarchy> H;
            std::unique_ptr<Precond> P;
            Method m = Method::PCG;
            bool flexible = false, restart = false;
            if (r->method == SERVE_AMG_MIXED || r->method == SERVE_AMG_FP64) {
                // every level smoothed by Chebyshev steps of degree 3: no
                // wavefront chains, which dominate small systems' V-cycles
                AmgParams ap;
                ap.precision = r->method == SERVE_AMG_MIXED ? 1 : 0;
                ap.smoother = 1;
                ap.chebyDegree = 3;
                ap.chebyFrom = 0;
                ap.eigRatio = g_serverEigRatio10.load() / 10.0;
                ap.nCoarsest = g_serverCoarsest.load();
                H = std::make_unique<AmgHierarchy>(A, ap);
                P = std::make_unique<AmgPrecond>(*H);
                flexible = ap.precision == 1;
                restart = true;
            } else if (r->method == SERVE_PCG_DIC) {
                P = make_ldu_precond(2, A);
            } else {
                P = make_ldu_precond(3, A);
                m = Method::PBiCGStab;
            }
            Krylov K(A, P.get(), m);
            K.relTol = r->relTol;
            K.maxIter = r->maxIter;
            K.flexible = flexible;
            K.fusedOuter = r->method == SERVE_AMG_MIXED;
            K.trueResidualRestart = restart;
            // concurrent slots share the SMs: the persistent cooperative
            // executor needs every SM, so slots run per-step kernels,
            // replayed from CUDA graphs.  The slot's allocations are
            // stream-ordered, so a capture never meets another slot's
            // device-synchronizing allocation.
            K.useMega = params.maxSlots == 1;
            K.useGraph = server_graphs() != 0;
            // a PCG/PBiCGStab request runs as one whole-solve launch on a
            // thread-block cluster: it holds a few SMs for the whole solve
            // instead of issuing tens of thousands of wavefront launches
            // that contend with the other slots' launches
            K.teamCells = g_serverTeamCells.load();
            r->tSetup = now_seconds();
            r->st = K.solveDevice(dx.p, db.p);
            r->x.resize(n);
            UNAP_CK(cudaMemcpyAsync(r->x.data(), dx.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
            UNAP_CK(cudaStreamSynchronize(s));
        } catch (const std::exception& e) {
            r->status = -1;
            r->error = e.what();
        }
        finish(r);
    }
    if (s) cudaStreamDestroy(s);
}

void Server::batchWorker()
{
    cudaStream_t s = nullptr;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    {
        StreamAllocScope scope(s);
        set_thread_wave_pdl(0);
        BatchSolver B(s);
        for (;;) {
            std::vector<ServeRequest*> take;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] {
                    return stopping || (!pendingSmall.empty() && admissible(*pendingSmall.front()));
                });
                while (!pendingSmall.empty() && admissible(*pendingSmall.front())) {
                    ServeRequest* r = pendingSmall.front();
                    pendingSmall.pop_front();
                    used += r->bytes;
                    take.push_back(r);
                }
                if (take.empty()) {
                    if (stopping) break;
                    continue;
                }
            }
            const double t0 = now_seconds();
            std::vector<std::unique_ptr<Matrix>> mats;
            std::vector<DevArray<double>> xs, bs;
            std::vector<BatchItem> items;
            try {
                for (ServeRequest* r : take) {
                    r->tStart = t0;
                    mats.push_back(std::make_unique<Matrix>(std::move(r->A), s));
                    const size_t n = (size_t)mats.back()->n();
                    xs.emplace_back(n);
                    bs.emplace_back(n);
                    bs.back().upload(r->b, s);
                    xs.back().zero(s);
                }
                for (size_t i = 0; i < take.size(); ++i) {
                    BatchItem it;
                    it.A = mats[i].get();
                    it.method = take[i]->method == SERVE_BICG_DILU ? 1 : 0;
                    it.precond = take[i]->method == SERVE_BICG_DILU ? 3 : 2;
                    it.relTol = take[i]->relTol;
                    it.maxIter = take[i]->maxIter;
                    it.x = xs[i].p;
                    it.b = bs[i].p;
                    items.push_back(it);
                    take[i]->tSetup = now_seconds();
                }
                UNAP_CK(cudaStreamSynchronize(s));
                std::vector<SolveStats> st = B.solve(items);
                for (size_t i = 0; i < take.size(); ++i) {
                    ServeRequest* r = take[i];
                    r->st = st[i];
                    r->x.resize(xs[i].n);
                    UNAP_CK(cudaMemcpyAsync(r->x.data(), xs[i].p, xs[i].n * sizeof(double),
                                            cudaMemcpyDeviceToHost, s));
                }
                UNAP_CK(cudaStreamSynchronize(s));
            } catch (const std::exception& e) {
                for (ServeRequest* r : take) {
                    r->status = -1;
                    r->error = e.what();
                }
            }
            for (auto& m : mats) B.forget(m.get());
            mats.clear();
            xs.clear();
            bs.clear();
            for (ServeRequest* r : take) finish(r);
        }
    }
    if (s) cudaStreamDestroy(s);
}

}  // namespace unapgpu
