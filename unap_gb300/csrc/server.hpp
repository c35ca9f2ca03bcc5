// Continuous-batching solve server (server.cpp).
#pragma once

#include <atomic>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "batch.hpp"
#include "engine.hpp"

namespace unapgpu {

enum ServeMethod : int {
    SERVE_AMG_MIXED = 0,  // AMG-PCG, FP32 Chebyshev V-cycle, flexible FP64 PCG
    SERVE_AMG_FP64 = 1,   // AMG-PCG, FP64 Chebyshev V-cycle
    SERVE_PCG_DIC = 2,    // PCG + DIC
    SERVE_BICG_DILU = 3,  // PBiCGStab + DILU
};

struct ServeRequest {
    long long id = 0;
    HostLdu A;
    std::vector<double> b, x;
    int method = 0;
    double relTol = 1e-8;
    int maxIter = 1000;
    size_t bytes = 0;      // admission estimate
    bool batched = false;  // solved in a fused small-system launch
    double tSubmit = 0, tStart = 0, tSetup = 0, tEnd = 0;
    SolveStats st;
    int status = 0;  // 0 ok, < 0 error
    std::string error;
    bool done = false;
};

// Slots replay each Krylov iteration from a CUDA graph (1, default) or
// launch its kernels one by one (0); returns the previous setting.
int server_graphs();
int set_server_graphs(int on);
// PCG/PBiCGStab requests of up to this many cells that a slot (not the
// batch lane) solves run as one whole-solve launch (default: all; 0: never);
// returns the previous value.
int set_server_team_cells(int cells);
// AMG requests: coarsest level target (default 200 cells) and Chebyshev
// interval ratio (default 30), for requests started afterwards
void set_server_amg(int nCoarsest, double eigRatio);

struct ServerParams {
    long long memoryBudget = 0;  // bytes; 0: 80% of free device memory at start
    int maxSlots = 4;            // concurrent large solves (one stream each)
    int smallCells = 65536;      // PCG/PBiCGStab requests up to this size are batched
};

// Requests arrive with their matrix; a request is admitted when a slot (large
// lane) or the batch lane is free and its device-memory estimate fits the
// budget left by the solves in flight.  Large solves run on their own
// streams, so work of different requests overlaps on the GPU; the batch lane
// collects every small request that is pending when it starts and solves
// them in one fused launch.  Results are the same as a solve alone up to
// the summation order of dot products.
class Server {
public:
    explicit Server(const ServerParams& p);
    ~Server();
    long long submit(std::unique_ptr<ServeRequest> r);
    // blocks until request `id` is done; hands the request over
    std::unique_ptr<ServeRequest> wait(long long id);
    size_t inFlightBytes() const { return used.load(); }
    long long budget() const { return params.memoryBudget; }

private:
    ServerParams params;
    std::mutex mu;
    std::condition_variable cv;       // new work or freed memory
    std::condition_variable doneCv;   // a request finished
    std::deque<ServeRequest*> pendingLarge, pendingSmall;
    std::map<long long, std::unique_ptr<ServeRequest>> all;
    std::atomic<size_t> used{0};
    std::atomic<long long> nextId{1};
    bool stopping = false;
    std::vector<std::thread> workers;
    std::thread batchThread;
    void largeWorker();
    void batchWorker();
    bool admissible(const ServeRequest& r) const;
    void finish(ServeRequest* r);
};

double now_seconds();

}  // namespace unapgpu
