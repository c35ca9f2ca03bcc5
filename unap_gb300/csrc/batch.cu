// Batched solves of many LDU systems of uneven size.
//
// Systems of at most team_solve_cells() cells are solved together in ONE
// launch: a team of CTAs per system (one CTA, or a thread-block cluster) runs
// the whole PCG or PBiCGStab solve (small_solve.cu), so a batch of hundreds
// of small systems costs one launch instead of hundreds of iterations x
// kernels.  Larger systems of the batch are solved one after another with
// the per-system Krylov driver.  Vectors enter and leave in the caller's
// cell order through one batched gather/scatter launch each.
//
// The launch shape (CTA size x CTAs per system) is picked by an autotuner:
// the first batch of each (size class, count class) is timed with every
// launchable shape, iterations capped, x reset between trials, and the
// fastest is cached for the pair.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <map>
#include <mutex>

#include "batch.hpp"
#include "device_common.cuh"

namespace unapgpu {

namespace {

struct PermJob {
    int n;
    const int* perm;
    const double* in;
    double* out;
    int toInternal;
};

// one block per job: out[i] = in[perm[i]] (to internal) or out[perm[i]] = in[i]
__global__ void batch_perm_kernel(const PermJob* jobs)
{
    const PermJob J = jobs[blockIdx.x];
    for (int i = threadIdx.x; i < J.n; i += blockDim.x) {
        if (J.toInternal)
            J.out[i] = J.in[J.perm[i]];
        else
            J.out[J.perm[i]] = J.in[i];
    }
}

std::mutex g_tune_mutex;
std::map<std::pair<int, int>, TeamShape> g_tuned;  // (size class, count class) -> shape
std::map<std::pair<int, int>, float> g_tunedMs;    // the shape's capped trial time
std::atomic<int> g_teamCells{kTeamSolveCells};
std::atomic<int> g_forceThreads{0}, g_forceCluster{0};  // shape override (0: tuner)
constexpr int kTuneIters = 10;  // iterations per timed trial

int size_class(int n)
{
    int c = 1;
    while (c < n) c <<= 1;
    return c;
}

int count_class(int m)
{
    return m <= 1 ? 1 : m <= 4 ? 4 : m <= 16 ? 16 : m <= 64 ? 64 : 1 << 30;
}

}  // namespace

int team_solve_cells() { return g_teamCells.load(); }

int set_team_solve_cells(int cells) { return g_teamCells.exchange(std::max(cells, 0)); }

void force_team_shape(int threads, int cluster)
{
    if (threads && !small_team_size_ok(threads, cluster))
        throw std::invalid_argument("team shape: threads 128, 256, 512 or 1024; cluster 1, 2, "
                                    "4, 8 or 16");
    if (threads && cluster > 1 && small_team_capacity(threads, cluster) <= 0)
        throw std::invalid_argument("team shape: this cluster cannot be scheduled on the device");
    g_forceThreads = threads;
    g_forceCluster = threads ? cluster : 0;
}

// tuner cache key: large groups (clusters of 16 only) apart from the rest
static std::pair<int, int> tune_key(int nMax, int m, bool largeGroup)
{
    return {size_class(nMax), count_class(m) + (largeGroup ? 1 : 0)};
}

TeamShape cached_team_shape(int nMax, int m, bool largeGroup)
{
    if (g_forceThreads.load()) return TeamShape{g_forceThreads.load(), g_forceCluster.load()};
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tuned.find(tune_key(nMax, m, largeGroup));
    return it == g_tuned.end() ? TeamShape{0, 0} : it->second;
}

TeamShape tuned_team_shape(cudaStream_t stream, const SmallSystem* dSys, int m, int nMax,
                           bool largeGroup, float* bestMs)
{
    const TeamShape have = cached_team_shape(nMax, m, largeGroup);
    if (have.threads) {
        // a forced shape was never timed: *bestMs is left as it is
        if (bestMs && !g_forceThreads.load()) {
            std::lock_guard<std::mutex> lock(g_tune_mutex);
            auto it = g_tunedMs.find(tune_key(nMax, m, largeGroup));
            if (it != g_tunedMs.end()) *bestMs = it->second;
        }
        return have;
    }
    std::vector<SmallSystem> sys((size_t)m);
    UNAP_CK(cudaMemcpyAsync(sys.data(), dSys, sizeof(SmallSystem) * (size_t)m,
                            cudaMemcpyDeviceToHost, stream));
    UNAP_CK(cudaStreamSynchronize(stream));
    // trial copies: iterations capped, no result written; a one-iteration
    // copy runs first for every shape (loads its kernel) untimed
    std::vector<SmallSystem> trial = sys, warm = sys;
    for (auto& S : trial) {
        S.maxIter = std::min(S.maxIter, kTuneIters);
        S.minIter = std::min(S.minIter, kTuneIters);
        S.result = nullptr;
    }
    for (auto& S : warm) {
        S.maxIter = 1;
        S.minIter = 0;
        S.result = nullptr;
    }
    DevArray<SmallSystem> dTrial, dWarm;
    dTrial.upload(trial.data(), trial.size(), stream);
    dWarm.upload(warm.data(), warm.size(), stream);
    size_t total = 0;
    for (auto& S : sys) total += (size_t)S.A.n;
    DevArray<double> x0(total);
    auto copy_x = [&](bool save) {
        size_t off = 0;
        for (auto& S : sys) {
            double* a = x0.p + off;
            UNAP_CK(cudaMemcpyAsync(save ? a : S.x, save ? S.x : a, sizeof(double) * (size_t)S.A.n,
                                    cudaMemcpyDeviceToDevice, stream));
            off += (size_t)S.A.n;
        }
    };
    copy_x(true);
    cudaEvent_t e0, e1;
    UNAP_CK(cudaEventCreate(&e0));
    UNAP_CK(cudaEventCreate(&e1));
    float best = 1e30f;
    TeamShape bestS;
    for (int C : {1, 2, 4, 8, 16}) {
        // systems above the whole-solve size: clusters of 16 CTAs of 256 or
        // more threads only (smaller teams take many times longer there)
        if (largeGroup && C != 16) continue;
        for (int t : {128, 256, 512, 1024}) {
            if (largeGroup && t < 256) continue;
            if (C > 1 && small_team_capacity(t, C) <= 0) continue;
            copy_x(false);
            launch_small_krylov(stream, dWarm.p, m, nullptr, t, C);
            copy_x(false);
            UNAP_CK(cudaEventRecord(e0, stream));
            launch_small_krylov(stream, dTrial.p, m, nullptr, t, C);
            UNAP_CK(cudaEventRecord(e1, stream));
            UNAP_CK(cudaEventSynchronize(e1));
            float ms = 0;
            UNAP_CK(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) {
                best = ms;
                bestS = TeamShape{t, C};
            }
        }
    }
    copy_x(false);
    UNAP_CK(cudaStreamSynchronize(stream));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tuned[tune_key(nMax, m, largeGroup)] = bestS;
        g_tunedMs[tune_key(nMax, m, largeGroup)] = best;
    }
    if (bestMs) *bestMs = best;
    return bestS;
}

// large groups: whole-solve launch (1) or one system after another (0),
// per (size class, count class); -1 while not measured
static std::map<std::pair<int, int>, int> g_largeMode;

int cached_large_mode(int nMax, int m)
{
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_largeMode.find(tune_key(nMax, m, true));
    return it == g_largeMode.end() ? -1 : it->second;
}

static void set_large_mode(int nMax, int m, int mode)
{
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_largeMode[tune_key(nMax, m, true)] = mode;
}

BatchSolver::BatchSolver(cudaStream_t s) : stream(s) {}

BatchSolver::~BatchSolver() = default;

const double* BatchSolver::factor(Matrix& A, int precond)
{
    // reciprocal diagonal for Diag (1/D), DIC or DILU, cached per matrix and
    // coefficient version
    Key k{&A, precond};
    auto it = factors.find(k);
    if (it != factors.end() && it->second.version == A.L->version) return it->second.rD.p;
    Fac f;
    f.version = A.L->version;
    f.rD.alloc((size_t)A.n());
    if (precond == 1) {
        std::vector<double> h((size_t)A.n());
        for (int i = 0; i < A.n(); ++i) h[(size_t)i] = 1.0 / A.host.diag[(size_t)A.L->perm[(size_t)i]];
        f.rD.upload(h, stream);
    } else {
        DevArray<double> dfac((size_t)A.n());
        Exec ex{stream, device_max_blocks()};
        dic_factor(ex, *A.L, precond == 3, dfac.p, f.rD.p);
        UNAP_CK(cudaStreamSynchronize(stream));
    }
    UNAP_CK(cudaStreamSynchronize(stream));
    auto& slot = factors[k];
    slot = std::move(f);
    return slot.rD.p;
}

void BatchSolver::forget(const Matrix* A)
{
    for (auto it = factors.begin(); it != factors.end();)
        it = it->first.A == A ? factors.erase(it) : std::next(it);
}

std::vector<SolveStats> BatchSolver::solve(const std::vector<BatchItem>& items)
{
    std::vector<SolveStats> out(items.size());
    std::vector<int> small, large;
    for (size_t i = 0; i < items.size(); ++i) {
        const BatchItem& it = items[i];
        if (!it.A->L->sweepable && (it.precond == 2 || it.precond == 3))
            throw std::invalid_argument("DIC/DILU need oriented, owner-sorted faces");
        (it.A->n() <= team_solve_cells() ? small : large).push_back((int)i);
    }
    if (!small.empty()) solveSmall(items, small, out);
    if (large.empty()) return out;
    // Larger systems: one whole-solve launch for the group (clusters of 16
    // CTAs, every system at once) or one system after another with the
    // per-step driver (each over the whole GPU), whichever the autotuner
    // measured faster for this (size class, count class): both run with
    // iterations capped, the group's initial guesses restored after each.
    int nMax = 0;
    for (int i : large) nMax = std::max(nMax, items[(size_t)i].A->n());
    const int m = (int)large.size();
    int mode = m >= 2 ? cached_large_mode(nMax, m) : 0;
    if (mode < 0) {
        const double tSeq = timeSequential(items, large);
        float tTeam = -1.0f;
        solveSmall(items, large, out, true, &tTeam);
        if (tTeam >= 0.0f) {
            mode = tTeam < tSeq * 1e3 ? 1 : 0;
            set_large_mode(nMax, m, mode);
        } else {
            mode = 1;  // a forced shape, never timed: nothing is cached
        }
        lastLargeMode = mode;
        return out;  // solved by the group launch already
    }
    lastLargeMode = mode;
    if (mode == 1) {
        solveSmall(items, large, out, true, nullptr);
        return out;
    }
    for (int i : large) out[(size_t)i] = solveOne(items[(size_t)i], items[(size_t)i].maxIter);
    return out;
}

SolveStats BatchSolver::solveOne(const BatchItem& it, int maxIter)
{
    auto P = make_ldu_precond(it.precond, *it.A);
    Krylov K(*it.A, P.get(), it.method == 1 ? Method::PBiCGStab : Method::PCG);
    K.tol = it.tol;
    K.relTol = it.relTol;
    K.maxIter = maxIter;
    K.minIter = std::min(it.minIter, maxIter);
    K.teamCells = 0;  // the per-step driver: this is the sequential arm
    return K.solveDevice(it.x, it.b);
}

double BatchSolver::timeSequential(const std::vector<BatchItem>& items, const std::vector<int>& idx)
{
    // each system solved alone with its iterations capped; the caller's
    // initial guesses are saved first and restored afterwards
    size_t total = 0;
    for (int i : idx) total += (size_t)items[(size_t)i].A->n();
    DevArray<double> x0(total);
    size_t off = 0;
    for (int i : idx) {
        const BatchItem& it = items[(size_t)i];
        UNAP_CK(cudaMemcpyAsync(x0.p + off, it.x, sizeof(double) * (size_t)it.A->n(),
                                cudaMemcpyDeviceToDevice, stream));
        off += (size_t)it.A->n();
    }
    UNAP_CK(cudaStreamSynchronize(stream));
    const auto t0 = std::chrono::steady_clock::now();
    for (int i : idx) (void)solveOne(items[(size_t)i], kTuneIters);
    const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    off = 0;
    for (int i : idx) {
        const BatchItem& it = items[(size_t)i];
        UNAP_CK(cudaMemcpyAsync(it.x, x0.p + off, sizeof(double) * (size_t)it.A->n(),
                                cudaMemcpyDeviceToDevice, stream));
        off += (size_t)it.A->n();
    }
    UNAP_CK(cudaStreamSynchronize(stream));
    return t;
}

void BatchSolver::solveSmall(const std::vector<BatchItem>& items, const std::vector<int>& idx,
                             std::vector<SolveStats>& out, bool largeGroup, float* tunedMs)
{
    const int m = (int)idx.size();
    size_t total = 0;
    int nMax = 0;
    for (int i : idx) {
        total += (size_t)items[(size_t)i].A->n();
        nMax = std::max(nMax, items[(size_t)i].A->n());
    }
    // workspace: internal x, b and 8 work vectors per system (reused)
    if (ws.n < total * 10) ws.alloc(total * 10);
    std::vector<SmallSystem> sys((size_t)m);
    std::vector<PermJob> in((size_t)2 * m), outJobs((size_t)m);
    std::vector<std::vector<int>> waves;
    waveDev.resize((size_t)m);
    size_t off = 0;
    for (int j = 0; j < m; ++j) {
        const BatchItem& it = items[(size_t)idx[(size_t)j]];
        Matrix& A = *it.A;
        const int n = A.n();
        double* xi = ws.p + off;
        double* bi = xi + n;
        double* wk = bi + n;
        off += (size_t)n * 10;
        SmallSystem& S = sys[(size_t)j];
        S = SmallSystem{};
        S.A = rows64(*A.L);
        S.nWave = A.L->nWave;
        waveDev[(size_t)j].upload(A.L->waveStart, stream);
        S.waveStart = waveDev[(size_t)j].p;
        S.rD = (it.precond >= 1 && it.precond <= 3) ? factor(A, it.precond) : nullptr;
        S.method = it.method == 1 ? 1 : 0;
        S.precond = (it.precond >= 1 && it.precond <= 3) ? it.precond : 0;
        S.tol = it.tol;
        S.relTol = it.relTol;
        S.maxIter = it.maxIter;
        S.minIter = it.minIter;
        S.zeroX = 0;
        S.x = xi;
        S.b = bi;
        S.work = wk;
        in[(size_t)2 * j] = PermJob{n, A.L->d_perm.p, it.x, xi, 1};
        in[(size_t)2 * j + 1] = PermJob{n, A.L->d_perm.p, it.b, bi, 1};
        outJobs[(size_t)j] = PermJob{n, A.L->d_perm.p, xi, it.x, 0};
    }
    if (results.n < (size_t)m) results.alloc((size_t)m);
    for (int j = 0; j < m; ++j) sys[(size_t)j].result = results.p + j;
    dSys.upload(sys.data(), sys.size(), stream);
    dIn.upload(reinterpret_cast<const unsigned char*>(in.data()), in.size() * sizeof(PermJob),
               stream);
    dOut.upload(reinterpret_cast<const unsigned char*>(outJobs.data()),
                outJobs.size() * sizeof(PermJob), stream);
    if (!capturing()) count_launches(1);
    batch_perm_kernel<<<2 * m, 256, 0, stream>>>(reinterpret_cast<const PermJob*>(dIn.p));

    const TeamShape shape = tuned_team_shape(stream, dSys.p, m, nMax, largeGroup, tunedMs);
    launch_small_krylov(stream, dSys.p, m, nullptr, shape.threads, shape.cluster);
    if (!capturing()) count_launches(1);
    batch_perm_kernel<<<m, 256, 0, stream>>>(reinterpret_cast<const PermJob*>(dOut.p));
    std::vector<SmallResult> res((size_t)m);
    UNAP_CK(cudaMemcpyAsync(res.data(), results.p, sizeof(SmallResult) * (size_t)m,
                            cudaMemcpyDeviceToHost, stream));
    UNAP_CK(cudaStreamSynchronize(stream));
    UNAP_CK(cudaGetLastError());
    for (int j = 0; j < m; ++j) {
        SolveStats& s = out[(size_t)idx[(size_t)j]];
        s.nIter = res[(size_t)j].nIter;
        s.converged = res[(size_t)j].converged;
        s.singular = res[(size_t)j].singular;
        s.initRes = res[(size_t)j].initRes;
        s.finalRes = res[(size_t)j].finalRes;
    }
    lastShape = shape;
}

}  // namespace unapgpu
