// Host-side engine: matrices, LDU preconditioners and the PCG / PBiCGStab
// drivers.  One solve keeps every vector and scalar on the device; the host
// only enqueues gated iterations (captured once into a CUDA graph) and polls
// the `done` flag of the device solver state between batches.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "engine.hpp"
#include "batch.hpp"

namespace unapgpu {

// ---- error text ---------------------------------------------------------
static thread_local std::string g_last_error;
std::shared_mutex& capture_gate()
{
    static std::shared_mutex m;
    return m;
}
bool& thread_in_capture()
{
    static thread_local bool v = false;
    return v;
}
cudaStream_t& thread_alloc_stream()
{
    static thread_local cudaStream_t s = nullptr;
    return s;
}
void keep_pool_memory()
{
    static std::mutex m;
    static std::vector<int> done;
    int dev = 0;
    UNAP_CK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(m);
    if (std::find(done.begin(), done.end(), dev) != done.end()) return;
    cudaMemPool_t pool;
    UNAP_CK(cudaDeviceGetDefaultMemPool(&pool, dev));
    // freed blocks stay in the pool (up to 32 GiB) for the next allocations
    unsigned long long keep = 32ull << 30;
    UNAP_CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    done.push_back(dev);
}
namespace {
std::mutex g_pinnedMutex;
std::map<size_t, std::vector<void*>> g_pinnedFree;  // block size -> free blocks
std::map<void*, size_t> g_pinnedSize;
}  // namespace
void* pinned_block_alloc(size_t bytes)
{
    const size_t sz = (bytes + 255) / 256 * 256;
    {
        std::lock_guard<std::mutex> lk(g_pinnedMutex);
        auto& f = g_pinnedFree[sz];
        if (!f.empty()) {
            void* p = f.back();
            f.pop_back();
            return p;
        }
    }
    void* p = nullptr;
    UNAP_CK(gated_malloc_host(&p, sz));
    std::lock_guard<std::mutex> lk(g_pinnedMutex);
    g_pinnedSize[p] = sz;
    return p;
}
void pinned_block_free(void* p)
{
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_pinnedMutex);
    auto it = g_pinnedSize.find(p);
    if (it == g_pinnedSize.end()) return;
    g_pinnedFree[it->second].push_back(p);
}
void order_after_default_stream(cudaStream_t s)
{
    // an event on the legacy default stream, waited for by s: everything
    // issued before the call to the legacy stream (and so to every blocking
    // stream) is done before s runs the call's kernels
    cudaEvent_t e;
    UNAP_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    UNAP_CK(cudaEventRecord(e, cudaStreamLegacy));
    UNAP_CK(cudaStreamWaitEvent(s, e, 0));
    UNAP_CK(cudaEventDestroy(e));  // released once it has completed
}
void set_last_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

// ---- Matrix ----------------------------------------------------------------
static std::atomic<int> g_matrixWavefronts{1};
int set_matrix_wavefronts(int on) { return g_matrixWavefronts.exchange(on ? 1 : 0); }
int matrix_wavefronts() { return g_matrixWavefronts.load(); }

Matrix::Matrix(HostLdu&& h, cudaStream_t s, bool wavefronts) : host(std::move(h)), stream(s)
{
    UNAP_CK(cudaGetDevice(&device));
    if (!stream) {
        UNAP_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        ownsStream = true;
    }
    host.validate();
    L = build_level(host, nullptr, false, stream, wavefronts);
}

Matrix::~Matrix()
{
    L.reset();
    if (ownsStream && stream) cudaStreamDestroy(stream);
}

void Matrix::setValues(const double* diag, const double* upper, const double* lower)
{
    std::memcpy(host.diag.data(), diag, sizeof(double) * (size_t)host.n);
    std::memcpy(host.upper.data(), upper, sizeof(double) * (size_t)host.nf);
    bool symm = (lower == nullptr || lower == upper);
    host.symm = symm;
    if (symm)
        host.lower.clear();
    else
        host.lower.assign(lower, lower + host.nf);
    update_level_values(*L, host, stream);
}

// ---- preconditioners -------------------------------------------------------
namespace {

Step diag_step(int n, const double* rD, const double* r, double* w, int slot);

class NoPrecond : public Precond {
public:
    explicit NoPrecond(int n) : n(n) {}
    bool fusesDot() const override { return true; }
    void apply(const Exec& ex, const double* r, double* w, const RedPool* pool, int site,
               KState* st, int fin, Gate g) override
    {
        // identity preconditioner (unapMatrixPrecond.cpp:4-17)
        diag_apply(ex, n, nullptr, r, w, pool ? pool->site(site, st, fin) : RSpec{}, g);
    }
    bool appendSteps(std::vector<Step>& out, std::vector<LevelRows>&, const double* r, double* w,
                     int slot, bool* dotFused) override
    {
        out.push_back(diag_step(n, nullptr, r, w, slot));
        *dotFused = true;
        return true;
    }
    int lduType() const override { return 0; }
    int n;
};

// w = rD r (rD == null: w = r) with the partial of w.r in `slot`
Step diag_step(int n, const double* rD, const double* r, double* w, int slot)
{
    Step s;
    s.op = ST_DIAG;
    s.single = mega_single_level(n);
    s.r1 = n;
    s.a = r;
    s.c = w;
    s.e = rD;
    s.red = slot;
    s.bytes = (rD ? 24.0 : 16.0) * n;
    return s;
}

class DiagPrecond : public Precond {
public:
    explicit DiagPrecond(Matrix& A) : n(A.n())
    {
        // lduDiagPrecond.cpp:13-41: rD = 1 / D
        std::vector<double> h((size_t)n);
        for (int i = 0; i < n; ++i) h[(size_t)i] = 1.0 / A.host.diag[(size_t)A.L->perm[(size_t)i]];
        rD.upload(h, A.stream);
        UNAP_CK(cudaStreamSynchronize(A.stream));
    }
    bool fusesDot() const override { return true; }
    void apply(const Exec& ex, const double* r, double* w, const RedPool* pool, int site,
               KState* st, int fin, Gate g) override
    {
        diag_apply(ex, n, rD.p, r, w, pool ? pool->site(site, st, fin) : RSpec{}, g);
    }
    bool appendSteps(std::vector<Step>& out, std::vector<LevelRows>&, const double* r, double* w,
                     int slot, bool* dotFused) override
    {
        out.push_back(diag_step(n, rD.p, r, w, slot));
        *dotFused = true;
        return true;
    }
    int lduType() const override { return 1; }
    const double* lduRD() const override { return rD.p; }
    int n;
    DevArray<double> rD;
};

class DicPrecond : public Precond {
public:
    DicPrecond(Matrix& A, bool dilu) : L(*A.L), dilu(dilu)
    {
        if (!L.sweepable)
            throw std::invalid_argument(
                "DIC/DILU need faces oriented lowerAddr < upperAddr and sorted by owner, "
                "and a matrix built with wavefronts");
        Exec ex;
        ex.s = A.stream;
        ex.maxBlocks = device_max_blocks();
        dfac.alloc((size_t)L.n);
        rD.alloc((size_t)L.n);
        dic_factor(ex, L, dilu, dfac.p, rD.p);
        UNAP_CK(cudaGetLastError());
        UNAP_CK(cudaStreamSynchronize(A.stream));
    }
    bool fusesDot() const override { return true; }
    void apply(const Exec& ex, const double* r, double* w, const RedPool* pool, int site,
               KState* st, int fin, Gate g) override
    {
        dic_apply(ex, L, dilu, rD.p, r, w, pool, site, st, fin, g);
    }
    bool appendSteps(std::vector<Step>& out, std::vector<LevelRows>& lv, const double* r,
                     double* w, int slot, bool* dotFused) override
    {
        // level 0 of the table is this matrix
        Rows<double> A = rows64(L);
        const bool single = mega_single_level(L.n);
        for (int k = 0; k < L.nWave; ++k) {
            Step s;
            s.op = ST_DIC_FWD;
            s.single = single;
            s.r0 = L.waveStart[k];
            s.r1 = L.waveStart[k + 1];
            s.a = r;
            s.c = w;
            s.e = rD.p;
            s.d = dilu ? A.val : A.valT;
            // DIC/DILU apply: 40 N + 32 F over both sweeps, half each
            s.bytes = 0.5 * ((s.r1 - s.r0) * 40.0 + (double)(s.r1 - s.r0) / L.n * L.nf * 32.0);
            out.push_back(s);
        }
        bool firstBwd = true;
        for (int k = L.nWave - 1; k >= 0; --k) {
            Step s;
            s.op = ST_DIC_BWD;
            s.single = single;
            s.r0 = L.waveStart[k];
            s.r1 = L.waveStart[k + 1];
            s.a = r;
            s.c = w;
            s.e = rD.p;
            s.red = slot;
            s.f0 = firstBwd ? 0 : 1;
            firstBwd = false;
            s.bytes = 0.5 * ((s.r1 - s.r0) * 40.0 + (double)(s.r1 - s.r0) / L.n * L.nf * 32.0);
            out.push_back(s);
        }
        (void)lv;
        *dotFused = L.nWave > 0;
        return true;
    }
    int lduType() const override { return dilu ? 3 : 2; }
    const double* lduRD() const override { return rD.p; }
    const Level& L;
    bool dilu;
    DevArray<double> dfac, rD;
};

}  // namespace

std::unique_ptr<Precond> make_ldu_precond(int type, Matrix& A)
{
    // fortranInterface.cpp:227-238: 1 Diag, 2 DIC, 3 DILU, otherwise none
    if (type == 1) return std::make_unique<DiagPrecond>(A);
    if (type == 2) return std::make_unique<DicPrecond>(A, false);
    if (type == 3) return std::make_unique<DicPrecond>(A, true);
    return std::make_unique<NoPrecond>(A.n());
}

// ---- Krylov driver -------------------------------------------------------------
enum { S_INIT = 0, S_WR, S_ALPHA, S_RES, S_TRUE, S_BS, S_BOMEGA, S_NSITES };

// per-step launches in CUDA graphs measured faster than the persistent
// executor on the 256^3 AMG-PCG solve, so they are the default
static std::atomic<int> g_persistent{0};
int set_default_executor(int persistent) { return g_persistent.exchange(persistent ? 1 : 0); }

Krylov::Krylov(Matrix& A_, Precond* P_, Method m) : A(A_), P(P_), method(m)
{
    useMega = g_persistent.load() != 0;
    teamCells = team_solve_cells();
    n = A.n();
    ex.s = A.stream;
    ex.maxBlocks = device_max_blocks();
    size_t N = (size_t)n;
    x.alloc(N);
    b.alloc(N);
    r.alloc(N);
    z.alloc(N);
    p.alloc(N);
    q.alloc(N);
    if (method == Method::PBiCGStab) {
        r0.alloc(N);
        y.alloc(N);
        Ay.alloc(N);
        s.alloc(N);
        t.alloc(N);
    }
    UNAP_CK(gated_malloc((void**)&d_st, sizeof(KState)));
    h_st = static_cast<KState*>(pinned_block_alloc(sizeof(KState)));
    // partial buffers for one CTA per 256 rows (row kernels launch that many)
    pool.init(S_NSITES, std::max(ex.maxBlocks, div_up(n, kBlock)), std::max(1, A.L->nWave) + 1,
              ex.s);
    UNAP_CK(cudaEventCreate(&ev0));
    UNAP_CK(cudaEventCreate(&ev1));
}

Krylov::~Krylov()
{
    if (graphExec) cudaGraphExecDestroy(graphExec);
    if (graph) cudaGraphDestroy(graph);
    if (d_st) gated_free(d_st);
    pinned_block_free(h_st);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
}

void Krylov::initState()
{
    KState h;
    std::memset(&h, 0, sizeof(h));
    h.wArA = 1.0e37;  // GREAT, PCG.cpp:57
    h.tol = tol;
    h.relTol = relTol;
    h.maxIter = maxIter;
    h.minIter = minIter;
    h.first = 1;
    h.flexible = flexible ? 1 : 0;
    h.trueRes = -1.0;
    *h_st = h;
    UNAP_CK(cudaMemcpyAsync(d_st, h_st, sizeof(KState), cudaMemcpyHostToDevice, ex.s));
}

void Krylov::readState()
{
    UNAP_CK(cudaMemcpyAsync(h_st, d_st, sizeof(KState), cudaMemcpyDeviceToHost, ex.s));
    UNAP_CK(cudaStreamSynchronize(ex.s));
}

// PCG.cpp:97-180 with the vector work fused into four kernels (plus the
// preconditioner's own sweeps).  wA of the reference is split into z
// (preconditioned residual) and q (A p) so flexible PCG can use z.q.
void Krylov::enqueuePcgIteration()
{
    Gate g{d_st, 1};
    Rows<double> Ar = rows64(*A.L);
    if (P->fusesDot() && !flexible) {
        P->apply(ex, r.p, z.p, &pool, S_WR, d_st, FIN_PCG_WR, g);
    } else {
        P->apply(ex, r.p, z.p, nullptr, 0, d_st, FIN_NONE, g);
        k_dot2(ex, n, z.p, r.p, flexible ? z.p : nullptr, flexible ? q.p : nullptr,
               pool.site(S_WR, d_st, FIN_PCG_WR), g, fusedOuter);
    }
    k_pcg_direction(ex, n, z.p, p.p, d_st, g, fusedOuter);
    k_spmv<double>(ex, Ar, p.p, q.p, p.p, pool.site(S_ALPHA, d_st, FIN_PCG_ALPHA), g, fusedOuter);
    k_pcg_update(ex, n, x.p, r.p, p.p, q.p, pool.site(S_RES, d_st, FIN_PCG_RES), g, fusedOuter);
}

// PBiCGStab.cpp:155-456.  rA0.rA of the next iteration is fused into the
// update kernel; `early` (converged on ||s||) gates the second half.
void Krylov::enqueueBicgIteration()
{
    Gate g3{d_st, 3}, g1{d_st, 1};
    Rows<double> Ar = rows64(*A.L);
    k_bicg_direction(ex, n, r.p, Ay.p, p.p, d_st, g3);
    P->apply(ex, p.p, y.p, nullptr, 0, d_st, FIN_NONE, g3);
    k_spmv<double>(ex, Ar, y.p, Ay.p, r0.p, pool.site(S_ALPHA, d_st, FIN_BICG_ALPHA), g3);
    k_bicg_s(ex, n, r.p, Ay.p, s.p, pool.site(S_BS, d_st, FIN_BICG_S), g3);
    P->apply(ex, s.p, z.p, nullptr, 0, d_st, FIN_NONE, g3);
    // t = A z; tAtA = t.t and omega numerator t.s
    k_spmv<double>(ex, Ar, z.p, t.p, nullptr, RSpec{}, g3);
    k_dot2(ex, n, t.p, t.p, t.p, s.p, pool.site(S_BOMEGA, d_st, FIN_BICG_OMEGA), g3);
    k_bicg_update(ex, n, x.p, r.p, y.p, z.p, s.p, t.p, r0.p, pool.site(S_RES, d_st, FIN_BICG_RES),
                  g1);
}

// PCG.cpp:35-183 as one step program: init = r = b - A x and its norm, then
// per iteration the preconditioner's steps, w.r (+ z.q), direction, q = A p
// with q.p, and the x/r update with r.r, each reduction followed by the
// scalar finalize the per-launch kernels run in their last block.
bool Krylov::stepProgram(std::vector<Step>& steps, std::vector<LevelRows>& lv, int& nInitOut)
{
    if (method != Method::PCG) return false;
    steps.clear();
    lv.assign(1, LevelRows{});
    lv[0].r64 = rows64(*A.L);
    if (A.L->d_val32.p) lv[0].r32 = rows32(*A.L);
    const bool single = mega_single_level(n);
    auto scalar = [&](int fin, int slot) {
        Step s;
        s.op = ST_SCALAR;
        s.f0 = fin;
        s.red = slot;
        s.r1 = -1;
        steps.push_back(s);
    };
    Step s0;
    s0.op = ST_RESID_NORM;
    s0.single = single;
    s0.a = x.p;
    s0.b = b.p;
    s0.c = r.p;
    s0.red = 4;
    s0.bytes = 32.0 * n + 16.0 * A.L->nf;
    steps.push_back(s0);
    scalar(FIN_INIT_RES, 4);
    const int nInit = (int)steps.size();
    bool fused = false;
    if (!P->appendSteps(steps, lv, r.p, z.p, 0, &fused)) return false;
    if (!fused || flexible) {
        Step d;
        d.op = ST_DOT2;
        d.single = single;
        d.r1 = n;
        d.a = z.p;
        d.b = r.p;
        d.c = flexible ? z.p : nullptr;
        d.d = flexible ? q.p : nullptr;
        d.red = 0;
        d.bytes = (flexible ? 24.0 : 16.0) * n;
        steps.push_back(d);
    }
    scalar(FIN_PCG_WR, 0);
    Step dir;
    dir.op = ST_PCG_DIR;
    dir.r1 = n;
    dir.a = z.p;
    dir.c = p.p;
    dir.bytes = 24.0 * n;
    steps.push_back(dir);
    Step mv;
    mv.op = ST_SPMV_DOT;
    mv.single = single;
    mv.a = p.p;
    mv.c = q.p;
    mv.red = 2;
    mv.bytes = 24.0 * n + 16.0 * A.L->nf;
    steps.push_back(mv);
    scalar(FIN_PCG_ALPHA, 2);
    Step up;
    up.op = ST_PCG_UPD;
    up.r1 = n;
    up.c = x.p;
    up.d = r.p;
    up.a = p.p;
    up.b = q.p;
    up.red = 4;
    up.bytes = 48.0 * n;
    steps.push_back(up);
    scalar(FIN_PCG_RES, 4);
    nInitOut = nInit;
    megaInitBytes = megaIterBytes = 0;
    for (int i = 0; i < (int)steps.size(); ++i)
        (i < nInit ? megaInitBytes : megaIterBytes) += steps[(size_t)i].bytes;
    bytesKnown = true;
    return true;
}

bool Krylov::buildMega()
{
    megaTried = true;
    std::vector<Step> steps;
    std::vector<LevelRows> lv;
    int nInit = 0;
    if (!stepProgram(steps, lv, nInit)) return false;
    mega = std::make_unique<MegaRunner>();
    mega->setProgram(steps, nInit, lv, 6, ex.s);
    megaSteps = (int)steps.size();
    return true;
}

void Krylov::enqueueIteration()
{
    if (method == Method::PCG)
        enqueuePcgIteration();
    else
        enqueueBicgIteration();
}

void Krylov::runIterations()
{
    if (useGraph && !graphExec) {
        CaptureGate gate;
        UNAP_CK(cudaStreamBeginCapture(ex.s, cudaStreamCaptureModeThreadLocal));
        set_capturing(true);
        try {
            enqueueIteration();
        } catch (...) {
            set_capturing(false);
            cudaStreamEndCapture(ex.s, &graph);
            throw;
        }
        set_capturing(false);
        UNAP_CK(cudaStreamEndCapture(ex.s, &graph));
        UNAP_CK(cudaGraphInstantiate(&graphExec, graph, 0));
        size_t nodes = 0;
        UNAP_CK(cudaGraphGetNodes(graph, nullptr, &nodes));
        graphKernels = (long long)nodes;
    }
    int batch = 1;
    int launched = 0;
    for (;;) {
        for (int k = 0; k < batch; ++k) {
            if (useGraph) {
                UNAP_CK(cudaGraphLaunch(graphExec, ex.s));
                count_launches(graphKernels);
            } else {
                enqueueIteration();
            }
        }
        launched += batch;
        UNAP_CK(cudaGetLastError());
        readState();
        if (h_st->done || h_st->singular) break;
        if (launched > maxIter + 2) break;  // safety: every iteration advances nIter
        batch = std::min(batch * 2, 16);
    }
}

SolveStats Krylov::solveTeam(double* x_ref, const double* b_ref)
{
    // the whole solve in one launch: a team of CTAs (one, or a cluster)
    // runs PCG.cpp:35-183 / PBiCGStab.cpp:45-459 with the preconditioner's
    // own reciprocal diagonal; the launch shape comes from the autotuner
    const Level& L = *A.L;
    const size_t N = (size_t)n;
    if (!teamWork.p) {
        teamWork.alloc(N * (method == Method::PBiCGStab ? 8 : 3));
        teamWaves.upload(L.waveStart, ex.s);
        teamSys.alloc(sizeof(SmallSystem) + sizeof(SmallResult));
    }
    SmallSystem* dS = reinterpret_cast<SmallSystem*>(teamSys.p);
    SmallResult* dR = reinterpret_cast<SmallResult*>(teamSys.p + sizeof(SmallSystem));
    SmallSystem S{};
    S.A = rows64(L);
    S.waveStart = teamWaves.p;
    S.nWave = L.nWave;
    S.precond = P->lduType();
    S.rD = S.precond ? P->lduRD() : nullptr;
    S.method = method == Method::PBiCGStab ? 1 : 0;
    S.tol = tol;
    S.relTol = relTol;
    S.maxIter = maxIter;
    S.minIter = minIter;
    S.zeroX = 0;
    S.x = x.p;
    S.b = b.p;
    S.work = teamWork.p;
    S.result = dR;
    UNAP_CK(cudaMemcpyAsync(dS, &S, sizeof(S), cudaMemcpyHostToDevice, ex.s));
    if (!cached_team_shape(n, 1).threads) {
        // first solve of this size class: the tuner's trials run on this
        // system (x restored after each), before the timed solve
        k_to_internal<double>(ex, n, L.d_perm.p, x_ref, x.p);
        k_to_internal<double>(ex, n, L.d_perm.p, b_ref, b.p);
        (void)tuned_team_shape(ex.s, dS, 1, n);
    }
    const TeamShape shape = cached_team_shape(n, 1);
    UNAP_CK(cudaEventRecord(ev0, ex.s));
    k_to_internal<double>(ex, n, L.d_perm.p, x_ref, x.p);
    k_to_internal<double>(ex, n, L.d_perm.p, b_ref, b.p);
    launch_small_krylov(ex.s, dS, 1, nullptr, shape.threads, shape.cluster);
    k_to_reference<double>(ex, n, L.d_perm.p, x.p, x_ref);
    UNAP_CK(cudaEventRecord(ev1, ex.s));
    SmallResult R{};
    UNAP_CK(cudaMemcpyAsync(&R, dR, sizeof(R), cudaMemcpyDeviceToHost, ex.s));
    UNAP_CK(cudaStreamSynchronize(ex.s));
    UNAP_CK(cudaGetLastError());
    SolveStats out;
    float ms = 0;
    UNAP_CK(cudaEventElapsedTime(&ms, ev0, ev1));
    out.seconds = ms * 1e-3;
    out.nIter = R.nIter;
    out.initRes = R.initRes;
    out.finalRes = R.finalRes;
    out.converged = R.converged;
    out.singular = R.singular;
    if (!bytesKnown && method == Method::PCG) {
        std::vector<Step> steps;
        std::vector<LevelRows> lv;
        int nInit = 0;
        stepProgram(steps, lv, nInit);
    }
    if (bytesKnown) out.bytes = megaInitBytes + (double)out.nIter * megaIterBytes;
    lastShape = shape;
    return out;
}

SolveStats Krylov::solveDevice(double* x_ref, const double* b_ref)
{
    if (n > 0 && n <= teamCells && !flexible && !trueResidualRestart && P && P->lduType() >= 0)
        return solveTeam(x_ref, b_ref);
    SolveStats out;
    const Level& L = *A.L;
    UNAP_CK(cudaEventRecord(ev0, ex.s));
    k_to_internal<double>(ex, n, L.d_perm.p, x_ref, x.p);
    k_to_internal<double>(ex, n, L.d_perm.p, b_ref, b.p);
    initState();
    Rows<double> Ar = rows64(L);
    if (useMega && !megaTried) megaReady = buildMega();
    const bool viaMega = useMega && megaReady;
    if (viaMega) {
        // the step program's init part computes r = b - A x and its norm
    } else if (method == Method::PCG) {
        // PCG.cpp:61-75: r = b - A x, initialResidual = normFactor(r)
        k_residual<double>(ex, Ar, x.p, b.p, r.p, pool.site(S_INIT, d_st, FIN_INIT_RES), Gate{});
    } else {
        // PBiCGStab.cpp:72-91: yA = A x; r = r0 = b - yA
        k_spmv<double>(ex, Ar, x.p, y.p, nullptr, RSpec{}, Gate{});
        k_bicg_init(ex, n, b.p, y.p, r.p, r0.p, pool.site(S_INIT, d_st, FIN_BICG_INIT));
    }
    if (n > 0) {
        bool restarted = false;
        for (;;) {
            if (viaMega) {
                if (!mega->run(d_st, maxIter + 1, ex.s, restarted))
                    throw CudaError("step executor: a grid barrier wait timed out");
                readState();
            } else {
                runIterations();
            }
            if (!trueResidualRestart || h_st->singular || !h_st->converged) break;
            // true residual check: restart from b - A x if the recurrence drifted
            k_residual<double>(ex, Ar, x.p, b.p, z.p, pool.site(S_TRUE, d_st, FIN_TRUE_RES),
                               Gate{});
            readState();
            double tr = h_st->trueRes;
            bool ok = (tr < tol) || (relTol > 1e-37 && tr <= relTol * h_st->initRes);
            if (ok || h_st->nIter >= maxIter) break;
            UNAP_CK(cudaMemcpyAsync(r.p, z.p, sizeof(double) * (size_t)n,
                                    cudaMemcpyDeviceToDevice, ex.s));
            h_st->done = 0;
            h_st->converged = 0;
            h_st->first = 1;
            h_st->finalRes = tr;
            h_st->wArA = 1.0e37;
            UNAP_CK(cudaMemcpyAsync(d_st, h_st, sizeof(KState), cudaMemcpyHostToDevice, ex.s));
            restarted = true;
        }
    }
    k_to_reference<double>(ex, n, L.d_perm.p, x.p, x_ref);
    UNAP_CK(cudaEventRecord(ev1, ex.s));
    readState();
    float ms = 0;
    UNAP_CK(cudaEventElapsedTime(&ms, ev0, ev1));
    out.seconds = ms * 1e-3;
    out.nIter = h_st->nIter;
    out.initRes = h_st->initRes;
    out.finalRes = h_st->finalRes;
    out.trueRes = h_st->trueRes;
    out.converged = h_st->converged;
    out.singular = h_st->singular;
    out.status = h_st->status;
    // algorithmic bytes of the iteration's steps (the same for both executors)
    if (!bytesKnown && method == Method::PCG) {
        std::vector<Step> steps;
        std::vector<LevelRows> lv;
        int nInit = 0;
        stepProgram(steps, lv, nInit);
    }
    if (bytesKnown) out.bytes = megaInitBytes + (double)out.nIter * megaIterBytes;
    return out;
}

SolveStats Krylov::solveHost(double* xh, const double* bh)
{
    DevArray<double> dx((size_t)n), db((size_t)n);
    dx.upload(xh, (size_t)n, ex.s);
    db.upload(bh, (size_t)n, ex.s);
    SolveStats st = solveDevice(dx.p, db.p);
    if (n) UNAP_CK(cudaMemcpyAsync(xh, dx.p, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, ex.s));
    UNAP_CK(cudaStreamSynchronize(ex.s));
    return st;
}

// ---- dense SPD inverse (coarsest level) --------------------------------------
// Cholesky A = L L^T column by column, L^-1 by forward substitution,
// A^-1 = L^-T L^-1; every sum runs over ascending index from 0 (same
// operation order as the oracle's restatement, so both produce the same
// bits).
bool dense_spd_inverse(int n, const std::vector<double>& A, std::vector<double>& inv)
{
    // Cholesky A = L L^T, then Li = L^-1, then inv = Li^T Li.  Every element
    // is a sum in ascending k, the order the oracle uses; the loops run four
    // independent sums side by side over contiguous rows for speed.
    const size_t N = (size_t)n;
    std::vector<double> L(N * N, 0.0), LiT(N * N, 0.0);  // LiT[j*N + k] = Li[k][j]
    inv.assign(N * N, 0.0);
    for (int j = 0; j < n; ++j) {
        const double* Lj = &L[(size_t)j * N];
        double s = A[(size_t)j * N + j];
        for (int k = 0; k < j; ++k) s -= Lj[k] * Lj[k];
        if (!(s > 0.0)) return false;
        const double djj = std::sqrt(s);
        L[(size_t)j * N + j] = djj;
        int i = j + 1;
        for (; i + 3 < n; i += 4) {
            const double* a0 = &L[(size_t)i * N];
            const double* a1 = a0 + N;
            const double* a2 = a1 + N;
            const double* a3 = a2 + N;
            double t0 = A[(size_t)i * N + j], t1 = A[(size_t)(i + 1) * N + j];
            double t2 = A[(size_t)(i + 2) * N + j], t3 = A[(size_t)(i + 3) * N + j];
            for (int k = 0; k < j; ++k) {
                const double l = Lj[k];
                t0 -= a0[k] * l;
                t1 -= a1[k] * l;
                t2 -= a2[k] * l;
                t3 -= a3[k] * l;
            }
            L[(size_t)i * N + j] = t0 / djj;
            L[(size_t)(i + 1) * N + j] = t1 / djj;
            L[(size_t)(i + 2) * N + j] = t2 / djj;
            L[(size_t)(i + 3) * N + j] = t3 / djj;
        }
        for (; i < n; ++i) {
            const double* ai = &L[(size_t)i * N];
            double t = A[(size_t)i * N + j];
            for (int k = 0; k < j; ++k) t -= ai[k] * Lj[k];
            L[(size_t)i * N + j] = t / djj;
        }
    }
    // Li row by row: Li[i][j] = -(sum_{k=j}^{i-1} L[i][k] Li[k][j]) / L[i][i]
    for (int i = 0; i < n; ++i) {
        const double* Lr = &L[(size_t)i * N];
        const double lii = Lr[i];
        LiT[(size_t)i * N + i] = 1.0 / lii;
        int j = 0;
        for (; j + 3 < i; j += 4) {
            const double* c0 = &LiT[(size_t)j * N];
            const double* c1 = c0 + N;
            const double* c2 = c1 + N;
            const double* c3 = c2 + N;
            double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
            // sums start at k = j, j+1, j+2, j+3 respectively
            t0 += Lr[j] * c0[j];
            t0 += Lr[j + 1] * c0[j + 1];
            t1 += Lr[j + 1] * c1[j + 1];
            t0 += Lr[j + 2] * c0[j + 2];
            t1 += Lr[j + 2] * c1[j + 2];
            t2 += Lr[j + 2] * c2[j + 2];
            for (int k = j + 3; k < i; ++k) {
                const double l = Lr[k];
                t0 += l * c0[k];
                t1 += l * c1[k];
                t2 += l * c2[k];
                t3 += l * c3[k];
            }
            LiT[(size_t)j * N + i] = -t0 / lii;
            LiT[(size_t)(j + 1) * N + i] = -t1 / lii;
            LiT[(size_t)(j + 2) * N + i] = -t2 / lii;
            LiT[(size_t)(j + 3) * N + i] = -t3 / lii;
        }
        for (; j < i; ++j) {
            const double* c = &LiT[(size_t)j * N];
            double t = 0.0;
            for (int k = j; k < i; ++k) t += Lr[k] * c[k];
            LiT[(size_t)j * N + i] = -t / lii;
        }
    }
    // inv[i][j] = sum_{k=i}^{n-1} Li[k][i] Li[k][j], j <= i
    for (int i = 0; i < n; ++i) {
        const double* ci = &LiT[(size_t)i * N];
        int j = 0;
        for (; j + 3 <= i; j += 4) {
            const double* c0 = &LiT[(size_t)j * N];
            const double* c1 = c0 + N;
            const double* c2 = c1 + N;
            const double* c3 = c2 + N;
            double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
            for (int k = i; k < n; ++k) {
                const double a = ci[k];
                t0 += a * c0[k];
                t1 += a * c1[k];
                t2 += a * c2[k];
                t3 += a * c3[k];
            }
            const double t[4] = {t0, t1, t2, t3};
            for (int q = 0; q < 4; ++q) {
                inv[(size_t)i * N + j + q] = t[q];
                inv[(size_t)(j + q) * N + i] = t[q];
            }
        }
        for (; j <= i; ++j) {
            const double* cj = &LiT[(size_t)j * N];
            double t = 0.0;
            for (int k = i; k < n; ++k) t += ci[k] * cj[k];
            inv[(size_t)i * N + j] = t;
            inv[(size_t)j * N + i] = t;
        }
    }
    return true;
}

}  // namespace unapgpu
