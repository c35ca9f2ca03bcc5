// C ABI of the AMG-PCG solver (declared in include/unap_cuda.h).
#include <cstring>
#include <cstdio>
#include <memory>

#include "amg.hpp"
#include "capi_handles.hpp"
#include "../../include/unap_cuda.h"

using namespace unapgpu;

namespace {

struct AmgHandle {
    static constexpr unsigned kMagic = 0x414d4731u;  // "AMG1"
    unsigned magic = kMagic;
    Matrix* A = nullptr;
    unap_cuda_amg_params p{};
    std::unique_ptr<AmgHierarchy> H;
    std::unique_ptr<AmgPrecond> P;
    std::unique_ptr<Krylov> K;
    DevArray<double> dx, db;  // staging for host solves (reference order)
    ~AmgHandle() { magic = 0; }
};

AmgHandle* amg_from(long int h)
{
    AmgHandle* a = reinterpret_cast<AmgHandle*>(h);
    if (!a || a->magic != AmgHandle::kMagic) throw std::invalid_argument("invalid AMG handle");
    return a;
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

void put(const SolveStats& s, unap_cuda_stats* o)
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

}  // namespace

extern "C" {

void unap_cuda_amg_default_params(unap_cuda_amg_params* p)
{
    if (!p) return;
    p->nCoarsest = 1000;
    p->maxLevels = 50;
    p->nPreSweeps = 2;
    p->nPostSweeps = 2;
    p->precision = 0;
    p->flexible = 0;
    p->tol = 0.0;
    p->relTol = 1e-10;
    p->maxIter = 500;
    p->minIter = 0;
    p->smoother = 0;
    p->chebyDegree = 3;
    p->chebyFrom = 0;
    p->eigRatio = 30.0;
    p->fusedOuter = 1;
}

int unap_cuda_amg_create(long int* amg, long int matrix, const unap_cuda_amg_params* p)
{
    return guarded([&] {
        if (!amg) throw std::invalid_argument("null handle pointer");
        auto h = std::make_unique<AmgHandle>();
        if (p)
            h->p = *p;
        else
            unap_cuda_amg_default_params(&h->p);
        if (h->p.precision != 0 && h->p.precision != 1)
            throw std::invalid_argument("precision must be 0 (FP64) or 1 (FP32 V-cycle)");
        h->A = &mat_from(matrix)->get();
        AmgParams ap;
        ap.nCoarsest = h->p.nCoarsest;
        ap.maxLevels = h->p.maxLevels;
        ap.nPre = h->p.nPreSweeps;
        ap.nPost = h->p.nPostSweeps;
        ap.precision = h->p.precision;
        ap.smoother = h->p.smoother;
        ap.chebyDegree = h->p.chebyDegree;
        ap.chebyFrom = h->p.chebyFrom;
        ap.eigRatio = h->p.eigRatio;
        h->H = std::make_unique<AmgHierarchy>(*h->A, ap);
        h->P = std::make_unique<AmgPrecond>(*h->H);
        h->K = std::make_unique<Krylov>(*h->A, h->P.get(), Method::PCG);
        h->K->tol = h->p.tol;
        h->K->relTol = h->p.relTol;
        h->K->maxIter = h->p.maxIter;
        h->K->minIter = h->p.minIter;
        h->K->flexible = h->p.flexible != 0;
        h->K->fusedOuter = h->p.precision == 1 && h->p.fusedOuter != 0;
        h->K->trueResidualRestart = true;
        *amg = reinterpret_cast<long int>(h.release());
    });
}

int unap_cuda_amg_level_layout(long int amg, int level, int* nCells, long long* nFaces,
                               int* nWavefronts, int* perm, int* waveStart)
{
    return guarded([&] {
        AmgHandle* h = amg_from(amg);
        if (level < 0 || level >= h->H->nLevels()) throw std::invalid_argument("no such level");
        const Level& L = *h->H->lv[(size_t)level].L;
        if (nCells) *nCells = L.n;
        if (nFaces) *nFaces = L.nf;
        if (nWavefronts) *nWavefronts = L.nWave;
        if (perm) std::memcpy(perm, L.perm.data(), sizeof(int) * L.perm.size());
        if (waveStart) std::memcpy(waveStart, L.waveStart.data(), sizeof(int) * L.waveStart.size());
    });
}

int unap_cuda_amg_info(long int amg, int* nLevels, int* cells, int* wavefronts, int maxOut,
                       double* setupSeconds, long long* deviceBytes)
{
    return guarded([&] {
        AmgHandle* h = amg_from(amg);
        std::vector<int> c = h->H->levelCells(), w = h->H->levelWavefronts();
        if (nLevels) *nLevels = (int)c.size();
        for (int k = 0; k < (int)c.size() && k < maxOut; ++k) {
            if (cells) cells[k] = c[(size_t)k];
            if (wavefronts) wavefronts[k] = w[(size_t)k];
        }
        if (setupSeconds) *setupSeconds = h->H->setupSeconds;
        if (deviceBytes) *deviceBytes = (long long)h->H->deviceBytes();
    });
}

int unap_cuda_amg_vcycle(long int amg, const double* r, double* z)
{
    return guarded([&] {
        AmgHandle* h = amg_from(amg);
        Matrix& A = *h->A;
        order_after_default_stream(A.stream);
        Exec ex{A.stream, device_max_blocks()};
        const int n = A.n();
        DevArray<double> ri((size_t)n), zi((size_t)n);
        k_to_internal<double>(ex, n, A.L->d_perm.p, r, ri.p);
        h->H->vcycle(ex, ri.p, zi.p, Gate{});
        k_to_reference<double>(ex, n, A.L->d_perm.p, zi.p, z);
        UNAP_CK(cudaGetLastError());
        UNAP_CK(cudaStreamSynchronize(A.stream));
    });
}

int unap_cuda_amg_profile_vcycle(long int amg, int reps, double* ms, int maxOut, int* written)
{
    return guarded([&] {
        AmgHandle* h = amg_from(amg);
        if (reps < 1 || maxOut < 1) throw std::invalid_argument("reps and maxOut must be >= 1");
        int w = h->H->profile(h->A->stream, reps, ms, maxOut);
        if (written) *written = w;
    });
}

int unap_cuda_amg_profile_smoother(long int amg, int level, int reps, double* ms, double* bytes,
                                   int* launches)
{
    return guarded([&] {
        AmgHandle* h = amg_from(amg);
        if (reps < 1) throw std::invalid_argument("reps must be >= 1");
        double t = h->H->profileSmoother(h->A->stream, level, reps, bytes, launches);
        if (ms) *ms = t;
    });
}

int unap_cuda_amg_setup_phases(long int amg, double* seconds)
{
    return guarded([&] {
        AmgHandle* h = amg_from(amg);
        for (int i = 0; i < 6; ++i)
            if (seconds) seconds[i] = h->H->setupPhase[i];
    });
}

int unap_cuda_amg_eigenvalues(long int amg, double* lam, int maxOut, int* written)
{
    return guarded([&] {
        AmgHandle* h = amg_from(amg);
        std::vector<double> v = h->H->eigenvalues();
        int w = 0;
        for (; w < (int)v.size() && w < maxOut; ++w)
            if (lam) lam[w] = v[(size_t)w];
        if (written) *written = w;
    });
}

int unap_cuda_amg_solve(long int amg, double* x, const double* b, unap_cuda_stats* stats)
{
    return guarded([&] {
        AmgHandle* h = amg_from(amg);
        order_after_default_stream(h->A->stream);
        put(h->K->solveDevice(x, b), stats);
    });
}

int unap_cuda_amg_solve_host(long int amg, double* x, const double* b, unap_cuda_stats* stats)
{
    return guarded([&] {
        AmgHandle* h = amg_from(amg);
        Matrix& A = *h->A;
        const size_t n = (size_t)A.n();
        if (h->dx.n != n) h->dx.alloc(n);
        if (h->db.n != n) h->db.alloc(n);
        UNAP_CK(cudaMemcpyAsync(h->db.p, b, n * sizeof(double), cudaMemcpyHostToDevice, A.stream));
        UNAP_CK(cudaMemcpyAsync(h->dx.p, x, n * sizeof(double), cudaMemcpyHostToDevice, A.stream));
        SolveStats st = h->K->solveDevice(h->dx.p, h->db.p);
        UNAP_CK(cudaMemcpyAsync(x, h->dx.p, n * sizeof(double), cudaMemcpyDeviceToHost, A.stream));
        UNAP_CK(cudaStreamSynchronize(A.stream));
        put(st, stats);
    });
}

int unap_cuda_amg_destroy(long int amg)
{
    return guarded([&] { delete amg_from(amg); });
}

long long unap_cuda_launch_count(void) { return launch_count(); }

int unap_cuda_set_executor(int persistent) { return set_default_executor(persistent); }

int unap_cuda_set_host_wait(int mode)
{
    return guarded([&] {
        unsigned flags = mode == 1   ? cudaDeviceScheduleSpin
                         : mode == 2 ? cudaDeviceScheduleYield
                         : mode == 3 ? cudaDeviceScheduleBlockingSync
                                     : cudaDeviceScheduleAuto;
        if (mode < 0 || mode > 3) throw std::invalid_argument("host wait mode must be 0 to 3");
        UNAP_CK(cudaSetDeviceFlags(flags));
    });
}

int unap_cuda_set_wave_pdl(int on) { return set_wave_pdl(on); }

int unap_cuda_set_wave_grid(int oneRowPerThread) { return set_wave_grid(oneRowPerThread); }

int unap_cuda_set_packed_sweeps(int mode) { return set_packed_sweeps(mode); }

int unap_cuda_set_cheby_small_rows(int rows) { return set_cheby_small_rows(rows); }

int unap_cuda_set_cheby_tail_rows(int rows) { return set_cheby_tail_rows(rows); }

int unap_cuda_set_matrix_wavefronts(int on) { return set_matrix_wavefronts(on); }

int unap_cuda_set_cheby_chunk(int entries)
{
    try {
        return set_cheby_chunk(entries);
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return UNAP_CUDA_EINVAL;
    }
}

int unap_cuda_set_tail_rows(int precision, long long tailRows, long long singleRows,
                            long long* oldTailRows, long long* oldSingleRows)
{
    return guarded([&] { set_tail_rows(precision, tailRows, singleRows, oldTailRows, oldSingleRows); });
}

int unap_cuda_tail_cluster_size(int* clusterSize)
{
    return guarded([&] { *clusterSize = tail_cluster_size(); });
}

int unap_cuda_selftest_barrier_timeout(int* timedOut, int* recovered)
{
    return guarded([&] {
        cudaStream_t s;
        UNAP_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        // CTA 0 sleeps 20 ms inside a single-CTA segment while the other CTAs
        // wait at the following grid barrier with a ~64 us bound
        std::vector<Step> steps(1);
        steps[0].op = ST_SLEEP;
        steps[0].single = 1;
        steps[0].f0 = 20000;
        std::vector<LevelRows> lv(1);
        MegaRunner R;
        R.setProgram(steps, 1, lv, 1, s);
        DevArray<KState> st(1);
        st.zero(s);
        bool ok = R.run(st.p, 1, s, false, 2000);
        if (timedOut) *timedOut = ok ? 0 : 1;
        // the context stays usable: the same program with the default bound
        bool ok2 = R.run(st.p, 1, s, false, 0);
        UNAP_CK(cudaStreamSynchronize(s));
        UNAP_CK(cudaStreamDestroy(s));
        if (recovered) *recovered = ok2 ? 1 : 0;
    });
}

}  // extern "C"
