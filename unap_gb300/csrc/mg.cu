// The reference's MGSolver on the device (see mg.hpp).
#include <climits>
#include <cmath>
#include <cstring>

#include "device_common.cuh"
#include "mg.hpp"

namespace unapgpu {

namespace {

__global__ void prolong_set_kernel(int nf, const int* __restrict__ cmap,
                                   const double* __restrict__ coarse, double* __restrict__ fine)
{
    // prolongField (unapMatrix.hpp:410-438): injection
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += gridDim.x * blockDim.x)
        fine[i] = coarse[cmap[i]];
}

__global__ void scale_dev_kernel(int n, double* __restrict__ x, const double* a)
{
    const double s = *a;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] *= s;
}

__global__ void axpy_dev_kernel(int n, const double* a, const double* __restrict__ x,
                                double* __restrict__ y)
{
    const double s = *a;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] += s * x[i];
}

__global__ void add_kernel(int n, const double* __restrict__ x, double* __restrict__ y)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] += x[i];
}

__global__ void copy_kernel(int n, const double* __restrict__ x, double* __restrict__ y)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] = x[i];
}

// scalingFactor.cpp:35-64: sums s.f and Af.f, Jacobi step f += (s - Af)/D;
// sf = sum0 / (sum1 + SMALL)
__global__ void __launch_bounds__(kBlock) scaling_kernel(int n, const double* __restrict__ src,
                                                         const double* __restrict__ Acf,
                                                         double* field,
                                                         const double* __restrict__ D,
                                                         double* sfOut, RSpec red)
{
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double f = field[i];
        v[0] += src[i] * f;
        v[1] += Acf[i] * f;
        field[i] = f + (src[i] - Acf[i]) / D[i];
    }
    reduce_launch<2>(v, red, [&](const double (&t)[2]) { *sfOut = t[0] / (t[1] + SMALL_D); });
}

// ---- chebySmoother::smooth (chebySmoother.cpp:44-148) ---------------------
__device__ __forceinline__ void cheby_coeffs(double maxEigPCG, int k, double& dtemp1,
                                             double& dtemp2, double& Rtheta)
{
    const double maxEig = maxEigPCG * 1.1;
    const double minEig = maxEigPCG / 1.5;
    const double delta = 2.0 / (maxEig - minEig);
    const double theta = 0.5 * (maxEig + minEig);
    const double s1 = theta * delta;
    double rhok = 1.0 / s1;
    Rtheta = 1.0 / theta;
    dtemp1 = dtemp2 = 0.0;
    for (int j = 1; j <= k; ++j) {
        double rhokp1 = 1.0 / (2.0 * s1 - rhok);
        dtemp1 = rhokp1 * rhok;
        dtemp2 = 2.0 * rhokp1 * delta;
        rhok = rhokp1;
    }
}

__global__ void cheby0_kernel(int n, const double* __restrict__ rD, const double* __restrict__ b,
                              double* __restrict__ w, double* __restrict__ x, const EigState* es)
{
    double d1, d2, Rtheta;
    cheby_coeffs(es->maxEig, 0, d1, d2, Rtheta);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double wi = rD[i] * (b[i] - w[i]) * Rtheta;
        w[i] = wi;
        x[i] += wi;
    }
}

__global__ void chebyk_kernel(int n, const double* __restrict__ rD, const double* __restrict__ b,
                              const double* __restrict__ p, double* __restrict__ w,
                              double* __restrict__ x, const EigState* es, int k)
{
    double d1, d2, Rtheta;
    cheby_coeffs(es->maxEig, k, d1, d2, Rtheta);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double wi = d1 * w[i] + d2 * rD[i] * (b[i] - p[i]);
        w[i] = wi;
        x[i] += wi;
    }
}

void tick() { if (!capturing()) count_launches(1); }

}  // namespace

enum { M_RES = 0, M_SCALE, M_EIGWR, M_EIGA, M_NSITES };

MgSolver::MgSolver(Matrix& A_, const std::vector<double>& weights, const MgParams& p)
    : params(p), A(A_)
{
    if (!A.L->sweepable)
        throw std::invalid_argument("MGSolver needs faces oriented lowerAddr < upperAddr and sorted by owner");
    if ((int)weights.size() != A.host.nf) throw std::invalid_argument("one weight per face expected");
    cudaStream_t s = A.stream;
    ex.s = s;
    ex.maxBlocks = device_max_blocks();
    scale = params.scaleCorr < 0 ? A.host.symm : (params.scaleCorr != 0);
    std::vector<CoarseHost> coarse =
        agglomerate_levels(A.host, weights, params.nCoarsest, params.maxLevels, 0, s);
    const int nC = (int)coarse.size();
    lv.resize((size_t)nC + 1);
    lv[0].L = A.L.get();
    lv[0].n = A.n();
    for (int k = 1; k <= nC; ++k) {
        CoarseHost& c = coarse[(size_t)k - 1];
        const Level& F = *lv[(size_t)k - 1].L;
        std::vector<int> key((size_t)c.A.n, INT_MAX);
        for (int i = 0; i < F.n; ++i) {
            int C = c.restrictAddr[(size_t)i];
            key[(size_t)C] = std::min(key[(size_t)C], F.iperm[(size_t)i]);
        }
        lv[(size_t)k].own = build_level(c.A, &key, false, s);
        lv[(size_t)k].L = lv[(size_t)k].own.get();
        lv[(size_t)k].n = c.A.n;
        const Level& Cl = *lv[(size_t)k].L;
        const int nc = c.A.n;
        std::vector<int> refStart((size_t)nc + 1, 0);
        for (int i = 0; i < F.n; ++i) refStart[(size_t)c.restrictAddr[(size_t)i] + 1]++;
        for (int C = 0; C < nc; ++C) refStart[(size_t)C + 1] += refStart[(size_t)C];
        std::vector<int> refChild((size_t)F.n);
        {
            std::vector<int> pos(refStart.begin(), refStart.end() - 1);
            for (int i = 0; i < F.n; ++i) refChild[(size_t)pos[(size_t)c.restrictAddr[(size_t)i]]++] = i;
        }
        std::vector<int> cs((size_t)nc + 1, 0), ch((size_t)F.n), cmap((size_t)F.n);
        for (int Ci = 0; Ci < nc; ++Ci) {
            int C = Cl.perm[(size_t)Ci];
            int len = refStart[(size_t)C + 1] - refStart[(size_t)C];
            cs[(size_t)Ci + 1] = cs[(size_t)Ci] + len;
            for (int j = 0; j < len; ++j)
                ch[(size_t)(cs[(size_t)Ci] + j)] = F.iperm[(size_t)refChild[(size_t)(refStart[(size_t)C] + j)]];
        }
        for (int i = 0; i < F.n; ++i) cmap[(size_t)i] = Cl.iperm[(size_t)c.restrictAddr[(size_t)F.perm[(size_t)i]]];
        Lv& K = lv[(size_t)k];
        K.childStart.upload(cs, s);
        K.child.upload(ch, s);
        K.cmap.upload(cmap, s);
        K.corr.alloc((size_t)nc);
        K.src.alloc((size_t)nc);
        UNAP_CK(cudaStreamSynchronize(s));
    }
    // per-level scratch, Chebyshev 1/D (lduDiagPrecond.cpp:13-41)
    for (int k = 0; k <= nC; ++k) {
        Lv& K = lv[(size_t)k];
        K.acf.alloc((size_t)K.n);
        K.pre.alloc((size_t)K.n);
        if (params.smoother == 2) {
            const HostLdu& H = k == 0 ? A.host : coarse[(size_t)k - 1].A;
            std::vector<double> rd((size_t)K.n);
            for (int i = 0; i < K.n; ++i) rd[(size_t)i] = 1.0 / H.diag[(size_t)K.L->perm[(size_t)i]];
            K.rD.upload(rd, s);
            K.w.alloc((size_t)K.n);
            K.p.alloc((size_t)K.n);
        }
    }
    // coarsest: PCG+DIC (symmetric) or PBiCGStab+DILU, relTol 1e-2, maxIter 100
    if (nC > 0) {
        Lv& C = lv[(size_t)nC];
        const bool symm = C.L->symm;
        C.dfac.alloc((size_t)C.n);
        C.pfac.alloc((size_t)C.n);
        dic_factor(ex, *C.L, !symm, C.dfac.p, C.pfac.p);
        coarseWork.alloc((size_t)8 * C.n);
        static_assert(sizeof(SmallSystem) % 8 == 0, "SmallSystem layout");
        SmallSystem S{};
        S.A = rows64(*C.L);
        S.nWave = C.L->nWave;
        S.rD = C.pfac.p;
        S.method = symm ? 0 : 1;
        S.precond = symm ? 2 : 3;
        S.tol = 0.0;
        S.relTol = 1.0e-2;
        S.maxIter = 100;
        S.minIter = 0;
        S.zeroX = 1;
        S.x = C.corr.p;
        S.b = C.src.p;
        S.work = coarseWork.p;
        S.result = nullptr;
        waveDev.upload(C.L->waveStart, s);
        S.waveStart = waveDev.p;
        coarseSys.upload(&S, 1, s);
    }
    x.alloc((size_t)A.n());
    b.alloc((size_t)A.n());
    Apsi.alloc((size_t)A.n());
    fc.alloc((size_t)A.n());
    fr.alloc((size_t)A.n());
    sfs.alloc((size_t)2 * (nC + 2));
    eig.alloc((size_t)nC + 1);
    chebyFirst.assign((size_t)nC + 1, 1);
    UNAP_CK(gated_malloc((void**)&d_st, sizeof(KState)));
    h_st = static_cast<KState*>(pinned_block_alloc(sizeof(KState)));
    pool.init(M_NSITES, ex.maxBlocks, 2, s);
    UNAP_CK(cudaEventCreate(&ev0));
    UNAP_CK(cudaEventCreate(&ev1));
    UNAP_CK(cudaStreamSynchronize(s));
}

MgSolver::~MgSolver()
{
    if (d_st) gated_free(d_st);
    pinned_block_free(h_st);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
}

std::vector<int> MgSolver::levelCells() const
{
    std::vector<int> v;
    for (auto& l : lv) v.push_back(l.n);
    return v;
}

void MgSolver::initSmoothers() { std::fill(chebyFirst.begin(), chebyFirst.end(), 1); }

void MgSolver::eigen_estimate(int slot, int k, double* xk, const double* bk)
{
    // eigenDiagPCG ctor: 10 diagonal-PCG iterations on (x, b), x updated
    Lv& K = lv[(size_t)k];
    const int n = K.n;
    EigState h{};
    h.wArA = 1.0e37;  // GREAT, eigenDiagPCG.cpp:75
    EigState* es = eig.p + slot;
    UNAP_CK(cudaMemcpyAsync(es, &h, sizeof(EigState), cudaMemcpyHostToDevice, ex.s));
    Rows<double> R = rows64(*K.L);
    (void)n;
    eig_diag_pcg(ex, R, K.rD.p, xk, bk, K.acf.p, K.w.p, K.p.p, es,
                 pool.site(M_EIGWR, nullptr, FIN_RES_ONLY), pool.site(M_EIGA, nullptr, FIN_RES_ONLY),
                 10);
    k_eig_sturm(ex, es, 10);
}

void MgSolver::chebyshev(int slot, int k, double* xk, const double* bk, int nSweeps)
{
    Lv& K = lv[(size_t)k];
    const int n = K.n;
    const EigState* es = eig.p + slot;
    Rows<double> R = rows64(*K.L);
    k_spmv<double>(ex, R, xk, K.w.p, nullptr, RSpec{}, Gate{});
    tick();
    cheby0_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, K.rD.p, bk, K.w.p, xk, es);
    for (int sw = 1; sw < nSweeps; ++sw) {
        k_spmv<double>(ex, R, xk, K.p.p, nullptr, RSpec{}, Gate{});
        tick();
        chebyk_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, K.rD.p, bk, K.p.p, K.w.p, xk, es, sw);
    }
}

void MgSolver::smooth(int slot, int k, double* xk, const double* bk, int nSweeps)
{
    if (params.smoother == 2) {
        if (chebyFirst[(size_t)slot]) {
            // chebySmoother.cpp:22-42: the first call only estimates
            eigen_estimate(slot, k, xk, bk);
            chebyFirst[(size_t)slot] = 0;
        } else {
            chebyshev(slot, k, xk, bk, nSweeps);
        }
        return;
    }
    const Level& L = *lv[(size_t)k].L;
    Rows<double> R = rows64(L);
    for (int s = 0; s < nSweeps; ++s) gs_sweep<double>(ex, L, R, xk, bk, false, false, Gate{});
}

void MgSolver::scaling(int k, double* field, const double* source, double* Acf, int sfSlot)
{
    Lv& K = lv[(size_t)k];
    Rows<double> R = rows64(*K.L);
    k_spmv<double>(ex, R, field, Acf, nullptr, RSpec{}, Gate{});
    tick();
    scaling_kernel<<<ex.grid(K.n), kBlock, 0, ex.s>>>(K.n, source, Acf, field, R.diag,
                                                      sfs.p + sfSlot,
                                                      pool.site(M_SCALE, nullptr, FIN_RES_ONLY));
}

// MGSolver::Vcycle, Vcycle.cpp:27-332 (coarse level c of the reference is lv[c+1])
void MgSolver::vcycle()
{
    const int L = nCoarseLevels() - 1;
    int sf = 0;
    if (L >= 0) k_restrict<double>(ex, lv[1].n, lv[1].childStart.p, lv[1].child.p, fr.p, lv[1].src.p, Gate{});
    for (int c = 0; c < L; ++c) {
        Lv& C = lv[(size_t)c + 1];
        Rows<double> R = rows64(*C.L);
        if (params.nPre) {
            k_fill<double>(ex, C.n, C.corr.p, 0.0);
            smooth(c + 1, c + 1, C.corr.p, C.src.p, params.nPre + c);
            if (scale && c < L - 1) {
                scaling(c + 1, C.corr.p, C.src.p, C.acf.p, sf);
                tick();
                scale_dev_kernel<<<ex.grid(C.n), kBlock, 0, ex.s>>>(C.n, C.corr.p, sfs.p + sf);
                ++sf;
            }
            k_spmv<double>(ex, R, C.corr.p, C.acf.p, nullptr, RSpec{}, Gate{});
            k_axpby<double>(ex, C.n, -1.0, C.acf.p, 1.0, C.src.p, Gate{});
        }
        Lv& N = lv[(size_t)c + 2];
        k_restrict<double>(ex, N.n, N.childStart.p, N.child.p, C.src.p, N.src.p, Gate{});
    }
    if (L >= 0) launch_small_krylov(ex.s, coarseSys.p, 1, nullptr);
    for (int c = L - 1; c >= 0; --c) {
        Lv& C = lv[(size_t)c + 1];
        Lv& N = lv[(size_t)c + 2];
        if (params.nPre) {
            tick();
            copy_kernel<<<ex.grid(C.n), kBlock, 0, ex.s>>>(C.n, C.corr.p, C.pre.p);
        }
        tick();
        prolong_set_kernel<<<ex.grid(C.n), kBlock, 0, ex.s>>>(C.n, N.cmap.p, N.corr.p, C.corr.p);
        if (scale && c < L - 1) {
            scaling(c + 1, C.corr.p, C.src.p, C.acf.p, sf);
            tick();
            scale_dev_kernel<<<ex.grid(C.n), kBlock, 0, ex.s>>>(C.n, C.corr.p, sfs.p + sf);
            ++sf;
        }
        if (params.nPre) {
            tick();
            add_kernel<<<ex.grid(C.n), kBlock, 0, ex.s>>>(C.n, C.pre.p, C.corr.p);
        }
        smooth(c + 1, c + 1, C.corr.p, C.src.p, params.nPost + c);
    }
    const int n = A.n();
    if (L >= 0) {
        tick();
        prolong_set_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, lv[1].cmap.p, lv[1].corr.p, fc.p);
    }
    if (scale) {
        scaling(0, fc.p, fr.p, Apsi.p, sf);
        tick();
        axpy_dev_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, sfs.p + sf, fc.p, x.p);
        ++sf;
    } else {
        tick();
        add_kernel<<<ex.grid(n), kBlock, 0, ex.s>>>(n, fc.p, x.p);
    }
    smooth(0, 0, x.p, b.p, params.nFinest);
}

SolveStats MgSolver::solveDevice(double* x_ref, const double* b_ref)
{
    SolveStats out;
    const Level& L0 = *A.L;
    const int n = A.n();
    UNAP_CK(cudaEventRecord(ev0, ex.s));
    k_to_internal<double>(ex, n, L0.d_perm.p, x_ref, x.p);
    k_to_internal<double>(ex, n, L0.d_perm.p, b_ref, b.p);
    k_fill<double>(ex, n, fc.p, 0.0);
    KState h;
    std::memset(&h, 0, sizeof(h));
    h.tol = params.tol;
    h.relTol = params.relTol;
    h.maxIter = params.maxIter;
    h.minIter = params.minIter;
    *h_st = h;
    UNAP_CK(cudaMemcpyAsync(d_st, h_st, sizeof(KState), cudaMemcpyHostToDevice, ex.s));
    Rows<double> R0 = rows64(L0);
    // MGSolve.cpp:31-58: finestResidual = b - A x, initialResidual
    k_residual<double>(ex, R0, x.p, b.p, fr.p, pool.site(M_RES, d_st, FIN_INIT_RES), Gate{});
    UNAP_CK(cudaMemcpyAsync(h_st, d_st, sizeof(KState), cudaMemcpyDeviceToHost, ex.s));
    UNAP_CK(cudaStreamSynchronize(ex.s));
    const double init = h_st->initRes;
    bool conv0 = ((init < params.tol || (params.relTol > 1e-37 && init <= params.relTol * init)) &&
                  0 >= params.minIter);
    if (!conv0 && n > 0) {
        for (;;) {
            vcycle();
            k_residual<double>(ex, R0, x.p, b.p, fr.p, pool.site(M_RES, d_st, FIN_MG_RES), Gate{});
            UNAP_CK(cudaGetLastError());
            UNAP_CK(cudaMemcpyAsync(h_st, d_st, sizeof(KState), cudaMemcpyDeviceToHost, ex.s));
            UNAP_CK(cudaStreamSynchronize(ex.s));
            if (h_st->done) break;
        }
    } else {
        h_st->converged = 1;
    }
    k_to_reference<double>(ex, n, L0.d_perm.p, x.p, x_ref);
    UNAP_CK(cudaEventRecord(ev1, ex.s));
    UNAP_CK(cudaStreamSynchronize(ex.s));
    float ms = 0;
    UNAP_CK(cudaEventElapsedTime(&ms, ev0, ev1));
    out.seconds = ms * 1e-3;
    out.nIter = h_st->nIter;
    out.initRes = init;
    out.finalRes = conv0 ? init : h_st->finalRes;
    out.converged = h_st->converged;
    out.singular = 0;
    return out;
}

SolveStats MgSolver::solveHost(double* xh, const double* bh)
{
    const size_t n = (size_t)A.n();
    DevArray<double> dx(n), db(n);
    dx.upload(xh, n, ex.s);
    db.upload(bh, n, ex.s);
    SolveStats st = solveDevice(dx.p, db.p);
    if (n) UNAP_CK(cudaMemcpyAsync(xh, dx.p, n * sizeof(double), cudaMemcpyDeviceToHost, ex.s));
    UNAP_CK(cudaStreamSynchronize(ex.s));
    return st;
}

}  // namespace unapgpu
