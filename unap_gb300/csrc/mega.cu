// Persistent cooperative step-program executor (see mega.hpp).
#include <cstring>

#include "device_common.cuh"
#include "mega.hpp"

namespace unapgpu {

namespace {

constexpr int kMegaThreads = 1024;
constexpr int kMaxDense = 4096;             // doubles of shared memory for ST_DENSE
constexpr unsigned kSpinLimit = 1u << 22;   // bounded barrier wait

// Sense-reversing grid barrier over a cooperative launch.  A wait that
// exceeds kSpinLimit sets status->timeout; every later barrier then returns
// false at once so the kernel unwinds instead of hanging.
__device__ bool grid_barrier(MegaStatus* gs, unsigned spinLimit)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned* vgen = &gs->gen;
        volatile int* vto = &gs->timeout;
        if (*vto) {
            ok = 0;
        } else {
            const unsigned g = *vgen;
            __threadfence();
            const unsigned arrived = atomicAdd(&gs->count, 1u);
            if (arrived == gridDim.x - 1) {
                atomicExch(&gs->count, 0u);
                __threadfence();
                atomicAdd(&gs->gen, 1u);
            } else {
                unsigned spins = 0;
                while (*vgen == g) {
                    if (*vto) {
                        ok = 0;
                        break;
                    }
                    if (++spins > spinLimit) {
                        atomicExch(&gs->timeout, 1);
                        ok = 0;
                        break;
                    }
                    __nanosleep(32);
                }
            }
            __threadfence();
        }
    }
    __syncthreads();
    return ok != 0;
}

template <class T>
__device__ __forceinline__ const Rows<T>& rows_of(const LevelRows& L);
template <>
__device__ __forceinline__ const Rows<double>& rows_of<double>(const LevelRows& L)
{
    return L.r64;
}
template <>
__device__ __forceinline__ const Rows<float>& rows_of<float>(const LevelRows& L)
{
    return L.r32;
}

// write this block's partial of a reduction step (overwrite or accumulate);
// a single-CTA step also zeroes the other blocks' entries, so finalize can
// always sum every block's entry
template <int K>
__device__ __forceinline__ void put_partial(double (&v)[K], const MegaArgs& g, int slot,
                                            bool accumulate, bool single)
{
    block_sum<K>(v);
    if (single && !accumulate) {
        for (int b = 1 + threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
            for (int k = 0; k < K; ++k) g.partials[(size_t)(slot + k) * gridDim.x + b] = 0.0;
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double* p = g.partials + (size_t)(slot + k) * gridDim.x + blockIdx.x;
            *p = accumulate ? *p + v[k] : v[k];
        }
    }
}

template <class T>
__device__ void exec_gs(const Step& s, const LevelRows& L, int first, int stride)
{
    const Rows<T>& A = rows_of<T>(L);
    T* x = (T*)s.c;
    const T* b = (const T*)s.b;
    for (int r = s.r0 + first; r < s.r1; r += stride) {
        const int info = ldg(A.rowInfo + r);
        const int len = info & 0xffff;
        const int nLow = info >> 16;
        const int base = ldg(A.sliceOff + (r >> 5)) + (r & 31);
        T acc = b[r];
        acc = row_subtract<T>(A, A.val, base, 0, nLow, x, acc);
        if (!s.f0) acc = row_subtract<T>(A, A.val, base, nLow, len, x, acc);
        x[r] = acc / ldg(A.diag + r);
    }
}

template <class T>
__device__ void exec_resid(const Step& s, const LevelRows& L, int first, int stride)
{
    const Rows<T>& A = rows_of<T>(L);
    const T* x = (const T*)s.a;
    const T* b = (const T*)s.b;
    T* r = (T*)s.c;
    for (int i = first; i < A.n; i += stride) r[i] = b[i] - row_apply<T, XL_CG>(A, i, x);
}

template <class T>
__device__ void exec_restrict(const Step& s, int first, int stride)
{
    const T* fine = (const T*)s.a;
    T* coarse = (T*)s.c;
    for (int c = first; c < s.r1; c += stride) {
        T acc = T(0);
        for (int k = s.i0[c]; k < s.i0[c + 1]; ++k) acc += fine[s.i1[k]];
        coarse[c] = acc;
    }
}

template <class T>
__device__ void exec_prolong(const Step& s, int first, int stride)
{
    const T* coarse = (const T*)s.a;
    T* fine = (T*)s.c;
    for (int i = first; i < s.r1; i += stride) fine[i] += coarse[s.i0[i]];
}

template <class T>
__device__ void exec_dense(const Step& s, int first, int stride, bool single)
{
    extern __shared__ double sb[];
    const int n = s.r1;
    const T* b = (const T*)s.a;
    T* x = (T*)s.c;
    const double* M = (const double*)s.e;
    for (int j = threadIdx.x; j < n; j += blockDim.x) sb[j] = (double)b[s.i0 ? s.i0[j] : j];
    __syncthreads();
    for (int i = first; i < n; i += stride) x[i] = (T)dense_row_chunked(M, n, i, sb);
    (void)single;
}

__device__ void exec_dic_fwd(const Step& s, const LevelRows& L, int first, int stride)
{
    const Rows<double>& A = L.r64;
    const double* rr = (const double*)s.a;
    double* w = (double*)s.c;
    const double* rD = (const double*)s.e;
    const double* coef = (const double*)s.d;
    for (int r = s.r0 + first; r < s.r1; r += stride) {
        const int nLow = ldg(A.rowInfo + r) >> 16;
        const int base = ldg(A.sliceOff + (r >> 5)) + (r & 31);
        const double rd = ldg(rD + r);
        double acc = rd * rr[r];
        for (int j = 0; j < nLow; ++j) {
            const int e = base + 32 * j;
            acc -= rd * ldg(coef + e) * w[ldg(A.col + e)];
        }
        w[r] = acc;
    }
}

__device__ void exec_dic_bwd(const Step& s, const LevelRows& L, const MegaArgs& g, int first,
                             int stride, bool single)
{
    const Rows<double>& A = L.r64;
    const double* rr = (const double*)s.a;
    double* w = (double*)s.c;
    const double* rD = (const double*)s.e;
    double v[1] = {0.0};
    for (int r = s.r0 + first; r < s.r1; r += stride) {
        const int info = ldg(A.rowInfo + r);
        const int len = info & 0xffff;
        const int nLow = info >> 16;
        const int base = ldg(A.sliceOff + (r >> 5)) + (r & 31);
        const double rd = ldg(rD + r);
        double acc = w[r];
        for (int j = len - 1; j >= nLow; --j) {
            const int e = base + 32 * j;
            acc -= rd * ldg(A.val + e) * w[ldg(A.col + e)];
        }
        w[r] = acc;
        v[0] += acc * rr[r];
    }
    put_partial<1>(v, g, s.red, s.f0 != 0, single);
}

template <class T>
__device__ void exec_cheb(const Step& s, const LevelRows& L, int first, int stride)
{
    const Rows<T>& A = rows_of<T>(L);
    const T* xin = (const T*)s.a;
    const T* b = (const T*)s.b;
    T* xout = (T*)s.c;
    T* w = (T*)s.d;
    const T c1 = (T)s.k1, c2 = (T)s.k2;
    for (int r = first; r < A.n; r += stride) {
        const T acc = row_apply<T, XL_CG>(A, r, xin);
        const T rD = T(1) / ldg(A.diag + r);
        const T bb = __ldcg(b + r);
        T wi;
        if (s.f0)
            wi = rD * (bb - acc) * c1;
        else
            wi = c1 * __ldcg(w + r) + c2 * rD * (bb - acc);
        w[r] = wi;
        xout[r] = __ldcg(xin + r) + wi;
    }
}

template <class T>
__device__ void exec_cheb0(const Step& s, const LevelRows& L, int first, int stride)
{
    const Rows<T>& A = rows_of<T>(L);
    T* b = (T*)s.b;
    const double* r64 = (const double*)s.e;
    T* x = (T*)s.c;
    T* w = (T*)s.d;
    const T Rth = (T)s.k1;
    for (int i = first; i < A.n; i += stride) {
        T bi;
        if (r64) {
            bi = (T)__ldcg(r64 + i);
            b[i] = bi;
        } else {
            bi = __ldcg(b + i);
        }
        const T rD = T(1) / ldg(A.diag + i);
        const T wi = rD * bi * Rth;
        w[i] = wi;
        x[i] = wi;
    }
}

template <class T>
__device__ void exec_restrict_cheb0(const Step& s, const LevelRows& L, int first, int stride)
{
    const Rows<T>& A = rows_of<T>(L);
    const T* fine = (const T*)s.a;
    T* coarse = (T*)s.c;
    T* x = (T*)s.d;
    T* w = (T*)s.e;
    const T Rth = (T)s.k1;
    for (int c = first; c < s.r1; c += stride) {
        T acc = T(0);
        for (int k = s.i0[c]; k < s.i0[c + 1]; ++k) acc += __ldcg(fine + s.i1[k]);
        coarse[c] = acc;
        const T rD = T(1) / ldg(A.diag + c);
        const T wi = rD * acc * Rth;
        w[c] = wi;
        x[c] = wi;
    }
}

template <class T>
__device__ void exec_prolong_to(const Step& s, int first, int stride)
{
    const T* coarse = (const T*)s.a;
    const T* xin = (const T*)s.b;
    T* xout = (T*)s.c;
    for (int i = first; i < s.r1; i += stride) xout[i] = __ldcg(xin + i) + __ldcg(coarse + s.i0[i]);
}

__device__ void exec_step(const Step& s, const MegaArgs& g, bool single)
{
    const int first = single ? threadIdx.x : blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = single ? blockDim.x : gridDim.x * blockDim.x;
    const LevelRows& L = g.levels[s.lvl];
    switch (s.op) {
    case ST_GS:
        if (s.prec)
            exec_gs<float>(s, L, first, stride);
        else
            exec_gs<double>(s, L, first, stride);
        break;
    case ST_RESID:
        if (s.prec)
            exec_resid<float>(s, L, first, stride);
        else
            exec_resid<double>(s, L, first, stride);
        break;
    case ST_RESTRICT:
        if (s.prec)
            exec_restrict<float>(s, first, stride);
        else
            exec_restrict<double>(s, first, stride);
        break;
    case ST_PROLONG_ADD:
        if (s.prec)
            exec_prolong<float>(s, first, stride);
        else
            exec_prolong<double>(s, first, stride);
        break;
    case ST_DENSE:
        if (s.prec)
            exec_dense<float>(s, first, stride, single);
        else
            exec_dense<double>(s, first, stride, single);
        break;
    case ST_FILL0:
        if (s.prec) {
            for (int i = first; i < s.r1; i += stride) ((float*)s.c)[i] = 0.0f;
        } else {
            for (int i = first; i < s.r1; i += stride) ((double*)s.c)[i] = 0.0;
        }
        break;
    case ST_D2F:
        for (int i = first; i < s.r1; i += stride) ((float*)s.c)[i] = (float)((const double*)s.a)[i];
        break;
    case ST_F2D:
        for (int i = first; i < s.r1; i += stride) ((double*)s.c)[i] = (double)((const float*)s.a)[i];
        break;
    case ST_COPY:
        for (int i = first; i < s.r1; i += stride) ((double*)s.c)[i] = ((const double*)s.a)[i];
        break;
    case ST_SLEEP:
        if (blockIdx.x == 0 && threadIdx.x == 0)
            for (int us = 0; us < s.f0 && us < 1000000; ++us) __nanosleep(1000);
        break;
    case ST_CHEB:
        if (s.prec)
            exec_cheb<float>(s, L, first, stride);
        else
            exec_cheb<double>(s, L, first, stride);
        break;
    case ST_CHEB0:
        if (s.prec)
            exec_cheb0<float>(s, L, first, stride);
        else
            exec_cheb0<double>(s, L, first, stride);
        break;
    case ST_RESTRICT_CHEB0:
        if (s.prec)
            exec_restrict_cheb0<float>(s, L, first, stride);
        else
            exec_restrict_cheb0<double>(s, L, first, stride);
        break;
    case ST_PROLONG_TO:
        if (s.prec)
            exec_prolong_to<float>(s, first, stride);
        else
            exec_prolong_to<double>(s, first, stride);
        break;
    case ST_DIC_FWD: exec_dic_fwd(s, L, first, stride); break;
    case ST_DIC_BWD: exec_dic_bwd(s, L, g, first, stride, single); break;
    case ST_DIAG: {
        const double* r = (const double*)s.a;
        double* w = (double*)s.c;
        const double* rD = (const double*)s.e;
        double v[1] = {0.0};
        for (int i = first; i < s.r1; i += stride) {
            double wi = rD ? rD[i] * r[i] : r[i];
            w[i] = wi;
            v[0] += wi * r[i];
        }
        put_partial<1>(v, g, s.red, false, single);
        break;
    }
    case ST_SPMV_DOT: {
        const Rows<double>& A = L.r64;
        const double* p = (const double*)s.a;
        double* q = (double*)s.c;
        double v[1] = {0.0};
        for (int i = first; i < A.n; i += stride) {
            double qi = row_apply<double, XL_CG>(A, i, p);
            q[i] = qi;
            v[0] += qi * p[i];
        }
        put_partial<1>(v, g, s.red, false, single);
        break;
    }
    case ST_RESID_NORM: {
        const Rows<double>& A = L.r64;
        const double* x = (const double*)s.a;
        const double* b = (const double*)s.b;
        double* r = (double*)s.c;
        double v[1] = {0.0};
        for (int i = first; i < A.n; i += stride) {
            double ri = b[i] - row_apply<double, XL_CG>(A, i, x);
            r[i] = ri;
            v[0] += ri * ri;
        }
        put_partial<1>(v, g, s.red, false, single);
        break;
    }
    case ST_DOT2: {
        const double* a = (const double*)s.a;
        const double* b = (const double*)s.b;
        const double* c = (const double*)s.c;
        const double* d = (const double*)s.d;
        double v[2] = {0.0, 0.0};
        for (int i = first; i < s.r1; i += stride) {
            v[0] += a[i] * b[i];
            if (c) v[1] += c[i] * d[i];
        }
        put_partial<2>(v, g, s.red, false, single);
        break;
    }
    default: break;
    }
}

__global__ void __launch_bounds__(kMegaThreads, 1) mega_kernel(MegaArgs g)
{
    __shared__ KState S;
    if (threadIdx.x == 0) S = *g.st;
    __syncthreads();
    int loops = 0;
    int p = g.skipInit ? g.nInit : 0;
    int end = g.skipInit ? g.nSteps : g.nInit;
    bool init = !g.skipInit;
    bool ok = true;
    for (;;) {
        int q = p;
        while (q < end) {
            const Step& s = g.steps[q];
            if (s.op == ST_SCALAR) {
                // every block finalizes the same partials in the same order
                if (threadIdx.x == 0) {
                    double t[2] = {0.0, 0.0};
                    const int parts = s.r1 < 0 ? (int)gridDim.x : s.r1;
                    for (int k = 0; k < 2; ++k)
                        for (int b = 0; b < parts; ++b)
                            t[k] += __ldcg(g.partials + (size_t)(s.red + k) * gridDim.x + b);
                    apply_fin(&S, s.f0, t, 2);
                }
                __syncthreads();
                ++q;
                if (S.done) break;  // singular: the reference breaks mid-iteration
                continue;
            }
            if (s.op == ST_PCG_DIR || s.op == ST_PCG_UPD) {
                const int first = blockIdx.x * blockDim.x + threadIdx.x;
                const int stride = gridDim.x * blockDim.x;
                if (s.op == ST_PCG_DIR) {
                    const double* z = (const double*)s.a;
                    double* pp = (double*)s.c;
                    const bool useBeta = S.useBeta;
                    const double beta = S.beta;
                    for (int i = first; i < s.r1; i += stride)
                        pp[i] = useBeta ? z[i] + beta * pp[i] : z[i];
                } else {
                    double* x = (double*)s.c;
                    double* r = (double*)s.d;
                    const double* pp = (const double*)s.a;
                    const double* qq = (const double*)s.b;
                    const double alpha = S.alpha;
                    double v[1] = {0.0};
                    for (int i = first; i < s.r1; i += stride) {
                        x[i] += alpha * pp[i];
                        double ri = r[i] - alpha * qq[i];
                        r[i] = ri;
                        v[0] += ri * ri;
                    }
                    put_partial<1>(v, g, s.red, false, false);
                }
                ++q;
            } else if (s.single) {
                int q2 = q;
                while (q2 < end && g.steps[q2].single && g.steps[q2].op != ST_SCALAR) ++q2;
                if (blockIdx.x == 0) {
                    for (int k = q; k < q2; ++k) {
                        exec_step(g.steps[k], g, true);
                        __syncthreads();
                    }
                }
                q = q2;
            } else {
                exec_step(s, g, false);
                ++q;
            }
            if (!grid_barrier(g.status, g.spinLimit)) {
                ok = false;
                break;
            }
        }
        if (!ok || S.done) break;
        if (init)
            init = false;
        else if (++loops >= g.maxLoops)
            break;
        p = g.nInit;
        end = g.nSteps;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *g.st = S;
}

}  // namespace

bool mega_single_level(int nRows) { return nRows <= 48 * 1024; }

MegaRunner::MegaRunner()
{
    h_status = static_cast<MegaStatus*>(pinned_block_alloc(sizeof(MegaStatus)));
    d_status.alloc(1);
}

MegaRunner::~MegaRunner()
{
    pinned_block_free(h_status);
}

int MegaRunner::threads() const { return kMegaThreads; }

void MegaRunner::setProgram(const std::vector<Step>& steps, int nInit_,
                            const std::vector<LevelRows>& lv, int nSlots_, cudaStream_t s)
{
    for (const Step& st : steps)
        if (st.op == ST_DENSE && st.r1 > kMaxDense)
            throw std::invalid_argument("dense coarsest level too large for the step executor");
    d_steps.upload(steps.data(), steps.size(), s);
    d_levels.upload(lv.data(), lv.size(), s);
    nSteps = (int)steps.size();
    nInit = nInit_;
    nSlots = nSlots_;
    int dev = 0, sms = 0, perSm = 0;
    UNAP_CK(cudaGetDevice(&dev));
    UNAP_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    UNAP_CK(cudaFuncSetAttribute(mega_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kMaxDense * (int)sizeof(double)));
    UNAP_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, mega_kernel, kMegaThreads,
                                                          kMaxDense * sizeof(double)));
    if (perSm < 1) throw std::runtime_error("step executor does not fit on an SM");
    blocks = sms * 1;  // one CTA per SM: the grid barrier cost grows with CTAs
    d_partials.alloc((size_t)std::max(1, nSlots) * blocks);
    d_partials.zero(s);
    UNAP_CK(cudaStreamSynchronize(s));
}

bool MegaRunner::run(KState* d_st, int maxLoops, cudaStream_t s, bool skipInit,
                     unsigned spinLimit)
{
    std::memset(h_status, 0, sizeof(MegaStatus));
    UNAP_CK(cudaMemcpyAsync(d_status.p, h_status, sizeof(MegaStatus), cudaMemcpyHostToDevice, s));
    MegaArgs a;
    a.steps = d_steps.p;
    a.nSteps = nSteps;
    a.nInit = nInit;
    a.levels = d_levels.p;
    a.st = d_st;
    a.status = d_status.p;
    a.partials = d_partials.p;
    a.nSlots = nSlots;
    a.maxLoops = maxLoops;
    a.skipInit = skipInit ? 1 : 0;
    a.spinLimit = spinLimit ? spinLimit : kSpinLimit;
    void* params[] = {&a};
    if (!capturing()) count_launches(1);
    UNAP_CK(cudaLaunchCooperativeKernel((const void*)mega_kernel, dim3(blocks),
                                        dim3(kMegaThreads), params,
                                        kMaxDense * sizeof(double), s));
    UNAP_CK(cudaMemcpyAsync(h_status, d_status.p, sizeof(MegaStatus), cudaMemcpyDeviceToHost, s));
    UNAP_CK(cudaStreamSynchronize(s));
    return h_status->timeout == 0;
}

}  // namespace unapgpu
