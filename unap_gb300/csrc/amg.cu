// AMG hierarchy on the device and its V-cycle (see amg.hpp).
#include <chrono>
#include <climits>
#include <type_traits>

#include "amg.hpp"

namespace unapgpu {

namespace {

template <class T>
Rows<T> rowsT(const Level& L);
template <>
Rows<double> rowsT<double>(const Level& L)
{
    return rows64(L);
}
template <>
Rows<float> rowsT<float>(const Level& L)
{
    return rows32(L);
}

struct Ext {
    const double* r = nullptr;
    double* z = nullptr;
};
thread_local Ext g_ext;

}  // namespace

AmgHierarchy::AmgHierarchy(Matrix& A_, const AmgParams& p) : params(p), A(A_)
{
    auto t0 = std::chrono::steady_clock::now();
    if (!A.host.symm) throw std::invalid_argument("AMG-PCG needs a symmetric matrix");
    if (params.smoother != 0 && params.smoother != 1)
        throw std::invalid_argument("smoother must be 0 (Gauss-Seidel) or 1 (Chebyshev)");
    if (params.smoother == 1) {
        if (params.chebyDegree < 1 || params.chebyDegree > kChebyMaxDegree)
            throw std::invalid_argument("Chebyshev degree must be 1 to 16");
        if (params.chebyFrom < 0) throw std::invalid_argument("chebyFrom must be >= 0");
        if (params.eigRatio <= 0) params.eigRatio = 1.5;  // chebySmoother.hpp:47
        if (!(params.eigRatio > 1.0))
            throw std::invalid_argument("Chebyshev eigenvalue ratio must be > 1");
    }
    // Gauss-Seidel on the finest level sweeps the matrix's wavefronts
    if (!A.L->sweepable && !(params.smoother == 1 && params.chebyFrom == 0))
        throw std::invalid_argument(
            "AMG Gauss-Seidel smoothing needs oriented, owner-sorted faces and a matrix built "
            "with wavefronts");
    cudaStream_t s = A.stream;
    auto tp = t0;
    auto phase = [&](int i) {
        const auto t = std::chrono::steady_clock::now();
        setupPhase[i] = std::chrono::duration<double>(t - tp).count();
        tp = t;
    };
    std::vector<double> w = mg_face_weights(A.host);
    std::vector<CoarseHost> coarse =
        agglomerate_levels(A.host, w, params.nCoarsest, params.maxLevels, 1, s);
    phase(0);
    const int L = (int)coarse.size();
    lv.resize((size_t)L + 1);
    lv[0].L = A.L.get();
    lv[0].n = A.n();
    for (int k = 1; k <= L; ++k) {
        CoarseHost& c = coarse[(size_t)k - 1];
        const Level& F = *lv[(size_t)k - 1].L;
        const int nC = c.A.n;
        // locality key of a coarse cell: the first locality rank of its
        // cells on the finer level (BFS order on the finest)
        std::vector<int> key((size_t)nC, INT_MAX);
        for (int i = 0; i < F.n; ++i) {
            int C = c.restrictAddr[(size_t)i];
            key[(size_t)C] = std::min(key[(size_t)C], F.locRank[(size_t)i]);
        }
        // Chebyshev levels are never swept: locality order, no wavefronts
        lv[(size_t)k].own = build_level(c.A, &key, k == L, s, !isCheby(k));
        lv[(size_t)k].L = lv[(size_t)k].own.get();
        lv[(size_t)k].n = nC;
        const Level& Cl = *lv[(size_t)k].L;
        // restriction: children of every coarse cell, ascending finer cell
        // index (the summation order of restrictField), in internal indices
        std::vector<int> refStart((size_t)nC + 1, 0);
        for (int i = 0; i < F.n; ++i) refStart[(size_t)c.restrictAddr[(size_t)i] + 1]++;
        for (int C = 0; C < nC; ++C) refStart[(size_t)C + 1] += refStart[(size_t)C];
        std::vector<int> refChild((size_t)F.n);
        {
            std::vector<int> pos(refStart.begin(), refStart.end() - 1);
            for (int i = 0; i < F.n; ++i) refChild[(size_t)pos[(size_t)c.restrictAddr[(size_t)i]]++] = i;
        }
        std::vector<int> cs((size_t)nC + 1, 0), ch((size_t)F.n);
        for (int Ci = 0; Ci < nC; ++Ci) {
            int C = Cl.perm[(size_t)Ci];
            int len = refStart[(size_t)C + 1] - refStart[(size_t)C];
            cs[(size_t)Ci + 1] = cs[(size_t)Ci] + len;
            for (int j = 0; j < len; ++j)
                ch[(size_t)(cs[(size_t)Ci] + j)] = F.iperm[(size_t)refChild[(size_t)(refStart[(size_t)C] + j)]];
        }
        std::vector<int> cmap((size_t)F.n);
        for (int i = 0; i < F.n; ++i) cmap[(size_t)i] = Cl.iperm[(size_t)c.restrictAddr[(size_t)F.perm[(size_t)i]]];
        lv[(size_t)k].childStart.upload(cs, s);
        lv[(size_t)k].child.upload(ch, s);
        lv[(size_t)k].cmap.upload(cmap, s);
        UNAP_CK(cudaStreamSynchronize(s));
    }
    phase(1);
    // coarsest: dense FP64 inverse (identity internal order when L >= 1)
    const HostLdu& Ch = L ? coarse[(size_t)L - 1].A : A.host;
    nc = Ch.n;
    if (nc > 8192) throw std::invalid_argument("coarsest level too large for the dense solve");
    {
        const size_t N = (size_t)nc;
        std::vector<double> dense(N * N, 0.0), inv;
        for (int c = 0; c < nc; ++c) dense[(size_t)c * N + c] = Ch.diag[(size_t)c];
        for (int f = 0; f < Ch.nf; ++f) {
            dense[(size_t)Ch.l[(size_t)f] * N + Ch.u[(size_t)f]] += Ch.upper[(size_t)f];
            dense[(size_t)Ch.u[(size_t)f] * N + Ch.l[(size_t)f]] += Ch.lowerPtr()[f];
        }
        // column-major copy with rows in the coarsest level's internal order
        // and columns in its own cell order: column j, row I holds
        // inv[perm[I]][j].  The product then sums each row in cell order,
        // gathering b through iperm (identity, so no gather, when L >= 1;
        // the finest level's order when no coarse level exists).
        const Level& CL = *lv[(size_t)L].L;
        denseGather = L ? nullptr : CL.d_iperm.p;
        if (nc >= kDeviceInverseCells) {
            // the same bits computed on the device (dense_dev.cu)
            Minv.alloc(N * N);
            if (!dense_spd_inverse_device(nc, dense, CL.d_iperm.p, Minv.p, s))
                throw std::invalid_argument("coarsest matrix is not positive definite");
        } else {
            if (!dense_spd_inverse(nc, dense, inv))
                throw std::invalid_argument("coarsest matrix is not positive definite");
            std::vector<double> cm(N * N);
            for (int j = 0; j < nc; ++j)
                for (int I = 0; I < nc; ++I)
                    cm[(size_t)j * N + I] = inv[(size_t)CL.perm[(size_t)I] * N + (size_t)j];
            Minv.upload(cm, s);
        }
    }
    phase(2);
    {
        std::vector<int> all;
        waveOff.assign((size_t)L + 2, 0);
        for (int k = 0; k <= L; ++k) {
            waveOff[(size_t)k] = (int)all.size();
            const std::vector<int>& w = lv[(size_t)k].L->waveStart;
            all.insert(all.end(), w.begin(), w.end());
        }
        waveOff[(size_t)L + 1] = (int)all.size();
        dWaves.upload(all, s);
    }
    for (int k = 0; k <= L; ++k) {
        size_t n = (size_t)lv[(size_t)k].n;
        if (k > 0) {
            lv[(size_t)k].x.alloc(n);
            lv[(size_t)k].b.alloc(n);
        }
        lv[(size_t)k].r.alloc(n);
        if (params.precision == 1) {
            lv[(size_t)k].xf.alloc(n);
            lv[(size_t)k].bf.alloc(n);
            lv[(size_t)k].rf.alloc(n);
            if (k < L) make_fp32(const_cast<Level&>(*lv[(size_t)k].L), s);
        }
    }
    UNAP_CK(cudaStreamSynchronize(s));
    phase(3);
    // row-packed copies of the levels the cluster tail may run (in the
    // precision of the V-cycle)
    for (int k = 0; k < L; ++k) {
        if (lv[(size_t)k].n > kTailPackRows || isCheby(k)) continue;
        if (params.precision == 1)
            pack_rows<float>(rows32(*lv[(size_t)k].L), lv[(size_t)k].pack, s);
        else
            pack_rows<double>(rows64(*lv[(size_t)k].L), lv[(size_t)k].pack, s);
    }
    UNAP_CK(cudaStreamSynchronize(s));
    phase(4);
    if (params.smoother == 1) setupCheby(s);
    tail_cluster_size();  // function attributes and the cluster query, outside any capture
    // the Chebyshev levels of at most cheby_tail_rows() rows, and all below,
    // in one cluster launch
    if (params.smoother == 1 && cheby_tail_rows() > 0 && cheby_tail_cluster() > 0) {
        for (int k = std::max(1, params.chebyFrom); k < L; ++k)
            if (lv[(size_t)k].n <= cheby_tail_rows() && L - k <= kChebTailMaxLevels) {
                chebTail = k;
                break;
            }
        if (chebTail > 0)
            chebTailPart.alloc((size_t)nc * (size_t)((nc + kDenseChunk - 1) / kDenseChunk));
    }
    phase(5);
    setupSeconds =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

std::vector<int> AmgHierarchy::levelCells() const
{
    std::vector<int> v;
    for (auto& l : lv) v.push_back(l.n);
    return v;
}

std::vector<int> AmgHierarchy::levelWavefronts() const
{
    std::vector<int> v;
    for (auto& l : lv) v.push_back(l.L->nWave);
    return v;
}

size_t AmgHierarchy::deviceBytes() const
{
    size_t b = Minv.bytes();
    for (size_t k = 0; k < lv.size(); ++k) {
        const Lv& l = lv[k];
        if (l.own) b += l.own->deviceBytes();
        b += l.childStart.bytes() + l.child.bytes() + l.cmap.bytes() + l.x.bytes() + l.b.bytes() +
             l.r.bytes() + l.xf.bytes() + l.bf.bytes() + l.rf.bytes() + l.pack.bytes() +
             l.t.bytes() + l.tf.bytes();
    }
    return b;
}

template <>
double* AmgHierarchy::X<double>(int k)
{
    return k == 0 ? g_ext.z : lv[(size_t)k].x.p;
}
template <>
double* AmgHierarchy::B<double>(int k)
{
    return k == 0 ? const_cast<double*>(g_ext.r) : lv[(size_t)k].b.p;
}
template <>
double* AmgHierarchy::R<double>(int k)
{
    return lv[(size_t)k].r.p;
}
template <>
float* AmgHierarchy::X<float>(int k)
{
    return lv[(size_t)k].xf.p;
}
template <>
float* AmgHierarchy::B<float>(int k)
{
    return lv[(size_t)k].bf.p;
}
template <>
float* AmgHierarchy::R<float>(int k)
{
    return lv[(size_t)k].rf.p;
}
template <>
double* AmgHierarchy::Tmp<double>(int k)
{
    return lv[(size_t)k].t.p;
}
template <>
float* AmgHierarchy::Tmp<float>(int k)
{
    return lv[(size_t)k].tf.p;
}

template <class T>
T* AmgHierarchy::chebBuf(int k, int j)
{
    return ((params.chebyDegree - 1 - j) % 2 == 0) ? X<T>(k) : Tmp<T>(k);
}

void AmgHierarchy::setupCheby(cudaStream_t s)
{
    const int L = nLevels() - 1;
    Exec ex{s, device_max_blocks()};
    size_t nMax = 0;
    for (int k = 0; k < L; ++k)
        if (isCheby(k)) nMax = std::max(nMax, (size_t)lv[(size_t)k].n);
    if (!nMax) return;
    DevArray<double> x(nMax), b(nMax), rD(nMax), rA(nMax), wA(nMax), pA(nMax);
    DevArray<EigState> es(1);
    RedPool pool;
    pool.init(2, ex.maxBlocks, 1, s);
    for (int k = 0; k < L; ++k) {
        if (!isCheby(k)) continue;
        Lv& V = lv[(size_t)k];
        const Level& Lk = *V.L;
        const int n = V.n;
        // eigenDiagPCG from x = 0 on b = the splitmix64 start vector, FP64
        k_fill<double>(ex, n, x.p, 0.0);
        k_eig_start(ex, n, Lk.d_perm.p, b.p);
        k_reciprocal(ex, n, Lk.d_diag.p, rD.p);
        EigState h{};
        h.wArA = 1.0e37;  // GREAT, eigenDiagPCG.cpp:75
        UNAP_CK(cudaMemcpyAsync(es.p, &h, sizeof(EigState), cudaMemcpyHostToDevice, s));
        eig_diag_pcg(ex, rows64(Lk), rD.p, x.p, b.p, rA.p, wA.p, pA.p, es.p,
                     pool.site(0, nullptr, FIN_RES_ONLY), pool.site(1, nullptr, FIN_RES_ONLY), 10);
        k_eig_sturm(ex, es.p, 10);
        UNAP_CK(cudaMemcpyAsync(&h, es.p, sizeof(EigState), cudaMemcpyDeviceToHost, s));
        UNAP_CK(cudaStreamSynchronize(s));
        V.lam = h.maxEig;
        cheby_coeffs(V.lam, params.eigRatio, params.chebyDegree, &V.Rth, V.d1, V.d2);
        if (params.precision == 1)
            V.tf.alloc((size_t)n);
        else
            V.t.alloc((size_t)n);
    }
    UNAP_CK(cudaStreamSynchronize(s));
}

std::vector<double> AmgHierarchy::eigenvalues() const
{
    std::vector<double> v;
    for (int k = 0; k + 1 < nLevels(); ++k) v.push_back(lv[(size_t)k].lam);
    return v;
}

int AmgHierarchy::tailFirst(size_t elemBytes) const
{
    const int L = nLevels() - 1;
    const long long rows = tail_rows(params.precision);
    if (L < 1 || rows <= 0 || nc > kTailMaxCoarsest) return L;
    // the tail kernel runs Gauss-Seidel levels only, and a tail is a suffix
    if (params.smoother == 1 && params.chebyFrom < L) return L;
    const int C = tail_cluster_size();
    if (C < 1) return L;
    const long long single = single_rows(params.precision);
    const size_t budget = tail_smem_bytes();
    // the tail is the suffix of levels with at most `rows` rows whose x fits
    // in the cluster's shared memory and whose tables fit the kernel's
    std::vector<int> sizes{nc};
    int t = L;
    while (t > 0) {
        const int k = t - 1;
        if (lv[(size_t)k].n > rows || !lv[(size_t)k].pack.rec.p || L - k > kTailMaxLevels ||
            waveOff[(size_t)L] - waveOff[(size_t)k] > kTailMaxWaves)
            break;
        std::vector<int> s2{lv[(size_t)k].n};
        s2.insert(s2.end(), sizes.begin(), sizes.end());
        const long long e = tail_x_elems(s2, C, single);
        const size_t bytes = (((size_t)e * elemBytes + 15) & ~(size_t)15) + (size_t)nc * sizeof(double);
        if (bytes > budget) break;
        sizes.swap(s2);
        t = k;
    }
    return t;
}

template <class T>
void AmgHierarchy::launch_tail(const Exec& ex, int t, Gate g)
{
    const int L = nLevels() - 1;
    const long long single = single_rows(params.precision);
    const int C = tail_cluster_size();
    TailArgs a;
    a.nLv = L - t;
    a.nPre = params.nPre;
    a.nPost = params.nPost;
    int off = 0;
    for (int k = t; k < L; ++k) {
        const Level& Lk = *lv[(size_t)k].L;
        const Rows<T> rw = rowsT<T>(Lk);
        const Lv& Cn = lv[(size_t)k + 1];
        TailLevel& d = a.lv[k - t];
        d.n = Lk.n;
        d.nWave = Lk.nWave;
        d.waveOff = waveOff[(size_t)k] - waveOff[(size_t)t];
        d.single = Lk.n <= single ? 1 : 0;
        d.nNext = Cn.n;
        d.xOff = off;
        off += (int)tail_x_elems({Lk.n, 0}, C, single);
        d.sliceOff = rw.sliceOff;
        d.rowInfo = rw.rowInfo;
        d.col = rw.col;
        d.val = rw.val;
        d.diag = rw.diag;
        d.b = B<T>(k);
        d.r = R<T>(k);
        d.childStart = Cn.childStart.p;
        d.child = Cn.child.p;
        d.cmap = Cn.cmap.p;
        d.pmeta = lv[(size_t)k].pack.meta.p;
        d.prec = lv[(size_t)k].pack.rec.p;
    }
    a.nc = nc;
    a.xcOff = off;
    off += (int)tail_x_elems({nc}, C, single);
    a.xElems = off;
    a.Minv = Minv.p;
    a.bc = B<T>(L);
    a.xOut = X<T>(t);
    a.waves = dWaves.p + waveOff[(size_t)t];
    a.nWaveTotal = waveOff[(size_t)L] - waveOff[(size_t)t];
    a.g = g;
    launch_tail_vcycle<T>(a, C, ex.s);
}

template <class T>
void AmgHierarchy::sweep(const Exec& ex, int k, const Level& Lk, const Rows<T>& Rk, T* x,
                         const T* b, bool backward, bool xIsZero, Gate g)
{
    const PackedRows& P = lv[(size_t)k].pack;
    // the row-packed form on levels whose rows are long (more than 8
    // entries on average), where the SELL chunks would chain two loads
    const int mode = packed_sweeps();
    if (P.rec.p && mode != 0 && Rk.wide) {
        // register window by mean row length (measured per level on 256^3)
        const bool wide = mode == 3 || (mode == 1 && 2.0 * Lk.nf > 12.5 * Lk.n);
        gs_sweep_packed<T>(ex, Lk, P, Rk.diag, x, b, backward, xIsZero, wide, g);
    }
    else
        gs_sweep<T>(ex, Lk, Rk, x, b, backward, xIsZero, g);
}

template <class T>
ChebTailArgs<T> AmgHierarchy::chebTailArgs(int k)
{
    const int L = nLevels() - 1;
    ChebTailArgs<T> a{};
    a.nLev = L - k;
    a.deg = params.chebyDegree;
    for (int l = 0; l < a.nLev; ++l) {
        const int kk = k + l;
        Lv& V = lv[(size_t)kk];
        ChebTailLevel<T>& t = a.lev[l];
        t.A = rowsT<T>(*V.L);
        t.childStart = V.childStart.p;
        t.child = V.child.p;
        t.cmap = V.cmap.p;
        t.x = X<T>(kk);
        t.b = B<T>(kk);
        t.w = R<T>(kk);
        t.cb[0] = chebBuf<T>(kk, 0);
        t.cb[1] = chebBuf<T>(kk, 1);
        t.post = (params.chebyDegree % 2 == 0) ? X<T>(kk) : Tmp<T>(kk);
        t.Rth = (T)V.Rth;
        for (int j = 0; j < kChebyMaxDegree; ++j) {
            t.d1[j] = (T)V.d1[j];
            t.d2[j] = (T)V.d2[j];
        }
    }
    a.nc = nc;
    a.cChildStart = lv[(size_t)L].childStart.p;
    a.cChild = lv[(size_t)L].child.p;
    a.cCmap = lv[(size_t)L].cmap.p;
    a.cb = B<T>(L);
    a.cx = X<T>(L);
    a.Minv = Minv.p;
    a.part = chebTailPart.p;
    return a;
}

template <class T>
void AmgHierarchy::vcycle_level(const Exec& ex, int k, Gate g)
{
    const int L = nLevels() - 1;
    T* x = X<T>(k);
    T* b = B<T>(k);
    if (profIn) UNAP_CK(cudaEventRecordWithFlags((*profIn)[(size_t)k], ex.s, cudaEventRecordExternal));
    if (k == curTail && k < L) {
        launch_tail<T>(ex, k, g);
        if (profOut) UNAP_CK(cudaEventRecordWithFlags((*profOut)[(size_t)k], ex.s, cudaEventRecordExternal));
        return;
    }
    if (k == chebTail) {
        launch_cheb_tail<T>(ex, chebTailArgs<T>(k), g);
        if (profOut) UNAP_CK(cudaEventRecordWithFlags((*profOut)[(size_t)k], ex.s, cudaEventRecordExternal));
        return;
    }
    if (k == L) {
        k_dense_apply<T>(ex, nc, Minv.p, b, denseGather, x, g);
        if (profOut) UNAP_CK(cudaEventRecordWithFlags((*profOut)[(size_t)k], ex.s, cudaEventRecordExternal));
        return;
    }
    const Level& Lk = *lv[(size_t)k].L;
    Rows<T> Rk = rowsT<T>(Lk);
    T* r = R<T>(k);
    const bool cheb = isCheby(k);
    const Lv& V = lv[(size_t)k];
    const int deg = params.chebyDegree;
    if (cheb) {
        // pre-smoothing from x = 0 (w shares the residual's buffer); the
        // first step of a coarse level ran inside the restriction
        if (k == 0) {
            if (std::is_same<T, float>::value)
                k_cheb_zero<T>(ex, Lk.n, Rk.diag, b, g_ext.r, chebBuf<T>(k, 0), r, (T)V.Rth, g);
            else
                k_cheb_zero<T>(ex, Lk.n, Rk.diag, b, nullptr, chebBuf<T>(k, 0), r, (T)V.Rth, g);
        }
        for (int j = 1; j < deg; ++j)
            k_cheb_step<T>(ex, Rk, chebBuf<T>(k, j - 1), chebBuf<T>(k, j), b, r, (T)V.d1[j],
                           (T)V.d2[j], 0, g);
    } else if (params.nPre > 0) {
        for (int s = 0; s < params.nPre; ++s) sweep<T>(ex, k, Lk, Rk, x, b, false, s == 0, g);
    } else {
        k_fill<T>(ex, Lk.n, x, T(0));
    }
    k_residual<T>(ex, Rk, x, b, r, RSpec{}, g);
    const Lv& C = lv[(size_t)k + 1];
    if (isCheby(k + 1))
        k_restrict_cheb_zero<T>(ex, C.n, C.childStart.p, C.child.p, r, B<T>(k + 1),
                                rowsT<T>(*C.L).diag, chebBuf<T>(k + 1, 0), R<T>(k + 1),
                                (T)C.Rth, g);
    else
        k_restrict<T>(ex, C.n, C.childStart.p, C.child.p, r, B<T>(k + 1), g);
    vcycle_level<T>(ex, k + 1, g);
    if (cheb) {
        // post-smoothing from x + P e: the prolongation writes the buffer the
        // chain starts from
        T* prev = (deg % 2 == 0) ? x : Tmp<T>(k);
        if (prev == x)
            k_prolong_add<T>(ex, Lk.n, C.cmap.p, X<T>(k + 1), x, g);
        else
            k_prolong_add_to<T>(ex, Lk.n, C.cmap.p, X<T>(k + 1), x, prev, g);
        for (int j = 0; j < deg; ++j) {
            T* out = chebBuf<T>(k, j);
            k_cheb_step<T>(ex, Rk, prev, out, b, r, j == 0 ? (T)V.Rth : (T)V.d1[j],
                           j == 0 ? T(0) : (T)V.d2[j], j == 0 ? 1 : 0, g);
            prev = out;
        }
    } else {
        k_prolong_add<T>(ex, Lk.n, C.cmap.p, X<T>(k + 1), x, g);
        for (int s = 0; s < params.nPost; ++s) sweep<T>(ex, k, Lk, Rk, x, b, true, false, g);
    }
    if (profOut) UNAP_CK(cudaEventRecordWithFlags((*profOut)[(size_t)k], ex.s, cudaEventRecordExternal));
}

template <class T>
void AmgHierarchy::append_level(std::vector<Step>& out, int k, int tableBase)
{
    const int L = nLevels() - 1;
    const int prec = std::is_same<T, float>::value ? 1 : 0;
    const int lvl = k == 0 ? 0 : tableBase + k - 1;
    T* x = X<T>(k);
    T* b = B<T>(k);
    auto step = [&](int op, bool single) {
        Step s;
        s.op = op;
        s.prec = prec;
        s.single = single ? 1 : 0;
        s.lvl = lvl;
        return s;
    };
    if (k == L) {
        Step s = step(ST_DENSE, true);
        s.r1 = nc;
        s.e = Minv.p;
        s.i0 = denseGather;
        s.a = b;
        s.c = x;
        s.bytes = 8.0 * nc * nc + 2.0 * sizeof(T) * nc;
        out.push_back(s);
        return;
    }
    const Level& Lk = *lv[(size_t)k].L;
    const bool single = mega_single_level(Lk.n);
    const bool cheb = isCheby(k);
    const Lv& V = lv[(size_t)k];
    const int deg = params.chebyDegree;
    const bool fp32 = prec == 1;
    auto chebStep = [&](const T* xin, T* xout, int j) {
        Step s = step(ST_CHEB, single);
        s.a = xin;
        s.b = b;
        s.c = xout;
        s.d = R<T>(k);
        s.f0 = j == 0 ? 1 : 0;
        s.k1 = j == 0 ? V.Rth : V.d1[j];
        s.k2 = j == 0 ? 0.0 : V.d2[j];
        s.bytes = cheb_bytes(Lk.n, Lk.nf, fp32, j != 0);
        out.push_back(s);
    };
    if (cheb) {
        if (k == 0) {
            Step s = step(ST_CHEB0, single);
            s.b = b;
            s.e = fp32 ? g_ext.r : nullptr;
            s.c = chebBuf<T>(k, 0);
            s.d = R<T>(k);
            s.k1 = V.Rth;
            s.bytes = (double)sizeof(T) * 4 * Lk.n + (fp32 ? 12.0 * Lk.n : 0.0);
            out.push_back(s);
        }
        for (int j = 1; j < deg; ++j) chebStep(chebBuf<T>(k, j - 1), chebBuf<T>(k, j), j);
    } else if (params.nPre > 0) {
        for (int sw = 0; sw < params.nPre; ++sw)
            for (int w = 0; w < Lk.nWave; ++w) {
                Step s = step(ST_GS, single);
                s.r0 = Lk.waveStart[(size_t)w];
                s.r1 = Lk.waveStart[(size_t)w + 1];
                s.f0 = sw == 0 ? 1 : 0;  // first sweep from x = 0: upper side is zero
                s.b = b;
                s.c = x;
                s.bytes = sweep_bytes(s.r1 - s.r0, Lk.n, Lk.nf, prec == 1);
                out.push_back(s);
            }
    } else {
        Step s = step(ST_FILL0, single);
        s.r1 = Lk.n;
        s.c = x;
        s.bytes = (double)sizeof(T) * Lk.n;
        out.push_back(s);
    }
    {
        Step s = step(ST_RESID, single);
        s.a = x;
        s.b = b;
        s.c = R<T>(k);
        s.bytes = sweep_bytes(Lk.n, Lk.n, Lk.nf, prec == 1);
        out.push_back(s);
    }
    const Lv& C = lv[(size_t)k + 1];
    if (isCheby(k + 1)) {
        Step s = step(ST_RESTRICT_CHEB0, single);
        s.lvl = tableBase + k;  // the coarse level's rows (diagonal)
        s.r1 = C.n;
        s.i0 = C.childStart.p;
        s.i1 = C.child.p;
        s.a = R<T>(k);
        s.c = B<T>(k + 1);
        s.d = chebBuf<T>(k + 1, 0);
        s.e = R<T>(k + 1);
        s.k1 = C.Rth;
        s.bytes = (sizeof(T) + 4.0) * Lk.n + (4.0 * sizeof(T) + 4.0) * C.n;
        out.push_back(s);
    } else {
        Step s = step(ST_RESTRICT, single);
        s.r1 = C.n;
        s.i0 = C.childStart.p;
        s.i1 = C.child.p;
        s.a = R<T>(k);
        s.c = B<T>(k + 1);
        s.bytes = (sizeof(T) + 4.0) * Lk.n + (sizeof(T) + 4.0) * C.n;
        out.push_back(s);
    }
    append_level<T>(out, k + 1, tableBase);
    if (cheb) {
        T* prev = (deg % 2 == 0) ? x : Tmp<T>(k);
        Step s = step(prev == x ? ST_PROLONG_ADD : ST_PROLONG_TO, single);
        s.r1 = Lk.n;
        s.i0 = C.cmap.p;
        s.a = X<T>(k + 1);
        s.b = x;
        s.c = prev;
        s.bytes = (2.0 * sizeof(T) + 4.0) * Lk.n + (double)sizeof(T) * C.n;
        out.push_back(s);
        for (int j = 0; j < deg; ++j) {
            T* o = chebBuf<T>(k, j);
            chebStep(prev, o, j);
            prev = o;
        }
        return;
    }
    {
        Step s = step(ST_PROLONG_ADD, single);
        s.r1 = Lk.n;
        s.i0 = C.cmap.p;
        s.a = X<T>(k + 1);
        s.c = x;
        s.bytes = (2.0 * sizeof(T) + 4.0) * Lk.n + (double)sizeof(T) * C.n;
        out.push_back(s);
    }
    for (int sw = 0; sw < params.nPost; ++sw)
        for (int w = Lk.nWave - 1; w >= 0; --w) {
            Step s = step(ST_GS, single);
            s.r0 = Lk.waveStart[(size_t)w];
            s.r1 = Lk.waveStart[(size_t)w + 1];
            s.b = b;
            s.c = x;
            s.bytes = sweep_bytes(s.r1 - s.r0, Lk.n, Lk.nf, prec == 1);
            out.push_back(s);
        }
}

void AmgHierarchy::appendVcycle(std::vector<Step>& out, std::vector<LevelRows>& table,
                                const double* r, double* z)
{
    g_ext.r = r;
    g_ext.z = z;
    const int tableBase = (int)table.size();
    for (int k = 1; k < nLevels(); ++k) {
        LevelRows e;
        e.r64 = rows64(*lv[(size_t)k].L);
        if (lv[(size_t)k].L->d_val32.p) e.r32 = rows32(*lv[(size_t)k].L);
        table.push_back(e);
    }
    const int n0 = lv[0].n;
    if (params.precision == 1) {
        table[0].r32 = rows32(*lv[0].L);
        Step s;
        s.op = ST_D2F;
        s.single = mega_single_level(n0);
        s.r1 = n0;
        s.a = r;
        s.c = lv[0].bf.p;
        s.bytes = 12.0 * n0;
        // a Chebyshev finest level converts r inside its first step
        if (!isCheby(0)) out.push_back(s);
        append_level<float>(out, 0, tableBase);
        Step t;
        t.op = ST_F2D;
        t.single = s.single;
        t.r1 = n0;
        t.a = lv[0].xf.p;
        t.c = z;
        t.bytes = 12.0 * n0;
        out.push_back(t);
    } else {
        append_level<double>(out, 0, tableBase);
    }
}

void AmgHierarchy::vcycle(const Exec& ex, const double* r, double* z, Gate g)
{
    g_ext.r = r;
    g_ext.z = z;
    curTail = tailFirst(params.precision == 1 ? sizeof(float) : sizeof(double));
    if (params.precision == 1) {
        // a Chebyshev finest level converts r inside its first step
        if (!isCheby(0)) k_d2f(ex, lv[0].n, r, lv[0].bf.p);
        vcycle_level<float>(ex, 0, g);
        k_f2d(ex, lv[0].n, lv[0].xf.p, z);
    } else {
        vcycle_level<double>(ex, 0, g);
    }
}

template <class T>
static double time_smoother(AmgHierarchy& H, cudaStream_t s, int k, int reps, double* bytes,
                            int* launches)
{
    const AmgHierarchy::Lv& V = H.lv[(size_t)k];
    const Level& Lk = *V.L;
    const Rows<T> R = rowsT<T>(Lk);
    const bool fp32 = std::is_same<T, float>::value;
    Exec ex{s, device_max_blocks()};
    DevArray<T> x((size_t)V.n), t((size_t)V.n), b((size_t)V.n), w((size_t)V.n);
    k_fill<T>(ex, V.n, x.p, T(0));
    k_fill<T>(ex, V.n, t.p, T(0));
    k_fill<T>(ex, V.n, b.p, T(1));
    k_fill<T>(ex, V.n, w.p, T(0));
    const bool cheb = H.isCheby(k);
    auto run = [&]() {
        if (cheb)
            k_cheb_step<T>(ex, R, x.p, t.p, b.p, w.p, (T)V.d1[1 % H.params.chebyDegree],
                           (T)V.d2[1 % H.params.chebyDegree], 0, Gate{});
        else if (V.pack.rec.p && packed_sweeps() != 0 && R.wide)
            gs_sweep_packed<T>(ex, Lk, V.pack, R.diag, x.p, b.p, false, false,
                               packed_sweeps() == 3 ||
                                   (packed_sweeps() == 1 && 2.0 * Lk.nf > 12.5 * Lk.n),
                               Gate{});
        else
            gs_sweep<T>(ex, Lk, R, x.p, b.p, false, false, Gate{});
    };
    run();
    cudaEvent_t e0, e1;
    UNAP_CK(cudaEventCreate(&e0));
    UNAP_CK(cudaEventCreate(&e1));
    UNAP_CK(cudaEventRecord(e0, s));
    for (int i = 0; i < reps; ++i) run();
    UNAP_CK(cudaEventRecord(e1, s));
    UNAP_CK(cudaEventSynchronize(e1));
    float ms = 0;
    UNAP_CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (bytes)
        *bytes = cheb ? cheb_bytes(V.n, Lk.nf, fp32, true) : sweep_bytes(V.n, V.n, Lk.nf, fp32);
    if (launches) *launches = cheb ? 1 : Lk.nWave;
    return (double)ms / std::max(reps, 1);
}

double AmgHierarchy::profileSmoother(cudaStream_t s, int k, int reps, double* bytes,
                                     int* launches)
{
    if (k < 0 || k >= nLevels() - 1) throw std::invalid_argument("no smoothed level there");
    return params.precision == 1 ? time_smoother<float>(*this, s, k, reps, bytes, launches)
                                 : time_smoother<double>(*this, s, k, reps, bytes, launches);
}

int AmgHierarchy::profile(cudaStream_t s, int reps, double* ms, int maxOut)
{
    const int nl = nLevels();
    const size_t n0 = (size_t)lv[0].n;
    DevArray<double> r(n0), z(n0);
    Exec ex{s, device_max_blocks()};
    k_fill<double>(ex, (int)n0, r.p, 1.0);
    cudaEvent_t e0, e1;
    UNAP_CK(cudaEventCreate(&e0));
    UNAP_CK(cudaEventCreate(&e1));
    std::vector<cudaEvent_t> in((size_t)nl), out((size_t)nl);
    for (int k = 0; k < nl; ++k) {
        UNAP_CK(cudaEventCreate(&in[(size_t)k]));
        UNAP_CK(cudaEventCreate(&out[(size_t)k]));
    }
    // levels below a tail (the Gauss-Seidel cluster tail or the Chebyshev
    // one) record no events: the tail's first level holds the whole tail
    const int tail = chebTail >= 0
                         ? chebTail
                         : tailFirst(params.precision == 1 ? sizeof(float) : sizeof(double));
    // one V-cycle captured as a CUDA graph (as inside a solve), with an
    // event node around every level
    cudaGraph_t gr = nullptr;
    cudaGraphExec_t ge = nullptr;
    profIn = &in;
    profOut = &out;
    {
        CaptureGate gate;
        UNAP_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        set_capturing(true);
        try {
            vcycle(ex, r.p, z.p, Gate{});
        } catch (...) {
            set_capturing(false);
            profIn = profOut = nullptr;
            cudaStreamEndCapture(s, &gr);
            if (gr) cudaGraphDestroy(gr);
            throw;
        }
        set_capturing(false);
        profIn = profOut = nullptr;
        UNAP_CK(cudaStreamEndCapture(s, &gr));
    }
    UNAP_CK(cudaGraphInstantiate(&ge, gr, 0));
    UNAP_CK(cudaGraphLaunch(ge, s));
    UNAP_CK(cudaEventRecord(e0, s));
    for (int i = 0; i < reps; ++i) UNAP_CK(cudaGraphLaunch(ge, s));
    UNAP_CK(cudaEventRecord(e1, s));
    UNAP_CK(cudaEventSynchronize(e1));
    float t = 0;
    UNAP_CK(cudaEventElapsedTime(&t, e0, e1));
    if (maxOut > 0) ms[0] = (double)t / std::max(reps, 1);
    UNAP_CK(cudaStreamSynchronize(s));
    cudaGraphExecDestroy(ge);
    cudaGraphDestroy(gr);
    int written = 1;
    for (int k = 0; k < nl && 1 + k < maxOut; ++k) {
        double own = 0;
        if (k <= tail || k == nl - 1) {
            float a = 0, b = 0;
            const bool inner = k + 1 < nl && !(k == tail && tail < nl - 1);
            if (inner) {
                UNAP_CK(cudaEventElapsedTime(&a, in[(size_t)k], in[(size_t)k + 1]));
                UNAP_CK(cudaEventElapsedTime(&b, out[(size_t)k + 1], out[(size_t)k]));
                own = (double)a + (double)b;
            } else if (k <= tail || tail == nl - 1) {
                UNAP_CK(cudaEventElapsedTime(&a, in[(size_t)k], out[(size_t)k]));
                own = a;
            }
        }
        ms[1 + k] = own;
        written = 2 + k;
    }
    for (int k = 0; k < nl; ++k) {
        cudaEventDestroy(in[(size_t)k]);
        cudaEventDestroy(out[(size_t)k]);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return written;
}

}  // namespace unapgpu
