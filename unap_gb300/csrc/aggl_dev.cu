// One level of the reference's pairwise agglomeration on the device, with
// the same result as the host form in agglomeration.cpp (restrict map, coarse
// addressing, coarse coefficients, restricted face weights), bit for bit.
//
// The matching (lduAgglomerate.cpp:94-271) is a sequential greedy: cell c,
// if still free at its turn, pairs with the neighbour across its heaviest
// face among free neighbours, else joins the cluster across its heaviest
// face.  Its turn depends only on the state of its neighbours at that time,
// which only cells d < c within two faces can change.  So c can take its
// turn as soon as every such d has taken its own (or, per neighbour, the
// neighbour is already assigned): a round computes, for every cell v, the
// smallest cell around v (v and its neighbours) that has not taken its turn,
// marks c ready when that is c itself around c and around every free
// neighbour, and runs all ready cells at once.  Ready cells never touch
// each other's state (each would have to be around the other), so every
// turn sees exactly what it sees in the sequential order.  On randomly
// numbered matrices the rounds number tens; on structured numberings the
// chains can be long, so after kMaxRounds the level goes back to the host.
//
// Cluster numbers follow the sequential counter: pairs in the order of the
// cell whose turn formed them, then the cells left alone, in cell order.
// Coarse faces are numbered per coarse owner in the order its fine
// boundary faces (in face order) first meet each neighbour, and coarse
// coefficients and weights are summed per coarse face in fine face order,
// the coarse diagonal over the aggregate's cells in cell order and then its
// interior faces in face order -- the host's summation orders.
#include <algorithm>
#include <climits>

#include "amg.hpp"

namespace unapgpu {

namespace {

constexpr int kThreads = 256;
constexpr double kSmall = 1.0e-37;  // SMALL, src/base/unap.hpp:88
constexpr int kMaxList = 2048;      // longer per-cell lists: host
constexpr int kMaxRounds = 512;

template <class T>
using Scratch = StreamScratch<T>;

int grid_for(long long n)
{
    long long b = (n + kThreads - 1) / kThreads;
    return (int)std::max(1LL, std::min(b, 1LL << 30));
}

#define GRID_LOOP(i, n) \
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); \
         i += (long long)gridDim.x * blockDim.x)

// per-cell counts of the two sides of every face
__global__ void k_adj_count(const int* __restrict__ l, const int* __restrict__ u, int nf, int* deg)
{
    GRID_LOOP(f, nf)
    {
        atomicAdd(&deg[u[f]], 1);
        atomicAdd(&deg[l[f]], 1);
    }
}

// key of a list entry: the face where the cell is the neighbour (u side)
// sorts before the faces where it is the owner, each by face index
__global__ void k_adj_fill(const int* __restrict__ l, const int* __restrict__ u, int nf,
                           int* cursor, long long* key)
{
    GRID_LOOP(f, nf)
    {
        key[atomicAdd(&cursor[u[f]], 1)] = f;
        key[atomicAdd(&cursor[l[f]], 1)] = (long long)nf + f;
    }
}

template <class K>
__global__ void k_sort_lists(const int* __restrict__ start, long long n, K* key, int* tooLong)
{
    GRID_LOOP(c, n)
    {
        const int a = start[c], e = start[c + 1];
        if (e - a > kMaxList) {
            atomicOr(tooLong, 1);
            continue;
        }
        for (int i = a + 1; i < e; ++i) {
            const K v = key[i];
            int j = i - 1;
            while (j >= a && key[j] > v) {
                key[j + 1] = key[j];
                --j;
            }
            key[j + 1] = v;
        }
    }
}

__global__ void k_adj_expand(const long long* __restrict__ key, long long m, const int* __restrict__ l,
                             const int* __restrict__ u, const double* __restrict__ w, int nf,
                             int* nbr, double* wt)
{
    GRID_LOOP(e, m)
    {
        const long long k = key[e];
        const int f = (int)(k < nf ? k : k - nf);
        nbr[e] = k < nf ? l[f] : u[f];
        wt[e] = w[f];
    }
}

// smallest cell among v and its neighbours that has not taken its turn
__global__ void k_min_pending(const int* __restrict__ start, const int* __restrict__ nbr, int n,
                              const unsigned char* __restrict__ done, int* mp)
{
    GRID_LOOP(v, n)
    {
        int m = done[v] ? INT_MAX : (int)v;
        for (int e = start[v]; e < start[v + 1]; ++e) {
            const int x = nbr[e];
            if (!done[x] && x < m) m = x;
        }
        mp[v] = m;
    }
}

__global__ void k_ready(const int* __restrict__ start, const int* __restrict__ nbr, int n,
                        const unsigned char* __restrict__ done, const int* __restrict__ lead,
                        const int* __restrict__ mp, unsigned char* ready, int* pending)
{
    GRID_LOOP(c, n)
    {
        unsigned char r = 0;
        if (!done[c]) {
            *pending = 1;  // every writer stores the same value
            bool ok = mp[c] == c;
            for (int e = start[c]; ok && e < start[c + 1]; ++e) {
                const int v = nbr[e];
                ok = lead[v] >= 0 || mp[v] == c;
            }
            r = ok;
        }
        ready[c] = r;
    }
}

// the turns of the ready cells (pairwise_pass's loop body)
__global__ void k_turn(const int* __restrict__ start, const int* __restrict__ nbr,
                       const double* __restrict__ wt, int n, const unsigned char* __restrict__ ready,
                       int* lead, unsigned char* done, unsigned char* former)
{
    GRID_LOOP(c, n)
    {
        if (!ready[c]) continue;
        const int a = start[c], e = start[c + 1];
        int match = -1;
        double maxW = kSmall;
        for (int k = a; k < e; ++k)
            if (lead[nbr[k]] < 0 && wt[k] > maxW) {
                match = nbr[k];
                maxW = wt[k];
            }
        done[c] = 1;
        if (match >= 0) {
            lead[c] = (int)c;
            lead[match] = (int)c;
            done[match] = 1;
            former[c] = 1;
            continue;
        }
        int cmatch = -1;
        double cmax = kSmall;
        for (int k = a; k < e; ++k)
            if (wt[k] > cmax) {
                cmatch = nbr[k];
                cmax = wt[k];
            }
        if (cmatch >= 0) lead[c] = lead[cmatch];
    }
}

__global__ void k_flags(const unsigned char* __restrict__ former, const int* __restrict__ lead, int n,
                        int* pairF, int* aloneF)
{
    GRID_LOOP(c, n)
    {
        pairF[c] = former[c];
        aloneF[c] = lead[c] < 0;
    }
}

__global__ void k_map(const int* __restrict__ lead, const int* __restrict__ pairId,
                      const int* __restrict__ aloneId, int nPairs, int n, int* map)
{
    GRID_LOOP(c, n)
    map[c] = lead[c] >= 0 ? pairId[lead[c]] : nPairs + aloneId[c];
}

// coarse owner of every fine face (-1: inside an aggregate, with its
// faceRestrict written) and counts per coarse owner / aggregate
__global__ void k_face_owner(const int* __restrict__ l, const int* __restrict__ u,
                             const int* __restrict__ map, int nf, int* own, int* faceRestrict,
                             int* segCnt, int* inCnt)
{
    GRID_LOOP(f, nf)
    {
        const int a = map[u[f]], b = map[l[f]];
        if (a != b) {
            const int o = min(a, b);
            own[f] = o;
            atomicAdd(&segCnt[o], 1);
        } else {
            own[f] = -1;
            faceRestrict[f] = -(a + 1);
            atomicAdd(&inCnt[a], 1);
        }
    }
}

__global__ void k_face_fill(const int* __restrict__ own, const int* __restrict__ l,
                            const int* __restrict__ map, int nf, int* segCur, int* seg, int* inCur,
                            int* in)
{
    GRID_LOOP(f, nf)
    {
        const int o = own[f];
        if (o >= 0)
            seg[atomicAdd(&segCur[o], 1)] = (int)f;
        else
            in[atomicAdd(&inCur[map[l[f]]], 1)] = (int)f;
    }
}

__global__ void k_count_kids(const int* __restrict__ map, int n, int* cnt)
{
    GRID_LOOP(i, n)
    atomicAdd(&cnt[map[i]], 1);
}

__global__ void k_cell_fill(const int* __restrict__ map, int n, int* cur, int* kids)
{
    GRID_LOOP(i, n)
    kids[atomicAdd(&cur[map[i]], 1)] = (int)i;
}

// distinct neighbours of every coarse owner in discovery order
__global__ void k_owner_faces(const int* __restrict__ segStart, const int* __restrict__ seg, int nc,
                              const int* __restrict__ l, const int* __restrict__ u,
                              const int* __restrict__ map, int* nei, int* local, int* cnt)
{
    GRID_LOOP(c, nc)
    {
        const int a = segStart[c], e = segStart[c + 1];
        int m = 0;
        for (int i = a; i < e; ++i) {
            const int f = seg[i];
            const int ne = max(map[u[f]], map[l[f]]);
            int j = 0;
            while (j < m && nei[a + j] != ne) ++j;
            if (j == m) nei[a + m++] = ne;
            local[i] = j;
        }
        cnt[c] = m;
    }
}

// coarse faces of every owner: addressing, faceRestrict, coefficients and
// weights summed in fine face order
__global__ void k_owner_coeffs(const int* __restrict__ segStart, const int* __restrict__ seg, int nc,
                               const int* __restrict__ nei, const int* __restrict__ local,
                               const int* __restrict__ cfStart, const int* __restrict__ l,
                               const int* __restrict__ map, const double* __restrict__ upper,
                               const double* __restrict__ lower, const double* __restrict__ w,
                               int* Cl, int* Cu, double* Cup, double* Clo, double* cw,
                               int* faceRestrict)
{
    GRID_LOOP(c, nc)
    {
        const int a = segStart[c], e = segStart[c + 1], k0 = cfStart[c], m = cfStart[c + 1] - k0;
        for (int j = 0; j < m; ++j) {
            Cl[k0 + j] = (int)c;
            Cu[k0 + j] = nei[a + j];
        }
        for (int i = a; i < e; ++i) {
            const int f = seg[i], cf = k0 + local[i];
            faceRestrict[f] = cf;
            if (Clo) {
                // the fine face's owner side decides which coarse side it feeds
                if (map[l[f]] == (int)c) {
                    Cup[cf] += upper[f];
                    Clo[cf] += lower[f];
                } else {
                    Cup[cf] += lower[f];
                    Clo[cf] += upper[f];
                }
            } else {
                Cup[cf] += upper[f];
            }
            cw[cf] += w[f];
        }
    }
}

__global__ void k_coarse_diag(const int* __restrict__ kidStart, const int* __restrict__ kids,
                              const int* __restrict__ inStart, const int* __restrict__ in, int nc,
                              const double* __restrict__ diag, const double* __restrict__ upper,
                              const double* __restrict__ lower, double* Cdiag)
{
    GRID_LOOP(c, nc)
    {
        double t = 0.0;
        for (int i = kidStart[c]; i < kidStart[c + 1]; ++i) t += diag[kids[i]];
        for (int i = inStart[c]; i < inStart[c + 1]; ++i) {
            const int f = in[i];
            t += lower ? upper[f] + lower[f] : 2 * upper[f];
        }
        Cdiag[c] = t;
    }
}

template <class T>
void up(Scratch<T>& d, const std::vector<T>& h, cudaStream_t s)
{
    if (!h.empty())
        UNAP_CK(cudaMemcpyAsync(d.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s));
}

template <class T>
void down(std::vector<T>& h, const T* d, size_t n, cudaStream_t s)
{
    h.resize(n);
    if (n) UNAP_CK(cudaMemcpyAsync(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost, s));
}

int read_int(const int* d, cudaStream_t s)
{
    int h = 0;
    UNAP_CK(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s));
    UNAP_CK(cudaStreamSynchronize(s));
    return h;
}

}  // namespace

// One level: returns false (nothing produced) when the device form leaves
// the level to the host (a list longer than kMaxList, or more than
// kMaxRounds rounds).  On success `out` and `cw` are what pairwise_pass,
// coarse_addressing, coarse_coefficients and the weight restriction give.
bool agglomerate_level_device(const HostLdu& A, const std::vector<double>& w, CoarseHost& out,
                              std::vector<double>& cw, int& nCoarse, cudaStream_t s)
{
    const int n = A.n, nf = A.nf;
    if (n <= 0) return false;
    const bool symm = A.symm;
    Scratch<int> l((size_t)nf, s), u((size_t)nf, s), flag(2, s);
    Scratch<double> dw((size_t)nf, s);
    up(l, A.l, s);
    up(u, A.u, s);
    up(dw, w, s);
    UNAP_CK(cudaMemsetAsync(flag.p, 0, 2 * sizeof(int), s));

    // cell lists in the host pass's order
    Scratch<int> start((size_t)n + 1, s);
    Scratch<long long> key((size_t)2 * nf, s);
    Scratch<int> nbr((size_t)2 * nf, s);
    Scratch<double> wt((size_t)2 * nf, s);
    UNAP_CK(cudaMemsetAsync(start.p, 0, sizeof(int) * ((size_t)n + 1), s));
    if (nf) k_adj_count<<<grid_for(nf), kThreads, 0, s>>>(l.p, u.p, nf, start.p);
    device_exclusive_scan(start.p, start.p, n, s);
    {
        Scratch<int> cur((size_t)n, s);
        UNAP_CK(cudaMemcpyAsync(cur.p, start.p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s));
        if (nf) k_adj_fill<<<grid_for(nf), kThreads, 0, s>>>(l.p, u.p, nf, cur.p, key.p);
    }
    k_sort_lists<long long><<<grid_for(n), kThreads, 0, s>>>(start.p, n, key.p, flag.p);
    if (nf) k_adj_expand<<<grid_for(2LL * nf), kThreads, 0, s>>>(key.p, 2LL * nf, l.p, u.p, dw.p, nf,
                                                                nbr.p, wt.p);
    if (read_int(flag.p, s)) return false;

    // turns in dependency rounds
    Scratch<int> lead((size_t)n, s), mp((size_t)n, s);
    Scratch<unsigned char> done((size_t)n, s), ready((size_t)n, s), former((size_t)n, s);
    UNAP_CK(cudaMemsetAsync(lead.p, 0xff, sizeof(int) * (size_t)n, s));
    UNAP_CK(cudaMemsetAsync(done.p, 0, (size_t)n, s));
    UNAP_CK(cudaMemsetAsync(former.p, 0, (size_t)n, s));
    for (int round = 0;; ++round) {
        k_min_pending<<<grid_for(n), kThreads, 0, s>>>(start.p, nbr.p, n, done.p, mp.p);
        UNAP_CK(cudaMemsetAsync(flag.p + 1, 0, sizeof(int), s));
        k_ready<<<grid_for(n), kThreads, 0, s>>>(start.p, nbr.p, n, done.p, lead.p, mp.p, ready.p,
                                                 flag.p + 1);
        if (read_int(flag.p + 1, s) == 0) break;
        if (round >= kMaxRounds) return false;
        k_turn<<<grid_for(n), kThreads, 0, s>>>(start.p, nbr.p, wt.p, n, ready.p, lead.p, done.p,
                                                former.p);
    }
    UNAP_CK(cudaGetLastError());

    // cluster numbers
    Scratch<int> pairF((size_t)n + 1, s), aloneF((size_t)n + 1, s), map((size_t)n, s);
    k_flags<<<grid_for(n), kThreads, 0, s>>>(former.p, lead.p, n, pairF.p, aloneF.p);
    device_exclusive_scan(pairF.p, pairF.p, n, s);
    device_exclusive_scan(aloneF.p, aloneF.p, n, s);
    const int nPairs = read_int(pairF.p + n, s);
    const int nAlone = read_int(aloneF.p + n, s);
    const int nc = nPairs + nAlone;
    nCoarse = nc;
    k_map<<<grid_for(n), kThreads, 0, s>>>(lead.p, pairF.p, aloneF.p, nPairs, n, map.p);

    // coarse addressing
    Scratch<int> own((size_t)nf, s), fr((size_t)nf, s);
    Scratch<int> segStart((size_t)nc + 1, s), inStart((size_t)nc + 1, s), kidStart((size_t)nc + 1, s);
    UNAP_CK(cudaMemsetAsync(segStart.p, 0, sizeof(int) * ((size_t)nc + 1), s));
    UNAP_CK(cudaMemsetAsync(inStart.p, 0, sizeof(int) * ((size_t)nc + 1), s));
    UNAP_CK(cudaMemsetAsync(kidStart.p, 0, sizeof(int) * ((size_t)nc + 1), s));
    if (nf)
        k_face_owner<<<grid_for(nf), kThreads, 0, s>>>(l.p, u.p, map.p, nf, own.p, fr.p, segStart.p,
                                                      inStart.p);
    k_count_kids<<<grid_for(n), kThreads, 0, s>>>(map.p, n, kidStart.p);
    device_exclusive_scan(segStart.p, segStart.p, nc, s);
    device_exclusive_scan(inStart.p, inStart.p, nc, s);
    device_exclusive_scan(kidStart.p, kidStart.p, nc, s);
    const int nSeg = read_int(segStart.p + nc, s);
    const int nIn = read_int(inStart.p + nc, s);
    Scratch<int> seg((size_t)nSeg, s), in((size_t)nIn, s), kids((size_t)n, s);
    {
        Scratch<int> c1((size_t)nc, s), c2((size_t)nc, s), c3((size_t)nc, s);
        UNAP_CK(cudaMemcpyAsync(c1.p, segStart.p, sizeof(int) * (size_t)nc, cudaMemcpyDeviceToDevice, s));
        UNAP_CK(cudaMemcpyAsync(c2.p, inStart.p, sizeof(int) * (size_t)nc, cudaMemcpyDeviceToDevice, s));
        UNAP_CK(cudaMemcpyAsync(c3.p, kidStart.p, sizeof(int) * (size_t)nc, cudaMemcpyDeviceToDevice, s));
        if (nf) k_face_fill<<<grid_for(nf), kThreads, 0, s>>>(own.p, l.p, map.p, nf, c1.p, seg.p, c2.p, in.p);
        k_cell_fill<<<grid_for(n), kThreads, 0, s>>>(map.p, n, c3.p, kids.p);
    }
    UNAP_CK(cudaMemsetAsync(flag.p, 0, sizeof(int), s));
    k_sort_lists<int><<<grid_for(nc), kThreads, 0, s>>>(segStart.p, nc, seg.p, flag.p);
    k_sort_lists<int><<<grid_for(nc), kThreads, 0, s>>>(inStart.p, nc, in.p, flag.p);
    k_sort_lists<int><<<grid_for(nc), kThreads, 0, s>>>(kidStart.p, nc, kids.p, flag.p);
    if (read_int(flag.p, s)) return false;
    Scratch<int> nei((size_t)nSeg, s), local((size_t)nSeg, s), cfStart((size_t)nc + 1, s);
    k_owner_faces<<<grid_for(nc), kThreads, 0, s>>>(segStart.p, seg.p, nc, l.p, u.p, map.p, nei.p,
                                                    local.p, cfStart.p);
    device_exclusive_scan(cfStart.p, cfStart.p, nc, s);
    const int nCF = read_int(cfStart.p + nc, s);

    // coarse coefficients and weights
    Scratch<double> up_((size_t)nf, s), lo_(symm ? 0 : (size_t)nf, s), dg((size_t)n, s);
    up(up_, A.upper, s);
    if (!symm) up(lo_, A.lower, s);
    up(dg, A.diag, s);
    Scratch<int> Cl((size_t)nCF, s), Cu((size_t)nCF, s);
    Scratch<double> Cup((size_t)nCF, s), Clo(symm ? 0 : (size_t)nCF, s), Cw((size_t)nCF, s),
        Cdiag((size_t)nc, s);
    if (nCF) {
        UNAP_CK(cudaMemsetAsync(Cup.p, 0, sizeof(double) * (size_t)nCF, s));
        UNAP_CK(cudaMemsetAsync(Cw.p, 0, sizeof(double) * (size_t)nCF, s));
        if (!symm) UNAP_CK(cudaMemsetAsync(Clo.p, 0, sizeof(double) * (size_t)nCF, s));
    }
    k_owner_coeffs<<<grid_for(nc), kThreads, 0, s>>>(segStart.p, seg.p, nc, nei.p, local.p, cfStart.p,
                                                     l.p, map.p, up_.p, symm ? nullptr : lo_.p, dw.p,
                                                     Cl.p, Cu.p, Cup.p, symm ? nullptr : Clo.p, Cw.p,
                                                     fr.p);
    k_coarse_diag<<<grid_for(nc), kThreads, 0, s>>>(kidStart.p, kids.p, inStart.p, in.p, nc, dg.p,
                                                    up_.p, symm ? nullptr : lo_.p, Cdiag.p);
    UNAP_CK(cudaGetLastError());

    out = CoarseHost();
    down(out.restrictAddr, map.p, (size_t)n, s);
    down(out.faceRestrict, fr.p, (size_t)nf, s);
    HostLdu& C = out.A;
    C.n = nc;
    C.nf = nCF;
    C.symm = symm;
    down(C.l, Cl.p, (size_t)nCF, s);
    down(C.u, Cu.p, (size_t)nCF, s);
    down(C.upper, Cup.p, (size_t)nCF, s);
    if (!symm) down(C.lower, Clo.p, (size_t)nCF, s);
    down(C.diag, Cdiag.p, (size_t)nc, s);
    down(cw, Cw.p, (size_t)nCF, s);
    UNAP_CK(cudaStreamSynchronize(s));
    C.validate();
    return true;
}

}  // namespace unapgpu
