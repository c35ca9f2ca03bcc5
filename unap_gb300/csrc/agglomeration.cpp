// Host-side pairwise agglomeration of an LDU matrix into a coarse hierarchy.
//
// The matching is the reference's sequential greedy algorithm, kept exact so
// the hierarchy (restrict maps, coarse addressing, coarse coefficients) is
// bit-identical to lduAgglomeration's:
//   pairwise pass        lduAgglomerate.cpp:94-271
//   coarse addressing    lduAgglomerationAddressing.cpp:8-178
//   coarse coefficients  lduAgglomerateMatrix.cpp:3-104
//   level loop           lduAgglomerate.cpp:4-91, lduAgglomeration.cpp:26-43
// Storage is flat (per-cell segments sized by a counting pass) so a 16.7M-cell
// level agglomerates in a few hundred milliseconds.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <thread>

#include "amg.hpp"

namespace unapgpu {

static constexpr double kSmall = 1.0e-37;  // SMALL, src/base/unap.hpp:88

namespace {

// f(begin, end) over [0, n) split across host threads (at least minPer
// items each)
template <class F>
void parallel_ranges(int n, int minPer, F&& f)
{
    unsigned hw = std::thread::hardware_concurrency();
    int nt = (int)std::min<long long>({(long long)(hw ? hw : 1), 32LL, (long long)n / minPer});
    if (nt <= 1) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    th.reserve((size_t)nt);
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            f((int)((long long)n * t / nt), (int)((long long)n * (t + 1) / nt));
        });
    for (auto& x : th) x.join();
}

}  // namespace

std::vector<int> pairwise_pass(const HostLdu& A, const std::vector<double>& w, int& nCoarse)
{
    const int n = A.n, nf = A.nf;
    const int* l = A.l.data();
    const int* u = A.u.data();
    // faces of every cell: those where it is the neighbour, then those where
    // it is the owner, each in face order (lduAgglomerate.cpp:23-71)
    std::vector<int> off((size_t)n + 1, 0);
    for (int f = 0; f < nf; ++f) {
        off[(size_t)u[f] + 1]++;
        off[(size_t)l[f] + 1]++;
    }
    for (int c = 0; c < n; ++c) off[(size_t)c + 1] += off[(size_t)c];
    std::vector<int> cellFaces((size_t)2 * nf);
    {
        std::vector<int> pos(off.begin(), off.end() - 1);
        for (int f = 0; f < nf; ++f) cellFaces[(size_t)pos[(size_t)u[f]]++] = f;
        for (int f = 0; f < nf; ++f) cellFaces[(size_t)pos[(size_t)l[f]]++] = f;
    }
    std::vector<int> map((size_t)n, -1);
    int nc = 0;
    for (int c = 0; c < n; ++c) {
        if (map[(size_t)c] >= 0) continue;
        int match = -1;
        double maxW = kSmall;
        for (int k = off[(size_t)c]; k < off[(size_t)c + 1]; ++k) {
            int f = cellFaces[(size_t)k];
            if (map[(size_t)u[f]] < 0 && map[(size_t)l[f]] < 0 && w[(size_t)f] > maxW) {
                match = f;
                maxW = w[(size_t)f];
            }
        }
        if (match >= 0) {
            map[(size_t)u[match]] = nc;
            map[(size_t)l[match]] = nc;
            ++nc;
            continue;
        }
        // no free neighbour: join the cluster across the heaviest face
        int cmatch = -1;
        double cmax = kSmall;
        for (int k = off[(size_t)c]; k < off[(size_t)c + 1]; ++k) {
            int f = cellFaces[(size_t)k];
            if (w[(size_t)f] > cmax) {
                cmatch = f;
                cmax = w[(size_t)f];
            }
        }
        if (cmatch >= 0) map[(size_t)c] = std::max(map[(size_t)u[cmatch]], map[(size_t)l[cmatch]]);
    }
    for (int c = 0; c < n; ++c)
        if (map[(size_t)c] < 0) map[(size_t)c] = nc++;
    nCoarse = nc;
    return map;
}

// Coarse faces are numbered by coarse owner, then by the order in which
// each owner's fine boundary faces (in fine face order) first meet a
// neighbour -- the reference's numbering.  Owners are independent, so after
// two serial counting passes the owners are split over host threads.
void coarse_addressing(const HostLdu& fine, const std::vector<int>& map, int nCoarse,
                       CoarseHost& out)
{
    const int nf = fine.nf;
    const int* l = fine.l.data();
    const int* u = fine.u.data();
    const int* mp = map.data();
    out.faceRestrict.assign((size_t)nf, 0);
    // coarse owner of every fine boundary face (-1: inside an aggregate)
    std::vector<int> own((size_t)nf);
    parallel_ranges(nf, 65536, [&](int f0, int f1) {
        for (int f = f0; f < f1; ++f) {
            int a = mp[u[f]], b = mp[l[f]];
            own[(size_t)f] = a != b ? std::min(a, b) : -1;
            if (a == b) out.faceRestrict[(size_t)f] = -(a + 1);
        }
    });
    // fine boundary faces of every coarse owner, in fine face order
    std::vector<int> segStart((size_t)nCoarse + 1, 0);
    for (int f = 0; f < nf; ++f)
        if (own[(size_t)f] >= 0) segStart[(size_t)own[(size_t)f] + 1]++;
    for (int c = 0; c < nCoarse; ++c) segStart[(size_t)c + 1] += segStart[(size_t)c];
    const size_t total = (size_t)segStart[(size_t)nCoarse];
    std::vector<int> segFace(total);
    {
        std::vector<int> pos(segStart.begin(), segStart.end() - 1);
        for (int f = 0; f < nf; ++f)
            if (own[(size_t)f] >= 0) segFace[(size_t)pos[(size_t)own[(size_t)f]]++] = f;
    }
    // per owner: distinct neighbours in discovery order, each boundary
    // face's index among them
    std::vector<int> nei(total), local(total), cnt((size_t)nCoarse, 0);
    parallel_ranges(nCoarse, 4096, [&](int c0, int c1) {
        for (int c = c0; c < c1; ++c) {
            const size_t a = (size_t)segStart[(size_t)c], e = (size_t)segStart[(size_t)c + 1];
            int m = 0;
            for (size_t i = a; i < e; ++i) {
                const int f = segFace[i];
                const int ne = std::max(mp[u[f]], mp[l[f]]);
                int j = 0;
                while (j < m && nei[a + (size_t)j] != ne) ++j;
                if (j == m) nei[a + (size_t)m++] = ne;
                local[i] = j;
            }
            cnt[(size_t)c] = m;
        }
    });
    std::vector<int> cfStart((size_t)nCoarse + 1, 0);
    for (int c = 0; c < nCoarse; ++c) cfStart[(size_t)c + 1] = cfStart[(size_t)c] + cnt[(size_t)c];
    const int nCF = cfStart[(size_t)nCoarse];
    out.A.n = nCoarse;
    out.A.nf = nCF;
    out.A.l.resize((size_t)nCF);
    out.A.u.resize((size_t)nCF);
    parallel_ranges(nCoarse, 4096, [&](int c0, int c1) {
        for (int c = c0; c < c1; ++c) {
            const size_t a = (size_t)segStart[(size_t)c];
            const int k0 = cfStart[(size_t)c];
            for (int j = 0; j < cnt[(size_t)c]; ++j) {
                out.A.l[(size_t)(k0 + j)] = c;
                out.A.u[(size_t)(k0 + j)] = nei[a + (size_t)j];
            }
            for (size_t i = a; i < (size_t)segStart[(size_t)c + 1]; ++i)
                out.faceRestrict[(size_t)segFace[i]] = k0 + local[i];
        }
    });
    out.restrictAddr = map;
}

void coarse_coefficients(const HostLdu& fine, CoarseHost& c)
{
    HostLdu& C = c.A;
    C.symm = fine.symm;
    C.diag.assign((size_t)C.n, 0.0);
    C.upper.assign((size_t)C.nf, 0.0);
    // restrictField of the diagonal (unapMatrix.hpp:378-407)
    for (int i = 0; i < fine.n; ++i) C.diag[(size_t)c.restrictAddr[(size_t)i]] += fine.diag[(size_t)i];
    const int* fr = c.faceRestrict.data();
    if (fine.symm) {
        C.lower.clear();
        for (int f = 0; f < fine.nf; ++f) {
            int cf = fr[f];
            if (cf >= 0)
                C.upper[(size_t)cf] += fine.upper[(size_t)f];
            else
                C.diag[(size_t)(-1 - cf)] += 2 * fine.upper[(size_t)f];
        }
    } else {
        C.lower.assign((size_t)C.nf, 0.0);
        for (int f = 0; f < fine.nf; ++f) {
            int cf = fr[f];
            if (cf >= 0) {
                int cl = c.restrictAddr[(size_t)fine.l[(size_t)f]];
                if (C.l[(size_t)cf] == cl) {
                    C.upper[(size_t)cf] += fine.upper[(size_t)f];
                    C.lower[(size_t)cf] += fine.lower[(size_t)f];
                } else if (C.u[(size_t)cf] == cl) {
                    C.upper[(size_t)cf] += fine.lower[(size_t)f];
                    C.lower[(size_t)cf] += fine.upper[(size_t)f];
                } else {
                    throw std::runtime_error("inconsistent addressing between fine and coarse grids");
                }
            } else {
                C.diag[(size_t)(-1 - cf)] += fine.upper[(size_t)f] + fine.lower[(size_t)f];
            }
        }
    }
    C.validate();
}

std::vector<CoarseHost> agglomerate_levels(const HostLdu& fine, const std::vector<double>& weights,
                                           int nCoarsest, int maxLevels, int stopRule,
                                           cudaStream_t s)
{
    if (maxLevels <= 0) maxLevels = 50;
    if (nCoarsest <= 0) nCoarsest = 50;
    std::vector<CoarseHost> levels;
    std::vector<double> w = weights;
    while ((int)levels.size() < maxLevels - 1) {
        const HostLdu& fm = levels.empty() ? fine : levels.back().A;
        if (stopRule == 1 && fm.n <= nCoarsest) break;
        const long long minCells = device_setup_min_cells();
        if (minCells >= 0 && fm.n >= minCells) {
            CoarseHost c;
            std::vector<double> cw;
            int nc = -1;
            if (agglomerate_level_device(fm, w, c, cw, nc, s)) {
                bool keep = stopRule == 1 ? (nc < fm.n) : (nc >= nCoarsest);
                if (!keep) break;
                w.swap(cw);
                levels.push_back(std::move(c));
                continue;
            }
        }
        int nc = -1;
        std::vector<int> map = pairwise_pass(fm, w, nc);
        bool keep = stopRule == 1 ? (nc < fm.n) : (nc >= nCoarsest);
        if (!keep) break;
        CoarseHost c;
        coarse_addressing(fm, map, nc, c);
        coarse_coefficients(fm, c);
        // restrictFaceField of the weights (unapMatrix.hpp:441-475)
        std::vector<double> cw((size_t)c.A.nf, 0.0);
        for (int f = 0; f < fm.nf; ++f)
            if (c.faceRestrict[(size_t)f] >= 0) cw[(size_t)c.faceRestrict[(size_t)f]] += w[(size_t)f];
        w.swap(cw);
        levels.push_back(std::move(c));
    }
    return levels;
}

std::vector<double> mg_face_weights(const HostLdu& A)
{
    // fortranInterface.cpp:383-395: |upper| / sqrt(sum upper^2)
    double s = 0.0;
    for (int f = 0; f < A.nf; ++f) s += A.upper[(size_t)f] * A.upper[(size_t)f];
    double avg = std::sqrt(s);
    std::vector<double> w((size_t)A.nf);
    for (int f = 0; f < A.nf; ++f) w[(size_t)f] = std::fabs(A.upper[(size_t)f]) / avg;
    return w;
}

}  // namespace unapgpu
