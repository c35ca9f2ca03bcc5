// Host-side construction of one device Level (see unap_internal.hpp).
#include <algorithm>
#include <atomic>
#include <cstring>
#include <numeric>

#include "unap_internal.hpp"

namespace unapgpu {

// Coefficient versions are unique across all Levels of the process, so a
// cache keyed by (matrix address, version) cannot match a new matrix that
// happens to reuse a freed one's address.
static std::atomic<int> g_version{0};
static int next_version() { return ++g_version; }

void HostLdu::validate()
{
    oriented = true;
    ownerSorted = true;
    for (int f = 0; f < nf; ++f) {
        if (l[f] < 0 || l[f] >= n || u[f] < 0 || u[f] >= n)
            throw std::invalid_argument("face " + std::to_string(f) + " addresses a cell out of range");
        if (!(l[f] < u[f])) oriented = false;
        if (f && l[f] < l[f - 1]) ownerSorted = false;
    }
}

size_t Level::deviceBytes() const
{
    return d_perm.bytes() + d_iperm.bytes() + d_sliceOff.bytes() + d_rowInfo.bytes() +
           d_col.bytes() + d_val.bytes() + d_valT.bytes() + d_diag.bytes() + d_val32.bytes() +
           d_diag32.bytes();
}

namespace {

// faces grouped by a cell array (counting sort, stable in face order)
void group_faces(int n, int nf, const int* key, std::vector<int>& start, std::vector<int>& list)
{
    start.assign((size_t)n + 1, 0);
    for (int f = 0; f < nf; ++f) start[(size_t)key[f] + 1]++;
    for (int c = 0; c < n; ++c) start[(size_t)c + 1] += start[c];
    list.resize((size_t)nf);
    std::vector<int> pos(start.begin(), start.end() - 1);
    for (int f = 0; f < nf; ++f) list[(size_t)pos[(size_t)key[f]]++] = f;
}

// BFS visit rank of every cell (components started in index order)
std::vector<int> bfs_rank(int n, const std::vector<int>& loStart, const std::vector<int>& loList,
                          const std::vector<int>& ownStart, const std::vector<int>& ownList,
                          const int* l, const int* u)
{
    std::vector<int> rank((size_t)n, -1);
    std::vector<int> queue((size_t)n);
    int head = 0, tail = 0, next = 0;
    for (int seed = 0; seed < n; ++seed) {
        if (rank[(size_t)seed] >= 0) continue;
        rank[(size_t)seed] = next++;
        queue[(size_t)tail++] = seed;
        while (head < tail) {
            int c = queue[(size_t)head++];
            for (int k = loStart[(size_t)c]; k < loStart[(size_t)c + 1]; ++k) {
                int o = l[loList[(size_t)k]];
                if (rank[(size_t)o] < 0) {
                    rank[(size_t)o] = next++;
                    queue[(size_t)tail++] = o;
                }
            }
            for (int k = ownStart[(size_t)c]; k < ownStart[(size_t)c + 1]; ++k) {
                int o = u[ownList[(size_t)k]];
                if (rank[(size_t)o] < 0) {
                    rank[(size_t)o] = next++;
                    queue[(size_t)tail++] = o;
                }
            }
        }
    }
    return rank;
}

}  // namespace

std::unique_ptr<Level> build_level(const HostLdu& A, const std::vector<int>* key,
                                   bool identityOrder, cudaStream_t s, bool wavefronts)
{
    const long long minCells = device_setup_min_cells();
    if (!identityOrder && A.oriented && A.ownerSorted && minCells >= 0 && A.n > 0 &&
        A.n >= minCells) {
        if (auto D = build_level_device(A, key, s, wavefronts)) {
            D->version = next_version();
            return D;
        }
    }
    auto L = std::make_unique<Level>();
    L->version = next_version();
    const int n = A.n, nf = A.nf;
    L->n = n;
    L->nf = nf;
    L->symm = A.symm;
    L->sweepable = A.oriented && A.ownerSorted && (wavefronts || identityOrder);
    const int* l = A.l.data();
    const int* u = A.u.data();

    std::vector<int> loStart, loList, ownStart, ownList;
    group_faces(n, nf, u, loStart, loList);    // faces with upperAddr == c (losort)
    group_faces(n, nf, l, ownStart, ownList);  // faces with lowerAddr == c

    // forward wavefront of every cell: 1 + max over lower neighbours
    std::vector<int> wave((size_t)n, 0);
    int nWave = 1;
    if (L->sweepable && !identityOrder && wavefronts) {
        for (int c = 0; c < n; ++c) {
            int w = 0;
            for (int k = loStart[(size_t)c]; k < loStart[(size_t)c + 1]; ++k) {
                int o = l[loList[(size_t)k]];
                w = std::max(w, wave[(size_t)o] + 1);
            }
            wave[(size_t)c] = w;
            nWave = std::max(nWave, w + 1);
        }
    } else if (L->sweepable && identityOrder) {
        // identity order keeps one cell per wavefront position only when the
        // sweep needs it; a dense coarsest level is never swept, so a single
        // range with sequential semantics is not required here.
        nWave = 1;
    }
    if (n == 0) nWave = 0;

    // internal order: wavefront-major, locality key inside a wavefront
    L->perm.resize((size_t)n);
    L->iperm.resize((size_t)n);
    L->locRank.resize((size_t)n);
    if (identityOrder) {
        std::iota(L->perm.begin(), L->perm.end(), 0);
        std::iota(L->locRank.begin(), L->locRank.end(), 0);
        L->waveStart = {0, n};
        L->nWave = n ? 1 : 0;
    } else {
        std::vector<int> rank;
        if (key && (int)key->size() == n)
            rank = *key;
        else
            rank = bfs_rank(n, loStart, loList, ownStart, ownList, l, u);
        // cells in key order (keys may repeat: stable on cell index), by a
        // counting sort over the key range
        int maxKey = 0;
        for (int c = 0; c < n; ++c) {
            if (rank[(size_t)c] < 0) throw std::invalid_argument("negative locality key");
            maxKey = std::max(maxKey, rank[(size_t)c]);
        }
        std::vector<int> byKey((size_t)n);
        {
            std::vector<int> cnt((size_t)maxKey + 2, 0);
            for (int c = 0; c < n; ++c) cnt[(size_t)rank[(size_t)c] + 1]++;
            for (int k = 0; k <= maxKey; ++k) cnt[(size_t)k + 1] += cnt[(size_t)k];
            for (int c = 0; c < n; ++c) byKey[(size_t)cnt[(size_t)rank[(size_t)c]]++] = c;
        }
        for (int i = 0; i < n; ++i) L->locRank[(size_t)byKey[(size_t)i]] = i;
        L->waveStart.assign((size_t)nWave + 1, 0);
        for (int c = 0; c < n; ++c) L->waveStart[(size_t)wave[(size_t)c] + 1]++;
        for (int w = 0; w < nWave; ++w) L->waveStart[(size_t)w + 1] += L->waveStart[(size_t)w];
        std::vector<int> pos(L->waveStart.begin(), L->waveStart.end() - 1);
        for (int c : byKey) L->perm[(size_t)pos[(size_t)wave[(size_t)c]]++] = c;
        L->nWave = nWave;
        if (!wavefronts) {
            // rows of similar length share SELL-32 slices: inside every
            // window of 256 rows, decreasing row length (stable)
            auto deg = [&](int c) {
                return loStart[(size_t)c + 1] - loStart[(size_t)c] + ownStart[(size_t)c + 1] -
                       ownStart[(size_t)c];
            };
            for (int w0 = 0; w0 < n; w0 += 256) {
                const int w1 = std::min(n, w0 + 256);
                std::stable_sort(L->perm.begin() + w0, L->perm.begin() + w1,
                                 [&](int a, int b) { return deg(a) > deg(b); });
            }
        }
    }
    for (int i = 0; i < n; ++i) L->iperm[(size_t)L->perm[(size_t)i]] = i;

    // SELL-32 layout; a row's entries are its faces in ascending face order
    L->nSlices = div_up(n, 32);
    std::vector<int> rowLen((size_t)n), rowLow((size_t)n);
    for (int i = 0; i < n; ++i) {
        int c = L->perm[(size_t)i];
        rowLow[(size_t)i] = loStart[(size_t)c + 1] - loStart[(size_t)c];
        rowLen[(size_t)i] = rowLow[(size_t)i] + ownStart[(size_t)c + 1] - ownStart[(size_t)c];
        if (rowLen[(size_t)i] > 0xffff) throw std::invalid_argument("row with more than 65535 faces");
    }
    std::vector<int> sliceOff((size_t)L->nSlices + 1, 0);
    long long total = 0;
    int maxLen = 0;
    for (int sl = 0; sl < L->nSlices; ++sl) {
        int w = 0;
        for (int r = sl * 32; r < std::min(n, sl * 32 + 32); ++r) w = std::max(w, rowLen[(size_t)r]);
        maxLen = std::max(maxLen, w);
        sliceOff[(size_t)sl] = (int)total;
        total += 32LL * w;
        if (total > 0x7fffffffLL) throw std::invalid_argument("matrix too large for int32 SELL offsets");
    }
    sliceOff[(size_t)L->nSlices] = (int)total;
    L->nEntries = total;
    L->maxRowLen = maxLen;

    std::vector<int> col((size_t)total), rowInfo((size_t)n);
    L->entLo.assign((size_t)nf, -1);
    L->entUp.assign((size_t)nf, -1);
    for (int i = 0; i < n; ++i) {
        int c = L->perm[(size_t)i];
        long long base = sliceOff[(size_t)(i >> 5)] + (i & 31);
        int a = loStart[(size_t)c], ae = loStart[(size_t)c + 1];
        int b = ownStart[(size_t)c], be = ownStart[(size_t)c + 1];
        int j = 0;
        // merge the two face lists by face index (for owner-sorted matrices
        // every lower-side face precedes every upper-side face)
        while (a < ae || b < be) {
            bool takeLow;
            if (a >= ae)
                takeLow = false;
            else if (b >= be)
                takeLow = true;
            else
                takeLow = loList[(size_t)a] < ownList[(size_t)b];
            long long e = base + 32LL * j;
            if (takeLow) {
                int f = loList[(size_t)a++];
                col[(size_t)e] = L->iperm[(size_t)l[f]];
                L->entLo[(size_t)f] = (int)e;
            } else {
                int f = ownList[(size_t)b++];
                col[(size_t)e] = L->iperm[(size_t)u[f]];
                L->entUp[(size_t)f] = (int)e;
            }
            ++j;
        }
        rowInfo[(size_t)i] = rowLen[(size_t)i] | (rowLow[(size_t)i] << 16);
    }
    // padding entries point at the row itself with zero value
    for (int sl = 0; sl < L->nSlices; ++sl) {
        int w = (sliceOff[(size_t)sl + 1] - sliceOff[(size_t)sl]) / 32;
        for (int r = sl * 32; r < sl * 32 + 32; ++r) {
            int len = r < n ? rowLen[(size_t)r] : 0;
            for (int j = len; j < w; ++j)
                col[(size_t)sliceOff[(size_t)sl] + 32 * j + (r & 31)] = r < n ? r : 0;
        }
    }
    L->d_perm.upload(L->perm, s);
    L->d_iperm.upload(L->iperm, s);
    L->d_sliceOff.upload(sliceOff, s);
    L->d_rowInfo.upload(rowInfo, s);
    L->d_col.upload(col, s);
    UNAP_CK(cudaStreamSynchronize(s));  // host vectors die here
    update_level_values(*L, A, s);
    return L;
}

void update_level_values(Level& L, const HostLdu& A, cudaStream_t s)
{
    if (A.n != L.n || A.nf != L.nf) throw std::invalid_argument("coefficient update changes the size");
    const double* lower = A.lowerPtr();
    const double* upper = A.upper.data();
    std::vector<double> val((size_t)L.nEntries, 0.0), valT;
    if (!A.symm) valT.assign((size_t)L.nEntries, 0.0);
    for (int f = 0; f < A.nf; ++f) {
        // row u (lower side) holds lower[f]; row l (upper side) holds upper[f]
        val[(size_t)L.entLo[(size_t)f]] = lower[f];
        val[(size_t)L.entUp[(size_t)f]] = upper[f];
        if (!A.symm) {
            valT[(size_t)L.entLo[(size_t)f]] = upper[f];
            valT[(size_t)L.entUp[(size_t)f]] = lower[f];
        }
    }
    std::vector<double> diag((size_t)L.n);
    for (int i = 0; i < L.n; ++i) diag[(size_t)i] = A.diag[(size_t)L.perm[(size_t)i]];
    L.symm = A.symm;
    L.d_val.upload(val, s);
    if (!A.symm)
        L.d_valT.upload(valT, s);
    else
        L.d_valT.release();
    L.d_diag.upload(diag, s);
    L.d_val32.release();
    L.d_diag32.release();
    L.version = next_version();
    UNAP_CK(cudaStreamSynchronize(s));
}

}  // namespace unapgpu
