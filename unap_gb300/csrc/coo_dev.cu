// Device form of the COO/CSR ingest: reorderCOO
// (tools/matrixConversion/matrixConversion.cpp:38-98) followed by coo2ldu
// (tools/matrixConversion/coo2ldu.cpp:3-113), giving the same LDU arrays as
// the host form in capi.cpp (coo_to_ldu) bit for bit.
//
//   1. 1-based -> 0-based (the Fortran entry points), range and row-order
//      checks, row counts and offsets (CSR: the row pointer expanded);
//   2. each entry's place in its row = its row's start plus the number of
//      the row's entries with a smaller column (reorderCOO's posInRow);
//   3. upper faces are the (row < col) entries in row-major order (an
//      exclusive scan of that flag numbers them); the diagonal is scattered;
//   4. asymmetric values: the (row > col) entries are bucketed by column in
//      row-major order (atomic fill, then each bucket sorted by position),
//      and the k-th one of column o becomes lower[first face of owner o + k]
//      (sortData, matrixConversion.cpp:4-35).
// Malformed input the reference leaves undefined is an error here: rows
// out of order, repeated (row, col) pairs, per-column counts of lower
// entries that differ from the upper ones (not structurally symmetric).
#include <algorithm>

#include "unap_internal.hpp"

namespace unapgpu {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBucket = 1024;

int grid_for(long long n)
{
    long long b = (n + kThreads - 1) / kThreads;
    return (int)std::max(1LL, std::min(b, 1LL << 30));
}

template <class T>
using Scratch = StreamScratch<T>;

// error bits
constexpr int kBadRange = 1, kBadOrder = 2, kBadDup = 4, kBadSym = 8, kBadBucket = 16,
              kBadPtr = 32;

// CSR row pointer -> row of every entry
__global__ void k_expand_rows(const int* __restrict__ ptr, int n, int size, int* rows, int* bad)
{
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
         r += (long long)gridDim.x * blockDim.x) {
        const int a = ptr[r], e = ptr[r + 1];
        if (a < 0 || e < a || e > size || (r == 0 && a != 0) || (r == n - 1 && e != size)) {
            atomicOr(bad, kBadPtr);
            continue;
        }
        for (int j = a; j < e; ++j) rows[j] = (int)r;
    }
}

__global__ void k_coo_prepare(const int* __restrict__ rowsIn, const int* __restrict__ colsIn,
                              int base, int n, int size, int* rows, int* cols, int* cnt, int* bad)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < size;
         i += (long long)gridDim.x * blockDim.x) {
        const int r = rowsIn[i] - base, c = colsIn[i] - base;
        rows[i] = r;
        cols[i] = c;
        if (r < 0 || r >= n || c < 0 || c >= n) {
            atomicOr(bad, kBadRange);
            continue;
        }
        if (i && rowsIn[i - 1] - base > r) atomicOr(bad, kBadOrder);
        atomicAdd(&cnt[r], 1);
    }
}

// sorted position of every entry within its row (posInRow)
__global__ void k_coo_sort(const int* __restrict__ rows, const int* __restrict__ cols,
                           const double* __restrict__ vals, int size, const int* __restrict__ off,
                           int* scol, double* sval)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < size;
         i += (long long)gridDim.x * blockDim.x) {
        const int r = rows[i], c = cols[i];
        const int a = off[r], e = off[r + 1];
        // entries with a smaller column, and equal ones earlier in the row
        // (a repeated entry then takes the next slot and is reported)
        int pos = a;
        for (int k = a; k < e; ++k) pos += (c > cols[k]) + (k < i && cols[k] == c);
        scol[pos] = c;
        sval[pos] = vals[i];
    }
}

// classify sorted entries; up[p] = 1 for an upper face
__global__ void k_coo_classify(const int* __restrict__ rows, const int* __restrict__ scol,
                               const double* __restrict__ sval, int size, double* diag, int* up,
                               int* lowCnt, int* bad)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < size;
         p += (long long)gridDim.x * blockDim.x) {
        const int r = rows[p], c = scol[p];
        if (p && rows[p - 1] == r && scol[p - 1] >= c) atomicOr(bad, kBadDup);
        up[p] = c > r;
        if (c == r) diag[r] = sval[p];
        if (lowCnt && c < r) atomicAdd(&lowCnt[c], 1);
    }
}

__global__ void k_coo_faces(const int* __restrict__ rows, const int* __restrict__ scol,
                            const double* __restrict__ sval, int size, const int* __restrict__ fidx,
                            int* l, int* u, double* upper)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < size;
         p += (long long)gridDim.x * blockDim.x) {
        if (fidx[p + 1] == fidx[p]) continue;  // not an upper entry
        const int f = fidx[p];
        l[f] = rows[p];
        u[f] = scol[p];
        upper[f] = sval[p];
    }
}

// first face of every owner o = upper entries before row o's first entry;
// lower entries of column o must number as many as o's upper faces
__global__ void k_owner_start(const int* __restrict__ off, const int* __restrict__ fidx, int n,
                              const int* __restrict__ lowCnt, int* faceStart, int* bad)
{
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o <= n;
         o += (long long)gridDim.x * blockDim.x) {
        faceStart[o] = fidx[off[o]];
        if (o < n && lowCnt) {
            const int nUp = fidx[off[o + 1]] - fidx[off[o]];
            if (lowCnt[o] != nUp) atomicOr(bad, kBadSym);
            if (lowCnt[o] > kMaxBucket) atomicOr(bad, kBadBucket);
        }
    }
}

__global__ void k_lower_fill(const int* __restrict__ rows, const int* __restrict__ scol, int size,
                             int* cursor, int* bucket)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < size;
         p += (long long)gridDim.x * blockDim.x) {
        const int r = rows[p], c = scol[p];
        if (c < r) bucket[atomicAdd(&cursor[c], 1)] = (int)p;
    }
}

// each owner's lower entries in row-major order, then their values
__global__ void k_lower_place(const int* __restrict__ faceStart, int n, int* bucket,
                              const double* __restrict__ sval, double* lower)
{
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < n;
         o += (long long)gridDim.x * blockDim.x) {
        const int a = faceStart[o], e = faceStart[o + 1];
        for (int i = a + 1; i < e; ++i) {
            const int v = bucket[i];
            int j = i - 1;
            while (j >= a && bucket[j] > v) {
                bucket[j + 1] = bucket[j];
                --j;
            }
            bucket[j + 1] = v;
        }
        for (int i = a; i < e; ++i) lower[i] = sval[bucket[i]];
    }
}

}  // namespace

// rowsOrPtr: 1-based rows (csr == false) or a 0-based row pointer of n + 1
// entries (csr == true, columns 0-based as the reference's csr2ldu takes
// them).  Returns false (nothing done) when the device form declines: a
// column with more than kMaxBucket lower entries.
bool coo_to_ldu_device(const double* val, const int* rowsOrPtr, const int* colsIn, int n, int size,
                       bool symm, bool csr, cudaStream_t s, HostLdu& out)
{
    if (n <= 0 || size < 0) throw std::invalid_argument("bad COO sizes");
    const int base = csr ? 0 : 1;
    Scratch<int> rowsIn(csr ? 0 : (size_t)size, s), ptr(csr ? (size_t)n + 1 : 0, s);
    Scratch<int> colsRaw((size_t)size, s), rows((size_t)size, s), cols((size_t)size, s);
    Scratch<double> vals((size_t)size, s);
    Scratch<int> cnt((size_t)n + 1, s), bad(1, s);
    UNAP_CK(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
    UNAP_CK(cudaMemsetAsync(cnt.p, 0, sizeof(int) * ((size_t)n + 1), s));
    if (size) {
        UNAP_CK(cudaMemcpyAsync(colsRaw.p, colsIn, sizeof(int) * (size_t)size, cudaMemcpyHostToDevice, s));
        UNAP_CK(cudaMemcpyAsync(vals.p, val, sizeof(double) * (size_t)size, cudaMemcpyHostToDevice, s));
    }
    const int* rowsSrc;
    Scratch<int> expanded(csr ? (size_t)size : 0, s);
    if (csr) {
        UNAP_CK(cudaMemcpyAsync(ptr.p, rowsOrPtr, sizeof(int) * ((size_t)n + 1), cudaMemcpyHostToDevice, s));
        k_expand_rows<<<grid_for(n), kThreads, 0, s>>>(ptr.p, n, size, expanded.p, bad.p);
        rowsSrc = expanded.p;
    } else {
        if (size)
            UNAP_CK(cudaMemcpyAsync(rowsIn.p, rowsOrPtr, sizeof(int) * (size_t)size, cudaMemcpyHostToDevice, s));
        rowsSrc = rowsIn.p;
    }
    int hbad = 0;
    if (csr) {  // the expansion must be valid before rows are read
        UNAP_CK(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        UNAP_CK(cudaStreamSynchronize(s));
        if (hbad) throw std::invalid_argument("CSR row pointer is not a valid partition of the entries");
    }
    if (size)
        k_coo_prepare<<<grid_for(size), kThreads, 0, s>>>(rowsSrc, colsRaw.p, base, n, size, rows.p,
                                                         cols.p, cnt.p, bad.p);
    UNAP_CK(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    UNAP_CK(cudaStreamSynchronize(s));
    if (hbad & kBadRange) throw std::invalid_argument("COO entry out of range");
    if (hbad & kBadOrder)
        throw std::invalid_argument("COO entries must be grouped by row in ascending row order");
    Scratch<int> off((size_t)n + 1, s);
    device_exclusive_scan(cnt.p, off.p, n, s);

    Scratch<int> scol((size_t)size, s), up((size_t)size + 1, s), fidx((size_t)size + 1, s);
    Scratch<double> sval((size_t)size, s), diag((size_t)n, s);
    Scratch<int> lowCnt(symm ? 0 : (size_t)n, s);
    UNAP_CK(cudaMemsetAsync(diag.p, 0, sizeof(double) * (size_t)n, s));
    if (!symm) UNAP_CK(cudaMemsetAsync(lowCnt.p, 0, sizeof(int) * (size_t)n, s));
    if (size) {
        k_coo_sort<<<grid_for(size), kThreads, 0, s>>>(rows.p, cols.p, vals.p, size, off.p, scol.p, sval.p);
        k_coo_classify<<<grid_for(size), kThreads, 0, s>>>(rows.p, scol.p, sval.p, size, diag.p, up.p,
                                                          symm ? nullptr : lowCnt.p, bad.p);
    }
    device_exclusive_scan(up.p, fidx.p, size, s);
    int nf = 0;
    UNAP_CK(cudaMemcpyAsync(&nf, fidx.p + size, sizeof(int), cudaMemcpyDeviceToHost, s));
    UNAP_CK(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    UNAP_CK(cudaStreamSynchronize(s));
    if (hbad & kBadDup) throw std::invalid_argument("COO matrix repeats an entry");
    if (nf != (size - n) / 2) throw std::invalid_argument("COO matrix is not structurally symmetric");

    Scratch<int> l((size_t)nf, s), u((size_t)nf, s), faceStart((size_t)n + 1, s);
    Scratch<double> upper((size_t)nf, s), lower(symm ? 0 : (size_t)nf, s);
    if (size)
        k_coo_faces<<<grid_for(size), kThreads, 0, s>>>(rows.p, scol.p, sval.p, size, fidx.p, l.p, u.p,
                                                       upper.p);
    k_owner_start<<<grid_for((long long)n + 1), kThreads, 0, s>>>(off.p, fidx.p, n,
                                                                 symm ? nullptr : lowCnt.p,
                                                                 faceStart.p, bad.p);
    if (!symm) {
        UNAP_CK(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        UNAP_CK(cudaStreamSynchronize(s));
        if (hbad & kBadSym) throw std::invalid_argument("COO matrix is not structurally symmetric");
        if (hbad & kBadBucket) return false;
        Scratch<int> cursor((size_t)n, s), bucket((size_t)nf, s);
        UNAP_CK(cudaMemcpyAsync(cursor.p, faceStart.p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s));
        if (size) k_lower_fill<<<grid_for(size), kThreads, 0, s>>>(rows.p, scol.p, size, cursor.p, bucket.p);
        k_lower_place<<<grid_for(n), kThreads, 0, s>>>(faceStart.p, n, bucket.p, sval.p, lower.p);
    }
    UNAP_CK(cudaGetLastError());

    out = HostLdu();
    out.n = n;
    out.nf = nf;
    out.symm = symm;
    out.l.resize((size_t)nf);
    out.u.resize((size_t)nf);
    out.upper.resize((size_t)nf);
    out.diag.resize((size_t)n);
    if (nf) {
        UNAP_CK(cudaMemcpyAsync(out.l.data(), l.p, sizeof(int) * (size_t)nf, cudaMemcpyDeviceToHost, s));
        UNAP_CK(cudaMemcpyAsync(out.u.data(), u.p, sizeof(int) * (size_t)nf, cudaMemcpyDeviceToHost, s));
        UNAP_CK(cudaMemcpyAsync(out.upper.data(), upper.p, sizeof(double) * (size_t)nf,
                                cudaMemcpyDeviceToHost, s));
    }
    UNAP_CK(cudaMemcpyAsync(out.diag.data(), diag.p, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, s));
    if (!symm) {
        out.lower.resize((size_t)nf);
        if (nf)
            UNAP_CK(cudaMemcpyAsync(out.lower.data(), lower.p, sizeof(double) * (size_t)nf,
                                    cudaMemcpyDeviceToHost, s));
    }
    UNAP_CK(cudaStreamSynchronize(s));
    return true;
}

}  // namespace unapgpu
