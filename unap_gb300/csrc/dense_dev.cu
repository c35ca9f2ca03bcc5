// Dense SPD inverse of the AMG coarsest level on the device, bit-identical
// to the host form (dense_spd_inverse in engine.cu) and to the oracle's:
// every element is the same sum in the same ascending-k order with separate
// multiplies and adds (the library is built with --fmad=false), and every
// division and square root is IEEE-rounded on both sides.
//
//   1. Cholesky A = L L^T, right-looking: step k subtracts L[i][k] L[j][k]
//      from the trailing lower triangle, which is the host's left-looking
//      sum A[i][j] - sum_k L[i][k] L[j][k] term by term in the same order;
//      the threads that update column k + 1 also finish it (its diagonal
//      and the division by it), so one launch per column.
//   2. Li = L^-1 row by row, right-looking in the same way: step k adds
//      L[i][k] Li[k][j] to the accumulator of every later row; the threads of
//      row k + 1 then finish that row (-t / L[k+1][k+1]).
//   3. inv = Li^T Li, one independent ascending-k dot product per element,
//      scattered into the column-major array the V-cycle reads (rows in
//      internal order, columns in cell order).
// The factorization is n dependent steps of shrinking rank-1 updates (n^3/6
// multiply-adds each for steps 1-3, FP64), so for the coarsest sizes used
// (hundreds to a few thousand cells) it is launch- and FP64-bound; it moves
// the O(n^3) work off the host, which matters when many solves set up at
// once.
#include "unap_internal.hpp"

namespace unapgpu {

namespace {

constexpr int kTx = 32, kTy = 8;

// step k of the Cholesky: W[i][j] -= L[i][k] L[j][k] for k + 1 < j <= i.
// Column k + 1 is then complete: its threads finish it instead of writing W
// (nobody reads that column of W again), each recomputing the diagonal from
// the unchanged W[k+1][k+1] exactly as the diagonal's own thread does.  W
// and L are row-major n x n.
__global__ void k_chol_step(int n, int k, double* __restrict__ W, double* __restrict__ L,
                            int* bad)
{
    const int j = k + 1 + blockIdx.x * kTx + threadIdx.x;
    const int i = k + 1 + blockIdx.y * kTy + threadIdx.y;
    if (i >= n || j > i) return;
    const double lik = L[(size_t)i * n + k], ljk = L[(size_t)j * n + k];
    const double w = W[(size_t)i * n + j] - lik * ljk;
    if (j != k + 1) {
        W[(size_t)i * n + j] = w;
        return;
    }
    const double s = i == j ? w : W[(size_t)j * n + j] - ljk * ljk;
    if (!(s > 0.0)) {
        if (i == j) atomicOr(bad, 1);
        return;
    }
    const double d = sqrt(s);
    L[(size_t)i * n + j] = i == j ? d : w / d;
}

// column 0 of the Cholesky
__global__ void k_chol_first(int n, const double* __restrict__ W, double* __restrict__ L, int* bad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double s = W[0];
    if (!(s > 0.0)) {
        if (i == 0) atomicOr(bad, 1);
        return;
    }
    const double d = sqrt(s);
    L[(size_t)i * n] = i == 0 ? d : W[(size_t)i * n] / d;
}

// step k of L^-1: T[i][j] += L[i][k] Li[k][j] for i > k, j <= k; the
// threads of row k + 1 then finish it.  Li and T are row-major.
__global__ void k_linv_step(int n, int k, const double* __restrict__ L, double* __restrict__ Li,
                            double* __restrict__ T)
{
    const int j = blockIdx.x * kTx + threadIdx.x;
    const int i = k + 1 + blockIdx.y * kTy + threadIdx.y;
    if (i >= n || j > k) return;
    const double t = T[(size_t)i * n + j] + L[(size_t)i * n + k] * Li[(size_t)k * n + j];
    T[(size_t)i * n + j] = t;
    if (i == k + 1) {
        const double lii = L[(size_t)i * n + i];
        Li[(size_t)i * n + j] = -t / lii;
        if (j == k) Li[(size_t)i * n + i] = 1.0 / lii;
    }
}

__global__ void k_linv_first(int n, const double* __restrict__ L, double* __restrict__ Li)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) Li[0] = 1.0 / L[0];
}

// inv[i][j] = sum_{k=i}^{n-1} Li[k][i] Li[k][j] (j <= i), written column-
// major with rows in internal order and columns in cell order:
// out[b*n + iperm[a]] = inv[a][b], for (a, b) = (i, j) and its mirror.
__global__ void k_inv_product(int n, const double* __restrict__ Li, const int* __restrict__ iperm,
                              double* __restrict__ out)
{
    const int j = blockIdx.x * kTx + threadIdx.x;
    const int i = blockIdx.y * kTy + threadIdx.y;
    if (i >= n || j > i) return;
    double t = 0.0;
    for (int k = i; k < n; ++k) t += Li[(size_t)k * n + i] * Li[(size_t)k * n + j];
    out[(size_t)j * n + (iperm ? iperm[i] : i)] = t;
    out[(size_t)i * n + (iperm ? iperm[j] : j)] = t;
}

}  // namespace

// A: row-major dense n x n SPD matrix (host).  On return `out` (device, n*n)
// holds A^-1 column-major, rows in the internal order given by iperm
// (device, cell -> internal row; null for the identity), columns in cell
// order.
// Returns false when A is not positive definite.
bool dense_spd_inverse_device(int n, const std::vector<double>& A, const int* iperm, double* out,
                              cudaStream_t s)
{
    if (n <= 0) return true;
    const size_t N = (size_t)n;
    DevArray<double> W(N * N), L(N * N), Li(N * N), T(N * N);
    DevArray<int> bad(1);
    W.upload(A, s);
    L.zero(s);
    Li.zero(s);
    T.zero(s);
    bad.zero(s);
    const dim3 blk(kTx, kTy);
    k_chol_first<<<(n + 255) / 256, 256, 0, s>>>(n, W.p, L.p, bad.p);
    for (int k = 0; k + 1 < n; ++k) {
        const int m = n - k - 1;
        k_chol_step<<<dim3((m + kTx - 1) / kTx, (m + kTy - 1) / kTy), blk, 0, s>>>(n, k, W.p, L.p,
                                                                                 bad.p);
    }
    k_linv_first<<<1, 32, 0, s>>>(n, L.p, Li.p);
    for (int k = 0; k + 1 < n; ++k) {
        const int m = n - k - 1;
        k_linv_step<<<dim3((k + 1 + kTx - 1) / kTx, (m + kTy - 1) / kTy), blk, 0, s>>>(n, k, L.p,
                                                                                     Li.p, T.p);
    }
    k_inv_product<<<dim3((n + kTx - 1) / kTx, (n + kTy - 1) / kTy), blk, 0, s>>>(n, Li.p, iperm,
                                                                               out);
    UNAP_CK(cudaGetLastError());
    int hbad = 0;
    UNAP_CK(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    UNAP_CK(cudaStreamSynchronize(s));
    return hbad == 0;
}

}  // namespace unapgpu
