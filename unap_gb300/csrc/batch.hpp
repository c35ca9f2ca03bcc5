// Batched solves of many LDU systems (batch.cu).
#pragma once

#include <map>
#include <vector>

#include "engine.hpp"
#include "small_solve.hpp"

namespace unapgpu {

constexpr int kBatchSmallCells = 65536;  // systems solved by one CTA each

struct BatchItem {
    Matrix* A = nullptr;
    int method = 0;   // 0 PCG, 1 PBiCGStab
    int precond = 0;  // 0 none, 1 Diag, 2 DIC, 3 DILU
    double tol = 0.0, relTol = 1e-6;
    int maxIter = 1000, minIter = 0;
    double* x = nullptr;        // device, caller's order (initial guess in, solution out)
    const double* b = nullptr;  // device, caller's order
};

class BatchSolver {
public:
    explicit BatchSolver(cudaStream_t s);
    ~BatchSolver();
    std::vector<SolveStats> solve(const std::vector<BatchItem>& items);
    int lastThreads = 0;  // CTA size of the last fused launch

    // drop the cached preconditioner diagonals of a matrix that is going away
    void forget(const Matrix* A);

private:
    struct Key {
        const Matrix* A;
        int precond;
        bool operator<(const Key& o) const
        {
            return A < o.A || (A == o.A && precond < o.precond);
        }
    };
    struct Fac {
        int version = -1;
        DevArray<double> rD;
    };
    cudaStream_t stream;
    std::map<Key, Fac> factors;       // preconditioner diagonals per matrix
    DevArray<double> ws;              // internal-order x, b and work vectors
    DevArray<SmallSystem> dSys;
    DevArray<SmallResult> results;
    std::vector<DevArray<int>> waveDev;
    DevArray<unsigned char> dIn, dOut;  // gather / scatter job lists
    const double* factor(Matrix& A, int precond);
    void solveSmall(const std::vector<BatchItem>& items, const std::vector<int>& idx,
                    std::vector<SolveStats>& out);
    int autotune(int sizeClass, int m);
};

// CTA size the autotuner chose for a size class (0: not tuned yet)
int batch_tuned_threads(int sizeClass);

}  // namespace unapgpu
