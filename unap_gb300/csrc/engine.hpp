// Host-side engine: matrices, preconditioners and Krylov drivers on one GPU.
#pragma once

#include <memory>
#include <vector>

#include "kernels.hpp"
#include "mega.hpp"
#include "small_solve.hpp"

namespace unapgpu {

struct SolveStats {
    int nIter = 0;
    double initRes = 0, finalRes = 0, trueRes = -1;
    int converged = 0, singular = 0, status = 0;
    double seconds = 0;  // device time of the solve (CUDA events)
    double bytes = 0;    // algorithmic DRAM bytes of the solve (step executor)
};

// A device-resident LDU matrix (one system).  The host copy keeps the
// reference layout; the device Level holds the internal order and SELL rows.
class Matrix {
public:
    // wavefronts == false: locality order without wavefront ranges, for a
    // matrix used only by SpMV-shaped work (SpMV, Chebyshev smoothing,
    // AMG without Gauss-Seidel on it); DIC, DILU and Gauss-Seidel refuse it
    Matrix(HostLdu&& h, cudaStream_t s, bool wavefronts = true);
    ~Matrix();
    HostLdu host;
    std::unique_ptr<Level> L;
    cudaStream_t stream;
    bool ownsStream = false;
    int device = 0;  // the GPU the matrix was built on (current at construction)
    int n() const { return host.n; }
    // replace the coefficients (same addressing)
    void setValues(const double* diag, const double* upper, const double* lower);
};

// Preconditioner interface: w = M^-1 r on internal-order vectors.
class Precond {
public:
    virtual ~Precond() = default;
    // true when apply() also reduces w.r into `site` and finalizes with `fin`
    virtual bool fusesDot() const { return false; }
    virtual void apply(const Exec& ex, const double* r, double* w, const RedPool* pool, int site,
                       KState* st, int fin, Gate g) = 0;
    // Step-program form of apply (mega.hpp): appends the steps computing
    // w = M^-1 r; level 0 of `lv` is the system matrix.  When the steps
    // also leave w.r in partial slot `slot`, *dotFused is set.  Returns false
    // when the preconditioner has no step form.
    virtual bool appendSteps(std::vector<Step>& out, std::vector<LevelRows>& lv, const double* r,
                             double* w, int slot, bool* dotFused)
    {
        (void)out, (void)lv, (void)r, (void)w, (void)slot, (void)dotFused;
        return false;
    }
    // LDU preconditioner type (0 none, 1 Diag, 2 DIC, 3 DILU; -1 other) and
    // its reciprocal diagonal in internal order, for whole-solve launches
    virtual int lduType() const { return -1; }
    virtual const double* lduRD() const { return nullptr; }
};

std::unique_ptr<Precond> make_ldu_precond(int type, Matrix& A);  // 1 Diag, 2 DIC, 3 DILU, else none

enum class Method { PCG, PBiCGStab };

// Krylov driver with device-resident scalars and CUDA-graph iterations.
class Krylov {
public:
    Krylov(Matrix& A, Precond* P, Method m);
    ~Krylov();
    double tol = 0.0, relTol = 1e-6;
    int maxIter = 1000, minIter = 0;
    bool flexible = false;   // PCG only
    // PCG's outer vector work (SpMV, dots, updates) in fused multiply-adds:
    // half the FP64 instructions (the mixed-precision AMG-PCG's outer loop)
    bool fusedOuter = false;
    bool trueResidualRestart = false;  // re-check ||b - Ax|| and restart if needed
    bool useGraph = true;
    bool useMega = true;     // PCG as one persistent cooperative launch when possible
    // systems of at most this many cells with an LDU preconditioner (none,
    // Diag, DIC, DILU) are solved by one whole-solve launch (small_solve.cu)
    int teamCells = 0;
    TeamShape lastShape{0, 0};  // shape of the last whole-solve launch
    // solve on device vectors in reference order (x in/out, b in)
    SolveStats solveDevice(double* x_ref, const double* b_ref);
    // solve on host vectors (copies in and out)
    SolveStats solveHost(double* x, const double* b);
    Matrix& A;

private:
    Precond* P;
    Method method;
    Exec ex;
    int n;
    DevArray<double> x, b, r, z, p, q, r0, y, Ay, s, t, zz;
    DevArray<double> hx_ref;  // staging for host solves
    KState* d_st = nullptr;
    KState* h_st = nullptr;   // pinned
    RedPool pool;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graphExec = nullptr;
    long long graphKernels = 0;
    cudaEvent_t ev0, ev1;
    std::unique_ptr<MegaRunner> mega;
    bool megaReady = false, megaTried = false;
    int megaSteps = 0;
    double megaInitBytes = 0, megaIterBytes = 0;  // algorithmic bytes of the program
    bool bytesKnown = false;
    // one PCG iteration (and the init part) as a step program; false for
    // methods or preconditioners without one
    DevArray<double> teamWork;      // whole-solve launch: work vectors
    DevArray<int> teamWaves;        // and wavefront ranges
    DevArray<unsigned char> teamSys;  // its SmallSystem and SmallResult
    SolveStats solveTeam(double* x_ref, const double* b_ref);
    bool stepProgram(std::vector<Step>& steps, std::vector<LevelRows>& lv, int& nInit);
    bool buildMega();
    void enqueueIteration();
    void enqueuePcgIteration();
    void enqueueBicgIteration();
    void initState();
    void runIterations();
    void readState();
};

// default executor of Krylov objects created afterwards; returns the old one
int set_default_executor(int persistent);
// whether matrices created through the C ABI afterwards get wavefront
// ranges (1, default) or only a locality order (0); returns the old value
int set_matrix_wavefronts(int on);
int matrix_wavefronts();

// Dense FP64 SPD inverse by Cholesky (row-major in, row-major out).
// Returns false when the matrix is not positive definite.
bool dense_spd_inverse(int n, const std::vector<double>& A, std::vector<double>& inv);
// The same inverse computed on the device (dense_dev.cu), written
// column-major to out (n * n doubles on the device) with rows in the
// internal order iperm gives (null: identity) and columns in cell order.
// Used from this many coarsest cells up.
constexpr int kDeviceInverseCells = 128;
bool dense_spd_inverse_device(int n, const std::vector<double>& A, const int* iperm, double* out,
                              cudaStream_t s);

}  // namespace unapgpu
