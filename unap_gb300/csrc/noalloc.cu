// unap_cuda_spmv_noalloc: y = A x for callers that cannot allocate device
// memory at call time.
//
// unap_cuda_spmv reorders x and A x through two scratch vectors that the
// matrix handle allocates with cudaMalloc the first time they are needed
// (and again when the matrix size changes).  Some callers cannot allow an
// allocation at that point: a time-stepping code that reserved its whole
// device-memory budget up front and must not fail with out-of-memory half
// way through a run, or a host thread that must not take the CUDA
// allocator's locks while other threads allocate.  This variant takes its
// scratch from a fixed array compiled into the library instead:
//
//   * the array is a file-scope __device__ array of 2 * kNoAllocMaxCells
//     doubles (16 MiB); every GPU that loads the library holds it until the
//     process exits;
//   * matrices with more than kNoAllocMaxCells cells are rejected with
//     UNAP_CUDA_EINVAL and a message (there is no fallback that allocates);
//   * host code cannot use the array's name as a device address, so the
//     first call for a matrix on each device looks the address up with
//     cudaGetSymbolAddress, with the matrix's device current, and keeps it;
//   * the call runs on the device the matrix was built on whatever device
//     is current (it makes that one current for the call and restores the
//     caller's afterwards); it is synchronous -- it returns when its kernels
//     have finished -- so it must not be called while a stream capture is
//     active on the calling thread;
//   * every call uses the same array: calls whose work overlaps on the GPU
//     (different streams or host threads at the same time) race on it;
//     calls on one stream, or one after another, are safe.  Both halves are
//     fully overwritten by every call, so nothing has to start at zero;
//   * the matrix handle must already be built on the device (coefficients
//     filled), because building it allocates.
//
// Nothing here calls cudaMalloc, cudaFree or a routine that allocates.
#include <mutex>

#include "capi_handles.hpp"
#include "../../include/unap_cuda.h"

namespace unapgpu {

constexpr int kNoAllocMaxCells = 1 << 20;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[2 * (size_t)kNoAllocMaxCells];

namespace {

std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// device address of the scratch array on device `dev` (current), looked up
// once per device
double* noalloc_scratch(int dev)
{
    if (dev < 0 || dev >= kNoAllocMaxDevices) throw std::invalid_argument("device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            throw CudaError(std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") +
                            cudaGetErrorString(e));
        g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
    return g_noalloc_ptr[dev];
}

// makes `dev` current for its lifetime, then restores the caller's device
struct DeviceScope {
    int old = -1;
    explicit DeviceScope(int dev)
    {
        UNAP_CK(cudaGetDevice(&old));
        if (old != dev) UNAP_CK(cudaSetDevice(dev));
    }
    ~DeviceScope()
    {
        int cur = -1;
        if (cudaGetDevice(&cur) == cudaSuccess && cur != old && old >= 0) cudaSetDevice(old);
    }
};

}  // namespace

}  // namespace unapgpu

using namespace unapgpu;

extern "C" int unap_cuda_spmv_noalloc(long int handle, const double* x, double* y)
{
    try {
        MatHandle* h = mat_from(handle);
        if (!h->M) throw std::invalid_argument("matrix handle is not built on the device yet");
        Matrix& A = *h->M;
        const int n = A.n();
        if (n > kNoAllocMaxCells)
            throw std::invalid_argument("unap_cuda_spmv_noalloc: " + std::to_string(n) +
                                        " cells exceed the static scratch limit of " +
                                        std::to_string(kNoAllocMaxCells));
        DeviceScope scope(A.device);
        double* scratch = noalloc_scratch(A.device);
        double* xi = scratch;
        double* yi = scratch + kNoAllocMaxCells;
        Exec ex{A.stream, device_max_blocks()};
        order_after_default_stream(A.stream);
        k_to_internal<double>(ex, n, A.L->d_perm.p, x, xi);
        k_spmv<double>(ex, rows64(*A.L), xi, yi, nullptr, RSpec{}, Gate{});
        k_to_reference<double>(ex, n, A.L->d_perm.p, yi, y);
        UNAP_CK(cudaGetLastError());
        UNAP_CK(cudaStreamSynchronize(A.stream));
        return UNAP_CUDA_OK;
    } catch (const CudaError& e) {
        set_last_error(e.what());
        return UNAP_CUDA_ECUDA;
    } catch (const std::invalid_argument& e) {
        set_last_error(e.what());
        return UNAP_CUDA_EINVAL;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return UNAP_CUDA_EINTERNAL;
    }
}
