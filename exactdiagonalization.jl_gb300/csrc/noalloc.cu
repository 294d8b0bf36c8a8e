// edgpu_coupling_grad_device_noalloc: the fused product + coupling-gradient launch for callers that
// must not allocate device memory.
//
// Some callers own all device memory through their own allocator: a Julia or PyTorch memory pool
// that has reserved the device's memory for itself, or an application that pre-allocates everything
// at start-up and must keep cudaMalloc/cudaFree (and the device-wide synchronisation they can imply)
// out of its time-step loop.  edgpu_coupling_grad_device may allocate on its first calls (the
// per-block partial sums, the reduced gradient, the operator's tables); this variant takes its
// scratch from a fixed array that is part of the library instead and allocates nothing.  It runs the
// same kernel as edgpu_coupling_grad_device (the pair-flip gradient kernel when the operator has a
// target table or its space a parent-state map, else the row-per-lane or queued term scan).
//
// The scratch is a file-scope __device__ array of NOALLOC_SCRATCH_BYTES (2 MiB).  Every GPU on which
// the library is loaded holds it for the life of the process.  All calls share it: calls whose
// executions overlap on the GPU (different streams, or different host threads with different
// operators) race on it and must be serialised by the caller.  Each call overwrites every scratch
// word it later reads (one partial sum per block and coupling, then the totals), so nothing needs
// clearing between calls.
#include <mutex>
#include <vector>

#include "edgpu_internal.h"

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)2 << 20;
constexpr size_t NOALLOC_SCRATCH_DOUBLES = NOALLOC_SCRATCH_BYTES / sizeof(double);

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

std::mutex g_scratch_mu;
std::vector<double*> g_scratch_by_device;   // device address of g_noalloc_scratch, per device

// Device address of the scratch array on the current device.  In host code g_noalloc_scratch is only
// a host-side stand-in, so its address is looked up once per device with that device current.
double* scratch_on_current_device() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) throw edgpu::Error(EDGPU_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if ((int)g_scratch_by_device.size() <= dev) g_scratch_by_device.resize(dev + 1, nullptr);
    if (!g_scratch_by_device[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || ptr == nullptr)
            throw edgpu::Error(EDGPU_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_scratch_by_device[dev] = (double*)ptr;
    }
    return g_scratch_by_device[dev];
}

}  // namespace

extern "C" int edgpu_coupling_grad_device_noalloc(edgpu_op op, int32_t precision, const void* x, const void* gy,
                                                  void* y, int64_t n, double* grad_out, void* stream) {
    using namespace edgpu;
    try {
        if (!op) throw Error(EDGPU_ERR_ARG, "null operator handle");
        if (precision != EDGPU_FP64 && precision != EDGPU_MIXED) throw Error(EDGPU_ERR_ARG, "bad precision");
        if (!x || !gy || !y || !grad_out) throw Error(EDGPU_ERR_ARG, "x, gy, y and grad_out are required");
        auto lk = lock_op(op);   // calls on one operator handle are serialised
        const int n_coupl = coupling_count(op);
        const int64_t dim = op_dimension(op);
        if (n != dim)
            throw Error(EDGPU_ERR_DIM, "state has length " + std::to_string(n) + " != dimension " + std::to_string(dim));
        // at least one block's partial sums plus the totals must fit; operator creation already limits
        // n_couplings to 8192, far below this guard
        if ((size_t)2 * n_coupl > NOALLOC_SCRATCH_DOUBLES)
            throw Error(EDGPU_ERR_ARG, "n_couplings = " + std::to_string(n_coupl) + " exceeds the no-allocation limit of " +
                                           std::to_string(NOALLOC_SCRATCH_DOUBLES / 2) + " couplings");
        cudaStream_t st = (cudaStream_t)stream;
        double* scratch = scratch_on_current_device();
        if (n == 0) {
            for (int c = 0; c < n_coupl; ++c) grad_out[c] = 0.0;
            return EDGPU_OK;
        }
        // partial sums [blocks][n_coupl] followed by the totals [n_coupl]
        const int cap = (int)std::max<long long>(1, (long long)(NOALLOC_SCRATCH_DOUBLES / n_coupl) - 1);
        int blocks = 0;
        if (!coupling_grad_launch_built(op, precision, x, gy, y, scratch, cap, st, &blocks))
            throw Error(EDGPU_ERR_STATE,
                        "the operator's gradient tables for this precision are not built yet: call "
                        "edgpu_coupling_grad_device once (it may allocate) before the no-allocation variant");
        double* totals = scratch + (size_t)blocks * n_coupl;
        launch_reduce_grad(blocks, n_coupl, scratch, totals, st);
        cudaError_t e = cudaMemcpyAsync(grad_out, totals, n_coupl * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("no-allocation gradient: ") + cudaGetErrorString(e));
        return EDGPU_OK;
    } catch (const Error& e) {
        return record_api_error(e.code, e.what());
    } catch (const std::exception& e) {
        return record_api_error(EDGPU_ERR_STATE, e.what());
    }
}
