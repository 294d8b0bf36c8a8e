// edgpu_coupling_grad_device_noalloc: the fused product + coupling-gradient launch for callers that
// must not allocate device memory.
//
// Some callers own all device memory through their own allocator: a Julia or PyTorch memory pool
// that has reserved the device's memory for itself, or an application that pre-allocates everything
// at start-up and must keep cudaMalloc/cudaFree (and the device-wide synchronisation they can imply)
// out of its time-step loop.  edgpu_coupling_grad_device may allocate on its first calls (the
// per-block partial sums, the reduced gradient, the operator's gradient tables); this variant takes
// its scratch from a fixed array that is part of the library instead and allocates nothing.
//
// The scratch is a file-scope __device__ array of NOALLOC_SCRATCH_BYTES (2 MiB).  Every GPU on which
// the library is loaded holds it for the life of the process.  All calls share it: calls whose
// executions overlap on the GPU (different streams, or different host threads) race on it and must
// be serialised by the caller.  Each call overwrites every scratch word it later reads (one partial
// sum per block and coupling, then the totals), so nothing needs clearing between calls.
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
        GradTables t;
        if (!coupling_grad_tables(op, precision, &t))
            throw Error(EDGPU_ERR_STATE,
                        "the operator's gradient tables for this precision are not built yet: call "
                        "edgpu_coupling_grad_device once (it may allocate) before the no-allocation variant");
        if (n != t.dim)
            throw Error(EDGPU_ERR_DIM, "state has length " + std::to_string(n) + " != dimension " + std::to_string(t.dim));
        if ((size_t)2 * t.n_coupl > NOALLOC_SCRATCH_DOUBLES)
            throw Error(EDGPU_ERR_ARG, "n_couplings = " + std::to_string(t.n_coupl) + " exceeds the no-allocation limit of " +
                                           std::to_string(NOALLOC_SCRATCH_DOUBLES / 2) + " couplings");
        cudaStream_t st = (cudaStream_t)stream;
        double* scratch = scratch_on_current_device();
        if (n == 0) {
            for (int c = 0; c < t.n_coupl; ++c) grad_out[c] = 0.0;
            return EDGPU_OK;
        }
        // partial sums [blocks][n_coupl] followed by the totals [n_coupl] must fit the scratch array
        const long long tiles = (t.dim + t.rows_per_tile - 1) / t.rows_per_tile;
        long long blocks = std::min<long long>((tiles + HX_THREADS / 32 - 1) / (HX_THREADS / 32), t.max_blocks);
        blocks = std::max<long long>(1, std::min<long long>(blocks, (long long)(NOALLOC_SCRATCH_DOUBLES / t.n_coupl) - 1));
        double* partial = scratch;
        double* totals = scratch + (size_t)blocks * t.n_coupl;
        HxParams p = t.tmpl;
        p.rows_per_tile = t.rows_per_tile;
        p.x = x;
        p.y = y;
        p.gy = gy;
        p.grad_partial = partial;
        p.accumulate = 0;
        if (t.w32) hx_launch_w32(t.gk, precision, 1, p, (int)blocks, t.smem, st);
        else hx_launch_w64(t.gk, precision, 1, p, (int)blocks, t.smem, st);
        launch_reduce_grad((int)blocks, t.n_coupl, partial, totals, st);
        cudaError_t e = cudaMemcpyAsync(grad_out, totals, t.n_coupl * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("no-allocation gradient: ") + cudaGetErrorString(e));
        return EDGPU_OK;
    } catch (const Error& e) {
        return record_api_error(e.code, e.what());
    } catch (const std::exception& e) {
        return record_api_error(EDGPU_ERR_STATE, e.what());
    }
}
