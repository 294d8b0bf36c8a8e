// Vector kernels around the product: seeded start vectors, precision conversion, deterministic FP64
// reductions (dots, norms, Gram-Schmidt projections) and the Lanczos three-term update.
// All reductions use a fixed grid and a fixed second-stage order, so results are reproducible.
#include <cmath>

#include "edgpu_internal.h"

namespace edgpu {

namespace {

constexpr int RED_BLOCKS = 1024;
constexpr int RED_THREADS = 256;
constexpr int MD_BLOCKS = 64;   // blocks per vector in the multi-dot

unsigned grid_for(int64_t n, int threads = 256) {
    int64_t b = (n + threads - 1) / threads;
    if (b > 1048576) b = 1048576;
    if (b < 1) b = 1;
    return (unsigned)b;
}

__device__ __forceinline__ unsigned long long splitmix64_at(unsigned long long seed, unsigned long long k) {
    unsigned long long z = seed + (k + 1ull) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_random_c128(long long n, unsigned long long seed, double2* dst) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double u = (double)(splitmix64_at(seed, 2ull * i) >> 11) * (1.0 / 9007199254740992.0);
        const double u2 = (double)(splitmix64_at(seed, 2ull * i + 1ull) >> 11) * (1.0 / 9007199254740992.0);
        const double u1 = 1.0 - u;
        const double r = sqrt(-2.0 * log(u1));
        const double ang = 2.0 * M_PI * u2;
        const double s = 0.70710678118654752440;   // 1/sqrt(2)
        dst[i] = make_double2(r * cos(ang) * s, r * sin(ang) * s);
    }
}

__global__ void k_c128_to_c64(long long n, const double2* src, float2* dst) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double2 v = src[i];
        dst[i] = make_float2((float)v.x, (float)v.y);
    }
}

__global__ void k_c64_to_c128(long long n, const float2* src, double2* dst, int accumulate) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = src[i];
        double2 o = make_double2((double)v.x, (double)v.y);
        if (accumulate) {
            const double2 a = dst[i];
            o.x += a.x;
            o.y += a.y;
        }
        dst[i] = o;
    }
}

__global__ void k_scale_c128(long long n, double s, double2* v) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double2 a = v[i];
        v[i] = make_double2(a.x * s, a.y * s);
    }
}

__global__ void k_conj_c128(long long n, double2* v) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[i].y = -v[i].y;
}

__device__ __forceinline__ double2 block_sum2(double2 v, double2* sh) {
    for (int d = 16; d > 0; d >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, d);
        v.y += __shfl_down_sync(0xffffffffu, v.y, d);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double2 r = make_double2(0.0, 0.0);
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            r.x += sh[w].x;
            r.y += sh[w].y;
        }
    __syncthreads();
    return r;
}

// Stage 1: <a, b> = sum conj(a_i) b_i over a grid-stride slice; partial per block.
__global__ void k_dot_stage1(long long n, const double2* a, const double2* b, double2* partial, int norm_only) {
    __shared__ double2 sh[32];
    double2 s = make_double2(0.0, 0.0);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double2 u = a[i];
        if (norm_only) {
            s.x += u.x * u.x + u.y * u.y;
        } else {
            const double2 v = b[i];
            s.x += u.x * v.x + u.y * v.y;
            s.y += u.x * v.y - u.y * v.x;
        }
    }
    const double2 r = block_sum2(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

// Stage 2: fixed-order sum of the partials; out = sum (or sqrt of its real part for a norm).
__global__ void k_dot_stage2(int nparts, const double2* partial, double* out, int take_sqrt) {
    __shared__ double2 sh[32];
    double2 s = make_double2(0.0, 0.0);
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        s.x += partial[i].x;
        s.y += partial[i].y;
    }
    const double2 r = block_sum2(s, sh);
    if (threadIdx.x == 0) {
        if (take_sqrt) out[0] = sqrt(r.x);
        else {
            out[0] = r.x;
            out[1] = r.y;
        }
    }
}

__global__ void k_reduce_grad(int nblocks, int ncoupl, const double* partial, double* out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncoupl) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += partial[(size_t)b * ncoupl + c];
    out[c] = s;
}

__global__ void k_lanczos_update(long long n, double2* w, const double2* v, const double2* u, const double* alpha,
                                 const double* beta) {
    const double a = alpha[0];
    const double b = (u && beta) ? beta[0] : 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double2 x = w[i];
        const double2 vv = v[i];
        x.x -= a * vv.x;
        x.y -= a * vv.y;
        if (u) {
            const double2 uu = u[i];
            x.x -= b * uu.x;
            x.y -= b * uu.y;
        }
        w[i] = x;
    }
}

// h_k = <V_k, w>: grid (MD_BLOCKS, k); partial[k][block].
__global__ void k_multi_dot_stage1(long long n, const double2* V, long long ldv, const double2* w, double2* partial) {
    __shared__ double2 sh[32];
    const int k = blockIdx.y;
    const double2* vk = V + (size_t)k * ldv;
    double2 s = make_double2(0.0, 0.0);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double2 u = vk[i];
        const double2 v = w[i];
        s.x += u.x * v.x + u.y * v.y;
        s.y += u.x * v.y - u.y * v.x;
    }
    const double2 r = block_sum2(s, sh);
    if (threadIdx.x == 0) partial[(size_t)k * gridDim.x + blockIdx.x] = r;
}

__global__ void k_multi_dot_stage2(int nparts, const double2* partial, double2* h) {
    __shared__ double2 sh[32];
    const int k = blockIdx.x;
    double2 s = make_double2(0.0, 0.0);
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        s.x += partial[(size_t)k * nparts + i].x;
        s.y += partial[(size_t)k * nparts + i].y;
    }
    const double2 r = block_sum2(s, sh);
    if (threadIdx.x == 0) h[k] = r;
}

__global__ void k_multi_axpy(long long n, int K, const double2* V, long long ldv, const double2* h, double2* w) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double2 x = w[i];
        for (int k = 0; k < K; ++k) {
            const double2 c = h[k];
            const double2 u = V[(size_t)k * ldv + i];
            x.x -= c.x * u.x - c.y * u.y;
            x.y -= c.x * u.y + c.y * u.x;
        }
        w[i] = x;
    }
}

// The same over a complex64 basis (the stored Krylov basis of a mixed-precision run).
__global__ void k_multi_dot_stage1_c64(long long n, const float2* V, long long ldv, const double2* w, double2* partial) {
    __shared__ double2 sh[32];
    const int k = blockIdx.y;
    const float2* vk = V + (size_t)k * ldv;
    double2 s = make_double2(0.0, 0.0);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 u = vk[i];
        const double2 v = w[i];
        s.x += (double)u.x * v.x + (double)u.y * v.y;
        s.y += (double)u.x * v.y - (double)u.y * v.x;
    }
    const double2 r = block_sum2(s, sh);
    if (threadIdx.x == 0) partial[(size_t)k * gridDim.x + blockIdx.x] = r;
}

__global__ void k_multi_axpy_c64(long long n, int K, const float2* V, long long ldv, const double2* h, double2* w) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double2 x = w[i];
        for (int k = 0; k < K; ++k) {
            const double2 c = h[k];
            const float2 u = V[(size_t)k * ldv + i];
            x.x -= c.x * (double)u.x - c.y * (double)u.y;
            x.y -= c.x * (double)u.y + c.y * (double)u.x;
        }
        w[i] = x;
    }
}

__global__ void k_normalize(long long n, const double2* w, const double* beta, double2* v, float2* v32) {
    const double inv = 1.0 / beta[0];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double2 a = w[i];
        const double2 o = make_double2(a.x * inv, a.y * inv);
        v[i] = o;
        if (v32) v32[i] = make_float2((float)o.x, (float)o.y);
    }
}

__global__ void k_axpy_real(long long n, double a, const double2* x, double2* y) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double2 u = x[i];
        double2 v = y[i];
        v.x += a * u.x;
        v.y += a * u.y;
        y[i] = v;
    }
}

}  // namespace

void launch_random_c128(int64_t n, uint64_t seed, double* dst, cudaStream_t st) {
    if (n <= 0) return;
    k_random_c128<<<grid_for(n), 256, 0, st>>>(n, seed, (double2*)dst);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_c128_to_c64(int64_t n, const double* src, float* dst, cudaStream_t st) {
    if (n <= 0) return;
    k_c128_to_c64<<<grid_for(n), 256, 0, st>>>(n, (const double2*)src, (float2*)dst);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_c64_to_c128(int64_t n, const float* src, double* dst, int accumulate, cudaStream_t st) {
    if (n <= 0) return;
    k_c64_to_c128<<<grid_for(n), 256, 0, st>>>(n, (const float2*)src, (double2*)dst, accumulate);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_scale_c128(int64_t n, double s, double* v, cudaStream_t st) {
    if (n <= 0) return;
    k_scale_c128<<<grid_for(n), 256, 0, st>>>(n, s, (double2*)v);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_conj_c128(int64_t n, double* v, cudaStream_t st) {
    if (n <= 0) return;
    k_conj_c128<<<grid_for(n), 256, 0, st>>>(n, (double2*)v);
    EDGPU_CUDA(cudaGetLastError());
}

size_t dot_scratch_doubles() { return 2 * (size_t)RED_BLOCKS; }

void launch_dot_c128(int64_t n, const double* a, const double* b, double* scratch, double* out_dev, cudaStream_t st) {
    k_dot_stage1<<<RED_BLOCKS, RED_THREADS, 0, st>>>(n, (const double2*)a, (const double2*)b, (double2*)scratch, 0);
    k_dot_stage2<<<1, 1024, 0, st>>>(RED_BLOCKS, (const double2*)scratch, out_dev, 0);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_norm2_c128(int64_t n, const double* a, double* scratch, double* out_dev, cudaStream_t st) {
    k_dot_stage1<<<RED_BLOCKS, RED_THREADS, 0, st>>>(n, (const double2*)a, nullptr, (double2*)scratch, 1);
    k_dot_stage2<<<1, 1024, 0, st>>>(RED_BLOCKS, (const double2*)scratch, out_dev, 1);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_reduce_grad(int nblocks, int ncoupl, const double* partial, double* out_dev, cudaStream_t st) {
    if (ncoupl <= 0) return;
    k_reduce_grad<<<(ncoupl + 127) / 128, 128, 0, st>>>(nblocks, ncoupl, partial, out_dev);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_lanczos_update(int64_t n, double* w, const double* v, const double* u, const double* alpha_dev,
                           const double* beta_dev, cudaStream_t st) {
    if (n <= 0) return;
    k_lanczos_update<<<grid_for(n), 256, 0, st>>>(n, (double2*)w, (const double2*)v, (const double2*)u, alpha_dev,
                                                  beta_dev);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_multi_dot(int64_t n, int k, const double* V, int64_t ldv, const double* w, double* scratch, double* h_dev,
                      cudaStream_t st) {
    if (k <= 0) return;
    dim3 grid(MD_BLOCKS, k);
    k_multi_dot_stage1<<<grid, RED_THREADS, 0, st>>>(n, (const double2*)V, ldv, (const double2*)w, (double2*)scratch);
    k_multi_dot_stage2<<<k, 64, 0, st>>>(MD_BLOCKS, (const double2*)scratch, (double2*)h_dev);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_multi_axpy(int64_t n, int k, const double* V, int64_t ldv, const double* h_dev, double* w, cudaStream_t st) {
    if (k <= 0 || n <= 0) return;
    k_multi_axpy<<<grid_for(n), 256, 0, st>>>(n, k, (const double2*)V, ldv, (const double2*)h_dev, (double2*)w);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_multi_dot_c64(int64_t n, int k, const float* V, int64_t ldv, const double* w, double* scratch, double* h_dev,
                          cudaStream_t st) {
    if (k <= 0) return;
    dim3 grid(MD_BLOCKS, k);
    k_multi_dot_stage1_c64<<<grid, RED_THREADS, 0, st>>>(n, (const float2*)V, ldv, (const double2*)w, (double2*)scratch);
    k_multi_dot_stage2<<<k, 64, 0, st>>>(MD_BLOCKS, (const double2*)scratch, (double2*)h_dev);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_multi_axpy_c64(int64_t n, int k, const float* V, int64_t ldv, const double* h_dev, double* w,
                           cudaStream_t st) {
    if (k <= 0 || n <= 0) return;
    k_multi_axpy_c64<<<grid_for(n), 256, 0, st>>>(n, k, (const float2*)V, ldv, (const double2*)h_dev, (double2*)w);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_normalize(int64_t n, const double* w, const double* beta_dev, double* v_next, float* v32, cudaStream_t st) {
    if (n <= 0) return;
    k_normalize<<<grid_for(n), 256, 0, st>>>(n, (const double2*)w, beta_dev, (double2*)v_next, (float2*)v32);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_axpy_real(int64_t n, double a, const double* x, double* y, cudaStream_t st) {
    if (n <= 0) return;
    k_axpy_real<<<grid_for(n), 256, 0, st>>>(n, a, (const double2*)x, (double2*)y);
    EDGPU_CUDA(cudaGetLastError());
}

}  // namespace edgpu
