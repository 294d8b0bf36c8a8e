// Product kernels for basis words of at most 31 bits (uint32 tables).
#include "hx_kernel.cuh"
#include "hx_rows.cuh"

namespace edgpu {

void hx_launch_w32(int gk, int prec, int mode, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    switch (gk * 4 + prec * 2 + mode) {
        EDGPU_HX_CASES(unsigned int, 0, hx_launch_one, p, blocks, smem, st)
        EDGPU_HX_CASES(unsigned int, 1, hx_launch_one, p, blocks, smem, st)
        EDGPU_HX_CASES(unsigned int, 2, hx_launch_one, p, blocks, smem, st)
        EDGPU_HX_CASES(unsigned int, 3, hx_launch_one, p, blocks, smem, st)
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");
    }
}

int hx_occupancy_w32(int gk, int prec, int mode, size_t smem) {
    switch (gk * 4 + prec * 2 + mode) {
        EDGPU_HX_CASES(unsigned int, 0, hx_occupancy_one, smem)
        EDGPU_HX_CASES(unsigned int, 1, hx_occupancy_one, smem)
        EDGPU_HX_CASES(unsigned int, 2, hx_occupancy_one, smem)
        EDGPU_HX_CASES(unsigned int, 3, hx_occupancy_one, smem)
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");
    }
}

// Row-per-lane strategy (product mode only).
void hx_rows_launch_w32(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    switch (gk * 2 + prec) {
        case 0 * 2 + 0: return hx_rows_launch_one<unsigned int, 0, 0, 0>(p, blocks, smem, st);
        case 0 * 2 + 1: return hx_rows_launch_one<unsigned int, 0, 1, 0>(p, blocks, smem, st);
        case 1 * 2 + 0: return hx_rows_launch_one<unsigned int, 1, 0, 0>(p, blocks, smem, st);
        case 1 * 2 + 1: return hx_rows_launch_one<unsigned int, 1, 1, 0>(p, blocks, smem, st);
        case 2 * 2 + 0: return hx_rows_launch_one<unsigned int, 2, 0, 0>(p, blocks, smem, st);
        case 2 * 2 + 1: return hx_rows_launch_one<unsigned int, 2, 1, 0>(p, blocks, smem, st);
        case 3 * 2 + 0: return hx_rows_launch_one<unsigned int, 3, 0, 0>(p, blocks, smem, st);
        case 3 * 2 + 1: return hx_rows_launch_one<unsigned int, 3, 1, 0>(p, blocks, smem, st);
        case 4 * 2 + 0: return hx_rows_launch_one<unsigned int, 4, 0, 0>(p, blocks, smem, st);
        case 4 * 2 + 1: return hx_rows_launch_one<unsigned int, 4, 1, 0>(p, blocks, smem, st);
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");
    }
}

int hx_rows_occupancy_w32(int gk, int prec, size_t smem) {
    switch (gk * 2 + prec) {
        case 0 * 2 + 0: return hx_rows_occupancy_one<unsigned int, 0, 0, 0>(smem);
        case 0 * 2 + 1: return hx_rows_occupancy_one<unsigned int, 0, 1, 0>(smem);
        case 1 * 2 + 0: return hx_rows_occupancy_one<unsigned int, 1, 0, 0>(smem);
        case 1 * 2 + 1: return hx_rows_occupancy_one<unsigned int, 1, 1, 0>(smem);
        case 2 * 2 + 0: return hx_rows_occupancy_one<unsigned int, 2, 0, 0>(smem);
        case 2 * 2 + 1: return hx_rows_occupancy_one<unsigned int, 2, 1, 0>(smem);
        case 3 * 2 + 0: return hx_rows_occupancy_one<unsigned int, 3, 0, 0>(smem);
        case 3 * 2 + 1: return hx_rows_occupancy_one<unsigned int, 3, 1, 0>(smem);
        case 4 * 2 + 0: return hx_rows_occupancy_one<unsigned int, 4, 0, 0>(smem);
        case 4 * 2 + 1: return hx_rows_occupancy_one<unsigned int, 4, 1, 0>(smem);
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");
    }
}

// Batched sectors in one persistent launch (product mode only).
void hx_multi_launch_w32(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    switch (gk * 2 + prec) {
        case 0 * 2 + 0: return hx_multi_launch_one<unsigned int, 0, 0>(p, blocks, smem, st);
        case 0 * 2 + 1: return hx_multi_launch_one<unsigned int, 0, 1>(p, blocks, smem, st);
        case 1 * 2 + 0: return hx_multi_launch_one<unsigned int, 1, 0>(p, blocks, smem, st);
        case 1 * 2 + 1: return hx_multi_launch_one<unsigned int, 1, 1>(p, blocks, smem, st);
        case 2 * 2 + 0: return hx_multi_launch_one<unsigned int, 2, 0>(p, blocks, smem, st);
        case 2 * 2 + 1: return hx_multi_launch_one<unsigned int, 2, 1>(p, blocks, smem, st);
        case 3 * 2 + 0: return hx_multi_launch_one<unsigned int, 3, 0>(p, blocks, smem, st);
        case 3 * 2 + 1: return hx_multi_launch_one<unsigned int, 3, 1>(p, blocks, smem, st);
        case 4 * 2 + 0: return hx_multi_launch_one<unsigned int, 4, 0>(p, blocks, smem, st);
        case 4 * 2 + 1: return hx_multi_launch_one<unsigned int, 4, 1>(p, blocks, smem, st);
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");
    }
}

int hx_multi_occupancy_w32(int gk, int prec, size_t smem) {
    switch (gk * 2 + prec) {
        case 0 * 2 + 0: return hx_multi_occupancy_one<unsigned int, 0, 0>(smem);
        case 0 * 2 + 1: return hx_multi_occupancy_one<unsigned int, 0, 1>(smem);
        case 1 * 2 + 0: return hx_multi_occupancy_one<unsigned int, 1, 0>(smem);
        case 1 * 2 + 1: return hx_multi_occupancy_one<unsigned int, 1, 1>(smem);
        case 2 * 2 + 0: return hx_multi_occupancy_one<unsigned int, 2, 0>(smem);
        case 2 * 2 + 1: return hx_multi_occupancy_one<unsigned int, 2, 1>(smem);
        case 3 * 2 + 0: return hx_multi_occupancy_one<unsigned int, 3, 0>(smem);
        case 3 * 2 + 1: return hx_multi_occupancy_one<unsigned int, 3, 1>(smem);
        case 4 * 2 + 0: return hx_multi_occupancy_one<unsigned int, 4, 0>(smem);
        case 4 * 2 + 1: return hx_multi_occupancy_one<unsigned int, 4, 1>(smem);
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");
    }
}

// Sparse assembly (FP64).
void hx_sparse_launch_w32(int gk, const HxParams& p, long long row0, long long n_run, int conj_vals, double tol,
                         long long* counts, const long long* row_ptr, long long* cols, double2* vals, size_t smem,
                         cudaStream_t st) {
    switch (gk) {
        case 0: return hx_sparse_launch_one<unsigned int, 0>(p, row0, n_run, conj_vals, tol, counts, row_ptr, cols, vals, smem, st);
        case 1: return hx_sparse_launch_one<unsigned int, 1>(p, row0, n_run, conj_vals, tol, counts, row_ptr, cols, vals, smem, st);
        case 2: return hx_sparse_launch_one<unsigned int, 2>(p, row0, n_run, conj_vals, tol, counts, row_ptr, cols, vals, smem, st);
        case 3: return hx_sparse_launch_one<unsigned int, 3>(p, row0, n_run, conj_vals, tol, counts, row_ptr, cols, vals, smem, st);
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");
    }
}

// Adjoint by scatter (terms that do not commute with the group).
void hx_scatter_launch_w32(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    switch (gk * 2 + prec) {
        case 0 * 2 + 0: return hx_scatter_launch_one<unsigned int, 0, 0>(p, blocks, smem, st);
        case 0 * 2 + 1: return hx_scatter_launch_one<unsigned int, 0, 1>(p, blocks, smem, st);
        case 1 * 2 + 0: return hx_scatter_launch_one<unsigned int, 1, 0>(p, blocks, smem, st);
        case 1 * 2 + 1: return hx_scatter_launch_one<unsigned int, 1, 1>(p, blocks, smem, st);
        case 2 * 2 + 0: return hx_scatter_launch_one<unsigned int, 2, 0>(p, blocks, smem, st);
        case 2 * 2 + 1: return hx_scatter_launch_one<unsigned int, 2, 1>(p, blocks, smem, st);
        case 3 * 2 + 0: return hx_scatter_launch_one<unsigned int, 3, 0>(p, blocks, smem, st);
        case 3 * 2 + 1: return hx_scatter_launch_one<unsigned int, 3, 1>(p, blocks, smem, st);
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");
    }
}

// Row-per-lane gradient mode (per-thread coupling accumulators in shared memory).
void hx_rows_grad_launch_w32(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    switch (gk * 2 + prec) {
        case 0 * 2 + 0: return hx_rows_launch_one<unsigned int, 0, 0, 1>(p, blocks, smem, st);
        case 0 * 2 + 1: return hx_rows_launch_one<unsigned int, 0, 1, 1>(p, blocks, smem, st);
        case 1 * 2 + 0: return hx_rows_launch_one<unsigned int, 1, 0, 1>(p, blocks, smem, st);
        case 1 * 2 + 1: return hx_rows_launch_one<unsigned int, 1, 1, 1>(p, blocks, smem, st);
        case 2 * 2 + 0: return hx_rows_launch_one<unsigned int, 2, 0, 1>(p, blocks, smem, st);
        case 2 * 2 + 1: return hx_rows_launch_one<unsigned int, 2, 1, 1>(p, blocks, smem, st);
        case 3 * 2 + 0: return hx_rows_launch_one<unsigned int, 3, 0, 1>(p, blocks, smem, st);
        case 3 * 2 + 1: return hx_rows_launch_one<unsigned int, 3, 1, 1>(p, blocks, smem, st);
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");
    }
}

int hx_rows_grad_occupancy_w32(int gk, int prec, size_t smem) {
    switch (gk * 2 + prec) {
        case 0 * 2 + 0: return hx_rows_occupancy_one<unsigned int, 0, 0, 1>(smem);
        case 0 * 2 + 1: return hx_rows_occupancy_one<unsigned int, 0, 1, 1>(smem);
        case 1 * 2 + 0: return hx_rows_occupancy_one<unsigned int, 1, 0, 1>(smem);
        case 1 * 2 + 1: return hx_rows_occupancy_one<unsigned int, 1, 1, 1>(smem);
        case 2 * 2 + 0: return hx_rows_occupancy_one<unsigned int, 2, 0, 1>(smem);
        case 2 * 2 + 1: return hx_rows_occupancy_one<unsigned int, 2, 1, 1>(smem);
        case 3 * 2 + 0: return hx_rows_occupancy_one<unsigned int, 3, 0, 1>(smem);
        case 3 * 2 + 1: return hx_rows_occupancy_one<unsigned int, 3, 1, 1>(smem);
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");
    }
}

}  // namespace edgpu
