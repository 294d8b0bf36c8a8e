// Product kernels for basis words of at most 31 bits (uint32 tables).
#include "hx_kernel.cuh"

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

}  // namespace edgpu
