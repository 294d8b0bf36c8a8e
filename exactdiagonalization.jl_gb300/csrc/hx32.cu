// Product kernels for basis words of at most 31 bits (uint32 tables).
#include "hx_kernel.cuh"

namespace edgpu {

void hx_launch_w32(int gk, int prec, int mode, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    EDGPU_HX_DISPATCH(unsigned int, hx_launch_one, p, blocks, smem, st)
}

int hx_occupancy_w32(int gk, int prec, int mode, size_t smem) {
    EDGPU_HX_DISPATCH(unsigned int, hx_occupancy_one, smem)
}

}  // namespace edgpu
