// Product kernels for basis words of 32 to 63 bits (uint64 tables).
#include "hx_kernel.cuh"

namespace edgpu {

void hx_launch_w64(int gk, int prec, int mode, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    switch (gk * 4 + prec * 2 + mode) {
        EDGPU_HX_CASES(unsigned long long, 0, hx_launch_one, p, blocks, smem, st)
        EDGPU_HX_CASES(unsigned long long, 1, hx_launch_one, p, blocks, smem, st)
        EDGPU_HX_CASES(unsigned long long, 2, hx_launch_one, p, blocks, smem, st)
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");
    }
}

int hx_occupancy_w64(int gk, int prec, int mode, size_t smem) {
    switch (gk * 4 + prec * 2 + mode) {
        EDGPU_HX_CASES(unsigned long long, 0, hx_occupancy_one, smem)
        EDGPU_HX_CASES(unsigned long long, 1, hx_occupancy_one, smem)
        EDGPU_HX_CASES(unsigned long long, 2, hx_occupancy_one, smem)
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");
    }
}

int hx_warp_bytes(bool w32) {
    return w32 ? hx_warp_bytes_t<unsigned int>() : hx_warp_bytes_t<unsigned long long>();
}

int hx_max_blocks_per_sm(bool w32, int gk, int prec, int mode, size_t smem) {
    int hx_occupancy_w32(int, int, int, size_t);
    return w32 ? hx_occupancy_w32(gk, prec, mode, smem) : hx_occupancy_w64(gk, prec, mode, smem);
}

}  // namespace edgpu
