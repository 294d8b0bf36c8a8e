// Pair-flip schedule kernels (hx_bond.cuh) for both word widths, precisions and target lookups
// (GK_TRIVIAL search, GK_TORUS / GK_GENERIC / GK_RING canonicalisation and search, GK_MAP parent-state
// map).  Two targets per lane and step, and four for the parent-state map flavour (nt = 4).
#include "hx_bond.cuh"

namespace edgpu {

// Rings of 1-bit sites in 32-bit words only (GK_RING is never selected for 64-bit tables).
#define RING_OR_TORUS(W) (sizeof(W) == 4 ? GK_RING : GK_TORUS)

#define EDGPU_BOND_CASES(W, FN, ...)                                                                   \
    if (gk == GK_MAP && nt == 4) {                                                                     \
        if (prec == 0) return FN<W, GK_MAP, 0, 4>(__VA_ARGS__);                                        \
        return FN<W, GK_MAP, 1, 4>(__VA_ARGS__);                                                       \
    }                                                                                                  \
    switch (gk * 2 + prec) {                                                                           \
        case 0 * 2 + 0: return FN<W, 0, 0, 2>(__VA_ARGS__);                                            \
        case 0 * 2 + 1: return FN<W, 0, 1, 2>(__VA_ARGS__);                                            \
        case 1 * 2 + 0: return FN<W, 1, 0, 2>(__VA_ARGS__);                                            \
        case 1 * 2 + 1: return FN<W, 1, 1, 2>(__VA_ARGS__);                                            \
        case 2 * 2 + 0: return FN<W, 2, 0, 2>(__VA_ARGS__);                                            \
        case 2 * 2 + 1: return FN<W, 2, 1, 2>(__VA_ARGS__);                                            \
        case 3 * 2 + 0: return FN<W, RING_OR_TORUS(W), 0, 2>(__VA_ARGS__);                             \
        case 3 * 2 + 1: return FN<W, RING_OR_TORUS(W), 1, 2>(__VA_ARGS__);                             \
        case 4 * 2 + 0: return FN<W, 4, 0, 2>(__VA_ARGS__);                                            \
        case 4 * 2 + 1: return FN<W, 4, 1, 2>(__VA_ARGS__);                                            \
        default: throw Error(EDGPU_ERR_ARG, "bad pair-flip kernel selector");                          \
    }

void hx_bond_launch_w32(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    const int nt = p.bond_nt;
    EDGPU_BOND_CASES(unsigned int, hx_bond_launch_one, p, blocks, smem, st)
}
void hx_bond_launch_w64(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    const int nt = p.bond_nt;
    EDGPU_BOND_CASES(unsigned long long, hx_bond_launch_one, p, blocks, smem, st)
}
int hx_bond_occupancy_w32(int gk, int prec, int nt, size_t smem) {
    EDGPU_BOND_CASES(unsigned int, hx_bond_occupancy_one, smem)
}
int hx_bond_occupancy_w64(int gk, int prec, int nt, size_t smem) {
    EDGPU_BOND_CASES(unsigned long long, hx_bond_occupancy_one, smem)
}
void hx_bond_multi_launch_w32(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    const int nt = p.bond_nt;
    EDGPU_BOND_CASES(unsigned int, hx_bond_multi_launch_one, p, blocks, smem, st)
}
void hx_bond_multi_launch_w64(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    const int nt = p.bond_nt;
    EDGPU_BOND_CASES(unsigned long long, hx_bond_multi_launch_one, p, blocks, smem, st)
}
int hx_bond_multi_occupancy_w32(int gk, int prec, int nt, size_t smem) {
    EDGPU_BOND_CASES(unsigned int, hx_bond_multi_occupancy_one, smem)
}
int hx_bond_multi_occupancy_w64(int gk, int prec, int nt, size_t smem) {
    EDGPU_BOND_CASES(unsigned long long, hx_bond_multi_occupancy_one, smem)
}

}  // namespace edgpu
