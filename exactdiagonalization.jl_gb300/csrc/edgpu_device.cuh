// Device helpers shared by the enumeration and product kernels: group action on basis words
// (orbit minimum, stabiliser size, representative test) and the branch-free sorted-table search.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "edgpu_internal.h"

namespace edgpu {

// Word type of the basis table: uint32 when the state has <= 31 bits, else uint64.
template <typename W>
__device__ __forceinline__ W ldg_w(const W* p) { return __ldg(p); }

// T(a,b).q for the torus: rotate every row (rowbits wide) left by s = a*w bits.
// keep = bits at in-row positions [0, rowbits - s), replicated over the rows.
template <typename W>
__device__ __forceinline__ W torus_row_rotate(W r, int s, W keep, W full, int rowbits) {
    return (W)(((r & keep) << s) | ((r & (full ^ keep)) >> (rowbits - s)));
}

// Minimum of the orbit of q (the representative), the element g with g.q == rep that is found
// first, and the stabiliser size |{g : g.q == q}|.
// TORUS: loop over row shifts b (rotate the word by rowbits) and in-row shifts a.
template <typename W>
__device__ __forceinline__ void canon_torus(W q, int L1, int L2, int w, int rowbits, int nbits, W full,
                                            const W* keep, W& rep, int& gbest, int& stab) {
    rep = q;
    gbest = 0;
    stab = 0;
    W r = q;
    for (int b = 0; b < L2; ++b) {
        for (int a = 0; a < L1; ++a) {
            const W t = torus_row_rotate<W>(r, a * w, keep[a], full, rowbits);
            if (t < rep) { rep = t; gbest = a + L1 * b; }
            stab += (t == q);
        }
        r = (W)(((r << rowbits) | (r >> (nbits - rowbits))) & full);
    }
}

// GENERIC: g.q = OR_c lut[g][c][nibble_c(q)] XOR flips[g].
template <typename W>
__device__ __forceinline__ W generic_apply(W q, int g, int nchunks, const W* lut, const W* flips) {
    W t = 0;
    const W* L = lut + (size_t)g * nchunks * 16;
#pragma unroll 4
    for (int c = 0; c < nchunks; ++c) t |= L[c * 16 + (int)((q >> (4 * c)) & 15u)];
    return t ^ flips[g];
}

template <typename W>
__device__ __forceinline__ void canon_generic(W q, int G, int nchunks, const W* lut, const W* flips, W& rep,
                                              int& gbest, int& stab) {
    rep = q;
    gbest = 0;
    stab = 0;
    for (int g = 0; g < G; ++g) {
        const W t = generic_apply<W>(q, g, nchunks, lut, flips);
        if (t < rep) { rep = t; gbest = g; }
        stab += (t == q);
    }
}

// Representative test of symmetry_reduce_generic.jl:55-69: q is kept iff no element maps it to a
// smaller word and every element fixing q has character 1 (exact: num == 0 mod den).
template <typename W>
__device__ __forceinline__ bool is_rep_torus(W q, int L1, int L2, int w, int rowbits, int nbits, W full,
                                             const W* keep, const int32_t* num) {
    W r = q;
    for (int b = 0; b < L2; ++b) {
        for (int a = 0; a < L1; ++a) {
            if (a == 0 && b == 0) continue;
            const W t = torus_row_rotate<W>(r, a * w, keep[a], full, rowbits);
            if (t < q) return false;
            if (t == q && num[a + L1 * b] != 0) return false;
        }
        r = (W)(((r << rowbits) | (r >> (nbits - rowbits))) & full);
    }
    return true;
}

template <typename W>
__device__ __forceinline__ bool is_rep_generic(W q, int G, int nchunks, const W* lut, const W* flips,
                                               const int32_t* num) {
    for (int g = 1; g < G; ++g) {
        const W t = generic_apply<W>(q, g, nchunks, lut, flips);
        if (t < q) return false;
        if (t == q && num[g] != 0) return false;
    }
    return true;
}

// Branch-free search of a sorted table: the iteration count depends on n only, so the lanes of a
// warp stay converged.  Returns the index of key or -1 (get(FrozenSortedArrayIndex, key, -1)).
template <typename W>
__device__ __forceinline__ long long sorted_find(const W* __restrict__ keys, long long n, W key) {
    long long lo = 0, len = n;
    while (len > 1) {
        const long long half = len >> 1;
        lo = (ldg_w(keys + lo + half) <= key) ? lo + half : lo;
        len -= half;
    }
    return (n > 0 && ldg_w(keys + lo) == key) ? lo : -1;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Block-wide exclusive scan of one int64 per thread (blockDim.x <= 1024, multiple of 32).
// tmp: shared array of at least 32 long longs.  Returns the exclusive prefix; *total = block sum.
__device__ __forceinline__ long long block_exclusive_scan(long long v, long long* tmp, long long* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    long long inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const long long u = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += u;
    }
    if (lane == 31) tmp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        long long s = (lane < nw) ? tmp[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const long long u = __shfl_up_sync(0xffffffffu, s, d);
            if (lane >= d) s += u;
        }
        if (lane < nw) tmp[lane] = s;   // inclusive warp totals
    }
    __syncthreads();
    const long long warp_off = (warp > 0) ? tmp[warp - 1] : 0;
    const long long res = warp_off + inc - v;
    if (total) *total = tmp[nw - 1];
    __syncthreads();
    return res;
}

}  // namespace edgpu
