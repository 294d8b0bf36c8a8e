// Matrix-free (symmetry-reduced) Hamiltonian application y = H x on the GPU.
//
// Replaces the row loop of apply_serial!/apply_parallel! (abstract_operator_representation.jl:296-316,
// :358-378) over get_row_iterator(::ReducedOperatorRepresentation) (reduced_operator_representation.jl:
// 57-85) and get_row_iterator(::OperatorRepresentation) (operator_representation.jl:66-79).
//
// Work decomposition.  A warp owns a tile of up to 32 consecutive rows (basis words b_r).
//  1. Each lane loads one row word, counts its stabiliser (orbit norm) and sums the diagonal terms
//     (row == col projectors) into acc[r] = E(b_r) x[r].
//  2. The (row, off-diagonal term) pairs of the tile are scanned in row-major order, 32 per step; a
//     match (b & mask == row) is compacted by warp ballot into a per-warp queue of targets
//     q = b ^ (row ^ col), so the queue stays ordered by row.
//  3. Whenever 32 targets are queued, every lane takes one: orbit minimum of q and the element h with
//     h.q = rep (recomputed, never stored), branch-free search of rep in the sorted table, gather of
//     x[c], element amp * chi(h) * sqrt(|O_r| / |O_c|), and a segmented warp scan by row that adds
//     each row's partial sum into acc[r].  The summation order is fixed: results are deterministic.
//  4. acc is written to y (coalesced); apply! semantics add the old y.
// MODE 1 also accumulates dL/dJ_c = Re <gy | H_c x> per coupling c into per-block partial sums.
#pragma once

#include "edgpu_internal.h"
#include "edgpu_device.cuh"

namespace edgpu {

template <int PREC>
struct Cx;
template <>
struct Cx<0> {
    typedef double2 V;
    typedef double R;
};
template <>
struct Cx<1> {
    typedef float2 V;
    typedef float R;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
template <typename V>
__device__ __forceinline__ V czero();
template <>
__device__ __forceinline__ double2 czero<double2>() { return make_double2(0.0, 0.0); }
template <>
__device__ __forceinline__ float2 czero<float2>() { return make_float2(0.f, 0.f); }
template <typename V>
__device__ __forceinline__ V from_d2(double2 a);
template <>
__device__ __forceinline__ double2 from_d2<double2>(double2 a) { return a; }
template <>
__device__ __forceinline__ float2 from_d2<float2>(double2 a) { return make_float2((float)a.x, (float)a.y); }
__device__ __forceinline__ double2 shfl_up_v(double2 v, int d) {
    return make_double2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
}
__device__ __forceinline__ float2 shfl_up_v(float2 v, int d) {
    return make_float2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
}

template <typename W>
__host__ __device__ constexpr int hx_warp_bytes_t() {
    return HX_QCAP * (int)sizeof(W) + HX_QCAP * 4 + 32 * 16 + 32 * 4 + 32 * 16;
}

template <typename W, int GK, int PREC, int MODE>
__global__ void __launch_bounds__(HX_THREADS) hx_kernel(const HxParams p) {
    typedef typename Cx<PREC>::V V;
    typedef typename Cx<PREC>::R R;
    extern __shared__ __align__(16) unsigned char sm[];
    {
        const int4* src = (const int4*)p.blob;
        int4* dst = (int4*)sm;
        for (int i = threadIdx.x; i < p.blob_words16; i += blockDim.x) dst[i] = src[i];
    }
    double* sgrad = (double*)(sm + p.o_grad);
    if (MODE)
        for (int i = threadIdx.x; i < p.n_coupl; i += blockDim.x) sgrad[i] = 0.0;
    __syncthreads();

    const W* om = (const W*)(sm + p.o_om);
    const W* orw = (const W*)(sm + p.o_or);
    const W* ofl = (const W*)(sm + p.o_of);
    const V* oa = (const V*)(sm + p.o_oa);
    const V* ou = (const V*)(sm + p.o_ou);
    const int* oc = (const int*)(sm + p.o_oc);
    const W* dm = (const W*)(sm + p.o_dm);
    const W* dr = (const W*)(sm + p.o_dr);
    const double2* da = (const double2*)(sm + p.o_da);
    const double2* du = (const double2*)(sm + p.o_du);
    const int* dc = (const int*)(sm + p.o_dc);
    const V* ph = (const V*)(sm + p.o_ph);
    const int* num = (const int*)(sm + p.o_num);
    const int* divi = (const int*)(sm + p.o_divi);
    const R* ratio = (const R*)(sm + p.o_ratio);
    const W* keep = (const W*)(sm + p.o_keep);
    const W* lut = (const W*)(sm + p.o_lut);
    const W* flips = (const W*)(sm + p.o_flip);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    unsigned char* ws = sm + p.warp_base + warp * hx_warp_bytes_t<W>();
    W* qs = (W*)ws;
    int* qi = (int*)(ws + HX_QCAP * sizeof(W));
    V* acc = (V*)(ws + HX_QCAP * sizeof(W) + HX_QCAP * 4);
    int* rdi = (int*)(ws + HX_QCAP * sizeof(W) + HX_QCAP * 4 + 32 * 16);
    V* gyr = (V*)(ws + HX_QCAP * sizeof(W) + HX_QCAP * 4 + 32 * 16 + 32 * 4);

    const W* __restrict__ keys = (const W*)p.keys;
    const V* __restrict__ x = (const V*)p.x;
    V* y = (V*)p.y;
    const V* gy = (const V*)p.gy;
    const int RT = p.rows_per_tile;
    const long long n_tiles = (p.n_rows + RT - 1) / RT;
    const W full = (W)p.full;
    const int T_o = p.T_o;
    const int inc_i = T_o ? 32 / T_o : 0, inc_j = T_o ? 32 % T_o : 0;

    int head = 0;
    // Process cnt queued targets, one per lane (see step 3 above).
    auto process = [&](int cnt) {
        V contrib = czero<V>();
        int myi = -1;
        if (lane < cnt) {
            const int pos = (head + lane) & (HX_QCAP - 1);
            const W q = qs[pos];
            const int info = qi[pos];
            myi = info >> 16;
            const int j = info & 0xffff;
            W rep = q;
            int g = 0, stab = 1;
            if (GK == GK_TORUS) canon_torus<W>(q, p.L1, p.L2, p.w, p.rowbits, p.nbits, full, keep, rep, g, stab);
            else if (GK == GK_GENERIC) canon_generic<W>(q, p.G, p.nchunks, lut, flips, rep, g, stab);
            const long long c = sorted_find<W>(keys, p.n_rows, rep);
            if (c >= 0) {
                V coef = oa[j];
                V phv = czero<V>();
                R f = (R)1;
                if (GK != GK_TRIVIAL) {
                    phv = ph[num[g]];
                    f = ratio[rdi[myi] * p.nd + divi[stab]];
                    coef = cscale(cmul(coef, phv), f);
                }
                const V xv = x[c];
                contrib = cmul(coef, xv);
                if (MODE) {
                    V cu = ou[j];
                    if (GK != GK_TRIVIAL) cu = cscale(cmul(cu, phv), f);
                    const V t = cmul(cu, xv);
                    const V gg = gyr[myi];
                    atomicAdd(&sgrad[oc[j]], (double)gg.x * (double)t.x + (double)gg.y * (double)t.y);
                }
            }
        }
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const V up = shfl_up_v(contrib, d);
            const int iu = __shfl_up_sync(0xffffffffu, myi, d);
            if (lane >= d && iu == myi) contrib = cadd(contrib, up);
        }
        const int inext = __shfl_down_sync(0xffffffffu, myi, 1);
        if (lane < cnt && (lane == cnt - 1 || inext != myi)) acc[myi] = cadd(acc[myi], contrib);
        __syncwarp();
    };

    for (long long tile = (long long)blockIdx.x * wpb + warp; tile < n_tiles; tile += (long long)gridDim.x * wpb) {
        const long long row0 = tile * RT;
        const int nrows = (int)min((long long)RT, p.n_rows - row0);
        const bool rowact = lane < nrows;
        const W b = rowact ? keys[row0 + lane] : (W)0;

        int stab_r = 1;
        if (GK == GK_TORUS) {
            W rp;
            int gg;
            canon_torus<W>(b, p.L1, p.L2, p.w, p.rowbits, p.nbits, full, keep, rp, gg, stab_r);
        } else if (GK == GK_GENERIC) {
            W rp;
            int gg;
            canon_generic<W>(b, p.G, p.nchunks, lut, flips, rp, gg, stab_r);
        }

        double2 e = make_double2(0.0, 0.0);
        for (int t = 0; t < p.T_d; ++t)
            if ((b & dm[t]) == dr[t]) {
                e.x += da[t].x;
                e.y += da[t].y;
            }
        const V xr = rowact ? x[row0 + lane] : czero<V>();
        acc[lane] = cmul(from_d2<V>(e), xr);
        rdi[lane] = divi[stab_r];
        if (MODE) {
            const V gv = rowact ? gy[row0 + lane] : czero<V>();
            gyr[lane] = gv;
            if (rowact)
                for (int t = 0; t < p.T_d; ++t)
                    if ((b & dm[t]) == dr[t]) {
                        const V cu = cmul(from_d2<V>(du[t]), xr);
                        atomicAdd(&sgrad[dc[t]], (double)gv.x * (double)cu.x + (double)gv.y * (double)cu.y);
                    }
        }
        __syncwarp();

        head = 0;
        int tail = 0;
        if (T_o > 0) {
            int i = lane / T_o, j = lane - (lane / T_o) * T_o;
            const int total = nrows * T_o;
            for (int p0 = 0; p0 < total; p0 += 32) {
                const bool act = (p0 + lane) < total;
                const W bi = __shfl_sync(0xffffffffu, b, i & 31);
                const bool m = act && ((bi & om[j]) == orw[j]);
                const unsigned bal = __ballot_sync(0xffffffffu, m);
                if (m) {
                    const int pos = (tail + __popc(bal & lanemask_lt())) & (HX_QCAP - 1);
                    qs[pos] = bi ^ ofl[j];
                    qi[pos] = (i << 16) | j;
                }
                tail += __popc(bal);
                j += inc_j;
                i += inc_i;
                if (j >= T_o) {
                    j -= T_o;
                    ++i;
                }
                if (tail - head >= 32) {
                    __syncwarp();
                    process(32);
                    head += 32;
                }
            }
            __syncwarp();
            while (tail > head) {
                const int cnt = min(32, tail - head);
                process(cnt);
                head += cnt;
            }
        }
        __syncwarp();
        if (rowact) {
            V v = acc[lane];
            if (p.accumulate) v = cadd(v, y[row0 + lane]);
            y[row0 + lane] = v;
        }
        __syncwarp();
    }
    if (MODE) {
        __syncthreads();
        for (int i = threadIdx.x; i < p.n_coupl; i += blockDim.x)
            p.grad_partial[(size_t)blockIdx.x * p.n_coupl + i] = sgrad[i];
    }
}

template <typename W, int GK, int PREC, int MODE>
void hx_launch_one(const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    auto kern = hx_kernel<W, GK, PREC, MODE>;
    EDGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<blocks, HX_THREADS, smem, st>>>(p);
    EDGPU_CUDA(cudaGetLastError());
}

template <typename W, int GK, int PREC, int MODE>
int hx_occupancy_one(size_t smem) {
    auto kern = hx_kernel<W, GK, PREC, MODE>;
    EDGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int n = 0;
    EDGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, HX_THREADS, smem));
    return n;
}

#define EDGPU_HX_DISPATCH(W, FN, ...)                                                        \
    switch (gk * 4 + prec * 2 + mode) {                                                      \
        case 0: return FN<W, GK_TRIVIAL, 0, 0>(__VA_ARGS__);                                 \
        case 1: return FN<W, GK_TRIVIAL, 0, 1>(__VA_ARGS__);                                 \
        case 2: return FN<W, GK_TRIVIAL, 1, 0>(__VA_ARGS__);                                 \
        case 3: return FN<W, GK_TRIVIAL, 1, 1>(__VA_ARGS__);                                 \
        case 4: return FN<W, GK_TORUS, 0, 0>(__VA_ARGS__);                                   \
        case 5: return FN<W, GK_TORUS, 0, 1>(__VA_ARGS__);                                   \
        case 6: return FN<W, GK_TORUS, 1, 0>(__VA_ARGS__);                                   \
        case 7: return FN<W, GK_TORUS, 1, 1>(__VA_ARGS__);                                   \
        case 8: return FN<W, GK_GENERIC, 0, 0>(__VA_ARGS__);                                 \
        case 9: return FN<W, GK_GENERIC, 0, 1>(__VA_ARGS__);                                 \
        case 10: return FN<W, GK_GENERIC, 1, 0>(__VA_ARGS__);                                \
        case 11: return FN<W, GK_GENERIC, 1, 1>(__VA_ARGS__);                                \
        default: throw Error(EDGPU_ERR_ARG, "bad product kernel selector");                  \
    }

}  // namespace edgpu
