// Matrix-free (symmetry-reduced) Hamiltonian application y = H x on the GPU.
//
// Replaces the row loop of apply_serial!/apply_parallel! (abstract_operator_representation.jl:296-316,
// :358-378) over get_row_iterator(::ReducedOperatorRepresentation) (reduced_operator_representation.jl:
// 57-85) and get_row_iterator(::OperatorRepresentation) (operator_representation.jl:66-79).
//
// Work decomposition.  A warp owns a tile of up to 32 consecutive rows (keys of representatives).
//  1. Each lane loads one row key (state + orbit-size index) and the row's diagonal element E(b_r)
//     (sum of the row == col projector terms, precomputed once per operator) into acc[r] = E x[r].
//  2. The (row, off-diagonal term) pairs of the tile are scanned in row-major order, 32 per step; a
//     match (b & mask == row) is compacted by warp ballot into a per-warp queue of targets
//     q = b ^ (row ^ col), so the queue stays ordered by row.
//  3. Whenever 64 targets are queued, every lane takes two: orbit minimum of q and the element h with
//     h.q = rep (recomputed, never stored), bucketed branch-free search of rep (one directory load,
//     then a few probes inside the bucket), gather of x[c], element amp * chi(h) * sqrt(|O_r| / |O_c|), and a segmented warp scan by
//     row that adds each row's partial sum into acc[r].  The summation order is fixed: results are
//     deterministic run to run.
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
__device__ __forceinline__ double2 make_conj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ float2 make_conj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
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
__device__ __forceinline__ double2 shfl_xor_v(double2 v, int d) {
    return make_double2(__shfl_xor_sync(0xffffffffu, v.x, d), __shfl_xor_sync(0xffffffffu, v.y, d));
}
__device__ __forceinline__ float2 shfl_xor_v(float2 v, int d) {
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, d), __shfl_xor_sync(0xffffffffu, v.y, d));
}

// One off-diagonal term record (mask, row, row^col) from shared memory in a single vector load.
template <typename W>
__device__ __forceinline__ void load_rec3(const W* r, W& m, W& row, W& f);
template <>
__device__ __forceinline__ void load_rec3<unsigned int>(const unsigned int* r, unsigned int& m, unsigned int& row,
                                                        unsigned int& f) {
    const uint4 v = *(const uint4*)r;
    m = v.x;
    row = v.y;
    f = v.z;
}
template <>
__device__ __forceinline__ void load_rec3<unsigned long long>(const unsigned long long* r, unsigned long long& m,
                                                              unsigned long long& row, unsigned long long& f) {
    const ulonglong2 a = *(const ulonglong2*)r;
    m = a.x;
    row = a.y;
    f = r[2];
}

template <typename W>
__host__ __device__ constexpr int hx_warp_bytes_t() {
    return HX_QCAP * (int)sizeof(W) + HX_QCAP * 4 + 32 * 16 + 32 * 4 + 32 * 16;
}

// Orbit minimum of q and the element reaching it, for each group kind.
template <typename W, int GK>
__device__ __forceinline__ void canon_rep(W q, const HxParams& p, const W* keep, const W* lut, const W* flips,
                                          const unsigned* rlut, const unsigned* keep32, W& rep, int& g) {
    if (GK == GK_TRIVIAL) {
        rep = q;
        g = 0;
    } else if (GK == GK_RING) {
        unsigned r;
        canon_ring((unsigned)q, p.nbits, p.L1, p.w, p.pb, p.want_arg != 0, r, g);
        rep = (W)r;
    } else if (GK == GK_TORUS) {
        if (p.o_rlut >= 0 && p.rlut_pair) {
            canon_torus_pair<W>(q, p.L1, p.L2, p.w, p.rowbits, p.nbits, (W)p.full, (const W*)keep32, keep, rlut, rep, g);
        } else if (p.o_rlut >= 0) {
            canon_torus_pruned<W>(q, p.L1, p.L2, p.w, p.rowbits, p.nbits, (W)p.full, keep, rlut, p.l1inv, rep, g);
        } else {
            int s;
            canon_torus<W>(q, p.L1, p.L2, p.w, p.rowbits, p.nbits, (W)p.full, keep, p.want_arg != 0, false, rep, g, s);
        }
    } else {
        int s;
        canon_generic<W>(q, p.G, p.nchunks, lut, flips, false, rep, g, s);
    }
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

    const W* orec = (const W*)(sm + p.o_om);   // off-diagonal term t: orec[4t] mask, [4t+1] row, [4t+2] row^col
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
    const R* ratio = (const R*)(sm + p.o_ratio);
    const W* keep = (const W*)(sm + p.o_keep);
    const W* lut = p.o_lut >= 0 ? (const W*)(sm + p.o_lut) : (const W*)p.lut_g;
    const W* flips = (const W*)(sm + p.o_flip);
    const unsigned* rlut = (const unsigned*)(sm + (p.o_rlut >= 0 ? p.o_rlut : 0));
    const unsigned* keep32 = (const unsigned*)(sm + p.o_keep32);

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
    const int sb = p.sb;
    const W smask = (W)((((W)1) << sb) - 1);
    const int T_o = p.T_o;
    const int inc_i = T_o ? 32 / T_o : 0, inc_j = T_o ? 32 % T_o : 0;
    const bool want_arg = p.want_arg != 0;

    int head = 0;
    // Process cnt (<= 64) queued targets (step 3 above): lane handles entries lane and lane + 32, whose
    // searches and gathers overlap.  Each half of the batch is a row-ordered run of the queue.
    auto process = [&](int cnt) {
        V contrib[2];
        int myi[2], jj[2], g[2];
        W q[2], rep[2];
        bool act[2];
        long long c[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int e = lane + 32 * h;
            contrib[h] = czero<V>();
            act[h] = e < cnt;
            myi[h] = -1;
            jj[h] = 0;
            q[h] = 0;
            g[h] = 0;
            if (act[h]) {
                const int pos = (head + e) & (HX_QCAP - 1);
                q[h] = qs[pos];
                const int info = qi[pos];
                myi[h] = info >> 16;
                jj[h] = info & 0xffff;
            }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            rep[h] = q[h];
            if (act[h]) canon_rep<W, GK>(q[h], p, keep, lut, flips, rlut, keep32, rep[h], g[h]);
        }
        int sx[2];
        key_find_sum2<W>(keys, p.ds, rep, act, c, sx);
        V xv[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) xv[h] = (c[h] >= 0) ? x[c[h]] : czero<V>();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (c[h] >= 0) {
                V coef = oa[jj[h]];
                V phv = czero<V>();
                R f = (R)1;
                if (GK != GK_TRIVIAL) {
                    f = ratio[rdi[myi[h]] * p.nd + sx[h]];
                    if (want_arg) {
                        phv = ph[num[g[h]]];
                        coef = cmul(coef, phv);
                    }
                    coef = cscale(coef, f);
                }
                contrib[h] = cmul(coef, xv[h]);
                if (MODE) {
                    V cu = ou[jj[h]];
                    if (GK != GK_TRIVIAL) {
                        if (want_arg) cu = cmul(cu, phv);
                        cu = cscale(cu, f);
                    }
                    const V t = cmul(cu, xv[h]);
                    const V gg = gyr[myi[h]];
                    atomicAdd(&sgrad[oc[jj[h]]], (double)gg.x * (double)t.x + (double)gg.y * (double)t.y);
                }
            }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const V up = shfl_up_v(contrib[h], d);
                const int iu = __shfl_up_sync(0xffffffffu, myi[h], d);
                if (lane >= d && iu == myi[h]) contrib[h] = cadd(contrib[h], up);
            }
            const int inext = __shfl_down_sync(0xffffffffu, myi[h], 1);
            const int e = lane + 32 * h;
            if (act[h] && (lane == 31 || e == cnt - 1 || inext != myi[h])) acc[myi[h]] = cadd(acc[myi[h]], contrib[h]);
            __syncwarp();
        }
    };

    for (long long tile = (long long)blockIdx.x * wpb + warp; tile < n_tiles; tile += (long long)gridDim.x * wpb) {
        const long long row0 = tile * RT;
        const int nrows = (int)min((long long)RT, p.n_rows - row0);
        const bool rowact = lane < nrows;
        const W kr = rowact ? keys[row0 + lane] : (W)0;
        const W b = kr >> sb;

        const V xr = rowact ? x[row0 + lane] : czero<V>();
        if (MODE == 0) {
            const V* dtab = (const V*)p.diag;
            acc[lane] = rowact ? cmul(dtab[row0 + lane], xr) : czero<V>();
        } else {
            double2 e = make_double2(0.0, 0.0);
            for (int t = 0; t < p.T_d; ++t)
                if ((b & dm[t]) == dr[t]) {
                    e.x += da[t].x;
                    e.y += da[t].y;
                }
            acc[lane] = cmul(from_d2<V>(e), xr);
        }
        rdi[lane] = (int)(kr & smask);
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
                W tm, tr, tf;
                load_rec3<W>(orec + 4 * j, tm, tr, tf);
                const bool m = act && ((bi & tm) == tr);
                const unsigned bal = __ballot_sync(0xffffffffu, m);
                if (m) {
                    const int pos = (tail + __popc(bal & lanemask_lt())) & (HX_QCAP - 1);
                    qs[pos] = bi ^ tf;
                    qi[pos] = (i << 16) | j;
                }
                tail += __popc(bal);
                j += inc_j;
                i += inc_i;
                if (j >= T_o) {
                    j -= T_o;
                    ++i;
                }
                if (tail - head >= 64) {
                    __syncwarp();
                    process(64);
                    head += 64;
                }
            }
            __syncwarp();
            while (tail > head) {
                const int cnt = min(64, tail - head);
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
    raise_smem_limit((const void*)kern, smem);
    kern<<<blocks, HX_THREADS, smem, st>>>(p);
    EDGPU_CUDA(cudaGetLastError());
}

template <typename W, int GK, int PREC, int MODE>
int hx_occupancy_one(size_t smem) {
    auto kern = hx_kernel<W, GK, PREC, MODE>;
    raise_smem_limit((const void*)kern, smem);
    int n = 0;
    EDGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, HX_THREADS, smem));
    return n;
}

#define EDGPU_HX_CASES(W, GKV, FN, ...)                                                      \
    case GKV * 4 + 0: return FN<W, GKV, 0, 0>(__VA_ARGS__);                                  \
    case GKV * 4 + 1: return FN<W, GKV, 0, 1>(__VA_ARGS__);                                  \
    case GKV * 4 + 2: return FN<W, GKV, 1, 0>(__VA_ARGS__);                                  \
    case GKV * 4 + 3: return FN<W, GKV, 1, 1>(__VA_ARGS__);

}  // namespace edgpu
