// Row-per-lane strategy of the matrix-free product y = H x (same result as hx_kernel, other schedule);
// lpr = 1, 2 or 4 lanes may share a row, each taking every lpr-th term.
//
// Replaces the same reference loop as hx_kernel.cuh (apply_serial!/apply_parallel! over
// get_row_iterator, abstract_operator_representation.jl:296-316, reduced_operator_representation.jl:
// 57-85).  Every lane owns one row: it reads the row's key and diagonal element, tests its state
// against the off-diagonal term records (broadcast shared-memory loads) into a bitmask of matching
// terms, then walks its matches two at a time: orbit minimum and element of each target, the two
// bucketed searches in lockstep, gathers, and accumulation in registers in term order (the order of
// the reference's row iterator).  No queue and no cross-lane reduction: the warp runs as long as its
// busiest row, which costs less than the bookkeeping when rows have similar numbers of targets.
#pragma once

#include "hx_kernel.cuh"

namespace edgpu {

// Shared-memory views of the tables of one product launch (common to all sectors of a batch).
template <typename W, int PREC>
struct RowsTables {
    typedef typename Cx<PREC>::V V;
    typedef typename Cx<PREC>::R R;
    const W *orec, *dm, *dr, *keep, *lut, *flips;
    const V *oa, *ou;
    const int *oc, *dc;
    const double2 *da, *du;
    const R* ratio;
    const unsigned* rlut;
    const unsigned* keep32;
    __device__ __forceinline__ RowsTables(const HxParams& p, const unsigned char* sm) {
        orec = (const W*)(sm + p.o_om);
        oa = (const V*)(sm + p.o_oa);
        ou = (const V*)(sm + p.o_ou);
        oc = (const int*)(sm + p.o_oc);
        dm = (const W*)(sm + p.o_dm);
        dr = (const W*)(sm + p.o_dr);
        da = (const double2*)(sm + p.o_da);
        du = (const double2*)(sm + p.o_du);
        dc = (const int*)(sm + p.o_dc);
        ratio = (const R*)(sm + p.o_ratio);
        keep = (const W*)(sm + p.o_keep);
        lut = p.o_lut >= 0 ? (const W*)(sm + p.o_lut) : (const W*)p.lut_g;
        flips = (const W*)(sm + p.o_flip);
        rlut = (const unsigned*)(sm + (p.o_rlut >= 0 ? p.o_rlut : 0));
        keep32 = (const unsigned*)(sm + p.o_keep32);
    }
};

// The sector a warp tile belongs to: its basis table, search directory, vectors, diagonal and
// character table.
template <int PREC>
struct RowsSector {
    typedef typename Cx<PREC>::V V;
    const void* keys;
    const V* x;
    V* y;
    const V* diag;
    long long n_rows;
    DirSearch ds;
    const V* ph;
    const int* num;
    bool want_arg;
    const void* map;   // parent-state map (null: canonicalise and search)
    int map_wide, map_cb, map_direct;
    // target table of the pair-flip schedule (GK_TABLE): the map-format entry of every (row, target),
    // rows in warp tiles of 32, each tile's entries from tile_off[tile], row after row
    const void* tab;
    const long long* tile_off;
    int tab_wide, tab_cb;
};

// Colex rank of a state with rank_k set bits among the parent's bits: sum over 6-bit chunks of the
// chunk table entry for (chunk, set bits below the chunk, chunk value).  The chunk loop is unrolled
// (constant shifts) and skips the chunks past the parent's bits; T is the table entry type (uint32 when
// every rank fits in 32 bits).
template <typename T, typename W>
__device__ __forceinline__ T colex_rank_t(W q, const T* __restrict__ tab, unsigned k1x64, int nc) {
    T r = 0;
    unsigned base = 0u, ones64 = 0u;
#pragma unroll
    for (int c = 0; c < (int)(8 * sizeof(W) + RANK_CHUNK - 1) / RANK_CHUNK; ++c) {
        if (c < nc) {
            const unsigned v = (unsigned)(q >> (RANK_CHUNK * c)) & 63u;
            r += __ldg(tab + (base + ones64 + v));
            ones64 += (unsigned)__popc(v) << 6;
            base += k1x64;
        }
    }
    return r;
}

// Row c of the representative of a target q in the sector's table (-1: its orbit has no
// representative there), the representative's orbit-size index sx and the group element g reaching
// it, through the parent-state map: the entry of q (indexed by q itself for a direct map, else by its
// colex rank among the parent's states) packs c | sx << map_cb | g << (map_cb + sb).
template <typename W, int PREC>
__device__ __forceinline__ void map_lookup(const HxParams& p, const RowsSector<PREC>& sc, W q, bool on, long long& c,
                                           int& sx, int& g) {
    const unsigned long long cmask = (1ull << sc.map_cb) - 1ull;
    unsigned long long e = ~0ull;
    if (sc.map_direct) {
        // direct map: every state of the parent's bits has an entry (invalid: all ones)
        if (on)
            e = sc.map_wide ? __ldg((const unsigned long long*)sc.map + (unsigned long long)q)
                            : (unsigned long long)__ldg((const unsigned*)sc.map + (unsigned long long)q);
    } else if (on && __popcll((unsigned long long)q) == p.rank_k) {
        unsigned long long r;
        if (p.rank_split) {
            // split tables: rank = A[high part] + B[low part] (entries of the same width)
            const unsigned long long qq = (unsigned long long)q;
            const unsigned long long hi = qq >> p.rank_split;
            const unsigned long long lo = qq & ((1ull << p.rank_split) - 1ull);
            const unsigned long long nb_a = 1ull << (p.nbits - p.rank_split);
            r = p.rank_wide ? __ldg((const unsigned long long*)p.rank_tab + hi) +
                                  __ldg((const unsigned long long*)p.rank_tab + nb_a + lo)
                            : (unsigned long long)__ldg((const unsigned*)p.rank_tab + hi) +
                                  (unsigned long long)__ldg((const unsigned*)p.rank_tab + nb_a + lo);
        } else {
            const unsigned k1x64 = ((unsigned)p.rank_k + 1u) << 6;
            r = p.rank_wide ? colex_rank_t<unsigned long long, W>(q, (const unsigned long long*)p.rank_tab, k1x64,
                                                                  p.rank_nc)
                            : (unsigned long long)colex_rank_t<unsigned, W>(q, (const unsigned*)p.rank_tab, k1x64,
                                                                            p.rank_nc);
        }
        e = sc.map_wide ? __ldg((const unsigned long long*)sc.map + r) : (unsigned long long)__ldg((const unsigned*)sc.map + r);
    }
    const unsigned long long ci = e & cmask;
    c = (ci == cmask) ? -1 : (long long)ci;
    sx = (int)((e >> sc.map_cb) & ((1ull << p.sb) - 1ull));
    g = (int)(e >> (sc.map_cb + p.sb)) & 0xfff;
}

// Resolve two targets q[0..1] (on[h]: the slot holds a target): row c[h] (-1: none), orbit-size
// index sx[h] and group element g[h], by the parent-state map (GK_MAP) or by canonicalisation to the
// orbit minimum and the bucketed search of the sector's table (both searches in lockstep).
template <typename W, int GK, int PREC>
__device__ __forceinline__ void resolve_targets2(const HxParams& p, const RowsTables<W, PREC>& tb,
                                                 const RowsSector<PREC>& sc, const W* q, const bool* on, long long* c,
                                                 int* sx, int* g) {
    if constexpr (GK == GK_MAP) {
#pragma unroll
        for (int h = 0; h < 2; ++h) map_lookup<W, PREC>(p, sc, q[h], on[h], c[h], sx[h], g[h]);
    } else {
        W rep[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            rep[h] = q[h];
            g[h] = 0;
            if (on[h]) canon_rep<W, GK>(q[h], p, tb.keep, tb.lut, tb.flips, tb.rlut, tb.keep32, rep[h], g[h]);
        }
        key_find_sum2<W>((const W*)sc.keys, sc.ds, rep, on, c, sx);
    }
}

// One warp tile of rows (rows_per_tile = 32 / lpr consecutive rows of the sector, lpr lanes each).
template <typename W, int GK, int PREC, int MODE>
__device__ __forceinline__ void rows_tile(const HxParams& p, const RowsTables<W, PREC>& tb, const RowsSector<PREC>& sc,
                                          long long tile, int lane, double* sgrad) {
    typedef typename Cx<PREC>::V V;
    typedef typename Cx<PREC>::R R;
    const W* __restrict__ keys = (const W*)sc.keys;
    const V* __restrict__ x = sc.x;
    const int sb = p.sb;
    const W smask = (W)((((W)1) << sb) - 1);
    const int T_o = p.T_o;
    // lpr lanes share a row: lane sub = lane % lpr takes the terms t with t % lpr == sub
    const int lpr = p.lpr, sub = lane & (lpr - 1), rpw = 32 / lpr;
    const long long row = tile * rpw + lane / lpr;
    const bool act = row < sc.n_rows;
    const W kr = act ? keys[row] : (W)0;
    const W b = kr >> sb;
    const int ri = (int)(kr & smask);
    const V xr = act ? x[row] : czero<V>();
    V acc = czero<V>();
    V gv = czero<V>();
    if (MODE == 0) {
        if (act && sub == 0) acc = cmul(sc.diag[row], xr);
    } else {
        // forward diagonal from the diagonal table; the gradient's diagonal part scans the row == col
        // terms, forms each contribution Re(conj(gy_r) u_t x_r) in the product's precision and adds it
        // to the coupling's FP64 accumulator
        gv = act ? ((const V*)p.gy)[row] : czero<V>();
        if (act && sub == 0) {
            acc = cmul(sc.diag[row], xr);
            for (int t = 0; t < p.T_d; ++t)
                if ((b & tb.dm[t]) == tb.dr[t]) {
                    const V cu = cmul(from_d2<V>(tb.du[t]), xr);
                    sgrad[tb.dc[t] * HX_THREADS + threadIdx.x] += (double)(gv.x * cu.x + gv.y * cu.y);
                }
        }
    }
    // this lane's terms: t = sub + lpr * k, in chunks of 64
    const int my_terms = (T_o - sub + lpr - 1) / lpr;
    for (int k0 = 0; k0 < my_terms; k0 += 64) {
        const int kn = min(64, my_terms - k0);
        unsigned long long mm = 0ull;
        for (int k = 0; k < kn; ++k) {
            W tm, tr, tf;
            load_rec3<W>(tb.orec + 4 * (sub + lpr * (k0 + k)), tm, tr, tf);
            mm |= (unsigned long long)((b & tm) == tr) << k;
        }
        if (!act) mm = 0ull;
        constexpr int NT = 2;   // targets per lane and step (the search takes two in lockstep)
        while (__any_sync(0xffffffffu, mm != 0ull)) {
            int tt[NT];
            bool on[NT];
            W q[NT];
            int g[NT];
            long long c[NT];
            int sx[NT];
#pragma unroll
            for (int h = 0; h < NT; ++h) {
                on[h] = mm != 0ull;
                tt[h] = on[h] ? sub + lpr * (k0 + __ffsll((long long)mm) - 1) : 0;
                mm &= mm - 1ull;
                W tm, tr, tf;
                load_rec3<W>(tb.orec + 4 * tt[h], tm, tr, tf);
                q[h] = b ^ tf;
            }
            resolve_targets2<W, GK, PREC>(p, tb, sc, q, on, c, sx, g);
            V xv[NT];
#pragma unroll
            for (int h = 0; h < NT; ++h) xv[h] = (c[h] >= 0) ? x[c[h]] : czero<V>();
#pragma unroll
            for (int h = 0; h < NT; ++h) {
                if (c[h] >= 0) {
                    V coef = tb.oa[tt[h]];
                    V phv = czero<V>();
                    R f = (R)1;
                    if (GK != GK_TRIVIAL) {
                        f = tb.ratio[ri * p.nd + sx[h]];
                        if (sc.want_arg) {
                            phv = sc.ph[sc.num[g[h]]];
                            coef = cmul(coef, phv);
                        }
                        coef = cscale(coef, f);
                    }
                    acc = cadd(acc, cmul(coef, xv[h]));
                    if (MODE) {
                        V cu = tb.ou[tt[h]];
                        if (GK != GK_TRIVIAL) {
                            if (sc.want_arg) cu = cmul(cu, phv);
                            cu = cscale(cu, f);
                        }
                        const V t = cmul(cu, xv[h]);
                        sgrad[tb.oc[tt[h]] * HX_THREADS + threadIdx.x] += (double)(gv.x * t.x + gv.y * t.y);
                    }
                }
            }
        }
    }
    // partial sums of the row's lanes (fixed butterfly order)
    for (int d = 1; d < lpr; d <<= 1) acc = cadd(acc, shfl_xor_v(acc, d));
    if (act && sub == 0) {
        if (p.accumulate) acc = cadd(acc, sc.y[row]);
        sc.y[row] = acc;
    }
}

template <typename W, int GK, int PREC, int MODE>
__global__ void __launch_bounds__(HX_THREADS) hx_rows_kernel(const HxParams p) {
    typedef typename Cx<PREC>::V V;
    extern __shared__ __align__(16) unsigned char sm[];
    {
        const int4* src = (const int4*)p.blob;
        int4* dst = (int4*)sm;
        for (int i = threadIdx.x; i < p.blob_words16; i += blockDim.x) dst[i] = src[i];
    }
    // gradient mode: one FP64 accumulator per coupling and thread ([coupling][thread]), reduced per
    // block in a fixed order at the end (no atomics)
    double* sgrad = (double*)(sm + p.o_grad);
    if (MODE)
        for (int i = threadIdx.x; i < p.n_coupl * HX_THREADS; i += blockDim.x) sgrad[i] = 0.0;
    __syncthreads();

    const RowsTables<W, PREC> tb(p, sm);
    RowsSector<PREC> sc;
    sc.keys = p.keys;
    sc.x = (const V*)p.x;
    sc.y = (V*)p.y;
    sc.diag = (const V*)p.diag;
    sc.n_rows = p.n_rows;
    sc.ds = p.ds;
    sc.ph = (const V*)(sm + p.o_ph);
    sc.num = (const int*)(sm + p.o_num);
    sc.want_arg = p.want_arg != 0;
    sc.map = p.map;
    sc.map_wide = p.map_wide;
    sc.map_cb = p.map_cb;
    sc.map_direct = p.map_direct;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const int rpw = 32 / p.lpr;
    const long long n_tiles = (p.n_rows + rpw - 1) / rpw;
    for (long long tile = (long long)blockIdx.x * wpb + warp; tile < n_tiles; tile += (long long)gridDim.x * wpb)
        rows_tile<W, GK, PREC, MODE>(p, tb, sc, tile, lane, sgrad);
    if (MODE) {
        __syncthreads();
        for (int i = threadIdx.x; i < p.n_coupl; i += blockDim.x) {
            double sum = 0.0;
            for (int t = 0; t < HX_THREADS; ++t) sum += sgrad[i * HX_THREADS + t];
            p.grad_partial[(size_t)blockIdx.x * p.n_coupl + i] = sum;
        }
    }
}

// Batched sectors in one persistent launch: the warp tiles of all sectors are numbered one after the
// other (sector s owns tiles [tile_end[s-1], tile_end[s])), and the grid strides over them.  Each
// warp's tiles increase, so its sector index only moves forward.  The common term and group tables
// and each sector's descriptor and character table are staged in shared memory once per block.
template <typename W, int GK, int PREC>
__global__ void __launch_bounds__(HX_THREADS) hx_multi_kernel(const HxParams p) {
    typedef typename Cx<PREC>::V V;
    extern __shared__ __align__(16) unsigned char sm[];
    {
        const int4* src = (const int4*)p.blob;
        int4* dst = (int4*)sm;
        for (int i = threadIdx.x; i < p.blob_words16; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const RowsTables<W, PREC> tb(p, sm);
    const SectorDesc* sec = (const SectorDesc*)(sm + p.o_sec);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    int s = 0;
    long long tile0 = 0;   // first tile of sector s
    for (long long tile = (long long)blockIdx.x * wpb + warp; tile < p.n_tiles; tile += (long long)gridDim.x * wpb) {
        while (s + 1 < p.n_sec && tile >= sec[s].tile_end) {
            tile0 = sec[s].tile_end;
            ++s;
        }
        const SectorDesc& d = sec[s];
        RowsSector<PREC> sc;
        sc.keys = d.keys;
        sc.x = (const V*)d.x;
        sc.y = (V*)d.y;
        sc.diag = (const V*)d.diag;
        sc.n_rows = d.n_rows;
        sc.ds = d.ds;
        sc.ph = (const V*)(sm + d.o_ph);
        sc.num = (const int*)(sm + d.o_num);
        sc.want_arg = d.want_arg != 0;
        sc.map = d.map;
        sc.map_wide = d.map_wide;
        sc.map_cb = d.map_cb;
        sc.map_direct = d.map_direct;
        rows_tile<W, GK, PREC, 0>(p, tb, sc, tile - tile0, lane, nullptr);
    }
}

// Adjoint of the product's matrix by scatter, for terms that do not commute with the group (where the
// reduced row and column iterators are not transposes of each other): one thread per row r adds
// conj(H[r, c]) x[r] into y[c] for every target c of the row, and conj(E_r) x[r] into y[r], by atomic
// adds.  The elements are formed exactly as in the product (rows_tile).
template <typename W, int GK, int PREC>
__global__ void __launch_bounds__(HX_THREADS) hx_scatter_adjoint_kernel(const HxParams p) {
    typedef typename Cx<PREC>::V V;
    typedef typename Cx<PREC>::R R;
    extern __shared__ __align__(16) unsigned char sm[];
    {
        const int4* src = (const int4*)p.blob;
        int4* dst = (int4*)sm;
        for (int i = threadIdx.x; i < p.blob_words16; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const RowsTables<W, PREC> tb(p, sm);
    const W* __restrict__ keys = (const W*)p.keys;
    const V* ph = (const V*)(sm + p.o_ph);
    const int* num = (const int*)(sm + p.o_num);
    const V* xin = (const V*)p.gy;
    R* yout = (R*)p.y;
    const int sb = p.sb;
    const W smask = (W)((((W)1) << sb) - 1);
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < p.n_rows;
         r += (long long)gridDim.x * blockDim.x) {
        const W kr = keys[r];
        const W b = kr >> sb;
        const int ri = (int)(kr & smask);
        const V xr = xin[r];
        {
            const V d = ((const V*)p.diag)[r];
            const V t = cmul(make_conj(d), xr);
            atomicAdd(yout + 2 * r, t.x);
            atomicAdd(yout + 2 * r + 1, t.y);
        }
        for (int k = 0; k < p.T_o; ++k) {
            W tm, tr, tf;
            load_rec3<W>(tb.orec + 4 * k, tm, tr, tf);
            if ((b & tm) != tr) continue;
            const W q = b ^ tf;
            W rep[2] = {q, q};
            int g = 0;
            canon_rep<W, GK>(q, p, tb.keep, tb.lut, tb.flips, tb.rlut, tb.keep32, rep[0], g);
            const bool act[2] = {true, false};
            long long c[2];
            int sx[2];
            key_find_sum2<W>(keys, p.ds, rep, act, c, sx);
            if (c[0] < 0) continue;
            V coef = tb.oa[k];
            if (GK != GK_TRIVIAL) {
                if (p.want_arg) coef = cmul(coef, ph[num[g]]);
                coef = cscale(coef, tb.ratio[ri * p.nd + sx[0]]);
            }
            const V t = cmul(make_conj(coef), xr);
            atomicAdd(yout + 2 * c[0], t.x);
            atomicAdd(yout + 2 * c[0] + 1, t.y);
        }
    }
}

template <typename W, int GK, int PREC>
void hx_scatter_launch_one(const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    auto kern = hx_scatter_adjoint_kernel<W, GK, PREC>;
    raise_smem_limit((const void*)kern, smem);
    kern<<<blocks, HX_THREADS, smem, st>>>(p);
    EDGPU_CUDA(cudaGetLastError());
}

// Sparse assembly of the representation in FP64 (sparse(opr) and get_row,
// abstract_operator_representation.jl:135-213): one warp per row.  The lanes evaluate the row's
// off-diagonal terms (term t in slot t, no match: column -1) and lane 0 adds the diagonal in slot
// T_o; lane 0 then merges the slots into a list sorted by column, summing entries of equal column,
// and drops entries with |value| < tol (choptol!, util.jl:88-94).  Count pass (row_ptr == null):
// counts[row] = entries; fill pass: entries written at row_ptr[row], optionally conjugated.
constexpr int SPARSE_THREADS = 128;

template <typename W, int GK>
__global__ void __launch_bounds__(SPARSE_THREADS) hx_sparse_kernel(const HxParams p, long long row0, long long n_run,
                                                                 int conj_vals, double tol, long long* counts,
                                                                 const long long* row_ptr, long long* cols,
                                                                 double2* vals) {
    extern __shared__ __align__(16) unsigned char sm[];
    {
        const int4* src = (const int4*)p.blob;
        int4* dst = (int4*)sm;
        for (int i = threadIdx.x; i < p.blob_words16; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const RowsTables<W, 0> tb(p, sm);
    const W* __restrict__ keys = (const W*)p.keys;
    const double2* ph = (const double2*)(sm + p.o_ph);
    const int* num = (const int*)(sm + p.o_num);
    const int T1 = p.T_o + 1;
    const int T1p = (T1 + 1) & ~1;   // even, so that every double2 array below starts on 16 bytes
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    // per-warp scratch after the tables (warp_base is 16-byte aligned): slots (column, value), then
    // the merged list; sizes in units of T1p entries: 8 + 16 + 8 + 16 = 48 bytes
    unsigned char* base = sm + p.warp_base + (size_t)warp * (size_t)T1p * 48;
    long long* sc = (long long*)base;
    double2* sv = (double2*)(base + (size_t)T1p * 8);
    long long* lc = (long long*)(base + (size_t)T1p * 24);
    double2* lv = (double2*)(base + (size_t)T1p * 32);
    const int sb = p.sb;
    const W smask = (W)((((W)1) << sb) - 1);
    for (long long rr = (long long)blockIdx.x * wpb + warp; rr < n_run; rr += (long long)gridDim.x * wpb) {
        const long long row = row0 + rr;
        const W kr = keys[row];
        const W b = kr >> sb;
        const int ri = (int)(kr & smask);
        for (int t = lane; t < p.T_o; t += 32) {
            W tm, tr, tf;
            load_rec3<W>(tb.orec + 4 * t, tm, tr, tf);
            long long c = -1;
            double2 v = make_double2(0.0, 0.0);
            if ((b & tm) == tr) {
                const W q = b ^ tf;
                W rep[2] = {q, q};
                int g = 0;
                canon_rep<W, GK>(q, p, tb.keep, tb.lut, tb.flips, tb.rlut, tb.keep32, rep[0], g);
                const bool act[2] = {true, false};
                long long cc[2];
                int sx[2];
                key_find_sum2<W>(keys, p.ds, rep, act, cc, sx);
                if (cc[0] >= 0) {
                    c = cc[0];
                    v = tb.oa[t];
                    if (GK != GK_TRIVIAL) {
                        if (p.want_arg) v = cmul(v, ph[num[g]]);
                        v = cscale(v, tb.ratio[ri * p.nd + sx[0]]);
                    }
                }
            }
            sc[t] = c;
            sv[t] = v;
        }
        if (lane == 0) {
            sc[p.T_o] = row;
            sv[p.T_o] = ((const double2*)p.diag)[row];
        }
        __syncwarp();
        if (lane == 0) {
            int n = 0;
            for (int i = 0; i < T1; ++i) {
                const long long c = sc[i];
                if (c < 0) continue;
                int j = n;
                while (j > 0 && lc[j - 1] > c) --j;
                if (j > 0 && lc[j - 1] == c) {
                    lv[j - 1].x += sv[i].x;
                    lv[j - 1].y += sv[i].y;
                    continue;
                }
                for (int k = n; k > j; --k) {
                    lc[k] = lc[k - 1];
                    lv[k] = lv[k - 1];
                }
                lc[j] = c;
                lv[j] = sv[i];
                ++n;
            }
            int m = 0;
            for (int k = 0; k < n; ++k)
                if (!(sqrt(lv[k].x * lv[k].x + lv[k].y * lv[k].y) < tol)) {
                    lc[m] = lc[k];
                    lv[m] = lv[k];
                    ++m;
                }
            if (!row_ptr) {
                counts[rr] = m;
            } else {
                const long long o = row_ptr[rr];
                for (int k = 0; k < m; ++k) {
                    cols[o + k] = lc[k];
                    vals[o + k] = conj_vals ? make_double2(lv[k].x, -lv[k].y) : lv[k];
                }
            }
        }
        __syncwarp();
    }
}

template <typename W, int GK>
void hx_sparse_launch_one(const HxParams& p, long long row0, long long n_run, int conj_vals, double tol,
                          long long* counts, const long long* row_ptr, long long* cols, double2* vals, size_t smem,
                          cudaStream_t st) {
    auto kern = hx_sparse_kernel<W, GK>;
    raise_smem_limit((const void*)kern, smem);
    const long long warps = n_run;
    const int blocks = (int)std::max<long long>(1, std::min<long long>((warps + 3) / 4, 152ll * 16));
    kern<<<blocks, SPARSE_THREADS, smem, st>>>(p, row0, n_run, conj_vals, tol, counts, row_ptr, cols, vals);
    EDGPU_CUDA(cudaGetLastError());
}

template <typename W, int GK, int PREC>
void hx_multi_launch_one(const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    auto kern = hx_multi_kernel<W, GK, PREC>;
    raise_smem_limit((const void*)kern, smem);
    kern<<<blocks, HX_THREADS, smem, st>>>(p);
    EDGPU_CUDA(cudaGetLastError());
}

template <typename W, int GK, int PREC>
int hx_multi_occupancy_one(size_t smem) {
    auto kern = hx_multi_kernel<W, GK, PREC>;
    raise_smem_limit((const void*)kern, smem);
    int n = 0;
    EDGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, HX_THREADS, smem));
    return n;
}

template <typename W, int GK, int PREC, int MODE>
void hx_rows_launch_one(const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    auto kern = hx_rows_kernel<W, GK, PREC, MODE>;
    raise_smem_limit((const void*)kern, smem);
    kern<<<blocks, HX_THREADS, smem, st>>>(p);
    EDGPU_CUDA(cudaGetLastError());
}

template <typename W, int GK, int PREC, int MODE>
int hx_rows_occupancy_one(size_t smem) {
    auto kern = hx_rows_kernel<W, GK, PREC, MODE>;
    raise_smem_limit((const void*)kern, smem);
    int n = 0;
    EDGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, HX_THREADS, smem));
    return n;
}

}  // namespace edgpu
