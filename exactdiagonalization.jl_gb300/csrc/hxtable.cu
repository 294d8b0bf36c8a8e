// Target table of the pair-flip schedule: the map-format entry of every (row, target) of the product,
// stored once per operator in the order the product walks them (warp tiles of 32 rows, row after row,
// each row's targets by bond class and start bit).  The product then streams the table instead of
// looking every target up (a parent-state map read or canonicalisation plus search per target), and
// gathers x: the entries are the same, so the results are bit-identical to the looked-up product.
//
// This is the compact, index-only form of the reference's precomputed parent-sized
// basis_mapping_index (symmetry_reduce_generic.jl:33-35), taken one step further: indexed by (row,
// target) rather than by parent state, as read by the row iterator (reduced_operator_representation.jl
// :57-85).
#include "hx_bond.cuh"

namespace edgpu {

namespace {

// Targets of every warp tile of 32 rows (the pair-flip schedule with one lane per row).
template <typename W, int PREC>
__global__ void __launch_bounds__(HX_THREADS) hx_table_count_kernel(const HxParams p, long long n_tiles,
                                                                  long long* tile_cnt) {
    extern __shared__ __align__(16) unsigned char sm[];
    {
        const int4* src = (const int4*)p.blob;
        int4* dst = (int4*)sm;
        for (int i = threadIdx.x; i < p.blob_words16; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const BondTables<W, PREC> bt(p, sm);
    const W* __restrict__ keys = (const W*)p.keys;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const W smask = (W)((((W)1) << p.sb) - 1);
    for (long long tile = (long long)blockIdx.x * wpb + warp; tile < n_tiles; tile += (long long)gridDim.x * wpb) {
        const long long row = tile * 32 + lane;
        const bool act = row < p.n_rows;
        const W b = act ? (W)(keys[row] >> p.sb) : (W)0;
        (void)smask;
        int cnt = bond_row_count<W, PREC>(b, bt, act ? p.bond_ncls : 0, p.nbits, (W)p.full);
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, d);
        if (lane == 0) tile_cnt[tile] = cnt;
    }
}

// Exclusive scan of n counts in one block (each thread a contiguous run); *total = their sum.
__global__ void k_table_scan(const long long* cnt, long long n, long long* off, long long* total) {
    __shared__ long long tmp[32];
    const long long per = (n + blockDim.x - 1) / blockDim.x;
    const long long beg = min(n, (long long)threadIdx.x * per), end = min(n, beg + per);
    long long s = 0;
    for (long long i = beg; i < end; ++i) s += cnt[i];
    long long tot = 0;
    long long ex = block_exclusive_scan(s, tmp, &tot);
    for (long long i = beg; i < end; ++i) {
        off[i] = ex;
        ex += cnt[i];
    }
    if (threadIdx.x == 0) *total = tot;
}

// The build pass: every target of every row looked up with flavour GK and written to the table.
template <typename W, int GK, int PREC>
__global__ void __launch_bounds__(HX_THREADS) hx_table_fill_kernel(const HxParams p, long long n_tiles) {
    typedef typename Cx<PREC>::V V;
    extern __shared__ __align__(16) unsigned char sm[];
    {
        const int4* src = (const int4*)p.blob;
        int4* dst = (int4*)sm;
        for (int i = threadIdx.x; i < p.blob_words16; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const RowsTables<W, PREC> tb(p, sm);
    const BondTables<W, PREC> bt(p, sm);
    RowsSector<PREC> sc{};
    sc.keys = p.keys;
    sc.n_rows = p.n_rows;
    sc.ds = p.ds;
    sc.ph = (const V*)(sm + p.o_ph);
    sc.num = (const int*)(sm + p.o_num);
    sc.want_arg = p.want_arg != 0;
    sc.map = p.map;
    sc.map_wide = p.map_wide;
    sc.map_cb = p.map_cb;
    sc.map_direct = p.map_direct;
    sc.tab = p.tab;
    sc.tile_off = p.tile_off;
    sc.tab_wide = p.tab_wide;
    sc.tab_cb = p.tab_cb;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    for (long long tile = (long long)blockIdx.x * wpb + warp; tile < n_tiles; tile += (long long)gridDim.x * wpb)
        bond_tile<W, GK, PREC, 2, true>(p, tb, bt, sc, tile, lane);
}

template <typename K>
void set_smem(K kern, size_t smem) {
    raise_smem_limit((const void*)kern, smem);
}

int grid_for(long long n_tiles) {
    return (int)std::max<long long>(1, std::min<long long>((n_tiles + HX_THREADS / 32 - 1) / (HX_THREADS / 32),
                                                           (long long)sm_count() * 8));
}

template <typename W>
void fill_one(int gk, const HxParams& p, long long n_tiles, size_t smem, cudaStream_t st) {
    const int blocks = grid_for(n_tiles);
    switch (gk) {
        case GK_TRIVIAL: set_smem(hx_table_fill_kernel<W, GK_TRIVIAL, 1>, smem);
            hx_table_fill_kernel<W, GK_TRIVIAL, 1><<<blocks, HX_THREADS, smem, st>>>(p, n_tiles); break;
        case GK_TORUS: set_smem(hx_table_fill_kernel<W, GK_TORUS, 1>, smem);
            hx_table_fill_kernel<W, GK_TORUS, 1><<<blocks, HX_THREADS, smem, st>>>(p, n_tiles); break;
        case GK_GENERIC: set_smem(hx_table_fill_kernel<W, GK_GENERIC, 1>, smem);
            hx_table_fill_kernel<W, GK_GENERIC, 1><<<blocks, HX_THREADS, smem, st>>>(p, n_tiles); break;
        case GK_RING:
            if constexpr (sizeof(W) == 4) {
                set_smem(hx_table_fill_kernel<W, GK_RING, 1>, smem);
                hx_table_fill_kernel<W, GK_RING, 1><<<blocks, HX_THREADS, smem, st>>>(p, n_tiles);
                break;
            }
            throw Error(EDGPU_ERR_ARG, "ring lookups need 32-bit tables");
        case GK_MAP: set_smem(hx_table_fill_kernel<W, GK_MAP, 1>, smem);
            hx_table_fill_kernel<W, GK_MAP, 1><<<blocks, HX_THREADS, smem, st>>>(p, n_tiles); break;
        default: throw Error(EDGPU_ERR_ARG, "bad target-table lookup flavour");
    }
    EDGPU_CUDA(cudaGetLastError());
}

template <typename W>
void launch_t(int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st, bool multi) {
    const int nt = p.bond_nt == 8 ? 8 : p.bond_nt == 4 ? 4 : 2;
#define EDGPU_TABLE_CASE(PR, NTV)                                                                          \
    if (prec == PR && nt == NTV) {                                                                         \
        if (multi) return hx_bond_multi_launch_one<W, GK_TABLE, PR, NTV>(p, blocks, smem, st);             \
        return hx_bond_launch_one<W, GK_TABLE, PR, NTV>(p, blocks, smem, st);                              \
    }
    // warp-uniform pair steps: one-sector launches with 4 or 8 targets per step
    if (p.bond_uni && !multi && (nt == 4 || nt == 8)) {
        if (prec == 0) return nt == 8 ? hx_bond_launch_one<W, GK_TABLE, 0, 8, true>(p, blocks, smem, st)
                                      : hx_bond_launch_one<W, GK_TABLE, 0, 4, true>(p, blocks, smem, st);
        return nt == 8 ? hx_bond_launch_one<W, GK_TABLE, 1, 8, true>(p, blocks, smem, st)
                       : hx_bond_launch_one<W, GK_TABLE, 1, 4, true>(p, blocks, smem, st);
    }
    EDGPU_TABLE_CASE(0, 2)
    EDGPU_TABLE_CASE(0, 4)
    EDGPU_TABLE_CASE(1, 2)
    EDGPU_TABLE_CASE(1, 4)
    // eight targets per step (one-sector and batched launches)
    if (nt == 8) {
        if (multi) {
            if (prec == 0) return hx_bond_multi_launch_one<W, GK_TABLE, 0, 8>(p, blocks, smem, st);
            return hx_bond_multi_launch_one<W, GK_TABLE, 1, 8>(p, blocks, smem, st);
        }
        if (prec == 0) return hx_bond_launch_one<W, GK_TABLE, 0, 8>(p, blocks, smem, st);
        return hx_bond_launch_one<W, GK_TABLE, 1, 8>(p, blocks, smem, st);
    }
#undef EDGPU_TABLE_CASE
    throw Error(EDGPU_ERR_ARG, "bad target-table kernel selector");
}

template <typename W>
int occupancy_t(int prec, int nt, size_t smem, bool multi, bool uni) {
    if (uni && !multi && (nt == 4 || nt == 8)) {
        if (prec == 0) return nt == 8 ? hx_bond_occupancy_one<W, GK_TABLE, 0, 8, true>(smem)
                                      : hx_bond_occupancy_one<W, GK_TABLE, 0, 4, true>(smem);
        return nt == 8 ? hx_bond_occupancy_one<W, GK_TABLE, 1, 8, true>(smem)
                       : hx_bond_occupancy_one<W, GK_TABLE, 1, 4, true>(smem);
    }
    if (nt == 8 && !multi)
        return prec == 0 ? hx_bond_occupancy_one<W, GK_TABLE, 0, 8>(smem) : hx_bond_occupancy_one<W, GK_TABLE, 1, 8>(smem);
    if (nt == 8)
        return prec == 0 ? hx_bond_multi_occupancy_one<W, GK_TABLE, 0, 8>(smem)
                         : hx_bond_multi_occupancy_one<W, GK_TABLE, 1, 8>(smem);
    if (prec == 0 && nt != 4) return multi ? hx_bond_multi_occupancy_one<W, GK_TABLE, 0, 2>(smem) : hx_bond_occupancy_one<W, GK_TABLE, 0, 2>(smem);
    if (prec == 0) return multi ? hx_bond_multi_occupancy_one<W, GK_TABLE, 0, 4>(smem) : hx_bond_occupancy_one<W, GK_TABLE, 0, 4>(smem);
    if (nt != 4) return multi ? hx_bond_multi_occupancy_one<W, GK_TABLE, 1, 2>(smem) : hx_bond_occupancy_one<W, GK_TABLE, 1, 2>(smem);
    return multi ? hx_bond_multi_occupancy_one<W, GK_TABLE, 1, 4>(smem) : hx_bond_occupancy_one<W, GK_TABLE, 1, 4>(smem);
}

}  // namespace

void hx_table_count(bool w32, const HxParams& p, long long n_tiles, long long* tile_cnt, size_t smem, cudaStream_t st) {
    const int blocks = grid_for(n_tiles);
    if (w32) {
        set_smem(hx_table_count_kernel<unsigned, 1>, smem);
        hx_table_count_kernel<unsigned, 1><<<blocks, HX_THREADS, smem, st>>>(p, n_tiles, tile_cnt);
    } else {
        set_smem(hx_table_count_kernel<unsigned long long, 1>, smem);
        hx_table_count_kernel<unsigned long long, 1><<<blocks, HX_THREADS, smem, st>>>(p, n_tiles, tile_cnt);
    }
    EDGPU_CUDA(cudaGetLastError());
}

long long hx_table_scan(const long long* tile_cnt, long long n_tiles, long long* tile_off, cudaStream_t st) {
    long long* d_total = nullptr;
    EDGPU_CUDA(cudaMalloc(&d_total, sizeof(long long)));
    k_table_scan<<<1, 1024, 0, st>>>(tile_cnt, n_tiles, tile_off, d_total);
    cudaError_t e = cudaGetLastError();
    long long total = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, d_total, sizeof(long long), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_total);
    if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("target table scan: ") + cudaGetErrorString(e));
    return total;
}

void hx_table_fill(bool w32, int gk, const HxParams& p, long long n_tiles, size_t smem, cudaStream_t st) {
    if (w32) fill_one<unsigned>(gk, p, n_tiles, smem, st);
    else fill_one<unsigned long long>(gk, p, n_tiles, smem, st);
}

void hx_table_launch(bool w32, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    if (w32) launch_t<unsigned>(prec, p, blocks, smem, st, false);
    else launch_t<unsigned long long>(prec, p, blocks, smem, st, false);
}

int hx_table_occupancy(bool w32, int prec, int nt, size_t smem, bool uni) {
    return w32 ? occupancy_t<unsigned>(prec, nt, smem, false, uni)
               : occupancy_t<unsigned long long>(prec, nt, smem, false, uni);
}

void hx_table_multi_launch(bool w32, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    if (w32) launch_t<unsigned>(prec, p, blocks, smem, st, true);
    else launch_t<unsigned long long>(prec, p, blocks, smem, st, true);
}

int hx_table_multi_occupancy(bool w32, int prec, int nt, size_t smem) {
    return w32 ? occupancy_t<unsigned>(prec, nt, smem, true, false)
               : occupancy_t<unsigned long long>(prec, nt, smem, true, false);
}

}  // namespace edgpu

namespace edgpu {

// The product fused with the coupling gradient (hx_bond_grad_kernel): target table or parent-state
// map, four targets per lane and step.
void hx_bond_grad_launch(bool w32, bool table, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    if (w32) {
        if (table) return prec == 0 ? hx_bond_grad_launch_one<unsigned, GK_TABLE, 0, 4>(p, blocks, smem, st)
                                    : hx_bond_grad_launch_one<unsigned, GK_TABLE, 1, 4>(p, blocks, smem, st);
        return prec == 0 ? hx_bond_grad_launch_one<unsigned, GK_MAP, 0, 4>(p, blocks, smem, st)
                         : hx_bond_grad_launch_one<unsigned, GK_MAP, 1, 4>(p, blocks, smem, st);
    }
    if (table) return prec == 0 ? hx_bond_grad_launch_one<unsigned long long, GK_TABLE, 0, 4>(p, blocks, smem, st)
                                : hx_bond_grad_launch_one<unsigned long long, GK_TABLE, 1, 4>(p, blocks, smem, st);
    return prec == 0 ? hx_bond_grad_launch_one<unsigned long long, GK_MAP, 0, 4>(p, blocks, smem, st)
                     : hx_bond_grad_launch_one<unsigned long long, GK_MAP, 1, 4>(p, blocks, smem, st);
}

int hx_bond_grad_occupancy(bool w32, bool table, int prec, size_t smem) {
    if (w32) {
        if (table) return prec == 0 ? hx_bond_grad_occupancy_one<unsigned, GK_TABLE, 0, 4>(smem)
                                    : hx_bond_grad_occupancy_one<unsigned, GK_TABLE, 1, 4>(smem);
        return prec == 0 ? hx_bond_grad_occupancy_one<unsigned, GK_MAP, 0, 4>(smem)
                         : hx_bond_grad_occupancy_one<unsigned, GK_MAP, 1, 4>(smem);
    }
    if (table) return prec == 0 ? hx_bond_grad_occupancy_one<unsigned long long, GK_TABLE, 0, 4>(smem)
                                : hx_bond_grad_occupancy_one<unsigned long long, GK_TABLE, 1, 4>(smem);
    return prec == 0 ? hx_bond_grad_occupancy_one<unsigned long long, GK_MAP, 0, 4>(smem)
                     : hx_bond_grad_occupancy_one<unsigned long long, GK_MAP, 1, 4>(smem);
}

}  // namespace edgpu

// ---- adjoint target table ------------------------------------------------------------------------
// For operators whose terms do not commute with the group, the adjoint of the product's matrix
// (dL/dx = H^dagger gy) is not the row formula applied to the adjoint terms.  Its rows are the
// columns of H: this table lists, per column c, every (row r, slot) whose target lands on c, sorted,
// so that (H^dagger gy)[c] = sum conj(H[r, c]) gy[r] is a gather in a fixed order instead of a
// scatter with atomics.
namespace edgpu {
namespace {

template <typename W, int PASS>
__global__ void __launch_bounds__(HX_THREADS) hx_adj_pass_kernel(const HxParams p, long long n_tiles) {
    typedef typename Cx<1>::V V;
    extern __shared__ __align__(16) unsigned char sm[];
    {
        const int4* src = (const int4*)p.blob;
        int4* dst = (int4*)sm;
        for (int i = threadIdx.x; i < p.blob_words16; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const RowsTables<W, 1> tb(p, sm);
    const BondTables<W, 1> bt(p, sm);
    RowsSector<1> sc{};
    sc.keys = p.keys;
    sc.n_rows = p.n_rows;
    sc.ds = p.ds;
    sc.ph = (const V*)(sm + p.o_ph);
    sc.num = (const int*)(sm + p.o_num);
    sc.want_arg = p.want_arg != 0;
    sc.tab = p.tab;
    sc.tile_off = p.tile_off;
    sc.tab_wide = p.tab_wide;
    sc.tab_cb = p.tab_cb;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    for (long long tile = (long long)blockIdx.x * wpb + warp; tile < n_tiles; tile += (long long)gridDim.x * wpb)
        bond_tile<W, GK_TABLE, 1, 4, false, false, false, PASS>(p, tb, bt, sc, tile, lane);
}

// Each column's run sorted ascending (the entries of a column are distinct): the order of the
// adjoint's sum no longer depends on the order in which the fill pass wrote them.
__global__ void k_adj_sort(const long long* off, unsigned long long* tab, long long n) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const long long a = off[c], b = off[c + 1];
        for (long long i = a + 1; i < b; ++i) {
            const unsigned long long v = tab[i];
            long long j = i - 1;
            while (j >= a && tab[j] > v) {
                tab[j + 1] = tab[j];
                --j;
            }
            tab[j + 1] = v;
        }
    }
}

// y[c] = conj(diag[c]) x[c] + sum over c's run of conj(amp(slot) chi(g) sqrt(|O_r| / |O_c|)) x[r].
template <typename W, int PREC>
__global__ void __launch_bounds__(HX_THREADS) hx_adj_kernel(const HxParams p) {
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
    const BondTables<W, PREC> bt(p, sm);
    const V* ph = (const V*)(sm + p.o_ph);
    const int* num = (const int*)(sm + p.o_num);
    const W* __restrict__ keys = (const W*)p.keys;
    const V* __restrict__ x = (const V*)p.gy;
    V* __restrict__ y = (V*)p.y;
    const V* __restrict__ diag = (const V*)p.diag;
    const W smask = (W)((((W)1) << p.sb) - 1);
    const bool want_arg = p.want_arg != 0;
    const bool real_fast = p.bond_real && !want_arg;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < p.n_rows; c += (long long)gridDim.x * blockDim.x) {
        const int sxc = (int)(keys[c] & smask);
        V acc = cmul(cconj(diag[c]), x[c]);
        const long long a = p.adj_off[c], b = p.adj_off[c + 1];
        for (long long i = a; i < b; ++i) {
            const unsigned long long e = p.adj_tab[i];
            const long long r = (long long)(e >> 32);
            const int ti = (int)((e >> 19) & 0x1fffu);
            const int sxr = (int)((e >> 14) & 0x1fu);
            const int g = (int)(e & 0x3fffu);
            const V xr = x[r];
            if (real_fast) {
                // real amplitude, trivial characters: the element is its own conjugate
                const R f = bt.amp[ti].x * tb.ratio[sxr * p.nd + sxc];
                acc.x = fma_r(f, xr.x, acc.x);
                acc.y = fma_r(f, xr.y, acc.y);
                continue;
            }
            V coef = bt.amp[ti];
            if (want_arg) coef = cmul(coef, ph[num[g]]);
            coef = cscale(coef, tb.ratio[sxr * p.nd + sxc]);
            acc = cadd(acc, cmul(cconj(coef), xr));
        }
        if (p.accumulate) acc = cadd(acc, y[c]);
        y[c] = acc;
    }
}

}  // namespace

void hx_adj_pass(bool w32, int pass, const HxParams& p, long long n_tiles, size_t smem, cudaStream_t st) {
    const int blocks = grid_for(n_tiles);
    if (w32) {
        if (pass == 1) {
            set_smem(hx_adj_pass_kernel<unsigned, 1>, smem);
            hx_adj_pass_kernel<unsigned, 1><<<blocks, HX_THREADS, smem, st>>>(p, n_tiles);
        } else {
            set_smem(hx_adj_pass_kernel<unsigned, 2>, smem);
            hx_adj_pass_kernel<unsigned, 2><<<blocks, HX_THREADS, smem, st>>>(p, n_tiles);
        }
    } else {
        if (pass == 1) {
            set_smem(hx_adj_pass_kernel<unsigned long long, 1>, smem);
            hx_adj_pass_kernel<unsigned long long, 1><<<blocks, HX_THREADS, smem, st>>>(p, n_tiles);
        } else {
            set_smem(hx_adj_pass_kernel<unsigned long long, 2>, smem);
            hx_adj_pass_kernel<unsigned long long, 2><<<blocks, HX_THREADS, smem, st>>>(p, n_tiles);
        }
    }
    EDGPU_CUDA(cudaGetLastError());
}

void hx_adj_sort(const long long* off, unsigned long long* tab, long long n, cudaStream_t st) {
    const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)sm_count() * 16));
    k_adj_sort<<<blocks, 256, 0, st>>>(off, tab, n);
    EDGPU_CUDA(cudaGetLastError());
}

void hx_adj_launch(bool w32, int prec, const HxParams& p, size_t smem, cudaStream_t st) {
    const int blocks = (int)std::max<long long>(1, std::min<long long>((p.n_rows + HX_THREADS - 1) / HX_THREADS,
                                                                      (long long)sm_count() * 8));
    if (w32) {
        if (prec == 0) {
            set_smem(hx_adj_kernel<unsigned, 0>, smem);
            hx_adj_kernel<unsigned, 0><<<blocks, HX_THREADS, smem, st>>>(p);
        } else {
            set_smem(hx_adj_kernel<unsigned, 1>, smem);
            hx_adj_kernel<unsigned, 1><<<blocks, HX_THREADS, smem, st>>>(p);
        }
    } else {
        if (prec == 0) {
            set_smem(hx_adj_kernel<unsigned long long, 0>, smem);
            hx_adj_kernel<unsigned long long, 0><<<blocks, HX_THREADS, smem, st>>>(p);
        } else {
            set_smem(hx_adj_kernel<unsigned long long, 1>, smem);
            hx_adj_kernel<unsigned long long, 1><<<blocks, HX_THREADS, smem, st>>>(p);
        }
    }
    EDGPU_CUDA(cudaGetLastError());
}

}  // namespace edgpu
