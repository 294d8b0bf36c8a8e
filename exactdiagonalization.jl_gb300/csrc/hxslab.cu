// Column-slab table of the pair-flip schedule and its multi-pass product (both precisions).
//
// On a large sector the target-table product (hx_bond.cuh, GK_TABLE) gathers x at random: with x
// many times the size of L2, nearly every gather is a DRAM sector of 32 bytes for 8 bytes of x.  The
// slab table regroups the same entries by the column slab their target lies in.  Pass q of the
// product reads only the entries whose columns lie in slab q, so while it runs the gathers hit a
// window of x small enough to stay in L2; its share is added to y.  y is then read and written once
// per pass, which is streamed traffic, instead of one random DRAM sector per target.
//
// The entries are those of the target table (itself the (row, target) form of the reference's
// basis_mapping_index, symmetry_reduce_generic.jl:33-35), with the coefficient of each element
// (amplitude x character x orbit-size ratio, reduced_operator_representation.jl:57-85) replaced by an
// index into a small table of the distinct coefficients.  Within a pass every row adds its entries
// in the target table's order and the passes are added in order, so results are reproducible run to
// run; they differ from the one-pass product by the order of the additions.  A scaled table's index
// leaves the orbit-size ratio sqrt(|O_c| / |O_r|) out: x is scaled by sqrt(|O_c|) before the passes
// (k_slab_xscale) and each row's result by 1 / sqrt(|O_r|) in the last pass.
#include "hx_bond.cuh"

#include <type_traits>

namespace edgpu {

namespace {

// Calls f(slot, c, sx, g) for every target of the row state b in the target table's order (class,
// then start bit), reading the entries from position tpos on; slot = (class n + i) << 2 | v.
template <typename W, int PREC, typename F>
__device__ __forceinline__ void slab_walk(const HxParams& p, const BondTables<W, PREC>& bt,
                                          const RowsSector<PREC>& sc, W b, long long tpos, F&& f) {
    const int n = p.nbits;
    const W full = (W)p.full;
    for (int cls = 0; cls < p.bond_ncls; ++cls) {
        W m = bond_class_mask<W, PREC>(b, bt, cls, n, full);
        const bool cpar = (bt.ninfo[cls] >> 8) != 0;
        while (m) {
            const int i = lowest_bit<W>(m);
            m &= m - 1;
            const int ti = cls * n + i;
            int v = (int)(b >> i) & 1;
            if (cpar) v |= (__popcll((unsigned long long)(b & bt.flip[ti])) != 1) << 1;
            long long c;
            int sx, g;
            table_entry<PREC>(sc, tpos, true, p.sb, c, sx, g);
            ++tpos;
            f((ti << 2) | v, c, sx, g);
        }
    }
}

// Pass 1 counts every row's targets per slab (counts[q][row], tile sums); pass 2 writes every entry
// at its place (a per-thread cursor per slab, started at the tile's offset plus the counts of the
// tile's earlier rows).
template <typename W, int PREC, int PASS>
__global__ void __launch_bounds__(HX_THREADS) hx_slab_build_kernel(const HxParams p, const SlabBuild s) {
    extern __shared__ __align__(16) unsigned char sm[];
    {
        const int4* src = (const int4*)p.blob;
        int4* dst = (int4*)sm;
        for (int i = threadIdx.x; i < p.blob_words16; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const BondTables<W, PREC> bt(p, sm);
    RowsSector<PREC> sc{};
    sc.tab = p.tab;
    sc.tile_off = p.tile_off;
    sc.tab_wide = p.tab_wide;
    sc.tab_cb = p.tab_cb;
    const int* num = (const int*)(sm + p.o_num);
    const W* __restrict__ keys = (const W*)p.keys;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const W smask = (W)((((W)1) << p.sb) - 1);
    const unsigned wc = (unsigned)s.wc;
    const int P = s.n_pass;
    for (long long tile = (long long)blockIdx.x * wpb + warp; tile < s.n_tiles; tile += (long long)gridDim.x * wpb) {
        const long long row = tile * 32 + lane;
        const bool act = row < p.n_rows;
        const W kr = act ? keys[row] : (W)0;
        const W b = kr >> p.sb;
        const int ri = (int)(kr & smask);
        const int cnt = bond_row_count<W, PREC>(b, bt, act ? p.bond_ncls : 0, p.nbits, (W)p.full);
        int incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += u;
        }
        const long long tpos = p.tile_off[tile] + (incl - cnt);
        if constexpr (PASS == 1) {
            if (s.cls && act) s.cls[row] = (unsigned char)ri;
            unsigned char* ctr = sm + s.o_ctr;
            for (int q = 0; q < P; ++q) ctr[q * HX_THREADS + threadIdx.x] = 0;
            if (act)
                slab_walk<W, PREC>(p, bt, sc, b, tpos, [&](int, long long c, int, int) {
                    if (c >= 0) ++ctr[((unsigned)c / wc) * HX_THREADS + threadIdx.x];
                });
            for (int q = 0; q < P; ++q) {
                const unsigned v = ctr[q * HX_THREADS + threadIdx.x];
                if (act) s.counts[(size_t)q * p.n_rows + row] = (unsigned char)v;
                unsigned t = v;
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) t += __shfl_xor_sync(0xffffffffu, t, d);
                if (lane == 0) s.tile_sum[(size_t)q * s.n_tiles + tile] = t;
            }
        } else {
            unsigned* cur = (unsigned*)(sm + s.o_ctr);
            for (int q = 0; q < P; ++q) {
                const unsigned v = act ? s.counts[(size_t)q * p.n_rows + row] : 0u;
                unsigned inc = v;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const unsigned u = __shfl_up_sync(0xffffffffu, inc, d);
                    if (lane >= d) inc += u;
                }
                cur[q * HX_THREADS + threadIdx.x] = s.off[(size_t)q * s.n_tiles + tile] + (inc - v);
            }
            if (act)
                slab_walk<W, PREC>(p, bt, sc, b, tpos, [&](int slot, long long c, int sx, int g) {
                    if (c < 0) return;
                    const unsigned q = (unsigned)c / wc;
                    const unsigned rel = cur[q * HX_THREADS + threadIdx.x]++;
                    const unsigned ph = p.want_arg ? (unsigned)num[g] : 0u;
                    const unsigned ap = (unsigned)__ldg(s.amp_id + slot) * (unsigned)p.den + ph;
                    const unsigned id = s.scaled ? ap : (ap * (unsigned)p.nd + (unsigned)ri) * (unsigned)p.nd + (unsigned)sx;
                    s.tab[s.base[q] + rel] = ((unsigned)c - q * wc) | (id << s.colbits);
                });
        }
    }
}

// Exclusive scan of the tile sums of every pass, in chunks of SLAB_CHUNK per block (blockIdx.y =
// pass): chunk totals, then a scan of the chunk totals per pass, then the offsets.
constexpr int SLAB_CHUNK = HX_THREADS * 16;

__global__ void k_slab_scan_part(const unsigned* ts, long long n_tiles, unsigned long long* part, int nb) {
    __shared__ long long tmp[32];
    const int q = blockIdx.y;
    const unsigned* a = ts + (size_t)q * n_tiles;
    const long long beg = (long long)blockIdx.x * SLAB_CHUNK + (long long)threadIdx.x * 16;
    long long s = 0;
    for (long long i = beg; i < min(n_tiles, beg + 16); ++i) s += a[i];
    long long tot = 0;
    block_exclusive_scan(s, tmp, &tot);
    if (threadIdx.x == 0) part[(size_t)q * nb + blockIdx.x] = (unsigned long long)tot;
}

__global__ void k_slab_scan_mid(unsigned long long* part, int nb, unsigned long long* totals) {
    __shared__ long long tmp[32];
    unsigned long long* a = part + (size_t)blockIdx.x * nb;
    long long carry = 0;
    for (int b0 = 0; b0 < nb; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        const long long v = i < nb ? (long long)a[i] : 0;
        long long tot = 0;
        const long long ex = block_exclusive_scan(v, tmp, &tot);
        if (i < nb) a[i] = (unsigned long long)(carry + ex);
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = (unsigned long long)carry;
}

__global__ void k_slab_scan_out(const unsigned* ts, long long n_tiles, const unsigned long long* part, int nb,
                                unsigned* off) {
    __shared__ long long tmp[32];
    const int q = blockIdx.y;
    const unsigned* a = ts + (size_t)q * n_tiles;
    unsigned* o = off + (size_t)q * n_tiles;
    const long long beg = (long long)blockIdx.x * SLAB_CHUNK + (long long)threadIdx.x * 16;
    const long long end = min(n_tiles, beg + 16);
    long long s = 0;
    for (long long i = beg; i < end; ++i) s += a[i];
    long long ex = block_exclusive_scan(s, tmp, nullptr) + (long long)part[(size_t)q * nb + blockIdx.x];
    for (long long i = beg; i < end; ++i) {
        o[i] = (unsigned)ex;
        ex += a[i];
    }
}

// acc += c x with explicit fused multiply-adds (the same roundings in every kernel of this file)
template <typename V>
__device__ __forceinline__ V cfma_acc(V acc, V c, V x) {
    acc.x = fma_r(c.x, x.x, acc.x);
    acc.x = fma_r(-c.y, x.y, acc.x);
    acc.y = fma_r(c.x, x.y, acc.y);
    acc.y = fma_r(c.y, x.x, acc.y);
    return acc;
}

// Loads and stores with or without cache hints (CH): the gathers of x cached in L2 only (they have
// no reuse in L1), the streamed count bytes, offsets and y marked evict-first, so that the slab of x
// keeps its place in L2.
template <bool CH, typename T>
__device__ __forceinline__ T ld_gather(const T* p) {
    if constexpr (CH) return __ldcg(p);
    else return *p;
}
template <bool CH, typename T>
__device__ __forceinline__ T ld_stream(const T* p) {
    if constexpr (CH) return __ldcs(p);
    else return *p;
}
template <bool CH, typename T>
__device__ __forceinline__ void st_stream(T* p, T v) {
    if constexpr (CH) __stcs(p, v);
    else *p = v;
}

// One pass of the product: a warp per tile of 32 rows with one lane per row (LPR = 1), or per part of
// 32 / LPR rows of a tile with LPR lanes per row (lane sub of a row takes the row's entries sub,
// sub + LPR, ...; the partial sums are added by a fixed butterfly).  A lane adds its entries of this
// pass (NT per step, loads then gathers); the row's sum is then added to y (the first pass writes it,
// the last adds the diagonal term too and may write complex128 to y_c128 instead).  LUTM: where the
// coefficients are read (SlabRun::lut_mode).
template <int PREC, bool REAL, int NT, bool CH, int LPR, int LUTM>
__global__ void __launch_bounds__(HX_THREADS) hx_slab_kernel(const SlabRun r) {
    typedef typename Cx<PREC>::V V;
    typedef typename Cx<PREC>::R R;
    typedef typename std::conditional<REAL, R, V>::type C;
    constexpr int REPS = 128 / (int)sizeof(C);   // copies per coefficient: one per bank group
    extern __shared__ __align__(16) unsigned char sm[];
    pdl_launch_dependents();
    const C* src = (const C*)r.lut;
    R c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    if constexpr (LUTM == 2) {
        const R* lr0 = (const R*)r.lut;
        c0 = __ldg(lr0);
        c1 = __ldg(lr0 + min(1, r.n_lut - 1));
        c2 = __ldg(lr0 + min(2, r.n_lut - 1));
        c3 = __ldg(lr0 + min(3, r.n_lut - 1));
    } else if constexpr (LUTM == 1) {
        for (int i = threadIdx.x; i < r.n_lut * REPS; i += blockDim.x) ((C*)sm)[i] = src[i / REPS];
        __syncthreads();
    } else {
        for (int i = threadIdx.x; i < r.n_lut; i += blockDim.x) ((C*)sm)[i] = src[i];
        __syncthreads();
    }
    pdl_wait();
    const C* lut = (const C*)sm;
    const V* __restrict__ xs = (const V*)r.xs;
    const unsigned* __restrict__ tab = r.tab;
    V* y = (V*)r.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const int sub = lane & (LPR - 1);
    const int rep = lane & (REPS - 1);
    const bool to_c128 = r.last && r.y_c128 != nullptr;
    const long long n_parts = r.n_tiles * LPR;
    for (long long part = (long long)blockIdx.x * wpb + warp; part < n_parts; part += (long long)gridDim.x * wpb) {
        const long long tile = r.tile0 + part / LPR;
        // the counts of the tile's 32 rows and their exclusive prefix
        const long long row32 = tile * 32 + lane;
        const int c32 = row32 < r.n_rows ? (int)ld_stream<CH>(r.cnt + row32) : 0;
        int incl = c32;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += u;
        }
        // this lane's row in the tile
        const int rl = LPR == 1 ? lane : (int)(part % LPR) * (32 / LPR) + lane / LPR;
        const int cnt = LPR == 1 ? c32 : __shfl_sync(0xffffffffu, c32, rl);
        const int excl = LPR == 1 ? incl - c32 : __shfl_sync(0xffffffffu, incl - c32, rl);
        const long long row = tile * 32 + rl;
        const bool act = row < r.n_rows;
        const long long start = (long long)ld_stream<CH>(r.off + tile) + excl;
        V acc = czero<V>();
        for (int j = sub; __any_sync(0xffffffffu, j < cnt); j += NT * LPR) {
            unsigned e[NT];
#pragma unroll
            for (int h = 0; h < NT; ++h) e[h] = (j + h * LPR < cnt) ? __ldg(tab + start + j + h * LPR) : 0u;
            V xv[NT];
#pragma unroll
            for (int h = 0; h < NT; ++h)
                xv[h] = (j + h * LPR < cnt) ? ld_gather<CH>(xs + (e[h] & r.colmask)) : czero<V>();
#pragma unroll
            for (int h = 0; h < NT; ++h) {
                if (j + h * LPR >= cnt) continue;
                const unsigned id = e[h] >> r.colbits;
                C f;
                if constexpr (LUTM == 2) {
                    f = (id & 2u) ? ((id & 1u) ? c3 : c2) : ((id & 1u) ? c1 : c0);
                } else if constexpr (LUTM == 1) {
                    f = lut[id * REPS + rep];
                } else {
                    f = lut[id];
                }
                if constexpr (REAL) {
                    acc.x = fma_r(f, xv[h].x, acc.x);
                    acc.y = fma_r(f, xv[h].y, acc.y);
                } else {
                    acc = cfma_acc(acc, f, xv[h]);
                }
            }
        }
#pragma unroll
        for (int d = 1; d < LPR; d <<= 1) {
            acc.x += __shfl_xor_sync(0xffffffffu, acc.x, d);
            acc.y += __shfl_xor_sync(0xffffffffu, acc.y, d);
        }
        if (!act || sub != 0) continue;
        // passes add their sums in order; the last adds the diagonal term diag x (so that a pass needs
        // only its own slab of x, the last one all of it)
        V t;
        if (r.first) {
            if (r.accumulate) {
                V yo = ld_stream<CH>(y + row);
                if (r.scaled) {
                    // y += H x on a scaled table: the old y_r enters the row's scaled sum as sqrt(|O_r|) y_r
                    const R sr = __ldg((const R*)r.scale + r.cls[row]);
                    yo.x *= sr;
                    yo.y *= sr;
                }
                t = cadd(yo, acc);
            } else {
                t = acc;
            }
        } else {
            if (cnt == 0 && !r.last) continue;   // nothing to add to this row
            t = cadd(ld_stream<CH>(y + row), acc);
        }
        if (r.last) {
            t = cfma_acc(t, ld_stream<CH>((const V*)r.diag + row), ld_stream<CH>((const V*)r.x + row));
            if (r.scaled) {
                const R rs = __ldg((const R*)r.scale + r.nd + r.cls[row]);
                t.x *= rs;
                t.y *= rs;
            }
        }
        if (to_c128) {
            double2 o = make_double2((double)t.x, (double)t.y);
            double2* yc = (double2*)r.y_c128;
            if (r.acc_c128) {
                const double2 old = yc[row];
                o.x += old.x;
                o.y += old.y;
            }
            yc[row] = o;
        } else {
            st_stream<CH>(y + row, t);
        }
    }
}

// x_c -> sqrt(|O_c|) x_c over the columns [c0, c1)
template <typename V, typename R>
__global__ void k_slab_xscale(const V* __restrict__ x, const unsigned char* __restrict__ cls,
                              const R* __restrict__ scale, V* __restrict__ out, long long c0, long long c1) {
    for (long long c = c0 + (long long)blockIdx.x * blockDim.x + threadIdx.x; c < c1;
         c += (long long)gridDim.x * blockDim.x) {
        const R f = scale[cls[c]];
        V v = x[c];
        v.x *= f;
        v.y *= f;
        out[c] = v;
    }
}

// the same from complex128 to complex64: x_c rounded to complex64, then scaled in FP32 (as the
// device-buffer path scales a complex64 x)
__global__ void k_slab_xscale_c128_c64(const double2* __restrict__ x, const unsigned char* __restrict__ cls,
                                       const float* __restrict__ scale, float2* __restrict__ out, long long c0,
                                       long long c1) {
    for (long long c = c0 + (long long)blockIdx.x * blockDim.x + threadIdx.x; c < c1;
         c += (long long)gridDim.x * blockDim.x) {
        const float f = scale[cls[c]];
        const double2 v = x[c];
        out[c] = make_float2((float)v.x * f, (float)v.y * f);
    }
}

int xscale_blocks(long long n) {
    const long long need = (n + 255) / 256;
    return (int)std::max<long long>(1, std::min<long long>(need, (long long)sm_count() * 8));
}

template <typename K>
void slab_pdl_launch(K kern, const SlabRun& r, int blocks, size_t smem, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(HX_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    EDGPU_CUDA(cudaLaunchKernelEx(&cfg, kern, r));
}

template <typename K>
int slab_blocks(K kern, size_t smem, long long n_tiles, int per_sm = 0) {
    raise_smem_limit((const void*)kern, smem);
    int n = 0;
    EDGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, HX_THREADS, smem));
    if (per_sm > 0) n = std::min(n, per_sm);
    else if (per_sm < 0) n = std::max(1, n + per_sm);
    const long long need = (n_tiles + HX_THREADS / 32 - 1) / (HX_THREADS / 32);
    return (int)std::max<long long>(1, std::min<long long>(need, (long long)std::max(1, n) * sm_count()));
}

template <typename W, int PREC>
void slab_build_t(int pass, const HxParams& p, const SlabBuild& s, size_t smem, cudaStream_t st) {
    const int blocks = (int)std::max<long long>(
        1, std::min<long long>((s.n_tiles + HX_THREADS / 32 - 1) / (HX_THREADS / 32), (long long)sm_count() * 8));
    if (pass == 1) {
        auto k = hx_slab_build_kernel<W, PREC, 1>;
        raise_smem_limit((const void*)k, smem);
        k<<<blocks, HX_THREADS, smem, st>>>(p, s);
    } else {
        auto k = hx_slab_build_kernel<W, PREC, 2>;
        raise_smem_limit((const void*)k, smem);
        k<<<blocks, HX_THREADS, smem, st>>>(p, s);
    }
    EDGPU_CUDA(cudaGetLastError());
}

}  // namespace

void hx_slab_build(bool w32, int prec, int pass, const HxParams& p, const SlabBuild& s, size_t smem,
                   cudaStream_t st) {
    if (w32) {
        if (prec == 0) slab_build_t<unsigned, 0>(pass, p, s, smem, st);
        else slab_build_t<unsigned, 1>(pass, p, s, smem, st);
    } else {
        if (prec == 0) slab_build_t<unsigned long long, 0>(pass, p, s, smem, st);
        else slab_build_t<unsigned long long, 1>(pass, p, s, smem, st);
    }
}

void hx_slab_scan(const unsigned* tile_sum, unsigned* off, int n_pass, long long n_tiles,
                  std::vector<unsigned long long>& totals, cudaStream_t st) {
    totals.assign((size_t)n_pass, 0);
    if (n_pass == 0 || n_tiles == 0) return;
    const int nb = (int)((n_tiles + SLAB_CHUNK - 1) / SLAB_CHUNK);
    unsigned long long* part = nullptr;
    unsigned long long* tot = nullptr;
    EDGPU_CUDA(cudaMalloc(&part, (size_t)nb * n_pass * sizeof(unsigned long long)));
    cudaError_t e = cudaMalloc(&tot, (size_t)n_pass * sizeof(unsigned long long));
    if (e != cudaSuccess) {
        cudaFree(part);
        throw Error(EDGPU_ERR_OOM, std::string("slab scan: ") + cudaGetErrorString(e));
    }
    const dim3 grid((unsigned)nb, (unsigned)n_pass);
    k_slab_scan_part<<<grid, HX_THREADS, 0, st>>>(tile_sum, n_tiles, part, nb);
    k_slab_scan_mid<<<n_pass, 1024, 0, st>>>(part, nb, tot);
    k_slab_scan_out<<<grid, HX_THREADS, 0, st>>>(tile_sum, n_tiles, part, nb, off);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(totals.data(), tot, (size_t)n_pass * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(part);
    cudaFree(tot);
    if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("slab scan: ") + cudaGetErrorString(e));
}

template <int PREC, bool REAL, bool CH, int NT, int LPR>
void slab_launch_m(const SlabRun& r, size_t smem, cudaStream_t st) {
    if constexpr (REAL) {
        if (r.lut_mode == 2) {
            auto k = hx_slab_kernel<PREC, true, NT, CH, LPR, 2>;
            slab_pdl_launch(k, r, slab_blocks(k, 0, r.n_tiles * LPR, r.blocks_per_sm), 0, st);
            return;
        }
    }
    if (r.lut_mode == 1) {
        auto k = hx_slab_kernel<PREC, REAL, NT, CH, LPR, 1>;
        slab_pdl_launch(k, r, slab_blocks(k, smem, r.n_tiles * LPR, r.blocks_per_sm), smem, st);
    } else {
        auto k = hx_slab_kernel<PREC, REAL, NT, CH, LPR, 0>;
        slab_pdl_launch(k, r, slab_blocks(k, smem, r.n_tiles * LPR, r.blocks_per_sm), smem, st);
    }
}

template <int PREC, bool CH, int NT, int LPR>
void slab_launch_t(const SlabRun& r, size_t smem, cudaStream_t st) {
    if (r.lut_real) slab_launch_m<PREC, true, CH, NT, LPR>(r, smem, st);
    else slab_launch_m<PREC, false, CH, NT, LPR>(r, smem, st);
}

// hints: 0 to 3 one lane per row (bit 0 the cache hints, bit 1 eight entries per lane and step
// instead of four); 4 and 5: two and four lanes per row, four entries per lane and step
template <int PREC>
void slab_launch_p(const SlabRun& r, size_t smem, cudaStream_t st) {
    switch (r.hints) {
        case 0: slab_launch_t<PREC, false, 4, 1>(r, smem, st); break;
        case 1: slab_launch_t<PREC, true, 4, 1>(r, smem, st); break;
        case 2: slab_launch_t<PREC, false, 8, 1>(r, smem, st); break;
        case 3: slab_launch_t<PREC, true, 8, 1>(r, smem, st); break;
        case 4: slab_launch_t<PREC, false, 4, 2>(r, smem, st); break;
        default: slab_launch_t<PREC, false, 4, 4>(r, smem, st); break;
    }
}

void hx_slab_launch(int prec, const SlabRun& r, cudaStream_t st) {
    if (r.n_tiles == 0) return;
    const size_t csize = (size_t)(r.lut_real ? 1 : 2) * (prec == 0 ? 8 : 4);
    const size_t smem = (size_t)r.n_lut * (r.lut_mode == 1 ? 128 : csize);
    if (prec == 0) slab_launch_p<0>(r, smem, st);
    else slab_launch_p<1>(r, smem, st);
}

void launch_slab_xscale(int prec, const void* x, const unsigned char* cls, const void* scale, void* out,
                        int64_t c0, int64_t c1, cudaStream_t st) {
    if (c1 <= c0) return;
    const int blocks = xscale_blocks(c1 - c0);
    if (prec == 0)
        k_slab_xscale<double2, double><<<blocks, 256, 0, st>>>((const double2*)x, cls, (const double*)scale,
                                                              (double2*)out, c0, c1);
    else
        k_slab_xscale<float2, float><<<blocks, 256, 0, st>>>((const float2*)x, cls, (const float*)scale,
                                                            (float2*)out, c0, c1);
    EDGPU_CUDA(cudaGetLastError());
}

void launch_slab_xscale_c128_c64(const double* x, const unsigned char* cls, const float* scale, float* out,
                                 int64_t c0, int64_t c1, cudaStream_t st) {
    if (c1 <= c0) return;
    k_slab_xscale_c128_c64<<<xscale_blocks(c1 - c0), 256, 0, st>>>((const double2*)x, cls, scale, (float2*)out,
                                                                  c0, c1);
    EDGPU_CUDA(cudaGetLastError());
}

}  // namespace edgpu
