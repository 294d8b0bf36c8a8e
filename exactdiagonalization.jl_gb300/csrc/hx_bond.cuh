// Pair-flip schedule of the matrix-free product y = H x, for operators whose off-diagonal terms all
// flip two sites of one bit each (spin-1/2 exchange S+S- + S-S+, and S+S+ / S-S- pair terms): every
// XXZ, Heisenberg and J1-J2 Hamiltonian built from pauli_matrix products.
//
// Replaces the same reference loop as hx_rows.cuh (apply_serial!/apply_parallel! over
// get_row_iterator, abstract_operator_representation.jl:296-316, reduced_operator_representation.jl:
// 57-85), with the same elements; only the way a row finds its matching terms differs.  The
// reference tests every term of the SumOperator against the row (operator_iterator.jl:48-54); for a
// pair-flip term on sites (i, j) the match depends only on whether bits i and j are equal.
//
// The pairs are grouped on the host into bond classes.  Within a class every pair (i, j) is oriented
// so that its start bits i are distinct, and the class is a union of at most BOND_MAXC rotation
// components: pairs with j = (i + s) mod n for one shift s.  For a row state b, the bits of
//     x_s = b ^ rotr_n(b, s)                       (bit i of x_s: b_i != b_{i+s})
// give every pair of component s whose two bits differ, so
//     D = OR_s (x_s & A_s) | (~x_s & P_s)
// (A_s: starts of pairs with a term on antiparallel bits, P_s: on parallel bits) is the set of the
// class's matching pairs, found with a handful of word operations instead of one test per term.  On
// a translation-invariant lattice a class is one bond direction (a chain: one class of one component;
// the 6x6 J1-J2 torus: four classes).  Each lane owns one row (or 1/lpr of its pairs, split by start
// bit) and walks its classes' set bits, two targets per step: flip mask and amplitude from shared
// memory (amplitude indexed by the start bit's value and parallel/antiparallel), then the parent-state
// map or canonicalisation plus search, the gather of x, and accumulation in registers.  The summation
// order (class, then start bit) is fixed, so results are bit-identical run to run.
#pragma once

#include "hx_rows.cuh"

namespace edgpu {

// Shared-memory views of the bond-class tables (offsets in HxParams):
//   comp  [ncls][BOND_MAXC][4] words: shift s, antiparallel starts A, parallel starts P, unused
//   ninfo [ncls] ints: components | has_parallel << 8
//   flip  [ncls][n] words: flip mask of the pair starting at bit i (0 when there is none)
//   amp   [ncls][n][4] amplitudes by v = b_i | (b_i == b_j) << 1
template <typename W, int PREC>
struct BondTables {
    typedef typename Cx<PREC>::V V;
    const W* comp;
    const int* ninfo;
    const W* flip;
    const V* amp;
    __device__ __forceinline__ BondTables(const HxParams& p, const unsigned char* sm) {
        comp = (const W*)(sm + p.o_bcomp);
        ninfo = (const int*)(sm + p.o_binfo);
        flip = (const W*)(sm + p.o_bflip);
        amp = (const V*)(sm + p.o_bamp);
    }
};

// Matching pairs of class cls for the row state b (n parent bits, full = the n-bit mask).
template <typename W, int PREC>
__device__ __forceinline__ W bond_class_mask(W b, const BondTables<W, PREC>& bt, int cls, int n, W full) {
    const int info = bt.ninfo[cls];
    const int nc = info & 0xff;
    W D = 0;
    for (int k = 0; k < nc; ++k) {
        const W* cp = bt.comp + 4 * (cls * BOND_MAXC + k);
        W s_w, A, P;
        load_rec3<W>(cp, s_w, A, P);
        const int s = (int)s_w;
        const W r = (W)(((b >> s) | (b << (n - s))) & full);   // bit i = b_{(i + s) mod n}
        const W xs = b ^ r;
        D |= (xs & A) | (~xs & P);
    }
    return D;
}

// Programmatic dependent launch (griddepcontrol): no-ops when the launch did not enable it.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ double fma_r(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_r(float a, float b, float c) { return __fmaf_rn(a, b, c); }

template <typename W>
__device__ __forceinline__ int lowest_bit(W m) {
    if constexpr (sizeof(W) == 8) return __ffsll((long long)m) - 1;
    else return __ffs((int)m) - 1;
}

// Entry of the target table at pos (map format: c | sx << cb | g << (cb + sb); all ones when the
// target's orbit has no representative in the table).
template <int PREC>
__device__ __forceinline__ void table_entry(const RowsSector<PREC>& sc, long long pos, bool on, int sb, long long& c,
                                            int& sx, int& g) {
    if (!sc.tab_wide) {
        const unsigned e = on ? __ldg((const unsigned*)sc.tab + pos) : 0xffffffffu;
        const unsigned cmask = (sc.tab_cb >= 32) ? 0xffffffffu : ((1u << sc.tab_cb) - 1u);
        const unsigned ci = e & cmask;
        c = (ci == cmask) ? -1 : (long long)ci;
        sx = (int)((e >> sc.tab_cb) & ((1u << sb) - 1u));
        g = (int)((e >> (sc.tab_cb + sb)) & 0xfffu);
    } else {
        const unsigned long long e = on ? __ldg((const unsigned long long*)sc.tab + pos) : ~0ull;
        const unsigned long long cmask = (1ull << sc.tab_cb) - 1ull;
        const unsigned long long ci = e & cmask;
        c = (ci == cmask) ? -1 : (long long)ci;
        sx = (int)((e >> sc.tab_cb) & ((1ull << sb) - 1ull));
        g = (int)((e >> (sc.tab_cb + sb)) & 0xfffull);
    }
}

// Prefetch into L2 the x element of the target-table entry at pos (nothing for an entry without a
// representative), so that the product's later gather of it does not wait for DRAM.
template <int PREC>
__device__ __forceinline__ void table_prefetch_x(const RowsSector<PREC>& sc, long long pos, int sb) {
    long long c;
    int sx, g;
    table_entry<PREC>(sc, pos, true, sb, c, sx, g);
    if (c >= 0) asm volatile("prefetch.global.L2 [%0];" ::"l"(sc.x + c));
}

// OR of a word over the warp.
template <typename W>
__device__ __forceinline__ W warp_or(W v) {
    if constexpr (sizeof(W) == 8) {
        const unsigned lo = __reduce_or_sync(0xffffffffu, (unsigned)v);
        const unsigned hi = __reduce_or_sync(0xffffffffu, (unsigned)(v >> 32));
        return (W)lo | ((W)hi << 32);
    } else {
        return (W)__reduce_or_sync(0xffffffffu, (unsigned)v);
    }
}

// Matching pairs of every class of the row state b (lpr == 1): the row's number of targets.
template <typename W, int PREC>
__device__ __forceinline__ int bond_row_count(W b, const BondTables<W, PREC>& bt, int ncls, int n, W full) {
    int cnt = 0;
    for (int c = 0; c < ncls; ++c) cnt += __popcll((unsigned long long)bond_class_mask<W, PREC>(b, bt, c, n, full));
    return cnt;
}

// One warp tile of rows (32 / lpr consecutive rows of the sector, lpr lanes each) of the pair-flip
// schedule; lane sub of a row takes the pairs whose start bit i has i % lpr == sub.  NT targets per
// lane and step (2 or 4): their lookups, then their gathers, are issued together.
//   GK_TABLE  the targets' entries are read from the sector's target table (lpr == 1) in this order;
//   FILL      the build pass of that table: the entries are looked up with the flavour GK and written
//             to the table (sc.tab) instead of being gathered and accumulated;
//   UNI       warp-uniform steps (lpr == 1): the warp walks the union of its lanes' matching pairs,
//             class by class and start bit by start bit, and in every step each lane takes the pairs
//             of that step its row matches.  Lanes of one step gather the targets of one bond pair of
//             32 consecutive representatives, which often share a DRAM sector of x (a target whose
//             representative is itself lies next to the targets of the neighbouring rows), so a warp
//             issues fewer sector requests than when each lane walks its own matches.  Every lane still
//             visits its pairs by class, then start bit, so the table positions and the summation
//             order, hence the results, are the same as without UNI;
//   GRAD      the coupling gradient fused with the product: every target also adds
//             Re(conj(gy_r) u x_c), with u its unit-coupling element, to the accumulator of its slot's
//             coupling (sgrad[coupling][thread], one slot per thread: no atomics, so the sums are
//             reproducible), and every diagonal term matching the row adds Re(u_t z_r) with
//             z_r = conj(gy_r) x_r.  The accumulators have the product's arithmetic type R (FP32 in
//             mixed precision: a thread adds a few dozen terms before the block sums them in FP64).
//   ADJ       (1 or 2, with GK_TABLE) the passes that build the adjoint target table: 1 counts every
//             target on its column, 2 writes row, slot, the row's orbit-size index and the group
//             element into the column's run.
template <typename W, int GK, int PREC, int NT, bool FILL = false, bool UNI = false, bool GRAD = false, int ADJ = 0>
__device__ __forceinline__ void bond_tile(const HxParams& p, const RowsTables<W, PREC>& tb,
                                          const BondTables<W, PREC>& bt, const RowsSector<PREC>& sc, long long tile,
                                          int lane, typename Cx<PREC>::R* sgrad = nullptr) {
    typedef typename Cx<PREC>::V V;
    typedef typename Cx<PREC>::R R;
    const W* __restrict__ keys = (const W*)sc.keys;
    const V* __restrict__ x = sc.x;
    const int sb = p.sb;
    const W smask = (W)((((W)1) << sb) - 1);
    const int lpr = p.lpr, sub = lane & (lpr - 1), rpw = 32 / lpr;
    const long long row = tile * rpw + lane / lpr;
    const bool act = row < sc.n_rows;
    const W kr = act ? keys[row] : (W)0;
    const W b = kr >> sb;
    const int ri = (int)(kr & smask);
    V acc = czero<V>();
    V gv = czero<V>();   // GRAD: gy of the row
    if (!FILL && ADJ == 0) {
        const V xr = act ? x[row] : czero<V>();
        if (act && sub == 0) acc = cmul(sc.diag[row], xr);
        if (GRAD) {
            gv = act ? ((const V*)p.gy)[row] : czero<V>();
            if (act && sub == 0) {
                const unsigned char* smb = (const unsigned char*)bt.comp - p.o_bcomp;
                const W* dm = (const W*)(smb + p.o_pdm);
                const W* dr = (const W*)(smb + p.o_pdr);
                const V* du = (const V*)(smb + p.o_pdu);
                const int* dc = (const int*)(smb + p.o_pdc);
                // z = conj(gy_r) x_r; a term's share is Re(u z) = u.x z.x - u.y z.y
                const R zr = gv.x * xr.x + gv.y * xr.y, zi = gv.x * xr.y - gv.y * xr.x;
                if (p.n_pdb >= 0) {
                    // one entry per (site pair, coupling): the unit amplitude of the row's two bits
                    const int* db = (const int*)(smb + p.o_pdb);
                    const V* dv = (const V*)(smb + p.o_pdv);
                    for (int k = 0; k < p.n_pdb; ++k) {
                        const int e = db[k];
                        const int pat = (int)((b >> (e & 0xff)) & 1) | ((int)((b >> ((e >> 8) & 0xff)) & 1) << 1);
                        const V u = dv[k * 4 + pat];
                        R& a = sgrad[(e >> 16) * HX_THREADS + threadIdx.x];
                        a = fma_r(u.x, zr, fma_r(-u.y, zi, a));
                    }
                } else {
                    for (int t = 0; t < p.T_d; ++t)
                        if ((b & dm[t]) == dr[t]) {
                            R& a = sgrad[dc[t] * HX_THREADS + threadIdx.x];
                            a = fma_r(du[t].x, zr, fma_r(-du[t].y, zi, a));
                        }
                }
            }
        }
    }
    const int n = p.nbits;
    const W full = (W)p.full;
    // start bits of this lane: i % lpr == sub
    const W split = lpr == 1 ? (W)~(W)0
                             : (W)((lpr == 2 ? (W)0x5555555555555555ull : (W)0x1111111111111111ull) << sub);
    const int ncls = act ? p.bond_ncls : 0;
    const R* __restrict__ rrow = tb.ratio + ri * p.nd;
    const bool real_fast = p.bond_real && !sc.want_arg;
    // target table position of this lane's first target: the tile's offset plus the targets of the
    // rows before it in the tile
    long long tpos = 0, tend = 0, tpf = 0;
    if (GK == GK_TABLE || FILL) {
        const int cnt = bond_row_count<W, PREC>(b, bt, ncls, n, full);
        int incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += u;
        }
        tpos = sc.tile_off[tile] + (incl - cnt);
        tend = tpos + cnt;
        tpf = tpos;
        // software prefetch of the gathers: the x elements of the first bond_pf steps' targets now,
        // then NT more each step (bond_pf steps ahead)
        if (GK == GK_TABLE && !FILL && p.bond_pf > 0) {
            const long long lim = min(tend, tpos + (long long)p.bond_pf * NT);
            for (; tpf < lim; ++tpf) table_prefetch_x<PREC>(sc, tpf, sb);
        }
    }
    int cls = -1;
    bool cpar = false;   // the current class has terms on parallel bits
    W m = 0;
    while (true) {
        if constexpr (UNI) {
            // the warp moves on to the next class once no lane has pairs left in this one
            while (!__any_sync(0xffffffffu, m != 0) && cls + 1 < p.bond_ncls) {
                ++cls;
                m = act ? (bond_class_mask<W, PREC>(b, bt, cls, n, full) & split) : (W)0;
                cpar = (bt.ninfo[cls] >> 8) != 0;
            }
        } else {
            // lanes whose class ran out move on to their next class with matching pairs
            while (m == 0 && cls + 1 < ncls) {
                ++cls;
                m = bond_class_mask<W, PREC>(b, bt, cls, n, full) & split;
                cpar = (bt.ninfo[cls] >> 8) != 0;
            }
        }
        if (!__any_sync(0xffffffffu, m != 0)) break;
        int ti[NT];
        bool on[NT];
        W q[NT];
        int g[NT], sx[NT];
        long long c[NT];
        W u = 0;   // UNI: the pairs of this class some lane of the warp still has to visit
        if constexpr (UNI) u = warp_or<W>(m);
#pragma unroll
        for (int h = 0; h < NT; ++h) {
            int i;
            if constexpr (UNI) {
                const bool any = u != 0;
                i = any ? lowest_bit<W>(u) : 0;
                u &= u - 1;
                on[h] = any && ((m >> i) & 1);
                if (on[h]) m &= ~((W)1 << i);
            } else {
                on[h] = m != 0;
                i = on[h] ? lowest_bit<W>(m) : 0;
                m &= m - 1;
            }
            ti[h] = on[h] ? cls * n + i : 0;
            // (a table read needs the flip mask only for the parallel test)
            const W f = (GK != GK_TABLE || cpar) ? bt.flip[ti[h]] : (W)0;
            q[h] = b ^ f;
            // amplitude slot: b_i, and whether the pair's bits are parallel (classes with such terms)
            int v = (int)(b >> i) & 1;
            if (cpar) v |= (__popcll((unsigned long long)(b & f)) != 1) << 1;
            ti[h] = (ti[h] << 2) | v;
        }
        if constexpr (GK == GK_TABLE) {
#pragma unroll
            for (int h = 0; h < NT; ++h) {
                table_entry<PREC>(sc, tpos, on[h], sb, c[h], sx[h], g[h]);
                tpos += on[h] ? 1 : 0;
            }
            if (!FILL && p.bond_pf > 0) {
                const long long lim = min(tend, tpf + NT);
                for (; tpf < lim; ++tpf) table_prefetch_x<PREC>(sc, tpf, sb);
            }
        } else {
#pragma unroll
            for (int h = 0; h < NT; h += 2)
                resolve_targets2<W, GK, PREC>(p, tb, sc, q + h, on + h, c + h, sx + h, g + h);
        }
        if constexpr (ADJ != 0) {
#pragma unroll
            for (int h = 0; h < NT; ++h) {
                if (!on[h] || c[h] < 0) continue;
                if (ADJ == 1) {
                    atomicAdd(p.adj_cnt + c[h], 1u);
                } else {
                    const long long pos = p.adj_off[c[h]] + (long long)atomicAdd(p.adj_cur + c[h], 1u);
                    p.adj_tab[pos] = ((unsigned long long)row << 32) | ((unsigned long long)ti[h] << 19) |
                                     ((unsigned long long)ri << 14) | (unsigned long long)(g[h] & 0x3fff);
                }
            }
            continue;
        }
        if constexpr (FILL) {
            const bool with_g = sc.want_arg;
#pragma unroll
            for (int h = 0; h < NT; ++h) {
                if (!on[h]) continue;
                unsigned long long e = ~0ull;
                if (c[h] >= 0) {
                    e = (unsigned long long)c[h] | ((unsigned long long)sx[h] << sc.tab_cb);
                    if (with_g) e |= (unsigned long long)g[h] << (sc.tab_cb + sb);
                }
                if (sc.tab_wide) ((unsigned long long*)sc.tab)[tpos] = e;
                else ((unsigned*)sc.tab)[tpos] = (unsigned)e;
                ++tpos;
            }
            continue;
        }
        V xv[NT];
#pragma unroll
        for (int h = 0; h < NT; ++h) xv[h] = (c[h] >= 0) ? x[c[h]] : czero<V>();
#pragma unroll
        for (int h = 0; h < NT; ++h) {
            if (GRAD && c[h] >= 0) {
                const unsigned char* smb = (const unsigned char*)bt.comp - p.o_bcomp;
                const V u0 = ((const V*)(smb + p.o_bunit))[ti[h]];
                const int cid = ((const int*)(smb + p.o_bcid))[ti[h]];
                R& a = sgrad[cid * HX_THREADS + threadIdx.x];
                if (p.bunit_real && !sc.want_arg) {
                    // real unit amplitude, trivial characters: u x_c is a real multiple of x_c
                    const R f = GK == GK_TRIVIAL ? u0.x : u0.x * rrow[sx[h]];
                    a = fma_r(f, gv.x * xv[h].x + gv.y * xv[h].y, a);
                } else {
                    V u = u0;
                    if (GK != GK_TRIVIAL) {
                        if (sc.want_arg) u = cmul(u, sc.ph[sc.num[g[h]]]);
                        u = cscale(u, rrow[sx[h]]);
                    }
                    const V t = cmul(u, xv[h]);
                    a += gv.x * t.x + gv.y * t.y;
                }
            }
            if (c[h] >= 0) {
                const V a = bt.amp[ti[h]];
                if (GK == GK_TRIVIAL) {
                    acc = cadd(acc, cmul(a, xv[h]));
                } else if (real_fast) {
                    // real amplitude, trivial characters: one scale and two fused multiply-adds
                    const R f = a.x * rrow[sx[h]];
                    acc.x = fma_r(f, xv[h].x, acc.x);
                    acc.y = fma_r(f, xv[h].y, acc.y);
                } else if (p.bond_real) {
                    // real amplitude times the character: chi(g) (a sqrt(|O_r| / |O_c|))
                    const R f = a.x * rrow[sx[h]];
                    const V ph = sc.ph[sc.num[g[h]]];
                    acc = cadd(acc, cmul(cscale(ph, f), xv[h]));
                } else {
                    V coef = a;
                    if (sc.want_arg) coef = cmul(coef, sc.ph[sc.num[g[h]]]);
                    coef = cscale(coef, rrow[sx[h]]);
                    acc = cadd(acc, cmul(coef, xv[h]));
                }
            }
        }
    }
    if (FILL || ADJ != 0) return;
    // partial sums of the row's lanes (fixed butterfly order)
    for (int d = 1; d < lpr; d <<= 1) acc = cadd(acc, shfl_xor_v(acc, d));
    if (act && sub == 0) {
        if (PREC == 1 && p.y_c128) {
            // complex128 output (the host-buffer product, written to the caller's buffer): the
            // complex64 result widened, plus the old value for apply!, as the separate conversion does
            double2* y2 = (double2*)p.y_c128;
            double2 o = make_double2((double)acc.x, (double)acc.y);
            if (p.accumulate) {
                const double2 a = y2[row];
                o.x += a.x;
                o.y += a.y;
            }
            y2[row] = o;
        } else {
            if (p.accumulate) acc = cadd(acc, sc.y[row]);
            sc.y[row] = acc;
        }
    }
}

template <typename W, int GK, int PREC, int NT, bool UNI = false>
__global__ void __launch_bounds__(HX_THREADS) hx_bond_kernel(const HxParams p) {
    typedef typename Cx<PREC>::V V;
    extern __shared__ __align__(16) unsigned char sm[];
    // programmatic dependent launch: the next kernel in the stream may start its own prologue now;
    // this kernel copies its (constant) tables, then waits for the previous kernel in the stream to
    // complete before touching any vector or table it may have written
    pdl_launch_dependents();
    {
        const int4* src = (const int4*)p.blob;
        int4* dst = (int4*)sm;
        for (int i = threadIdx.x; i < p.blob_words16; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    pdl_wait();
    const RowsTables<W, PREC> tb(p, sm);
    const BondTables<W, PREC> bt(p, sm);
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
    sc.tab = p.tab;
    sc.tile_off = p.tile_off;
    sc.tab_wide = p.tab_wide;
    sc.tab_cb = p.tab_cb;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const int rpw = 32 / p.lpr;
    const long long n_tiles = (p.n_rows + rpw - 1) / rpw;
    for (long long tile = (long long)blockIdx.x * wpb + warp; tile < n_tiles; tile += (long long)gridDim.x * wpb)
        bond_tile<W, GK, PREC, NT, false, UNI>(p, tb, bt, sc, tile, lane);
}

// All sectors of a batch in one persistent launch (the tile numbering of hx_multi_kernel).  With eight
// targets per step the kernel is held to three resident blocks per SM instead of four, so that like the
// one-sector launch it keeps its eight entries and gathers in registers.
template <typename W, int GK, int PREC, int NT>
__global__ void __launch_bounds__(HX_THREADS, NT == 8 ? 3 : 4) hx_bond_multi_kernel(const HxParams p) {
    typedef typename Cx<PREC>::V V;
    extern __shared__ __align__(16) unsigned char sm[];
    // programmatic dependent launch: the next kernel in the stream may start its own prologue now;
    // this kernel copies its (constant) tables, then waits for the previous kernel in the stream to
    // complete before touching any vector or table it may have written
    pdl_launch_dependents();
    {
        const int4* src = (const int4*)p.blob;
        int4* dst = (int4*)sm;
        for (int i = threadIdx.x; i < p.blob_words16; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    pdl_wait();
    const RowsTables<W, PREC> tb(p, sm);
    const BondTables<W, PREC> bt(p, sm);
    const SectorDesc* sec = (const SectorDesc*)(sm + p.o_sec);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    int s = 0;
    long long tile0 = 0;
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
        sc.tab = d.tab;
        sc.tile_off = d.tile_off;
        sc.tab_wide = d.tab_wide;
        sc.tab_cb = d.tab_cb;
        bond_tile<W, GK, PREC, NT>(p, tb, bt, sc, tile - tile0, lane);
    }
}

// The product fused with the coupling gradient (GRAD), one sector; GK is GK_MAP or GK_TABLE.  Shared
// memory: the pair-flip image, then n_couplings x HX_THREADS FP64 accumulators (p.o_grad); each
// block writes its sums, reduced over its threads in a fixed order, to grad_partial[block][coupling].
template <typename W, int GK, int PREC, int NT>
__global__ void __launch_bounds__(HX_THREADS) hx_bond_grad_kernel(const HxParams p) {
    typedef typename Cx<PREC>::V V;
    extern __shared__ __align__(16) unsigned char sm[];
    {
        const int4* src = (const int4*)p.blob;
        int4* dst = (int4*)sm;
        for (int i = threadIdx.x; i < p.blob_words16; i += blockDim.x) dst[i] = src[i];
    }
    typedef typename Cx<PREC>::R R;
    R* sgrad = (R*)(sm + p.o_grad);
    for (int i = threadIdx.x; i < p.n_coupl * HX_THREADS; i += blockDim.x) sgrad[i] = (R)0;
    __syncthreads();
    const RowsTables<W, PREC> tb(p, sm);
    const BondTables<W, PREC> bt(p, sm);
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
    sc.tab = p.tab;
    sc.tile_off = p.tile_off;
    sc.tab_wide = p.tab_wide;
    sc.tab_cb = p.tab_cb;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const int rpw = 32 / p.lpr;
    const long long n_tiles = (p.n_rows + rpw - 1) / rpw;
    for (long long tile = (long long)blockIdx.x * wpb + warp; tile < n_tiles; tile += (long long)gridDim.x * wpb)
        bond_tile<W, GK, PREC, NT, false, false, true>(p, tb, bt, sc, tile, lane, sgrad);
    __syncthreads();
    // block sums in FP64, one warp per coupling: lane l adds the accumulators of threads l, l + 32, ...
    // in turn, then a butterfly over the lanes (a fixed order)
    for (int i = warp; i < p.n_coupl; i += wpb) {
        double sum = 0.0;
        for (int t = lane; t < HX_THREADS; t += 32) sum += (double)sgrad[i * HX_THREADS + t];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, d);
        if (lane == 0) p.grad_partial[(size_t)blockIdx.x * p.n_coupl + i] = sum;
    }
}

// Launch with programmatic stream serialisation: the kernel may begin while the previous kernel in
// the stream finishes (it waits for it with griddepcontrol.wait before reading any vector).
template <typename K>
void pdl_launch(K kern, const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
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
    EDGPU_CUDA(cudaLaunchKernelEx(&cfg, kern, p));
}

template <typename W, int GK, int PREC, int NT, bool UNI = false>
void hx_bond_launch_one(const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    auto kern = hx_bond_kernel<W, GK, PREC, NT, UNI>;
    raise_smem_limit((const void*)kern, smem);
    pdl_launch(kern, p, blocks, smem, st);
}

template <typename W, int GK, int PREC, int NT, bool UNI = false>
int hx_bond_occupancy_one(size_t smem) {
    auto kern = hx_bond_kernel<W, GK, PREC, NT, UNI>;
    raise_smem_limit((const void*)kern, smem);
    int n = 0;
    EDGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, HX_THREADS, smem));
    return n;
}

template <typename W, int GK, int PREC, int NT>
void hx_bond_multi_launch_one(const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    auto kern = hx_bond_multi_kernel<W, GK, PREC, NT>;
    raise_smem_limit((const void*)kern, smem);
    pdl_launch(kern, p, blocks, smem, st);
}

template <typename W, int GK, int PREC, int NT>
int hx_bond_multi_occupancy_one(size_t smem) {
    auto kern = hx_bond_multi_kernel<W, GK, PREC, NT>;
    raise_smem_limit((const void*)kern, smem);
    int n = 0;
    EDGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, HX_THREADS, smem));
    return n;
}

}  // namespace edgpu

namespace edgpu {

template <typename W, int GK, int PREC, int NT>
void hx_bond_grad_launch_one(const HxParams& p, int blocks, size_t smem, cudaStream_t st) {
    auto kern = hx_bond_grad_kernel<W, GK, PREC, NT>;
    raise_smem_limit((const void*)kern, smem);
    kern<<<blocks, HX_THREADS, smem, st>>>(p);
    EDGPU_CUDA(cudaGetLastError());
}

template <typename W, int GK, int PREC, int NT>
int hx_bond_grad_occupancy_one(size_t smem) {
    auto kern = hx_bond_grad_kernel<W, GK, PREC, NT>;
    raise_smem_limit((const void*)kern, smem);
    int n = 0;
    EDGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, HX_THREADS, smem));
    return n;
}

}  // namespace edgpu
