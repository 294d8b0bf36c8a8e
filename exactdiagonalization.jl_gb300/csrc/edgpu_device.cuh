// Device helpers shared by the enumeration and product kernels: group action on basis words
// (orbit minimum and the element that reaches it, stabiliser size, representative test), the key
// encoding of representative tables and the branch-free sorted-table search.
//
// Key encoding.  A table of representatives stores key = (state << sb) | sidx, where sidx (sb bits)
// is the index of the representative's stabiliser size among the divisors of the group order, so the
// orbit norm of any row or found column comes with the key.  Unreduced tables have sb = 0 (key =
// state).  Keys sort like states, so the search compares against (rep << sb) | (2^sb - 1).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "edgpu_internal.h"

namespace edgpu {

template <typename W>
__device__ __forceinline__ W ldg_w(const W* p) { return __ldg(p); }

// T(a,b).q for the torus: rotate every row (rowbits wide) left by s = a*w bits.
// keep = bits at in-row positions [0, rowbits - s), replicated over the rows.
template <typename W>
__device__ __forceinline__ W torus_row_rotate(W r, int s, W keep, W full, int rowbits) {
    return (W)(((r & keep) << s) | ((r & (full ^ keep)) >> (rowbits - s)));
}

// Orbit minimum of q under the torus translations, the first element g (= a + L1*b) reaching it
// (only when want_arg), and the stabiliser size |{g : g.q == q}| (only when want_stab).
template <typename W>
__device__ __forceinline__ void canon_torus(W q, int L1, int L2, int w, int rowbits, int nbits, W full,
                                            const W* keep, bool want_arg, bool want_stab, W& rep, int& gbest,
                                            int& stab) {
    rep = q;
    gbest = 0;
    stab = 0;
    W r = q;
    for (int b = 0; b < L2; ++b) {
        for (int a = 0; a < L1; ++a) {
            const W t = torus_row_rotate<W>(r, a * w, keep[a], full, rowbits);
            if (want_arg) {
                if (t < rep) { rep = t; gbest = a + L1 * b; }
            } else {
                rep = t < rep ? t : rep;
            }
            if (want_stab) stab += (t == q);
        }
        r = (W)(((r << rowbits) | (r >> (nbits - rowbits))) & full);
    }
}

// Torus canonicalisation with top-row pruning (rows of rowbits <= 10 bits, at most TORUS_MAXR rows).
// The numerically smallest translate has the smallest possible top row, M = min over rows j of the
// smallest rotation of row j, so only translates T(a,b) whose top row (row j = L2-1-b rotated by a)
// equals M can be the representative.  rlut[v] = smallest rotation of the row value v (low 16 bits) |
// the set of rotation steps a reaching it (high 16 bits).  The candidates (j, a) are collected into
// one bit set (bit j*L1 + a) first, so the lanes of a warp loop over their own candidates only
// (usually one or two) instead of over the rows.  Exact: candidates are compared as whole words.
// l1inv = ceil(2^16 / L1): j = (c * l1inv) >> 16 for the candidate bit c < 64.

template <typename W>
__device__ __forceinline__ void canon_torus_pruned(W q, int L1, int L2, int w, int rowbits, int nbits, W full,
                                                   const W* keep, const unsigned* rlut, unsigned l1inv, W& rep,
                                                   int& gbest) {
    const unsigned rmask = (1u << rowbits) - 1u;
    unsigned e[TORUS_MAXR];
    unsigned M = 0xffffu;
#pragma unroll
    for (int j = 0; j < TORUS_MAXR; ++j) {
        e[j] = (j < L2) ? rlut[(unsigned)(q >> (j * rowbits)) & rmask] : 0xffffffffu;
        M = min(M, e[j] & 0xffffu);
    }
    unsigned long long cand = 0ull;
#pragma unroll
    for (int j = 0; j < TORUS_MAXR; ++j)
        if ((e[j] & 0xffffu) == M) cand |= (unsigned long long)(e[j] >> 16) << (j * L1);
    rep = full;
    gbest = 0;
    bool first = true;
    while (cand) {
        const int c = __ffsll((long long)cand) - 1;
        cand &= cand - 1ull;
        const int j = (int)(((unsigned)c * l1inv) >> 16);
        const int a = c - j * L1;
        const int b = L2 - 1 - j;
        const int sh = b * rowbits;
        const W rb = sh ? (W)(((q << sh) | (q >> (nbits - sh))) & full) : q;
        const W t = torus_row_rotate<W>(rb, a * w, keep[a], full, rowbits);
        if (first || t < rep) {
            rep = t;
            gbest = a + L1 * b;
            first = false;
        }
    }
}

// The same search with the two top rows (rowbits <= 6, so L1 <= 6): plut[(v_hi << rowbits) | v_lo] =
// the smallest of rot_a(v_hi) << rowbits | rot_a(v_lo) over the row rotations a (high 16 bits) | the
// set of a reaching it (low 8 bits).  A candidate (j, a) must give the smallest pair of top rows (row
// j and the row below it, j-1 mod L2, rotated by a), which leaves far fewer ties than the top row
// alone.  Rows are peeled off 32-bit halves by funnel shifts, candidates sit in 8-bit slots (bit
// 8*j + a of clo:chi), and states of at most 32 bits are translated in 32-bit arithmetic.
// R = the number of rows L2 when it is known at compile time (R == L2), else TORUS_MAXR with the rows
// beyond L2 masked off.
template <typename S, int R>
__device__ __forceinline__ void torus_pair_search(S q, int L1, int L2, int w, int rowbits, int nbits, S full,
                                                  const S* keep, const unsigned* plut, S& rep, int& gbest) {
    const bool exact = R < TORUS_MAXR;
    const unsigned rmask = (1u << rowbits) - 1u;
    unsigned lo = (unsigned)q, hi = sizeof(S) == 8 ? (unsigned)((unsigned long long)q >> 32) : 0u;
    unsigned v[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
        v[j] = lo & rmask;
        lo = __funnelshift_r(lo, hi, rowbits);
        hi >>= rowbits;
    }
    const unsigned vtop = exact ? v[R - 1] : ((unsigned)(q >> ((L2 - 1) * rowbits)) & rmask);
    const unsigned rmul = rmask + 1u;   // table index v_hi * 2^rowbits + v_lo as one multiply-add
    unsigned e[R];
    unsigned Mf = 0xffffffffu;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        e[j] = (exact || j < L2) ? plut[v[j] * rmul + (j ? v[j > 0 ? j - 1 : 0] : vtop)] : 0xffffffffu;
        Mf = min(Mf, e[j]);
    }
    unsigned clo = 0u, chi = 0u;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const unsigned st = ((e[j] ^ Mf) < 0x10000u) ? (e[j] & 0xffu) : 0u;
        if (j < 4) clo |= st << (8 * j);
        else chi |= st << (8 * (j - 4));
    }
    // row-cyclic rotations of a state of at most 32 bits come from one funnel shift of q | q << nbits
    unsigned dlo = 0u, dhi = 0u;
    if constexpr (sizeof(S) == 4) {
        const unsigned long long d = (unsigned long long)q | ((unsigned long long)q << nbits);
        dlo = (unsigned)d;
        dhi = (unsigned)(d >> 32);
    }
    rep = full;
    gbest = 0;
    bool first = true;
    while ((clo | chi) != 0u) {
        const bool use_lo = clo != 0u;
        unsigned x = use_lo ? clo : chi;
        const int c = __ffs((int)x) - 1 + (use_lo ? 0 : 32);
        x &= x - 1u;
        clo = use_lo ? x : clo;
        chi = use_lo ? chi : x;
        const int j = c >> 3, a = c & 7;
        const int b = L2 - 1 - j;
        const int sh = b * rowbits;
        S rb;
        if constexpr (sizeof(S) == 4) rb = (S)(__funnelshift_r(dlo, dhi, nbits - sh) & (unsigned)full);
        else rb = sh ? (S)(((q << sh) | (q >> (nbits - sh))) & full) : q;
        const S t = torus_row_rotate<S>(rb, a * w, keep[a], full, rowbits);
        if (first || t < rep) {
            rep = t;
            gbest = a + L1 * b;
            first = false;
        }
    }
}

template <typename S>
__device__ __forceinline__ void torus_pair_dispatch(S q, int L1, int L2, int w, int rowbits, int nbits, S full,
                                                    const S* keep, const unsigned* plut, S& rep, int& gbest) {
    switch (L2) {   // uniform over the launch
        case 4: torus_pair_search<S, 4>(q, L1, L2, w, rowbits, nbits, full, keep, plut, rep, gbest); return;
        case 5: torus_pair_search<S, 5>(q, L1, L2, w, rowbits, nbits, full, keep, plut, rep, gbest); return;
        case 6: torus_pair_search<S, 6>(q, L1, L2, w, rowbits, nbits, full, keep, plut, rep, gbest); return;
        default: torus_pair_search<S, TORUS_MAXR>(q, L1, L2, w, rowbits, nbits, full, keep, plut, rep, gbest);
    }
}

template <typename W>
__device__ __forceinline__ void canon_torus_pair(W q, int L1, int L2, int w, int rowbits, int nbits, W full,
                                                 const W* keep32, const W* keep, const unsigned* plut, W& rep,
                                                 int& gbest) {
    if (sizeof(W) == 8 && nbits <= 32) {   // 64-bit keys, 32-bit states: canonicalise in 32 bits
        unsigned r;
        torus_pair_dispatch<unsigned>((unsigned)q, L1, L2, w, rowbits, nbits, (unsigned)full, (const unsigned*)keep32,
                                      plut, r, gbest);
        rep = (W)r;
    } else {
        torus_pair_dispatch<W>(q, L1, L2, w, rowbits, nbits, full, keep, plut, rep, gbest);
    }
}

// Ring (L2 == 1) of n <= 31 bits in 32-bit words: rotations by funnel shifts of the doubled word
// d = q | q << n, since bits [n - s, 2n - s) of d are q rotated left by s.  With pb index bits
// (n + pb <= 32) the element index rides in the low bits of each candidate, so a single unsigned
// min yields both the representative and the element reaching it: 3 instructions per element.
__device__ __forceinline__ void canon_ring32(unsigned q, int n, int L1, int w, int pb, bool want_arg,
                                             unsigned& rep, int& gbest) {
    const unsigned mask = (n >= 32) ? 0xffffffffu : ((1u << n) - 1u);
    if (!want_arg) {
        // top-aligned rotations: X holds q twice from its top bit down, so the top 32 bits of X << s
        // are rot_s(q) << (32 - n) followed by bits that only break ties between equal rotations
        const unsigned long long X = ((unsigned long long)q << (64 - n)) | ((unsigned long long)q << (64 - 2 * n));
        const unsigned lo = (unsigned)X, hi = (unsigned)(X >> 32);
        unsigned best = 0xffffffffu;
#pragma unroll 4
        for (int a = 0; a < L1; ++a) best = min(best, __funnelshift_l(lo, hi, a * w));
        rep = best >> (32 - n);
        gbest = 0;
        return;
    }
    if (pb > 0) {
        const unsigned long long d = ((unsigned long long)q | ((unsigned long long)q << n)) << pb;
        const unsigned lo = (unsigned)d, hi = (unsigned)(d >> 32);
        const unsigned kmask = mask << pb;
        unsigned best = 0xffffffffu;
#pragma unroll 4
        for (int a = 0; a < L1; ++a) {
            const unsigned t = (__funnelshift_r(lo, hi, n - a * w) & kmask) | (unsigned)a;
            best = min(best, t);
        }
        rep = best >> pb;
        gbest = (int)(best & ((1u << pb) - 1u));
        return;
    }
    const unsigned long long d = (unsigned long long)q | ((unsigned long long)q << n);
    const unsigned lo = (unsigned)d, hi = (unsigned)(d >> 32);
    unsigned best = 0xffffffffu;
#pragma unroll 4
    for (int a = 0; a < L1; ++a) best = min(best, __funnelshift_r(lo, hi, n - a * w) & mask);
    rep = best;
    gbest = 0;
    if (want_arg) {
#pragma unroll 4
        for (int a = L1 - 1; a >= 0; --a)
            if ((__funnelshift_r(lo, hi, n - a * w) & mask) == best) gbest = a;
    }
}

// The same for 1-bit sites and a compile-time ring length N: fully unrolled with constant shifts.
template <int N>
__device__ __forceinline__ void canon_ring_n(unsigned q, int pb, bool want_arg, unsigned& rep, int& gbest) {
    const unsigned mask = (N >= 32) ? 0xffffffffu : ((1u << N) - 1u);
    if (!want_arg) {   // top-aligned rotations (see canon_ring32): 2 instructions per element
        const unsigned long long X = ((unsigned long long)q << (64 - N)) | ((unsigned long long)q << (64 - 2 * N));
        const unsigned lo = (unsigned)X, hi = (unsigned)(X >> 32);
        unsigned best = 0xffffffffu;
#pragma unroll
        for (int a = 0; a < N; ++a) best = min(best, __funnelshift_l(lo, hi, a));
        rep = best >> (32 - N);
        gbest = 0;
        return;
    }
    if (pb > 0) {
        const unsigned long long d = ((unsigned long long)q | ((unsigned long long)q << N)) << pb;
        const unsigned lo = (unsigned)d, hi = (unsigned)(d >> 32);
        const unsigned kmask = mask << pb;
        unsigned best = 0xffffffffu;
#pragma unroll
        for (int a = 0; a < N; ++a) best = min(best, (__funnelshift_r(lo, hi, N - a) & kmask) | (unsigned)a);
        rep = best >> pb;
        gbest = (int)(best & ((1u << pb) - 1u));
        return;
    }
    const unsigned long long d = (unsigned long long)q | ((unsigned long long)q << N);
    const unsigned lo = (unsigned)d, hi = (unsigned)(d >> 32);
    unsigned best = 0xffffffffu;
#pragma unroll
    for (int a = 0; a < N; ++a) best = min(best, __funnelshift_r(lo, hi, N - a) & mask);
    rep = best;
    gbest = 0;
    if (want_arg) {
#pragma unroll
        for (int a = N - 1; a >= 0; --a)
            if ((__funnelshift_r(lo, hi, N - a) & mask) == best) gbest = a;
    }
}

// Ring canonicalisation dispatched on the (warp-uniform) ring length for 1-bit sites.
__device__ __forceinline__ void canon_ring(unsigned q, int n, int L1, int w, int pb, bool want_arg, unsigned& rep,
                                           int& gbest) {
    if (w == 1) {
        switch (n) {
            case 8: canon_ring_n<8>(q, pb, want_arg, rep, gbest); return;
            case 10: canon_ring_n<10>(q, pb, want_arg, rep, gbest); return;
            case 12: canon_ring_n<12>(q, pb, want_arg, rep, gbest); return;
            case 14: canon_ring_n<14>(q, pb, want_arg, rep, gbest); return;
            case 16: canon_ring_n<16>(q, pb, want_arg, rep, gbest); return;
            case 18: canon_ring_n<18>(q, pb, want_arg, rep, gbest); return;
            case 20: canon_ring_n<20>(q, pb, want_arg, rep, gbest); return;
            case 22: canon_ring_n<22>(q, pb, want_arg, rep, gbest); return;
            case 24: canon_ring_n<24>(q, pb, want_arg, rep, gbest); return;
            case 26: canon_ring_n<26>(q, pb, want_arg, rep, gbest); return;
            case 28: canon_ring_n<28>(q, pb, want_arg, rep, gbest); return;
            case 30: canon_ring_n<30>(q, pb, want_arg, rep, gbest); return;
            default: break;
        }
    }
    canon_ring32(q, n, L1, w, pb, want_arg, rep, gbest);
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
__device__ __forceinline__ void canon_generic(W q, int G, int nchunks, const W* lut, const W* flips,
                                              bool want_stab, W& rep, int& gbest, int& stab) {
    rep = q;
    gbest = 0;
    stab = 0;
    for (int g = 0; g < G; ++g) {
        const W t = generic_apply<W>(q, g, nchunks, lut, flips);
        if (t < rep) { rep = t; gbest = g; }
        if (want_stab) stab += (t == q);
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

// Branch-free search of a sorted key table for the state `rep` (keys carry sb low index bits).
// The iteration count depends on n only, so the lanes of a warp stay converged.  Returns the index
// or -1 (get(FrozenSortedArrayIndex, key, -1)); *key_out receives the key found.
template <typename W>
__device__ __forceinline__ long long key_find(const W* __restrict__ keys, long long n, W rep, int sb, W* key_out) {
    const W target = (W)((rep << sb) | (W)((((W)1) << sb) - 1));
    long long lo = 0, len = n;
    while (len > 1) {
        const long long half = len >> 1;
        lo = (ldg_w(keys + lo + half) <= target) ? lo + half : lo;
        len -= half;
    }
    const W k = (n > 0) ? ldg_w(keys + lo) : (W)0;
    if (key_out) *key_out = k;
    return (n > 0 && (k >> sb) == rep) ? lo : -1;
}

// Bucketed branch-free search with bucket summaries.  The table of keys is split into buckets by
// state >> shift; dir[b] summarises bucket b in one 64-bit word:
//     bits  0..31  index of the bucket's first key (start)
//     bits 32..35  number of keys in the bucket, saturated at 15
//     bits 36..63  the low mb = shift + sb bits of each key of the bucket, K of them (K*mb <= 28)
// A bucket with at most K keys is answered from its summary alone; a larger one by a branch-free
// window search of `steps` halvings in the sorted keys between start and the next bucket's start.
// dir[nb] is a sentinel (start = n, count 0); buckets past the last key clamp to it.
template <typename W>
__device__ __forceinline__ void key_find_sum2(const W* __restrict__ keys, const DirSearch& d, const W* rep,
                                              const bool* act, long long* c, int* sidx) {
    const unsigned smask = (1u << d.sb) - 1u;
    unsigned long long e[2];
    unsigned bk[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const unsigned long long b = (unsigned long long)(rep[h] >> d.shift);
        bk[h] = (unsigned)min(b, (unsigned long long)d.nb);
        e[h] = act[h] ? __ldg(d.dir + bk[h]) : 0ull;
    }
    bool slow[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const unsigned start = (unsigned)e[h];
        const unsigned hi = (unsigned)(e[h] >> 32);
        const int cnt = (int)(hi & 15u);
        const unsigned field = hi >> 4;                                   // K members of mb bits
        const unsigned want = ((unsigned)rep[h] & ((1u << d.shift) - 1u)) << d.sb;   // member bits without sidx
        // fields equal to want (state bits only) have all-zero x; the top bit of t marks nonzero fields
        const unsigned x = (field ^ (want * d.unit)) & d.keybits;
        const unsigned t = ((x & d.low) + d.low) | x;
        slow[h] = act[h] && cnt > d.K;
        const unsigned valid = slow[h] ? 0u : (d.top & ((1u << (cnt * d.mb)) - 1u));   // the bucket's members
        const unsigned hits = ~t & valid;
        const int pos = __ffs((int)hits) - 1;                             // top bit of the first match
        const bool found = act[h] && hits != 0u;
        c[h] = found ? (long long)(start + (unsigned)__popc(d.top & ((1u << pos) - 1u))) : -1;
        sidx[h] = found ? (int)((field >> (pos + 1 - d.mb)) & smask) : 0;
    }
    if (slow[0] || slow[1]) {   // buckets larger than K: search the keys
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (!slow[h]) continue;
            unsigned lo = (unsigned)e[h];
            int len = (int)((unsigned)__ldg(d.dir + bk[h] + 1) - lo);
            const W target = (W)((rep[h] << d.sb) | (W)smask);
            for (int k = 0; k < d.steps; ++k) {
                const int half = len >> 1;
                if (half > 0) {
                    lo = (ldg_w(keys + lo + half) <= target) ? lo + half : lo;
                    len -= half;
                }
            }
            const W kk = ldg_w(keys + lo);
            if ((kk >> d.sb) == rep[h]) {
                c[h] = lo;
                sidx[h] = (int)(kk & (W)smask);
            }
        }
    }
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
