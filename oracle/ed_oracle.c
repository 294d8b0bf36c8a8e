/*
 * ed_oracle.c -- CPU restatement of ExactDiagonalization.jl's symmetry-reduced
 * Hamiltonian application, used ONLY as test infrastructure (the checker in
 * tests/, the parity check in __graft_entry__.smoke() and the CPU baseline leg
 * of bench.py).  Nothing in the product library links or calls this file.
 *
 * Every function follows the reference's algorithm and data structures
 * (parent-sized mapping tables, binary search over the parent basis, the
 * visited-flag orbit sweep), not the GPU design.  Citations are to files of
 * kyungminlee/ExactDiagonalization.jl v0.14.3.
 *
 * Conventions: indices are 0-based here (the reference is 1-based); "absent"
 * is -1 in both.  Complex numbers are interleaved (re, im) doubles.  Compile
 * with -ffp-contract=off so products are not fused, as in Julia's Complex{Float64}
 * arithmetic.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cplx;

static inline cplx c_mul(cplx a, cplx b) {
    /* Base.:*(::Complex, ::Complex): (ar*br - ai*bi) + (ar*bi + ai*br)i */
    cplx r; r.re = a.re * b.re - a.im * b.im; r.im = a.re * b.im + a.im * b.re; return r;
}
static inline cplx c_add(cplx a, cplx b) { cplx r; r.re = a.re + b.re; r.im = a.im + b.im; return r; }
static inline cplx c_conj(cplx a) { cplx r; r.re = a.re; r.im = -a.im; return r; }
static inline cplx c_inv(cplx a) {
    /* one(S) / a for |a| ~ 1/sqrt(k): the naive formula is within an ulp of Julia's scaled division */
    double d = a.re * a.re + a.im * a.im; cplx r; r.re = a.re / d; r.im = -a.im / d; return r;
}

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* fs_index / get(lookup, key, -1): searchsortedfirst then equality check.
 * frozensortedarray.jl:29-32, :45-48 */
int64_t or_lookup(const uint64_t* keys, int64_t n, uint64_t key) {
    int64_t lo = 0, len = n;
    while (len > 0) {                       /* searchsortedfirst */
        int64_t half = len >> 1;
        if (keys[lo + half] < key) { lo = lo + half + 1; len = len - half - 1; }
        else len = half;
    }
    return (lo < n && keys[lo] == key) ? lo : -1;
}

void or_lookup_many(const uint64_t* keys, int64_t n, const uint64_t* q, int64_t m, int64_t* out) {
    for (int64_t i = 0; i < m; ++i) out[i] = or_lookup(keys, n, q[i]);
}

/* symmetry_apply(hs, ::SitePermutation, bitrep): the field of site i moves to
 * site map[i].  symmetry_apply.jl:82-92.  A GlobalBitFlip factor (bitflipsymmetry.jl:23-35)
 * is applied afterwards as XOR with flip (the DirectProductOperation order of
 * symmetry_apply.jl:65-77 is immaterial: both commute with each other on bits). */
uint64_t or_symmetry_apply(int n_sites, const int32_t* bitwidths, const int32_t* bitoffsets,
                           const int32_t* map, uint64_t flip, uint64_t b) {
    uint64_t out = 0;
    for (int i = 0; i < n_sites; ++i) {
        uint64_t m = (bitwidths[i] >= 64) ? ~0ull : ((1ull << bitwidths[i]) - 1ull);
        out |= ((b >> bitoffsets[i]) & m) << bitoffsets[map[i]];
    }
    return out ^ flip;
}

/* symmetry_reduce_serial(hsr, symops_and_amplitudes; tol) -- symmetry_reduce_generic.jl:22-106.
 * Element 0 must be the identity (":20  The irreps have to follow certain order").
 * ampl[g] are the amplitudes y of the (symop, y) pairs; the phase of member g.b is conj(y*sgn), sgn=1.
 * Outputs: reps_out (capacity n_parent) -> returns the reduced dimension;
 *          map_index[n_parent] (reduced index or -1); map_ampl[2*n_parent]. */
int64_t or_symmetry_reduce(const uint64_t* parent, int64_t n_parent,
                           int n_sites, const int32_t* bitwidths, const int32_t* bitoffsets,
                           int G, const int32_t* maps, const uint64_t* flips,
                           const double* ampl, double tol,
                           uint64_t* reps_out, int64_t* map_index, double* map_ampl) {
    int64_t* rep_of = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n_parent > 0 ? n_parent : 1));
    uint8_t* visited = (uint8_t*)calloc((size_t)(n_parent > 0 ? n_parent : 1), 1);
    uint64_t* states = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)G);
    cplx* phases = (cplx*)malloc(sizeof(cplx) * (size_t)G);
    uint64_t* dk = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)G);   /* "Dict" keys */
    cplx* dv = (cplx*)malloc(sizeof(cplx) * (size_t)G);               /* "Dict" values */
    cplx* map_a = (cplx*)map_ampl;
    int64_t n_r = 0;
    for (int64_t p = 0; p < n_parent; ++p) { rep_of[p] = -1; map_a[p].re = 0.0; map_a[p].im = 0.0; }
    for (int g = 0; g < G; ++g) { phases[g].re = 1.0; phases[g].im = 0.0; }   /* ones(ScalarType, G) */

    for (int64_t ivec_p = 0; ivec_p < n_parent; ++ivec_p) {              /* :50 */
        if (visited[ivec_p]) continue;                                   /* :51 */
        uint64_t bvec = parent[ivec_p];
        int compatible = 1;
        for (int i = 1; i < G; ++i) {                                    /* :55 */
            cplx y; y.re = ampl[2 * i]; y.im = ampl[2 * i + 1];
            uint64_t bp = or_symmetry_apply(n_sites, bitwidths, bitoffsets, maps + (size_t)i * n_sites,
                                            flips ? flips[i] : 0ull, bvec);
            if (bp < bvec) { compatible = 0; break; }                     /* :58-60 */
            if (bp == bvec) {                                            /* :61-64 isapprox(ampl*sgn, 1; atol=tol) */
                double dr = y.re - 1.0, di = y.im;
                if (!(sqrt(dr * dr + di * di) <= tol)) { compatible = 0; break; }
            }
            states[i] = bp;
            phases[i] = c_conj(y);                                       /* :67 conj(ampl * sgn) */
        }
        if (!compatible) continue;
        states[0] = bvec;
        reps_out[n_r++] = bvec;                                          /* :72 */
        int nd = 0;                                                      /* :74-78 Dict, last write wins */
        for (int i = 0; i < G; ++i) {
            int f = -1;
            for (int k = 0; k < nd; ++k) if (dk[k] == states[i]) { f = k; break; }
            if (f < 0) { dk[nd] = states[i]; dv[nd] = phases[i]; ++nd; }
            else dv[f] = phases[i];
        }
        double inv_norm = 1.0 / sqrt((double)nd);                        /* :39, :79 */
        for (int k = 0; k < nd; ++k) {                                   /* :80-85 */
            int64_t ip = or_lookup(parent, n_parent, dk[k]);
            visited[ip] = 1;
            rep_of[ip] = ivec_p;
            map_a[ip].re = dv[k].re * inv_norm;
            map_a[ip].im = dv[k].im * inv_norm;
        }
    }
    for (int64_t p = 0; p < n_parent; ++p) map_index[p] = -1;            /* :88-89 */
    for (int64_t r = 0; r < n_r; ++r) map_index[or_lookup(parent, n_parent, reps_out[r])] = r;   /* :91-94 */
    for (int64_t pp = 0; pp < n_parent; ++pp) {                          /* :96-101 */
        int64_t p = rep_of[pp];
        if (p < 0 || p == pp) continue;
        map_index[pp] = map_index[p];
    }
    free(rep_of); free(visited); free(states); free(phases); free(dk); free(dv);
    return n_r;
}

/* One row of get_row_iterator(::ReducedOperatorRepresentation, irow_r) summed into out[irow],
 * reduced_operator_representation.jl:57-85, operator_iterator.jl:48-54, and the accumulation of
 * apply_serial!/apply_parallel! (abstract_operator_representation.jl:308-313, :370-375).
 * When map_index == NULL this is the unreduced OperatorRepresentation row
 * (operator_representation.jl:66-79): the column index is the parent lookup itself. */
static cplx row_sum(int64_t irow, const uint64_t* basis, const uint64_t* parent, int64_t n_parent,
                    const int64_t* map_index, const cplx* map_a,
                    int T, const uint64_t* masks, const uint64_t* rows, const uint64_t* cols,
                    const cplx* amps, const cplx* state, int64_t ncols, cplx acc) {
    uint64_t brow = basis[irow];
    cplx inv_ampl_row; inv_ampl_row.re = 1.0; inv_ampl_row.im = 0.0;
    if (map_index) {
        int64_t irow_p = or_lookup(parent, n_parent, brow);              /* :65 */
        inv_ampl_row = c_inv(map_a[irow_p]);                             /* :66, :69 */
    }
    for (int t = 0; t < T; ++t) {
        if ((brow & masks[t]) != rows[t]) continue;                      /* match */
        uint64_t bcol = (brow & ~masks[t]) | cols[t];                     /* element */
        int64_t icol = or_lookup(parent, n_parent, bcol);                /* :75 get(basis_lookup, bcol, -1) */
        if (icol < 0) continue;                                          /* :76 -> (-1 => ampl), dropped */
        cplx el = amps[t];
        if (map_index) {
            int64_t icol_p = icol;
            icol = map_index[icol_p];                                    /* :77 */
            if (icol < 0) continue;                                      /* :78 */
            el = c_mul(c_mul(amps[t], map_a[icol_p]), inv_ampl_row);     /* :79-80 ampl*ampl_col*inv_ampl_row */
        }
        if (icol >= ncols) continue;                                     /* 1 <= icol <= ncols */
        acc = c_add(acc, c_mul(el, state[icol]));                        /* out[irow] += amplitude * state[icol] */
    }
    return acc;
}

/* apply!(out, opr, state) restricted to rows [r0, r1): out += opr * state (accumulate=1) or mul!:
 * fill!(out,0) then apply! (abstract_operator_representation.jl:110-118).  Rows are split statically
 * over threads like Threads.@threads in apply_parallel! (:358-378).  When nnz_out is not NULL it
 * receives the number of off-diagonal elements with a valid column in those rows. */
void or_apply_rows_range(const uint64_t* basis, int64_t nrows, const uint64_t* parent, int64_t n_parent,
                         const int64_t* map_index, const double* map_ampl,
                         int T, const uint64_t* masks, const uint64_t* rows, const uint64_t* cols,
                         const double* amps, const double* state, double* out, int accumulate, int nthreads,
                         int64_t r0, int64_t r1, int64_t* nnz_out) {
    const cplx* a = (const cplx*)amps; const cplx* x = (const cplx*)state; cplx* y = (cplx*)out;
    const cplx* ma = (const cplx*)map_ampl;
    if (r0 < 0) r0 = 0;
    if (r1 > nrows) r1 = nrows;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t r = r0; r < r1; ++r) {
        cplx acc = accumulate ? y[r] : (cplx){0.0, 0.0};
        y[r] = row_sum(r, basis, parent, n_parent, map_index, ma, T, masks, rows, cols, a, x, nrows, acc);
    }
    if (nnz_out) {
        int64_t nnz = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads) reduction(+:nnz)
#endif
        for (int64_t r = r0; r < r1; ++r) {
            uint64_t brow = basis[r];
            for (int t = 0; t < T; ++t) {
                if (rows[t] == cols[t] || (brow & masks[t]) != rows[t]) continue;
                int64_t icol = or_lookup(parent, n_parent, (brow & ~masks[t]) | cols[t]);
                if (icol >= 0 && map_index) icol = map_index[icol];
                if (icol >= 0) ++nnz;
            }
        }
        *nnz_out = nnz;
    }
    (void)nthreads;
}

void or_apply_rows(const uint64_t* basis, int64_t nrows, const uint64_t* parent, int64_t n_parent,
                   const int64_t* map_index, const double* map_ampl,
                   int T, const uint64_t* masks, const uint64_t* rows, const uint64_t* cols,
                   const double* amps, const double* state, double* out, int accumulate, int nthreads) {
    or_apply_rows_range(basis, nrows, parent, n_parent, map_index, map_ampl, T, masks, rows, cols, amps, state,
                        out, accumulate, nthreads, 0, nrows, NULL);
}

/* apply!(out, state, opr): out += transpose(state) * opr via get_column_iterator
 * (abstract_operator_representation.jl:327-347, :389-409).  The reduced column element is
 * ampl * conj(ampl_row_p) / conj(ampl_col) (reduced_operator_representation.jl:88-116);
 * the unreduced one is operator_representation.jl:90-103. */
void or_apply_cols(const uint64_t* basis, int64_t ncols, const uint64_t* parent, int64_t n_parent,
                   const int64_t* map_index, const double* map_ampl,
                   int T, const uint64_t* masks, const uint64_t* rows, const uint64_t* cols,
                   const double* amps, const double* state, double* out, int accumulate, int nthreads) {
    const cplx* a = (const cplx*)amps; const cplx* x = (const cplx*)state; cplx* y = (cplx*)out;
    const cplx* ma = (const cplx*)map_ampl;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t c = 0; c < ncols; ++c) {
        uint64_t bcol = basis[c];
        cplx inv_ampl_col; inv_ampl_col.re = 1.0; inv_ampl_col.im = 0.0;
        if (map_index) {
            int64_t icol_p = or_lookup(parent, n_parent, bcol);
            inv_ampl_col = c_inv(c_conj(ma[icol_p]));                      /* one(S) / conj(ampl_col) */
        }
        cplx acc = accumulate ? y[c] : (cplx){0.0, 0.0};
        for (int t = 0; t < T; ++t) {
            if ((bcol & masks[t]) != cols[t]) continue;                     /* operator_iterator.jl:57-63 */
            uint64_t brow = (bcol & ~masks[t]) | rows[t];
            int64_t irow = or_lookup(parent, n_parent, brow);
            if (irow < 0) continue;
            cplx el = a[t];
            if (map_index) {
                int64_t irow_p = irow;
                irow = map_index[irow_p];
                if (irow < 0) continue;
                el = c_mul(c_mul(a[t], c_conj(ma[irow_p])), inv_ampl_col);
            }
            if (irow >= ncols) continue;
            acc = c_add(acc, c_mul(x[irow], el));                           /* out[icol] += state[irow] * amplitude */
        }
        y[c] = acc;
    }
    (void)nthreads;
}

/* symmetry_unreduce(rhsr, small_vector): large[i_p] += ampl[i_p] * small[i_r] (symmetry_reduce.jl:208-225) */
void or_unreduce(const int64_t* map_index, const double* map_ampl, int64_t n_parent,
                 const double* small_v, double* large_v) {
    const cplx* ma = (const cplx*)map_ampl; const cplx* s = (const cplx*)small_v; cplx* l = (cplx*)large_v;
    for (int64_t p = 0; p < n_parent; ++p) {
        l[p].re = 0.0; l[p].im = 0.0;
        int64_t r = map_index[p];
        if (r >= 0) l[p] = c_mul(ma[p], s[r]);
    }
}

/* symmetry_reduce(rhsr, large_vector): small[i_r] += conj(ampl[i_p]) * large[i_p] (symmetry_reduce.jl:38-56) */
void or_reduce_vector(const int64_t* map_index, const double* map_ampl, int64_t n_parent,
                      const double* large_v, double* small_v, int64_t n_r) {
    const cplx* ma = (const cplx*)map_ampl; const cplx* l = (const cplx*)large_v; cplx* s = (cplx*)small_v;
    for (int64_t r = 0; r < n_r; ++r) { s[r].re = 0.0; s[r].im = 0.0; }
    for (int64_t p = 0; p < n_parent; ++p) {
        int64_t r = map_index[p];
        if (r >= 0) s[r] = c_add(s[r], c_mul(c_conj(ma[p]), l[p]));
    }
}

/* Sorted list of all n-bit words with popcount k: the 2Sz sector of a spin-1/2 chain
 * (hs_get_basis_list for HilbertSpaceSector(hs, n-2k), hilbert_space_representation.jl:127-206,
 * produces exactly this ascending list).  Used to build large parent bases quickly; the tests
 * cross-check it against the Python restatement of the QN dynamic programme. */
int64_t or_popcount_basis(int n, int k, uint64_t* out, int64_t cap) {
    if (k < 0 || k > n || n > 63) return -1;
    int64_t cnt = 0;
    if (k == 0) { if (cap > 0) out[0] = 0; return 1; }
    uint64_t v = (1ull << k) - 1ull, lim = 1ull << n;
    while (v < lim) {
        if (cnt < cap) out[cnt] = v;
        ++cnt;
        uint64_t t = v | (v - 1ull);                      /* Gosper's hack: next word with the same popcount */
        v = (t + 1ull) | (((~t & (t + 1ull)) - 1ull) >> (__builtin_ctzll(v) + 1));
    }
    return cnt;
}

/* ---- the reference's tables evaluated for one orbit at a time --------------------------------
 * symmetry_reduce_generic.jl:22-106 fills basis_mapping_index / basis_mapping_amplitude for every
 * parent state in one ascending sweep.  For sectors whose parent-sized tables do not fit in host
 * memory (the 6x6 torus: 9.1e9 parent states, ~290 GB of tables), the entries a row needs are
 * evaluated here for the orbit of one state, with the same semantics:
 *   - the sweep meets an orbit first at its minimum, which becomes the representative (:50-51, :72);
 *   - the orbit is kept only if every g with g.rep == rep has amplitude ~1 (:55-64, atol = tol);
 *   - the "Dict" of members keeps the LAST element i with g_i.rep == q (:74-78), so q's amplitude is
 *     conj(y_i) of that i over sqrt(#distinct members) (:39, :79-85).
 * Restricted to parents that are one popcount sector of 1-bit sites (every spin-1/2 2Sz sector):
 * get(basis_lookup, bcol, -1) on such a parent is -1 exactly when popcount(bcol) differs. */
static uint64_t torus_apply(uint64_t v, int L1, int L2, int a, int b, const uint64_t* keep) {
    const int n = L1 * L2;
    const uint64_t full = (n >= 64) ? ~0ull : ((1ull << n) - 1ull);
    /* rows up by b: bit x + L1*y -> x + L1*((y+b) mod L2), a rotation of the n-bit word by L1*b */
    const int s = (L1 * b) % n;
    if (s) v = ((v << s) | (v >> (n - s))) & full;
    /* every row rotated by a within its L1 bits: bits that do not wrap move up by a, the others
     * move down by L1 - a (keep[a] marks the bits of each row that do not wrap) */
    if (a) v = ((v & keep[a]) << a) | ((v & ~keep[a] & full) >> (L1 - a));
    return v;
}

/* Row masks of the torus rotations: keep[a] marks, in every row of L1 bits, the bits that a rotation
 * by a within the row moves up without wrapping. */
static void torus_keep(int L1, int L2, uint64_t* keep) {
    for (int a = 0; a < L1; ++a) {
        uint64_t row = 0;
        for (int x = 0; x + a < L1; ++x) row |= 1ull << x;
        keep[a] = 0;
        for (int y = 0; y < L2; ++y) keep[a] |= row << (L1 * y);
    }
}

typedef struct { uint64_t rep; int compatible; int n_distinct; cplx ampl; } orbit_info;

/* g.v for element g: the site permutation (symmetry_apply.jl:82-92), or, when the group is the
 * translation group of an L1 x L2 torus of 1-bit sites listed as g = a + L1 b (tor != NULL: L1, L2 and
 * the row masks), the same permutation by word rotations. */
typedef struct { int L1, L2; uint64_t keep[33]; } torus_spec;

static inline uint64_t group_apply(int g, uint64_t v, int n_sites, const int32_t* bw, const int32_t* off,
                                   const int32_t* maps, const uint64_t* flips, const torus_spec* tor) {
    if (tor) return torus_apply(v, tor->L1, tor->L2, g % tor->L1, g / tor->L1, tor->keep);
    return or_symmetry_apply(n_sites, bw, off, maps + (size_t)g * n_sites, flips ? flips[g] : 0ull, v);
}

static orbit_info orbit_of_t(uint64_t q, int n_sites, const int32_t* bw, const int32_t* off, int G,
                             const int32_t* maps, const uint64_t* flips, const cplx* y, double tol,
                             const torus_spec* tor) {
    orbit_info o;
    uint64_t rep = q;
    for (int g = 1; g < G; ++g) {
        uint64_t t = group_apply(g, q, n_sites, bw, off, maps, flips, tor);
        if (t < rep) rep = t;
    }
    o.rep = rep;
    o.compatible = 1;
    o.n_distinct = 0;
    o.ampl.re = 0.0; o.ampl.im = 0.0;
    /* states[i] = g_i.rep, phase conj(y_i); Dict with last write winning */
    uint64_t dk[4096];
    int nd = 0, last_q = -1;
    if (G > 4096) { o.compatible = -1; return o; }
    for (int i = 0; i < G; ++i) {
        uint64_t s = (i == 0) ? rep : group_apply(i, rep, n_sites, bw, off, maps, flips, tor);
        if (i > 0 && s == rep) {
            double dr = y[i].re - 1.0, di = y[i].im;
            if (!(sqrt(dr * dr + di * di) <= tol)) o.compatible = 0;
        }
        int f = 0;
        for (int k = 0; k < nd; ++k) if (dk[k] == s) { f = 1; break; }
        if (!f) dk[nd++] = s;
        if (s == q) last_q = i;
    }
    o.n_distinct = nd;
    if (last_q >= 0) {
        /* phases start as ones(ScalarType, G) (:46); only elements i >= 1 get conj(y_i) (:67) */
        cplx ph = (last_q == 0) ? (cplx){1.0, 0.0} : c_conj(y[last_q]);
        double inv_norm = 1.0 / sqrt((double)nd);
        o.ampl.re = ph.re * inv_norm;
        o.ampl.im = ph.im * inv_norm;
    }
    return o;
}

static orbit_info orbit_of(uint64_t q, int n_sites, const int32_t* bw, const int32_t* off, int G,
                           const int32_t* maps, const uint64_t* flips, const cplx* y, double tol) {
    return orbit_of_t(q, n_sites, bw, off, G, maps, flips, y, tol, NULL);
}

/* Orbit data of m states: representative, compatibility (1/0), #distinct members and the mapping
 * amplitude the reference's tables hold for the state. */
void or_orbit_info(int n_sites, const int32_t* bw, const int32_t* off, int G, const int32_t* maps,
                   const uint64_t* flips, const double* ampl, double tol, const uint64_t* states, int64_t m,
                   uint64_t* rep_out, int32_t* compatible_out, int32_t* n_distinct_out, double* ampl_out) {
    const cplx* y = (const cplx*)ampl;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t j = 0; j < m; ++j) {
        orbit_info o = orbit_of(states[j], n_sites, bw, off, G, maps, flips, y, tol);
        rep_out[j] = o.rep;
        compatible_out[j] = o.compatible;
        n_distinct_out[j] = o.n_distinct;
        ampl_out[2 * j] = o.ampl.re;
        ampl_out[2 * j + 1] = o.ampl.im;
    }
}

/* Selected rows of mul!(out, represent(rhsr, op), state): for each sampled row index r,
 * out[j] = sum over the row iterator's elements (reduced_operator_representation.jl:57-85):
 *   brow = basis_list[r]; ampl_row = mapping amplitude of brow (:65-66); for every matching term t
 *   (operator_iterator.jl:48-54) with bcol = (brow & ~mask) | col in the parent sector (:75-76), the
 *   column is the index of bcol's representative (:77; dropped when its orbit is not kept, :78), with
 *   amplitude amp_t * ampl_col / ampl_row (:79-80); summed in term order into a zero (mul! fills out
 *   with zero first, abstract_operator_representation.jl:115-116).
 * status[j]: 0 ok; 1 basis_list[r] is not its orbit's representative; 2 its orbit is not kept;
 * 3 a column's representative is missing from basis_list.  nnz_out[j]: off-diagonal elements with a
 * valid column (row == col terms are diagonal). */
static void sampled_rows(const uint64_t* basis, int64_t n_r, int parent_popcount, int n_sites, const int32_t* bw,
                         const int32_t* off, int G, const int32_t* maps, const uint64_t* flips, const double* ampl,
                         double tol, int T, const uint64_t* masks, const uint64_t* rows, const uint64_t* cols,
                         const double* amps, const double* state, const int64_t* sample, int64_t m, double* out,
                         int32_t* status, int64_t* nnz_out, const torus_spec* tor);

void or_sampled_rows(const uint64_t* basis, int64_t n_r, int parent_popcount, int n_sites, const int32_t* bw,
                     const int32_t* off, int G, const int32_t* maps, const uint64_t* flips, const double* ampl,
                     double tol, int T, const uint64_t* masks, const uint64_t* rows, const uint64_t* cols,
                     const double* amps, const double* state, const int64_t* sample, int64_t m, double* out,
                     int32_t* status, int64_t* nnz_out) {
    sampled_rows(basis, n_r, parent_popcount, n_sites, bw, off, G, maps, flips, ampl, tol, T, masks, rows, cols,
                 amps, state, sample, m, out, status, nnz_out, NULL);
}

/* The same rows with the translations of an L1 x L2 torus (elements g = a + L1 b, as listed by the
 * caller's maps) applied by word rotations instead of the site loop: identical results, used where
 * the host time of the restatement is measured. */
void or_sampled_rows_torus(int L1, int L2, const uint64_t* basis, int64_t n_r, int parent_popcount, int n_sites,
                           const int32_t* bw, const int32_t* off, int G, const int32_t* maps, const double* ampl,
                           double tol, int T, const uint64_t* masks, const uint64_t* rows, const uint64_t* cols,
                           const double* amps, const double* state, const int64_t* sample, int64_t m, double* out,
                           int32_t* status, int64_t* nnz_out) {
    torus_spec tor;
    tor.L1 = L1;
    tor.L2 = L2;
    torus_keep(L1, L2, tor.keep);
    sampled_rows(basis, n_r, parent_popcount, n_sites, bw, off, G, maps, NULL, ampl, tol, T, masks, rows, cols,
                 amps, state, sample, m, out, status, nnz_out, &tor);
}

static void sampled_rows(const uint64_t* basis, int64_t n_r, int parent_popcount, int n_sites, const int32_t* bw,
                         const int32_t* off, int G, const int32_t* maps, const uint64_t* flips, const double* ampl,
                         double tol, int T, const uint64_t* masks, const uint64_t* rows, const uint64_t* cols,
                         const double* amps, const double* state, const int64_t* sample, int64_t m, double* out,
                         int32_t* status, int64_t* nnz_out, const torus_spec* tor) {
    const cplx* y = (const cplx*)ampl;
    const cplx* a = (const cplx*)amps;
    const cplx* x = (const cplx*)state;
    cplx* o = (cplx*)out;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t j = 0; j < m; ++j) {
        const int64_t r = sample[j];
        const uint64_t brow = basis[r];
        int st = 0;
        int64_t nnz = 0;
        cplx acc = {0.0, 0.0};
        orbit_info orow = orbit_of_t(brow, n_sites, bw, off, G, maps, flips, y, tol, tor);
        if (orow.rep != brow) st = 1;
        else if (orow.compatible != 1) st = 2;
        const cplx inv_ampl_row = c_inv(orow.ampl);
        for (int t = 0; t < T && st == 0; ++t) {
            if ((brow & masks[t]) != rows[t]) continue;
            const uint64_t bcol = (brow & ~masks[t]) | cols[t];
            if (parent_popcount >= 0 && __builtin_popcountll(bcol) != parent_popcount) continue;
            orbit_info oc = orbit_of_t(bcol, n_sites, bw, off, G, maps, flips, y, tol, tor);
            if (oc.compatible != 1) continue;
            const int64_t icol = or_lookup(basis, n_r, oc.rep);
            if (icol < 0) { st = 3; break; }
            if (rows[t] != cols[t]) ++nnz;
            const cplx el = c_mul(c_mul(a[t], oc.ampl), inv_ampl_row);
            acc = c_add(acc, c_mul(el, x[icol]));
        }
        o[j] = acc;
        status[j] = st;
        nnz_out[j] = nnz;
    }
}

/* ---- representatives of a translation sector, enumerated without a parent basis ----------------
 * The set symmetry_reduce_generic.jl:22-106 keeps: the sweep over the ascending parent basis meets
 * every orbit first at its minimum (:50-51), and keeps it when every element fixing it has amplitude
 * 1 (:55-64).  So the representatives are exactly the states of the sector that are the minimum of
 * their orbit and whose stabiliser has trivial character.  This enumerates them for the translations
 * T(a,b) of an L1 x L2 torus of 1-bit sites (site x + L1*y at bit x + L1*y; T(a,b) moves site (x,y)
 * to (x+a, y+b)) in the popcount-n_up sector, with chi(T(a,b)) = exp(2 pi i num[a + L1 b] / den), in
 * ascending order, without materialising the parent sector (9.1e9 states for the 6x6 torus).
 * The sector is split into nchunks colex-ranked chunks handled by OpenMP threads; each chunk's
 * representatives are counted first, then written at their offsets.  Returns the number of
 * representatives (out may be NULL to count only). */
static double binom_d(int n, int k) {
    if (k < 0 || k > n) return 0.0;
    double r = 1.0;
    for (int i = 1; i <= k; ++i) r = r * (double)(n - k + i) / (double)i;
    return r;
}

/* colex unranking of the r-th n-bit word with popcount k (ascending order of the words) */
static uint64_t colex_unrank(uint64_t r, int n, int k) {
    uint64_t v = 0;
    for (int i = n - 1; i >= 0 && k > 0; --i) {
        const uint64_t c = (uint64_t)binom_d(i, k);   /* words with the top set bit below i */
        if (r >= c) { v |= 1ull << i; r -= c; --k; }
    }
    return v;
}

static int torus_is_rep(uint64_t v, int L1, int L2, const uint64_t* keep, const int32_t* num, int den) {
    for (int b = 0; b < L2; ++b)
        for (int a = 0; a < L1; ++a) {
            if (a == 0 && b == 0) continue;
            const uint64_t t = torus_apply(v, L1, L2, a, b, keep);
            if (t < v) return 0;
            if (t == v && (num[a + L1 * b] % den) != 0) return 0;
        }
    return 1;
}

int64_t or_torus_reps(int L1, int L2, int n_up, const int32_t* num, int den, int nchunks, uint64_t* out) {
    const int n = L1 * L2;
    if (n < 1 || n > 63 || n_up < 0 || n_up > n || L1 > 32) return -1;
    uint64_t keep[33];
    torus_keep(L1, L2, keep);
    const uint64_t total = (uint64_t)binom_d(n, n_up);
    if (nchunks < 1) nchunks = 1;
    int64_t* cnt = (int64_t*)calloc((size_t)nchunks + 1, sizeof(int64_t));
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) {   /* exclusive scan of the chunk counts */
            int64_t s = 0;
            for (int c = 0; c < nchunks; ++c) { int64_t t = cnt[c]; cnt[c] = s; s += t; }
            cnt[nchunks] = s;
            if (!out) break;
        }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
        for (int c = 0; c < nchunks; ++c) {
            const uint64_t r0 = total / (uint64_t)nchunks * (uint64_t)c + ((uint64_t)c < total % (uint64_t)nchunks ? (uint64_t)c : total % (uint64_t)nchunks);
            const uint64_t r1 = r0 + total / (uint64_t)nchunks + ((uint64_t)c < total % (uint64_t)nchunks ? 1u : 0u);
            if (r1 <= r0) continue;
            uint64_t v = colex_unrank(r0, n, n_up);
            int64_t k = 0, pos = (pass == 1) ? cnt[c] : 0;
            for (uint64_t r = r0; r < r1; ++r) {
                if (torus_is_rep(v, L1, L2, keep, num, den)) {
                    if (pass == 1) out[pos++] = v;
                    else ++k;
                }
                if (n_up == 0) break;
                const uint64_t t = v | (v - 1ull);   /* next word with the same popcount (Gosper) */
                v = (t + 1ull) | (((~t & (t + 1ull)) - 1ull) >> (__builtin_ctzll(v) + 1));
            }
            if (pass == 0) cnt[c] = k;
        }
    }
    const int64_t res = cnt[nchunks];
    free(cnt);
    return res;
}
