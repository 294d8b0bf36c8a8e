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
