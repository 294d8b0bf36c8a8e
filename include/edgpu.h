/*
 * edgpu.h -- C ABI of libedgpu.so, the GB300 (sm_103a) implementation of
 * ExactDiagonalization.jl's sector basis, translation-symmetry reduction and
 * matrix-free (reduced) Hamiltonian application.
 *
 * Every entry point replaces one reference interface, cited as file:line of
 * kyungminlee/ExactDiagonalization.jl v0.14.3.  Plain pointers and sizes only.
 *
 * Conventions
 *   - Every function returns an int status (EDGPU_OK == 0).  On failure a
 *     message is available from edgpu_last_error() (per calling thread).
 *     The status maps to the reference's exception types:
 *       EDGPU_ERR_ARG    ArgumentError     (bad masks, non-unit amplitudes, BR too small)
 *       EDGPU_ERR_DIM    DimensionMismatch (vector lengths)
 *       EDGPU_ERR_BOUNDS BoundsError       (row/column index out of range)
 *       EDGPU_ERR_KEY    KeyError          (state not in the basis)
 *   - Indices are 0-based; "absent" is -1 (the reference is 1-based, -1 absent).
 *   - Basis states are uint64 words; site i occupies bits
 *     [bitoffset(i), bitoffset(i)+bitwidth(i)) with bitwidth = ceil(log2(dim_i))
 *     (hilbert_space.jl:25-41, site.jl:93); local state index s is stored as code s-1.
 *   - Complex vectors are interleaved (re, im).  Host-buffer entry points take
 *     complex128 (ComplexF64).  Device-buffer entry points take complex128 for
 *     EDGPU_FP64 and complex64 for EDGPU_MIXED.
 *   - Device-buffer entry points take a cudaStream_t as void* (NULL = the CUDA default stream) and
 *     are asynchronous on it; host-buffer entry points return after the result is in host memory.
 *   - Threading: every handle (space, operator, batch) owns a lock and its own CUDA stream.  Calls
 *     on one handle are serialised by its lock; calls on distinct handles run concurrently from
 *     different host threads.  Calls without a stream argument (builds, host-buffer products, the
 *     autotuners, Lanczos) run on the handle's own stream; a call blocks only its calling thread.
 *     An operator's calls also take its space's lock while they enqueue work, so a space's
 *     parent-state map cannot be freed while a product is being issued on it.
 */
#ifndef EDGPU_H
#define EDGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EDGPU_OK          0
#define EDGPU_ERR_ARG     1
#define EDGPU_ERR_DIM     2
#define EDGPU_ERR_BOUNDS  3
#define EDGPU_ERR_KEY     4
#define EDGPU_ERR_OOM     5
#define EDGPU_ERR_CUDA    6
#define EDGPU_ERR_TIMEOUT 7
#define EDGPU_ERR_STATE   8

/* Arithmetic of the matrix-free product. */
#define EDGPU_FP64   0   /* complex128 vectors, FP64 accumulation                               */
#define EDGPU_MIXED  1   /* complex64 vectors, FP32 accumulation; phases and orbit-normalisation
                            factors computed in FP64 and rounded once                            */

/* Flags of edgpu_space_create. */
#define EDGPU_SPACE_LAZY 1  /* do not materialise the sector basis (only its definition is kept);
                               edgpu_reduce then enumerates representatives directly          */

typedef struct edgpu_space_s* edgpu_space;  /* HilbertSpaceRepresentation or ReducedHilbertSpaceRepresentation */
typedef struct edgpu_op_s* edgpu_op;        /* OperatorRepresentation or ReducedOperatorRepresentation         */
typedef struct edgpu_batch_s* edgpu_batch;  /* several operator representations applied in one launch          */

/* ---- library --------------------------------------------------------------------------- */
const char* edgpu_last_error(void);
const char* edgpu_version(void);
/* Number of visible CUDA devices (0 when no driver or device is present). */
int edgpu_device_count(int32_t* out);

/* ---- Hilbert space sector and its basis ------------------------------------------------ */
/* represent(HilbertSpaceSector(hs, allowed)) with the sorted basis enumerated on the GPU.
 * Replaces hs_get_basis_list(::HilbertSpaceSector) + represent_array
 * (hilbert_space_representation.jl:127-206, :215-230) and the sector constructor
 * (hilbert_space_sector.jl:20-63).
 *   site_dims[n_sites]          number of local states of each site (Site.states)
 *   state_qn[sum(site_dims)*qn_len]  quantum-number tuple of each local state, site-major
 *   allowed_qn[n_allowed*qn_len]     allowed total quantum numbers (n_allowed < 0: all sectors,
 *                                    i.e. represent(hs), hilbert_space_representation.jl:109-119)
 * EDGPU_ERR_ARG when the total bit width is >= 64 ("BR too small", :63-69). */
int edgpu_space_create(int32_t n_sites, const int32_t* site_dims, int32_t qn_len, const int64_t* state_qn,
                       int32_t n_allowed, const int64_t* allowed_qn, int32_t flags, edgpu_space* out);
/* represent(hs, basis_list): basis given by the caller, sorted here if needed, duplicates rejected
 * (hilbert_space_representation.jl:239-256, frozensortedarray.jl:14-22). */
int edgpu_space_from_basis(int32_t n_sites, const int32_t* site_dims, const uint64_t* basis, int64_t n,
                           edgpu_space* out);
/* dimension(hsr) / dimension(rhsr) (hilbert_space_representation.jl:82, reduced_hilbert_space_representation.jl:38) */
int edgpu_space_dim(edgpu_space s, int64_t* out);
/* bitwidth(hs) (hilbert_space.jl:96) */
int edgpu_space_nbits(edgpu_space s, int32_t* out);
/* basis_list (sorted uint64) copied to host memory of n entries. */
int edgpu_space_get_basis(edgpu_space s, uint64_t* out, int64_t n);
/* get(basis_lookup, key, -1) for n keys on the device (frozensortedarray.jl:29-48). */
int edgpu_space_lookup(edgpu_space s, const uint64_t* keys, int64_t n, int64_t* idx_out);
void edgpu_space_destroy(edgpu_space s);
/* Shape of the search directory that replaces the binary search of FrozenSortedArrayIndex
 * (frozensortedarray.jl:29-32) in the product: number of buckets, bucket = state >> shift, keys
 * summarised inline per bucket, halvings for larger buckets, and the fraction of rows whose bucket is
 * answered by its summary alone (all outputs nullable). */
int edgpu_space_search_stats(edgpu_space s, int64_t* buckets, int32_t* shift, int32_t* inline_keys_per_bucket,
                             int32_t* window_steps, double* inline_fraction);

/* Parent-state map of a reduced representation whose parent is one fixed-popcount sector.  The
 * reference keeps parent-sized tables basis_mapping_index / basis_mapping_amplitude (24 bytes per parent
 * state, symmetry_reduce_translation.jl:22-24,82-87 and symmetry_reduce_generic.jl:33-35) and its row
 * iterator reads them for every target (reduced_operator_representation.jl:57-85).  This is the compact
 * form: 4 (or 8) bytes per parent state, indexed by the colex rank of the state, holding the
 * representative's index, its orbit-size index and the group element reaching it; the product then
 * replaces orbit canonicalisation and search by one rank and one load per target (results identical).
 * Built when it applies and needs at most max_bytes (*built = 1), else *built = 0 and nothing changes.
 * The map belongs to the space and is used by every operator on it until edgpu_space_free_map. */
int edgpu_space_build_map(edgpu_space s, int64_t max_bytes, int32_t* built);
int edgpu_space_free_map(edgpu_space s);
/* entries = parent states covered (0 without a map), entry_bytes = 4 or 8. */
int edgpu_space_map_info(edgpu_space s, int64_t* entries, int32_t* entry_bytes);

/* ---- symmetry reduction ------------------------------------------------------------------ */
/* symmetry_reduce(hsr, symops_and_amplitudes) (symmetry_reduce_generic.jl:7-106), and the
 * IrrepComponent forms (symmetry_reduce.jl:12-20, symmetry_reduce_translation.jl) once their
 * elements are listed.  Element g acts as: the field of site i moves to site site_maps[g*n+i]
 * (SitePermutation, symmetry_apply.jl:82-92), then the word is XORed with flip_masks[g]
 * (GlobalBitFlip, bitflipsymmetry.jl:23-35; NULL = no flips).  Its amplitude (the y of the
 * reference's (op, y) pairs) is exp(2*pi*i*char_num[g]/char_den).  Element 0 must be the
 * identity with char_num 0; the elements must form a group and the amplitudes a 1-D
 * representation of it (EDGPU_ERR_ARG otherwise).
 * Representatives (orbit minima whose stabiliser has character 1) are enumerated on the GPU
 * into a sorted table; phases and orbit norms are recomputed on the fly by the product, so no
 * parent-sized table is built. */
int edgpu_reduce(edgpu_space parent, int32_t n_elems, const int32_t* site_maps, const uint64_t* flip_masks,
                 const int32_t* char_num, int32_t char_den, edgpu_space* out);
/* ReducedHilbertSpaceRepresentation.basis_mapping_index / basis_mapping_amplitude
 * (reduced_hilbert_space_representation.jl:13-22) materialised for a parent of n_parent states:
 * index_out[n_parent] (reduced index or -1), ampl_out[2*n_parent].  Requires a materialised parent. */
int edgpu_reduce_mapping(edgpu_space reduced, int64_t* index_out, double* ampl_out, int64_t n_parent);
/* Dimension of the parent of a reduced representation (its sector's size; for a lazy parent the number
 * of words of its popcount). */
int edgpu_space_parent_dim(edgpu_space reduced, int64_t* out);
/* symmetry_unreduce(rhsr, small) (symmetry_reduce.jl:208-225): large[i] = ampl(p_i) small[rep(p_i)] for
 * every parent state p_i (0 where its orbit has no representative), and symmetry_reduce(rhsr, large)
 * (symmetry_reduce.jl:38-56): small[c] = sum over the orbit of rep_c of conj(ampl(p)) large[i(p)], on
 * DEVICE vectors (complex128 for EDGPU_FP64, complex64 for EDGPU_MIXED).  The reference reads its
 * parent-sized tables; here each entry's representative, stabiliser and group element are recomputed,
 * so no table is built (the 6x6 torus's parent vector of 9.1e9 entries fits where the tables do not).
 * Parent index i: position in the materialised parent basis, or the colex rank for a lazy parent.
 * The reduction sums each orbit in a fixed element order (reproducible, no atomics).  The calls return
 * after the work is done; stream NULL uses the space's own stream. */
int edgpu_symmetry_unreduce_device(edgpu_space reduced, int32_t precision, const void* small, int64_t n, void* large,
                                   int64_t n_parent, void* stream);
int edgpu_symmetry_reduce_device(edgpu_space reduced, int32_t precision, const void* large, int64_t n_parent, void* small,
                                 int64_t n, void* stream);
/* Orbit size |O| of every representative (1/sqrt(|O|) is the reference's amplitude of a representative). */
int edgpu_space_orbit_sizes(edgpu_space reduced, int32_t* out, int64_t n);

/* ---- operator representation and the product ------------------------------------------- */
/* represent(hsr, op) / represent(rhsr, op) (operator_representation.jl:34-36,
 * reduced_operator_representation.jl:40-42) for a SumOperator given as its terms
 * (sum_operator.jl:13-23): term t is amps[t] * prod_i (|row_i><col_i| on the bits of masks[t]).
 * coupling_ids (nullable) tags each term with a coupling index in [0, n_couplings) for
 * edgpu_coupling_grad; amps are then the per-unit-coupling amplitudes and the operator is
 * sum_t couplings[coupling_ids[t]] * amps[t] * P_t.  EDGPU_ERR_ARG when (~mask) & row != 0 or
 * (~mask) & col != 0 (pure_operator.jl:32-36). */
int edgpu_op_create(edgpu_space s, int32_t n_terms, const uint64_t* masks, const uint64_t* rows,
                    const uint64_t* cols, const double* amps, const int32_t* coupling_ids,
                    int32_t n_couplings, const double* couplings, edgpu_op* out);
/* Change the coupling values of an operator created with coupling_ids.  Tables already built are
 * rewritten in place (same device buffers, nothing allocated) after the device has finished the work
 * that may read the old values; the target table does not depend on coupling values and is kept. */
int edgpu_op_set_couplings(edgpu_op op, const double* couplings, int32_t n_couplings);
int edgpu_op_dim(edgpu_op op, int64_t* out);
void edgpu_op_destroy(edgpu_op op);
/* Schedule of the product kernel: -1, -2 or -4 for 1, 2 or 4 lanes per row (0 = default, one lane
 * per row), or the rows per warp tile of the queued schedule (a divisor of 32). */
int edgpu_op_set_tiling(edgpu_op op, int32_t precision, int32_t rows_per_tile);
/* In-library autotuner: times the product for each candidate schedule (1, 2 or 4 lanes per row, each
 * with and without the pair-flip schedule where it applies; queued with 32 or 16 rows per warp tile)
 * on this operator and keeps the fastest per launch in back-to-back bursts of launches
 * (rows_per_tile_out: the schedule as in edgpu_op_set_tiling; best_ms_out nullable). */
int edgpu_op_autotune(edgpu_op op, int32_t precision, int32_t* rows_per_tile_out, double* best_ms_out);
/* Pair-flip schedule of the row-per-lane product (enable = 1, the default): when every off-diagonal
 * term flips two 1-bit sites (spin-1/2 exchange and pair terms), a row finds its matching terms from
 * bond classes (a few word operations per class) instead of testing every term.  Same elements as the
 * term scan of get_row_iterator (operator_iterator.jl:48-54, reduced_operator_representation.jl:57-85);
 * the targets are summed by bond class, then start bit, rather than in term order.  enable = 0 keeps
 * the term scan; 2, 4 or 8 sets the targets each lane looks up per step (4 applies with a
 * parent-state map or a target table, 8 with a target table; 1 = 2).  edgpu_op_autotune may change
 * the choice. */
int edgpu_op_set_pair_schedule(edgpu_op op, int32_t enable);
/* Flag of edgpu_op_set_pair_schedule (with 4 or 8 targets per step) and of the pair_flips output of
 * edgpu_op_get_schedule: the target-table product walks warp-uniform steps -- the 32 lanes of a warp
 * step through the union of their rows' matching pairs together, so that the gathers of one step
 * are the targets of one bond pair across 32 consecutive representatives and share DRAM sectors more
 * often.  The visiting order of every row, hence the result, is unchanged. */
#define EDGPU_PAIR_UNIFORM 16
/* Bond classes of the pair-flip schedule for this operator (0 when the terms do not allow it) and
 * their rotation components in total. */
int edgpu_op_pair_classes(edgpu_op op, int32_t* n_classes, int32_t* n_components);
/* Host-only inspection of the pair-flip schedule's bond classes for a term table over n_bits sites
 * of one bit each (no device work; no reference counterpart).  *n_classes = 0 when some off-diagonal
 * term is not a two-site flip.  When cap_classes >= *n_classes, the nullable outputs receive, per
 * class: info (components | has_parallel << 8), comps [BOND_MAXC = 4][3] (shift s, starts of pairs
 * with antiparallel terms, starts with parallel terms), flips [n_bits] (flip mask of the pair starting
 * at each bit, 0 if none) and class_amps [n_bits][4][2] (amplitude by b_i | (b_i == b_j) << 1). */
int edgpu_pair_classes_of_terms(int32_t n_bits, int32_t n_terms, const uint64_t* masks, const uint64_t* rows,
                                const uint64_t* cols, const double* amps, int32_t cap_classes, int32_t* n_classes,
                                int32_t* info, uint64_t* comps, uint64_t* flips, double* class_amps);
/* The schedule the product uses for this precision: rows_per_tile as in edgpu_op_set_tiling (0 =
 * default), pair_flips = 0 when every row tests every term, else the targets each lane looks up per
 * step in the pair-flip schedule (2; 4 with a parent-state map or a target table; 8 with a table),
 * with EDGPU_PAIR_UNIFORM set for warp-uniform steps, and
 * target_table = 1 when the product reads the target table; every pointer nullable. */
int edgpu_op_get_schedule(edgpu_op op, int32_t precision, int32_t* rows_per_tile, int32_t* pair_flips,
                          int32_t* target_table);
/* Target table of the pair-flip schedule: the entry (representative row, orbit-size index and, for
 * characters other than 1, group element; 4 or 8 bytes) of every (row, target) of the product, stored
 * once in the order the product walks them.  It is the (row, target)-indexed form of the
 * reference's parent-sized basis_mapping_index, read per target by the row iterator
 * (reduced_operator_representation.jl:57-85; symmetry_reduce_generic.jl:33-35): products then stream
 * it instead of looking every target up, with bit-identical results.  Built (with the space's
 * parent-state map when it has one, else by canonicalisation and search) when the operator's terms
 * allow the pair-flip schedule and the table needs at most max_bytes; *built = 0 otherwise. */
int edgpu_op_build_targets(edgpu_op op, int64_t max_bytes, int32_t* built);
int edgpu_op_free_targets(edgpu_op op);
/* x prefetch distance of the target-table product for this precision, in steps of targets (0: none;
 * steps < 0 only queries; *current nullable).  Chosen by edgpu_op_autotune; results do not depend on it. */
int edgpu_op_table_prefetch(edgpu_op op, int32_t precision, int32_t steps, int32_t* current);
/* Adjoint target table (no reference counterpart): for every column c of the product's matrix, the
 * rows r whose targets land on c with their slots, sorted.  It serves edgpu_mul_adjoint_device for
 * terms that do not commute with the group (whose adjoint is not the row formula of the adjoint
 * terms): y[c] = sum conj(H[r, c]) x[r] is then a gather in a fixed order (reproducible bit for bit)
 * instead of a scatter with atomics.  Built from the operator's target table (which must exist) when
 * it needs at most max_bytes (8 bytes per nonzero plus 8 per row); *built = 0 otherwise. */
int edgpu_op_build_adjoint_targets(edgpu_op op, int64_t max_bytes, int32_t* built);
int edgpu_op_free_adjoint_targets(edgpu_op op);
/* Entries of the target table and bytes per entry; 0 and 0 without a table. */
int edgpu_op_targets_info(edgpu_op op, int64_t* entries, int32_t* entry_bytes);
/* Column-slab table, built from the target table (which must exist) for products on large sectors
 * (both precisions).  The columns are cut into slabs of slab_bytes of complex64 x (at most 64 slabs);
 * the product then runs one pass per slab, gathering only from that slab (sized to stay in L2) and
 * adding its share to y, instead of gathering at random from all of x.  Results equal the one-pass
 * product up to the order of the additions (the passes are added in order: reproducible run to
 * run).  *built = 0 (nothing kept) when the table would exceed max_bytes, the sector has 2^32 rows or
 * more, a row has more than 255 targets, the terms of one pair slot have different couplings, or the
 * coefficient table does not fit; the autotuner then never picks it.  A new build replaces the old
 * one; new coupling values rewrite its coefficient table in place. */
int edgpu_op_build_slabs(edgpu_op op, int64_t slab_bytes, int64_t max_bytes, int32_t* built);
int edgpu_op_free_slabs(edgpu_op op);
/* Slabs (passes), columns per slab and entries of the slab table; zeros without one. */
int edgpu_op_slabs_info(edgpu_op op, int32_t* passes, int64_t* columns_per_slab, int64_t* entries);
/* Whether products of this precision read the slab table, and how: use = 0 (no), or 1 + v for the
 * variant v = 0 to 5 sets it (1 to 6 need the table: EDGPU_ERR_STATE otherwise), -1 only queries;
 * *current = the setting.  v = 0 to 3: one lane per row (bit 0: cache hints, the gathers of x cached
 * in L2 only and the streamed counts, offsets and y evict-first; bit 1: eight entries per lane and
 * step instead of four), all four bit-identical; v = 4 and 5: two and four lanes per row (for sectors
 * too small to fill the GPU), whose partial sums are added in another fixed order, so their results
 * differ from v = 0 to 3 by rounding (each is deterministic).  Building the table sets 1 for both
 * precisions; the autotuner times the variants against the one-pass schedules. */
int edgpu_op_slab_use(edgpu_op op, int32_t precision, int32_t use, int32_t* current);
/* Layout of the next slab table: mode 0 (default) scaled on sectors of 2^22 representatives or more
 * where that saves passes or the coefficients are complex (and wherever the unscaled ids do not fit in
 * an entry), 1 never, 2 always; -1 only queries.  *scaled = whether the current table is scaled.  A scaled
 * table's entries carry the coefficient without the orbit-size ratio sqrt(|O_c| / |O_r|): each product
 * first scales x by sqrt(|O_c|) into a buffer of the table (slab by slab on the handle's second
 * stream while the earlier passes run), and the last pass scales row r by 1 / sqrt(|O_r|).  Fewer
 * distinct coefficients (a few in registers, or a conflict-free shared-memory copy per bank group)
 * and more column bits per entry (fewer passes) against one more streamed pass over x.  Results agree
 * with the unscaled layout to rounding.  Products of one operator through a scaled table are ordered
 * by the calling stream (the scaled x is one buffer per table). */
int edgpu_op_slab_scaling(edgpu_op op, int32_t mode, int32_t* scaled);
/* Host-buffer products through the slab table (pinned complex128 buffers the device can address) run
 * their passes in row blocks: each block's last pass, which writes the block's rows of the result
 * into the host buffer, runs on a second stream of the handle beside the next block's passes.  Two
 * blocks for mixed precision on sectors of 2^22 rows or more with at least 4 passes, else one; the
 * environment variable EDGPU_SLAB_ROW_BLOCKS (1 to 64) sets the count.  The sums are the same, in the
 * same order, for every count. */
/* Sparse matrix of the representation, assembled on the device in FP64: rows sorted by column,
 * entries of equal column summed, entries with |value| < tol dropped (tol: the reference's
 * Base.rtoldefault(Float64) = sqrt(eps) gives its default).  This is sparse(opr)
 * (abstract_operator_representation.jl:135-198, a SparseMatrixCSC built column by column) as CSR:
 * transpose == 0 gives the rows of H, transpose == 1 the rows of H^T (= the columns of H, the
 * reference's CSC arrays).  Call with row_ptr == NULL for *nnz only; then with host buffers
 * row_ptr[dim + 1], col_idx[nnz] and values[2 * nnz] (interleaved complex128). */
int edgpu_op_sparse(edgpu_op op, int32_t transpose, double tol, int64_t* nnz, int64_t* row_ptr, int64_t* col_idx,
                    double* values);
/* One row (transpose == 0: get_row, abstract_operator_representation.jl:201-213) or column
 * (transpose == 1: get_column, :216-228) as sorted (index, value) entries, summed and chopped as in
 * edgpu_op_sparse.  *count = entries; col_idx/values (capacity cap entries) may be NULL to count only.
 * EDGPU_ERR_BOUNDS for a row outside [0, dim). */
int edgpu_op_get_row(edgpu_op op, int32_t transpose, int64_t row, double tol, int64_t cap, int64_t* count,
                     int64_t* col_idx, double* values);

/* Number of off-diagonal (row, term) matches over all rows, and how many of them land on a row of
 * the representation (the nonzero off-diagonal elements the row iterator yields with a valid column,
 * reduced_operator_representation.jl:57-85) -- the NNZ_off of the product's byte model. */
int edgpu_op_count_nnz(edgpu_op op, int64_t* n_targets, int64_t* nnz_off);

/* LinearAlgebra.mul!(out, opr, state) (accumulate = 0) and apply!(out, opr, state)
 * (accumulate = 1) on HOST complex128 vectors of length n: copies in, applies, copies out.
 * abstract_operator_representation.jl:110-118, :260-267, :296-316, :358-378.
 * EDGPU_ERR_DIM when n != dimension. */
int edgpu_mul(edgpu_op op, int32_t precision, const double* x, double* y, int64_t n, int32_t accumulate);
/* The same on DEVICE vectors (complex128 for EDGPU_FP64, complex64 for EDGPU_MIXED) on a
 * caller stream (cudaStream_t; NULL = the CUDA default stream).  Asynchronous. */
int edgpu_mul_device(edgpu_op op, int32_t precision, const void* x, void* y, int64_t n, int32_t accumulate,
                     void* stream);
/* apply!(out, state, opr): out += transpose(state) * opr (transpose product,
 * abstract_operator_representation.jl:278-285, :327-347; reduced_operator_representation.jl:88-116),
 * host complex128 vectors. */
int edgpu_mul_transpose(edgpu_op op, int32_t precision, const double* x, double* y, int64_t n, int32_t accumulate);
/* Whether every element of the space's symmetry group maps the operator's terms onto themselves (no
 * reference counterpart).  Only then are the reference's reduced row iterator (mul!,
 * reduced_operator_representation.jl:57-85) and column iterator (transpose, :88-116) transposes of
 * each other; edgpu_mul_adjoint_device is the adjoint of the mul! matrix in both cases. */
int edgpu_op_is_invariant(edgpu_op op, int32_t* invariant);

/* y = H^dagger x on device vectors (the adjoint product dL/dx = H^dagger gy).  For a reduced
 * representation the orbit phases are recomputed, not stored. */
int edgpu_mul_adjoint_device(edgpu_op op, int32_t precision, const void* x, void* y, int64_t n,
                             int32_t accumulate, void* stream);
/* dL/dJ_c = Re <gy | H_c x> for every coupling c (H = sum_c J_c H_c), fused with y = H x
 * (y may be NULL).  grad_out: n_couplings doubles in HOST memory.  Device vectors.  With a target table
 * (or a parent-state map) and pair-flip terms whose every (pair, pattern) slot belongs to one coupling,
 * the pair-flip kernel runs it; otherwise the term scan.  Both accumulate per thread in FP64 and reduce
 * per block in a fixed order (reproducible bit for bit) while n_couplings x 2 KiB fits in shared
 * memory (about 90 couplings); beyond that the queued term scan adds per block with shared-memory
 * atomics (reproducible only to rounding). */
int edgpu_coupling_grad_device(edgpu_op op, int32_t precision, const void* x, const void* gy, void* y,
                               int64_t n, double* grad_out, void* stream);

/* Which kernel edgpu_coupling_grad_device runs for this precision (no reference counterpart): 2 the
 * pair-flip gradient kernel through the target table, 1 through the parent-state map, 0 the
 * row-per-lane term scan, -1 the queued term scan (couplings beyond the shared-memory accumulators). */
int edgpu_op_grad_kernel(edgpu_op op, int32_t precision, int32_t* kind);
/* The same fused product and coupling gradient for callers that cannot allocate device memory (their
 * device memory is owned by another allocator, e.g. a Julia or PyTorch memory pool, or they keep
 * allocation out of a time-step loop).  This entry point has no counterpart in the reference.  It
 * allocates nothing: its scratch is a 2 MiB array inside the library (held on every GPU that loads
 * the library), shared by all calls, so calls that overlap on the GPU race and must be serialised by
 * the caller.  It launches the kernel edgpu_coupling_grad_device would (same schedule); the block
 * count is limited to what the scratch holds (2^18 / n_couplings - 1 blocks), which changes only the
 * order in which per-block partial sums are added.  y is required.  The operator's tables for this
 * precision must have been built by one earlier edgpu_coupling_grad_device call (EDGPU_ERR_STATE
 * otherwise); edgpu_op_set_couplings rewrites them in place, so coupling changes keep them built and
 * allocate nothing.  n_couplings is at most 8192 (set at operator creation).  The first call on a
 * device looks up the scratch address (cudaGetSymbolAddress).  grad_out is host memory: the call
 * synchronises its stream before returning, so it must not be issued while that stream is being
 * captured into a CUDA graph. */
int edgpu_coupling_grad_device_noalloc(edgpu_op op, int32_t precision, const void* x, const void* gy, void* y,
                                       int64_t n, double* grad_out, void* stream);

/* ---- batched sectors --------------------------------------------------------------------- */
/* Several operator representations (e.g. every momentum sector of one Hamiltonian) applied in ONE
 * persistent launch: the warp tiles of all sectors are numbered one after the other and the grid
 * strides over them.  No reference counterpart (the reference applies one representation per
 * mul!, abstract_operator_representation.jl:110-118); each sector's result equals edgpu_mul_device
 * on that sector with the same lanes per row, bit for bit.  The operators must share the operator
 * terms, the basis layout and the symmetry group (they differ only in the sector: basis table,
 * characters, diagonal); EDGPU_ERR_ARG otherwise, at the first product.  The operators must outlive
 * the batch; changing an operator's couplings rebuilds the batch's tables at the next product. */
int edgpu_batch_create(int32_t n_ops, const edgpu_op* ops, edgpu_batch* out);
/* Lanes per row of the batched launch for this precision: 0 (default: 1), 1, 2 or 4. */
int edgpu_batch_set_tiling(edgpu_batch b, int32_t precision, int32_t lanes_per_row);
/* In-library autotuner: times the batched launch for 1, 2 and 4 lanes per row, with and without the
 * pair-flip schedule where it applies (and the first operator allows it), and for the pair-flip
 * schedules also per-sector launches on 1, 2 and 3 streams (edgpu_batch_set_launch), with the batch's
 * schedule and with each operator's own, on scratch vectors (allocated and freed here), and keeps the
 * fastest. */
int edgpu_batch_autotune(edgpu_batch b, int32_t precision, int32_t* lanes_per_row_out, double* best_ms_out);
/* The batched launch's lanes per row (0 = default), and pair_flips and target_table as in
 * edgpu_op_get_schedule (the batch reads target tables when every operator has one). */
int edgpu_batch_get_schedule(edgpu_batch b, int32_t precision, int32_t* lanes_per_row, int32_t* pair_flips,
                             int32_t* target_table);
/* How the batch launches (autotuned with the schedule; default 0):
 *   0       all sectors in ONE persistent launch (above);
 *   1       one product launch per sector, in order on the call's stream: each sector's own product
 *           kernel with the batch's schedule (results equal edgpu_mul_device on the sector, bit for bit);
 *   2 or 3  the same per-sector launches spread over that many streams of the batch (sector k on
 *           stream k mod streams), forked from and joined back into the call's stream, so that a
 *           sector's launch fills the SMs that the previous sector's last blocks leave idle;
 *   5 to 7  per-sector launches on 1 to 3 streams, each with its operator's own schedule (the one
 *           edgpu_op_autotune chose for it: slab table, target table or term scan; the best may differ
 *           between sectors).  Results equal edgpu_mul_device on each sector bit for bit.
 * The per-sector modes read the operators' own tables, not a batched image. */
int edgpu_batch_set_launch(edgpu_batch b, int32_t precision, int32_t streams);
int edgpu_batch_get_launch(edgpu_batch b, int32_t precision, int32_t* streams);
/* y_k = H_k x_k for every k, device vectors (arrays of n_ops pointers).  The first call with a set of
 * pointers uploads the sector descriptors (synchronous); if use_graph != 0 that launch is also
 * captured once into a CUDA graph and replayed on the later calls with the same pointers. */
int edgpu_batch_mul_device(edgpu_batch b, int32_t precision, const void* const* xs, void* const* ys,
                           int32_t use_graph, void* stream);
void edgpu_batch_destroy(edgpu_batch b);

/* ---- Lanczos driver ---------------------------------------------------------------------- */
/* Lowest eigenvalue by Lanczos on the device: at most n_steps steps from a seeded complex Gaussian
 * start vector (or v0, host complex128 of length dim, if not NULL), full reorthogonalisation when
 * reorth != 0.  Scalars, dots, norms and the tridiagonal eigensolve are FP64; precision selects the
 * product.  tol > 0 stops once the lowest Ritz value moved by less than tol |E| over the last 5 steps,
 * or (without ground_state) from step 10 on once the Kato-Temple estimate of its error,
 * (beta s_last)^2 / (theta_2 - theta_1) from the tridiagonal matrix, is at most tol max(1, |E|).  With
 * refine != 0 and EDGPU_MIXED: a mixed-precision run until that estimate is at most tol / 4, or 6 steps
 * after its Ritz value settled to max(tol, 1e-9); then one FP64 product gives the Rayleigh quotient
 * E_RQ of its Ritz vector psi and the residual r = H psi - E_RQ psi; E_RQ is returned when the
 * Kato-Temple estimate |r|^2 / (theta_2 - E_RQ) (theta_2 the second Ritz value) is at most
 * tol max(1, |E_RQ|), else FP64 Lanczos continues from psi until the eigenvalue settles to tol or the
 * estimate (with the mixed run's theta_2) certifies it.  Outputs: e0, alphas/betas of the last run (n_steps
 * each, nullable), steps_done (all runs).  ground_state (nullable, host complex128 dim): Ritz vector.
 * The Krylov basis is stored (FP64, or the complex64 product inputs of a mixed run) only when
 * reorthogonalisation or a Ritz vector needs it and it fits under the Krylov limit (EDGPU_ERR_OOM when
 * reorthogonalisation cannot be stored); otherwise two vectors roll and a Ritz vector costs a second
 * pass of the recurrence.  No reference counterpart: the reference leaves eigensolvers to dense
 * eigvals or Arpack (docs/src/examples/spinhalf.md:26). */
int edgpu_lanczos(edgpu_op op, int32_t precision, int32_t n_steps, int32_t reorth, uint64_t seed,
                  const double* v0, int32_t refine, double tol, double* e0, double* alphas, double* betas,
                  int32_t* steps_done, double* ground_state);
/* Largest Krylov basis in bytes that edgpu_lanczos may store (0, the default: half of the free device
 * memory at the call).  The complex64 basis of a mixed-precision run with refine is also held to the
 * device memory left once the run's other buffers are allocated, less 2 GiB. */
int edgpu_set_krylov_limit(int64_t bytes);

/* ---- utilities --------------------------------------------------------------------------- */
/* Seeded complex Gaussian vector (SplitMix64 + Box-Muller, (g1 + i g2)/sqrt(2), normalised in FP64)
 * written to a DEVICE buffer as complex128 (precision EDGPU_FP64) or complex64 (EDGPU_MIXED). */
int edgpu_random_vector_device(int64_t n, uint64_t seed, int32_t precision, void* dst, void* stream);
/* Wait for all work the library has enqueued on the current device (every handle stream and every
 * caller stream): a device-wide synchronisation. */
int edgpu_sync(void);
/* Pinned host memory for the host-buffer entry points (cudaMallocHost / cudaFreeHost). */
int edgpu_host_alloc(int64_t bytes, void** out);
void edgpu_host_free(void* p);

#ifdef __cplusplus
}
#endif

#endif /* EDGPU_H */
