// Internal declarations shared by the translation units of libedgpu.so.
#pragma once

#include <cstdint>
#include <cstddef>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/edgpu.h"

namespace edgpu {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define EDGPU_CUDA(call)                                                                               \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            throw ::edgpu::Error(e_ == cudaErrorMemoryAllocation ? EDGPU_ERR_OOM : EDGPU_ERR_CUDA,     \
                                 std::string(#call) + ": " + cudaGetErrorString(e_));                 \
    } while (0)

enum GroupKind { GK_TRIVIAL = 0, GK_TORUS = 1, GK_GENERIC = 2, GK_RING = 3 };
// Product-kernel flavour for targets looked up in a parent-state map (no canonicalisation code).
constexpr int GK_MAP = 4;
// Pair-flip product flavour that reads every target's map-format entry from the operator's target
// table (row after row, in the schedule's order) instead of looking it up.
constexpr int GK_TABLE = 5;

// Symmetry group acting on basis words: element g maps word q to g.q.
//  TRIVIAL  the identity only (unreduced representation).
//  TORUS    translations T(a,b) of an L1 x L2 torus of w-bit sites numbered x + L1*y;
//           g = a + L1*b; T(a,b).q rotates every row of L1*w bits left by a*w and the rows
//           up by b rows.  num[] is in this order.
//  GENERIC  arbitrary site permutations (+ XOR flip), applied through 4-bit chunk tables.
//  RING     (product kernel only) a TORUS with L2 == 1 in 32-bit words: funnel-shift rotations.
struct Group {
    int kind = GK_TRIVIAL;
    int G = 1;
    int den = 1;
    std::vector<int32_t> num{0};     // character numerators: chi(g) = exp(2 pi i num[g] / den)
    int L1 = 1, L2 = 1, w = 1;       // TORUS
    std::vector<int32_t> maps;       // GENERIC: [G][n_sites] site maps in user order
    std::vector<uint64_t> flips;     // GENERIC: [G]
};

struct Layout {
    int n_sites = 0, nbits = 0, qlen = 0;
    std::vector<int32_t> dims, bw, off;
    std::vector<int64_t> state_qn;   // [sum(dims)][qlen], site-major
    std::vector<int64_t> allowed;    // [n_allowed][qlen]
    bool all_sectors = false;
    int popcount = -1;               // >= 0: spin-1/2-like sector = all words of nbits with this popcount
};

struct Space {
    Layout lay;
    bool reduced = false;
    bool lazy = false;
    Space* parent = nullptr;         // reduced: the parent representation (not owned)
    Group group;
    int64_t dim = 0;
    bool w32 = false;                // keys are uint32 (nbits + sb <= 32) else uint64
    int sb = 0;                      // low key bits holding the orbit-size index (0: unreduced)
    void* d_keys = nullptr;          // sorted keys: (state << sb) | orbit-size index
    unsigned long long* d_dir = nullptr;   // search directory of bucket summaries (see DirSearch)
    int dir_shift = 0;               // bucket of a state = state >> dir_shift
    long long dir_nb = 0;            // number of buckets (entry dir_nb is a sentinel)
    int dir_steps = 0;               // ceil(log2(largest bucket)) for buckets searched in the keys
    int dir_K = 0;                   // keys summarised inline per bucket
    double dir_inline = 0.0;         // fraction of keys in buckets answered by their summary
    // Parent-state map of a reduced table whose parent is one fixed-popcount sector (optional):
    // entry r, for the parent state q of colex rank r (its index in the sorted parent basis; or r = q
    // itself when the map is direct), holds the
    // index c of q's representative | orbit-size index << map_cb | group element g (g.q = rep)
    // << (map_cb + sb), or all ones when q's orbit has no representative in the table.
    void* d_map = nullptr;
    int map_wide = 0;                // entries are uint64 (else uint32)
    int map_cb = 0;                  // bits of the index field
    int map_direct = 0;              // entries indexed by the state itself (2^nbits entries), not the rank
    int64_t map_n = 0;               // entries: C(nbits, popcount), or 2^nbits when direct
    void* d_rank = nullptr;          // colex rank chunk table [chunk][ones before][64 values]
    int rank_wide = 0;               // rank table entries are uint64 (else uint32)
    int rank_split = 0;              // > 0: split rank tables A (high bits) and B (rank_split low bits)
    uint64_t map_gen = 0;            // bumped whenever the map is built or freed
    ~Space();
};
// Build (or free) the parent-state map of a reduced space; false when it does not apply or would
// exceed max_bytes.
bool build_parent_map(Space& red, int64_t max_bytes, cudaStream_t st);
void free_parent_map(Space& red);
constexpr int RANK_CHUNK = 6;      // bits per chunk of the colex rank tables

// ---- device-side descriptors -------------------------------------------------------------------

struct GroupDev {
    int kind, G, den;
    int L1, L2, w, rowbits, nbits, nchunks;
    unsigned long long full;
    const int32_t* num;              // [G]
    const unsigned long long* keep;  // [L1] TORUS row-rotation masks (bits that do not wrap)
    const unsigned long long* lut;   // [G][nchunks][16] GENERIC
    const unsigned long long* flips; // [G] GENERIC
};

struct SectorDev {
    int n_sites, qlen, n_allowed, all_sectors;
    const int32_t* off;
    const int32_t* bw;
    const int32_t* dims;
    const int32_t* qbase;            // [n_sites] first local-state row of each site in qn
    const long long* qn;             // [sum dims][qlen]
    const long long* allowed;        // [n_allowed][qlen]
};

// Device copy of a Group (owned).
struct GroupBuffers {
    GroupDev dev{};
    int32_t* d_num = nullptr;
    unsigned long long* d_keep = nullptr;
    unsigned long long* d_lut = nullptr;
    unsigned long long* d_flips = nullptr;
    void upload(const Group& g, const Layout& lay);
    void release();
    ~GroupBuffers() { release(); }
};

// Host helpers used by several units.
std::vector<unsigned long long> torus_keep_masks(const Group& g, int nbits);
std::vector<unsigned long long> generic_luts(const Group& g, const Layout& lay, int* nchunks);

// ---- enumeration (enumerate.cu) ---------------------------------------------------------------
cudaStream_t lib_stream();
// Raise a kernel's dynamic shared-memory limit to at least smem bytes, never lowering it, under a
// process-wide lock (launches from several host threads must not leave a smaller limit in place).
void raise_smem_limit(const void* kern, size_t smem);
int sm_count();
void enumerate_parent(Space& s, cudaStream_t st);
void enumerate_reps(Space& red, const Space& parent, cudaStream_t st);
void build_mapping(const Space& red, const Space& parent, int64_t* index_out, double* ampl_out, cudaStream_t st);
void orbit_sizes(const Space& red, int32_t* out_host, cudaStream_t st);
void lookup_keys(const Space& s, const uint64_t* keys_host, int64_t n, int64_t* out_host, cudaStream_t st);
// Number of index bits for the divisors of G, and the divisor index of every stabiliser size.
int orbit_index_bits(int G);
// Rewrite a freshly enumerated representative table as keys (state << sb) | orbit-size index, and
// build the shared-memory search tree of any table.
void embed_orbit_index(Space& red, cudaStream_t st);
void build_search_directory(Space& s, cudaStream_t st);
void get_states(const Space& s, uint64_t* out_host, cudaStream_t st);
// Vectors between a reduced space and its parent on the device (symmetry_unreduce / symmetry_reduce):
// unreduce: out[n_parent] from in[dim]; reduce: out[dim] from in[n_parent].  complex128 (EDGPU_FP64) or
// complex64 (EDGPU_MIXED) vectors; the parent is materialised or a lazy popcount sector.
void reduce_vector(const Space& red, const Space& parent, int prec, bool unreduce, const void* in, void* out,
                   cudaStream_t st);
int64_t parent_dimension(const Space& parent);
// Diagonal element of every row: sum of the amplitudes of the row == col terms matching the row's state
// (FP64), written as complex128 (out64) and/or complex64 (out32).  scratch: device room for the T terms
// (4 words each), or null to allocate it for the call.
void compute_diagonal(const Space& s, int T, const uint64_t* masks, const uint64_t* rows, const double* amps,
                      double* out64, float* out32, unsigned long long* scratch, cudaStream_t st);
// Off-diagonal targets of every row (T terms: masks/rows/flips = row ^ col) and how many land in the table.
void count_nnz(const Space& s, int T, const uint64_t* masks, const uint64_t* rows, const uint64_t* flips,
               int64_t* n_targets, int64_t* n_found, cudaStream_t st);

constexpr int TORUS_MAXR = 8;      // most rows of a torus canonicalised with top-row pruning

// Search directory of a key table (bucket summaries; see key_find_sum2 in edgpu_device.cuh) with the
// constants of the in-register compare of a bucket's K member fields (mb bits each):
// unit = 1 in the lowest bit of every field, keybits = the state bits of every field (above the sb
// orbit-index bits), low = all but the top bit of every field, top = the top bit of every field.
struct DirSearch {
    const unsigned long long* dir;
    long long nb;
    int shift, mb, K, steps, sb;
    unsigned unit, keybits, low, top;
};
DirSearch dir_search_of(const Space& s);

// ---- matrix-free product (hx*.cu) ----------------------------------------------------------------
struct HxParams {
    const void* keys;
    long long n_rows;
    const void* x;
    void* y;
    const void* gy;
    double* grad_partial;
    int accumulate, rows_per_tile, n_coupl;
    const void* blob;
    int blob_words16;
    int o_om, o_or, o_of, o_oa, o_ou, o_oc;   // off-diagonal terms: mask,row,flip,amp,unit amp,coupling id
    int o_dm, o_dr, o_da, o_du, o_dc;         // diagonal terms
    DirSearch ds;                             // the search directory of the table
    const void* diag;                         // per-row diagonal element (V), product mode
    int o_ph, o_num, o_ratio, o_keep, o_lut, o_flip, o_grad;
    const void* lut_g;                        // GENERIC permutation tables in global memory (o_lut < 0)
    int o_rlut;                               // torus row table for top-row pruning, -1 when absent
    unsigned l1inv;                           // ceil(2^16 / L1) (candidate bit -> row of the pruned torus search)
    int rlut_pair;                            // the row table holds pairs of rows (rowbits <= 6)
    int o_keep32;                             // the torus keep masks as 32-bit words (states of <= 32 bits)
    int T_o, T_d, G, den, nd;
    int L1, L2, w, rowbits, nbits, nchunks;
    int sb, pb, want_arg, lpr;
    unsigned long long full;
    int warp_base;
    int o_sec, n_sec;                         // batched launch: shared-memory offset and count of SectorDesc
    long long n_tiles;                        // batched launch: warp tiles over all sectors
    // parent-state map (replaces canonicalisation and search when map != null)
    const void* map;
    int map_wide, map_cb, map_direct;
    const void* rank_tab;                     // colex rank chunk table
    int rank_wide, rank_k, rank_nc;           // entry width, popcount of the parent sector, chunks
    int rank_split;                           // > 0: rank = A[q >> rank_split] + B[q & low bits]
    // pair-flip schedule (hx_bond.cuh): bond classes of the off-diagonal terms, 0 when the terms are not
    // all two-site flips of 1-bit sites
    int bond_ncls;
    int o_bcomp, o_binfo, o_bflip, o_bamp;    // shared-memory offsets of the class tables
    int bond_real;                            // every pair amplitude is real
    int bond_nt;                              // targets per lane and step: 2, or 4 (parent-state map only)
    int bond_pf;                              // target tables: x prefetched this many steps ahead (0: none)
    int bond_uni;                             // target tables: warp-uniform pair steps (bond_tile UNI)
    // gradient mode of the pair-flip kernel (offsets into its shared-memory image, -1 when absent): the
    // slots' unit amplitudes and coupling ids, and the diagonal term records
    int o_bunit, o_bcid, o_pdm, o_pdr, o_pdu, o_pdc;
    int bunit_real;                           // every unit pair amplitude is real
    // the diagonal records by site pair (n_pdb entries; -1: a record has a mask of more than two bits):
    // i | j << 8 | coupling id << 16, and per entry the unit amplitudes of the pair's four bit patterns
    int o_pdb, o_pdv, n_pdb;
    // adjoint target table (column-sorted; built by the ADJ passes of bond_tile): per column the
    // count, the offset of its run, a fill cursor, and the entries (row << 32 | slot << 19 |
    // row's orbit-size index << 14 | group element)
    unsigned* adj_cnt;
    const long long* adj_off;
    unsigned* adj_cur;
    unsigned long long* adj_tab;
    // target table of the pair-flip schedule (GK_TABLE launches and the table's build pass)
    const void* tab;
    const long long* tile_off;
    int tab_wide, tab_cb;
    void* y_c128;                             // mixed precision: write y as complex128 here instead (or null)
};

// One sector of a batched launch (hx_multi_kernel), kept in shared memory after the common tables.
// The term, group and orbit-normalisation tables are common to all sectors; the basis table, its
// search directory, the diagonal, the vectors and the character table belong to the sector.
struct __align__(16) SectorDesc {
    const void* keys;
    const void* x;
    void* y;
    const void* diag;
    long long n_rows;
    long long tile_end;                       // cumulative warp tiles through this sector
    DirSearch ds;
    const void* map;                          // the sector's parent-state map (or null)
    int map_wide, map_cb, map_direct;
    int o_ph, o_num, want_arg;
    const void* tab;                          // the sector's target table (pair-flip schedule, or null)
    const long long* tile_off;
    int tab_wide, tab_cb;
};

constexpr int BOND_MAXC = 4;       // rotation components per bond class of the pair-flip schedule
constexpr int BOND_MAXCLS = 24;    // bond classes at most (more: the term-matching schedule)

constexpr size_t GENERIC_SMEM_LUT = 64 * 1024;   // larger GENERIC permutation tables stay in global memory
constexpr int HX_QCAP = 128;         // per-warp target queue capacity (entries; 2 batches of 32 + 31)
constexpr int HX_THREADS = 256;      // threads per block of the product kernel
int hx_warp_bytes(bool w32);

// Launch the product kernel for (word width, group kind, precision, gradient mode).
void hx_launch_w32(int gk, int prec, int mode, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
void hx_launch_w64(int gk, int prec, int mode, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
int hx_max_blocks_per_sm(bool w32, int gk, int prec, int mode, size_t smem);
// Row-per-lane strategy (hx_rows.cuh), product mode only.
void hx_rows_launch_w32(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
void hx_rows_launch_w64(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
int hx_rows_occupancy_w32(int gk, int prec, size_t smem);
int hx_rows_occupancy_w64(int gk, int prec, size_t smem);
// Sparse assembly of a representation in FP64 (hx_rows.cuh, hx_sparse_kernel); shared memory:
// the blob's warp_base plus 4 warps x (T_o + 1) x 48 bytes.
void hx_sparse_launch_w32(int gk, const HxParams& p, long long row0, long long n_run, int conj_vals, double tol,
                          long long* counts, const long long* row_ptr, long long* cols, double2* vals, size_t smem,
                          cudaStream_t st);
void hx_sparse_launch_w64(int gk, const HxParams& p, long long row0, long long n_run, int conj_vals, double tol,
                          long long* counts, const long long* row_ptr, long long* cols, double2* vals, size_t smem,
                          cudaStream_t st);
// Row-per-lane gradient mode (hx_rows_kernel MODE 1): shared memory o_grad + n_coupl x HX_THREADS x 8.
void hx_rows_grad_launch_w32(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
void hx_rows_grad_launch_w64(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
int hx_rows_grad_occupancy_w32(int gk, int prec, size_t smem);
int hx_rows_grad_occupancy_w64(int gk, int prec, size_t smem);
// Adjoint of the product's matrix by scatter (hx_rows.cuh, hx_scatter_adjoint_kernel): p.gy = input,
// p.y = output (zeroed or accumulated by the caller); shared memory as the row-per-lane kernel.
void hx_scatter_launch_w32(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
void hx_scatter_launch_w64(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
// Batched sectors in one persistent launch (hx_rows.cuh, hx_multi_kernel), product mode only.
void hx_multi_launch_w32(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
void hx_multi_launch_w64(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
int hx_multi_occupancy_w32(int gk, int prec, size_t smem);
int hx_multi_occupancy_w64(int gk, int prec, size_t smem);

// Pair-flip schedule (hx_bond.cuh), product mode only: one sector, and all sectors of a batch.
void hx_bond_launch_w32(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
void hx_bond_launch_w64(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
int hx_bond_occupancy_w32(int gk, int prec, int nt, size_t smem);
int hx_bond_occupancy_w64(int gk, int prec, int nt, size_t smem);
void hx_bond_multi_launch_w32(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
void hx_bond_multi_launch_w64(int gk, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
int hx_bond_multi_occupancy_w32(int gk, int prec, int nt, size_t smem);
int hx_bond_multi_occupancy_w64(int gk, int prec, int nt, size_t smem);

// Target table of the pair-flip schedule (hxtable.cu): count the targets of every warp tile of 32 rows,
// scan the counts into tile offsets (returns the total), and write every target's map-format entry,
// looked up with flavour gk (GK_MAP or a canonicalising kind).  p: the pair-flip launch template with
// lpr = 1; p.tab / p.tile_off / p.tab_wide / p.tab_cb set for the fill.
void hx_table_count(bool w32, const HxParams& p, long long n_tiles, long long* tile_cnt, size_t smem, cudaStream_t st);
long long hx_table_scan(const long long* tile_cnt, long long n_tiles, long long* tile_off, cudaStream_t st);
void hx_table_fill(bool w32, int gk, const HxParams& p, long long n_tiles, size_t smem, cudaStream_t st);
// The product through the table (GK_TABLE), one sector and all sectors of a batch.
void hx_table_launch(bool w32, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
int hx_table_occupancy(bool w32, int prec, int nt, size_t smem, bool uni = false);
void hx_table_multi_launch(bool w32, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
int hx_table_multi_occupancy(bool w32, int prec, int nt, size_t smem);
// The product fused with the coupling gradient on the pair-flip schedule (hx_bond.cuh, GRAD mode):
// targets from the target table (table) or the parent-state map, four per lane and step.  Shared
// memory: the pair-flip image up to p.o_grad, then n_couplings x HX_THREADS doubles.
void hx_bond_grad_launch(bool w32, bool table, int prec, const HxParams& p, int blocks, size_t smem, cudaStream_t st);
int hx_bond_grad_occupancy(bool w32, bool table, int prec, size_t smem);
// Adjoint target table (hxtable.cu): pass 1 counts every column's targets (p.adj_cnt), pass 2 writes
// each target's entry into its column's run (p.adj_off, p.adj_cur, p.adj_tab); the runs are then
// sorted so that the summation order is fixed.  p: the table-flavour pair-flip template (lpr = 1).
void hx_adj_pass(bool w32, int pass, const HxParams& p, long long n_tiles, size_t smem, cudaStream_t st);
void hx_adj_sort(const long long* off, unsigned long long* tab, long long n, cudaStream_t st);
// y = H^dagger x through the adjoint target table: one lane per column, its run in order; p.gy = x.
void hx_adj_launch(bool w32, int prec, const HxParams& p, size_t smem, cudaStream_t st);

// ---- column-slab table of the pair-flip schedule (hxslab.cu) -------------------------------------
// The target table's entries regrouped by column slab: slab q holds the columns [q wc, (q + 1) wc).
// Pass q of the product gathers only from slab q (sized to stay in L2 while the pass runs) and adds
// its share to y.  Per pass: a count byte per row, a 32-bit offset per warp tile of 32 rows
// (relative to the pass's first entry), and the entries tile by tile, row by row, each row's
// entries in the target table's order; an entry is (column - q wc) | id << colbits, where id
// indexes the coefficient table: id = ((amplitude id x den + character index) x nd + orbit-size
// index of the row) x nd + orbit-size index of the column.
struct SlabBuild {
    long long wc;                   // columns per slab
    int n_pass;
    long long n_tiles;
    unsigned char* counts;          // [n_pass][n_rows] (written by the count pass)
    unsigned* tile_sum;             // [n_pass][n_tiles] (written by the count pass)
    const unsigned* off;            // [n_pass][n_tiles] tile offsets relative to the pass (fill pass)
    const long long* base;          // [n_pass] first entry of each pass (fill pass)
    unsigned* tab;                  // the entries (fill pass)
    const unsigned short* amp_id;   // [n_slots] amplitude id of every pair-flip slot (fill pass)
    unsigned char* cls;             // [n_rows] every row's orbit-size index (count pass; null: not kept)
    int n_slots;
    int colbits;
    int scaled;                     // ids without the orbit-size indices (amplitude id x den + character)
    int o_ctr;                      // shared-memory offset of the per-thread pass counters / cursors
};
struct SlabRun {
    const unsigned char* cnt;       // this pass's count bytes [n_rows]
    const unsigned* off;            // this pass's tile offsets [n_tiles]
    const unsigned* tab;            // this pass's entries
    const void* xs;                 // x from the slab's first column
    const void* x;                  // x (first pass: the diagonal's product)
    void* y;
    const void* diag;
    const void* lut;                // coefficients by id: V, or R when lut_real
    void* y_c128;                   // last pass: complex128 output instead of y (host buffers)
    long long n_rows, n_tiles;
    unsigned colmask;
    int colbits, n_lut, lut_real;
    int first, last, accumulate, acc_c128;
    int hints;                      // 0 to 3: one lane per row (bit 0: gathers cached in L2 only,
                                    // streamed data evict-first; bit 1: eight entries per lane and step
                                    // instead of four); 4, 5: two, four lanes per row
    int lut_mode;                   // 0: one shared-memory copy of the coefficients; 1: a copy per
                                    // bank group (conflict-free lookups); 2: real, at most 4, in registers
    // scaled tables: xs and x hold sqrt(|O_c|) x_c; the last pass multiplies row r by 1/sqrt(|O_r|)
    // (and the first pass of y += H x the old y_r by sqrt(|O_r|))
    int scaled;
    const unsigned char* cls;       // [n_rows] orbit-size index of every row
    const void* scale;              // R[2 nd]: sqrt(|O|) by orbit-size index, then 1 / sqrt(|O|)
    int nd;
    long long tile0;                // the launch covers the tiles [tile0, tile0 + n_tiles)
    int blocks_per_sm;              // 0: as many as fit; > 0: at most that many; < 0: leave -blocks_per_sm free
};
// Coefficient tables of at most this many entries go to registers (real) or to one copy per shared-
// memory bank group (SLAB_REP_BYTES in all, which keeps eight blocks of the slab kernel per SM).
constexpr int SLAB_REG_LUT = 4;
constexpr int SLAB_REP_BYTES = 24 * 1024;
// x_c -> sqrt(|O_c|) x_c for the columns [c0, c1) of x (R = float for complex64, double for complex128;
// scale = the column scales by orbit-size index), written to out at the same columns.  From a complex128
// source to a complex64 result (mixed precision from host buffers) x_c is rounded to complex64 first.
void launch_slab_xscale(int prec, const void* x, const unsigned char* cls, const void* scale, void* out,
                        int64_t c0, int64_t c1, cudaStream_t st);
void launch_slab_xscale_c128_c64(const double* x, const unsigned char* cls, const float* scale, float* out,
                                 int64_t c0, int64_t c1, cudaStream_t st);
// Count pass (1) or fill pass (2) of the slab table from the target table.  p: the table-flavour
// pair-flip template (tab, tile_off set; lpr = 1); smem: its image plus s.o_ctr's counters.
void hx_slab_build(bool w32, int prec, int pass, const HxParams& p, const SlabBuild& s, size_t smem,
                   cudaStream_t st);
// Per pass: exclusive scan of the tile sums [n_pass][n_tiles] into 32-bit offsets relative to the
// pass; totals[q] = entries of pass q (host, after a synchronisation).
void hx_slab_scan(const unsigned* tile_sum, unsigned* off, int n_pass, long long n_tiles,
                  std::vector<unsigned long long>& totals, cudaStream_t st);
// One pass of the slab product.
void hx_slab_launch(int prec, const SlabRun& r, cudaStream_t st);

// ---- the coupling-gradient launch for callers that cannot allocate (noalloc.cu) -----------------
// The fused product and coupling gradient exactly as edgpu_coupling_grad_device launches it (same
// kernel choice), with the per-block partial sums written to partial[blocks][n_couplings] and at most
// cap_blocks blocks.  False, with nothing launched or allocated, when the operator's tables for this
// precision (gradient and product mode) have not been built yet.
bool coupling_grad_launch_built(edgpu_op op, int prec, const void* x, const void* gy, void* y, double* partial,
                                int cap_blocks, cudaStream_t st, int* blocks_used);
int coupling_count(edgpu_op op);
int64_t op_dimension(edgpu_op op);
// The call lock of an operator handle (calls on one handle are serialised).
std::unique_lock<std::mutex> lock_op(edgpu_op op);
// Record an error message for edgpu_last_error() and return code.
int record_api_error(int code, const std::string& msg);

// ---- vector kernels (linalg.cu) ------------------------------------------------------------------
void launch_random_c128(int64_t n, uint64_t seed, double* dst, cudaStream_t st);
void launch_c128_to_c64(int64_t n, const double* src, float* dst, cudaStream_t st);
void launch_c64_to_c128(int64_t n, const float* src, double* dst, int accumulate, cudaStream_t st);
void launch_scale_c128(int64_t n, double s, double* v, cudaStream_t st);
void launch_conj_c128(int64_t n, double* v, cudaStream_t st);
// Deterministic FP64 reductions through a per-call scratch buffer of at least dot_scratch_doubles().
size_t dot_scratch_doubles();
void launch_dot_c128(int64_t n, const double* a, const double* b, double* scratch, double* out_dev, cudaStream_t st);
void launch_norm2_c128(int64_t n, const double* a, double* scratch, double* out_dev, cudaStream_t st);
void launch_reduce_grad(int nblocks, int ncoupl, const double* partial, double* out_dev, cudaStream_t st);
// Lanczos helpers: w = w - a*v - b*u (a, b device scalars, b may be null)
void launch_lanczos_update(int64_t n, double* w, const double* v, const double* u, const double* alpha_dev,
                           const double* beta_dev, cudaStream_t st);
// w = w - V h (h: k complex device values), and h = V^H w
void launch_multi_dot(int64_t n, int k, const double* V, int64_t ldv, const double* w, double* scratch,
                      double* h_dev, cudaStream_t st);
void launch_multi_axpy(int64_t n, int k, const double* V, int64_t ldv, const double* h_dev, double* w,
                       cudaStream_t st);
// the same with a complex64 basis V (FP64 accumulation)
void launch_multi_dot_c64(int64_t n, int k, const float* V, int64_t ldv, const double* w, double* scratch,
                          double* h_dev, cudaStream_t st);
void launch_multi_axpy_c64(int64_t n, int k, const float* V, int64_t ldv, const double* h_dev, double* w,
                           cudaStream_t st);
// v_next = w / beta (beta device scalar); also writes a complex64 copy when v32 != null
void launch_normalize(int64_t n, const double* w, const double* beta_dev, double* v_next, float* v32,
                      cudaStream_t st);
void launch_axpy_real(int64_t n, double a, const double* x, double* y, cudaStream_t st);

}  // namespace edgpu
