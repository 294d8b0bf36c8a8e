// C ABI of libedgpu.so (declared in include/edgpu.h): handle management, argument validation with
// the reference's error classes, precision staging, the product launcher, the batched launcher and the
// Lanczos driver.  All arithmetic on vectors runs in the CUDA kernels of enumerate.cu, hx*.cu and
// linalg.cu; there is no CPU fallback.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>
#include <memory>
#include <mutex>
#include <thread>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "edgpu_internal.h"

using namespace edgpu;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

#define API_BEGIN try {
#define API_END                                                        \
    }                                                                  \
    catch (const Error& e) { return fail(e.code, e.what()); }          \
    catch (const std::bad_alloc&) { return fail(EDGPU_ERR_OOM, "host allocation failed"); } \
    catch (const std::exception& e) { return fail(EDGPU_ERR_STATE, e.what()); }            \
    return EDGPU_OK;

void require(bool cond, int code, const std::string& msg) {
    if (!cond) throw Error(code, msg);
}

std::mutex g_init_mu;
cudaStream_t g_stream = nullptr;   // stream of the calls that belong to no handle
int g_sm_count = 0;

void init_device() {
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (g_stream) return;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        throw Error(EDGPU_ERR_CUDA, std::string("no CUDA device available: ") + cudaGetErrorString(e));
    int dev = 0;
    EDGPU_CUDA(cudaGetDevice(&dev));
    EDGPU_CUDA(cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev));
    EDGPU_CUDA(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking));
}

// NULL selects the CUDA default stream, like the stream argument of CUDA's own libraries.
cudaStream_t pick_stream(void* s) { return (cudaStream_t)s; }

// What every handle (space, operator, batch) owns for concurrency: the mutex that serialises calls on
// the handle, and its own non-blocking stream (created on first use) for the work of calls that take
// no stream argument (builds, host-buffer products, the autotuner, Lanczos).  Distinct handles run
// concurrently from different host threads, each on its own stream.
template <typename M>
struct HandleSyncT {
    M mu;
    cudaStream_t st = nullptr;
    cudaStream_t stream() {
        if (!st) EDGPU_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        return st;
    }
    HandleSyncT() = default;
    HandleSyncT(const HandleSyncT&) = delete;
    HandleSyncT& operator=(const HandleSyncT&) = delete;
    ~HandleSyncT() {
        if (st) cudaStreamDestroy(st);
    }
};
using HandleSync = HandleSyncT<std::mutex>;
// Spaces use a recursive mutex: a batch holds the locks of its sectors' spaces while it launches, and
// an operator's launch takes its space's lock again.
using SpaceSync = HandleSyncT<std::recursive_mutex>;
using OpLock = std::lock_guard<std::mutex>;
using SpaceLock = std::lock_guard<std::recursive_mutex>;

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    void ensure(size_t count) {
        if (count <= n && p) return;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        EDGPU_CUDA(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
        n = count;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DevBuf() { release(); }
};

int bitwidth_of(int dim) {
    int w = 0;
    while ((1LL << w) < dim) ++w;
    return w;
}

unsigned long long binom_u64(int n, int k) {
    if (k < 0 || k > n) return 0;
    unsigned long long r = 1;
    for (int i = 1; i <= k; ++i) r = r * (unsigned long long)(n - k + i) / (unsigned long long)i;
    return r;
}

// ---- operator representation ------------------------------------------------------------------

struct Blob {
    bool ready = false;
    int gk = 0;              // product-kernel group kind (GK_RING for 32-bit rings)
    void* d = nullptr;
    HxParams tmpl{};
    size_t smem = 0;
    int max_blocks = 0;      // resident blocks for the whole GPU
    int rows_per_tile = 32;
    void* d_diag = nullptr;  // per-row diagonal element in the blob's precision (product mode)
    size_t cap_d = 0, cap_pair = 0, cap_diag = 0;   // bytes allocated at d, d_pair, d_diag
    void* d_lut = nullptr;   // GENERIC permutation tables in global memory (when too large for shared memory)
    size_t cap_lut = 0;
    size_t smem_rows = 0;    // shared memory of the row-per-lane kernel (no per-warp queues)
    int max_blocks_rows = 0;
    int max_blocks_map = 0;  // resident blocks of the parent-state-map kernel (computed on first use)
    int max_blocks_grad = 0; // resident blocks of the row-per-lane gradient kernel (computed on first use)
    int max_blocks_pgrad[2] = {0, 0};   // of the pair-flip gradient kernel [target table]
    size_t smem_bond = 0;    // shared memory of the mapped pair-flip kernel (the blob's prefix up to the bond tables)
    size_t smem_bond_canon = 0;   // of the canonicalising one (through the torus row table)
    size_t term_start = 0;   // offset of the term records in the term image (before: group and torus tables)
    size_t bond_end = 0;     // end of the bond classes in the pair-flip image (the torus row table follows)
    void* d_pair = nullptr;  // the pair-flip image: group tables, bond classes, torus row table
    std::vector<unsigned char> pair_host;   // its host copy (batched images start from it)
    HxParams tmpl_pair{};    // launch template of the pair-flip kernel (offsets into d_pair)
    int max_blocks_bond[2][2] = {{0, 0}, {0, 0}};   // resident blocks of the pair-flip kernel [mapped][4 targets]
    int max_blocks_table[2][3] = {{0, 0, 0}, {0, 0, 0}};   // of its target-table flavour [warp-uniform][2, 4, 8 targets]
    ~Blob() {
        if (d) cudaFree(d);
        if (d_diag) cudaFree(d_diag);
        if (d_pair) cudaFree(d_pair);
        if (d_lut) cudaFree(d_lut);
    }
};

}  // namespace

// A space handle: the space plus its call lock and stream.  Operators on the space take the lock while
// they enqueue work that reads the space's parent-state map, so the map cannot be freed under them.
struct edgpu_space_s : public Space {
    SpaceSync hs;
};

// Largest Krylov basis (bytes) the Lanczos driver stores; 0: half of the free device memory.
int64_t g_krylov_limit = 0;

struct edgpu_op_s {
    HandleSync hs;                    // call lock and stream of this handle
    edgpu_space_s* space = nullptr;
    int T = 0;
    std::vector<uint64_t> masks, rows, cols;
    std::vector<double> unit;         // 2T: per-unit-coupling amplitudes (the amplitudes when uncoupled)
    std::vector<int32_t> cid;         // T
    int n_coupl = 1;
    std::vector<double> coupl{1.0};
    Blob blob[2][2][2];               // [precision][direction 0 = H, 1 = H^dagger][mode 0 = product, 1 = gradient]
    int tuned_rows[2] = {0, 0};
    int pair_allowed = 1;             // the caller allows the pair-flip schedule (edgpu_op_set_pair_schedule)
    int pair_use[2] = {1, 1};         // [precision]: use it where the terms allow it (chosen by the autotuner)
    int pair_nt[2] = {2, 2};          // [precision]: targets per lane and step with a parent-state map (2 or 4)
    uint64_t gen = 0;                 // bumped whenever the device tables are rebuilt
    uint64_t invariant_gen = ~0ull;   // table generation the invariance flag belongs to
    bool invariant = true;            // the terms commute with every element of the space's group
    DevBuf<double> x64, y64, z64;
    DevBuf<float> x32, y32;
    DevBuf<double> grad_partial, grad_dev;
    DevBuf<unsigned long long> diag_scratch;   // device copy of the diagonal terms while the diagonal is computed
    std::map<std::vector<const void*>, cudaGraphExec_t> host_graphs;   // replayed host-buffer products
    // target table of the pair-flip schedule (optional, edgpu_op_build_targets)
    void* d_tab = nullptr;
    long long* d_tile_off = nullptr;
    int tab_wide = 0, tab_cb = 0;
    int64_t tab_n = 0;
    int tab_use[2] = {1, 1};          // [precision]: products read the table (chosen by the autotuner)
    int tab_pf[2] = {0, 0};           // [precision]: x prefetched this many steps ahead (chosen by the autotuner)
    int tab_uni[2] = {0, 0};          // [precision]: warp-uniform pair steps (chosen by the autotuner)
    // adjoint target table (optional, edgpu_op_build_adjoint_targets): per column its sorted run of
    // (row, slot, orbit-size index of the row, group element) entries
    long long* d_adj_off = nullptr;
    unsigned long long* d_adj_tab = nullptr;
    int64_t adj_n = 0;
    // column-slab table (optional, edgpu_op_build_slabs; mixed-precision products, hxslab.cu)
    struct Slab {
        unsigned* tab = nullptr;            // entries, pass after pass
        unsigned char* counts = nullptr;    // [n_pass][dim] entries of each row in each pass
        unsigned* off = nullptr;            // [n_pass][tiles] tile offsets relative to the pass
        std::vector<long long> base;        // [n_pass + 1] first entry of each pass
        int n_pass = 0, colbits = 0, n_ids = 0, den = 1, nd = 1;
        long long wc = 0;                   // columns per slab
        int64_t n = 0;                      // entries
        std::vector<int> amp_cid;           // per amplitude id: its coupling id (-1: none)
        std::vector<double> amp_unit;       // per amplitude id: unit amplitude (re, im)
        std::vector<int> divs;              // orbit sizes by orbit-size index
        DevBuf<float> lut;                  // coefficients by id: float, or (re, im) when !lut_real
        DevBuf<double> lut64;               // the same in FP64
        int lut_real = 1;
        int lut_mode = 0;                   // SlabRun::lut_mode
        // scaled table: ids carry no orbit-size indices; x is scaled by sqrt(|O_c|) into xsc before the
        // passes and row r of the result by 1 / sqrt(|O_r|) in the last pass
        int scaled = 0;
        unsigned char* cls = nullptr;       // [dim] orbit-size index of every representative
        DevBuf<float> sc32;                 // [2 nd] sqrt(|O|), then 1 / sqrt(|O|), by orbit-size index
        DevBuf<double> sc64;
        DevBuf<double> xsc;                 // [2 dim] the scaled x (complex64 or complex128)
    } slab;
    int slab_scaling = 0;             // scaled slab tables: 0 for sectors of 2^22 rows or more, 1 never, 2 always
    int slab_use[2] = {0, 0};         // [precision]: products read the slab table (chosen by the autotuner)
    // host-buffer slab products: a second stream converting x slab by slab while the passes run
    cudaStream_t aux_st = nullptr;
    cudaEvent_t aux_fork = nullptr;
    std::vector<cudaEvent_t> slab_ready;
    void ensure_slab_events(int n) {
        if (!aux_st) EDGPU_CUDA(cudaStreamCreateWithFlags(&aux_st, cudaStreamNonBlocking));
        if (!aux_fork) EDGPU_CUDA(cudaEventCreateWithFlags(&aux_fork, cudaEventDisableTiming));
        while ((int)slab_ready.size() < n) {
            cudaEvent_t e = nullptr;
            EDGPU_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            slab_ready.push_back(e);
        }
    }
    // host-buffer slab products in row blocks: each block's last pass (which writes the host buffer)
    // runs on this stream while the next block's passes run
    cudaStream_t blk_st = nullptr;
    std::vector<cudaEvent_t> blk_ev;   // [block] its passes before the last are done; then: all done
    void ensure_block_events(int n) {
        if (!blk_st) EDGPU_CUDA(cudaStreamCreateWithFlags(&blk_st, cudaStreamNonBlocking));
        while ((int)blk_ev.size() < n + 1) {
            cudaEvent_t e = nullptr;
            EDGPU_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            blk_ev.push_back(e);
        }
    }
    int slab_hint[2] = {0, 0};        // [precision]: the slab product's cache hints (chosen by the autotuner)
    // the optional tables change: cached graphs (this handle's host-buffer graphs, and batches, which
    // compare gen) must not replay launches that read the old ones
    void drop_host_graphs() {
        for (auto& kv : host_graphs) cudaGraphExecDestroy(kv.second);
        host_graphs.clear();
        ++gen;
    }
    void free_slabs() {
        drop_host_graphs();
        if (slab.tab) cudaFree(slab.tab);
        if (slab.counts) cudaFree(slab.counts);
        if (slab.off) cudaFree(slab.off);
        if (slab.cls) cudaFree(slab.cls);
        slab.lut.release();
        slab.lut64.release();
        slab.sc32.release();
        slab.sc64.release();
        slab.xsc.release();
        slab = Slab();
        slab_use[0] = slab_use[1] = 0;
    }
    void free_table() {
        drop_host_graphs();
        if (d_tab) cudaFree(d_tab);
        if (d_tile_off) cudaFree(d_tile_off);
        d_tab = nullptr;
        d_tile_off = nullptr;
        tab_n = 0;
    }
    void free_adjoint() {
        drop_host_graphs();
        if (d_adj_off) cudaFree(d_adj_off);
        if (d_adj_tab) cudaFree(d_adj_tab);
        d_adj_off = nullptr;
        d_adj_tab = nullptr;
        adj_n = 0;
    }
    ~edgpu_op_s() {
        drop_host_graphs();
        free_table();
        free_adjoint();
        free_slabs();
        if (aux_st) {
            cudaStreamSynchronize(aux_st);
            cudaStreamDestroy(aux_st);
        }
        if (aux_fork) cudaEventDestroy(aux_fork);
        for (auto e : slab_ready) cudaEventDestroy(e);
        if (blk_st) {
            cudaStreamSynchronize(blk_st);
            cudaStreamDestroy(blk_st);
        }
        for (auto e : blk_ev) cudaEventDestroy(e);
    }
};

// Sectors applied in one persistent launch (hx_multi_kernel).  Per precision: the common shared-memory
// image (term, group and orbit-normalisation tables of the first operator, then every sector's
// character table), and per set of vector pointers and lanes per row a device copy of that image
// followed by the sector descriptors, plus the CUDA graph replaying the launch.
struct edgpu_batch_s {
    HandleSync hs;                                 // call lock and stream of this handle
    std::vector<edgpu_op_s*> ops;
    int lpr[2] = {0, 0};                           // lanes per row (0: default 1)
    int pair_use[2] = {1, 1};                      // pair-flip schedule where the terms allow it (autotuned)
    int pair_nt[2] = {2, 2};                       // its targets per lane and step with sector maps
    int tab_use[2] = {1, 1};                       // read the sectors' target tables (autotuned)
    int tab_pf[2] = {0, 0};                        // their x prefetch distance in steps (autotuned)
    // launch: 0 = all sectors in one persistent launch; k >= 1 = one product launch per sector (the
    // operator's product kernel with the batch's schedule), spread over k streams that run
    // concurrently (the calling stream alone for k = 1)
    int seq[2] = {0, 0};
    int seq_own[2] = {0, 0};                       // per-sector launches keep each operator's own schedule
    cudaStream_t lane_st[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t fork_ev = nullptr, join_ev[3] = {nullptr, nullptr, nullptr};
    void ensure_lanes(int k) {
        if (!fork_ev) EDGPU_CUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
        for (int i = 0; i < k; ++i) {
            if (!lane_st[i]) EDGPU_CUDA(cudaStreamCreateWithFlags(&lane_st[i], cudaStreamNonBlocking));
            if (!join_ev[i]) EDGPU_CUDA(cudaEventCreateWithFlags(&join_ev[i], cudaEventDisableTiming));
        }
    }
    struct Fused {
        bool ready = false;
        std::vector<uint64_t> gens;                // operator table generations the image was built from
        std::vector<unsigned char> image;          // common tables + per-sector character tables + descriptors
                                                   // + term records
        size_t smem_pair = 0;                      // the image's part before the term records
        size_t smem_lookup = 0;                    // its part before the torus row table
        std::vector<int> o_ph, o_num, want_arg;
        HxParams tmpl{};
        int gk = 0, per_sm = 1, per_sm_map = 0;
        int per_sm_bond[2][2] = {{0, 0}, {0, 0}};   // pair-flip kernel [mapped][4 targets per step]
        int per_sm_table[3] = {0, 0, 0};            // its target-table flavour [2, 4, 8 targets per step]
        size_t smem = 0;
        int64_t rows = 0;
    } fused[2];
    std::map<std::vector<const void*>, void*> images[2];
    std::map<std::vector<const void*>, cudaGraphExec_t> graphs[2];
    void drop(int prec) {
        for (auto& kv : images[prec]) cudaFree(kv.second);
        for (auto& kv : graphs[prec]) cudaGraphExecDestroy(kv.second);
        images[prec].clear();
        graphs[prec].clear();
        fused[prec] = Fused();
    }
    ~edgpu_batch_s() {
        drop(0);
        drop(1);
        for (int i = 0; i < 3; ++i) {
            if (lane_st[i]) {
                cudaStreamSynchronize(lane_st[i]);
                cudaStreamDestroy(lane_st[i]);
            }
            if (join_ev[i]) cudaEventDestroy(join_ev[i]);
        }
        if (fork_ev) cudaEventDestroy(fork_ev);
    }
};

namespace edgpu {
cudaStream_t lib_stream() { return g_stream; }

void raise_smem_limit(const void* kern, size_t smem) {
    static std::mutex mu;
    static std::unordered_map<const void*, size_t> set;
    std::lock_guard<std::mutex> lk(mu);
    size_t& cur = set[kern];
    if (smem <= cur) return;
    EDGPU_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    cur = smem;
}
int sm_count() { return g_sm_count; }
int hx_max_blocks_per_sm(bool w32, int gk, int prec, int mode, size_t smem);
}  // namespace edgpu

namespace {

size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

// Bond classes of the pair-flip schedule (hx_bond.cuh).  Applies when every off-diagonal term flips
// two sites of one bit each (mask = two bits = row ^ col) and each pair's terms come in complete
// antiparallel (01, 10) and/or parallel (00, 11) couples, as in every Hermitian spin-1/2 exchange.
// Pairs are sorted by their ring distance and assigned greedily to the first class where one of
// their two orientations (start, shift) has a free start bit, preferring a class that already has the
// shift as a component (at most BOND_MAXC components per class).
struct BondClasses {
    int ncls = 0;
    std::vector<int32_t> info;        // [ncls] components | has_parallel << 8
    std::vector<uint64_t> comp;       // [ncls][BOND_MAXC][4]: shift, antiparallel starts, parallel starts, 0
    std::vector<uint64_t> flip;       // [ncls][n]
    std::vector<double> amp;          // [ncls][n][4][2]
    std::vector<int32_t> cid;         // [ncls][n][4] coupling id of each slot's terms (-1: no term)
    bool cid_ok = true;               // the terms of every slot share one coupling id
    bool real = true;
};

bool build_bond_classes(const Layout& lay, const std::vector<uint64_t>& masks, const std::vector<uint64_t>& rows,
                        const std::vector<uint64_t>& flips, const std::vector<double>& amps, BondClasses& out,
                        const std::vector<int32_t>* cids = nullptr) {
    const int n = lay.nbits;
    if (masks.empty() || n < 2 || n > 64) return false;
    for (int i = 0; i < lay.n_sites; ++i)
        if (lay.bw[i] != 1) return false;
    struct Pair {
        int a, b;                      // bits a < b
        double amp[4][2];              // by (b_a, b_b) pattern: index b_a | b_b << 1
        bool have[4];
        int cid[4];                    // coupling id of the pattern's terms (-1: none yet)
    };
    std::map<std::pair<int, int>, Pair> pairs;
    for (size_t t = 0; t < masks.size(); ++t) {
        const uint64_t m = masks[t];
        if (__builtin_popcountll(m) != 2 || flips[t] != m || (rows[t] & ~m) != 0) return false;
        const int a = __builtin_ctzll(m), b = 63 - __builtin_clzll(m);
        Pair& P = pairs[{a, b}];
        if (P.a == P.b) {
            P.a = a;
            P.b = b;
            for (int v = 0; v < 4; ++v) {
                P.amp[v][0] = P.amp[v][1] = 0.0;
                P.have[v] = false;
                P.cid[v] = -1;
            }
        }
        const int pat = (int)((rows[t] >> a) & 1u) | (int)(((rows[t] >> b) & 1u) << 1);
        P.amp[pat][0] += amps[2 * t];
        P.amp[pat][1] += amps[2 * t + 1];
        P.have[pat] = true;
        if (cids) {
            const int c = (*cids)[t];
            if (P.cid[pat] >= 0 && P.cid[pat] != c) out.cid_ok = false;
            P.cid[pat] = c;
        }
    }
    std::vector<Pair> list;
    for (auto& kv : pairs) {
        const Pair& P = kv.second;
        // complete couples only: a row whose bits match one pattern of a couple must have its term
        if (P.have[1] != P.have[2] || P.have[0] != P.have[3]) return false;
        list.push_back(P);
    }
    auto dist = [n](const Pair& P) { const int d = P.b - P.a; return std::min(d, n - d); };
    std::stable_sort(list.begin(), list.end(), [&](const Pair& x, const Pair& y) { return dist(x) < dist(y); });
    struct Cls {
        uint64_t used = 0;
        std::vector<int> shifts;
        std::vector<uint64_t> A, P;
        std::vector<int> partner = std::vector<int>(64, -1);
        std::vector<std::array<double, 8>> amp = std::vector<std::array<double, 8>>(64);
        std::vector<std::array<int, 4>> cid = std::vector<std::array<int, 4>>(64, std::array<int, 4>{-1, -1, -1, -1});
        bool par = false;
    };
    std::vector<Cls> cls;
    for (const Pair& P : list) {
        const int starts[2] = {P.a, P.b};
        const int parts[2] = {P.b, P.a};
        int best_c = -1, best_o = -1, best_score = 3;
        for (int c = 0; c < (int)cls.size() && best_score > 0; ++c)
            for (int o = 0; o < 2; ++o) {
                if ((cls[c].used >> starts[o]) & 1ull) continue;
                const int sh = ((parts[o] - starts[o]) % n + n) % n;
                const bool has = std::find(cls[c].shifts.begin(), cls[c].shifts.end(), sh) != cls[c].shifts.end();
                const int score = has ? 0 : ((int)cls[c].shifts.size() < BOND_MAXC ? 1 : 3);
                if (score < best_score) {
                    best_score = score;
                    best_c = c;
                    best_o = o;
                }
            }
        if (best_c < 0) {
            if ((int)cls.size() >= BOND_MAXCLS) return false;
            cls.emplace_back();
            best_c = (int)cls.size() - 1;
            best_o = 0;
        }
        Cls& C = cls[best_c];
        const int st = starts[best_o], pt = parts[best_o];
        const int sh = ((pt - st) % n + n) % n;
        int k = (int)(std::find(C.shifts.begin(), C.shifts.end(), sh) - C.shifts.begin());
        if (k == (int)C.shifts.size()) {
            C.shifts.push_back(sh);
            C.A.push_back(0);
            C.P.push_back(0);
        }
        C.used |= 1ull << st;
        C.partner[st] = pt;
        // v = b_start | (b_start == b_partner) << 1; pattern index = b_a | b_b << 1 of the pair
        for (int v = 0; v < 4; ++v) {
            const int bs = v & 1;
            const int bp = (v >> 1) ? bs : 1 - bs;
            const int pat = (st == P.a) ? (bs | (bp << 1)) : (bp | (bs << 1));
            C.amp[st][2 * v] = P.amp[pat][0];
            C.amp[st][2 * v + 1] = P.amp[pat][1];
            C.cid[st][v] = P.cid[pat];
            if (P.amp[pat][1] != 0.0) out.real = false;
        }
        if (P.have[1]) C.A[k] |= 1ull << st;
        if (P.have[0]) {
            C.P[k] |= 1ull << st;
            C.par = true;
        }
    }
    out.ncls = (int)cls.size();
    out.info.assign(out.ncls, 0);
    out.comp.assign((size_t)out.ncls * BOND_MAXC * 4, 0);
    out.flip.assign((size_t)out.ncls * n, 0);
    out.amp.assign((size_t)out.ncls * n * 8, 0.0);
    out.cid.assign((size_t)out.ncls * n * 4, -1);
    for (int c = 0; c < out.ncls; ++c) {
        const Cls& C = cls[c];
        out.info[c] = (int32_t)C.shifts.size() | (C.par ? 1 << 8 : 0);
        for (size_t k = 0; k < C.shifts.size(); ++k) {
            out.comp[((size_t)c * BOND_MAXC + k) * 4 + 0] = (uint64_t)C.shifts[k];
            out.comp[((size_t)c * BOND_MAXC + k) * 4 + 1] = C.A[k];
            out.comp[((size_t)c * BOND_MAXC + k) * 4 + 2] = C.P[k];
        }
        for (int i = 0; i < n; ++i) {
            if (C.partner[i] < 0) continue;
            out.flip[(size_t)c * n + i] = (1ull << i) | (1ull << C.partner[i]);
            for (int e = 0; e < 8; ++e) out.amp[((size_t)c * n + i) * 8 + e] = C.amp[i][e];
            for (int v = 0; v < 4; ++v) out.cid[((size_t)c * n + i) * 4 + v] = C.cid[i][v];
        }
    }
    return true;
}

// Build the shared-memory image of the term, phase and group tables for one (precision, direction,
// mode) and the kernel parameter template.
void build_blob(edgpu_op_s* op, int prec, int dir, int mode) {
    Blob& B = op->blob[prec][dir][mode];
    if (B.ready) return;
    const Space& s = *op->space;
    const bool w32 = s.w32;
    const size_t wsz = w32 ? 4 : 8;
    const size_t vsz = prec == EDGPU_FP64 ? 16 : 8;
    const size_t rsz = prec == EDGPU_FP64 ? 8 : 4;
    const Group& g = s.group;

    // term split (keeps the reference's term order inside each class)
    std::vector<int> diag, offd;
    for (int t = 0; t < op->T; ++t) {
        const uint64_t r = dir ? op->cols[t] : op->rows[t];
        const uint64_t c = dir ? op->rows[t] : op->cols[t];
        (r == c ? diag : offd).push_back(t);
    }
    const int T_o = (int)offd.size(), T_d = (int)diag.size();
    require(T_o < 65536, EDGPU_ERR_ARG, "too many off-diagonal terms (max 65535)");

    // divisors of G for the orbit-normalisation table
    std::vector<int> divs;
    for (int d = 1; d <= g.G; ++d)
        if (g.G % d == 0) divs.push_back(d);
    const int nd = (int)divs.size();

    int nchunks = 0;
    std::vector<unsigned long long> keep, lut;
    if (g.kind == GK_TORUS) keep = torus_keep_masks(g, s.lay.nbits);
    if (g.kind == GK_GENERIC) lut = generic_luts(g, s.lay, &nchunks);

    size_t off = 0;
    auto alloc = [&](size_t bytes) {
        const size_t o = off;
        off = align16(off + bytes);
        return (int)o;
    };
    auto amp_of = [&](int t, bool unit_only, double& re, double& im) {
        double a = op->unit[2 * t], b = op->unit[2 * t + 1];
        if (!unit_only) {
            const double c = op->coupl[op->cid[t]];
            a *= c;
            b *= c;
        }
        re = a;
        im = dir ? -b : b;   // adjoint: conj(amplitude) (pure_operator.jl adjoint)
    };
    HxParams p{};
    // One host image: group tables, the pair-flip schedule's bond classes, the torus row table, then
    // the term records.  Two device images are cut from it: the pair-flip image (everything before the
    // term records) and the term image (everything but the bond classes, later offsets moved down).
    p.o_ph = alloc(g.den * vsz);
    p.o_num = alloc(g.G * 4);
    p.o_ratio = alloc(nd * nd * rsz);
    p.o_keep = alloc(keep.size() * wsz);
    p.o_keep32 = alloc(keep.size() * 4);
    // permutation tables of a large general group stay in global memory (read through L1/L2) so
    // that the rest of the image fits in shared memory
    const bool lut_global = lut.size() * wsz > GENERIC_SMEM_LUT;
    p.o_lut = lut_global ? -1 : alloc(lut.size() * wsz);
    p.lut_g = nullptr;
    p.o_flip = alloc((g.kind == GK_GENERIC ? g.G : 0) * wsz);
    // torus row table: smallest rotation of every row value and the rotation steps reaching it
    const int rowbits = g.L1 * g.w;
    const bool use_rlut = g.kind == GK_TORUS && g.L2 >= 2 && g.L2 <= TORUS_MAXR && rowbits <= 10 && g.L1 <= 16;
    const bool use_pair = use_rlut && rowbits <= 6;
    const int lut_bits = use_pair ? 2 * rowbits : rowbits;
    p.rlut_pair = use_pair ? 1 : 0;
    BondClasses bc, bcu;   // bond classes with the coupled amplitudes; (gradient mode) with the unit ones
    bool grad_pair = false;  // gradient mode: the pair-flip gradient kernel applies
    struct DiagPair { int i, j, cid; double u[4][2]; };
    std::vector<DiagPair> dpairs;   // gradient mode: the diagonal records by site pair (below)
    int n_pdb = -1;
    if (mode == 0 || dir == 0) {
        std::vector<uint64_t> bm, br, bf;
        std::vector<double> ba, bu;
        std::vector<int32_t> bc_id;
        for (int t : offd) {
            const uint64_t r = dir ? op->cols[t] : op->rows[t];
            const uint64_t c = dir ? op->rows[t] : op->cols[t];
            bm.push_back(op->masks[t]);
            br.push_back(r);
            bf.push_back(r ^ c);
            double re, im;
            amp_of(t, false, re, im);
            ba.push_back(re);
            ba.push_back(im);
            amp_of(t, true, re, im);
            bu.push_back(re);
            bu.push_back(im);
            bc_id.push_back(op->cid[t]);
        }
        if (!build_bond_classes(s.lay, bm, br, bf, ba, bc, &bc_id)) bc = BondClasses();
        if (mode == 1 && bc.ncls > 0 && bc.cid_ok) {
            // the unit-coupling amplitudes of the same classes (the structure depends only on the terms'
            // masks and patterns)
            grad_pair = build_bond_classes(s.lay, bm, br, bf, bu, bcu) && bcu.ncls == bc.ncls;
        }
        // the diagonal records by site pair: when every record's mask has at most two bits, the records of
        // one (pair, coupling) become one entry with a unit amplitude per pattern of the pair's two bits
        // (a one-bit mask is the pair (i, i), patterns 0 and 3; an empty mask adds to both), so that the
        // gradient kernel looks up one value per entry and row instead of testing every record
        if (grad_pair) {
            std::map<std::tuple<int, int, int>, int> at;
            bool ok = true;
            for (int k = 0; k < T_d && ok; ++k) {
                const int t = diag[k];
                const uint64_t m = op->masks[t];
                const uint64_t r = dir ? op->cols[t] : op->rows[t];
                const int pc = __builtin_popcountll(m);
                if (pc > 2) {
                    ok = false;
                    break;
                }
                const int i = pc ? __builtin_ctzll(m) : 0;
                const int j = pc == 2 ? 63 - __builtin_clzll(m) : i;
                const auto key = std::make_tuple(i, j, op->cid[t]);
                auto it = at.find(key);
                if (it == at.end()) {
                    it = at.emplace(key, (int)dpairs.size()).first;
                    DiagPair d{};
                    d.i = i;
                    d.j = j;
                    d.cid = op->cid[t];
                    dpairs.push_back(d);
                }
                double v[2];
                amp_of(t, true, v[0], v[1]);
                DiagPair& d = dpairs[it->second];
                for (int pat = 0; pat < 4; ++pat) {
                    const int bi = pat & 1, bj = pat >> 1;
                    if (pc == 1 && bi != bj) continue;   // pattern of the pair (i, i)
                    const bool match = pc == 0 || (((r >> i) & 1) == (uint64_t)bi && ((r >> j) & 1) == (uint64_t)bj);
                    if (match) {
                        d.u[pat][0] += v[0];
                        d.u[pat][1] += v[1];
                    }
                }
            }
            if (!ok) dpairs.clear();
            else n_pdb = (int)dpairs.size();
        }
        // keep the pair-flip kernel's shared memory within 48 KB (five or more blocks per SM)
        size_t bond_bytes = (size_t)bc.ncls * (BOND_MAXC * 4 * wsz + 16 + s.lay.nbits * (wsz + 4 * vsz));
        if (grad_pair)
            bond_bytes += (size_t)bc.ncls * s.lay.nbits * 4 * (vsz + 4) +
                          (n_pdb >= 0 ? (size_t)n_pdb * (4 + 4 * vsz) : (size_t)T_d * (2 * wsz + vsz + 4));
        const size_t rlut_bytes = use_rlut ? ((size_t)1 << lut_bits) * 4 : 0;
        if (off + bond_bytes + rlut_bytes > 48 * 1024) {
            bc = BondClasses();
            grad_pair = false;
        }
        if (mode == 1 && !grad_pair) bc = BondClasses();
    }
    const int n_b = s.lay.nbits;
    p.bond_ncls = bc.ncls;
    p.bond_real = bc.real ? 1 : 0;
    p.o_bcomp = alloc((size_t)bc.ncls * BOND_MAXC * 4 * wsz);
    p.o_binfo = alloc((size_t)bc.ncls * 4);
    p.o_bflip = alloc((size_t)bc.ncls * n_b * wsz);
    p.o_bamp = alloc((size_t)bc.ncls * n_b * 4 * vsz);
    // gradient mode of the pair-flip kernel: unit amplitudes and coupling ids of the slots, and a copy
    // of the diagonal term records (mask, row, unit amplitude, coupling id)
    p.o_bunit = p.o_bcid = p.o_pdm = p.o_pdr = p.o_pdu = p.o_pdc = -1;
    p.o_pdb = p.o_pdv = -1;
    p.n_pdb = grad_pair ? n_pdb : -1;
    p.bunit_real = 0;
    if (grad_pair) {
        p.o_bunit = alloc((size_t)bc.ncls * n_b * 4 * vsz);
        p.o_bcid = alloc((size_t)bc.ncls * n_b * 4 * 4);
        if (p.n_pdb >= 0) {
            p.o_pdb = alloc(dpairs.size() * 4);
            p.o_pdv = alloc(dpairs.size() * 4 * vsz);
        } else {
            p.o_pdm = alloc((size_t)T_d * wsz);
            p.o_pdr = alloc((size_t)T_d * wsz);
            p.o_pdu = alloc((size_t)T_d * vsz);
            p.o_pdc = alloc((size_t)T_d * 4);
        }
    }
    // the prefix a mapped pair-flip launch copies ends here; the torus row table follows (needed by
    // canonicalisation only)
    const size_t bond_prefix = align16(off);
    p.o_rlut = use_rlut ? alloc(((size_t)1 << lut_bits) * 4) : -1;
    const size_t bond_prefix_canon = align16(off);
    p.o_om = alloc(T_o * 4 * wsz);   // packed records (mask, row, row ^ col, 0)
    p.o_or = p.o_om;
    p.o_of = p.o_om;
    p.o_oa = alloc(T_o * vsz);
    p.o_ou = alloc(mode ? T_o * vsz : 0);
    p.o_oc = alloc(mode ? T_o * 4 : 0);
    p.o_dm = alloc(mode ? T_d * wsz : 0);
    p.o_dr = alloc(mode ? T_d * wsz : 0);
    p.o_da = alloc(mode ? T_d * 16 : 0);
    p.o_du = alloc(mode ? T_d * 16 : 0);
    p.o_dc = alloc(mode ? T_d * 4 : 0);
    const size_t blob_bytes = align16(off);
    std::vector<unsigned char> h(blob_bytes, 0);
    auto putw = [&](int o, size_t i, uint64_t v) {
        if (w32) { uint32_t u = (uint32_t)v; memcpy(&h[o + i * 4], &u, 4); }
        else memcpy(&h[o + i * 8], &v, 8);
    };
    auto putv = [&](int o, size_t i, double re, double im) {
        if (prec == EDGPU_FP64) { double v[2] = {re, im}; memcpy(&h[o + i * 16], v, 16); }
        else { float v[2] = {(float)re, (float)im}; memcpy(&h[o + i * 8], v, 8); }
    };
    for (int k = 0; k < T_o; ++k) {
        const int t = offd[k];
        const uint64_t r = dir ? op->cols[t] : op->rows[t];
        const uint64_t c = dir ? op->rows[t] : op->cols[t];
        putw(p.o_om, 4 * k, op->masks[t]);
        putw(p.o_om, 4 * k + 1, r);
        putw(p.o_om, 4 * k + 2, r ^ c);
        double re, im;
        amp_of(t, false, re, im);
        putv(p.o_oa, k, re, im);
        if (mode) {
            amp_of(t, true, re, im);
            putv(p.o_ou, k, re, im);
            memcpy(&h[p.o_oc + k * 4], &op->cid[t], 4);
        }
    }
    std::vector<uint64_t> dg_mask(T_d), dg_row(T_d);
    std::vector<double> dg_amp(2 * (size_t)T_d);
    for (int k = 0; k < T_d; ++k) {
        const int t = diag[k];
        const uint64_t r = dir ? op->cols[t] : op->rows[t];
        double v[2];
        amp_of(t, false, v[0], v[1]);
        dg_mask[k] = op->masks[t];
        dg_row[k] = r;
        dg_amp[2 * k] = v[0];
        dg_amp[2 * k + 1] = v[1];
        if (mode) {
            putw(p.o_dm, k, op->masks[t]);
            putw(p.o_dr, k, r);
            memcpy(&h[p.o_da + k * 16], v, 16);
            amp_of(t, true, v[0], v[1]);
            memcpy(&h[p.o_du + k * 16], v, 16);
            memcpy(&h[p.o_dc + k * 4], &op->cid[t], 4);
        }
    }
    for (int j = 0; j < g.den; ++j) {
        const double ang = 2.0 * M_PI * (double)j / (double)g.den;
        putv(p.o_ph, j, std::cos(ang), std::sin(ang));
    }
    memcpy(&h[p.o_num], g.num.data(), g.G * 4);
    for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j) {
            const double f = std::sqrt((double)divs[j] / (double)divs[i]);   // sqrt(|O_r| / |O_c|)
            if (prec == EDGPU_FP64) memcpy(&h[p.o_ratio + (i * nd + j) * 8], &f, 8);
            else { float ff = (float)f; memcpy(&h[p.o_ratio + (i * nd + j) * 4], &ff, 4); }
        }
    for (size_t i = 0; i < keep.size(); ++i) putw(p.o_keep, i, keep[i]);
    for (size_t i = 0; i < keep.size(); ++i) {
        const uint32_t k32 = (uint32_t)keep[i];
        memcpy(&h[p.o_keep32 + i * 4], &k32, 4);
    }
    if (use_rlut) {
        // smallest rotation of a row (or of a pair of rows: top row << rowbits | the row below it,
        // both rotated by the same a) and the rotations a reaching it
        const uint32_t rmask = (1u << rowbits) - 1u;
        auto rot = [&](uint32_t v, int a) {
            const int sh = a * g.w;
            return sh ? (((v << sh) | (v >> (rowbits - sh))) & rmask) : v;
        };
        const uint32_t n_entries = 1u << lut_bits;
        for (uint32_t v = 0; v < n_entries; ++v) {
            uint32_t best = 0xffffffffu, steps = 0;
            for (int a = 0; a < g.L1; ++a) {
                const uint32_t r = use_pair ? ((rot(v >> rowbits, a) << rowbits) | rot(v & rmask, a)) : rot(v, a);
                if (r < best) {
                    best = r;
                    steps = 0;
                }
                if (r == best) steps |= 1u << a;
            }
            // pair table: value in the high half so that one min finds the smallest pair
            const uint32_t e = use_pair ? ((best << 16) | steps) : (best | (steps << 16));
            memcpy(&h[p.o_rlut + v * 4], &e, 4);
        }
    }
    if (!lut_global)
        for (size_t i = 0; i < lut.size(); ++i) putw(p.o_lut, i, lut[i]);
    if (g.kind == GK_GENERIC)
        for (int e = 0; e < g.G; ++e) putw(p.o_flip, e, e < (int)g.flips.size() ? g.flips[e] : 0ull);
    if (bc.ncls > 0) {
        for (size_t i = 0; i < bc.comp.size(); ++i) putw(p.o_bcomp, i, bc.comp[i]);
        memcpy(&h[p.o_binfo], bc.info.data(), bc.info.size() * 4);
        for (size_t i = 0; i < bc.flip.size(); ++i) putw(p.o_bflip, i, bc.flip[i]);
        for (size_t i = 0; i < bc.flip.size() * 4; ++i) putv(p.o_bamp, i, bc.amp[2 * i], bc.amp[2 * i + 1]);
    }
    if (grad_pair) {
        p.bunit_real = bcu.real ? 1 : 0;
        for (size_t i = 0; i < bcu.flip.size() * 4; ++i) putv(p.o_bunit, i, bcu.amp[2 * i], bcu.amp[2 * i + 1]);
        memcpy(&h[p.o_bcid], bc.cid.data(), bc.cid.size() * 4);
        for (int k = 0; k < T_d && p.n_pdb < 0; ++k) {
            const int t = diag[k];
            const uint64_t r = dir ? op->cols[t] : op->rows[t];
            putw(p.o_pdm, k, op->masks[t]);
            putw(p.o_pdr, k, r);
            double v[2];
            amp_of(t, true, v[0], v[1]);
            putv(p.o_pdu, k, v[0], v[1]);
            memcpy(&h[p.o_pdc + k * 4], &op->cid[t], 4);
        }
        for (size_t k = 0; k < dpairs.size(); ++k) {
            const int32_t e = dpairs[k].i | (dpairs[k].j << 8) | (dpairs[k].cid << 16);
            memcpy(&h[p.o_pdb + k * 4], &e, 4);
            for (int pat = 0; pat < 4; ++pat) putv(p.o_pdv, k * 4 + pat, dpairs[k].u[pat][0], dpairs[k].u[pat][1]);
        }
    }

    // cut the pair-flip image and the term image
    const size_t bstart = (size_t)p.o_bcomp, bshift = bond_prefix - bstart;
    std::vector<unsigned char> hp(h.begin(), h.begin() + bond_prefix_canon);
    HxParams pp = p;
    std::vector<unsigned char> ht(h.begin(), h.begin() + bstart);
    ht.insert(ht.end(), h.begin() + bond_prefix, h.end());
    for (int* o : {&p.o_rlut, &p.o_om, &p.o_or, &p.o_of, &p.o_oa, &p.o_ou, &p.o_oc, &p.o_dm, &p.o_dr, &p.o_da,
                   &p.o_du, &p.o_dc})
        if (*o >= (int)bond_prefix) *o -= (int)bshift;
    const size_t term_start = bond_prefix_canon - bshift;   // term records in the term image
    h.swap(ht);
    const size_t blob_bytes_t = h.size();

    size_t tot = blob_bytes_t;
    p.o_grad = (int)tot;
    tot = align16(tot + (mode ? op->n_coupl * 8 : 0));
    p.warp_base = (int)tot;
    tot += (size_t)(HX_THREADS / 32) * hx_warp_bytes(w32);
    require(tot <= 227 * 1024, EDGPU_ERR_ARG,
            "operator tables do not fit in shared memory (" + std::to_string(tot) + " bytes)");

    // device buffers are reused when they are large enough (a rebuild after a change of coupling
    // values has the same layout and allocates nothing)
    auto ensure = [](void*& d, size_t& cap, size_t bytes) {
        bytes = std::max<size_t>(bytes, 16);
        if (d && cap >= bytes) return;
        if (d) cudaFree(d);
        d = nullptr;
        cap = 0;
        EDGPU_CUDA(cudaMalloc(&d, bytes));
        cap = bytes;
    };
    if (!mode) {
        ensure(B.d_diag, B.cap_diag, (size_t)std::max<int64_t>(s.dim, 1) * vsz);
        op->diag_scratch.ensure((size_t)std::max(T_d, 1) * 4);
        compute_diagonal(s, T_d, dg_mask.data(), dg_row.data(), dg_amp.data(),
                         prec == EDGPU_FP64 ? (double*)B.d_diag : nullptr,
                         prec == EDGPU_FP64 ? nullptr : (float*)B.d_diag, op->diag_scratch.p, op->hs.stream());
    }
    ensure(B.d, B.cap_d, blob_bytes_t);
    EDGPU_CUDA(cudaMemcpy(B.d, h.data(), blob_bytes_t, cudaMemcpyHostToDevice));
    if (lut_global) {
        std::vector<unsigned char> lh(lut.size() * wsz);
        for (size_t i = 0; i < lut.size(); ++i) {
            if (w32) {
                const uint32_t u = (uint32_t)lut[i];
                memcpy(&lh[i * 4], &u, 4);
            } else {
                memcpy(&lh[i * 8], &lut[i], 8);
            }
        }
        ensure(B.d_lut, B.cap_lut, lh.size());
        EDGPU_CUDA(cudaMemcpy(B.d_lut, lh.data(), lh.size(), cudaMemcpyHostToDevice));
        p.lut_g = B.d_lut;
    }
    if (bc.ncls > 0) {
        ensure(B.d_pair, B.cap_pair, hp.size());
        EDGPU_CUDA(cudaMemcpy(B.d_pair, hp.data(), hp.size(), cudaMemcpyHostToDevice));
    } else if (B.d_pair) {
        cudaFree(B.d_pair);
        B.d_pair = nullptr;
        B.cap_pair = 0;
    }
    B.pair_host = hp;
    p.blob = B.d;
    p.blob_words16 = (int)(blob_bytes_t / 16);
    p.T_o = T_o;
    p.T_d = T_d;
    p.G = g.G;
    p.den = g.den;
    p.nd = nd;
    p.L1 = g.L1;
    p.l1inv = (65536u + (unsigned)g.L1 - 1u) / (unsigned)g.L1;
    p.L2 = g.L2;
    p.w = g.w;
    p.rowbits = g.L1 * g.w;
    p.nbits = s.lay.nbits;
    p.nchunks = nchunks;
    p.full = (s.lay.nbits >= 64) ? ~0ull : ((1ull << s.lay.nbits) - 1ull);
    p.keys = s.d_keys;
    p.n_rows = s.dim;
    p.n_coupl = op->n_coupl;
    p.sb = s.sb;
    p.want_arg = g.den > 1 ? 1 : 0;
    p.ds = dir_search_of(s);
    p.diag = B.d_diag;
    int gk = g.kind;
    p.pb = 0;
    if (gk == GK_TORUS && g.L2 == 1 && w32 && s.lay.nbits <= 31) {
        gk = GK_RING;
        int pb = 0;
        while ((1 << pb) < g.L1) ++pb;
        p.pb = (s.lay.nbits + pb <= 32) ? pb : 0;
    }
    B.gk = gk;
    B.tmpl = p;
    // the pair-flip template: the term template with the pair image's offsets
    B.tmpl_pair = p;
    B.tmpl_pair.blob = B.d_pair;
    B.tmpl_pair.o_rlut = pp.o_rlut;
    B.tmpl_pair.o_bcomp = pp.o_bcomp;
    B.tmpl_pair.o_binfo = pp.o_binfo;
    B.tmpl_pair.o_bflip = pp.o_bflip;
    B.tmpl_pair.o_bamp = pp.o_bamp;
    B.smem = tot;
    B.smem_bond = std::max<size_t>(bond_prefix, 16);
    B.smem_bond_canon = std::max<size_t>(bond_prefix_canon, 16);
    B.term_start = term_start;
    B.bond_end = bond_prefix;
    B.max_blocks_bond[0][0] = B.max_blocks_bond[0][1] = B.max_blocks_bond[1][0] = B.max_blocks_bond[1][1] = 0;
    for (auto& a : B.max_blocks_table) a[0] = a[1] = a[2] = 0;
    B.max_blocks_pgrad[0] = B.max_blocks_pgrad[1] = 0;
    const int per_sm = std::max(1, hx_max_blocks_per_sm(w32, gk, prec, mode, tot));
    B.max_blocks = per_sm * std::max(1, g_sm_count);
    if (!mode) {
        B.smem_rows = std::max<size_t>(p.warp_base, 16);
        const int per_sm_rows = std::max(1, w32 ? hx_rows_occupancy_w32(gk, prec, B.smem_rows)
                                                : hx_rows_occupancy_w64(gk, prec, B.smem_rows));
        B.max_blocks_rows = per_sm_rows * std::max(1, g_sm_count);
    }
    B.ready = true;
}

void invalidate_blobs(edgpu_op_s* op) {
    ++op->gen;
    for (auto& a : op->blob)
        for (auto& b : a)
            for (auto& c : b) {
                if (c.d) cudaFree(c.d);
                if (c.d_diag) cudaFree(c.d_diag);
                if (c.d_pair) cudaFree(c.d_pair);
                if (c.d_lut) cudaFree(c.d_lut);
                c.d = nullptr;
                c.d_diag = nullptr;
                c.d_pair = nullptr;
                c.d_lut = nullptr;
                c.cap_d = c.cap_pair = c.cap_diag = c.cap_lut = 0;
                c.ready = false;
            }
}

// Coefficient tables of the slab product (FP32 and FP64) for the current coupling values, written
// into the tables' existing buffers: id = ((amplitude id x den + character index) x nd + orbit-size
// index of the row) x nd + orbit-size index of the column, coefficient = J_c u_a chi sqrt(|O_c| / |O_r|)
// as the one-pass product forms it (hx_bond.cuh), here in FP64 and rounded once.  A scaled table's
// id is amplitude id x den + character index and its coefficient J_c u_a chi: the ratio's factors
// sqrt(|O_c|) and 1 / sqrt(|O_r|) go to x and to the row's result.
void slab_refresh_lut(edgpu_op_s* op) {
    auto& S = op->slab;
    if (!S.tab) return;
    const int na = (int)S.amp_cid.size();
    bool real = S.den == 1;
    for (int a = 0; a < na && real; ++a)
        if (S.amp_unit[2 * a + 1] != 0.0) real = false;
    std::vector<float> h((size_t)S.n_ids * 2, 0.f);
    std::vector<double> h64((size_t)S.n_ids * 2, 0.0);
    for (int id = 0; id < S.n_ids; ++id) {
        int rest = id, sxc = 0, sxr = 0;
        if (!S.scaled) {
            sxc = rest % S.nd;
            rest /= S.nd;
            sxr = rest % S.nd;
            rest /= S.nd;
        }
        const int ph = rest % S.den;
        const int a = rest / S.den;
        if (a >= na) continue;
        const double J = S.amp_cid[a] >= 0 ? op->coupl[S.amp_cid[a]] : 0.0;
        const double ur = S.amp_unit[2 * a] * J, ui = S.amp_unit[2 * a + 1] * J;
        const double ang = 2.0 * M_PI * (double)ph / (double)S.den;
        const double cr = std::cos(ang), ci = std::sin(ang);
        // the orbit-size ratio; on a scaled table it is applied to x and y instead
        const double f = S.scaled ? 1.0 : std::sqrt((double)S.divs[sxc] / (double)S.divs[sxr]);
        const double re = (ur * cr - ui * ci) * f, im = (ur * ci + ui * cr) * f;
        if (real) {
            h[id] = (float)re;
            h64[id] = re;
        } else {
            h[2 * (size_t)id] = (float)re;
            h[2 * (size_t)id + 1] = (float)im;
            h64[2 * (size_t)id] = re;
            h64[2 * (size_t)id + 1] = im;
        }
    }
    S.lut_real = real ? 1 : 0;
    // registers for a few real coefficients, one copy per bank group for a small complex table (its
    // lookups then never conflict), else one shared-memory copy
    S.lut_mode = (real && S.n_ids <= SLAB_REG_LUT) ? 2 : (!real && (size_t)S.n_ids * 128 <= (size_t)SLAB_REP_BYTES) ? 1 : 0;
    EDGPU_CUDA(cudaMemcpy(S.lut.p, h.data(), (size_t)S.n_ids * (real ? 1 : 2) * sizeof(float), cudaMemcpyHostToDevice));
    EDGPU_CUDA(cudaMemcpy(S.lut64.p, h64.data(), (size_t)S.n_ids * (real ? 1 : 2) * sizeof(double),
                          cudaMemcpyHostToDevice));
}

// New coupling values: every table built so far is rewritten in place (same layout, same device
// buffers: nothing is allocated or freed), after the device has finished the work that may still
// read the old values.  Tables not built yet are built on first use, as before.
void refresh_blobs(edgpu_op_s* op) {
    ++op->gen;
    bool any = false;
    for (auto& a : op->blob)
        for (auto& b : a)
            for (auto& c : b) any = any || c.ready;
    if (!any && !op->slab.tab) return;
    EDGPU_CUDA(cudaDeviceSynchronize());
    for (int prec = 0; prec < 2; ++prec)
        for (int dir = 0; dir < 2; ++dir)
            for (int mode = 0; mode < 2; ++mode) {
                Blob& B = op->blob[prec][dir][mode];
                if (!B.ready) continue;
                B.ready = false;
                build_blob(op, prec, dir, mode);
            }
    slab_refresh_lut(op);
}

int blocks_for(const Blob& B, long long n_rows, int rows_per_tile) {
    const long long tiles = (n_rows + rows_per_tile - 1) / rows_per_tile;
    const long long need = (tiles + HX_THREADS / 32 - 1) / (HX_THREADS / 32);
    return (int)std::max<long long>(1, std::min<long long>(need, B.max_blocks));
}

// Colex rank parameters of a mapped space (the chunk table and the parent sector's popcount).
void set_map_params(HxParams& p, const Space& sp) {
    p.rank_tab = sp.d_rank;
    p.rank_wide = sp.rank_wide;
    p.rank_k = sp.lay.popcount;
    p.rank_nc = (sp.lay.nbits + RANK_CHUNK - 1) / RANK_CHUNK;
    p.rank_split = sp.rank_split;
}

// Whether a product launch (mode 0 = product) goes through the column-slab table.
bool slab_active(const edgpu_op_s* op, int prec, int dir, int mode, int rows) {
    return mode == 0 && dir == 0 && op->slab.tab && op->slab_use[prec] && op->pair_allowed && op->pair_use[prec] &&
           rows < 0;
}

// The column-slab product: one launch per slab (hxslab.cu); the last pass adds the diagonal term and
// writes complex128 to y_c128 when given.  With ready != null, pass q first waits for ready[q] (the
// event after which slab q of x, and for the last pass all of x, is in place).  On a scaled table x
// is the caller's unscaled vector, unless pre_scaled: the caller has written the scaled x to the
// table's buffer (slab q by the event ready[q]).  Otherwise slab q of x is scaled into that buffer on
// the handle's second stream while the earlier passes run.
void launch_slab_passes(edgpu_op_s* op, int prec, const Blob& B, const void* x, void* y, int accumulate,
                        void* y_c128, int acc_c128, cudaStream_t st, const cudaEvent_t* ready,
                        bool pre_scaled = false, int row_blocks = 1) {
    auto& S = op->slab;
    const size_t esz = prec == EDGPU_FP64 ? 16 : 8;
    const void* scale = prec == EDGPU_FP64 ? (const void*)S.sc64.p : (const void*)S.sc32.p;
    if (S.scaled) {
        if (!pre_scaled) {
            const int64_t n = B.tmpl.n_rows;
            if (S.n_pass == 1) {
                launch_slab_xscale(prec, x, S.cls, scale, S.xsc.p, 0, n, st);
                ready = nullptr;
            } else {
                op->ensure_slab_events(S.n_pass);
                EDGPU_CUDA(cudaEventRecord(op->aux_fork, st));
                EDGPU_CUDA(cudaStreamWaitEvent(op->aux_st, op->aux_fork, 0));
                for (int q = 0; q < S.n_pass; ++q) {
                    const int64_t c0 = (int64_t)q * S.wc, c1 = std::min<int64_t>(n, c0 + S.wc);
                    launch_slab_xscale(prec, x, S.cls, scale, S.xsc.p, c0, c1, op->aux_st);
                    EDGPU_CUDA(cudaEventRecord(op->slab_ready[q], op->aux_st));
                }
                ready = op->slab_ready.data();
            }
        }
        x = S.xsc.p;
    }
    SlabRun r{};
    r.x = x;
    r.y = y;
    r.diag = B.d_diag;
    r.lut = prec == EDGPU_FP64 ? (const void*)S.lut64.p : (const void*)S.lut.p;
    r.n_lut = S.n_ids;
    r.lut_real = S.lut_real;
    r.lut_mode = S.lut_mode;
    r.scaled = S.scaled;
    r.cls = S.cls;
    r.scale = scale;
    r.nd = S.nd;
    r.n_rows = B.tmpl.n_rows;
    r.n_tiles = (r.n_rows + 31) / 32;
    r.colbits = S.colbits;
    r.colmask = (unsigned)((1ull << S.colbits) - 1ull);
    r.y_c128 = y_c128;
    r.acc_c128 = acc_c128;
    r.accumulate = y_c128 ? 0 : accumulate;
    r.hints = op->slab_hint[prec];
    const long long n_tiles = r.n_tiles;
    auto set_pass = [&](int q) {
        r.cnt = S.counts + (size_t)q * r.n_rows;
        r.off = S.off + (size_t)q * n_tiles;
        r.tab = S.tab + S.base[q];
        r.xs = (const char*)x + (size_t)q * S.wc * esz;
        r.first = q == 0;
        r.last = q == S.n_pass - 1;
    };
    if (row_blocks > 1 && S.n_pass > 1 && n_tiles >= row_blocks) {
        // rows in blocks: a block's passes before the last run on st with one block slot per SM left
        // free; its last pass (which writes y, e.g. to a host buffer) runs on the handle's block stream
        // with one block per SM, beside the next block's passes
        op->ensure_block_events(row_blocks);
        const long long per = (n_tiles + row_blocks - 1) / row_blocks;
        for (int b = 0; b < row_blocks; ++b) {
            const long long t0 = (long long)b * per, t1 = std::min(n_tiles, t0 + per);
            if (t0 >= t1) break;
            r.tile0 = t0;
            r.n_tiles = t1 - t0;
            r.blocks_per_sm = -1;
            for (int q = 0; q + 1 < S.n_pass; ++q) {
                if (ready && b == 0) EDGPU_CUDA(cudaStreamWaitEvent(st, ready[q], 0));
                set_pass(q);
                hx_slab_launch(prec, r, st);
            }
            EDGPU_CUDA(cudaEventRecord(op->blk_ev[b], st));
            EDGPU_CUDA(cudaStreamWaitEvent(op->blk_st, op->blk_ev[b], 0));
            if (ready && b == 0) EDGPU_CUDA(cudaStreamWaitEvent(op->blk_st, ready[S.n_pass - 1], 0));
            r.blocks_per_sm = 1;
            set_pass(S.n_pass - 1);
            hx_slab_launch(prec, r, op->blk_st);
        }
        EDGPU_CUDA(cudaEventRecord(op->blk_ev[row_blocks], op->blk_st));
        EDGPU_CUDA(cudaStreamWaitEvent(st, op->blk_ev[row_blocks], 0));
        return;
    }
    for (int q = 0; q < S.n_pass; ++q) {
        if (ready) EDGPU_CUDA(cudaStreamWaitEvent(st, ready[q], 0));
        set_pass(q);
        hx_slab_launch(prec, r, st);
    }
}

// Row blocks of a host-buffer slab product (launch_slab_passes): EDGPU_SLAB_ROW_BLOCKS when set (1 to
// 64); else 2 for mixed precision on sectors of 2^22 rows or more with at least 4 passes (on 6x6 k=0,
// 252M rows: 101.8 -> 96.9 ms per H x with pinned complex128 buffers; 4 and 8 blocks gain no more,
// and the FP64 product is slower in blocks), 1 otherwise.
int slab_row_blocks(const edgpu_op_s* op, int prec, int64_t n) {
    const char* v = std::getenv("EDGPU_SLAB_ROW_BLOCKS");
    if (v && *v) {
        const int k = std::atoi(v);
        if (k >= 1 && k <= 64) return k;
    }
    return (prec == EDGPU_MIXED && n >= ((int64_t)1 << 22) && op->slab.n_pass >= 4) ? 2 : 1;
}

// Shared memory of the pair-flip gradient kernel's per-thread coupling accumulators (the product's
// real type: FP32 in mixed precision, FP64 in FP64).
static size_t pair_grad_acc_bytes(const edgpu_op_s* op, int prec) {
    return (size_t)op->n_coupl * HX_THREADS * (prec == EDGPU_MIXED ? 4 : 8);
}

// y_c128 (mixed precision, product mode): when the launch goes through the pair-flip kernel, it writes
// y as complex128 to y_c128 (adding the old value there when acc_c128) instead of complex64 to y, and
// *wrote_c128 is set; otherwise y is written as usual.
// max_blocks_cap > 0 limits the grid (the gradient's per-block partial sums must fit a caller's buffer).
void launch_product(edgpu_op_s* op, int prec, int dir, int mode, const void* x, void* y, int accumulate,
                    const void* gy, double* grad_partial, cudaStream_t st, int* blocks_used = nullptr,
                    int rows_override = 0, void* y_c128 = nullptr, int acc_c128 = 0, bool* wrote_c128 = nullptr,
                    int max_blocks_cap = 0) {
    if (wrote_c128) *wrote_c128 = false;
    // the space's parent-state map is read below and by the launched kernel: hold the space's lock
    // while enqueueing so that the map is not freed in between
    SpaceLock space_lk(op->space->hs.mu);
    build_blob(op, prec, dir, mode);
    Blob& B = op->blob[prec][dir][mode];
    HxParams p = B.tmpl;
    if (p.n_rows == 0) {
        if (blocks_used) *blocks_used = 0;
        return;
    }
    int rows = rows_override ? rows_override : (op->tuned_rows[prec] ? op->tuned_rows[prec] : (mode ? B.rows_per_tile : -1));
    const Space& sp = *op->space;
    if (mode == 0 && sp.d_map) {
        // parent-state map: targets are looked up, not canonicalised (row-per-lane schedule only)
        set_map_params(p, sp);
        p.map = sp.d_map;
        p.map_wide = sp.map_wide;
        p.map_cb = sp.map_cb;
        p.map_direct = sp.map_direct;
        if (rows > 0) rows = -1;
    }
    if (slab_active(op, prec, dir, mode, rows)) {
        launch_slab_passes(op, prec, B, x, y, accumulate, y_c128, acc_c128, st, nullptr);
        if (wrote_c128) *wrote_c128 = y_c128 != nullptr;
        if (blocks_used) *blocks_used = 0;
        return;
    }
    if (rows < 0 && mode == 0) {
        // row-per-lane strategy: -lpr lanes per row, one warp per 32/lpr consecutive rows
        p.lpr = -rows;
        p.rows_per_tile = 32 / p.lpr;
        p.x = x;
        p.y = y;
        p.gy = gy;
        p.grad_partial = grad_partial;
        p.accumulate = accumulate;
        const bool mapped = p.map != nullptr;
        const int gk = mapped ? GK_MAP : B.gk;
        if (p.bond_ncls > 0 && op->pair_allowed && op->pair_use[prec]) {
            // pair-flip schedule: matching pairs from bond classes (hx_bond.cuh); copies only the
            // blob's prefix up to the bond tables
            const bool table = op->d_tab && op->tab_use[prec];
            const size_t smem = (mapped || table) ? B.smem_bond : B.smem_bond_canon;
            if (y_c128 && prec == EDGPU_MIXED) {
                p.y_c128 = y_c128;
                p.accumulate = acc_c128;
                if (wrote_c128) *wrote_c128 = true;
            }
            p.blob = B.d_pair;
            p.o_rlut = B.tmpl_pair.o_rlut;
            p.o_bcomp = B.tmpl_pair.o_bcomp;
            p.o_binfo = B.tmpl_pair.o_binfo;
            p.o_bflip = B.tmpl_pair.o_bflip;
            p.o_bamp = B.tmpl_pair.o_bamp;
            p.blob_words16 = (int)(smem / 16);
            // targets per lane and step: 2; 4 with a map or a table; 8 with a table (one product launch)
            p.bond_nt = op->pair_nt[prec] == 8 ? (table ? 8 : 4) : op->pair_nt[prec] == 4 ? 4 : 2;
            if (!(mapped || table)) p.bond_nt = 2;
            const bool w32 = op->space->w32;
            if (table) {
                // the target table: one lane per row, entries streamed in the schedule's order
                p.lpr = 1;
                p.rows_per_tile = 32;
                p.tab = op->d_tab;
                p.tile_off = op->d_tile_off;
                p.tab_wide = op->tab_wide;
                p.tab_cb = op->tab_cb;
                p.bond_pf = op->tab_pf[prec];
                p.bond_uni = (op->tab_uni[prec] && p.bond_nt >= 4) ? 1 : 0;
                int& mt = B.max_blocks_table[p.bond_uni][p.bond_nt == 8 ? 2 : p.bond_nt == 4 ? 1 : 0];
                if (mt == 0)
                    mt = std::max(1, hx_table_occupancy(w32, prec, p.bond_nt, smem, p.bond_uni != 0)) *
                         std::max(1, g_sm_count);
                const long long warps = (p.n_rows + 31) / 32;
                const int blocks = (int)std::max<long long>(1, std::min<long long>((warps + HX_THREADS / 32 - 1) / (HX_THREADS / 32), mt));
                if (blocks_used) *blocks_used = blocks;
                hx_table_launch(w32, prec, p, blocks, smem, st);
                return;
            }
            int& mb = B.max_blocks_bond[mapped ? 1 : 0][p.bond_nt == 4 ? 1 : 0];
            if (mb == 0) {
                const int per_sm = std::max(1, w32 ? hx_bond_occupancy_w32(gk, prec, p.bond_nt, smem)
                                                   : hx_bond_occupancy_w64(gk, prec, p.bond_nt, smem));
                mb = per_sm * std::max(1, g_sm_count);
            }
            const long long warps = (p.n_rows + p.rows_per_tile - 1) / p.rows_per_tile;
            const int blocks = (int)std::max<long long>(1, std::min<long long>((warps + HX_THREADS / 32 - 1) / (HX_THREADS / 32), mb));
            if (blocks_used) *blocks_used = blocks;
            if (w32) hx_bond_launch_w32(gk, prec, p, blocks, smem, st);
            else hx_bond_launch_w64(gk, prec, p, blocks, smem, st);
            return;
        }
        if (mapped && B.max_blocks_map == 0) {
            const int per_sm = std::max(1, op->space->w32 ? hx_rows_occupancy_w32(GK_MAP, prec, B.smem_rows)
                                                           : hx_rows_occupancy_w64(GK_MAP, prec, B.smem_rows));
            B.max_blocks_map = per_sm * std::max(1, g_sm_count);
        }
        const long long warps = (p.n_rows + p.rows_per_tile - 1) / p.rows_per_tile;
        const int blocks = (int)std::max<long long>(1, std::min<long long>((warps + HX_THREADS / 32 - 1) / (HX_THREADS / 32),
                                                                          mapped ? B.max_blocks_map : B.max_blocks_rows));
        if (blocks_used) *blocks_used = blocks;
        if (op->space->w32) hx_rows_launch_w32(gk, prec, p, blocks, B.smem_rows, st);
        else hx_rows_launch_w64(gk, prec, p, blocks, B.smem_rows, st);
        return;
    }
    auto cap_blocks = [&](int b) { return max_blocks_cap > 0 ? std::max(1, std::min(b, max_blocks_cap)) : b; };
    if (mode == 1 && B.tmpl.o_bunit >= 0 && op->pair_allowed && (op->d_tab || sp.d_map)) {
        // gradient on the pair-flip schedule: targets from the target table (or the parent-state map),
        // per-thread FP64 coupling accumulators in shared memory after the pair-flip image
        const bool table = op->d_tab != nullptr;
        HxParams q = B.tmpl_pair;
        q.o_grad = (int)align16(B.smem_bond);
        const size_t gsmem = (size_t)q.o_grad + pair_grad_acc_bytes(op, prec);
        if (gsmem <= 200 * 1024) {
            build_blob(op, prec, dir, 0);   // the forward diagonal table
            q.diag = op->blob[prec][dir][0].d_diag;
            q.blob = B.d_pair;
            q.blob_words16 = (int)(B.smem_bond / 16);
            q.lpr = 1;
            q.rows_per_tile = 32;
            q.bond_nt = 4;
            q.bond_pf = 0;
            q.bond_uni = 0;
            q.x = x;
            q.y = y;
            q.gy = gy;
            q.grad_partial = grad_partial;
            q.accumulate = accumulate;
            if (table) {
                q.tab = op->d_tab;
                q.tile_off = op->d_tile_off;
                q.tab_wide = op->tab_wide;
                q.tab_cb = op->tab_cb;
            } else {
                set_map_params(q, sp);
                q.map = sp.d_map;
                q.map_wide = sp.map_wide;
                q.map_cb = sp.map_cb;
                q.map_direct = sp.map_direct;
            }
            int& mb = B.max_blocks_pgrad[table ? 1 : 0];
            if (mb == 0) mb = std::max(1, hx_bond_grad_occupancy(sp.w32, table, prec, gsmem)) * std::max(1, g_sm_count);
            const long long warps = (q.n_rows + 31) / 32;
            const int blocks = cap_blocks((int)std::max<long long>(1, std::min<long long>((warps + HX_THREADS / 32 - 1) / (HX_THREADS / 32), mb)));
            if (blocks_used) *blocks_used = blocks;
            hx_bond_grad_launch(sp.w32, table, prec, q, blocks, gsmem, st);
            return;
        }
    }
    if (mode == 1) {
        // gradient: the row-per-lane kernel with per-thread coupling accumulators when they fit in
        // shared memory (deterministic block sums, no atomics), else the queued kernel below
        const size_t gsmem = (size_t)p.o_grad + (size_t)op->n_coupl * HX_THREADS * 8;
        if (gsmem <= 200 * 1024) {
            build_blob(op, prec, dir, 0);   // the forward diagonal table
            p.diag = op->blob[prec][dir][0].d_diag;
            const int lpr = rows < 0 ? -rows : 1;
            p.lpr = lpr;
            p.rows_per_tile = 32 / lpr;
            p.x = x;
            p.y = y;
            p.gy = gy;
            p.grad_partial = grad_partial;
            p.accumulate = accumulate;
            if (B.max_blocks_grad == 0) {
                const int per_sm = std::max(1, op->space->w32 ? hx_rows_grad_occupancy_w32(B.gk, prec, gsmem)
                                                               : hx_rows_grad_occupancy_w64(B.gk, prec, gsmem));
                B.max_blocks_grad = per_sm * std::max(1, g_sm_count);
            }
            const long long warps = (p.n_rows + p.rows_per_tile - 1) / p.rows_per_tile;
            const int blocks = cap_blocks((int)std::max<long long>(
                1, std::min<long long>((warps + HX_THREADS / 32 - 1) / (HX_THREADS / 32), B.max_blocks_grad)));
            if (blocks_used) *blocks_used = blocks;
            if (op->space->w32) hx_rows_grad_launch_w32(B.gk, prec, p, blocks, gsmem, st);
            else hx_rows_grad_launch_w64(B.gk, prec, p, blocks, gsmem, st);
            return;
        }
    }
    if (rows < 0) rows = 32;
    p.rows_per_tile = rows;
    p.x = x;
    p.y = y;
    p.gy = gy;
    p.grad_partial = grad_partial;
    p.accumulate = accumulate;
    const int blocks = mode == 1 ? cap_blocks(blocks_for(B, p.n_rows, rows)) : blocks_for(B, p.n_rows, rows);
    if (blocks_used) *blocks_used = blocks;
    if (op->space->w32) hx_launch_w32(B.gk, prec, mode, p, blocks, B.smem, st);
    else hx_launch_w64(B.gk, prec, mode, p, blocks, B.smem, st);
}

edgpu_space_s* as_space(edgpu_space s) {
    require(s != nullptr, EDGPU_ERR_ARG, "null space handle");
    return static_cast<edgpu_space_s*>(s);
}

// The operators of a batch, then their spaces, each locked once in address order (so two batches
// sharing operators cannot deadlock).
struct BatchLocks {
    std::vector<std::unique_lock<std::mutex>> ops;
    std::vector<std::unique_lock<std::recursive_mutex>> spaces;
    explicit BatchLocks(const std::vector<edgpu_op_s*>& v);
};

BatchLocks::BatchLocks(const std::vector<edgpu_op_s*>& v) {
    std::vector<edgpu_op_s*> o(v);
    std::sort(o.begin(), o.end());
    o.erase(std::unique(o.begin(), o.end()), o.end());
    std::vector<edgpu_space_s*> sp;
    for (auto* x : o) {
        ops.emplace_back(x->hs.mu);
        sp.push_back(x->space);
    }
    std::sort(sp.begin(), sp.end());
    sp.erase(std::unique(sp.begin(), sp.end()), sp.end());
    for (auto* x : sp) spaces.emplace_back(x->hs.mu);
}

edgpu_op_s* as_op(edgpu_op o) {
    require(o != nullptr, EDGPU_ERR_ARG, "null operator handle");
    return static_cast<edgpu_op_s*>(o);
}

void check_prec(int prec) { require(prec == EDGPU_FP64 || prec == EDGPU_MIXED, EDGPU_ERR_ARG, "bad precision"); }

void check_dim(const edgpu_op_s* op, int64_t n, const char* what) {
    if (n != op->space->dim)
        throw Error(EDGPU_ERR_DIM, std::string(what) + " has length " + std::to_string(n) + " != dimension " +
                                       std::to_string(op->space->dim));
}

// ---- symmetric tridiagonal helpers (Lanczos) ----------------------------------------------------

// Number of eigenvalues of tridiag(a, b) below x (Sturm sequence / LDL^T pivot signs).
int sturm_count(const std::vector<double>& a, const std::vector<double>& b, double x) {
    int cnt = 0;
    double d = 1.0;
    for (size_t i = 0; i < a.size(); ++i) {
        const double bb = i ? b[i - 1] * b[i - 1] : 0.0;
        d = (a[i] - x) - (i ? bb / d : 0.0);
        if (d == 0.0) d = -1e-300;
        if (d < 0) ++cnt;
    }
    return cnt;
}

// k-th lowest eigenvalue (k = 1, 2, ...) of tridiag(a, b) by Sturm bisection.
double kth_eigenvalue(const std::vector<double>& a, const std::vector<double>& b, int k) {
    double lo = a[0], hi = a[0];
    for (size_t i = 0; i < a.size(); ++i) {
        const double r = (i ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < a.size() ? std::fabs(b[i]) : 0.0);
        lo = std::min(lo, a[i] - r);
        hi = std::max(hi, a[i] + r);
    }
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (sturm_count(a, b, mid) >= k) hi = mid;
        else lo = mid;
    }
    return 0.5 * (lo + hi);
}

double lowest_eigenvalue(const std::vector<double>& a, const std::vector<double>& b) {
    double lo = a[0], hi = a[0];
    for (size_t i = 0; i < a.size(); ++i) {
        const double r = (i ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < a.size() ? std::fabs(b[i]) : 0.0);
        lo = std::min(lo, a[i] - r);
        hi = std::max(hi, a[i] + r);
    }
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (sturm_count(a, b, mid) >= 1) hi = mid;
        else lo = mid;
    }
    return 0.5 * (lo + hi);
}

// Eigenvector of tridiag(a, b) for eigenvalue lam by inverse iteration (LU with partial pivoting).
std::vector<double> tridiag_eigvec(const std::vector<double>& a, const std::vector<double>& b, double lam) {
    const int n = (int)a.size();
    std::vector<double> z(n, 1.0 / std::sqrt((double)n));
    if (n == 1) return {1.0};
    double scale = 0.0;
    for (int i = 0; i < n; ++i) scale = std::max(scale, std::fabs(a[i]) + (i < n - 1 ? std::fabs(b[i]) : 0.0));
    const double shift = lam - 1e-13 * std::max(1.0, scale);
    for (int iter = 0; iter < 4; ++iter) {
        // factor T - shift I = L U with row interchanges (U has 3 diagonals)
        std::vector<double> d(n), du(n, 0.0), du2(n, 0.0), dl(n, 0.0), rhs = z;
        std::vector<int> piv(n, 0);
        for (int i = 0; i < n; ++i) d[i] = a[i] - shift;
        std::vector<double> sub(n, 0.0), sup(n, 0.0);
        for (int i = 0; i < n - 1; ++i) { sub[i] = b[i]; sup[i] = b[i]; }
        for (int i = 0; i < n; ++i) du[i] = sup[i];
        for (int i = 0; i < n - 1; ++i) {
            if (std::fabs(d[i]) >= std::fabs(sub[i])) {
                const double f = (d[i] != 0.0) ? sub[i] / d[i] : 0.0;
                dl[i] = f;
                d[i + 1] -= f * du[i];
                piv[i] = 0;
            } else {
                const double f = d[i] / sub[i];
                d[i] = sub[i];
                dl[i] = f;
                const double tmp = du[i];
                du[i] = d[i + 1];
                d[i + 1] = tmp - f * d[i + 1];
                if (i < n - 2) {
                    du2[i] = du[i + 1];
                    du[i + 1] = -f * du[i + 1];
                }
                piv[i] = 1;
            }
        }
        for (int i = 0; i < n; ++i)
            if (d[i] == 0.0) d[i] = 1e-300;
        for (int i = 0; i < n - 1; ++i) {   // forward: apply L^-1 with interchanges
            if (piv[i]) std::swap(rhs[i], rhs[i + 1]);
            rhs[i + 1] -= dl[i] * rhs[i];
        }
        for (int i = n - 1; i >= 0; --i) {   // back substitution with U
            double v = rhs[i];
            if (i + 1 < n) v -= du[i] * rhs[i + 1];
            if (i + 2 < n) v -= du2[i] * rhs[i + 2];
            rhs[i] = v / d[i];
        }
        double nrm = 0.0;
        for (double v : rhs) nrm += v * v;
        nrm = std::sqrt(nrm);
        for (int i = 0; i < n; ++i) z[i] = rhs[i] / nrm;
    }
    return z;
}

}  // namespace

// Support for the entry point in noalloc.cu: expose already-built gradient tables and the error slot.
namespace edgpu {
std::unique_lock<std::mutex> lock_op(edgpu_op oh) { return std::unique_lock<std::mutex>(as_op(oh)->hs.mu); }

bool coupling_grad_launch_built(edgpu_op oh, int prec, const void* x, const void* gy, void* y, double* partial,
                                int cap_blocks, cudaStream_t st, int* blocks_used) {
    edgpu_op_s* op = as_op(oh);
    if (!op->blob[prec][0][1].ready || !op->blob[prec][0][0].ready) return false;
    launch_product(op, prec, 0, 1, x, y, 0, gy, partial, st, blocks_used, 0, nullptr, 0, nullptr, cap_blocks);
    return true;
}

int coupling_count(edgpu_op oh) { return as_op(oh)->n_coupl; }
int64_t op_dimension(edgpu_op oh) { return as_op(oh)->space->dim; }

int record_api_error(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace edgpu

// =================================================================================================
extern "C" {

const char* edgpu_last_error(void) { return g_last_error.c_str(); }

const char* edgpu_version(void) { return "edgpu 0.1.0 (sm_103a)"; }

int edgpu_device_count(int32_t* out) {
    API_BEGIN
    require(out, EDGPU_ERR_ARG, "null output");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
    cudaGetLastError();
    *out = n;
    API_END
}

int edgpu_space_create(int32_t n_sites, const int32_t* site_dims, int32_t qn_len, const int64_t* state_qn,
                       int32_t n_allowed, const int64_t* allowed_qn, int32_t flags, edgpu_space* out) {
    API_BEGIN
    require(out != nullptr, EDGPU_ERR_ARG, "null output handle");
    *out = nullptr;
    require(n_sites >= 1 && n_sites <= 64, EDGPU_ERR_ARG, "n_sites must be in [1, 64]");
    require(site_dims != nullptr, EDGPU_ERR_ARG, "null site_dims");
    require(qn_len >= 0 && qn_len <= 4, EDGPU_ERR_ARG, "quantum-number tuples of length 0..4 are supported");
    std::unique_ptr<edgpu_space_s> s(new edgpu_space_s());
    Layout& L = s->lay;
    L.n_sites = n_sites;
    L.qlen = qn_len;
    L.off.push_back(0);
    int total_states = 0;
    for (int i = 0; i < n_sites; ++i) {
        require(site_dims[i] >= 1 && site_dims[i] <= 65536, EDGPU_ERR_ARG, "site dimension out of range");
        L.dims.push_back(site_dims[i]);
        L.bw.push_back(bitwidth_of(site_dims[i]));
        L.off.push_back(L.off.back() + L.bw.back());
        total_states += site_dims[i];
    }
    L.nbits = L.off.back();
    if (L.nbits >= 64)
        throw Error(EDGPU_ERR_ARG, "type UInt64 not enough to represent the hilbert space (need " +
                                       std::to_string(L.nbits) + " bits)");
    if (qn_len > 0) {
        require(state_qn != nullptr, EDGPU_ERR_ARG, "null state_qn");
        L.state_qn.assign(state_qn, state_qn + (size_t)total_states * qn_len);
    }
    if (n_allowed < 0) {
        L.all_sectors = true;
    } else if (n_allowed > 0) {
        require(qn_len > 0, EDGPU_ERR_ARG, "allowed quantum numbers given for a space without quantum numbers");
        require(allowed_qn != nullptr, EDGPU_ERR_ARG, "null allowed_qn");
        L.allowed.assign(allowed_qn, allowed_qn + (size_t)n_allowed * qn_len);
    }
    if (qn_len == 0) L.all_sectors = true;
    // spin-1/2-like single sector: every word of nbits with a fixed popcount
    if (!L.all_sectors && n_allowed == 1 && qn_len == 1) {
        bool ok = true;
        for (int i = 0; i < n_sites && ok; ++i) ok = (L.dims[i] == 2);
        if (ok) {
            const int64_t q0 = L.state_qn[0], q1 = L.state_qn[1];
            for (int i = 0; i < n_sites && ok; ++i) ok = (L.state_qn[2 * i] == q0 && L.state_qn[2 * i + 1] == q1);
            ok = ok && (q0 != q1);
            if (ok) {
                const int64_t v = L.allowed[0] - (int64_t)n_sites * q0, d = q1 - q0;
                if (v % d == 0 && v / d >= 0 && v / d <= n_sites) L.popcount = (int)(v / d);
                else L.popcount = -2;   // unreachable sector: empty basis
            }
        }
    }
    s->lazy = (flags & EDGPU_SPACE_LAZY) != 0;
    s->w32 = L.nbits <= 31;
    if (L.popcount == -2 || (!L.all_sectors && n_allowed == 0)) {
        s->dim = 0;
        L.popcount = -1;
        if (!s->lazy) EDGPU_CUDA(cudaMalloc(&s->d_keys, 16));
        *out = s.release();
        return EDGPU_OK;
    }
    init_device();
    enumerate_parent(*s, s->hs.stream());
    if (!s->lazy) build_search_directory(*s, s->hs.stream());
    *out = s.release();
    API_END
}

int edgpu_space_from_basis(int32_t n_sites, const int32_t* site_dims, const uint64_t* basis, int64_t n,
                           edgpu_space* out) {
    API_BEGIN
    require(out != nullptr, EDGPU_ERR_ARG, "null output handle");
    *out = nullptr;
    require(n_sites >= 1 && n_sites <= 64 && site_dims, EDGPU_ERR_ARG, "bad site layout");
    require(n >= 0 && (n == 0 || basis), EDGPU_ERR_ARG, "bad basis");
    std::unique_ptr<edgpu_space_s> s(new edgpu_space_s());
    Layout& L = s->lay;
    L.n_sites = n_sites;
    L.off.push_back(0);
    for (int i = 0; i < n_sites; ++i) {
        require(site_dims[i] >= 1, EDGPU_ERR_ARG, "site dimension out of range");
        L.dims.push_back(site_dims[i]);
        L.bw.push_back(bitwidth_of(site_dims[i]));
        L.off.push_back(L.off.back() + L.bw.back());
    }
    L.nbits = L.off.back();
    if (L.nbits >= 64)
        throw Error(EDGPU_ERR_ARG, "type UInt64 not enough to represent the hilbert space (need " +
                                       std::to_string(L.nbits) + " bits)");
    L.all_sectors = true;
    std::vector<uint64_t> b(basis, basis + n);
    if (!std::is_sorted(b.begin(), b.end())) std::sort(b.begin(), b.end());
    for (int64_t i = 1; i < n; ++i)
        if (b[i] == b[i - 1]) throw Error(EDGPU_ERR_ARG, "vals contains duplicates " + std::to_string(b[i]));
    const uint64_t full = (1ull << L.nbits) - 1ull;
    for (int64_t i = 0; i < n; ++i)
        require((b[i] & ~full) == 0, EDGPU_ERR_ARG, "basis state has bits beyond the site layout");
    s->w32 = L.nbits <= 31;
    s->dim = n;
    init_device();
    if (s->w32) {
        std::vector<uint32_t> b32(b.begin(), b.end());
        EDGPU_CUDA(cudaMalloc(&s->d_keys, std::max<int64_t>(n, 1) * 4));
        EDGPU_CUDA(cudaMemcpy(s->d_keys, b32.data(), n * 4, cudaMemcpyHostToDevice));
    } else {
        EDGPU_CUDA(cudaMalloc(&s->d_keys, std::max<int64_t>(n, 1) * 8));
        EDGPU_CUDA(cudaMemcpy(s->d_keys, b.data(), n * 8, cudaMemcpyHostToDevice));
    }
    build_search_directory(*s, s->hs.stream());
    *out = s.release();
    API_END
}

int edgpu_space_dim(edgpu_space s, int64_t* out) {
    API_BEGIN
    require(out, EDGPU_ERR_ARG, "null output");
    *out = as_space(s)->dim;
    API_END
}

int edgpu_space_nbits(edgpu_space s, int32_t* out) {
    API_BEGIN
    require(out, EDGPU_ERR_ARG, "null output");
    *out = as_space(s)->lay.nbits;
    API_END
}

int edgpu_space_get_basis(edgpu_space sh, uint64_t* out, int64_t n) {
    API_BEGIN
    edgpu_space_s* s = as_space(sh);
    SpaceLock lk_(s->hs.mu);
    require(s->d_keys != nullptr || s->dim == 0, EDGPU_ERR_STATE, "basis of a lazy space is not materialised");
    if (n != s->dim) throw Error(EDGPU_ERR_DIM, "output has length " + std::to_string(n) + " != dimension " +
                                                     std::to_string(s->dim));
    if (n == 0) return EDGPU_OK;
    require(out, EDGPU_ERR_ARG, "null output");
    get_states(*s, out, s->hs.stream());
    API_END
}

int edgpu_space_lookup(edgpu_space sh, const uint64_t* keys, int64_t n, int64_t* idx_out) {
    API_BEGIN
    edgpu_space_s* s = as_space(sh);
    SpaceLock lk_(s->hs.mu);
    require(s->d_keys != nullptr, EDGPU_ERR_STATE, "basis of a lazy space is not materialised");
    require(n >= 0 && (n == 0 || (keys && idx_out)), EDGPU_ERR_ARG, "bad arguments");
    if (s->dim == 0) {
        for (int64_t i = 0; i < n; ++i) idx_out[i] = -1;
        return EDGPU_OK;
    }
    lookup_keys(*s, keys, n, idx_out, s->hs.stream());
    API_END
}

void edgpu_space_destroy(edgpu_space s) { delete static_cast<edgpu_space_s*>(s); }

int edgpu_space_search_stats(edgpu_space sh, int64_t* buckets, int32_t* shift, int32_t* inline_keys_per_bucket,
                             int32_t* window_steps, double* inline_fraction) {
    API_BEGIN
    edgpu_space_s* s = as_space(sh);
    SpaceLock lk_(s->hs.mu);
    require(s->d_dir != nullptr || s->dim == 0, EDGPU_ERR_STATE, "no search directory (lazy or empty space)");
    if (buckets) *buckets = s->dir_nb;
    if (shift) *shift = s->dir_shift;
    if (inline_keys_per_bucket) *inline_keys_per_bucket = s->dir_K;
    if (window_steps) *window_steps = s->dir_steps;
    if (inline_fraction) *inline_fraction = s->dir_inline;
    API_END
}

int edgpu_space_build_map(edgpu_space sh, int64_t max_bytes, int32_t* built) {
    API_BEGIN
    edgpu_space_s* s = as_space(sh);
    SpaceLock lk_(s->hs.mu);
    require(max_bytes >= 0, EDGPU_ERR_ARG, "negative byte limit");
    require(s->reduced, EDGPU_ERR_ARG, "parent-state maps belong to reduced representations");
    if (!s->d_dir && s->dim > 0) build_search_directory(*s, s->hs.stream());
    const bool ok = build_parent_map(*s, max_bytes, s->hs.stream());
    if (built) *built = ok ? 1 : 0;
    API_END
}

int edgpu_space_free_map(edgpu_space sh) {
    API_BEGIN
    edgpu_space_s* s = as_space(sh);
    SpaceLock lk_(s->hs.mu);
    EDGPU_CUDA(cudaDeviceSynchronize());
    free_parent_map(*s);
    API_END
}

int edgpu_space_map_info(edgpu_space sh, int64_t* entries, int32_t* entry_bytes) {
    API_BEGIN
    edgpu_space_s* s = as_space(sh);
    SpaceLock lk_(s->hs.mu);
    if (entries) *entries = s->d_map ? s->map_n : 0;
    if (entry_bytes) *entry_bytes = s->d_map ? (s->map_wide ? 8 : 4) : 0;
    API_END
}

int edgpu_reduce(edgpu_space parent_h, int32_t n_elems, const int32_t* site_maps, const uint64_t* flip_masks,
                 const int32_t* char_num, int32_t char_den, edgpu_space* out) {
    API_BEGIN
    require(out != nullptr, EDGPU_ERR_ARG, "null output handle");
    *out = nullptr;
    edgpu_space_s* parent = as_space(parent_h);
    SpaceLock lk_(parent->hs.mu);
    require(!parent->reduced, EDGPU_ERR_ARG, "the parent must be an unreduced representation");
    const Layout& L = parent->lay;
    const int n = L.n_sites;
    require(n_elems >= 1 && n_elems <= 4096, EDGPU_ERR_ARG, "group order must be in [1, 4096]");
    require(site_maps && char_num, EDGPU_ERR_ARG, "null group data");
    require(char_den >= 1 && char_den <= 4096, EDGPU_ERR_ARG, "character denominator must be in [1, 4096]");
    const uint64_t full = (1ull << L.nbits) - 1ull;
    Group g;
    g.G = n_elems;
    g.den = char_den;
    g.maps.assign(site_maps, site_maps + (size_t)n_elems * n);
    g.flips.assign(n_elems, 0ull);
    if (flip_masks) g.flips.assign(flip_masks, flip_masks + n_elems);
    g.num.resize(n_elems);
    for (int e = 0; e < n_elems; ++e) g.num[e] = ((char_num[e] % char_den) + char_den) % char_den;
    // each element: a site permutation between sites of equal bit width; flips inside the word
    for (int e = 0; e < n_elems; ++e) {
        std::vector<char> seen(n, 0);
        for (int i = 0; i < n; ++i) {
            const int j = g.maps[(size_t)e * n + i];
            require(j >= 0 && j < n && !seen[j], EDGPU_ERR_ARG, "site map of element " + std::to_string(e) +
                                                                   " is not a permutation");
            seen[j] = 1;
            require(L.bw[i] == L.bw[j], EDGPU_ERR_ARG, "a permutation maps sites of different bit widths");
        }
        require((g.flips[e] & ~full) == 0, EDGPU_ERR_ARG, "flip mask has bits beyond the site layout");
    }
    for (int i = 0; i < n; ++i)
        require(g.maps[i] == i, EDGPU_ERR_ARG, "element 0 must be the identity");
    require(g.flips[0] == 0 && g.num[0] == 0, EDGPU_ERR_ARG, "element 0 must be the identity with amplitude 1");
    // closure and the 1-D representation property: chi(g h) = chi(g) chi(h)
    {
        std::map<std::pair<std::vector<int32_t>, uint64_t>, int> index;
        for (int e = 0; e < n_elems; ++e) {
            std::vector<int32_t> m(g.maps.begin() + (size_t)e * n, g.maps.begin() + (size_t)(e + 1) * n);
            auto key = std::make_pair(m, g.flips[e]);
            require(index.find(key) == index.end(), EDGPU_ERR_ARG, "repeated group element");
            index[key] = e;
        }
        auto apply_bits = [&](int e, uint64_t b) {
            uint64_t o = 0;
            for (int i = 0; i < n; ++i) {
                const uint64_t m = (1ull << L.bw[i]) - 1ull;
                o |= ((b >> L.off[i]) & m) << L.off[g.maps[(size_t)e * n + i]];
            }
            return o;
        };
        for (int a = 0; a < n_elems; ++a)
            for (int b = 0; b < n_elems; ++b) {
                std::vector<int32_t> m(n);
                for (int i = 0; i < n; ++i) m[i] = g.maps[(size_t)a * n + g.maps[(size_t)b * n + i]];
                const uint64_t f = apply_bits(a, g.flips[b]) ^ g.flips[a];
                auto it = index.find(std::make_pair(m, f));
                require(it != index.end(), EDGPU_ERR_ARG, "the symmetry operations do not form a group");
                require((g.num[a] + g.num[b]) % char_den == g.num[it->second], EDGPU_ERR_ARG,
                        "the amplitudes are not a one-dimensional representation of the group");
            }
    }
    // torus translation structure (fast path): uniform bit width, no flips, G == n_sites
    bool uniform = true;
    for (int i = 0; i < n; ++i) uniform = uniform && (L.bw[i] == L.bw[0]);
    bool noflip = true;
    for (int e = 0; e < n_elems; ++e) noflip = noflip && g.flips[e] == 0;
    g.kind = GK_GENERIC;
    if (n_elems == 1) {
        g.kind = GK_TRIVIAL;
        g.num = {0};
        g.den = 1;
    } else if (uniform && noflip && n_elems == n && L.bw[0] >= 1) {
        for (int L1 = n; L1 >= 1 && g.kind == GK_GENERIC; --L1) {
            if (n % L1 != 0 || L1 > 64) continue;
            const int L2 = n / L1;
            std::vector<int> slot(n_elems, -1);
            bool ok = true;
            for (int e = 0; e < n_elems && ok; ++e) {
                const int32_t* m = &g.maps[(size_t)e * n];
                const int a = m[0] % L1, b = m[0] / L1;
                for (int y = 0; y < L2 && ok; ++y)
                    for (int x = 0; x < L1 && ok; ++x)
                        ok = (m[x + L1 * y] == (x + a) % L1 + L1 * ((y + b) % L2));
                if (ok) {
                    const int t = a + L1 * b;
                    ok = slot[t] < 0;
                    slot[t] = e;
                }
            }
            if (ok) {
                std::vector<int32_t> num(n_elems);
                for (int t = 0; t < n_elems; ++t) num[t] = g.num[slot[t]];
                g.kind = GK_TORUS;
                g.L1 = L1;
                g.L2 = L2;
                g.w = L.bw[0];
                g.num = num;
            }
        }
    }
    std::unique_ptr<edgpu_space_s> s(new edgpu_space_s());
    s->lay = L;
    s->reduced = true;
    s->parent = parent;
    s->group = g;
    s->sb = g.kind == GK_TRIVIAL ? 0 : orbit_index_bits(g.G);
    require(L.nbits + s->sb <= 64, EDGPU_ERR_ARG, "state plus orbit index does not fit a 64-bit key");
    s->w32 = L.nbits + s->sb <= 32;
    init_device();
    if (parent->dim == 0) {
        s->dim = 0;
        EDGPU_CUDA(cudaMalloc(&s->d_keys, 16));
    } else {
        enumerate_reps(*s, *parent, s->hs.stream());
        embed_orbit_index(*s, s->hs.stream());
    }
    build_search_directory(*s, s->hs.stream());
    *out = s.release();
    API_END
}

int edgpu_reduce_mapping(edgpu_space reduced, int64_t* index_out, double* ampl_out, int64_t n_parent) {
    API_BEGIN
    edgpu_space_s* s = as_space(reduced);
    SpaceLock lk_(s->hs.mu);
    require(s->reduced && s->parent, EDGPU_ERR_ARG, "not a reduced representation");
    require(s->parent->d_keys != nullptr || s->parent->dim == 0, EDGPU_ERR_STATE, "the parent basis is not materialised");
    if (n_parent != s->parent->dim) throw Error(EDGPU_ERR_DIM, "output length != parent dimension");
    if (n_parent == 0) return EDGPU_OK;
    require(index_out && ampl_out, EDGPU_ERR_ARG, "null output");
    build_mapping(*s, *s->parent, index_out, ampl_out, s->hs.stream());
    API_END
}

int edgpu_space_parent_dim(edgpu_space reduced, int64_t* out) {
    API_BEGIN
    edgpu_space_s* s = as_space(reduced);
    SpaceLock lk_(s->hs.mu);
    require(out, EDGPU_ERR_ARG, "null output");
    require(s->reduced && s->parent, EDGPU_ERR_ARG, "not a reduced representation");
    *out = parent_dimension(*s->parent);
    API_END
}

int edgpu_symmetry_unreduce_device(edgpu_space reduced, int32_t precision, const void* small, int64_t n, void* large,
                                   int64_t n_parent, void* stream) {
    API_BEGIN
    edgpu_space_s* s = as_space(reduced);
    SpaceLock lk_(s->hs.mu);
    check_prec(precision);
    require(s->reduced && s->parent, EDGPU_ERR_ARG, "not a reduced representation");
    require(n == s->dim, EDGPU_ERR_DIM, "small vector has length " + std::to_string(n) + " != dimension " + std::to_string(s->dim));
    require(n_parent == parent_dimension(*s->parent), EDGPU_ERR_DIM, "large vector length differs from the parent dimension");
    if (n_parent == 0) return EDGPU_OK;
    require(large && (small || n == 0), EDGPU_ERR_ARG, "null vector");
    cudaStream_t st = stream ? pick_stream(stream) : s->hs.stream();
    reduce_vector(*s, *s->parent, precision, true, small, large, st);
    API_END
}

int edgpu_symmetry_reduce_device(edgpu_space reduced, int32_t precision, const void* large, int64_t n_parent, void* small,
                                 int64_t n, void* stream) {
    API_BEGIN
    edgpu_space_s* s = as_space(reduced);
    SpaceLock lk_(s->hs.mu);
    check_prec(precision);
    require(s->reduced && s->parent, EDGPU_ERR_ARG, "not a reduced representation");
    require(n == s->dim, EDGPU_ERR_DIM, "small vector has length " + std::to_string(n) + " != dimension " + std::to_string(s->dim));
    require(n_parent == parent_dimension(*s->parent), EDGPU_ERR_DIM, "large vector length differs from the parent dimension");
    if (n == 0) return EDGPU_OK;
    require(small && (large || n_parent == 0), EDGPU_ERR_ARG, "null vector");
    cudaStream_t st = stream ? pick_stream(stream) : s->hs.stream();
    reduce_vector(*s, *s->parent, precision, false, large, small, st);
    API_END
}

int edgpu_space_orbit_sizes(edgpu_space reduced, int32_t* out, int64_t n) {
    API_BEGIN
    edgpu_space_s* s = as_space(reduced);
    SpaceLock lk_(s->hs.mu);
    if (n != s->dim) throw Error(EDGPU_ERR_DIM, "output length != dimension");
    if (n == 0) return EDGPU_OK;
    require(out, EDGPU_ERR_ARG, "null output");
    orbit_sizes(*s, out, s->hs.stream());
    API_END
}

int edgpu_op_create(edgpu_space sh, int32_t n_terms, const uint64_t* masks, const uint64_t* rows, const uint64_t* cols,
                    const double* amps, const int32_t* coupling_ids, int32_t n_couplings, const double* couplings,
                    edgpu_op* out) {
    API_BEGIN
    require(out != nullptr, EDGPU_ERR_ARG, "null output handle");
    *out = nullptr;
    edgpu_space_s* s = as_space(sh);
    SpaceLock lk_(s->hs.mu);
    require(s->d_keys != nullptr, EDGPU_ERR_STATE, "the representation's basis is not materialised");
    require(n_terms >= 0, EDGPU_ERR_ARG, "negative term count");
    require(n_terms == 0 || (masks && rows && cols && amps), EDGPU_ERR_ARG, "null term arrays");
    const uint64_t full = (s->lay.nbits >= 64) ? ~0ull : ((1ull << s->lay.nbits) - 1ull);
    std::unique_ptr<edgpu_op_s> op(new edgpu_op_s());
    op->space = s;
    op->T = n_terms;
    for (int t = 0; t < n_terms; ++t) {
        if ((~masks[t]) & rows[t]) throw Error(EDGPU_ERR_ARG, "every bit of bitrow not in bitmask should be set to zero");
        if ((~masks[t]) & cols[t]) throw Error(EDGPU_ERR_ARG, "every bit of bitcol not in bitmask should be set to zero");
        require((masks[t] & ~full) == 0, EDGPU_ERR_ARG, "term mask has bits beyond the site layout");
    }
    op->masks.assign(masks, masks + n_terms);
    op->rows.assign(rows, rows + n_terms);
    op->cols.assign(cols, cols + n_terms);
    op->unit.assign(amps, amps + 2 * (size_t)n_terms);
    if (coupling_ids) {
        require(n_couplings >= 1 && n_couplings <= 8192, EDGPU_ERR_ARG, "n_couplings must be in [1, 8192]");
        require(couplings != nullptr, EDGPU_ERR_ARG, "null couplings");
        op->cid.assign(coupling_ids, coupling_ids + n_terms);
        for (int t = 0; t < n_terms; ++t)
            require(op->cid[t] >= 0 && op->cid[t] < n_couplings, EDGPU_ERR_ARG, "coupling id out of range");
        op->n_coupl = n_couplings;
        op->coupl.assign(couplings, couplings + n_couplings);
    } else {
        op->cid.assign(n_terms, 0);
        op->n_coupl = 1;
        op->coupl = {1.0};
    }
    init_device();
    *out = op.release();
    API_END
}

int edgpu_op_set_couplings(edgpu_op oh, const double* couplings, int32_t n_couplings) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    require(n_couplings == op->n_coupl && couplings, EDGPU_ERR_DIM, "coupling count mismatch");
    op->coupl.assign(couplings, couplings + n_couplings);
    refresh_blobs(op);
    API_END
}

int edgpu_op_dim(edgpu_op oh, int64_t* out) {
    API_BEGIN
    require(out, EDGPU_ERR_ARG, "null output");
    *out = as_op(oh)->space->dim;
    API_END
}

void edgpu_op_destroy(edgpu_op o) {
    edgpu_op_s* op = static_cast<edgpu_op_s*>(o);
    if (!op) return;
    invalidate_blobs(op);
    delete op;
}

int edgpu_op_set_tiling(edgpu_op oh, int32_t precision, int32_t rows_per_tile) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    check_prec(precision);
    require(rows_per_tile == 0 || rows_per_tile == -1 || rows_per_tile == -2 || rows_per_tile == -4 ||
                (rows_per_tile >= 1 && rows_per_tile <= 32 && (32 % rows_per_tile) == 0),
            EDGPU_ERR_ARG, "rows_per_tile must be 0 (default), -1/-2/-4 (1, 2 or 4 lanes per row) or a divisor of 32");
    op->tuned_rows[precision] = rows_per_tile;
    API_END
}

int edgpu_op_set_pair_schedule(edgpu_op oh, int32_t enable) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    const int uni = (enable & EDGPU_PAIR_UNIFORM) ? 1 : 0;
    const int nt = enable & ~EDGPU_PAIR_UNIFORM;
    require(nt == 0 || nt == 1 || nt == 2 || nt == 4 || nt == 8, EDGPU_ERR_ARG,
            "enable must be 0, 1, 2, 4 or 8, optionally with EDGPU_PAIR_UNIFORM");
    require(!uni || nt >= 4, EDGPU_ERR_ARG, "warp-uniform pair steps need 4 or 8 targets per step");
    op->pair_allowed = nt ? 1 : 0;
    op->pair_use[0] = op->pair_use[1] = nt ? 1 : 0;
    op->pair_nt[0] = op->pair_nt[1] = nt >= 4 ? nt : 2;
    op->tab_uni[0] = op->tab_uni[1] = uni;
    API_END
}

int edgpu_op_table_prefetch(edgpu_op oh, int32_t precision, int32_t steps, int32_t* current) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    check_prec(precision);
    require(steps <= 1024, EDGPU_ERR_ARG, "prefetch distance above 1024 steps");
    if (steps >= 0) op->tab_pf[precision] = steps;
    if (current) *current = op->tab_pf[precision];
    API_END
}

int edgpu_op_get_schedule(edgpu_op oh, int32_t precision, int32_t* rows_per_tile, int32_t* pair_flips,
                          int32_t* target_table) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    check_prec(precision);
    if (rows_per_tile) *rows_per_tile = op->tuned_rows[precision];
    build_blob(op, precision, 0, 0);
    const int rows = op->tuned_rows[precision];
    const bool on = op->blob[precision][0][0].tmpl.bond_ncls > 0 && op->pair_allowed && op->pair_use[precision] &&
                    rows <= 0;
    const bool table = on && op->d_tab && op->tab_use[precision];
    int nt = 2;
    if (on && (op->space->d_map || table) && op->pair_nt[precision] >= 4) nt = (table && op->pair_nt[precision] == 8) ? 8 : 4;
    if (pair_flips) *pair_flips = on ? (nt | ((table && nt >= 4 && op->tab_uni[precision]) ? EDGPU_PAIR_UNIFORM : 0)) : 0;
    if (target_table) *target_table = table ? 1 : 0;
    API_END
}

int edgpu_op_build_targets(edgpu_op oh, int64_t max_bytes, int32_t* built) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    require(max_bytes >= 0, EDGPU_ERR_ARG, "negative byte limit");
    if (built) *built = 0;
    op->free_table();
    const Space& sp = *op->space;
    // the pair-flip tables of either precision (the bond classes do not depend on it)
    int prec = EDGPU_MIXED;
    build_blob(op, prec, 0, 0);
    if (op->blob[prec][0][0].tmpl.bond_ncls == 0) {
        prec = EDGPU_FP64;
        build_blob(op, prec, 0, 0);
    }
    Blob& B = op->blob[prec][0][0];
    if (B.tmpl.bond_ncls == 0 || sp.dim == 0) return EDGPU_OK;
    const bool mapped = sp.d_map != nullptr;
    HxParams p = B.tmpl;
    if (mapped) {
        set_map_params(p, sp);
        p.map = sp.d_map;
        p.map_wide = sp.map_wide;
        p.map_cb = sp.map_cb;
        p.map_direct = sp.map_direct;
    }
    const size_t smem = mapped ? B.smem_bond : B.smem_bond_canon;
    p.blob = B.d_pair;
    p.o_rlut = B.tmpl_pair.o_rlut;
    p.o_bcomp = B.tmpl_pair.o_bcomp;
    p.o_binfo = B.tmpl_pair.o_binfo;
    p.o_bflip = B.tmpl_pair.o_bflip;
    p.o_bamp = B.tmpl_pair.o_bamp;
    p.blob_words16 = (int)(smem / 16);
    p.lpr = 1;
    p.rows_per_tile = 32;
    // entry format of the parent-state map: c | sx << cb | g << (cb + sb), g only for characters other
    // than 1; all ones = no representative
    int cb = 1;
    while (cb < 63 && ((int64_t)1 << cb) <= sp.dim) ++cb;
    int gbits = 0;
    if (sp.group.den > 1)
        while (gbits < 12 && (1 << gbits) < sp.group.G) ++gbits;
    require(cb + sp.sb + gbits <= 64, EDGPU_ERR_ARG, "target entries do not fit in 64 bits");
    const int wide = cb + sp.sb + gbits > 32 ? 1 : 0;
    const long long n_tiles = (sp.dim + 31) / 32;
    DevBuf<long long> cnt;
    cnt.ensure((size_t)n_tiles);
    long long* d_off = nullptr;
    EDGPU_CUDA(cudaMalloc(&d_off, (size_t)n_tiles * sizeof(long long)));
    try {
        hx_table_count(sp.w32, p, n_tiles, cnt.p, smem, op->hs.stream());
        const long long total = hx_table_scan(cnt.p, n_tiles, d_off, op->hs.stream());
        const double bytes = (double)total * (wide ? 8.0 : 4.0) + (double)n_tiles * 8.0;
        if (bytes > (double)max_bytes) {
            cudaFree(d_off);
            return EDGPU_OK;
        }
        void* d_tab = nullptr;
        EDGPU_CUDA(cudaMalloc(&d_tab, std::max<size_t>((size_t)total * (wide ? 8 : 4), 16)));
        p.tab = d_tab;
        p.tile_off = d_off;
        p.tab_wide = wide;
        p.tab_cb = cb;
        try {
            hx_table_fill(sp.w32, mapped ? GK_MAP : B.gk, p, n_tiles, smem, op->hs.stream());
            EDGPU_CUDA(cudaStreamSynchronize(op->hs.stream()));
        } catch (...) {
            cudaFree(d_tab);
            throw;
        }
        op->d_tab = d_tab;
        op->d_tile_off = d_off;
        op->tab_wide = wide;
        op->tab_cb = cb;
        op->tab_n = total;
        op->tab_use[0] = op->tab_use[1] = 1;
    } catch (...) {
        if (!op->d_tile_off) cudaFree(d_off);
        throw;
    }
    if (built) *built = 1;
    API_END
}

int edgpu_op_free_targets(edgpu_op oh) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    // products on caller streams may still read the table
    EDGPU_CUDA(cudaDeviceSynchronize());
    op->free_table();
    API_END
}

int edgpu_op_build_adjoint_targets(edgpu_op oh, int64_t max_bytes, int32_t* built) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    require(max_bytes >= 0, EDGPU_ERR_ARG, "negative byte limit");
    if (built) *built = 0;
    op->free_adjoint();
    const Space& sp = *op->space;
    if (!op->d_tab || sp.dim == 0) return EDGPU_OK;
    int prec = EDGPU_MIXED;
    build_blob(op, prec, 0, 0);
    if (op->blob[prec][0][0].tmpl.bond_ncls == 0) {
        prec = EDGPU_FP64;
        build_blob(op, prec, 0, 0);
    }
    const Blob& B = op->blob[prec][0][0];
    if (B.tmpl.bond_ncls == 0) return EDGPU_OK;
    require(sp.dim < ((int64_t)1 << 32) && sp.sb <= 5 && sp.group.G <= (1 << 14), EDGPU_ERR_ARG,
            "the adjoint table's entries hold rows below 2^32, 5 orbit-size bits and 2^14 group elements");
    const int64_t n = sp.dim;
    if ((double)op->tab_n * 8.0 + (double)(n + 1) * 8.0 > (double)max_bytes) return EDGPU_OK;
    HxParams p = B.tmpl_pair;
    p.blob = B.d_pair;
    p.blob_words16 = (int)(B.smem_bond / 16);
    p.lpr = 1;
    p.rows_per_tile = 32;
    p.bond_nt = 4;
    p.bond_pf = 0;
    p.bond_uni = 0;
    p.tab = op->d_tab;
    p.tile_off = op->d_tile_off;
    p.tab_wide = op->tab_wide;
    p.tab_cb = op->tab_cb;
    const long long n_tiles = (n + 31) / 32;
    cudaStream_t st = op->hs.stream();
    DevBuf<unsigned> cnt;
    cnt.ensure((size_t)n);
    EDGPU_CUDA(cudaMemsetAsync(cnt.p, 0, (size_t)n * sizeof(unsigned), st));
    p.adj_cnt = cnt.p;
    hx_adj_pass(sp.w32, 1, p, n_tiles, B.smem_bond, st);
    std::vector<unsigned> hc((size_t)n);
    EDGPU_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, (size_t)n * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    EDGPU_CUDA(cudaStreamSynchronize(st));
    std::vector<long long> ho((size_t)n + 1);
    ho[0] = 0;
    for (int64_t c = 0; c < n; ++c) ho[c + 1] = ho[c] + hc[c];
    const long long total = ho[n];
    long long* d_off = nullptr;
    unsigned long long* d_tab = nullptr;
    EDGPU_CUDA(cudaMalloc(&d_off, (size_t)(n + 1) * sizeof(long long)));
    cudaError_t e = cudaMalloc(&d_tab, std::max<size_t>((size_t)total * 8, 16));
    if (e != cudaSuccess) {
        cudaFree(d_off);
        throw Error(e == cudaErrorMemoryAllocation ? EDGPU_ERR_OOM : EDGPU_ERR_CUDA,
                    std::string("adjoint table: ") + cudaGetErrorString(e));
    }
    op->d_adj_off = d_off;
    op->d_adj_tab = d_tab;
    EDGPU_CUDA(cudaMemcpyAsync(d_off, ho.data(), (size_t)(n + 1) * sizeof(long long), cudaMemcpyHostToDevice, st));
    EDGPU_CUDA(cudaMemsetAsync(cnt.p, 0, (size_t)n * sizeof(unsigned), st));
    p.adj_off = d_off;
    p.adj_cur = cnt.p;
    p.adj_tab = d_tab;
    hx_adj_pass(sp.w32, 2, p, n_tiles, B.smem_bond, st);
    hx_adj_sort(d_off, d_tab, n, st);
    EDGPU_CUDA(cudaStreamSynchronize(st));
    op->adj_n = total;
    if (built) *built = 1;
    API_END
}

int edgpu_op_free_adjoint_targets(edgpu_op oh) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    EDGPU_CUDA(cudaDeviceSynchronize());
    op->free_adjoint();
    API_END
}

int edgpu_op_targets_info(edgpu_op oh, int64_t* entries, int32_t* entry_bytes) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    if (entries) *entries = op->d_tab ? op->tab_n : 0;
    if (entry_bytes) *entry_bytes = op->d_tab ? (op->tab_wide ? 8 : 4) : 0;
    API_END
}

int edgpu_op_build_slabs(edgpu_op oh, int64_t slab_bytes, int64_t max_bytes, int32_t* built) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    require(slab_bytes > 0 && max_bytes >= 0, EDGPU_ERR_ARG, "slab_bytes must be positive and max_bytes >= 0");
    if (built) *built = 0;
    EDGPU_CUDA(cudaDeviceSynchronize());   // products on caller streams may still read an old slab table
    op->free_slabs();
    const Space& sp = *op->space;
    if (!op->d_tab || sp.dim == 0 || sp.dim >= ((int64_t)1 << 32)) return EDGPU_OK;
    int prec = EDGPU_MIXED;
    build_blob(op, prec, 0, 0);
    if (op->blob[prec][0][0].tmpl.bond_ncls == 0) {
        prec = EDGPU_FP64;
        build_blob(op, prec, 0, 0);
    }
    const Blob& B = op->blob[prec][0][0];
    if (B.tmpl.bond_ncls == 0) return EDGPU_OK;
    // the slots' coupling ids and unit amplitudes: the bond classes of the terms, once with the coupled
    // amplitudes (and coupling ids), once with the unit ones; their pairs must be the product's
    const int nb = sp.lay.nbits, ncls = B.tmpl.bond_ncls;
    BondClasses bc, bcu;
    {
        std::vector<uint64_t> bm, br, bf;
        std::vector<double> ba, bu;
        std::vector<int32_t> bid;
        for (int t = 0; t < op->T; ++t) {
            if (op->rows[t] == op->cols[t]) continue;
            bm.push_back(op->masks[t]);
            br.push_back(op->rows[t]);
            bf.push_back(op->rows[t] ^ op->cols[t]);
            const double c = op->coupl[op->cid[t]];
            ba.push_back(op->unit[2 * t] * c);
            ba.push_back(op->unit[2 * t + 1] * c);
            bu.push_back(op->unit[2 * t]);
            bu.push_back(op->unit[2 * t + 1]);
            bid.push_back(op->cid[t]);
        }
        if (!build_bond_classes(sp.lay, bm, br, bf, ba, bc, &bid) || !bc.cid_ok ||
            !build_bond_classes(sp.lay, bm, br, bf, bu, bcu) || bc.ncls != ncls || bcu.ncls != ncls)
            return EDGPU_OK;
    }
    const size_t wsz = sp.w32 ? 4 : 8;
    if ((size_t)B.tmpl_pair.o_bflip + (size_t)ncls * nb * wsz > B.pair_host.size()) return EDGPU_OK;
    int n_pairs = 0;
    for (int k = 0; k < ncls * nb; ++k) {
        uint64_t f = 0;
        memcpy(&f, &B.pair_host[B.tmpl_pair.o_bflip + k * wsz], wsz);
        if (f != bc.flip[k] || f != bcu.flip[k]) return EDGPU_OK;
        n_pairs += f != 0;
    }
    // a row's targets in one slab are counted in a byte: at most 255 pairs
    if (n_pairs > 255) return EDGPU_OK;
    auto& S = op->slab;
    const int n_slots = ncls * nb * 4;
    std::vector<unsigned short> amp_id((size_t)n_slots, 0);
    std::map<std::tuple<int, double, double>, int> ids;
    for (int k = 0; k < n_slots; ++k) {
        const int32_t c = bc.cid[k];
        if (c < 0) continue;
        const double u0 = bcu.amp[2 * (size_t)k], u1 = bcu.amp[2 * (size_t)k + 1];
        const auto key = std::make_tuple((int)c, u0, u1);
        auto it = ids.find(key);
        if (it == ids.end()) {
            it = ids.emplace(key, (int)S.amp_cid.size()).first;
            S.amp_cid.push_back(c);
            S.amp_unit.push_back(u0);
            S.amp_unit.push_back(u1);
        }
        amp_id[k] = (unsigned short)it->second;
    }
    const int n_amp = std::max<int>(1, (int)S.amp_cid.size());
    S.den = std::max(1, sp.group.den);
    S.divs.clear();
    for (int d = 1; d <= sp.group.G; ++d)
        if (sp.group.G % d == 0) S.divs.push_back(d);
    S.nd = (int)S.divs.size();
    // columns per slab and passes of a layout with n_ids coefficient ids (0 passes: ids too many)
    auto layout = [&](long long n_ids, long long& wc) {
        int idbits = 1;
        while (((long long)1 << idbits) < n_ids) ++idbits;
        if (32 - idbits < 12 || n_ids * 8 > 48 * 1024) return 0;
        wc = std::max<long long>(1024, std::min<long long>(slab_bytes / 8, (long long)1 << (32 - idbits)));
        return (int)((sp.dim + wc - 1) / wc);
    };
    bool complex_coef = S.den > 1;
    for (size_t a = 0; a < S.amp_cid.size(); ++a) complex_coef = complex_coef || S.amp_unit[2 * a + 1] != 0.0;
    const long long ids_full = (long long)n_amp * S.den * S.nd * S.nd, ids_scaled = (long long)n_amp * S.den;
    long long wc_full = 0, wc_scaled = 0;
    const int pass_full = layout(ids_full, wc_full), pass_scaled = layout(ids_scaled, wc_scaled);
    // the scaled layout pays a scaling pass over x per product; by default it is taken on sectors of
    // 2^22 rows or more where it saves passes or replaces a complex coefficient table (whose lookups
    // conflict in shared memory)
    bool scaled = false;
    if (S.nd > 1 && pass_scaled > 0) {
        if (op->slab_scaling == 2) scaled = true;
        else if (op->slab_scaling == 0)
            scaled = pass_full == 0 || (sp.dim >= ((int64_t)1 << 22) && (pass_scaled < pass_full || complex_coef));
    }
    const long long n_ids = scaled ? ids_scaled : ids_full;
    const long long wc = scaled ? wc_scaled : wc_full;
    const int n_pass = scaled ? pass_scaled : pass_full;
    if (n_pass == 0 || n_amp > 65535) {
        op->free_slabs();
        return EDGPU_OK;
    }
    int idbits = 1;
    while (((long long)1 << idbits) < n_ids) ++idbits;
    const int colbits = 32 - idbits;
    const long long n_tiles = (sp.dim + 31) / 32;
    if (n_pass > 64) {
        op->free_slabs();
        return EDGPU_OK;
    }
    HxParams p = B.tmpl_pair;
    p.blob = B.d_pair;
    p.blob_words16 = (int)(B.smem_bond / 16);
    p.lpr = 1;
    p.rows_per_tile = 32;
    p.tab = op->d_tab;
    p.tile_off = op->d_tile_off;
    p.tab_wide = op->tab_wide;
    p.tab_cb = op->tab_cb;
    cudaStream_t st = op->hs.stream();
    SlabBuild sb{};
    sb.wc = wc;
    sb.n_pass = n_pass;
    sb.n_tiles = n_tiles;
    sb.colbits = colbits;
    sb.n_slots = n_slots;
    sb.scaled = scaled ? 1 : 0;
    sb.o_ctr = (int)align16(B.smem_bond);
    // counts and tile offsets; a scaled table's orbit-size bytes and scaled-x buffer (complex128)
    const size_t meta = (size_t)n_pass * sp.dim + (size_t)n_pass * n_tiles * 4 + (scaled ? (size_t)sp.dim * 17 : 0);
    if ((double)meta > (double)max_bytes) {
        op->free_slabs();
        return EDGPU_OK;
    }
    DevBuf<unsigned> tile_sum;
    DevBuf<unsigned short> d_amp;
    DevBuf<long long> d_base;
    try {
        EDGPU_CUDA(cudaMalloc(&S.counts, std::max<size_t>((size_t)n_pass * sp.dim, 16)));
        EDGPU_CUDA(cudaMalloc(&S.off, std::max<size_t>((size_t)n_pass * n_tiles * 4, 16)));
        tile_sum.ensure((size_t)n_pass * n_tiles);
        if (scaled) {
            EDGPU_CUDA(cudaMalloc(&S.cls, (size_t)sp.dim));
            S.xsc.ensure(2 * (size_t)sp.dim);
        }
        sb.cls = S.cls;
        sb.counts = S.counts;
        sb.tile_sum = tile_sum.p;
        hx_slab_build(sp.w32, prec, 1, p, sb, (size_t)sb.o_ctr + (size_t)n_pass * HX_THREADS, st);
        std::vector<unsigned long long> totals;
        hx_slab_scan(tile_sum.p, S.off, n_pass, n_tiles, totals, st);
        S.base.assign((size_t)n_pass + 1, 0);
        for (int q = 0; q < n_pass; ++q) {
            require(totals[q] < ((unsigned long long)1 << 32), EDGPU_ERR_ARG, "slab pass with 2^32 entries or more");
            S.base[q + 1] = S.base[q] + (long long)totals[q];
        }
        S.n = S.base[n_pass];
        if ((double)meta + (double)S.n * 4.0 > (double)max_bytes) {
            op->free_slabs();
            return EDGPU_OK;
        }
        EDGPU_CUDA(cudaMalloc(&S.tab, std::max<size_t>((size_t)S.n * 4, 16)));
        d_amp.ensure((size_t)n_slots);
        d_base.ensure((size_t)n_pass);
        EDGPU_CUDA(cudaMemcpyAsync(d_amp.p, amp_id.data(), (size_t)n_slots * 2, cudaMemcpyHostToDevice, st));
        EDGPU_CUDA(cudaMemcpyAsync(d_base.p, S.base.data(), (size_t)n_pass * 8, cudaMemcpyHostToDevice, st));
        sb.off = S.off;
        sb.base = d_base.p;
        sb.tab = S.tab;
        sb.amp_id = d_amp.p;
        hx_slab_build(sp.w32, prec, 2, p, sb, (size_t)sb.o_ctr + (size_t)n_pass * HX_THREADS * 4, st);
        EDGPU_CUDA(cudaStreamSynchronize(st));
        S.n_pass = n_pass;
        S.wc = wc;
        S.colbits = colbits;
        S.n_ids = (int)n_ids;
        S.scaled = scaled ? 1 : 0;
        if (scaled && n_pass > 1) op->ensure_slab_events(n_pass);
        if (scaled) {
            std::vector<float> f(2 * (size_t)S.nd);
            std::vector<double> d(2 * (size_t)S.nd);
            for (int k = 0; k < S.nd; ++k) {
                d[k] = std::sqrt((double)S.divs[k]);
                d[S.nd + k] = 1.0 / std::sqrt((double)S.divs[k]);
                f[k] = (float)d[k];
                f[S.nd + k] = (float)d[S.nd + k];
            }
            S.sc32.ensure(f.size());
            S.sc64.ensure(d.size());
            EDGPU_CUDA(cudaMemcpy(S.sc32.p, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
            EDGPU_CUDA(cudaMemcpy(S.sc64.p, d.data(), d.size() * sizeof(double), cudaMemcpyHostToDevice));
        }
        S.lut.ensure((size_t)n_ids * 2);
        S.lut64.ensure((size_t)n_ids * 2);
        slab_refresh_lut(op);
    } catch (...) {
        cudaStreamSynchronize(st);
        op->free_slabs();
        throw;
    }
    op->slab_use[EDGPU_MIXED] = op->slab_use[EDGPU_FP64] = 1;
    if (built) *built = 1;
    API_END
}

int edgpu_op_free_slabs(edgpu_op oh) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    EDGPU_CUDA(cudaDeviceSynchronize());
    op->free_slabs();
    API_END
}

int edgpu_op_slabs_info(edgpu_op oh, int32_t* passes, int64_t* columns_per_slab, int64_t* entries) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    const bool on = op->slab.tab != nullptr;
    if (passes) *passes = on ? op->slab.n_pass : 0;
    if (columns_per_slab) *columns_per_slab = on ? op->slab.wc : 0;
    if (entries) *entries = on ? op->slab.n : 0;
    API_END
}

int edgpu_op_slab_scaling(edgpu_op oh, int32_t mode, int32_t* scaled) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    require(mode >= -1 && mode <= 2, EDGPU_ERR_ARG, "mode must be -1 (query), 0, 1 or 2");
    if (mode >= 0) op->slab_scaling = mode;
    if (scaled) *scaled = op->slab.tab ? op->slab.scaled : 0;
    API_END
}

int edgpu_op_slab_use(edgpu_op oh, int32_t precision, int32_t use, int32_t* current) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    check_prec(precision);
    require(use >= -1 && use <= 6, EDGPU_ERR_ARG, "use must be -1 (query) or 0 to 6");
    require(use <= 0 || op->slab.tab, EDGPU_ERR_STATE, "no slab table (edgpu_op_build_slabs)");
    if (use >= 0) {
        op->slab_use[precision] = use > 0 ? 1 : 0;
        op->slab_hint[precision] = use > 0 ? use - 1 : 0;
    }
    if (current) *current = op->slab_use[precision] ? 1 + op->slab_hint[precision] : 0;
    API_END
}

int edgpu_pair_classes_of_terms(int32_t n_bits, int32_t n_terms, const uint64_t* masks, const uint64_t* rows,
                                const uint64_t* cols, const double* amps, int32_t cap_classes, int32_t* n_classes,
                                int32_t* info, uint64_t* comps, uint64_t* flips, double* class_amps) {
    API_BEGIN
    require(n_bits >= 1 && n_bits <= 64, EDGPU_ERR_ARG, "n_bits = " + std::to_string(n_bits) + " is not in [1, 64]");
    require(n_terms >= 0 && n_classes, EDGPU_ERR_ARG, "bad arguments");
    require(n_terms == 0 || (masks && rows && cols && amps), EDGPU_ERR_ARG, "null term arrays");
    Layout lay;
    lay.n_sites = lay.nbits = n_bits;
    lay.bw.assign(n_bits, 1);
    std::vector<uint64_t> bm, br, bf;
    std::vector<double> ba;
    for (int t = 0; t < n_terms; ++t) {
        if (rows[t] == cols[t]) continue;
        bm.push_back(masks[t]);
        br.push_back(rows[t]);
        bf.push_back(rows[t] ^ cols[t]);
        ba.push_back(amps[2 * t]);
        ba.push_back(amps[2 * t + 1]);
    }
    BondClasses bc;
    *n_classes = build_bond_classes(lay, bm, br, bf, ba, bc) ? bc.ncls : 0;
    if (*n_classes > 0 && cap_classes >= *n_classes) {
        for (int c = 0; c < bc.ncls; ++c) {
            if (info) info[c] = bc.info[c];
            for (int k = 0; k < BOND_MAXC; ++k)
                for (int f = 0; f < 3; ++f)
                    if (comps) comps[((size_t)c * BOND_MAXC + k) * 3 + f] = bc.comp[((size_t)c * BOND_MAXC + k) * 4 + f];
        }
        if (flips) std::copy(bc.flip.begin(), bc.flip.end(), flips);
        if (class_amps) std::copy(bc.amp.begin(), bc.amp.end(), class_amps);
    }
    API_END
}

int edgpu_op_pair_classes(edgpu_op oh, int32_t* n_classes, int32_t* n_components) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    std::vector<uint64_t> bm, br, bf;
    std::vector<double> ba;
    for (int t = 0; t < op->T; ++t) {
        if (op->rows[t] == op->cols[t]) continue;
        bm.push_back(op->masks[t]);
        br.push_back(op->rows[t]);
        bf.push_back(op->rows[t] ^ op->cols[t]);
        const double c = op->coupl[op->cid[t]];
        ba.push_back(op->unit[2 * t] * c);
        ba.push_back(op->unit[2 * t + 1] * c);
    }
    BondClasses bc;
    int nc = 0, ncomp = 0;
    if (build_bond_classes(op->space->lay, bm, br, bf, ba, bc)) {
        nc = bc.ncls;
        for (int c = 0; c < nc; ++c) ncomp += bc.info[c] & 0xff;
    }
    if (n_classes) *n_classes = nc;
    if (n_components) *n_components = ncomp;
    API_END
}

int edgpu_op_autotune(edgpu_op oh, int32_t precision, int32_t* rows_per_tile_out, double* best_ms_out) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    check_prec(precision);
    const int64_t n = op->space->dim;
    // Candidates: the term scan with 1, 2 or 4 lanes per row (and the queued schedule with 32 or 16
    // rows per warp tile when there is no parent-state map); where the pair-flip schedule applies
    // (and the caller allows it), that schedule with 2 or 4 targets per step (4 with a map or a
    // target table) and 1, 2 or 4 lanes per row, and its target-table flavour (one lane per row).
    // With a slab table (mixed precision), also its multi-pass product.
    struct Cand { int pair, nt, table, rows, pf, uni, slab = 0, hint = 0; };
    std::vector<Cand> cands;
    build_blob(op, precision, 0, 0);
    const bool pair_ok = op->blob[precision][0][0].tmpl.bond_ncls > 0 && op->pair_allowed;
    const bool mapped = op->space->d_map != nullptr;
    if (pair_ok) {
        if (op->slab.tab)
            for (int hint : {0, 1, 2, 3, 4, 5}) cands.push_back({1, 4, 1, -1, 0, 0, 1, hint});
        if (op->d_tab) {
            for (int nt : {8, 4, 2})
                for (int pf : {0, 4, 64}) cands.push_back({1, nt, 1, -1, pf, 0});
            for (int nt : {8, 4})
                for (int pf : {0, 4}) cands.push_back({1, nt, 1, -1, pf, 1});
        }
        for (int nt : (mapped ? std::vector<int>{4, 2} : std::vector<int>{2}))
            for (int r : {-1, -2, -4}) cands.push_back({1, nt, 0, r, 0, 0});
    }
    for (int r : {-1, -2, -4}) cands.push_back({0, 2, 0, r, 0, 0});
    if (!mapped)
        for (int r : {32, 16}) cands.push_back({0, 2, 0, r, 0, 0});
    Cand best = cands.front();
    double best_ms = 1e30;
    const int keep_pair = op->pair_use[precision], keep_nt = op->pair_nt[precision], keep_tab = op->tab_use[precision];
    const int keep_uni = op->tab_uni[precision], keep_slab = op->slab_use[precision], keep_hint = op->slab_hint[precision];
    if (n > 0) {
        const size_t vs = precision == EDGPU_FP64 ? 16 : 8;
        void *x = nullptr, *y = nullptr;
        EDGPU_CUDA(cudaMalloc(&x, n * vs));
        EDGPU_CUDA(cudaMalloc(&y, n * vs));
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        try {
            EDGPU_CUDA(cudaMemsetAsync(x, 0, n * vs, op->hs.stream()));
            for (const Cand& c : cands) {
                op->pair_use[precision] = c.pair;
                op->pair_nt[precision] = c.nt;
                op->tab_use[precision] = c.table;
                op->tab_pf[precision] = c.pf;
                op->tab_uni[precision] = c.uni;
                op->slab_use[precision] = c.slab;
                op->slab_hint[precision] = c.hint;
                launch_product(op, precision, 0, 0, x, y, 0, nullptr, nullptr, op->hs.stream(), nullptr, c.rows);
                // one timed launch, then two back-to-back bursts of enough launches to cover about 2 ms
                // (1 to 50 per burst), as a solver issues them; the faster burst's time per launch
                float t_min = 1e30f;
                EDGPU_CUDA(cudaEventRecord(e0, op->hs.stream()));
                launch_product(op, precision, 0, 0, x, y, 0, nullptr, nullptr, op->hs.stream(), nullptr, c.rows);
                EDGPU_CUDA(cudaEventRecord(e1, op->hs.stream()));
                EDGPU_CUDA(cudaEventSynchronize(e1));
                float ms1 = 0.f;
                cudaEventElapsedTime(&ms1, e0, e1);
                const int reps = std::max(1, std::min(50, (int)(2.0f / std::max(ms1, 1e-3f))));
                for (int burst = 0; burst < 2; ++burst) {
                    EDGPU_CUDA(cudaEventRecord(e0, op->hs.stream()));
                    for (int k = 0; k < reps; ++k)
                        launch_product(op, precision, 0, 0, x, y, 0, nullptr, nullptr, op->hs.stream(), nullptr, c.rows);
                    EDGPU_CUDA(cudaEventRecord(e1, op->hs.stream()));
                    EDGPU_CUDA(cudaEventSynchronize(e1));
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    t_min = std::min(t_min, ms / reps);
                }
                if (t_min < best_ms) {
                    best_ms = t_min;
                    best = c;
                }
            }
        } catch (...) {
            op->pair_use[precision] = keep_pair;
            op->pair_nt[precision] = keep_nt;
            op->tab_use[precision] = keep_tab;
            op->tab_uni[precision] = keep_uni;
            op->slab_use[precision] = keep_slab;
            op->slab_hint[precision] = keep_hint;
            cudaFree(x);
            cudaFree(y);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            throw;
        }
        cudaFree(x);
        cudaFree(y);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    op->pair_use[precision] = best.pair;
    op->pair_nt[precision] = best.nt;
    op->tab_use[precision] = best.table ? 1 : (op->d_tab ? 0 : 1);
    op->tab_pf[precision] = best.pf;
    op->tab_uni[precision] = best.uni;
    op->slab_use[precision] = best.slab;
    op->slab_hint[precision] = best.hint;
    op->tuned_rows[precision] = best.rows;
    if (rows_per_tile_out) *rows_per_tile_out = best.rows;
    if (best_ms_out) *best_ms_out = best_ms;
    API_END
}

// ---- sparse assembly ---------------------------------------------------------------------------

namespace {

// Count (row_ptr == null) or fill the CSR rows [row0, row0 + n_run) of H (transpose == 0) or of H^T
// (transpose == 1, as the conjugated rows of H^dagger) on the device.
void sparse_pass(edgpu_op_s* op, int transpose, double tol, long long row0, long long n_run, long long* d_counts,
                 const long long* d_row_ptr, long long* d_cols, double2* d_vals) {
    build_blob(op, EDGPU_FP64, transpose, 0);
    const Blob& B = op->blob[EDGPU_FP64][transpose][0];
    const HxParams& p = B.tmpl;
    const size_t t1p = (size_t)((p.T_o + 2) & ~1);   // T_o + 1 rounded up to even (see hx_sparse_kernel)
    require(p.warp_base % 16 == 0, EDGPU_ERR_ARG, "internal: unaligned sparse scratch");
    const size_t smem = (size_t)p.warp_base + 4 * t1p * 48;
    require(smem <= 227 * 1024, EDGPU_ERR_ARG, "too many off-diagonal terms per row for sparse assembly");
    if (n_run <= 0) return;
    if (op->space->w32)
        hx_sparse_launch_w32(B.gk, p, row0, n_run, transpose, tol, d_counts, d_row_ptr, d_cols, d_vals, smem, op->hs.stream());
    else
        hx_sparse_launch_w64(B.gk, p, row0, n_run, transpose, tol, d_counts, d_row_ptr, d_cols, d_vals, smem, op->hs.stream());
}

}  // namespace

int edgpu_op_sparse(edgpu_op oh, int32_t transpose, double tol, int64_t* nnz, int64_t* row_ptr, int64_t* col_idx,
                    double* values) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    require(nnz && tol >= 0.0 && (transpose == 0 || transpose == 1), EDGPU_ERR_ARG, "bad sparse arguments");
    require(!row_ptr || (col_idx && values), EDGPU_ERR_ARG, "row_ptr, col_idx and values go together");
    const long long n = op->space->dim;
    DevBuf<long long> counts, rp, cols;
    DevBuf<double> vals;
    counts.ensure(std::max<long long>(n, 1));
    sparse_pass(op, transpose, tol, 0, n, counts.p, nullptr, nullptr, nullptr);
    std::vector<long long> hc(n);
    if (n) EDGPU_CUDA(cudaMemcpyAsync(hc.data(), counts.p, n * sizeof(long long), cudaMemcpyDeviceToHost, op->hs.stream()));
    EDGPU_CUDA(cudaStreamSynchronize(op->hs.stream()));
    std::vector<long long> hp(n + 1, 0);
    for (long long i = 0; i < n; ++i) hp[i + 1] = hp[i] + hc[i];
    *nnz = hp[n];
    if (!row_ptr) return EDGPU_OK;
    for (long long i = 0; i <= n; ++i) row_ptr[i] = hp[i];
    if (hp[n] == 0) return EDGPU_OK;
    rp.ensure(n + 1);
    cols.ensure(hp[n]);
    vals.ensure(2 * hp[n]);
    EDGPU_CUDA(cudaMemcpyAsync(rp.p, hp.data(), (n + 1) * sizeof(long long), cudaMemcpyHostToDevice, op->hs.stream()));
    sparse_pass(op, transpose, tol, 0, n, nullptr, rp.p, cols.p, (double2*)vals.p);
    EDGPU_CUDA(cudaMemcpyAsync(col_idx, cols.p, hp[n] * sizeof(long long), cudaMemcpyDeviceToHost, op->hs.stream()));
    EDGPU_CUDA(cudaMemcpyAsync(values, vals.p, 2 * hp[n] * sizeof(double), cudaMemcpyDeviceToHost, op->hs.stream()));
    EDGPU_CUDA(cudaStreamSynchronize(op->hs.stream()));
    API_END
}

int edgpu_op_get_row(edgpu_op oh, int32_t transpose, int64_t row, double tol, int64_t cap, int64_t* count,
                     int64_t* col_idx, double* values) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    require(count && tol >= 0.0 && (transpose == 0 || transpose == 1) && cap >= 0, EDGPU_ERR_ARG,
            "bad get_row arguments");
    require(row >= 0 && row < op->space->dim, EDGPU_ERR_BOUNDS, "row index out of range");
    DevBuf<long long> c, rp, cols;
    DevBuf<double> vals;
    c.ensure(1);
    sparse_pass(op, transpose, tol, row, 1, c.p, nullptr, nullptr, nullptr);
    long long k = 0;
    EDGPU_CUDA(cudaMemcpyAsync(&k, c.p, sizeof(long long), cudaMemcpyDeviceToHost, op->hs.stream()));
    EDGPU_CUDA(cudaStreamSynchronize(op->hs.stream()));
    *count = k;
    if (!col_idx || k == 0) return EDGPU_OK;
    require(values && cap >= k, EDGPU_ERR_DIM, "output buffers hold fewer entries than the row");
    const long long zero = 0;
    rp.ensure(1);
    cols.ensure(k);
    vals.ensure(2 * k);
    EDGPU_CUDA(cudaMemcpyAsync(rp.p, &zero, sizeof(long long), cudaMemcpyHostToDevice, op->hs.stream()));
    sparse_pass(op, transpose, tol, row, 1, nullptr, rp.p, cols.p, (double2*)vals.p);
    EDGPU_CUDA(cudaMemcpyAsync(col_idx, cols.p, k * sizeof(long long), cudaMemcpyDeviceToHost, op->hs.stream()));
    EDGPU_CUDA(cudaMemcpyAsync(values, vals.p, 2 * k * sizeof(double), cudaMemcpyDeviceToHost, op->hs.stream()));
    EDGPU_CUDA(cudaStreamSynchronize(op->hs.stream()));
    API_END
}

int edgpu_op_count_nnz(edgpu_op oh, int64_t* n_targets, int64_t* nnz_off) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    require(n_targets && nnz_off, EDGPU_ERR_ARG, "null output");
    std::vector<uint64_t> m, r, f;
    for (int t = 0; t < op->T; ++t)
        if (op->rows[t] != op->cols[t]) {
            m.push_back(op->masks[t]);
            r.push_back(op->rows[t]);
            f.push_back(op->rows[t] ^ op->cols[t]);
        }
    count_nnz(*op->space, (int)m.size(), m.data(), r.data(), f.data(), n_targets, nnz_off, op->hs.stream());
    API_END
}

// ---- products ----------------------------------------------------------------------------------

static bool is_pinned(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// The device's address of pinned host memory (null when the device cannot address it): kernels then
// read and write the host buffer directly over the host link, without a staging copy.
static void* device_alias(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Wait for the library stream by polling an event (lower wake-up latency than a blocking wait for the
// short products of the host-buffer entry points).
static void wait_stream(cudaStream_t st) {
    static thread_local cudaEvent_t ev = nullptr;
    if (!ev) EDGPU_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    EDGPU_CUDA(cudaEventRecord(ev, st));
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {   // poll for up to 2 ms, then block
        const cudaError_t e = cudaEventQuery(ev);
        if (e == cudaSuccess) return;
        if (e != cudaErrorNotReady) throw Error(EDGPU_ERR_CUDA, std::string("wait: ") + cudaGetErrorString(e));
        if (std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(2)) break;
    }
    EDGPU_CUDA(cudaEventSynchronize(ev));
}

static void host_product_issue(edgpu_op_s* op, int prec, int dir, const double* x, double* y, int64_t n,
                               int accumulate, bool conj_io, cudaStream_t st);

// The host-buffer product: copies in, the product (with complex64 conversions in mixed precision),
// copies out.  With pinned host buffers the sequence is captured once into a CUDA graph per set of
// buffers and replayed; pageable buffers take the plain stream path.
static void host_product(edgpu_op_s* op, int prec, int dir, const double* x, double* y, int64_t n, int accumulate,
                         bool conj_io) {
    cudaStream_t st = op->hs.stream();
    op->x64.ensure(2 * n);
    op->y64.ensure(2 * n);
    if (prec == EDGPU_MIXED) {
        op->x32.ensure(2 * n);
        op->y32.ensure(2 * n);
    }
    if (!is_pinned(x) || !is_pinned(y)) {
        host_product_issue(op, prec, dir, x, y, n, accumulate, conj_io, st);
        wait_stream(st);
        return;
    }
    build_blob(op, prec, dir, 0);
    // the graph replays the launches of this call: the key holds everything they depend on (buffers,
    // tables, the schedule)
    const std::vector<const void*> key = {(const void*)x, (const void*)y, (const void*)(intptr_t)n,
                                          (const void*)(intptr_t)(prec * 8 + dir * 4 + accumulate * 2 + (conj_io ? 1 : 0)),
                                          (const void*)op->x64.p, (const void*)op->y64.p,
                                          (const void*)op->x32.p, (const void*)op->y32.p,
                                          (const void*)op->space->d_map, (const void*)(uintptr_t)op->gen,
                                          (const void*)(intptr_t)op->tuned_rows[prec],
                                          op->d_tab, (const void*)op->slab.tab,
                                          (const void*)(intptr_t)(op->pair_allowed + 2 * op->pair_use[prec] +
                                                                  4 * op->pair_nt[prec] + 64 * op->tab_use[prec] +
                                                                  128 * op->tab_uni[prec] + 256 * op->slab_use[prec] +
                                                                  512 * op->tab_pf[prec] + (1 << 20) * op->slab_hint[prec]),
                                          (const void*)(intptr_t)slab_row_blocks(op, prec, n)};
    auto it = op->host_graphs.find(key);
    if (it == op->host_graphs.end()) {
        cudaStream_t cap = nullptr;
        EDGPU_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            try {
                host_product_issue(op, prec, dir, x, y, n, accumulate, conj_io, cap);
            } catch (...) {
                cudaStreamEndCapture(cap, &graph);
                if (graph) cudaGraphDestroy(graph);
                cudaStreamDestroy(cap);
                throw;
            }
            e = cudaStreamEndCapture(cap, &graph);
        }
        cudaStreamDestroy(cap);
        cudaGraphExec_t exec = nullptr;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("host product graph: ") + cudaGetErrorString(e));
        if (op->host_graphs.size() >= 16) {   // bounded cache
            for (auto& kv : op->host_graphs) cudaGraphExecDestroy(kv.second);
            op->host_graphs.clear();
        }
        it = op->host_graphs.emplace(key, exec).first;
    }
    EDGPU_CUDA(cudaGraphLaunch(it->second, st));
    wait_stream(st);
}

static void host_product_issue(edgpu_op_s* op, int prec, int dir, const double* x, double* y, int64_t n,
                               int accumulate, bool conj_io, cudaStream_t st) {
    if (prec == EDGPU_MIXED && !conj_io) {
        // pinned buffers the device can address: the complex64 conversion kernels read x from and
        // write y to host memory directly (no staging copies)
        const double* xd = (const double*)device_alias(x);
        double* yd = (double*)device_alias(y);
        const int rows = op->tuned_rows[prec] ? op->tuned_rows[prec] : -1;
        if (xd && yd && slab_active(op, prec, dir, 0, (rows > 0 && op->space->d_map) ? -1 : rows)) {
            // the slab passes: slab q of x is converted on a second stream while the earlier passes
            // run (pass q waits for it; the last pass, which adds the diagonal term, for all of x), and
            // the last pass writes the complex128 result to the host buffer
            build_blob(op, prec, dir, 0);
            const auto& S = op->slab;
            op->ensure_slab_events(S.n_pass);
            EDGPU_CUDA(cudaEventRecord(op->aux_fork, st));
            EDGPU_CUDA(cudaStreamWaitEvent(op->aux_st, op->aux_fork, 0));
            // (on a scaled table the conversion writes the scaled x to the table's buffer)
            float* xdst = S.scaled ? (float*)S.xsc.p : op->x32.p;
            for (int q = 0; q < S.n_pass; ++q) {
                const int64_t c0 = (int64_t)q * S.wc, c1 = std::min<int64_t>(n, c0 + S.wc);
                if (S.scaled) launch_slab_xscale_c128_c64(xd, S.cls, S.sc32.p, xdst, c0, c1, op->aux_st);
                else launch_c128_to_c64(c1 - c0, xd + 2 * c0, xdst + 2 * c0, op->aux_st);
                EDGPU_CUDA(cudaEventRecord(op->slab_ready[q], op->aux_st));
            }
            launch_slab_passes(op, prec, op->blob[prec][dir][0], xdst, op->y32.p, 0, yd, accumulate, st,
                               op->slab_ready.data(), true, slab_row_blocks(op, prec, n));
            return;
        }
        if (xd && yd) {
            launch_c128_to_c64(n, xd, op->x32.p, st);
            // the pair-flip kernel writes the complex128 result to the host buffer itself
            bool fused = false;
            launch_product(op, prec, dir, 0, op->x32.p, op->y32.p, 0, nullptr, nullptr, st, nullptr, 0, yd,
                           accumulate, &fused);
            if (!fused) launch_c64_to_c128(n, op->y32.p, yd, accumulate, st);
            return;
        }
    }
    if (prec == EDGPU_FP64 && !conj_io) {
        // pinned buffers the device can address: x is copied in (the product gathers it at random),
        // and the product writes (or, for apply!, updates) y in the host buffer itself
        double* yd = (double*)device_alias(y);
        if (yd) {
            const int rows = op->tuned_rows[prec] ? op->tuned_rows[prec] : -1;
            if (slab_active(op, prec, dir, 0, (rows > 0 && op->space->d_map) ? -1 : rows)) {
                // the slab passes add into the device buffer and the last writes the host buffer; x is
                // copied in slab by slab on a second stream (one copy per slab) while the earlier
                // passes run
                build_blob(op, prec, dir, 0);
                const auto& S = op->slab;
                op->ensure_slab_events(S.n_pass);
                EDGPU_CUDA(cudaEventRecord(op->aux_fork, st));
                EDGPU_CUDA(cudaStreamWaitEvent(op->aux_st, op->aux_fork, 0));
                // (on a scaled table each copied slab is then scaled into the table's buffer)
                for (int q = 0; q < S.n_pass; ++q) {
                    const int64_t c0 = (int64_t)q * S.wc, c1 = std::min<int64_t>(n, c0 + S.wc);
                    EDGPU_CUDA(cudaMemcpyAsync(op->x64.p + 2 * c0, x + 2 * c0, (size_t)(c1 - c0) * 16,
                                               cudaMemcpyHostToDevice, op->aux_st));
                    if (S.scaled) launch_slab_xscale(prec, op->x64.p, S.cls, S.sc64.p, S.xsc.p, c0, c1, op->aux_st);
                    EDGPU_CUDA(cudaEventRecord(op->slab_ready[q], op->aux_st));
                }
                launch_slab_passes(op, prec, op->blob[prec][dir][0], S.scaled ? (const void*)S.xsc.p : op->x64.p,
                                   op->y64.p, 0, yd, accumulate, st, op->slab_ready.data(), true,
                                   slab_row_blocks(op, prec, n));
                return;
            }
            EDGPU_CUDA(cudaMemcpyAsync(op->x64.p, x, n * 16, cudaMemcpyHostToDevice, st));
            launch_product(op, prec, dir, 0, op->x64.p, yd, accumulate, nullptr, nullptr, st);
            return;
        }
    }
    EDGPU_CUDA(cudaMemcpyAsync(op->x64.p, x, n * 16, cudaMemcpyHostToDevice, st));
    if (conj_io) launch_conj_c128(n, op->x64.p, st);
    if (accumulate) {
        EDGPU_CUDA(cudaMemcpyAsync(op->y64.p, y, n * 16, cudaMemcpyHostToDevice, st));
        if (conj_io) launch_conj_c128(n, op->y64.p, st);
    }
    if (prec == EDGPU_FP64) {
        launch_product(op, prec, dir, 0, op->x64.p, op->y64.p, accumulate, nullptr, nullptr, st);
    } else {
        launch_c128_to_c64(n, op->x64.p, op->x32.p, st);
        launch_product(op, prec, dir, 0, op->x32.p, op->y32.p, 0, nullptr, nullptr, st);
        launch_c64_to_c128(n, op->y32.p, op->y64.p, accumulate, st);
    }
    if (conj_io) launch_conj_c128(n, op->y64.p, st);
    EDGPU_CUDA(cudaMemcpyAsync(y, op->y64.p, n * 16, cudaMemcpyDeviceToHost, st));
}

int edgpu_mul(edgpu_op oh, int32_t precision, const double* x, double* y, int64_t n, int32_t accumulate) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    check_prec(precision);
    check_dim(op, n, "state");
    if (n == 0) return EDGPU_OK;
    require(x && y, EDGPU_ERR_ARG, "null vector");
    host_product(op, precision, 0, x, y, n, accumulate ? 1 : 0, false);
    API_END
}

int edgpu_mul_device(edgpu_op oh, int32_t precision, const void* x, void* y, int64_t n, int32_t accumulate,
                     void* stream) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    check_prec(precision);
    check_dim(op, n, "state");
    if (n == 0) return EDGPU_OK;
    require(x && y, EDGPU_ERR_ARG, "null vector");
    require(x != y, EDGPU_ERR_ARG, "out and state must be distinct buffers");
    launch_product(op, precision, 0, 0, x, y, accumulate ? 1 : 0, nullptr, nullptr, pick_stream(stream));
    API_END
}

int edgpu_mul_transpose(edgpu_op oh, int32_t precision, const double* x, double* y, int64_t n, int32_t accumulate) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    check_prec(precision);
    check_dim(op, n, "state");
    if (n == 0) return EDGPU_OK;
    require(x && y, EDGPU_ERR_ARG, "null vector");
    // transpose(A) x = conj(A^dagger conj(x))
    host_product(op, precision, 1, x, y, n, accumulate ? 1 : 0, true);
    API_END
}

namespace {

// Site maps and flip masks of every element of a space's group, on the host.
void host_group(const Space& s, std::vector<std::vector<int>>& maps, std::vector<uint64_t>& flips) {
    const Group& g = s.group;
    const int n = s.lay.n_sites;
    std::vector<int> id(n);
    for (int i = 0; i < n; ++i) id[i] = i;
    if (!s.reduced || g.kind == GK_TRIVIAL) {
        maps.push_back(id);
        flips.push_back(0);
    } else if (g.kind == GK_TORUS) {
        for (int b = 0; b < g.L2; ++b)
            for (int a = 0; a < g.L1; ++a) {
                std::vector<int> m(n);
                for (int y = 0; y < g.L2; ++y)
                    for (int x = 0; x < g.L1; ++x) m[x + g.L1 * y] = (x + a) % g.L1 + g.L1 * ((y + b) % g.L2);
                maps.push_back(m);
                flips.push_back(0);
            }
    } else {
        for (int e = 0; e < g.G; ++e) {
            maps.emplace_back(g.maps.begin() + (size_t)e * n, g.maps.begin() + (size_t)(e + 1) * n);
            flips.push_back(e < (int)g.flips.size() ? g.flips[e] : 0ull);
        }
    }
}

uint64_t permute_bits(uint64_t v, const std::vector<int>& m, const Layout& lay) {
    uint64_t r = 0;
    for (int i = 0; i < lay.n_sites; ++i) {
        const uint64_t w = lay.bw[i] >= 64 ? ~0ull : ((1ull << lay.bw[i]) - 1ull);
        r |= ((v >> lay.off[i]) & w) << lay.off[m[i]];
    }
    return r;
}

// Whether every group element maps the operator's term table onto itself (equal summed amplitude per
// (mask, row, col)).  Then the reduced row and column iterators give transposed matrices.
bool op_invariant(edgpu_op_s* op) {
    if (op->invariant_gen == op->gen) return op->invariant;
    const Space& s = *op->space;
    std::vector<std::vector<int>> maps;
    std::vector<uint64_t> flips;
    host_group(s, maps, flips);
    struct K {
        uint64_t m, r, c;
        bool operator<(const K& o) const { return m != o.m ? m < o.m : (r != o.r ? r < o.r : c < o.c); }
    };
    std::map<K, std::pair<double, double>> base;
    double scale = 0.0;
    for (int t = 0; t < op->T; ++t) {
        const double c = op->coupl[op->cid[t]];
        auto& a = base[K{op->masks[t], op->rows[t], op->cols[t]}];
        a.first += op->unit[2 * t] * c;
        a.second += op->unit[2 * t + 1] * c;
        scale = std::max(scale, std::hypot(op->unit[2 * t] * c, op->unit[2 * t + 1] * c));
    }
    bool inv = true;
    for (size_t e = 0; e < maps.size() && inv; ++e) {
        std::map<K, std::pair<double, double>> img;
        for (const auto& kv : base) {
            const uint64_t m = permute_bits(kv.first.m, maps[e], s.lay);
            const uint64_t f = flips[e] & m;
            auto& a = img[K{m, permute_bits(kv.first.r, maps[e], s.lay) ^ f, permute_bits(kv.first.c, maps[e], s.lay) ^ f}];
            a.first += kv.second.first;
            a.second += kv.second.second;
        }
        for (const auto& kv : img) {
            auto it = base.find(kv.first);
            const double re = it == base.end() ? 0.0 : it->second.first;
            const double im = it == base.end() ? 0.0 : it->second.second;
            if (std::hypot(kv.second.first - re, kv.second.second - im) > 1e-12 * std::max(scale, 1e-300)) inv = false;
        }
        if (img.size() != base.size()) inv = inv && false;
    }
    op->invariant = inv;
    op->invariant_gen = op->gen;
    return inv;
}

}  // namespace

int edgpu_op_is_invariant(edgpu_op oh, int32_t* invariant) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    require(invariant, EDGPU_ERR_ARG, "null output");
    *invariant = op_invariant(op) ? 1 : 0;
    API_END
}

int edgpu_mul_adjoint_device(edgpu_op oh, int32_t precision, const void* x, void* y, int64_t n, int32_t accumulate,
                             void* stream) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    check_prec(precision);
    check_dim(op, n, "state");
    if (n == 0) return EDGPU_OK;
    require(x && y && x != y, EDGPU_ERR_ARG, "bad vectors");
    cudaStream_t st = pick_stream(stream);
    if (op_invariant(op)) {
        // the adjoint term table, applied by the row formula, is the adjoint of the product's matrix
        launch_product(op, precision, 1, 0, x, y, accumulate ? 1 : 0, nullptr, nullptr, st);
        return EDGPU_OK;
    }
    if (op->d_adj_tab) {
        // the adjoint target table: every column gathers its run in a fixed order
        build_blob(op, precision, 0, 0);
        const Blob& B = op->blob[precision][0][0];
        HxParams p = B.tmpl_pair;
        p.blob = B.d_pair;
        p.blob_words16 = (int)(B.smem_bond / 16);
        p.gy = x;
        p.y = y;
        p.diag = B.d_diag;
        p.accumulate = accumulate ? 1 : 0;
        p.adj_off = op->d_adj_off;
        p.adj_tab = op->d_adj_tab;
        SpaceLock space_lk(op->space->hs.mu);
        hx_adj_launch(op->space->w32, precision, p, B.smem_bond, st);
        return EDGPU_OK;
    }
    // terms that do not commute with the group, no adjoint table: the rows of the product's matrix are
    // scattered, y[c] += conj(H[r, c]) x[r] by atomic adds (summation order not fixed)
    const size_t vs = precision == EDGPU_FP64 ? 16 : 8;
    if (!accumulate) EDGPU_CUDA(cudaMemsetAsync(y, 0, n * vs, st));
    build_blob(op, precision, 0, 0);
    const Blob& B = op->blob[precision][0][0];
    HxParams p = B.tmpl;
    p.gy = x;
    p.y = y;
    const int blocks = (int)std::max<long long>(1, std::min<long long>((n + HX_THREADS - 1) / HX_THREADS, 152ll * 32));
    if (op->space->w32) hx_scatter_launch_w32(B.gk, precision, p, blocks, B.smem_rows, st);
    else hx_scatter_launch_w64(B.gk, precision, p, blocks, B.smem_rows, st);
    API_END
}

int edgpu_op_grad_kernel(edgpu_op oh, int32_t precision, int32_t* kind) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    check_prec(precision);
    require(kind, EDGPU_ERR_ARG, "null output");
    build_blob(op, precision, 0, 1);
    const Blob& B = op->blob[precision][0][1];
    const size_t gsmem = align16(B.smem_bond) + pair_grad_acc_bytes(op, precision);
    if (B.tmpl.o_bunit >= 0 && op->pair_allowed && (op->d_tab || op->space->d_map) && gsmem <= 200 * 1024)
        *kind = op->d_tab ? 2 : 1;
    else
        *kind = ((size_t)B.tmpl.o_grad + (size_t)op->n_coupl * HX_THREADS * 8 <= 200 * 1024) ? 0 : -1;
    API_END
}

int edgpu_coupling_grad_device(edgpu_op oh, int32_t precision, const void* x, const void* gy, void* y, int64_t n,
                               double* grad_out, void* stream) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    check_prec(precision);
    check_dim(op, n, "state");
    require(grad_out, EDGPU_ERR_ARG, "null gradient output");
    if (n == 0) {
        for (int c = 0; c < op->n_coupl; ++c) grad_out[c] = 0.0;
        return EDGPU_OK;
    }
    require(x && gy, EDGPU_ERR_ARG, "null vector");
    cudaStream_t st = pick_stream(stream);
    void* yy = y;
    if (!yy) {
        if (precision == EDGPU_FP64) {
            op->z64.ensure(2 * n);
            yy = op->z64.p;
        } else {
            op->y32.ensure(2 * n);
            yy = op->y32.p;
        }
    }
    build_blob(op, precision, 0, 1);
    build_blob(op, precision, 0, 0);   // the forward tables (diagonal), so that every gradient kernel finds them
    // partial sums of either gradient kernel: at most 8 resident blocks of 256 threads per SM
    const int max_blocks = std::max(op->blob[precision][0][1].max_blocks, 8 * std::max(1, g_sm_count));
    op->grad_partial.ensure((size_t)max_blocks * op->n_coupl);
    op->grad_dev.ensure(op->n_coupl);
    int blocks = 0;
    launch_product(op, precision, 0, 1, x, yy, 0, gy, op->grad_partial.p, st, &blocks);
    launch_reduce_grad(blocks, op->n_coupl, op->grad_partial.p, op->grad_dev.p, st);
    EDGPU_CUDA(cudaMemcpyAsync(grad_out, op->grad_dev.p, op->n_coupl * sizeof(double), cudaMemcpyDeviceToHost, st));
    EDGPU_CUDA(cudaStreamSynchronize(st));
    API_END
}

// ---- batched sectors ---------------------------------------------------------------------------

namespace {

// Common tables of a batch, checked for sameness: one term table, basis layout and symmetry group.
void batch_prepare(edgpu_batch_s* b, int prec) {
    edgpu_batch_s::Fused& F = b->fused[prec];
    const int n = (int)b->ops.size();
    std::vector<uint64_t> gens(n);
    for (int i = 0; i < n; ++i) build_blob(b->ops[i], prec, 0, 0);
    for (int i = 0; i < n; ++i) gens[i] = b->ops[i]->gen;
    if (F.ready && F.gens == gens) return;
    b->drop(prec);
    const edgpu_op_s* o0 = b->ops[0];
    const Space& s0 = *o0->space;
    for (int i = 1; i < n; ++i) {
        const edgpu_op_s* o = b->ops[i];
        const Space& s = *o->space;
        const bool same = s.w32 == s0.w32 && s.sb == s0.sb && s.lay.nbits == s0.lay.nbits &&
                          s.group.kind == s0.group.kind && s.group.G == s0.group.G && s.group.L1 == s0.group.L1 &&
                          s.group.L2 == s0.group.L2 && s.group.w == s0.group.w && s.group.maps == s0.group.maps &&
                          s.group.flips == s0.group.flips && o->T == o0->T && o->masks == o0->masks &&
                          o->rows == o0->rows && o->cols == o0->cols && o->unit == o0->unit && o->cid == o0->cid &&
                          o->coupl == o0->coupl && o->blob[prec][0][0].gk == o0->blob[prec][0][0].gk;
        require(same, EDGPU_ERR_ARG,
                "batched operators must share the operator terms, the basis layout and the symmetry group "
                "(operator " + std::to_string(i) + " differs from operator 0)");
    }
    const Blob& B0 = o0->blob[prec][0][0];
    const size_t vsz = prec == EDGPU_FP64 ? 16 : 8;
    // image: the blob's group tables and bond classes, every sector's character tables (phase tables
    // shared between sectors of the same denominator), room for the sector descriptors, the torus row
    // table, then the blob's term records (relocated).  The pair-flip kernel copies the part before the
    // torus row table when it reads parent-state maps or target tables, through it when it
    // canonicalises; the term scan copies everything.  Shared memory left to L1 keeps the lanes' table
    // runs cached.
    const size_t full = (size_t)B0.tmpl.blob_words16 * 16;
    const size_t tstart = std::min(B0.term_start, full);
    std::vector<unsigned char> blob_h(full, 0);
    if (full) EDGPU_CUDA(cudaMemcpy(blob_h.data(), B0.d, full, cudaMemcpyDeviceToHost));
    const size_t bend = std::min(B0.bond_end, B0.pair_host.size());
    F.image.assign(B0.pair_host.begin(), B0.pair_host.begin() + bend);   // group tables, bond classes
    F.o_ph.assign(n, 0);
    F.o_num.assign(n, 0);
    F.want_arg.assign(n, 0);
    int any_arg = 0;
    F.rows = 0;
    std::map<int, int> ph_of_den;
    for (int i = 0; i < n; ++i) {
        const Group& g = b->ops[i]->space->group;
        auto known = ph_of_den.find(g.den);
        if (known != ph_of_den.end()) {
            F.o_ph[i] = known->second;
        } else {
        F.o_ph[i] = (int)F.image.size();
        ph_of_den[g.den] = F.o_ph[i];
        F.image.resize(align16(F.image.size() + g.den * vsz), 0);
        for (int j = 0; j < g.den; ++j) {
            const double ang = 2.0 * M_PI * (double)j / (double)g.den;
            if (prec == EDGPU_FP64) {
                const double v[2] = {std::cos(ang), std::sin(ang)};
                memcpy(&F.image[F.o_ph[i] + j * 16], v, 16);
            } else {
                const float v[2] = {(float)std::cos(ang), (float)std::sin(ang)};
                memcpy(&F.image[F.o_ph[i] + j * 8], v, 8);
            }
        }
        }
        F.o_num[i] = (int)F.image.size();
        F.image.resize(align16(F.image.size() + g.G * 4), 0);
        memcpy(&F.image[F.o_num[i]], g.num.data(), g.G * 4);
        F.want_arg[i] = g.den > 1 ? 1 : 0;
        any_arg |= F.want_arg[i];
        F.rows += b->ops[i]->space->dim;
    }
    F.tmpl = B0.tmpl_pair;   // offsets of the pair image; the torus table and term records are relocated
    F.tmpl.o_sec = (int)F.image.size();
    F.image.resize(align16(F.image.size() + (size_t)n * sizeof(SectorDesc)), 0);
    F.smem_lookup = F.image.size();
    if (F.tmpl.o_rlut >= 0) {
        F.tmpl.o_rlut = (int)F.image.size();
        F.image.insert(F.image.end(), B0.pair_host.begin() + bend, B0.pair_host.end());
        F.image.resize(align16(F.image.size()), 0);
    }
    F.smem_pair = F.image.size();
    const int delta = (int)F.image.size() - (int)tstart;   // term records move by this many bytes
    F.image.insert(F.image.end(), blob_h.begin() + tstart, blob_h.end());
    for (int* o : {&F.tmpl.o_om, &F.tmpl.o_or, &F.tmpl.o_of, &F.tmpl.o_oa, &F.tmpl.o_ou, &F.tmpl.o_oc, &F.tmpl.o_dm,
                   &F.tmpl.o_dr, &F.tmpl.o_da, &F.tmpl.o_du, &F.tmpl.o_dc})
        *o += delta;
    F.tmpl.o_grad += delta;
    F.tmpl.warp_base += delta;
    F.smem = F.image.size();
    require(F.smem <= 227 * 1024, EDGPU_ERR_ARG,
            "batched tables do not fit in shared memory (" + std::to_string(F.smem) + " bytes)");
    F.tmpl.want_arg = any_arg;
    F.tmpl.n_sec = n;
    F.tmpl.accumulate = 0;
    F.gk = B0.gk;
    F.per_sm = std::max(1, s0.w32 ? hx_multi_occupancy_w32(F.gk, prec, F.smem) : hx_multi_occupancy_w64(F.gk, prec, F.smem));
    F.gens = gens;
    F.ready = true;
}

// Launch parameters of one batched product for a set of vector pointers (device image built once).
HxParams batch_params(edgpu_batch_s* b, int prec, const void* const* xs, void* const* ys, int* blocks_out) {
    edgpu_batch_s::Fused& F = b->fused[prec];
    const int n = (int)b->ops.size();
    // sector maps are used when every sector has one (one colex rank table for all); target tables
    // when every sector's operator has one (pair-flip schedule, one lane per row)
    bool mapped = true, tabled = true;
    for (int i = 0; i < n; ++i) {
        mapped = mapped && (b->ops[i]->space->d_map != nullptr || b->ops[i]->space->dim == 0);
        tabled = tabled && (b->ops[i]->d_tab != nullptr || b->ops[i]->space->dim == 0);
    }
    const bool pair = F.tmpl.bond_ncls > 0 && b->ops[0]->pair_allowed && b->pair_use[prec];
    tabled = tabled && pair && b->tab_use[prec];
    const int lpr = tabled ? 1 : (b->lpr[prec] ? b->lpr[prec] : 1);
    const int rpw = 32 / lpr;
    std::vector<const void*> key;
    key.push_back((const void*)(intptr_t)lpr);
    for (int i = 0; i < n; ++i) {
        key.push_back(xs[i]);
        key.push_back(ys[i]);
        key.push_back(mapped ? b->ops[i]->space->d_map : nullptr);
        key.push_back(tabled ? b->ops[i]->d_tab : nullptr);
    }
    std::vector<SectorDesc> d(n);
    long long tiles = 0;
    for (int i = 0; i < n; ++i) {
        const edgpu_op_s* o = b->ops[i];
        const Space& s = *o->space;
        require(s.dim == 0 || (xs[i] && ys[i]), EDGPU_ERR_ARG, "null vector in batch");
        d[i] = SectorDesc{};
        d[i].keys = s.d_keys;
        d[i].x = xs[i];
        d[i].y = ys[i];
        d[i].diag = o->blob[prec][0][0].d_diag;
        d[i].n_rows = s.dim;
        tiles += (s.dim + rpw - 1) / rpw;
        d[i].tile_end = tiles;
        d[i].ds = dir_search_of(s);
        d[i].map = mapped ? s.d_map : nullptr;
        d[i].map_wide = s.map_wide;
        d[i].map_cb = s.map_cb;
        d[i].map_direct = s.map_direct;
        d[i].o_ph = F.o_ph[i];
        d[i].o_num = F.o_num[i];
        d[i].want_arg = F.want_arg[i];
        if (tabled) {
            d[i].tab = o->d_tab;
            d[i].tile_off = o->d_tile_off;
            d[i].tab_wide = o->tab_wide;
            d[i].tab_cb = o->tab_cb;
        }
    }
    auto it = b->images[prec].find(key);
    if (it == b->images[prec].end()) {
        std::vector<unsigned char> img(F.image);
        memcpy(&img[F.tmpl.o_sec], d.data(), n * sizeof(SectorDesc));
        void* dev = nullptr;
        EDGPU_CUDA(cudaMalloc(&dev, img.size()));
        cudaError_t e = cudaMemcpy(dev, img.data(), img.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(dev);
            throw Error(EDGPU_ERR_CUDA, std::string("batch image: ") + cudaGetErrorString(e));
        }
        it = b->images[prec].emplace(key, dev).first;
    }
    HxParams p = F.tmpl;
    if (mapped) {
        for (int i = 0; i < n; ++i)
            if (b->ops[i]->space->d_map) {
                set_map_params(p, *b->ops[i]->space);
                break;
            }
    }
    p.blob = it->second;
    p.blob_words16 = (int)(F.smem / 16);   // the pair-flip launch below copies only F.smem_pair
    p.lpr = lpr;
    p.rows_per_tile = rpw;
    p.n_tiles = tiles;
    const bool w32 = b->ops[0]->space->w32;
    int per_sm = mapped ? F.per_sm_map : F.per_sm;
    p.bond_nt = (tabled && b->pair_nt[prec] == 8) ? 8 : ((mapped || tabled) && b->pair_nt[prec] >= 4) ? 4 : 2;
    p.tab = nullptr;
    if (tabled) {
        for (int i = 0; i < n; ++i)
            if (b->ops[i]->d_tab) {
                p.tab = b->ops[i]->d_tab;   // marks the target-table launch; the kernel reads each sector's
                break;
            }
        p.blob_words16 = (int)(F.smem_lookup / 16);
        p.bond_pf = b->tab_pf[prec];
        int& ps = F.per_sm_table[p.bond_nt == 8 ? 2 : p.bond_nt == 4 ? 1 : 0];
        if (ps == 0) ps = std::max(1, hx_table_multi_occupancy(w32, prec, p.bond_nt, F.smem_lookup));
        per_sm = ps;
    } else if (pair) {
        const size_t sm_b = mapped ? F.smem_lookup : F.smem_pair;
        p.blob_words16 = (int)(sm_b / 16);
        int& ps = F.per_sm_bond[mapped ? 1 : 0][p.bond_nt == 4 ? 1 : 0];
        if (ps == 0) {
            const int gk = mapped ? GK_MAP : F.gk;
            ps = std::max(1, w32 ? hx_bond_multi_occupancy_w32(gk, prec, p.bond_nt, sm_b)
                                 : hx_bond_multi_occupancy_w64(gk, prec, p.bond_nt, sm_b));
        }
        per_sm = ps;
    } else if (mapped && F.per_sm_map == 0) {
        F.per_sm_map = std::max(1, w32 ? hx_multi_occupancy_w32(GK_MAP, prec, F.smem) : hx_multi_occupancy_w64(GK_MAP, prec, F.smem));
        per_sm = F.per_sm_map;
    }
    const long long need = (tiles + HX_THREADS / 32 - 1) / (HX_THREADS / 32);
    *blocks_out = (int)std::max<long long>(1, std::min<long long>(need, (long long)per_sm * std::max(1, g_sm_count)));
    return p;
}

void batch_launch(edgpu_batch_s* b, int prec, const HxParams& p, int blocks, cudaStream_t st) {
    if (p.n_tiles == 0) return;
    const int gk = p.rank_tab ? GK_MAP : b->fused[prec].gk;   // sector maps present: the map flavour
    const bool w32 = b->ops[0]->space->w32;
    if (p.tab) {
        hx_table_multi_launch(w32, prec, p, blocks, b->fused[prec].smem_lookup, st);
        return;
    }
    if (p.bond_ncls > 0 && b->ops[0]->pair_allowed && b->pair_use[prec]) {
        const size_t sm_b = gk == GK_MAP ? b->fused[prec].smem_lookup : b->fused[prec].smem_pair;
        if (w32) hx_bond_multi_launch_w32(gk, prec, p, blocks, sm_b, st);
        else hx_bond_multi_launch_w64(gk, prec, p, blocks, sm_b, st);
        return;
    }
    if (w32) hx_multi_launch_w32(gk, prec, p, blocks, b->fused[prec].smem, st);
    else hx_multi_launch_w64(gk, prec, p, blocks, b->fused[prec].smem, st);
}

// One sector of a batch launched on its own: the operator's product kernel with the batch's schedule
// (pair flips, targets per step, target table, prefetch, lanes per row; no slab table) in place of
// the operator's own for this launch, or (seq_own) with the operator's own schedule.  The caller holds
// the operators' locks.
void batch_sector_launch(edgpu_batch_s* b, int prec, int i, const void* x, void* y, cudaStream_t st) {
    edgpu_op_s* op = b->ops[i];
    if (op->space->dim == 0) return;
    if (b->seq_own[prec]) {
        // the operator's own (autotuned) schedule, as edgpu_mul_device on the sector
        launch_product(op, prec, 0, 0, x, y, 0, nullptr, nullptr, st);
        return;
    }
    const int keep[6] = {op->pair_use[prec], op->pair_nt[prec], op->tab_use[prec], op->tab_pf[prec], op->tab_uni[prec],
                         op->slab_use[prec]};
    op->pair_use[prec] = b->pair_use[prec];
    op->pair_nt[prec] = b->pair_nt[prec];
    op->tab_use[prec] = b->tab_use[prec];
    op->tab_pf[prec] = b->tab_pf[prec];
    op->tab_uni[prec] = 0;
    op->slab_use[prec] = 0;
    auto restore = [&] {
        op->pair_use[prec] = keep[0];
        op->pair_nt[prec] = keep[1];
        op->tab_use[prec] = keep[2];
        op->tab_pf[prec] = keep[3];
        op->tab_uni[prec] = keep[4];
        op->slab_use[prec] = keep[5];
    };
    try {
        launch_product(op, prec, 0, 0, x, y, 0, nullptr, nullptr, st, nullptr, -(b->lpr[prec] ? b->lpr[prec] : 1));
    } catch (...) {
        restore();
        throw;
    }
    restore();
}

// The batched product y_k = H_k x_k in the batch's launch mode (edgpu_batch_s::seq), enqueued on st.
// Per-sector launches on k > 1 streams fork from st and join back into it, so that st orders them
// after the work before the call and the work after it after all of them (also under stream capture).
void batch_run(edgpu_batch_s* b, int prec, const void* const* xs, void* const* ys, cudaStream_t st) {
    const int k = b->seq[prec];
    const int n = (int)b->ops.size();
    if (k <= 0) {
        int blocks = 0;
        const HxParams p = batch_params(b, prec, xs, ys, &blocks);
        batch_launch(b, prec, p, blocks, st);
        return;
    }
    for (int i = 0; i < n; ++i)
        require(b->ops[i]->space->dim == 0 || (xs[i] && ys[i]), EDGPU_ERR_ARG, "null vector in batch");
    if (k == 1) {
        for (int i = 0; i < n; ++i) batch_sector_launch(b, prec, i, xs[i], ys[i], st);
        return;
    }
    b->ensure_lanes(k);
    EDGPU_CUDA(cudaEventRecord(b->fork_ev, st));
    for (int j = 0; j < k; ++j) EDGPU_CUDA(cudaStreamWaitEvent(b->lane_st[j], b->fork_ev, 0));
    for (int i = 0; i < n; ++i) batch_sector_launch(b, prec, i, xs[i], ys[i], b->lane_st[i % k]);
    for (int j = 0; j < k; ++j) {
        EDGPU_CUDA(cudaEventRecord(b->join_ev[j], b->lane_st[j]));
        EDGPU_CUDA(cudaStreamWaitEvent(st, b->join_ev[j], 0));
    }
}

}  // namespace

int edgpu_batch_create(int32_t n_ops, const edgpu_op* ops, edgpu_batch* out) {
    API_BEGIN
    require(out && n_ops >= 1 && ops, EDGPU_ERR_ARG, "bad batch arguments");
    *out = nullptr;
    std::unique_ptr<edgpu_batch_s> b(new edgpu_batch_s());
    for (int i = 0; i < n_ops; ++i) b->ops.push_back(as_op(ops[i]));
    *out = b.release();
    API_END
}

int edgpu_batch_set_tiling(edgpu_batch bh, int32_t precision, int32_t lanes_per_row) {
    API_BEGIN
    require(bh, EDGPU_ERR_ARG, "null batch");
    std::lock_guard<std::mutex> blk_(bh->hs.mu);
    BatchLocks locks_(bh->ops);
    check_prec(precision);
    require(lanes_per_row == 0 || lanes_per_row == 1 || lanes_per_row == 2 || lanes_per_row == 4, EDGPU_ERR_ARG,
            "lanes_per_row must be 0 (default), 1, 2 or 4");
    bh->lpr[precision] = lanes_per_row;
    API_END
}

int edgpu_batch_autotune(edgpu_batch bh, int32_t precision, int32_t* lanes_per_row_out, double* best_ms_out) {
    API_BEGIN
    require(bh, EDGPU_ERR_ARG, "null batch");
    std::lock_guard<std::mutex> blk_(bh->hs.mu);
    BatchLocks locks_(bh->ops);
    check_prec(precision);
    edgpu_batch_s* b = bh;
    batch_prepare(b, precision);
    const int n = (int)b->ops.size();
    const size_t vs = precision == EDGPU_FP64 ? 16 : 8;
    int64_t tot = 0;
    for (auto* o : b->ops) tot += o->space->dim;
    int best = 1, best_pair = 1, best_nt = 2, best_tab = 1, best_pf = 0, best_seq = 0, best_slab = 0;
    double best_ms = 1e30;
    if (tot > 0) {
        void *x = nullptr, *y = nullptr;
        EDGPU_CUDA(cudaMalloc(&x, tot * vs));
        cudaError_t e = cudaMalloc(&y, tot * vs);
        if (e != cudaSuccess) {
            cudaFree(x);
            throw Error(EDGPU_ERR_OOM, "batch autotune: no room for scratch vectors");
        }
        std::vector<const void*> xs(n);
        std::vector<void*> ys(n);
        int64_t off = 0;
        for (int i = 0; i < n; ++i) {
            xs[i] = (const char*)x + off * vs;
            ys[i] = (char*)y + off * vs;
            off += b->ops[i]->space->dim;
        }
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        const int keep = b->lpr[precision];
        try {
            EDGPU_CUDA(cudaMemsetAsync(x, 0, tot * vs, bh->hs.stream()));
            // lanes per row, with and without the pair-flip schedule where it applies
            const bool pair_ok = b->fused[precision].tmpl.bond_ncls > 0 && b->ops[0]->pair_allowed;
            bool mapped = true;
            for (auto* o : b->ops) mapped = mapped && (o->space->d_map != nullptr || o->space->dim == 0);
            bool tabled = pair_ok;
            for (auto* o : b->ops) tabled = tabled && (o->d_tab != nullptr || o->space->dim == 0);
            // cand 5/4/3: target tables with 8/4/2 targets per step; 2/1: pair flips with 4/2; 0: term scan.
            // l: target tables: one lane per row, x prefetched 0 (l = 1), 4 (l = 5) or 64 (l = 6) steps
            // ahead; the other schedules: l lanes per row.  sq: the launch mode (edgpu_batch_s::seq),
            // per-sector launches only with one lane per row and no prefetch.
            // per-sector launches also with each operator's own schedule (its autotuned one: the slab
            // table, the target table or the term scan, which may differ from sector to sector)
            struct Cand { int cand, l, sq, slab; };
            std::vector<Cand> cands;
            for (int cand = tabled ? 5 : (pair_ok ? (mapped ? 2 : 1) : 0); cand >= 0; --cand)
                for (int l : {1, 2, 4, 5, 6}) {
                    if (cand >= 3 && !(l == 1 || l >= 5)) continue;
                    if (cand < 3 && l >= 5) continue;
                    for (int sq = 0; sq <= 3; ++sq)
                        if (sq == 0 || (l == 1 && cand > 0)) cands.push_back({cand, l, sq, 0});
                }
            for (int sq = 1; sq <= 3; ++sq) cands.push_back({4, 1, sq, 1});
            for (const Cand& cd : cands) {
                const int cand = cd.cand;
                int l = cd.l;
                const int pf = l == 5 ? 4 : (l == 6 ? 64 : 0);
                b->tab_pf[precision] = pf;
                if (l >= 5) l = 1;
                b->lpr[precision] = l;
                b->pair_use[precision] = cand > 0 ? 1 : 0;
                b->pair_nt[precision] = cand == 5 ? 8 : (cand == 2 || cand == 4) ? 4 : 2;
                b->tab_use[precision] = cand >= 3 ? 1 : 0;
                b->seq[precision] = cd.sq;
                b->seq_own[precision] = cd.slab;
                auto run = [&] { batch_run(b, precision, xs.data(), ys.data(), bh->hs.stream()); };
                run();
                float t_min = 1e30f;
                EDGPU_CUDA(cudaEventRecord(e0, bh->hs.stream()));
                run();
                EDGPU_CUDA(cudaEventRecord(e1, bh->hs.stream()));
                EDGPU_CUDA(cudaEventSynchronize(e1));
                float ms1 = 0.f;
                cudaEventElapsedTime(&ms1, e0, e1);
                const int reps = std::max(1, std::min(50, (int)(2.0f / std::max(ms1, 1e-3f))));
                for (int burst = 0; burst < 2; ++burst) {
                    EDGPU_CUDA(cudaEventRecord(e0, bh->hs.stream()));
                    for (int k = 0; k < reps; ++k) run();
                    EDGPU_CUDA(cudaEventRecord(e1, bh->hs.stream()));
                    EDGPU_CUDA(cudaEventSynchronize(e1));
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    t_min = std::min(t_min, ms / reps);
                }
                if (t_min < best_ms) {
                    best_ms = t_min;
                    best = l;
                    best_pf = pf;
                    best_pair = cand > 0 ? 1 : 0;
                    best_nt = cand == 5 ? 8 : (cand == 2 || cand == 4) ? 4 : 2;
                    best_tab = cand >= 3 ? 1 : 0;
                    best_seq = cd.sq;
                    best_slab = cd.slab;
                }
            }
        } catch (...) {
            b->lpr[precision] = keep;
            b->pair_use[precision] = 1;
            b->pair_nt[precision] = 2;
            b->tab_use[precision] = 1;
            b->seq[precision] = 0;
            b->seq_own[precision] = 0;
            cudaStreamSynchronize(bh->hs.stream());
            cudaFree(x);
            cudaFree(y);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            throw;
        }
        cudaStreamSynchronize(bh->hs.stream());
        // the scratch images refer to freed vectors: forget them
        for (auto& kv : b->images[precision]) cudaFree(kv.second);
        b->images[precision].clear();
        for (auto& kv : b->graphs[precision]) cudaGraphExecDestroy(kv.second);
        b->graphs[precision].clear();
        cudaFree(x);
        cudaFree(y);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    b->lpr[precision] = best;
    b->pair_use[precision] = best_pair;
    b->pair_nt[precision] = best_nt;
    b->tab_use[precision] = best_tab;
    b->tab_pf[precision] = best_pf;
    b->seq[precision] = best_seq;
    b->seq_own[precision] = best_slab;
    if (lanes_per_row_out) *lanes_per_row_out = best;
    if (best_ms_out) *best_ms_out = best_ms;
    API_END
}

int edgpu_batch_get_schedule(edgpu_batch bh, int32_t precision, int32_t* lanes_per_row, int32_t* pair_flips,
                             int32_t* target_table) {
    API_BEGIN
    require(bh, EDGPU_ERR_ARG, "null batch");
    std::lock_guard<std::mutex> blk_(bh->hs.mu);
    BatchLocks locks_(bh->ops);
    check_prec(precision);
    if (lanes_per_row) *lanes_per_row = bh->lpr[precision];
    if (pair_flips) {
        batch_prepare(bh, precision);
        bool mapped = true;
        for (auto* o : bh->ops) mapped = mapped && (o->space->d_map != nullptr || o->space->dim == 0);
        bool tabled = true;
        for (auto* o : bh->ops) tabled = tabled && (o->d_tab != nullptr || o->space->dim == 0);
        const bool on = bh->fused[precision].tmpl.bond_ncls > 0 && bh->ops[0]->pair_allowed && bh->pair_use[precision];
        tabled = tabled && on && bh->tab_use[precision];
        *pair_flips = on ? ((tabled && bh->pair_nt[precision] == 8) ? 8 : ((mapped || tabled) && bh->pair_nt[precision] >= 4) ? 4 : 2) : 0;
        if (target_table) *target_table = tabled ? 1 : 0;
    } else if (target_table) {
        bool tabled = true;
        for (auto* o : bh->ops) tabled = tabled && (o->d_tab != nullptr || o->space->dim == 0);
        batch_prepare(bh, precision);
        *target_table = (tabled && bh->fused[precision].tmpl.bond_ncls > 0 && bh->ops[0]->pair_allowed &&
                         bh->pair_use[precision] && bh->tab_use[precision]) ? 1 : 0;
    }
    API_END
}

int edgpu_batch_set_launch(edgpu_batch bh, int32_t precision, int32_t streams) {
    API_BEGIN
    require(bh, EDGPU_ERR_ARG, "null batch");
    std::lock_guard<std::mutex> blk_(bh->hs.mu);
    BatchLocks locks_(bh->ops);
    check_prec(precision);
    require(streams >= 0 && streams <= 7 && streams != 4, EDGPU_ERR_ARG,
            "streams must be 0 (one persistent launch), 1 to 3, or 5 to 7 (per-sector launches with each "
            "operator's own schedule)");
    bh->seq[precision] = streams & 3;
    bh->seq_own[precision] = streams >= 5 ? 1 : 0;
    API_END
}

int edgpu_batch_get_launch(edgpu_batch bh, int32_t precision, int32_t* streams) {
    API_BEGIN
    require(bh && streams, EDGPU_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> blk_(bh->hs.mu);
    check_prec(precision);
    *streams = bh->seq[precision] + (bh->seq_own[precision] ? 4 : 0);
    API_END
}

int edgpu_batch_mul_device(edgpu_batch bh, int32_t precision, const void* const* xs, void* const* ys, int32_t use_graph,
                           void* stream) {
    API_BEGIN
    require(bh && xs && ys, EDGPU_ERR_ARG, "bad batch arguments");
    std::lock_guard<std::mutex> blk_(bh->hs.mu);
    BatchLocks locks_(bh->ops);
    check_prec(precision);
    edgpu_batch_s* b = bh;
    cudaStream_t st = pick_stream(stream);
    const int n = (int)b->ops.size();
    batch_prepare(b, precision);
    if (!use_graph) {
        batch_run(b, precision, xs, ys, st);
        return EDGPU_OK;
    }
    const int sq = b->seq[precision];
    std::vector<const void*> key;
    key.push_back((const void*)(intptr_t)b->lpr[precision]);
    key.push_back((const void*)(intptr_t)(b->pair_use[precision] * 8 + b->pair_nt[precision] +
                                          b->tab_use[precision] * 16 + 32 * b->tab_pf[precision]));   // the kernel
    key.push_back((const void*)(intptr_t)(sq + 8 * b->seq_own[precision]));   // the launch mode
    if (sq == 0) {
        int blocks = 0;
        key.push_back(batch_params(b, precision, xs, ys, &blocks).blob);   // the image (vectors, sector maps)
    } else {
        for (int i = 0; i < n; ++i) {
            // per-sector launches read the operators' own tables (and their slab variants)
            key.push_back(b->ops[i]->d_tab);
            key.push_back(b->ops[i]->space->d_map);
            const edgpu_op_s* o = b->ops[i];
            key.push_back(o->slab.tab);
            // the operator's own schedule (modes 5 to 7 launch with it)
            key.push_back((const void*)(intptr_t)(o->pair_allowed + 2 * o->pair_use[precision] + 4 * o->pair_nt[precision] +
                                                  64 * o->tab_use[precision] + 128 * o->tab_uni[precision] +
                                                  256 * o->slab_use[precision] + 512 * o->tab_pf[precision] +
                                                  (1 << 20) * o->slab_hint[precision]));
            key.push_back((const void*)(intptr_t)o->tuned_rows[precision]);
            key.push_back((const void*)(uintptr_t)o->gen);
        }
    }
    for (int i = 0; i < n; ++i) {
        key.push_back(xs[i]);
        key.push_back(ys[i]);
    }
    auto& cache = b->graphs[precision];
    auto it = cache.find(key);
    if (it == cache.end()) {
        // Capture on a private stream (the caller's stream may be the legacy default stream, which
        // cannot be captured); the graph is then launched on the caller's stream.
        cudaStream_t cap = nullptr;
        EDGPU_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaStreamDestroy(cap);
            throw Error(EDGPU_ERR_CUDA, std::string("begin capture: ") + cudaGetErrorString(e));
        }
        try {
            batch_run(b, precision, xs, ys, cap);
        } catch (...) {
            cudaStreamEndCapture(cap, &graph);
            if (graph) cudaGraphDestroy(graph);
            cudaStreamDestroy(cap);
            throw;
        }
        e = cudaStreamEndCapture(cap, &graph);
        cudaStreamDestroy(cap);
        if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e));
        cudaGraphExec_t exec = nullptr;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        it = cache.emplace(key, exec).first;
    }
    EDGPU_CUDA(cudaGraphLaunch(it->second, st));
    API_END
}

void edgpu_batch_destroy(edgpu_batch b) { delete b; }

// ---- Lanczos -------------------------------------------------------------------------------------

int edgpu_set_krylov_limit(int64_t bytes) {
    API_BEGIN
    require(bytes >= 0, EDGPU_ERR_ARG, "negative limit");
    g_krylov_limit = bytes;
    API_END
}

int edgpu_lanczos(edgpu_op oh, int32_t precision, int32_t n_steps, int32_t reorth, uint64_t seed, const double* v0,
                  int32_t refine, double tol, double* e0, double* alphas, double* betas, int32_t* steps_done,
                  double* ground_state) {
    API_BEGIN
    edgpu_op_s* op = as_op(oh);
    OpLock lk_(op->hs.mu);
    check_prec(precision);
    require(n_steps >= 1 && e0 && tol >= 0.0, EDGPU_ERR_ARG, "bad Lanczos arguments");
    const int64_t N = op->space->dim;
    require(N >= 1, EDGPU_ERR_ARG, "empty representation");
    cudaStream_t st = op->hs.stream();
    const int m = (int)std::min<int64_t>(n_steps, N);
    const bool two_phase = refine && precision == EDGPU_MIXED;
    const bool want_vec = ground_state != nullptr;

    // Krylov basis storage of one run: rolling (two FP64 vectors), FP64 basis, or the complex64 product
    // inputs of a mixed-precision run.  A basis is stored only when reorthogonalisation or a Ritz vector
    // needs it and it fits under the Krylov limit; a Ritz vector of a rolling run is rebuilt by a second
    // pass of the recurrence from the saved start vector (every kernel on the path is deterministic,
    // so the pass regenerates the same vectors bit for bit).
    enum Store { ROLL = 0, F64 = 1, F32 = 2 };
    size_t free_b = 0, total_b = 0;
    EDGPU_CUDA(cudaMemGetInfo(&free_b, &total_b));
    double limit = g_krylov_limit > 0 ? (double)g_krylov_limit : 0.5 * (double)free_b;
    auto fits64 = [&](int k) { return (double)(k + 1) * (double)N * 16.0 <= limit; };
    auto fits32 = [&](int k) { return (double)(k + 1) * (double)N * 8.0 <= limit; };

    DevBuf<double> V64, w, scal, scratch, h, md, psi, vstart;
    DevBuf<float> V32, y32;
    scal.ensure(8);
    scratch.ensure(dot_scratch_doubles());
    h.ensure(2 * (size_t)(m + 1));
    md.ensure(2 * (size_t)(m + 1) * 64);
    w.ensure(2 * N);
    double* d_alpha = scal.p;      // [0]=re [1]=im of <v, w>
    double* d_beta = scal.p + 2;   // current beta
    double* d_bprev = scal.p + 3;  // previous beta
    double* d_tmp = scal.p + 4;

    // per-run layout
    int cur_prec = precision, cur_store = ROLL, cur_cap = m;
    bool cur_reorth = false;
    auto vec64 = [&](int j) { return V64.p + (size_t)(cur_store == F64 ? j : (j & 1)) * 2 * N; };
    auto vin32 = [&](int j) { return V32.p + (size_t)(cur_store == F32 ? j : 0) * 2 * N; };
    auto setup = [&](int prec, int store, int cap, bool reo) {
        cur_prec = prec;
        cur_store = store;
        cur_cap = cap;
        cur_reorth = reo;
        V64.ensure((size_t)(store == F64 ? cap + 1 : 2) * 2 * N);
        if (prec == EDGPU_MIXED) {
            V32.ensure((size_t)(store == F32 ? cap + 1 : 1) * 2 * N);
            y32.ensure(2 * N);
        }
        if (store == ROLL) vstart.ensure(2 * N);
    };
    // vec64(0) <- src / |src| (and its complex64 copy); saved as the start vector of a rolling run
    auto start_from = [&](const double* src_dev, const double* src_host) {
        if (src_host) EDGPU_CUDA(cudaMemcpyAsync(vec64(0), src_host, N * 16, cudaMemcpyHostToDevice, st));
        else if (src_dev) EDGPU_CUDA(cudaMemcpyAsync(vec64(0), src_dev, N * 16, cudaMemcpyDeviceToDevice, st));
        else launch_random_c128(N, seed, vec64(0), st);
        launch_norm2_c128(N, vec64(0), scratch.p, d_tmp, st);
        launch_normalize(N, vec64(0), d_tmp, vec64(0), cur_prec == EDGPU_MIXED ? vin32(0) : nullptr, st);
        if (cur_store == ROLL) EDGPU_CUDA(cudaMemcpyAsync(vstart.p, vec64(0), N * 16, cudaMemcpyDeviceToDevice, st));
    };

    // Kato-Temple estimate of the lowest Ritz value's error after a step with the next beta:
    // (beta s_last)^2 / (theta_2 - theta_1) <= kt max(1, |theta_1|), s the lowest eigenvector of the
    // tridiagonal matrix (beta |s_last| is the Ritz pair's residual norm) and theta_2 its second
    // eigenvalue (or the given one when not NaN).
    auto kt_ok = [&](const std::vector<double>& A, const std::vector<double>& B, double beta, double th1,
                     double th2_given, double kt) {
        if (A.size() < 2) return false;
        const double th2 = std::isnan(th2_given) ? kth_eigenvalue(A, B, 2) : th2_given;
        if (!(th2 > th1)) return false;
        const std::vector<double> sv = tridiag_eigvec(A, B, th1);
        double nrm = 0.0;
        for (double v : sv) nrm += v * v;
        const double res = beta * std::fabs(sv.back()) / std::sqrt(nrm);
        return res * res / (th2 - th1) <= kt * std::max(1.0, std::fabs(th1));
    };
    // Lanczos steps j = 0 .. steps-1 from vec64(0); fills A, B.  conv_tol > 0: stop once the lowest Ritz
    // value moved by less than conv_tol |E| over the last 5 steps (with kt > 0: once that has held for
    // `patience` steps, or earlier when the Kato-Temple estimate is below kt, from step kt_min on).
    // With acc: psi += acc[j] v_j only.
    auto run = [&](int steps, double conv_tol, std::vector<double>& A, std::vector<double>& B,
                   const std::vector<double>* acc, double kt = 0.0, double kt_th2 = NAN, int kt_min = 10,
                   int patience = 1) {
        std::vector<double> hist;   // lowest Ritz value after every step (with conv_tol > 0)
        int settled_for = 0;
        for (int j = 0; j < steps; ++j) {
            double* vj = vec64(j);
            if (acc) {
                launch_axpy_real(N, (*acc)[j], vj, psi.p, st);
                if (j + 1 >= (int)acc->size()) break;
            }
            if (cur_prec == EDGPU_FP64) {
                launch_product(op, EDGPU_FP64, 0, 0, vj, w.p, 0, nullptr, nullptr, st);
            } else {
                launch_product(op, EDGPU_MIXED, 0, 0, vin32(j), y32.p, 0, nullptr, nullptr, st);
                launch_c64_to_c128(N, y32.p, w.p, 0, st);
            }
            launch_dot_c128(N, vj, w.p, scratch.p, d_alpha, st);
            launch_lanczos_update(N, w.p, vj, j > 0 ? vec64(j - 1) : nullptr, d_alpha, j > 0 ? d_bprev : nullptr, st);
            if (cur_reorth) {
                for (int pass = 0; pass < 2; ++pass) {
                    if (cur_store == F64) {
                        launch_multi_dot(N, j + 1, V64.p, N, w.p, md.p, h.p, st);
                        launch_multi_axpy(N, j + 1, V64.p, N, h.p, w.p, st);
                    } else {
                        launch_multi_dot_c64(N, j + 1, V32.p, N, w.p, md.p, h.p, st);
                        launch_multi_axpy_c64(N, j + 1, V32.p, N, h.p, w.p, st);
                    }
                }
            }
            launch_norm2_c128(N, w.p, scratch.p, d_beta, st);
            double hb[2];
            EDGPU_CUDA(cudaMemcpyAsync(hb, d_alpha, sizeof(double), cudaMemcpyDeviceToHost, st));
            EDGPU_CUDA(cudaMemcpyAsync(hb + 1, d_beta, sizeof(double), cudaMemcpyDeviceToHost, st));
            EDGPU_CUDA(cudaStreamSynchronize(st));
            A.push_back(hb[0]);
            const double beta = hb[1];
            if (j == steps - 1 || beta <= 1e-12 * std::max(1.0, std::fabs(hb[0]))) break;
            if (conv_tol > 0.0 && !acc) {
                const double e = lowest_eigenvalue(A, B);
                hist.push_back(e);
                const size_t h = hist.size();
                const bool settled = h > 5 && std::fabs(e - hist[h - 6]) < conv_tol * std::max(1.0, std::fabs(e));
                settled_for = settled ? settled_for + 1 : 0;
                if (kt > 0.0 && (int)A.size() >= kt_min && kt_ok(A, B, beta, e, kt_th2, kt)) break;
                if (settled_for >= (kt > 0.0 ? patience : 1)) break;
            }
            B.push_back(beta);
            launch_normalize(N, w.p, d_beta, vec64(j + 1), cur_prec == EDGPU_MIXED ? vin32(j + 1) : nullptr, st);
            EDGPU_CUDA(cudaMemcpyAsync(d_bprev, d_beta, sizeof(double), cudaMemcpyDeviceToDevice, st));
        }
    };
    auto lowest = [&](const std::vector<double>& A, const std::vector<double>& B) {
        return lowest_eigenvalue(A, std::vector<double>(B.begin(), B.begin() + (A.size() - 1)));
    };
    // psi = sum_k s_k v_k for the lowest eigenvector s of the current run's tridiagonal matrix
    auto ritz_vector = [&](const std::vector<double>& A, const std::vector<double>& B, double lam) {
        std::vector<double> s = tridiag_eigvec(A, std::vector<double>(B.begin(), B.begin() + (A.size() - 1)), lam);
        psi.ensure(2 * N);
        EDGPU_CUDA(cudaMemsetAsync(psi.p, 0, N * 16, st));
        if (cur_store == ROLL) {
            EDGPU_CUDA(cudaMemcpyAsync(vec64(0), vstart.p, N * 16, cudaMemcpyDeviceToDevice, st));
            if (cur_prec == EDGPU_MIXED) launch_c128_to_c64(N, vec64(0), vin32(0), st);
            std::vector<double> A2, B2;
            run((int)s.size(), 0.0, A2, B2, &s);
        } else {
            std::vector<double> coef(2 * s.size());
            for (size_t k = 0; k < s.size(); ++k) {
                coef[2 * k] = -s[k];
                coef[2 * k + 1] = 0.0;
            }
            EDGPU_CUDA(cudaMemcpyAsync(h.p, coef.data(), coef.size() * sizeof(double), cudaMemcpyHostToDevice, st));
            if (cur_store == F64) launch_multi_axpy(N, (int)s.size(), V64.p, N, h.p, psi.p, st);
            else launch_multi_axpy_c64(N, (int)s.size(), V32.p, N, h.p, psi.p, st);
        }
        EDGPU_CUDA(cudaStreamSynchronize(st));
    };

    std::vector<double> A, B;
    double E = 0.0;
    int done = 0;
    bool want_vec_done = false;
    if (!two_phase) {
        int store = ROLL;
        if (reorth || want_vec) {
            if (fits64(m)) store = F64;
            else if (precision == EDGPU_MIXED && fits32(m)) store = F32;
        }
        require(!reorth || store != ROLL, EDGPU_ERR_OOM,
                "the Krylov basis for full reorthogonalisation does not fit in device memory (" +
                    std::to_string((long long)((m + 1) * N * (precision == EDGPU_MIXED ? 8 : 16) >> 20)) +
                    " MiB); use reorth = 0");
        setup(precision, store, m, reorth != 0);
        start_from(nullptr, v0);
        // the Kato-Temple rule certifies the eigenvalue, not the vector: a wanted ground state runs on
        // until the eigenvalue has settled
        run(m, tol, A, B, nullptr, want_vec ? 0.0 : tol);
        E = lowest(A, B);
        done = (int)A.size();
    } else {
        // 1. mixed-precision Lanczos to about 1e-9 with a stored basis (FP64, else complex64, capped by
        //    the Krylov limit and by the device memory left once the run's other buffers are in place,
        //    less 2 GiB), or rolling with a second pass for the Ritz vector
        psi.ensure(2 * N);
        V64.ensure(2 * 2 * N);
        y32.ensure(2 * N);
        {
            size_t fb = 0, tb = 0;
            EDGPU_CUDA(cudaMemGetInfo(&fb, &tb));
            const double room = (double)fb + (double)V32.n * sizeof(float) - (double)(2ull << 30);
            limit = std::max(0.0, std::min(limit, room));
        }
        int store = ROLL, m1 = m;
        if (fits64(m)) store = F64;
        else if (fits32(m)) store = F32;
        else {
            int cap = 0;
            while (cap < m && fits32(cap + 1)) ++cap;
            if (cap >= 40 && !reorth) {
                store = F32;
                m1 = cap;
            }
        }
        require(!reorth || store != ROLL, EDGPU_ERR_OOM,
                "the Krylov basis for full reorthogonalisation does not fit in device memory; use reorth = 0");
        setup(EDGPU_MIXED, store, m1, reorth != 0);
        start_from(nullptr, v0);
        // restarted from its Ritz vector while the stored basis fills up before the eigenvalue settles
        // (at most n_steps mixed steps in all)
        const double tol1 = std::max(tol, 1e-9);
        for (;;) {
            A.clear();
            B.clear();
            const int budget = std::min(m1, m - done);
            // on until the Ritz pair's residual predicts that the FP64 Rayleigh quotient below will be
            // certified (a quarter of tol, for the complex64 roundings), or for 6 steps after the Ritz
            // value has settled to tol1 (the roundings may hold the residual above that)
            run(budget, tol1, A, B, nullptr, 0.25 * tol, NAN, 10, 6);
            E = lowest(A, B);
            done += (int)A.size();
            ritz_vector(A, B, E);
            if ((int)A.size() < budget || done >= m || store != F32 || m1 == m) break;
            start_from(psi.p, nullptr);
        }
        // 2. the FP64 Rayleigh quotient of the mixed-precision Ritz vector psi, one FP64 product:
        //    E_RQ = <psi|H psi>, r = H psi - E_RQ psi.  Its error is of second order in the error of
        //    psi and is estimated by the Kato-Temple bound |r|^2 / (theta_2 - E_RQ), theta_2 the
        //    second-lowest Ritz value of the mixed run; accepted when that is below tol |E_RQ|.
        bool certified = false;
        double theta2_mixed = NAN;
        if (A.size() >= 2) {
            launch_norm2_c128(N, psi.p, scratch.p, d_tmp, st);
            launch_normalize(N, psi.p, d_tmp, psi.p, nullptr, st);
            launch_product(op, EDGPU_FP64, 0, 0, psi.p, w.p, 0, nullptr, nullptr, st);
            launch_dot_c128(N, psi.p, w.p, scratch.p, d_alpha, st);
            launch_lanczos_update(N, w.p, psi.p, nullptr, d_alpha, nullptr, st);
            launch_norm2_c128(N, w.p, scratch.p, d_beta, st);
            double hb[2];
            EDGPU_CUDA(cudaMemcpyAsync(hb, d_alpha, sizeof(double), cudaMemcpyDeviceToHost, st));
            EDGPU_CUDA(cudaMemcpyAsync(hb + 1, d_beta, sizeof(double), cudaMemcpyDeviceToHost, st));
            EDGPU_CUDA(cudaStreamSynchronize(st));
            const double e_rq = hb[0], rn = hb[1];
            const double theta2 = kth_eigenvalue(A, std::vector<double>(B.begin(), B.begin() + (A.size() - 1)), 2);
            theta2_mixed = theta2;
            ++done;
            if (theta2 > e_rq && rn * rn / (theta2 - e_rq) <= tol * std::max(1.0, std::fabs(e_rq))) {
                E = e_rq;
                certified = true;
            }
        }
        // 3. otherwise FP64 Lanczos from the mixed-precision Ritz vector until the eigenvalue settles to tol
        const bool store2 = (reorth || want_vec) && fits64(m);
        if (!certified) {
            V32.release();   // the mixed run's basis makes room for the FP64 run's
            setup(EDGPU_FP64, store2 ? F64 : ROLL, m, reorth != 0 && store2);
            start_from(psi.p, nullptr);
            std::vector<double> A2, B2;
            // stopped by the Kato-Temple estimate with the mixed run's second Ritz value as the gap
            run(m, tol, A2, B2, nullptr, tol, theta2_mixed, std::isnan(theta2_mixed) ? 10 : 2);
            A = A2;
            B = B2;
            E = lowest(A, B);
            done += (int)A.size();
        } else if (want_vec) {
            // psi is the certified ground state: return it as is
            EDGPU_CUDA(cudaMemcpyAsync(ground_state, psi.p, N * 16, cudaMemcpyDeviceToHost, st));
            EDGPU_CUDA(cudaStreamSynchronize(st));
            want_vec_done = true;
        }
    }
    *e0 = E;
    if (alphas)
        for (size_t k = 0; k < (size_t)n_steps; ++k) alphas[k] = k < A.size() ? A[k] : 0.0;
    if (betas)
        for (size_t k = 0; k < (size_t)n_steps; ++k) betas[k] = k < B.size() ? B[k] : 0.0;
    if (steps_done) *steps_done = done;
    if (ground_state && !want_vec_done) {
        ritz_vector(A, B, E);
        launch_norm2_c128(N, psi.p, scratch.p, d_tmp, st);
        launch_normalize(N, psi.p, d_tmp, psi.p, nullptr, st);
        EDGPU_CUDA(cudaMemcpyAsync(ground_state, psi.p, N * 16, cudaMemcpyDeviceToHost, st));
    }
    EDGPU_CUDA(cudaStreamSynchronize(st));
    API_END
}

// ---- utilities ---------------------------------------------------------------------------------

int edgpu_random_vector_device(int64_t n, uint64_t seed, int32_t precision, void* dst, void* stream) {
    API_BEGIN
    check_prec(precision);
    require(n >= 0 && (n == 0 || dst), EDGPU_ERR_ARG, "bad arguments");
    if (n == 0) return EDGPU_OK;
    init_device();
    cudaStream_t st = pick_stream(stream);
    DevBuf<double> tmp, scratch, nrm;
    double* target = nullptr;
    if (precision == EDGPU_FP64) target = (double*)dst;
    else {
        tmp.ensure(2 * n);
        target = tmp.p;
    }
    scratch.ensure(dot_scratch_doubles());
    nrm.ensure(1);
    launch_random_c128(n, seed, target, st);
    launch_norm2_c128(n, target, scratch.p, nrm.p, st);
    launch_normalize(n, target, nrm.p, target, precision == EDGPU_MIXED ? (float*)dst : nullptr, st);
    EDGPU_CUDA(cudaStreamSynchronize(st));
    API_END
}

int edgpu_sync(void) {
    API_BEGIN
    // every handle's stream and the caller streams the library was given
    if (g_stream) EDGPU_CUDA(cudaDeviceSynchronize());
    API_END
}

int edgpu_host_alloc(int64_t bytes, void** out) {
    API_BEGIN
    require(out && bytes >= 0, EDGPU_ERR_ARG, "bad arguments");
    init_device();
    EDGPU_CUDA(cudaMallocHost(out, std::max<int64_t>(bytes, 1)));
    API_END
}

void edgpu_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"
