// Sector basis and representative enumeration on the GPU.
//
// Replaces hs_get_basis_list(::HilbertSpaceSector) (hilbert_space_representation.jl:127-206) and the
// representative sweep of symmetry_reduce (symmetry_reduce_generic.jl:22-106).  Candidates are
// scanned in increasing order, 32 per thread (one bitmap word per thread, written coalesced);
// a predicate marks the kept ones, per-block popcounts are scanned into offsets, and a second pass
// regenerates the candidates and writes the kept ones in order: the output is sorted by
// construction.  Candidate sources:
//   RANGE  every word below 2^nbits (general sites: local-code validity + QN sum in the allowed set)
//   COMBO  every nbits-bit word with k set bits, by combinatorial unranking + Gosper's next-
//          combination step (spin-1/2 2Sz sectors; the parent basis then needs no predicate)
//   LIST   a materialised parent basis
#include <algorithm>
#include <cmath>
#include <mutex>

#include "edgpu_internal.h"
#include "edgpu_device.cuh"

namespace edgpu {

namespace {

constexpr int ENUM_THREADS = 256;

unsigned long long* binomial_table() {
    // C(i, j) for 0 <= i, j <= 64 (row stride 65); C(64, 32) < 2^63 so no entry overflows.
    static unsigned long long* d_tab = nullptr;
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (!d_tab) {
        std::vector<unsigned long long> h(65 * 65, 0ull);
        for (int i = 0; i <= 64; ++i) {
            h[i * 65] = 1;
            for (int j = 1; j <= i; ++j) h[i * 65 + j] = h[(i - 1) * 65 + j - 1] + (j <= i - 1 ? h[(i - 1) * 65 + j] : 0ull);
        }
        EDGPU_CUDA(cudaMalloc(&d_tab, h.size() * sizeof(unsigned long long)));
        EDGPU_CUDA(cudaMemcpy(d_tab, h.data(), h.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice));
    }
    return d_tab;
}

unsigned long long host_binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    unsigned long long r = 1;
    for (int i = 1; i <= k; ++i) r = r * (unsigned long long)(n - k + i) / (unsigned long long)i;
    return r;
}

template <typename W>
__device__ __forceinline__ int ctz_w(W v);
template <>
__device__ __forceinline__ int ctz_w<uint32_t>(uint32_t v) { return __ffs((int)v) - 1; }
template <>
__device__ __forceinline__ int ctz_w<unsigned long long>(unsigned long long v) { return __ffsll((long long)v) - 1; }

// Colex unranking: the rank-r word with k set bits among n (rank order == numeric order).
template <typename W>
__device__ __forceinline__ W unrank_combo(unsigned long long r, int n, int k, const unsigned long long* C) {
    W v = 0;
    int c = n;
    for (int i = k; i >= 1; --i) {
        do { --c; } while (C[c * 65 + i] > r);
        v |= (W)1 << c;
        r -= C[c * 65 + i];
    }
    return v;
}

// Next word with the same popcount (Gosper).
template <typename W>
__device__ __forceinline__ W gosper_next(W v) {
    const W t = v | (v - 1);
    return (W)((t + 1) | (((~t & (t + 1)) - 1) >> (ctz_w<W>(v) + 1)));
}

enum { SRC_RANGE = 0, SRC_COMBO = 1, SRC_LIST = 2 };

struct EnumParams {
    int src;
    long long total;
    int n, k;
    const unsigned long long* C;
    const void* list;
    int list_w32;
    int check_sector;
    SectorDev sec;
    int check_rep;
    GroupDev grp;
    unsigned* bitmap;
    long long* block_counts;
    long long* block_offsets;
    void* out;
};

template <typename W>
__device__ __forceinline__ bool sector_ok(W s, const SectorDev& d) {
    long long acc[4] = {0, 0, 0, 0};
    for (int i = 0; i < d.n_sites; ++i) {
        const int c = (int)((s >> d.off[i]) & (W)(((W)1 << d.bw[i]) - 1));
        if (c >= d.dims[i]) return false;
        const long long* q = d.qn + (size_t)(d.qbase[i] + c) * d.qlen;
        for (int k = 0; k < d.qlen; ++k) acc[k] += q[k];
    }
    if (d.all_sectors) return true;
    for (int a = 0; a < d.n_allowed; ++a) {
        bool m = true;
        for (int k = 0; k < d.qlen; ++k) m = m && (d.allowed[a * d.qlen + k] == acc[k]);
        if (m) return true;
    }
    return false;
}

template <typename W>
__device__ __forceinline__ bool rep_ok(W s, const GroupDev& g) {
    if (g.kind == GK_TORUS) {
        W keep[64];
        for (int a = 0; a < g.L1; ++a) keep[a] = (W)g.keep[a];
        return is_rep_torus<W>(s, g.L1, g.L2, g.w, g.rowbits, g.nbits, (W)g.full, keep, g.num);
    }
    if (g.kind == GK_GENERIC) {
        for (int e = 1; e < g.G; ++e) {
            W t = 0;
            const unsigned long long* L = g.lut + (size_t)e * g.nchunks * 16;
            for (int c = 0; c < g.nchunks; ++c) t |= (W)L[c * 16 + (int)((s >> (4 * c)) & 15u)];
            t ^= (W)g.flips[e];
            if (t < s) return false;
            if (t == s && g.num[e] != 0) return false;
        }
        return true;
    }
    return true;
}

template <typename W>
__device__ __forceinline__ W first_candidate(const EnumParams& p, long long r0) {
    if (p.src == SRC_RANGE) return (W)r0;
    if (p.src == SRC_COMBO) return unrank_combo<W>((unsigned long long)r0, p.n, p.k, p.C);
    return p.list_w32 ? (W)((const unsigned*)p.list)[r0] : (W)((const unsigned long long*)p.list)[r0];
}

template <typename W>
__device__ __forceinline__ W next_candidate(const EnumParams& p, W v, long long r) {
    if (p.src == SRC_RANGE) return (W)(v + 1);
    if (p.src == SRC_COMBO) return gosper_next<W>(v);
    return p.list_w32 ? (W)((const unsigned*)p.list)[r] : (W)((const unsigned long long*)p.list)[r];
}

template <typename W>
__global__ void __launch_bounds__(ENUM_THREADS) k_mark(EnumParams p) {
    __shared__ long long tmp[32];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long r0 = t * 32;
    unsigned word = 0;
    if (r0 < p.total) {
        const int cnt = (int)min(32LL, p.total - r0);
        W v = first_candidate<W>(p, r0);
        for (int j = 0; j < cnt; ++j) {
            bool ok = true;
            if (p.check_sector) ok = sector_ok<W>(v, p.sec);
            if (ok && p.check_rep) ok = rep_ok<W>(v, p.grp);
            if (ok) word |= 1u << j;
            if (j + 1 < cnt) v = next_candidate<W>(p, v, r0 + j + 1);
        }
        p.bitmap[t] = word;
    }
    long long tot = 0;
    block_exclusive_scan((long long)__popc(word), tmp, &tot);
    if (threadIdx.x == 0) p.block_counts[blockIdx.x] = tot;
}

__global__ void k_scan_counts(const long long* counts, long long n, long long* offsets, long long* total) {
    __shared__ long long tmp[32];
    const long long per = (n + blockDim.x - 1) / blockDim.x;
    const long long beg = min(n, (long long)threadIdx.x * per), end = min(n, beg + per);
    long long s = 0;
    for (long long i = beg; i < end; ++i) s += counts[i];
    long long tot = 0;
    long long ex = block_exclusive_scan(s, tmp, &tot);
    for (long long i = beg; i < end; ++i) {
        offsets[i] = ex;
        ex += counts[i];
    }
    if (threadIdx.x == 0) *total = tot;
}

template <typename W>
__global__ void __launch_bounds__(ENUM_THREADS) k_compact(EnumParams p) {
    __shared__ long long tmp[32];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long r0 = t * 32;
    const unsigned word = (r0 < p.total) ? p.bitmap[t] : 0u;
    long long pos = block_exclusive_scan((long long)__popc(word), tmp, nullptr) + p.block_offsets[blockIdx.x];
    if (word) {
        const int cnt = (int)min(32LL, p.total - r0);
        W v = first_candidate<W>(p, r0);
        W* out = (W*)p.out;
        for (int j = 0; j < cnt; ++j) {
            if ((word >> j) & 1u) out[pos++] = v;
            if (j + 1 < cnt) v = next_candidate<W>(p, v, r0 + j + 1);
        }
    }
}

template <typename W>
__global__ void k_combo_write(long long total, int n, int k, const unsigned long long* C, W* out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long r0 = t * 32;
    if (r0 >= total) return;
    W v = unrank_combo<W>((unsigned long long)r0, n, k, C);
    const int cnt = (int)min(32LL, total - r0);
    for (int j = 0; j < cnt; ++j) {
        out[r0 + j] = v;
        if (j + 1 < cnt) v = gosper_next<W>(v);
    }
}

// Device copies of the sector definition for the RANGE predicate.
struct SectorBuffers {
    SectorDev dev{};
    std::vector<void*> ptrs;
    template <typename T>
    const T* put(const std::vector<T>& v) {
        if (v.empty()) return nullptr;
        void* d = nullptr;
        EDGPU_CUDA(cudaMalloc(&d, v.size() * sizeof(T)));
        ptrs.push_back(d);
        EDGPU_CUDA(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        return (const T*)d;
    }
    explicit SectorBuffers(const Layout& lay) {
        std::vector<int32_t> qbase(lay.n_sites);
        int acc = 0;
        for (int i = 0; i < lay.n_sites; ++i) { qbase[i] = acc; acc += lay.dims[i]; }
        std::vector<long long> qn(lay.state_qn.begin(), lay.state_qn.end());
        std::vector<long long> al(lay.allowed.begin(), lay.allowed.end());
        dev.n_sites = lay.n_sites;
        dev.qlen = lay.qlen;
        dev.n_allowed = lay.qlen ? (int)(lay.allowed.size() / lay.qlen) : 0;
        dev.all_sectors = lay.all_sectors ? 1 : 0;
        dev.off = put(lay.off);
        dev.bw = put(lay.bw);
        dev.dims = put(lay.dims);
        dev.qbase = put(qbase);
        dev.qn = put(qn);
        dev.allowed = put(al);
    }
    ~SectorBuffers() {
        for (void* p : ptrs) cudaFree(p);
    }
};

template <typename W>
int64_t run_filtered(EnumParams p, void** out_keys, bool write, cudaStream_t st) {
    const long long n_words = (p.total + 31) / 32;
    const long long n_blocks = (n_words + ENUM_THREADS - 1) / ENUM_THREADS;
    if (n_blocks > 0x7fffffffLL) throw Error(EDGPU_ERR_ARG, "enumeration too large");
    unsigned* d_bitmap = nullptr;
    long long* d_counts = nullptr;
    long long* d_offsets = nullptr;
    long long* d_total = nullptr;
    int64_t total = 0;
    try {
        EDGPU_CUDA(cudaMalloc(&d_bitmap, std::max<long long>(n_words, 1) * sizeof(unsigned)));
        EDGPU_CUDA(cudaMalloc(&d_counts, std::max<long long>(n_blocks, 1) * sizeof(long long)));
        EDGPU_CUDA(cudaMalloc(&d_offsets, std::max<long long>(n_blocks, 1) * sizeof(long long)));
        EDGPU_CUDA(cudaMalloc(&d_total, sizeof(long long)));
        p.bitmap = d_bitmap;
        p.block_counts = d_counts;
        p.block_offsets = d_offsets;
        if (n_blocks > 0) {
            k_mark<W><<<(unsigned)n_blocks, ENUM_THREADS, 0, st>>>(p);
            EDGPU_CUDA(cudaGetLastError());
            k_scan_counts<<<1, 1024, 0, st>>>(d_counts, n_blocks, d_offsets, d_total);
            EDGPU_CUDA(cudaGetLastError());
            long long h_total = 0;
            EDGPU_CUDA(cudaMemcpyAsync(&h_total, d_total, sizeof(long long), cudaMemcpyDeviceToHost, st));
            EDGPU_CUDA(cudaStreamSynchronize(st));
            total = h_total;
        }
        if (write) {
            void* keys = nullptr;
            EDGPU_CUDA(cudaMalloc(&keys, std::max<int64_t>(total, 1) * sizeof(W)));
            p.out = keys;
            if (total > 0) {
                k_compact<W><<<(unsigned)n_blocks, ENUM_THREADS, 0, st>>>(p);
                cudaError_t e = cudaGetLastError();
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                if (e != cudaSuccess) {
                    cudaFree(keys);
                    throw Error(EDGPU_ERR_CUDA, std::string("k_compact: ") + cudaGetErrorString(e));
                }
            }
            *out_keys = keys;
        }
    } catch (...) {
        cudaFree(d_bitmap);
        cudaFree(d_counts);
        cudaFree(d_offsets);
        cudaFree(d_total);
        throw;
    }
    cudaFree(d_bitmap);
    cudaFree(d_counts);
    cudaFree(d_offsets);
    cudaFree(d_total);
    return total;
}

template <typename W>
void enumerate_parent_t(Space& s, cudaStream_t st) {
    const Layout& lay = s.lay;
    if (lay.popcount >= 0) {
        const long long total = (long long)host_binom(lay.nbits, lay.popcount);
        s.dim = total;
        if (s.lazy) return;
        EDGPU_CUDA(cudaMalloc(&s.d_keys, std::max<long long>(total, 1) * sizeof(W)));
        const long long threads = (total + 31) / 32;
        if (threads > 0) {
            k_combo_write<W><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(total, lay.nbits, lay.popcount,
                                                                             binomial_table(), (W*)s.d_keys);
            EDGPU_CUDA(cudaGetLastError());
            EDGPU_CUDA(cudaStreamSynchronize(st));
        }
        return;
    }
    if (lay.nbits > 34)
        throw Error(EDGPU_ERR_ARG, "sector enumeration over a generic site layout is limited to 34 bits "
                                   "(spin-1/2 single-sector spaces have no limit)");
    SectorBuffers sb(lay);
    EnumParams p{};
    p.src = SRC_RANGE;
    p.total = 1LL << lay.nbits;
    p.check_sector = 1;
    p.sec = sb.dev;
    p.check_rep = 0;
    s.dim = run_filtered<W>(p, &s.d_keys, !s.lazy, st);
}

template <typename W>
void enumerate_reps_t(Space& red, const Space& parent, cudaStream_t st) {
    const Layout& lay = parent.lay;
    GroupBuffers gb;
    gb.upload(red.group, lay);
    EnumParams p{};
    p.check_rep = 1;
    p.grp = gb.dev;
    if (parent.d_keys) {
        p.src = SRC_LIST;
        p.list = parent.d_keys;
        p.list_w32 = parent.w32 ? 1 : 0;
        p.total = parent.dim;
        red.dim = run_filtered<W>(p, &red.d_keys, true, st);
    } else if (lay.popcount >= 0) {
        p.src = SRC_COMBO;
        p.total = (long long)host_binom(lay.nbits, lay.popcount);
        p.n = lay.nbits;
        p.k = lay.popcount;
        p.C = binomial_table();
        red.dim = run_filtered<W>(p, &red.d_keys, true, st);
    } else {
        if (lay.nbits > 34) throw Error(EDGPU_ERR_ARG, "lazy generic sector limited to 34 bits");
        SectorBuffers sb(lay);
        p.src = SRC_RANGE;
        p.total = 1LL << lay.nbits;
        p.check_sector = 1;
        p.sec = sb.dev;
        red.dim = run_filtered<W>(p, &red.d_keys, true, st);
    }
}

// basis_mapping_index / basis_mapping_amplitude for every parent word: orbit minimum, its index in
// the representative table (-1 when the orbit is incompatible), chi(h)/sqrt(|O|) with h.p = rep.
template <typename W, typename PW>
__global__ void k_mapping(const PW* parent, long long n_parent, const W* reps, long long n_reps, int sb, GroupDev g,
                          const double2* phase, long long* index_out, double2* ampl_out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_parent) return;
    const W q = (W)parent[i];
    W rep = q;
    int gb = 0, stab = 1;
    if (g.kind == GK_TORUS) {
        W keep[64];
        for (int a = 0; a < g.L1; ++a) keep[a] = (W)g.keep[a];
        canon_torus<W>(q, g.L1, g.L2, g.w, g.rowbits, g.nbits, (W)g.full, keep, true, true, rep, gb, stab);
    } else if (g.kind == GK_GENERIC) {
        rep = q; gb = 0; stab = 0;
        for (int e = 0; e < g.G; ++e) {
            W t = 0;
            const unsigned long long* L = g.lut + (size_t)e * g.nchunks * 16;
            for (int c = 0; c < g.nchunks; ++c) t |= (W)L[c * 16 + (int)((q >> (4 * c)) & 15u)];
            t ^= (W)g.flips[e];
            if (t < rep) { rep = t; gb = e; }
            stab += (t == q);
        }
    }
    const long long c = key_find<W>(reps, n_reps, rep, sb, nullptr);
    index_out[i] = c;
    double2 a = make_double2(0.0, 0.0);
    if (c >= 0) {
        const double s = sqrt((double)stab / (double)g.G);
        const double2 ph = phase[g.num[gb]];
        a = make_double2(ph.x * s, ph.y * s);
    }
    ampl_out[i] = a;
}

template <typename W>
__global__ void k_orbit_sizes(const W* reps, long long n, int sb, GroupDev g, int32_t* out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const W q = reps[i] >> sb;
    int stab = 1;
    if (g.kind == GK_TORUS) {
        W keep[64];
        for (int a = 0; a < g.L1; ++a) keep[a] = (W)g.keep[a];
        W rep;
        int gb;
        canon_torus<W>(q, g.L1, g.L2, g.w, g.rowbits, g.nbits, (W)g.full, keep, false, true, rep, gb, stab);
    } else if (g.kind == GK_GENERIC) {
        stab = 0;
        for (int e = 0; e < g.G; ++e) {
            W t = 0;
            const unsigned long long* L = g.lut + (size_t)e * g.nchunks * 16;
            for (int c = 0; c < g.nchunks; ++c) t |= (W)L[c * 16 + (int)((q >> (4 * c)) & 15u)];
            t ^= (W)g.flips[e];
            stab += (t == q);
        }
    }
    out[i] = g.G / stab;
}

template <typename W>
__global__ void k_lookup(const W* keys, long long n, int sb, const unsigned long long* q, long long m, long long* out,
                         unsigned long long smax) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const unsigned long long k = q[i];
    out[i] = (k > smax) ? -1 : key_find<W>(keys, n, (W)k, sb, nullptr);
}

template <typename W>
__global__ void k_get_states(const W* keys, long long n, int sb, unsigned long long* out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (unsigned long long)(keys[i] >> sb);
}

// key = (state << sb) | index of the stabiliser size among the divisors of G
template <typename W>
__global__ void k_embed(W* keys, long long n, int sb, GroupDev g, const int32_t* divi) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const W q = keys[i];
    int stab = 1;
    if (g.kind == GK_TORUS) {
        W keep[64];
        for (int a = 0; a < g.L1; ++a) keep[a] = (W)g.keep[a];
        W rep;
        int gb;
        canon_torus<W>(q, g.L1, g.L2, g.w, g.rowbits, g.nbits, (W)g.full, keep, false, true, rep, gb, stab);
    } else if (g.kind == GK_GENERIC) {
        stab = 0;
        for (int e = 0; e < g.G; ++e) {
            W t = 0;
            const unsigned long long* L = g.lut + (size_t)e * g.nchunks * 16;
            for (int c = 0; c < g.nchunks; ++c) t |= (W)L[c * 16 + (int)((q >> (4 * c)) & 15u)];
            t ^= (W)g.flips[e];
            stab += (t == q);
        }
    }
    keys[i] = (W)((q << sb) | (W)divi[stab]);
}

// Bucket width of a search directory: for every candidate shift s in [s_lo, s_lo + n_shift) count
// the keys whose bucket (state >> s) holds at most K(s) keys, K(s) = min(4, 28 / (s + sb)) (the keys
// a bucket summary can carry).  A bucket holds more than K keys exactly when some K+1 consecutive
// keys around key i share its bucket, so each key reads its K neighbours on either side.
template <typename W>
__global__ void k_dir_survey(const W* keys, long long n, int sb, int s_lo, int n_shift, unsigned long long* counts) {
    __shared__ unsigned long long part[64];
    for (int j = threadIdx.x; j < n_shift; j += blockDim.x) part[j] = 0ull;
    __syncthreads();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < n;
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long v[9];   // states of keys i-4 .. i+4 (v valid where 0 <= index < n)
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        const long long w = i - 4 + j;
        v[j] = (act && w >= 0 && w < n) ? (unsigned long long)(keys[w] >> sb) : 0ull;
    }
    for (int j = 0; j < n_shift; ++j) {
        const int sh = s_lo + j, mb = sh + sb;
        const int K = mb == 0 ? 4 : min(4, 28 / mb);
        bool ok = act;
#pragma unroll
        for (int a = 0; a <= 4; ++a) {   // the K+1 keys from w = i-4+a (windows through i: a >= 4-K)
            const long long w = i - 4 + a;
            if (a >= 4 - K && w >= 0 && w + K < n && (v[a] >> sh) == (v[a + K] >> sh)) ok = false;
        }
        ok = ok && act;
        const unsigned cnt = __popc(__ballot_sync(0xffffffffu, ok));
        if (lane == 0 && cnt) atomicAdd(&part[j], (unsigned long long)cnt);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < n_shift; j += blockDim.x)
        if (part[j]) atomicAdd(&counts[j], part[j]);
}

// Search directory, one entry per bucket b in [0, nb) plus the sentinel dir[nb] = n:
// dir[b] = start | min(count, 15) << 32 | the low mb bits of each key << (36 + k*mb) when the bucket
// holds at most K keys (start = index of the bucket's first key, or of the next key when empty).
// Each thread builds DIR_CHUNK consecutive buckets: one binary search for the first key of its
// chunk, then a walk over the chunk's keys.  stats[0] receives the largest bucket and stats[1] the
// number of keys answered by their bucket summary.
constexpr int DIR_CHUNK = 128;

template <typename W>
__global__ void k_dir_build(const W* keys, long long n, int sb, int shift, long long nb, int mb, int K,
                            unsigned long long* dir, unsigned long long* stats) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long b0 = t * DIR_CHUNK;
    unsigned long long mx = 0ull, inl = 0ull;
    if (b0 <= nb) {
        long long lo = 0, len = n;   // first key with bucket >= b0
        while (len > 0) {
            const long long half = len >> 1;
            if ((long long)((keys[lo + half] >> sb) >> shift) < b0) {
                lo += half + 1;
                len -= half + 1;
            } else {
                len = half;
            }
        }
        long long i = lo;
        const unsigned long long mbmask = (mb >= 64) ? ~0ull : ((1ull << mb) - 1ull);
        const long long b1 = min(b0 + DIR_CHUNK, nb + 1);
        for (long long bb = b0; bb < b1; ++bb) {
            if (bb == nb) {
                dir[bb] = (unsigned long long)n;
                break;
            }
            const long long st = i;
            unsigned long long mem = 0ull;
            int k = 0;
            while (i < n && (long long)((keys[i] >> sb) >> shift) == bb) {
                if (k < K) mem |= ((unsigned long long)keys[i] & mbmask) << (36 + k * mb);
                ++k;
                ++i;
            }
            const unsigned long long cnt = (unsigned long long)k;
            if ((long long)cnt <= K) inl += cnt;
            else mem = 0ull;
            if (cnt > mx) mx = cnt;
            dir[bb] = (unsigned long long)st | (min(cnt, 15ull) << 32) | mem;
        }
    }
    for (int d = 16; d > 0; d >>= 1) {
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, d));
        inl += __shfl_xor_sync(0xffffffffu, inl, d);
    }
    if ((threadIdx.x & 31) == 0) {
        if (mx > 1) atomicMax(stats, mx);
        if (inl) atomicAdd(stats + 1, inl);
    }
}

template <typename W>
__global__ void k_count_nnz(const W* keys, long long n, int sb, GroupDev g, int T, const unsigned long long* masks,
                            const unsigned long long* rows, const unsigned long long* flips,
                            unsigned long long* counts /* [0] targets, [1] found */) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long nt = 0, nf = 0;
    if (r < n) {
        const W b = keys[r] >> sb;
        for (int t = 0; t < T; ++t) {
            if ((b & (W)masks[t]) != (W)rows[t]) continue;
            const W q = b ^ (W)flips[t];
            ++nt;
            W rep = q;
            int gb = 0, stab = 1;
            if (g.kind == GK_TORUS) {
                W keep[64];
                for (int a = 0; a < g.L1; ++a) keep[a] = (W)g.keep[a];
                canon_torus<W>(q, g.L1, g.L2, g.w, g.rowbits, g.nbits, (W)g.full, keep, false, false, rep, gb, stab);
            } else if (g.kind == GK_GENERIC) {
                for (int e = 0; e < g.G; ++e) {
                    W tt = 0;
                    const unsigned long long* L = g.lut + (size_t)e * g.nchunks * 16;
                    for (int c = 0; c < g.nchunks; ++c) tt |= (W)L[c * 16 + (int)((q >> (4 * c)) & 15u)];
                    tt ^= (W)g.flips[e];
                    if (tt < rep) rep = tt;
                }
            }
            nf += (key_find<W>(keys, n, rep, sb, nullptr) >= 0);
        }
    }
    for (int d = 16; d > 0; d >>= 1) {
        nt += __shfl_down_sync(0xffffffffu, nt, d);
        nf += __shfl_down_sync(0xffffffffu, nf, d);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counts, nt);
        atomicAdd(counts + 1, nf);
    }
}

template <typename W>
void count_nnz_t(const Space& s, int T, const uint64_t* masks, const uint64_t* rows, const uint64_t* flips,
                 int64_t* n_targets, int64_t* n_found, cudaStream_t st) {
    GroupBuffers gb;
    gb.upload(s.group, s.lay);
    unsigned long long* d = nullptr;
    const size_t tb = std::max(T, 1) * sizeof(unsigned long long);
    EDGPU_CUDA(cudaMalloc(&d, 3 * tb + 2 * sizeof(unsigned long long)));
    unsigned long long* dm = d;
    unsigned long long* dr = d + std::max(T, 1);
    unsigned long long* df = d + 2 * std::max(T, 1);
    unsigned long long* dc = d + 3 * std::max(T, 1);
    cudaError_t e = cudaSuccess;
    unsigned long long h[2] = {0, 0};
    if (T > 0) e = cudaMemcpyAsync(dm, masks, T * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && T > 0) e = cudaMemcpyAsync(dr, rows, T * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && T > 0) e = cudaMemcpyAsync(df, flips, T * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dc, 0, 2 * sizeof(unsigned long long), st);
    if (e == cudaSuccess && s.dim > 0) {
        k_count_nnz<W><<<(unsigned)((s.dim + 255) / 256), 256, 0, st>>>((const W*)s.d_keys, s.dim, s.sb, gb.dev, T, dm, dr, df, dc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, dc, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d);
    if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("count_nnz: ") + cudaGetErrorString(e));
    *n_targets = (int64_t)h[0];
    *n_found = (int64_t)h[1];
}

}  // namespace

// ---- host side ----------------------------------------------------------------------------------

std::vector<unsigned long long> torus_keep_masks(const Group& g, int nbits) {
    const int rowbits = g.L1 * g.w;
    std::vector<unsigned long long> keep(g.L1);
    for (int a = 0; a < g.L1; ++a) {
        const int s = a * g.w;
        const unsigned long long row_keep = (rowbits - s >= 64) ? ~0ull : ((1ull << (rowbits - s)) - 1ull);
        unsigned long long m = 0;
        for (int r = 0; r < g.L2; ++r) m |= row_keep << (r * rowbits);
        keep[a] = m;
    }
    (void)nbits;
    return keep;
}

std::vector<unsigned long long> generic_luts(const Group& g, const Layout& lay, int* nchunks) {
    const int nc = (lay.nbits + 3) / 4;
    *nchunks = nc;
    std::vector<unsigned long long> lut((size_t)g.G * nc * 16, 0ull);
    for (int e = 0; e < g.G; ++e) {
        const int32_t* map = g.maps.data() + (size_t)e * lay.n_sites;
        for (int c = 0; c < nc; ++c) {
            for (int v = 0; v < 16; ++v) {
                const unsigned long long word = (unsigned long long)v << (4 * c);
                unsigned long long out = 0;
                for (int i = 0; i < lay.n_sites; ++i) {
                    const unsigned long long m = (lay.bw[i] >= 64) ? ~0ull : ((1ull << lay.bw[i]) - 1ull);
                    out |= ((word >> lay.off[i]) & m) << lay.off[map[i]];
                }
                lut[((size_t)e * nc + c) * 16 + v] = out;
            }
        }
    }
    return lut;
}

void GroupBuffers::upload(const Group& g, const Layout& lay) {
    release();
    dev = GroupDev{};
    dev.kind = g.kind;
    dev.G = g.G;
    dev.den = g.den;
    dev.L1 = g.L1;
    dev.L2 = g.L2;
    dev.w = g.w;
    dev.rowbits = g.L1 * g.w;
    dev.nbits = lay.nbits;
    dev.full = (lay.nbits >= 64) ? ~0ull : ((1ull << lay.nbits) - 1ull);
    EDGPU_CUDA(cudaMalloc(&d_num, std::max<size_t>(g.num.size(), 1) * sizeof(int32_t)));
    EDGPU_CUDA(cudaMemcpy(d_num, g.num.data(), g.num.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    dev.num = d_num;
    if (g.kind == GK_TORUS) {
        auto keep = torus_keep_masks(g, lay.nbits);
        EDGPU_CUDA(cudaMalloc(&d_keep, keep.size() * sizeof(unsigned long long)));
        EDGPU_CUDA(cudaMemcpy(d_keep, keep.data(), keep.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice));
        dev.keep = d_keep;
    } else if (g.kind == GK_GENERIC) {
        int nc = 0;
        auto lut = generic_luts(g, lay, &nc);
        dev.nchunks = nc;
        EDGPU_CUDA(cudaMalloc(&d_lut, lut.size() * sizeof(unsigned long long)));
        EDGPU_CUDA(cudaMemcpy(d_lut, lut.data(), lut.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice));
        EDGPU_CUDA(cudaMalloc(&d_flips, g.G * sizeof(unsigned long long)));
        std::vector<unsigned long long> fl(g.flips.begin(), g.flips.end());
        fl.resize(g.G, 0ull);
        EDGPU_CUDA(cudaMemcpy(d_flips, fl.data(), g.G * sizeof(unsigned long long), cudaMemcpyHostToDevice));
        dev.lut = d_lut;
        dev.flips = d_flips;
    }
}

void GroupBuffers::release() {
    cudaFree(d_num);
    cudaFree(d_keep);
    cudaFree(d_lut);
    cudaFree(d_flips);
    d_num = nullptr;
    d_keep = nullptr;
    d_lut = nullptr;
    d_flips = nullptr;
}

Space::~Space() {
    if (d_keys) cudaFree(d_keys);
    if (d_dir) cudaFree(d_dir);
    if (d_map) cudaFree(d_map);
    if (d_rank) cudaFree(d_rank);
}

void enumerate_parent(Space& s, cudaStream_t st) {
    if (s.w32) enumerate_parent_t<uint32_t>(s, st);
    else enumerate_parent_t<unsigned long long>(s, st);
}

void enumerate_reps(Space& red, const Space& parent, cudaStream_t st) {
    if (red.w32) enumerate_reps_t<uint32_t>(red, parent, st);
    else enumerate_reps_t<unsigned long long>(red, parent, st);
}

namespace {
template <typename W>
void build_mapping_t(const Space& red, const Space& parent, int64_t* index_out, double* ampl_out, cudaStream_t st) {
    GroupBuffers gb;
    gb.upload(red.group, parent.lay);
    std::vector<double> ph(2 * (size_t)red.group.den);
    for (int j = 0; j < red.group.den; ++j) {
        const double ang = 2.0 * M_PI * (double)j / (double)red.group.den;
        ph[2 * j] = std::cos(ang);
        ph[2 * j + 1] = std::sin(ang);
    }
    double2* d_ph = nullptr;
    long long* d_idx = nullptr;
    double2* d_amp = nullptr;
    const long long n = parent.dim;
    try {
        EDGPU_CUDA(cudaMalloc(&d_ph, ph.size() * sizeof(double)));
        EDGPU_CUDA(cudaMemcpy(d_ph, ph.data(), ph.size() * sizeof(double), cudaMemcpyHostToDevice));
        EDGPU_CUDA(cudaMalloc(&d_idx, std::max<long long>(n, 1) * sizeof(long long)));
        EDGPU_CUDA(cudaMalloc(&d_amp, std::max<long long>(n, 1) * sizeof(double2)));
        if (n > 0) {
            if (parent.w32)
                k_mapping<W, unsigned><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
                    (const unsigned*)parent.d_keys, n, (const W*)red.d_keys, red.dim, red.sb, gb.dev, d_ph, d_idx, d_amp);
            else
                k_mapping<W, unsigned long long><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
                    (const unsigned long long*)parent.d_keys, n, (const W*)red.d_keys, red.dim, red.sb, gb.dev, d_ph,
                    d_idx, d_amp);
            EDGPU_CUDA(cudaGetLastError());
            EDGPU_CUDA(cudaMemcpyAsync(index_out, d_idx, n * sizeof(long long), cudaMemcpyDeviceToHost, st));
            EDGPU_CUDA(cudaMemcpyAsync(ampl_out, d_amp, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
            EDGPU_CUDA(cudaStreamSynchronize(st));
        }
    } catch (...) {
        cudaFree(d_ph);
        cudaFree(d_idx);
        cudaFree(d_amp);
        throw;
    }
    cudaFree(d_ph);
    cudaFree(d_idx);
    cudaFree(d_amp);
}

// Parent-state map over the fixed-popcount parent sector (see Space::d_map): one thread per colex rank
// r: the parent state q = unrank(r), its orbit minimum and an element reaching it, the representative's
// index by the search directory, packed into one entry (all ones when the orbit is not in the table).
template <typename W, typename E>
__global__ void k_build_map(long long n_parent, int n, int k, const unsigned long long* C, const W* reps,
                            DirSearch ds, GroupDev g, int cb, int direct, E* out) {
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n_parent;
         r += (long long)gridDim.x * blockDim.x) {
        const W q = unrank_combo<W>((unsigned long long)r, n, k, C);
        W rep = q;
        int gb = 0, stab = 1;
        if (g.kind == GK_TORUS) {
            W keep[64];
            for (int a = 0; a < g.L1; ++a) keep[a] = (W)g.keep[a];
            canon_torus<W>(q, g.L1, g.L2, g.w, g.rowbits, g.nbits, (W)g.full, keep, true, false, rep, gb, stab);
        } else if (g.kind == GK_GENERIC) {
            for (int e = 0; e < g.G; ++e) {
                W t = 0;
                const unsigned long long* L = g.lut + (size_t)e * g.nchunks * 16;
                for (int c = 0; c < g.nchunks; ++c) t |= (W)L[c * 16 + (int)((q >> (4 * c)) & 15u)];
                t ^= (W)g.flips[e];
                if (t < rep) {
                    rep = t;
                    gb = e;
                }
            }
        }
        W reps2[2] = {rep, rep};
        const bool act[2] = {true, false};
        long long c[2];
        int sx[2];
        key_find_sum2<W>(reps, ds, reps2, act, c, sx);
        E e = (E)~(E)0;
        if (c[0] >= 0) e = (E)c[0] | ((E)sx[0] << cb) | (g.den > 1 ? (E)gb << (cb + ds.sb) : (E)0);
        out[direct ? (long long)q : r] = e;
    }
}

template <typename W>
void orbit_sizes_t(const Space& red, int32_t* out_host, cudaStream_t st) {
    GroupBuffers gb;
    gb.upload(red.group, red.lay);
    int32_t* d = nullptr;
    const long long n = red.dim;
    EDGPU_CUDA(cudaMalloc(&d, std::max<long long>(n, 1) * sizeof(int32_t)));
    if (n > 0) {
        k_orbit_sizes<W><<<(unsigned)((n + 255) / 256), 256, 0, st>>>((const W*)red.d_keys, n, red.sb, gb.dev, d);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(out_host, d, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            cudaFree(d);
            throw Error(EDGPU_ERR_CUDA, std::string("orbit sizes: ") + cudaGetErrorString(e));
        }
    }
    cudaFree(d);
}

template <typename W>
void lookup_t(const Space& s, const uint64_t* keys_host, int64_t n, int64_t* out_host, cudaStream_t st) {
    unsigned long long* dq = nullptr;
    long long* dout = nullptr;
    try {
        EDGPU_CUDA(cudaMalloc(&dq, std::max<int64_t>(n, 1) * sizeof(unsigned long long)));
        EDGPU_CUDA(cudaMalloc(&dout, std::max<int64_t>(n, 1) * sizeof(long long)));
        EDGPU_CUDA(cudaMemcpyAsync(dq, keys_host, n * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
        const unsigned long long smax = (s.lay.nbits >= 64) ? ~0ull : ((1ull << s.lay.nbits) - 1ull);
        k_lookup<W><<<(unsigned)((n + 255) / 256), 256, 0, st>>>((const W*)s.d_keys, s.dim, s.sb, dq, n, dout, smax);
        EDGPU_CUDA(cudaGetLastError());
        EDGPU_CUDA(cudaMemcpyAsync(out_host, dout, n * sizeof(long long), cudaMemcpyDeviceToHost, st));
        EDGPU_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        cudaFree(dq);
        cudaFree(dout);
        throw;
    }
    cudaFree(dq);
    cudaFree(dout);
}
}  // namespace

void build_mapping(const Space& red, const Space& parent, int64_t* index_out, double* ampl_out, cudaStream_t st) {
    if (red.w32) build_mapping_t<uint32_t>(red, parent, index_out, ampl_out, st);
    else build_mapping_t<unsigned long long>(red, parent, index_out, ampl_out, st);
}

void orbit_sizes(const Space& red, int32_t* out_host, cudaStream_t st) {
    if (red.w32) orbit_sizes_t<uint32_t>(red, out_host, st);
    else orbit_sizes_t<unsigned long long>(red, out_host, st);
}

void lookup_keys(const Space& s, const uint64_t* keys_host, int64_t n, int64_t* out_host, cudaStream_t st) {
    if (n <= 0) return;
    if (s.w32) lookup_t<uint32_t>(s, keys_host, n, out_host, st);
    else lookup_t<unsigned long long>(s, keys_host, n, out_host, st);
}

}  // namespace edgpu

namespace edgpu {
void count_nnz(const Space& s, int T, const uint64_t* masks, const uint64_t* rows, const uint64_t* flips,
               int64_t* n_targets, int64_t* n_found, cudaStream_t st) {
    if (s.w32) count_nnz_t<uint32_t>(s, T, masks, rows, flips, n_targets, n_found, st);
    else count_nnz_t<unsigned long long>(s, T, masks, rows, flips, n_targets, n_found, st);
}
}  // namespace edgpu

namespace edgpu {

int orbit_index_bits(int G) {
    int nd = 0;
    for (int d = 1; d <= G; ++d) nd += (G % d == 0);
    int b = 0;
    while ((1 << b) < nd) ++b;
    return b;
}

namespace {
template <typename W>
void embed_t(Space& red, cudaStream_t st) {
    GroupBuffers gb;
    gb.upload(red.group, red.lay);
    std::vector<int32_t> divi(red.group.G + 1, 0);
    int k = 0;
    for (int d = 1; d <= red.group.G; ++d)
        if (red.group.G % d == 0) divi[d] = k++;
    int32_t* d_divi = nullptr;
    EDGPU_CUDA(cudaMalloc(&d_divi, divi.size() * sizeof(int32_t)));
    cudaError_t e = cudaMemcpy(d_divi, divi.data(), divi.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && red.dim > 0) {
        k_embed<W><<<(unsigned)((red.dim + 255) / 256), 256, 0, st>>>((W*)red.d_keys, red.dim, red.sb, gb.dev, d_divi);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaFree(d_divi);
    if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("embed: ") + cudaGetErrorString(e));
}

template <typename W>
void dir_t(Space& s, cudaStream_t st) {
    const long long n = s.dim;
    if (n >= (1ll << 32)) throw Error(EDGPU_ERR_ARG, "tables of 2^32 or more rows are not supported");
    unsigned long long max_state = 0;
    if (n > 0) {
        W last;
        EDGPU_CUDA(cudaMemcpy(&last, (const W*)s.d_keys + (n - 1), sizeof(W), cudaMemcpyDeviceToHost));
        max_state = (unsigned long long)(last >> s.sb);
    }
    int bitlen = 0;
    while (bitlen < 64 && (max_state >> bitlen) != 0ull) ++bitlen;
    int nbits_n = 0;
    while ((1ll << nbits_n) < std::max<long long>(n, 1)) ++nbits_n;
    // the directory may use up to 16x the key table (HBM is plentiful; a clustered table needs small
    // buckets before most of its keys fit in their bucket summaries)
    const size_t cap_bytes = std::max<size_t>((size_t)512 << 20, 16 * (size_t)n * sizeof(W));
    // candidate shifts: from about one bucket per key (s_hi) down to the smallest the cap allows
    // bucket summaries need member fields of at least one bit (shift + sb >= 1): a dense table of
    // unreduced keys (every state present) gets buckets of two states
    const int min_shift = s.sb == 0 ? 1 : 0;
    const int s_hi = std::max(min_shift, bitlen - std::max(1, std::min(nbits_n, bitlen)));
    int s_lo = s_hi;
    while (s_lo > min_shift && s_hi - s_lo < 63 &&
           (size_t)((max_state >> (s_lo - 1)) + 2) * sizeof(unsigned long long) <= cap_bytes)
        --s_lo;
    const int n_shift = s_hi - s_lo + 1;
    unsigned long long* d_stats = nullptr;   // survey counts [n_shift], then [largest bucket, inline keys]
    EDGPU_CUDA(cudaMalloc(&d_stats, (n_shift + 2) * sizeof(unsigned long long)));
    std::vector<unsigned long long> cnt(n_shift + 2, 0ull);
    cudaError_t e = cudaMemsetAsync(d_stats, 0, (n_shift + 2) * sizeof(unsigned long long), st);
    if (e == cudaSuccess && n > 0) {
        k_dir_survey<W><<<(unsigned)((n + 255) / 256), 256, 0, st>>>((const W*)s.d_keys, n, s.sb, s_lo, n_shift, d_stats);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnt.data(), d_stats, n_shift * sizeof(unsigned long long),
                                              cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaFree(d_stats);
        throw Error(EDGPU_ERR_CUDA, std::string("search directory survey: ") + cudaGetErrorString(e));
    }
    // the widest buckets whose summaries answer at least 98% of the keys, else the best fraction
    int shift = s_hi;
    double best = -1.0;
    for (int sh = s_hi; sh >= s_lo; --sh) {
        const double f = n > 0 ? (double)cnt[sh - s_lo] / (double)n : 1.0;
        if (f > best) {
            best = f;
            shift = sh;
        }
        if (f >= 0.98) break;
    }
    const long long nb = (bitlen == 0) ? 1 : ((long long)(max_state >> shift) + 1);
    const int mb = shift + s.sb;
    const int K = mb == 0 ? 4 : std::min(4, 28 / mb);
    if (s.d_dir) cudaFree(s.d_dir);
    s.d_dir = nullptr;
    e = cudaMalloc(&s.d_dir, (nb + 1) * sizeof(unsigned long long));
    if (e == cudaSuccess) {
        const long long threads = nb / DIR_CHUNK + 1;
        k_dir_build<W><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>((const W*)s.d_keys, n, s.sb, shift, nb, mb, K,
                                                                          s.d_dir, d_stats + n_shift);
        e = cudaGetLastError();
    }
    unsigned long long hs[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(hs, d_stats + n_shift, sizeof(hs), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_stats);
    if (e != cudaSuccess) {
        if (s.d_dir) cudaFree(s.d_dir);
        s.d_dir = nullptr;
        throw Error(e == cudaErrorMemoryAllocation ? EDGPU_ERR_OOM : EDGPU_ERR_CUDA,
                    std::string("search directory: ") + cudaGetErrorString(e));
    }
    s.dir_shift = shift;
    s.dir_nb = nb;
    s.dir_K = K;
    s.dir_inline = n > 0 ? (double)hs[1] / (double)n : 1.0;
    int steps = 0;
    while ((1ull << steps) < std::max<unsigned long long>(hs[0], 1ull)) ++steps;
    s.dir_steps = steps;
}

template <typename W>
void states_t(const Space& s, uint64_t* out_host, cudaStream_t st) {
    unsigned long long* d = nullptr;
    EDGPU_CUDA(cudaMalloc(&d, std::max<int64_t>(s.dim, 1) * 8));
    k_get_states<W><<<(unsigned)((s.dim + 255) / 256), 256, 0, st>>>((const W*)s.d_keys, s.dim, s.sb, d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out_host, d, s.dim * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d);
    if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("get_states: ") + cudaGetErrorString(e));
}
}  // namespace

DirSearch dir_search_of(const Space& s) {
    DirSearch d{};
    d.dir = s.d_dir;
    d.nb = s.dir_nb;
    d.shift = s.dir_shift;
    d.mb = s.dir_shift + s.sb;
    d.K = s.dir_K;
    d.steps = s.dir_steps;
    d.sb = s.sb;
    const unsigned mbmask = d.mb >= 32 ? 0xffffffffu : ((1u << d.mb) - 1u);
    const unsigned smask = (1u << d.sb) - 1u;
    for (int k = 0; k < d.K; ++k) {
        const int o = k * d.mb;
        d.unit |= 1u << o;
        d.keybits |= (mbmask & ~smask) << o;
        d.low |= (mbmask >> 1) << o;
        d.top |= (1u << (d.mb - 1)) << o;
    }
    return d;
}

void embed_orbit_index(Space& red, cudaStream_t st) {
    if (red.sb == 0 || red.dim == 0) return;
    if (red.w32) embed_t<uint32_t>(red, st);
    else embed_t<unsigned long long>(red, st);
}

void build_search_directory(Space& s, cudaStream_t st) {
    if (s.w32) dir_t<uint32_t>(s, st);
    else dir_t<unsigned long long>(s, st);
}

namespace {
int bitlen_u64(unsigned long long v) {
    int b = 0;
    while (b < 64 && (v >> b) != 0ull) ++b;
    return b;
}

template <typename W>
void build_map_t(Space& red, cudaStream_t st) {
    const Layout& L = red.lay;
    const int n = L.nbits, k = L.popcount;
    const long long np = (long long)host_binom(n, k);   // parent states (the map may be larger when direct)
    GroupBuffers gb;
    gb.upload(red.group, L);
    const DirSearch ds = dir_search_of(red);
    const unsigned blocks = (unsigned)std::min<long long>((np + 255) / 256, 152ll * 64);
    if (red.map_wide)
        k_build_map<W, unsigned long long><<<blocks, 256, 0, st>>>(np, n, k, binomial_table(), (const W*)red.d_keys, ds,
                                                                  gb.dev, red.map_cb, red.map_direct,
                                                                  (unsigned long long*)red.d_map);
    else
        k_build_map<W, unsigned><<<blocks, 256, 0, st>>>(np, n, k, binomial_table(), (const W*)red.d_keys, ds, gb.dev,
                                                        red.map_cb, red.map_direct, (unsigned*)red.d_map);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("parent map: ") + cudaGetErrorString(e));
}
}  // namespace

void free_parent_map(Space& red) {
    if (red.d_map) cudaFree(red.d_map);
    if (red.d_rank) cudaFree(red.d_rank);
    red.d_map = nullptr;
    red.d_rank = nullptr;
    red.map_n = 0;
    ++red.map_gen;
}

bool build_parent_map(Space& red, int64_t max_bytes, cudaStream_t st) {
    const Layout& L = red.lay;
    if (!red.reduced || L.popcount < 0 || L.nbits > 64 || red.dim == 0 || !red.d_keys || !red.d_dir) return false;
    const int n = L.nbits, k = L.popcount;
    const unsigned long long np = host_binom(n, k);
    const int cb = bitlen_u64((unsigned long long)red.dim);
    // the element is needed only for characters other than 1
    const int gbits = red.group.den > 1 ? bitlen_u64((unsigned long long)std::max(red.group.G - 1, 0)) : 0;
    const int wide = (cb + red.sb + gbits <= 32) ? 0 : 1;
    if (cb + red.sb + gbits > 64) return false;
    const double bytes = (double)np * (wide ? 8.0 : 4.0);
    if (bytes > (double)max_bytes) return false;
    // direct indexing (entry index = the state itself, no rank) when the whole state range is small:
    // at most 2^30 entries and 4 GB, within the limit
    const double dbytes = n <= 30 ? (double)(1ull << n) * (wide ? 8.0 : 4.0) : 1e300;
    const bool direct = dbytes <= std::min((double)max_bytes, 4.0 * (1ull << 30));
    // Colex rank tables.  Split form (n <= 44): with lb = n / 2 low bits, the rank of q = (H << lb) | L
    // is A[H] + B[L], where A[H] counts the sector's states whose high part is below H (sum over
    // H' < H of C(lb, k - popc(H'))) and B[L] is the rank of L among the lb-bit words of its popcount.
    // Chunk form (larger n): T[(c * (k + 1) + j) * 64 + v] = sum over the set bits b of v, in ascending
    // order t = 0, 1, ..., of C(6c + b, j + t + 1).
    const int rank_wide = np > 0xffffffffull ? 1 : 0;
    const int split = n <= 44 ? n / 2 : 0;
    std::vector<unsigned long long> T;
    if (split) {
        const int lb = split, hb = n - split;
        T.assign(((size_t)1 << hb) + ((size_t)1 << lb), 0ull);
        unsigned long long acc = 0;
        for (size_t h = 0; h < ((size_t)1 << hb); ++h) {
            T[h] = acc;
            const int need = k - __builtin_popcountll(h);
            acc += (need >= 0 && need <= lb) ? host_binom(lb, need) : 0ull;
        }
        std::vector<unsigned long long> cnt(lb + 1, 0ull);
        for (size_t l = 0; l < ((size_t)1 << lb); ++l) T[((size_t)1 << hb) + l] = cnt[__builtin_popcountll(l)]++;
    } else {
        const int nc = (n + RANK_CHUNK - 1) / RANK_CHUNK;
        T.assign((size_t)nc * (k + 1) * 64, 0ull);
        for (int c = 0; c < nc; ++c)
            for (int j = 0; j <= k; ++j)
                for (int v = 0; v < 64; ++v) {
                    unsigned long long sum = 0;
                    int t = 0;
                    for (int bb = 0; bb < RANK_CHUNK; ++bb)
                        if ((v >> bb) & 1) {
                            sum += host_binom(RANK_CHUNK * c + bb, j + t + 1);
                            ++t;
                        }
                    T[((size_t)c * (k + 1) + j) * 64 + v] = sum;
                }
    }
    free_parent_map(red);
    std::vector<unsigned> T32;
    if (!rank_wide) T32.assign(T.begin(), T.end());
    const size_t tbytes = T.size() * (rank_wide ? 8 : 4);
    cudaError_t e = cudaMalloc(&red.d_rank, tbytes);
    if (e == cudaSuccess)
        e = cudaMemcpy(red.d_rank, rank_wide ? (const void*)T.data() : (const void*)T32.data(), tbytes,
                       cudaMemcpyHostToDevice);
    const size_t entries = direct ? ((size_t)1 << n) : (size_t)np;
    if (e == cudaSuccess) e = cudaMalloc(&red.d_map, entries * (wide ? 8 : 4));
    if (e == cudaSuccess && direct) e = cudaMemsetAsync(red.d_map, 0xff, entries * (wide ? 8 : 4), st);   // invalid
    if (e != cudaSuccess) {
        free_parent_map(red);
        if (e == cudaErrorMemoryAllocation) return false;
        throw Error(EDGPU_ERR_CUDA, std::string("parent map: ") + cudaGetErrorString(e));
    }
    red.map_direct = direct ? 1 : 0;
    red.map_n = (int64_t)entries;
    red.map_wide = wide;
    red.map_cb = cb;
    red.rank_wide = rank_wide;
    red.rank_split = split;
    try {
        if (red.w32) build_map_t<uint32_t>(red, st);
        else build_map_t<unsigned long long>(red, st);
    } catch (...) {
        free_parent_map(red);
        throw;
    }
    ++red.map_gen;
    return true;
}

void get_states(const Space& s, uint64_t* out_host, cudaStream_t st) {
    if (s.dim == 0) return;
    if (s.w32) states_t<uint32_t>(s, out_host, st);
    else states_t<unsigned long long>(s, out_host, st);
}

}  // namespace edgpu

namespace edgpu {
namespace {
template <typename W>
__global__ void k_diag(const W* keys, long long n, int sb, int T, const unsigned long long* masks,
                       const unsigned long long* rows, const double2* amps, double2* out64, float2* out32) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const W b = keys[i] >> sb;
    double2 e = make_double2(0.0, 0.0);
    for (int t = 0; t < T; ++t)
        if ((b & (W)masks[t]) == (W)rows[t]) {
            e.x += amps[t].x;
            e.y += amps[t].y;
        }
    if (out64) out64[i] = e;
    if (out32) out32[i] = make_float2((float)e.x, (float)e.y);
}

template <typename W>
void diag_t(const Space& s, int T, const uint64_t* masks, const uint64_t* rows, const double* amps, double* out64,
            float* out32, unsigned long long* scratch, cudaStream_t st) {
    unsigned long long* d = scratch;
    const size_t Tm = std::max(T, 1);
    if (!scratch) EDGPU_CUDA(cudaMalloc(&d, Tm * (8 + 8 + 16)));
    unsigned long long* dm = d;
    unsigned long long* dr = d + Tm;
    double2* da = (double2*)(d + 2 * Tm);
    cudaError_t e = cudaSuccess;
    if (T > 0) {
        e = cudaMemcpyAsync(dm, masks, T * 8, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dr, rows, T * 8, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(da, amps, T * 16, cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess && s.dim > 0) {
        k_diag<W><<<(unsigned)((s.dim + 255) / 256), 256, 0, st>>>((const W*)s.d_keys, s.dim, s.sb, T, dm, dr, da,
                                                                  (double2*)out64, (float2*)out32);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (!scratch) cudaFree(d);
    if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("diagonal: ") + cudaGetErrorString(e));
}
}  // namespace

void compute_diagonal(const Space& s, int T, const uint64_t* masks, const uint64_t* rows, const double* amps,
                      double* out64, float* out32, unsigned long long* scratch, cudaStream_t st) {
    if (s.w32) diag_t<uint32_t>(s, T, masks, rows, amps, out64, out32, scratch, st);
    else diag_t<unsigned long long>(s, T, masks, rows, amps, out64, out32, scratch, st);
}
}  // namespace edgpu

// ---- vectors between the parent space and the reduced space, on the device -----------------------
// symmetry_unreduce(rhsr, small) and symmetry_reduce(rhsr, large) (symmetry_reduce.jl:208-225 and
// :38-56): the reference reads its parent-sized tables basis_mapping_index / basis_mapping_amplitude;
// here every parent entry's representative, stabiliser and group element are recomputed, so they run
// for parents whose tables do not fit (a parent vector of 9.1e9 entries for the 6x6 torus does).
// Parent index i <-> state: the materialised parent's sorted basis, or for a lazy popcount sector the
// colex rank (rank = sum over the set bits, lowest first, of C(position, count so far)).
namespace edgpu {
namespace {

// g.q for element e of the group (T(a, b) with e = a + L1 b for a torus: rows rotated left by a sites,
// then the rows moved up by b; the chunk tables and flip mask for a general group).
template <typename W>
__device__ __forceinline__ W group_elem_apply(W q, int e, const GroupDev& g) {
    if (g.kind == GK_TORUS) {
        const int a = e % g.L1, b = e / g.L1;
        const W full = (W)g.full;
        W v = q;
        if (a) {
            const int s = a * g.w;
            const W keep = (W)g.keep[a];
            v = (W)(((v & keep) << s) | ((v & ~keep & full) >> (g.rowbits - s)));
        }
        const int sr = b * g.rowbits;
        if (sr) v = (W)(((v << sr) | (v >> (g.nbits - sr))) & full);
        return v;
    }
    if (g.kind == GK_GENERIC) {
        W t = 0;
        const unsigned long long* L = g.lut + (size_t)e * g.nchunks * 16;
        for (int c = 0; c < g.nchunks; ++c) t |= (W)L[c * 16 + (int)((q >> (4 * c)) & 15u)];
        return t ^ (W)g.flips[e];
    }
    return q;
}

template <typename W>
__device__ __forceinline__ long long colex_rank(W q, const unsigned long long* C) {
    long long r = 0;
    int j = 0;
    while (q) {
        const int pos = (sizeof(W) == 8) ? __ffsll((long long)q) - 1 : __ffs((int)q) - 1;
        ++j;
        r += (long long)C[pos * 65 + j];
        q &= q - 1;
    }
    return r;
}

// large[i] = ampl(p_i) small[c(p_i)] (0 where the orbit has no representative), the parent index i
// running over [0, n_parent).
template <typename W, typename PW, typename V>
__global__ void k_unreduce(const PW* parent, long long n_parent, int n, int k, const unsigned long long* C,
                           const W* reps, long long n_reps, int sb, GroupDev g, const double2* phase, const V* small,
                           V* large) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_parent;
         i += (long long)gridDim.x * blockDim.x) {
        const W q = parent ? (W)parent[i] : unrank_combo<W>((unsigned long long)i, n, k, C);
        W rep = q;
        int gb = 0, stab = 1;
        if (g.kind == GK_TORUS) {
            W keep[64];
            for (int a = 0; a < g.L1; ++a) keep[a] = (W)g.keep[a];
            canon_torus<W>(q, g.L1, g.L2, g.w, g.rowbits, g.nbits, (W)g.full, keep, true, true, rep, gb, stab);
        } else if (g.kind == GK_GENERIC) {
            stab = 0;
            for (int e = 0; e < g.G; ++e) {
                const W t = group_elem_apply<W>(q, e, g);
                if (t < rep) {
                    rep = t;
                    gb = e;
                }
                stab += (t == q);
            }
        }
        const long long c = key_find<W>(reps, n_reps, rep, sb, nullptr);
        V out;
        out.x = 0;
        out.y = 0;
        if (c >= 0) {
            const double s = sqrt((double)stab / (double)g.G);
            const double2 ph = phase[g.num[gb]];
            const V v = small[c];
            const double ar = ph.x * s, ai = ph.y * s;
            out.x = (decltype(out.x))(ar * (double)v.x - ai * (double)v.y);
            out.y = (decltype(out.y))(ar * (double)v.y + ai * (double)v.x);
        }
        large[i] = out;
    }
}

// small[c] = sum over the orbit members p of rep_c of conj(ampl(p)) large[i(p)].  Every element e of
// the group gives the member e.rep_c with ampl = conj(chi(e)) sqrt(|stab| / |G|); each distinct
// member occurs |stab| times among the |G| elements, so the sum over all elements is divided by
// |stab|.  One thread per representative, elements in a fixed order (reproducible, no atomics).
template <typename W, typename PW, typename V>
__global__ void k_reduce(const PW* parent, long long n_parent, const unsigned long long* C, const W* reps,
                         long long n_reps, int sb, GroupDev g, const double2* phase, const V* large, V* small) {
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n_reps;
         c += (long long)gridDim.x * blockDim.x) {
        const W rep = reps[c] >> sb;
        int stab = 0;
        for (int e = 0; e < g.G; ++e) stab += (group_elem_apply<W>(rep, e, g) == rep);
        const double s = sqrt((double)stab / (double)g.G) / (double)stab;
        double ar = 0.0, ai = 0.0;
        for (int e = 0; e < g.G; ++e) {
            const W t = group_elem_apply<W>(rep, e, g);
            long long i;
            if (parent) {
                long long lo = 0, len = n_parent;
                while (len > 0) {   // searchsortedfirst over the parent basis
                    const long long half = len >> 1;
                    if ((W)parent[lo + half] < t) {
                        lo += half + 1;
                        len -= half + 1;
                    } else {
                        len = half;
                    }
                }
                i = (lo < n_parent && (W)parent[lo] == t) ? lo : -1;
            } else {
                i = colex_rank<W>(t, C);
            }
            if (i < 0) continue;
            // conj(ampl(t)) = chi(e) sqrt(|stab| / |G|); chi(e) = phase[num[e]]
            const double2 ph = phase[g.num[e]];
            const V v = large[i];
            ar += ph.x * (double)v.x - ph.y * (double)v.y;
            ai += ph.x * (double)v.y + ph.y * (double)v.x;
        }
        V out;
        out.x = (decltype(out.x))(ar * s);
        out.y = (decltype(out.y))(ai * s);
        small[c] = out;
    }
}

template <typename W, typename PW, typename V>
void reduce_vector_t(const Space& red, const Space& parent, bool unreduce, const void* in, void* out,
                     cudaStream_t st) {
    GroupBuffers gb;
    gb.upload(red.group, parent.lay);
    std::vector<double> ph(2 * (size_t)red.group.den);
    for (int j = 0; j < red.group.den; ++j) {
        const double ang = 2.0 * M_PI * (double)j / (double)red.group.den;
        ph[2 * j] = std::cos(ang);
        ph[2 * j + 1] = std::sin(ang);
    }
    double2* d_ph = nullptr;
    EDGPU_CUDA(cudaMalloc(&d_ph, ph.size() * sizeof(double)));
    cudaError_t e = cudaMemcpyAsync(d_ph, ph.data(), ph.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    const PW* pk = parent.d_keys ? (const PW*)parent.d_keys : nullptr;
    const long long n_parent = parent.d_keys ? parent.dim : (long long)host_binom(parent.lay.nbits, parent.lay.popcount);
    const int blocks = std::max(1, sm_count() * 16);
    if (e == cudaSuccess) {
        if (unreduce)
            k_unreduce<W, PW, V><<<blocks, 256, 0, st>>>(pk, n_parent, parent.lay.nbits, parent.lay.popcount,
                                                          binomial_table(), (const W*)red.d_keys, red.dim, red.sb, gb.dev,
                                                          d_ph, (const V*)in, (V*)out);
        else
            k_reduce<W, PW, V><<<blocks, 256, 0, st>>>(pk, n_parent, binomial_table(), (const W*)red.d_keys, red.dim,
                                                        red.sb, gb.dev, d_ph, (const V*)in, (V*)out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_ph);
    if (e != cudaSuccess) throw Error(EDGPU_ERR_CUDA, std::string("vector reduction: ") + cudaGetErrorString(e));
}

}  // namespace

int64_t parent_dimension(const Space& parent) {
    return parent.d_keys ? parent.dim : (int64_t)host_binom(parent.lay.nbits, parent.lay.popcount);
}

void reduce_vector(const Space& red, const Space& parent, int prec, bool unreduce, const void* in, void* out,
                   cudaStream_t st) {
    if (!parent.d_keys && parent.lay.popcount < 0)
        throw Error(EDGPU_ERR_STATE, "a lazy parent must be one popcount sector of 1-bit sites");
    const bool pw32 = parent.d_keys && parent.w32;
#define EDGPU_RV(W)                                                                                         \
    if (prec == EDGPU_FP64) {                                                                              \
        if (pw32) reduce_vector_t<W, uint32_t, double2>(red, parent, unreduce, in, out, st);                \
        else reduce_vector_t<W, unsigned long long, double2>(red, parent, unreduce, in, out, st);           \
    } else {                                                                                                \
        if (pw32) reduce_vector_t<W, uint32_t, float2>(red, parent, unreduce, in, out, st);                 \
        else reduce_vector_t<W, unsigned long long, float2>(red, parent, unreduce, in, out, st);            \
    }
    if (red.w32) {
        EDGPU_RV(uint32_t)
    } else {
        EDGPU_RV(unsigned long long)
    }
#undef EDGPU_RV
}

}  // namespace edgpu
