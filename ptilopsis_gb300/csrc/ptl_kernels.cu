// CUDA kernels of the GB300 code generator.  Per-thread logic lives in ptl_stages.cuh and
// ptl_sort.cuh; this file holds the launch shapes, the cross-thread primitives (scans,
// the depth-order rounds, the lock-step register allocator of lane-0 functions) and
// their bounded waits.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <atomic>
#include <map>
#include <mutex>
#include <utility>

#include "ptl_kernels.cuh"
#include "ptl_ra.cuh"

namespace ptl {

// A kernel's largest dynamic shared memory is one attribute per function and device,
// shared by every host thread: batched pipelines on several threads (the compile server's
// lanes) launch the same kernels with different sizes.  So the attribute is only ever
// raised, under a lock, to the largest size requested so far; a launch that set it never
// finds it lowered by another thread before it runs.
cudaError_t allow_dynamic_smem(const void* kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> granted;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    size_t& g = granted[{dev, kernel}];
    if (bytes <= g) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
    if (e == cudaSuccess) g = bytes;
    return e;
}

}  // namespace ptl

namespace ptl {

namespace {

std::atomic<uint64_t> g_launches{0};

constexpr int kThreads = 256;

inline unsigned grid_for(uint64_t n, int threads = kThreads) {
    uint64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > 152ull * 64ull) g = 152ull * 64ull;  // grid-stride beyond 64 CTAs per SM
    return static_cast<unsigned>(g);
}

#define PTL_FOR(i, count)                                                                \
    for (uint64_t i##_ = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;   \
         i##_ < (count); i##_ += static_cast<uint64_t>(gridDim.x) * blockDim.x)          \
        if (const uint32_t i = static_cast<uint32_t>(i##_); true)

// ------------------------------------------------------------------ element-wise stages
__global__ void k_ingest(Prog P) {
    PTL_FOR(i, P.nb8) if (st_ingest(P, i)) P.flags[3] = 1u;
}
__global__ void k_pre_lists(Prog P) { PTL_FOR(i, P.nb8) st_pre_lists(P, i); }
__global__ void k_pre_float(Prog P) { PTL_FOR(i, P.nb8) st_pre_float(P, i); }
__global__ void k_pre_float_apply(Prog P) { PTL_FOR(i, P.nb8) st_pre_float_apply(P, i); }
__global__ void k_fix_own(Prog P) { PTL_FOR(i, P.nb8) st_fix_own(P, i); }
__global__ void k_fix_cond(Prog P) { PTL_FOR(i, P.nb8) st_fix_cond(P, i); }

// ------------------------------------------------------------------ decoupled look-back scan
// Exclusive scan (mod 2^32) of load(i) over [0, count), single pass: tiles take tickets
// in order, publish their aggregate, look back over predecessors until one has published
// its inclusive prefix, then publish their own.  A look-back that waits too long gives
// up and records ST_DEVICE_TIMEOUT instead of spinning forever.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;
constexpr uint32_t kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x) {
    const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
        if (lane >= static_cast<uint32_t>(d)) x += y;
    }
    return x;
}

// The look-back of a tile past its program's first tile, by one whole warp: lane k reads
// the status of tile j-k, so each round trip to L2 examines 32 predecessors.  Partial
// aggregates (flag 1) are summed up to the nearest tile that has published its inclusive
// prefix (flag 2); a window with a tile that has published nothing yet (flag 0) in front
// of that one is read again.  Every lane gets the exclusive prefix.  Bounded like every
// device wait: after kSpinLimit re-reads it records ST_DEVICE_TIMEOUT and returns what it
// has, so the tile still publishes and no successor waits forever.
__device__ uint32_t warp_lookback(unsigned long long* status, uint32_t tile, uint32_t first, ErrorWord* err) {
    constexpr unsigned full = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t prefix = 0, spins = 0;
    int64_t j = static_cast<int64_t>(tile) - 1;
    for (;;) {
        const int64_t idx = j - static_cast<int64_t>(lane);
        // tiles before the first one never matter: the first tile publishes its inclusive
        // prefix directly and is met before them
        const unsigned long long st = idx >= static_cast<int64_t>(first)
                                          ? *reinterpret_cast<volatile unsigned long long*>(&status[idx])
                                          : (2ull << 32);
        const uint32_t flag = static_cast<uint32_t>(st >> 32);
        const unsigned incl = __ballot_sync(full, flag == 2u);
        const unsigned none = __ballot_sync(full, flag == 0u);
        const uint32_t k = incl ? static_cast<uint32_t>(__ffs(static_cast<int>(incl)) - 1) : 31u;
        const unsigned upto = k == 31u ? full : ((1u << (k + 1u)) - 1u);
        if (none & upto) {
            if (++spins > kSpinLimit) {
                if (lane == 0) record_error(err, ST_DEVICE_TIMEOUT, W_SCAN, tile);
                return prefix;
            }
            continue;
        }
        uint32_t v = lane <= k ? static_cast<uint32_t>(st) : 0u;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(full, v, d);
        prefix += v;
        if (incl) return prefix;
        j -= 32;
    }
}

template <class Load, class Store>
__global__ void __launch_bounds__(kScanThreads) k_scan(Load load, Store store, uint32_t count, ScanScratch sc, ErrorWord* err) {
    constexpr int kWarps = kScanThreads / 32;
    __shared__ uint32_t s_tile, s_prefix;
    __shared__ uint32_t s_warp[kWarps];
    if (threadIdx.x == 0) s_tile = atomicAdd(sc.counter, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint64_t wbase = static_cast<uint64_t>(tile) * kScanTile + static_cast<uint64_t>(warp) * 32u * kScanItems;
    uint32_t v[kScanItems];
    uint32_t carry = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const uint64_t idx = wbase + static_cast<uint64_t>(k) * 32u + lane;
        const uint32_t x = idx < count ? load(static_cast<uint32_t>(idx)) : 0u;
        const uint32_t incl = warp_incl_scan(x);
        v[k] = carry + incl - x;
        carry += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    if (lane == 0) s_warp[warp] = carry;
    __syncthreads();
    if (warp == 0) {
        const uint32_t t = lane < kWarps ? s_warp[lane] : 0u;
        const uint32_t incl = warp_incl_scan(t);
        if (lane < kWarps) s_warp[lane] = incl - t;
        const uint32_t aggregate = __shfl_sync(0xFFFFFFFFu, incl, kWarps - 1);
        uint32_t prefix = 0;
        if (tile == 0) {
            if (lane == 0) atomicExch(&sc.status[0], (2ull << 32) | aggregate);
        } else {
            if (lane == 0) atomicExch(&sc.status[tile], (1ull << 32) | aggregate);
            prefix = warp_lookback(sc.status, tile, 0u, err);
            if (lane == 0) atomicExch(&sc.status[tile], (2ull << 32) | (prefix + aggregate));
        }
        if (lane == 0) s_prefix = prefix;
    }
    __syncthreads();
    const uint32_t base = s_prefix + s_warp[warp];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const uint64_t idx = wbase + static_cast<uint64_t>(k) * 32u + lane;
        if (idx < count) store(static_cast<uint32_t>(idx), base + v[k]);
    }
}

static_assert(kScanTile == kScanTileElems, "scan tile size shared with the host");

template <class Load, class Store>
void run_scan(Load load, Store store, uint32_t count, const ScanScratch& sc, ErrorWord* err, cudaStream_t s) {
    const uint32_t tiles = (count + kScanTile - 1) / kScanTile;
    if (tiles == 0) return;
    if (tiles > sc.tile_cap) {  // the caller sizes the scratch; never write past it
        ErrorWord e{ST_UNSUPPORTED, W_SCAN, tiles, 0};
        cudaMemcpyAsync(err, &e, sizeof(e), cudaMemcpyHostToDevice, s);
        cudaStreamSynchronize(s);
        return;
    }
    cudaMemsetAsync(sc.status, 0, sizeof(unsigned long long) * tiles, s);
    cudaMemsetAsync(sc.counter, 0, sizeof(uint32_t), s);
    g_launches++;
    k_scan<<<tiles, kScanThreads, 0, s>>>(load, store, count, sc, err);
}

struct CountLoad {
    Prog P;
    __device__ uint32_t operator()(uint32_t i) const {
        const uint32_t v = st_count(P, i);
        P.sizes[i] = v;
        return v;
    }
};
struct StoreTo {
    uint32_t* out;
    __device__ void operator()(uint32_t i, uint32_t v) const { out[i] = v; }
};
struct DeclLoad {
    Prog P;
    __device__ uint32_t operator()(uint32_t i) const { return P.nt[i] == RV_FUNC_DECL ? 1u : 0u; }
};
struct DeclStore {
    Prog P;
    uint32_t* meta;
    uint32_t count;
    __device__ void operator()(uint32_t i, uint32_t v) const {
        const bool is_decl = P.nt[i] == RV_FUNC_DECL;
        if (is_decl) P.decl[v] = i;
        if (i == count - 1) meta[0] = v + (is_decl ? 1u : 0u);
    }
};
struct RaCountLoad {
    Prog P;
    __device__ uint32_t operator()(uint32_t i) const { return st_ra_count(P, i); }
};
struct FjSizeLoad {
    Prog P;
    __device__ uint32_t operator()(uint32_t i) const {
        const uint32_t v = i < P.W2 ? st_fj_size(P, i) : 0u;
        P.fsz[i] = v;
        return v;
    }
};

// ------------------------------------------------------------------ function table
__global__ void k_functab(Prog P, const uint32_t* meta) {
    const uint32_t F = meta[0];
    const uint32_t fb8 = (F + 7u) & ~7u;
    PTL_FOR(f, fb8) st_functab(P, f);
}
__global__ void k_functab_end(Prog P, uint32_t* meta) {
    const uint32_t F = meta[0];
    const uint32_t fb8 = (F + 7u) & ~7u;
    PTL_FOR(f, fb8) {
        st_functab_end(P, f);
        if (f < F) atomicMax(&meta[2], P.fn_size[f]);  // longest function, in steps
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) meta[1] = P.loc[P.n - 1];  // word count
}

// ------------------------------------------------------------------ depth order
__global__ void k_sort_init(Prog P, SortScratch ss) {
    PTL_FOR(i, P.n) ss.a[i] = (static_cast<unsigned long long>(u32(P.dep[i])) << 32) | i;
}

// The round kernels read this round's segment and tile counts on the device, so that
// rounds run back to back without the host.  A capacity overflow (impossible by the
// bounds the host sizes with, but checked) raises counters[5] and idles later kernels.
__device__ __forceinline__ bool sort_overflow(const SortScratch& ss) {
    return *reinterpret_cast<const volatile uint32_t*>(&ss.counters[5]) != 0;
}
__device__ __forceinline__ uint32_t sort_nseg(const SortScratch& ss) { return min(ss.counters[4], ss.seg_cap); }
__device__ __forceinline__ uint32_t sort_ntiles(const SortScratch& ss) { return min(ss.counters[0], ss.tile_cap); }

// Round start: the segments emitted by the previous round become this round's.
__global__ void k_sort_round(SortScratch ss) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ss.counters[4] = ss.counters[1];
        ss.counters[1] = 0;
        ss.counters[0] = 0;
    }
}

__global__ void k_sort_tiles(SortScratch ss, const SortSeg* cur, SortSeg* curw) {
    if (sort_overflow(ss)) return;
    const uint32_t nseg = sort_nseg(ss);
    PTL_FOR(s, nseg) {
        SortSeg g = cur[s];
        median_to_first(ss.a, g.first, g.last);
        g.pivot = skey(ss.a[g.first]);
        g.kmin = g.kmax = g.pivot;  // k_sort_count folds in the other keys
        const uint32_t m1 = g.last - g.first - 1;
        g.tcount = (m1 + kSortTile - 1) / kSortTile;
        g.tbase = atomicAdd(&ss.counters[0], g.tcount);
        curw[s] = g;
        if (g.tbase + g.tcount > ss.tile_cap) {
            ss.counters[5] = 1;
            continue;
        }
        for (uint32_t k = 0; k < g.tcount; ++k) ss.tile_seg[g.tbase + k] = s;
    }
}
__device__ __forceinline__ uint32_t block_reduce_add(uint32_t v, uint32_t* sm) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, d);
    if (lane == 0) sm[warp] = v;
    __syncthreads();
    uint32_t t = 0;
    if (threadIdx.x == 0) {
        for (uint32_t w = 0; w < blockDim.x / 32; ++w) t += sm[w];
    }
    __syncthreads();
    return t;  // valid in thread 0
}

constexpr uint32_t kSortItems = kSortTile / kThreads;  // 8 per thread

// Exclusive prefix sums of a and b over the block's threads (kThreads), by warp shuffles
// and one pass over the warp totals; *tot receives the two block totals.  sm holds
// 2 * kThreads / 32 + 2 words; the caller synchronises before reusing it.
__device__ __forceinline__ void block_excl_scan2(uint32_t a, uint32_t b, uint32_t* sm, uint32_t* ea, uint32_t* eb,
                                                 uint32_t* tot) {
    constexpr uint32_t W = kThreads / 32;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t ia = warp_incl_scan(a), ib = warp_incl_scan(b);
    if (lane == 31) { sm[warp] = ia; sm[W + warp] = ib; }
    __syncthreads();
    if (warp == 0) {
        const uint32_t va = lane < W ? sm[lane] : 0u, vb = lane < W ? sm[W + lane] : 0u;
        const uint32_t sa = warp_incl_scan(va), sb = warp_incl_scan(vb);
        if (lane < W) { sm[lane] = sa - va; sm[W + lane] = sb - vb; }
        if (lane == W - 1) { sm[2 * W] = sa; sm[2 * W + 1] = sb; }
    }
    __syncthreads();
    *ea = sm[warp] + ia - a;
    *eb = sm[W + warp] + ib - b;
    tot[0] = sm[2 * W];
    tot[1] = sm[2 * W + 1];
}

// Stop counts per tile, and the least and greatest key of each segment (atomics on the
// segment record; a part of the next split is known to hold one key when its bound on
// the pivot's side meets the pivot).  The tile's stop bits go to ss.stops (tile-local
// key j at word j / 32, bit j % 32), so the position pass reads 2 bits per key, not 8
// bytes.
constexpr uint32_t kStopWords = kSortTile / 32;  // per kind and tile
__global__ void __launch_bounds__(kThreads) k_sort_count(SortScratch ss, SortSeg* cur) {
    __shared__ uint32_t sm[kThreads / 32];
    __shared__ int32_t smn[kThreads / 32], smx[kThreads / 32];
    if (sort_overflow(ss)) return;
    const uint32_t ntiles = sort_ntiles(ss);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const uint32_t si = ss.tile_seg[t];
        const SortSeg g = cur[si];
        const uint32_t lo = g.first + 1 + (t - g.tbase) * kSortTile;
        const uint32_t hi = min(g.last, lo + kSortTile);
        uint32_t cl = 0, cr = 0;
        int32_t mn = g.pivot, mx = g.pivot;
        int32_t key[kSortItems];  // the tile's keys of this thread, loaded together
#pragma unroll
        for (uint32_t u = 0; u < kSortItems; ++u) {
            const uint32_t p = lo + threadIdx.x + u * kThreads;
            key[u] = p < hi ? skey(ss.a[p]) : g.pivot;
        }
        uint32_t* bits = ss.stops + static_cast<size_t>(t) * 2u * kStopWords;
#pragma unroll
        for (uint32_t u = 0; u < kSortItems; ++u) {  // tile-local j = warp * 32 + lane + u * kThreads
            const bool in = lo + threadIdx.x + u * kThreads < hi;
            const unsigned bl = __ballot_sync(0xFFFFFFFFu, in && is_lstop(key[u], g.pivot));
            const unsigned br = __ballot_sync(0xFFFFFFFFu, in && is_rstop(key[u], g.pivot));
            if (lane == 0) {
                bits[warp + u * (kThreads / 32)] = bl;
                bits[kStopWords + warp + u * (kThreads / 32)] = br;
            }
        }
#pragma unroll
        for (uint32_t u = 0; u < kSortItems; ++u) {
            if (lo + threadIdx.x + u * kThreads >= hi) continue;
            cl += is_lstop(key[u], g.pivot);
            cr += is_rstop(key[u], g.pivot);
            mn = min(mn, key[u]);
            mx = max(mx, key[u]);
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            mn = min(mn, __shfl_down_sync(0xFFFFFFFFu, mn, d));
            mx = max(mx, __shfl_down_sync(0xFFFFFFFFu, mx, d));
        }
        if (lane == 0) { smn[warp] = mn; smx[warp] = mx; }
        const uint32_t tl = block_reduce_add(cl, sm);  // its barriers publish smn / smx
        const uint32_t tr = block_reduce_add(cr, sm);
        if (threadIdx.x == 0) {
            ss.tile_l[t] = tl;
            ss.tile_r[t] = tr;
            for (uint32_t w = 1; w < kThreads / 32; ++w) { mn = min(mn, smn[w]); mx = max(mx, smx[w]); }
            if (mn < g.pivot) atomicMin(&cur[si].kmin, mn);
            if (mx > g.pivot) atomicMax(&cur[si].kmax, mx);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kThreads) k_sort_segscan(SortScratch ss, SortSeg* cur) {
    __shared__ uint32_t sm[2 * kThreads / 32 + 2];
    if (sort_overflow(ss)) return;
    const uint32_t nseg = sort_nseg(ss);
    for (uint32_t si = blockIdx.x; si < nseg; si += gridDim.x) {
        SortSeg& g = cur[si];
        uint32_t carry_l = 0, carry_r = 0;
        for (uint32_t c = 0; c < g.tcount; c += kThreads) {
            const uint32_t k = c + threadIdx.x;
            const uint32_t vl = k < g.tcount ? ss.tile_l[g.tbase + k] : 0u;
            const uint32_t vr = k < g.tcount ? ss.tile_r[g.tbase + k] : 0u;
            uint32_t el, er, tot[2];
            block_excl_scan2(vl, vr, sm, &el, &er, tot);
            if (k < g.tcount) {
                ss.tile_l[g.tbase + k] = carry_l + el;
                ss.tile_r[g.tbase + k] = carry_r + er;
            }
            carry_l += tot[0];
            carry_r += tot[1];
            __syncthreads();
        }
        // A bound on the pair count K: at any position x, K <= max(L-stops before x,
        // R-stops from x on) -- were K larger, the K-th L-stop would sit at or after x and
        // its pair, further right, would leave K R-stops from x on.  The minimum over the
        // tile starts (and the end) keeps it in g.K until the cut; stops ranked past it
        // are never swapped, so their positions need not be written.
        uint32_t kb = carry_l;
        for (uint32_t k = threadIdx.x; k < g.tcount; k += kThreads)
            kb = min(kb, max(ss.tile_l[g.tbase + k], carry_r - ss.tile_r[g.tbase + k]));
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) kb = min(kb, __shfl_down_sync(0xFFFFFFFFu, kb, d));
        if ((threadIdx.x & 31u) == 0) sm[threadIdx.x >> 5] = kb;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (uint32_t w = 1; w < kThreads / 32; ++w) kb = min(kb, sm[w]);
            g.nL = carry_l;
            g.nR = carry_r;
            g.K = kb;
        }
        __syncthreads();
    }
}

// Stop positions by rank: A[rank] for L-stops, B[rank from the right] for R-stops, for
// ranks up to the segment's bound on K (g.K, from k_sort_segscan) -- the cut reads
// A[0..K] and B[0..K-1].  A tile with no stop in that range is not read.
__global__ void __launch_bounds__(kThreads) k_sort_pos(SortScratch ss, const SortSeg* cur) {
    __shared__ uint32_t sm[2 * kThreads / 32 + 2];
    if (sort_overflow(ss)) return;
    const uint32_t ntiles = sort_ntiles(ss);
    for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const SortSeg g = cur[ss.tile_seg[t]];
        const uint32_t kb1 = g.K + 1u;  // ranks below this are written
        const uint32_t rnext = t + 1u < g.tbase + g.tcount ? ss.tile_r[t + 1u] : g.nR;
        if (ss.tile_l[t] >= kb1 && g.nR - rnext >= kb1) continue;  // block-uniform
        const uint32_t lo = g.first + 1 + (t - g.tbase) * kSortTile;
        const uint32_t hi = min(g.last, lo + kSortTile);
        const uint32_t p0 = lo + threadIdx.x * kSortItems;
        // this thread's kSortItems keys: tile-local j = threadIdx.x * 8 .. + 7, one byte of
        // a stop word (bits past the tile's end are clear)
        static_assert(kSortItems == 8, "a thread's stop bits are one byte of a word");
        const uint32_t* bits = ss.stops + static_cast<size_t>(t) * 2u * kStopWords;
        const uint32_t sh = (threadIdx.x & 3u) * 8u;
        const uint32_t fl = (bits[threadIdx.x >> 2] >> sh) & 0xFFu;
        const uint32_t fr = (bits[kStopWords + (threadIdx.x >> 2)] >> sh) & 0xFFu;
        const uint32_t cl = __popc(fl), cr = __popc(fr);
        (void)hi;
        uint32_t el, er, tot[2];
        block_excl_scan2(cl, cr, sm, &el, &er, tot);
        uint32_t rl = ss.tile_l[t] + el;
        uint32_t rr = ss.tile_r[t] + er;
#pragma unroll
        for (uint32_t k = 0; k < kSortItems; ++k) {
            const uint32_t p = p0 + k;
            if ((fl >> k) & 1u) {
                if (rl < kb1) ss.apos[g.first + rl] = p;
                ++rl;
            }
            if ((fr >> k) & 1u) {
                const uint32_t rk = g.nR - 1u - rr++;
                if (rk < kb1) ss.bpos[g.first + rk] = p;
            }
        }
        __syncthreads();
    }
}

// Routes a part of a split: eq says its keys are all equal.
__device__ void sort_emit(SortScratch ss, SortSeg* next, uint32_t first, uint32_t last, uint32_t dl, bool eq) {
    if (eq && last - first <= kSortThreshold) return;  // a stable sort of equal keys moves nothing
    if (eq && dl >= equal_levels(last - first)) {      // final order in closed form (k_sort_equal)
        const uint32_t k = atomicAdd(&ss.counters[7], 1u);
        if (k < ss.seg_cap) { ss.equal[2 * k] = first; ss.equal[2 * k + 1] = last; }
        else ss.counters[5] = 1;
        return;
    }
    if (last - first <= kSortThreshold) {
        if (last - first > 1) {
            const uint32_t k = atomicAdd(&ss.counters[2], 1u);
            if (k < ss.leaf_cap) { ss.leaf[2 * k] = first; ss.leaf[2 * k + 1] = last; }
            else ss.counters[5] = 1;
        }
        return;
    }
    if (dl > 0 && last - first <= kSortBlock) {  // finishes in one block after the rounds
        const uint32_t k = atomicAdd(&ss.counters[6], 1u);
        if (k < ss.seg_cap) { ss.local[3 * k] = first; ss.local[3 * k + 1] = last; ss.local[3 * k + 2] = dl; }
        else ss.counters[5] = 1;
        return;
    }
    if (dl == 0) {
        const uint32_t k = atomicAdd(&ss.counters[3], 1u);
        if (k < ss.leaf_cap) { ss.heap[2 * k] = first; ss.heap[2 * k + 1] = last; }
        else ss.counters[5] = 1;
        return;
    }
    const uint32_t k = atomicAdd(&ss.counters[1], 1u);
    if (k < ss.seg_cap) {
        SortSeg c{};
        c.first = first;
        c.last = last;
        c.dl = dl;
        next[k] = c;
    } else {
        ss.counters[5] = 1;
    }
}

__global__ void k_sort_cut(SortScratch ss, SortSeg* cur, SortSeg* next, ErrorWord* err) {
    if (sort_overflow(ss)) return;
    const uint32_t nseg = sort_nseg(ss);
    PTL_FOR(s, nseg) {
        SortSeg& g = cur[s];
        if (g.nL == 0 || g.nR == 0) {  // the median move guarantees both kinds of stop
            record_error(err, ST_UNSUPPORTED, W_SORT, g.first);
            g.K = 0;
            continue;
        }
        // positions are written for ranks up to the bound g.K only; K <= g.K
        g.K = partition_k(ss.apos + g.first, ss.bpos + g.first, min(g.nL, g.K), g.nR);
        g.cut = partition_cut(ss.apos + g.first, ss.bpos + g.first, g.nL, g.K);
        if (g.cut <= g.first || g.cut >= g.last) {
            record_error(err, ST_UNSUPPORTED, W_SORT, g.first);
            g.K = 0;
            continue;
        }
        sort_emit(ss, next, g.first, g.cut, g.dl - 1, g.kmin == g.pivot);
        sort_emit(ss, next, g.cut, g.last, g.dl - 1, g.kmax == g.pivot);
    }
}

// The K swaps of a segment touch disjoint positions (every A[k] lies left of every B[k'],
// k, k' < K), so a thread loads all of its tile's pairs and their keys before it stores
// any: the loads of a tile are in flight together instead of one dependent pair at a time.
__global__ void __launch_bounds__(kThreads) k_sort_swap(SortScratch ss, const SortSeg* cur) {
    if (sort_overflow(ss)) return;
    const uint32_t ntiles = sort_ntiles(ss);
    for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const SortSeg g = cur[ss.tile_seg[t]];
        const uint32_t k0 = (t - g.tbase) * kSortTile;
        const uint32_t k1 = min(g.K, k0 + kSortTile);
        if (k0 >= k1) continue;
        uint32_t pa[kSortItems], pb[kSortItems];
        unsigned long long va[kSortItems], vb[kSortItems];
#pragma unroll
        for (uint32_t u = 0; u < kSortItems; ++u) {
            const uint32_t k = k0 + threadIdx.x + u * kThreads;
            if (k < k1) {
                pa[u] = ss.apos[g.first + k];
                pb[u] = ss.bpos[g.first + k];
            }
        }
#pragma unroll
        for (uint32_t u = 0; u < kSortItems; ++u) {
            if (k0 + threadIdx.x + u * kThreads < k1) {
                va[u] = ss.a[pa[u]];
                vb[u] = ss.a[pb[u]];
            }
        }
#pragma unroll
        for (uint32_t u = 0; u < kSortItems; ++u) {
            if (k0 + threadIdx.x + u * kThreads < k1) {
                ss.a[pa[u]] = vb[u];
                ss.a[pb[u]] = va[u];
            }
        }
    }
}

__global__ void k_sort_leaves(SortScratch ss, uint32_t count) {
    PTL_FOR(k, count) leaf_sort(ss.a, ss.leaf[2 * k], ss.leaf[2 * k + 1]);
}
// ---- ranges of at most kSortBlock keys: one block each, in shared memory
// The partition steps are the closed form of the rounds above.  Parts longer than
// kSortLocal are split by the whole block (stop positions by ballot and a scan over
// (sweep, warp) counts, K by binary search, the K disjoint swaps in parallel); shorter
// parts are finished by one warp each.  Every part's start is marked in a bitmask, so
// the final ranges tile the buffer: a range of at most 16 keys (a leaf) is written back
// by stable rank, a range of equal keys in closed form, a heap-sorted range as it is.
// The smaller part of a split is taken first, so the pending stacks stay within
// log2(kSortBlock) entries.
constexpr int kSortBlockThreads = 512;
constexpr int kSortBlockWarps = kSortBlockThreads / 32;
constexpr uint32_t kSortBlockSweeps = (kSortBlock + kSortBlockThreads - 1) / kSortBlockThreads;
constexpr uint32_t kSortBlockLists = kSortBlock / (kSortThreshold + 1) + 2;
constexpr uint32_t kSortStack = 16;
static_assert(kSortBlock <= 65535 && kSortBlockSweeps <= 32, "16-bit positions, 32-bit sweep masks");

struct BlockSortSmem {
    unsigned long long buf[kSortBlock];
    uint16_t A[kSortBlock], R[kSortBlock];  // stop positions of the part being split (at its offset)
    uint32_t starts[kSortBlock / 32 + 1];   // bit j: a part starts at j (bit m: the end)
    uint16_t sm_f[kSortBlockLists], sm_l[kSortBlockLists], sm_d[kSortBlockLists];     // warp parts
    uint16_t fin_f[kSortBlockLists], fin_l[kSortBlockLists], fin_h[kSortBlockLists];  // equal (0) / heap (1)
    uint16_t st_f[kSortBlockWarps][kSortStack], st_l[kSortBlockWarps][kSortStack], st_d[kSortBlockWarps][kSortStack];
    uint32_t bst_f[kSortStack], bst_l[kSortStack], bst_d[kSortStack];
    uint32_t cntL[kSortBlockSweeps * kSortBlockWarps], cntR[kSortBlockSweeps * kSortBlockWarps];
    int32_t wmin[kSortBlockWarps], wmax[kSortBlockWarps];
    int32_t kmin, kmax;
    uint32_t nL, nR, K, cut;
    uint32_t n_sm, n_fin, next_sm, n_bst, bad;
    uint32_t cur_f, cur_l, cur_d, have;
};

// Marks the start of part [f, l) (depth budget d, eq: its keys are all equal) and lists
// it if it is final; returns whether it must be split further.
__device__ bool bsort_route(BlockSortSmem& w, uint32_t f, uint32_t l, uint32_t d, bool eq) {
    atomicOr(&w.starts[f >> 5], 1u << (f & 31u));
    const uint32_t m = l - f;
    if (m <= kSortThreshold) return false;  // a leaf
    const bool closed = eq && d >= equal_levels(m);
    if (closed || d == 0) {
        const uint32_t k = atomicAdd(&w.n_fin, 1u);
        if (k < kSortBlockLists) {
            w.fin_f[k] = static_cast<uint16_t>(f);
            w.fin_l[k] = static_cast<uint16_t>(l);
            w.fin_h[k] = closed ? 0 : 1;
        } else {
            w.bad = 1;
        }
        return false;
    }
    return true;
}

__device__ void bsort_push_small(BlockSortSmem& w, uint32_t f, uint32_t l, uint32_t d) {
    const uint32_t k = atomicAdd(&w.n_sm, 1u);
    if (k < kSortBlockLists) {
        w.sm_f[k] = static_cast<uint16_t>(f);
        w.sm_l[k] = static_cast<uint16_t>(l);
        w.sm_d[k] = static_cast<uint16_t>(d);
    } else {
        w.bad = 1;
    }
}

__device__ __forceinline__ int32_t warp_min_i32(int32_t v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = min(v, __shfl_xor_sync(0xFFFFFFFFu, v, d));
    return v;
}
__device__ __forceinline__ int32_t warp_max_i32(int32_t v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = max(v, __shfl_xor_sync(0xFFFFFFFFu, v, d));
    return v;
}

// One block-wide split of [f, l); sets w.K / w.cut / w.kmin / w.kmax (w.bad on a broken
// invariant).  Every thread calls it; it ends with a barrier.
// The caller has moved the median to f (thread 0, before the barrier that publishes the
// part).
__device__ void bsort_split_block(BlockSortSmem& w, uint32_t f, uint32_t l) {
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const unsigned full = 0xFFFFFFFFu, lt = (1u << lane) - 1u;
    constexpr uint32_t T = kSortBlockThreads;
    const int32_t pivot = skey(w.buf[f]);
    const uint32_t sweeps = (l - f - 1u + T - 1u) / T;
    uint32_t fl = 0, fr = 0;
    int32_t mn = pivot, mx = pivot;
    for (uint32_t k = 0; k < sweeps; ++k) {
        const uint32_t p = f + 1u + k * T + tid;
        const bool in = p < l;
        const int32_t key = in ? skey(w.buf[p]) : pivot;
        const bool isL = in && is_lstop(key, pivot), isR = in && is_rstop(key, pivot);
        mn = min(mn, key);
        mx = max(mx, key);
        fl |= static_cast<uint32_t>(isL) << k;
        fr |= static_cast<uint32_t>(isR) << k;
        const unsigned bL = __ballot_sync(full, isL), bR = __ballot_sync(full, isR);
        if (lane == 0) {
            w.cntL[k * kSortBlockWarps + warp] = __popc(bL);
            w.cntR[k * kSortBlockWarps + warp] = __popc(bR);
        }
    }
    mn = warp_min_i32(mn);
    mx = warp_max_i32(mx);
    if (lane == 0) { w.wmin[warp] = mn; w.wmax[warp] = mx; }
    __syncthreads();
    if (warp == 0) {
        // exclusive scan of the (sweep, warp) counts in that order, 8 entries per lane
        constexpr uint32_t E = kSortBlockSweeps * kSortBlockWarps, per = E / 32;
        const uint32_t used = sweeps * kSortBlockWarps;
        uint32_t vl[per], vr[per], sl = 0, sr = 0;
#pragma unroll
        for (uint32_t q = 0; q < per; ++q) {
            const uint32_t e = lane * per + q;
            vl[q] = e < used ? w.cntL[e] : 0u;
            vr[q] = e < used ? w.cntR[e] : 0u;
            sl += vl[q];
            sr += vr[q];
        }
        uint32_t il = sl, ir = sr;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t al = __shfl_up_sync(full, il, d), ar = __shfl_up_sync(full, ir, d);
            if (lane >= static_cast<uint32_t>(d)) { il += al; ir += ar; }
        }
        uint32_t ol = il - sl, orr = ir - sr;
#pragma unroll
        for (uint32_t q = 0; q < per; ++q) {
            const uint32_t e = lane * per + q;
            if (e < used) { w.cntL[e] = ol; w.cntR[e] = orr; }
            ol += vl[q];
            orr += vr[q];
        }
        int32_t a = lane < kSortBlockWarps ? w.wmin[lane] : pivot, b = lane < kSortBlockWarps ? w.wmax[lane] : pivot;
        a = warp_min_i32(a);
        b = warp_max_i32(b);
        if (lane == 31) { w.nL = il; w.nR = ir; }
        if (lane == 0) { w.kmin = a; w.kmax = b; }
    }
    __syncthreads();
    for (uint32_t k = 0; k < sweeps; ++k) {
        const bool isL = (fl >> k) & 1u, isR = (fr >> k) & 1u;
        const unsigned bL = __ballot_sync(full, isL), bR = __ballot_sync(full, isR);
        const uint32_t p = f + 1u + k * T + tid;
        if (isL) w.A[f + w.cntL[k * kSortBlockWarps + warp] + __popc(bL & lt)] = static_cast<uint16_t>(p);
        if (isR) w.R[f + w.cntR[k * kSortBlockWarps + warp] + __popc(bR & lt)] = static_cast<uint16_t>(p);
    }
    __syncthreads();
    if (warp == 0) {
        const uint32_t nL = w.nL, nR = w.nR;
        uint32_t K = 0, cut = 0;
        if (nL == 0 || nR == 0) {  // the median move guarantees both kinds of stop
            if (lane == 0) w.bad = 1;
        } else {
            // K: A[k] < B[k] holds on a prefix of k, and K is in [lo, hi].  32 probes per
            // round narrow the range to one of 33 slices; the last round tests each index.
            uint32_t lo = 0, hi = nL < nR ? nL : nR;
            while (hi - lo > 32u) {
                const uint64_t span = hi - lo;
                const uint32_t q = lo + static_cast<uint32_t>(span * (lane + 1u) / 33u);
                const uint32_t c = __popc(__ballot_sync(full, w.A[f + q] < w.R[f + nR - 1u - q]));
                const uint32_t nlo = c == 0 ? lo : lo + static_cast<uint32_t>(span * c / 33u) + 1u;
                const uint32_t nhi = c == 32 ? hi : lo + static_cast<uint32_t>(span * (c + 1u) / 33u);
                lo = nlo;
                hi = nhi;
            }
            const uint32_t q = lo + lane;
            K = lo + __popc(__ballot_sync(full, q < hi && w.A[f + q] < w.R[f + nR - 1u - q]));
            if (K == 0) {
                cut = w.A[f];
            } else {
                const uint32_t bk = w.R[f + nR - K];  // B[K-1]
                cut = (K < nL && w.A[f + K] < bk) ? w.A[f + K] : bk;
            }
            if (cut <= f || cut >= l) {
                if (lane == 0) w.bad = 1;
                K = 0;
            }
        }
        if (lane == 0) {
            w.K = K;
            w.cut = cut;
        }
    }
    __syncthreads();
    const uint32_t K = w.K, nR = w.nR;
    for (uint32_t k = tid; k < K; k += T) sswap(w.buf, w.A[f + k], w.R[f + nR - 1u - k]);
    __syncthreads();
}

// One warp finishes part [f, l) (more than 16 keys, depth budget d > 0) and every part
// of it that must be split further.
__device__ void bsort_warp(BlockSortSmem& w, uint32_t f, uint32_t l, uint32_t d) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned full = 0xFFFFFFFFu, lt = (1u << lane) - 1u;
    uint32_t sp = 0;
    for (;;) {
        if (lane == 0) median_to_first(w.buf, f, l);
        __syncwarp();
        const int32_t pivot = skey(w.buf[f]);
        uint32_t nL = 0, nR = 0;
        int32_t mn = pivot, mx = pivot;
        for (uint32_t base = f + 1; base < l; base += 32) {
            const uint32_t p = base + lane;
            const bool in = p < l;
            const int32_t k = in ? skey(w.buf[p]) : pivot;
            const bool isL = in && is_lstop(k, pivot), isR = in && is_rstop(k, pivot);
            mn = min(mn, k);
            mx = max(mx, k);
            const unsigned bL = __ballot_sync(full, isL), bR = __ballot_sync(full, isR);
            if (isL) w.A[f + nL + __popc(bL & lt)] = static_cast<uint16_t>(p);
            if (isR) w.R[f + nR + __popc(bR & lt)] = static_cast<uint16_t>(p);  // B[k] = R[nR - 1 - k]
            nL += __popc(bL);
            nR += __popc(bR);
        }
        mn = warp_min_i32(mn);
        mx = warp_max_i32(mx);
        __syncwarp();
        if (nL == 0 || nR == 0) {  // the median move guarantees both kinds of stop
            if (lane == 0) w.bad = 1;
            return;
        }
        const uint32_t mnc = nL < nR ? nL : nR;
        uint32_t K = mnc;
        for (uint32_t c = 0; c < mnc; c += 32) {
            const uint32_t k = c + lane;
            const unsigned b = __ballot_sync(full, k < mnc && !(w.A[f + k] < w.R[f + nR - 1u - k]));
            if (b) {
                K = c + static_cast<uint32_t>(__ffs(b) - 1);
                break;
            }
        }
        uint32_t cut;
        if (K == 0) {
            cut = w.A[f];
        } else {
            const uint32_t bk = w.R[f + nR - K];
            cut = (K < nL && w.A[f + K] < bk) ? w.A[f + K] : bk;
        }
        if (cut <= f || cut >= l) {
            if (lane == 0) w.bad = 1;
            return;
        }
        for (uint32_t k = lane; k < K; k += 32) sswap(w.buf, w.A[f + k], w.R[f + nR - 1u - k]);
        __syncwarp();
        uint32_t go = 0;
        if (lane == 0) {
            go = (bsort_route(w, f, cut, d - 1, mn == pivot) ? 1u : 0u) |
                 (bsort_route(w, cut, l, d - 1, mx == pivot) ? 2u : 0u);
        }
        go = __shfl_sync(full, go, 0);
        --d;
        if (go == 3u) {  // take the smaller part, keep the larger
            const bool left_small = cut - f <= l - cut;
            if (lane == 0) {
                if (sp < kSortStack) {
                    w.st_f[warp][sp] = static_cast<uint16_t>(left_small ? cut : f);
                    w.st_l[warp][sp] = static_cast<uint16_t>(left_small ? l : cut);
                    w.st_d[warp][sp] = static_cast<uint16_t>(d);
                } else {
                    w.bad = 1;
                }
            }
            ++sp;
            if (sp > kSortStack) return;
            if (left_small) l = cut; else f = cut;
        } else if (go == 1u) {
            l = cut;
        } else if (go == 2u) {
            f = cut;
        } else {
            if (sp == 0) return;
            --sp;
            __syncwarp();
            f = w.st_f[warp][sp];
            l = w.st_l[warp][sp];
            d = w.st_d[warp][sp];
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(kSortBlockThreads) k_sort_block(SortScratch ss, uint32_t count, ErrorWord* err) {
    extern __shared__ __align__(16) unsigned char bsm[];
    BlockSortSmem& w = *reinterpret_cast<BlockSortSmem*>(bsm);
    const uint32_t tid = threadIdx.x, lane = tid & 31u;
    constexpr uint32_t T = kSortBlockThreads;
    for (uint32_t r = blockIdx.x; r < count; r += gridDim.x) {
        const uint32_t first = ss.local[3 * r], last = ss.local[3 * r + 1], dl = ss.local[3 * r + 2];
        const uint32_t m = last - first;
        if (m > kSortBlock || m < 2) {  // emitted only up to kSortBlock (block-uniform)
            if (tid == 0) record_error(err, ST_UNSUPPORTED, W_SORT, first);
            continue;
        }
        for (uint32_t j = tid; j < m; j += T) w.buf[j] = ss.a[first + j];
        for (uint32_t j = tid; j < kSortBlock / 32 + 1; j += T) w.starts[j] = 0;
        if (tid == 0) {
            w.n_sm = w.n_fin = w.next_sm = w.n_bst = w.bad = 0;
            w.have = 0;
        }
        __syncthreads();
        if (tid == 0) {
            w.starts[m >> 5] |= 1u << (m & 31u);
            if (bsort_route(w, 0, m, dl, false)) {
                if (m <= kSortLocal) {
                    bsort_push_small(w, 0, m, dl);
                } else {
                    w.cur_f = 0; w.cur_l = m; w.cur_d = dl; w.have = 1;
                    median_to_first(w.buf, 0, m);
                }
            }
        }
        __syncthreads();
        // parts longer than kSortLocal: the whole block
        while (w.have) {
            const uint32_t f = w.cur_f, l = w.cur_l, d = w.cur_d;
            bsort_split_block(w, f, l);
            if (tid == 0) {
                w.have = 0;
                if (!w.bad) {
                    const uint32_t cut = w.cut;
                    const int32_t pivot = skey(w.buf[f]);
                    const bool gl = bsort_route(w, f, cut, d - 1, w.kmin == pivot);
                    const bool gr = bsort_route(w, cut, l, d - 1, w.kmax == pivot);
                    // warp-sized parts are listed; of two block-sized parts the larger waits
                    const bool bl = gl && cut - f > kSortLocal, br = gr && l - cut > kSortLocal;
                    if (gl && !bl) bsort_push_small(w, f, cut, d - 1);
                    if (gr && !br) bsort_push_small(w, cut, l, d - 1);
                    if (bl && br) {
                        const bool left_small = cut - f <= l - cut;
                        if (w.n_bst < kSortStack) {
                            w.bst_f[w.n_bst] = left_small ? cut : f;
                            w.bst_l[w.n_bst] = left_small ? l : cut;
                            w.bst_d[w.n_bst] = d - 1;
                            ++w.n_bst;
                        } else {
                            w.bad = 1;
                        }
                        w.cur_f = left_small ? f : cut; w.cur_l = left_small ? cut : l; w.cur_d = d - 1; w.have = 1;
                    } else if (bl || br) {
                        w.cur_f = bl ? f : cut; w.cur_l = bl ? cut : l; w.cur_d = d - 1; w.have = 1;
                    }
                    if (!w.have && w.n_bst > 0 && !w.bad) {
                        --w.n_bst;
                        w.cur_f = w.bst_f[w.n_bst]; w.cur_l = w.bst_l[w.n_bst]; w.cur_d = w.bst_d[w.n_bst];
                        w.have = 1;
                    }
                    if (w.have) median_to_first(w.buf, w.cur_f, w.cur_l);  // the next split's pivot
                }
            }
            __syncthreads();
        }
        // parts of at most kSortLocal keys: a warp each
        const uint32_t n_sm = min(w.n_sm, kSortBlockLists);
        for (;;) {
            uint32_t idx = 0;
            if (lane == 0) idx = atomicAdd(&w.next_sm, 1u);
            idx = __shfl_sync(0xFFFFFFFFu, idx, 0);
            if (idx >= n_sm) break;
            bsort_warp(w, w.sm_f[idx], w.sm_l[idx], w.sm_d[idx]);
        }
        __syncthreads();
        const uint32_t n_fin = min(w.n_fin, kSortBlockLists);
        for (uint32_t k = tid; k < n_fin; k += T)
            if (w.fin_h[k]) heap_sort_range(w.buf + w.fin_f[k], static_cast<uint32_t>(w.fin_l[k] - w.fin_f[k]));
        __syncthreads();
        // write-back: leaves by stable rank
        for (uint32_t j = tid; j < m; j += T) {
            const uint32_t wi = j >> 5, b = j & 31u;
            uint32_t x = w.starts[wi] & (0xFFFFFFFFu >> (31u - b));
            int32_t s0 = -1;
            if (x) s0 = static_cast<int32_t>(wi * 32u + 31u - __clz(x));
            else if (wi > 0 && (x = w.starts[wi - 1]) != 0) s0 = static_cast<int32_t>((wi - 1u) * 32u + 31u - __clz(x));
            if (s0 < 0 || j - static_cast<uint32_t>(s0) >= kSortThreshold) continue;
            x = b == 31u ? 0u : (w.starts[wi] & (0xFFFFFFFFu << (b + 1u)));
            uint32_t e0;
            if (x) e0 = wi * 32u + __ffs(x) - 1u;
            else if ((x = w.starts[wi + 1]) != 0) e0 = (wi + 1u) * 32u + __ffs(x) - 1u;
            else continue;
            const uint32_t s = static_cast<uint32_t>(s0);
            if (e0 - s > kSortThreshold) continue;
            const int32_t kj = skey(w.buf[j]);
            uint32_t rank = 0;
            for (uint32_t q = s; q < e0; ++q) {
                const int32_t kq = skey(w.buf[q]);
                rank += (kq < kj || (kq == kj && q < j)) ? 1u : 0u;
            }
            ss.a[first + s + rank] = w.buf[j];
        }
        // equal-key ranges in closed form, heap-sorted ranges as they are
        for (uint32_t k = 0; k < n_fin; ++k) {
            const uint32_t f = w.fin_f[k], len = w.fin_l[k] - w.fin_f[k];
            const bool heap = w.fin_h[k] != 0;
            for (uint32_t i = tid; i < len; i += T)
                ss.a[first + f + (heap ? i : equal_final_index(i, len))] = w.buf[f + i];
        }
        if (tid == 0 && w.bad) record_error(err, ST_UNSUPPORTED, W_SORT, first);
        __syncthreads();
    }
}

// Equal-key ranges found by the rounds: one block per range places each (key, index)
// pair at its closed-form position, through apos (free after the rounds).
__global__ void __launch_bounds__(kThreads) k_sort_equal(SortScratch ss, uint32_t count) {
    for (uint32_t r = blockIdx.x; r < count; r += gridDim.x) {
        const uint32_t first = ss.equal[2 * r], m = ss.equal[2 * r + 1] - first;
        for (uint32_t i = threadIdx.x; i < m; i += kThreads) ss.apos[first + equal_final_index(i, m)] = sidx(ss.a[first + i]);
        __syncthreads();
        const unsigned long long key = ss.a[first] & 0xFFFFFFFF00000000ull;
        for (uint32_t i = threadIdx.x; i < m; i += kThreads) ss.a[first + i] = key | ss.apos[first + i];
        __syncthreads();
    }
}
__global__ void k_sort_heaps(SortScratch ss, uint32_t count) {
    PTL_FOR(k, count) heap_sort_range(ss.a + ss.heap[2 * k], ss.heap[2 * k + 1] - ss.heap[2 * k]);
}
__global__ void k_sort_out(Prog P, SortScratch ss) { PTL_FOR(p, P.n) P.pos[sidx(ss.a[p])] = p; }

// ------------------------------------------------------------------ isn_gen / optimize
__global__ void k_gen_prop(Prog P) { PTL_FOR(x, P.n) st_gen_prop(P, x); }
__global__ void k_gen_claim(Prog P) { PTL_FOR(x, P.n) st_gen_claim(P, x); }
__global__ void k_gen_write(Prog P) { PTL_FOR(x, P.n) st_gen_write(P, x); }

__global__ void k_opt_mark(Prog P) { PTL_FOR(i, P.wb8) st_opt_mark(P, i); }
__global__ void k_opt_sweep(Prog P) {
    bool any = false;
    PTL_FOR(i, P.wb8) any |= st_opt_sweep(P, i);
    if (__syncthreads_or(any) && threadIdx.x == 0) P.flags[0] = 1;
}
__global__ void k_opt_final(Prog P) { PTL_FOR(i, P.wb8) st_opt_final(P, i); }

// ------------------------------------------------------------------ regalloc
// Independent functions with an on-chip symbol cache per thread (used when the fused
// launch below cannot be made co-resident).
constexpr int kRaFreeThreads = 64;
constexpr uint32_t kRaFreeK = 64;

__device__ __forceinline__ uint32_t free_function_of(uint32_t k) {
    return (k / 7u) * 8u + (k % 7u) + 1u;  // the k-th function index that is not a multiple of 8
}

__global__ void __launch_bounds__(kRaFreeThreads) k_ra_free_cached(Prog P) {
    __shared__ uint32_t tag[kRaFreeThreads * kRaFreeK];
    __shared__ uint32_t val[kRaFreeThreads * kRaFreeK];
    const SymCache c{tag, val, kRaFreeK};
    const uint32_t f = free_function_of(blockIdx.x * kRaFreeThreads + threadIdx.x);
    if (f < P.F) ra_free_function_cached(P, c, threadIdx.x, f);
}

// The independent functions of each listed program, longest first, into ra_order: a
// warp's lanes step together until its longest function ends, so functions of similar
// length side by side waste few lane-steps (the functions are independent, so any order
// gives the same result).  One block per program: a bitonic sort of (size, index) in
// shared memory; programs with more than kOrderMax independent functions keep the
// function order.
constexpr uint32_t kOrderMax = 4096;
constexpr uint32_t kOrderThreads = 256;
__global__ void __launch_bounds__(kOrderThreads) k_free_order(const Prog* progs, const uint32_t* list,
                                                               uint32_t count) {
    __shared__ unsigned long long key[kOrderMax];
    const uint32_t tid = threadIdx.x;
    for (uint32_t k = blockIdx.x; k < count; k += gridDim.x) {
        const Prog& P = progs[list[k]];
        const uint32_t nfree = P.F - (P.F + 7u) / 8u;
        if (nfree > kOrderMax) {
            for (uint32_t x = tid; x < nfree; x += kOrderThreads) P.ra_order[x] = free_function_of(x);
            continue;
        }
        uint32_t m = 1;
        while (m < nfree) m <<= 1;
        for (uint32_t x = tid; x < m; x += kOrderThreads) {
            unsigned long long v = ~0ull;
            if (x < nfree) {
                const uint32_t size = P.fn_size0[free_function_of(x)];
                v = (static_cast<unsigned long long>(~(s32(size) > 0 ? size : 0u)) << 32) | x;
            }
            key[x] = v;
        }
        __syncthreads();
        for (uint32_t len = 2; len <= m; len <<= 1) {
            for (uint32_t stride = len >> 1; stride > 0; stride >>= 1) {
                for (uint32_t x = tid; x < m; x += kOrderThreads) {
                    const uint32_t y = x ^ stride;
                    if (y > x) {
                        const unsigned long long a = key[x], b = key[y];
                        if ((a > b) == ((x & len) == 0)) {
                            key[x] = b;
                            key[y] = a;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t x = tid; x < nfree; x += kOrderThreads)
            P.ra_order[x] = free_function_of(static_cast<uint32_t>(key[x]));
        __syncthreads();  // before the next program refills key
    }
}

// Progress chunks: hist[x] = independent functions whose last step falls in chunk x.
__global__ void k_ra_chunk_hist(Prog P, uint32_t nfree) {
    PTL_FOR(k, nfree) {
        const uint32_t f = free_function_of(k);
        if (f >= P.F) continue;
        const uint32_t size = P.fn_size0[f];
        if (s32(size) > 0) atomicAdd(&P.ra_chunks[(size - 1u) / kRaChunk], 1u);
    }
}

constexpr uint32_t kRaWaitLimit = 1u << 23;  // polls of 128 ns or more: about a second

// Lane-0 block: waits until every independent function has finished chunk c, i.e. until
// done[c] reaches need.  Gives up (false) on an error word or after the poll limit.
__device__ bool ra_wait_chunk(const uint32_t* done, uint32_t c, uint32_t need, ErrorWord* err) {
    for (uint32_t polls = 0;; ++polls) {
        if (*reinterpret_cast<const volatile uint32_t*>(&done[c]) >= need) {
            __threadfence();
            return true;
        }
        if (*reinterpret_cast<const volatile uint32_t*>(&err->code) != 0) return false;
        if (polls > kRaWaitLimit) {
            record_error(err, ST_DEVICE_TIMEOUT, W_RA2, c);
            return false;
        }
        __nanosleep(128);
    }
}

// The lane-0 pass of a program with one lane-0 function (at most 8 functions) whose
// registers are each defined once.  Every other function is in group 0, so no mark of an
// earlier group exists (the check and the Jacobi rounds never act), no later group
// triggers a position the slot reads (no swapped rewrites), and the slot wins every row-0
// position it writes.  Lane 0 of warp 0 runs the slot; the warp turns each step's trigger
// records into a 64-bit mask by ballot.  Row 0 stays in shared memory beside a mask of
// the positions that hold virtual registers.  No block barrier: the other warps return.
__device__ void ra_lane0_single(const Prog& P, uint32_t S, uint32_t K, uint32_t chunks, unsigned char* smem) {
    constexpr uint32_t kNone = 0xFFFFFFFFu;
    constexpr unsigned full = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x;  // warp 0 only
    const uint32_t* hist = P.ra_chunks;
    const uint32_t* done = P.ra_chunks + chunks;
    Ra2Shared& sh = *reinterpret_cast<Ra2Shared*>(smem);
    uint32_t* cur = reinterpret_cast<uint32_t*>(smem + sizeof(Ra2Shared));
    uint32_t* ctag = cur + 4u;
    uint32_t* cval = ctag + K;
    const SymCache c{ctag, cval, K};
    uint32_t need = 0, wc = 0, waited = 0;  // lane 0: progress of the other functions
    auto wait_for = [&](uint32_t chunk) -> int {
        while (wc < chunk) need -= hist[wc++];
        waited = chunk + 1;
        return ra_wait_chunk(done, chunk, need, P.err) ? 0 : 1;
    };
    int abort = 0;
    Ra2Slot L;
    L.act = false;
    L.have_next = false;
    uint32_t s0 = 0;
    if (lane == 0) {
        for (uint32_t x = 0; x < chunks; ++x) need += hist[x];
        if (chunks > 0 && S > 0) abort = wait_for(0);
        ra2_slot_init(P, c, L, 0, 0);
        s0 = min(ra2_lane0_size(L), S);
    }
    sh.R0[lane] = sh.R0[lane + 32] = kNone;
    sh.R0own[lane] = sh.R0own[lane + 32] = kNone;
    s0 = __shfl_sync(full, s0, 0);
    if (__shfl_sync(full, abort, 0)) return;
    unsigned long long occ = 0;  // lane 0: positions whose row-0 entry is a virtual register
    uint32_t t0 = 0, t1 = 0;     // this step's records at positions lane and lane + 32
    if (s0 > 0) {
        t0 = __ldcg(&P.trig_max[lane]);
        t1 = __ldcg(&P.trig_max[32u + lane]);
    }
    __syncwarp();
    for (uint32_t i = 0; i < s0; ++i) {
        if (chunks > 0 && i + 2 < S && (i + 2) % kRaChunk == 0) {
            int ab = 0;
            if (lane == 0) ab = wait_for((i + 2) / kRaChunk);
            if (__shfl_sync(full, ab, 0)) return;
        }
        const unsigned long long others = static_cast<unsigned long long>(__ballot_sync(full, t0 != 0)) |
                                          (static_cast<unsigned long long>(__ballot_sync(full, t1 != 0)) << 32);
        if (i + 1 < S) {  // records of the next step (its chunk is complete: waited above)
            t0 = __ldcg(&P.trig_max[static_cast<size_t>(i + 1) * 64u + lane]);
            t1 = __ldcg(&P.trig_max[static_cast<size_t>(i + 1) * 64u + 32u + lane]);
        }
        if (lane == 0) {
            ra2_load(P, L, i, cur);
            RaStep& St = L.S;
            unsigned long long marks = others & occ;
            if (L.act) {
                uint32_t r1reg = 0, r2reg = 0;
                bool r1s = false, r2s = false;
                if (s32(St.r1) > 63) sym_read(P, c, 0, St.r1, &r1reg, &r1s);
                if (s32(St.r2) > 63) sym_read(P, c, 0, St.r2, &r2reg, &r2s);
                ra_compute(St, L.lifetime, r1reg, r1s, r2reg, r2s);
                L.lt_new = St.cleared | St.rdm;
                if (s32(St.ord) > 63) sym_write(P, c, 0, St.ord, St.rdr, false, (St.rdr & 63u) + 1u);
                if (s32(St.r1) > 63) sym_write(P, c, 0, St.r1, St.r1r, false);
                if (s32(St.r2) > 63) sym_write(P, c, 0, St.r2, St.r2r, false);
                marks = (others | St.trig) & occ;
            }
            // marks on the symbols row 0 held at the step's start, unless the slot updated them
            for (unsigned long long m = marks; m; m &= m - 1) {
                const uint32_t v = sh.R0[ctz64(m)];
                const bool updated = L.act && ((s32(St.ord) > 63 && St.ord == v) || (s32(St.r1) > 63 && St.r1 == v) ||
                                               (s32(St.r2) > 63 && St.r2 == v));
                if (!updated) sym_mark(P, c, 0, v);
            }
            // row 0: the defined register at its position, cleared entries at rs1 / rs2
            if (L.act) {
                if (St.ord != 0) {
                    const uint32_t q = St.rdr & 63u;
                    sh.R0[q] = St.ord;
                    sh.R0own[q] = 0;
                    occ = s32(St.ord - 64u) >= 0 ? (occ | (1ull << q)) : (occ & ~(1ull << q));
                }
                for (const uint32_t r : {St.r1r, St.r2r}) {
                    if (r != St.rdr && s32(r) >= 0 && r < 64u) {
                        sh.R0[r] = kNone;
                        sh.R0own[r] = 0;
                        occ &= ~(1ull << r);
                    }
                }
            }
        }
        __syncwarp();
    }
    if (s0 >= S) return;
    // the steps after the slot's last one only mark row 0's symbols
    int ab = 0;
    if (lane == 0)
        for (uint32_t x = waited; x < chunks && !ab; ++x) ab = wait_for(x);
    if (__shfl_sync(full, ab, 0)) return;
    __syncwarp();
    ra2_tail_p(P, c, sh, lane, s0, S);
    ra2_tail_p(P, c, sh, lane + 32u, s0, S);
}

// Register allocation steps in one launch.  Block 0 runs the lane-0 functions (f % 8 ==
// 0) in lock-step; thread t runs slots t, t+T, ... (Q per thread), slot = group index.
// Blocks 1.. run the independent functions, one per thread, and count finished chunks
// of trigger records; block 0 waits for a chunk before it loads that chunk's records.
// With chunks == 0 there are no other blocks: the independent functions ran before.
// Per step of block 0:
//   1. each active function computes its step; a symbol reads as swapped if a function
//      of an earlier group triggered the physical register holding it in row 0.  The
//      other functions' triggers are known (trig_min/trig_max); earlier lane-0 triggers
//      depend on the same computation, so when an operand sits in row 0 the CTA
//      iterates until the per-register minimum trigger group stops changing (a DAG in
//      group order);
//   2. symbol updates: a symbol updated by its owner ends swapped only if a later group
//      also triggered it; other triggered symbols end swapped;
//   3. row 0 takes, per physical register, the write of the highest group.
// The lane-0 block: P's lane-0 functions in lock-step over S steps, K cache entries per
// function in smem.  With chunks > 0 it waits on the independent functions' progress.
template <int Q>
__device__ void ra_lane0_block(const Prog& P, uint32_t S, uint32_t K, uint32_t chunks, unsigned char* smem) {
    if (P.F <= 8u && P.defpos) {  // one lane-0 function: warp 0 alone, no block barriers
        if (threadIdx.x < 32) ra_lane0_single(P, S, K, chunks, smem);
        return;
    }
    const uint32_t tid = threadIdx.x, T = blockDim.x;
    __shared__ uint32_t s_abort, s_s0;
    const uint32_t* hist = P.ra_chunks;
    const uint32_t* done = P.ra_chunks + chunks;
    Ra2Shared& sh = *reinterpret_cast<Ra2Shared*>(smem);
    const uint32_t G0 = (P.F + 7u) / 8u;
    uint32_t* cur = reinterpret_cast<uint32_t*>(smem + sizeof(Ra2Shared));
    uint32_t* ctag = cur + 4u * G0;
    uint32_t* cval = ctag + G0 * K;
    const SymCache c{ctag, cval, K};
    const bool hashed = P.defpos == nullptr;
    // Row-0 phases: thread tid handles physical registers tid, tid + T, ... (two each in a
    // one-warp block, which small programs get: its barriers cost next to nothing).
    constexpr uint32_t kRow = 64;
    // thread 0: independent functions still running in chunk wc (need); chunks below
    // `waited` are complete
    uint32_t need = 0, wc = 0, waited = 0;
    auto wait_for = [&](uint32_t chunk) {
        while (wc < chunk) need -= hist[wc++];
        if (!ra_wait_chunk(done, chunk, need, P.err)) s_abort = 1;
        waited = chunk + 1;
    };
    if (tid == 0) {
        s_abort = 0;
        s_s0 = 0;
        for (uint32_t x = 0; x < chunks; ++x) need += hist[x];
        if (chunks > 0 && S > 0) wait_for(0);
    }
    __syncthreads();
    Ra2Slot L[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const uint32_t j = tid + static_cast<uint32_t>(q) * T;
        L[q].act = false;
        L[q].have_next = false;
        if (j < G0) {
            ra2_slot_init(P, c, L[q], j, j);
            atomicMax(&s_s0, ra2_lane0_size(L[q]));
        }
    }
    uint32_t tmin[2] = {0xFFFFFFFFu, 0xFFFFFFFFu}, tmax[2] = {0, 0};  // trigger records, one step ahead
    for (uint32_t p = tid; p < kRow; p += T) {
        sh.R0[p] = 0xFFFFFFFFu;
        sh.R0own[p] = 0xFFFFFFFFu;
    }
    for (uint32_t k = tid; k < kSnapHash; k += T) {
        sh.hkey[0][k] = sh.hkey[1][k] = 0;
        sh.hmask[0][k] = sh.hmask[1][k] = 0;
    }
    __syncthreads();
    if (s_abort) return;
    // trigger records are read from L2: lines of a chunk may sit in L1 from the chunk before
    if (S > 0) {
#pragma unroll
        for (uint32_t r = 0; r < 2; ++r) {  // T >= 32: at most two positions per thread
            const uint32_t p = tid + r * T;
            if (p >= kRow) continue;
            ra2_begin_p(sh, 0, p, __ldcg(&P.trig_min[p]), __ldcg(&P.trig_max[p]), hashed);
            if (S > 1) { tmin[r] = __ldcg(&P.trig_min[kRow + p]); tmax[r] = __ldcg(&P.trig_max[kRow + p]); }
        }
    }
    __syncthreads();
    // Per step, three barriers: (load+compute) | (check + speculative apply + clear next
    // hash) | (marks, row 0, next step's snapshot).  Steps run while a lane-0 function is
    // still running (s0); the rest come down to ra2_tail_p.
    const uint32_t s0 = min(s_s0, S);
    for (uint32_t i = 0; i < s0; ++i) {
        if (tid == 0 && chunks > 0 && i + 2 < S && (i + 2) % kRaChunk == 0) wait_for((i + 2) / kRaChunk);
        bool in_row0 = false;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const uint32_t j = tid + static_cast<uint32_t>(q) * T;
            if (j < G0) {
                ra2_load(P, L[q], i, cur + 4u * j);
                in_row0 |= ra2_compute0(P, c, sh, L[q], j, i);
            }
        }
        const bool any_row0 = __syncthreads_or(in_row0);
        if (s_abort) break;  // set before the barrier: every thread leaves together
        // Apply speculatively; if an earlier lane-0 trigger changes what some slot read
        // (rare), undo the row-0 writes, iterate to the fixed point and apply again.
        bool flag = false;
        if (any_row0) {
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const uint32_t j = tid + static_cast<uint32_t>(q) * T;
                if (j < G0) flag |= ra2_check(sh, L[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const uint32_t j = tid + static_cast<uint32_t>(q) * T;
            if (j < G0) ra2_apply(P, c, sh, L[q], j, i, cur + 4u * j);
        }
        if (hashed)
            for (uint32_t p = tid; p < kRow; p += T) snap_clear_next(sh, i, p);
        if (__syncthreads_or(flag)) {
            for (uint32_t p = tid; p < kRow; p += T) sh.r0grp[p] = 0;
            for (uint32_t round = 0;; ++round) {
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    const uint32_t j = tid + static_cast<uint32_t>(q) * T;
                    if (j < G0) ra2_round(sh, L[q]);
                }
                __syncthreads();
                bool changed = false;
                for (uint32_t p = tid; p < kRow; p += T) changed |= ra2_round_p(sh, p);
                if (!__syncthreads_or(changed)) break;
                if (round > G0 + 2u) {
                    if (tid == 0) record_error(P.err, ST_DEVICE_TIMEOUT, W_RA2, i);
                    break;
                }
            }
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const uint32_t j = tid + static_cast<uint32_t>(q) * T;
                if (j < G0) ra2_apply(P, c, sh, L[q], j, i, cur + 4u * j);
            }
            __syncthreads();
        }
#pragma unroll
        for (uint32_t r = 0; r < 2; ++r) {
            const uint32_t p = tid + r * T;
            if (p < kRow) {
                ra2_end_p(P, c, sh, p, cur);
                if (i + 1 < S) {
                    ra2_begin_p(sh, i + 1, p, tmin[r], tmax[r], hashed);
                    if (i + 2 < S) {
                        tmin[r] = __ldcg(&P.trig_min[static_cast<size_t>(i + 2) * kRow + p]);
                        tmax[r] = __ldcg(&P.trig_max[static_cast<size_t>(i + 2) * kRow + p]);
                    }
                }
            }
        }
        __syncthreads();
    }
    if (s0 >= S || s_abort) return;
    // the remaining steps' trigger records, then one check per row-0 position
    if (tid == 0)
        for (uint32_t x = waited; x < chunks && !s_abort; ++x) wait_for(x);
    __syncthreads();
    if (s_abort) return;
    for (uint32_t p = tid; p < kRow; p += T) ra2_tail_p(P, c, sh, p, s0, S);
}


template <int Q>
__global__ void __launch_bounds__(1024) k_ra_steps(Prog P, uint32_t S, uint32_t K, uint32_t Kf, uint32_t chunks) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t tid = threadIdx.x, T = blockDim.x;
    if (blockIdx.x > 0) {
        uint32_t* tag = reinterpret_cast<uint32_t*>(smem);
        const SymCache cf{tag, tag + T * Kf, Kf};
        // the independent functions never need definition positions
        Prog Pf = P;
        Pf.defpos = nullptr;
        const uint32_t f = free_function_of((blockIdx.x - 1u) * T + tid);
        if (f < P.F) ra_free_function_cached(Pf, cf, tid, f, P.ra_chunks + chunks);
        return;
    }
    ra_lane0_block<Q>(P, S, K, chunks, smem);
}

// ------------------------------------------------------- the lane-0 pass on a cluster
// A program with more lane-0 groups than one block runs at one slot per thread (above
// 1,024) spreads its slots over the CTAs of a thread-block cluster: one per thread (Q
// per thread above 8 x 512).  Each CTA keeps its own copy of row 0 and of the step
// state the slots read (Ra2Shared) and runs the end-of-step phase on it itself (one
// thread per physical register), so that phase needs no cluster barrier after it: the
// copies stay equal because they are computed from the same values.  What all slots add
// to in a step -- lane-0 triggers and the highest group writing each position (Ra2Agg)
// -- lives in CTA 0's shared memory, reached through distributed shared memory, one set
// per step parity; the slots' step records are kept per parity too, so a CTA that has
// gone on to the next step never overwrites what a slower CTA's end phase still reads
// (no CTA gets two steps ahead: each step starts with a cluster barrier).  A CTA marks
// only the symbols of its own slots (cache and global memory); the others see the marks
// of their own.  A barrier that ORs a flag adds to a word in CTA 0: three words in
// rotation, the one the next such barrier uses cleared before this one.  The
// independent functions ran before, so every trigger record is complete and nothing
// waits.
namespace cg = cooperative_groups;
constexpr uint32_t kRaClusterThreads = 512;
constexpr uint32_t kRaClusterMax = 8;  // the portable cluster size

struct Ra2Agg {
    uint32_t lcur[64], lmax[64];       // lane-0 triggers of the current round
    uint32_t lnew[64], lmaxnew[64];    // of the next Jacobi round
    uint32_t r0grp[64];                // highest group (+1) writing each position
};

__device__ bool c_marked_before(const Ra2Shared& loc, const Ra2Agg& ag, uint64_t m, uint32_t j, bool with_lane0) {
    for (; m; m &= m - 1) {
        const uint32_t p = ctz64(m);
        uint32_t g = loc.omin[p];
        if (with_lane0 && ag.lcur[p] < g) g = ag.lcur[p];
        if (g <= j) return true;
    }
    return false;
}
__device__ void c_add_triggers(Ra2Agg& ag, uint64_t trig, uint32_t g1, bool into_new) {
    for (uint64_t t = trig; t; t &= t - 1) {
        const uint32_t p = ctz64(t);
        if (into_new) {
            atomicMin(&ag.lnew[p], g1);
            atomicMax(&ag.lmaxnew[p], g1);
        } else {
            atomicMin(&ag.lcur[p], g1);
            atomicMax(&ag.lmax[p], g1);
        }
    }
}
// ra2_compute0, ra2_check, ra2_round, ra2_round_p and ra2_apply (ptl_ra.cuh) with the
// aggregates apart from the CTA's copy of the step state.
__device__ bool c_compute0(const Prog& P, const SymCache& c, const Ra2Shared& loc, Ra2Agg& ag, Ra2Slot& L,
                           uint32_t slot, uint32_t i) {
    if (!L.act) return false;
    RaStep& S = L.S;
    L.r1reg = L.r2reg = 0;
    L.r1stored = L.r2stored = false;
    L.m1 = L.m2 = 0;
    if (s32(S.r1) > 63) {
        uint32_t d;
        sym_read(P, c, slot, S.r1, &L.r1reg, &L.r1stored, &d);
        L.m1 = snap_positions(P, loc, i, S.r1, d);
    }
    if (s32(S.r2) > 63) {
        uint32_t d;
        sym_read(P, c, slot, S.r2, &L.r2reg, &L.r2stored, &d);
        L.m2 = snap_positions(P, loc, i, S.r2, d);
    }
    L.r1m = c_marked_before(loc, ag, L.m1, L.j, false);
    L.r2m = c_marked_before(loc, ag, L.m2, L.j, false);
    ra_compute(S, L.lifetime, L.r1reg, L.r1stored || L.r1m, L.r2reg, L.r2stored || L.r2m);
    c_add_triggers(ag, S.trig, L.j + 1u, false);
    return (L.m1 | L.m2) != 0;
}
__device__ bool c_check(const Ra2Shared& loc, const Ra2Agg& ag, const Ra2Slot& L) {
    if (!L.act || (L.m1 | L.m2) == 0) return false;
    return c_marked_before(loc, ag, L.m1, L.j, true) != L.r1m || c_marked_before(loc, ag, L.m2, L.j, true) != L.r2m;
}
__device__ void c_round(const Ra2Shared& loc, Ra2Agg& ag, Ra2Slot& L) {
    if (!L.act) return;
    if (L.m1 | L.m2) {
        L.r1m = c_marked_before(loc, ag, L.m1, L.j, true);
        L.r2m = c_marked_before(loc, ag, L.m2, L.j, true);
        ra_compute(L.S, L.lifetime, L.r1reg, L.r1stored || L.r1m, L.r2reg, L.r2stored || L.r2m);
    }
    c_add_triggers(ag, L.S.trig, L.j + 1u, true);
}
__device__ bool c_round_p(Ra2Agg& ag, uint32_t p) {
    const bool changed = ag.lnew[p] != ag.lcur[p];
    ag.lcur[p] = ag.lnew[p];
    ag.lmax[p] = ag.lmaxnew[p];
    ag.lnew[p] = 0xFFFFFFFFu;
    ag.lmaxnew[p] = 0;
    return changed;
}
__device__ void c_apply(const Prog& P, const SymCache& c, const Ra2Shared& loc, Ra2Agg& ag, Ra2Slot& L, uint32_t slot,
                        uint32_t i, uint32_t* cur) {
    if (!L.act) return;
    const RaStep& S = L.S;
    L.lt_new = S.cleared | S.rdm;
    const uint32_t g1 = L.j + 1u;
    auto later = [&](uint64_t m) {
        for (; m; m &= m - 1) {
            const uint32_t p = ctz64(m);
            const uint32_t g = loc.omax[p] > ag.lmax[p] ? loc.omax[p] : ag.lmax[p];
            if (g > g1) return true;
        }
        return false;
    };
    const bool l_ord = !P.defpos && s32(S.ord) > 63 && later(snap_positions_hashed(loc, i, S.ord));
    const bool l_r1 = s32(S.r1) > 63 && later(L.m1);
    const bool l_r2 = s32(S.r2) > 63 && later(L.m2);
    if (s32(S.ord) > 63) sym_write(P, c, slot, S.ord, S.rdr, false, (S.rdr & 63u) + 1u);
    if (s32(S.r1) > 63) sym_write(P, c, slot, S.r1, S.r1r, false);
    if (s32(S.r2) > 63) sym_write(P, c, slot, S.r2, S.r2r, false);
    const bool r2v = s32(S.r2) > 63, r1v = s32(S.r1) > 63;
    if (l_ord) sym_write(P, c, slot, S.ord, (r2v && S.r2 == S.ord) ? S.r2r : ((r1v && S.r1 == S.ord) ? S.r1r : S.rdr), true);
    if (l_r1) sym_write(P, c, slot, S.r1, (r2v && S.r2 == S.r1) ? S.r2r : S.r1r, true);
    if (l_r2) sym_write(P, c, slot, S.r2, S.r2r, true);
    cur[3] = S.rdr & 63u;
    if (S.ord != 0) atomicMax(&ag.r0grp[S.rdr & 63u], g1);
    if (S.r1r != S.rdr && s32(S.r1r) >= 0 && S.r1r < 64u) atomicMax(&ag.r0grp[S.r1r], g1);
    if (S.r2r != S.rdr && s32(S.r2r) >= 0 && S.r2r < 64u) atomicMax(&ag.r0grp[S.r2r], g1);
}
// ra2_end_p on this CTA's copy of row 0: the marks of the symbols of its own slots (the
// owner's record is local), then row 0 takes the highest group's write, whose record
// may sit in any CTA.  cur: this CTA's records of the step (parity); recs(slot): any
// slot's, through distributed shared memory.
__device__ void c_end_p(const Prog& P, const SymCache& c, Ra2Shared& loc, const Ra2Agg& ag, uint32_t p, uint32_t rank,
                        uint32_t per_cta, const uint32_t* cur) {
    const bool triggered = loc.omin[p] != 0xFFFFFFFFu || ag.lcur[p] != 0xFFFFFFFFu;
    const uint32_t v = loc.snap[p];
    const uint32_t own = loc.snapown[p];
    const bool mine = own == 0xFFFFFFFFu ? rank == 0 : own / per_cta == rank;
    if (triggered && s32(v - 64u) >= 0 && mine) {
        bool updated = false;
        if (own != 0xFFFFFFFFu) {
            const uint32_t* u = cur + 4u * (own % per_cta);
            updated = (s32(u[0]) > 63 && u[0] == v) || (s32(u[1]) > 63 && u[1] == v) || (s32(u[2]) > 63 && u[2] == v);
        }
        if (!updated) sym_mark(P, c, own == 0xFFFFFFFFu ? 0xFFFFFFFFu : own % per_cta, v);
    }
    const uint32_t g = ag.r0grp[p];
    if (g != 0) {
        const uint32_t w = g - 1u;
        const uint32_t* r = cg::this_cluster().map_shared_rank(const_cast<uint32_t*>(cur), w / per_cta) + 4u * (w % per_cta);
        loc.R0[p] = (r[0] != 0 && r[3] == p) ? r[0] : 0xFFFFFFFFu;
        loc.R0own[p] = w;
    }
}

template <int Q>
__global__ void __launch_bounds__(kRaClusterThreads, 1)
    k_ra_lane0_cluster(Prog P, uint32_t S, uint32_t K, uint32_t per_cta) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t s_s0, s_or[3];
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t rank = cl.block_rank(), tid = threadIdx.x, T = blockDim.x;
    const uint32_t G0 = (P.F + 7u) / 8u;
    Ra2Shared& loc = *reinterpret_cast<Ra2Shared*>(smem);  // this CTA's copy of row 0 and the step state
    Ra2Agg* agl = reinterpret_cast<Ra2Agg*>(smem + sizeof(Ra2Shared));  // [2]: used in CTA 0
    uint32_t* cur = reinterpret_cast<uint32_t*>(smem + sizeof(Ra2Shared) + 2 * sizeof(Ra2Agg));  // [2][per_cta][4]
    uint32_t* ctag = cur + 8u * per_cta;
    uint32_t* cval = ctag + per_cta * K;
    const SymCache c{ctag, cval, K};  // this CTA's slots, by local index
    const bool row = tid < 64u;       // the CTA's row-0 threads (T >= 64)
    const bool hashed = P.defpos == nullptr;
    if (tid == 0) {
        s_s0 = 0;
        s_or[0] = s_or[1] = s_or[2] = 0;
    }
    cl.sync();  // every CTA has started (its shared memory exists) before remote accesses
    Ra2Agg* ag = cl.map_shared_rank(agl, 0);
    uint32_t* s0p = cl.map_shared_rank(&s_s0, 0);
    uint32_t* orp = cl.map_shared_rank(s_or, 0);
    uint32_t nbar = 0;  // OR barriers so far (the same count in every thread)
    auto cluster_or = [&](bool v) -> bool {
        const uint32_t k = nbar % 3u;
        if (rank == 0 && tid == 0) orp[(k + 1u) % 3u] = 0;
        if (__any_sync(0xFFFFFFFFu, v) && (tid & 31u) == 0) atomicOr(&orp[k], 1u);
        cl.sync();
        ++nbar;
        return *reinterpret_cast<volatile uint32_t*>(&orp[k]) != 0;
    };
    auto reset_agg = [&](Ra2Agg& a, uint32_t p) {
        a.lcur[p] = 0xFFFFFFFFu;
        a.lmax[p] = 0;
        a.lnew[p] = 0xFFFFFFFFu;
        a.lmaxnew[p] = 0;
        a.r0grp[p] = 0;
    };
    Ra2Slot L[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const uint32_t l = tid + static_cast<uint32_t>(q) * T;
        L[q].act = false;
        L[q].have_next = false;
        if (l < per_cta && rank * per_cta + l < G0) {
            ra2_slot_init(P, c, L[q], l, rank * per_cta + l);
            atomicMax(s0p, ra2_lane0_size(L[q]));
        }
    }
    if (row) {
        loc.R0[tid] = 0xFFFFFFFFu;
        loc.R0own[tid] = 0xFFFFFFFFu;
        if (rank == 0) {
            reset_agg(agl[0], tid);
            reset_agg(agl[1], tid);
        }
    }
    for (uint32_t k = tid; k < kSnapHash; k += T) {
        loc.hkey[0][k] = loc.hkey[1][k] = 0;
        loc.hmask[0][k] = loc.hmask[1][k] = 0;
    }
    __syncthreads();
    uint32_t tmin = 0xFFFFFFFFu, tmax = 0;  // a row-0 thread's trigger records, one step ahead
    if (row && S > 0) {
        ra2_begin_p(loc, 0, tid, __ldcg(&P.trig_min[tid]), __ldcg(&P.trig_max[tid]), hashed);
        if (S > 1) {
            tmin = __ldcg(&P.trig_min[64u + tid]);
            tmax = __ldcg(&P.trig_max[64u + tid]);
        }
    }
    cl.sync();  // the slots' step lengths and CTA 0's aggregates, for every CTA
    const uint32_t s0 = min(*reinterpret_cast<volatile uint32_t*>(s0p), S);
    for (uint32_t i = 0; i < s0; ++i) {
        const uint32_t par = i & 1u;
        Ra2Agg& a = ag[par];
        uint32_t* curp = cur + par * 4u * per_cta;
        bool in_row0 = false;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const uint32_t l = tid + static_cast<uint32_t>(q) * T;
            if (l < per_cta && rank * per_cta + l < G0) {
                ra2_load(P, L[q], i, curp + 4u * l);
                in_row0 |= c_compute0(P, c, loc, a, L[q], l, i);
            }
        }
        const bool any_row0 = cluster_or(in_row0);
        // the other parity's aggregates: every CTA read them last in the previous step's
        // end phase, before the barrier above; the next step's first writes come after the
        // barrier below
        if (rank == 0 && row) reset_agg(ag[par ^ 1u], tid);
        bool flag = false;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const uint32_t l = tid + static_cast<uint32_t>(q) * T;
            if (l < per_cta && rank * per_cta + l < G0) {
                if (any_row0) flag |= c_check(loc, a, L[q]);
                c_apply(P, c, loc, a, L[q], l, i, curp + 4u * l);
            }
        }
        if (hashed && row) snap_clear_next(loc, i, tid);
        if (cluster_or(flag)) {
            if (rank == 0 && row) a.r0grp[tid] = 0;
            for (uint32_t round = 0;; ++round) {
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    const uint32_t l = tid + static_cast<uint32_t>(q) * T;
                    if (l < per_cta && rank * per_cta + l < G0) c_round(loc, a, L[q]);
                }
                cl.sync();
                const bool changed = rank == 0 && row && c_round_p(a, tid);
                if (!cluster_or(changed)) break;
                if (round > G0 + 2u) {
                    if (rank == 0 && tid == 0) record_error(P.err, ST_DEVICE_TIMEOUT, W_RA2, i);
                    break;
                }
            }
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const uint32_t l = tid + static_cast<uint32_t>(q) * T;
                if (l < per_cta && rank * per_cta + l < G0) c_apply(P, c, loc, a, L[q], l, i, curp + 4u * l);
            }
            cl.sync();
        }
        if (row) {
            c_end_p(P, c, loc, a, tid, rank, per_cta, curp);
            if (i + 1 < S) {
                ra2_begin_p(loc, i + 1, tid, tmin, tmax, hashed);
                if (i + 2 < S) {
                    tmin = __ldcg(&P.trig_min[static_cast<size_t>(i + 2) * 64u + tid]);
                    tmax = __ldcg(&P.trig_max[static_cast<size_t>(i + 2) * 64u + tid]);
                }
            }
        }
        __syncthreads();  // this CTA's copy of row 0 is ready for the next step
    }
    cl.sync();  // every end phase has read the other CTAs' records: none exits before
    if (s0 >= S) return;
    // the steps after the last lane-0 one only mark row 0's symbols (global memory)
    if (rank == 0 && row && ra2_tail_hit(P, loc, tid, s0, S)) P.symswp[loc.R0[tid] - 64u] = 0xFFFFFFFFu;
}

// flags[1]: functions share symbols; flags[2]: a lane-0 virtual register has two
// definitions.  stamp counts the definitions (zeroed before).
__global__ void k_ra_cross(Prog P) {
    uint32_t any = 0;
    PTL_FOR(i, P.W) any |= st_ra_cross(P, i, P.stamp);
    if (__syncthreads_or(any & 1u) && threadIdx.x == 0) P.flags[1] = 1;
    if (__syncthreads_or(any & 2u) && threadIdx.x == 0) P.flags[2] = 1;
}
__global__ void k_ra_serial(Prog P) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st_ra_serial(P, P.stamp);
}
__global__ void k_ra_spill(Prog P) { PTL_FOR(v, P.W) st_ra_spill(P, v); }
__global__ void k_ra_scatter(Prog P) { PTL_FOR(i, P.wb8) st_ra_scatter(P, i); }
__global__ void k_ra_functab(Prog P) { PTL_FOR(f, P.F) st_fix_functab(P, f, P.roffs, P.W); }
__global__ void k_ra_frame(Prog P) { PTL_FOR(f, P.F) st_ra_frame(P, f); }
__global__ void k_fj_emit(Prog P) { PTL_FOR(i, P.W2) st_fj_emit(P, i); }
__global__ void k_fj_functab(Prog P) { PTL_FOR(f, P.F) st_fix_functab(P, f, P.joffs, P.W2); }

// ------------------------------------------------------------------ scalar semantics
// The stages where the scalar generator differs (ptl_scalar.cuh).
__global__ void k_s_pre_lists(Prog P) { PTL_FOR(i, P.nb8) st_s_pre_lists(P, i); }
__global__ void k_s_pre_float(Prog P) { PTL_FOR(i, P.nb8) st_s_pre_float(P, i); }
__global__ void k_s_gen_prop(Prog P) { PTL_FOR(x, P.n) st_s_gen_prop(P, x); }
__global__ void k_s_gen_claim(Prog P) { PTL_FOR(x, P.n) st_s_gen_claim(P, x); }
__global__ void k_s_gen_write(Prog P) { PTL_FOR(x, P.n) st_s_gen_write(P, x); }
// Functions on their own: one warp per tile of the word space (the functions starting in
// it, one per lane), their symbols as bytes in shared memory (cap bytes; a tile whose
// words exceed it works on the program's arrays), the 64-entry register state of each
// function in local memory.
constexpr int kScalarRaThreads = 32;
constexpr uint32_t kScalarTileWords = 4096;
__global__ void __launch_bounds__(kScalarRaThreads) k_s_ra_tiles(Prog P, unsigned long long* preserve, uint32_t cap) {
    extern __shared__ uint8_t s_sym[];
    uint32_t first, last, base;
    s_ra_tile_functions(P, blockIdx.x, kScalarTileWords, &first, &last);
    const uint32_t count = s_ra_tile_span(P, first, last, &base);
    if (first >= last) return;
    int32_t regs[64];
    if (count > cap) {
        for (uint32_t f = first + threadIdx.x; f < last; f += blockDim.x) s_ra_function(P, SymGlobal{P}, f, regs, preserve);
        return;
    }
    for (uint32_t k = threadIdx.x; k < count; k += blockDim.x) s_sym[k] = 0;
    __syncthreads();
    const SymBytes sy{s_sym, base, count, P.err};
    for (uint32_t f = first + threadIdx.x; f < last; f += blockDim.x) s_ra_function(P, sy, f, regs, preserve);
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < count; k += blockDim.x) s_ra_tile_writeback(P, s_sym, base, count, k);
}
// The same steps (s_ra_function, ptl_scalar.cuh) with one warp per function, for the
// latency of one program's longest function: every lane runs the step's scalar logic on
// the same values (no divergence), lane k holds registers k and k + 32 of the register
// state in registers, a swap reads the register it needs by a shuffle, and the
// function's symbols are bytes in shared memory (register in bits 0..5, swapped in bit
// 7).  Every lane performs every symbol write with the same value, so each lane reads
// back what all wrote without a barrier.  Functions of at most `stride` words.
constexpr uint32_t kScalarWarpFns = 4;          // functions (warps) per block
constexpr uint32_t kScalarWarpSymCap = 12288;   // symbol bytes per warp
// Function f of P by the calling warp; sym: the warp's `stride` symbol bytes.
__device__ void s_ra_warp_function(const Prog& P, uint32_t f, unsigned long long* preserve, uint32_t stride,
                                   uint8_t* sym) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    if (!s_ra_function_ok(P, f) || P.fn_size0[f] > stride) {
        if (lane == 0) record_error(P.err, ST_UNSUPPORTED, W_RA1, f);
        return;
    }
    const uint32_t start = P.fn_start0[f], size = P.fn_size0[f];
    for (uint32_t k = lane; k < size; k += 32u) sym[k] = 0;
    __syncwarp();
    int32_t rlo = -1, rhi = -1;  // regs[lane], regs[lane + 32]
    unsigned long long mask = 0x1Full, pm = 0;
    bool bad = false;
    // a symbol's byte index; the cross check keeps it inside the function
    auto at = [&](uint32_t r) -> uint32_t {
        const uint32_t w = r - 64u - start;
        if (w >= size) bad = true;
        return w < size ? w : 0u;
    };
    auto mark = [&](uint64_t regs_swapped) {
        for (uint64_t m = regs_swapped; m; m &= m - 1ull) {
            const uint32_t j = ctz64(m);
            const int32_t v = __shfl_sync(kFull, j < 32u ? rlo : rhi, j & 31u);
            if (v >= 64) {
                const uint32_t w = at(u32(v));
                sym[w] = static_cast<uint8_t>(sym[w] | 0x80u);
            }
        }
    };
    SWord cur = size > 0 ? s_word(P, start) : SWord{};
    for (uint32_t i = 0; i < size && !bad; ++i) {
        const SWord next = i + 1 < size ? s_word(P, start + i + 1) : SWord{};
        if (cur.used) {
            const uint32_t ins = cur.ins;
            if (ins == 0x000000EFu && cur.jt - start >= size) {  // a call out of the function
                mark(mask & ~kPreservedRegisterMask);
                mask &= kPreservedRegisterMask;
                if (!((mask >> lane) & 1ull)) rlo = -1;
                if (!((mask >> (lane + 32u)) & 1ull)) rhi = -1;
            } else {
                const uint32_t r1 = cur.r1, r2 = cur.r2, rdv = cur.rd;
                uint32_t rs1 = r1, rs2 = r2;
                if (r1 >= 64u) {
                    const uint32_t b = sym[at(r1)];
                    rs1 = (b & 0x80u) ? (s_needs_float(ins, 1) ? 37u : 5u) : (b & 0x3Fu);
                }
                if (r2 >= 64u) {
                    const uint32_t b = sym[at(r2)];
                    rs2 = (b & 0x80u) ? (s_needs_float(ins, 2) ? 38u : 6u) : (b & 0x3Fu);
                }
                unsigned long long cleared = mask;
                if (rs1 != 0) cleared &= ~(1ull << rs1);
                if (rs2 != 0) cleared &= ~(1ull << rs2);
                uint32_t rdr = rdv;
                if (rdv >= 64u) {
                    const bool fl = s_needs_float(ins, 0);
                    const uint32_t r = ffz_low32(cleared | (fl ? 0x00000000FFFFFFFFull : 0xFFFFFFFF00000000ull));
                    rdr = r == 64u ? (fl ? 37u : 5u) : r;
                }
                unsigned long long swap = 0;
                if (rdr != 0 && ((cleared >> rdr) & 1ull)) swap |= 1ull << rdr;
                if (rs1 != 0 && ((mask >> rs1) & 1ull)) swap |= 1ull << rs1;
                if (rs2 != 0 && ((mask >> rs2) & 1ull)) swap |= 1ull << rs2;
                mark(swap);  // from the register state before the step
                if (rdv >= 64u) sym[at(rdv)] = static_cast<uint8_t>(rdr);  // rd, rs1, rs2: a later write wins
                if (r1 >= 64u) sym[at(r1)] = static_cast<uint8_t>(rs1);
                if (r2 >= 64u) sym[at(r2)] = static_cast<uint8_t>(rs2);
                if ((rdr & 31u) == lane) (rdr < 32u ? rlo : rhi) = s32(rdv);
                if (rs1 != rdr && (rs1 & 31u) == lane) (rs1 < 32u ? rlo : rhi) = -1;
                if (rs2 != rdr && (rs2 & 31u) == lane) (rs2 < 32u ? rlo : rhi) = -1;
                mask = cleared | (1ull << rdr);
            }
        }
        pm |= mask;
        cur = next;
    }
    if (bad) {
        if (lane == 0) record_error(P.err, ST_UNSUPPORTED, W_RA1, f);
        return;
    }
    if (lane == 0) preserve[f] = pm & kNonscratchRegisters;
    __syncwarp();
    for (uint32_t k = lane; k < size; k += 32u) {
        const uint32_t b = sym[k];
        P.symreg[start + k] = b & 0x3Fu;
        P.symswp[start + k] = (b & 0x80u) ? 0xFFFFFFFFu : 0u;
    }
}
__global__ void __launch_bounds__(32 * kScalarWarpFns) k_s_ra_warp(Prog P, unsigned long long* preserve,
                                                                   uint32_t stride) {
    extern __shared__ uint8_t s_wsym[];
    const uint32_t f = blockIdx.x * kScalarWarpFns + (threadIdx.x >> 5);
    if (f >= P.F) return;  // the whole warp
    s_ra_warp_function(P, f, preserve, stride, s_wsym + (threadIdx.x >> 5) * stride);
}
__device__ __forceinline__ uint32_t batch_program(const uint32_t* off, uint32_t B, uint32_t t);
// The same for the listed programs of a batch: a tile is kScalarWarpFns functions of one
// program (off: the per-program tile table over F), one warp each.
__global__ void __launch_bounds__(32 * kScalarWarpFns) k_batch_s_ra_warp(const Prog* progs, const uint32_t* off,
                                                                         uint32_t B, uint32_t total, uint32_t stride) {
    extern __shared__ uint8_t s_wsym[];
    for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
        const uint32_t p = batch_program(off, B, t);
        const Prog& P = progs[p];
        const uint32_t f = (t - off[p]) * kScalarWarpFns + (threadIdx.x >> 5);
        // each warp's symbol bytes are its own, reused only by its next function: the warps
        // of a block go on to their next tiles without waiting for one another
        if (f < P.F) s_ra_warp_function(P, f, P.s_preserve, stride, s_wsym + (threadIdx.x >> 5) * stride);
    }
}

__global__ void k_s_ra_serial(Prog P, int32_t* regs, SRaStep* steps, unsigned long long* preserve) {
    if (blockIdx.x == 0 && threadIdx.x == 0) s_ra_serial(P, regs, steps, preserve);
}
__global__ void k_s_preserve_counts(Prog P, const unsigned long long* preserve, uint32_t* extra) {
    PTL_FOR(f, P.F) st_s_preserve_counts(P, f, preserve, extra);
}
__global__ void k_s_ra_scatter(Prog P) { PTL_FOR(i, P.wb8) st_s_ra_scatter(P, i); }
__global__ void k_s_frame(Prog P, const unsigned long long* preserve, int mode, unsigned long long* claim) {
    PTL_FOR(t, 3ull * P.F) st_s_frame(P, t % P.F, t / P.F, preserve, mode, claim);
}
struct SRaCountLoad {
    Prog P;
    const uint32_t* extra;
    __device__ uint32_t operator()(uint32_t i) const { return st_s_ra_count(P, i, extra); }
};

}  // namespace

uint64_t launch_count() { return g_launches.load(); }
void note_launch() { g_launches++; }

// ====================================================================== launchers
void launch_ingest(const Prog& P, cudaStream_t s) {
    g_launches++;
    k_ingest<<<grid_for(P.nb8), kThreads, 0, s>>>(P);
}

void launch_preprocess(const Prog& P, cudaStream_t s) {
    g_launches++;
    k_pre_lists<<<grid_for(P.nb8), kThreads, 0, s>>>(P);
    g_launches++;
    k_pre_float<<<grid_for(P.nb8), kThreads, 0, s>>>(P);
    g_launches++;
    k_pre_float_apply<<<grid_for(P.nb8), kThreads, 0, s>>>(P);
}

void launch_count_scan(const Prog& P, const ScanScratch& sc, cudaStream_t s) {
    run_scan(CountLoad{P}, StoreTo{P.loc0}, P.nb8, sc, P.err, s);
}

void launch_fix(const Prog& P, cudaStream_t s) {
    g_launches++;
    k_fix_own<<<grid_for(P.nb8), kThreads, 0, s>>>(P);
    g_launches++;
    k_fix_cond<<<grid_for(P.nb8), kThreads, 0, s>>>(P);
}

void launch_decl_scan(const Prog& P, uint32_t* meta, const ScanScratch& sc, cudaStream_t s) {
    run_scan(DeclLoad{P}, DeclStore{P, meta, P.nb8}, P.nb8, sc, P.err, s);
}

void launch_functab(const Prog& P, uint32_t* meta, cudaStream_t s) {
    // F is known on the device only; launch for the node count's upper bound.
    const uint64_t bound = P.nb8 / 8u + 8u;
    g_launches++;
    k_functab<<<grid_for(bound), kThreads, 0, s>>>(P, meta);
    g_launches++;
    k_functab_end<<<grid_for(bound), kThreads, 0, s>>>(P, meta);
}

// Introsort rounds over the nseg0 segments in ss.seg[0] (leaves and heaps already
// recorded in the counters), then the heap and leaf passes.  The rounds run back to back on
// the device; the host checks for the end (no segments left) after a first batch of
// first_batch rounds and then every few rounds.  Rounds after the end find no segments and
// return at once.
namespace {
constexpr uint32_t kRoundLaunches = 7;  // kernels per partition round

void launch_sort_round(const SortScratch& ss, SortSeg* segs, SortSeg* next, ErrorWord* err, cudaStream_t s) {
    const unsigned seg_grid = static_cast<unsigned>(std::min<uint64_t>(ss.seg_cap, 152ull * 8));
    const unsigned tile_grid = static_cast<unsigned>(std::min<uint64_t>(ss.tile_cap, 152ull * 8));
    k_sort_round<<<1, 32, 0, s>>>(ss);
    k_sort_tiles<<<grid_for(ss.seg_cap), kThreads, 0, s>>>(ss, segs, segs);
    k_sort_count<<<tile_grid, kThreads, 0, s>>>(ss, segs);
    k_sort_segscan<<<seg_grid, kThreads, 0, s>>>(ss, segs);
    k_sort_pos<<<tile_grid, kThreads, 0, s>>>(ss, segs);
    k_sort_cut<<<grid_for(ss.seg_cap), kThreads, 0, s>>>(ss, segs, next, err);
    k_sort_swap<<<tile_grid, kThreads, 0, s>>>(ss, segs);
}

bool same_layout(const SortScratch& a, const SortScratch& b) {
    return a.a == b.a && a.apos == b.apos && a.bpos == b.bpos && a.seg[0] == b.seg[0] && a.seg[1] == b.seg[1] &&
           a.seg_cap == b.seg_cap && a.tile_seg == b.tile_seg && a.tile_l == b.tile_l && a.tile_r == b.tile_r &&
           a.stops == b.stops &&
           a.tile_cap == b.tile_cap && a.leaf == b.leaf && a.heap == b.heap && a.leaf_cap == b.leaf_cap &&
           a.local == b.local && a.equal == b.equal && a.counters == b.counters;
}

// The graph of two rounds for this layout (captured when it has none or another).
cudaError_t round_pair_graph(SortRoundGraph& g, const SortScratch& ss, ErrorWord* err, cudaStream_t s) {
    if (g.exec && g.err == err && same_layout(g.ss, ss)) return cudaSuccess;
    if (g.exec) {
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
    }
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    launch_sort_round(ss, ss.seg[0], ss.seg[1], err, s);
    launch_sort_round(ss, ss.seg[1], ss.seg[0], err, s);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(s, &graph);
    if (e != cudaSuccess) return e;
    e = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        g.exec = nullptr;
        return e;
    }
    g.ss = ss;
    g.err = err;
    return cudaSuccess;
}
}  // namespace

cudaError_t run_sort_rounds(const SortScratch& ss, uint32_t nseg0, uint32_t first_batch, uint32_t max_rounds,
                            ErrorWord* err, cudaStream_t s, uint32_t* rounds_out, SortRoundGraph* graph) {
    cudaMemcpyAsync(ss.counters + 1, &nseg0, sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    uint32_t rounds = 0, nseg = nseg0;
    int cur = 0;
    uint32_t batch = std::max<uint32_t>(first_batch, 1u);
    if (graph && nseg > 0) {
        const cudaError_t e = round_pair_graph(*graph, ss, err, s);
        if (e != cudaSuccess) return e;
        batch += batch & 1u;  // whole pairs; a round after the end finds no segments
    }
    while (nseg > 0) {
        if (graph) {
            for (uint32_t r = 0; r < batch; r += 2) {
                const cudaError_t e = cudaGraphLaunch(graph->exec, s);
                if (e != cudaSuccess) return e;
                g_launches += 2 * kRoundLaunches;
                rounds += 2;
            }
        } else {
            for (uint32_t r = 0; r < batch; ++r) {
                launch_sort_round(ss, ss.seg[cur], ss.seg[cur ^ 1], err, s);
                g_launches += kRoundLaunches;
                cur ^= 1;
                ++rounds;
            }
        }
        uint32_t c[6] = {0, 0, 0, 0, 0, 0};
        cudaMemcpyAsync(c, ss.counters, sizeof(c), cudaMemcpyDeviceToHost, s);
        const cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        if (c[5]) return cudaErrorMemoryAllocation;
        nseg = c[1];
        // every round shortens each segment and the depth budget ends partitioning
        // after 2*floor(log2 n) levels
        if (nseg > 0 && rounds > max_rounds) return cudaErrorLaunchFailure;
        batch = 4;
    }
    uint32_t lh[6] = {0, 0, 0, 0, 0, 0};  // leaves, heaps, -, overflow, block ranges, equal ranges
    cudaMemcpyAsync(lh, ss.counters + 2, sizeof(lh), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    if (lh[3] || lh[0] > ss.leaf_cap || lh[1] > ss.leaf_cap || lh[4] > ss.seg_cap || lh[5] > ss.seg_cap)
        return cudaErrorMemoryAllocation;
    if (lh[1]) { g_launches++; k_sort_heaps<<<grid_for(lh[1]), kThreads, 0, s>>>(ss, lh[1]); }
    if (lh[0]) { g_launches++; k_sort_leaves<<<grid_for(lh[0]), kThreads, 0, s>>>(ss, lh[0]); }
    if (lh[5]) {
        g_launches++;
        k_sort_equal<<<static_cast<unsigned>(std::min<uint32_t>(lh[5], 152u * 8u)), kThreads, 0, s>>>(ss, lh[5]);
    }
    if (lh[4]) {
        const size_t smem = sizeof(BlockSortSmem);
        e = allow_dynamic_smem(reinterpret_cast<const void*>(k_sort_block), smem);
        if (e != cudaSuccess) return e;
        g_launches++;
        k_sort_block<<<lh[4], kSortBlockThreads, smem, s>>>(ss, lh[4], err);
    }
    if (rounds_out) *rounds_out = rounds;
    return cudaGetLastError();
}

cudaError_t run_depth_sort(const Prog& P, const SortScratch& ss, cudaStream_t s, uint32_t* rounds_out,
                           SortRoundGraph* graph) {
    const uint32_t n = P.n;
    g_launches++;
    k_sort_init<<<grid_for(n), kThreads, 0, s>>>(P, ss);
    cudaMemsetAsync(ss.counters, 0, sizeof(uint32_t) * 8, s);
    uint32_t nseg = 0;
    if (n > kSortBlock) {
        SortSeg g{};
        g.first = 0;
        g.last = n;
        g.dl = 2u * floor_log2(n);
        cudaMemcpyAsync(ss.seg[0], &g, sizeof(g), cudaMemcpyHostToDevice, s);
        nseg = 1;
    } else if (n > kSortThreshold) {  // one block sorts it all
        static const uint32_t one = 1;
        const uint32_t range[3] = {0, n, 2u * floor_log2(n)};
        cudaMemcpyAsync(ss.local, range, sizeof(range), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(ss.counters + 6, &one, sizeof(one), cudaMemcpyHostToDevice, s);
    } else if (n > 1) {
        const uint32_t leaf[2] = {0, n};
        cudaMemcpyAsync(ss.leaf, leaf, sizeof(leaf), cudaMemcpyHostToDevice, s);
        const uint32_t one = 1;
        cudaMemcpyAsync(ss.counters + 2, &one, sizeof(one), cudaMemcpyHostToDevice, s);
    }
    const uint32_t lg = floor_log2(std::max<uint32_t>(n, 2u));
    const uint32_t lb = floor_log2(kSortBlock);
    const cudaError_t e = run_sort_rounds(ss, nseg, lg > lb ? lg - lb : 1u, 2u * lg + 4u, P.err, s, rounds_out, graph);
    if (e != cudaSuccess) return e;
    g_launches++;
    k_sort_out<<<grid_for(n), kThreads, 0, s>>>(P, ss);
    return cudaGetLastError();
}
void launch_gen(const Prog& P, cudaStream_t s) {
    g_launches++;
    k_gen_prop<<<grid_for(P.n), kThreads, 0, s>>>(P);
    g_launches++;
    k_gen_claim<<<grid_for(P.n), kThreads, 0, s>>>(P);
    g_launches++;
    k_gen_write<<<grid_for(P.n), kThreads, 0, s>>>(P);
}

cudaError_t run_optimize(const Prog& P, cudaStream_t s, uint32_t* sweeps_out) {
    g_launches++;
    k_opt_mark<<<grid_for(P.wb8), kThreads, 0, s>>>(P);
    uint32_t sweeps = 0;
    for (;;) {
        cudaMemsetAsync(P.flags, 0, sizeof(uint32_t), s);
        for (int k = 0; k < 4; ++k) {
            g_launches++;
            k_opt_sweep<<<grid_for(P.wb8), kThreads, 0, s>>>(P);
        }
        sweeps += 4;
        uint32_t changed = 0;
        cudaMemcpyAsync(&changed, P.flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        const cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        if (!changed) break;
        if (sweeps > P.W + 8u) break;  // cannot happen: every sweep clears a mark
    }
    g_launches++;
    k_opt_final<<<grid_for(P.wb8), kThreads, 0, s>>>(P);
    if (sweeps_out) *sweeps_out = sweeps;
    return cudaGetLastError();
}

// Shape of the register allocation launch: T threads (at least 64, one per physical
// register in the row-0 phases), Q lane-0 slots per thread, K symbol-cache entries per
// lane-0 function and Kf per independent function, within about 160 KB of shared memory.
template <int Q>
cudaError_t launch_ra_steps_q(const Prog& P0, const Prog& Pfree, uint32_t G0, uint32_t T, cudaStream_t s) {
    const uint32_t free_fns = P0.F - G0;
    constexpr size_t kBudget = 160u * 1024u;
    uint32_t K = 64;
    const size_t fixed = sizeof(Ra2Shared) + 16ull * G0;
    while (K > 1 && fixed + static_cast<size_t>(G0) * K * 8u > kBudget) K >>= 1;
    uint32_t Kf = 64;
    while (Kf > 1 && static_cast<size_t>(T) * Kf * 8u > kBudget) Kf >>= 1;
    const size_t smem = std::max(fixed + static_cast<size_t>(G0) * K * 8u, static_cast<size_t>(T) * Kf * 8u) + 16;
    cudaError_t ce = allow_dynamic_smem(reinterpret_cast<const void*>(k_ra_steps<Q>), smem);
    if (ce != cudaSuccess) return ce;
    uint32_t S = P0.S;
    // One launch when its blocks can all be resident: the independent functions run
    // beside the lane-0 block, which waits on their progress (so the launch must be
    // cooperative).  Otherwise the independent functions run first.
    bool fused = false;
    const uint32_t free_blocks = (free_fns + T - 1u) / T;
    if (free_fns > 0) {
        int dev = 0, coop = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ra_steps<Q>, static_cast<int>(T), smem);
        fused = coop != 0 && static_cast<long long>(per_sm) * sms >= 1ll + free_blocks;
    }
    if (fused) {
        uint32_t chunks = (S + kRaChunk - 1u) / kRaChunk;
        cudaMemsetAsync(P0.ra_chunks, 0, 2ull * chunks * sizeof(uint32_t), s);
        g_launches++;
        k_ra_chunk_hist<<<grid_for(free_fns), kThreads, 0, s>>>(P0, free_fns);
        Prog Pl = P0;
        void* args[] = {&Pl, &S, &K, &Kf, &chunks};
        g_launches++;
        return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_ra_steps<Q>), dim3(1 + free_blocks),
                                           dim3(T), args, smem, s);
    }
    if (free_fns) {
        g_launches++;
        k_ra_free_cached<<<(free_fns + kRaFreeThreads - 1) / kRaFreeThreads, kRaFreeThreads, 0, s>>>(Pfree);
    }
    g_launches++;
    k_ra_steps<Q><<<1, T, smem, s>>>(P0, S, K, Kf, 0u);
    return cudaGetLastError();
}

// The independent functions, then the lane-0 pass on a cluster of C CTAs
// (k_ra_lane0_cluster) -- when the device can place such a cluster; *launched tells
// (nothing is launched otherwise; with dry set, nothing is launched either way).
template <int Q>
cudaError_t launch_ra_cluster_q(const Prog& P0, const Prog& Pfree, uint32_t G0, cudaStream_t s, bool* launched,
                                bool dry = false) {
    *launched = false;
    const uint32_t C = std::min(kRaClusterMax, (G0 + kRaClusterThreads * Q - 1u) / (kRaClusterThreads * Q));
    const uint32_t per_cta = (G0 + C - 1u) / C;
    const uint32_t T = std::max(64u, ((per_cta + Q - 1u) / Q + 31u) & ~31u);
    constexpr size_t kBudget = 160u * 1024u;
    const size_t fixed = sizeof(Ra2Shared) + 2 * sizeof(Ra2Agg) + 32ull * per_cta;  // records per step parity
    uint32_t K = 64;
    while (K > 1 && fixed + static_cast<size_t>(per_cta) * K * 8u > kBudget) K >>= 1;
    const size_t smem = fixed + static_cast<size_t>(per_cta) * K * 8u + 16;
    const void* fn = reinterpret_cast<const void*>(k_ra_lane0_cluster<Q>);
    cudaError_t ce = allow_dynamic_smem(fn, smem);
    if (ce != cudaSuccess) return ce;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(T);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) != cudaSuccess || clusters < 1) {
        cudaGetLastError();  // not placeable here: the caller takes the one-block pass
        return cudaSuccess;
    }
    if (dry) {
        *launched = true;
        return cudaSuccess;
    }
    const uint32_t free_fns = P0.F - G0;
    if (free_fns) {
        g_launches++;
        k_ra_free_cached<<<(free_fns + kRaFreeThreads - 1) / kRaFreeThreads, kRaFreeThreads, 0, s>>>(Pfree);
    }
    g_launches++;
    ce = cudaLaunchKernelEx(&cfg, k_ra_lane0_cluster<Q>, P0, P0.S, K, per_cta);
    *launched = true;
    return ce;
}

// PTL_RA_ONE_BLOCK=1 in the environment keeps every lane-0 pass in one block (the pass a
// device that cannot place the cluster takes), so that both paths can be compared.
bool ra_cluster_disabled() {
    static const bool off = [] {
        const char* v = std::getenv("PTL_RA_ONE_BLOCK");
        return v && v[0] == '1';
    }();
    return off;
}

cudaError_t launch_ra_wide(const Prog& P0, const Prog& Pfree, uint32_t G0, cudaStream_t s, bool* launched) {
    *launched = false;
    if (G0 <= kRaClusterMin || G0 > 2u * kRaClusterThreads * kRaClusterMax || ra_cluster_disabled()) return cudaSuccess;
    return G0 <= kRaClusterThreads * kRaClusterMax ? launch_ra_cluster_q<1>(P0, Pfree, G0, s, launched)
                                                   : launch_ra_cluster_q<2>(P0, Pfree, G0, s, launched);
}

bool ra_cluster_fits(uint32_t G0) {
    if (G0 <= kRaClusterMin || G0 > 2u * kRaClusterThreads * kRaClusterMax || ra_cluster_disabled()) return false;
    Prog none{};
    bool fits = false;
    const cudaError_t ce = G0 <= kRaClusterThreads * kRaClusterMax
                               ? launch_ra_cluster_q<1>(none, none, G0, nullptr, &fits, true)
                               : launch_ra_cluster_q<2>(none, none, G0, nullptr, &fits, true);
    return ce == cudaSuccess && fits;
}

cudaError_t launch_ra_steps(const Prog& P0, const Prog& Pfree, uint32_t G0, cudaStream_t s) {
    bool launched = false;
    const cudaError_t ce = launch_ra_wide(P0, Pfree, G0, s, &launched);
    if (ce != cudaSuccess || launched) return ce;
    const uint32_t T = G0 <= 1024u ? std::max(32u, (G0 + 31u) & ~31u) : 1024u;
    const uint32_t Q = (G0 + T - 1u) / T;
    switch (Q) {
        case 1: return launch_ra_steps_q<1>(P0, Pfree, G0, T, s);
        case 2: return launch_ra_steps_q<2>(P0, Pfree, G0, T, s);
        case 3:
        case 4: return launch_ra_steps_q<4>(P0, Pfree, G0, T, s);
        default: return launch_ra_steps_q<8>(P0, Pfree, G0, T, s);
    }
}

cudaError_t run_regalloc_steps(const Prog& P, cudaStream_t s, bool* serial_out, bool row0_hash) {
    // Programs whose functions share symbols need the reference's serial order.
    cudaMemsetAsync(P.flags + 1, 0, 2 * sizeof(uint32_t), s);
    cudaMemsetAsync(P.stamp, 0, sizeof(uint32_t) * P.W, s);
    cudaMemsetAsync(P.defpos, 0, P.W, s);
    g_launches++;
    k_ra_cross<<<grid_for(P.W), kThreads, 0, s>>>(P);
    uint32_t fl[2] = {0, 0};
    cudaMemcpyAsync(fl, P.flags + 1, sizeof(fl), cudaMemcpyDeviceToHost, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    const uint32_t cross = fl[0];
    // independent functions never need the definition positions; the lane-0 pass hashes
    // row 0 when a virtual register has two definitions
    Prog Pfree = P, P0 = P;
    Pfree.defpos = nullptr;
    if (fl[1] || row0_hash) P0.defpos = nullptr;
    const uint32_t G0 = (P.F + 7u) / 8u;
    if (cross || G0 > 8192u) {
        // functions share symbols (or too many lane-0 functions for one CTA): serial path
        g_launches++;
        k_ra_serial<<<1, 1, 0, s>>>(P);
    } else {
        const cudaError_t ce = launch_ra_steps(P0, Pfree, G0, s);
        if (ce != cudaSuccess) return ce;
    }
    g_launches++;
    k_ra_spill<<<grid_for(P.W), kThreads, 0, s>>>(P);
    if (serial_out) *serial_out = cross != 0;
    return cudaGetLastError();
}

void launch_regalloc_count_scan(const Prog& P, const ScanScratch& sc, cudaStream_t s) {
    run_scan(RaCountLoad{P}, StoreTo{P.roffs}, P.wb8, sc, P.err, s);
}

void launch_regalloc_emit(const Prog& P, cudaStream_t s) {
    g_launches++;
    k_ra_scatter<<<grid_for(P.wb8), kThreads, 0, s>>>(P);
    g_launches++;
    k_ra_functab<<<grid_for(P.F), kThreads, 0, s>>>(P);
    g_launches++;
    k_ra_frame<<<grid_for(P.F), kThreads, 0, s>>>(P);
}

void launch_preprocess_scalar(const Prog& P, cudaStream_t s) {
    g_launches++;
    k_s_pre_lists<<<grid_for(P.nb8), kThreads, 0, s>>>(P);
    g_launches++;
    k_s_pre_float<<<grid_for(P.nb8), kThreads, 0, s>>>(P);
    g_launches++;
    k_pre_float_apply<<<grid_for(P.nb8), kThreads, 0, s>>>(P);
}

void launch_gen_scalar(const Prog& P, cudaStream_t s) {
    g_launches++;
    k_s_gen_prop<<<grid_for(P.n), kThreads, 0, s>>>(P);
    g_launches++;
    k_s_gen_claim<<<grid_for(P.n), kThreads, 0, s>>>(P);
    g_launches++;
    k_s_gen_write<<<grid_for(P.n), kThreads, 0, s>>>(P);
}

cudaError_t scalar_regalloc_cross(const Prog& P, cudaStream_t s, bool* cross) {
    cudaMemsetAsync(P.flags + 1, 0, 2 * sizeof(uint32_t), s);
    cudaMemsetAsync(P.stamp, 0, sizeof(uint32_t) * P.W, s);
    g_launches++;
    k_ra_cross<<<grid_for(P.W), kThreads, 0, s>>>(P);
    uint32_t fl = 0;
    cudaMemcpyAsync(&fl, P.flags + 1, sizeof(fl), cudaMemcpyDeviceToHost, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    *cross = fl != 0;
    return e;
}

void launch_scalar_ra_free(const Prog& P, unsigned long long* preserve, cudaStream_t s) {
    if (P.S <= kScalarWarpSymCap) {  // one warp per function
        const uint32_t stride = (std::max<uint32_t>(P.S, 1u) + 15u) & ~15u;
        const size_t bytes = static_cast<size_t>(stride) * kScalarWarpFns;
        if (allow_dynamic_smem(reinterpret_cast<const void*>(&k_s_ra_warp), bytes) == cudaSuccess) {
            g_launches++;
            k_s_ra_warp<<<(P.F + kScalarWarpFns - 1u) / kScalarWarpFns, 32u * kScalarWarpFns, bytes, s>>>(P, preserve,
                                                                                                     stride);
            return;
        }
    }
    // a tile's words: at most one tile plus the longest function
    const uint64_t want = (static_cast<uint64_t>(kScalarTileWords) + P.S + 15u) & ~uint64_t(15);
    const uint32_t cap = static_cast<uint32_t>(std::min<uint64_t>(want, 96u * 1024u));
    if (allow_dynamic_smem(reinterpret_cast<const void*>(&k_s_ra_tiles), cap) != cudaSuccess) {
        ErrorWord e{ST_UNSUPPORTED, W_RA1, 0, 0};
        cudaMemcpyAsync(P.err, &e, sizeof(e), cudaMemcpyHostToDevice, s);
        cudaStreamSynchronize(s);
        return;
    }
    const uint32_t tiles = P.W / kScalarTileWords + 1u;
    g_launches++;
    k_s_ra_tiles<<<tiles, kScalarRaThreads, cap, s>>>(P, preserve, cap);
}

void launch_scalar_ra_serial(const Prog& P, int32_t* regs, SRaStep* steps, unsigned long long* preserve,
                             cudaStream_t s) {
    g_launches++;
    k_s_ra_serial<<<1, 1, 0, s>>>(P, regs, steps, preserve);
}

void launch_scalar_ra_count_scan(const Prog& P, const unsigned long long* preserve, uint32_t* extra,
                                 const ScanScratch& sc, cudaStream_t s) {
    g_launches++;
    k_ra_spill<<<grid_for(P.W), kThreads, 0, s>>>(P);
    cudaMemsetAsync(extra, 0, sizeof(uint32_t) * P.wb8, s);
    g_launches++;
    k_s_preserve_counts<<<grid_for(P.F), kThreads, 0, s>>>(P, preserve, extra);
    run_scan(SRaCountLoad{P, extra}, StoreTo{P.roffs}, P.wb8, sc, P.err, s);
}

void launch_scalar_ra_emit(const Prog& P, const unsigned long long* preserve, unsigned long long* claim,
                           cudaStream_t s) {
    g_launches++;
    k_s_ra_scatter<<<grid_for(P.wb8), kThreads, 0, s>>>(P);
    g_launches++;
    k_ra_functab<<<grid_for(P.F), kThreads, 0, s>>>(P);
    cudaMemsetAsync(claim, 0, sizeof(unsigned long long) * P.W2, s);
    g_launches++;
    k_s_frame<<<grid_for(3ull * P.F), kThreads, 0, s>>>(P, preserve, 1, claim);
    g_launches++;
    k_s_frame<<<grid_for(3ull * P.F), kThreads, 0, s>>>(P, preserve, 2, claim);
}

void launch_fixjumps_scan(const Prog& P, const ScanScratch& sc, cudaStream_t s) {
    run_scan(FjSizeLoad{P}, StoreTo{P.joffs}, P.w2b8, sc, P.err, s);
}

void launch_fixjumps_emit(const Prog& P, cudaStream_t s) {
    g_launches++;
    k_fj_emit<<<grid_for(P.W2), kThreads, 0, s>>>(P);
    g_launches++;
    k_fj_functab<<<grid_for(P.F), kThreads, 0, s>>>(P);
}


// ====================================================================== batched programs
// Many programs per launch.  Each program keeps its own Prog view (device memory, one
// per program) into arenas laid out per program with the generator's zero pads, so the
// per-element stage functions run unchanged.  Work is cut into tiles that never straddle
// programs: off[p] is the first tile of program p (exclusive prefix over the programs;
// programs left out of a stage have no tiles).
namespace {

constexpr uint32_t kBTile = 1024;  // default; the tile is a launch parameter (BatchLaunch::tile)

__device__ __forceinline__ uint32_t batch_program(const uint32_t* off, uint32_t B, uint32_t t) {
    uint32_t lo = 0, hi = B;  // off[lo] <= t < off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= t) lo = mid; else hi = mid;
    }
    return lo;
}

template <class Op>
__global__ void __launch_bounds__(kThreads) k_batch(const Prog* progs, const uint32_t* off, uint32_t B, uint32_t total,
                                                    uint32_t tile, Op op) {
    Op o = op;  // per-thread copy: an op may carry state from element to element
    if constexpr (Op::kViewInShared) {
        // The tile's program view in shared memory: read from global memory, its
        // pointers would be reloaded after every store an op makes (the compiler cannot
        // rule out that the store hit the view).  Worth its copy and two barriers for the
        // ops with many fields per element (regalloc, isn_gen).
        __shared__ Prog sP;
        uint32_t have = 0xFFFFFFFFu;
        for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
            const uint32_t p = batch_program(off, B, t);
            if (p != have) {  // block-uniform
                __syncthreads();  // every thread is done with the previous view
                const uint64_t* src = reinterpret_cast<const uint64_t*>(&progs[p]);
                uint64_t* dst = reinterpret_cast<uint64_t*>(&sP);
                for (uint32_t k = threadIdx.x; k < sizeof(Prog) / 8; k += kThreads) dst[k] = src[k];
                __syncthreads();
                have = p;
            }
            const uint32_t cnt = Op::count(sP);
            const uint32_t base = (t - off[p]) * tile;
            for (uint32_t k = threadIdx.x; k < tile; k += kThreads) {
                const uint32_t i = base + k;
                if (i < cnt) o(sP, i, p);
            }
        }
    } else {
        for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
            const uint32_t p = batch_program(off, B, t);
            const Prog& P = progs[p];
            const uint32_t cnt = Op::count(P);
            const uint32_t base = (t - off[p]) * tile;
            for (uint32_t k = threadIdx.x; k < tile; k += kThreads) {
                const uint32_t i = base + k;
                if (i < cnt) o(P, i, p);
            }
        }
    }
}

#define PTL_BATCH_OP_V(NAME, SHARED, COUNT, BODY)                                               \
    struct NAME {                                                                              \
        static constexpr bool kViewInShared = SHARED;                                          \
        __device__ static uint32_t count(const Prog& P) { return COUNT; }                      \
        __device__ void operator()(const Prog& P, uint32_t i, uint32_t p) const { BODY; }      \
    };
#define PTL_BATCH_OP(NAME, COUNT, BODY) PTL_BATCH_OP_V(NAME, true, COUNT, BODY)

PTL_BATCH_OP_V(BIngest, false, P.nb8, if (st_ingest(P, i)) P.flags[3] = 1u)
PTL_BATCH_OP_V(BPreLists, false, P.nb8, st_pre_lists(P, i))
PTL_BATCH_OP_V(BPreFloat, false, P.nb8, st_pre_float(P, i))
PTL_BATCH_OP_V(BPreFloatApply, false, P.nb8, st_pre_float_apply(P, i))
PTL_BATCH_OP(BFixOwn, P.nb8, st_fix_own(P, i))
PTL_BATCH_OP(BFixCond, P.nb8, st_fix_cond(P, i))
PTL_BATCH_OP(BFunctab, P.fb8, st_functab(P, i))
PTL_BATCH_OP(BGenProp, P.n, st_gen_prop(P, i))
PTL_BATCH_OP(BGenClaim, P.n, st_gen_claim(P, i))
PTL_BATCH_OP(BGenWrite, P.n, st_gen_write(P, i))
// the scalar generator's stages where they differ (ptl_scalar.cuh)
PTL_BATCH_OP_V(BSPreLists, false, P.nb8, st_s_pre_lists(P, i))
PTL_BATCH_OP_V(BSPreFloat, false, P.nb8, st_s_pre_float(P, i))
PTL_BATCH_OP(BSGenProp, P.n, st_s_gen_prop(P, i))
PTL_BATCH_OP(BSGenClaim, P.n, st_s_gen_claim(P, i))
PTL_BATCH_OP(BSGenWrite, P.n, st_s_gen_write(P, i))
PTL_BATCH_OP(BSPreserveCounts, P.F, st_s_preserve_counts(P, i, P.s_preserve, P.s_extra))
PTL_BATCH_OP(BSRaScatter, P.wb8, st_s_ra_scatter(P, i))
struct BSFrame {
    static constexpr bool kViewInShared = true;
    int mode;
    __device__ static uint32_t count(const Prog& P) { return 3u * P.F; }
    __device__ void operator()(const Prog& P, uint32_t t, uint32_t) const {
        st_s_frame(P, t % P.F, t / P.F, P.s_preserve, mode, P.s_claim);
    }
};
// Pads of the families the stages write in full (ArenaGuard): guard element j of a
// program is j - kArenaFront before its first element, then written + (j - kArenaFront).
__device__ __forceinline__ int64_t guard_index(uint32_t j, uint32_t written) {
    return j < kArenaFront ? static_cast<int64_t>(j) - static_cast<int64_t>(kArenaFront)
                           : static_cast<int64_t>(written) + static_cast<int64_t>(j - kArenaFront);
}
struct BGuardNodes {
    static constexpr bool kViewInShared = false;
    __device__ static uint32_t count(const Prog& P) { return static_cast<uint32_t>(arena_region(P.nb8) - P.nb8); }
    __device__ void operator()(const Prog& P, uint32_t j, uint32_t) const {
        const int64_t x = guard_index(j, P.nb8);
        P.nt[x] = 0; P.rt[x] = 0; P.nd1[x] = 0; P.nd[x] = 0; P.par[x] = 0; P.ci[x] = 0; P.dep[x] = 0;
        P.loc0[x] = 0; P.loc[x] = 0; P.fflag[x] = 0;
    }
};
struct BGuardWords {
    static constexpr bool kViewInShared = false;
    __device__ static uint32_t count(const Prog& P) { return static_cast<uint32_t>(arena_region(P.wb8) - P.W); }
    __device__ void operator()(const Prog& P, uint32_t j, uint32_t) const {
        const int64_t x = guard_index(j, P.W);
        P.used_instrs[x] = 0; P.spill[x] = 0; P.roffs[x] = 0;
    }
};
struct BGuardWords2 {
    static constexpr bool kViewInShared = false;
    __device__ static uint32_t count(const Prog& P) {
        return static_cast<uint32_t>(arena_region(P.w2b8 + 16u) - P.w2b8);
    }
    __device__ void operator()(const Prog& P, uint32_t j, uint32_t) const { P.joffs[guard_index(j, P.w2b8)] = 0; }
};
// marks, and odd = 1 when some virtual result is not its instruction's own word (what
// the optimize sweeps' worklist needs to know)
struct BOptMark {
    static constexpr bool kViewInShared = true;
    uint32_t* odd;
    __device__ static uint32_t count(const Prog& P) { return P.wb8; }
    __device__ void operator()(const Prog& P, uint32_t i, uint32_t) const {
        st_opt_mark(P, i);
        const uint32_t r = P.rd[i];
        if (s32(r) > 63 && r - 64u != i) atomicOr(odd, 1u);
    }
};
PTL_BATCH_OP(BOptFinal, P.wb8, st_opt_final(P, i))
PTL_BATCH_OP(BInitLifetime, P.F, P.lifetime[i] = 0x1Full)
// spill flags and cross checks find each word's function from the thread's previous
// word (the same program, 256 words earlier within a tile)
struct BSpill {
    static constexpr bool kViewInShared = true;
    uint32_t hint = 0xFFFFFFFFu, hp = 0xFFFFFFFFu;
    __device__ static uint32_t count(const Prog& P) { return P.W; }
    __device__ void operator()(const Prog& P, uint32_t i, uint32_t p) {
        if (p != hp) { hp = p; hint = 0xFFFFFFFFu; }
        st_ra_spill(P, i, &hint);
    }
};
PTL_BATCH_OP(BScatter, P.wb8, st_ra_scatter(P, i))
PTL_BATCH_OP(BRaFunctab, P.F, st_fix_functab(P, i, P.roffs, P.W))
PTL_BATCH_OP(BRaFrame, P.F, st_ra_frame(P, i))
PTL_BATCH_OP_V(BFjEmit, false, P.W2, st_fj_emit(P, i))
PTL_BATCH_OP_V(BFjFunctab, false, P.F, st_fix_functab(P, i, P.joffs, P.W2))
// chunk histogram of a program's independent functions (see k_ra_chunk_hist)
PTL_BATCH_OP(BRaHist, P.F - (P.F + 7u) / 8u,
             const uint32_t f = free_function_of(i);
             const uint32_t size = P.fn_size0[f];
             if (s32(size) > 0) atomicAdd(&P.ra_chunks[(size - 1u) / kRaChunk], 1u))
struct BCross {
    static constexpr bool kViewInShared = true;
    uint32_t hint = 0xFFFFFFFFu, hp = 0xFFFFFFFFu;
    __device__ static uint32_t count(const Prog& P) { return P.W; }
    __device__ void operator()(const Prog& P, uint32_t i, uint32_t p) {
        if (p != hp) { hp = p; hint = 0xFFFFFFFFu; }
        const uint32_t r = st_ra_cross(P, i, P.stamp, &hint);
        if (r & 1u) atomicOr(&P.flags[1], 1u);
        if (r & 2u) atomicOr(&P.flags[2], 1u);
    }
};

// per program: word count and longest function (meta[4p + 1], meta[4p + 2])
struct BFunctabEnd {
    static constexpr bool kViewInShared = true;
    uint32_t* meta;
    __device__ static uint32_t count(const Prog& P) { return P.fb8; }
    __device__ void operator()(const Prog& P, uint32_t f, uint32_t p) const {
        st_functab_end(P, f);
        if (f < P.F) atomicMax(&meta[4u * p + 2u], P.fn_size[f]);
        if (f == 0) meta[4u * p + 1u] = P.loc[P.n - 1];
    }
};
// depth-order keys of all programs in one array, program p from aoff[p]
struct BSortInit {
    static constexpr bool kViewInShared = true;
    unsigned long long* a;
    const uint64_t* aoff;
    __device__ static uint32_t count(const Prog& P) { return P.n; }
    __device__ void operator()(const Prog& P, uint32_t i, uint32_t p) const {
        a[aoff[p] + i] = (static_cast<unsigned long long>(u32(P.dep[i])) << 32) | i;
    }
};
struct BSortOut {
    static constexpr bool kViewInShared = true;
    const unsigned long long* a;
    const uint64_t* aoff;
    __device__ static uint32_t count(const Prog& P) { return P.n; }
    __device__ void operator()(const Prog& P, uint32_t i, uint32_t p) const { P.pos[sidx(a[aoff[p] + i])] = i; }
};

// Optimize sweeps over the tiles marked in cur (all tiles when cur is null).  A block
// takes a tile's used marks into shared memory and sweeps the tile to its own fixed
// point (clearing only ever removes marks, so any fair order of the updates reaches the
// same fixed point); marks it clears in other tiles are cleared in global memory and
// queue those tiles in next.  When every virtual result is the instruction's own word
// (cur given), an instruction acts only on a mark of its own tile, so only such cross-tile
// clears make another sweep necessary; otherwise every tile is swept until a sweep
// changes nothing.  The block writes back zeros only, so clears by other blocks are
// never undone.
template <uint32_t TILE>
__global__ void __launch_bounds__(kThreads) k_batch_sweep(const Prog* progs, const uint32_t* off, uint32_t B,
                                                          uint32_t total, uint32_t* changed, const uint8_t* cur,
                                                          uint8_t* next) {
    constexpr uint32_t kSweepItems = TILE / kThreads;
    static_assert(kSweepItems >= 1 && kSweepItems <= 32, "pending bits");
    __shared__ uint8_t s_used[TILE];
    if (cur && !cur[total]) return;  // no tile was marked: nothing to sweep
    for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
        if (cur && !cur[t]) continue;  // block-uniform
        const uint32_t p = batch_program(off, B, t);
        const Prog& P = progs[p];
        const uint32_t base = (t - off[p]) * TILE;
        const uint32_t W = P.W, lim = min(TILE, P.wb8 - base);
        uint32_t rd[kSweepItems], r1[kSweepItems], r2[kSweepItems];
        uint32_t pending = 0;  // bit e: instruction e of this thread may still act
#pragma unroll
        for (uint32_t e = 0; e < kSweepItems; ++e) {
            const uint32_t k = threadIdx.x + e * kThreads;
            if (k < lim) {
                s_used[k] = P.used[base + k];
                rd[e] = P.rd[base + k];
                r1[e] = P.rs1[base + k];
                r2[e] = P.rs2[base + k];
                if (s32(rd[e]) > 63) pending |= 1u << e;
            }
        }
        __syncthreads();
        bool cross = false, local = false;
        for (;;) {
            bool ch = false;
#pragma unroll
            for (uint32_t e = 0; e < kSweepItems; ++e) {
                if (!((pending >> e) & 1u)) continue;
                const uint32_t r = rd[e] - 64u;
                if (r >= W) {
                    record_error(P.err, ST_UNSUPPORTED, W_OPT, base + threadIdx.x + e * kThreads);
                    pending &= ~(1u << e);
                    continue;
                }
                const bool live = r - base < lim ? s_used[r - base] != 0
                                                 : *reinterpret_cast<const volatile uint8_t*>(&P.used[r]) != 0;
                if (live) continue;
                pending &= ~(1u << e);  // dead: its operands lose their marks, once
#pragma unroll
                for (uint32_t o = 0; o < 2; ++o) {
                    const int32_t a = s32((o == 0 ? r1[e] : r2[e]) - 64u);
                    if (a < 0 || u32(a) >= W || P.smark[a]) continue;
                    if (u32(a) - base < lim) {
                        if (s_used[u32(a) - base]) { s_used[u32(a) - base] = 0; ch = true; }
                    } else if (*reinterpret_cast<volatile uint8_t*>(&P.used[a])) {
                        P.used[a] = 0;
                        next[off[p] + u32(a) / TILE] = 1;
                        next[total] = 1;  // some tile is marked
                        cross = true;
                    }
                }
            }
            local |= ch;
            if (!__syncthreads_or(ch)) break;
        }
#pragma unroll
        for (uint32_t e = 0; e < kSweepItems; ++e) {
            const uint32_t k = threadIdx.x + e * kThreads;
            if (k < lim && s_used[k] == 0) P.used[base + k] = 0;
        }
        if (__syncthreads_or(cross || (cur == nullptr && local)) && threadIdx.x == 0) *changed = 1u;
    }
}

// Input gather from host memory: a tile is kGatherTile elements of one program; 16-byte
// moves when the host array is 16-byte aligned (the device side always is), bytes
// otherwise.  Each thread has kGatherDepth reads in flight, so a grid of two blocks per
// SM covers the host link's latency and leaves the SMs to kernels of other streams (the
// compile server's lanes).
constexpr int kGatherDepth = 8;
__global__ void __launch_bounds__(kThreads) k_gather_host(HostGather g, const uint32_t* off, uint32_t B,
                                                          uint32_t total) {
    for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
        const uint32_t p = batch_program(off, B, t);
        const uint64_t e0 = static_cast<uint64_t>(t - off[p]) * kGatherTile;
        if (e0 >= g.n[p]) continue;
        const uint64_t nb = min(static_cast<uint64_t>(kGatherTile), g.n[p] - e0) * g.esize;
        const uint8_t* s = static_cast<const uint8_t*>(g.src[p]) + e0 * g.esize;
        uint8_t* d = g.dst + (g.din[p] + e0) * g.esize;
        uint64_t done = 0;
        if ((reinterpret_cast<uintptr_t>(s) & 15u) == 0) {
            const uint64_t n16 = nb / 16;
            const uint4* s16 = reinterpret_cast<const uint4*>(s);
            uint4* d16 = reinterpret_cast<uint4*>(d);
            for (uint64_t base = threadIdx.x; base < n16; base += static_cast<uint64_t>(kThreads) * kGatherDepth) {
                uint4 v[kGatherDepth];
#pragma unroll
                for (int u = 0; u < kGatherDepth; ++u) {
                    const uint64_t k = base + static_cast<uint64_t>(u) * kThreads;
                    if (k < n16) v[u] = s16[k];
                }
#pragma unroll
                for (int u = 0; u < kGatherDepth; ++u) {
                    const uint64_t k = base + static_cast<uint64_t>(u) * kThreads;
                    if (k < n16) d16[k] = v[u];
                }
            }
            done = n16 * 16;
        }
        for (uint64_t k = done + threadIdx.x; k < nb; k += kThreads) d[k] = s[k];
    }
}

// per-program sizes after the regalloc and fix_jumps scans
__global__ void k_batch_w2(const Prog* progs, const uint32_t* list, uint32_t count, uint32_t* meta) {
    PTL_FOR(k, count) {
        const Prog& P = progs[list[k]];
        meta[4u * list[k]] = P.roffs[P.W - 1u] + 1u;
    }
}
__global__ void k_batch_w3(const Prog* progs, const uint32_t* list, uint32_t count, uint32_t* meta) {
    PTL_FOR(k, count) {
        const Prog& P = progs[list[k]];
        meta[4u * list[k] + 1u] = st_fj_size(P, P.W2 - 1u) + P.joffs[P.W2 - 1u];
    }
}

// ---- batched scan: the decoupled look-back scan with tiles per program; a tile looks
// back only as far as its program's first tile.
struct BScanCount {
    static constexpr bool kBlocked = false;
    __device__ static uint32_t count(const Prog& P) { return P.nb8; }
    __device__ uint32_t load(const Prog& P, uint32_t i) const { return st_count(P, i); }
    __device__ void store(const Prog& P, uint32_t i, uint32_t v, uint32_t) const { P.loc0[i] = v; }
};
struct BScanDecl {
    static constexpr bool kBlocked = false;
    uint32_t* meta;
    __device__ static uint32_t count(const Prog& P) { return P.nb8; }
    __device__ uint32_t load(const Prog& P, uint32_t i) const { return P.nt[i] == RV_FUNC_DECL ? 1u : 0u; }
    __device__ void store(const Prog& P, uint32_t i, uint32_t v, uint32_t p) const {
        const bool is_decl = P.nt[i] == RV_FUNC_DECL;
        if (is_decl) P.decl[v] = i;
        if (i == P.nb8 - 1u) meta[4u * p] = v + (is_decl ? 1u : 0u);
    }
};
struct BScanRaCount {
    static constexpr bool kBlocked = true;
    __device__ static uint32_t count(const Prog& P) { return P.wb8; }
    __device__ uint32_t load(const Prog& P, uint32_t i) const { return st_ra_count(P, i); }
    __device__ void store(const Prog& P, uint32_t i, uint32_t v, uint32_t) const { P.roffs[i] = v; }
};
struct BScanSRaCount {
    static constexpr bool kBlocked = true;
    __device__ static uint32_t count(const Prog& P) { return P.wb8; }
    __device__ uint32_t load(const Prog& P, uint32_t i) const { return st_s_ra_count(P, i, P.s_extra); }
    __device__ void store(const Prog& P, uint32_t i, uint32_t v, uint32_t) const { P.roffs[i] = v; }
};
struct BScanFjSize {
    static constexpr bool kBlocked = true;
    __device__ static uint32_t count(const Prog& P) { return P.w2b8; }
    __device__ uint32_t load(const Prog& P, uint32_t i) const { return i < P.W2 ? st_fj_size(P, i) : 0u; }
    __device__ void store(const Prog& P, uint32_t i, uint32_t v, uint32_t) const { P.joffs[i] = v; }
};

template <class Op>
__global__ void __launch_bounds__(kScanThreads) k_bscan(const Prog* progs, const uint32_t* off, uint32_t B, Op op,
                                                        ScanScratch sc) {
    constexpr int kWarps = kScanThreads / 32;
    __shared__ uint32_t s_tile, s_prefix;
    __shared__ uint32_t s_warp[kWarps];
    __shared__ Prog sP;  // the program view, out of reach of the ops' stores (as in k_batch)
    if (threadIdx.x == 0) s_tile = atomicAdd(sc.counter, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t p = batch_program(off, B, tile);
    {
        const uint64_t* src = reinterpret_cast<const uint64_t*>(&progs[p]);
        uint64_t* dst = reinterpret_cast<uint64_t*>(&sP);
        for (uint32_t k = threadIdx.x; k < sizeof(Prog) / 8; k += kScanThreads) dst[k] = src[k];
    }
    __syncthreads();
    const Prog& P = sP;
    const uint32_t first = off[p];  // the program's first tile
    const uint32_t count = Op::count(P);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint64_t wbase = static_cast<uint64_t>(tile - first) * kScanTile + static_cast<uint64_t>(warp) * 32u * kScanItems;
    // Element k of a lane: striped (k*32 + lane: each load instruction coalesced) or
    // blocked (lane*kScanItems + k: a thread sums its run, then one warp scan instead of
    // one per element).  Measured: blocked is faster for the regalloc count and jump-size
    // scans over words, slower for the node count scan, whose loads of a node's
    // neighbour and parent fields then spread over more sectors per instruction.
    auto elem = [&](int k) -> uint64_t {
        return Op::kBlocked ? wbase + static_cast<uint64_t>(lane) * kScanItems + static_cast<uint64_t>(k)
                            : wbase + static_cast<uint64_t>(k) * 32u + lane;
    };
    uint32_t v[kScanItems];
    uint32_t carry = 0;
    if constexpr (Op::kBlocked) {
        uint32_t run = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            const uint64_t idx = elem(k);
            const uint32_t x = idx < count ? op.load(P, static_cast<uint32_t>(idx)) : 0u;
            v[k] = run;
            run += x;
        }
        const uint32_t incl = warp_incl_scan(run);
        carry = __shfl_sync(0xFFFFFFFFu, incl, 31);
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) v[k] += incl - run;
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            const uint64_t idx = elem(k);
            const uint32_t x = idx < count ? op.load(P, static_cast<uint32_t>(idx)) : 0u;
            const uint32_t incl = warp_incl_scan(x);
            v[k] = carry + incl - x;
            carry += __shfl_sync(0xFFFFFFFFu, incl, 31);
        }
    }
    if (lane == 0) s_warp[warp] = carry;
    __syncthreads();
    if (warp == 0) {
        const uint32_t t = lane < kWarps ? s_warp[lane] : 0u;
        const uint32_t incl = warp_incl_scan(t);
        if (lane < kWarps) s_warp[lane] = incl - t;
        const uint32_t aggregate = __shfl_sync(0xFFFFFFFFu, incl, kWarps - 1);
        uint32_t prefix = 0;
        if (tile == first) {
            if (lane == 0) atomicExch(&sc.status[tile], (2ull << 32) | aggregate);
        } else {
            if (lane == 0) atomicExch(&sc.status[tile], (1ull << 32) | aggregate);
            prefix = warp_lookback(sc.status, tile, first, P.err);
            if (lane == 0) atomicExch(&sc.status[tile], (2ull << 32) | (prefix + aggregate));
        }
        if (lane == 0) s_prefix = prefix;
    }
    __syncthreads();
    const uint32_t base = s_prefix + s_warp[warp];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const uint64_t idx = elem(k);
        if (idx < count) op.store(P, static_cast<uint32_t>(idx), base + v[k], p);
    }
}

// ---- batched register allocation
__global__ void k_batch_serial(const Prog* progs, const uint32_t* list, uint32_t count) {
    PTL_FOR(k, count) {
        const Prog& P = progs[list[k]];
        st_ra_serial(P, P.stamp);
    }
}

// Register allocation of every listed program in one persistent launch.  Blocks take
// work items in order from a queue; program order[k] owns items item_off[k] ..
// item_off[k+1]: first the tiles of its independent functions (T per tile), then its
// lane-0 pass.  The independent functions count the finished 32-step chunks of trigger
// records in the program's ra_chunks record, and the lane-0 pass waits for each chunk
// before it reads it, as the fused single-program launch does.  Every tile of a program
// is handed out before its lane-0 item, to blocks that are running and never wait, so
// the waits end; they are bounded all the same (DEVICE_TIMEOUT after about a second).
struct BatchRa {
    const Prog* progs;
    const uint32_t* item_off;   // [n+1]
    const uint32_t* order;      // [n] programs, longest first
    uint32_t n, items;
    uint32_t* queue;
    uint32_t K, Kf;
};

template <int Q, int MAXT>
__global__ void __launch_bounds__(MAXT) k_batch_ra(BatchRa ra) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t s_item;
    __shared__ Prog sP;
    const uint32_t tid = threadIdx.x, T = blockDim.x;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(ra.queue, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= ra.items) break;
        const uint32_t pos = batch_program(ra.item_off, ra.n, item);
        const uint32_t p = ra.order[pos];
        const uint32_t local = item - ra.item_off[pos];
        const uint32_t free_tiles = ra.item_off[pos + 1] - ra.item_off[pos] - 1u;
        if (local < free_tiles) {
            Prog Pf = ra.progs[p];
            Pf.defpos = nullptr;  // the independent functions never need definition positions
            uint32_t* tag = reinterpret_cast<uint32_t*>(smem);
            const SymCache cf{tag, tag + T * ra.Kf, ra.Kf};
            const uint32_t x = local * T + tid;
            const uint32_t nfree = Pf.F - (Pf.F + 7u) / 8u;
            const uint32_t f = x < nfree ? (Pf.ra_order ? Pf.ra_order[x] : free_function_of(x)) : Pf.F;
            const uint32_t chunks = (Pf.S + kRaChunk - 1u) / kRaChunk;
            if (f < Pf.F) ra_free_function_cached(Pf, cf, tid, f, Pf.ra_chunks + chunks);
        } else {
            const uint64_t* src = reinterpret_cast<const uint64_t*>(&ra.progs[p]);
            uint64_t* dst = reinterpret_cast<uint64_t*>(&sP);
            for (uint32_t k = tid; k < sizeof(Prog) / 8; k += T) dst[k] = src[k];
            __syncthreads();
            ra_lane0_block<Q>(sP, sP.S, ra.K, (sP.S + kRaChunk - 1u) / kRaChunk, smem);
        }
        __syncthreads();  // before the next item reuses shared memory and s_item
    }
}

template <class Op>
void batch_launch(const BatchLaunch& bl, uint32_t total, const Op& op) {
    if (total == 0) return;
    g_launches++;
    k_batch<Op><<<std::min<uint32_t>(total, 152u * 16u), kThreads, 0, bl.s>>>(bl.progs, bl.off, bl.B, total, bl.tile,
                                                                               op);
}

}  // namespace

static_assert(sizeof(Prog) % 8 == 0, "Prog copies in 8-byte words");

uint32_t batch_tile() { return kBTile; }
uint32_t batch_scan_tile() { return kScanTile; }

void batch_guards(ArenaGuard g, const BatchLaunch& bl, uint32_t total) {
    switch (g) {
        case ArenaGuard::Nodes: batch_launch(bl, total, BGuardNodes{}); break;
        case ArenaGuard::Words: batch_launch(bl, total, BGuardWords{}); break;
        case ArenaGuard::Words2: batch_launch(bl, total, BGuardWords2{}); break;
    }
}

void batch_stage(BatchStage st, const BatchLaunch& bl, uint32_t total, uint32_t* meta) {
    switch (st) {
        case BatchStage::Ingest: batch_launch(bl, total, BIngest{}); break;
        case BatchStage::Preprocess:
            batch_launch(bl, total, BPreLists{});
            batch_launch(bl, total, BPreFloat{});
            batch_launch(bl, total, BPreFloatApply{});
            break;
        case BatchStage::Fix:
            batch_launch(bl, total, BFixOwn{});
            batch_launch(bl, total, BFixCond{});
            break;
        case BatchStage::Functab:
            batch_launch(bl, total, BFunctab{});
            batch_launch(bl, total, BFunctabEnd{meta});
            break;
        case BatchStage::Gen:
            batch_launch(bl, total, BGenProp{});
            batch_launch(bl, total, BGenClaim{});
            batch_launch(bl, total, BGenWrite{});
            break;
        case BatchStage::PreprocessScalar:
            batch_launch(bl, total, BSPreLists{});
            batch_launch(bl, total, BSPreFloat{});
            batch_launch(bl, total, BPreFloatApply{});
            break;
        case BatchStage::GenScalar:
            batch_launch(bl, total, BSGenProp{});
            batch_launch(bl, total, BSGenClaim{});
            batch_launch(bl, total, BSGenWrite{});
            break;
        case BatchStage::SPreserveCounts: batch_launch(bl, total, BSPreserveCounts{}); break;
        case BatchStage::SScatter: batch_launch(bl, total, BSRaScatter{}); break;
        case BatchStage::SFunctab: batch_launch(bl, total, BRaFunctab{}); break;
        case BatchStage::SFrames:  // the frame words, then the preserve stores and loads over them
            batch_launch(bl, total, BSFrame{1});
            batch_launch(bl, total, BSFrame{2});
            break;
        case BatchStage::OptMark: batch_launch(bl, total, BOptMark{meta}); break;  // meta: the odd flag
        case BatchStage::OptFinal: batch_launch(bl, total, BOptFinal{}); break;
        case BatchStage::InitLifetime: batch_launch(bl, total, BInitLifetime{}); break;
        case BatchStage::Cross: batch_launch(bl, total, BCross{}); break;
        case BatchStage::RaHist: batch_launch(bl, total, BRaHist{}); break;
        case BatchStage::Spill: batch_launch(bl, total, BSpill{}); break;
        case BatchStage::Scatter: batch_launch(bl, total, BScatter{}); break;
        case BatchStage::RaFunctab:
            batch_launch(bl, total, BRaFunctab{});
            batch_launch(bl, total, BRaFrame{});
            break;
        case BatchStage::FjEmit: batch_launch(bl, total, BFjEmit{}); break;
        case BatchStage::FjFunctab: batch_launch(bl, total, BFjFunctab{}); break;
    }
}

void batch_scalar_ra_warp(const BatchLaunch& bl, uint32_t total, uint32_t stride) {
    if (total == 0) return;
    const size_t bytes = static_cast<size_t>(stride) * kScalarWarpFns;
    if (allow_dynamic_smem(reinterpret_cast<const void*>(&k_batch_s_ra_warp), bytes) != cudaSuccess) return;
    g_launches++;
    const uint32_t grid = std::min<uint32_t>(total, 152u * 16u);
    k_batch_s_ra_warp<<<grid, 32u * kScalarWarpFns, bytes, bl.s>>>(bl.progs, bl.off, bl.B, total, stride);
}
uint32_t scalar_warp_fns() { return kScalarWarpFns; }
uint32_t scalar_warp_cap() { return kScalarWarpSymCap; }

void batch_sort_keys(const BatchLaunch& bl, uint32_t total, unsigned long long* a, const uint64_t* aoff, bool out) {
    if (out) batch_launch(bl, total, BSortOut{a, aoff});
    else batch_launch(bl, total, BSortInit{a, aoff});
}

// Plain 16-byte copy from host memory the device reads directly (the probe of the host
// input path, below).
__global__ void __launch_bounds__(kThreads) k_read_host(const uint4* src, uint4* dst, uint64_t n) {
    for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        dst[i] = src[i];
}

cudaError_t read_host(const void* src, void* dst, size_t bytes, cudaStream_t s) {
    g_launches++;
    k_read_host<<<152u * 2u, kThreads, 0, s>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst), bytes / 16u);
    return cudaGetLastError();
}

// A copy by kernel loads and stores (kernel_copy): 16-byte elements, four in flight per
// thread, the last bytes one at a time.
__global__ void __launch_bounds__(kThreads) k_copy16(const uint4* src, uint4* dst, uint64_t n16,
                                                         const uint8_t* tsrc, uint8_t* tdst, uint32_t tail) {
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n16; i += 4 * stride) {
        const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n16; i += stride) dst[i] = src[i];
    if (blockIdx.x == 0 && threadIdx.x < tail) tdst[threadIdx.x] = tsrc[threadIdx.x];
}

cudaError_t kernel_copy(const void* src, void* dst, size_t bytes, cudaStream_t s) {
    if (bytes == 0) return cudaSuccess;
    const uint64_t n16 = bytes / 16u;
    const uint32_t tail = static_cast<uint32_t>(bytes - n16 * 16u);
    g_launches++;
    k_copy16<<<152u * 4u, kThreads, 0, s>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst), n16,
                                                static_cast<const uint8_t*>(src) + n16 * 16u,
                                                static_cast<uint8_t*>(dst) + n16 * 16u, tail);
    return cudaGetLastError();
}

void batch_gather_host(const BatchLaunch& bl, uint32_t total, const HostGather& g) {
    if (total == 0) return;
    g_launches++;
    k_gather_host<<<std::min<uint32_t>(total, 152u * 2u), kThreads, 0, bl.s>>>(g, bl.off, bl.B, total);
}

bool batch_tile_ok(uint32_t tile) { return tile >= kThreads && tile <= 65536u && (tile & (tile - 1)) == 0; }
bool batch_sweep_tile_ok(uint32_t tile) { return tile == 512u || tile == 1024u || tile == 2048u; }

void batch_sweep(const BatchLaunch& bl, uint32_t total, uint32_t* changed, const uint8_t* cur, uint8_t* next) {
    if (total == 0) return;
    g_launches++;
    const unsigned grid = std::min<uint32_t>(total, 152u * 16u);
    switch (bl.tile) {
        case 512u: k_batch_sweep<512u><<<grid, kThreads, 0, bl.s>>>(bl.progs, bl.off, bl.B, total, changed, cur, next); break;
        case 2048u: k_batch_sweep<2048u><<<grid, kThreads, 0, bl.s>>>(bl.progs, bl.off, bl.B, total, changed, cur, next); break;
        default: k_batch_sweep<1024u><<<grid, kThreads, 0, bl.s>>>(bl.progs, bl.off, bl.B, total, changed, cur, next); break;
    }
}

void batch_scan(BatchScan which, const BatchLaunch& bl, uint32_t tiles, const ScanScratch& sc, uint32_t* meta) {
    if (tiles == 0) return;
    cudaMemsetAsync(sc.status, 0, sizeof(unsigned long long) * tiles, bl.s);
    cudaMemsetAsync(sc.counter, 0, sizeof(uint32_t), bl.s);
    g_launches++;
    switch (which) {
        case BatchScan::Count: k_bscan<<<tiles, kScanThreads, 0, bl.s>>>(bl.progs, bl.off, bl.B, BScanCount{}, sc); break;
        case BatchScan::Decl: k_bscan<<<tiles, kScanThreads, 0, bl.s>>>(bl.progs, bl.off, bl.B, BScanDecl{meta}, sc); break;
        case BatchScan::RaCount: k_bscan<<<tiles, kScanThreads, 0, bl.s>>>(bl.progs, bl.off, bl.B, BScanRaCount{}, sc); break;
        case BatchScan::SRaCount: k_bscan<<<tiles, kScanThreads, 0, bl.s>>>(bl.progs, bl.off, bl.B, BScanSRaCount{}, sc); break;
        case BatchScan::FjSize: k_bscan<<<tiles, kScanThreads, 0, bl.s>>>(bl.progs, bl.off, bl.B, BScanFjSize{}, sc); break;
    }
}

void batch_free_order(const Prog* progs, const uint32_t* list, uint32_t count, cudaStream_t s) {
    if (count == 0) return;
    g_launches++;
    k_free_order<<<std::min<uint32_t>(count, 152u * 8u), kOrderThreads, 0, s>>>(progs, list, count);
}

void batch_sizes(bool w3, const Prog* progs, const uint32_t* list, uint32_t count, uint32_t* meta, cudaStream_t s) {
    if (count == 0) return;
    g_launches++;
    if (w3) k_batch_w3<<<grid_for(count), kThreads, 0, s>>>(progs, list, count, meta);
    else k_batch_w2<<<grid_for(count), kThreads, 0, s>>>(progs, list, count, meta);
}

cudaError_t batch_regalloc(const Prog* progs, const uint32_t* item_off, const uint32_t* order, uint32_t n,
                           uint32_t items, uint32_t max_g0, uint32_t* queue, cudaStream_t s, double share) {
    if (items == 0) return cudaSuccess;
    const uint32_t T = batch_ra_threads(max_g0);
    const uint32_t Q = (max_g0 + T - 1u) / T;
    constexpr size_t kBudget = 160u * 1024u;
    // Many programs share each SM here, so the symbol caches are kept small (16 entries)
    // for occupancy; the single-program launch gives one program all it can use.
    uint32_t K = 16;
    const size_t fixed = sizeof(Ra2Shared) + 16ull * max_g0;
    while (K > 1 && fixed + static_cast<size_t>(max_g0) * K * 8u > kBudget) K >>= 1;
    uint32_t Kf = 16;
    while (Kf > 1 && static_cast<size_t>(T) * Kf * 8u > kBudget) Kf >>= 1;
    const size_t smem = std::max(fixed + static_cast<size_t>(max_g0) * K * 8u, static_cast<size_t>(T) * Kf * 8u) + 16;
    BatchRa ra{progs, item_off, order, n, items, queue, K, Kf};
    auto go = [&](auto kernel) -> cudaError_t {
        cudaError_t ce = allow_dynamic_smem(reinterpret_cast<const void*>(kernel), smem);
        if (ce != cudaSuccess) return ce;
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, static_cast<int>(T), smem);
        const uint64_t resident = static_cast<uint64_t>(std::max(per_sm, 1)) * sms;
        const uint64_t allowed = std::max<uint64_t>(1, static_cast<uint64_t>(static_cast<double>(resident) * share));
        const unsigned grid = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>(items, allowed)));
        cudaMemsetAsync(queue, 0, sizeof(uint32_t), s);
        g_launches++;
        kernel<<<grid, T, smem, s>>>(ra);
        return cudaGetLastError();
    };
    if (T <= 256u) return go(k_batch_ra<1, 256>);  // one slot per thread, registers to spare
    switch (Q) {
        case 1: return go(k_batch_ra<1, 1024>);
        case 2: return go(k_batch_ra<2, 1024>);
        case 3:
        case 4: return go(k_batch_ra<4, 1024>);
        default: return go(k_batch_ra<8, 1024>);
    }
}

uint32_t batch_ra_threads(uint32_t max_g0) {
    return max_g0 <= 1024u ? std::max(32u, (max_g0 + 31u) & ~31u) : 1024u;
}

void batch_serial(const Prog* progs, const uint32_t* list, uint32_t count, cudaStream_t s) {
    if (count == 0) return;
    g_launches++;
    k_batch_serial<<<grid_for(count), kThreads, 0, s>>>(progs, list, count);
}

}  // namespace ptl
