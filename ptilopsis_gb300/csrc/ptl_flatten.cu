// AST flattening on the GPU (ptl_flatten in include/ptl_codegen.h).
//
// Replaces DepthTree::DepthTree(ASTNode*) (pareas-ast/src/codegen/depthtree.cpp:11-100):
// a depth-first walk of the parser's pointer tree that emits each node after its
// children (children in order), with its depth, its child index (SIZE_MAX, -1 as int32,
// for the root) and its parent rewritten to the emitted index.  A pointer tree does not
// cross to a GPU, so the input here is the same tree as arrays in any node order -- what a
// parser that builds nodes in parallel produces: node v's parent is parent[v] (-1 for the
// root) and its place among the parent's children is child_idx[v].
//
// The walk becomes an Euler tour and a list ranking:
//   1. children per node (counts, an exclusive scan, each child in its slot
//      off[parent] + child_idx: a child index out of range or taken twice is an error);
//   2. the tour: events enter(v) = 2v and exit(v) = 2v+1, plus an end event 2n.  enter(v)
//      goes to enter(first child) or exit(v); exit(v) to enter(next sibling), exit(parent)
//      or, for the root, the end;
//   3. pointer jumping, ceil(log2(2n+1)) rounds: each event sums two weights over the rest
//      of the tour -- 1 per exit (post-order: v's index is n minus the exits from exit(v)
//      on) and +1 per enter / -1 per exit (depth: minus the sum from enter(v) on);
//   4. the scatter of the six arrays to post-order.
// The root's enter must see all n exits; fewer means nodes the root does not reach (a
// cycle of parents), an INVALID_AST.  No kernel waits on another block.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/ptl_codegen.h"
#include "ptl_device.h"

namespace {

constexpr int kThreads = 256;
constexpr uint32_t kEmpty = 0xFFFFFFFFu;
constexpr int kScanThreads = 1024;
constexpr uint32_t kScanTile = 4096;  // elements per scan tile (4 per thread)

struct Event {
    uint32_t succ;  // next event of the tour (2n: the end)
    uint32_t exits; // exits from here to the end
    int32_t level;  // enters minus exits from here to the end
    uint32_t pad;
};

struct FlatErr {
    uint32_t code;     // 0 ok, 1 invalid
    uint32_t detail;   // the first node found bad
    uint32_t roots;    // nodes with parent -1
    uint32_t root;     // one of them
    uint32_t max_depth;
    uint32_t reached;  // exits the root's enter sees
};

__device__ void flag(FlatErr* e, uint32_t v) {
    if (atomicCAS(&e->code, 0u, 1u) == 0u) e->detail = v;
}

#define FL_FOR(i, count)                                                                  \
    for (uint64_t i##_ = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;    \
         i##_ < (count); i##_ += static_cast<uint64_t>(gridDim.x) * blockDim.x)           \
        if (const uint32_t i = static_cast<uint32_t>(i##_); true)

unsigned grid_of(uint64_t n) {
    return static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>((n + kThreads - 1) / kThreads, 152u * 16u)));
}

// children per node; the root
__global__ void k_fl_count(const int32_t* parent, const int32_t* child, uint32_t n, uint32_t* deg, FlatErr* e) {
    FL_FOR(v, n) {
        const int32_t p = parent[v];
        if (p == -1) {
            atomicAdd(&e->roots, 1u);
            e->root = v;
        } else if (p < 0 || static_cast<uint32_t>(p) >= n || child[v] < 0) {
            flag(e, v);
        } else {
            atomicAdd(&deg[p], 1u);
        }
    }
}

// exclusive scan of deg into off[0..n] (three passes: tile sums, their scan, the tiles)
__device__ uint32_t block_excl(uint32_t x, uint32_t* total) {
    __shared__ uint32_t warp_sum[kScanThreads / 32];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    uint32_t incl = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= static_cast<uint32_t>(d)) incl += y;
    }
    if (lane == 31) warp_sum[w] = incl;
    __syncthreads();
    if (w == 0) {
        const uint32_t t = lane < kScanThreads / 32 ? warp_sum[lane] : 0u;
        uint32_t s = t;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, d);
            if (lane >= static_cast<uint32_t>(d)) s += y;
        }
        if (lane < kScanThreads / 32) warp_sum[lane] = s - t;
        if (lane == 31) *total = s;
    }
    __syncthreads();
    const uint32_t r = warp_sum[w] + incl - x;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) k_fl_tile_sums(const uint32_t* deg, uint32_t n, uint32_t* tsum) {
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kScanTile;
    uint32_t s = 0;
    for (uint32_t k = threadIdx.x; k < kScanTile; k += kScanThreads)
        if (base + k < n) s += deg[base + k];
    __shared__ uint32_t total;
    block_excl(s, &total);
    if (threadIdx.x == 0) tsum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_fl_scan_sums(uint32_t* tsum, uint32_t tiles) {
    __shared__ uint32_t total;
    uint32_t carry = 0;
    for (uint32_t b = 0; b < tiles; b += kScanThreads) {
        const uint32_t k = b + threadIdx.x;
        const uint32_t x = k < tiles ? tsum[k] : 0u;
        const uint32_t ex = block_excl(x, &total);
        if (k < tiles) tsum[k] = carry + ex;
        carry += total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanThreads) k_fl_tiles(const uint32_t* deg, uint32_t n, const uint32_t* tsum,
                                                           uint32_t* off) {
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kScanTile;
    constexpr uint32_t kItems = kScanTile / kScanThreads;
    uint32_t v[kItems], s = 0;
#pragma unroll
    for (uint32_t j = 0; j < kItems; ++j) {  // thread t takes elements t*kItems .. +kItems-1
        const uint64_t i = base + threadIdx.x * kItems + j;
        v[j] = i < n ? deg[i] : 0u;
        s += v[j];
    }
    __shared__ uint32_t total;
    uint32_t run = tsum[blockIdx.x] + block_excl(s, &total);
#pragma unroll
    for (uint32_t j = 0; j < kItems; ++j) {
        const uint64_t i = base + threadIdx.x * kItems + j;
        if (i <= n) off[i] = run;  // off[n]: the total
        run += v[j];
    }
}

// each child into its slot
__global__ void k_fl_place(const int32_t* parent, const int32_t* child, uint32_t n, const uint32_t* deg,
                           const uint32_t* off, uint32_t* kids, FlatErr* e) {
    FL_FOR(v, n) {
        const int32_t p = parent[v];
        if (p < 0 || static_cast<uint32_t>(p) >= n || child[v] < 0) continue;  // the root, or flagged
        const uint32_t c = static_cast<uint32_t>(child[v]);
        if (c >= deg[p] || atomicCAS(&kids[off[p] + c], kEmpty, v) != kEmpty) flag(e, v);
    }
}

// the tour's events; an unfilled slot (flagged input) ends the tour there
__global__ void k_fl_tour(const int32_t* parent, const int32_t* child, uint32_t n, const uint32_t* deg,
                          const uint32_t* off, const uint32_t* kids, Event* ev) {
    const uint32_t end = 2u * n;
    FL_FOR(v, n) {
        uint32_t s = 2u * v + 1u;  // enter(v) -> exit(v) for a leaf
        if (deg[v] > 0) {
            const uint32_t c = kids[off[v]];
            s = c < n ? 2u * c : end;
        }
        ev[2u * v] = Event{s, 0u, 1, 0u};
        const int32_t p = parent[v];
        uint32_t x = end;  // exit(root) -> the end
        if (p >= 0 && static_cast<uint32_t>(p) < n && child[v] >= 0) {
            const uint32_t c = static_cast<uint32_t>(child[v]) + 1u;
            if (c < deg[p]) {
                const uint32_t sib = kids[off[p] + c];
                x = sib < n ? 2u * sib : end;
            } else {
                x = 2u * static_cast<uint32_t>(p) + 1u;
            }
        }
        ev[2u * v + 1u] = Event{x, 1u, -1, 0u};
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ev[end] = Event{end, 0u, 0, 0u};
}

// one round of pointer jumping
__global__ void k_fl_jump(const Event* __restrict__ in, Event* __restrict__ out, uint32_t events) {
    FL_FOR(x, events) {
        const Event a = in[x];
        const Event b = in[a.succ];
        out[x] = Event{b.succ, a.exits + b.exits, a.level + b.level, 0u};
    }
}

// post-order index and depth of every node
__global__ void k_fl_rank(const Event* ev, uint32_t n, int32_t* post, FlatErr* e) {
    FL_FOR(v, n) {
        const uint32_t q = n - ev[2u * v + 1u].exits;
        if (q >= n) flag(e, v);  // a node the root does not reach
        post[v] = static_cast<int32_t>(q);
        const int32_t d = -ev[2u * v].level;
        if (d >= 0) atomicMax(&e->max_depth, static_cast<uint32_t>(d));
        if (v == e->root && e->roots == 1u) e->reached = ev[2u * v].exits;
    }
}

__global__ void k_fl_scatter(const uint8_t* type, const uint8_t* rtype, const int32_t* parent, const int32_t* child,
                             const uint32_t* data, uint32_t n, const int32_t* post, const Event* ev, uint8_t* o_type,
                             uint8_t* o_rtype, int32_t* o_parent, int32_t* o_depth, int32_t* o_child,
                             uint32_t* o_data, int32_t* order) {
    FL_FOR(v, n) {
        const int32_t q = post[v];
        if (q < 0 || static_cast<uint32_t>(q) >= n) continue;
        const int32_t p = parent[v];
        const bool ok_p = p >= 0 && static_cast<uint32_t>(p) < n;
        o_type[q] = type[v];
        o_rtype[q] = rtype[v];
        o_parent[q] = ok_p ? post[p] : -1;
        o_depth[q] = -ev[2u * v].level;
        o_child[q] = ok_p ? child[v] : -1;
        o_data[q] = data[v];
        if (order) order[v] = q;
    }
}

template <class T>
cudaError_t dev_alloc(T** p, size_t count, cudaStream_t s) {
    return cudaMallocAsync(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T), s);
}

}  // namespace

extern "C" ptl_status ptl_flatten(const ptl_tree_view* in, ptl_depth_tree_out* out, int device, void* stream) {
    if (!in || !out) return PTL_BAD_ARGUMENT;
    const size_t n64 = in->n;
    if (n64 == 0 || n64 >= (1ull << 31)) return PTL_BAD_ARGUMENT;
    if (!in->type || !in->rtype || !in->parent || !in->child_idx || !in->data || !out->type || !out->rtype ||
        !out->parent || !out->depth || !out->child_idx || !out->data)
        return PTL_BAD_ARGUMENT;
    const uint32_t n = static_cast<uint32_t>(n64);
    const ptl::DeviceScope on_device(device);
    if (!on_device.ok()) return PTL_CUDA_ERROR;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // device copies of the inputs (or the caller's device arrays) and of the outputs
    const uint8_t *d_type = in->type, *d_rtype = in->rtype;
    const int32_t *d_parent = in->parent, *d_child = in->child_idx;
    const uint32_t* d_data = in->data;
    uint8_t *o_type = out->type, *o_rtype = out->rtype;
    int32_t *o_parent = out->parent, *o_depth = out->depth, *o_child = out->child_idx, *o_order = out->order;
    uint32_t* o_data = out->data;
    uint8_t* in_bytes = nullptr;   // staged inputs (host views): 18 bytes per node
    uint8_t* out_bytes = nullptr;  // staged outputs (host views): 22 bytes per node
    uint32_t *deg = nullptr, *off = nullptr, *kids = nullptr, *tsum = nullptr;
    int32_t* post = nullptr;
    Event *ev0 = nullptr, *ev1 = nullptr;
    FlatErr* err = nullptr;
    FlatErr herr{};
    const uint32_t tiles = static_cast<uint32_t>((n64 + 1 + kScanTile - 1) / kScanTile);
    const uint32_t events = 2u * n + 1u;
    ptl_status st = PTL_OK;
    cudaError_t ce = cudaSuccess;
#define FL_CU(x)                       \
    do {                               \
        ce = (x);                      \
        if (ce != cudaSuccess) goto done; \
    } while (0)
    if (!in->on_device) {
        FL_CU(dev_alloc(&in_bytes, 18 * n64, s));
        uint8_t* b = in_bytes;
        FL_CU(cudaMemcpyAsync(b, in->parent, 4 * n64, cudaMemcpyHostToDevice, s));
        d_parent = reinterpret_cast<const int32_t*>(b);
        FL_CU(cudaMemcpyAsync(b + 4 * n64, in->child_idx, 4 * n64, cudaMemcpyHostToDevice, s));
        d_child = reinterpret_cast<const int32_t*>(b + 4 * n64);
        FL_CU(cudaMemcpyAsync(b + 8 * n64, in->data, 4 * n64, cudaMemcpyHostToDevice, s));
        d_data = reinterpret_cast<const uint32_t*>(b + 8 * n64);
        FL_CU(cudaMemcpyAsync(b + 12 * n64, in->type, n64, cudaMemcpyHostToDevice, s));
        d_type = b + 12 * n64;
        FL_CU(cudaMemcpyAsync(b + 13 * n64, in->rtype, n64, cudaMemcpyHostToDevice, s));
        d_rtype = b + 13 * n64;
    }
    if (!out->on_device) {
        FL_CU(dev_alloc(&out_bytes, 22 * n64, s));
        uint8_t* b = out_bytes;
        o_parent = reinterpret_cast<int32_t*>(b);
        o_depth = reinterpret_cast<int32_t*>(b + 4 * n64);
        o_child = reinterpret_cast<int32_t*>(b + 8 * n64);
        o_data = reinterpret_cast<uint32_t*>(b + 12 * n64);
        o_order = out->order ? reinterpret_cast<int32_t*>(b + 16 * n64) : nullptr;
        o_type = b + 20 * n64;
        o_rtype = b + 21 * n64;
    }
    FL_CU(dev_alloc(&deg, n64, s));
    FL_CU(dev_alloc(&off, n64 + 1, s));
    FL_CU(dev_alloc(&kids, n64, s));
    FL_CU(dev_alloc(&tsum, tiles, s));
    FL_CU(dev_alloc(&post, n64, s));
    FL_CU(dev_alloc(&ev0, events, s));
    FL_CU(dev_alloc(&ev1, events, s));
    FL_CU(dev_alloc(&err, 1, s));
    FL_CU(cudaMemsetAsync(deg, 0, 4 * n64, s));
    FL_CU(cudaMemsetAsync(kids, 0xFF, 4 * n64, s));
    FL_CU(cudaMemsetAsync(err, 0, sizeof(FlatErr), s));

    k_fl_count<<<grid_of(n), kThreads, 0, s>>>(d_parent, d_child, n, deg, err);
    k_fl_tile_sums<<<tiles, kScanThreads, 0, s>>>(deg, n, tsum);
    k_fl_scan_sums<<<1, kScanThreads, 0, s>>>(tsum, tiles);
    k_fl_tiles<<<tiles, kScanThreads, 0, s>>>(deg, n, tsum, off);
    k_fl_place<<<grid_of(n), kThreads, 0, s>>>(d_parent, d_child, n, deg, off, kids, err);
    k_fl_tour<<<grid_of(n), kThreads, 0, s>>>(d_parent, d_child, n, deg, off, kids, ev0);
    {
        uint32_t rounds = 0;
        while ((1ull << rounds) < events) ++rounds;
        for (uint32_t r = 0; r < rounds; ++r) {
            k_fl_jump<<<grid_of(events), kThreads, 0, s>>>(ev0, ev1, events);
            std::swap(ev0, ev1);
        }
    }
    k_fl_rank<<<grid_of(n), kThreads, 0, s>>>(ev0, n, post, err);
    k_fl_scatter<<<grid_of(n), kThreads, 0, s>>>(d_type, d_rtype, d_parent, d_child, d_data, n, post, ev0, o_type,
                                                 o_rtype, o_parent, o_depth, o_child, o_data, o_order);
    FL_CU(cudaGetLastError());
    FL_CU(cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, s));
    if (!out->on_device) {
        FL_CU(cudaMemcpyAsync(out->parent, o_parent, 4 * n64, cudaMemcpyDeviceToHost, s));
        FL_CU(cudaMemcpyAsync(out->depth, o_depth, 4 * n64, cudaMemcpyDeviceToHost, s));
        FL_CU(cudaMemcpyAsync(out->child_idx, o_child, 4 * n64, cudaMemcpyDeviceToHost, s));
        FL_CU(cudaMemcpyAsync(out->data, o_data, 4 * n64, cudaMemcpyDeviceToHost, s));
        if (out->order) FL_CU(cudaMemcpyAsync(out->order, o_order, 4 * n64, cudaMemcpyDeviceToHost, s));
        FL_CU(cudaMemcpyAsync(out->type, o_type, n64, cudaMemcpyDeviceToHost, s));
        FL_CU(cudaMemcpyAsync(out->rtype, o_rtype, n64, cudaMemcpyDeviceToHost, s));
    }
    FL_CU(cudaStreamSynchronize(s));
    if (herr.code != 0 || herr.roots != 1 || herr.reached != n) st = PTL_INVALID_AST;
    out->max_depth = herr.max_depth;
done:
#undef FL_CU
    for (void* p : {static_cast<void*>(in_bytes), static_cast<void*>(out_bytes), static_cast<void*>(deg),
                    static_cast<void*>(off), static_cast<void*>(kids), static_cast<void*>(tsum),
                    static_cast<void*>(post), static_cast<void*>(ev0), static_cast<void*>(ev1),
                    static_cast<void*>(err)})
        if (p) cudaFreeAsync(p, s);
    if (ce != cudaSuccess) {
        cudaStreamSynchronize(s);
        return ce == cudaErrorMemoryAllocation ? PTL_OOM : PTL_CUDA_ERROR;
    }
    return st;
}
