// C ABI of the GB300 code generator (include/ptl_codegen.h): generator objects, the
// device arena and the stage sequence.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <initializer_list>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <cstdlib>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/ptl_codegen.h"
#include "ptl_kernels.cuh"

namespace ptl {
namespace {

constexpr size_t kFrontPad = 16;  // elements before index 0 (the reference reads [-1])
constexpr size_t kBackPad = 80;   // elements after the last 8-lane block

// A device buffer with the reference's padding around it.  Allocated and freed in the
// order of its generator's stream (cudaMallocAsync / cudaFreeAsync): growing or freeing
// it does not wait for the whole device, so generators on other threads keep running.
struct DevBuf {
    void* base = nullptr;
    size_t bytes = 0;
    size_t elem = 4;
    size_t count = 0;  // logical capacity in elements (without pads)
    cudaStream_t s = nullptr;  // the owner's stream

    template <typename T>
    T* at() const { return base ? reinterpret_cast<T*>(static_cast<char*>(base) + kFrontPad * elem) : nullptr; }

    cudaError_t ensure(size_t n, size_t esize) {
        const size_t need = (n + kFrontPad + kBackPad) * esize;
        if (base && bytes >= need && elem == esize) {
            count = n;
            return cudaSuccess;
        }
        if (base) cudaFreeAsync(base, s);
        base = nullptr;
        bytes = 0;
        const size_t grow = need + need / 4;  // room to grow without reallocating
        cudaError_t e = cudaMallocAsync(&base, grow, s);
        if (e != cudaSuccess) { base = nullptr; return e; }
        bytes = grow;
        elem = esize;
        count = n;
        return cudaSuccess;
    }
    cudaError_t zero(cudaStream_t s) const { return base ? cudaMemsetAsync(base, 0, (count + kFrontPad + kBackPad) * elem, s) : cudaSuccess; }
    cudaError_t fill(cudaStream_t s, int byte) const { return base ? cudaMemsetAsync(base, byte, (count + kFrontPad + kBackPad) * elem, s) : cudaSuccess; }
    void release() { if (base) cudaFreeAsync(base, s); base = nullptr; bytes = 0; }
    // elements the allocation holds (at least the last ensure's n)
    size_t capacity() const { return base ? bytes / elem - kFrontPad - kBackPad : 0; }
};

const CodeTables& host_tables() {
    static CodeTables t;
    static std::once_flag once;
    std::call_once(once, [] { build_code_tables(&t); });
    return t;
}

inline size_t r8(size_t n) { return (n + 7) & ~size_t(7); }

}  // namespace

__global__ void k_init_lifetime(unsigned long long* lt, uint32_t F) {
    for (uint64_t k = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < F;
         k += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        lt[k] = 0x1Full;
}

}  // namespace ptl

using namespace ptl;

struct ptl_generator {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;

    // input (device copy)
    size_t n = 0, max_depth = 0;
    DevBuf in_type, in_rtype, in_parent, in_depth, in_child, in_data;
    // node arrays
    DevBuf nt, rt, nd1, nd, par, ci, dep, fflag, sizes, loc0, loc, pos, regs;
    DevBuf decl, fn_id, fn_start, fn_size, fn_end, fn_start0, fn_size0, fn_end0;
    DevBuf fn_ra_start, fn_ra_end, fn_ra_size;
    DevBuf instr, rd, rs1, rs2, jt, owner, used, smark, used_instrs;
    DevBuf symreg, symswp, stamp, defpos, lifetime, trig_min, trig_max, ra_chunks, spill, roffs;
    DevBuf ni, nrd, nr1, nr2, njt, fsz, joffs, out;
    DevBuf sort_a, sort_apos, sort_bpos, sort_seg0, sort_seg1, sort_tile_seg, sort_tile_l, sort_tile_r, sort_stops,
        sort_leaf, sort_heap, sort_counters, sort_local, sort_equal;
    DevBuf scan_status, scan_counter, meta, flags, errw, tables;
    DevBuf preserve, sregs, ssteps, sextra, sclaim;  // scalar register allocation
    bool scalar = false;  // the scalar generator's semantics (rv_generator_st)

    // results
    uint32_t F = 0, W = 0, W2 = 0, W3 = 0, S = 0;
    std::vector<uint32_t> words, fn_start_h, fn_end_h, fn_size_h, fn_id_h;
    bool words_valid = false, table_valid = false;  // the last result's host copies are current
    uint64_t stage_ns[7] = {0, 0, 0, 0, 0, 0, 0};
    uint32_t sort_rounds = 0, opt_sweeps = 0;
    SortRoundGraph sort_graph;  // a pair of depth-sort rounds, replayed
    bool ra_serial = false;

    ~ptl_generator() {
        for (DevBuf* b : all()) b->release();
        if (stream) cudaStreamDestroy(stream);
    }
    // The buffers allocate and free in this generator's stream order (after it exists).
    void bind_stream() {
        for (DevBuf* b : all()) b->s = stream;
    }
    std::vector<DevBuf*> all() {
        return {&in_type, &in_rtype, &in_parent, &in_depth, &in_child, &in_data, &nt, &rt, &nd1, &nd,
                &par, &ci, &dep, &fflag, &sizes, &loc0, &loc, &pos, &regs, &decl, &fn_id, &fn_start,
                &fn_size, &fn_end, &fn_start0, &fn_size0, &fn_end0, &fn_ra_start, &fn_ra_end, &fn_ra_size,
                &instr, &rd, &rs1, &rs2, &jt, &owner, &used, &smark, &used_instrs, &symreg, &symswp,
                &stamp, &defpos, &lifetime, &trig_min, &trig_max, &ra_chunks, &spill, &roffs, &ni, &nrd, &nr1, &nr2, &njt,
                &fsz, &joffs, &out, &sort_a, &sort_apos, &sort_bpos, &sort_seg0, &sort_seg1, &sort_stops,
                &sort_tile_seg, &sort_tile_l, &sort_tile_r, &sort_leaf, &sort_heap, &sort_counters, &sort_local, &sort_equal,
                &scan_status, &scan_counter, &meta, &flags, &errw, &tables, &preserve, &sregs, &ssteps,
                &sextra, &sclaim};
    }
};

namespace {

// How the plain pipeline moves the caller's arrays, per device, decided once: by a copy
// kernel that reads (writes) pageable host memory in place, where the device accesses
// it coherently (cudaDevAttrPageableMemoryAccess) and a 32 MB probe of each direction
// shows that faster than the copy engine's staged copy of pageable memory; else staged.
// (On some hosts in-place access to pageable memory runs far below the link.)
struct PageablePaths {
    bool read = false, write = false;
};
PageablePaths probe_pageable(int device) {
    PageablePaths out;
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess || !v) {
        cudaGetLastError();
        return out;
    }
    constexpr size_t kBytes = size_t(32) << 20;
    void* host = std::malloc(kBytes);
    void* dev = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t ev[5] = {};
    bool ok = host && cudaMalloc(&dev, kBytes) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess;
    for (auto& e : ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    float t[4] = {0, 0, 0, 0};
    if (ok) {
        std::memset(host, 1, kBytes);
        for (int rep = 0; rep < 2 && ok; ++rep) {  // the first round warms every path
            ok = cudaEventRecord(ev[0], s) == cudaSuccess && kernel_copy(host, dev, kBytes, s) == cudaSuccess &&
                 cudaEventRecord(ev[1], s) == cudaSuccess &&
                 cudaMemcpyAsync(dev, host, kBytes, cudaMemcpyHostToDevice, s) == cudaSuccess &&
                 cudaEventRecord(ev[2], s) == cudaSuccess && kernel_copy(dev, host, kBytes, s) == cudaSuccess &&
                 cudaEventRecord(ev[3], s) == cudaSuccess &&
                 cudaMemcpyAsync(host, dev, kBytes, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                 cudaEventRecord(ev[4], s) == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess;
        }
        for (int k = 0; k < 4 && ok; ++k) ok = cudaEventElapsedTime(&t[k], ev[k], ev[k + 1]) == cudaSuccess;
        if (ok) {
            out.read = t[0] <= t[1];
            out.write = t[2] <= t[3];
        }
    }
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    if (s) cudaStreamDestroy(s);
    if (dev) cudaFree(dev);
    std::free(host);
    cudaGetLastError();  // a failed probe leaves no error behind
    return out;
}
const PageablePaths& pageable_paths(int device) {
    static std::mutex mu;
    static std::map<int, PageablePaths> known;
    std::lock_guard<std::mutex> lk(mu);
    auto it = known.find(device);
    if (it == known.end()) {
        const DeviceScope on_device(device);
        it = known.emplace(device, on_device.ok() ? probe_pageable(device) : PageablePaths{}).first;
    }
    return it->second;
}

ptl_status fail(ptl_generator* g, ptl_status st, const std::string& msg) {
    if (g) g->last_error = msg;
    return st;
}

ptl_status cuda_fail(ptl_generator* g, cudaError_t e, const char* what) {
    const ptl_status st = (e == cudaErrorMemoryAllocation) ? PTL_OOM : PTL_CUDA_ERROR;
    return fail(g, st, std::string(what) + ": " + cudaGetErrorString(e));
}

#define PTL_CU(expr)                                          \
    do {                                                      \
        const cudaError_t e_ = (expr);                        \
        if (e_ != cudaSuccess) return cuda_fail(g, e_, #expr); \
    } while (0)

// A kernel must never see a pointer to a buffer that is not allocated yet; the views
// are rebuilt after each allocation and checked here before use.
bool prog_ready(const Prog& P, std::initializer_list<const void*> need) {
    for (const void* p : need) if (!p) return false;
    return P.err && P.flags && P.tab.t;
}

Prog make_prog(ptl_generator* g) {
    Prog P{};
    P.n = static_cast<uint32_t>(g->n);
    P.nb8 = static_cast<uint32_t>(r8(g->n));
    P.max_depth = static_cast<uint32_t>(g->max_depth);
    P.F = g->F;
    P.fb8 = static_cast<uint32_t>(r8(g->F));
    P.W = g->W;
    P.wb8 = static_cast<uint32_t>(r8(g->W));
    P.W2 = g->W2;
    P.w2b8 = static_cast<uint32_t>(r8(g->W2));
    P.W3 = g->W3;
    P.S = g->S;
    P.in_type = g->in_type.at<uint8_t>();
    P.in_rtype = g->in_rtype.at<uint8_t>();
    P.in_parent = g->in_parent.at<int32_t>();
    P.in_depth = g->in_depth.at<int32_t>();
    P.in_child = g->in_child.at<int32_t>();
    P.in_data = g->in_data.at<uint32_t>();
    P.nt = g->nt.at<uint8_t>();
    P.rt = g->rt.at<uint8_t>();
    P.nd1 = g->nd1.at<uint32_t>();
    P.nd = g->nd.at<uint32_t>();
    P.par = g->par.at<int32_t>();
    P.ci = g->ci.at<int32_t>();
    P.dep = g->dep.at<int32_t>();
    P.fflag = g->fflag.at<uint8_t>();
    P.sizes = g->sizes.at<uint32_t>();
    P.loc0 = g->loc0.at<uint32_t>();
    P.loc = g->loc.at<uint32_t>();
    P.regs = g->regs.at<uint32_t>();
    P.pos = g->pos.at<uint32_t>();
    P.owner = g->owner.at<unsigned long long>();
    P.decl = g->decl.at<uint32_t>();
    P.fn_id = g->fn_id.at<uint32_t>();
    P.fn_start = g->fn_start.at<uint32_t>();
    P.fn_size = g->fn_size.at<uint32_t>();
    P.fn_end = g->fn_end.at<uint32_t>();
    P.fn_start0 = g->fn_start0.at<uint32_t>();
    P.fn_size0 = g->fn_size0.at<uint32_t>();
    P.instr = g->instr.at<uint32_t>();
    P.rd = g->rd.at<uint32_t>();
    P.rs1 = g->rs1.at<uint32_t>();
    P.rs2 = g->rs2.at<uint32_t>();
    P.jt = g->jt.at<uint32_t>();
    P.used = g->used.at<uint8_t>();
    P.smark = g->smark.at<uint8_t>();
    P.used_instrs = g->used_instrs.at<uint32_t>();
    P.symreg = g->symreg.at<uint32_t>();
    P.symswp = g->symswp.at<uint32_t>();
    P.stamp = g->stamp.at<uint32_t>();
    P.defpos = g->defpos.at<uint8_t>();
    P.lifetime = g->lifetime.at<unsigned long long>();
    P.trig_min = g->trig_min.at<uint32_t>();
    P.trig_max = g->trig_max.at<uint32_t>();
    P.ra_chunks = g->ra_chunks.at<uint32_t>();
    P.spill = g->spill.at<uint32_t>();
    P.roffs = g->roffs.at<uint32_t>();
    P.ni = g->ni.at<uint32_t>();
    P.nrd = g->nrd.at<uint32_t>();
    P.nr1 = g->nr1.at<uint32_t>();
    P.nr2 = g->nr2.at<uint32_t>();
    P.njt = g->njt.at<uint32_t>();
    P.fsz = g->fsz.at<uint32_t>();
    P.joffs = g->joffs.at<uint32_t>();
    P.out = g->out.at<uint32_t>();
    P.tab.t = g->tables.at<CodeTables>();
    P.err = g->errw.at<ErrorWord>();
    P.flags = g->flags.at<uint32_t>();
    P.scalar = g->scalar ? 1u : 0u;
    return P;
}

ptl_status check_error_word(ptl_generator* g) {
    ErrorWord e{};
    cudaError_t ce = cudaMemcpyAsync(&e, g->errw.at<ErrorWord>(), sizeof(e), cudaMemcpyDeviceToHost, g->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(g->stream);
    if (ce != cudaSuccess) return cuda_fail(g, ce, "error word");
    if (e.code == ST_OK) return PTL_OK;
    static const char* stages[] = {"input", "preprocess", "isn_cnt", "depth sort", "isn_gen", "optimize",
                                   "regalloc", "regalloc (lane 0)", "regalloc scatter", "fix_jumps", "scan"};
    char buf[256];
    std::snprintf(buf, sizeof buf, "%s: %s at index %u",
                  e.where < sizeof(stages) / sizeof(stages[0]) ? stages[e.where] : "?",
                  e.code == ST_INVALID_AST ? "input violates the DepthTree contract"
                  : e.code == ST_DEVICE_TIMEOUT ? "bounded device wait gave up"
                                                : "input reaches behaviour the reference leaves undefined",
                  e.detail);
    return fail(g, static_cast<ptl_status>(e.code), buf);
}

template <typename T>
cudaError_t read1(ptl_generator* g, const T* dptr, T* out) {
    cudaError_t e = cudaMemcpyAsync(out, dptr, sizeof(T), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    return e;
}

struct StageTimer {
    ptl_generator* g;
    bool on;
    cudaEvent_t ev[8] = {};
    int k = 0;
    StageTimer(ptl_generator* gen, bool enable) : g(gen), on(enable) {
        if (!on) return;
        for (auto& e : ev) cudaEventCreate(&e);
        cudaEventRecord(ev[0], g->stream);
    }
    void mark() {
        if (on && k < 7) cudaEventRecord(ev[++k], g->stream);
    }
    void finish() {
        if (!on) return;
        cudaEventSynchronize(ev[k]);
        for (int s = 0; s < 7; ++s) {
            float ms = 0;
            if (s < k) cudaEventElapsedTime(&ms, ev[s], ev[s + 1]);
            g->stage_ns[s] = static_cast<uint64_t>(ms * 1e6);
        }
    }
    ~StageTimer() {
        if (on) for (auto& e : ev) cudaEventDestroy(e);
    }
};

// The depth sort's scratch for n keys (grown as needed), in ss.
cudaError_t sort_scratch(ptl_generator* g, size_t n, SortScratch* ss) {
#define E(expr)                                   \
    do {                                          \
        const cudaError_t e_ = (expr);            \
        if (e_ != cudaSuccess) return e_;         \
    } while (0)
    // a round's segments are disjoint and longer than kSortBlock, each with one partial tile
    const size_t seg_cap = n / 17 + 16, tile_cap = n / kSortTile + n / kSortBlock + 16, leaf_cap = n / 2 + 16;
    E(g->sort_a.ensure(n, 8));
    E(g->sort_apos.ensure(n, 4));
    E(g->sort_bpos.ensure(n, 4));
    E(g->sort_seg0.ensure(seg_cap, sizeof(SortSeg)));
    E(g->sort_seg1.ensure(seg_cap, sizeof(SortSeg)));
    E(g->sort_tile_seg.ensure(tile_cap, 4));
    E(g->sort_tile_l.ensure(tile_cap, 4));
    E(g->sort_tile_r.ensure(tile_cap, 4));
    E(g->sort_stops.ensure(tile_cap * 2 * (kSortTile / 32), 4));
    E(g->sort_leaf.ensure(2 * leaf_cap, 4));
    E(g->sort_heap.ensure(2 * leaf_cap, 4));
    E(g->sort_counters.ensure(8, 4));
    E(g->sort_local.ensure(3 * seg_cap, 4));
    E(g->sort_equal.ensure(2 * seg_cap, 4));
    ss->a = g->sort_a.at<unsigned long long>();
    ss->apos = g->sort_apos.at<uint32_t>();
    ss->bpos = g->sort_bpos.at<uint32_t>();
    ss->seg[0] = g->sort_seg0.at<SortSeg>();
    ss->seg[1] = g->sort_seg1.at<SortSeg>();
    // The capacities are what the allocations hold, so that they (and the captured round
    // graph that bakes them in) change only when a buffer is reallocated, not with n.
    const size_t seg_room = std::min({g->sort_seg0.capacity(), g->sort_seg1.capacity(), g->sort_local.capacity() / 3,
                                      g->sort_equal.capacity() / 2});
    const size_t tile_room = std::min({g->sort_tile_seg.capacity(), g->sort_tile_l.capacity(),
                                       g->sort_tile_r.capacity(), g->sort_stops.capacity() / (2 * (kSortTile / 32))});
    const size_t leaf_room = std::min(g->sort_leaf.capacity(), g->sort_heap.capacity()) / 2;
    ss->seg_cap = static_cast<uint32_t>(std::min<size_t>(seg_room, UINT32_MAX));
    ss->tile_seg = g->sort_tile_seg.at<uint32_t>();
    ss->tile_l = g->sort_tile_l.at<uint32_t>();
    ss->tile_r = g->sort_tile_r.at<uint32_t>();
    ss->stops = g->sort_stops.at<uint32_t>();
    ss->tile_cap = static_cast<uint32_t>(std::min<size_t>(tile_room, UINT32_MAX));
    ss->leaf = g->sort_leaf.at<uint32_t>();
    ss->heap = g->sort_heap.at<uint32_t>();
    ss->leaf_cap = static_cast<uint32_t>(std::min<size_t>(leaf_room, UINT32_MAX));
    ss->counters = g->sort_counters.at<uint32_t>();
    ss->local = g->sort_local.at<uint32_t>();
    ss->equal = g->sort_equal.at<uint32_t>();
#undef E
    return cudaSuccess;
}

// row0_hash: the AVX allocator's general row-0 lookup; serial: the scalar allocator in
// the reference's order for every program.  Both leave the output unchanged.
ptl_status run_pipeline(ptl_generator* g, bool profile, bool to_host, bool row0_hash, bool serial) {
    cudaStream_t s = g->stream;
    const size_t n = g->n;
    const size_t nb8 = r8(n);
    g->words_valid = g->table_valid = false;
    StageTimer timer(g, profile);

    // fixed-size scratch first, so every Prog view below sees it
    PTL_CU(g->flags.ensure(4, 4));
    PTL_CU(g->flags.zero(s));
    PTL_CU(g->errw.zero(s));
    PTL_CU(g->meta.zero(s));
    // node arrays
    for (DevBuf* b : {&g->nt, &g->rt}) {
        PTL_CU(b->ensure(nb8, 1));
        PTL_CU(b->zero(s));
    }
    for (DevBuf* b : {&g->nd1, &g->nd, &g->par, &g->ci, &g->dep, &g->sizes, &g->loc0, &g->loc, &g->pos}) {
        PTL_CU(b->ensure(nb8, 4));
        PTL_CU(b->zero(s));
    }
    PTL_CU(g->fflag.ensure(nb8, 1));
    PTL_CU(g->fflag.zero(s));
    PTL_CU(g->decl.ensure(nb8, 4));
    PTL_CU(g->decl.zero(s));
    PTL_CU(g->regs.ensure(3 * n, 4));
    PTL_CU(g->regs.zero(s));
    PTL_CU(g->scan_counter.ensure(1, 4));
    // Tile-status scratch for a scan over `count` elements (grows with the word counts).
    auto scan_for = [&](size_t count, ScanScratch* sc) -> cudaError_t {
        const size_t tiles = (std::max(count, size_t(1)) + kScanTileElems - 1) / kScanTileElems + 8;
        const cudaError_t e = g->scan_status.ensure(tiles, 8);
        if (e != cudaSuccess) return e;
        *sc = ScanScratch{g->scan_status.at<unsigned long long>(), g->scan_counter.at<uint32_t>(),
                          static_cast<uint32_t>(tiles)};
        return cudaSuccess;
    };
    ScanScratch sc{};
    PTL_CU(scan_for(nb8, &sc));

    g->F = g->W = g->W2 = g->W3 = g->S = 0;
    Prog P = make_prog(g);

    // ---- input checks and copy, one pass; then preprocess
    if (!prog_ready(P, {P.nt, P.rt, P.nd1, P.nd, P.par, P.ci, P.dep, P.fflag, P.sizes, P.loc0, P.loc, P.decl}))
        return fail(g, PTL_CUDA_ERROR, "internal: unallocated node arrays");
    launch_ingest(P, s);
    {
        uint32_t reach = 0;  // some node sits at max_depth (read with the error word's sync)
        PTL_CU(cudaMemcpyAsync(&reach, P.flags + 3, sizeof(reach), cudaMemcpyDeviceToHost, s));
        if (ptl_status st = check_error_word(g); st != PTL_OK) return st;
        if (!reach) return fail(g, PTL_INVALID_AST, "input: depths 0..max_depth are not all populated");
    }
    if (g->scalar) launch_preprocess_scalar(P, s);
    else launch_preprocess(P, s);
    timer.mark();

    // ---- isn_cnt: count + scan, fixes, function table
    launch_count_scan(P, sc, s);
    launch_fix(P, s);
    launch_decl_scan(P, g->meta.at<uint32_t>(), sc, s);
    uint32_t meta[3] = {0, 0, 0};
    PTL_CU(cudaMemcpyAsync(meta, g->meta.at<uint32_t>(), sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PTL_CU(cudaStreamSynchronize(s));
    if (ptl_status st = check_error_word(g); st != PTL_OK) return st;
    g->F = meta[0];
    if (g->F == 0) return fail(g, PTL_UNSUPPORTED, "isn_cnt: program has no function (the reference takes the max of an empty range)");
    const size_t fb8 = r8(g->F);
    for (DevBuf* b : {&g->fn_id, &g->fn_start, &g->fn_size, &g->fn_end, &g->fn_start0, &g->fn_size0, &g->fn_end0,
                      &g->fn_ra_start, &g->fn_ra_end, &g->fn_ra_size}) {
        PTL_CU(b->ensure(fb8 + 8, 4));
        PTL_CU(b->zero(s));
    }
    P = make_prog(g);
    if (!prog_ready(P, {P.fn_id, P.fn_start, P.fn_size, P.fn_end, P.fn_start0, P.fn_size0}))
        return fail(g, PTL_CUDA_ERROR, "internal: unallocated function table");
    launch_functab(P, g->meta.at<uint32_t>(), s);
    PTL_CU(cudaMemcpyAsync(meta, g->meta.at<uint32_t>(), sizeof(meta), cudaMemcpyDeviceToHost, s));
    PTL_CU(cudaStreamSynchronize(s));
    g->W = meta[1];
    g->S = meta[2];
    PTL_CU(cudaMemcpyAsync(g->fn_end0.at<uint32_t>(), g->fn_end.at<uint32_t>(), g->F * 4, cudaMemcpyDeviceToDevice, s));
    timer.mark();

    // ---- isn_gen: depth order, register propagation, instruction writes
    SortScratch ss{};
    PTL_CU(sort_scratch(g, n, &ss));

    const size_t wb8 = r8(g->W);
    for (DevBuf* b : {&g->instr, &g->rd, &g->rs1, &g->rs2, &g->jt, &g->used_instrs, &g->symreg, &g->symswp,
                      &g->stamp, &g->spill, &g->roffs}) {
        PTL_CU(b->ensure(wb8, 4));
        PTL_CU(b->zero(s));
    }
    PTL_CU(g->owner.ensure(wb8, 8));
    PTL_CU(g->owner.zero(s));
    PTL_CU(g->used.ensure(wb8, 1));
    PTL_CU(g->used.zero(s));
    PTL_CU(g->smark.ensure(wb8, 1));
    PTL_CU(g->smark.zero(s));
    PTL_CU(g->defpos.ensure(wb8, 1));
    P = make_prog(g);
    if (!prog_ready(P, {P.instr, P.rd, P.rs1, P.rs2, P.jt, P.used_instrs, P.symreg, P.symswp, P.stamp, P.spill,
                        P.defpos, P.roffs, P.owner, P.used, P.smark, P.pos, P.regs}))
        return fail(g, PTL_CUDA_ERROR, "internal: unallocated word arrays");
    PTL_CU(run_depth_sort(P, ss, s, &g->sort_rounds, &g->sort_graph));
    if (g->scalar) launch_gen_scalar(P, s);
    else launch_gen(P, s);
    if (ptl_status st = check_error_word(g); st != PTL_OK) return st;
    timer.mark();

    // ---- optimize
    PTL_CU(run_optimize(P, s, &g->opt_sweeps));
    if (ptl_status st = check_error_word(g); st != PTL_OK) return st;
    timer.mark();

    // ---- regalloc
    PTL_CU(g->lifetime.ensure(fb8, 8));
    PTL_CU(g->lifetime.zero(s));
    if (g->scalar) {
        PTL_CU(g->preserve.ensure(fb8, 8));
        PTL_CU(g->preserve.zero(s));
        PTL_CU(g->sextra.ensure(wb8, 4));
        P = make_prog(g);
        if (!prog_ready(P, {P.lifetime, g->preserve.at<void>(), g->sextra.at<void>()}))
            return fail(g, PTL_CUDA_ERROR, "internal: unallocated regalloc state");
        bool cross = false;
        PTL_CU(scalar_regalloc_cross(P, s, &cross));
        if (cross || serial) {
            PTL_CU(g->sregs.ensure(static_cast<size_t>(g->F) * 64, 4));
            PTL_CU(g->ssteps.ensure(g->F, sizeof(SRaStep)));
            launch_scalar_ra_serial(P, g->sregs.at<int32_t>(), g->ssteps.at<SRaStep>(),
                                    g->preserve.at<unsigned long long>(), s);
        } else {
            launch_scalar_ra_free(P, g->preserve.at<unsigned long long>(), s);
        }
        g->ra_serial = cross || serial;
        PTL_CU(scan_for(wb8, &sc));
        launch_scalar_ra_count_scan(P, g->preserve.at<unsigned long long>(), g->sextra.at<uint32_t>(), sc, s);
    } else {
        note_launch();
        k_init_lifetime<<<std::min<size_t>((g->F + 255) / 256, 1024), 256, 0, s>>>(g->lifetime.at<unsigned long long>(), g->F);
        const size_t trig = static_cast<size_t>(std::max<uint32_t>(g->S, 1)) * 64;
        PTL_CU(g->trig_min.ensure(trig, 4));
        PTL_CU(g->trig_min.fill(s, 0xFF));
        PTL_CU(g->trig_max.ensure(trig, 4));
        PTL_CU(g->trig_max.zero(s));
        PTL_CU(g->ra_chunks.ensure(2 * (static_cast<size_t>(g->S) / 32 + 2), 4));
        P = make_prog(g);
        if (!prog_ready(P, {P.lifetime, P.trig_min, P.trig_max, P.ra_chunks}))
            return fail(g, PTL_CUDA_ERROR, "internal: unallocated regalloc state");
        PTL_CU(run_regalloc_steps(P, s, &g->ra_serial, row0_hash));
        PTL_CU(scan_for(wb8, &sc));
        launch_regalloc_count_scan(P, sc, s);
    }
    uint32_t last_off = 0;
    PTL_CU(read1(g, P.roffs + (g->W - 1), &last_off));
    if (ptl_status st = check_error_word(g); st != PTL_OK) return st;
    g->W2 = last_off + 1;
    const size_t w2b8 = r8(g->W2);
    for (DevBuf* b : {&g->ni, &g->nrd, &g->nr1, &g->nr2, &g->njt, &g->fsz, &g->joffs}) {
        PTL_CU(b->ensure(w2b8 + 16, 4));
        PTL_CU(b->zero(s));
    }
    P = make_prog(g);
    if (!prog_ready(P, {P.ni, P.nrd, P.nr1, P.nr2, P.njt, P.fsz, P.joffs}))
        return fail(g, PTL_CUDA_ERROR, "internal: unallocated regalloc output");
    if (g->scalar) {
        PTL_CU(g->sclaim.ensure(g->W2, 8));
        launch_scalar_ra_emit(P, g->preserve.at<unsigned long long>(), g->sclaim.at<unsigned long long>(), s);
    } else {
        launch_regalloc_emit(P, s);
    }
    for (int k = 0; k < 3; ++k) {
        DevBuf* src[3] = {&g->fn_start, &g->fn_end, &g->fn_size};
        DevBuf* dst[3] = {&g->fn_ra_start, &g->fn_ra_end, &g->fn_ra_size};
        PTL_CU(cudaMemcpyAsync(dst[k]->at<uint32_t>(), src[k]->at<uint32_t>(), g->F * 4, cudaMemcpyDeviceToDevice, s));
    }
    timer.mark();

    // ---- fix_jumps (+ postprocess)
    PTL_CU(scan_for(w2b8, &sc));
    launch_fixjumps_scan(P, sc, s);
    uint32_t last_size = 0, last_joff = 0;
    PTL_CU(read1(g, P.fsz + (g->W2 - 1), &last_size));
    PTL_CU(read1(g, P.joffs + (g->W2 - 1), &last_joff));
    if (ptl_status st = check_error_word(g); st != PTL_OK) return st;
    g->W3 = last_size + last_joff;
    PTL_CU(g->out.ensure(r8(g->W3) + 8, 4));
    PTL_CU(g->out.zero(s));
    P = make_prog(g);
    if (!prog_ready(P, {P.out})) return fail(g, PTL_CUDA_ERROR, "internal: unallocated output");
    launch_fixjumps_emit(P, s);
    timer.mark();
    timer.mark();  // postprocess is fused into fix_jumps
    if (ptl_status st = check_error_word(g); st != PTL_OK) return st;
    timer.finish();

    if (to_host) {
        g->words.resize(g->W3);
        g->fn_start_h.resize(g->F);
        g->fn_end_h.resize(g->F);
        g->fn_size_h.resize(g->F);
        g->fn_id_h.resize(g->F);
        if (g->W3) {
            // Where the device accesses pageable memory coherently (ATS), kernel stores put
            // the words straight into the vector; otherwise the copy engine stages them.
            if (pageable_paths(g->device).write && (reinterpret_cast<uintptr_t>(g->words.data()) & 15u) == 0)
                PTL_CU(kernel_copy(P.out, g->words.data(), g->W3 * 4ull, s));
            else
                PTL_CU(cudaMemcpyAsync(g->words.data(), P.out, g->W3 * 4ull, cudaMemcpyDeviceToHost, s));
        }
        PTL_CU(cudaMemcpyAsync(g->fn_start_h.data(), P.fn_start, g->F * 4ull, cudaMemcpyDeviceToHost, s));
        PTL_CU(cudaMemcpyAsync(g->fn_end_h.data(), P.fn_end, g->F * 4ull, cudaMemcpyDeviceToHost, s));
        PTL_CU(cudaMemcpyAsync(g->fn_size_h.data(), P.fn_size, g->F * 4ull, cudaMemcpyDeviceToHost, s));
        PTL_CU(cudaMemcpyAsync(g->fn_id_h.data(), P.fn_id, g->F * 4ull, cudaMemcpyDeviceToHost, s));
        PTL_CU(cudaStreamSynchronize(s));
        g->words_valid = g->table_valid = true;
    }
    return PTL_OK;
}

}  // namespace

extern "C" {

namespace {

cudaError_t upload_inputs(ptl_generator* g, const ptl_ast_view* tree) {
    const cudaMemcpyKind kind = tree->on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const size_t n = tree->n;
    struct { DevBuf* b; const void* src; size_t es; } in[] = {
        {&g->in_type, tree->type, 1}, {&g->in_rtype, tree->rtype, 1}, {&g->in_parent, tree->parent, 4},
        {&g->in_depth, tree->depth, 4}, {&g->in_child, tree->child_idx, 4}, {&g->in_data, tree->data, 4}};
    // Where the device reads pageable memory coherently (ATS) and that is faster here, a
    // kernel reads the caller's arrays in place, else the copy engine copies them; either
    // way the call waits, so that the caller may reuse host arrays on return.
    bool direct = !tree->on_device && pageable_paths(g->device).read;
    for (auto& x : in) direct = direct && (reinterpret_cast<uintptr_t>(x.src) & 15u) == 0;
    cudaError_t e = cudaSuccess;
    for (auto& x : in) {
        e = x.b->ensure(n, x.es);
        if (e == cudaSuccess) {
            e = direct ? kernel_copy(x.src, x.b->at<char>(), n * x.es, g->stream)
                       : cudaMemcpyAsync(x.b->at<char>(), x.src, n * x.es, kind, g->stream);
        }
        if (e != cudaSuccess) return e;
    }
    if (!tree->on_device) {  // the caller may reuse host arrays once this returns
        e = cudaStreamSynchronize(g->stream);
        if (e != cudaSuccess) return e;
    }
    g->n = tree->n;
    g->max_depth = tree->max_depth;
    g->words_valid = g->table_valid = false;
    return cudaSuccess;
}

bool view_ok(const ptl_ast_view* tree) {
    return tree && tree->n > 0 && tree->n < (1ull << 31) && tree->type && tree->rtype && tree->parent &&
           tree->depth && tree->child_idx && tree->data;
}

}  // namespace

ptl_status ptl_generator_upload(ptl_generator* g, const ptl_ast_view* tree) {
    if (!g || !view_ok(tree)) return PTL_BAD_ARGUMENT;
    if (tree->max_depth == 0) return PTL_INVALID_AST;
    const DeviceScope on_device(g->device);
    if (!on_device.ok()) return fail(g, PTL_CUDA_ERROR, "cudaSetDevice");
    const cudaError_t e = upload_inputs(g, tree);
    if (e != cudaSuccess) return cuda_fail(g, e, "upload");
    return PTL_OK;
}

uint64_t ptl_kernel_launches(void) { return ptl::launch_count(); }

ptl_status ptl_generator_create(const ptl_ast_view* tree, int device, ptl_generator** out) {
    if (!out) return PTL_BAD_ARGUMENT;
    *out = nullptr;
    if (!view_ok(tree)) return PTL_BAD_ARGUMENT;
    if (tree->max_depth == 0) return PTL_INVALID_AST;  // the reference divides by it (rv_generator_avx.cpp:583)
    ptl_generator* g = new (std::nothrow) ptl_generator();
    if (!g) return PTL_OOM;
    g->device = device;
    g->n = tree->n;
    g->max_depth = tree->max_depth;
    const DeviceScope on_device(device);
    cudaError_t e = on_device.err;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) g->bind_stream();
    if (e == cudaSuccess) e = upload_inputs(g, tree);
    if (e == cudaSuccess) e = g->tables.ensure(sizeof(CodeTables), 1);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g->tables.at<char>(), &host_tables(), sizeof(CodeTables), cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = g->errw.ensure(1, sizeof(ErrorWord));
    if (e == cudaSuccess) e = g->meta.ensure(4, 4);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) {
        const ptl_status st = e == cudaErrorMemoryAllocation ? PTL_OOM : PTL_CUDA_ERROR;
        delete g;
        return st;
    }
    *out = g;
    return PTL_OK;
}

ptl_status ptl_generator_create_scalar(const ptl_ast_view* tree, int device, ptl_generator** out) {
    const ptl_status st = ptl_generator_create(tree, device, out);
    if (st == PTL_OK) (*out)->scalar = true;
    return st;
}

ptl_status ptl_generator_process(ptl_generator* g, int profile) {
    if (!g) return PTL_BAD_ARGUMENT;
    const DeviceScope on_device(g->device);
    if (!on_device.ok()) return fail(g, PTL_CUDA_ERROR, "cudaSetDevice");
    const ptl_status st =
        run_pipeline(g, (profile & 1) != 0, (profile & 2) == 0, (profile & 4) != 0, (profile & 8) != 0);
    if (st == PTL_OK) g->last_error.clear();
    return st;
}

namespace {
// The last result's words from the device into dst (count words), by kernel stores where
// the device writes pageable memory coherently and dst is 16-byte aligned.
cudaError_t fetch_words(ptl_generator* g, uint32_t* dst, size_t count) {
    if (count == 0) return cudaSuccess;
    const DeviceScope on_device(g->device);
    if (!on_device.ok()) return on_device.err;
    cudaError_t e = (pageable_paths(g->device).write && (reinterpret_cast<uintptr_t>(dst) & 15u) == 0)
                        ? kernel_copy(g->out.at<uint32_t>(), dst, count * 4ull, g->stream)
                        : cudaMemcpyAsync(dst, g->out.at<uint32_t>(), count * 4ull, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    return e;
}
}  // namespace

ptl_status ptl_generator_instructions(ptl_generator* g, const uint32_t** words, size_t* count) {
    if (!g || !words || !count) return PTL_BAD_ARGUMENT;
    if (!g->words_valid) {
        g->words.resize(g->W3);
        if (const cudaError_t e = fetch_words(g, g->words.data(), g->W3); e != cudaSuccess)
            return cuda_fail(g, e, "instructions");
        g->words_valid = true;
    }
    *words = g->words.data();
    *count = g->W3;
    return PTL_OK;
}

ptl_status ptl_generator_copy_instructions(ptl_generator* g, uint32_t* dst, size_t capacity, size_t* count) {
    if (!g || !count) return PTL_BAD_ARGUMENT;
    *count = g->W3;
    if (!dst) return PTL_OK;
    if (capacity < g->W3) return PTL_BAD_ARGUMENT;
    if (g->words_valid) {
        if (g->W3) std::memcpy(dst, g->words.data(), g->W3 * 4ull);
        return PTL_OK;
    }
    if (const cudaError_t e = fetch_words(g, dst, g->W3); e != cudaSuccess) return cuda_fail(g, e, "instructions");
    return PTL_OK;
}

ptl_status ptl_generator_device_instructions(ptl_generator* g, const uint32_t** words, size_t* count) {
    if (!g || !words || !count) return PTL_BAD_ARGUMENT;
    *words = g->out.at<uint32_t>();
    *count = g->W3;
    return PTL_OK;
}

ptl_status ptl_generator_function_table(ptl_generator* g, const uint32_t** starts, const uint32_t** ends,
                                        const uint32_t** sizes, const uint32_t** ids, size_t* count) {
    if (!g || !count) return PTL_BAD_ARGUMENT;
    if (!g->table_valid) {
        const DeviceScope on_device(g->device);
        if (!on_device.ok()) return fail(g, PTL_CUDA_ERROR, "cudaSetDevice");
        g->fn_start_h.resize(g->F);
        g->fn_end_h.resize(g->F);
        g->fn_size_h.resize(g->F);
        g->fn_id_h.resize(g->F);
        cudaMemcpyAsync(g->fn_start_h.data(), g->fn_start.at<uint32_t>(), g->F * 4ull, cudaMemcpyDeviceToHost, g->stream);
        cudaMemcpyAsync(g->fn_end_h.data(), g->fn_end.at<uint32_t>(), g->F * 4ull, cudaMemcpyDeviceToHost, g->stream);
        cudaMemcpyAsync(g->fn_size_h.data(), g->fn_size.at<uint32_t>(), g->F * 4ull, cudaMemcpyDeviceToHost, g->stream);
        cudaMemcpyAsync(g->fn_id_h.data(), g->fn_id.at<uint32_t>(), g->F * 4ull, cudaMemcpyDeviceToHost, g->stream);
        const cudaError_t e = cudaStreamSynchronize(g->stream);
        if (e != cudaSuccess) return cuda_fail(g, e, "function table");
        g->table_valid = true;
    }
    if (starts) *starts = g->fn_start_h.data();
    if (ends) *ends = g->fn_end_h.data();
    if (sizes) *sizes = g->fn_size_h.data();
    if (ids) *ids = g->fn_id_h.data();
    *count = g->F;
    return PTL_OK;
}

ptl_status ptl_generator_stage_ns(ptl_generator* g, uint64_t ns[7]) {
    if (!g || !ns) return PTL_BAD_ARGUMENT;
    std::memcpy(ns, g->stage_ns, sizeof(g->stage_ns));
    return PTL_OK;
}

const char* ptl_generator_last_error(const ptl_generator* g) { return g ? g->last_error.c_str() : "null generator"; }

void ptl_generator_destroy(ptl_generator* g) { delete g; }

ptl_status ptl_compile(const ptl_ast_view* tree, int device, uint32_t* words, size_t capacity, size_t* count) {
    if (!count) return PTL_BAD_ARGUMENT;
    ptl_generator* g = nullptr;
    ptl_status st = ptl_generator_create(tree, device, &g);
    if (st != PTL_OK) return st;
    st = ptl_generator_process(g, 0);
    if (st == PTL_OK) {
        *count = g->W3;
        if (words) {
            if (capacity < g->W3) st = PTL_BAD_ARGUMENT;
            else std::memcpy(words, g->words.data(), g->W3 * 4ull);
        }
    }
    ptl_generator_destroy(g);
    return st;
}

ptl_status ptl_depth_order(const int32_t* keys, size_t n, uint32_t* pos, int device) {
    if (!keys || !pos || n == 0 || n >= (1ull << 31)) return PTL_BAD_ARGUMENT;
    for (size_t i = 0; i < n; ++i) if (keys[i] < 0) return PTL_BAD_ARGUMENT;
    const DeviceScope on_device(device);
    if (!on_device.ok()) return PTL_CUDA_ERROR;
    ptl_generator g;  // its buffers and stream only
    g.device = device;
    g.n = n;
    cudaError_t e = cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) g.bind_stream();
    if (e == cudaSuccess) e = g.dep.ensure(r8(n), 4);
    if (e == cudaSuccess) e = g.pos.ensure(r8(n), 4);
    if (e == cudaSuccess) e = g.errw.ensure(1, sizeof(ErrorWord));
    if (e == cudaSuccess) e = g.flags.ensure(4, 4);
    if (e == cudaSuccess) e = g.errw.zero(g.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g.dep.at<int32_t>(), keys, n * 4, cudaMemcpyHostToDevice, g.stream);
    SortScratch ss{};
    if (e == cudaSuccess) e = sort_scratch(&g, n, &ss);
    if (e == cudaSuccess) {
        const Prog P = make_prog(&g);
        uint32_t rounds = 0;
        e = run_depth_sort(P, ss, g.stream, &rounds, nullptr);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(pos, g.pos.at<uint32_t>(), n * 4, cudaMemcpyDeviceToHost, g.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g.stream);
    if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? PTL_OOM : PTL_CUDA_ERROR;
    return check_error_word(&g);
}

ptl_status ptl_generator_snapshot(ptl_generator* g, int which, uint32_t* out, size_t capacity, size_t* count) {
    if (!g || !count) return PTL_BAD_ARGUMENT;
    const DevBuf* b = nullptr;
    size_t len = 0;
    switch (which) {
        case 0: b = &g->out; len = g->W3; break;
        case 1: b = &g->fn_start; len = g->F; break;
        case 2: b = &g->fn_end; len = g->F; break;
        case 3: b = &g->fn_size; len = g->F; break;
        case 4: b = &g->fn_id; len = g->F; break;
        case 5: b = &g->nt; len = g->n; break;
        case 6: b = &g->rt; len = g->n; break;
        case 7: b = &g->nd; len = g->n; break;
        case 8: b = &g->sizes; len = g->n; break;
        case 9: b = &g->loc; len = g->n; break;
        case 10: b = &g->fn_id; len = g->F; break;
        case 11: b = &g->fn_start0; len = g->F; break;
        case 12: b = &g->fn_end0; len = g->F; break;
        case 13: b = &g->fn_size0; len = g->F; break;
        case 14: b = &g->instr; len = g->W; break;
        case 15: b = &g->rd; len = g->W; break;
        case 16: b = &g->rs1; len = g->W; break;
        case 17: b = &g->rs2; len = g->W; break;
        case 18: b = &g->jt; len = g->W; break;
        case 19: b = &g->used_instrs; len = g->W; break;
        case 20: b = &g->ni; len = g->W2; break;
        case 21: b = &g->nrd; len = g->W2; break;
        case 22: b = &g->nr1; len = g->W2; break;
        case 23: b = &g->nr2; len = g->W2; break;
        case 24: b = &g->njt; len = g->W2; break;
        case 25: b = &g->fn_ra_start; len = g->F; break;
        case 26: b = &g->fn_ra_end; len = g->F; break;
        case 27: b = &g->fn_ra_size; len = g->F; break;
        case 40: b = &g->pos; len = g->n; break;
        case 41: b = &g->regs; len = 3 * g->n; break;
        case 42: b = &g->symreg; len = g->W; break;
        case 43: b = &g->symswp; len = g->W; break;
        default: return fail(g, PTL_BAD_ARGUMENT, "snapshot not kept by the GPU pipeline");
    }
    *count = len;
    if (!out) return PTL_OK;
    if (capacity < len) return PTL_BAD_ARGUMENT;
    if (len && b->elem == 1) {  // byte arrays (node and data types), widened
        std::vector<uint8_t> bytes(len);
        cudaError_t e = cudaMemcpyAsync(bytes.data(), b->at<uint8_t>(), len, cudaMemcpyDeviceToHost, g->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
        if (e != cudaSuccess) return cuda_fail(g, e, "snapshot");
        for (size_t k = 0; k < len; ++k) out[k] = bytes[k];
    } else if (len) {
        cudaError_t e = cudaMemcpyAsync(out, b->at<uint32_t>(), len * 4, cudaMemcpyDeviceToHost, g->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
        if (e != cudaSuccess) return cuda_fail(g, e, "snapshot");
    }
    return PTL_OK;
}

size_t ptl_code_table(int which, uint32_t* out) {
    const CodeTables& t = host_tables();
    auto flat = [&](size_t count, auto value) {
        if (out) for (size_t k = 0; k < count; ++k) out[k] = value(k);
        return count;
    };
    switch (which) {
        case 0: return flat(256 * 6, [&](size_t k) { return static_cast<uint32_t>(t.size[t.row_of[k / 6]][k % 6]); });
        case 1: return flat(256 * 24, [&](size_t k) { return ((t.has_instr[t.row_of[k / 24]][(k / 6) % 4] >> (k % 6)) & 1u) ? 0xFFFFFFFFu : 0u; });
        case 2: return flat(256 * 24, [&](size_t k) { return ((t.has_output[t.row_of[k / 24]][(k / 6) % 4] >> (k % 6)) & 1u) ? 0xFFFFFFFFu : 0u; });
        case 3: return flat(256 * 24, [&](size_t k) { return static_cast<uint32_t>(t.pai[t.row_of[k / 24]][(k / 6) % 4][k % 6]); });
        case 4: return flat(256 * 24, [&](size_t k) { return static_cast<uint32_t>(t.out[t.row_of[k / 24]][(k / 6) % 4][k % 6]); });
        case 5: return flat(256 * 24, [&](size_t k) { return t.instr[t.row_of[k / 24]][(k / 6) % 4][k % 6]; });
        case 6: return flat(256 * 4, [&](size_t k) { return static_cast<uint32_t>(t.cnst[t.row_of[k / 4]][k % 4]); });
        case 7: return flat(256 * 48, [&](size_t k) { return static_cast<uint32_t>(t.opd[t.row_of[k / 48]][(k / 12) % 4][(k / 2) % 6][k % 2]); });
        case 8: return flat(256 * 4, [&](size_t k) { return static_cast<uint32_t>(t.jt[t.row_of[k / 4]][k % 4]); });
        case 9: return flat(kNumPareasTypes, [&](size_t k) { return static_cast<uint32_t>(t.pareas_to_rv[k]); });
        default: return 0;
    }
}

ptl_status ptl_device_info(int device, char* name, size_t name_len, int* sm_count, int* cc_major, int* cc_minor) {
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return PTL_CUDA_ERROR;
    if (name && name_len) std::snprintf(name, name_len, "%s", prop.name);
    if (sm_count) *sm_count = prop.multiProcessorCount;
    if (cc_major) *cc_major = prop.major;
    if (cc_minor) *cc_minor = prop.minor;
    return PTL_OK;
}

}  // extern "C"
