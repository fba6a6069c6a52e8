// Batched pipeline (ptl_bpipe.h): the seven stages of rv_generator_avx::process
// (rv_generator_avx.cpp:104-120) for many programs at once, one launch per stage step for
// the whole batch.
//
// Every per-program array lives in an arena shared by the batch: program p's array of a
// family starts at element off[p] + 16 of the family's buffers and is followed by at
// least 80 zero elements, the same pads a single generator gives its arrays, so the
// stage functions see exactly what they see for that program alone.  Each program has
// its own Prog view (device memory); kernels cut their work into tiles that never
// straddle programs.  The host reads sizes between stages (function counts, word counts,
// steps) once per batch, and a program that fails a check drops out of the later stages
// without affecting the others.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <map>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "ptl_bpipe.h"
#include "ptl_kernels.cuh"

namespace ptl {
namespace {

constexpr uint64_t kFront = kArenaFront, kBack = kArenaBack;
inline uint64_t r8(uint64_t n) { return (n + 7) & ~uint64_t(7); }
inline uint64_t region(uint64_t count) { return arena_region(count); }

struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need) {
        if (need <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        const size_t grow = need + need / 4 + 4096;
        const cudaError_t e = cudaMalloc(&p, grow);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        bytes = grow;
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* at(uint64_t elem = 0) const { return static_cast<T*>(p) + elem; }
};

struct PBuf {  // pinned host memory
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need) {
        if (need <= bytes && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        const size_t grow = need + need / 4 + 4096;
        const cudaError_t e = cudaHostAlloc(&p, grow, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        bytes = grow;
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* at(uint64_t elem = 0) const { return static_cast<T*>(p) + elem; }
};

// Per-program regions of one array family.
struct Layout {
    std::vector<uint64_t> off;
    uint64_t total = 0;
    void build(const std::vector<uint64_t>& counts, const std::vector<uint8_t>& active) {
        off.assign(counts.size(), 0);
        total = 0;
        for (size_t p = 0; p < counts.size(); ++p) {
            off[p] = total;
            if (active[p]) total += region(counts[p]);
        }
        total += kFront + kBack;
    }
    uint64_t elem(size_t p) const { return off[p] + kFront; }
};

const CodeTables& tables() {
    static CodeTables t;
    static std::once_flag once;
    std::call_once(once, [] { build_code_tables(&t); });
    return t;
}

#define BP_CU(x)                                                     \
    do {                                                             \
        const cudaError_t e_ = (x);                                  \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x);             \
    } while (0)

void direct_host_slow(int device);  // later pipelines on the device gather through pinned memory

class Pipeline final : public BatchPipeline {
public:
    int device = 0;
    int threads = 8;
    cudaStream_t s = nullptr;
    cudaEvent_t ev[8] = {};
    cudaEvent_t ev_in = nullptr, ev_out0 = nullptr, ev_out1 = nullptr;  // input copy start, output copy
    cudaEvent_t ev_sort0 = nullptr, ev_sort1 = nullptr;  // the depth sort inside isn_gen
    uint64_t hns[3] = {0, 0, 0};
    uint64_t ns[7] = {0, 0, 0, 0, 0, 0, 0};
    uint64_t h2d = 0, d2h = 0;
    std::string err_text;

    DBuf tab;  // CodeTables
    DBuf in_type, in_rtype, in_parent, in_depth, in_child, in_data;
    DBuf nt, rt, nd1, nd, par, ci, dep, loc0, loc, pos, decl, fflag, regs;
    DBuf fn_id, fn_start, fn_size, fn_end, fn_start0, fn_size0, ra_order, lifetime;
    DBuf instr, rd, rs1, rs2, jt, used_instrs, symreg, symswp, stamp, spill, roffs, owner, used, smark, defpos;
    DBuf trig_min, trig_max, ra_chunks;
    DBuf ni, nrd, nr1, nr2, njt, joffs, out;
    DBuf errw, flags, meta, progs, tabs, lists, changed, sort_err, a_off, dirty, ra_sync;
    DBuf sa, sapos, sbpos, seg0, seg1, tile_seg, tile_l, tile_r, sort_stops, leaf, heap, counters, scan_status,
        scan_counter, sort_local, sort_equal;
    DBuf s_preserve, s_extra, s_claim, s_sregs, s_ssteps;  // the scalar generator's allocation
    bool scalar_mode = false;  // rv_generator_st's semantics for the whole batch
    PBuf h_in, h_out, h_fn, h_small, h_gp;
    DBuf d_gp;                 // host-gather parameters (source pointers, offsets, counts)
    bool direct_host = false;  // the device reads pageable host memory coherently
    uint64_t last_in_bytes = 0;  // input bytes of the last compile

    std::vector<uint8_t> active;
    std::vector<ptl_status> status;

    ~Pipeline() override {
        for (DBuf* b : all()) b->release();
        h_in.release();
        h_out.release();
        h_fn.release();
        h_small.release();
        h_gp.release();
        d_gp.release();
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t e : {ev_in, ev_out0, ev_out1, ev_sort0, ev_sort1})
            if (e) cudaEventDestroy(e);
        if (s) cudaStreamDestroy(s);
    }
    std::vector<DBuf*> all() {
        return {&tab, &in_type, &in_rtype, &in_parent, &in_depth, &in_child, &in_data, &nt, &rt, &nd1, &nd, &par,
                &ci, &dep, &loc0, &loc, &pos, &decl, &fflag, &regs, &fn_id, &fn_start, &fn_size,
                &fn_end, &fn_start0, &fn_size0, &ra_order, &lifetime, &instr, &rd, &rs1, &rs2, &jt, &used_instrs, &symreg,
                &symswp, &stamp, &spill, &roffs, &owner, &used, &smark, &defpos, &trig_min, &trig_max, &ra_chunks, &ni, &nrd,
                &nr1, &nr2, &njt, &joffs, &out, &errw, &flags, &meta, &progs, &tabs, &lists, &changed,
                &sort_err, &a_off, &dirty, &ra_sync, &sa, &sapos, &sbpos, &seg0, &seg1, &tile_seg, &tile_l, &tile_r,
                &sort_stops, &leaf, &heap, &counters, &scan_status, &scan_counter, &sort_local, &sort_equal,
                &s_preserve, &s_extra, &s_claim, &s_sregs, &s_ssteps};
    }

    ptl_status cuda_fail(cudaError_t e, const char* what) {
        err_text = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? PTL_OOM : PTL_CUDA_ERROR;
    }

    void stage_ns(uint64_t out_ns[7]) const override {
        for (int k = 0; k < 7; ++k) out_ns[k] = ns[k];
    }
    void copied_bytes(uint64_t* a, uint64_t* b) const override {
        if (a) *a = h2d;
        if (b) *b = d2h;
    }
    const char* last_error() const override { return err_text.c_str(); }
    uint64_t device_bytes() const override {
        uint64_t t = d_gp.bytes;
        for (const DBuf* b : const_cast<Pipeline*>(this)->all()) t += b->bytes;
        return t;
    }
    void release_memory() override {
        const DeviceScope on_device(device);
        for (DBuf* b : all()) b->release();
        d_gp.release();
    }
    void set_regalloc_share(double share) override { ra_share = std::min(1.0, std::max(0.05, share)); }
    void set_scalar(bool on) override { scalar_mode = on; }
    ptl_status scalar_regalloc(const std::vector<uint64_t>& F, const std::vector<uint64_t>& W,
                               const std::vector<uint64_t>& S, const Layout& Lf, const Layout& Lw, uint32_t* hfl,
                               std::vector<uint32_t>& active_list);
    bool set_tiles(uint32_t e, uint32_t w) override {
        if (!batch_tile_ok(e) || !batch_sweep_tile_ok(w)) return false;
        elem_tile = e;
        sweep_tile = w;
        return true;
    }
    void tiles(uint32_t out[2]) const override {
        out[0] = elem_tile;
        out[1] = sweep_tile;
    }
    void host_ns(uint64_t out_ns[3]) const override {
        for (int k = 0; k < 3; ++k) out_ns[k] = hns[k];
    }

    // Zeroed family of per-program arrays.
    cudaError_t family(const Layout& L, std::initializer_list<DBuf*> bufs, size_t es) {
        for (DBuf* b : bufs) {
            cudaError_t e = b->ensure(L.total * es);
            if (e == cudaSuccess) e = cudaMemsetAsync(b->p, 0, L.total * es, s);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    // A family the stages write in full (ArenaGuard): no zeroing, batch_guards clears the
    // pads.  With poison set (PTL_POISON_ARENAS=1 in the environment) its bytes are filled
    // with 0xA5 first, so a stage that read an element before writing it would show.
    bool poison = false;
    cudaError_t family_written(const Layout& L, std::initializer_list<DBuf*> bufs, size_t es) {
        for (DBuf* b : bufs) {
            cudaError_t e = b->ensure(L.total * es);
            if (e == cudaSuccess && poison) e = cudaMemsetAsync(b->p, 0xA5, L.total * es, s);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }

    // Pinned small-area slots: tile tables, lists, host copies of per-program words.
    size_t B = 0;
    uint32_t* table_slot(int k) { return h_small.at<uint32_t>(static_cast<uint64_t>(k) * (B + 1)); }
    uint32_t* dtable_slot(int k) { return tabs.at<uint32_t>(static_cast<uint64_t>(k) * (B + 1)); }

    // Tile table for per-program counts (inactive programs get none); uploads to slot k
    // and returns the total tile count.
    uint32_t tiles(int k, const std::vector<uint64_t>& counts, uint64_t tile, const std::vector<uint8_t>* only = nullptr) {
        slot_tile[k] = static_cast<uint32_t>(tile);
        uint32_t* h = table_slot(k);
        uint64_t t = 0;
        for (size_t p = 0; p < B; ++p) {
            h[p] = static_cast<uint32_t>(t);
            const bool on = active[p] && (!only || (*only)[p]);
            if (on) t += (counts[p] + tile - 1) / tile;
        }
        h[B] = static_cast<uint32_t>(t);
        cudaMemcpyAsync(dtable_slot(k), h, (B + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
        return static_cast<uint32_t>(t);
    }
    BatchLaunch bl(int k) {
        return BatchLaunch{progs.at<Prog>(), dtable_slot(k), static_cast<uint32_t>(B), s, slot_tile[k]};
    }
    // tile sizes: element-wise stages, optimize sweeps (chosen by the autotuner or the defaults)
    uint32_t elem_tile = batch_tile(), sweep_tile = 1024;
    double ra_share = 1.0;  // part of the resident blocks the persistent regalloc launch takes
    SortRoundGraph sort_graph;  // a pair of depth-sort rounds, replayed
    uint32_t slot_tile[32] = {};

    std::vector<Prog> hp;  // host copies of the views
    Prog* h_progs() { return reinterpret_cast<Prog*>(h_small.at<uint8_t>(small_progs_off)); }
    size_t small_progs_off = 0, small_meta_off = 0, small_err_off = 0, small_list_off = 0, small_up_off = 0;

    void upload_progs() {
        std::memcpy(h_progs(), hp.data(), B * sizeof(Prog));
        cudaMemcpyAsync(progs.p, h_progs(), B * sizeof(Prog), cudaMemcpyHostToDevice, s);
    }

    // Per-program error words: marks failed programs.  Syncs the stream.
    cudaError_t collect_errors() {
        ErrorWord* he = reinterpret_cast<ErrorWord*>(h_small.at<uint8_t>(small_err_off));
        cudaError_t e = cudaMemcpyAsync(he, errw.p, B * sizeof(ErrorWord), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        for (size_t p = 0; p < B; ++p) {
            if (active[p] && he[p].code != ST_OK) {
                active[p] = 0;
                status[p] = static_cast<ptl_status>(he[p].code);
            }
        }
        return cudaSuccess;
    }
    uint32_t* read_meta() {
        uint32_t* hm = reinterpret_cast<uint32_t*>(h_small.at<uint8_t>(small_meta_off));
        cudaMemcpyAsync(hm, meta.p, B * 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        return hm;
    }
    uint32_t* upload_list(int k, const std::vector<uint32_t>& v) {
        uint32_t* h = reinterpret_cast<uint32_t*>(h_small.at<uint8_t>(small_list_off)) + static_cast<uint64_t>(k) * (B + 1);
        std::copy(v.begin(), v.end(), h);
        uint32_t* d = lists.at<uint32_t>(static_cast<uint64_t>(k) * (B + 1));
        if (!v.empty()) cudaMemcpyAsync(d, h, v.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
        return d;
    }

    ptl_status compile(const ptl_ast_view* trees, size_t count, std::vector<BatchResult>& res) override;
    uint64_t sort_ns = 0;  // device time of the last compile's depth sort
    uint64_t depth_sort_ns() const override { return sort_ns; }
    uint64_t device_ns() const override {
        float ms = 0;
        return cudaEventElapsedTime(&ms, ev[0], ev[7]) == cudaSuccess ? static_cast<uint64_t>(ms * 1e6) : 0;
    }
};

// The scalar generator's register allocation (rv_generator.cpp:1213-1335) of every active
// program: each function on its own, with its preserve mask.  Programs whose functions
// share symbols take the serial order, one launch each; the others run one warp per
// function in one launch for the batch, except a program with a function longer than a
// warp's symbol bytes, which takes the tile form on its own.
ptl_status Pipeline::scalar_regalloc(const std::vector<uint64_t>& F, const std::vector<uint64_t>& W,
                                     const std::vector<uint64_t>& S, const Layout& Lf, const Layout& Lw,
                                     uint32_t* hfl, std::vector<uint32_t>& active_list) {
    BP_CU(family(Lf, {&s_preserve}, 8));
    BP_CU(family(Lw, {&s_extra}, 4));
    for (size_t p = 0; p < B; ++p) {
        hp[p].s_preserve = s_preserve.at<unsigned long long>(Lf.elem(p));
        hp[p].s_extra = s_extra.at<uint32_t>(Lw.elem(p));
    }
    upload_progs();
    const uint32_t t_w = tiles(7, W, elem_tile);
    batch_stage(BatchStage::Cross, bl(7), t_w, nullptr);  // flags[1]: functions share symbols
    BP_CU(cudaMemcpyAsync(hfl, flags.p, B * 16, cudaMemcpyDeviceToHost, s));
    BP_CU(collect_errors());
    std::vector<uint8_t> on_warp(B, 0);
    std::vector<uint32_t> serial, alone;
    uint64_t longest = 1, serial_f = 1;
    for (size_t p = 0; p < B; ++p) {
        if (!active[p]) continue;
        active_list.push_back(static_cast<uint32_t>(p));
        if (hfl[4 * p + 1]) {
            serial.push_back(static_cast<uint32_t>(p));
            serial_f = std::max(serial_f, F[p]);
        } else if (S[p] <= scalar_warp_cap()) {
            on_warp[p] = 1;
            longest = std::max(longest, S[p]);
        } else {
            alone.push_back(static_cast<uint32_t>(p));
        }
    }
    const uint32_t t_sw = tiles(16, F, scalar_warp_fns(), &on_warp);
    batch_scalar_ra_warp(bl(16), t_sw, static_cast<uint32_t>((longest + 15) & ~uint64_t(15)));
    if (!serial.empty()) {  // per program, one after another: they share the scratch
        BP_CU(s_sregs.ensure(serial_f * 64 * 4));
        BP_CU(s_ssteps.ensure(serial_f * sizeof(SRaStep)));
        for (const uint32_t p : serial)
            launch_scalar_ra_serial(hp[p], s_sregs.at<int32_t>(), s_ssteps.at<SRaStep>(), hp[p].s_preserve, s);
    }
    for (const uint32_t p : alone) launch_scalar_ra_free(hp[p], hp[p].s_preserve, s);
    BP_CU(cudaGetLastError());
    return PTL_OK;
}

ptl_status Pipeline::compile(const ptl_ast_view* trees, size_t count, std::vector<BatchResult>& res) {
    res.assign(count, BatchResult{});
    err_text.clear();
    h2d = d2h = 0;
    for (auto& x : ns) x = 0;
    if (count == 0) return PTL_OK;
    if (!trees) return PTL_BAD_ARGUMENT;
    if (count > (1u << 24)) return PTL_BAD_ARGUMENT;
    const DeviceScope on_device(device);
    BP_CU(on_device.err);
    {
        const char* pz = std::getenv("PTL_POISON_ARENAS");
        poison = pz && pz[0] == '1';
    }
    B = count;
    active.assign(B, 1);
    status.assign(B, PTL_OK);
    std::vector<uint64_t> n(B), nb8(B), n3(B);
    uint64_t ntot = 0;
    for (size_t p = 0; p < B; ++p) {
        const ptl_ast_view& t = trees[p];
        const bool ok = t.n > 0 && t.n < (1ull << 31) && t.type && t.rtype && t.parent && t.depth && t.child_idx &&
                        t.data && !t.on_device;
        if (!ok || t.max_depth == 0 || t.max_depth >= t.n) {
            active[p] = 0;
            status[p] = ok ? PTL_INVALID_AST : PTL_BAD_ARGUMENT;
            continue;
        }
        n[p] = t.n;
        nb8[p] = r8(t.n);
        n3[p] = 3 * t.n;
        ntot += t.n;
    }
    for (auto& e : ev)
        if (!e) BP_CU(cudaEventCreate(&e));
    for (cudaEvent_t* e : {&ev_in, &ev_out0, &ev_out1, &ev_sort0, &ev_sort1})
        if (!*e) BP_CU(cudaEventCreate(e));
    for (auto& x : hns) x = 0;

    // ---- small per-program state and the pinned small area
    constexpr int kTables = 23, kLists = 4;  // table slots 0..22 are used
    small_progs_off = static_cast<size_t>(kTables) * (B + 1) * 4;
    small_meta_off = small_progs_off + B * sizeof(Prog);
    small_err_off = small_meta_off + B * 16;
    small_list_off = small_err_off + B * sizeof(ErrorWord);
    small_up_off = small_list_off + static_cast<size_t>(kLists) * (B + 1) * 4;  // 8-byte aligned
    small_up_off = (small_up_off + 15) & ~size_t(15);
    BP_CU(h_small.ensure(small_up_off + B * (8 + 8 + sizeof(SortSeg) + 8 + 12) + 64));
    BP_CU(tabs.ensure(static_cast<size_t>(kTables) * (B + 1) * 4));
    BP_CU(lists.ensure(static_cast<size_t>(kLists) * (B + 1) * 4));
    BP_CU(progs.ensure(B * sizeof(Prog)));
    BP_CU(errw.ensure(B * sizeof(ErrorWord)));
    BP_CU(flags.ensure(B * 16));
    BP_CU(meta.ensure(B * 16));
    BP_CU(changed.ensure(16));
    BP_CU(sort_err.ensure(sizeof(ErrorWord)));
    BP_CU(cudaMemsetAsync(errw.p, 0, B * sizeof(ErrorWord), s));
    BP_CU(cudaMemsetAsync(flags.p, 0, B * 16, s));
    BP_CU(cudaMemsetAsync(meta.p, 0, B * 16, s));
    BP_CU(cudaMemsetAsync(sort_err.p, 0, sizeof(ErrorWord), s));
    if (!tab.p) {
        BP_CU(tab.ensure(sizeof(CodeTables)));
        BP_CU(cudaMemcpyAsync(tab.p, &tables(), sizeof(CodeTables), cudaMemcpyHostToDevice, s));
        BP_CU(cudaStreamSynchronize(s));
    }

    // ---- inputs.  A program's input region starts at a multiple of 16 elements.  On a
    // device with coherent access to pageable host memory a kernel reads the caller's
    // arrays directly; otherwise host threads gather them into pinned memory, one copy per
    // field and chunk, and a chunk's copies start as soon as its programs are gathered, so
    // the copy engine runs under the gather of the next chunks
    {
        std::vector<uint64_t> din(B + 1);
        uint64_t o = 0, nodes_in = 0;
        for (size_t p = 0; p < B; ++p) {
            din[p] = o;
            if (active[p]) {
                o += (n[p] + 15) & ~uint64_t(15);
                nodes_in += n[p];
            }
        }
        din[B] = o;
        const uint64_t cap = std::max<uint64_t>(o, 16);
        BP_CU(in_type.ensure(cap));
        BP_CU(in_rtype.ensure(cap));
        BP_CU(in_parent.ensure(cap * 4));
        BP_CU(in_depth.ensure(cap * 4));
        BP_CU(in_child.ensure(cap * 4));
        BP_CU(in_data.ensure(cap * 4));
        if (direct_host) {
            const auto g0 = std::chrono::steady_clock::now();
            BP_CU(h_gp.ensure(B * 8 * 8));
            BP_CU(d_gp.ensure(B * 8 * 8));
            const void** hsrc = reinterpret_cast<const void**>(h_gp.p);  // [6][B]
            uint64_t* hdin = reinterpret_cast<uint64_t*>(hsrc + 6 * B);
            uint64_t* hn = hdin + B;
            for (size_t p = 0; p < B; ++p) {
                const ptl_ast_view& t = trees[p];
                const void* f[6] = {t.type, t.rtype, t.parent, t.depth, t.child_idx, t.data};
                for (int k = 0; k < 6; ++k) hsrc[k * B + p] = f[k];
                hdin[p] = din[p];
                hn[p] = active[p] ? n[p] : 0;
            }
            BP_CU(cudaMemcpyAsync(d_gp.p, h_gp.p, B * 8 * 8, cudaMemcpyHostToDevice, s));
            const uint32_t t_g = tiles(18, n, kGatherTile);
            hns[0] = static_cast<uint64_t>(std::chrono::duration_cast<std::chrono::nanoseconds>(
                                               std::chrono::steady_clock::now() - g0).count());
            BP_CU(cudaEventRecord(ev_in, s));
            const void* const* dsrc = static_cast<const void* const*>(d_gp.p);
            const uint64_t* ddin = reinterpret_cast<const uint64_t*>(dsrc + 6 * B);
            uint8_t* dsts[6] = {in_type.at<uint8_t>(), in_rtype.at<uint8_t>(), in_parent.at<uint8_t>(),
                                in_depth.at<uint8_t>(), in_child.at<uint8_t>(), in_data.at<uint8_t>()};
            for (int k = 0; k < 6; ++k)
                batch_gather_host(bl(18), t_g, HostGather{dsrc + k * B, ddin, ddin + B, dsts[k], k < 2 ? 1u : 4u});
        } else {
            const size_t bytes = cap * (1 + 1 + 4 + 4 + 4 + 4);
            BP_CU(h_in.ensure(bytes));
            uint8_t* ht = h_in.at<uint8_t>();
            uint8_t* hr = ht + cap;
            int32_t* hpar = reinterpret_cast<int32_t*>(hr + cap);
            int32_t* hdep = hpar + cap;
            int32_t* hch = hdep + cap;
            uint32_t* hdat = reinterpret_cast<uint32_t*>(hch + cap);
            // chunks of about o / kInChunks nodes, cut at program boundaries
            constexpr size_t kInChunks = 8;
            std::vector<size_t> cfirst{0};
            std::vector<uint32_t> chunk_of(B);
            for (size_t p = 0; p < B; ++p) {
                const size_t c = cfirst.size() - 1;
                chunk_of[p] = static_cast<uint32_t>(c);
                if (p + 1 < B && cfirst.size() < kInChunks && din[p + 1] * kInChunks >= o * cfirst.size())
                    cfirst.push_back(p + 1);
            }
            const size_t C = cfirst.size();
            cfirst.push_back(B);
            std::vector<std::atomic<uint32_t>> left(C);
            for (size_t c = 0; c < C; ++c) {
                uint32_t k = 0;
                for (size_t p = cfirst[c]; p < cfirst[c + 1]; ++p) k += active[p] ? 1u : 0u;
                left[c].store(k, std::memory_order_relaxed);
            }
            std::atomic<size_t> next{0};
            const auto g0 = std::chrono::steady_clock::now();
            const int nt_ = std::max(1, std::min<int>(threads, static_cast<int>(B)));
            std::vector<std::thread> pool;
            for (int w = 0; w < nt_; ++w) {
                pool.emplace_back([&] {
                    for (size_t p = next.fetch_add(1, std::memory_order_relaxed); p < B;
                         p = next.fetch_add(1, std::memory_order_relaxed)) {
                        if (!active[p]) continue;
                        const ptl_ast_view& t = trees[p];
                        const uint64_t d = din[p];
                        std::memcpy(ht + d, t.type, n[p]);
                        std::memcpy(hr + d, t.rtype, n[p]);
                        std::memcpy(hpar + d, t.parent, 4 * n[p]);
                        std::memcpy(hdep + d, t.depth, 4 * n[p]);
                        std::memcpy(hch + d, t.child_idx, 4 * n[p]);
                        std::memcpy(hdat + d, t.data, 4 * n[p]);
                        left[chunk_of[p]].fetch_sub(1, std::memory_order_release);
                    }
                });
            }
            // every program is gathered by some worker, so each chunk's count reaches zero
            cudaError_t ce = cudaEventRecord(ev_in, s);
            for (size_t c = 0; c < C && ce == cudaSuccess; ++c) {
                while (left[c].load(std::memory_order_acquire) != 0) std::this_thread::yield();
                const uint64_t a = din[cfirst[c]], m = din[cfirst[c + 1]] - a;
                if (m == 0) continue;
                for (auto [dst, src, w] : {std::tuple<void*, const void*, uint64_t>{in_type.p, ht, 1},
                                           {in_rtype.p, hr, 1},
                                           {in_parent.p, hpar, 4},
                                           {in_depth.p, hdep, 4},
                                           {in_child.p, hch, 4},
                                           {in_data.p, hdat, 4}}) {
                    ce = cudaMemcpyAsync(static_cast<uint8_t*>(dst) + w * a, static_cast<const uint8_t*>(src) + w * a,
                                         w * m, cudaMemcpyHostToDevice, s);
                    if (ce != cudaSuccess) break;
                }
            }
            for (auto& t : pool) t.join();
            hns[0] = static_cast<uint64_t>(std::chrono::duration_cast<std::chrono::nanoseconds>(
                                               std::chrono::steady_clock::now() - g0).count());
            BP_CU(ce);
        }
        h2d += 18 * nodes_in;
        last_in_bytes = 18 * nodes_in;
        BP_CU(cudaEventRecord(ev[0], s));  // stage times start with the inputs on the device

        // node, register and depth families
        Layout Ln, Lr;
        Ln.build(nb8, active);
        Lr.build(n3, active);
        BP_CU(family_written(Ln, {&nd1, &nd, &par, &ci, &dep, &loc0, &loc}, 4));
        BP_CU(family_written(Ln, {&nt, &rt, &fflag}, 1));
        BP_CU(family(Ln, {&pos, &decl}, 4));
        BP_CU(family(Lr, {&regs}, 4));
        hp.assign(B, Prog{});
        for (size_t p = 0; p < B; ++p) {
            Prog& P = hp[p];
            P.n = static_cast<uint32_t>(n[p]);
            P.nb8 = static_cast<uint32_t>(nb8[p]);
            P.max_depth = static_cast<uint32_t>(trees[p].max_depth);
            P.in_type = in_type.at<uint8_t>(din[p]);
            P.in_rtype = in_rtype.at<uint8_t>(din[p]);
            P.in_parent = in_parent.at<int32_t>(din[p]);
            P.in_depth = in_depth.at<int32_t>(din[p]);
            P.in_child = in_child.at<int32_t>(din[p]);
            P.in_data = in_data.at<uint32_t>(din[p]);
            const uint64_t e = Ln.elem(p);
            P.nt = nt.at<uint8_t>(e);
            P.rt = rt.at<uint8_t>(e);
            P.nd1 = nd1.at<uint32_t>(e);
            P.nd = nd.at<uint32_t>(e);
            P.par = par.at<int32_t>(e);
            P.ci = ci.at<int32_t>(e);
            P.dep = dep.at<int32_t>(e);
            P.loc0 = loc0.at<uint32_t>(e);
            P.loc = loc.at<uint32_t>(e);
            P.pos = pos.at<uint32_t>(e);
            P.decl = decl.at<uint32_t>(e);
            P.fflag = fflag.at<uint8_t>(e);
            P.regs = regs.at<uint32_t>(Lr.elem(p));
            P.tab.t = tab.at<CodeTables>();
            P.err = errw.at<ErrorWord>(p);
            P.flags = flags.at<uint32_t>(4 * p);
            P.scalar = scalar_mode ? 1u : 0u;
        }
        upload_progs();

        // ---- input checks and copy, one pass; then preprocess on the valid programs
        {
            std::vector<uint64_t> gc(B);
            for (size_t p = 0; p < B; ++p) gc[p] = region(nb8[p]) - nb8[p];
            const uint32_t t_g = tiles(0, gc, elem_tile);
            batch_guards(ArenaGuard::Nodes, bl(0), t_g);
        }
        const uint32_t t_in = tiles(19, nb8, elem_tile);
        batch_stage(BatchStage::Ingest, bl(19), t_in, nullptr);
        {
            uint32_t* hfl = reinterpret_cast<uint32_t*>(h_small.at<uint8_t>(small_meta_off));
            BP_CU(cudaMemcpyAsync(hfl, flags.p, B * 16, cudaMemcpyDeviceToHost, s));
            BP_CU(collect_errors());
            for (size_t p = 0; p < B; ++p) {
                if (active[p] && !hfl[4 * p + 3]) {  // depths 0..max_depth must all be populated
                    active[p] = 0;
                    status[p] = PTL_INVALID_AST;
                }
            }
        }
        const uint32_t t_nb8 = tiles(1, nb8, elem_tile);
        batch_stage(scalar_mode ? BatchStage::PreprocessScalar : BatchStage::Preprocess, bl(1), t_nb8, nullptr);
        BP_CU(cudaEventRecord(ev[1], s));

        // ---- isn_cnt
        const uint32_t st_nb8 = tiles(2, nb8, batch_scan_tile());
        BP_CU(scan_status.ensure((static_cast<size_t>(st_nb8) + 8) * 8));
        BP_CU(scan_counter.ensure(16));
        ScanScratch sc{scan_status.at<unsigned long long>(), scan_counter.at<uint32_t>(), st_nb8 + 8};
        batch_scan(BatchScan::Count, bl(2), st_nb8, sc, nullptr);
        batch_stage(BatchStage::Fix, bl(1), t_nb8, nullptr);
        batch_scan(BatchScan::Decl, bl(2), st_nb8, sc, meta.at<uint32_t>());
        uint32_t* hm = read_meta();
        BP_CU(collect_errors());
        std::vector<uint64_t> F(B), fb8(B), fr(B);
        for (size_t p = 0; p < B; ++p) {
            if (!active[p]) continue;
            F[p] = hm[4 * p];
            if (F[p] == 0) {  // the reference takes the max of an empty range
                active[p] = 0;
                status[p] = PTL_UNSUPPORTED;
                continue;
            }
            fb8[p] = r8(F[p]);
            fr[p] = fb8[p] + 8;
        }
        Layout Lf;
        Lf.build(fr, active);
        BP_CU(family(Lf, {&fn_id, &fn_start, &fn_size, &fn_end, &fn_start0, &fn_size0, &ra_order}, 4));
        BP_CU(family(Lf, {&lifetime}, 8));
        for (size_t p = 0; p < B; ++p) {
            Prog& P = hp[p];
            P.F = static_cast<uint32_t>(F[p]);
            P.fb8 = static_cast<uint32_t>(fb8[p]);
            const uint64_t e = Lf.elem(p);
            P.fn_id = fn_id.at<uint32_t>(e);
            P.fn_start = fn_start.at<uint32_t>(e);
            P.fn_size = fn_size.at<uint32_t>(e);
            P.fn_end = fn_end.at<uint32_t>(e);
            P.fn_start0 = fn_start0.at<uint32_t>(e);
            P.fn_size0 = fn_size0.at<uint32_t>(e);
            P.ra_order = ra_order.at<uint32_t>(e);
            P.lifetime = lifetime.at<unsigned long long>(e);
        }
        upload_progs();
        const uint32_t t_fb8 = tiles(3, fb8, elem_tile);
        batch_stage(BatchStage::Functab, bl(3), t_fb8, meta.at<uint32_t>());
        hm = read_meta();
        BP_CU(collect_errors());
        std::vector<uint64_t> W(B), wb8(B), S(B), trig(B);
        uint32_t min_lg = 31, max_lg = 1;
        for (size_t p = 0; p < B; ++p) {
            if (!active[p]) continue;
            W[p] = hm[4 * p + 1];
            S[p] = hm[4 * p + 2];
            wb8[p] = r8(W[p]);
            trig[p] = std::max<uint64_t>(S[p], 1) * 64;
            if (W[p] == 0) {
                active[p] = 0;
                status[p] = PTL_UNSUPPORTED;
            }
        }
        BP_CU(cudaEventRecord(ev[2], s));

        // ---- isn_gen: depth order of every program in one introsort run, then the writes
        Layout Lw;
        Lw.build(wb8, active);
        BP_CU(family(Lw, {&instr, &rd, &rs1, &rs2, &jt, &symreg, &symswp, &stamp}, 4));
        BP_CU(family_written(Lw, {&used_instrs, &spill, &roffs}, 4));
        BP_CU(family(Lw, {&owner}, 8));
        BP_CU(family(Lw, {&used, &smark, &defpos}, 1));
        for (size_t p = 0; p < B; ++p) {
            Prog& P = hp[p];
            P.W = static_cast<uint32_t>(W[p]);
            P.wb8 = static_cast<uint32_t>(wb8[p]);
            P.S = static_cast<uint32_t>(S[p]);
            const uint64_t e = Lw.elem(p);
            P.instr = instr.at<uint32_t>(e);
            P.rd = rd.at<uint32_t>(e);
            P.rs1 = rs1.at<uint32_t>(e);
            P.rs2 = rs2.at<uint32_t>(e);
            P.jt = jt.at<uint32_t>(e);
            P.used_instrs = used_instrs.at<uint32_t>(e);
            P.symreg = symreg.at<uint32_t>(e);
            P.symswp = symswp.at<uint32_t>(e);
            P.stamp = stamp.at<uint32_t>(e);
            P.spill = spill.at<uint32_t>(e);
            P.roffs = roffs.at<uint32_t>(e);
            P.owner = owner.at<unsigned long long>(e);
            P.used = used.at<uint8_t>(e);
            P.smark = smark.at<uint8_t>(e);
            P.defpos = defpos.at<uint8_t>(e);
        }
        upload_progs();
        {
            std::vector<uint64_t> gc(B);
            for (size_t p = 0; p < B; ++p) gc[p] = region(wb8[p]) - W[p];
            const uint32_t t_g = tiles(20, gc, elem_tile);
            batch_guards(ArenaGuard::Words, bl(20), t_g);
        }
        // sort scratch over all active programs' nodes
        std::vector<uint64_t> aoff(B);
        uint64_t at = 0, seg_cap = 16, tile_cap = 16, leaf_cap = 16;
        std::vector<SortSeg> segs;
        std::vector<uint32_t> leaves, blocks;
        for (size_t p = 0; p < B; ++p) {
            aoff[p] = at;
            if (!active[p]) continue;
            const uint64_t np = n[p];
            seg_cap += np / 17 + 16;
            // a round's segments are disjoint and longer than kSortBlock: at most
            // np / kSortBlock of them, each with one partial tile
            tile_cap += np / kSortTile + np / kSortBlock + 16;
            leaf_cap += np / 2 + 16;
            if (np > kSortBlock) {
                SortSeg g{};
                g.first = static_cast<uint32_t>(at);
                g.last = static_cast<uint32_t>(at + np);
                g.dl = 2u * floor_log2(static_cast<uint32_t>(np));
                segs.push_back(g);
                const uint32_t lg = floor_log2(static_cast<uint32_t>(np));
                min_lg = std::min(min_lg, lg);
                max_lg = std::max(max_lg, lg);
            } else if (np > kSortThreshold) {  // one block sorts the whole program
                blocks.push_back(static_cast<uint32_t>(at));
                blocks.push_back(static_cast<uint32_t>(at + np));
                blocks.push_back(2u * floor_log2(static_cast<uint32_t>(np)));
            } else if (np > 1) {
                leaves.push_back(static_cast<uint32_t>(at));
                leaves.push_back(static_cast<uint32_t>(at + np));
            }
            at += np;
        }
        if (at >= (1ull << 32)) return cuda_fail(cudaErrorInvalidValue, "batch larger than 2^32 nodes");
        BP_CU(sa.ensure(std::max<uint64_t>(at, 1) * 8));
        BP_CU(sapos.ensure(std::max<uint64_t>(at, 1) * 4));
        BP_CU(sbpos.ensure(std::max<uint64_t>(at, 1) * 4));
        BP_CU(seg0.ensure(seg_cap * sizeof(SortSeg)));
        BP_CU(seg1.ensure(seg_cap * sizeof(SortSeg)));
        BP_CU(tile_seg.ensure(tile_cap * 4));
        BP_CU(tile_l.ensure(tile_cap * 4));
        BP_CU(tile_r.ensure(tile_cap * 4));
        BP_CU(sort_stops.ensure(tile_cap * 2 * (kSortTile / 32) * 4));
        BP_CU(leaf.ensure(2 * leaf_cap * 4));
        BP_CU(heap.ensure(2 * leaf_cap * 4));
        BP_CU(counters.ensure(64));
        BP_CU(sort_local.ensure(3 * seg_cap * 4));
        BP_CU(sort_equal.ensure(2 * seg_cap * 4));
        BP_CU(a_off.ensure(B * 8));
        uint64_t* up_aoff = reinterpret_cast<uint64_t*>(h_small.at<uint8_t>(small_up_off + B * 8));
        std::copy(aoff.begin(), aoff.end(), up_aoff);
        BP_CU(cudaMemcpyAsync(a_off.p, up_aoff, B * 8, cudaMemcpyHostToDevice, s));
        SortScratch ss{};
        ss.a = sa.at<unsigned long long>();
        ss.apos = sapos.at<uint32_t>();
        ss.bpos = sbpos.at<uint32_t>();
        ss.seg[0] = seg0.at<SortSeg>();
        ss.seg[1] = seg1.at<SortSeg>();
        // capacities as allocated: the captured round graph bakes them in, and they change
        // only when a buffer is reallocated, not with each batch's sizes
        ss.seg_cap = static_cast<uint32_t>(std::min<uint64_t>(
            {seg0.bytes / sizeof(SortSeg), seg1.bytes / sizeof(SortSeg), sort_local.bytes / 12, sort_equal.bytes / 8,
             UINT32_MAX}));
        ss.tile_seg = tile_seg.at<uint32_t>();
        ss.tile_l = tile_l.at<uint32_t>();
        ss.tile_r = tile_r.at<uint32_t>();
        ss.stops = sort_stops.at<uint32_t>();
        ss.tile_cap = static_cast<uint32_t>(std::min<uint64_t>(
            {tile_seg.bytes / 4, tile_l.bytes / 4, tile_r.bytes / 4, sort_stops.bytes / (8 * (kSortTile / 32)),
             UINT32_MAX}));
        ss.leaf = leaf.at<uint32_t>();
        ss.heap = heap.at<uint32_t>();
        ss.leaf_cap = static_cast<uint32_t>(std::min<uint64_t>({leaf.bytes / 8, heap.bytes / 8, UINT32_MAX}));
        ss.counters = counters.at<uint32_t>();
        ss.local = sort_local.at<uint32_t>();
        ss.equal = sort_equal.at<uint32_t>();
        const uint32_t t_n2 = tiles(4, n, elem_tile);
        BP_CU(cudaEventRecord(ev_sort0, s));
        batch_sort_keys(bl(4), t_n2, sa.at<unsigned long long>(), a_off.at<uint64_t>(), false);
        BP_CU(cudaMemsetAsync(counters.p, 0, 64, s));
        SortSeg* up_segs = reinterpret_cast<SortSeg*>(h_small.at<uint8_t>(small_up_off + 2 * B * 8));
        uint32_t* up_leaves = reinterpret_cast<uint32_t*>(h_small.at<uint8_t>(small_up_off + 2 * B * 8 + B * sizeof(SortSeg)));
        uint32_t* up_nl = up_leaves + 2 * B;
        uint32_t* up_blocks = up_nl + 4;
        uint32_t* up_nb = up_blocks + 3 * B;
        if (!blocks.empty()) {
            std::copy(blocks.begin(), blocks.end(), up_blocks);
            *up_nb = static_cast<uint32_t>(blocks.size() / 3);
            BP_CU(cudaMemcpyAsync(sort_local.p, up_blocks, blocks.size() * 4, cudaMemcpyHostToDevice, s));
            BP_CU(cudaMemcpyAsync(counters.at<uint32_t>(6), up_nb, 4, cudaMemcpyHostToDevice, s));
        }
        if (!segs.empty()) {
            std::copy(segs.begin(), segs.end(), up_segs);
            BP_CU(cudaMemcpyAsync(seg0.p, up_segs, segs.size() * sizeof(SortSeg), cudaMemcpyHostToDevice, s));
        }
        if (!leaves.empty()) {
            std::copy(leaves.begin(), leaves.end(), up_leaves);
            *up_nl = static_cast<uint32_t>(leaves.size() / 2);
            BP_CU(cudaMemcpyAsync(leaf.p, up_leaves, leaves.size() * 4, cudaMemcpyHostToDevice, s));
            BP_CU(cudaMemcpyAsync(counters.at<uint32_t>(2), up_nl, 4, cudaMemcpyHostToDevice, s));
        }
        uint32_t rounds = 0;
        const uint32_t lb = floor_log2(kSortBlock);
        BP_CU(run_sort_rounds(ss, static_cast<uint32_t>(segs.size()), min_lg > lb ? min_lg - lb : 1, 2 * max_lg + 4,
                              sort_err.at<ErrorWord>(), s, &rounds, &sort_graph));
        batch_sort_keys(bl(4), t_n2, sa.at<unsigned long long>(), a_off.at<uint64_t>(), true);
        BP_CU(cudaEventRecord(ev_sort1, s));
        batch_stage(scalar_mode ? BatchStage::GenScalar : BatchStage::Gen, bl(4), t_n2, nullptr);
        {
            ErrorWord se{};
            BP_CU(cudaMemcpyAsync(&se, sort_err.p, sizeof(se), cudaMemcpyDeviceToHost, s));
            BP_CU(collect_errors());
            if (se.code != ST_OK) return cuda_fail(cudaErrorLaunchFailure, "depth order");
        }
        BP_CU(cudaEventRecord(ev[3], s));

        // ---- optimize
        const uint32_t t_wb8 = tiles(5, wb8, elem_tile);
        BP_CU(cudaMemsetAsync(changed.p, 0, 8, s));
        // the marks, and whether some virtual result is not its instruction's own word
        batch_stage(BatchStage::OptMark, bl(5), t_wb8, changed.at<uint32_t>(1));
        uint32_t* hflag = reinterpret_cast<uint32_t*>(h_small.at<uint8_t>(small_meta_off));  // B*16 >= 8
        // sweeps after the first revisit only the tiles whose marks changed (when every
        // virtual result is its instruction's own word; else every tile, every sweep);
        // they have their own tile size
        const uint32_t t_sw = tiles(17, wb8, sweep_tile);
        BP_CU(dirty.ensure(2ull * t_sw + 64));
        BP_CU(cudaMemcpyAsync(hflag + 1, changed.at<uint32_t>(1), 4, cudaMemcpyDeviceToHost, s));
        BP_CU(cudaStreamSynchronize(s));
        const bool worklist = hflag[1] == 0;
        // a worklist holds one byte per tile and, after them, whether any tile is marked
        uint8_t* dbuf[2] = {dirty.at<uint8_t>(), dirty.at<uint8_t>(t_sw + 32)};
        BP_CU(cudaMemsetAsync(dbuf[0], 1, t_sw + 1, s));
        BP_CU(cudaMemsetAsync(dbuf[1], 0, t_sw + 1, s));
        int cur = 0;
        for (uint32_t sweeps = 0;;) {
            BP_CU(cudaMemsetAsync(changed.p, 0, 4, s));
            for (int k = 0; k < 4; ++k) {
                batch_sweep(bl(17), t_sw, changed.at<uint32_t>(), worklist ? dbuf[cur] : nullptr, dbuf[cur ^ 1]);
                BP_CU(cudaMemsetAsync(dbuf[cur], 0, t_sw + 1, s));
                cur ^= 1;
            }
            sweeps += 4;
            BP_CU(cudaMemcpyAsync(hflag, changed.p, 4, cudaMemcpyDeviceToHost, s));
            BP_CU(cudaStreamSynchronize(s));
            if (!*hflag) break;
            if (sweeps > 64u + 4u * static_cast<uint32_t>(*std::max_element(W.begin(), W.end()))) break;
        }
        batch_stage(BatchStage::OptFinal, bl(5), t_wb8, nullptr);
        BP_CU(collect_errors());
        BP_CU(cudaEventRecord(ev[4], s));

        // ---- regalloc
        std::vector<uint32_t> active_list;
        uint32_t* hfl = reinterpret_cast<uint32_t*>(h_small.at<uint8_t>(small_meta_off));
        if (scalar_mode) {
            const ptl_status sr = scalar_regalloc(F, W, S, Lf, Lw, hfl, active_list);
            if (sr != PTL_OK) return sr;
        } else {
        const uint32_t t_f = tiles(6, F, elem_tile);
        batch_stage(BatchStage::InitLifetime, bl(6), t_f, nullptr);
        Layout Lt, Lc;
        Lt.build(trig, active);
        std::vector<uint64_t> chunk_words(B);
        for (size_t p = 0; p < B; ++p) chunk_words[p] = 2 * (S[p] / 32 + 2);
        Lc.build(chunk_words, active);
        BP_CU(trig_min.ensure(Lt.total * 4));
        BP_CU(trig_max.ensure(Lt.total * 4));
        BP_CU(cudaMemsetAsync(trig_min.p, 0xFF, Lt.total * 4, s));
        BP_CU(cudaMemsetAsync(trig_max.p, 0, Lt.total * 4, s));
        BP_CU(family(Lc, {&ra_chunks}, 4));
        for (size_t p = 0; p < B; ++p) {
            hp[p].trig_min = trig_min.at<uint32_t>(Lt.elem(p));
            hp[p].trig_max = trig_max.at<uint32_t>(Lt.elem(p));
            hp[p].ra_chunks = ra_chunks.at<uint32_t>(Lc.elem(p));
        }
        upload_progs();
        const uint32_t t_w = tiles(7, W, elem_tile);
        batch_stage(BatchStage::Cross, bl(7), t_w, nullptr);
        BP_CU(cudaMemcpyAsync(hfl, flags.p, B * 16, cudaMemcpyDeviceToHost, s));
        BP_CU(collect_errors());
        std::vector<uint32_t> lane0_list, serial_list, wide_list;
        std::vector<uint8_t> lane0(B, 0);
        std::vector<uint64_t> nfree(B, 0);
        uint32_t max_g0 = 1;
        for (size_t p = 0; p < B; ++p) {
            if (!active[p]) continue;
            active_list.push_back(static_cast<uint32_t>(p));
            const uint64_t g0 = (F[p] + 7) / 8;
            if (hfl[4 * p + 1] || g0 > 8192) {  // functions share symbols: the serial order
                serial_list.push_back(static_cast<uint32_t>(p));
                continue;
            }
            if (hfl[4 * p + 2]) hp[p].defpos = nullptr;  // a register with two definitions: hash row 0
            if (g0 > kRaClusterMin && ra_cluster_fits(static_cast<uint32_t>(g0))) {
                wide_list.push_back(static_cast<uint32_t>(p));  // its own launches, on a cluster
                continue;
            }
            lane0[p] = 1;
            lane0_list.push_back(static_cast<uint32_t>(p));
            nfree[p] = F[p] - g0;
            max_g0 = std::max<uint32_t>(max_g0, static_cast<uint32_t>(g0));
        }
        upload_progs();
        // independent functions and lane-0 passes of all programs in one persistent launch,
        // longest programs (most steps) first
        std::stable_sort(lane0_list.begin(), lane0_list.end(), [&](uint32_t x, uint32_t y) { return S[x] > S[y]; });
        const uint32_t ra_T = batch_ra_threads(max_g0);
        uint32_t ra_items = 0;  // per program: its independent-function tiles, then its lane-0 pass
        {
            uint32_t* h = table_slot(8);
            for (size_t k = 0; k < lane0_list.size(); ++k) {
                h[k] = ra_items;
                ra_items += static_cast<uint32_t>((nfree[lane0_list[k]] + ra_T - 1) / ra_T) + 1u;
            }
            for (size_t k = lane0_list.size(); k <= B; ++k) h[k] = ra_items;
            BP_CU(cudaMemcpyAsync(dtable_slot(8), h, (B + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        }
        const uint32_t* d_lane0 = upload_list(0, lane0_list);
        batch_free_order(progs.at<Prog>(), d_lane0, static_cast<uint32_t>(lane0_list.size()), s);
        BP_CU(ra_sync.ensure(64));
        // per program: histogram of the independent functions' last chunks, then counts
        const uint32_t t_hist = tiles(16, nfree, elem_tile, &lane0);
        batch_stage(BatchStage::RaHist, bl(16), t_hist, nullptr);
        BP_CU(batch_regalloc(progs.at<Prog>(), dtable_slot(8), d_lane0, static_cast<uint32_t>(lane0_list.size()),
                             ra_items, max_g0, ra_sync.at<uint32_t>(), s, ra_share));
        const uint32_t* d_serial = upload_list(1, serial_list);
        batch_serial(progs.at<Prog>(), d_serial, static_cast<uint32_t>(serial_list.size()), s);
        for (const uint32_t p : wide_list) {
            Prog Pfree = hp[p];
            Pfree.defpos = nullptr;  // the independent functions never need definition positions
            bool launched = false;
            BP_CU(launch_ra_wide(hp[p], Pfree, static_cast<uint32_t>((F[p] + 7) / 8), s, &launched));
            if (!launched) return cuda_fail(cudaErrorLaunchFailure, "lane-0 cluster pass");
        }
        }  // the AVX generator's allocation
        const uint32_t t_w_sp = tiles(13, W, elem_tile);
        batch_stage(BatchStage::Spill, bl(13), t_w_sp, nullptr);
        if (scalar_mode) {  // preserve counts at each function's two preserve positions
            const uint32_t t_fp = tiles(6, F, elem_tile);
            batch_stage(BatchStage::SPreserveCounts, bl(6), t_fp, nullptr);
        }
        const uint32_t st_wb8 = tiles(9, wb8, batch_scan_tile());
        BP_CU(scan_status.ensure((static_cast<size_t>(st_wb8) + 8) * 8));
        sc = ScanScratch{scan_status.at<unsigned long long>(), scan_counter.at<uint32_t>(), st_wb8 + 8};
        batch_scan(scalar_mode ? BatchScan::SRaCount : BatchScan::RaCount, bl(9), st_wb8, sc, nullptr);
        const uint32_t* d_active = upload_list(2, active_list);
        batch_sizes(false, progs.at<Prog>(), d_active, static_cast<uint32_t>(active_list.size()), meta.at<uint32_t>(), s);
        hm = read_meta();
        BP_CU(collect_errors());
        std::vector<uint64_t> W2(B), w2b8(B), w2r(B);
        for (size_t p = 0; p < B; ++p) {
            if (!active[p]) continue;
            W2[p] = hm[4 * p];
            w2b8[p] = r8(W2[p]);
            w2r[p] = w2b8[p] + 16;
        }
        Layout L2;
        L2.build(w2r, active);
        BP_CU(family(L2, {&ni, &nrd, &nr1, &nr2, &njt}, 4));
        BP_CU(family_written(L2, {&joffs}, 4));
        if (scalar_mode) BP_CU(family(L2, {&s_claim}, 8));  // the frame writes' claims, zeroed
        for (size_t p = 0; p < B; ++p) {
            Prog& P = hp[p];
            P.W2 = static_cast<uint32_t>(W2[p]);
            P.w2b8 = static_cast<uint32_t>(w2b8[p]);
            const uint64_t e = L2.elem(p);
            P.ni = ni.at<uint32_t>(e);
            P.nrd = nrd.at<uint32_t>(e);
            P.nr1 = nr1.at<uint32_t>(e);
            P.nr2 = nr2.at<uint32_t>(e);
            P.njt = njt.at<uint32_t>(e);
            P.joffs = joffs.at<uint32_t>(e);
            if (scalar_mode) P.s_claim = s_claim.at<unsigned long long>(e);
        }
        upload_progs();
        {
            std::vector<uint64_t> gc(B);
            for (size_t p = 0; p < B; ++p) gc[p] = region(w2r[p]) - w2b8[p];
            const uint32_t t_g = tiles(21, gc, elem_tile);
            batch_guards(ArenaGuard::Words2, bl(21), t_g);
        }
        const uint32_t t_wb8_sc = tiles(14, wb8, elem_tile);
        batch_stage(scalar_mode ? BatchStage::SScatter : BatchStage::Scatter, bl(14), t_wb8_sc, nullptr);
        if (scalar_mode) {
            const uint32_t t_f2 = tiles(10, F, elem_tile);
            batch_stage(BatchStage::SFunctab, bl(10), t_f2, nullptr);
            std::vector<uint64_t> f3(B);
            for (size_t p = 0; p < B; ++p) f3[p] = 3 * F[p];
            const uint32_t t_f3 = tiles(22, f3, elem_tile);
            batch_stage(BatchStage::SFrames, bl(22), t_f3, nullptr);
        } else {
            const uint32_t t_f2 = tiles(10, F, elem_tile);
            batch_stage(BatchStage::RaFunctab, bl(10), t_f2, nullptr);
        }
        BP_CU(cudaEventRecord(ev[5], s));

        // ---- fix_jumps (+ postprocess)
        const uint32_t st_w2 = tiles(11, w2b8, batch_scan_tile());
        BP_CU(scan_status.ensure((static_cast<size_t>(st_w2) + 8) * 8));
        sc = ScanScratch{scan_status.at<unsigned long long>(), scan_counter.at<uint32_t>(), st_w2 + 8};
        batch_scan(BatchScan::FjSize, bl(11), st_w2, sc, nullptr);
        std::vector<uint32_t> active_now;  // programs still running after regalloc
        for (size_t p = 0; p < B; ++p)
            if (active[p]) active_now.push_back(static_cast<uint32_t>(p));
        const uint32_t* d_active2 = upload_list(3, active_now);
        batch_sizes(true, progs.at<Prog>(), d_active2, static_cast<uint32_t>(active_now.size()), meta.at<uint32_t>(), s);
        hm = read_meta();
        BP_CU(collect_errors());
        std::vector<uint64_t> W3(B), w3r(B);
        for (size_t p = 0; p < B; ++p) {
            if (!active[p]) continue;
            W3[p] = hm[4 * p + 1];
            w3r[p] = r8(W3[p]) + 8;
        }
        Layout Lo;
        Lo.build(w3r, active);
        BP_CU(family_written(Lo, {&out}, 4));  // fix_jumps writes words [0, W3); only those are read
        for (size_t p = 0; p < B; ++p) {
            hp[p].W3 = static_cast<uint32_t>(W3[p]);
            hp[p].out = out.at<uint32_t>(Lo.elem(p));
        }
        upload_progs();
        const uint32_t t_w2 = tiles(12, W2, elem_tile);
        batch_stage(BatchStage::FjEmit, bl(12), t_w2, nullptr);
        const uint32_t t_f3 = tiles(15, F, elem_tile);
        batch_stage(BatchStage::FjFunctab, bl(15), t_f3, nullptr);
        BP_CU(cudaEventRecord(ev[6], s));
        BP_CU(cudaEventRecord(ev[7], s));

        // ---- results: the output words and function tables of every program, one copy each
        BP_CU(h_out.ensure(Lo.total * 4));
        BP_CU(h_fn.ensure(Lf.total * 4 * 4));
        BP_CU(cudaEventRecord(ev_out0, s));
        {
            // kernel stores over the host link: 5.3 ms for the 4,096-program batch's 1 GB
            // against 9-10 ms through the copy engine
            void* dout = nullptr;  // the pinned output buffer's address on the device
            if (cudaHostGetDevicePointer(&dout, h_out.p, 0) == cudaSuccess && dout) {
                BP_CU(kernel_copy(out.p, dout, Lo.total * 4, s));
            } else {
                cudaGetLastError();
                BP_CU(cudaMemcpyAsync(h_out.p, out.p, Lo.total * 4, cudaMemcpyDeviceToHost, s));
            }
        }
        uint32_t* hf = h_fn.at<uint32_t>();
        BP_CU(cudaMemcpyAsync(hf, fn_start.p, Lf.total * 4, cudaMemcpyDeviceToHost, s));
        BP_CU(cudaMemcpyAsync(hf + Lf.total, fn_end.p, Lf.total * 4, cudaMemcpyDeviceToHost, s));
        BP_CU(cudaMemcpyAsync(hf + 2 * Lf.total, fn_size.p, Lf.total * 4, cudaMemcpyDeviceToHost, s));
        BP_CU(cudaMemcpyAsync(hf + 3 * Lf.total, fn_id.p, Lf.total * 4, cudaMemcpyDeviceToHost, s));
        d2h += Lo.total * 4 + 4 * Lf.total * 4;
        BP_CU(cudaEventRecord(ev_out1, s));
        BP_CU(collect_errors());
        for (size_t p = 0; p < B; ++p) {
            BatchResult& r = res[p];
            r.status = status[p];
            if (!active[p]) continue;
            r.words = h_out.at<uint32_t>(Lo.elem(p));
            r.count = W3[p];
            const uint64_t e = Lf.elem(p);
            r.starts = hf + e;
            r.ends = hf + Lf.total + e;
            r.sizes = hf + 2 * Lf.total + e;
            r.ids = hf + 3 * Lf.total + e;
            r.functions = F[p];
            r.nodes = n[p];
            r.words_gen = W[p];
            r.words_ra = W2[p];
        }
        float ms = 0;
        for (int k = 0; k < 6; ++k) {
            if (cudaEventElapsedTime(&ms, ev[k], ev[k + 1]) == cudaSuccess) ns[k] = static_cast<uint64_t>(ms * 1e6);
        }
        ns[6] = 0;  // postprocess is fused into fix_jumps
        if (cudaEventElapsedTime(&ms, ev_in, ev[0]) == cudaSuccess) hns[1] = static_cast<uint64_t>(ms * 1e6);
        // Direct reads of a large input slower than 40 GB/s (where the host's page
        // translation, not the link, bounds them): this pipeline and later ones on the
        // device take the inputs through pinned memory from now on.
        if (direct_host && last_in_bytes >= (uint64_t(256) << 20) && hns[1] > 0 &&
            static_cast<double>(last_in_bytes) < 40.0 * static_cast<double>(hns[1])) {
            direct_host = false;
            direct_host_slow(device);
        }
        sort_ns = cudaEventElapsedTime(&ms, ev_sort0, ev_sort1) == cudaSuccess ? static_cast<uint64_t>(ms * 1e6) : 0;
        if (cudaEventElapsedTime(&ms, ev_out0, ev_out1) == cudaSuccess) hns[2] = static_cast<uint64_t>(ms * 1e6);
    }
    return PTL_OK;
}

// Whether kernels should read the callers' pageable arrays directly rather than take
// them from pinned memory through the copy engine.  The link that direct reads use
// differs between hosts (on some the device reads host memory at a few GB/s while the
// copy engine still moves tens of GB/s), so it is measured once per device: 32 MB read
// each way; direct unless the copy engine is more than twice as fast, which pays for the
// host threads' gather into pinned memory.
struct DirectHostChoice {
    std::mutex mu;
    std::map<int, bool> known;
};
DirectHostChoice& direct_host_choice() {
    static DirectHostChoice c;
    return c;
}

void direct_host_slow(int device) {
    DirectHostChoice& c = direct_host_choice();
    std::lock_guard<std::mutex> lk(c.mu);
    c.known[device] = false;
}

bool direct_host_pays(int device, cudaStream_t s) {
    DirectHostChoice& c = direct_host_choice();
    std::lock_guard<std::mutex> lk(c.mu);
    std::map<int, bool>& known = c.known;
    const auto it = known.find(device);
    if (it != known.end()) return it->second;
    constexpr size_t kBytes = size_t(32) << 20;
    bool direct = true;  // if the probe cannot run: the reads it would have compared
    void* host = std::malloc(kBytes);
    void* pinned = nullptr;
    void* dev = nullptr;
    cudaEvent_t ev[4] = {};
    bool ok = host && cudaHostAlloc(&pinned, kBytes, cudaHostAllocDefault) == cudaSuccess &&
              cudaMalloc(&dev, kBytes) == cudaSuccess;
    for (auto& e : ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    if (ok) {
        std::memset(host, 1, kBytes);
        std::memset(pinned, 1, kBytes);
        for (int rep = 0; rep < 2 && ok; ++rep) {  // the first round warms both paths
            ok = cudaEventRecord(ev[0], s) == cudaSuccess && read_host(host, dev, kBytes, s) == cudaSuccess &&
                 cudaEventRecord(ev[1], s) == cudaSuccess &&
                 cudaMemcpyAsync(dev, pinned, kBytes, cudaMemcpyHostToDevice, s) == cudaSuccess &&
                 cudaEventRecord(ev[2], s) == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess;
        }
        float t_direct = 0, t_copy = 0;
        if (ok && cudaEventElapsedTime(&t_direct, ev[0], ev[1]) == cudaSuccess &&
            cudaEventElapsedTime(&t_copy, ev[1], ev[2]) == cudaSuccess && t_copy > 0)
            direct = t_direct <= 2.0f * t_copy;
    }
    for (auto& e : ev) if (e) cudaEventDestroy(e);
    if (dev) cudaFree(dev);
    if (pinned) cudaFreeHost(pinned);
    std::free(host);
    cudaGetLastError();  // a failed probe leaves no error behind
    known[device] = direct;
    return direct;
}

}  // namespace

BatchPipeline* BatchPipeline::create(int device, int host_threads, ptl_status* st, bool urgent) {
    Pipeline* p = new (std::nothrow) Pipeline;
    if (!p) {
        if (st) *st = PTL_OOM;
        return nullptr;
    }
    p->device = device;
    p->threads = std::max(1, host_threads);
    int lo = 0, hi = 0;  // stream priorities: numerically lower is more urgent
    const DeviceScope on_device(device);
    if (!on_device.ok() || cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&p->s, cudaStreamNonBlocking, urgent ? hi : lo) != cudaSuccess) {
        delete p;
        if (st) *st = PTL_CUDA_ERROR;
        return nullptr;
    }
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) pageable = 0;
    const char* env = std::getenv("PTL_HOST_GATHER");  // "1": gather through pinned memory regardless
    p->direct_host = pageable == 1 && !(env && env[0] == '1') && direct_host_pays(device, p->s);
    if (st) *st = PTL_OK;
    return p;
}

}  // namespace ptl
