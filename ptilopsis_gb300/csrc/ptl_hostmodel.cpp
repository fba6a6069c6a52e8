// Host model of the GPU pipeline -- test-only build.
//
// Runs the per-thread stage functions of ptl_stages.cuh / ptl_sort.cuh sequentially on
// the CPU, with sequential versions of the cross-thread steps (scans, the depth-order
// rounds, the lock-step lane-0 allocator).  The CPU test suite compares it with the
// oracle so the GPU algorithm is checked before it runs on a GPU.  The library API
// never calls it: without the CUDA library the package refuses to compile anything.
#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "ptl_common.cuh"
#include "ptl_sort.cuh"
#include "ptl_stages.cuh"
#include "ptl_ra.cuh"
#include "ptl_scalar.cuh"

using namespace ptl;

namespace {

uint32_t g_cache_k = 4;  // entries per function of the lane-0 symbol cache
bool g_force_hashed = false;  // lane-0 pass finds row-0 values by hashing even when definitions are unique
bool g_last_hashed = false;   // the last compile had a lane-0 virtual register with two definitions
bool g_last_cross = false;    // the last scalar compile took the serial register allocation
bool g_force_serial = false;  // scalar register allocation in the reference's order for every program

template <typename T>
struct HBuf {
    std::vector<T> v;
    T* p = nullptr;
    size_t n = 0;
    void ensure(size_t count, T fill = T{}) {
        n = count;
        v.assign(count + 16 + 80, fill);
        p = v.data() + 16;
    }
};

inline size_t r8(size_t n) { return (n + 7) & ~size_t(7); }

struct Model {
    CodeTables tab;
    ErrorWord err{};
    uint32_t flags[4] = {0, 0, 0, 0};
    HBuf<uint8_t> in_type, in_rtype, fflag, used, smark, defpos, nt, rt;
    HBuf<int32_t> in_parent, in_depth, in_child, par, ci, dep;
    HBuf<uint32_t> in_data, nd1, nd, sizes, loc0, loc, regs, pos, decl, fn_id, fn_start, fn_size,
        fn_end, fn_start0, fn_size0, fn_end0, fn_ra_start, fn_ra_end, fn_ra_size, instr, rd, rs1, rs2, jt,
        used_instrs, symreg, symswp, stamp, trig_min, trig_max, spill, roffs, ni, nrd, nr1, nr2, njt, fsz,
        joffs, out;
    HBuf<unsigned long long> owner, lifetime;
    Prog P{};

    void bind() {
        P.in_type = in_type.p; P.in_rtype = in_rtype.p; P.in_parent = in_parent.p; P.in_depth = in_depth.p;
        P.in_child = in_child.p; P.in_data = in_data.p;
        P.nt = nt.p; P.rt = rt.p; P.nd1 = nd1.p; P.nd = nd.p; P.par = par.p; P.ci = ci.p; P.dep = dep.p;
        P.fflag = fflag.p; P.sizes = sizes.p; P.loc0 = loc0.p; P.loc = loc.p; P.regs = regs.p; P.pos = pos.p;
        P.owner = owner.p; P.decl = decl.p; P.fn_id = fn_id.p; P.fn_start = fn_start.p; P.fn_size = fn_size.p;
        P.fn_end = fn_end.p; P.fn_start0 = fn_start0.p; P.fn_size0 = fn_size0.p; P.instr = instr.p;
        P.rd = rd.p; P.rs1 = rs1.p; P.rs2 = rs2.p; P.jt = jt.p; P.used = used.p; P.smark = smark.p;
        P.used_instrs = used_instrs.p; P.symreg = symreg.p; P.symswp = symswp.p; P.stamp = stamp.p;
        P.defpos = defpos.p;
        P.lifetime = lifetime.p; P.trig_min = trig_min.p; P.trig_max = trig_max.p; P.spill = spill.p;
        P.roffs = roffs.p; P.ni = ni.p; P.nrd = nrd.p; P.nr1 = nr1.p; P.nr2 = nr2.p; P.njt = njt.p;
        P.fsz = fsz.p; P.joffs = joffs.p; P.out = out.p;
        P.tab.t = &tab;
        P.err = &err;
        P.flags = flags;
    }

    template <class F>
    static void exclusive_scan(uint32_t count, F load, uint32_t* out) {
        uint32_t acc = 0;
        for (uint32_t i = 0; i < count; ++i) {
            const uint32_t v = load(i);
            out[i] = acc;
            acc += v;
        }
    }

    bool check() { return err.code == 0; }

    // Depth-order emulation with the same round structure as the kernels.
    void depth_sort(uint32_t n) {
        std::vector<unsigned long long> a(n);
        for (uint32_t i = 0; i < n; ++i) a[i] = (static_cast<unsigned long long>(static_cast<uint32_t>(dep.p[i])) << 32) | i;
        std::vector<uint32_t> apos(n), bpos(n);
        std::vector<SortSeg> cur, next;
        std::vector<std::pair<uint32_t, uint32_t>> leaves, heaps;
        std::vector<std::array<uint32_t, 3>> locals;
        std::vector<std::pair<uint32_t, uint32_t>> equal;
        auto emit = [&](uint32_t first, uint32_t last, uint32_t dl, bool eq) {
            if (eq && last - first <= kSortThreshold) return;  // a stable sort of equal keys
            if (eq && dl >= equal_levels(last - first)) { equal.push_back({first, last}); return; }
            if (last - first <= kSortThreshold) { if (last - first > 1) leaves.push_back({first, last}); return; }
            if (dl > 0 && last - first <= kSortBlock) { locals.push_back({first, last, dl}); return; }
            if (dl == 0) { heaps.push_back({first, last}); return; }
            SortSeg c{}; c.first = first; c.last = last; c.dl = dl;
            next.push_back(c);
        };
        if (n > 1) emit(0, n, 2u * floor_log2(n), false);  // the whole array: rounds, or one block
        cur.swap(next);
        while (!cur.empty()) {
            next.clear();
            for (SortSeg& g : cur) {
                median_to_first(a.data(), g.first, g.last);
                g.pivot = skey(a[g.first]);
                g.kmin = g.kmax = g.pivot;
                for (uint32_t p = g.first + 1; p < g.last; ++p) {
                    g.kmin = std::min(g.kmin, skey(a[p]));
                    g.kmax = std::max(g.kmax, skey(a[p]));
                }
                uint32_t nl = 0, nr_total = 0;
                for (uint32_t p = g.first + 1; p < g.last; ++p) nr_total += is_rstop(skey(a[p]), g.pivot);
                uint32_t rl = 0;
                for (uint32_t p = g.first + 1; p < g.last; ++p) {
                    const int32_t k = skey(a[p]);
                    if (is_lstop(k, g.pivot)) apos[g.first + nl++] = p;
                    if (is_rstop(k, g.pivot)) bpos[g.first + (nr_total - 1 - rl++)] = p;
                }
                g.nL = nl;
                g.nR = nr_total;
                g.K = partition_k(apos.data() + g.first, bpos.data() + g.first, g.nL, g.nR);
                g.cut = partition_cut(apos.data() + g.first, bpos.data() + g.first, g.nL, g.K);
                for (uint32_t k = 0; k < g.K; ++k) sswap(a.data(), apos[g.first + k], bpos[g.first + k]);
                emit(g.first, g.cut, g.dl - 1, g.kmin == g.pivot);
                emit(g.cut, g.last, g.dl - 1, g.kmax == g.pivot);
            }
            cur.swap(next);
        }
        for (auto& h : heaps) heap_sort_range(a.data() + h.first, h.second - h.first);
        for (auto& l : leaves) leaf_sort(a.data(), l.first, l.second);
        for (auto& r : locals) {  // one thread per range on the device, in a strided buffer
            std::vector<unsigned long long> buf(static_cast<size_t>(r[1] - r[0]) * 3);
            const Strided sb{buf.data() + 1, 3};
            for (uint32_t i = 0; i < r[1] - r[0]; ++i) sb[i] = a[r[0] + i];
            local_introsort(sb, 0u, r[1] - r[0], r[2]);
            for (uint32_t i = 0; i < r[1] - r[0]; ++i) a[r[0] + i] = sb[i];
        }
        for (auto& r : equal) {  // one block per range on the device, through apos
            const uint32_t m = r.second - r.first;
            for (uint32_t i = 0; i < m; ++i) apos[r.first + equal_final_index(i, m)] = sidx(a[r.first + i]);
            const unsigned long long key = a[r.first] & 0xFFFFFFFF00000000ull;
            for (uint32_t i = 0; i < m; ++i) a[r.first + i] = key | apos[r.first + i];
        }
        for (uint32_t p = 0; p < n; ++p) pos.p[sidx(a[p])] = p;
    }

    uint32_t hm_cache_k = g_cache_k;

    // The lane-0 pass with the same phase functions as k_ra_lane0_cached.
    void lane0_cached(uint32_t S, uint32_t K, bool hashed) {
        const uint32_t G0 = (P.F + 7) / 8;
        const Prog Psave = P;
        if (hashed) P.defpos = nullptr;
        Ra2Shared sh{};
        std::vector<uint32_t> cur(4 * G0), tag(static_cast<size_t>(G0) * K);
        std::vector<uint32_t> val(static_cast<size_t>(G0) * K);
        const SymCache c{tag.data(), val.data(), K};
        std::vector<Ra2Slot> L(G0);
        for (uint32_t j = 0; j < G0; ++j) {
            L[j].act = false;
            L[j].have_next = false;
            ra2_slot_init(P, c, L[j], j, j);
        }
        for (int p = 0; p < 64; ++p) { sh.R0[p] = 0xFFFFFFFFu; sh.R0own[p] = 0xFFFFFFFFu; }
        if (S > 0) for (uint32_t p = 0; p < 64; ++p) ra2_begin_p(sh, 0, p, P.trig_min[p], P.trig_max[p], hashed);
        uint32_t s0 = 0;  // steps with a lane-0 function still running
        for (uint32_t j = 0; j < G0; ++j) s0 = std::max(s0, ra2_lane0_size(L[j]));
        s0 = std::min(s0, S);
        for (uint32_t i = 0; i < s0; ++i) {
            bool in_row0 = false;
            for (uint32_t j = 0; j < G0; ++j) {
                ra2_load(P, L[j], i, cur.data() + 4 * j);
                in_row0 |= ra2_compute0(P, c, sh, L[j], j, i);
            }
            bool flag = false;
            if (in_row0) for (uint32_t j = 0; j < G0; ++j) flag |= ra2_check(sh, L[j]);
            for (uint32_t j = 0; j < G0; ++j) ra2_apply(P, c, sh, L[j], j, i, cur.data() + 4 * j);
            if (flag) {
                for (uint32_t p = 0; p < 64; ++p) sh.r0grp[p] = 0;
                for (uint32_t round = 0;; ++round) {
                    for (uint32_t j = 0; j < G0; ++j) ra2_round(sh, L[j]);
                    bool changed = false;
                    for (uint32_t p = 0; p < 64; ++p) changed |= ra2_round_p(sh, p);
                    if (!changed) break;
                    if (round > G0 + 2) { record_error(P.err, ST_DEVICE_TIMEOUT, W_RA2, i); break; }
                }
                for (uint32_t j = 0; j < G0; ++j) ra2_apply(P, c, sh, L[j], j, i, cur.data() + 4 * j);
            }
            if (hashed) for (uint32_t p = 0; p < 64; ++p) snap_clear_next(sh, i, p);
            for (uint32_t p = 0; p < 64; ++p) {
                ra2_end_p(P, c, sh, p, cur.data());
            }
            if (i + 1 < S) {
                for (uint32_t p = 0; p < 64; ++p) {
                    ra2_begin_p(sh, i + 1, p, P.trig_min[static_cast<size_t>(i + 1) * 64 + p],
                                P.trig_max[static_cast<size_t>(i + 1) * 64 + p], hashed);
                }
            }
        }
        {  // the steps after the last lane-0 function only mark row 0's symbols
            for (uint32_t p = 0; p < 64; ++p) ra2_tail_p(P, c, sh, p, s0, S);
        }
        P = Psave;
    }

    // The scalar generator's register allocation (ptl_scalar.cuh), from the optimized words
    // to the regalloc output (the spill offsets, the count scan, the scatter, the moved
    // function table and the frame words).
    void scalar_regalloc(uint32_t F, uint32_t W, uint32_t wb8) {
        uint32_t cross = 0;
        for (uint32_t i = 0; i < W; ++i) cross |= st_ra_cross(P, i, stamp.p) & 1u;
        std::vector<unsigned long long> preserve(F, 0);
        if (cross || g_force_serial) {
            std::vector<int32_t> sregs(static_cast<size_t>(F) * 64);
            std::vector<SRaStep> steps(F);
            s_ra_serial(P, sregs.data(), steps.data(), preserve.data());
        } else {
            // the GPU's word tiles (functions by their first word, symbols as bytes)
            int32_t sregs[64];
            constexpr uint32_t T = 4096;
            std::vector<uint8_t> sym;
            for (uint32_t b = 0; b <= W / T; ++b) {
                uint32_t first, last, base;
                s_ra_tile_functions(P, b, T, &first, &last);
                const uint32_t count = s_ra_tile_span(P, first, last, &base);
                sym.assign(count + 1, 0);
                const SymBytes sy{sym.data(), base, count, P.err};
                for (uint32_t f = first; f < last; ++f) s_ra_function(P, sy, f, sregs, preserve.data());
                for (uint32_t k = 0; k < count; ++k) s_ra_tile_writeback(P, sym.data(), base, count, k);
            }
        }
        g_last_cross = cross != 0;
        if (!check()) return;
        for (uint32_t v = 0; v < W; ++v) st_ra_spill(P, v);
        std::vector<uint32_t> extra(wb8 + 16, 0);
        for (uint32_t f = 0; f < F; ++f) st_s_preserve_counts(P, f, preserve.data(), extra.data());
        if (!check()) return;
        exclusive_scan(wb8, [&](uint32_t i) { return st_s_ra_count(P, i, extra.data()); }, roffs.p);
        if (!check()) return;
        const uint32_t W2 = roffs.p[W - 1] + 1;
        const uint32_t w2b8 = static_cast<uint32_t>(r8(W2));
        for (auto* b : {&ni, &nrd, &nr1, &nr2, &njt, &fsz, &joffs}) b->ensure(w2b8 + 16);
        P.W2 = W2; P.w2b8 = w2b8;
        bind();
        for (uint32_t i = 0; i < wb8; ++i) st_s_ra_scatter(P, i);
        for (uint32_t f = 0; f < F; ++f) st_fix_functab(P, f, P.roffs, W);
        for (uint32_t pass = 0; pass < 3; ++pass)
            for (uint32_t f = 0; f < F; ++f) st_s_frame(P, f, pass, preserve.data(), 0, nullptr);
    }

    int run(const uint8_t* type, const uint8_t* rtype, const int32_t* parent, const int32_t* depth,
            const int32_t* child, const uint32_t* data, size_t n_, size_t max_depth, bool scalar) {
        build_code_tables(&tab);
        const uint32_t n = static_cast<uint32_t>(n_);
        const uint32_t nb8 = static_cast<uint32_t>(r8(n));
        in_type.ensure(n); in_rtype.ensure(n); in_parent.ensure(n); in_depth.ensure(n); in_child.ensure(n); in_data.ensure(n);
        std::memcpy(in_type.p, type, n); std::memcpy(in_rtype.p, rtype, n);
        std::memcpy(in_parent.p, parent, 4ull * n); std::memcpy(in_depth.p, depth, 4ull * n);
        std::memcpy(in_child.p, child, 4ull * n); std::memcpy(in_data.p, data, 4ull * n);
        for (auto* b : {&nd1, &nd, &sizes, &loc0, &loc, &pos, &decl}) b->ensure(nb8);
        nt.ensure(nb8);
        rt.ensure(nb8);
        for (auto* b : {&par, &ci, &dep}) b->ensure(nb8);
        fflag.ensure(nb8);
        regs.ensure(3ull * n);
        P = Prog{};
        P.n = n; P.nb8 = nb8; P.max_depth = static_cast<uint32_t>(max_depth);
        P.scalar = scalar ? 1u : 0u;
        bind();
        bool reach = false;
        for (uint32_t i = 0; i < nb8; ++i) reach |= st_ingest(P, i);
        if (!check()) return err.code;
        if (!reach) return ST_INVALID_AST;
        if (scalar) {
            for (uint32_t i = 0; i < nb8; ++i) st_s_pre_lists(P, i);
            for (uint32_t i = 0; i < nb8; ++i) st_s_pre_float(P, i);
        } else {
            for (uint32_t i = 0; i < nb8; ++i) st_pre_lists(P, i);
            for (uint32_t i = 0; i < nb8; ++i) st_pre_float(P, i);
        }
        for (uint32_t i = 0; i < nb8; ++i) st_pre_float_apply(P, i);
        if (!check()) return err.code;
        exclusive_scan(nb8, [&](uint32_t i) { const uint32_t v = st_count(P, i); P.sizes[i] = v; return v; }, loc0.p);
        for (uint32_t i = 0; i < nb8; ++i) st_fix_own(P, i);
        for (uint32_t i = 0; i < nb8; ++i) st_fix_cond(P, i);
        uint32_t F = 0;
        for (uint32_t i = 0; i < nb8; ++i) if (P.nt[i] == RV_FUNC_DECL) P.decl[F++] = i;
        if (!check()) return err.code;
        if (F == 0) return ST_UNSUPPORTED;
        const uint32_t fb8 = static_cast<uint32_t>(r8(F));
        for (auto* b : {&fn_id, &fn_start, &fn_size, &fn_end, &fn_start0, &fn_size0, &fn_end0, &fn_ra_start, &fn_ra_end, &fn_ra_size}) b->ensure(fb8 + 8);
        P.F = F; P.fb8 = fb8;
        bind();
        for (uint32_t f = 0; f < fb8; ++f) st_functab(P, f);
        uint32_t S = 0;
        for (uint32_t f = 0; f < fb8; ++f) {
            st_functab_end(P, f);
            if (f < F) S = std::max(S, P.fn_size[f]);
        }
        for (uint32_t f = 0; f < F; ++f) fn_end0.p[f] = fn_end.p[f];
        const uint32_t W = P.loc[n - 1];
        const uint32_t wb8 = static_cast<uint32_t>(r8(W));
        for (auto* b : {&instr, &rd, &rs1, &rs2, &jt, &used_instrs, &symreg, &symswp, &stamp, &spill, &roffs}) b->ensure(wb8);
        owner.ensure(wb8);
        used.ensure(wb8);
        smark.ensure(wb8);
        P.W = W; P.wb8 = wb8; P.S = S;
        bind();
        depth_sort(n);
        if (scalar) {
            for (uint32_t x = 0; x < n; ++x) st_s_gen_prop(P, x);
            for (uint32_t x = 0; x < n; ++x) st_s_gen_claim(P, x);
            for (uint32_t x = 0; x < n; ++x) st_s_gen_write(P, x);
        } else {
            for (uint32_t x = 0; x < n; ++x) st_gen_prop(P, x);
            for (uint32_t x = 0; x < n; ++x) st_gen_claim(P, x);
            for (uint32_t x = 0; x < n; ++x) st_gen_write(P, x);
        }
        if (!check()) return err.code;
        for (uint32_t i = 0; i < wb8; ++i) st_opt_mark(P, i);
        for (;;) {
            bool changed = false;
            for (uint32_t i = 0; i < wb8; ++i) changed |= st_opt_sweep(P, i);
            if (!changed) break;
        }
        for (uint32_t i = 0; i < wb8; ++i) st_opt_final(P, i);
        if (!check()) return err.code;
        lifetime.ensure(fb8);
        for (uint32_t f = 0; f < F; ++f) lifetime.p[f] = 0x1Full;
        trig_min.ensure(static_cast<size_t>(std::max<uint32_t>(S, 1)) * 64, 0xFFFFFFFFu);
        trig_max.ensure(static_cast<size_t>(std::max<uint32_t>(S, 1)) * 64, 0u);
        bind();
        defpos.ensure(wb8);
        bind();
        if (scalar) {
            scalar_regalloc(F, W, wb8);
            if (!check()) return err.code;
        } else {
            uint32_t flagbits = 0;
            for (uint32_t i = 0; i < W; ++i) flagbits |= st_ra_cross(P, i, stamp.p);
            const uint32_t G0 = (F + 7) / 8;
            if ((flagbits & 1u) || G0 > 8192u) {
                st_ra_serial(P, stamp.p);
            } else {
                std::vector<uint32_t> tag(64), val(64);
                const SymCache c1{tag.data(), val.data(), 64};
                Prog Pfree = P;
                Pfree.defpos = nullptr;
                for (uint32_t f = 0; f < F; ++f) if (f & 7u) ra_free_function_cached(Pfree, c1, 0, f);
                lane0_cached(S, hm_cache_k, (flagbits & 2u) != 0 || g_force_hashed);
                g_last_hashed = (flagbits & 2u) != 0;
            }
            for (uint32_t v = 0; v < W; ++v) st_ra_spill(P, v);
            exclusive_scan(wb8, [&](uint32_t i) { return st_ra_count(P, i); }, roffs.p);
            if (!check()) return err.code;
            const uint32_t W2 = roffs.p[W - 1] + 1;
            const uint32_t w2b8 = static_cast<uint32_t>(r8(W2));
            for (auto* b : {&ni, &nrd, &nr1, &nr2, &njt, &fsz, &joffs}) b->ensure(w2b8 + 16);
            P.W2 = W2; P.w2b8 = w2b8;
            bind();
            for (uint32_t i = 0; i < wb8; ++i) st_ra_scatter(P, i);
            for (uint32_t f = 0; f < F; ++f) st_fix_functab(P, f, P.roffs, W);
            for (uint32_t f = 0; f < F; ++f) st_ra_frame(P, f);
        }
        for (uint32_t f = 0; f < F; ++f) { fn_ra_start.p[f] = fn_start.p[f]; fn_ra_end.p[f] = fn_end.p[f]; fn_ra_size.p[f] = fn_size.p[f]; }
        const uint32_t W2 = P.W2, w2b8 = P.w2b8;
        exclusive_scan(w2b8, [&](uint32_t i) { const uint32_t v = i < W2 ? st_fj_size(P, i) : 0u; P.fsz[i] = v; return v; }, joffs.p);
        const uint32_t W3 = fsz.p[W2 - 1] + joffs.p[W2 - 1];
        out.ensure(r8(W3) + 8);
        P.W3 = W3;
        bind();
        for (uint32_t i = 0; i < W2; ++i) st_fj_emit(P, i);
        for (uint32_t f = 0; f < F; ++f) st_fix_functab(P, f, P.joffs, W2);
        return check() ? 0 : err.code;
    }
};

}  // namespace

extern "C" {

struct ptlhm_buf {
    uint32_t* p;
    size_t n;
};

// Same slot numbers as ptl_generator_snapshot (include/ptl_codegen.h).
// scalar: the scalar generator's semantics.
int ptlhm_compile_mode(const uint8_t* type, const uint8_t* rtype, const int32_t* parent, const int32_t* depth,
                       const int32_t* child, const uint32_t* data, size_t n, size_t max_depth, ptlhm_buf* bufs,
                       int nbufs, uint32_t* err_out, int scalar) {
    Model* m = new Model();
    int rc = 0;
    try {
        rc = m->run(type, rtype, parent, depth, child, data, n, max_depth, scalar != 0);
    } catch (const std::exception&) {
        rc = ST_UNSUPPORTED;
    }
    if (err_out) { err_out[0] = m->err.code; err_out[1] = m->err.where; err_out[2] = m->err.detail; }
    auto put = [&](int k, const uint32_t* src, size_t len) {
        if (k >= nbufs) return;
        bufs[k].n = len;
        bufs[k].p = static_cast<uint32_t*>(std::malloc(std::max<size_t>(1, len) * 4));
        if (len) std::memcpy(bufs[k].p, src, len * 4);
    };
    for (int k = 0; k < nbufs; ++k) { bufs[k].p = nullptr; bufs[k].n = 0; }
    if (rc == 0) {
        const Prog& P = m->P;
        put(0, P.out, P.W3);
        put(1, P.fn_start, P.F); put(2, P.fn_end, P.F); put(3, P.fn_size, P.F); put(4, P.fn_id, P.F);
        {
            std::vector<uint32_t> wide(P.n);
            for (uint32_t i = 0; i < P.n; ++i) wide[i] = P.nt[i];
            put(5, wide.data(), P.n);
            for (uint32_t i = 0; i < P.n; ++i) wide[i] = P.rt[i];
            put(6, wide.data(), P.n);
        }
        put(7, P.nd, P.n);
        put(8, P.sizes, P.n); put(9, P.loc, P.n);
        put(10, P.fn_id, P.F); put(11, P.fn_start0, P.F); put(12, m->fn_end0.p, P.F); put(13, P.fn_size0, P.F);
        put(14, P.instr, P.W); put(15, P.rd, P.W); put(16, P.rs1, P.W); put(17, P.rs2, P.W); put(18, P.jt, P.W);
        put(19, P.used_instrs, P.W);
        put(20, P.ni, P.W2); put(21, P.nrd, P.W2); put(22, P.nr1, P.W2); put(23, P.nr2, P.W2); put(24, P.njt, P.W2);
        put(25, m->fn_ra_start.p, P.F); put(26, m->fn_ra_end.p, P.F); put(27, m->fn_ra_size.p, P.F);
        put(40, P.pos, P.n);
    }
    delete m;
    return rc;
}

int ptlhm_compile(const uint8_t* type, const uint8_t* rtype, const int32_t* parent, const int32_t* depth,
                  const int32_t* child, const uint32_t* data, size_t n, size_t max_depth, ptlhm_buf* bufs,
                  int nbufs, uint32_t* err_out) {
    return ptlhm_compile_mode(type, rtype, parent, depth, child, data, n, max_depth, bufs, nbufs, err_out, 0);
}

int ptlhm_last_cross(void) { return g_last_cross ? 1 : 0; }

// Whether isn_gen's packed table fields decode to the code tables.
int ptlhm_gen_desc_ok(void) {
    static CodeTables t;
    build_code_tables(&t);
    return gen_desc_ok(&t) ? 1 : 0;
}
void ptlhm_set_scalar_serial(int on) { g_force_serial = on != 0; }

void ptlhm_set_cache_entries(uint32_t k) { g_cache_k = k; }
void ptlhm_set_hashed(int on) { g_force_hashed = on != 0; }
int ptlhm_last_hashed(void) { return g_last_hashed ? 1 : 0; }

void ptlhm_free(ptlhm_buf* bufs, int nbufs) {
    for (int k = 0; k < nbufs; ++k) { std::free(bufs[k].p); bufs[k].p = nullptr; bufs[k].n = 0; }
}

// The sort emulation alone: perm receives the order of iota(n) sorted by keys.
void ptlhm_depth_sort(const int32_t* keys, size_t n, uint32_t* perm) {
    Model m;
    m.dep.ensure(n);
    m.pos.ensure(n);
    std::memcpy(m.dep.p, keys, 4 * n);
    m.depth_sort(static_cast<uint32_t>(n));
    for (size_t x = 0; x < n; ++x) perm[m.pos.p[x]] = static_cast<uint32_t>(x);
}

}  // extern "C"
