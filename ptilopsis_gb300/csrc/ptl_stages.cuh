// Per-thread stage logic of the GB300 code generator.
//
// Every function here is one thread's share of a stage and is called both by the CUDA
// kernels (ptl_kernels.cu) and by the host model used in CPU tests.  Comments cite the
// reference loop each function reproduces, in src/codegen/rv_generator_avx.cpp of the
// reference; the reference runs its loops over 8-lane blocks in ascending order with
// one worker thread, and the notes below say how each stage's ordering effects are
// resolved in parallel.
//
// Array conventions: node arrays hold nb8 = 8*ceil(n/8) elements plus zeroed pads on
// both sides (index -1 reads 0), like the reference's avx_buffer; instruction arrays
// likewise hold wb8 = 8*ceil(W/8) elements.
#pragma once

#include "ptl_common.cuh"

namespace ptl {

// Atomics that the host model runs single-threaded.  Each helper compiles for host and
// device; the device path is taken inside kernels.
PTL_HD void at_max_u64(unsigned long long* p, unsigned long long v) {
#if defined(__CUDA_ARCH__)
    atomicMax(p, v);
#else
    if (v > *p) *p = v;
#endif
}
PTL_HD void at_min_u32(uint32_t* p, uint32_t v) {
#if defined(__CUDA_ARCH__)
    atomicMin(p, v);
#else
    if (v < *p) *p = v;
#endif
}
PTL_HD void at_max_u32(uint32_t* p, uint32_t v) {
#if defined(__CUDA_ARCH__)
    atomicMax(p, v);
#else
    if (v > *p) *p = v;
#endif
}
PTL_HD void record_error(ErrorWord* e, uint32_t code, uint32_t where, uint32_t detail) {
#if defined(__CUDA_ARCH__)
    if (atomicCAS(&e->code, 0u, code) == 0u) {
        e->where = where;
        e->detail = detail;
    }
#else
    if (e->code == 0u) { e->code = code; e->where = where; e->detail = detail; }
#endif
}
PTL_HD void at_add_u32(uint32_t* p, uint32_t v) {
#if defined(__CUDA_ARCH__)
    atomicAdd(p, v);
#else
    *p += v;
#endif
}
PTL_HD int popcount64(uint64_t v) {
#if defined(__CUDA_ARCH__)
    return __popcll(static_cast<unsigned long long>(v));
#else
    return __builtin_popcountll(v);
#endif
}
PTL_HD uint32_t ctz64(uint64_t t) {
#if defined(__CUDA_ARCH__)
    return static_cast<uint32_t>(__ffsll(static_cast<long long>(t)) - 1);
#else
    return static_cast<uint32_t>(__builtin_ctzll(t));
#endif
}

// ------------------------------------------------------------------ table access
// Table reads: the tables never change while a kernel runs, so the device reads them
// through the read-only path, which also lets the compiler reuse a read across stores.
template <class T>
PTL_HD T tab_ld(const T* p) {
#if defined(__CUDA_ARCH__)
    return __ldg(p);
#else
    return *p;
#endif
}

struct Tab {
    const CodeTables* t;
    PTL_HD uint32_t row(uint32_t type) const { return tab_ld(&t->row_of[type & 0xFFu]); }
    // The reference indexes its tables with type*24 + slot*6 + rtype; types are < 256 and
    // validated data types are <= 5, so the dense row lookup is exact.
    PTL_HD uint32_t size(uint32_t type, uint32_t rt) const { return tab_ld(&t->size[row(type)][rt]); }
    PTL_HD bool has_instr(uint32_t type, uint32_t s, uint32_t rt) const {
        return (tab_ld(&t->has_instr[row(type)][s]) >> rt) & 1u;
    }
    PTL_HD bool has_output(uint32_t type, uint32_t s, uint32_t rt) const {
        return (tab_ld(&t->has_output[row(type)][s]) >> rt) & 1u;
    }
    PTL_HD uint32_t pai(uint32_t type, uint32_t s, uint32_t rt) const { return tab_ld(&t->pai[row(type)][s][rt]); }
    PTL_HD uint32_t out(uint32_t type, uint32_t s, uint32_t rt) const { return tab_ld(&t->out[row(type)][s][rt]); }
    PTL_HD uint32_t cnst(uint32_t type, uint32_t s) const { return tab_ld(&t->cnst[row(type)][s]); }
    PTL_HD uint32_t jt(uint32_t type, uint32_t s) const { return tab_ld(&t->jt[row(type)][s]); }
    PTL_HD uint32_t opd(uint32_t type, uint32_t s, uint32_t rt, uint32_t k) const {
        return tab_ld(&t->opd[row(type)][s][rt][k]);
    }
    PTL_HD uint32_t word(uint32_t type, uint32_t s, uint32_t rt) const { return tab_ld(&t->instr[row(type)][s][rt]); }
    // the four slots' packed fields / words of (type, rt) in one 16-byte read
    struct Slots4 {
        uint32_t v[4];
    };
    PTL_HD Slots4 slots4(const uint32_t (*tab)[6][4], uint32_t type, uint32_t rt) const {
        const uint32_t* p = &tab[row(type)][rt][0];
#if defined(__CUDA_ARCH__)
        const uint4 q = __ldg(reinterpret_cast<const uint4*>(p));
        return Slots4{{q.x, q.y, q.z, q.w}};
#else
        return Slots4{{p[0], p[1], p[2], p[3]}};
#endif
    }
    PTL_HD Slots4 gdesc(uint32_t type, uint32_t rt) const { return slots4(t->gdesc, type, rt); }
    PTL_HD Slots4 gword(uint32_t type, uint32_t rt) const { return slots4(t->gword, type, rt); }
};

// ------------------------------------------------------------------ program view
struct Prog {
    // sizes
    uint32_t n, nb8, max_depth;
    uint32_t F, fb8;       // functions
    uint32_t W, wb8;       // words after isn_gen
    uint32_t W2, w2b8;     // words after regalloc
    uint32_t W3;           // words after fix_jumps
    // inputs
    const uint8_t* in_type;
    const uint8_t* in_rtype;
    const int32_t* in_parent;
    const int32_t* in_depth;
    const int32_t* in_child;
    const uint32_t* in_data;
    // node arrays (padded)
    uint8_t* nt;      // rv node type (every type fits a byte)
    uint8_t* rt;      // data type (final after preprocess)
    uint32_t* nd1;    // node data after pass 1
    uint32_t* nd;     // node data after pass 2 (final)
    int32_t* par;
    int32_t* ci;
    int32_t* dep;
    uint8_t* fflag;   // pass 3: becomes FLOAT; from isn_gen on, each node's parent type
    uint32_t* sizes;  // node code sizes, kept for stage snapshots (null in a batch)
    uint32_t* loc0;   // scan result
    uint32_t* loc;    // after fix
    uint32_t* regs;   // isn_gen registers, 3 per node
    uint32_t* pos;    // position of a node in the reference's depth-sorted order
    unsigned long long* owner;  // isn_gen write priority per word
    // function table (padded; isn_cnt values, rewritten by fix_func_tab)
    uint32_t* decl;   // FUNC_DECL node indices
    uint32_t* fn_id;
    uint32_t* fn_start;
    uint32_t* fn_size;
    uint32_t* fn_end;
    uint32_t* fn_start0;  // copies of the isn_cnt table used by regalloc
    uint32_t* fn_size0;
    // isn_gen output (wb8 + pads)
    uint32_t* instr;
    uint32_t* rd;
    uint32_t* rs1;
    uint32_t* rs2;
    uint32_t* jt;
    // optimize
    uint8_t* used;
    uint8_t* smark;
    uint32_t* used_instrs;
    // regalloc
    uint32_t* symreg;
    uint32_t* symswp;
    uint32_t* stamp;      // definitions per virtual register (regalloc cross check)
    uint8_t* defpos;      // row-0 position + 1 of each lane-0 definition; null: use the row-0 hash
    unsigned long long* lifetime;
    uint32_t* trig_min;   // [S][64] min group+1 of non-lane-0 triggers, 0xFFFFFFFF = none
    uint32_t* trig_max;   // [S][64] max group+1, 0 = none
    uint32_t* ra_chunks;  // [2][S/32 + 2]: per progress chunk, independent functions ending there; chunks done
    uint32_t* ra_order;   // independent functions, longest first (null: function order)
    uint32_t S;           // longest function (steps)
    uint32_t* spill;
    uint32_t* roffs;
    uint32_t* ni;
    uint32_t* nrd;
    uint32_t* nr1;
    uint32_t* nr2;
    uint32_t* njt;
    // fix_jumps
    uint32_t* fsz;    // word sizes, kept for the size read-back (null in a batch)
    uint32_t* joffs;
    uint32_t* out;
    // tables, errors, scratch flags
    Tab tab;
    ErrorWord* err;
    uint32_t* flags;      // [0] optimize changed, [1] [2] regalloc checks, [3] a node at max_depth
    uint32_t scalar;      // 1: the scalar generator's semantics (ptl_scalar.cuh)
    uint32_t pad_;
    // the scalar generator's register allocation in a batch (null otherwise): per
    // function the preserve mask, per word the preserve counts, per word after
    // regalloc the frame writes' claims
    unsigned long long* s_preserve;
    uint32_t* s_extra;
    unsigned long long* s_claim;
};

// Function-argument registers and stack slots, rv_generator_avx.cpp:126-213, on one
// node's type t, data type rt, data nd and child index ci.  The reference runs it over
// 8-lane blocks, but every lane reads and writes only its own node (non-argument lanes
// keep their values), so the input pass applies it as it writes each node.
PTL_HD void pre_args(uint32_t& t, uint32_t rt, uint32_t& nd, uint32_t ci) {
    if ((t & 0xF0u) != 0xF0u) return;
    const bool is_float = rt == DT_FLOAT || rt == DT_FLOAT_REF;
    const bool is_int = !is_float;
    {
        const uint32_t float_data = is_float ? nd : 0u;
        const bool comp = s32(float_data) > 7;
        uint32_t reg_offset = (ci - float_data) + float_data - 8u;
        const bool on_stack = (s32(reg_offset) > 7) && comp;
        const bool as_int = !on_stack && comp;
        if (on_stack) t |= 0b10u;
        if (as_int) t |= 0b01u;
        if (on_stack) reg_offset -= 8u;
        if (comp) nd = reg_offset;
    }
    {
        const uint32_t int_data = is_int ? nd : 0u;
        const uint32_t float_args = ci - int_data;
        uint32_t reg_offset = int_data + (float_args - ((s32(float_args) > 7) ? 8u : 0u));
        // The reference ANDs its comparison mask with the data value itself (:198).
        const uint32_t on_stack = (s32(reg_offset) > 7 ? 0xFFFFFFFFu : 0u) & int_data;
        t |= on_stack & 0b10u;
        reg_offset -= 8u & on_stack;
        if (is_int) nd = reg_offset;
    }
}

// The scalar generator's argument placement, rv_generator.cpp:231-284, on one node.
// rt & 0b001 and rt & 0b110: a float or float reference.
PTL_HD void pre_args_scalar(uint32_t& t, uint32_t rt, uint32_t& nd, uint32_t ci) {
    if ((t & RV_FUNC_ARG) != RV_FUNC_ARG) return;
    const bool is_f = (rt & 1u) && (rt & 6u);
    if (is_f && nd < 8u) return;  // the first eight float arguments stay in float registers
    const int32_t preceding_integers = is_f ? s32(ci - nd) : s32(nd);
    const int32_t preceding_floats = s32(ci) - preceding_integers;
    const int32_t over = preceding_floats - 8;
    const int32_t ir_idx = preceding_integers + (over > 0 ? over : 0);
    if (ir_idx < 8) {
        nd = u32(ir_idx);
        if (is_f) t |= 0b01u;
    } else {
        t |= 0b10u;
        nd = u32(ir_idx - 8);
    }
}

// ================================================================== input checks and copy
// One pass over the six input arrays: the DepthTree contract (post-order, one root last,
// consistent depths, in-range types; a bad node records INVALID_AST with its index), then
// the constructor copy and the Pareas -> rv type map (src/codegen/rv_generator.cpp:41-67)
// and preprocess's function-argument pass (pre_args); lanes past n become zero.  Returns
// whether node i is valid and sits at max_depth: with
// every node one level below its parent, depths 0..max_depth are all populated exactly
// when some node reaches max_depth.
PTL_HD bool st_ingest(const Prog& P, uint32_t i) {
    P.fflag[i] = 0;
    if (i >= P.n) {
        P.nt[i] = 0; P.rt[i] = 0; P.par[i] = 0; P.ci[i] = 0; P.nd1[i] = 0; P.dep[i] = 0;
        return false;
    }
    const uint32_t n = P.n;
    const uint32_t ty = P.in_type[i];
    const uint32_t rty = P.in_rtype[i];
    const int32_t p = P.in_parent[i];
    const int32_t c = P.in_child[i];
    const int32_t d = P.in_depth[i];
    const uint32_t data = P.in_data[i];
    bool bad = ty >= kNumPareasTypes || rty > 5 || d < 0 || static_cast<uint32_t>(d) > P.max_depth;
    if (i == n - 1) {
        bad |= p != -1 || d != 0;
    } else {
        bad |= p <= static_cast<int32_t>(i) || p >= static_cast<int32_t>(n) || c < 0;
        if (!bad) bad |= d - 1 != P.in_depth[p];  // d >= 0 here
    }
    if (bad) record_error(P.err, ST_INVALID_AST, 0, i);
    uint32_t t = ty < kNumPareasTypes ? P.tab.t->pareas_to_rv[ty] : 0u;
    uint32_t nd = data;
    if (P.scalar) pre_args_scalar(t, rty, nd, u32(c));  // preprocess's first pass, fused
    else pre_args(t, rty, nd, u32(c));
    P.nt[i] = t;
    P.rt[i] = rty;
    P.par[i] = p;
    P.ci[i] = c;
    P.nd1[i] = nd;
    P.dep[i] = d;
    return !bad && static_cast<uint32_t>(d) == P.max_depth;
}

// Value the call-list pass stores into lane i (or the lane's own data):
// rv_generator_avx.cpp:217-266.  The stores are masked by the predecessor's type only.
PTL_HD bool pre_list_block(const Prog& P, uint32_t b) {
    bool any = false;
    for (uint32_t l = 0; l < 8; ++l) any |= P.nt[8 * b + l] == RV_FUNC_CALL_ARG_LIST;
    return any;
}

PTL_HD uint32_t pre_list_value(const Prog& P, int64_t i, uint32_t prev_nd) {
    const uint32_t pt = P.nt[i - 1];
    if (pt == RV_FUNC_CALL_ARG_ON_STACK) return prev_nd + 1u;
    if (pt == RV_FUNC_CALL_ARG && P.rt[i - 1] == DT_FLOAT) {
        const int32_t v = s32(u32(P.ci[i - 1]) - prev_nd - 8u);
        return u32(v > 0 ? v : 0);
    }
    return P.nd1[i];
}

PTL_HD bool pre_list_hit(const Prog& P, int64_t i) {
    const uint32_t pt = P.nt[i - 1];
    return pt == RV_FUNC_CALL_ARG_ON_STACK || (pt == RV_FUNC_CALL_ARG && P.rt[i - 1] == DT_FLOAT);
}

// A lane reads its predecessor's data as loaded at the top of its block: the
// predecessor's pass-2 value when it sits in the previous block (lane 7), else the
// pass-1 value.  The chain is at most two long.
PTL_HD void st_pre_lists(const Prog& P, uint32_t i) {
    const uint32_t b = i / 8;
    uint32_t v = P.nd1[i];
    if (pre_list_block(P, b) && pre_list_hit(P, i)) {
        uint32_t prev;
        if ((i & 7u) == 0 && i > 0) {
            const uint32_t j = i - 1;  // lane 7 of block b-1
            prev = (pre_list_block(P, b - 1) && pre_list_hit(P, j)) ? pre_list_value(P, j, P.nd1[j - 1]) : P.nd1[j];
        } else {
            prev = P.nd1[static_cast<int64_t>(i) - 1];
        }
        v = pre_list_value(P, i, prev);
    }
    P.nd[i] = v;
}

// Float comparisons, rv_generator_avx.cpp:270-305.  A block reads its nodes' data types
// once, then marks parents FLOAT; later blocks see the marks.  Node c therefore reads
// FLOAT when a child in an earlier block marked it.  Each node that starts FLOAT walks
// up while the mark would be read by the next block up; the walks only set flags.
PTL_HD bool pre_parent_eq(const Prog& P, uint32_t c) {
    const int32_t p = P.par[c];
    const uint32_t pt = P.nt[p > -1 ? p : 0];
    return (pt & RV_EQ) == RV_EQ;
}

PTL_HD void st_pre_float(const Prog& P, uint32_t c) {
    if (P.rt[c] != DT_FLOAT || !pre_parent_eq(P, c)) return;
    uint32_t cur = c;
    for (uint32_t guard = 0; guard < P.nb8 + 1; ++guard) {
        const int32_t p = P.par[cur];
        if (p < 0) {  // the reference would store in front of its buffer
            record_error(P.err, ST_UNSUPPORTED, W_PRE, cur);
            return;
        }
        P.fflag[p] = 1;
        if (cur / 8 < u32(p) / 8 && pre_parent_eq(P, u32(p))) {
            cur = u32(p);
            continue;
        }
        return;
    }
}

PTL_HD void st_pre_float_apply(const Prog& P, uint32_t i) {
    if (P.fflag[i]) P.rt[i] = DT_FLOAT;
}

// ================================================================== isn_cnt
// Instruction count per node, rv_generator_avx.cpp:315-369.
PTL_HD uint32_t st_count(const Prog& P, uint32_t i) {
    const uint32_t t = P.nt[i];
    const uint32_t rt = P.rt[i];
    uint32_t v = P.tab.size(t, rt);
    if (t == RV_FUNC_CALL_ARG_LIST && (i > 0 || !P.scalar)) {  // the scalar generator skips node 0 (:325)
        v += 1u;
        const int64_t q = static_cast<int64_t>(i) - 1;
        if ((P.nt[q] & RV_FUNC_CALL_ARG) == RV_FUNC_CALL_ARG) v += u32(P.ci[q]) + 1u;
    }
    const int32_t p = P.par[i];
    if (P.scalar && p == -1) return v;  // and the root's parent (rv_generator.cpp:334)
    const uint32_t pt = P.nt[p != -1 ? p : 0];
    const int32_t ci = P.ci[i];
    const bool if_else = pt == RV_IF_ELSE;
    if (ci == 0 && (if_else || pt == RV_IF)) v += 1u;
    if (ci == 1 && (if_else || pt == RV_WHILE)) v += 1u;
    return v;
}

// Location fix-ups, rv_generator_avx.cpp:398-447.  The condition child of an if/while
// (and the child of a declaration-side argument) moves its parent to just past its own
// code; call arguments are placed inside their list.  Neither write target is read by
// the other rule, so both run in parallel from the scanned locations: first every node
// takes its own (or its call-argument) location, then condition children overwrite
// their parents -- except call arguments, whose list rule comes later in the reference.
// The scanned location as the fixes read it: the scalar generator first sets the
// locations of invalid nodes to 0xFFFFFFFF (rv_generator.cpp:364-369).
PTL_HD uint32_t fix_loc0(const Prog& P, int64_t i) {
    return (P.scalar && P.nt[i] == RV_INVALID) ? 0xFFFFFFFFu : P.loc0[i];
}

PTL_HD void st_fix_own(const Prog& P, uint32_t i) {
    if ((P.nt[i] & RV_FUNC_CALL_ARG) == RV_FUNC_CALL_ARG) {
        P.loc[i] = fix_loc0(P, P.par[i]) + u32(P.ci[i]) + 1u;
    } else {
        P.loc[i] = fix_loc0(P, i);
    }
}

PTL_HD void st_fix_cond(const Prog& P, uint32_t i) {
    const int32_t p = P.par[i];
    const uint32_t pt = P.nt[p > -1 ? p : 0];
    const bool cond = ((pt & RV_IF) == RV_IF) && (P.ci[i] == s32(pt & 1u));
    if (!cond) return;
    if (p < 0) {
        record_error(P.err, ST_UNSUPPORTED, W_CNT, i);
        return;
    }
    if ((pt & RV_FUNC_CALL_ARG) == RV_FUNC_CALL_ARG) return;  // overwritten by the list rule
    P.loc[p] = fix_loc0(P, i) + P.tab.size(P.nt[i], P.rt[i]);
}

// Function table, rv_generator_avx.cpp:451-517.  decl[] holds the FUNC_DECL indices in
// order (zero past F, as the reference's padded buffer).
PTL_HD void st_functab(const Prog& P, uint32_t f) {
    const uint32_t d = P.decl[f];
    P.fn_id[f] = P.nd[d];
    const uint32_t off = 6u + P.loc[d];
    P.fn_start[f + 1] = off;
    // function_sizes[f] = offset[f] - offset[f-1], offset[-1] = 0
    const uint32_t prev = f == 0 ? 0u : 6u + P.loc[P.decl[f - 1]];
    P.fn_size[f] = off - prev;
}

PTL_HD void st_functab_end(const Prog& P, uint32_t f) {
    P.fn_end[f] = P.fn_start[f] + P.fn_size[f];
    P.fn_start0[f] = P.fn_start[f];
    P.fn_size0[f] = P.fn_size[f];
}

// ================================================================== isn_gen
// One lane of the reference's level loop body, rv_generator_avx.cpp:597-881: a node and
// one of its four instruction slots.  Lanes of the same node differ only in the slot.
struct GenLane {
    bool has, prop, nopar, lfp, nonc, call;
    uint32_t par, ci, pt, iib, rdv, dpv;
    int32_t pai;
};

// What the four lanes of node x read from the node arrays, read once per node (the
// stages store between lanes, so per-lane reads would be repeated after each store).
struct GenNode {
    uint32_t x, t, rt, par, ntp, ci, loc, nd;
};

// stored_ntp: the parent's type from the byte the propagation pass keeps per node (the
// AVX passes after it), instead of a read at the parent's index.
PTL_HD GenNode gen_node(const Prog& P, uint32_t x, bool stored_ntp = false) {
    GenNode N;
    N.x = x;
    N.t = P.nt[x];
    N.rt = P.rt[x];
    N.par = u32(P.par[x]);
    if (stored_ntp) N.ntp = P.fflag[x];
    else N.ntp = s32(N.par) == -1 ? 0u : P.nt[s32(N.par)];  // the parent's type
    N.ci = u32(P.ci[x]);
    N.loc = P.loc[x];
    N.nd = P.nd[x];
    return N;
}

// d: the slot's packed table fields (Tab::gdesc).
PTL_HD GenLane gen_lane(const GenNode& N, uint32_t s, uint32_t d) {
    GenLane L;
    const uint32_t rt = N.rt;
    L.has = gd_has(d);
    L.prop = L.has || s == 0;
    L.par = L.prop ? N.par : 0u;
    L.nopar = s32(L.par) == -1;
    L.lfp = !L.nopar && L.prop;
    L.pt = L.lfp ? N.ntp : 0u;
    L.ci = L.lfp ? N.ci : 0u;
    L.nonc = ((L.pt & RV_IF) == RV_IF) && !(L.ci == (L.pt & 1u));
    L.call = L.nonc;
    if ((L.nopar || !L.nonc) && L.prop) {
        const uint32_t calc = gd_pai(d);
        if (calc == 1) L.call = true;
        if (calc == 2 && s32(rt) > 1) L.call = true;
    }
    L.pai = L.call ? s32(L.par * 3u + L.ci) : -1;
    L.iib = s + (L.prop ? N.loc : 0u);
    uint32_t r = 0;
    if (L.has) {
        const uint32_t calc = gd_out(d);
        if (calc == 3) r |= 32u;
        if (calc == 4) r |= 10u;
        if (calc == 1) r |= N.nd + 10u;
        if (calc == 2) r |= N.nd + 42u;
        bool hov = L.call;
        if (calc == 0 && gd_has_output(d)) hov = true;
        if (hov) r |= L.iib + 64u;
    }
    L.rdv = r;
    const bool use_rd = L.nopar || (!L.nonc && L.lfp);
    const uint32_t instr_no = L.iib + (L.nonc ? gd_size(d) : 0u);
    L.dpv = (use_rd ? r : 0u) | (L.nonc ? instr_no : 0u);
    return L;
}

// Data propagated to the parent's registers, rv_generator_avx.cpp:872-881.  The value a
// node propagates never depends on the registers array, and every parent slot has one
// writer (child indices 0..2), so all nodes write at once; the node's last writing lane
// wins, as in the reference.
PTL_HD void st_gen_prop(const Prog& P, uint32_t x) {
    const GenNode N = gen_node(P, x);
    P.fflag[x] = static_cast<uint8_t>(N.ntp);  // rv node types fit a byte
    const Tab::Slots4 D = P.tab.gdesc(N.t, N.rt);
    int32_t target = -1;
    uint32_t value = 0;
    for (uint32_t s = 0; s < 4; ++s) {
        const GenLane L = gen_lane(N, s, D.v[s]);
        if (L.pai >= 0) {
            target = L.pai;
            value = L.dpv;
        }
    }
    if (target < 0) return;
    // A child index above 2 would write into another node's registers; the reference's
    // result then depends on its visiting order.  Programs from the front end never do.
    if (N.ci > 2u || u32(target) >= 3u * P.n) {
        record_error(P.err, ST_UNSUPPORTED, W_GEN, x);
        return;
    }
    P.regs[target] = value;
}

// Where the lane's instruction goes, rv_generator_avx.cpp:713-750.  r1 / r2: the node's
// registers 1 and 2 (read only by if-else and while nodes).
PTL_HD uint32_t gen_loc(const Prog& P, const GenNode& N, uint32_t s, const GenLane& L, uint32_t r1, uint32_t r2) {
    const uint32_t t = N.t;
    uint32_t loc = L.has ? L.iib : 0u;
    const bool ie = s == 1 && t == RV_IF_ELSE;
    const bool wh = s == 1 && t == RV_WHILE;
    if (ie) loc = r1;
    if (wh) loc = r2;
    const bool add2 = t == RV_FUNC_DECL || (s > 1 && t == RV_FUNC_DECL_DUMMY);
    const bool fcal = s == 1 && t == RV_FUNC_CALL_ARG_LIST;
    if (add2 || fcal) loc += 2u;
    if (fcal) {
        const int64_t prev = static_cast<int64_t>(N.x) - 1;
        if ((P.nt[prev] & RV_FUNC_CALL_ARG) == RV_FUNC_CALL_ARG) loc += u32(P.ci[prev]);
    }
    return loc;
}

// Levels run deepest first; within a level the reference visits nodes in its sorted
// order, two nodes per body and slots in order.  A later visit overwrites an earlier
// one at the same word, so the write with the largest key wins.  The slot is the key's
// low two bits.
PTL_HD unsigned long long gen_key(const Prog& P, uint32_t x) {
    const unsigned long long lvl = static_cast<unsigned long long>(P.max_depth - u32(P.dep[x]));
    return (lvl << 40) | (static_cast<unsigned long long>(P.pos[x]) << 2);
}

PTL_HD void st_gen_claim(const Prog& P, uint32_t x) {
    const Tab::Slots4 D = P.tab.gdesc(P.nt[x], P.rt[x]);
    if (!((D.v[0] | D.v[1] | D.v[2] | D.v[3]) & 1u)) return;  // no slot has an instruction
    const GenNode N = gen_node(P, x, true);
    const unsigned long long key = gen_key(P, x);
    const bool loop2 = N.t == RV_IF_ELSE || N.t == RV_WHILE;  // slot 1 goes where a register says
    const uint32_t r1 = loop2 ? P.regs[x * 3u + 1u] : 0u, r2 = loop2 ? P.regs[x * 3u + 2u] : 0u;
    for (uint32_t s = 0; s < 4; ++s) {
        if (!gd_has(D.v[s])) continue;  // most slots: no instruction
        const GenLane L = gen_lane(N, s, D.v[s]);
        const uint32_t loc = gen_loc(P, N, s, L, r1, r2);
        if (loc >= P.W) {
            record_error(P.err, ST_UNSUPPORTED, W_GEN, x);
            continue;
        }
        at_max_u64(&P.owner[loc], key | s);
    }
}

PTL_HD void st_gen_write(const Prog& P, uint32_t x) {
    const Tab::Slots4 D = P.tab.gdesc(P.nt[x], P.rt[x]);
    if (!((D.v[0] | D.v[1] | D.v[2] | D.v[3]) & 1u)) return;  // no slot has an instruction
    const GenNode N = gen_node(P, x, true);
    const uint32_t t = N.t;
    const uint32_t rt = N.rt;
    const unsigned long long key = gen_key(P, x);
    const uint32_t reg[3] = {P.regs[x * 3u], P.regs[x * 3u + 1u], P.regs[x * 3u + 2u]};
    const uint32_t nd = N.nd;
    const Tab::Slots4 Wd = P.tab.gword(t, rt);
    for (uint32_t s = 0; s < 4; ++s) {
        const uint32_t d = D.v[s];
        if (!gd_has(d)) continue;  // most slots: no instruction
        const GenLane L = gen_lane(N, s, d);
        const uint32_t loc = gen_loc(P, N, s, L, reg[1], reg[2]);
        if (loc >= P.W || P.owner[loc] != (key | s)) continue;
        // instruction word and constants, :752-779
        uint32_t w = Wd.v[s];
        const uint32_t cc = gd_cnst(d);
        if (cc == 1) w |= nd & 0xFFFFF000u;
        if (cc == 2) w |= (nd & 0xFFFu) << 20;
        const uint32_t m4 = nd * 4u;
        if (cc == 3) w |= (0u - (m4 + 8u)) << 20;
        if (cc == 4) w |= m4 << 20;
        if (cc == 5) w |= (0u - m4) << 20;
        // jump target, :781-814
        const uint32_t jc = gd_jt(d);
        uint32_t jv = 0;
        if (s32(jc) > 0 && !(s32(jc) > 5)) {
            uint32_t v = s32(jc) > 2 ? reg[2] : reg[1];
            if ((jc & 1u) == 0) v += 1u;
            jv = v;
        }
        if ((jc == 6 || jc == 7) && nd >= P.F) {  // a function id past the table
            record_error(P.err, ST_UNSUPPORTED, W_GEN, x);
            continue;
        }
        if (jc == 6) jv |= P.fn_end[s32(nd)] - 6u;
        if (jc == 7) jv |= P.fn_start[s32(nd)];
        // operands, :816-850
        uint32_t ops[2];
        for (uint32_t k = 0; k < 2; ++k) {
            const uint32_t c = gd_opd(d, k);
            uint32_t a = 0;
            if (c == 1 || c == 4 || c == 5 || c == 6) {
                uint32_t ri = 0;
                if (c == 1) ri += k;
                if (c == 4 || c == 5) ri += 1u;
                if (c == 5) ri -= k;
                a = ri == 0 ? reg[0] : (ri == 1 ? reg[1] : reg[2]);
            }
            if (c == 2) a |= nd + 10u;
            if (c == 3) a |= nd + 42u;
            if (c == 7) a |= L.iib + 63u;
            ops[k] = a;
        }
        P.instr[loc] = w;
        P.rd[loc] = L.rdv;
        P.rs1[loc] = ops[0];
        P.rs2[loc] = ops[1];
        P.jt[loc] = jv;
    }
}

// ================================================================== optimize
// rv_generator_avx.cpp:891-1016.  The reference iterates a Jacobi sweep until nothing
// changes: used[v] is cleared for operands of instructions whose (virtual) result is
// unused, while operands of stores are re-marked each sweep.  The sweep only ever
// clears bits and is monotone, so any fair order of the same updates reaches the same
// fixed point (the greatest one below the initial marks); the GPU sweeps in place.
PTL_HD void st_opt_mark(const Prog& P, uint32_t i) {
    const int32_t a = s32(P.rs1[i] - 64u);
    const int32_t b = s32(P.rs2[i] - 64u);
    const uint32_t f = P.instr[i] & 0x707Fu;
    const bool store = f == 0x2023u || f == 0x2027u;
    if (a >= 0) {
        if (u32(a) >= P.W) { record_error(P.err, ST_UNSUPPORTED, W_OPT, i); return; }
        P.used[a] = 1;
        if (store) P.smark[a] = 1;
    }
    if (b >= 0) {
        if (u32(b) >= P.W) { record_error(P.err, ST_UNSUPPORTED, W_OPT, i); return; }
        P.used[b] = 1;
        if (store) P.smark[b] = 1;
    }
}

// Clears the used marks of the operands of instruction i when its result is unused;
// returns how many it cleared, their word indices in cleared[0..].
PTL_HD uint32_t st_opt_sweep_cleared(const Prog& P, uint32_t i, uint32_t cleared[2]) {
    const uint32_t r = P.rd[i];
    if (!(s32(r) > 63)) return 0;
    if (r - 64u >= P.W) { record_error(P.err, ST_UNSUPPORTED, W_OPT, i); return 0; }
    if (P.used[r - 64u]) return 0;
    uint32_t nc = 0;
    const int32_t a = s32(P.rs1[i] - 64u);
    const int32_t b = s32(P.rs2[i] - 64u);
    if (a >= 0 && u32(a) < P.W && !P.smark[a] && P.used[a]) { P.used[a] = 0; cleared[nc++] = u32(a); }
    if (b >= 0 && u32(b) < P.W && !P.smark[b] && P.used[b]) { P.used[b] = 0; cleared[nc++] = u32(b); }
    return nc;
}

// Returns true when it cleared a mark.
PTL_HD bool st_opt_sweep(const Prog& P, uint32_t i) {
    uint32_t cleared[2];
    return st_opt_sweep_cleared(P, i, cleared) != 0;
}

PTL_HD void st_opt_final(const Prog& P, uint32_t i) {
    // used_instrs = ~(rd > 63) | used[i]; lanes past W read a zero used flag
    const bool keep = !(s32(P.rd[i]) > 63) || (i < P.W && P.used[i]);
    P.used_instrs[i] = keep ? 0xFFFFFFFFu : 0u;
}

// ================================================================== regalloc
// One step of the reference's per-function register allocator, rv_generator_avx.cpp:
// 1055-1397, for one function's instruction.
struct RaStep {
    uint32_t ins, r1, r2, ord;  // instruction and its virtual/physical operands
    uint32_t r1r, r2r, rdr;     // allocated physical registers
    unsigned long long cleared, rdm;
    uint64_t trig;              // physical registers whose current symbols get marked swapped
};

PTL_HD uint64_t bit_of(uint32_t r) {
    const int32_t sr = s32(r);
    return (sr >= 0 && sr < 64) ? (1ull << sr) : 0ull;
}

// ptilopsis::ffz(uint64_t) (include/utils.hpp:23-47) calls __builtin_ffs(int): only the
// low 32 bits are searched and 64 means "none".
PTL_HD uint32_t ffz_low32(unsigned long long m) {
    const uint32_t low = static_cast<uint32_t>(m);
    if (low == 0xFFFFFFFFu) return 64u;
#if defined(__CUDA_ARCH__)
    return static_cast<uint32_t>(__ffs(static_cast<int>(~low)) - 1);
#else
    return static_cast<uint32_t>(__builtin_ctz(~low));
#endif
}

// Lookups -> allocation -> swap triggers (:1150-1285).  r1s/r2s: whether the rs1/rs2
// symbols read as swapped at this point.
PTL_HD void ra_compute(RaStep& S, unsigned long long lifetime, uint32_t r1reg, bool r1s,
                       uint32_t r2reg, bool r2s) {
    const bool fop = (S.ins & 0x7Fu) == 0x53u;
    uint32_t r1r = r1reg, r2r = r2reg;
    if (r1s) r1r = (S.ins == 0xC0007053u || fop) ? 37u : 5u;
    if (r2s) r2r = fop ? 38u : 6u;
    S.r1r = r1r;
    S.r2r = r2r;
    const unsigned long long clear = (bit_of(r1r) | bit_of(r2r)) & ~1ull;
    S.cleared = lifetime & ~clear;
    uint32_t r = S.ord;
    if (s32(r) > 63) {
        const bool rdf = S.ins == 0xD0007053u || fop;
        const unsigned long long adj = rdf ? 0x00000000FFFFFFFFull : 0xFFFFFFFF00000000ull;
        r = ffz_low32(S.cleared | adj);
        if (r == 64u) r = rdf ? 37u : 5u;
    }
    S.rdr = r;
    S.rdm = bit_of(r);
    uint64_t trig = 0;
    if (r != 0 && (S.cleared & S.rdm)) trig |= S.rdm;
    if (r1r != 0 && (lifetime & bit_of(r1r))) trig |= bit_of(r1r);
    if (r2r != 0 && (lifetime & bit_of(r2r))) trig |= bit_of(r2r);
    S.trig = trig;
}

// Loads step i's instruction of a function with isn_cnt range [start, start+size).
PTL_HD bool ra_load_at(const Prog& P, uint32_t start, uint32_t size, uint32_t i, RaStep& S) {
    if (s32(i) >= s32(size)) return false;
    const uint32_t off = start + i;
    S.ins = P.instr[off];
    S.r1 = P.rs1[off];
    S.r2 = P.rs2[off];
    S.ord = P.rd[off];
    return true;
}

PTL_HD bool ra_load(const Prog& P, uint32_t f, uint32_t i, RaStep& S) {
    const uint32_t sz = P.fn_size0[f];
    if (s32(i) >= s32(sz)) return false;
    const uint32_t off = P.fn_start0[f] + i;
    S.ins = P.instr[off];
    S.r1 = P.rs1[off];
    S.r2 = P.rs2[off];
    S.ord = P.rd[off];
    return true;
}

// Virtual registers of function f must be its own instructions: that is what keeps
// functions outside lane 0 independent of each other.
PTL_HD bool ra_own(const Prog& P, uint32_t f, uint32_t r) {
    if (!(s32(r) > 63)) return true;
    const uint32_t v = r - 64u;
    const uint32_t st = P.fn_start0[f];
    return v >= st && v - st < P.fn_size0[f];
}

// A virtual register names an instruction of the program (checked where it is read).
PTL_HD bool ra_in_range(const Prog& P, uint32_t r) { return !(s32(r) > 63) || r - 64u < P.W; }

// Whether instruction i names a virtual register outside its own function (bit 0).  The
// reference lets that happen when an instruction number lands in a register operand
// (a child of a float-as-int call argument propagates its instruction count, which
// reads as virtual register count-64); such programs couple functions through the
// symbol table and take the serial path below.  Bit 1: a lane-0 instruction defines a
// virtual register that an earlier-counted instruction also defines (defcnt counts the
// definitions, zeroed beforehand); the lane-0 pass then finds row-0 values by hashing.
// The function holding word i: the last function start <= i (0 when the first start is
// past i).  The starts never decrease (6 + loc of the declarations, which no fix-up rule
// moves, over an exclusive scan of sizes), so "start <= i" holds on a prefix and both the
// bisection and a walk find its end.  hint: the answer for an earlier word of the same
// program; from it a short walk forward replaces the bisection.
PTL_HD uint32_t function_of(const Prog& P, uint32_t i, uint32_t hint = 0xFFFFFFFFu) {
    if (hint < P.F && P.fn_start0[hint] <= i) {
        uint32_t f = hint;
        for (int k = 0; k < 4; ++k) {
            if (f + 1u >= P.F || P.fn_start0[f + 1u] > i) return f;
            ++f;
        }
    }
    uint32_t lo = 0, hi = P.F;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (P.fn_start0[mid] <= i) lo = mid; else hi = mid;
    }
    return lo;
}

PTL_HD uint32_t st_ra_cross(const Prog& P, uint32_t i, uint32_t* defcnt, uint32_t* hint = nullptr) {
    const uint32_t lo = function_of(P, i, hint ? *hint : 0xFFFFFFFFu);
    if (hint) *hint = lo;
    const uint32_t rd = P.rd[i];
    if (!ra_own(P, lo, P.rs1[i]) || !ra_own(P, lo, P.rs2[i]) || !ra_own(P, lo, rd)) return 1u;
    if ((lo & 7u) != 0 || !(s32(rd) > 63)) return 0u;
#if defined(__CUDA_ARCH__)
    const uint32_t before = atomicAdd(&defcnt[rd - 64u], 1u);
#else
    const uint32_t before = defcnt[rd - 64u]++;
#endif
    return before != 0 ? 2u : 0u;
}

// The reference's step loop as written (rv_generator_avx.cpp:1400-1413 with one worker):
// for every step, the functions in index order, 8 to a group; within a group the
// lookups of all lanes precede the swap marks, which precede the updates.  One thread
// runs it; it serves programs whose functions share symbols.  active holds F entries.
PTL_HD void st_ra_serial(const Prog& P, uint32_t* active) {
    uint32_t row0[64];
    for (int p = 0; p < 64; ++p) row0[p] = 0xFFFFFFFFu;
    uint32_t na = 0;
    for (uint32_t f = 0; f < P.F; ++f) if (s32(P.fn_size0[f]) > 0) active[na++] = f;
    for (uint32_t i = 0; na > 0; ++i) {
        uint32_t snap[64];
        for (int p = 0; p < 64; ++p) snap[p] = row0[p];
        uint32_t a = 0;
        while (a < na) {
            const uint32_t j = active[a] / 8u;
            RaStep L[8];
            uint32_t fl[8];
            uint32_t m = 0;
            while (a < na && active[a] / 8u == j) {
                const uint32_t f = active[a++];
                RaStep S;
                if (!ra_load(P, f, i, S)) continue;
                if (S.ins == 0x000000EFu || !ra_in_range(P, S.r1) || !ra_in_range(P, S.r2) || !ra_in_range(P, S.ord)) {
                    record_error(P.err, ST_UNSUPPORTED, W_RA1, P.fn_start0[f] + i);
                    return;
                }
                fl[m] = f;
                L[m++] = S;
            }
            for (uint32_t k = 0; k < m; ++k) {
                RaStep& S = L[k];
                const bool v1 = s32(S.r1) > 63, v2 = s32(S.r2) > 63;
                ra_compute(S, P.lifetime[fl[k]], v1 ? P.symreg[S.r1 - 64u] : 0u, v1 && P.symswp[S.r1 - 64u] != 0,
                           v2 ? P.symreg[S.r2 - 64u] : 0u, v2 && P.symswp[S.r2 - 64u] != 0);
            }
            // marks: rd lanes, then rs1 lanes, then rs2 lanes
            for (int role = 0; role < 3; ++role) {
                for (uint32_t k = 0; k < m; ++k) {
                    const RaStep& S = L[k];
                    const uint32_t r = role == 0 ? S.rdr : (role == 1 ? S.r1r : S.r2r);
                    if (!(S.trig & bit_of(r))) continue;
                    const bool fires = role == 0 ? (r != 0 && (S.cleared & S.rdm))
                                                 : (r != 0 && (P.lifetime[fl[k]] & bit_of(r)));
                    if (!fires) continue;
                    const uint32_t v = snap[r & 63u];
                    if (s32(v - 64u) >= 0) P.symswp[v - 64u] = 0xFFFFFFFFu;
                }
            }
            for (uint32_t k = 0; k < m; ++k) P.lifetime[fl[k]] = L[k].cleared | L[k].rdm;
            for (uint32_t k = 0; k < m; ++k) {
                if ((fl[k] & 7u) != 0) continue;  // only lane 0 writes row 0
                const RaStep& S = L[k];
                if (S.ord != 0) row0[S.rdr & 63u] = S.ord;
                if (S.r1r != S.rdr && s32(S.r1r) >= 0 && S.r1r < 64u) row0[S.r1r] = 0xFFFFFFFFu;
                if (S.r2r != S.rdr && s32(S.r2r) >= 0 && S.r2r < 64u) row0[S.r2r] = 0xFFFFFFFFu;
            }
            for (uint32_t k = 0; k < m; ++k) if (s32(L[k].ord) > 63) { P.symreg[L[k].ord - 64u] = L[k].rdr; P.symswp[L[k].ord - 64u] = 0; }
            for (uint32_t k = 0; k < m; ++k) if (s32(L[k].r1) > 63) { P.symreg[L[k].r1 - 64u] = L[k].r1r; P.symswp[L[k].r1 - 64u] = 0; }
            for (uint32_t k = 0; k < m; ++k) if (s32(L[k].r2) > 63) { P.symreg[L[k].r2 - 64u] = L[k].r2r; P.symswp[L[k].r2 - 64u] = 0; }
        }
        uint32_t w = 0;
        for (uint32_t k = 0; k < na; ++k) if (s32(i + 1u) < s32(P.fn_size0[active[k]])) active[w++] = active[k];
        na = w;
    }
}

// Spill flag per virtual register: the reference copies swapped-ness of the symbol at
// each function start down to the function's other registers (:1464-1469).
PTL_HD void st_ra_spill(const Prog& P, uint32_t v, uint32_t* hint = nullptr) {
    // last function start <= v (starts are ascending in valid programs; the reference's
    // fill follows index order, which is what function_of's bisection reproduces)
    const uint32_t lo = function_of(P, v, hint ? *hint : 0xFFFFFFFFu);
    if (hint) *hint = lo;
    const uint32_t s = P.fn_start0[lo];
    P.spill[v] = s <= v ? (P.symswp[s] & 1u) : 0u;
}

PTL_HD uint32_t st_ra_count(const Prog& P, uint32_t i) {
    if (!P.used_instrs[i]) return 0;
    uint32_t c = 1;
    const uint32_t r1 = P.rs1[i], r2 = P.rs2[i], r = P.rd[i];
    if (!ra_in_range(P, r1) || !ra_in_range(P, r2) || !ra_in_range(P, r)) {
        record_error(P.err, ST_UNSUPPORTED, W_RA_SCATTER, i);
        return 1;
    }
    if (s32(r1) > 63 && P.symswp[r1 - 64u]) ++c;
    if (s32(r2) > 63 && P.symswp[r2 - 64u]) ++c;
    if (s32(r) > 63 && P.symswp[r - 64u]) ++c;
    return c;
}

// Emit the instruction with allocated registers plus reloads/spills, :1552-1697.
PTL_HD void st_ra_scatter(const Prog& P, uint32_t i) {
    if (!P.used_instrs[i]) return;
    if (!ra_in_range(P, P.rs1[i]) || !ra_in_range(P, P.rs2[i]) || !ra_in_range(P, P.rd[i]) ||
        P.jt[i] >= P.wb8 + 16u) {
        record_error(P.err, ST_UNSUPPORTED, W_RA_SCATTER, i);
        return;
    }
    const uint32_t base = P.roffs[i];
    const uint32_t ins = P.instr[i];
    const bool fop = (ins & 0x7Fu) == 0x53u;

    const uint32_t r1 = P.rs1[i];
    uint32_t l1 = 0xFFFFFFFFu, st1 = 0, al1 = (s32(r1) > 63) ? 0u : r1;
    if (s32(r1) > 63) {
        const uint32_t sw = P.symswp[r1 - 64u];
        l1 = ~sw | base;
        st1 = P.spill[r1 - 64u];
        al1 |= sw ? 0u : P.symreg[r1 - 64u];
        if (sw) al1 |= (ins == 0xC0007053u || fop) ? 37u : 5u;
    }
    const uint32_t r2 = P.rs2[i];
    uint32_t l2 = 0xFFFFFFFFu, st2 = 0, al2 = (s32(r2) > 63) ? 0u : r2;
    if (s32(r2) > 63) {
        const uint32_t sw = P.symswp[r2 - 64u];
        // The reference tests its own initial value here (:1598), so an rs2 reload lands
        // on the rs1 reload's slot.
        l2 = ~sw | base;
        st2 = P.spill[r2 - 64u];
        al2 |= sw ? 0u : P.symreg[r2 - 64u];
        if (sw) al2 |= fop ? 38u : 6u;
    }
    const uint32_t mo = base + (s32(l1) > 0 ? 1u : 0u) + (s32(l2) > 0 ? 1u : 0u);
    const uint32_t r = P.rd[i];
    uint32_t ro = 0xFFFFFFFFu, str = 0, ar = (s32(r) > 63) ? 0u : r;
    if (s32(r) > 63) {
        const uint32_t sw = P.symswp[r - 64u];
        ro = ~sw | (mo + 1u);
        str = P.spill[r - 64u];
        ar |= P.symreg[r - 64u];
    }
    const uint32_t cap = P.w2b8 + 16u;  // writes of the padding lanes stay in the pad
    if (s32(l1) >= 0 && l1 < cap) { P.ni[l1] = (((st1 - 1u) * 4u) << 20) | 0x2003u; P.nrd[l1] = 5; }
    if (s32(l2) >= 0 && l2 < cap) { P.ni[l2] = (((st2 - 1u) * 4u) << 20) | 0x2003u; P.nrd[l2] = 6; }
    if (s32(mo) >= 0 && mo < cap) {
        P.ni[mo] = ins;
        P.nrd[mo] = ar;
        P.nr1[mo] = al1;
        P.nr2[mo] = al2;
        P.njt[mo] = P.roffs[P.jt[i]];
    }
    if (s32(ro) >= 0 && ro < cap) {
        const uint32_t imm = (str - 1u) * 0xFFFFFFFCu;
        P.ni[ro] = 0x2023u | ((imm & 0x1Fu) << 7) | ((imm & 0xFEu) << 19);
        P.nr1[ro] = ar;
    }
}

// fix_func_tab_avx, rv_generator_avx.cpp:1816-1837, on function f < F.  (The reference
// also rewrites the padding lanes of the last block; nothing reads those lanes.)
PTL_HD void st_fix_functab(const Prog& P, uint32_t f, const uint32_t* offs, uint32_t offs_size) {
    const uint32_t si = P.fn_start[f];
    const uint32_t so = offs[s32(si)];
    const uint32_t ei = si + P.fn_size[f];
    const bool past = s32(ei) >= s32(offs_size);
    const uint32_t eo = past ? offs[static_cast<int64_t>(offs_size) - 1] + 1u : offs[s32(ei)];
    P.fn_start[f] = so;
    P.fn_end[f] = eo;
    P.fn_size[f] = eo - so;
}

// Frame-size words at each function's prologue and epilogue, :1701-1811.  Preserve
// masks stay zero in the reference, so every frame is 8 bytes.
PTL_HD void st_ra_frame(const Prog& P, uint32_t f) {
    const uint32_t upper = 0x00000437u;                  // lui s0, 0
    const uint32_t lower = (8u << 20) | 0x00040413u;     // addi s0, s0, 8
    const uint32_t st = P.fn_start[f];
    const uint32_t en = st + P.fn_size[f];
    const uint32_t at[4] = {st + 2u, st + 3u, en - 6u, en - 5u};
    const uint32_t w[4] = {upper, lower, upper, lower};
    for (int k = 0; k < 4; ++k) {
        const uint32_t p = at[k];
        if (p >= P.W2) { record_error(P.err, ST_UNSUPPORTED, W_RA_SCATTER, f); continue; }
        P.ni[p] = w[k]; P.nrd[p] = 0; P.nr1[p] = 0; P.nr2[p] = 0; P.njt[p] = 0;
    }
}

// ================================================================== fix_jumps
// rv_generator_avx.cpp:1853-1993 with postprocess (:1995-2011) folded in.
PTL_HD uint32_t st_fj_size(const Prog& P, uint32_t i) {
    const uint32_t w = P.ni[i];
    const bool jump = (w & 0x7Fu) == 0x67u && w != 0x8067u;
    return jump ? 2u : (w != 0 ? 1u : 0u);
}

PTL_HD void st_fj_emit(const Prog& P, uint32_t i) {
    if (i >= P.W2) return;
    const uint32_t w = P.ni[i];
    if (w == 0) return;  // zero words vanish; the next word takes the slot
    const uint32_t at = P.joffs[i];
    const bool jump = (w & 0x7Fu) == 0x67u && w != 0x8067u;
    const bool branch = (w & 0x7Fu) == 0x63u;
    const uint32_t post = ((P.nrd[i] & 31u) << 7) | ((P.nr1[i] & 31u) << 15) | ((P.nr2[i] & 31u) << 20);
    if (!jump && !branch) {
        P.out[at] = w | post;
        return;
    }
    const uint32_t delta = 4u * P.joffs[s32(P.njt[i])] - at * 4u;
    if (jump) {
        const uint32_t upper = (delta & 0xFFFFF000u) >> 12;
        const uint32_t lower = delta & 0xFFFu;
        const uint32_t sign = (delta >> 11) & 1u;
        P.out[at] = ((upper + sign) << 12) | 0x97u;
        P.out[at + 1] = w | (lower << 20) | (1u << 15);
        return;
    }
    const uint32_t word = w | (((delta >> 12) & 1u) << 31) | (((delta >> 11) & 1u) << 7) |
                          (((delta >> 5) & 0x1Fu) << 25) | (((delta >> 1) & 0xFu) << 8);
    P.out[at] = word | post;
}

}  // namespace ptl
