// Scalar-semantics mode: the reference's proof-of-concept generator rv_generator_st
// (src/codegen/rv_generator.cpp:227-1736, the -s flag of src/main.cpp), whose output
// differs from rv_generator_avx's in the argument pass, the call-list pass, the float
// comparison pass, isn_gen's parent-slot and jump-target rules, the lui constant, and a
// register allocator with one register state per function and real preserve masks.
//
// Stages that compute the same thing in both generators (the depth order, optimize's
// fixed point, fix_jumps, postprocess) run the AVX stage functions of ptl_stages.cuh, and
// so does isn_cnt, whose three scalar differences are branches there (st_count,
// fix_loc0); the functions here replace the others.  Each is one thread's share, shared
// by the CUDA kernels and the host model, as in ptl_stages.cuh (the warp-per-function
// register allocation kernel restates s_ra_function's steps in ptl_kernels.cu).
#pragma once

#include "ptl_stages.cuh"

namespace ptl {

// ================================================================== preprocess
// Call-list stack argument counts, rv_generator.cpp:287-304: each list reads its
// predecessor (the last argument, post-order) as the argument pass left it.
PTL_HD void st_s_pre_lists(const Prog& P, uint32_t i) {
    uint32_t v = P.nd1[i];
    if (i > 0 && i < P.n && P.nt[i] == RV_FUNC_CALL_ARG_LIST) {
        const uint32_t prev = i - 1;
        int64_t stack_args = 0;
        if (P.nt[prev] == RV_FUNC_CALL_ARG) {
            if (P.rt[prev] == DT_FLOAT) {
                const int64_t int_args = static_cast<int64_t>(P.ci[prev]) - static_cast<int64_t>(P.nd1[prev]);
                stack_args = int_args - 8 > 0 ? int_args - 8 : 0;
            }
        } else if (P.nt[prev] == RV_FUNC_CALL_ARG_ON_STACK) {
            stack_args = static_cast<int64_t>(static_cast<uint32_t>(P.nd1[prev] + 1u));
        }
        v = static_cast<uint32_t>(stack_args);
    }
    P.nd[i] = v;
}

// Float comparisons, rv_generator.cpp:306-313: one ascending pass, a parent that tests
// equal-like (mask 0b1110) and has a FLOAT child becomes FLOAT.  The pass sees the marks
// it made at lower indices, so a FLOAT climbs a chain of such parents while each parent
// comes later in index order than the node that marked it.  Each FLOAT node walks up that
// chain setting flags; st_pre_float_apply folds them in.
PTL_HD void st_s_pre_float(const Prog& P, uint32_t c) {
    if (c >= P.n || P.rt[c] != DT_FLOAT) return;
    uint32_t cur = c;
    for (uint32_t guard = 0; guard <= P.max_depth + 1u; ++guard) {
        const int32_t p = P.par[cur];
        if (p < 0 || (P.nt[p] & RV_EQ) != RV_EQ) return;
        P.fflag[p] = 1;
        if (u32(p) < cur) return;  // the pass visited the parent already: the mark stops there
        cur = u32(p);
    }
}

// ================================================================== isn_gen
// One (node, slot) of the level loop, rv_generator.cpp:591-776.
struct SGenLane {
    bool has;
    int64_t pai;    // parent slot index written (negative: none)
    uint32_t iib;   // the slot's own word
    uint32_t rd;    // output register
    uint32_t dpv;   // value propagated to the parent slot
};

// get_parent_arg_idx (:478-520).  The reference multiplies by a size_t and returns
// int64, so the root's -1 parent gives -3 + child_idx, which is not the -1 it tests for.
PTL_HD int64_t s_parent_arg_idx(const Prog& P, const GenNode& N, uint32_t s) {
    const int32_t par = s32(N.par);
    const int64_t pidx = static_cast<int64_t>(par) * 3 + static_cast<int64_t>(s32(N.ci));
    const int32_t ci = s32(N.ci);
    if (par != -1) {
        const uint32_t pt = N.ntp;
        if (ci > 0 && (pt == RV_IF || pt == RV_IF_ELSE)) return pidx;
        if ((ci == 0 || ci == 2) && pt == RV_WHILE) return pidx;
    }
    const uint32_t calc = P.tab.pai(N.t, s, N.rt);
    if (calc == 1) return pidx;
    if (calc == 2 && N.rt > 1u) return pidx;
    return -1;
}

// get_data_prop_value (:522-556).
PTL_HD uint32_t s_prop_value(const Prog& P, const GenNode& N, uint32_t rd, uint32_t instr_offset) {
    if (s32(N.par) == -1) return rd;
    const uint32_t pt = N.ntp;
    const int32_t ci = s32(N.ci);
    const uint32_t instr_no = instr_offset + P.tab.size(N.t, N.rt);
    if (pt == RV_IF || pt == RV_IF_ELSE) return (ci == 1 || ci == 2) ? instr_no : rd;
    if (pt == RV_WHILE) return (ci == 0 || ci == 2) ? instr_no : rd;
    return rd;
}

PTL_HD SGenLane s_gen_lane(const Prog& P, const GenNode& N, uint32_t s) {
    SGenLane L;
    L.has = P.tab.has_instr(N.t, s, N.rt);
    L.iib = N.loc + s;
    L.pai = -1;
    L.rd = 0;
    L.dpv = 0;
    if (L.has) {
        L.pai = s_parent_arg_idx(P, N, s);
        const uint32_t calc = P.tab.out(N.t, s, N.rt);  // get_output_register (:638-656)
        if (calc == 1) L.rd = N.nd + 10u;
        else if (calc == 2) L.rd = N.nd + 42u;
        else if (calc == 3) L.rd = 32u;
        else if (calc == 4) L.rd = 10u;
        else L.rd = (L.pai != -1 || P.tab.has_output(N.t, s, N.rt)) ? L.iib + 64u : 0u;
        L.dpv = s_prop_value(P, N, L.rd, L.iib);
    } else if (s == 0) {  // no instruction: slot 0 still propagates (:760-767)
        L.pai = s_parent_arg_idx(P, N, 0);
        L.dpv = s_prop_value(P, N, 0, N.loc);
    }
    return L;
}

// Registers the node propagates to its parent: the reference scatters each level after
// computing it, its slots in order, so the node's last slot with a parent index wins;
// the value never depends on the registers array, so all levels propagate at once.
PTL_HD void st_s_gen_prop(const Prog& P, uint32_t x) {
    const GenNode N = gen_node(P, x);
    int64_t target = -1;
    uint32_t value = 0;
    for (uint32_t s = 0; s < 4; ++s) {
        const SGenLane L = s_gen_lane(P, N, s);
        if (L.pai >= 0 && static_cast<int32_t>(L.pai) >= 0) {
            target = L.pai;
            value = L.dpv;
        }
    }
    if (target < 0) return;
    // A child index above 2 writes into another node's registers, where the reference's
    // result depends on its visiting order.  Programs from the front end never do.
    if (s32(N.ci) > 2 || target >= 3ll * P.n) {
        record_error(P.err, ST_UNSUPPORTED, W_GEN, x);
        return;
    }
    P.regs[target] = value;
}

// get_instr_loc (:661-685).  The reference keeps the location in an int32.
PTL_HD int64_t s_instr_loc(const Prog& P, const GenNode& N, uint32_t s, uint32_t iib, uint32_t r1, uint32_t r2) {
    const uint32_t t = N.t;
    if (s == 1 && t == RV_IF_ELSE) return s32(r1);
    if (s == 1 && t == RV_WHILE) return s32(r2);
    if ((s >= 2 && t == RV_FUNC_DECL_DUMMY) || t == RV_FUNC_DECL) return s32(iib + 2u);
    if (s == 1 && t == RV_FUNC_CALL_ARG_LIST) {
        uint32_t res = iib + 2u;
        if (N.x != 0) {
            const uint32_t pt = P.nt[N.x - 1];
            if (pt == RV_FUNC_CALL_ARG || pt == RV_FUNC_CALL_ARG_FLOAT_AS_INT || pt == RV_FUNC_CALL_ARG_ON_STACK)
                res += u32(P.ci[N.x - 1]);
        }
        return s32(res);
    }
    return s32(iib);
}

// Sign extension of a 12-bit immediate (rv_generator.cpp:69-73).
PTL_HD uint32_t extend12(uint32_t x) { return u32(s32(x << 20) >> 20); }

PTL_HD void st_s_gen_claim(const Prog& P, uint32_t x) {
    const GenNode N = gen_node(P, x);
    const unsigned long long key = gen_key(P, x);
    const bool loop2 = N.t == RV_IF_ELSE || N.t == RV_WHILE;
    const uint32_t r1 = loop2 ? P.regs[x * 3u + 1u] : 0u, r2 = loop2 ? P.regs[x * 3u + 2u] : 0u;
    for (uint32_t s = 0; s < 4; ++s) {
        if (!P.tab.has_instr(N.t, s, N.rt)) continue;
        const int64_t loc = s_instr_loc(P, N, s, N.loc + s, r1, r2);
        if (loc < 0 || loc >= static_cast<int64_t>(P.W)) continue;  // the reference skips those
        at_max_u64(&P.owner[loc], key | s);
    }
}

PTL_HD void st_s_gen_write(const Prog& P, uint32_t x) {
    const GenNode N = gen_node(P, x);
    const uint32_t t = N.t, rt = N.rt, nd = N.nd;
    const unsigned long long key = gen_key(P, x);
    const uint32_t reg[3] = {P.regs[x * 3u], P.regs[x * 3u + 1u], P.regs[x * 3u + 2u]};
    for (uint32_t s = 0; s < 4; ++s) {
        if (!P.tab.has_instr(t, s, rt)) continue;
        const SGenLane L = s_gen_lane(P, N, s);
        const int64_t loc = s_instr_loc(P, N, s, L.iib, reg[1], reg[2]);
        if (loc < 0 || loc >= static_cast<int64_t>(P.W) || P.owner[loc] != (key | s)) continue;
        // instr_constant (:687-705)
        uint32_t w = P.tab.word(t, s, rt);
        const uint32_t cc = P.tab.cnst(t, s);
        if (cc == 1) w |= (nd - extend12(nd & 0xFFFu)) & 0xFFFFF000u;
        if (cc == 2) w |= (nd & 0xFFFu) << 20;
        if (cc == 3) w |= (0u - 4u * (nd + 2u)) << 20;
        if (cc == 4) w |= (4u * nd) << 20;
        if (cc == 5) w |= (0u - 4u * nd) << 20;
        // node_get_instr_arg (:718-736)
        uint32_t ops[2];
        for (uint32_t k = 0; k < 2; ++k) {
            const uint32_t c = P.tab.opd(t, s, rt, k);
            uint32_t a = 0;
            if (c == 1) a = reg[k];
            else if (c == 2) a = nd + 10u;
            else if (c == 3) a = nd + 42u;
            else if (c == 4) a = reg[1];
            else if (c == 5) a = reg[1 - k];
            else if (c == 6) a = reg[0];
            else if (c == 7) a = L.iib + 63u;
            ops[k] = a;
        }
        // instr_jt (:738-752)
        const uint32_t jc = P.tab.jt(t, s);
        uint32_t jv = 0;
        if ((jc == 6 || jc == 7) && nd >= P.F) {  // a function id past the table
            record_error(P.err, ST_UNSUPPORTED, W_GEN, x);
            continue;
        }
        if (jc == 1) jv = reg[1];
        else if (jc == 2) jv = reg[1] + 1u;
        else if (jc == 3) jv = reg[2];
        else if (jc == 4) jv = reg[2] + 1u;
        else if (jc == 5) jv = reg[0];
        else if (jc == 6) jv = P.fn_end[nd] - 6u;
        else if (jc == 7) jv = P.fn_start[nd];
        P.instr[loc] = w;
        P.rd[loc] = L.rd;
        P.rs1[loc] = ops[0];
        P.rs2[loc] = ops[1];
        P.jt[loc] = jv;
    }
}

// ================================================================== regalloc
// rv_generator.cpp:902-1258: every function has its own 64-entry register state
// (physical register -> the register number its value came from, -1 free) and lifetime
// mask; one step per instruction, all functions at step i before any symbol is updated:
// first the swap marks (the symbol a reused register held is marked swapped, keeping its
// register), then the symbols of rd, rs1 and rs2.  preserve_masks OR every step's
// lifetime mask.  A function reads and writes only its own symbols unless one of its
// instructions names another function's word (the cross check); then the functions run
// in the reference's order, one step for all of them at a time (s_ra_serial).
constexpr uint64_t kPreservedRegisterMask = 0x0FFC03000FFC031Full;  // rv_nodetype.hpp:108
constexpr uint64_t kNonscratchRegisters = 0x0FFC03000FFC0200ull;    // rv_nodetype.hpp:110

PTL_HD bool s_needs_float(uint32_t ins, uint32_t which) {
    if (ins == 0xC0007053u) return which != 0;  // FCVT.W.S: the source
    if (ins == 0xD0007053u) return which == 0;  // FCVT.S.W: the destination
    return (ins & 0x7Fu) == 0x53u;
}

// One step's effect on a function, computed before any symbol or register state of the
// step is written (the reference works from copies of both).
struct SRaStep {
    uint32_t act;              // 0: no instruction, 1: an instruction, 2: a call
    uint32_t rdv;              // rd as named
    unsigned long long mask;   // lifetime after the step
    unsigned long long swap;   // physical registers whose symbols become swapped
    uint32_t use_v[3];         // rd, rs1, rs2 as named (>= 64: a symbol)
    uint32_t use_reg[3];       // their registers after the step
};

// The reference keeps register numbers in int64 made from non-negative values: >= 64
// names a symbol (word r - 64).
PTL_HD bool s_sym_ok(const Prog& P, uint32_t r) { return r < 64u || r - 64u < P.W; }

// Where the symbols (register, swapped flag per word) live while the steps run: the
// program's arrays, or one byte per word of a run of functions (register in bits 0..5,
// swapped in bit 7) in shared memory -- a function only reads and writes its own words'
// symbols when it runs on its own.
struct SymGlobal {
    const Prog& P;
    PTL_HD uint32_t reg(uint32_t w) const { return P.symreg[w] & 0xFFu; }
    PTL_HD bool swapped(uint32_t w) const { return P.symswp[w] != 0; }
    PTL_HD void mark(uint32_t w) const { P.symswp[w] = 0xFFFFFFFFu; }
    PTL_HD void assign(uint32_t w, uint32_t r) const {
        P.symreg[w] = r;
        P.symswp[w] = 0;
    }
};
struct SymBytes {
    uint8_t* b;     // byte of word base + k at b[k], k < count
    uint32_t base, count;
    ErrorWord* err;
    // the cross check keeps every access inside the run; one outside is refused
    PTL_HD bool in(uint32_t w) const {
        if (w - base < count) return true;
        record_error(err, ST_UNSUPPORTED, W_RA1, w);
        return false;
    }
    PTL_HD uint32_t reg(uint32_t w) const { return in(w) ? (b[w - base] & 0x3Fu) : 0u; }
    PTL_HD bool swapped(uint32_t w) const { return in(w) && (b[w - base] & 0x80u) != 0; }
    PTL_HD void mark(uint32_t w) const { if (in(w)) b[w - base] = static_cast<uint8_t>(b[w - base] | 0x80u); }
    PTL_HD void assign(uint32_t w, uint32_t r) const { if (in(w)) b[w - base] = static_cast<uint8_t>(r & 0x3Fu); }
};

// The fields of word off a step reads.
struct SWord {
    uint32_t used, ins, r1, r2, rd, jt;
};
PTL_HD SWord s_word(const Prog& P, uint32_t off) {
    return SWord{P.used_instrs[off], P.instr[off], P.rs1[off], P.rs2[off], P.rd[off], P.jt[off]};
}

// lifetime_analyze_valid (:959-1145) for function f's word wd under lifetime mask; false
// for an input the reference leaves undefined (a symbol past the words).
template <class Sym>
PTL_HD bool s_ra_compute(const Prog& P, const Sym& sy, uint32_t f, const SWord& wd, uint64_t mask, SRaStep& R) {
    const uint32_t ins = wd.ins, r1 = wd.r1, r2 = wd.r2, rdv = wd.rd, j = wd.jt;
    const uint32_t start = P.fn_start0[f];
    if (ins == 0x000000EFu && (j < start || j - start >= P.fn_size0[f])) {
        // a call out of the function: caller-saved registers are freed, the ones in use
        // are marked swapped, no symbol is assigned
        R.act = 2;
        R.rdv = 0;
        R.mask = mask & kPreservedRegisterMask;
        R.swap = mask & ~kPreservedRegisterMask;
        return true;
    }
    if (!s_sym_ok(P, r1) || !s_sym_ok(P, r2) || !s_sym_ok(P, rdv)) return false;
    auto sym = [&](uint32_t r, uint32_t* reg, bool* sw) {
        if (r < 64u) {
            *reg = r;
            *sw = false;
        } else {
            *reg = sy.reg(r - 64u);
            *sw = sy.swapped(r - 64u);
        }
    };
    uint32_t rs1_reg, rs2_reg;
    bool sw1, sw2;
    sym(r1, &rs1_reg, &sw1);
    sym(r2, &rs2_reg, &sw2);
    if (sw1) rs1_reg = s_needs_float(ins, 1) ? 37u : 5u;
    if (sw2) rs2_reg = s_needs_float(ins, 2) ? 38u : 6u;
    auto clear = [](uint32_t r, uint64_t m) { return r == 0 ? m : (m & ~(1ull << r)); };
    const uint64_t cleared = clear(rs2_reg, clear(rs1_reg, mask));
    uint32_t rd_register = rdv;
    if (rdv >= 64u) {
        // the first free register of the class; the reference's ffs sees the low 32 bits
        const bool fl = s_needs_float(ins, 0);
        const uint32_t r = ffz_low32(cleared | (fl ? 0x00000000FFFFFFFFull : 0xFFFFFFFF00000000ull));
        rd_register = r == 64u ? (fl ? 37u : 5u) : r;
    }
    uint64_t swap = 0;
    if (rd_register != 0 && ((cleared >> rd_register) & 1ull)) swap |= 1ull << rd_register;
    if (rs1_reg != 0 && ((mask >> rs1_reg) & 1ull)) swap |= 1ull << rs1_reg;
    if (rs2_reg != 0 && ((mask >> rs2_reg) & 1ull)) swap |= 1ull << rs2_reg;
    R.act = 1;
    R.rdv = rdv;
    R.mask = cleared | (1ull << rd_register);
    R.swap = swap;
    R.use_v[0] = rdv;
    R.use_v[1] = r1;
    R.use_v[2] = r2;
    R.use_reg[0] = rd_register;
    R.use_reg[1] = rs1_reg;
    R.use_reg[2] = rs2_reg;
    return true;
}

// The swap marks: the symbols the swapped registers held before the step (regs, the
// function's register state, not yet updated) keep their register and read as swapped.
template <class Sym>
PTL_HD void s_ra_swaps(const Prog& P, const Sym& sy, const SRaStep& R, const int32_t* regs) {
    unsigned long long m = R.swap;
    while (m) {
        const uint32_t j = ctz64(m);
        m &= m - 1ull;
        const int32_t v = regs[j];
        if (v >= 64 && u32(v) - 64u < P.W) sy.mark(u32(v) - 64u);
    }
}

// The step's symbols take their registers (after every swap mark of the step).
template <class Sym>
PTL_HD void s_ra_uses(const Prog& P, const Sym& sy, const SRaStep& R) {
    if (R.act != 1) return;
    for (int k = 0; k < 3; ++k) {
        const uint32_t v = R.use_v[k];
        if (v >= 64u && v - 64u < P.W) {
            sy.assign(v - 64u, R.use_reg[k]);
        }
    }
}

// The function's register state after the step.  Registers are below 64 by
// construction (symbols only ever take registers the step computed); the checks keep
// the 64-entry state in bounds regardless.
PTL_HD void s_ra_regs(const SRaStep& R, int32_t* regs) {
    if (R.act == 1) {
        const uint32_t rd = R.use_reg[0];
        if (rd < 64u) regs[rd] = s32(R.rdv);
        if (R.use_reg[1] != rd && R.use_reg[1] < 64u) regs[R.use_reg[1]] = -1;
        if (R.use_reg[2] != rd && R.use_reg[2] < 64u) regs[R.use_reg[2]] = -1;
    } else if (R.act == 2) {
        for (uint32_t j = 0; j < 64; ++j)
            if (!((R.mask >> j) & 1ull)) regs[j] = -1;
    }
}

// The words a function's steps visit lie in the program (the reference reads past its
// buffers otherwise).
PTL_HD bool s_ra_function_ok(const Prog& P, uint32_t f) {
    return P.fn_start0[f] <= P.W && P.fn_size0[f] <= P.W - P.fn_start0[f];
}

// One function on its own (no word of another function named): its steps in order.
// regs: its 64-entry register state (caller's storage).  preserve[f] receives the OR of
// its lifetime masks, masked to the callee-saved registers.  The next step's word is
// loaded while the current one runs.
template <class Sym>
PTL_HD void s_ra_function(const Prog& P, const Sym& sy, uint32_t f, int32_t* regs, unsigned long long* preserve) {
    for (int k = 0; k < 64; ++k) regs[k] = -1;
    uint64_t mask = 0x1Full, pm = 0;
    if (!s_ra_function_ok(P, f)) {
        record_error(P.err, ST_UNSUPPORTED, W_RA1, f);
        return;
    }
    const uint32_t start = P.fn_start0[f], size = P.fn_size0[f];
    SWord cur = size > 0 ? s_word(P, start) : SWord{};
    for (uint32_t i = 0; i < size; ++i) {
        const uint32_t off = start + i;
        const SWord next = i + 1 < size ? s_word(P, off + 1) : SWord{};
        if (cur.used) {
            SRaStep R;
            if (!s_ra_compute(P, sy, f, cur, mask, R)) {
                record_error(P.err, ST_UNSUPPORTED, W_RA1, off);
                return;
            }
            s_ra_swaps(P, sy, R, regs);
            s_ra_uses(P, sy, R);
            s_ra_regs(R, regs);
            mask = R.mask;
        }
        pm |= mask;
        cur = next;
    }
    preserve[f] = pm & kNonscratchRegisters;
}

// Functions on their own in tiles of the word space: tile b takes the functions whose
// first word lies in [b * T, (b + 1) * T); their words run from the first one's start to
// the last one's end, at most T + S bytes (S: the longest function).  Threads of the
// tile run its functions with their symbols in sym (zeroed by the caller), then copy
// the bytes back to the program's arrays.  first/last: the tile's function range.
PTL_HD void s_ra_tile_functions(const Prog& P, uint32_t b, uint32_t T, uint32_t* first, uint32_t* last) {
    auto lower = [&](uint64_t w) {  // first function starting at or after word w
        uint32_t lo = 0, hi = P.F;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) / 2;
            if (P.fn_start0[mid] < w) lo = mid + 1; else hi = mid;
        }
        return lo;
    };
    *first = lower(static_cast<uint64_t>(b) * T);
    *last = lower(static_cast<uint64_t>(b + 1) * T);
}

// The tile's words [base, base + count) (clipped to the program).
PTL_HD uint32_t s_ra_tile_span(const Prog& P, uint32_t first, uint32_t last, uint32_t* base) {
    if (first >= last) {
        *base = 0;
        return 0;
    }
    *base = P.fn_start0[first];
    uint64_t end = static_cast<uint64_t>(P.fn_start0[last - 1]) + P.fn_size0[last - 1];
    if (end > P.W) end = P.W;
    return end > *base ? static_cast<uint32_t>(end - *base) : 0u;
}

PTL_HD void s_ra_tile_writeback(const Prog& P, const uint8_t* sym, uint32_t base, uint32_t count, uint32_t k) {
    if (k >= count || base + k >= P.W) return;
    const uint8_t v = sym[k];
    P.symreg[base + k] = v & 0x3Fu;
    P.symswp[base + k] = (v & 0x80u) ? 0xFFFFFFFFu : 0u;
}

// All functions in the reference's order (:1167-1269): per step, every function computes
// from the symbols as the previous step left them, then all swap marks, then the symbol
// updates in function order (a later function wins).  regs: F x 64 register states;
// steps: F step results (caller's storage); lifetime masks in P.lifetime.
PTL_HD void s_ra_serial(const Prog& P, int32_t* regs, SRaStep* steps, unsigned long long* preserve) {
    const uint32_t F = P.F;
    uint32_t S = 0;
    for (uint32_t f = 0; f < F; ++f) {
        for (int k = 0; k < 64; ++k) regs[f * 64u + k] = -1;
        P.lifetime[f] = 0x1Full;
        preserve[f] = 0;
        if (!s_ra_function_ok(P, f)) {
            record_error(P.err, ST_UNSUPPORTED, W_RA1, f);
            return;
        }
        S = P.fn_size0[f] > S ? P.fn_size0[f] : S;
    }
    for (uint32_t i = 0; i < S; ++i) {
        for (uint32_t f = 0; f < F; ++f) {
            steps[f].act = 0;
            const uint32_t off = P.fn_start0[f] + i;
            if (i < P.fn_size0[f] && P.used_instrs[off]) {
                if (!s_ra_compute(P, SymGlobal{P}, f, s_word(P, off), P.lifetime[f], steps[f])) {
                    record_error(P.err, ST_UNSUPPORTED, W_RA1, off);
                    return;
                }
            }
        }
        for (uint32_t f = 0; f < F; ++f)
            if (steps[f].act) s_ra_swaps(P, SymGlobal{P}, steps[f], regs + f * 64u);
        for (uint32_t f = 0; f < F; ++f) {
            if (steps[f].act) {
                s_ra_uses(P, SymGlobal{P}, steps[f]);
                s_ra_regs(steps[f], regs + f * 64u);
                P.lifetime[f] = steps[f].mask;
            }
            preserve[f] |= P.lifetime[f];
        }
    }
    for (uint32_t f = 0; f < F; ++f) preserve[f] &= kNonscratchRegisters;
}

// Extra words for the preserve stores and loads (:1309-1322): popcount(mask) at the
// function's sixth word and at its sixth word from the end, added to the counts of
// st_ra_count (function f, device: atomically).
PTL_HD void st_s_preserve_counts(const Prog& P, uint32_t f, const unsigned long long* preserve, uint32_t* counts) {
    const uint32_t pc = static_cast<uint32_t>(popcount64(preserve[f]));
    const int64_t a = static_cast<int64_t>(P.fn_start0[f]) + 5;
    const int64_t b = static_cast<int64_t>(P.fn_start0[f]) + static_cast<int64_t>(P.fn_size0[f]) - 6;
    if (a < 0 || b < 0 || a >= static_cast<int64_t>(P.W) || b >= static_cast<int64_t>(P.W)) {
        record_error(P.err, ST_UNSUPPORTED, W_RA_SCATTER, f);  // the reference adds past its counts
        return;
    }
    if (pc == 0) return;
    at_add_u32(&counts[a], pc);
    at_add_u32(&counts[b], pc);
}

// Words instruction i takes (:1296-1328): itself and a reload or spill per swapped
// symbol, plus the preserve words counted at it.
PTL_HD uint32_t st_s_ra_count(const Prog& P, uint32_t i, const uint32_t* extra) {
    const uint32_t e = extra[i];
    if (i >= P.W || !P.used_instrs[i]) return e;
    const uint32_t r1 = P.rs1[i], r2 = P.rs2[i], r = P.rd[i];
    if (!s_sym_ok(P, r1) || !s_sym_ok(P, r2) || !s_sym_ok(P, r)) {
        record_error(P.err, ST_UNSUPPORTED, W_RA_SCATTER, i);
        return 1u + e;
    }
    uint32_t c = 1u + e;
    if (r1 >= 64u && P.symswp[r1 - 64u]) ++c;
    if (r2 >= 64u && P.symswp[r2 - 64u]) ++c;
    if (r >= 64u && P.symswp[r - 64u]) ++c;
    return c;
}

// The instruction with allocated registers plus its reloads and spill, :1341-1497.  The
// stack offsets add the function's stack size, which the reference leaves 0.  Quirk kept:
// the rs2 reload and the main word test the rs1 reload's offset for > 0, so in the
// program's first word they land on the same slot.
PTL_HD void st_s_ra_scatter(const Prog& P, uint32_t i) {
    if (i >= P.W || !P.used_instrs[i]) return;
    const uint32_t r1 = P.rs1[i], r2 = P.rs2[i], r = P.rd[i], ins = P.instr[i];
    // the reference's offsets array holds W values in a zeroed allocation: a jump target
    // just past the words reads 0, one further on is undefined
    if (!s_sym_ok(P, r1) || !s_sym_ok(P, r2) || !s_sym_ok(P, r) || P.jt[i] >= P.W + 8u) {
        record_error(P.err, ST_UNSUPPORTED, W_RA_SCATTER, i);
        return;
    }
    const int64_t base = P.roffs[i];
    const bool sw1 = r1 >= 64u && P.symswp[r1 - 64u] != 0;
    const bool sw2 = r2 >= 64u && P.symswp[r2 - 64u] != 0;
    const bool swd = r >= 64u && P.symswp[r - 64u] != 0;
    const int64_t l1 = sw1 ? base : -1;
    const int64_t l2 = sw2 ? base + (l1 > 0 ? 1 : 0) : -1;
    const int64_t at_main = base + (l1 > 0 ? 1 : 0) + (l2 > 0 ? 1 : 0);
    const int64_t so = swd ? at_main + 1 : -1;
    const uint32_t ard = r >= 64u ? (P.symreg[r - 64u] & 0xFFu) : r;
    uint32_t ar1 = r1, ar2 = r2;
    if (r1 >= 64u) ar1 = sw1 ? (s_needs_float(ins, 1) ? 37u : 5u) : (P.symreg[r1 - 64u] & 0xFFu);
    if (r2 >= 64u) ar2 = sw2 ? (s_needs_float(ins, 2) ? 38u : 6u) : (P.symreg[r2 - 64u] & 0xFFu);
    const int64_t cap = P.W2;
    auto put = [&](int64_t at, uint32_t w, uint32_t d, uint32_t a, uint32_t b, uint32_t j) {
        if (at < 0 || at >= cap) return;
        P.ni[at] = w;
        P.nrd[at] = d;
        P.nr1[at] = a;
        P.nr2[at] = b;
        P.njt[at] = j;
    };
    auto load = [](uint32_t stack) { return 0x2003u | ((4u * (stack - 1u)) << 20); };  // lw
    if (sw1) put(l1, load(P.spill[r1 - 64u]), 5u, 0, 0, 0);
    if (sw2) put(l2, load(P.spill[r2 - 64u]), 6u, 0, 0, 0);
    put(at_main, ins, ard, ar1, ar2, P.jt[i] < P.W ? P.roffs[P.jt[i]] : 0u);
    if (swd) {  // sw of the result; the reference keeps imm bits 7:1 in the upper field
        const uint32_t imm = 0u - 4u * (P.spill[r - 64u] - 1u);
        put(so, 0x2023u | ((imm & 0x1Fu) << 7) | ((imm & 0xFEu) << 19), 0, ard, 0, 0);
    }
}

// Prologue and epilogue stack words, then the preserve stores, then the preserve loads,
// :1509-1602, on the table fix_func_tab moved.  The reference writes them in one scatter
// in that order (all functions' stack words, then all stores, then all loads), so later
// writes win where a function with few words and many preserved registers reaches into
// a neighbour's words.  On the GPU each word is claimed for the item latest in that order
// (s_frame_key), then the claiming items write.
PTL_HD uint32_t s_frame_stack_size(uint64_t pm) { return (static_cast<uint32_t>(popcount64(pm)) + 2u) * 4u; }

PTL_HD void s_frame_put(const Prog& P, int64_t at, uint32_t w) {
    if (at < 0 || at >= static_cast<int64_t>(P.W2)) return;
    P.ni[at] = w;
    P.nrd[at] = 0;
    P.nr1[at] = 0;
    P.nr2[at] = 0;
    P.njt[at] = 0;
}

// Word k of function f's pass: pass 0 the four stack words (lui/addi x8 after the entry
// and before the exit, stack size (preserved + 2) * 4 with the upper part sign-
// compensated), pass 1 the store and pass 2 the load of preserved register k.  False
// when the item has no word.
PTL_HD bool s_frame_item(const Prog& P, uint32_t f, uint64_t pm, uint32_t pass, uint32_t k, int64_t* at, uint32_t* w) {
    const int64_t start = P.fn_start[f], size = P.fn_size[f];
    if (pass == 0) {
        const uint32_t ss = s_frame_stack_size(pm);
        const uint32_t lower = (ss & 0xFFFu) << 20;
        const uint32_t upper = (ss - extend12(ss & 0xFFFu)) & 0xFFFFF000u;
        const int64_t where[4] = {start + 2, start + 3, start + size - 6, start + size - 5};
        *at = where[k];
        *w = (k & 1u) ? (0x00040413u | lower) : (0x00000437u | upper);
        return true;
    }
    if (!((pm >> k) & 1ull)) return false;
    const int64_t leading = popcount64(pm & ((1ull << k) - 1ull));
    const int64_t offset = -(8 + leading * 4);  // (stack size + overflow + 2) * 4: both 0 in the reference
    if (pass == 1) {
        const uint32_t hi = static_cast<uint32_t>((offset & 0xFE0) << 25);  // the reference's shift
        const uint32_t lo = static_cast<uint32_t>((offset & 0x1F) << 7);
        *w = (k >= 32 ? 0x00042027u : 0x00042023u) | hi | lo | ((k % 32u) << 20);  // fsw / sw
        *at = start + leading + 6;
    } else {
        *w = (k >= 32 ? 0x00042007u : 0x00042003u) | (static_cast<uint32_t>(offset) << 20) | ((k % 32u) << 7);
        *at = start + size + leading - 7;  // flw / lw
    }
    return true;
}

// Scatter order of the reference: pass, then function, then item.
PTL_HD unsigned long long s_frame_key(const Prog& P, uint32_t f, uint32_t pass, uint32_t k) {
    return (((static_cast<unsigned long long>(pass) * P.F + f) << 6) | k) + 1ull;
}

// mode 0: write (the caller runs passes and functions in the reference's order);
// 1: claim each word for the latest item (claim[] zeroed before); 2: write the words
// this function's items claimed.
PTL_HD void st_s_frame(const Prog& P, uint32_t f, uint32_t pass, const unsigned long long* preserve, int mode,
                       unsigned long long* claim) {
    const uint64_t pm = preserve[f];
    const uint32_t items = pass == 0 ? 4u : 64u;
    for (uint32_t k = 0; k < items; ++k) {
        int64_t at;
        uint32_t w;
        if (!s_frame_item(P, f, pm, pass, k, &at, &w)) continue;
        if (at < 0 || at >= static_cast<int64_t>(P.W2)) continue;
        const unsigned long long key = s_frame_key(P, f, pass, k);
        if (mode == 1) at_max_u64(&claim[at], key);
        else if (mode == 0 || claim[at] == key) s_frame_put(P, at, w);
    }
}

}  // namespace ptl
