// Register allocation step loops (rv_generator_avx.cpp:1018-1420) with on-chip symbol
// caches.  The phases below are shared by the CUDA kernels (one thread per function
// slot, barriers between phases) and the host model (the same phases in loops).
//
// Symbol state (physical register, swapped flag) lives in global memory, which always
// holds the truth; each function keeps a direct-mapped copy of recently used symbols
// in shared memory.  A symbol is written only by the function that owns it (its own
// instruction range) and by swap marks, and a mark can only hit a symbol that sits in
// row 0 of the register state -- row 0 also records which function wrote each entry,
// so a mark updates that function's cached copy together with global memory.
#pragma once

#include "ptl_stages.cuh"

namespace ptl {

// ---------------------------------------------------------------- symbol caches
struct SymCache {
    uint32_t* tag;   // [slots * K] virtual register held, 0 = empty
    uint32_t* val;   // physical register | swapped << 8 | (row-0 position + 1) << 16
    uint32_t K;      // entries per function (power of two)
};

PTL_HD void cache_reset(const SymCache& c, uint32_t slot) {
    for (uint32_t k = 0; k < c.K; ++k) c.tag[slot * c.K + k] = 0;
}

// Looks up v (> 63); returns physical register, swapped flag and (through defp, when
// given) the row-0 position + 1 of v's definition.
PTL_HD void sym_read(const Prog& P, const SymCache& c, uint32_t slot, uint32_t v, uint32_t* reg, bool* swp,
                     uint32_t* defp = nullptr) {
    const uint32_t e = slot * c.K + ((v - 64u) & (c.K - 1u));
    uint32_t x;
    if (c.tag[e] == v) {
        x = c.val[e];
    } else {
        x = (P.symreg[v - 64u] & 0xFFu) | (P.symswp[v - 64u] != 0 ? 0x100u : 0u) |
            (P.defpos ? static_cast<uint32_t>(P.defpos[v - 64u]) << 16 : 0u);
        c.tag[e] = v;
        c.val[e] = x;
    }
    *reg = x & 0xFFu;
    *swp = ((x >> 8) & 1u) != 0;
    if (defp) *defp = x >> 16;
}

// Owner update of v.  defp = row-0 position + 1 of a definition, 0 for a use (kept).
PTL_HD void sym_write(const Prog& P, const SymCache& c, uint32_t slot, uint32_t v, uint32_t reg, bool swp,
                      uint32_t defp = 0) {
    P.symreg[v - 64u] = reg;
    P.symswp[v - 64u] = swp ? 0xFFFFFFFFu : 0u;
    const uint32_t e = slot * c.K + ((v - 64u) & (c.K - 1u));
    uint32_t keep = 0;
    if (defp) {
        if (P.defpos) P.defpos[v - 64u] = static_cast<uint8_t>(defp);
        keep = defp << 16;
    } else if (c.tag[e] == v) {
        keep = c.val[e] & 0xFFFF0000u;
    } else if (P.defpos) {
        keep = static_cast<uint32_t>(P.defpos[v - 64u]) << 16;
    }
    c.tag[e] = v;
    c.val[e] = (reg & 0xFFu) | (swp ? 0x100u : 0u) | keep;
}

// A swap mark: global memory, plus the owner's cached copy if it holds v.
PTL_HD void sym_mark(const Prog& P, const SymCache& c, uint32_t owner_slot, uint32_t v) {
    P.symswp[v - 64u] = 0xFFFFFFFFu;
    if (owner_slot == 0xFFFFFFFFu) return;
    const uint32_t e = owner_slot * c.K + ((v - 64u) & (c.K - 1u));
    if (c.tag[e] == v) c.val[e] |= 0x100u;
}

// Whether r is a physical register or a virtual register of the instruction range
// [start, start+size) (ra_own with the range in registers).
PTL_HD bool ra_own_in(uint32_t start, uint32_t size, uint32_t r) {
    return !(s32(r) > 63) || r - 64u - start < size;
}

// ---------------------------------------------------------------- independent functions
// Steps per progress chunk: when the lane-0 pass runs beside the independent functions,
// each function counts the chunks whose trigger records it has finished.
constexpr uint32_t kRaChunk = 32;

// Functions outside lane 0: no marks reach their symbols, so the loop needs only the
// physical registers (kept in the cache) and emits trigger records for the lane-0 pass.
// done (device only, may be null): per-chunk count of functions whose records for that
// chunk are complete; the fence orders the records before the count.
PTL_HD void ra_free_function_cached(const Prog& P, const SymCache& c, uint32_t slot, uint32_t f,
                                    uint32_t* done = nullptr) {
    cache_reset(c, slot);
    unsigned long long lifetime = 0x1Full;
    const uint32_t g1 = f / 8u + 1u;
    const uint32_t start = P.fn_start0[f], size = P.fn_size0[f];
    // Each thread walks its own function, so a warp's loads of one step touch 32 lines:
    // the instruction of step i+2 is loaded during step i, two steps of work ahead of
    // its use, which covers the latency of a read that misses the L1.
    RaStep next, next2;
    bool have = ra_load_at(P, start, size, 0, next);
    bool have2 = ra_load_at(P, start, size, 1, next2);
    for (uint32_t i = 0; have; ++i) {
        RaStep S = next;
        next = next2;
        have = have2;
        have2 = ra_load_at(P, start, size, i + 2, next2);
        if (S.ins == 0x000000EFu || !ra_own_in(start, size, S.r1) || !ra_own_in(start, size, S.r2) ||
            !ra_own_in(start, size, S.ord)) {
            record_error(P.err, ST_UNSUPPORTED, W_RA1, start + i);
            return;
        }
        uint32_t r1reg = 0, r2reg = 0;
        bool s1 = false, s2 = false;
        if (s32(S.r1) > 63) sym_read(P, c, slot, S.r1, &r1reg, &s1);
        if (s32(S.r2) > 63) sym_read(P, c, slot, S.r2, &r2reg, &s2);
        ra_compute(S, lifetime, r1reg, false, r2reg, false);
        lifetime = S.cleared | S.rdm;
        if (s32(S.ord) > 63) sym_write(P, c, slot, S.ord, S.rdr, false);
        if (s32(S.r1) > 63) sym_write(P, c, slot, S.r1, S.r1r, false);
        if (s32(S.r2) > 63) sym_write(P, c, slot, S.r2, S.r2r, false);
        for (uint64_t t = S.trig; t; t &= t - 1) {
            const uint32_t p = ctz64(t);
            at_min_u32(&P.trig_min[static_cast<size_t>(i) * 64u + p], g1);
            at_max_u32(&P.trig_max[static_cast<size_t>(i) * 64u + p], g1);
        }
#if defined(__CUDA_ARCH__)
        if (done && (!have || (i + 1u) % kRaChunk == 0)) {
            __threadfence();
            atomicAdd(&done[i / kRaChunk], 1u);
        }
#endif
    }
}

// ---------------------------------------------------------------- lane-0 lock-step
// Shared (on-chip) state of the lane-0 pass.  Groups are stored as group+1 ("g1"); 0 and
// 0xFFFFFFFF mean none for the max / min arrays.
constexpr uint32_t kSnapHash = 128;  // open-addressing table: virtual register -> row-0 positions

struct Ra2Shared {
    uint32_t hkey[2][kSnapHash];            // double-buffered by step parity; 0 = empty
    unsigned long long hmask[2][kSnapHash];
    uint32_t R0[64];       // row 0 of the register state
    uint32_t R0own[64];    // slot of the function that wrote the entry
    uint32_t snap[64];     // row 0 at the start of the step
    uint32_t snapown[64];
    uint32_t omin[64], omax[64];   // trigger groups of the other functions this step
    uint32_t lcur[64], lmax[64];   // lane-0 triggers of the current round
    uint32_t lnew[64], lmaxnew[64];
    uint32_t r0grp[64];    // highest group (+1) writing each position this step
};

// Per function slot (registers on the device).
struct Ra2Slot {
    uint32_t j;            // group index (function 8j)
    uint32_t start, size;  // the function's isn_cnt instruction range
    bool act;
    unsigned long long lifetime, lt_new;  // live mask before the step; after it (set by ra2_apply)
    RaStep S, next;
    bool have_next;
    uint32_t r1reg, r2reg;
    bool r1stored, r2stored;   // swapped flag as stored before the step
    bool r1m, r2m;             // marked by an earlier group this step (as used)
    uint64_t m1, m2;           // row-0 positions holding r1 / r2
};

PTL_HD uint32_t snap_hash(uint32_t v) { return (v * 2654435761u) >> 25; }

// Row-0 positions holding v at the start of step i (v > 63), from the hash of row 0.
PTL_HD uint64_t snap_positions_hashed(const Ra2Shared& sh, uint32_t i, uint32_t v) {
    const uint32_t t = i & 1u;
    uint32_t h = snap_hash(v);
    for (uint32_t probe = 0; probe < kSnapHash; ++probe) {
        const uint32_t k = sh.hkey[t][h];
        if (k == v) return sh.hmask[t][h];
        if (k == 0) return 0;
        h = (h + 1u) & (kSnapHash - 1u);
    }
    return 0;
}

PTL_HD void snap_insert(Ra2Shared& sh, uint32_t i, uint32_t v, uint32_t p) {
    const uint32_t t = i & 1u;
    uint32_t h = snap_hash(v);
    for (uint32_t probe = 0; probe < kSnapHash; ++probe) {
#if defined(__CUDA_ARCH__)
        const uint32_t prev = atomicCAS(&sh.hkey[t][h], 0u, v);
#else
        const uint32_t prev = sh.hkey[t][h];
        if (prev == 0) sh.hkey[t][h] = v;
#endif
        if (prev == 0 || prev == v) {
#if defined(__CUDA_ARCH__)
            atomicOr(&sh.hmask[t][h], 1ull << p);
#else
            sh.hmask[t][h] |= 1ull << p;
#endif
            return;
        }
        h = (h + 1u) & (kSnapHash - 1u);
    }
}

// Empties the table step i+1 will use (called during step i, before its last barrier).
PTL_HD void snap_clear_next(Ra2Shared& sh, uint32_t i, uint32_t p) {
    const uint32_t t = (i + 1u) & 1u;
    for (uint32_t k = p; k < kSnapHash; k += 64u) {
        sh.hkey[t][k] = 0;
        sh.hmask[t][k] = 0;
    }
}

// Row-0 positions holding v: a lane-0 value enters row 0 only where its definition put
// it, so one compare answers the question -- unless two instructions define the same
// virtual register, for which the row-0 hash is built instead (P.defpos == null).
PTL_HD uint64_t snap_positions(const Prog& P, const Ra2Shared& sh, uint32_t i, uint32_t v, uint32_t d) {
    if (!P.defpos) return snap_positions_hashed(sh, i, v);
    if (d == 0) return 0;
    return sh.snap[d - 1u] == v ? (1ull << (d - 1u)) : 0ull;
}

// Whether a symbol at row-0 positions m is marked by a group before j (g1 <= j).
PTL_HD bool marked_before(const Ra2Shared& sh, uint64_t m, uint32_t j, bool with_lane0) {
    for (; m; m &= m - 1) {
        const uint32_t p = ctz64(m);
        uint32_t g = sh.omin[p];
        if (with_lane0 && sh.lcur[p] < g) g = sh.lcur[p];
        if (g <= j) return true;
    }
    return false;
}

PTL_HD void ra2_slot_init(const Prog& P, const SymCache& c, Ra2Slot& L, uint32_t slot, uint32_t j) {
    L.j = j;
    L.lifetime = L.lt_new = 0x1Full;
    L.start = 8u * j < P.F ? P.fn_start0[8u * j] : 0u;
    L.size = 8u * j < P.F ? P.fn_size0[8u * j] : 0u;
    L.have_next = 8u * j < P.F && ra_load_at(P, L.start, L.size, 0, L.next);
    cache_reset(c, slot);
}

// Step start for row-0 position p (64 threads); tmin/tmax are the step's trigger
// records of the other functions (loaded a step ahead).
PTL_HD void ra2_begin_p(Ra2Shared& sh, uint32_t i, uint32_t p, uint32_t tmin, uint32_t tmax, bool hashed) {
    sh.snap[p] = sh.R0[p];
    sh.snapown[p] = sh.R0own[p];
    if (hashed && s32(sh.R0[p] - 64u) >= 0) snap_insert(sh, i, sh.R0[p], p);
    sh.omin[p] = tmin;
    sh.omax[p] = tmax;
    sh.lcur[p] = 0xFFFFFFFFu;
    sh.lmax[p] = 0;
    sh.lnew[p] = 0xFFFFFFFFu;
    sh.lmaxnew[p] = 0;
    sh.r0grp[p] = 0;
}

// Loads the slot's instruction of step i (prefetched in the previous step).  cur[0..2]:
// what the slot updates this step (for the mark phase); cur[3] is set by ra2_apply.
PTL_HD void ra2_load(const Prog& P, Ra2Slot& L, uint32_t i, uint32_t* cur) {
    L.lifetime = L.lt_new;
    L.act = L.have_next;
    if (L.act) {
        L.S = L.next;
        L.have_next = ra_load_at(P, L.start, L.size, i + 1, L.next);
        if (L.S.ins == 0x000000EFu || !ra_own_in(L.start, L.size, L.S.r1) || !ra_own_in(L.start, L.size, L.S.r2) ||
            !ra_own_in(L.start, L.size, L.S.ord)) {
            record_error(P.err, ST_UNSUPPORTED, W_RA2, P.fn_start0[8u * L.j] + i);
            L.act = false;
            L.have_next = false;
        }
    }
    cur[0] = L.act ? L.S.ord : 0u;
    cur[1] = L.act ? L.S.r1 : 0u;
    cur[2] = L.act ? L.S.r2 : 0u;
}

PTL_HD void ra2_add_triggers(Ra2Shared& sh, uint64_t trig, uint32_t g1, bool into_new) {
    for (uint64_t t = trig; t; t &= t - 1) {
        const uint32_t p = ctz64(t);
        if (into_new) {
            at_min_u32(&sh.lnew[p], g1);
            at_max_u32(&sh.lmaxnew[p], g1);
        } else {
            at_min_u32(&sh.lcur[p], g1);
            at_max_u32(&sh.lmax[p], g1);
        }
    }
}

// Round 0: lookups through the cache, marks of earlier groups among the other functions
// only, the allocation, and this slot's triggers into lcur/lmax.
// Returns whether the slot read a symbol that sits in row 0 (then the check phase runs).
PTL_HD bool ra2_compute0(const Prog& P, const SymCache& c, Ra2Shared& sh, Ra2Slot& L, uint32_t slot, uint32_t i) {
    if (!L.act) return false;
    RaStep& S = L.S;
    L.r1reg = L.r2reg = 0;
    L.r1stored = L.r2stored = false;
    L.m1 = L.m2 = 0;
    if (s32(S.r1) > 63) {
        uint32_t d;
        sym_read(P, c, slot, S.r1, &L.r1reg, &L.r1stored, &d);
        L.m1 = snap_positions(P, sh, i, S.r1, d);
    }
    if (s32(S.r2) > 63) {
        uint32_t d;
        sym_read(P, c, slot, S.r2, &L.r2reg, &L.r2stored, &d);
        L.m2 = snap_positions(P, sh, i, S.r2, d);
    }
    L.r1m = marked_before(sh, L.m1, L.j, false);
    L.r2m = marked_before(sh, L.m2, L.j, false);
    ra_compute(S, L.lifetime, L.r1reg, L.r1stored || L.r1m, L.r2reg, L.r2stored || L.r2m);
    ra2_add_triggers(sh, S.trig, L.j + 1u, false);
    return (L.m1 | L.m2) != 0;
}

// After round 0: does an earlier lane-0 trigger change what this slot read?
PTL_HD bool ra2_check(const Ra2Shared& sh, const Ra2Slot& L) {
    if (!L.act || (L.m1 | L.m2) == 0) return false;
    return marked_before(sh, L.m1, L.j, true) != L.r1m || marked_before(sh, L.m2, L.j, true) != L.r2m;
}

// Jacobi round (only when the check fired): recompute with the current lane-0 triggers
// and accumulate the next round's triggers.
PTL_HD void ra2_round(Ra2Shared& sh, Ra2Slot& L) {
    if (!L.act) return;
    if (L.m1 | L.m2) {
        L.r1m = marked_before(sh, L.m1, L.j, true);
        L.r2m = marked_before(sh, L.m2, L.j, true);
        ra_compute(L.S, L.lifetime, L.r1reg, L.r1stored || L.r1m, L.r2reg, L.r2stored || L.r2m);
    }
    ra2_add_triggers(sh, L.S.trig, L.j + 1u, true);
}

// Row-0 thread p after a Jacobi round: adopt the new triggers; report change.
PTL_HD bool ra2_round_p(Ra2Shared& sh, uint32_t p) {
    const bool changed = sh.lnew[p] != sh.lcur[p];
    sh.lcur[p] = sh.lnew[p];
    sh.lmax[p] = sh.lmaxnew[p];
    sh.lnew[p] = 0xFFFFFFFFu;
    sh.lmaxnew[p] = 0;
    return changed;
}

// Apply the step: lifetime, own symbol updates (swapped only when a later group marks
// the symbol in this step), row-0 writes as the highest writing group per position.
// Applying again after Jacobi rounds rewrites the same symbols and records (row-0
// group maxima are reset in between), so a step may be applied speculatively.
// The winner's value follows from its record: its defined register at its rd position
// (cur[3]), a cleared entry (0xFFFFFFFF) at its rs1/rs2 positions.
PTL_HD void ra2_apply(const Prog& P, const SymCache& c, Ra2Shared& sh, Ra2Slot& L, uint32_t slot, uint32_t i,
                      uint32_t* cur) {
    if (!L.act) return;
    const RaStep& S = L.S;
    L.lt_new = S.cleared | S.rdm;
    const uint32_t g1 = L.j + 1u;
    auto later = [&](uint64_t m) {
        for (; m; m &= m - 1) {
            const uint32_t p = ctz64(m);
            const uint32_t g = sh.omax[p] > sh.lmax[p] ? sh.omax[p] : sh.lmax[p];
            if (g > g1) return true;
        }
        return false;
    };
    // The swap flags need the row-0 positions at the step start: m1/m2 from the round-0
    // lookups.  The defined register sits in row 0 before its definition only when it
    // has two definitions, i.e. in hashed mode.
    const bool l_ord = !P.defpos && s32(S.ord) > 63 && later(snap_positions_hashed(sh, i, S.ord));
    const bool l_r1 = s32(S.r1) > 63 && later(L.m1);
    const bool l_r2 = s32(S.r2) > 63 && later(L.m2);
    // the reference's order: rd, rs1, rs2 (a later write of the same symbol wins); a
    // definition records the row-0 position it writes (when it writes row 0 at all)
    if (s32(S.ord) > 63) sym_write(P, c, slot, S.ord, S.rdr, false, (S.rdr & 63u) + 1u);
    if (s32(S.r1) > 63) sym_write(P, c, slot, S.r1, S.r1r, false);
    if (s32(S.r2) > 63) sym_write(P, c, slot, S.r2, S.r2r, false);
    // a swapped symbol keeps the register just written for it (the last of the three
    // writes above that names it): the values are known here, no global read needed
    const bool r2v = s32(S.r2) > 63, r1v = s32(S.r1) > 63;
    if (l_ord) sym_write(P, c, slot, S.ord, (r2v && S.r2 == S.ord) ? S.r2r : ((r1v && S.r1 == S.ord) ? S.r1r : S.rdr), true);
    if (l_r1) sym_write(P, c, slot, S.r1, (r2v && S.r2 == S.r1) ? S.r2r : S.r1r, true);
    if (l_r2) sym_write(P, c, slot, S.r2, S.r2r, true);
    // rdr < 64 always, and a clear never lands on the rd position, so each group writes
    // one value per position
    cur[3] = S.rdr & 63u;
    if (S.ord != 0) at_max_u32(&sh.r0grp[S.rdr & 63u], g1);
    if (S.r1r != S.rdr && s32(S.r1r) >= 0 && S.r1r < 64u) at_max_u32(&sh.r0grp[S.r1r], g1);
    if (S.r2r != S.rdr && s32(S.r2r) >= 0 && S.r2r < 64u) at_max_u32(&sh.r0grp[S.r2r], g1);
}

// The slots' step records (cur[0..3] of ra2_load / ra2_apply) and symbol caches, seen
// by slot index (== group index) from the row-0 phases.  One block holds them all; a
// thread-block cluster spreads them over its CTAs (k_ra_lane0_cluster has its own view).
struct BlockSlots {
    const uint32_t* cur;
    SymCache c;
    PTL_HD const uint32_t* rec(uint32_t slot) const { return cur + 4u * slot; }
    PTL_HD void mark(const Prog& P, uint32_t owner, uint32_t v) const { sym_mark(P, c, owner, v); }
};

// Step end for row-0 position p: marks on symbols their owner did not update this step,
// then row 0 takes the highest group's write.
template <class Slots>
PTL_HD void ra2_end_p_at(const Prog& P, const Slots& sl, Ra2Shared& sh, uint32_t p) {
    const bool triggered = sh.omin[p] != 0xFFFFFFFFu || sh.lcur[p] != 0xFFFFFFFFu;
    const uint32_t v = sh.snap[p];
    if (triggered && s32(v - 64u) >= 0) {
        const uint32_t own = sh.snapown[p];
        bool updated = false;
        if (own != 0xFFFFFFFFu) {
            const uint32_t* u = sl.rec(own);
            updated = (s32(u[0]) > 63 && u[0] == v) || (s32(u[1]) > 63 && u[1] == v) || (s32(u[2]) > 63 && u[2] == v);
        }
        if (!updated) sl.mark(P, own, v);
    }
    const uint32_t g = sh.r0grp[p];
    if (g != 0) {
        const uint32_t* w = sl.rec(g - 1u);
        sh.R0[p] = (w[0] != 0 && w[3] == p) ? w[0] : 0xFFFFFFFFu;
        sh.R0own[p] = g - 1u;
    }
}
// cur[4*slot..] are the slots' records (slot index == group index).
PTL_HD void ra2_end_p(const Prog& P, const SymCache& c, Ra2Shared& sh, uint32_t p, const uint32_t* cur) {
    ra2_end_p_at(P, BlockSlots{cur, c}, sh, p);
}

// ---------------------------------------------------------------- the tail of the pass
// Steps that change row 0: every lane-0 function has run its last step by s0 (the
// longest lane-0 function).  From s0 on no slot is active, so no slot writes row 0 or
// updates a symbol, and a step only marks the symbol row 0 holds at each position that
// another function triggers.  Row 0 no longer changes and a mark only sets a flag, so the
// steps s0..S-1 come down to one check per position (ra2_tail_p).
PTL_HD uint32_t ra2_lane0_size(const Ra2Slot& L) { return s32(L.size) > 0 ? L.size : 0u; }

PTL_HD uint32_t ld_records(const uint32_t* p) {
#if defined(__CUDA_ARCH__)
    return __ldcg(p);  // written by other blocks
#else
    return *p;
#endif
}

// Position p after step s0-1: whether its symbol is marked in a step of [s0, S), i.e.
// another function has a trigger record there.
PTL_HD bool ra2_tail_hit(const Prog& P, const Ra2Shared& sh, uint32_t p, uint32_t s0, uint32_t S) {
    const uint32_t v = sh.R0[p];
    if (s32(v - 64u) < 0) return false;
    bool hit = false;
    for (uint32_t i = s0; i < S && !hit; i += 8) {
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k)
            if (i + k < S) hit |= ld_records(&P.trig_min[static_cast<size_t>(i + k) * 64u + p]) != 0xFFFFFFFFu;
    }
    return hit;
}
PTL_HD void ra2_tail_p(const Prog& P, const SymCache& c, const Ra2Shared& sh, uint32_t p, uint32_t s0, uint32_t S) {
    if (ra2_tail_hit(P, sh, p, s0, S)) sym_mark(P, c, sh.R0own[p], sh.R0[p]);
}

}  // namespace ptl
