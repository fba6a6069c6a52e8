// ORACLE -- test infrastructure, not product code (see ptl_port.h).
//
// Scalar restatement of the reference AVX2 code generator,
// src/codegen/rv_generator_avx.cpp, with one worker thread.  Every "parallel" loop of
// the reference (run_basic, rv_generator_avx.hpp:118-147) then visits its 8-lane
// blocks in ascending order, so each loop below walks blocks in order and keeps the
// reference's block-level snapshots: values loaded at the top of a block body are
// not refreshed by stores the same body makes.
//
// Buffers mirror avx_buffer (include/codegen/avx_buffer.hpp:42-58): 64 zero bytes
// before element 0 and a zeroed tail rounded up to 64 bytes plus 64 more, because
// the reference reads element -1, reads past the end and stores into the tail.
#include "ptl_port.h"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "port_tables.inc"

namespace {

using port::Tables;

const Tables& tables() {
    static const Tables t = port::make_tables();
    return t;
}

template <typename T>
class PBuf {
public:
    PBuf() = default;
    explicit PBuf(size_t n) { resize(n); }
    void resize(size_t n) {
        n_ = n;
        size_t bytes = ((sizeof(T) * n + 63) & ~size_t(63)) + 128;
        store_.assign(bytes / sizeof(T) + 1, T{});
        p_ = store_.data() + 64 / sizeof(T);
        cap_ = bytes / sizeof(T) - 64 / sizeof(T);
    }
    size_t size() const { return n_; }
    T& operator[](int64_t i) { return at(i); }
    const T& operator[](int64_t i) const { return const_cast<PBuf*>(this)->at(i); }
    T* data() { return p_; }
    const T* data() const { return p_; }
    T& back() { return p_[n_ - 1]; }
    // Copy with the semantics of avx_buffer's copy constructor: the logical elements
    // only, into a fresh zeroed allocation.
    PBuf clone() const {
        PBuf o(n_);
        for (size_t i = 0; i < n_; ++i) o.p_[i] = p_[i];
        return o;
    }
    bool equal(const PBuf& o) const {
        if (n_ != o.n_) return false;
        for (size_t i = 0; i < n_; ++i) if (p_[i] != o.p_[i]) return false;
        return true;
    }

private:
    T& at(int64_t i) {
        int64_t lo = -static_cast<int64_t>(64 / sizeof(T));
        if (i < lo || i >= static_cast<int64_t>(cap_)) {
            throw std::out_of_range("oracle: access outside the reference's allocation");
        }
        return p_[i];
    }
    std::vector<T> store_;
    T* p_ = nullptr;
    size_t n_ = 0;
    size_t cap_ = 0;
};

// Number of 8 x u32 blocks of a u32 buffer of n elements (avx_buffer::size_m256i).
inline size_t blocks32(size_t n) { return (n * 4 + 31) / 32; }

inline int32_t s32(uint32_t v) { return static_cast<int32_t>(v); }

struct Unsupported : std::runtime_error {
    using std::runtime_error::runtime_error;
};

struct Gen {
    size_t n = 0;
    size_t max_depth = 0;
    PBuf<uint32_t> node_types, result_types, node_data, node_sizes, node_locations;
    PBuf<int32_t> parents, depth, child_idx;
    PBuf<uint32_t> func_starts, func_ends, function_sizes, function_ids;
    PBuf<uint32_t> instr, rd, rs1, rs2, jt, used_instrs;

    const Tables& T = tables();

    // ---------------------------------------------------------------- preprocess
    // rv_generator_avx.cpp:122-308
    void preprocess() {
        const size_t nb = blocks32(n);
        // Pass 1, function arguments: :126-213
        for (size_t b = 0; b < nb; ++b) {
            bool any_arg = false;
            for (int l = 0; l < 8; ++l) any_arg |= (node_types[8 * b + l] & 0xF0u) == 0xF0u;
            if (!any_arg) continue;
            for (int l = 0; l < 8; ++l) {
                const size_t i = 8 * b + l;
                uint32_t t = node_types[i];
                const bool is_arg = (t & 0xF0u) == 0xF0u;
                const uint32_t rt = result_types[i];
                const bool is_float = is_arg && (rt == port::D_FLOAT || rt == port::D_FLOAT_REF);
                const bool is_int = is_arg && !is_float;
                uint32_t nd = node_data[i];
                const uint32_t ci = static_cast<uint32_t>(child_idx[i]);
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
                    // The reference ANDs the comparison mask with the data value itself.
                    const uint32_t on_stack = (s32(reg_offset) > 7 ? 0xFFFFFFFFu : 0u) & int_data;
                    t |= on_stack & 0b10u;
                    reg_offset -= 8u & on_stack;
                    if (is_int) nd = reg_offset;
                }
                node_types[i] = t;
                node_data[i] = nd;
            }
        }
        // Pass 2, call argument lists: :217-266
        for (size_t b = 0; b < nb; ++b) {
            bool any_list = false;
            for (int l = 0; l < 8; ++l) any_list |= node_types[8 * b + l] == port::T_FUNC_CALL_ARG_LIST;
            if (!any_list) continue;
            uint32_t prev_t[8], prev_nd[8], prev_rt[8];
            int32_t prev_ci[8];
            for (int l = 0; l < 8; ++l) {
                const int64_t p = static_cast<int64_t>(8 * b + l) - 1;
                prev_t[l] = node_types[p];
                prev_nd[l] = node_data[p];
                prev_rt[l] = result_types[p];
                prev_ci[l] = child_idx[p];
            }
            // Stores are masked by the predecessor's type only (not by "is a list").
            for (int l = 0; l < 8; ++l) {
                if (prev_t[l] == port::T_FUNC_CALL_ARG_ON_STACK) node_data[8 * b + l] = prev_nd[l] + 1u;
            }
            for (int l = 0; l < 8; ++l) {
                if (prev_t[l] == port::T_FUNC_CALL_ARG && prev_rt[l] == port::D_FLOAT) {
                    int32_t v = s32(static_cast<uint32_t>(prev_ci[l]) - prev_nd[l] - 8u);
                    node_data[8 * b + l] = static_cast<uint32_t>(std::max(v, 0));
                }
            }
        }
        // Pass 3, float comparisons: :270-305.  Result types of the block are read once.
        for (size_t b = 0; b < nb; ++b) {
            bool store[8];
            int32_t par[8];
            for (int l = 0; l < 8; ++l) {
                const size_t i = 8 * b + l;
                par[l] = parents[i];
                const int32_t gi = par[l] > -1 ? par[l] : 0;
                const uint32_t pt = node_types[gi];
                const bool peq = (pt & port::T_EQ) == port::T_EQ;
                const uint32_t rt = result_types[i] & (peq ? 0xFFFFFFFFu : 0u);
                store[l] = rt == port::D_FLOAT;
            }
            for (int l = 0; l < 8; ++l) {
                if (store[l]) result_types[par[l]] = port::D_FLOAT;
            }
        }
    }

    // ---------------------------------------------------------------- isn_cnt
    // rv_generator_avx.cpp:310-518
    void isn_cnt() {
        const size_t nb = blocks32(n);
        for (size_t b = 0; b < nb; ++b) {  // :315-369
            for (int l = 0; l < 8; ++l) {
                const size_t i = 8 * b + l;
                const uint32_t t = node_types[i];
                const uint32_t rt = result_types[i];
                uint32_t base = size_flat(t * 6u + rt);
                uint32_t delta = 0;
                if (t == port::T_FUNC_CALL_ARG_LIST) {
                    delta += 1;
                    const uint32_t pt = node_types[static_cast<int64_t>(i) - 1];
                    if ((pt & port::T_FUNC_CALL_ARG) == port::T_FUNC_CALL_ARG) {
                        delta += static_cast<uint32_t>(child_idx[static_cast<int64_t>(i) - 1]) + 1u;
                    }
                }
                const int32_t p = parents[i];
                const uint32_t ptype = node_types[p != -1 ? p : 0];
                const int32_t ci = child_idx[i];
                const bool if_else = ptype == port::T_IF_ELSE;
                if (ci == 0 && (if_else || ptype == port::T_IF)) delta += 1;
                if (ci == 1 && (if_else || ptype == port::T_WHILE)) delta += 1;
                node_sizes[i] = base + delta;
            }
        }
        // Exclusive scan, :374-392 (shifted load of element -1).
        {
            uint32_t acc = 0;
            for (size_t i = 0; i < 8 * nb; ++i) {
                acc += node_sizes[static_cast<int64_t>(i) - 1];
                node_locations[i] = acc;
            }
        }
        // Fix conditions and call arguments, :398-447.
        for (size_t b = 0; b < nb; ++b) {
            int32_t par[8], ci[8];
            bool cond[8];
            bool any_cond = false;
            for (int l = 0; l < 8; ++l) {
                const size_t i = 8 * b + l;
                par[l] = parents[i];
                ci[l] = child_idx[i];
                const uint32_t pt = node_types[par[l] > -1 ? par[l] : 0];
                cond[l] = ((pt & port::T_IF) == port::T_IF) && (ci[l] == s32(pt & 1u));
                any_cond |= cond[l];
            }
            if (any_cond) {
                uint32_t vals[8];
                for (int l = 0; l < 8; ++l) {
                    const size_t i = 8 * b + l;
                    vals[l] = node_locations[i] + (cond[l] ? size_flat(node_types[i] * 6u + result_types[i]) : 0u);
                }
                for (int l = 0; l < 8; ++l) {
                    if (cond[l]) node_locations[par[l]] = vals[l];
                }
            }
            bool fca[8];
            bool any_fca = false;
            for (int l = 0; l < 8; ++l) {
                fca[l] = (node_types[8 * b + l] & port::T_FUNC_CALL_ARG) == port::T_FUNC_CALL_ARG;
                any_fca |= fca[l];
            }
            if (any_fca) {
                uint32_t nl[8];
                for (int l = 0; l < 8; ++l) {
                    nl[l] = fca[l] ? node_locations[par[l]] + static_cast<uint32_t>(ci[l]) + 1u : 0u;
                }
                for (int l = 0; l < 8; ++l) {
                    if (fca[l]) node_locations[8 * b + l] = nl[l];
                }
            }
        }
        // Function table, :451-517.
        std::vector<uint32_t> decls;
        for (size_t i = 0; i < 8 * nb; ++i) {
            if (node_types[i] == port::T_FUNC_DECL) decls.push_back(static_cast<uint32_t>(i));
        }
        const size_t F = decls.size();
        if (F == 0) throw Unsupported("program has no function (the reference takes the max of an empty range)");
        PBuf<uint32_t> func_decls(F);
        for (size_t f = 0; f < F; ++f) func_decls[f] = decls[f];
        function_ids.resize(F);
        func_starts.resize(F);
        PBuf<uint32_t> func_offsets(F);
        const size_t fb = blocks32(F);
        for (size_t b = 0; b < fb; ++b) {
            for (int l = 0; l < 8; ++l) {
                const size_t f = 8 * b + l;
                const uint32_t d = func_decls[f];
                function_ids[f] = node_data[d];
                const uint32_t off = 6u + node_locations[d];
                func_starts[f + 1] = off;
                func_offsets[f] = off;
            }
        }
        function_sizes.resize(F);
        for (size_t f = 0; f < 8 * fb; ++f) {
            function_sizes[f] = func_offsets[f] - func_offsets[static_cast<int64_t>(f) - 1];
        }
        func_ends.resize(F);
        for (size_t f = 0; f < 8 * fb; ++f) func_ends[f] = func_starts[f] + function_sizes[f];
    }

    uint32_t size_flat(uint32_t idx) const { return (&T.size[0][0])[idx]; }

    // ---------------------------------------------------------------- isn_gen
    // rv_generator_avx.cpp:520-889
    void isn_gen() {
        std::vector<uint32_t> idx_array(n);
        std::iota(idx_array.begin(), idx_array.end(), 0u);
        // :539-541, the one-thread branch of the reference
        std::sort(idx_array.begin(), idx_array.end(),
                  [this](uint32_t a, uint32_t b) { return depth[a] < depth[b]; });
        std::vector<uint32_t> depth_starts;
        for (size_t i = 0; i < n; ++i) {
            if (i == 0 || depth[idx_array[i]] != depth[idx_array[i - 1]]) depth_starts.push_back(static_cast<uint32_t>(i));
        }
        if (depth_starts.size() != max_depth + 1) {
            throw Unsupported("depths 0..max_depth are not all populated");
        }
        const uint32_t word_count = node_locations.back();
        PBuf<uint32_t> registers(n * 3);
        instr.resize(word_count);
        rd.resize(word_count);
        rs1.resize(word_count);
        rs2.resize(word_count);
        jt.resize(word_count);

        const uint32_t* has_instr = &T.has_instr[0][0][0];
        const uint32_t* has_output = &T.has_output[0][0][0];
        const uint32_t* pai_tab = &T.pai[0][0][0];
        const uint32_t* out_tab = &T.out[0][0][0];
        const uint32_t* instr_tab = &T.instr[0][0][0];
        const uint32_t* const_tab = &T.cnst[0][0];
        const uint32_t* operand_tab = &T.operand[0][0][0][0];
        const uint32_t* jt_tab = &T.jt[0][0];

        for (size_t lvl = 0; lvl < max_depth + 1; ++lvl) {
            const uint32_t cur = static_cast<uint32_t>(max_depth - lvl);
            const uint32_t start = depth_starts[cur];
            const uint32_t end = (cur == max_depth) ? static_cast<uint32_t>(n) : depth_starts[cur + 1];
            const uint32_t level_size = end - start;
            const uint32_t steps = (level_size + 1) / 2;
            const bool uneven = level_size & 1u;
            for (uint32_t j = 0; j < steps; ++j) {
                const bool skip_last = uneven && (steps == j + 1);
                const uint32_t idx0 = idx_array[start + 2 * j];
                const uint32_t idx1 = skip_last ? idx0 : idx_array[start + 2 * j + 1];
                uint32_t node[8], rt[8], t[8], hidx[8], has[8], par[8], ci[8], pt[8];
                bool prop[8], nopar[8], lfp[8], nonc[8], call[8];
                for (int k = 0; k < 8; ++k) {
                    node[k] = k < 4 ? idx0 : idx1;
                    const uint32_t s = k & 3;
                    rt[k] = result_types[node[k]];
                    t[k] = node_types[node[k]];
                    hidx[k] = t[k] * 24u + s * 6u + rt[k];
                    const bool load = (k < 4) || !skip_last;
                    has[k] = load ? has_instr[hidx[k]] : 0u;
                    prop[k] = has[k] != 0 || k == 0 || (k == 4 && !skip_last);
                    par[k] = prop[k] ? static_cast<uint32_t>(parents[node[k]]) : 0u;
                    nopar[k] = s32(par[k]) == -1;
                    lfp[k] = !nopar[k] && prop[k];
                    pt[k] = lfp[k] ? node_types[s32(par[k])] : 0u;
                    ci[k] = lfp[k] ? static_cast<uint32_t>(child_idx[node[k]]) : 0u;
                    nonc[k] = ((pt[k] & port::T_IF) == port::T_IF) && !(ci[k] == (pt[k] & 1u));
                    call[k] = nonc[k];
                }
                for (int k = 0; k < 8; ++k) {
                    const bool load = (nopar[k] || !nonc[k]) && prop[k];
                    const uint32_t calc = load ? pai_tab[hidx[k]] : 0u;
                    if (calc == 1) call[k] = true;
                    if (calc == 2 && s32(result_types[node[k]]) > 1) call[k] = true;
                }
                int32_t pai[8];
                uint32_t iib[8], rdv[8], dpv[8], loc[8];
                bool any_has = false;
                for (int k = 0; k < 8; ++k) any_has |= has[k] != 0;
                for (int k = 0; k < 8; ++k) {
                    pai[k] = call[k] ? s32(par[k] * 3u + ci[k]) : -1;
                    iib[k] = static_cast<uint32_t>(k & 3) + (prop[k] ? node_locations[node[k]] : 0u);
                    uint32_t r = 0;
                    if (any_has) {
                        const uint32_t calc = has[k] ? out_tab[hidx[k]] : 0xFFFFFFFFu;
                        if (calc == 3) r |= 32u;
                        if (calc == 4) r |= 10u;
                        if (calc == 1 || calc == 2) {
                            const uint32_t nd = node_data[node[k]];
                            if (calc == 1) r |= nd + 10u;
                            if (calc == 2) r |= nd + 42u;
                        }
                        bool hov = call[k] && has[k];
                        if (calc == 0 && has_output[hidx[k]]) hov = true;
                        if (hov) r |= iib[k] + 64u;
                    }
                    rdv[k] = r;
                    const bool use_rd = nopar[k] || (!nonc[k] && lfp[k]);
                    const uint32_t instr_no = iib[k] + (nonc[k] ? size_flat(t[k] * 6u + rt[k]) : 0u);
                    dpv[k] = (use_rd ? r : 0u) | (nonc[k] ? instr_no : 0u);
                    loc[k] = has[k] ? iib[k] : 0u;
                }
                for (int k = 0; k < 8; ++k) {
                    const uint32_t s = k & 3;
                    const bool ie = s == 1 && t[k] == port::T_IF_ELSE;
                    const bool wh = s == 1 && t[k] == port::T_WHILE;
                    if (ie || wh) loc[k] = registers[s32(node[k] * 3u + (ie ? 1u : 0u) + (wh ? 2u : 0u))];
                    const bool add2 = t[k] == port::T_FUNC_DECL || (s > 1 && t[k] == port::T_FUNC_DECL_DUMMY);
                    const bool fcal = s == 1 && t[k] == port::T_FUNC_CALL_ARG_LIST;
                    if (add2 || fcal) loc[k] += 2u;
                    if (fcal) {
                        const int64_t prev = static_cast<int64_t>(node[k]) - 1;
                        const uint32_t prev_t = node_types[prev];
                        if ((prev_t & port::T_FUNC_CALL_ARG) == port::T_FUNC_CALL_ARG) {
                            loc[k] += static_cast<uint32_t>(child_idx[prev]);
                        }
                    }
                }
                uint32_t words[8], jtv[8], r1[8], r2[8];
                for (int k = 0; k < 8; ++k) {
                    const uint32_t s = k & 3;
                    uint32_t w = has[k] ? instr_tab[hidx[k]] : 0u;
                    const uint32_t ici = t[k] * 4u + s;
                    const uint32_t nd = has[k] ? node_data[node[k]] : 0u;
                    const uint32_t cc = has[k] ? const_tab[ici] : 0u;
                    if (cc == 1) w |= nd & 0xFFFFF000u;
                    if (cc == 2) w |= (nd & 0xFFFu) << 20;
                    const uint32_t m4 = nd * 4u;
                    if (cc == 3) w |= (0u - (m4 + 8u)) << 20;
                    if (cc == 4) w |= m4 << 20;
                    if (cc == 5) w |= (0u - m4) << 20;
                    words[k] = w;

                    const uint32_t jc = has[k] ? jt_tab[ici] : 0u;
                    uint32_t jv = 0;
                    if (s32(jc) > 0 && !(s32(jc) > 5)) {
                        uint32_t v = registers[s32(node[k] * 3u + 1u + (s32(jc) > 2 ? 1u : 0u))];
                        if ((jc & 1u) == 0) v += 1u;
                        jv = v;
                    }
                    if (jc == 6) jv |= func_ends[s32(nd)] - 6u;
                    if (jc == 7) jv |= func_starts[s32(nd)];
                    jtv[k] = jv;

                    for (uint32_t p = 0; p < 2; ++p) {
                        const uint32_t c = has[k] ? operand_tab[hidx[k] * 2u + p] : 0u;
                        uint32_t a = 0;
                        if (c == 1 || c == 4 || c == 5 || c == 6) {
                            uint32_t ri = node[k] * 3u;
                            if (c == 1) ri += p;
                            if (c == 4 || c == 5) ri += 1u;
                            if (c == 5) ri -= p;
                            a = registers[s32(ri)];
                        }
                        if (c == 2) a |= nd + 10u;
                        if (c == 3) a |= nd + 42u;
                        if (c == 7) a |= iib[k] + 63u;
                        (p == 0 ? r1 : r2)[k] = a;
                    }
                }
                for (int k = 0; k < 8; ++k) {
                    if (has[k]) {
                        const uint32_t at = loc[k];
                        instr[at] = words[k];
                        rd[at] = rdv[k];
                        rs1[at] = r1[k];
                        rs2[at] = r2[k];
                        jt[at] = jtv[k];
                    }
                }
                for (int k = 0; k < 8; ++k) {
                    if (pai[k] >= 0) registers[pai[k]] = dpv[k];
                }
            }
        }
    }

    // ---------------------------------------------------------------- optimize
    // rv_generator_avx.cpp:891-1016
    void optimize() {
        const size_t W = instr.size();
        const size_t nb = blocks32(W);
        PBuf<uint32_t> used(W);
        for (size_t i = 0; i < 8 * nb; ++i) {
            const int32_t a = s32(rs1[i] - 64u);
            if (a >= 0) used[a] = 0xFFFFFFFFu;
        }
        for (size_t i = 0; i < 8 * nb; ++i) {
            const int32_t a = s32(rs2[i] - 64u);
            if (a >= 0) used[a] = 0xFFFFFFFFu;
        }
        // Store marks do not change between iterations.
        std::vector<int32_t> store_marks;
        for (size_t i = 0; i < 8 * nb; ++i) {
            const uint32_t f = instr[i] & 0x707Fu;
            if (f == 0x2023u || f == 0x2027u) {
                store_marks.push_back(s32(rs1[i] - 64u));
                store_marks.push_back(s32(rs2[i] - 64u));
            }
        }
        for (;;) {
            PBuf<uint32_t> next = used.clone();
            for (size_t i = 0; i < 8 * nb; ++i) {
                if (s32(rd[i]) > 63 && used[s32(rd[i] - 64u)] == 0) {
                    const int32_t a = s32(rs1[i] - 64u);
                    const int32_t b = s32(rs2[i] - 64u);
                    if (a >= 0) next[a] = 0;
                    if (b >= 0) next[b] = 0;
                }
            }
            for (int32_t m : store_marks) {
                if (m >= 0) next[m] = 0xFFFFFFFFu;
            }
            const bool same = used.equal(next);
            used = next.clone();
            if (same) break;
        }
        used_instrs.resize(W);
        for (size_t i = 0; i < 8 * nb; ++i) {
            used_instrs[i] = (!(s32(rd[i]) > 63)) ? 0xFFFFFFFFu : used[i];
        }
    }

    // ---------------------------------------------------------------- regalloc
    // rv_generator_avx.cpp:1018-1814
    void regalloc() {
        const size_t F = function_sizes.size();
        const size_t G = blocks32(F);
        uint32_t max_size = 0;
        for (size_t f = 0; f < F; ++f) max_size = std::max(max_size, function_sizes[f]);
        PBuf<uint64_t> lifetime(F);
        for (size_t f = 0; f < F; ++f) lifetime[f] = 0x1Full;
        const size_t W = used_instrs.size();
        PBuf<uint32_t> symreg(W), symswp(W);
        // Only row 0 of the register state is ever read (its index carries no function
        // offset, :1290/:1301/:1312); rows 1..7 are written and never read.
        uint32_t row0[64];
        std::fill(row0, row0 + 64, 0xFFFFFFFFu);

        // Functions still active at a step, in index order.
        std::vector<uint32_t> active(F);
        std::iota(active.begin(), active.end(), 0u);

        struct Lane {
            uint32_t f;
            bool valid;
            uint32_t ins, r1, r2, r1r, r2r, ord, rdr;
            uint64_t cleared, rdm;
            bool sw_rd, sw_r1, sw_r2;
        };
        std::vector<Lane> grp;
        grp.reserve(8);

        for (uint32_t i = 0; i < max_size; ++i) {
            uint32_t snap[64];
            std::copy(row0, row0 + 64, snap);
            size_t a = 0;
            while (a < active.size()) {
                const uint32_t j = active[a] / 8;
                grp.clear();
                while (a < active.size() && active[a] / 8 == j) {
                    const uint32_t f = active[a++];
                    Lane L{};
                    L.f = f;
                    const uint32_t st = func_starts[f];
                    const uint32_t sz = function_sizes[f];
                    const uint32_t off = (s32(i) >= s32(sz)) ? 0xFFFFFFFFu : st + i;
                    L.valid = off != 0xFFFFFFFFu;
                    if (!L.valid) continue;
                    L.ins = instr[off];
                    if (L.ins == 0x000000EFu) throw Unsupported("jal call word reaches the reference's unused call path");
                    L.r1 = rs1[off];
                    L.r2 = rs2[off];
                    L.ord = rd[off];
                    grp.push_back(L);
                }
                // Phase A: lookups, allocation, swap detection (all lanes of the group)
                for (Lane& L : grp) {
                    const bool r1v = s32(L.r1) > 63;
                    const bool r2v = s32(L.r2) > 63;
                    uint32_t r1r = r1v ? symreg[s32(L.r1 - 64u)] : 0u;
                    uint32_t r1s = r1v ? symswp[s32(L.r1 - 64u)] : 0u;
                    uint32_t r2r = r2v ? symreg[s32(L.r2 - 64u)] : 0u;
                    uint32_t r2s = r2v ? symswp[s32(L.r2 - 64u)] : 0u;
                    const bool fop = (L.ins & 0x7Fu) == 0x53u;
                    if (r1s) r1r = (L.ins == 0xC0007053u || fop) ? 37u : 5u;
                    if (r2s) r2r = fop ? 38u : 6u;
                    L.r1r = r1r;
                    L.r2r = r2r;
                    auto bit = [](uint32_t r) -> uint64_t {
                        const int64_t sr = s32(r);
                        return (sr >= 0 && sr < 64) ? (1ull << sr) : 0ull;
                    };
                    const uint64_t clear = (bit(r1r) | bit(r2r)) & ~1ull;
                    const uint64_t lt = lifetime[L.f];
                    L.cleared = lt & ~clear;
                    uint32_t r = L.ord;
                    if (s32(r) > 63) {
                        const bool rdf = L.ins == 0xD0007053u || fop;
                        const uint64_t adj = rdf ? 0x00000000FFFFFFFFull : 0xFFFFFFFF00000000ull;
                        const uint64_t m = L.cleared | adj;
                        // ptilopsis::ffz (include/utils.hpp:23-47) hands the 64-bit mask to
                        // __builtin_ffs(int): only the low 32 bits are searched.
                        const uint32_t low = static_cast<uint32_t>(m);
                        r = (low == 0xFFFFFFFFu) ? 64u : static_cast<uint32_t>(__builtin_ctz(~low));
                        if (r == 64) r = rdf ? 37u : 5u;
                    }
                    L.rdr = r;
                    L.rdm = bit(r);
                    L.sw_r1 = r1r != 0 && (lt & bit(r1r)) != 0;
                    L.sw_r2 = r2r != 0 && (lt & bit(r2r)) != 0;
                    L.sw_rd = r != 0 && (L.cleared & L.rdm) != 0;
                }
                // Phase B: swap marks through row 0 of the step snapshot (rd, rs1, rs2)
                auto mark = [&](uint32_t phys) {
                    const int32_t v = s32(snap[phys] - 64u);
                    if (v >= 0) symswp[v] = 0xFFFFFFFFu;
                };
                for (Lane& L : grp) if (L.sw_rd) mark(L.rdr);
                for (Lane& L : grp) if (L.sw_r1) mark(L.r1r);
                for (Lane& L : grp) if (L.sw_r2) mark(L.r2r);
                // Phase C: lifetimes
                for (Lane& L : grp) lifetime[L.f] = L.cleared | L.rdm;
                // Phase D: register-state rows; only lane 0 (f % 8 == 0) writes row 0
                for (Lane& L : grp) if ((L.f & 7u) == 0 && L.ord != 0) row0[L.rdr] = L.ord;
                for (Lane& L : grp) if ((L.f & 7u) == 0 && L.r1r != L.rdr && s32(L.r1r) >= 0) row0[L.r1r] = 0xFFFFFFFFu;
                for (Lane& L : grp) if ((L.f & 7u) == 0 && L.r2r != L.rdr && s32(L.r2r) >= 0) row0[L.r2r] = 0xFFFFFFFFu;
                // Phase E: symbol table
                for (Lane& L : grp) if (s32(L.ord) > 63) { symreg[s32(L.ord - 64u)] = L.rdr; symswp[s32(L.ord - 64u)] = 0; }
                for (Lane& L : grp) if (s32(L.r1) > 63) { symreg[s32(L.r1 - 64u)] = L.r1r; symswp[s32(L.r1 - 64u)] = 0; }
                for (Lane& L : grp) if (s32(L.r2) > 63) { symreg[s32(L.r2 - 64u)] = L.r2r; symswp[s32(L.r2 - 64u)] = 0; }
            }
            // Retire functions whose last instruction was this step.
            size_t w = 0;
            for (uint32_t f : active) if (function_sizes[f] > i + 1) active[w++] = f;
            active.resize(w);
        }
        (void)G;

        // Function-start flags and the spill "segmented fill", :1422-1469
        std::vector<uint8_t> is_start(W + 1, 0);
        for (size_t f = 0; f < F; ++f) {
            const uint32_t s = func_starts[f];
            if (s < W) is_start[s] = 1;
        }
        PBuf<uint32_t> spill(W);
        for (size_t v = 0; v < W; ++v) spill[v] = symswp[v] & 1u;
        for (size_t v = 0; v < W; ++v) {
            if (!is_start[v]) spill[v] = v > 0 ? spill[v - 1] : 0u;
        }
        // Instruction counts, :1473-1495 (padding lanes of used_instrs are enabled)
        const size_t nb = blocks32(W);
        PBuf<uint32_t> counts(W);
        for (size_t i = 0; i < 8 * nb; ++i) {
            if (!used_instrs[i]) continue;
            uint32_t c = 1;
            auto swp = [&](uint32_t r) { return s32(r) > 63 && symswp[s32(r - 64u)] != 0; };
            if (swp(rs1[i])) ++c;
            if (swp(rs2[i])) ++c;
            if (swp(rd[i])) ++c;
            counts[i] = c;
        }
        // Exclusive scan, :1524-1538
        PBuf<uint32_t> offs(W);
        {
            uint32_t acc = 0;
            for (size_t i = 0; i < 8 * nb; ++i) {
                acc += counts[static_cast<int64_t>(i) - 1];
                offs[i] = acc;
            }
        }
        const uint32_t new_count = (W == 0) ? 0 : offs[W - 1] + 1;
        PBuf<uint32_t> ni(new_count), nrd(new_count), nr1(new_count), nr2(new_count), njt(new_count);
        // Scatter with loads/stores of swapped registers, :1552-1697
        for (size_t b = 0; b < nb; ++b) {
            bool any_used = false;
            for (int l = 0; l < 8; ++l) any_used |= used_instrs[8 * b + l] != 0;
            if (!any_used) continue;
            int32_t ld1[8], ld2[8], mainoff[8], rdoff[8];
            uint32_t a1[8], a2[8], ad[8], i1[8], i2[8], id[8];
            for (int l = 0; l < 8; ++l) {
                const size_t i = 8 * b + l;
                const bool u = used_instrs[i] != 0;
                const uint32_t base = u ? offs[i] : 0xFFFFFFFFu;
                const uint32_t ins = u ? instr[i] : 0u;
                const bool fop = (ins & 0x7Fu) == 0x53u;

                const uint32_t r1 = u ? rs1[i] : 0u;
                uint32_t l1 = 0xFFFFFFFFu, st1 = 0, al1 = (s32(r1) > 63) ? 0u : r1;
                if (s32(r1) > 63) {
                    const uint32_t sw = symswp[s32(r1 - 64u)];
                    l1 = ~sw | base;
                    st1 = spill[s32(r1 - 64u)];
                    const bool nf = ins == 0xC0007053u || fop;
                    al1 |= sw ? 0u : symreg[s32(r1 - 64u)];
                    if (sw) al1 |= nf ? 37u : 5u;
                }
                const uint32_t r2 = u ? rs2[i] : 0u;
                uint32_t l2 = 0xFFFFFFFFu, st2 = 0, al2 = (s32(r2) > 63) ? 0u : r2;
                if (s32(r2) > 63) {
                    const uint32_t sw = symswp[s32(r2 - 64u)];
                    // The reference tests its own initial value (-1 > 0) here, so the
                    // rs2 load lands on the same slot as the rs1 load.
                    l2 = ~sw | base;
                    st2 = spill[s32(r2 - 64u)];
                    al2 |= sw ? 0u : symreg[s32(r2 - 64u)];
                    if (sw) al2 |= fop ? 38u : 6u;
                }
                const uint32_t mo = base + (s32(l1) > 0 ? 1u : 0u) + (s32(l2) > 0 ? 1u : 0u);
                const uint32_t r = u ? rd[i] : 0u;
                uint32_t ro = 0xFFFFFFFFu, str = 0, ar = (s32(r) > 63) ? 0u : r;
                if (s32(r) > 63) {
                    const uint32_t sw = symswp[s32(r - 64u)];
                    ro = ~sw | (mo + 1u);
                    str = spill[s32(r - 64u)];
                    ar |= symreg[s32(r - 64u)];
                }
                ld1[l] = s32(l1); ld2[l] = s32(l2); mainoff[l] = s32(mo); rdoff[l] = s32(ro);
                a1[l] = al1; a2[l] = al2; ad[l] = ar;
                i1[l] = (((st1 - 1u) * 4u) << 20) | 0x2003u;
                i2[l] = (((st2 - 1u) * 4u) << 20) | 0x2003u;
                const uint32_t imm = (str - 1u) * 0xFFFFFFFCu;
                id[l] = 0x2023u | ((imm & 0x1Fu) << 7) | ((imm & 0xFEu) << 19);
            }
            for (int l = 0; l < 8; ++l) if (ld1[l] >= 0) { ni[ld1[l]] = i1[l]; nrd[ld1[l]] = 5; }
            for (int l = 0; l < 8; ++l) if (ld2[l] >= 0) { ni[ld2[l]] = i2[l]; nrd[ld2[l]] = 6; }
            for (int l = 0; l < 8; ++l) {
                if (mainoff[l] >= 0) {
                    const size_t i = 8 * b + l;
                    const int32_t at = mainoff[l];
                    ni[at] = instr[i];
                    nrd[at] = ad[l];
                    nr1[at] = a1[l];
                    nr2[at] = a2[l];
                    njt[at] = offs[s32(jt[i])];
                }
            }
            for (int l = 0; l < 8; ++l) if (rdoff[l] >= 0) { ni[rdoff[l]] = id[l]; nr1[rdoff[l]] = ad[l]; }
        }
        instr = ni.clone();
        rd = nrd.clone();
        rs1 = nr1.clone();
        rs2 = nr2.clone();
        jt = njt.clone();
        fix_func_tab(offs, W);
        // Prologue/epilogue stack-size words, :1701-1811 (preserve masks stay 0,
        // so every frame is 8 bytes: lui s0, 0 ; addi s0, s0, 8)
        const uint32_t upper_instr = 0x00000437u;
        const uint32_t lower_instr = (8u << 20) | 0x00040413u;
        const size_t fb = blocks32(F);
        for (size_t b = 0; b < fb; ++b) {
            uint32_t st[8], en[8];
            bool ok[8];
            for (int l = 0; l < 8; ++l) {
                const size_t f = 8 * b + l;
                ok[l] = f < F;
                st[l] = ok[l] ? func_starts[f] : 0u;
                en[l] = st[l] + (ok[l] ? function_sizes[f] : 0u);
            }
            auto fix = [&](const uint32_t* at, int32_t delta, uint32_t word) {
                for (int l = 0; l < 8; ++l) {
                    if (!ok[l]) continue;
                    const uint32_t p = at[l] + static_cast<uint32_t>(delta);
                    instr[p] = word; rd[p] = 0; rs1[p] = 0; rs2[p] = 0; jt[p] = 0;
                }
            };
            fix(st, 2, upper_instr);
            fix(st, 3, lower_instr);
            fix(en, -6, upper_instr);
            fix(en, -5, lower_instr);
        }
    }

    // rv_generator_avx.cpp:1816-1837
    void fix_func_tab(PBuf<uint32_t>& offs, size_t offs_size) {
        const size_t fb = blocks32(func_starts.size());
        for (size_t b = 0; b < fb; ++b) {
            for (int l = 0; l < 8; ++l) {
                const size_t f = 8 * b + l;
                const uint32_t si = func_starts[f];
                const uint32_t so = offs[s32(si)];
                const uint32_t ei = si + function_sizes[f];
                const bool past = s32(ei) >= s32(static_cast<uint32_t>(offs_size));
                const uint32_t eo = past ? offs[static_cast<int64_t>(offs_size) - 1] + 1u : offs[s32(ei)];
                func_starts[f] = so;
                func_ends[f] = eo;
                function_sizes[f] = eo - so;
            }
        }
    }

    // ---------------------------------------------------------------- fix_jumps
    // rv_generator_avx.cpp:1853-1993
    void fix_jumps() {
        const size_t W = instr.size();
        const size_t nb = blocks32(W);
        PBuf<uint32_t> sizes(W), offs(W);
        for (size_t i = 0; i < 8 * nb; ++i) {
            const uint32_t w = instr[i];
            const bool jump = (w & 0x7Fu) == 0x67u && w != 0x8067u;
            sizes[i] = jump ? 2u : (w != 0 ? 1u : 0u);
        }
        {
            uint32_t acc = 0;
            for (size_t i = 0; i < 8 * nb; ++i) {
                acc += sizes[static_cast<int64_t>(i) - 1];
                offs[i] = acc;
            }
        }
        const uint32_t count = sizes.back() + offs.back();
        PBuf<uint32_t> ni(count), nrd(count), nr1(count), nr2(count), njt(count);
        for (size_t i = 0; i < W; ++i) {
            const uint32_t at = offs[i];
            ni[at] = instr[i]; nrd[at] = rd[i]; nr1[at] = rs1[i]; nr2[at] = rs2[i]; njt[at] = jt[i];
        }
        for (size_t i = 0; i < 8 * blocks32(count); ++i) njt[i] = offs[s32(njt[i])];
        for (size_t b = 0; b < nb; ++b) {
            uint32_t at[8], w[8];
            bool jump[8], branch[8];
            bool any = false;
            for (int l = 0; l < 8; ++l) {
                at[l] = offs[8 * b + l];
                w[l] = ni[s32(at[l])];
                jump[l] = (w[l] & 0x7Fu) == 0x67u && w[l] != 0x8067u;
                branch[l] = (w[l] & 0x7Fu) == 0x63u;
                any |= jump[l] || branch[l];
            }
            if (!any) continue;
            uint32_t delta[8];
            for (int l = 0; l < 8; ++l) {
                const uint32_t tgt = (jump[l] || branch[l]) ? 4u * njt[s32(at[l])] : 0u;
                delta[l] = tgt - at[l] * 4u;
            }
            for (int l = 0; l < 8; ++l) {
                if (!jump[l]) continue;
                const uint32_t upper = (delta[l] & 0xFFFFF000u) >> 12;
                const uint32_t lower = delta[l] & 0xFFFu;
                const uint32_t sign = (delta[l] >> 11) & 1u;
                const uint32_t auipc = ((upper + sign) << 12) | 0x97u;
                const uint32_t jalr = w[l] | (lower << 20) | (1u << 15);
                const int64_t p = at[l];
                ni[p] = auipc; njt[p] = 0; nrd[p] = 0; nr1[p] = 0; nr2[p] = 0;
                ni[p + 1] = jalr; njt[p + 1] = 0; nrd[p + 1] = 0; nr1[p + 1] = 0; nr2[p + 1] = 0;
            }
            for (int l = 0; l < 8; ++l) {
                if (!branch[l]) continue;
                const uint32_t d = delta[l];
                const uint32_t word = w[l] | (((d >> 12) & 1u) << 31) | (((d >> 11) & 1u) << 7) |
                                      (((d >> 5) & 0x1Fu) << 25) | (((d >> 1) & 0xFu) << 8);
                ni[s32(at[l])] = word;
            }
        }
        instr = ni.clone();
        jt = njt.clone();
        rd = nrd.clone();
        rs1 = nr1.clone();
        rs2 = nr2.clone();
        fix_func_tab(offs, W);
    }

    // ---------------------------------------------------------------- postprocess
    // rv_generator_avx.cpp:1995-2011
    void postprocess() {
        for (size_t i = 0; i < 8 * blocks32(instr.size()); ++i) {
            instr[i] |= ((rd[i] & 31u) << 7) | ((rs1[i] & 31u) << 15) | ((rs2[i] & 31u) << 20);
        }
    }
};

// ==================================================================== scalar generator
// Restatement of the reference's single-threaded proof of concept, rv_generator_st
// (src/codegen/rv_generator.cpp:227-1736, the -s flag of src/main.cpp), written as its
// own loops: preprocess, isn_cnt, isn_gen, optimize, regalloc and fix_jumps have their
// own rules there (fix_jumps differs only in the jump targets it leaves, which no output
// word reads); postprocess is the AVX generator's.  The reference keeps registers, rd, rs1 and rs2 in
// int64 built from u32 arithmetic; they are kept here as u32 and read zero-extended.
struct GenSt : Gen {
    static bool is_float_like(uint32_t rt) { return (rt & 1u) && (rt & 6u); }
    uint32_t tsize(uint32_t t, uint32_t rt) const { return size_flat(t * 6u + rt); }
    uint32_t tab3(const uint32_t* tab, uint32_t t, uint32_t s, uint32_t rt) const { return tab[t * 24u + s * 6u + rt]; }

    // rv_generator.cpp:227-314
    void preprocess_st() {
        for (size_t i = 0; i < n; ++i) {  // argument placement, :231-284
            uint32_t t = node_types[i];
            if ((t & port::T_FUNC_ARG) != port::T_FUNC_ARG) continue;
            const uint32_t rt = result_types[i];
            uint32_t nd = node_data[i];
            const bool fl = is_float_like(rt);
            if (fl && nd < 8u) continue;
            const int32_t ci = child_idx[i];
            const int32_t ints = fl ? static_cast<int32_t>(static_cast<uint32_t>(ci) - nd) : static_cast<int32_t>(nd);
            const int32_t floats = ci - ints;
            const int32_t ir = ints + std::max<int32_t>(floats - 8, 0);
            if (ir < 8) {
                nd = static_cast<uint32_t>(ir);
                if (fl) t |= 0b01u;
            } else {
                t |= 0b10u;
                nd = static_cast<uint32_t>(ir - 8);
            }
            node_types[i] = t;
            node_data[i] = nd;
        }
        for (size_t i = 1; i < n; ++i) {  // call argument lists, :287-304
            if (node_types[i] != port::T_FUNC_CALL_ARG_LIST) continue;
            const size_t prev = i - 1;
            int64_t stack_args = 0;
            if (node_types[prev] == port::T_FUNC_CALL_ARG) {
                if (result_types[prev] == port::D_FLOAT) {
                    const int64_t int_args = static_cast<int64_t>(child_idx[prev]) - static_cast<int64_t>(node_data[prev]);
                    stack_args = std::max<int64_t>(int_args - 8, 0);
                }
            } else if (node_types[prev] == port::T_FUNC_CALL_ARG_ON_STACK) {
                stack_args = static_cast<uint32_t>(node_data[prev] + 1u);
            }
            node_data[i] = static_cast<uint32_t>(stack_args);
        }
        for (size_t i = 0; i < n; ++i) {  // float comparisons, :306-313
            const int32_t p = parents[i];
            if (p >= 0 && (node_types[p] & port::T_EQ) == port::T_EQ && result_types[i] == port::D_FLOAT) {
                result_types[p] = port::D_FLOAT;
            }
        }
    }

    // rv_generator.cpp:316-446
    void isn_cnt_st() {
        for (size_t i = 0; i < n; ++i) {
            const uint32_t t = node_types[i];
            uint32_t delta = 0;
            if (i > 0 && t == port::T_FUNC_CALL_ARG_LIST) {
                delta = 1;
                if ((node_types[i - 1] & port::T_FUNC_CALL_ARG) == port::T_FUNC_CALL_ARG) {
                    delta += static_cast<uint32_t>(child_idx[i - 1]) + 1u;
                }
            }
            const int32_t p = parents[i];
            if (p != -1) {
                const uint32_t pt = p >= 0 ? node_types[p] : static_cast<uint32_t>(port::T_STATEMENT_LIST);
                const int32_t ci = child_idx[i];
                if (ci == 0 && (pt == port::T_IF || pt == port::T_IF_ELSE)) delta += 1;
                else if (ci == 1 && (pt == port::T_IF_ELSE || pt == port::T_WHILE)) delta += 1;
            }
            node_sizes[i] = tsize(t, result_types[i]) + delta;
        }
        uint32_t acc = 0;
        for (size_t i = 0; i < n; ++i) {
            node_locations[i] = acc;
            acc += node_sizes[i];
        }
        for (size_t i = 0; i < n; ++i) {
            if (node_types[i] == port::T_INVALID) node_locations[i] = 0xFFFFFFFFu;
        }
        std::vector<int64_t> fix_idx(n, -1);
        std::vector<uint32_t> fix_val(n, 0);
        for (size_t i = 0; i < n; ++i) {
            const int32_t p = parents[i];
            if (p == -1) continue;
            const uint32_t pt = node_types[p];
            if ((pt & port::T_IF) == port::T_IF && child_idx[i] == static_cast<int32_t>(pt & 1u)) {
                fix_idx[i] = p;
                fix_val[i] = node_locations[i] + tsize(node_types[i], result_types[i]);
            } else if ((node_types[i] & port::T_FUNC_CALL_ARG) == port::T_FUNC_CALL_ARG) {
                fix_idx[i] = static_cast<int64_t>(i);
                fix_val[i] = node_locations[p] + static_cast<uint32_t>(child_idx[i]) + 1u;
            }
        }
        for (size_t i = 0; i < n; ++i) {
            if (fix_idx[i] >= 0) node_locations[fix_idx[i]] = fix_val[i];
        }
        std::vector<uint32_t> decls;
        for (size_t i = 0; i < n; ++i) if (node_types[i] == port::T_FUNC_DECL) decls.push_back(static_cast<uint32_t>(i));
        const size_t F = decls.size();
        if (F == 0) throw Unsupported("program has no function (the reference takes the max of an empty range)");
        function_ids.resize(F);
        func_starts.resize(F);
        func_ends.resize(F);
        function_sizes.resize(F);
        for (size_t f = 0; f < F; ++f) {
            function_ids[f] = node_data[decls[f]];
            const uint32_t off = node_locations[decls[f]] + 6u;
            const uint32_t prev = f == 0 ? 0u : node_locations[decls[f - 1]] + 6u;
            function_sizes[f] = f == 0 ? off : off - prev;
            func_starts[f] = prev;
            func_ends[f] = prev + function_sizes[f];
        }
    }

    // rv_generator.cpp:448-809
    void isn_gen_st() {
        std::vector<uint32_t> idx_array(n);
        std::iota(idx_array.begin(), idx_array.end(), 0u);
        std::sort(idx_array.begin(), idx_array.end(), [this](uint32_t a, uint32_t b) { return depth[a] < depth[b]; });
        std::vector<uint32_t> depth_starts;
        for (size_t i = 0; i < n; ++i) {
            if (i == 0 || depth[idx_array[i]] != depth[idx_array[i - 1]]) depth_starts.push_back(static_cast<uint32_t>(i));
        }
        if (depth_starts.size() != max_depth + 1) throw Unsupported("depths 0..max_depth are not all populated");
        const uint32_t W = node_locations[static_cast<int64_t>(n) - 1];
        std::vector<int64_t> registers(n * 3, 0);
        instr.resize(W); rd.resize(W); rs1.resize(W); rs2.resize(W); jt.resize(W);
        const uint32_t* has_instr = &T.has_instr[0][0][0];
        const uint32_t* has_output = &T.has_output[0][0][0];
        const uint32_t* pai_tab = &T.pai[0][0][0];
        const uint32_t* out_tab = &T.out[0][0][0];
        const uint32_t* instr_tab = &T.instr[0][0][0];
        const uint32_t* const_tab = &T.cnst[0][0];
        const uint32_t* operand_tab = &T.operand[0][0][0][0];
        const uint32_t* jt_tab = &T.jt[0][0];
        const size_t F = func_starts.size();

        auto parent_arg_idx = [&](uint32_t node, uint32_t s) -> int64_t {
            const int64_t pidx = static_cast<int64_t>(parents[node]) * 3 + child_idx[node];
            auto lookup = [&]() -> int64_t {
                const uint32_t calc = tab3(pai_tab, node_types[node], s, result_types[node]);
                if (calc == 1) return pidx;
                if (calc == 2 && result_types[node] > 1u) return pidx;
                return -1;
            };
            const int32_t p = parents[node];
            if (p == -1) return lookup();
            const uint32_t pt = node_types[p];
            const int32_t ci = child_idx[node];
            if (ci > 0 && (pt == port::T_IF || pt == port::T_IF_ELSE)) return pidx;
            if ((ci == 0 || ci == 2) && pt == port::T_WHILE) return pidx;
            return lookup();
        };
        auto prop_value = [&](uint32_t node, int64_t rdv, int64_t off) -> int64_t {
            const int32_t p = parents[node];
            if (p == -1) return rdv;
            const uint32_t pt = node_types[p];
            const int32_t ci = child_idx[node];
            const int64_t instr_no = off + tsize(node_types[node], result_types[node]);
            if (pt == port::T_IF || pt == port::T_IF_ELSE) return (ci == 1 || ci == 2) ? instr_no : rdv;
            if (pt == port::T_WHILE) return (ci == 0 || ci == 2) ? instr_no : rdv;
            return rdv;
        };
        auto extend12 = [](uint32_t x) { return static_cast<uint32_t>(static_cast<int32_t>(x << 20) >> 20); };

        struct Entry { int64_t at, pidx; uint32_t word, jtv; int64_t rdv, r1, r2, reg; };
        std::vector<Entry> entries;
        for (size_t lvl = 0; lvl <= max_depth; ++lvl) {
            const size_t cur = max_depth - lvl;
            const uint32_t start = depth_starts[cur];
            const uint32_t end = cur == max_depth ? static_cast<uint32_t>(n) : depth_starts[cur + 1];
            entries.clear();
            for (uint32_t k = start; k < end; ++k) {
                const uint32_t idx = idx_array[k];
                const uint32_t t = node_types[idx], rt = result_types[idx], nd = node_data[idx];
                const int64_t* reg = &registers[static_cast<size_t>(idx) * 3];
                for (uint32_t s = 0; s < 4; ++s) {
                    Entry e{-1, -1, 0, 0, 0, 0, 0, 0};
                    if (tab3(has_instr, t, s, rt)) {
                        const uint32_t iib = node_locations[idx] + s;
                        const uint32_t oc = tab3(out_tab, t, s, rt);
                        int64_t rdv;
                        if (oc == 1) rdv = static_cast<uint32_t>(nd + 10u);
                        else if (oc == 2) rdv = static_cast<uint32_t>(nd + 42u);
                        else if (oc == 3) rdv = 32;
                        else if (oc == 4) rdv = 10;
                        else rdv = (parent_arg_idx(idx, s) != -1 || tab3(has_output, t, s, rt)) ? static_cast<uint32_t>(iib + 64u) : 0;
                        int64_t at;
                        if (s == 1 && t == port::T_IF_ELSE) at = reg[1];
                        else if (s == 1 && t == port::T_WHILE) at = reg[2];
                        else if ((s >= 2 && t == port::T_FUNC_DECL_DUMMY) || t == port::T_FUNC_DECL) at = static_cast<uint32_t>(iib + 2u);
                        else if (s == 1 && t == port::T_FUNC_CALL_ARG_LIST) {
                            uint32_t res = iib + 2u;
                            if (idx != 0) {
                                const uint32_t pv = node_types[idx - 1];
                                if (pv == port::T_FUNC_CALL_ARG || pv == port::T_FUNC_CALL_ARG_FLOAT_AS_INT ||
                                    pv == port::T_FUNC_CALL_ARG_ON_STACK) {
                                    res += static_cast<uint32_t>(child_idx[idx - 1]);
                                }
                            }
                            at = res;
                        } else {
                            at = iib;
                        }
                        e.at = static_cast<int32_t>(at);
                        e.pidx = static_cast<int32_t>(parent_arg_idx(idx, s));
                        uint32_t w = tab3(instr_tab, t, s, rt);
                        switch (const_tab[t * 4u + s]) {
                            case 1: w |= (nd - extend12(nd & 0xFFFu)) & 0xFFFFF000u; break;
                            case 2: w |= (nd & 0xFFFu) << 20; break;
                            case 3: w |= static_cast<uint32_t>(-(4 * (static_cast<int64_t>(static_cast<int32_t>(nd)) + 2))) << 20; break;
                            case 4: w |= (4u * nd) << 20; break;
                            case 5: w |= static_cast<uint32_t>(-(4 * static_cast<int64_t>(static_cast<int32_t>(nd)))) << 20; break;
                            default: break;
                        }
                        e.word = w;
                        e.rdv = rdv;
                        for (uint32_t a = 0; a < 2; ++a) {
                            int64_t v = 0;
                            switch (operand_tab[(t * 24u + s * 6u + rt) * 2u + a]) {
                                case 1: v = reg[a]; break;
                                case 2: v = static_cast<uint32_t>(nd + 10u); break;
                                case 3: v = static_cast<uint32_t>(nd + 42u); break;
                                case 4: v = reg[1]; break;
                                case 5: v = reg[1 - a]; break;
                                case 6: v = reg[0]; break;
                                case 7: v = static_cast<int64_t>(iib) + 64 - 1; break;
                                default: break;
                            }
                            (a == 0 ? e.r1 : e.r2) = v;
                        }
                        int64_t j = 0;
                        switch (jt_tab[t * 4u + s]) {
                            case 1: j = reg[1]; break;
                            case 2: j = reg[1] + 1; break;
                            case 3: j = reg[2]; break;
                            case 4: j = reg[2] + 1; break;
                            case 5: j = reg[0]; break;
                            case 6: if (nd >= F) throw Unsupported("jump to a function past the table"); j = func_ends[nd] - 6u; break;
                            case 7: if (nd >= F) throw Unsupported("jump to a function past the table"); j = func_starts[nd]; break;
                            default: break;
                        }
                        e.jtv = static_cast<uint32_t>(j);
                        e.reg = prop_value(idx, rdv, iib);
                    } else if (s == 0) {
                        e.pidx = static_cast<int32_t>(parent_arg_idx(idx, 0));
                        e.reg = prop_value(idx, 0, node_locations[idx]);
                    } else {
                        continue;
                    }
                    entries.push_back(e);
                }
            }
            for (const Entry& e : entries) {
                if (e.at >= 0 && e.at < static_cast<int64_t>(W)) {
                    instr[e.at] = e.word;
                    rd[e.at] = static_cast<uint32_t>(e.rdv);
                    rs1[e.at] = static_cast<uint32_t>(e.r1);
                    rs2[e.at] = static_cast<uint32_t>(e.r2);
                    jt[e.at] = e.jtv;
                }
            }
            for (const Entry& e : entries) {
                if (e.pidx >= 0 && e.pidx < static_cast<int64_t>(registers.size())) registers[e.pidx] = e.reg;
            }
        }
    }

    // rv_generator.cpp:811-900 (Jacobi iterations to the fixed point)
    void optimize_st() {
        const size_t W = instr.size();
        std::vector<uint8_t> used(W, 0);
        auto in_range = [W](int64_t v) { return v >= 0 && v < static_cast<int64_t>(W); };
        for (size_t i = 0; i < W; ++i) {
            if (in_range(int64_t(rs1[i]) - 64)) used[rs1[i] - 64] = 1;
            if (in_range(int64_t(rs2[i]) - 64)) used[rs2[i] - 64] = 1;
        }
        for (;;) {
            const std::vector<uint8_t> before = used;
            std::vector<uint8_t> next = used;
            for (size_t i = 0; i < W; ++i) {
                if (rd[i] < 64u) continue;
                if (!in_range(int64_t(rd[i]) - 64)) throw Unsupported("rd names a word past the program");
                if (before[rd[i] - 64]) continue;
                if (in_range(int64_t(rs1[i]) - 64)) next[rs1[i] - 64] = 0;
                if (in_range(int64_t(rs2[i]) - 64)) next[rs2[i] - 64] = 0;
            }
            for (size_t i = 0; i < W; ++i) {
                const uint32_t m = instr[i] & 0x707Fu;
                if (m != 0x2023u && m != 0x2027u) continue;  // sw, fsw
                if (in_range(int64_t(rs1[i]) - 64)) next[rs1[i] - 64] = 1;
                if (in_range(int64_t(rs2[i]) - 64)) next[rs2[i] - 64] = 1;
            }
            used = next;
            if (used == before) break;
        }
        used_instrs.resize(W);
        for (size_t i = 0; i < W; ++i) used_instrs[i] = (rd[i] < 64u || used[i]) ? 1u : 0u;
    }

    // rv_generator.cpp:1619-1720
    void fix_jumps_st() {
        const size_t W = instr.size();
        auto is_jump = [](uint32_t w) { return (w & 0x7Fu) == 0x67u && w != 0x00008067u; };
        std::vector<int64_t> sizes(W), offs(W);
        for (size_t i = 0; i < W; ++i) sizes[i] = is_jump(instr[i]) ? 2 : (instr[i] == 0 ? 0 : 1);
        int64_t acc = 0;
        for (size_t i = 0; i < W; ++i) { offs[i] = acc; acc += sizes[i]; }
        const int64_t count = W == 0 ? 0 : sizes[W - 1] + offs[W - 1];
        PBuf<uint32_t> ni(count), nrd(count), nr1(count), nr2(count), njt(count);
        for (size_t i = 0; i < W; ++i) {
            const int64_t at = offs[i];
            if (at >= count) throw Unsupported("word past the output");
            ni[at] = instr[i]; nrd[at] = rd[i]; nr1[at] = rs1[i]; nr2[at] = rs2[i]; njt[at] = jt[i];
        }
        for (int64_t i = 0; i < count; ++i) {
            if (njt[i] >= W) throw Unsupported("jump target past the words");
            njt[i] = static_cast<uint32_t>(offs[njt[i]]);
        }
        struct Put { int64_t at; uint32_t w, d, a, b; };
        std::vector<Put> puts;
        for (size_t i = 0; i < W; ++i) {
            const int64_t at = offs[i];
            const uint32_t w = ni[at];
            const bool jump = is_jump(w), branch = (w & 0x7Fu) == 0x63u;
            if (!jump && !branch) continue;
            const uint32_t delta = static_cast<uint32_t>(static_cast<int64_t>(njt[at]) * 4 - at * 4);
            if (jump) {
                const uint32_t upper = ((delta & 0xFFFFF000u) >> 12) + ((delta >> 11) & 1u);
                puts.push_back({at, 0x97u | (upper << 12), 0, 0, 0});
                puts.push_back({at + 1, w | ((delta & 0xFFFu) << 20) | (1u << 15), 0, 0, 0});
            } else {
                const uint32_t word = w | (((delta >> 12) & 1u) << 31) | (((delta >> 11) & 1u) << 7) |
                                      (((delta >> 5) & 0x1Fu) << 25) | (((delta >> 1) & 0xFu) << 8);
                puts.push_back({at, word, nrd[at], nr1[at], nr2[at]});
            }
        }
        for (const Put& p : puts) {
            if (p.at < 0 || p.at >= count) continue;
            ni[p.at] = p.w; njt[p.at] = 0; nrd[p.at] = p.d; nr1[p.at] = p.a; nr2[p.at] = p.b;
        }
        instr = ni.clone(); rd = nrd.clone(); rs1 = nr1.clone(); rs2 = nr2.clone(); jt = njt.clone();
        PBuf<uint32_t> o(W);
        for (size_t i = 0; i < W; ++i) o[i] = static_cast<uint32_t>(offs[i]);
        fix_func_tab(o, W);
    }

    // rv_generator.cpp:902-1602
    void regalloc_st() {
        const size_t W = instr.size();
        const size_t F = function_sizes.size();
        uint32_t S = 0;
        for (size_t f = 0; f < F; ++f) S = std::max(S, function_sizes[f]);
        for (size_t f = 0; f < F; ++f) {
            if (func_starts[f] > W || function_sizes[f] > W - func_starts[f]) throw Unsupported("function past the words");
        }
        constexpr uint64_t kPreserved = 0x0FFC03000FFC031Full, kNonscratch = 0x0FFC03000FFC0200ull;
        std::vector<uint64_t> lifetime(F, 0x1Full), preserve(F, 0);
        std::vector<uint8_t> sym_reg(W, 0), sym_swp(W, 0);
        std::vector<int64_t> state(F * 64, -1);
        auto needs_float = [](uint32_t w, int which) {
            if (w == 0xC0007053u) return which != 0;
            if (w == 0xD0007053u) return which == 0;
            return (w & 0x7Fu) == 0x53u;
        };
        auto check_sym = [W](uint32_t r) {
            if (r >= 64u && r - 64u >= W) throw Unsupported("a register names a word past the program");
        };
        struct Step {
            uint64_t mask = 0;
            int64_t sym[3] = {-1, -1, -1};  // symbols the step assigns
            uint8_t phys[3] = {0, 0, 0};
            uint64_t swapped = 0;           // physical registers whose symbols are swapped out
            bool act = false, call = false;
            uint32_t rdv = 0, rd_phys = 0, r1_phys = 0, r2_phys = 0;
        };
        std::vector<Step> steps(F);
        for (uint32_t i = 0; i < S; ++i) {
            for (size_t f = 0; f < F; ++f) {
                Step& st = steps[f];
                st = Step{};
                st.mask = lifetime[f];
                if (i >= function_sizes[f]) continue;
                const uint32_t off = func_starts[f] + i;
                if (!used_instrs[off]) continue;
                st.act = true;
                const uint32_t w = instr[off];
                const uint32_t start = func_starts[f], end = start + function_sizes[f];
                if (w == 0x000000EFu && (jt[off] < start || jt[off] >= end)) {  // a call, :967-1000
                    st.call = true;
                    st.mask = lifetime[f] & kPreserved;
                    const uint64_t spilled = lifetime[f] & ~kPreserved;
                    st.swapped = spilled;
                    continue;
                }
                check_sym(rs1[off]); check_sym(rs2[off]); check_sym(rd[off]);
                auto sym_of = [&](uint32_t r, uint32_t* reg, bool* sw) {
                    if (r < 64u) { *reg = r; *sw = false; }
                    else { *reg = sym_reg[r - 64u]; *sw = sym_swp[r - 64u] != 0; }
                };
                uint32_t p1, p2;
                bool s1, s2;
                sym_of(rs1[off], &p1, &s1);
                sym_of(rs2[off], &p2, &s2);
                if (s1) p1 = needs_float(w, 1) ? 37u : 5u;
                if (s2) p2 = needs_float(w, 2) ? 38u : 6u;
                uint64_t cleared = lifetime[f];
                if (p1 != 0) cleared &= ~(1ull << p1);
                if (p2 != 0) cleared &= ~(1ull << p2);
                uint32_t prd = rd[off];
                if (prd >= 64u) {
                    const bool fl = needs_float(w, 0);
                    const uint64_t fixed = cleared | (0xFFFFFFFFull << (fl ? 0 : 32));
                    const uint32_t low = ~static_cast<uint32_t>(fixed);  // the reference's ffs takes an int
                    if (low == 0) prd = fl ? 37u : 5u;
                    else prd = static_cast<uint32_t>(__builtin_ctz(low));
                }
                if (prd != 0 && ((cleared >> prd) & 1u)) st.swapped |= 1ull << prd;
                if (p1 != 0 && ((lifetime[f] >> p1) & 1u)) st.swapped |= 1ull << p1;
                if (p2 != 0 && ((lifetime[f] >> p2) & 1u)) st.swapped |= 1ull << p2;
                st.mask = cleared | (1ull << prd);
                const uint32_t named[3] = {rd[off], rs1[off], rs2[off]};
                const uint32_t phys[3] = {prd, p1, p2};
                for (int k = 0; k < 3; ++k) {
                    st.sym[k] = named[k] >= 64u ? static_cast<int64_t>(named[k]) - 64 : -1;
                    st.phys[k] = static_cast<uint8_t>(phys[k]);
                }
                st.rdv = rd[off];
                st.rd_phys = prd;
                st.r1_phys = p1;
                st.r2_phys = p2;
            }
            // swapped symbols keep their register and read as swapped; then the step's
            // symbols take their registers (later writes win, every swap first)
            for (size_t f = 0; f < F; ++f) {
                for (int p = 0; p < 64; ++p) {
                    if (!((steps[f].swapped >> p) & 1u)) continue;
                    const int64_t v = state[f * 64 + p];
                    if (v >= 64 && v - 64 < static_cast<int64_t>(W)) sym_swp[v - 64] = 1;
                }
            }
            for (size_t f = 0; f < F; ++f) {
                for (int k = 0; k < 3; ++k) {
                    const int64_t v = steps[f].sym[k];
                    if (v >= 0 && v < static_cast<int64_t>(W)) { sym_reg[v] = steps[f].phys[k]; sym_swp[v] = 0; }
                }
            }
            for (size_t f = 0; f < F; ++f) {
                const Step& st = steps[f];
                lifetime[f] = st.mask;
                preserve[f] |= lifetime[f];
                if (!st.act) continue;
                int64_t* rs = &state[f * 64];
                if (st.call) {
                    for (int p = 0; p < 64; ++p) if (!((st.mask >> p) & 1u)) rs[p] = -1;
                } else {
                    rs[st.rd_phys] = st.rdv;
                    if (st.r1_phys != st.rd_phys) rs[st.r1_phys] = -1;
                    if (st.r2_phys != st.rd_phys) rs[st.r2_phys] = -1;
                }
            }
        }
        for (size_t f = 0; f < F; ++f) preserve[f] &= kNonscratch;

        // spill slots: the swapped flag of each function's first word, held to the next
        // function start (:1290-1300)
        std::vector<uint8_t> is_start(W + 1, 0);
        for (size_t f = 0; f < F; ++f) if (func_starts[f] < W) is_start[func_starts[f]] = 1;
        std::vector<uint32_t> spill(W, 0);
        for (size_t v = 0; v < W; ++v) spill[v] = is_start[v] ? sym_swp[v] : (v > 0 ? spill[v - 1] : 0u);

        // counts, preserve words, offsets (:1302-1340)
        std::vector<int64_t> counts(W, 0);
        for (size_t i = 0; i < W; ++i) {
            if (!used_instrs[i]) continue;
            int64_t c = 1;
            for (uint32_t r : {rd[i], rs1[i], rs2[i]}) {
                check_sym(r);
                if (r >= 64u && sym_swp[r - 64u]) ++c;
            }
            counts[i] = c;
        }
        for (size_t f = 0; f < F; ++f) {
            const int64_t pc = __builtin_popcountll(preserve[f]);
            const int64_t a = static_cast<int64_t>(func_starts[f]) + 5;
            const int64_t b = static_cast<int64_t>(func_starts[f]) + function_sizes[f] - 6;
            if (a < 0 || b < 0 || a >= static_cast<int64_t>(W) || b >= static_cast<int64_t>(W))
                throw Unsupported("preserve words counted past the program");
            counts[a] += pc;
            counts[b] += pc;
        }
        PBuf<uint32_t> offs(W);
        {
            int64_t acc = 0;
            for (size_t i = 0; i < W; ++i) { offs[i] = static_cast<uint32_t>(acc); acc += counts[i]; }
        }
        const size_t W2 = W == 0 ? 0 : static_cast<size_t>(offs[static_cast<int64_t>(W) - 1]) + 1;
        PBuf<uint32_t> ni(W2), nrd(W2), nr1(W2), nr2(W2), njt(W2);
        auto put = [&](int64_t at, uint32_t w, uint32_t d, uint32_t a, uint32_t b, uint32_t j) {
            if (at < 0 || at >= static_cast<int64_t>(W2)) return;
            ni[at] = w; nrd[at] = d; nr1[at] = a; nr2[at] = b; njt[at] = j;
        };
        for (size_t i = 0; i < W; ++i) {  // :1354-1480
            if (!used_instrs[i]) continue;
            const int64_t base = offs[i];
            const uint32_t a1 = rs1[i], a2 = rs2[i], ad = rd[i];
            const bool sw1 = a1 >= 64u && sym_swp[a1 - 64u];
            const bool sw2 = a2 >= 64u && sym_swp[a2 - 64u];
            const bool swd = ad >= 64u && sym_swp[ad - 64u];
            const int64_t l1 = sw1 ? base : -1;
            const int64_t l2 = sw2 ? base + (l1 > 0 ? 1 : 0) : -1;
            const int64_t mo = base + (l1 > 0 ? 1 : 0) + (l2 > 0 ? 1 : 0);
            const int64_t so = swd ? mo + 1 : -1;
            const uint32_t prd = ad >= 64u ? sym_reg[ad - 64u] : ad;
            uint32_t p1 = a1, p2 = a2;
            if (a1 >= 64u) p1 = sw1 ? (needs_float(instr[i], 1) ? 37u : 5u) : sym_reg[a1 - 64u];
            if (a2 >= 64u) p2 = sw2 ? (needs_float(instr[i], 2) ? 38u : 6u) : sym_reg[a2 - 64u];
            const uint32_t st1 = sw1 ? spill[a1 - 64u] : 0u;
            const uint32_t st2 = sw2 ? spill[a2 - 64u] : 0u;
            const uint32_t std_ = swd ? spill[ad - 64u] : 0u;
            if (l1 >= 0) put(l1, 0x2003u | ((4u * (st1 - 1u)) << 20), 5, 0, 0, 0);
            if (l2 >= 0) put(l2, 0x2003u | ((4u * (st2 - 1u)) << 20), 6, 0, 0, 0);
            // the offsets hold W values in a zeroed allocation: just past them reads 0
            if (jt[i] >= W + 8) throw Unsupported("jump target past the program");
            put(mo, instr[i], prd, p1, p2, jt[i] < W ? offs[jt[i]] : 0u);
            if (so >= 0) {
                const uint32_t imm = 0u - 4u * (std_ - 1u);
                put(so, 0x2023u | ((imm & 0x1Fu) << 7) | ((imm & 0xFEu) << 19), 0, prd, 0, 0);
            }
        }
        instr = ni.clone(); rd = nrd.clone(); rs1 = nr1.clone(); rs2 = nr2.clone(); jt = njt.clone();
        fix_func_tab(offs, W);
        // frame words, preserve stores, preserve loads: one scatter in that order (:1509-1602)
        std::vector<std::pair<int64_t, uint32_t>> frame;
        for (size_t f = 0; f < F; ++f) {
            const uint32_t ss = (static_cast<uint32_t>(__builtin_popcountll(preserve[f])) + 2u) * 4u;
            const uint32_t lower = (ss & 0xFFFu) << 20;
            const uint32_t sx = static_cast<uint32_t>(static_cast<int32_t>((ss & 0xFFFu) << 20) >> 20);
            const uint32_t upper = (ss - sx) & 0xFFFFF000u;
            const int64_t st = func_starts[f], sz = function_sizes[f];
            frame.push_back({st + 2, 0x437u | upper});
            frame.push_back({st + 3, 0x40413u | lower});
            frame.push_back({st + sz - 6, 0x437u | upper});
            frame.push_back({st + sz - 5, 0x40413u | lower});
        }
        for (int pass = 0; pass < 2; ++pass) {
            for (size_t f = 0; f < F; ++f) {
                const uint64_t pm = preserve[f];
                const int64_t st = func_starts[f], sz = function_sizes[f];
                for (uint32_t j = 0; j < 64; ++j) {
                    if (!((pm >> j) & 1u)) continue;
                    const int64_t lead = __builtin_popcountll(pm & ((1ull << j) - 1));
                    const int64_t offset = -(8 + lead * 4);
                    if (pass == 0) {
                        const uint32_t w = (j >= 32 ? 0x42027u : 0x42023u) | static_cast<uint32_t>((offset & 0xFE0) << 25) |
                                           static_cast<uint32_t>((offset & 0x1F) << 7) | ((j % 32) << 20);
                        frame.push_back({st + lead + 6, w});
                    } else {
                        const uint32_t w = (j >= 32 ? 0x42007u : 0x42003u) | (static_cast<uint32_t>(offset) << 20) | ((j % 32) << 7);
                        frame.push_back({st + sz + lead - 7, w});
                    }
                }
            }
        }
        for (auto& fw : frame) {
            if (fw.first < 0 || fw.first >= static_cast<int64_t>(W2)) continue;
            instr[fw.first] = fw.second; rd[fw.first] = 0; rs1[fw.first] = 0; rs2[fw.first] = 0; jt[fw.first] = 0;
        }
    }
};

template <typename B>
ptlport_buf copy_out(const B& b) {
    ptlport_buf o{nullptr, b.size()};
    o.p = static_cast<uint32_t*>(std::malloc(std::max<size_t>(1, b.size()) * 4));
    for (size_t i = 0; i < b.size(); ++i) o.p[i] = static_cast<uint32_t>(b[i]);
    return o;
}

void set_err(char* err, size_t errlen, const char* msg) {
    if (err && errlen) std::snprintf(err, errlen, "%s", msg);
}

}  // namespace

namespace {

int compile_impl(const uint8_t* type, const uint8_t* rtype, const int32_t* parent, const int32_t* depth,
                 const int32_t* child_idx, const uint32_t* data, size_t n, size_t max_depth, int snapshots,
                 ptlport_result* out, char* err, size_t errlen, bool scalar) {
    std::memset(out, 0, sizeof(*out));
    if (n == 0) { set_err(err, errlen, "empty tree"); return PTLPORT_EINVAL; }
    if (max_depth == 0) { set_err(err, errlen, "max_depth is 0 (the reference divides by it)"); return PTLPORT_EINVAL; }
    for (size_t i = 0; i < n; ++i) {
        if (type[i] >= 44 || rtype[i] > 5) { set_err(err, errlen, "node type or data type out of range"); return PTLPORT_EINVAL; }
    }
    try {
        GenSt g;
        g.n = n;
        g.max_depth = max_depth;
        g.node_types.resize(n); g.result_types.resize(n); g.node_data.resize(n);
        g.node_sizes.resize(n); g.node_locations.resize(n);
        g.parents.resize(n); g.depth.resize(n); g.child_idx.resize(n);
        const Tables& T = tables();
        for (size_t i = 0; i < n; ++i) {  // rv_generator.cpp:41-67
            g.node_types[i] = T.pareas[type[i]];
            g.result_types[i] = rtype[i];
            g.parents[i] = parent[i];
            g.depth[i] = depth[i];
            g.child_idx[i] = child_idx[i];
            g.node_data[i] = data[i];
        }
        using clock = std::chrono::steady_clock;
        auto timed = [&](int idx, auto fn) {
            auto t0 = clock::now();
            fn();
            out->stage_ns[idx] = static_cast<uint64_t>(
                std::chrono::duration_cast<std::chrono::nanoseconds>(clock::now() - t0).count());
        };
        timed(0, [&] { if (scalar) g.preprocess_st(); else g.preprocess(); });
        if (snapshots) {
            out->bufs[PTLPORT_PRE_TYPE] = copy_out(g.node_types);
            out->bufs[PTLPORT_PRE_RTYPE] = copy_out(g.result_types);
            out->bufs[PTLPORT_PRE_DATA] = copy_out(g.node_data);
        }
        timed(1, [&] { if (scalar) g.isn_cnt_st(); else g.isn_cnt(); });
        if (snapshots) {
            out->bufs[PTLPORT_CNT_SIZE] = copy_out(g.node_sizes);
            out->bufs[PTLPORT_CNT_LOC] = copy_out(g.node_locations);
            out->bufs[PTLPORT_CNT_FN_ID] = copy_out(g.function_ids);
            out->bufs[PTLPORT_CNT_FN_START] = copy_out(g.func_starts);
            out->bufs[PTLPORT_CNT_FN_END] = copy_out(g.func_ends);
            out->bufs[PTLPORT_CNT_FN_SIZE] = copy_out(g.function_sizes);
        }
        timed(2, [&] { if (scalar) g.isn_gen_st(); else g.isn_gen(); });
        if (snapshots) {
            out->bufs[PTLPORT_GEN_INSTR] = copy_out(g.instr);
            out->bufs[PTLPORT_GEN_RD] = copy_out(g.rd);
            out->bufs[PTLPORT_GEN_RS1] = copy_out(g.rs1);
            out->bufs[PTLPORT_GEN_RS2] = copy_out(g.rs2);
            out->bufs[PTLPORT_GEN_JT] = copy_out(g.jt);
        }
        timed(3, [&] { if (scalar) g.optimize_st(); else g.optimize(); });
        if (snapshots) out->bufs[PTLPORT_OPT_USED] = copy_out(g.used_instrs);
        timed(4, [&] { if (scalar) g.regalloc_st(); else g.regalloc(); });
        if (snapshots) {
            out->bufs[PTLPORT_RA_INSTR] = copy_out(g.instr);
            out->bufs[PTLPORT_RA_RD] = copy_out(g.rd);
            out->bufs[PTLPORT_RA_RS1] = copy_out(g.rs1);
            out->bufs[PTLPORT_RA_RS2] = copy_out(g.rs2);
            out->bufs[PTLPORT_RA_JT] = copy_out(g.jt);
            out->bufs[PTLPORT_RA_FN_START] = copy_out(g.func_starts);
            out->bufs[PTLPORT_RA_FN_END] = copy_out(g.func_ends);
            out->bufs[PTLPORT_RA_FN_SIZE] = copy_out(g.function_sizes);
        }
        timed(5, [&] { if (scalar) g.fix_jumps_st(); else g.fix_jumps(); });
        if (snapshots) {
            out->bufs[PTLPORT_FJ_INSTR] = copy_out(g.instr);
            out->bufs[PTLPORT_FJ_RD] = copy_out(g.rd);
            out->bufs[PTLPORT_FJ_RS1] = copy_out(g.rs1);
            out->bufs[PTLPORT_FJ_RS2] = copy_out(g.rs2);
            out->bufs[PTLPORT_FJ_JT] = copy_out(g.jt);
            out->bufs[PTLPORT_FJ_FN_START] = copy_out(g.func_starts);
            out->bufs[PTLPORT_FJ_FN_END] = copy_out(g.func_ends);
            out->bufs[PTLPORT_FJ_FN_SIZE] = copy_out(g.function_sizes);
        }
        timed(6, [&] { g.postprocess(); });
        out->bufs[PTLPORT_OUT_WORDS] = copy_out(g.instr);
        out->bufs[PTLPORT_FN_START] = copy_out(g.func_starts);
        out->bufs[PTLPORT_FN_END] = copy_out(g.func_ends);
        out->bufs[PTLPORT_FN_SIZE] = copy_out(g.function_sizes);
        out->bufs[PTLPORT_FN_ID] = copy_out(g.function_ids);
        return PTLPORT_OK;
    } catch (const Unsupported& e) {
        set_err(err, errlen, e.what());
        ptlport_free_result(out);
        return PTLPORT_EUNSUPPORTED;
    } catch (const std::exception& e) {
        set_err(err, errlen, e.what());
        ptlport_free_result(out);
        return PTLPORT_EUNSUPPORTED;
    }
}

}  // namespace

extern "C" int ptlport_compile(const uint8_t* type, const uint8_t* rtype, const int32_t* parent,
                               const int32_t* depth, const int32_t* child_idx, const uint32_t* data,
                               size_t n, size_t max_depth, int snapshots, ptlport_result* out,
                               char* err, size_t errlen) {
    return compile_impl(type, rtype, parent, depth, child_idx, data, n, max_depth, snapshots, out, err, errlen,
                        false);
}

extern "C" int ptlport_compile_scalar(const uint8_t* type, const uint8_t* rtype, const int32_t* parent,
                                      const int32_t* depth, const int32_t* child_idx, const uint32_t* data,
                                      size_t n, size_t max_depth, int snapshots, ptlport_result* out,
                                      char* err, size_t errlen) {
    return compile_impl(type, rtype, parent, depth, child_idx, data, n, max_depth, snapshots, out, err, errlen,
                        true);
}

extern "C" void ptlport_free_result(ptlport_result* r) {
    for (auto& b : r->bufs) {
        std::free(b.p);
        b.p = nullptr;
        b.n = 0;
    }
}

extern "C" void ptlport_depth_sort(const int32_t* keys, size_t n, uint32_t* perm) {
    std::iota(perm, perm + n, 0u);
    std::sort(perm, perm + n, [keys](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
}

extern "C" size_t ptlport_table(int which, uint32_t* out) {
    const Tables& T = tables();
    const uint32_t* src = nullptr;
    size_t count = 0;
    switch (which) {
        case 0: src = &T.size[0][0]; count = sizeof(T.size) / 4; break;
        case 1: src = &T.has_instr[0][0][0]; count = sizeof(T.has_instr) / 4; break;
        case 2: src = &T.has_output[0][0][0]; count = sizeof(T.has_output) / 4; break;
        case 3: src = &T.pai[0][0][0]; count = sizeof(T.pai) / 4; break;
        case 4: src = &T.out[0][0][0]; count = sizeof(T.out) / 4; break;
        case 5: src = &T.instr[0][0][0]; count = sizeof(T.instr) / 4; break;
        case 6: src = &T.cnst[0][0]; count = sizeof(T.cnst) / 4; break;
        case 7: src = &T.operand[0][0][0][0]; count = sizeof(T.operand) / 4; break;
        case 8: src = &T.jt[0][0]; count = sizeof(T.jt) / 4; break;
        case 9: src = T.pareas; count = 44; break;
        default: return 0;
    }
    if (out) std::memcpy(out, src, count * 4);
    return count;
}

// ---------------------------------------------------------------- AST flattening
// DepthTree::construct (pareas-ast/src/codegen/depthtree.cpp:52-100): a depth-first walk
// from the root that pushes a node's children last-to-first and emits a node once all
// its children are emitted, so children come in order before their parent (post-order);
// depth is the walk depth, the root's child index is SIZE_MAX (-1 as int32), parents are
// rewritten to emitted indices.  Here the children come from child_idx instead of an
// ASTNode's child vector.
extern "C" int ptlport_flatten(size_t n, const uint8_t* type, const uint8_t* rtype, const int32_t* parent,
                               const int32_t* child_idx, const uint32_t* data, uint8_t* o_type, uint8_t* o_rtype,
                               int32_t* o_parent, int32_t* o_depth, int32_t* o_child, uint32_t* o_data,
                               int32_t* order, size_t* max_depth) {
    if (n == 0 || n >= (1ull << 31)) return PTLPORT_EINVAL;
    std::vector<uint32_t> deg(n, 0), off(n + 1, 0);
    int64_t root = -1;
    for (size_t v = 0; v < n; ++v) {
        const int32_t p = parent[v];
        if (p == -1) {
            if (root >= 0) return PTLPORT_EINVAL;  // two roots
            root = static_cast<int64_t>(v);
        } else if (p < 0 || static_cast<size_t>(p) >= n || child_idx[v] < 0) {
            return PTLPORT_EINVAL;
        } else {
            ++deg[static_cast<size_t>(p)];
        }
    }
    if (root < 0) return PTLPORT_EINVAL;
    for (size_t v = 0; v < n; ++v) off[v + 1] = off[v] + deg[v];
    std::vector<int64_t> kids(n, -1);
    for (size_t v = 0; v < n; ++v) {
        const int32_t p = parent[v];
        if (p == -1) continue;
        const uint32_t c = static_cast<uint32_t>(child_idx[v]);
        if (c >= deg[static_cast<size_t>(p)]) return PTLPORT_EINVAL;
        int64_t& slot = kids[off[static_cast<size_t>(p)] + c];
        if (slot >= 0) return PTLPORT_EINVAL;  // two children with one index
        slot = static_cast<int64_t>(v);
    }
    struct Frame { size_t v, depth, next; };
    std::vector<Frame> stack;
    stack.push_back({static_cast<size_t>(root), 0, 0});
    std::vector<int32_t> post(n, -1);
    size_t emitted = 0, md = 0;
    while (!stack.empty()) {
        Frame& f = stack.back();
        if (f.next < deg[f.v]) {
            const size_t c = static_cast<size_t>(kids[off[f.v] + f.next++]);
            const size_t d = f.depth + 1;
            stack.push_back({c, d, 0});
            continue;
        }
        const size_t v = f.v, d = f.depth;
        stack.pop_back();
        post[v] = static_cast<int32_t>(emitted);
        o_type[emitted] = type[v];
        o_rtype[emitted] = rtype[v];
        o_depth[emitted] = static_cast<int32_t>(d);
        o_child[emitted] = static_cast<int64_t>(v) == root ? -1 : child_idx[v];
        o_data[emitted] = data[v];
        if (d > md) md = d;
        ++emitted;
    }
    if (emitted != n) return PTLPORT_EINVAL;  // nodes the root does not reach
    for (size_t v = 0; v < n; ++v) {
        const int32_t p = parent[v];
        o_parent[post[v]] = p == -1 ? -1 : post[static_cast<size_t>(p)];
        if (order) order[v] = post[v];
    }
    *max_depth = md;
    return PTLPORT_OK;
}
