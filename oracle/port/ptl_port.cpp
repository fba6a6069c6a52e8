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

extern "C" int ptlport_compile(const uint8_t* type, const uint8_t* rtype, const int32_t* parent,
                               const int32_t* depth, const int32_t* child_idx, const uint32_t* data,
                               size_t n, size_t max_depth, int snapshots, ptlport_result* out,
                               char* err, size_t errlen) {
    std::memset(out, 0, sizeof(*out));
    if (n == 0) { set_err(err, errlen, "empty tree"); return PTLPORT_EINVAL; }
    if (max_depth == 0) { set_err(err, errlen, "max_depth is 0 (the reference divides by it)"); return PTLPORT_EINVAL; }
    for (size_t i = 0; i < n; ++i) {
        if (type[i] >= 44 || rtype[i] > 5) { set_err(err, errlen, "node type or data type out of range"); return PTLPORT_EINVAL; }
    }
    try {
        Gen g;
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
        timed(0, [&] { g.preprocess(); });
        if (snapshots) {
            out->bufs[PTLPORT_PRE_TYPE] = copy_out(g.node_types);
            out->bufs[PTLPORT_PRE_RTYPE] = copy_out(g.result_types);
            out->bufs[PTLPORT_PRE_DATA] = copy_out(g.node_data);
        }
        timed(1, [&] { g.isn_cnt(); });
        if (snapshots) {
            out->bufs[PTLPORT_CNT_SIZE] = copy_out(g.node_sizes);
            out->bufs[PTLPORT_CNT_LOC] = copy_out(g.node_locations);
            out->bufs[PTLPORT_CNT_FN_ID] = copy_out(g.function_ids);
            out->bufs[PTLPORT_CNT_FN_START] = copy_out(g.func_starts);
            out->bufs[PTLPORT_CNT_FN_END] = copy_out(g.func_ends);
            out->bufs[PTLPORT_CNT_FN_SIZE] = copy_out(g.function_sizes);
        }
        timed(2, [&] { g.isn_gen(); });
        if (snapshots) {
            out->bufs[PTLPORT_GEN_INSTR] = copy_out(g.instr);
            out->bufs[PTLPORT_GEN_RD] = copy_out(g.rd);
            out->bufs[PTLPORT_GEN_RS1] = copy_out(g.rs1);
            out->bufs[PTLPORT_GEN_RS2] = copy_out(g.rs2);
            out->bufs[PTLPORT_GEN_JT] = copy_out(g.jt);
        }
        timed(3, [&] { g.optimize(); });
        if (snapshots) out->bufs[PTLPORT_OPT_USED] = copy_out(g.used_instrs);
        timed(4, [&] { g.regalloc(); });
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
        timed(5, [&] { g.fix_jumps(); });
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
