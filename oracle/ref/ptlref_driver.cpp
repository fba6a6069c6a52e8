// Oracle harness: drives the reference code generator, compiled from its own sources,
// through a C ABI so Python tests and fixture scripts can call it.  Test
// infrastructure only (see ptlref.h).
//
// The harness needs the generator's private arrays for per-stage snapshots, so the
// reference headers are included with `private`/`protected` widened to `public` in
// this translation unit only; no reference file is modified.  Every standard header
// the reference pulls in is included first so the widening never touches the
// standard library.
#include <algorithm>
#include <array>
#include <atomic>
#include <barrier>
#include <bit>
#include <bitset>
#include <chrono>
#include <cmath>
#include <concepts>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <execution>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iosfwd>
#include <iostream>
#include <limits>
#include <memory>
#include <numeric>
#include <optional>
#include <ostream>
#include <queue>
#include <ranges>
#include <span>
#include <sstream>
#include <stack>
#include <string>
#include <string_view>
#include <thread>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <vector>
#include <immintrin.h>

#include <magic_enum.hpp>
#include <tbb/task_arena.h>

#include "codegen/lexer.hpp"
#include "codegen/parser.hpp"
#include "codegen/symtab.hpp"
#include "codegen/exception.hpp"
#include "codegen/astnode.hpp"

#define private public
#define protected public
#include "codegen/depthtree.hpp"
#include "codegen/rv_generator_avx.hpp"
#include "disassembler.hpp"
#undef private
#undef protected

#include "ptlref.h"

namespace {

void set_err(char* err, size_t errlen, const std::string& msg) {
    if (err != nullptr && errlen > 0) {
        std::snprintf(err, errlen, "%s", msg.c_str());
    }
}

template <typename T>
ptlref_buf copy_buf(const avx_buffer<T>& b) {
    ptlref_buf out{nullptr, b.size()};
    out.p = static_cast<uint32_t*>(std::malloc(std::max<size_t>(1, b.size()) * sizeof(uint32_t)));
    for (size_t i = 0; i < b.size(); ++i) {
        out.p[i] = static_cast<uint32_t>(b[i]);
    }
    return out;
}

// A DepthTree whose arrays are the caller's; built field by field because the
// reference only offers a constructor from a pointer-linked ASTNode tree.
struct borrowed_tree {
    alignas(DepthTree) unsigned char storage[sizeof(DepthTree)];
    DepthTree* get() { return reinterpret_cast<DepthTree*>(storage); }
};

void copy_tree(const DepthTree& tree, ptlref_tree* out) {
    size_t n = tree.filledNodes();
    out->n = n;
    out->max_depth = tree.maxDepth();
    out->type = static_cast<uint8_t*>(std::malloc(std::max<size_t>(1, n)));
    out->rtype = static_cast<uint8_t*>(std::malloc(std::max<size_t>(1, n)));
    out->parent = static_cast<int32_t*>(std::malloc(std::max<size_t>(1, n) * 4));
    out->depth = static_cast<int32_t*>(std::malloc(std::max<size_t>(1, n) * 4));
    out->child_idx = static_cast<int32_t*>(std::malloc(std::max<size_t>(1, n) * 4));
    out->data = static_cast<uint32_t*>(std::malloc(std::max<size_t>(1, n) * 4));
    std::memcpy(out->type, tree.getNodeTypes().data(), n);
    std::memcpy(out->rtype, tree.getResultingTypes().data(), n);
    std::memcpy(out->parent, tree.getParents().data(), n * 4);
    std::memcpy(out->depth, tree.getDepth().data(), n * 4);
    std::memcpy(out->child_idx, tree.getChildren().data(), n * 4);
    std::memcpy(out->data, tree.getNodeData().data(), n * 4);
}

}  // namespace

extern "C" int ptlref_flatten(size_t n, const uint8_t* type, const uint8_t* rtype, const int32_t* parent,
                              const int32_t* child_idx, const uint32_t* data, ptlref_tree* out) {
    // The pointer tree the reference flattens: one ASTNode per node, children in
    // child_idx order, built leaves first (an ASTNode takes its children when made).
    if (n == 0) return 1;
    std::vector<std::vector<size_t>> kids(n);
    size_t root = n;
    for (size_t v = 0; v < n; ++v) {
        if (parent[v] == -1) root = v;
        else kids[static_cast<size_t>(parent[v])].push_back(v);
    }
    if (root == n) return 1;
    for (auto& k : kids)
        std::sort(k.begin(), k.end(), [&](size_t a, size_t b) { return child_idx[a] < child_idx[b]; });
    std::vector<ASTNode*> made(n, nullptr);
    std::vector<std::pair<size_t, size_t>> stack{{root, 0}};
    while (!stack.empty()) {
        auto& [v, next] = stack.back();
        if (next < kids[v].size()) {
            const size_t c = kids[v][next++];
            stack.push_back({c, 0});
            continue;
        }
        std::vector<ASTNode*> ch;
        for (size_t c : kids[v]) ch.push_back(made[c]);
        made[v] = new ASTNode(static_cast<NodeType>(type[v]), static_cast<DataType>(rtype[v]), data[v], ch);
        stack.pop_back();
    }
    std::unique_ptr<ASTNode> node(made[root]);
    DepthTree tree(node.get());
    copy_tree(tree, out);
    return 0;
}

extern "C" int ptlref_parse_file(const char* path, ptlref_tree* out, char* err, size_t errlen) {
    try {
        std::ifstream input(path);
        if (!input.good()) {
            set_err(err, errlen, std::string("cannot open ") + path);
            return 1;
        }
        Lexer lexer(input);
        SymbolTable symtab;
        Parser parser(lexer, symtab);
        std::unique_ptr<ASTNode> node(parser.parse());
        node->resolveType();
        DepthTree tree(node.get());
        copy_tree(tree, out);
        return 0;
    } catch (const std::exception& e) {
        set_err(err, errlen, e.what());
        return 2;
    }
}

extern "C" void ptlref_free_tree(ptlref_tree* t) {
    std::free(t->type);
    std::free(t->rtype);
    std::free(t->parent);
    std::free(t->depth);
    std::free(t->child_idx);
    std::free(t->data);
    std::memset(t, 0, sizeof(*t));
}

// The reference's destructor (src/codegen/rv_generator_avx.cpp:70-80) releases its
// worker threads and detaches them; they then read the destroyed generator's fields as
// they wake, a use after free that crashed the calling process at random.  The harness
// never destroys a generator: each is kept in a list that is never freed (not even at
// exit), and its workers stay parked on its barrier.
static void keep_alive(std::unique_ptr<rv_generator_avx> gen) {
    static std::mutex mu;
    static auto* kept = new std::vector<std::unique_ptr<rv_generator_avx>>();
    std::lock_guard<std::mutex> lk(mu);
    kept->push_back(std::move(gen));
}

extern "C" int ptlref_compile(const ptlref_tree* in, int threads, int sync, int altblock,
                              uint32_t mininstr, int snapshots, ptlref_result* out,
                              char* err, size_t errlen) {
    std::memset(out, 0, sizeof(*out));
    borrowed_tree bt;
    DepthTree* tree = bt.get();
    tree->node_types = in->type;
    tree->resulting_types = in->rtype;
    tree->parents = in->parent;
    tree->depth = in->depth;
    tree->child_idx = in->child_idx;
    tree->node_data = in->data;
    tree->max_nodes = in->n;
    tree->filled_nodes = in->n;
    tree->max_depth = in->max_depth;

    try {
        // The generator reports its thread count on stderr; keep the harness quiet.
        std::streambuf* saved = std::cerr.rdbuf(nullptr);
        auto gen = std::make_unique<rv_generator_avx>(*tree, threads, sync, altblock != 0, mininstr);
        std::cerr.rdbuf(saved);
        rv_generator_avx* g = gen.get();
        keep_alive(std::move(gen));  // before any stage can throw
        out->threads_used = static_cast<int>(g->threads);

        using clock = std::chrono::steady_clock;
        auto timed = [&](int idx, auto fn) {
            auto t0 = clock::now();
            fn();
            auto t1 = clock::now();
            out->stage_ns[idx] = static_cast<uint64_t>(
                std::chrono::duration_cast<std::chrono::nanoseconds>(t1 - t0).count());
        };

        timed(0, [&] { g->preprocess(); });
        if (snapshots) {
            out->bufs[PTLREF_PRE_TYPE] = copy_buf(g->node_types);
            out->bufs[PTLREF_PRE_RTYPE] = copy_buf(g->result_types);
            out->bufs[PTLREF_PRE_DATA] = copy_buf(g->node_data);
        }
        timed(1, [&] { g->isn_cnt(); });
        if (snapshots) {
            out->bufs[PTLREF_CNT_SIZE] = copy_buf(g->node_sizes);
            out->bufs[PTLREF_CNT_LOC] = copy_buf(g->node_locations);
            out->bufs[PTLREF_CNT_FN_ID] = copy_buf(g->function_ids);
            out->bufs[PTLREF_CNT_FN_START] = copy_buf(g->func_starts);
            out->bufs[PTLREF_CNT_FN_END] = copy_buf(g->func_ends);
            out->bufs[PTLREF_CNT_FN_SIZE] = copy_buf(g->function_sizes);
        }
        timed(2, [&] { g->isn_gen(); });
        if (snapshots) {
            out->bufs[PTLREF_GEN_INSTR] = copy_buf(g->instr);
            out->bufs[PTLREF_GEN_RD] = copy_buf(g->rd_avx);
            out->bufs[PTLREF_GEN_RS1] = copy_buf(g->rs1_avx);
            out->bufs[PTLREF_GEN_RS2] = copy_buf(g->rs2_avx);
            out->bufs[PTLREF_GEN_JT] = copy_buf(g->jt_avx);
        }
        timed(3, [&] { g->optimize(); });
        if (snapshots) {
            out->bufs[PTLREF_OPT_USED] = copy_buf(g->used_instrs_avx);
        }
        timed(4, [&] { g->regalloc(); });
        if (snapshots) {
            out->bufs[PTLREF_RA_INSTR] = copy_buf(g->instr);
            out->bufs[PTLREF_RA_RD] = copy_buf(g->rd_avx);
            out->bufs[PTLREF_RA_RS1] = copy_buf(g->rs1_avx);
            out->bufs[PTLREF_RA_RS2] = copy_buf(g->rs2_avx);
            out->bufs[PTLREF_RA_JT] = copy_buf(g->jt_avx);
            out->bufs[PTLREF_RA_FN_START] = copy_buf(g->func_starts);
            out->bufs[PTLREF_RA_FN_END] = copy_buf(g->func_ends);
            out->bufs[PTLREF_RA_FN_SIZE] = copy_buf(g->function_sizes);
        }
        timed(5, [&] { g->fix_jumps(); });
        if (snapshots) {
            out->bufs[PTLREF_FJ_INSTR] = copy_buf(g->instr);
            out->bufs[PTLREF_FJ_RD] = copy_buf(g->rd_avx);
            out->bufs[PTLREF_FJ_RS1] = copy_buf(g->rs1_avx);
            out->bufs[PTLREF_FJ_RS2] = copy_buf(g->rs2_avx);
            out->bufs[PTLREF_FJ_JT] = copy_buf(g->jt_avx);
            out->bufs[PTLREF_FJ_FN_START] = copy_buf(g->func_starts);
            out->bufs[PTLREF_FJ_FN_END] = copy_buf(g->func_ends);
            out->bufs[PTLREF_FJ_FN_SIZE] = copy_buf(g->function_sizes);
        }
        timed(6, [&] { g->postprocess(); });

        out->bufs[PTLREF_OUT_WORDS] = copy_buf(g->instr);
        out->bufs[PTLREF_FN_START] = copy_buf(g->func_starts);
        out->bufs[PTLREF_FN_END] = copy_buf(g->func_ends);
        out->bufs[PTLREF_FN_SIZE] = copy_buf(g->function_sizes);
        out->bufs[PTLREF_FN_ID] = copy_buf(g->function_ids);

        return 0;
    } catch (const std::exception& e) {
        set_err(err, errlen, e.what());
        return 2;
    }
}

// The reference's scalar generator rv_generator_st (src/codegen/rv_generator.cpp:129-1736,
// the -s flag of src/main.cpp), stage by stage with the same snapshot slots.  It owns no
// threads, so it is destroyed normally.
extern "C" int ptlref_compile_scalar(const ptlref_tree* in, int snapshots, ptlref_result* out, char* err,
                                     size_t errlen) {
    std::memset(out, 0, sizeof(*out));
    borrowed_tree bt;
    DepthTree* tree = bt.get();
    tree->node_types = in->type;
    tree->resulting_types = in->rtype;
    tree->parents = in->parent;
    tree->depth = in->depth;
    tree->child_idx = in->child_idx;
    tree->node_data = in->data;
    tree->max_nodes = in->n;
    tree->filled_nodes = in->n;
    tree->max_depth = in->max_depth;
    try {
        rv_generator_st gen(*tree);
        rv_generator_st* g = &gen;
        out->threads_used = 1;
        using clock = std::chrono::steady_clock;
        auto timed = [&](int idx, auto fn) {
            auto t0 = clock::now();
            fn();
            auto t1 = clock::now();
            out->stage_ns[idx] = static_cast<uint64_t>(
                std::chrono::duration_cast<std::chrono::nanoseconds>(t1 - t0).count());
        };
        auto words = [&](int i, int r, int a, int b, int j) {
            out->bufs[i] = copy_buf(g->instructions);
            out->bufs[r] = copy_buf(g->rd);
            out->bufs[a] = copy_buf(g->rs1);
            out->bufs[b] = copy_buf(g->rs2);
            out->bufs[j] = copy_buf(g->jt);
        };
        timed(0, [&] { g->preprocess(); });
        if (snapshots) {
            out->bufs[PTLREF_PRE_TYPE] = copy_buf(g->node_types);
            out->bufs[PTLREF_PRE_RTYPE] = copy_buf(g->result_types);
            out->bufs[PTLREF_PRE_DATA] = copy_buf(g->node_data);
        }
        timed(1, [&] { g->isn_cnt(); });
        if (snapshots) {
            out->bufs[PTLREF_CNT_SIZE] = copy_buf(g->node_sizes);
            out->bufs[PTLREF_CNT_LOC] = copy_buf(g->node_locations);
            out->bufs[PTLREF_CNT_FN_ID] = copy_buf(g->function_ids);
            out->bufs[PTLREF_CNT_FN_START] = copy_buf(g->func_starts);
            out->bufs[PTLREF_CNT_FN_END] = copy_buf(g->func_ends);
            out->bufs[PTLREF_CNT_FN_SIZE] = copy_buf(g->function_sizes);
        }
        timed(2, [&] { g->isn_gen(); });
        if (snapshots) words(PTLREF_GEN_INSTR, PTLREF_GEN_RD, PTLREF_GEN_RS1, PTLREF_GEN_RS2, PTLREF_GEN_JT);
        timed(3, [&] { g->optimize(); });
        if (snapshots) out->bufs[PTLREF_OPT_USED] = copy_buf(g->used_instrs);
        timed(4, [&] { g->regalloc(); });
        if (snapshots) {
            words(PTLREF_RA_INSTR, PTLREF_RA_RD, PTLREF_RA_RS1, PTLREF_RA_RS2, PTLREF_RA_JT);
            out->bufs[PTLREF_RA_FN_START] = copy_buf(g->func_starts);
            out->bufs[PTLREF_RA_FN_END] = copy_buf(g->func_ends);
            out->bufs[PTLREF_RA_FN_SIZE] = copy_buf(g->function_sizes);
        }
        timed(5, [&] { g->fix_jumps(); });
        if (snapshots) {
            words(PTLREF_FJ_INSTR, PTLREF_FJ_RD, PTLREF_FJ_RS1, PTLREF_FJ_RS2, PTLREF_FJ_JT);
            out->bufs[PTLREF_FJ_FN_START] = copy_buf(g->func_starts);
            out->bufs[PTLREF_FJ_FN_END] = copy_buf(g->func_ends);
            out->bufs[PTLREF_FJ_FN_SIZE] = copy_buf(g->function_sizes);
        }
        timed(6, [&] { g->postprocess(); });
        out->bufs[PTLREF_OUT_WORDS] = copy_buf(g->instructions);
        out->bufs[PTLREF_FN_START] = copy_buf(g->func_starts);
        out->bufs[PTLREF_FN_END] = copy_buf(g->func_ends);
        out->bufs[PTLREF_FN_SIZE] = copy_buf(g->function_sizes);
        out->bufs[PTLREF_FN_ID] = copy_buf(g->function_ids);
        return 0;
    } catch (const std::exception& e) {
        set_err(err, errlen, e.what());
        return 2;
    }
}

extern "C" void ptlref_free_result(ptlref_result* r) {
    for (auto& b : r->bufs) {
        std::free(b.p);
        b.p = nullptr;
        b.n = 0;
    }
}

// Flat dumps of the reference's constexpr code-generation tables
// (include/codegen/rv_nodetype.hpp:197-1134), indexed like ptlport_table.
extern "C" size_t ptlref_table(int which, uint32_t* out) {
    const uint32_t* src = nullptr;
    size_t count = 0;
    switch (which) {
        case 0: src = &node_size_mapping[0][0]; count = sizeof(node_size_mapping) / 4; break;
        case 1: src = &has_instr_mapping[0][0][0]; count = sizeof(has_instr_mapping) / 4; break;
        case 2: src = &has_output[0][0][0]; count = sizeof(has_output) / 4; break;
        case 3: src = &parent_arg_idx_lookup[0][0][0]; count = sizeof(parent_arg_idx_lookup) / 4; break;
        case 4: src = &get_output_table[0][0][0]; count = sizeof(get_output_table) / 4; break;
        case 5: src = &instr_table[0][0][0]; count = sizeof(instr_table) / 4; break;
        case 6: src = &instr_constant_table[0][0]; count = sizeof(instr_constant_table) / 4; break;
        case 7: src = &operand_table[0][0][0][0]; count = sizeof(operand_table) / 4; break;
        case 8: src = &instr_jt_table[0][0]; count = sizeof(instr_jt_table) / 4; break;
        case 9: {
            count = sizeof(pareas_to_rv_nodetype) / sizeof(pareas_to_rv_nodetype[0]);
            if (out) {
                for (size_t i = 0; i < count; ++i) out[i] = static_cast<uint32_t>(pareas_to_rv_nodetype[i]);
            }
            return count;
        }
        default: return 0;
    }
    if (out) std::memcpy(out, src, count * 4);
    return count;
}

namespace {
size_t put_text(const std::string& t, char* out, size_t cap) {
    if (out) std::memcpy(out, t.data(), std::min(cap, t.size()));
    return t.size();
}
}  // namespace

extern "C" size_t ptlref_to_asm(const uint32_t* words, size_t n, char* out, size_t cap) {
    std::ostringstream os;
    for (size_t k = 0; k < n; ++k) os << rvdisasm::instruction(words[k]) << '\n';  // rv_generator::to_asm
    return put_text(os.str(), out, cap);
}

extern "C" size_t ptlref_disassemble(const uint32_t* words, size_t n, uint64_t start_addr, const uint64_t* func_starts,
                                     size_t nfunc, char* out, size_t cap) {
    std::vector<uint32_t> w(words, words + n);
    std::vector<uint64_t> f(func_starts, func_starts + nfunc);
    std::ostringstream os;
    rvdisasm::disassemble(os, w, start_addr, f);
    return put_text(os.str(), out, cap);
}
