/* rv_generator_gb300: the GB300 code generator inside the reference's own class
 * hierarchy.  A maintainer drops this header next to include/codegen/rv_generator.hpp of
 * Ptilopsis and links libptl_gb300.so; src/main.cpp:121-127 then constructs it like the
 * AVX generator:
 *
 *     gen = std::make_unique<rv_generator_gb300>(depth_tree);
 *
 * It replaces rv_generator_avx (include/codegen/rv_generator_avx.hpp:58,
 * src/codegen/rv_generator_avx.cpp:82-84, 104-120) behind the base class
 * rv_generator (include/codegen/rv_generator.hpp:19-75).  process() runs the seven
 * stages on the GPU through the C ABI of ptl_codegen.h, then fills the base class's
 * protected function table (func_starts, func_ends, function_sizes, function_ids), so
 * that the inherited print(), to_asm() and to_binary() work unchanged.  With profile
 * set it prints the stage CSV of the reference's -p flag (rv_generator.cpp:150-162:
 * the seven stage names, then their times in ns, on stdout), from device times.
 * Errors are thrown as std::runtime_error, as the reference does for its own.
 *
 * With scalar set it replaces the reference's scalar generator rv_generator_st instead
 * (include/codegen/rv_generator.hpp:82-100, picked by -s at src/main.cpp:123-124):
 *
 *     gen = std::make_unique<rv_generator_gb300>(depth_tree, 0, simple); */
#pragma once

#include <algorithm>
#include <cstdint>
#include <iostream>
#include <span>
#include <stdexcept>
#include <string>

#include <codegen/depthtree.hpp>
#include <codegen/rv_generator.hpp>

#include "ptl_codegen.h"

class rv_generator_gb300 : public rv_generator {
    ptl_generator* gen_ = nullptr;
    std::span<uint32_t> words_;

    static void check(ptl_status st, const ptl_generator* g, const char* what) {
        if (st == PTL_OK) return;
        const char* detail = g ? ptl_generator_last_error(g) : nullptr;
        throw std::runtime_error(std::string(what) + ": " +
                                 (detail && *detail ? std::string(detail) : "status " + std::to_string(st)));
    }

    static void fill(avx_buffer<uint32_t>& dst, const uint32_t* src, size_t n) {
        dst = avx_buffer<uint32_t>(n);
        std::copy_n(src, n, dst.begin());
    }

  public:
    /* device: the CUDA device to compile on; scalar: the scalar generator's semantics.
     * The tree is read here (DepthTree getters,
     * subprojects/pareas-ast/include/codegen/depthtree.hpp:32-58) and copied to the
     * device; the base class keeps its own host copy as the reference's constructor does. */
    explicit rv_generator_gb300(const DepthTree& tree, int device = 0, bool scalar = false) : rv_generator(tree) {
        const ptl_ast_view v{tree.filledNodes(),          tree.maxDepth(),
                             tree.getNodeTypes().data(),  tree.getResultingTypes().data(),
                             tree.getParents().data(),    tree.getDepth().data(),
                             tree.getChildren().data(),   tree.getNodeData().data(),
                             /*on_device=*/0};
        if (scalar) check(ptl_generator_create_scalar(&v, device, &gen_), nullptr, "ptl_generator_create_scalar");
        else check(ptl_generator_create(&v, device, &gen_), nullptr, "ptl_generator_create");
    }

    ~rv_generator_gb300() override { ptl_generator_destroy(gen_); }

    void process(bool profile) override {
        check(ptl_generator_process(gen_, profile ? 1 : 0), gen_, "ptl_generator_process");
        const uint32_t* w = nullptr;
        size_t n = 0;
        check(ptl_generator_instructions(gen_, &w, &n), gen_, "ptl_generator_instructions");
        words_ = {const_cast<uint32_t*>(w), n};  // owned by gen_, valid until it is destroyed
        const uint32_t *starts = nullptr, *ends = nullptr, *sizes = nullptr, *ids = nullptr;
        size_t f = 0;
        check(ptl_generator_function_table(gen_, &starts, &ends, &sizes, &ids, &f), gen_,
              "ptl_generator_function_table");
        fill(func_starts, starts, f);
        fill(func_ends, ends, f);
        fill(function_sizes, sizes, f);
        fill(function_ids, ids, f);
        if (profile) {
            uint64_t ns[7] = {};
            check(ptl_generator_stage_ns(gen_, ns), gen_, "ptl_generator_stage_ns");
            static const char* const names[7] = {"preprocess", "isn_cnt",  "isn_gen",    "optimize",
                                                 "regalloc",   "fix_jumps", "postprocess"};
            for (int k = 0; k < 7; ++k) std::cout << names[k] << (k < 6 ? ',' : '\n');
            for (int k = 0; k < 7; ++k) std::cout << ns[k] << (k < 6 ? ',' : '\n');
            std::cout.flush();
        }
    }

    [[nodiscard]] std::span<uint32_t> get_instructions() const override { return words_; }
};
