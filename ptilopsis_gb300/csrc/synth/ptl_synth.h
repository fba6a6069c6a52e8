/*
 * Seeded synthetic Pareas programs, emitted directly as the flattened post-order AST
 * arrays that pareas-ast's DepthTree produces (subprojects/pareas-ast/src/codegen/
 * depthtree.cpp:52-100): u8 node type, u8 result type, i32 parent, i32 depth,
 * i32 child index, u32 node data.  The construction follows the reference front
 * end's parser (parser.cpp) and type resolution (astnode.cpp:108-244): implicit
 * dereferences around variables read as values, FUNC_ARG wrapping a declaration,
 * per-type argument indices, FUNC_DECL = {FUNC_DECL_DUMMY, FUNC_ARG_LIST, body},
 * WHILE = {WHILE_DUMMY, cond, body}, RETURN data = function id, CALL data = callee.
 *
 * For small programs the generator can also print equivalent source text; parsing
 * that text with the reference front end reproduces the arrays exactly, which is how
 * the generator is pinned (tests/test_synth.py).
 *
 * The generator is deterministic across hosts: its random numbers come from a
 * counter-based integer generator and its lognormal sizes from IEEE-exact
 * arithmetic only (no libm), so a seed names the same program on x86-64 and aarch64.
 */
#ifndef PTL_SYNTH_H
#define PTL_SYNTH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    uint64_t seed;
    uint32_t n_functions;      /* functions in the program (>= 1) */
    double median_fn_nodes;    /* median body size in AST nodes */
    double sigma;              /* lognormal sigma of body sizes; 0 = all equal */
    uint32_t min_fn_nodes;     /* clip of body sizes */
    uint32_t max_fn_nodes;
    uint32_t max_expr_depth;   /* expression tree depth limit (>= 1) */
    double float_frac;         /* fraction of expressions computed in float */
    uint32_t max_nesting;      /* block nesting limit */
    double spill_frac;         /* fraction of functions given one statement that keeps
                                  more than 31 values live at once */
    int emit_source;           /* also print source text (small programs only) */
} ptl_synth_params;

typedef struct {
    size_t n;
    size_t max_depth;
    uint8_t* type;
    uint8_t* rtype;
    int32_t* parent;
    int32_t* depth;
    int32_t* child_idx;
    uint32_t* data;
    char* source;        /* NUL-terminated, or NULL */
    size_t source_len;
} ptl_synth_program;

/* Fills params with the defaults of the small seeded grammar (16 functions, about
 * 20k nodes, expression depth <= 6, 30% float). */
void ptl_synth_default_params(ptl_synth_params* p);

/* Returns 0 on success. */
int ptl_synth_generate(const ptl_synth_params* p, ptl_synth_program* out);
void ptl_synth_free(ptl_synth_program* prog);

#ifdef __cplusplus
}
#endif

#endif
