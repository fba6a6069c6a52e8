/*
 * Oracle harness around the reference code generator, built from the reference's
 * own sources (see oracle/ref/Makefile).  Test infrastructure only: the library it
 * describes (oracle/_ref/libptlref.so) is loaded by tests and fixture scripts in
 * this container, never by the product.
 *
 * ptlref_compile runs rv_generator_avx (src/codegen/rv_generator_avx.cpp:21) stage
 * by stage -- preprocess, isn_cnt, isn_gen, optimize, regalloc, fix_jumps,
 * postprocess, the order of rv_generator_st::process (src/codegen/rv_generator.cpp:142-148)
 * -- and copies out the generator's arrays after each stage.
 */
#ifndef PTLREF_H
#define PTLREF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    size_t n;          /* DepthTree::filledNodes() */
    size_t max_depth;  /* DepthTree::maxDepth() */
    uint8_t* type;     /* Pareas NodeType, post-order */
    uint8_t* rtype;    /* Pareas DataType */
    int32_t* parent;
    int32_t* depth;
    int32_t* child_idx;
    uint32_t* data;
} ptlref_tree;

typedef struct {
    uint32_t* p;
    size_t n;
} ptlref_buf;

enum {
    PTLREF_OUT_WORDS = 0,
    PTLREF_FN_START, PTLREF_FN_END, PTLREF_FN_SIZE, PTLREF_FN_ID,
    PTLREF_PRE_TYPE, PTLREF_PRE_RTYPE, PTLREF_PRE_DATA,
    PTLREF_CNT_SIZE, PTLREF_CNT_LOC, PTLREF_CNT_FN_ID, PTLREF_CNT_FN_START,
    PTLREF_CNT_FN_END, PTLREF_CNT_FN_SIZE,
    PTLREF_GEN_INSTR, PTLREF_GEN_RD, PTLREF_GEN_RS1, PTLREF_GEN_RS2, PTLREF_GEN_JT,
    PTLREF_OPT_USED,
    PTLREF_RA_INSTR, PTLREF_RA_RD, PTLREF_RA_RS1, PTLREF_RA_RS2, PTLREF_RA_JT,
    PTLREF_RA_FN_START, PTLREF_RA_FN_END, PTLREF_RA_FN_SIZE,
    PTLREF_FJ_INSTR, PTLREF_FJ_RD, PTLREF_FJ_RS1, PTLREF_FJ_RS2, PTLREF_FJ_JT,
    PTLREF_FJ_FN_START, PTLREF_FJ_FN_END, PTLREF_FJ_FN_SIZE,
    PTLREF_NUM_BUFS
};

typedef struct {
    ptlref_buf bufs[PTLREF_NUM_BUFS];
    uint64_t stage_ns[7];
    int threads_used;
} ptlref_result;

/* Build the reference's pointer tree (ASTNode, children in child_idx order) from a
 * parent-pointer tree in any node order (parent[v] = -1 for the root) and flatten it with
 * the reference's DepthTree constructor (pareas-ast/src/codegen/depthtree.cpp:11-100).
 * The input must be one tree; returns 0 on success (free with ptlref_free_tree). */
int ptlref_flatten(size_t n, const uint8_t* type, const uint8_t* rtype, const int32_t* parent,
                   const int32_t* child_idx, const uint32_t* data, ptlref_tree* out);

/* Parse a Pareas source file with the reference front end (pareas-ast) and flatten it
 * into a DepthTree.  Returns 0 on success; on failure writes a message into err. */
int ptlref_parse_file(const char* path, ptlref_tree* out, char* err, size_t errlen);
void ptlref_free_tree(ptlref_tree* t);

/* Run the reference AVX generator.  threads/sync/altblock/mininstr are the arguments of
 * rv_generator_avx's constructor; threads = 1 is the deterministic oracle.
 * snapshots = 0 copies only the final words and function table. */
int ptlref_compile(const ptlref_tree* in, int threads, int sync, int altblock,
                   uint32_t mininstr, int snapshots, ptlref_result* out,
                   char* err, size_t errlen);
/* Run the reference's scalar generator rv_generator_st (its -s flag), with the same
 * snapshot slots. */
int ptlref_compile_scalar(const ptlref_tree* in, int snapshots, ptlref_result* out, char* err, size_t errlen);
void ptlref_free_result(ptlref_result* r);

/* Flat dumps of the reference tables; see ptlport_table in oracle/port/ptl_port.h. */
size_t ptlref_table(int which, uint32_t* out);

/* The reference's text output of words (rv_generator::to_asm, rvdisasm::disassemble)
 * into out (at most cap bytes); returns the text's full length. */
size_t ptlref_to_asm(const uint32_t* words, size_t n, char* out, size_t cap);
size_t ptlref_disassemble(const uint32_t* words, size_t n, uint64_t start_addr, const uint64_t* func_starts,
                          size_t nfunc, char* out, size_t cap);

#ifdef __cplusplus
}
#endif

#endif
