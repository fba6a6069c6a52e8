/*
 * ORACLE -- test infrastructure, not product code.
 *
 * A scalar CPU restatement of the reference's AVX2 code generator
 * (src/codegen/rv_generator_avx.cpp), run with one worker thread, which is the
 * deterministic configuration whose output the GPU build must reproduce bit for bit,
 * and of its single-threaded scalar generator (src/codegen/rv_generator.cpp).
 * Parity of this restatement is pinned against the reference itself, compiled from
 * its sources by oracle/ref/Makefile, on the reference's Pareas test inputs and on
 * seeded synthetic programs (tests/test_oracle_pin.py); tests/golden/ carries the
 * reference's outputs for machines where the reference cannot be built.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 */
#ifndef PTL_PORT_H
#define PTL_PORT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Buffer slots, in the same order as oracle/ref/ptlref.h so results compare 1:1. */
enum {
    PTLPORT_OUT_WORDS = 0,
    PTLPORT_FN_START, PTLPORT_FN_END, PTLPORT_FN_SIZE, PTLPORT_FN_ID,
    PTLPORT_PRE_TYPE, PTLPORT_PRE_RTYPE, PTLPORT_PRE_DATA,
    PTLPORT_CNT_SIZE, PTLPORT_CNT_LOC, PTLPORT_CNT_FN_ID, PTLPORT_CNT_FN_START,
    PTLPORT_CNT_FN_END, PTLPORT_CNT_FN_SIZE,
    PTLPORT_GEN_INSTR, PTLPORT_GEN_RD, PTLPORT_GEN_RS1, PTLPORT_GEN_RS2, PTLPORT_GEN_JT,
    PTLPORT_OPT_USED,
    PTLPORT_RA_INSTR, PTLPORT_RA_RD, PTLPORT_RA_RS1, PTLPORT_RA_RS2, PTLPORT_RA_JT,
    PTLPORT_RA_FN_START, PTLPORT_RA_FN_END, PTLPORT_RA_FN_SIZE,
    PTLPORT_FJ_INSTR, PTLPORT_FJ_RD, PTLPORT_FJ_RS1, PTLPORT_FJ_RS2, PTLPORT_FJ_JT,
    PTLPORT_FJ_FN_START, PTLPORT_FJ_FN_END, PTLPORT_FJ_FN_SIZE,
    PTLPORT_NUM_BUFS
};

typedef struct {
    uint32_t* p;
    size_t n;
} ptlport_buf;

typedef struct {
    ptlport_buf bufs[PTLPORT_NUM_BUFS];
    uint64_t stage_ns[7];
} ptlport_result;

/* Return codes */
#define PTLPORT_OK 0
#define PTLPORT_EINVAL 1      /* input violates the reference's input contract */
#define PTLPORT_EUNSUPPORTED 2 /* input reaches reference behaviour that is undefined */

/* Compile one program.  snapshots != 0 also copies every stage's arrays. */
int ptlport_compile(const uint8_t* type, const uint8_t* rtype, const int32_t* parent,
                    const int32_t* depth, const int32_t* child_idx, const uint32_t* data,
                    size_t n, size_t max_depth, int snapshots, ptlport_result* out,
                    char* err, size_t errlen);
void ptlport_free_result(ptlport_result* r);

/* The same for the reference's scalar generator rv_generator_st
 * (src/codegen/rv_generator.cpp:227-1736, the -s flag of src/main.cpp). */
int ptlport_compile_scalar(const uint8_t* type, const uint8_t* rtype, const int32_t* parent,
                           const int32_t* depth, const int32_t* child_idx, const uint32_t* data,
                           size_t n, size_t max_depth, int snapshots, ptlport_result* out,
                           char* err, size_t errlen);

/* The permutation libstdc++'s std::sort leaves when it sorts iota(n) by key (the
 * reference's isn_gen sort, src/codegen/rv_generator_avx.cpp:539-541), written into
 * perm.  Exposed so tests can pin the GPU's emulation of that order. */
void ptlport_depth_sort(const int32_t* keys, size_t n, uint32_t* perm);

/* Dumps of the code-generation tables in the reference's flat layouts
 * (include/codegen/rv_nodetype.hpp:197-1134): which = 0 node_size[256][6],
 * 1 has_instr[256][4][6], 2 has_output[256][4][6], 3 parent_arg_idx[256][4][6],
 * 4 get_output[256][4][6], 5 instr[256][4][6], 6 instr_constant[256][4],
 * 7 operand[256][4][6][2], 8 instr_jt[256][4], 9 pareas_to_rv[44].
 * Returns the element count (out may be NULL to query it). */
size_t ptlport_table(int which, uint32_t* out);

/* DepthTree::DepthTree(ASTNode*) (pareas-ast/src/codegen/depthtree.cpp:11-100) over a
 * parent-pointer tree in any node order: node v's parent is parent[v] (-1 for the one
 * root) and its place among its parent's children is child_idx[v].  Writes the DepthTree
 * arrays in post-order (children in child_idx order before their parent), depth from the
 * root, parents as post-order indices, the root's child_idx -1, order[v] = v's post-order
 * index and *max_depth.  Returns PTLPORT_EINVAL when the arrays are not one tree with
 * child indices 0..k-1 at every node. */
int ptlport_flatten(size_t n, const uint8_t* type, const uint8_t* rtype, const int32_t* parent,
                    const int32_t* child_idx, const uint32_t* data, uint8_t* o_type, uint8_t* o_rtype,
                    int32_t* o_parent, int32_t* o_depth, int32_t* o_child, uint32_t* o_data, int32_t* order,
                    size_t* max_depth);

#ifdef __cplusplus
}
#endif

#endif
