// Common definitions of the GB300 code generator.
//
// Stage logic is written as __host__ __device__ functions of one thread's work so that
// the CUDA kernels and the host model build (PTL_HOST_MODEL, used only by the CPU test
// suite to check the GPU algorithm before it runs on a GPU) execute the same code.
#pragma once

#include <stddef.h>
#include <stdint.h>

#if defined(__CUDACC__) && !defined(PTL_HOST_MODEL)
#define PTL_HD __host__ __device__ __forceinline__
#define PTL_DEVICE_BUILD 1
#else
#define PTL_HD inline
#define PTL_DEVICE_BUILD 0
#endif

namespace ptl {

// ---------------------------------------------------------------- node encoding
// rv node types of the reference (include/codegen/rv_nodetype.hpp:13-86): the bit
// patterns matter, the code tests them with masks.
enum : uint32_t {
    RV_INVALID = 0, RV_STATEMENT_LIST = 1, RV_EMPTY = 2, RV_EXPRESSION = 3,
    RV_ADD = 4, RV_SUB = 5, RV_MUL = 6, RV_DIV = 7, RV_MOD = 8, RV_BITAND = 9, RV_BITOR = 10,
    RV_BITXOR = 11, RV_LSHIFT = 12, RV_RSHIFT = 13, RV_URSHIFT = 14, RV_LAND = 15, RV_LOR = 16,
    RV_BITNOT = 17, RV_LNOT = 18, RV_NEG = 19, RV_LITERAL = 20, RV_CAST = 21, RV_DEREF = 22,
    RV_ASSIGN = 23, RV_DECL = 24, RV_ID = 25, RV_WHILE_DUMMY = 26, RV_FUNC_DECL_DUMMY = 27,
    RV_RETURN = 28, RV_FUNC_DECL = 29, RV_FUNC_ARG_LIST = 30, RV_FUNC_CALL = 31,
    RV_FUNC_CALL_ARG_LIST = 32,
    RV_IF = 0xD0, RV_WHILE = 0xD1, RV_IF_ELSE = 0xD2,
    RV_EQ = 0xE0, RV_NEQ = 0xE1, RV_LT = 0xE2, RV_GT = 0xE3, RV_LTE = 0xE4, RV_GTE = 0xE5,
    RV_FUNC_ARG = 0xF0, RV_FUNC_ARG_FLOAT_AS_INT = 0xF1, RV_FUNC_ARG_ON_STACK = 0xF2,
    RV_FUNC_CALL_ARG = 0xF4, RV_FUNC_CALL_ARG_FLOAT_AS_INT = 0xF5,
    RV_FUNC_CALL_ARG_ON_STACK = 0xF6,
};
enum : uint32_t { DT_INVALID = 0, DT_VOID = 1, DT_INT = 2, DT_FLOAT = 3, DT_INT_REF = 4, DT_FLOAT_REF = 5 };

constexpr uint32_t kNumPareasTypes = 44;
constexpr uint32_t kNoInstr = 0x00000073u;  // placeholder word the reference emits for "no instruction"

// ---------------------------------------------------------------- code tables
// Dense layout of the reference's [256][4][6] tables (rv_nodetype.hpp:197-1134): rows
// are indexed by a dense id of the rv node type (kTypeRows rows; row kUndefRow is all
// zero, the value the reference's zero-initialised tables hold for unused types).
constexpr uint32_t kTypeRows = 49;
constexpr uint32_t kUndefRow = 48;

struct CodeTables {
    uint8_t row_of[256];             // rv node type -> dense row
    uint8_t pareas_to_rv[kNumPareasTypes];
    uint8_t size[kTypeRows][6];      // node_size_mapping
    uint8_t has_instr[kTypeRows][4]; // bit d set = has_instr_mapping[t][s][d]
    uint8_t has_output[kTypeRows][4];
    uint8_t pai[kTypeRows][4][6];    // parent_arg_idx_lookup
    uint8_t out[kTypeRows][4][6];    // get_output_table
    uint8_t cnst[kTypeRows][4];      // instr_constant_table
    uint8_t jt[kTypeRows][4];        // instr_jt_table
    uint8_t opd[kTypeRows][4][6][2]; // operand_table
    uint32_t instr[kTypeRows][4][6]; // instr_table
    // isn_gen's reads per (row, data type), the four slots side by side so that a node
    // loads them in one 16-byte read: gdesc packs the slot's fields (gd_* below), gword
    // its instruction word
    alignas(16) uint32_t gdesc[kTypeRows][6][4];
    alignas(16) uint32_t gword[kTypeRows][6][4];
};

// gdesc fields: has_instr (bit 0), parent_arg_idx calc (1-2), output calc (3-5),
// has_output (6), instr_constant calc (7-9), instr_jt calc (10-12), the two operand calcs
// (13-15, 16-18), node_size_mapping (19-22).
PTL_HD bool gd_has(uint32_t d) { return (d & 1u) != 0; }
PTL_HD uint32_t gd_pai(uint32_t d) { return (d >> 1) & 3u; }
PTL_HD uint32_t gd_out(uint32_t d) { return (d >> 3) & 7u; }
PTL_HD bool gd_has_output(uint32_t d) { return ((d >> 6) & 1u) != 0; }
PTL_HD uint32_t gd_cnst(uint32_t d) { return (d >> 7) & 7u; }
PTL_HD uint32_t gd_jt(uint32_t d) { return (d >> 10) & 7u; }
PTL_HD uint32_t gd_opd(uint32_t d, uint32_t k) { return (d >> (13u + 3u * k)) & 7u; }
PTL_HD uint32_t gd_size(uint32_t d) { return (d >> 19) & 15u; }

// Builds the tables (ptl_tables.cpp).
void build_code_tables(CodeTables* t);
// Whether the packed isn_gen fields decode to the tables (every value fit its field).
bool gen_desc_ok(const CodeTables* t);

PTL_HD int32_t s32(uint32_t v) { return static_cast<int32_t>(v); }
PTL_HD uint32_t u32(int32_t v) { return static_cast<uint32_t>(v); }

// ---------------------------------------------------------------- status
enum Status : int {
    ST_OK = 0,
    ST_INVALID_AST = 1,
    ST_UNSUPPORTED = 2,
    ST_OOM = 3,
    ST_ADMISSION_DENIED = 4,
    ST_DEVICE_TIMEOUT = 5,
    ST_CUDA_ERROR = 6,
    ST_BAD_ARGUMENT = 7,
};

// Device-side error word: kernels that meet an input the reference leaves undefined,
// or a bounded wait that gives up, record a code and a detail instead of trapping.
struct ErrorWord {
    uint32_t code;    // Status
    uint32_t where;   // kernel/stage id
    uint32_t detail;  // first offending index
    uint32_t pad;
};

enum : uint32_t {
    W_PRE = 1, W_CNT = 2, W_SORT = 3, W_GEN = 4, W_OPT = 5, W_RA1 = 6, W_RA2 = 7,
    W_RA_SCATTER = 8, W_FIX = 9, W_SCAN = 10,
};

}  // namespace ptl
