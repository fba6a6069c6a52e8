// The reference's code-generation tables (include/codegen/rv_nodetype.hpp:197-1134),
// re-encoded densely for the GPU (ptl_common.cuh, CodeTables).  The contents are the
// reference's -- the instruction words and operand rules are the compiler's ISA
// mapping and must be identical -- and tests compare the flattened tables with the
// reference's own constexpr arrays element by element.
//
// Each node type is described once, as a row spec: per slot, which data types emit an
// instruction, the instruction word per data type, and the operand / output / jump /
// constant rules.
#include <cstring>
#include <initializer_list>

#include "ptl_common.cuh"

namespace ptl {
namespace {

constexpr uint8_t kAll = 0x3F;
constexpr uint8_t kI = 1u << DT_INT;
constexpr uint8_t kF = 1u << DT_FLOAT;

constexpr uint32_t R(uint32_t f7, uint32_t rs2, uint32_t rs1, uint32_t f3, uint32_t rd, uint32_t op) {
    return (f7 << 25) | (rs2 << 20) | (rs1 << 15) | (f3 << 12) | (rd << 7) | op;
}
constexpr uint32_t I(uint32_t imm, uint32_t rs1, uint32_t f3, uint32_t rd, uint32_t op) {
    return ((imm & 0xFFFu) << 20) | (rs1 << 15) | (f3 << 12) | (rd << 7) | op;
}

// Order of the dense rows; row k describes rv type kRowTypes[k].
constexpr uint32_t kRowTypes[] = {
    RV_INVALID, RV_STATEMENT_LIST, RV_EMPTY, RV_EXPRESSION, RV_ADD, RV_SUB, RV_MUL, RV_DIV,
    RV_MOD, RV_BITAND, RV_BITOR, RV_BITXOR, RV_LSHIFT, RV_RSHIFT, RV_URSHIFT, RV_LAND, RV_LOR,
    RV_BITNOT, RV_LNOT, RV_NEG, RV_LITERAL, RV_CAST, RV_DEREF, RV_ASSIGN, RV_DECL, RV_ID,
    RV_WHILE_DUMMY, RV_FUNC_DECL_DUMMY, RV_RETURN, RV_FUNC_DECL, RV_FUNC_ARG_LIST, RV_FUNC_CALL,
    RV_FUNC_CALL_ARG_LIST, RV_IF, RV_WHILE, RV_IF_ELSE, RV_EQ, RV_NEQ, RV_LT, RV_GT, RV_LTE,
    RV_GTE, RV_FUNC_ARG, RV_FUNC_ARG_FLOAT_AS_INT, RV_FUNC_ARG_ON_STACK, RV_FUNC_CALL_ARG,
    RV_FUNC_CALL_ARG_FLOAT_AS_INT, RV_FUNC_CALL_ARG_ON_STACK,
};
static_assert(sizeof(kRowTypes) / sizeof(kRowTypes[0]) == 48, "48 named rv node types");
static_assert(kUndefRow == 48 && kTypeRows == 49, "unnamed types use their own zero row");

struct RowBuilder {
    CodeTables* t;
    uint32_t r;

    RowBuilder& size(uint32_t v) { for (int d = 0; d < 6; ++d) t->size[r][d] = static_cast<uint8_t>(v); return *this; }
    RowBuilder& size_by(std::initializer_list<uint32_t> v) { int d = 0; for (uint32_t x : v) t->size[r][d++] = static_cast<uint8_t>(x); return *this; }
    // Slots with instructions, as a data-type mask per slot.
    RowBuilder& emits(int s, uint8_t mask) { t->has_instr[r][s] = mask; return *this; }
    RowBuilder& output(int s, uint8_t mask) { t->has_output[r][s] = mask; return *this; }
    RowBuilder& pai(int s, uint32_t v) { for (int d = 0; d < 6; ++d) t->pai[r][s][d] = static_cast<uint8_t>(v); return *this; }
    RowBuilder& pai_at(int s, int d, uint32_t v) { t->pai[r][s][d] = static_cast<uint8_t>(v); return *this; }
    RowBuilder& out_at(int s, int d, uint32_t v) { t->out[r][s][d] = static_cast<uint8_t>(v); return *this; }
    // Every slot's word defaults to the reference's placeholder.
    RowBuilder& no_words() { for (int s = 0; s < 4; ++s) for (int d = 0; d < 6; ++d) t->instr[r][s][d] = kNoInstr; return *this; }
    RowBuilder& word(int s, uint32_t w) { for (int d = 0; d < 6; ++d) t->instr[r][s][d] = w; return *this; }
    RowBuilder& word_at(int s, int d, uint32_t w) { t->instr[r][s][d] = w; return *this; }
    RowBuilder& cnst(int s, uint32_t v) { t->cnst[r][s] = static_cast<uint8_t>(v); return *this; }
    RowBuilder& jt(int s, uint32_t v) { t->jt[r][s] = static_cast<uint8_t>(v); return *this; }
    RowBuilder& opd(int s, uint32_t a, uint32_t b) {
        for (int d = 0; d < 6; ++d) { t->opd[r][s][d][0] = static_cast<uint8_t>(a); t->opd[r][s][d][1] = static_cast<uint8_t>(b); }
        return *this;
    }
    RowBuilder& opd_at(int s, int d, uint32_t a, uint32_t b) {
        t->opd[r][s][d][0] = static_cast<uint8_t>(a); t->opd[r][s][d][1] = static_cast<uint8_t>(b);
        return *this;
    }
};

}  // namespace

void build_code_tables(CodeTables* t) {
    std::memset(t, 0, sizeof(*t));
    for (int k = 0; k < 256; ++k) t->row_of[k] = static_cast<uint8_t>(kUndefRow);
    for (uint32_t k = 0; k < 48; ++k) t->row_of[kRowTypes[k]] = static_cast<uint8_t>(k);
    auto row = [&](uint32_t type) { return RowBuilder{t, t->row_of[type]}; };

    for (uint32_t ty : {RV_INVALID, RV_STATEMENT_LIST, RV_EXPRESSION}) row(ty).no_words().pai(0, 2);
    row(RV_EMPTY).no_words();

    struct Bin { uint32_t ty, wi, wf; };
    const Bin bins[] = {
        {RV_ADD, R(0x00, 0, 0, 0, 0, 0x33), R(0x00, 0, 0, 7, 0, 0x53)},
        {RV_SUB, R(0x20, 0, 0, 0, 0, 0x33), R(0x04, 0, 0, 7, 0, 0x53)},
        {RV_MUL, R(0x01, 0, 0, 0, 0, 0x33), R(0x08, 0, 0, 7, 0, 0x53)},
        {RV_DIV, R(0x01, 0, 0, 4, 0, 0x33), R(0x0C, 0, 0, 7, 0, 0x53)},
        {RV_MOD, R(0x01, 0, 0, 6, 0, 0x33), kNoInstr},
        {RV_BITAND, R(0x00, 0, 0, 7, 0, 0x33), kNoInstr},
        {RV_BITOR, R(0x00, 0, 0, 6, 0, 0x33), kNoInstr},
        {RV_BITXOR, R(0x00, 0, 0, 4, 0, 0x33), kNoInstr},
        {RV_LSHIFT, R(0x00, 0, 0, 1, 0, 0x33), kNoInstr},
        {RV_RSHIFT, R(0x20, 0, 0, 5, 0, 0x33), kNoInstr},
        {RV_URSHIFT, R(0x00, 0, 0, 5, 0, 0x33), kNoInstr},
    };
    for (const Bin& b : bins) {
        row(b.ty).size(1).emits(0, kAll).pai(0, 2).no_words().word_at(0, DT_INT, b.wi)
            .word_at(0, DT_FLOAT, b.wf).opd(0, 1, 1);
    }
    for (uint32_t ty : {RV_LAND, RV_LOR}) row(ty).emits(0, kAll).pai(0, 2).no_words();
    row(RV_BITNOT).size(1).emits(0, kAll).pai(0, 2).no_words().word_at(0, DT_INT, I(0xFFF, 0, 4, 0, 0x13));
    row(RV_LNOT).size(1).emits(0, kAll).pai(0, 2).no_words().word_at(0, DT_INT, I(1, 0, 3, 0, 0x13));
    row(RV_NEG).size(1).emits(0, kAll).pai(0, 2).no_words().word_at(0, DT_INT, R(0x20, 0, 0, 0, 0, 0x33))
        .word_at(0, DT_FLOAT, R(0x10, 0, 0, 1, 0, 0x53));

    row(RV_LITERAL).size_by({0, 0, 2, 3, 0, 0}).emits(0, kAll).emits(1, kAll).emits(2, kF)
        .output(0, kAll).output(1, kF)
        .pai(1, 1).pai_at(1, DT_FLOAT, 0).pai_at(2, DT_FLOAT, 1)
        .no_words().word_at(0, DT_INT, 0x37).word_at(0, DT_FLOAT, 0x37)
        .word_at(1, DT_INT, 0x13).word_at(1, DT_FLOAT, 0x13).word_at(2, DT_FLOAT, R(0x78, 0, 0, 0, 0, 0x53))
        .cnst(0, 1).cnst(1, 2).opd(1, 7, 0).opd_at(2, DT_FLOAT, 7, 0);
    row(RV_CAST).size(1).emits(0, kAll).pai(0, 2).no_words().word_at(0, DT_INT, R(0x60, 0, 0, 7, 0, 0x53))
        .word_at(0, DT_FLOAT, R(0x68, 0, 0, 7, 0, 0x53)).opd(0, 1, 0);
    row(RV_DEREF).size(1).emits(0, kAll).pai(0, 2).no_words().word_at(0, DT_INT, I(0, 0, 2, 0, 0x03))
        .word_at(0, DT_FLOAT, I(0, 0, 2, 0, 0x07)).opd(0, 1, 0);
    row(RV_ASSIGN).size(2).emits(0, kAll).emits(1, kAll).pai(1, 1).no_words()
        .word_at(0, DT_INT, 0x2023).word_at(0, DT_FLOAT, 0x2027)
        .word_at(1, DT_INT, 0x33).word_at(1, DT_FLOAT, R(0x10, 0, 0, 0, 0, 0x53))
        .opd(0, 1, 1).opd(1, 4, 0).opd_at(1, DT_FLOAT, 4, 4);
    for (uint32_t ty : {RV_DECL, RV_ID}) {
        row(ty).size(1).emits(0, kAll).pai(0, 2).no_words().word(0, I(0, 8, 0, 0, 0x13)).cnst(0, 3);
    }
    row(RV_WHILE_DUMMY).emits(0, kAll).pai(0, 2).no_words();
    row(RV_FUNC_DECL_DUMMY).size(6).emits(0, kAll).emits(1, kAll).emits(2, kAll).emits(3, kAll).pai(0, 2)
        .word(0, 0xFE112E23u).word(1, 0xFE812C23u).word(2, R(0x20, 8, 2, 0, 2, 0x33)).word(3, R(0x00, 2, 8, 0, 8, 0x33));
    // Slot 0 of return lists four words in the reference; data types 4 and 5 stay 0.
    row(RV_RETURN).size(2).emits(0, kAll).emits(1, kAll).output(0, kAll)
        .out_at(0, 0, 4).out_at(0, 1, 4).out_at(0, 2, 4).out_at(0, 3, 3).out_at(0, 4, 4).out_at(0, 5, 4)
        .word_at(0, DT_INVALID, kNoInstr).word_at(0, DT_VOID, 0x33).word_at(0, DT_INT, 0x33)
        .word_at(0, DT_FLOAT, R(0x10, 0, 0, 0, 0, 0x53)).word(1, 0x67).word(2, kNoInstr).word(3, kNoInstr)
        .opd_at(0, DT_INT, 1, 0).opd_at(0, DT_FLOAT, 1, 0).jt(1, 6);
    row(RV_FUNC_DECL).size(6).emits(0, kAll).emits(1, kAll).emits(2, kAll).emits(3, kAll)
        .word(0, R(0x00, 8, 2, 0, 2, 0x33)).word(1, I(0xFFC, 2, 2, 1, 0x03)).word(2, I(0xFF8, 8, 2, 8, 0x03))
        .word(3, I(0, 1, 0, 0, 0x67));
    row(RV_FUNC_ARG_LIST).pai(0, 2).no_words();
    row(RV_FUNC_CALL).size_by({3, 2, 3, 3, 3, 3}).emits(0, kAll).emits(2, kI | kF)
        .pai_at(2, DT_INT, 1).pai_at(2, DT_FLOAT, 1).no_words().word(0, I(0, 0, 0, 1, 0x67))
        .word_at(2, DT_INT, R(0x00, 0, 10, 0, 0, 0x33)).word_at(2, DT_FLOAT, R(0x10, 10, 10, 0, 0, 0x53)).jt(0, 7);
    row(RV_FUNC_CALL_ARG_LIST).emits(0, kAll).emits(1, kAll).pai(0, 2).no_words()
        .word(0, I(0, 2, 7, 2, 0x13)).word(1, I(0, 2, 6, 2, 0x13)).cnst(0, 5).cnst(1, 4);

    row(RV_IF).emits(0, kAll).pai(0, 2).no_words().word(0, 0x63).opd(0, 1, 0).jt(0, 1);
    row(RV_WHILE).size(1).emits(0, kAll).emits(1, kAll).pai(0, 2).no_words().word(0, 0x63).word(1, 0x67)
        .opd(0, 4, 0).jt(0, 4).jt(1, 5);
    row(RV_IF_ELSE).emits(0, kAll).emits(1, kAll).pai(0, 2).no_words().word(0, 0x63).word(1, 0x67)
        .opd(0, 1, 0).jt(0, 2).jt(1, 3);

    const uint32_t sub_w = R(0x20, 0, 0, 0, 0, 0x33);
    const uint32_t feq_w = R(0x50, 0, 0, 2, 0, 0x53);
    const uint32_t sltiu1 = I(1, 0, 3, 0, 0x13);
    const uint32_t slt_w = R(0x00, 0, 0, 2, 0, 0x33);
    row(RV_EQ).size_by({0, 0, 2, 1, 0, 0}).emits(0, kAll).emits(1, kI | kF).output(0, kI).pai(0, 2)
        .pai_at(1, DT_INT, 1).no_words().word_at(0, DT_INT, sub_w).word_at(0, DT_FLOAT, feq_w)
        .word_at(1, DT_INT, sltiu1).opd(0, 1, 1).opd_at(1, DT_INT, 7, 0);
    row(RV_NEQ).size(2).emits(0, kAll).emits(1, kAll).output(0, kAll).pai(0, 2).no_words()
        .word_at(0, DT_INT, sub_w).word_at(0, DT_FLOAT, feq_w).word_at(1, DT_INT, R(0x00, 0, 0, 3, 0, 0x33))
        .word_at(1, DT_FLOAT, sltiu1).opd(0, 1, 1).opd_at(1, DT_INT, 0, 7).opd_at(1, DT_FLOAT, 7, 0);
    row(RV_LT).size(1).emits(0, kAll).pai(0, 2).no_words().word_at(0, DT_INT, slt_w)
        .word_at(0, DT_FLOAT, R(0x50, 0, 0, 1, 0, 0x53)).opd(0, 1, 1);
    row(RV_GT).size(1).emits(0, kAll).pai(0, 2).no_words().word_at(0, DT_INT, slt_w)
        .word_at(0, DT_FLOAT, R(0x50, 0, 0, 1, 0, 0x53)).opd(0, 5, 5);
    row(RV_LTE).size_by({0, 0, 2, 1, 0, 0}).emits(0, kAll).emits(1, kI).output(0, kI).pai(0, 2).no_words()
        .word_at(0, DT_INT, slt_w).word_at(0, DT_FLOAT, R(0x50, 0, 0, 0, 0, 0x53)).word_at(1, DT_INT, sltiu1)
        .opd_at(0, DT_INT, 5, 5).opd_at(0, DT_FLOAT, 1, 1).opd_at(1, DT_INT, 7, 0);
    row(RV_GTE).size_by({0, 0, 2, 1, 0, 0}).emits(0, kAll).emits(1, kI).output(0, kI).pai(0, 2).no_words()
        .word_at(0, DT_INT, slt_w).word_at(0, DT_FLOAT, R(0x50, 0, 0, 0, 0, 0x53)).word_at(1, DT_INT, sltiu1)
        .opd_at(0, DT_INT, 1, 1).opd_at(0, DT_FLOAT, 5, 5).opd_at(1, DT_INT, 7, 0);

    row(RV_FUNC_ARG).size(1).emits(0, kAll).no_words().word_at(0, DT_INT_REF, 0x2023)
        .word_at(0, DT_FLOAT_REF, 0x2027).opd(0, 1, 0).opd_at(0, DT_INT_REF, 1, 2).opd_at(0, DT_FLOAT_REF, 1, 3);
    row(RV_FUNC_ARG_FLOAT_AS_INT).size(1).emits(0, kAll).no_words().word(0, R(0x70, 0, 0, 0, 0, 0x53)).opd(0, 1, 2);
    row(RV_FUNC_ARG_ON_STACK).size(2).emits(0, kAll).emits(1, kAll).output(0, kAll).no_words()
        .word_at(0, DT_INT, 0x2123).word_at(0, DT_FLOAT, 0x2127).cnst(0, 4).opd(1, 1, 7);
    row(RV_FUNC_CALL_ARG).emits(0, kAll).no_words().word_at(0, DT_INT, 0x33)
        .word_at(0, DT_FLOAT, R(0x10, 0, 0, 0, 0, 0x53)).out_at(0, DT_INT, 1).out_at(0, DT_FLOAT, 2)
        .opd(0, 1, 0).opd_at(0, DT_FLOAT, 1, 6);
    row(RV_FUNC_CALL_ARG_FLOAT_AS_INT).emits(0, kAll).no_words().word(0, R(0x70, 0, 0, 0, 0, 0x53))
        .out_at(0, 0, 1).out_at(0, 1, 1).out_at(0, 2, 1).out_at(0, 3, 1).out_at(0, 4, 1).out_at(0, 5, 1).opd(0, 1, 0);
    row(RV_FUNC_CALL_ARG_ON_STACK).emits(0, kAll).emits(1, kAll).no_words().word_at(0, DT_INT, 0x2123)
        .word_at(0, DT_FLOAT, 0x2127).cnst(0, 4).opd(0, 6, 0);

    // Pareas NodeType -> rv type (rv_nodetype.hpp:1089-1134)
    const uint32_t pareas[kNumPareasTypes] = {
        RV_INVALID, RV_STATEMENT_LIST, RV_EMPTY, RV_FUNC_DECL, RV_FUNC_ARG, RV_FUNC_ARG_LIST,
        RV_EXPRESSION, RV_IF, RV_IF_ELSE, RV_WHILE, RV_FUNC_CALL, RV_FUNC_CALL_ARG,
        RV_FUNC_CALL_ARG_LIST, RV_ADD, RV_SUB, RV_MUL, RV_DIV, RV_MOD, RV_BITAND, RV_BITOR,
        RV_BITXOR, RV_LSHIFT, RV_RSHIFT, RV_URSHIFT, RV_LAND, RV_LOR, RV_EQ, RV_NEQ, RV_LT, RV_GT,
        RV_LTE, RV_GTE, RV_BITNOT, RV_LNOT, RV_NEG, RV_LITERAL, RV_CAST, RV_DEREF, RV_ASSIGN,
        RV_DECL, RV_ID, RV_WHILE_DUMMY, RV_FUNC_DECL_DUMMY, RV_RETURN,
    };
    for (uint32_t k = 0; k < kNumPareasTypes; ++k) t->pareas_to_rv[k] = static_cast<uint8_t>(pareas[k]);

    // isn_gen's packed per-slot fields; a value that does not fit its field is stored as
    // all ones there (gen_desc_ok reports it)
    auto fit = [](uint32_t v, uint32_t bits) { return v < (1u << bits) ? v : (1u << bits) - 1u; };
    for (uint32_t r = 0; r < kTypeRows; ++r) {
        for (uint32_t d = 0; d < 6; ++d) {
            for (uint32_t s = 0; s < 4; ++s) {
                uint32_t v = (t->has_instr[r][s] >> d) & 1u;
                v |= fit(t->pai[r][s][d], 2) << 1;
                v |= fit(t->out[r][s][d], 3) << 3;
                v |= ((t->has_output[r][s] >> d) & 1u) << 6;
                v |= fit(t->cnst[r][s], 3) << 7;
                v |= fit(t->jt[r][s], 3) << 10;
                v |= fit(t->opd[r][s][d][0], 3) << 13;
                v |= fit(t->opd[r][s][d][1], 3) << 16;
                v |= fit(t->size[r][d], 4) << 19;
                t->gdesc[r][d][s] = v;
                t->gword[r][d][s] = t->instr[r][s][d];
            }
        }
    }
}

bool gen_desc_ok(const CodeTables* t) {
    for (uint32_t r = 0; r < kTypeRows; ++r) {
        for (uint32_t d = 0; d < 6; ++d) {
            for (uint32_t s = 0; s < 4; ++s) {
                const uint32_t v = t->gdesc[r][d][s];
                const bool ok = gd_has(v) == (((t->has_instr[r][s] >> d) & 1u) != 0) && gd_pai(v) == t->pai[r][s][d] &&
                                gd_out(v) == t->out[r][s][d] &&
                                gd_has_output(v) == (((t->has_output[r][s] >> d) & 1u) != 0) &&
                                gd_cnst(v) == t->cnst[r][s] && gd_jt(v) == t->jt[r][s] &&
                                gd_opd(v, 0) == t->opd[r][s][d][0] && gd_opd(v, 1) == t->opd[r][s][d][1] &&
                                gd_size(v) == t->size[r][d] && t->gword[r][d][s] == t->instr[r][s][d];
                if (!ok) return false;
            }
        }
    }
    return true;
}

}  // namespace ptl
