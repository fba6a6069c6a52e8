// RISC-V text output of the generated words: the reference's to_asm
// (src/codegen/rv_generator.cpp:121-127, one rvdisasm::instruction line per word) and its
// listing rvdisasm::disassemble (src/disassembler.cpp:411-451).  The text is the
// reference's, byte for byte, including its decoding choices for words outside what the
// generator emits: instruction names resolve through the reference's case order, where a
// case with no match continues with the next one (a branch with funct3 = 2 reads "lw",
// an OP word with an unknown funct7 "fence"); fused multiply-adds print integer registers;
// fsw prints the rs1 field as its float source; branch offsets drop immediate bit 10.
// Host code, no CUDA.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <ios>
#include <iomanip>
#include <optional>
#include <sstream>
#include <string>
#include <unordered_set>

#include "../../include/ptl_codegen.h"

namespace {

// RISC-V psABI register names.
const char* const kX[32] = {"zero", "ra", "sp",  "gp",  "tp", "t0", "t1", "t2", "s0", "s1", "a0",
                            "a1",   "a2", "a3",  "a4",  "a5", "a6", "a7", "s2", "s3", "s4", "s5",
                            "s6",   "s7", "s8",  "s9",  "s10", "s11", "t3", "t4", "t5", "t6"};
const char* const kF[32] = {"ft0", "ft1", "ft2", "ft3", "ft4", "ft5", "ft6",  "ft7",  "fs0", "fs1", "fa0",
                            "fa1", "fa2", "fa3", "fa4", "fa5", "fa6", "fa7",  "fs2",  "fs3", "fs4", "fs5",
                            "fs6", "fs7", "fs8", "fs9", "fs10", "fs11", "ft8", "ft9", "ft10", "ft11"};

// ANSI colours of the listing (include/disassembler.hpp:9-17).
const char* const kWhite = "\033[37m";
const char* const kInstr = "\033[38;5;186m";
const char* const kReg = "\033[38;5;117m";
const char* const kImm = "\033[38;5;114m";
const char* const kExtra = "\033[38;5;114m";

enum class Kind { unknown, r, i, s, b, u, j, r4 };

Kind kind_of(uint32_t w) {
    switch (w & 0x7Fu) {
        case 0x37: case 0x17: return Kind::u;
        case 0x6F: return Kind::j;
        case 0x67: case 0x03: case 0x13: case 0x0F: case 0x73: case 0x07: return Kind::i;
        case 0x63: return Kind::b;
        case 0x23: case 0x27: return Kind::s;
        case 0x33: case 0x53: return Kind::r;
        case 0x43: case 0x47: case 0x4B: case 0x4F: return Kind::r4;
        default: return Kind::unknown;
    }
}

using Name = const char*;

// One case of the name decoder: the name for word w, or null to continue with the next.
using Case = Name (*)(uint32_t w);

uint32_t f3(uint32_t w) { return (w >> 12) & 7u; }
uint32_t f7(uint32_t w) { return (w >> 25) & 0x7Fu; }
uint32_t f5(uint32_t w) { return (w >> 20) & 0x1Fu; }  // the rs2 field

Name pick(uint32_t key, std::initializer_list<std::pair<uint32_t, Name>> t) {
    for (const auto& [k, n] : t)
        if (k == key) return n;
    return nullptr;
}

// OP-IMM (0x13): every funct3 has a name; funct3 5 with an unknown funct7 reads as funct3 6.
Name op_imm(uint32_t w) {
    switch (f3(w)) {
        case 0: return "addi";
        case 1: return "slli";
        case 2: return "slti";
        case 3: return "sltiu";
        case 4: return "xori";
        case 5:
            if (f7(w) == 0x00) return "srli";
            if (f7(w) == 0x20) return "srai";
            return "ori";
        case 6: return "ori";
        default: return "andi";
    }
}

// OP (0x33): the funct3 rows in order from the word's own; a row without the word's
// funct7 hands on to the next; past the last row the word continues to the next case.
Name op(uint32_t w) {
    static const std::initializer_list<std::pair<uint32_t, Name>> rows[8] = {
        {{0x00, "add"}, {0x01, "mul"}, {0x20, "sub"}}, {{0, "sll"}, {1, "mulh"}},  {{0, "slt"}, {1, "mulhsu"}},
        {{0, "sltu"}, {1, "mulhu"}},                   {{0, "xor"}, {1, "div"}},   {{0x00, "srl"}, {0x01, "divu"}, {0x20, "sra"}},
        {{0, "or"}, {1, "rem"}},                       {{0, "and"}, {1, "remu"}}};
    for (uint32_t r = f3(w); r < 8; ++r)
        if (Name n = pick(f7(w), rows[r])) return n;
    return nullptr;
}

// OP-FP (0x53): the funct7 cases in order from the word's own; the first five always
// name the word, the later ones hand on to the next when their inner field has no entry.
Name op_fp(uint32_t w) {
    static const uint32_t order[] = {0x00, 0x04, 0x08, 0x0C, 0x2C, 0x10, 0x14, 0x60, 0x70, 0x50, 0x68, 0x78};
    size_t k = 0;
    while (k < sizeof(order) / sizeof(order[0]) && order[k] != f7(w)) ++k;
    for (; k < sizeof(order) / sizeof(order[0]); ++k) {
        Name n = nullptr;
        switch (order[k]) {
            case 0x00: return "fadd.s";
            case 0x04: return "fsub.s";
            case 0x08: return "fmul.s";
            case 0x0C: return "fdiv.s";
            case 0x2C: return "fsqrt.s";
            case 0x10: n = pick(f3(w), {{0, "fsgnj.s"}, {1, "fsgnjn.s"}, {2, "fsgnjx.s"}}); break;
            case 0x14: n = pick(f3(w), {{0, "fmin.s"}, {1, "fmax.s"}}); break;
            case 0x60: n = pick(f5(w), {{0, "fcvt.w.s"}, {1, "fcvt.wu.s"}}); break;
            case 0x70: n = pick(f3(w), {{0, "fmv.x.w"}, {1, "fclass.s"}}); break;
            case 0x50: n = pick(f3(w), {{0, "fle.s"}, {1, "flt.s"}, {2, "feq.s"}}); break;
            case 0x68: n = pick(f5(w), {{0, "fcvt.s.w"}, {1, "fcvt.s.wu"}}); break;
            default: return "fmv.w.x";
        }
        if (n) return n;
    }
    return nullptr;
}

// The decoder's cases, in the order a case without a match hands on to the next.
struct Entry {
    uint32_t opcode;
    Case decode;
};
const Entry kCases[] = {
    {0x37, [](uint32_t) -> Name { return "lui"; }},
    {0x17, [](uint32_t) -> Name { return "auipc"; }},
    {0x6F, [](uint32_t) -> Name { return "jal"; }},
    {0x67, [](uint32_t) -> Name { return "jalr"; }},
    {0x63, [](uint32_t w) { return pick(f3(w), {{0, "beq"}, {1, "bne"}, {4, "blt"}, {5, "bge"}, {6, "bltu"}, {7, "bgeu"}}); }},
    {0x03, [](uint32_t w) { return pick(f3(w), {{0, "lb"}, {1, "lh"}, {2, "lw"}, {4, "lbu"}, {5, "lhu"}}); }},
    {0x23, [](uint32_t w) { return pick(f3(w), {{0, "sb"}, {1, "sh"}, {2, "sw"}}); }},
    {0x13, op_imm},
    {0x33, op},
    {0x0F, [](uint32_t) -> Name { return "fence"; }},
    {0x73, [](uint32_t w) { return pick(f7(w), {{0, "ecall"}, {1, "ebreak"}}); }},
    {0x07, [](uint32_t) -> Name { return "flw"; }},
    {0x27, [](uint32_t) -> Name { return "fsw"; }},
    {0x43, [](uint32_t) -> Name { return "fmadd.s"; }},
    {0x47, [](uint32_t) -> Name { return "fmsub.s"; }},
    {0x4B, [](uint32_t) -> Name { return "fnmsub.s"; }},
    {0x4F, [](uint32_t) -> Name { return "fnmadd.s"; }},
    {0x53, op_fp},
};

Name name_of(uint32_t w) {
    const size_t ncase = sizeof(kCases) / sizeof(kCases[0]);
    size_t k = 0;
    while (k < ncase && kCases[k].opcode != (w & 0x7Fu)) ++k;
    for (; k < ncase; ++k)
        if (Name n = kCases[k].decode(w)) return n;
    return w ? "unknown" : "(zero)";
}

struct Style {
    bool color;
    void reg(std::ostream& os, const char* name) const {
        if (color) os << kReg << name << kWhite;
        else os << name;
    }
    const char* imm() const { return color ? kImm : ""; }
    const char* white() const { return color ? kWhite : ""; }
};

uint32_t field(uint32_t w, int at) { return (w >> at) & 0x1Fu; }

int32_t sext12(uint32_t v) { return static_cast<int32_t>((v >> 11) ? (v | 0xFFFFF000u) : v); }

// The operands, as format_args writes them (decimal unless noted; addr is the word's
// address, used by branches).  Leaves the stream's format flags as it found them.
void operands(std::ostream& os, uint32_t w, bool color, uint64_t addr) {
    const std::ios_base::fmtflags saved = os.flags();
    const Style st{color};
    const uint32_t opc = w & 0x7Fu;
    os << std::dec;
    switch (kind_of(w)) {
        case Kind::r:
            if (opc == 0x53) {
                const uint32_t fn = f7(w);
                const bool to_f = fn == 0x78 || fn == 0x68;                  // fmv.w.x, fcvt.s.w[u]
                const bool to_x = fn == 0x60 || (fn == 0x70 && f3(w) == 0);  // fcvt.w[u].s, fmv.x.w
                if (to_f || to_x) {
                    st.reg(os, to_f ? kF[field(w, 7)] : kX[field(w, 7)]);
                    os << ", ";
                    st.reg(os, to_f ? kX[field(w, 15)] : kF[field(w, 15)]);
                } else {
                    st.reg(os, kF[field(w, 7)]);
                    os << ", ";
                    st.reg(os, kF[field(w, 15)]);
                    os << ", ";
                    st.reg(os, kF[field(w, 20)]);
                }
            } else {
                st.reg(os, kX[field(w, 7)]);
                os << ", ";
                st.reg(os, kX[field(w, 15)]);
                os << ", ";
                st.reg(os, kX[field(w, 20)]);
            }
            break;
        case Kind::i: {
            const int32_t imm = sext12(w >> 20);
            if (opc == 0x07 || opc == 0x03 || opc == 0x67) {  // loads and jalr: rd, imm(rs1)
                st.reg(os, opc == 0x07 ? kF[field(w, 7)] : kX[field(w, 7)]);
                os << ", " << st.imm() << imm << st.white() << "(";
                st.reg(os, kX[field(w, 15)]);
                os << ")";
            } else {
                st.reg(os, kX[field(w, 7)]);
                os << ", ";
                st.reg(os, kX[field(w, 15)]);
                os << ", " << st.imm() << imm << st.white();
            }
            break;
        }
        case Kind::s: {
            const int32_t imm = sext12(((w >> 7) & 0x1Fu) | ((w >> 20) & 0xFE0u));
            st.reg(os, opc == 0x27 ? kF[field(w, 15)] : kX[field(w, 20)]);
            os << ", " << st.imm() << imm << st.white() << "(";
            st.reg(os, kX[field(w, 15)]);
            os << ")";
            break;
        }
        case Kind::b: {
            uint32_t imm = ((w >> 7) & 0x1Eu) | ((w >> 20) & 0x3E0u) | (((w >> 7) & 1u) << 11);
            if (w >> 31) imm |= 0xFFFFF800u;
            st.reg(os, kX[field(w, 15)]);
            os << ", ";
            st.reg(os, kX[field(w, 20)]);
            os << ", " << st.imm() << std::hex << std::showbase
               << (addr + static_cast<uint64_t>(static_cast<int64_t>(static_cast<int32_t>(imm)))) << std::dec
               << st.white();
            break;
        }
        case Kind::u:
            st.reg(os, kX[field(w, 7)]);
            os << ", " << st.imm() << static_cast<int32_t>(w & 0xFFFFF000u) << st.white();
            break;
        case Kind::j: {
            uint32_t imm = ((w >> 20) & 0x7FEu) | (((w >> 20) & 1u) << 11) | (w & 0xFF000u);
            if (w >> 31) imm |= 0xFFF80000u;
            st.reg(os, kX[field(w, 7)]);
            os << ", " << st.imm() << static_cast<int32_t>(imm) << st.white();
            break;
        }
        case Kind::r4:
            st.reg(os, kX[field(w, 7)]);
            os << ", ";
            st.reg(os, kX[field(w, 15)]);
            os << ", ";
            st.reg(os, kX[field(w, 20)]);
            os << ", ";
            st.reg(os, kX[field(w, 27)]);
            break;
        case Kind::unknown:
            break;
    }
    os.flags(saved);
}

ptl_status put(const std::string& text, char* out, size_t cap, size_t* len) {
    if (!len) return PTL_BAD_ARGUMENT;
    *len = text.size();
    if (!out) return PTL_OK;
    if (cap < text.size()) return PTL_BAD_ARGUMENT;
    std::memcpy(out, text.data(), text.size());
    return PTL_OK;
}

}  // namespace

extern "C" ptl_status ptl_to_asm(const uint32_t* words, size_t n, char* out, size_t cap, size_t* len) {
    if (n && !words) return PTL_BAD_ARGUMENT;
    std::ostringstream os;
    for (size_t k = 0; k < n; ++k) {
        os << name_of(words[k]) << ' ';
        operands(os, words[k], false, 0);
        os << '\n';
    }
    return put(os.str(), out, cap, len);
}

extern "C" ptl_status ptl_disassemble(const uint32_t* words, size_t n, uint64_t start_addr, const uint64_t* func_starts,
                                      size_t nfunc, char* out, size_t cap, size_t* len) {
    if (n == 0 || !words || (nfunc && !func_starts)) return PTL_BAD_ARGUMENT;
    const std::unordered_set<uint64_t> starts(func_starts, func_starts + nfunc);
    const size_t digits = static_cast<size_t>(std::ceil(std::log(n) / std::log(16))) + 1;
    const size_t count_digits = static_cast<size_t>(std::log10(n)) + 1;
    std::ostringstream os;
    os << kExtra << std::setfill('0') << std::dec << n << kWhite << " instructions, starting at " << kImm << "0x"
       << std::hex << std::setw(static_cast<int>(digits)) << start_addr << kWhite << std::dec << '\n';
    size_t label = 0;
    uint64_t addr = start_addr;
    for (size_t k = 0; k < n; ++k, addr += 4) {
        const uint32_t w = words[k];
        if (starts.count(addr / 4)) {
            // the label number takes the stream's base as the previous line left it
            os << std::string(count_digits + 3 + digits + 2 + 12 + 1, ' ') << "func" << label++ << ":\n";
        }
        os << kExtra << std::dec << std::setw(static_cast<int>(count_digits)) << std::setfill(' ') << std::right
           << (addr / 4) << kWhite << "   " << std::hex << std::setw(static_cast<int>(digits)) << std::setfill('0')
           << std::right << addr << ": ";
        for (int b = 3; b >= 0; --b) os << ' ' << kExtra << std::setw(2) << ((w >> (8 * b)) & 0xFFu) << kWhite;
        os << "   " << kInstr << std::setw(9) << std::setfill(' ') << std::left << name_of(w) << kWhite << ' ';
        operands(os, w, true, addr);
        os << '\n';
    }
    return put(os.str(), out, cap, len);
}
