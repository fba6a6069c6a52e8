// ELF64 wrapping of a compiled program (ptl_write_elf in include/ptl_codegen.h).
//
// The reference writes raw little-endian words only (rv_generator::to_binary,
// src/codegen/rv_generator.cpp:116-119).  This writes the same words as the .text
// section of an ELF64 little-endian RISC-V relocatable object (EM_RISCV), with one
// global STT_FUNC symbol per function of the function table, named like the labels of
// the reference's disassembler listing (func0, func1, ... in address order,
// src/disassembler.cpp:425-431), value = start word * 4, size = (end - start) * 4.
// Every jump the generator emits is pc-relative inside the program (auipc/jalr pairs
// and branches, rv_generator_avx.cpp:1930-1975), so the object needs no relocations.
// e_flags is 0: the words use the F extension's registers for float values, but the
// generator follows no calling convention that a float-ABI flag would describe.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ptl_codegen.h"

namespace {

struct Ehdr {
    unsigned char ident[16];
    uint16_t type, machine;
    uint32_t version;
    uint64_t entry, phoff, shoff;
    uint32_t flags;
    uint16_t ehsize, phentsize, phnum, shentsize, shnum, shstrndx;
};
struct Shdr {
    uint32_t name, type;
    uint64_t flags, addr, offset, size;
    uint32_t link, info;
    uint64_t addralign, entsize;
};
struct Sym {
    uint32_t name;
    unsigned char info, other;
    uint16_t shndx;
    uint64_t value, size;
};
static_assert(sizeof(Ehdr) == 64 && sizeof(Shdr) == 64 && sizeof(Sym) == 24, "ELF64 record sizes");

constexpr uint16_t kEtRel = 1, kEmRiscv = 243;
constexpr uint32_t kShtProgbits = 1, kShtSymtab = 2, kShtStrtab = 3;
constexpr uint64_t kShfAlloc = 0x2, kShfExec = 0x4;
constexpr unsigned char kStbLocal = 0, kStbGlobal = 1, kSttSection = 3, kSttFunc = 2, kSttFile = 4;

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

template <class T>
void put(std::vector<unsigned char>& out, size_t at, const T& v) {
    std::memcpy(out.data() + at, &v, sizeof(T));  // the writer runs on little-endian hosts only
}

}  // namespace

extern "C" ptl_status ptl_write_elf(const uint32_t* words, size_t n_words, const uint32_t* func_starts,
                                    const uint32_t* func_ends, size_t n_funcs, uint8_t* out, size_t capacity,
                                    size_t* size) {
    if (!size || (n_words && !words) || (n_funcs && (!func_starts || !func_ends))) return PTL_BAD_ARGUMENT;
    if (n_words > (1ull << 40) || n_funcs > (1ull << 31)) return PTL_BAD_ARGUMENT;
    for (size_t f = 0; f < n_funcs; ++f) {
        if (func_starts[f] > func_ends[f] || func_ends[f] > n_words) return PTL_BAD_ARGUMENT;
        if (f && func_starts[f] < func_starts[f - 1]) return PTL_BAD_ARGUMENT;  // address order
    }
    // string tables
    const std::string shstr = std::string("\0.text\0.symtab\0.strtab\0.shstrtab\0", 33);
    const uint32_t n_text = 1, n_symtab = 7, n_strtab = 15, n_shstrtab = 23;
    std::string str(1, '\0');
    const uint32_t file_name = static_cast<uint32_t>(str.size());
    str += "ptilopsis_gb300";
    str.push_back('\0');
    std::vector<uint32_t> fname(n_funcs);
    for (size_t f = 0; f < n_funcs; ++f) {
        fname[f] = static_cast<uint32_t>(str.size());
        str += "func" + std::to_string(f);
        str.push_back('\0');
    }
    // layout: header, .text, .symtab, .strtab, .shstrtab, section headers
    const size_t text_off = 64, text_size = 4 * n_words;
    const size_t sym_off = align_up(text_off + text_size, 8), nsym = 3 + n_funcs, sym_size = 24 * nsym;
    const size_t str_off = sym_off + sym_size, shstr_off = str_off + str.size();
    const size_t sh_off = align_up(shstr_off + shstr.size(), 8), total = sh_off + 5 * 64;
    *size = total;
    if (!out) return PTL_OK;
    if (capacity < total) return PTL_BAD_ARGUMENT;

    std::vector<unsigned char> b(total, 0);
    Ehdr h{};
    const unsigned char ident[16] = {0x7F, 'E', 'L', 'F', 2 /*64-bit*/, 1 /*little-endian*/, 1 /*version*/, 0 /*SysV*/};
    std::memcpy(h.ident, ident, 16);
    h.type = kEtRel;
    h.machine = kEmRiscv;
    h.version = 1;
    h.shoff = sh_off;
    h.ehsize = 64;
    h.shentsize = 64;
    h.shnum = 5;
    h.shstrndx = 4;
    put(b, 0, h);
    if (text_size) std::memcpy(b.data() + text_off, words, text_size);
    // symbols: null, the file, the .text section, then the functions (all global)
    Sym s{};
    put(b, sym_off, s);
    s.name = file_name;
    s.info = static_cast<unsigned char>((kStbLocal << 4) | kSttFile);
    s.shndx = 0xFFF1;  // SHN_ABS
    put(b, sym_off + 24, s);
    s = Sym{};
    s.info = static_cast<unsigned char>((kStbLocal << 4) | kSttSection);
    s.shndx = 1;
    put(b, sym_off + 48, s);
    for (size_t f = 0; f < n_funcs; ++f) {
        Sym fs{};
        fs.name = fname[f];
        fs.info = static_cast<unsigned char>((kStbGlobal << 4) | kSttFunc);
        fs.shndx = 1;
        fs.value = 4ull * func_starts[f];
        fs.size = 4ull * (func_ends[f] - func_starts[f]);
        put(b, sym_off + 24 * (3 + f), fs);
    }
    std::memcpy(b.data() + str_off, str.data(), str.size());
    std::memcpy(b.data() + shstr_off, shstr.data(), shstr.size());
    // section headers: null, .text, .symtab, .strtab, .shstrtab
    Shdr t{};
    t.name = n_text;
    t.type = kShtProgbits;
    t.flags = kShfAlloc | kShfExec;
    t.offset = text_off;
    t.size = text_size;
    t.addralign = 4;
    put(b, sh_off + 64, t);
    Shdr y{};
    y.name = n_symtab;
    y.type = kShtSymtab;
    y.offset = sym_off;
    y.size = sym_size;
    y.link = 3;   // .strtab
    y.info = 3;   // first global symbol
    y.addralign = 8;
    y.entsize = 24;
    put(b, sh_off + 128, y);
    Shdr z{};
    z.name = n_strtab;
    z.type = kShtStrtab;
    z.offset = str_off;
    z.size = str.size();
    z.addralign = 1;
    put(b, sh_off + 192, z);
    Shdr q{};
    q.name = n_shstrtab;
    q.type = kShtStrtab;
    q.offset = shstr_off;
    q.size = shstr.size();
    q.addralign = 1;
    put(b, sh_off + 256, q);
    std::memcpy(out, b.data(), total);
    return PTL_OK;
}
