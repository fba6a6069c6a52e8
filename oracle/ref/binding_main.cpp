// Build check of include/rv_generator_gb300.hpp against the reference's own headers and
// objects (test infrastructure).  It does what src/main.cpp:119-157 does with the GPU
// generator in place of rv_generator_avx: parse a Pareas source with the reference's
// front end, flatten it (DepthTree), construct rv_generator_gb300, process, and write
// the assembly listing (inherited to_asm) and the raw words (inherited to_binary).
//
//   binding_check [-s] <input.in> <out.S> <out.bin>     (-s: the scalar generator)
//
// Exit status: 0 on success; 3 with the exception text on stderr when the GPU generator
// throws (for instance on a host without a GPU); 2 when the front end fails.
#include <fstream>
#include <iostream>
#include <memory>
#include <string>

#include "codegen/astnode.hpp"
#include "codegen/depthtree.hpp"
#include "codegen/lexer.hpp"
#include "codegen/parser.hpp"
#include "codegen/symtab.hpp"

#include "rv_generator_gb300.hpp"

int main(int argc, char** argv) {
    const bool scalar = argc == 5 && std::string(argv[1]) == "-s";
    if (scalar) ++argv, --argc;
    if (argc != 4) {
        std::cerr << "usage: binding_check [-s] <input.in> <out.S> <out.bin>\n";
        return 1;
    }
    std::unique_ptr<ASTNode> node;
    std::unique_ptr<DepthTree> tree;
    try {
        std::ifstream input(argv[1]);
        Lexer lexer(input);
        SymbolTable symtab;
        Parser parser(lexer, symtab);
        node.reset(parser.parse());
        node->resolveType();
        tree = std::make_unique<DepthTree>(node.get());
    } catch (const std::exception& e) {
        std::cerr << "front end: " << e.what() << '\n';
        return 2;
    }
    try {
        std::unique_ptr<rv_generator> gen = std::make_unique<rv_generator_gb300>(*tree, 0, scalar);
        gen->process(true);
        std::ofstream asm_out(argv[2]);
        gen->to_asm(asm_out);
        std::ofstream bin_out(argv[3], std::ios::binary);
        gen->to_binary(bin_out);
    } catch (const std::exception& e) {
        std::cerr << "rv_generator_gb300: " << e.what() << '\n';
        return 3;
    }
    return 0;
}
