"""ptilopsis_gb300: a GB300 (sm_103a) implementation of Ptilopsis's data-parallel RISC-V
code generator.

The compute path is hand-written CUDA behind the C ABI of include/ptl_codegen.h
(libptl_gb300.so); this package is the Python host mirror of the reference's
rv_generator interface plus the seeded synthetic program generator used by the
benchmarks.
"""
from .codegen import (DepthTree, PtlError, RvGenerator, SNAPSHOTS, STAGES, code_table,
                      compile_tree, depth_order, device_info, disassemble, flatten, library_path,
                      to_asm, to_elf)

__all__ = ["DepthTree", "PtlError", "RvGenerator", "SNAPSHOTS", "STAGES", "code_table", "compile_tree",
           "depth_order", "device_info", "disassemble", "flatten", "library_path", "to_asm", "to_elf"]
