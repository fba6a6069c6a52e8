"""ELF wrapping of compiled words (ptl_write_elf): an ELF64 little-endian RISC-V
relocatable object whose .text is the words and whose symbols are the functions of the
function table, named like the reference disassembler's labels.  Checked by parsing the
file here, and with readelf where the host has it; no GPU needed (the words are the
reference's golden output)."""
from __future__ import annotations

import shutil
import struct
import subprocess

import numpy as np
import pytest

from conftest import load_fixture


def _sections(blob: bytes):
    (shoff,) = struct.unpack_from("<Q", blob, 0x28)
    shnum, shstrndx = struct.unpack_from("<HH", blob, 0x3C)
    hdrs = [struct.unpack_from("<IIQQQQIIQQ", blob, shoff + 64 * k) for k in range(shnum)]
    names = hdrs[shstrndx]
    def name(off):
        s = blob[names[4] + off:]
        return s[:s.index(b"\0")].decode()
    return {name(h[0]): h for h in hdrs}


def test_elf_object_holds_the_words_and_functions(built_cuda, tmp_path):
    from ptilopsis_gb300 import to_elf
    _, gold = load_fixture("pareas_basic_3_in")
    words, starts, ends = gold["words"], gold["fn_start"], gold["fn_end"]
    blob = to_elf(words, starts, ends)
    assert blob[:4] == b"\x7fELF" and blob[4] == 2 and blob[5] == 1
    e_type, e_machine = struct.unpack_from("<HH", blob, 16)
    assert (e_type, e_machine) == (1, 243)  # ET_REL, EM_RISCV
    sec = _sections(blob)
    assert set(sec) >= {".text", ".symtab", ".strtab", ".shstrtab"}
    text = sec[".text"]
    np.testing.assert_array_equal(np.frombuffer(blob, "<u4", text[5] // 4, text[4]), words)
    sym, strtab = sec[".symtab"], sec[".strtab"]
    nsym = sym[5] // 24
    assert nsym == 3 + len(starts)
    for f in range(len(starts)):
        name_off, info, _, shndx, value, size = struct.unpack_from("<IBBHQQ", blob, sym[4] + 24 * (3 + f))
        s = blob[strtab[4] + name_off:]
        assert s[:s.index(b"\0")].decode() == f"func{f}"
        assert info == 0x12 and shndx == 1  # global function in .text
        assert value == 4 * int(starts[f]) and size == 4 * int(ends[f] - starts[f])
    if shutil.which("readelf"):
        path = tmp_path / "prog.o"
        path.write_bytes(blob)
        res = subprocess.run(["readelf", "-h", "-S", "-s", "-W", str(path)], capture_output=True, text=True)
        assert res.returncode == 0 and "RISC-V" in res.stdout and "func0" in res.stdout, res.stdout + res.stderr
        assert "Warning" not in res.stderr and "Error" not in res.stderr, res.stderr


def test_elf_rejects_inconsistent_tables(built_cuda):
    from ptilopsis_gb300 import PtlError, to_elf
    words = np.arange(10, dtype=np.uint32)
    with pytest.raises(PtlError):
        to_elf(words, np.array([0, 5], np.uint32), np.array([5, 11], np.uint32))  # past the words
    with pytest.raises(PtlError):
        to_elf(words, np.array([5, 0], np.uint32), np.array([10, 5], np.uint32))  # not in address order
    assert to_elf(np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.uint32))[:4] == b"\x7fELF"
