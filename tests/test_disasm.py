"""Text output (to_asm and the disassembler listing) against the reference's own
rv_generator::to_asm and rvdisasm::disassemble, built from its sources: the generated
words of the golden fixtures, and words that reach every decoding branch, including the
reference's choices for encodings the generator never emits.  Host code; no GPU."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import manifest


def _ref():
    from oracle import refbind
    if not refbind.build() or not refbind.available():
        pytest.skip("reference not buildable on this host")
    return refbind


def _corner_words():
    """Every opcode × funct3 × a spread of funct7 values, with random other fields."""
    rng = np.random.default_rng(0x50544D10)
    out = []
    for opc in range(128):
        for f3 in range(8):
            for f7 in (0x00, 0x01, 0x04, 0x08, 0x0C, 0x10, 0x14, 0x20, 0x2C, 0x50, 0x60, 0x68, 0x70, 0x78, 0x7F,
                       int(rng.integers(0, 128))):
                for rs2 in (0, 1, int(rng.integers(2, 32))):
                    w = (opc | (int(rng.integers(0, 32)) << 7) | (f3 << 12) | (int(rng.integers(0, 32)) << 15)
                         | (rs2 << 20) | (f7 << 25))
                    out.append(w)
    out += [0, 0xFFFFFFFF, 0x80000063, 0x80000067, 0x8000006F, 0xFFFFF0EF]
    return np.array(out, np.uint32)


def test_to_asm_matches_reference_on_generated_words(built):
    ref = _ref()
    from ptilopsis_gb300 import disassemble, to_asm
    from conftest import load_fixture
    for fx in manifest()["fixtures"]:
        _, golden = load_fixture(fx["name"])
        words = golden["words"]
        assert to_asm(words) == ref.to_asm(words), fx["name"]
        starts = golden["fn_start"].astype(np.uint64)
        assert disassemble(words, 0, starts) == ref.disassemble(words, 0, starts), fx["name"]


def test_to_asm_matches_reference_on_every_encoding(built):
    ref = _ref()
    from ptilopsis_gb300 import to_asm
    words = _corner_words()
    rng = np.random.default_rng(0x50544D11)
    words = np.concatenate([words, rng.integers(0, 1 << 32, 20000, dtype=np.uint64).astype(np.uint32)])
    got, want = to_asm(words).splitlines(), ref.to_asm(words).splitlines()
    assert len(got) == len(want) == len(words)
    bad = [(hex(int(w)), g, r) for w, g, r in zip(words, got, want) if g != r]
    assert not bad, bad[:5]


@pytest.mark.parametrize("n,start,funcs", [(1, 0, [0]), (17, 0x400, [0, 3, 16]), (300, 0, [0, 7, 11, 12, 299]),
                                           (5000, 0x1000, [1, 1024, 2049, 3000, 4096 + 0x400])])
def test_disassembly_listing_matches_reference(built, n, start, funcs):
    ref = _ref()
    from ptilopsis_gb300 import disassemble
    words = np.resize(_corner_words(), n)
    assert disassemble(words, start, funcs) == ref.disassemble(words, start, funcs)
