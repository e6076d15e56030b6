"""CPU-only checks of the product library: it builds, loads, exports every
symbol the public header declares, and its host-side pieces (the replay of
the reference's random stream, Philox) are right. No CUDA calls."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _lib():
    from beofaunus_gb300 import build
    build.build()
    return ctypes.CDLL(build.LIB)


def declared_symbols():
    names = set()
    for h in ("faunus_gb300.h",):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(fg_\w+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = _lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s


def test_philox_known_answers():
    """Random123's published known-answer vectors for Philox4x32-10."""
    from beofaunus_gb300.gpu import philox4x32_10
    kat = [
        ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
        ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
        ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
         (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
    ]
    for ctr, key, want in kat:
        got = philox4x32_10(ctr, key)
        assert [hex(x) for x in got] == [hex(x) for x in want]


def test_params_layout_matches_header():
    """ctypes mirror of fg_params has the C layout (offset of the last field)."""
    from beofaunus_gb300.params import FgParams
    # 2 int32, 3+1 double, 4x16 double, 5 double, 2 int32, 5 double, 1 double, 8 int32
    expected = 8 + 32 + 4 * 16 * 8 + 5 * 8 + 8 + 4 * 8 + 8 + 8 * 4
    assert ctypes.sizeof(FgParams) == expected


def test_oracle_philox_matches_library():
    """The oracle's Philox restatement and the library's agree."""
    from beofaunus_gb300.gpu import philox4x32_10
    from oracle.oracle import philox
    rng = np.random.default_rng(0)
    for _ in range(20):
        c = rng.integers(0, 2 ** 32, 4, dtype=np.uint64).astype(np.uint32)
        k = rng.integers(0, 2 ** 32, 2, dtype=np.uint64).astype(np.uint32)
        np.testing.assert_array_equal(philox(c, k), philox4x32_10(c, k))


def test_dipole_draws_match_oracle():
    """fg_dip_draw_stream (host code in the library) and the oracle's
    restatement of the reference's AtomicRotation / AtomicTranslation draws
    give the same trials, both with drawn and with given move kinds."""
    from beofaunus_gb300.gpu import dip_draw_stream, mol_draw_stream
    from oracle.oracle import dip_stream, mol_stream
    a = dip_draw_stream(5489, 100, 4000, p_rotate=0.4, dp=0.7, dprot=4.7)
    b = dip_stream(5489, 100, 4000, 0.4, 0.7, 4.7)
    for k in ("kind", "idx", "axis", "angle", "disp", "u"):
        np.testing.assert_array_equal(a[k], b[k])
    kinds = np.tile([1] * 50 + [2] * 50, 20)
    a = dip_draw_stream(7, 50, len(kinds), dp=0.5, dprot=1.0, kinds=kinds)
    b = dip_stream(7, 50, len(kinds), 0.0, 0.5, 1.0, kinds=kinds)
    for k in ("kind", "idx", "axis", "angle", "disp", "u"):
        np.testing.assert_array_equal(a[k], b[k])
    np.testing.assert_array_equal(a["kind"], kinds)
    m1 = mol_draw_stream(11, 1000, 500, 1.0, 0.3, True)
    m2 = mol_stream(11, 1000, 1.0, 0.3, True, 500)
    for k in ("group", "axis", "angle", "trans", "u"):
        np.testing.assert_array_equal(m1[k], m2[k])
