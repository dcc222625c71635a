"""Pins the oracle's numeric primitives to the reference's own Reactor
known-answer tests (tests/ReactorUnitTests/ReactorUnitTests.cpp) and to the x86
instruction semantics the reference's JIT emits."""
import struct

import numpy as np
import pytest


def f32(x):
    return struct.unpack("<f", struct.pack("<f", x))[0]


def test_round_int_known_answers(oracle_mod):
    L = oracle_mod.lib()
    # ReactorUnitTests.cpp:1495-1533 (RoundInt)
    assert [L.oracle_round_int(v) for v in (3.1, 3.6, -3.1, -3.6)] == [3, 4, -3, -4]
    # cvtps2dq rounds half to even and returns 0x80000000 out of range
    assert [L.oracle_round_int(v) for v in (2.5, 3.5, -2.5, 0.5)] == [2, 4, -2, 0]
    assert L.oracle_round_int(2147483648.0) == -2147483648
    assert L.oracle_round_int(float("nan")) == -2147483648


def test_round_int_clamped_known_answers(oracle_mod):
    L = oracle_mod.lib()
    # ReactorUnitTests.cpp:1503,1525-1533 (RoundIntClamped)
    assert L.oracle_round_int_clamped(2147483648.0) >= 2147483520
    assert L.oracle_round_int_clamped(-2147483648.0) < -2147483647
    assert L.oracle_round_int_clamped(2147483520.0) == 2147483520
    assert L.oracle_round_int_clamped(-2147483520.0) == -2147483520
    assert L.oracle_round_int_clamped(float("nan")) == 0  # fptosi.sat


def test_mulhigh_known_answers(oracle_mod):
    L = oracle_mod.lib()
    # ReactorUnitTests.cpp:1813-1878 (MulHigh, Short4 and UShort4 rows)
    a = (0x01AA, 0x02DD, 0x03EE, 0xF422)
    b = (0x01BB, 0x02CC, 0x03FF, 0xF411)
    s = [L.oracle_mulhigh_s16(np.int16(np.uint16(x)), np.int16(np.uint16(y))) & 0xFFFF for x, y in zip(a, b)]
    u = [L.oracle_mulhigh_u16(x, y) for x, y in zip(a, b)]
    assert (s[1] << 16 | s[0]) == 0x00080002 and (s[3] << 16 | s[2]) == 0x008D000F
    assert (u[1] << 16 | u[0]) == 0x00080002 and (u[3] << 16 | u[2]) == 0xE8C0000F


def test_fmuladd_is_fused(oracle_mod):
    L = oracle_mod.lib()
    # ReactorUnitTests.cpp:1207-1250: with FMA available MulAdd equals fmaf
    x, y, z = f32(1.00000011920929), 53400708.0, -53400708.0
    exact = float(np.float32(np.float64(np.float32(x)) * np.float64(np.float32(y)) + np.float64(np.float32(z))))
    assert L.oracle_fmuladd(x, y, z) == exact
    assert L.oracle_fmuladd(x, y, z) != float(np.float32(np.float32(x) * np.float32(y)) + np.float32(z))
    assert L.oracle_fmuladd(2.0, 3.0, 0.0) == 6.0 and L.oracle_fmuladd(4.0, 0.0, 7.0) == 7.0


def test_ftz_daz(oracle_mod):
    L = oracle_mod.lib()
    tiny = struct.unpack("<f", struct.pack("<I", 0x00000010))[0]
    assert L.oracle_ftz(tiny) == 0.0
    neg = struct.unpack("<f", struct.pack("<I", 0x80000010))[0]
    r = L.oracle_ftz(neg)
    assert r == 0.0 and struct.pack("<f", r) == struct.pack("<I", 0x80000000)
    # a product that underflows to a subnormal flushes to zero
    assert L.oracle_fmuladd(1e-20, 1e-20, 0.0) == 0.0


def test_trunc_and_log2sqrt(oracle_mod):
    L = oracle_mod.lib()
    assert [L.oracle_trunc_int(v) for v in (2.9, -2.9, 0.0)] == [2, -2, 0]
    assert L.oracle_trunc_int(3e9) == -2147483648  # cvttss2si overflow
    # log2sqrt(x) ~ log2(sqrt(x)) within the bit trick's error, exact at powers of 4
    for v in (1.0, 4.0, 16.0, 0.25):
        assert L.oracle_log2sqrt(v) == pytest.approx(np.log2(np.sqrt(v)), abs=1e-6)
    assert abs(L.oracle_log2sqrt(10.0) - np.log2(np.sqrt(10.0))) < 0.05
