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


def _ulp16(ref, val):
    """ULP_16 of the reference's MathUnitTests (tests/MathUnitTests/unittests.cpp:149-156):
    |val - ref| in units of ref's 16-bit-float last place."""
    ref = np.asarray(ref, dtype=np.float32)
    x1 = (ref.view(np.uint32) ^ np.uint32(0x2000)).view(np.float32).astype(np.float64)
    return np.abs(np.asarray(val, np.float64) - ref.astype(np.float64)) / np.abs(x1 - ref.astype(np.float64))


def test_log2_mediump_bounds(oracle_mod):
    """Log2 at relaxed precision (ShaderCore.cpp:406-470) against the bounds the
    reference's Log2RelaxedExhaustive asserts (unittests.cpp:183-247): exact at
    powers of two, within 2^-7 absolute on [0.5, 2], within 3 ULP-16 elsewhere.
    Sampled every 97th bit pattern of the positive floats instead of all."""
    bits = np.arange(0x00800000, 0x7F800000, 97, dtype=np.uint32)
    x = bits.view(np.float32)
    val = oracle_mod.transcendental("log2_mediump", x).astype(np.float64)
    ref = np.log2(x.astype(np.float64))
    exact = ref == np.round(ref)
    assert np.array_equal(val[exact], ref[exact])
    p2 = (2.0 ** np.arange(-126, 128)).astype(np.float32)
    assert np.array_equal(oracle_mod.transcendental("log2_mediump", p2), np.arange(-126, 128, dtype=np.float32))
    mid = (x >= 0.5) & (x <= 2.0) & ~exact
    assert np.max(np.abs(val[mid] - ref[mid])) <= 2.0 ** -7
    rest = ~mid & ~exact
    assert np.max(_ulp16(ref[rest].astype(np.float32), val[rest])) < 3.0
    assert oracle_mod.transcendental("log2_mediump", np.array([np.inf], np.float32))[0] == np.inf


def test_exp2_mediump_bounds(oracle_mod):
    """Exp2 at relaxed precision (ShaderCore.cpp:336-386) against
    Exp2RelaxedExhaustive (unittests.cpp:266-305): exact at integers, within
    (1 + 2|x|) ULP-16 on [-10, 10]; clamped to [-126.999992, 128]."""
    x = np.linspace(-10.0, 10.0, 2_000_001, dtype=np.float32)
    val = oracle_mod.transcendental("exp2_mediump", x)
    ref = np.exp2(x.astype(np.float64)).astype(np.float32)
    ints = np.arange(-10, 11, dtype=np.float32)
    assert np.array_equal(oracle_mod.transcendental("exp2_mediump", ints), np.exp2(ints))
    assert np.all(_ulp16(ref, val) <= 1.0 + 2.0 * np.abs(x))
    assert oracle_mod.transcendental("exp2_mediump", np.array([200.0], np.float32))[0] == np.inf  # 2^128 bits


def test_srgb_transfer(oracle_mod):
    """linearToSRGB / sRGBtoLinear of colour attachments (ShaderCore.cpp:914-930):
    the linear segment below the knee is exact arithmetic; above it the mediump
    power keeps the 8-bit encode within one step of the exact curve
    (sw::linearToSRGB, src/System/Math.hpp:338-348) and the decode within 2e-3."""
    c = np.linspace(0.0, 1.0, 100_001, dtype=np.float32)
    enc = oracle_mod.transcendental("linear_to_srgb", c).astype(np.float64)
    c64 = c.astype(np.float64)
    exact = np.where(c64 <= 0.0031308, c64 * 12.92, 1.055 * c64 ** (1 / 2.4) - 0.055)
    assert np.max(np.abs(np.rint(np.clip(enc, 0, 1) * 255) - np.rint(exact * 255))) <= 1
    low = c < np.float32(0.0031308)
    assert np.array_equal(enc[low], (c[low] * np.float32(12.92)).astype(np.float64))
    dec = oracle_mod.transcendental("srgb_to_linear", c).astype(np.float64)
    exact_d = np.where(c64 <= 0.04045, c64 / 12.92, ((c64 + 0.055) / 1.055) ** 2.4)
    assert np.max(np.abs(dec - exact_d)) < 2e-3
    # monotonic on the 8-bit decode grid the blend reads (b * 257 / 0xFFFF)
    grid = (np.arange(256, dtype=np.float32) * np.float32(257)) * np.float32(1.0 / 0xFFFF)
    assert np.all(np.diff(oracle_mod.transcendental("srgb_to_linear", grid)) > 0)
