"""The oracle's Blitter restatement (sw::Blitter, src/Device/Blitter.cpp) on
known answers: fastClear's packing, the byte-averaging resolve against the
float averaging blit, the bilinear 2x reduction, sRGB encode and decode, D16
clears, and the clamp of float into 8-bit formats."""
import numpy as np
import pytest

from swiftshader_gb300 import abi


def test_fast_clear_packing(oracle_mod):
    """fastClear (Blitter.cpp:216-227): (uint32_t)(255 * c + 0.5f) after the
    clamp to [0, 1], B8G8R8A8 stores B, G, R, A."""
    a = np.zeros((3, 5, 4), np.uint8)
    oracle_mod.clear(a, abi.FORMAT_R8G8B8A8_UNORM, (0.5, 1.2, -1.0, 0.25))
    assert (a == [128, 255, 0, 64]).all()
    oracle_mod.clear(a, abi.FORMAT_B8G8R8A8_UNORM, (0.5, 1.2, -1.0, 0.25))
    assert (a == [0, 255, 128, 64]).all()
    # 0.5 / 255 steps round half up, not to even: 2.5 -> 3
    oracle_mod.clear(a, abi.FORMAT_R8G8B8A8_UNORM, (2 / 255, 2.5 / 255, 3.5 / 255, 1.0))
    assert list(a[0, 0]) == [2, 3, 4, 255]


def test_clear_area_and_samples(oracle_mod):
    a = np.full((4, 6, 7), 9, np.uint8)
    oracle_mod.clear(a, abi.FORMAT_S8_UINT, 0x1A5, samples=4, area=(2, 1, 3, 4))
    assert (a[:, 1:5, 2:5] == 0xA5).all()
    a[:, 1:5, 2:5] = 9
    assert (a == 9).all()


def test_clear_depth(oracle_mod):
    """D32_SFLOAT keeps the float's bits (no clamp); D16_UNORM rounds
    z * 0xFFFF half to even after the clamp to [0, 1]."""
    d = np.zeros((2, 2), np.float32)
    oracle_mod.clear(d, abi.FORMAT_D32_SFLOAT, 1.5)
    assert (d == 1.5).all()
    h = np.zeros((2, 2), np.uint16)
    oracle_mod.clear(h, abi.FORMAT_D16_UNORM, 0.5)
    assert (h == 32768).all()  # 32767.5 -> even
    oracle_mod.clear(h, abi.FORMAT_D16_UNORM, 2.0)
    assert (h == 65535).all()


def test_clear_srgb_and_float(oracle_mod):
    """The blit routine's constant colour: sRGB encodes with linearToSRGB
    (Pow<Mediump>); half and float formats store the value unclamped."""
    a = np.zeros((2, 2, 4), np.uint8)
    oracle_mod.clear(a, abi.FORMAT_R8G8B8A8_SRGB, (0.5, 0.2, 0.0, 1.0))
    exact = [1.055 * 0.5 ** (1 / 2.4) - 0.055, 1.055 * 0.2 ** (1 / 2.4) - 0.055]
    assert abs(int(a[0, 0, 0]) - exact[0] * 255) <= 1 and abs(int(a[0, 0, 1]) - exact[1] * 255) <= 1
    assert list(a[0, 0, 2:]) == [0, 255]
    f = np.zeros((2, 2, 4), np.float32)
    oracle_mod.clear(f, abi.FORMAT_R32G32B32A32_SFLOAT, (1.5, -2.0, 1e-39, 0.25))
    assert f[0, 0, 0] == 1.5 and f[0, 0, 1] == -2.0 and f[0, 0, 2] == np.float32(1e-39)  # subnormal kept
    hf = np.zeros((2, 2, 4), np.uint16)
    oracle_mod.clear(hf, abi.FORMAT_R16G16B16A16_SFLOAT, (1.5, -2.0, 0.0, 65504.0))
    assert list(hf[0, 0].view(np.float16)) == [1.5, -2.0, 0.0, 65504.0]


def test_resolve_paths(oracle_mod):
    """Whole R8G8B8A8_UNORM images take the cascaded rounding-up byte average
    (averageByte4 / pavgb): samples 0, 0, 0, 1 give 1.  A region takes the
    float averaging blit: RoundInt(0.25) = 0."""
    s = np.zeros((4, 2, 2, 4), np.uint8)
    s[3] = 1
    d = np.full((2, 2, 4), 7, np.uint8)
    oracle_mod.resolve(s, d, abi.FORMAT_R8G8B8A8_UNORM)
    assert (d == 1).all()
    oracle_mod.resolve(s, d, abi.FORMAT_R8G8B8A8_UNORM, region=(0, 0, 0, 0, 1, 1))
    assert (d[0, 0] == 0).all() and (d[1, 1] == 1).all()
    # byte average of 255 and 0 twice: (255 + 0 + 1) >> 1 = 128, then 128
    s[:] = 0
    s[0] = 255
    s[2] = 255
    oracle_mod.resolve(s, d, abi.FORMAT_R8G8B8A8_UNORM)
    assert (d == 128).all()


def test_resolve_float_sum_order(oracle_mod):
    """Float resolves sum the samples in order and scale by 1/4:
    ((1e8 + 1) + -1e8 + 1) * 0.25 = 0.25 in binary32."""
    s = np.zeros((4, 1, 1, 4), np.float32)
    s[:, 0, 0, 0] = [1e8, 1.0, -1e8, 1.0]
    d = np.zeros((1, 1, 4), np.float32)
    oracle_mod.resolve(s, d, abi.FORMAT_R32G32B32A32_SFLOAT)
    assert d[0, 0, 0] == np.float32(((np.float32(1e8) + np.float32(1)) + np.float32(-1e8) + np.float32(1)) * np.float32(0.25))


def test_bilinear_half_reduction(oracle_mod):
    """A LINEAR 2x reduction samples between four texels with weights 1/2:
    the float result is ((a * .5 + b * .5) * .5 + (c * .5 + d * .5) * .5)."""
    t = np.arange(8 * 8 * 4, dtype=np.float32).reshape(8, 8, 4) * np.float32(0.37)
    m = np.zeros((4, 4, 4), np.float32)
    oracle_mod.blit(t, abi.FORMAT_R32G32B32A32_SFLOAT, m, abi.FORMAT_R32G32B32A32_SFLOAT, (0, 0, 8, 8), (0, 0, 4, 4),
                    abi.FILTER_LINEAR)
    h = np.float32(0.5)
    for y in range(4):
        for x in range(4):
            a, b, c, d = t[2 * y, 2 * x], t[2 * y, 2 * x + 1], t[2 * y + 1, 2 * x], t[2 * y + 1, 2 * x + 1]
            assert np.array_equal(m[y, x], (a * h + b * h) * h + (c * h + d * h) * h)


def test_nearest_copy_and_mirror(oracle_mod):
    """NEAREST at scale 1 copies texels; reversed destination corners mirror."""
    rng = np.random.default_rng(5)
    t = rng.integers(0, 256, size=(6, 9, 4), dtype=np.uint8)
    o = np.zeros_like(t)
    oracle_mod.blit(t, abi.FORMAT_R8G8B8A8_UNORM, o, abi.FORMAT_R8G8B8A8_UNORM, (0, 0, 9, 6), (0, 0, 9, 6),
                    abi.FILTER_NEAREST)
    assert np.array_equal(o, t)
    oracle_mod.blit(t, abi.FORMAT_R8G8B8A8_UNORM, o, abi.FORMAT_R8G8B8A8_UNORM, (0, 0, 9, 6), (9, 0, 0, 6),
                    abi.FILTER_NEAREST)
    assert np.array_equal(o, t[:, ::-1])
    b = np.zeros_like(t)
    oracle_mod.blit(t, abi.FORMAT_R8G8B8A8_UNORM, b, abi.FORMAT_B8G8R8A8_UNORM, (0, 0, 9, 6), (0, 0, 9, 6),
                    abi.FILTER_NEAREST)
    assert np.array_equal(b, t[..., [2, 1, 0, 3]])


def test_float_into_unorm_clamps(oracle_mod):
    """Float sources scale by 255 and clamp to [0, 255] before RoundInt."""
    t = np.array([[[-0.5, 0.5, 1.5, 0.2]]], np.float32)
    o = np.zeros((1, 1, 4), np.uint8)
    oracle_mod.blit(t, abi.FORMAT_R32G32B32A32_SFLOAT, o, abi.FORMAT_R8G8B8A8_UNORM, (0, 0, 1, 1), (0, 0, 1, 1),
                    abi.FILTER_NEAREST)
    assert list(o[0, 0]) == [0, 128, 255, 51]  # 127.5 -> 128 (even), 51.0


def test_srgb_round_trip(oracle_mod):
    """UNORM -> sRGB -> UNORM through two NEAREST blits returns every byte
    within one step (the mediump power curves are not exact inverses)."""
    t = np.tile(np.arange(256, dtype=np.uint8)[:, None], (1, 4)).reshape(16, 16, 4)
    e = np.zeros_like(t)
    back = np.zeros_like(t)
    oracle_mod.blit(t, abi.FORMAT_R8G8B8A8_UNORM, e, abi.FORMAT_R8G8B8A8_SRGB, (0, 0, 16, 16), (0, 0, 16, 16), 0)
    oracle_mod.blit(e, abi.FORMAT_R8G8B8A8_SRGB, back, abi.FORMAT_R8G8B8A8_UNORM, (0, 0, 16, 16), (0, 0, 16, 16), 0)
    assert np.max(np.abs(back.astype(int) - t.astype(int))) <= 1
    assert np.array_equal(back[..., 3], t[..., 3])  # alpha is linear
