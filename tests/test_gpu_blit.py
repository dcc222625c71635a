"""GPU parity of the Blitter steps either side of a draw (swgb_clear,
swgb_resolve, swgb_blit) against the oracle's restatement of sw::Blitter:
every byte of the destination compared, including the bytes around a cleared
or blitted area (pre-filled with noise)."""
import numpy as np
import pytest

from swiftshader_gb300 import abi

pytestmark = pytest.mark.gpu

COLOUR = [abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_B8G8R8A8_UNORM, abi.FORMAT_R8G8B8A8_SRGB, abi.FORMAT_B8G8R8A8_SRGB,
          abi.FORMAT_R16G16B16A16_SFLOAT, abi.FORMAT_R32G32B32A32_SFLOAT]
NP = {abi.FORMAT_R16G16B16A16_SFLOAT: (np.uint16, 4), abi.FORMAT_R32G32B32A32_SFLOAT: (np.float32, 4),
      abi.FORMAT_D32_SFLOAT: (np.float32, None), abi.FORMAT_D16_UNORM: (np.uint16, None), abi.FORMAT_S8_UINT: (np.uint8, None)}


def host_image(rng, fmt, h, w, samples=1, denormals=False):
    """Random contents of an image of fmt, as the numpy array the oracle takes."""
    dt, comps = NP.get(fmt, (np.uint8, 4))
    shape = ((samples,) if samples > 1 else ()) + (h, w) + ((comps,) if comps else ())
    if dt == np.float32:
        a = rng.uniform(-0.25, 1.5, size=shape).astype(np.float32)
        if denormals:
            a.reshape(-1)[::7] = np.float32(1e-39) * rng.integers(1, 100, size=a.reshape(-1)[::7].shape)
        return a
    if fmt == abi.FORMAT_R16G16B16A16_SFLOAT:
        a = rng.uniform(-0.25, 1.5, size=shape).astype(np.float16).view(np.uint16)
        if denormals:
            # half subnormals, zeros of both signs, infinities and NaNs (Reactor
            # reads exponent 31 as finite 65536+)
            flat = a.reshape(-1)
            flat[::5] = rng.integers(1, 0x400, size=flat[::5].shape) | (rng.integers(0, 2, size=flat[::5].shape) << 15)
            flat[3::41] = rng.choice(np.array([0x0000, 0x8000, 0x7C00, 0xFC00, 0x7E00, 0x7C01], np.uint16),
                                     size=flat[3::41].shape)
        return a
    return rng.integers(0, np.iinfo(dt).max + 1, size=shape, dtype=np.int64).astype(dt)


def to_device(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gpu_image(t, fmt, samples=1):
    from swiftshader_gb300.renderer import image_view
    return image_view(t, fmt, samples)


def assert_same(got, ref, what):
    g, r = np.ascontiguousarray(got).view(np.uint8), np.ascontiguousarray(ref).view(np.uint8)
    bad = np.flatnonzero(g.reshape(-1) != r.reshape(-1))
    assert bad.size == 0, "%s: %d of %d bytes differ (first at byte %d: %d vs %d)" % (
        what, bad.size, g.size, bad[0], g.reshape(-1)[bad[0]], r.reshape(-1)[bad[0]])


@pytest.fixture(scope="module")
def rend(gpu_lib):
    from swiftshader_gb300 import Renderer
    r = Renderer(0)
    yield r
    r.close()


@pytest.mark.parametrize("fmt", COLOUR + [abi.FORMAT_D32_SFLOAT, abi.FORMAT_D16_UNORM, abi.FORMAT_S8_UINT])
@pytest.mark.parametrize("samples", [1, 4])
def test_clear(rend, oracle_mod, fmt, samples):
    """Whole-image and sub-area clears of every sample plane; values outside
    [0, 1] clamp for normalized formats; odd areas exercise the unaligned row
    heads and tails."""
    import torch
    rng = np.random.default_rng(80 + fmt + samples)
    for (h, w), area, value in [((37, 53), None, (0.5, 1.25, -0.5, 0.2509804)),
                                ((37, 53), (3, 5, 41, 17), (0.1, 0.7354, 0.0031, 1.0)),
                                ((64, 96), (1, 0, 95, 64), (0.03, 0.999, 0.4, 0.5)),
                                ((9, 7), (6, 8, 1, 1), (1e-39, 3.5, 0.25, -0.0))]:
        host = host_image(rng, fmt, h, w, samples)
        dev = to_device(host)
        if fmt == abi.FORMAT_S8_UINT:
            v = int(value[1] * 200) + 1
        elif fmt in (abi.FORMAT_D32_SFLOAT, abi.FORMAT_D16_UNORM):
            v = value[0] if value[0] <= 1 else 0.37
        else:
            v = value
        rend.clear_area(gpu_image(dev, fmt, samples), v, area)
        torch.cuda.synchronize()
        oracle_mod.clear(host, fmt, v, samples=samples, area=area)
        assert_same(dev.cpu().numpy(), host, "clear fmt %d samples %d area %s" % (fmt, samples, area))


@pytest.mark.parametrize("fmt", COLOUR)
@pytest.mark.parametrize("h,w", [(32, 48), (19, 37)])
def test_resolve_whole(rend, oracle_mod, fmt, h, w):
    """Whole-image resolves: the byte-averaging fast path for R8G8B8A8_UNORM /
    B8G8R8A8_UNORM (16-byte and 4-byte accesses), the averaging blit for the
    rest (sRGB decoded per sample and re-encoded; float32 subnormals kept)."""
    import torch
    rng = np.random.default_rng(90 + fmt + w)
    src = host_image(rng, fmt, h, w, 4, denormals=True)
    dst = host_image(rng, fmt, h, w)
    ds, dd = to_device(src), to_device(dst)
    rend.resolve(gpu_image(ds, fmt, 4), gpu_image(dd, fmt))
    torch.cuda.synchronize()
    oracle_mod.resolve(src, dst, fmt)
    assert_same(dd.cpu().numpy(), dst, "resolve fmt %d" % fmt)


@pytest.mark.parametrize("fmt", [abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_R8G8B8A8_SRGB, abi.FORMAT_R16G16B16A16_SFLOAT])
def test_resolve_region(rend, oracle_mod, fmt):
    """A resolve of a region (not the whole image) is the averaging blit for
    every format, R8G8B8A8_UNORM included, with offsets on both sides."""
    import torch
    rng = np.random.default_rng(100 + fmt)
    src = host_image(rng, fmt, 40, 50, 4)
    dst = host_image(rng, fmt, 30, 45)
    ds, dd = to_device(src), to_device(dst)
    region = (7, 3, 2, 5, 33, 21)
    rend.resolve(gpu_image(ds, fmt, 4), gpu_image(dd, fmt), region)
    torch.cuda.synchronize()
    oracle_mod.resolve(src, dst, fmt, region)
    assert_same(dd.cpu().numpy(), dst, "resolve region fmt %d" % fmt)


BLIT_CASES = [
    # (src fmt, dst fmt, src shape, dst shape, src box, dst box, filter)
    (abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_R8G8B8A8_UNORM, (37, 53), (18, 26), (0, 0, 53, 37), (0, 0, 26, 18), 1),
    (abi.FORMAT_R8G8B8A8_SRGB, abi.FORMAT_R8G8B8A8_SRGB, (64, 64), (32, 32), (0, 0, 64, 64), (0, 0, 32, 32), 1),
    (abi.FORMAT_B8G8R8A8_SRGB, abi.FORMAT_B8G8R8A8_SRGB, (33, 17), (16, 8), (0, 0, 17, 33), (0, 0, 8, 16), 1),
    (abi.FORMAT_R16G16B16A16_SFLOAT, abi.FORMAT_R16G16B16A16_SFLOAT, (40, 40), (20, 20), (0, 0, 40, 40), (0, 0, 20, 20), 1),
    (abi.FORMAT_R32G32B32A32_SFLOAT, abi.FORMAT_R32G32B32A32_SFLOAT, (31, 45), (15, 22), (0, 0, 45, 31), (0, 0, 22, 15), 1),
    # magnify, nearest and linear; mirrored destination; source box past the edge
    (abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_R8G8B8A8_UNORM, (16, 16), (50, 40), (2, 3, 14, 12), (40, 45, 3, 1), 0),
    (abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_R8G8B8A8_UNORM, (16, 16), (50, 40), (-3, -2, 19, 20), (1, 2, 37, 47), 1),
    (abi.FORMAT_R32G32B32A32_SFLOAT, abi.FORMAT_R32G32B32A32_SFLOAT, (20, 24), (30, 30), (24, 20, 0, 0), (0, 0, 30, 30), 1),
    # format conversions: encode, decode, float into 8-bit (clamp), swizzle
    (abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_R8G8B8A8_SRGB, (24, 24), (24, 24), (0, 0, 24, 24), (0, 0, 24, 24), 0),
    (abi.FORMAT_B8G8R8A8_SRGB, abi.FORMAT_R32G32B32A32_SFLOAT, (24, 24), (12, 12), (0, 0, 24, 24), (0, 0, 12, 12), 1),
    (abi.FORMAT_R32G32B32A32_SFLOAT, abi.FORMAT_B8G8R8A8_UNORM, (24, 24), (24, 24), (0, 0, 24, 24), (0, 0, 24, 24), 0),
    (abi.FORMAT_R16G16B16A16_SFLOAT, abi.FORMAT_R8G8B8A8_SRGB, (24, 24), (10, 14), (0, 0, 24, 24), (0, 0, 14, 10), 1),
    # exact 2:1 reductions from the origin (the mip-level kernel): odd and even widths, every kind
    (abi.FORMAT_B8G8R8A8_UNORM, abi.FORMAT_B8G8R8A8_UNORM, (48, 66), (24, 33), (0, 0, 66, 48), (0, 0, 33, 24), 1),
    (abi.FORMAT_R32G32B32A32_SFLOAT, abi.FORMAT_R32G32B32A32_SFLOAT, (32, 34), (16, 17), (0, 0, 34, 32), (0, 0, 17, 16), 1),
    (abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_R8G8B8A8_SRGB, (32, 32), (16, 16), (0, 0, 32, 32), (0, 0, 16, 16), 1),
    (abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_R8G8B8A8_UNORM, (33, 35), (16, 17), (0, 0, 34, 32), (0, 0, 17, 16), 1),
]


@pytest.mark.parametrize("case", range(len(BLIT_CASES)))
def test_blit(rend, oracle_mod, case):
    import torch
    sf, df, ss, dsh, sbox, dbox, filt = BLIT_CASES[case]
    rng = np.random.default_rng(110 + case)
    src = host_image(rng, sf, *ss)
    dst = host_image(rng, df, *dsh)
    ds, dd = to_device(src), to_device(dst)
    rend.blit(gpu_image(ds, sf), gpu_image(dd, df), sbox, dbox, filt)
    torch.cuda.synchronize()
    oracle_mod.blit(src, sf, dst, df, sbox, dbox, filt)
    assert_same(dd.cpu().numpy(), dst, "blit case %d" % case)


@pytest.mark.parametrize("fmt", [abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_R8G8B8A8_SRGB, abi.FORMAT_R16G16B16A16_SFLOAT])
def test_generate_mipmaps(rend, oracle_mod, fmt):
    """A full mip chain of a 300 x 200 texture, one LINEAR blit per level
    (odd sizes on the way down), each level from the device's previous one."""
    import torch
    rng = np.random.default_rng(120 + fmt)
    sizes = [(200, 300)]
    while sizes[-1] != (1, 1):
        h, w = sizes[-1]
        sizes.append((max(1, h // 2), max(1, w // 2)))
    host = [host_image(rng, fmt, h, w) for h, w in sizes]
    dev = [to_device(a) for a in host]
    rend.generate_mipmaps([gpu_image(t, fmt) for t in dev])
    torch.cuda.synchronize()
    for i in range(1, len(sizes)):
        (h0, w0), (h1, w1) = sizes[i - 1], sizes[i]
        oracle_mod.blit(host[i - 1], fmt, host[i], fmt, (0, 0, w0, h0), (0, 0, w1, h1), 1)
        assert_same(dev[i].cpu().numpy(), host[i], "mip level %d" % i)


def test_blitter_errors(rend):
    """Host-side validation: mismatched resolve formats, sample counts, areas
    outside the image, value formats, unaligned pitches."""
    import torch
    from swiftshader_gb300._lib import SwgbError
    a = torch.zeros((4, 8, 8, 4), dtype=torch.uint8, device="cuda")
    b = torch.zeros((8, 8, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(SwgbError):
        rend.resolve(gpu_image(a, abi.FORMAT_R8G8B8A8_UNORM, 4), gpu_image(b, abi.FORMAT_R32G32B32A32_SFLOAT))
    with pytest.raises(SwgbError):
        rend.clear_area(gpu_image(b, abi.FORMAT_R32G32B32A32_SFLOAT), (0, 0, 0, 0), (4, 4, 5, 1))
    with pytest.raises(SwgbError):
        rend.blit(gpu_image(a, abi.FORMAT_R8G8B8A8_UNORM, 4), gpu_image(b, abi.FORMAT_R32G32B32A32_SFLOAT),
                  (0, 0, 8, 8), (0, 0, 8, 8))
    with pytest.raises(SwgbError):
        rend.blit(gpu_image(b, abi.FORMAT_R32G32B32A32_SFLOAT), gpu_image(b, abi.FORMAT_R32G32B32A32_SFLOAT),
                  (0, 0, 8, 8), (0, 0, 9, 8))
    img = gpu_image(b, abi.FORMAT_R32G32B32A32_SFLOAT)
    img.pitch_bytes = 8 * 16 + 4
    with pytest.raises(SwgbError):
        rend.clear_image(img, (0, 0, 0, 0))
    rend.synchronize()


@pytest.mark.parametrize("fmt,samples", [(abi.FORMAT_R8G8B8A8_UNORM, 1), (abi.FORMAT_B8G8R8A8_UNORM, 1),
                                         (abi.FORMAT_R32G32B32A32_SFLOAT, 1), (abi.FORMAT_R8G8B8A8_UNORM, 4)])
def test_scene_clear_through_blitter(gpu_lib, fmt, samples):
    """DeviceScene.clear(renderer) (the library's Blitter clear, which the
    benchmark's frames use) leaves the attachments exactly as the torch fills
    of DeviceScene.clear() do, and a draw after it gives the same bits."""
    import torch
    from swiftshader_gb300 import DeviceScene, Renderer, scenes
    s = scenes.scene_heightfield(quads_x=60, quads_y=30, width=160, height=96, tex_size=64)
    s.color_format = fmt
    s.samples = samples
    if fmt == abi.FORMAT_R32G32B32A32_SFLOAT:
        s.clear_color = (0.1, 0.2, 0.3, 0.4)
    r = Renderer(0)
    ds = DeviceScene(s)
    torch.cuda.synchronize()
    ref_c, ref_d = ds.color.clone(), ds.depth.clone()
    ds.color.fill_(7)
    ds.depth.fill_(-3.0)
    ds.clear(r)
    r.synchronize()
    assert torch.equal(ds.color, ref_c)
    assert torch.equal(ds.depth.view(torch.int32), ref_d.view(torch.int32))
    r.draw(ds.state(), ds.args())
    r.synchronize()
    c1, d1 = ds.color.clone(), ds.depth.clone()
    ds.clear()
    r.draw(ds.state(), ds.args())
    r.synchronize()
    assert torch.equal(ds.color, c1)
    assert torch.equal(ds.depth.view(torch.int32), d1.view(torch.int32))
