"""Helpers shared by the GPU parity tests: run a scene through the C-ABI on
the device and through the CPU oracle on the host, and compare."""
import numpy as np


def render_gpu(scene, renderer=None, repeat=1):
    import torch
    from swiftshader_gb300 import DeviceScene, Renderer
    r = renderer or Renderer(0)
    ds = DeviceScene(scene)
    torch.cuda.synchronize()
    r.reset_counters()
    for _ in range(repeat):
        r.draw(ds.state(), ds.args())
    r.synchronize()
    cnt = r.counters()
    color = ds.color.cpu().numpy()
    depth = ds.depth_numpy()
    return color, depth, cnt


def render_oracle(scene, nthreads=4):
    import oracle
    return oracle.render(scene, nthreads)


def assert_bit_exact(a, b, what):
    if a.dtype.kind == "f":
        au, bu = a.view(np.uint32 if a.itemsize == 4 else np.uint16), b.view(np.uint32 if b.itemsize == 4 else np.uint16)
    else:
        au, bu = a, b
    diff = au != bu
    if diff.any():
        idx = np.argwhere(diff)
        first = tuple(idx[0])
        raise AssertionError("%s: %d of %d values differ; first at %s: gpu=%r oracle=%r" % (
            what, int(diff.sum()), diff.size, first, a[first], b[first]))
