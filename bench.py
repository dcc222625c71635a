"""Benchmark of the GB300 draw path on the 1M-triangle textured 1080p frame.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload heightfield|small]

One step = one frame: clear colour + depth, then one draw of the whole scene
through the C-ABI (swgb_draw).  Inputs are resident in HBM for ``value``; the L2
(129 MB) is flushed by writing a 256 MiB buffer before every timed step,
outside the step's CUDA events.  ``e2e`` is the same metric through the same
public call with host buffers: every step copies the scene (vertices, indices,
texture chain) host->device from pinned memory and reads the colour + depth
attachments back, inside the timed region.

Multi-GPU (torchrun, N > 1): the frame does not shard, so every rank renders
its own replica ("replicas only"); value = all ranks' fragments / max time.

--impl reference times the CPU restatement of the reference's draw path (the
oracle; the reference's own JIT cannot be built here) on all host cores, same
workload, and prints the same JSON line with "impl": "reference".
"""
import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "heightfield": "1000x500-quad height field (1,000,000 tris, uint32 indices), 1920x1080 RGBA8 + D32F, "
                   "2048^2 RGBA8 12-level chain trilinear REPEAT, colour = texel * vertex colour, depth LESS, "
                   "blend SRC_ALPHA/ONE_MINUS_SRC_ALPHA",
    "small": "1000 independent Gouraud triangles, 256x256 RGBA8 + D32F, depth LESS, no blend, no texture",
}


def make_scene(name):
    from swiftshader_gb300 import scenes
    return scenes.scene_heightfield() if name == "heightfield" else scenes.scene_small()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons in the background."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(values, device=None):
    """Element-wise maximum of per-rank timings across the process group
    (the slowest rank defines a replicated step's time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(scene, cnt):
    """Algorithmic bytes of one frame (whole draw) and of the raster kernel.

    frame  = I*T + V*S_v + F_t*4 + F_p*(4 + 4 + 4*blend) + TexC
    raster = F_t*4 + F_p*(4 + 4 + 4*blend) + TexC
    F_t / F_p = fragments tested / passed (device counters, equal to the
    oracle's), TexC = every referenced mip level counted once."""
    from swiftshader_gb300 import abi
    blend = 1 if scene.blend is not None else 0
    bpp = 4
    frag = cnt["fragments_tested"] * 4 + cnt["fragments_passed"] * (4 + bpp + bpp * blend)
    texc = 0
    mask = cnt.get("texture_levels_mask", 0)
    for i, lv in enumerate(scene.texture_levels):
        if mask >> i & 1:
            texc += lv.nbytes
    idx = 0 if scene.indices is None else scene.indices.nbytes
    verts = scene.vertices.nbytes
    raster = frag + texc
    return idx + verts + raster, raster, texc


def run_ours(args):
    import torch
    from swiftshader_gb300 import DeviceScene, Renderer
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    scene = make_scene(args.workload)
    stream = torch.cuda.Stream(dev)  # every op of the bench (clears, copies, events, draws) is ordered on it
    torch.cuda.set_stream(stream)
    r = Renderer(local, stream)
    ds = DeviceScene(scene, dev)
    st, a = ds.state(), ds.args()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # warm-up
    for _ in range(args.warmup):
        ds.clear()
        r.draw(st, a)
    r.synchronize()
    r.reset_counters()
    r.kernel_times()

    # ---- device-resident timed region -----------------------------------
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    r.set_kernel_timing(True)
    barrier()
    torch.cuda.synchronize()
    launches0 = r.launch_count()
    for i in range(args.steps):
        flush.fill_(i & 0xFF)  # L2 flush, outside the step's events
        starts[i].record(stream)
        ds.clear()
        r.draw(st, a)
        ends[i].record(stream)
    r.synchronize()
    torch.cuda.synchronize()
    barrier()
    launches = r.launch_count() - launches0
    r.set_kernel_timing(False)
    ktimes = r.kernel_times()
    clk = clocks.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms_per_step = sum(step_ms) / len(step_ms)
    cnt = r.counters()
    frames = args.steps
    frag_per_frame = cnt["fragments_tested"] / frames
    tri_per_frame = cnt["triangles_in"] / frames
    per_frame = {k: v // frames if k != "texture_levels_mask" else v for k, v in cnt.items()}

    # ---- end to end through the API with host buffers --------------------
    pin = lambda arr: torch.from_numpy(arr).pin_memory()
    import numpy as np
    h_vert = pin(np.ascontiguousarray(scene.vertices))
    h_idx = None if scene.indices is None else pin(np.ascontiguousarray(scene.indices).view(np.int32))
    h_lv = [pin(np.ascontiguousarray(l)) for l in scene.texture_levels]
    h_color = torch.empty(ds.color.shape, dtype=ds.color.dtype).pin_memory()
    h_depth = torch.empty(ds.depth.shape, dtype=ds.depth.dtype).pin_memory()
    h2d = h_vert.numel() * 4 + (0 if h_idx is None else h_idx.numel() * 4) + sum(l.numel() for l in h_lv)
    d2h = h_color.numel() * h_color.element_size() + h_depth.numel() * 4

    def e2e_step():
        ds.vertices.copy_(h_vert, non_blocking=True)
        if h_idx is not None:
            ds.indices.copy_(h_idx, non_blocking=True)
        for d_l, h_l in zip(ds.levels, h_lv):
            d_l.copy_(h_l, non_blocking=True)
        ds.clear()
        r.draw(st, a)
        h_color.copy_(ds.color, non_blocking=True)
        h_depth.copy_(ds.depth, non_blocking=True)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    e_starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    e_ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        e_starts[i].record(stream)
        e2e_step()
        e_ends[i].record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = sum(s.elapsed_time(e) for s, e in zip(e_starts, e_ends)) / args.steps

    # max over ranks
    ms_per_step, e2e_ms = max_over_ranks([ms_per_step, e2e_ms], dev)

    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    frame_bytes, raster_bytes, texc = algorithmic_bytes(scene, per_frame)
    peak, peak_kind = measured_peaks()
    rast_ms, rast_n = ktimes.get("raster", (0.0, 0))
    rast_avg = rast_ms / max(1, rast_n)
    achieved = raster_bytes / (rast_avg * 1e-3) / 1e9 if rast_avg > 0 else 0.0
    kernels = {k: {"avg_ms": v[0] / max(1, v[1]), "launches": v[1]} for k, v in ktimes.items()}
    value = world * frag_per_frame / (ms_per_step * 1e-3) / 1e9
    line = {
        "metric": "Gfrag/s",
        "value": round(value, 4),
        "unit": "Gfrag/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 + int32 fixed point (RGBA8 / D32F out)",
        "data": "synthetic (seeded generator, swiftshader_gb300.scenes)",
        "config": {"workload": WORKLOADS[args.workload], "l2": "flushed before every timed step (256 MiB write)",
                   "parallelism": "replicas only" if world > 1 else "single GPU"},
        "mtri_per_s": round(world * tri_per_frame / (ms_per_step * 1e-3) / 1e6, 2),
        "frame_counters": per_frame,
        "frame_algorithmic_bytes": frame_bytes,
        "frame_achieved_gbs": round(frame_bytes / (ms_per_step * 1e-3) / 1e9, 1),
        "kernels": kernels,
        "roofline": {"kernel": "k_raster", "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "algorithmic_bytes_per_launch": raster_bytes, "traffic": None},
        "e2e": {"value": round(world * frag_per_frame / (e2e_ms * 1e-3) / 1e9, 4), "unit": "Gfrag/s",
                "ms_per_step": round(e2e_ms, 4), "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    traffic = os.path.join(ROOT, "profiles", "raster_traffic.json")
    if os.path.exists(traffic):
        try:
            with open(traffic) as f:
                tj = json.load(f)
            if tj.get("workload") == args.workload:
                line["roofline"]["traffic"] = tj["bytes_per_launch"]
        except Exception:
            pass
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, scene, bounded_s=args.cpu_seconds)
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def cpu_baseline(args, scene, bounded_s=12.0, threads=None):
    """Times the oracle (CPU restatement of the reference path) on host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    threads = threads or os.cpu_count() or 1
    frames, frags, t0 = 0, 0, time.perf_counter()
    while True:
        _, _, cnt = oracle.render(scene, threads)
        frames += 1
        frags += cnt["fragments_tested"]
        if time.perf_counter() - t0 >= bounded_s:
            break
    dt = time.perf_counter() - t0
    return {"value": round(frags / dt / 1e9, 5), "unit": "Gfrag/s", "cores": threads, "kind": "port",
            "sample": "%d full frame(s) of the same workload, %.1f s, %s %s" % (
                frames, dt, platform.machine(), platform.processor() or "")}


def run_reference(args):
    world, rank, local = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    scene = make_scene(args.workload)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        oracle.render(scene, threads)
    t = []
    frags = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, _, cnt = oracle.render(scene, threads)
        t.append(time.perf_counter() - t0)
        frags += cnt["fragments_tested"]
    ms = 1e3 * sum(t) / len(t)
    value = frags / sum(t) / 1e9
    line = {
        "impl": "reference",
        "metric": "Gfrag/s", "value": round(value, 5), "unit": "Gfrag/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 + int32 fixed point (RGBA8 / D32F out)",
        "data": "synthetic (seeded generator, swiftshader_gb300.scenes)",
        "config": {"workload": WORKLOADS[args.workload], "parallelism": "host threads"},
        "cpu_baseline": {"value": round(value, 5), "unit": "Gfrag/s", "cores": threads, "kind": "port",
                         "sample": "one full frame per step; the CPU restatement of the reference draw path "
                                   "(reference JIT unbuildable here), %s" % platform.machine()},
        "e2e": {"value": round(value, 5), "unit": "Gfrag/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="heightfield", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
