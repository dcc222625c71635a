"""Benchmark of the GB300 draw path on the 1M-triangle textured 1080p frame.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload heightfield|small|batch]

One step = one frame: clear colour + depth, then one draw of the whole scene
through the C-ABI (swgb_draw).  Inputs are resident in HBM for ``value``; the
L2 (129 MB) is flushed by writing a 256 MiB buffer before every timed step,
outside the step's CUDA events.  ``e2e`` is the same metric through the same
public call with host buffers: every step copies the scene (vertices, indices,
texture chain) host->device from pinned memory and reads the colour + depth
attachments back, inside the timed region.

``value`` counts fragments passed (written after the depth test) per second;
fragments tested are reported beside it as ``gfrag_tested_per_s``.

The default line also carries
  * "batched": the full 4096-draw atlas workload (triangle counts
    log-uniform in [16, 65536]), one swgb_draw_batch call per step against
    the same draws issued one swgb_draw each (the per-draw raster
    configuration picked on a seeded 256-draw sample, then timed on all
    4096 draws);
  * "adjoint": forward and adjoint times (and their ratio) of the two adjoint
    workloads at full size -- the 20k-triangle sphere at 512^2 RGBA32F and 256
    views of the 100k-triangle noisy sphere at 512^2 4x MSAA -- through the
    calls the autograd function makes;
  * "blitter": the Blitter steps either side of a draw on images larger than
    L2 -- 4x MSAA resolves (byte-averaging RGBA8 and averaging RGBA16F),
    a 13-level LINEAR mip chain of an 8192^2 RGBA8 texture, clears of 4x MSAA
    colour and depth -- each as achieved GB/s of its algorithmic bytes and the
    fraction of the measured HBM peak.
--workload batch measures the full 4096-draw atlas workload (log-uniform
[16, 65536] triangles) as the headline line: one step = clear the atlas + one
swgb_draw_batch of all draws.

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

DEFAULT_RUNS = 3

WORKLOADS = {
    "heightfield": "1000x500-quad height field (1,000,000 tris, uint32 indices), 1920x1080 RGBA8 + D32F, "
                   "2048^2 RGBA8 12-level chain trilinear REPEAT, colour = texel * vertex colour, depth LESS, "
                   "blend SRC_ALPHA/ONE_MINUS_SRC_ALPHA",
    "small": "1000 independent Gouraud triangles, 256x256 RGBA8 + D32F, depth LESS, no blend, no texture",
    "sphere": "adjoint: 20k-triangle uv-sphere, 512^2 RGBA32F, 1024^2 RGBA32F texture (forward + adjoint)",
    "views": "adjoint: views of a 100k-triangle noisy sphere, 512^2 4x MSAA RGBA16F, OVER (forward + adjoint)",
    "blitter": "Blitter steps: 4x MSAA 4096^2 RGBA8 and 2048^2 RGBA16F resolves, clears of 4x MSAA 4096^2 "
               "RGBA8 and D32F, 13-level LINEAR mip chain of an 8192^2 RGBA8 texture",
    "batch": "4096 independent draws, triangle counts log-uniform in [16, 65536], uniform clip-space triangles, "
             "square viewports with side uniform in {128,256,384,512} shelf-packed into 16384^2 RGBA8 + D32F "
             "atlas pages, each draw sampling its own 256^2 RGBA8 texture bilinearly, depth LESS, no blend",
}

BATCH_FULL = dict(n_draws=4096, tri_min=16, tri_max=65536)


def make_scene(name):
    from swiftshader_gb300 import scenes
    if name == "batch":
        return scenes.scene_batch(**BATCH_FULL)
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
    from swiftshader_gb300 import DeviceScene, Renderer, scenes
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
    # the frame's Blitter clears run on a stream of their own (a second
    # context) after the previous frame's raster; the draw lets only its raster
    # stage wait for them (swgb_draw_args.raster_wait_event), so they run
    # beside vertex processing, setup and binning
    clr = torch.cuda.Stream(dev)
    rc = Renderer(local, clr)
    ev_clear = torch.cuda.Event()
    ev_clear.record(clr)
    a_frame = ds.args()
    a_frame.raster_wait_event = ev_clear.cuda_event

    def frame():
        clr.wait_stream(stream)
        ds.clear(rc)
        ev_clear.record(clr)
        r.draw(st, a_frame)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # raster configuration chosen by the library's autotuner on this frame
    # (or fixed by --raster-config)
    tune = None
    if args.raster_config:
        wh, hz = args.raster_config.split(":")
        w, h = (int(x) for x in wh.split("x"))
        r.set_raster_config(w, h, bool(int(hz)))
        tune = {"best": r.raster_config(), "how": "fixed by --raster-config"}
    elif not args.no_autotune:
        ds.clear(r)
        tune = autotune_summary(*r.autotune([st], [a], batched=False))

    # warm-up
    for _ in range(args.warmup):
        frame()
    r.synchronize()
    r.reset_counters()
    r.kernel_times()

    # ---- device-resident timed region -----------------------------------
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    # live event pairs around k_raster only (the roofline's kernel); the
    # other kernels' times come from an untimed pass after the timed region
    r.set_kernel_timing(True, kinds=["raster"])
    barrier()
    torch.cuda.synchronize()
    launches0 = r.launch_count() + rc.launch_count()
    for i in range(args.steps):
        flush.fill_(i & 0xFF)  # L2 flush, outside the step's events
        starts[i].record(stream)
        frame()  # the raster waits for the clears: the end event follows both
        ends[i].record(stream)
    r.synchronize()
    torch.cuda.synchronize()
    barrier()
    launches = r.launch_count() + rc.launch_count() - launches0
    r.set_kernel_timing(False)
    ktimes = r.kernel_times()
    clk = clocks.stop()
    cnt = r.counters()
    # every kernel of the same frames, each launch timed (outside the timed region)
    r.set_kernel_timing(True)
    rc.set_kernel_timing(True)
    rc.kernel_times()
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        frame()
    torch.cuda.synchronize()
    r.set_kernel_timing(False)
    rc.set_kernel_timing(False)
    ktimes_all = r.kernel_times()
    ktimes_all.update(rc.kernel_times())
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms_per_step = sum(step_ms) / len(step_ms)
    frames = args.steps
    frag_per_frame = cnt["fragments_passed"] / frames
    tested_per_frame = cnt["fragments_tested"] / frames
    tri_per_frame = cnt["triangles_in"] / frames
    per_frame = {k: v // frames if k != "texture_levels_mask" else v for k, v in cnt.items()}

    # ---- end to end through the API with host buffers --------------------
    # the scene's geometry (vertices, indices) and texture levels sit in two
    # regions of the DeviceScene's allocation and its attachments in a third.
    # Per step: the geometry, then the textures, uploaded from pinned memory on
    # an upload stream; the draw waits for the geometry and lets only its
    # raster stage wait for the textures (swgb_draw_args.raster_wait_event),
    # so the texture upload runs beside vertex processing, setup and binning;
    # one read-back of colour and depth.
    h_geo = ds.geometry_region.cpu().pin_memory()
    h_tex = ds.texture_region.cpu().pin_memory()
    h2d = h_geo.numel() + h_tex.numel()
    d2h = ds.outputs().numel()
    e2e_ms, e2e_seq_ms = measure_e2e(r, rc, stream, clr, flush, [ds, DeviceScene(scene, dev)], h_geo, h_tex,
                                     args.steps, args.warmup, barrier)

    # batched vs per-draw on the reduced-size atlas workload (free the frame first)
    batched = None
    if args.workload == "heightfield" and not args.no_batched:
        del h_geo, h_tex
        _, db, batched = measure_batch(r, stream, flush, BATCH_FULL, 3, 1, 1, dev, tune=not args.no_autotune,
                                       pick_sample=256)
        batched["config"]["workload"] = WORKLOADS["batch"]
        del db

    blitter = None
    if args.workload == "heightfield" and not args.no_blitter:
        blitter = measure_blitter(r, stream, flush, dev)

    adjoint_lines = None
    if args.workload == "heightfield" and not args.no_adjoint:
        adjoint_lines = {"sphere": measure_adjoint(r, stream, flush, dev, "sphere"),
                         "views": measure_adjoint(r, stream, flush, dev, "views", steps=2, warmup=1)}

    # max over ranks
    ms_per_step, e2e_ms, e2e_seq_ms = max_over_ranks([ms_per_step, e2e_ms, e2e_seq_ms], dev)

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
    kernels = {k: {"avg_ms": v[0] / max(1, v[1]), "launches": v[1]} for k, v in ktimes_all.items()}
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
        "config": {"workload": WORKLOADS[args.workload]},
        "l2": "flushed before every timed step (256 MiB write)",
        "step_how": "the two Blitter clears (swgb_clear, a second context on its own stream, after the previous "
                    "frame's raster) and one swgb_draw whose raster stage waits for them "
                    "(swgb_draw_args.raster_wait_event); the step's end event follows both",
        "parallelism": "replicas only" if world > 1 else "single GPU",
        "value_counts": "fragments passed (F_p: written after the depth test) per second",
        "gfrag_tested_per_s": round(world * tested_per_frame / (ms_per_step * 1e-3) / 1e9, 4),
        "mtri_per_s": round(world * tri_per_frame / (ms_per_step * 1e-3) / 1e6, 2),
        "frame_counters": per_frame,
        "frame_algorithmic_bytes": frame_bytes,
        "frame_achieved_gbs": round(frame_bytes / (ms_per_step * 1e-3) / 1e9, 1),
        "kernels": kernels,
        "kernels_how": "k_raster (the roofline) timed by CUDA events inside the timed region; every kernel, "
                       "each launch between events, in an untimed pass of the same frames (the clears, 'blit', "
                       "run beside vertex processing and setup, so their event time includes sharing the GPU)",
        "roofline": {"kernel": "k_raster", "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "algorithmic_bytes_per_launch": raster_bytes, "traffic": None},
        "e2e": {"value": round(world * frag_per_frame / (e2e_ms * 1e-3) / 1e9, 4), "unit": "Gfrag/s",
                "ms_per_step": round(e2e_ms, 4), "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "how": "two frames in flight (two DeviceScenes): step i uploads its geometry and textures on "
                       "an upload stream while step i-1 renders, and reads its colour and depth back on a "
                       "read-back stream while step i+1 renders; L2 flushed inside every step; "
                       "K steps between one pair of events, fill and drain included",
                "sequential_ms_per_step": round(e2e_seq_ms, 4),
                "sequential_value": round(world * frag_per_frame / (e2e_seq_ms * 1e-3) / 1e9, 4)},
        "gpu_launches": int(launches),
        "clocks": clk,
        "raster_config": tune,
    }
    traffic = os.path.join(ROOT, "profiles", "raster_traffic.json")
    if os.path.exists(traffic):
        try:
            with open(traffic) as f:
                tj = json.load(f)
            if tj.get("workload") == args.workload:
                line["roofline"]["traffic"] = tj["bytes_per_launch"]
                # the issue-side bound the kernel runs against: its warp
                # instructions per launch (the same ncu capture) over the live
                # launch time, against one instruction per scheduler (4 per
                # SM) per cycle at the SM clock sampled during the timed steps
                inst = tj.get("warp_instructions_per_launch")
                mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz")
                if inst and mhz and rast_avg > 0:
                    sms = torch.cuda.get_device_properties(dev).multi_processor_count
                    ach = inst / (rast_avg * 1e-3) / 1e9
                    peak_i = sms * 4 * mhz * 1e6 / 1e9
                    line["roofline"]["issue"] = {"warp_instructions_per_launch": inst, "achieved": round(ach, 1),
                                                 "peak": round(peak_i, 1), "unit": "G warp instructions/s",
                                                 "frac": round(ach / peak_i, 4),
                                                 "how": "%d SMs x 4 schedulers x %g MHz; instructions from ncu" % (sms, mhz)}
        except Exception:
            pass
    if batched is not None:
        line["batched"] = batched
    if adjoint_lines is not None:
        line["adjoint"] = adjoint_lines
    if blitter is not None:
        line["blitter"] = blitter
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, scene, bounded_s=args.cpu_seconds)
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def measure_e2e(r, rc, stream, clr, flush, dss, h_geo, h_tex, steps, warmup, barrier):
    """Per-step milliseconds of the frame through the API with host buffers:
    (pipelined, sequential).

    Sequential: one frame at a time -- upload, clear, draw, read-back, the
    next step after the read-back.  Pipelined: two frames in flight on two
    DeviceScenes (``dss``); step i's uploads (upload stream) wait only until
    the draw of step i-2 has read that scene's inputs, its clear waits until
    the read-back of step i-2 has left that scene's attachments, and its
    read-back (read-back stream) runs while step i+1 renders.  The clears run
    on the clear stream (context rc) beside the draw's first stages; the
    raster waits for them and for the texture upload (one event).  Every step
    flushes L2 on the draw stream before its draw, inside the timed region;
    the pipelined K steps are timed between one pair of events, including the
    first upload and the last read-back."""
    import torch
    dev = stream.device
    up, down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    sts = [d.state() for d in dss]
    h_out = [torch.empty(d.outputs().shape, dtype=torch.uint8).pin_memory() for d in dss]
    ev_geo = [torch.cuda.Event() for _ in dss]
    ev_tex = [torch.cuda.Event() for _ in dss]
    ev_drawn = [torch.cuda.Event() for _ in dss]
    ev_read = [torch.cuda.Event() for _ in dss]
    ev_ready = [torch.cuda.Event() for _ in dss]  # clears done and textures up
    argl = []
    for d, e in zip(dss, ev_ready):
        e.record(clr)  # a recorded event before the first draw refers to it
        a = d.args()
        a.raster_wait_event = e.cuda_event
        argl.append(a)
    torch.cuda.synchronize()

    def upload(b):
        d = dss[b]
        up.wait_event(ev_drawn[b])  # the draw two steps back has read these inputs
        with torch.cuda.stream(up):
            d.geometry_region.copy_(h_geo, non_blocking=True)
            ev_geo[b].record(up)
            d.texture_region.copy_(h_tex, non_blocking=True)
            ev_tex[b].record(up)

    def render(i, b):
        d = dss[b]
        flush.fill_(i & 0xFF)
        clr.wait_stream(stream)
        clr.wait_event(ev_read[b])  # the read-back two steps back has left the attachments
        d.clear(rc)
        clr.wait_event(ev_tex[b])
        ev_ready[b].record(clr)
        stream.wait_event(ev_geo[b])
        r.draw(sts[b], argl[b])
        ev_drawn[b].record(stream)

    def read_back(b):
        down.wait_event(ev_drawn[b])
        with torch.cuda.stream(down):
            h_out[b].copy_(dss[b].outputs(), non_blocking=True)
            ev_read[b].record(down)

    def pipelined(n):
        for i in range(n):
            b = i & 1
            upload(b)
            render(i, b)
            read_back(b)
        stream.wait_stream(down)

    def sequential_step(i):
        upload(0)
        render(i, 0)
        read_back(0)
        stream.wait_stream(down)

    for i in range(max(1, warmup)):
        sequential_step(i)
    pipelined(max(2, warmup))
    torch.cuda.synchronize()
    # sequential: per-step event pairs
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    barrier()
    for i in range(steps):
        starts[i].record(stream)
        sequential_step(i)
        ends[i].record(stream)
    torch.cuda.synchronize()
    seq_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / steps
    # pipelined: one event pair around all steps
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    t0.record(stream)
    pipelined(steps)
    t1.record(stream)
    torch.cuda.synchronize()
    barrier()
    # both scenes rendered the same frame as the device-resident steps
    for b in range(len(dss)):
        assert torch.equal(h_out[b], h_out[0]), "pipelined frames differ"
    return t0.elapsed_time(t1) / steps, seq_ms


def measure_blitter(r, stream, flush, dev, steps=5, warmup=3):
    """GB/s of swgb_resolve / swgb_blit (mip chain) / swgb_clear on images
    larger than L2; algorithmic bytes = every byte read once + every byte
    written once."""
    import torch
    from swiftshader_gb300 import abi
    from swiftshader_gb300.renderer import image_view
    peak, peak_kind = measured_peaks()
    out = {}

    def run(name, body, nbytes, note):
        for _ in range(warmup):
            body()
        torch.cuda.synchronize()
        ms = statistics.median(time_steps(stream, flush, steps, body))
        gbs = nbytes / (ms * 1e-3) / 1e9
        out[name] = {"ms": round(ms, 4), "bytes": int(nbytes), "achieved_gbs": round(gbs, 1),
                     "frac": round(gbs / peak, 4), "what": note}

    g = torch.Generator(device=dev).manual_seed(9)
    n = 4096
    ms4 = torch.randint(0, 256, (4, n, n, 4), dtype=torch.uint8, device=dev, generator=g)
    one = torch.empty((n, n, 4), dtype=torch.uint8, device=dev)
    src, dst = image_view(ms4, abi.FORMAT_R8G8B8A8_UNORM, 4), image_view(one, abi.FORMAT_R8G8B8A8_UNORM)
    run("resolve_rgba8", lambda: r.resolve(src, dst), 5 * one.numel(),
        "4x MSAA 4096^2 R8G8B8A8_UNORM -> 1x (byte-averaging path)")
    clr = (0.25, 0.5, 0.75, 1.0)
    run("clear_rgba8_4x", lambda: r.clear_image(src, clr), ms4.numel(), "clear of 4x MSAA 4096^2 R8G8B8A8_UNORM")
    del ms4, one
    m = 2048
    h4 = torch.randn((4, m, m, 4), device=dev, generator=g).to(torch.float16).view(torch.int16)
    h1 = torch.empty((m, m, 4), dtype=torch.int16, device=dev)
    hs, hd = image_view(h4, abi.FORMAT_R16G16B16A16_SFLOAT, 4), image_view(h1, abi.FORMAT_R16G16B16A16_SFLOAT)
    run("resolve_rgba16f", lambda: r.resolve(hs, hd), 5 * h1.numel() * 2,
        "4x MSAA 2048^2 R16G16B16A16_SFLOAT -> 1x (averaging blit)")
    del h4, h1
    d4 = torch.empty((4, n, n), dtype=torch.float32, device=dev)
    di = image_view(d4, abi.FORMAT_D32_SFLOAT, 4)
    run("clear_d32f_4x", lambda: r.clear_image(di, 1.0), d4.numel() * 4, "clear of 4x MSAA 4096^2 D32_SFLOAT")
    del d4
    levels, size = [], 8192
    while True:
        levels.append(torch.empty((size, size, 4), dtype=torch.uint8, device=dev))
        if size == 1:
            break
        size //= 2
    levels[0].copy_(torch.randint(0, 256, levels[0].shape, dtype=torch.uint8, device=dev, generator=g))
    views = [image_view(t, abi.FORMAT_R8G8B8A8_UNORM) for t in levels]
    mip_bytes = sum(t.numel() for t in levels[:-1]) + sum(t.numel() for t in levels[1:])
    run("mip_chain_rgba8", lambda: r.generate_mipmaps(views), mip_bytes,
        "8192^2 R8G8B8A8_UNORM -> 13 levels, one LINEAR swgb_blit per level")
    del levels, views
    out["peak"] = {"value": peak, "kind": peak_kind, "unit": "GB/s"}
    return out


def batch_raster_bytes(b, cnt):
    """Algorithmic bytes of the batched raster kernel: F_t*4 + F_p*(4 + 4) +
    every draw's texture once (no blending in this workload)."""
    return cnt["fragments_tested"] * 4 + cnt["fragments_passed"] * 8 + int(b.textures.nbytes)


def time_steps(stream, flush, steps, body):
    import torch
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    for i in range(steps):
        flush.fill_(i & 0xFF)  # L2 flush, outside the step's events
        starts[i].record(stream)
        body()
        ends[i].record(stream)
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in zip(starts, ends)]


def autotune_summary(best, table):
    return {"best": best,
            "candidates_ms": {"%s hiz%d" % (c["bin"], c["hiz"]): {k: round(v, 3) for k, v in t.items()}
                              for c, t in table},
            "how": "swgb_autotune: one warm-up and %d runs per candidate, each timed alone with CUDA events, "
                   "attachments restored between; lowest median wins" % DEFAULT_RUNS}


def measure_batch(r, stream, flush, params, steps, warmup, per_draw_steps, dev, world=1, rank=0, tune=True,
                  pick_sample=0):
    """Batched vs per-draw on the atlas workload: one swgb_draw_batch call per
    step against one swgb_draw per draw, same draws, same kernels' work.  The
    batched arm runs the raster configuration the autotuner picks for the
    batch; the per-draw arm runs the faster of that one and the default (16x16
    bins, depth rejection on).  With pick_sample = 0 each candidate is timed
    on all draws; with pick_sample = S the candidates are compared on a seeded
    sample of S draws and only the faster one is timed on all draws.  On N
    ranks each rank draws its longest-processing-time-first share."""
    from swiftshader_gb300 import DeviceBatch, scenes, shard
    b = scenes.scene_batch(**params)
    if world > 1:
        b = b.subset(shard.lpt_partition(shard.draw_costs(b.tris, b.sides), world)[rank])
    db = DeviceBatch(b, dev)
    tuned = None
    if tune:
        db.clear()
        tuned = autotune_summary(*r.autotune(db.states, db.args, batched=True))
    best = r.raster_config()

    def batched():
        db.clear()
        db.draw_batch(r)

    def per_draw():
        db.clear()
        db.draw_each(r)

    for _ in range(warmup):
        batched()
    r.synchronize()
    r.reset_counters()
    l0 = r.launch_count()
    tb = time_steps(stream, flush, steps, batched)
    r.synchronize()
    launches = r.launch_count() - l0
    cnt = r.counters()
    per_draw_ms = {}
    sample_ms = {}
    if per_draw_steps:
        import numpy as np
        shapes = [best] + ([{"bin": "16x16", "hiz": 1}] if best != {"bin": "16x16", "hiz": 1} else [])
        key = lambda c: "%s hiz%d" % (c["bin"], c["hiz"])
        if pick_sample and pick_sample < b.n:
            sample = sorted(np.random.Generator(np.random.PCG64(11)).permutation(b.n)[:pick_sample].tolist())
            for c in shapes:
                w, h = (int(x) for x in c["bin"].split("x"))
                r.set_raster_config(w, h, bool(c["hiz"]))
                db.clear()
                db.draw_each(r, sample)
                r.synchronize()
                ts = time_steps(stream, flush, 3, lambda: db.draw_each(r, sample))
                sample_ms[key(c)] = round(statistics.median(ts), 3)
            shapes = [min(shapes, key=lambda c: sample_ms[key(c)])]
        for c in shapes:
            w, h = (int(x) for x in c["bin"].split("x"))
            r.set_raster_config(w, h, bool(c["hiz"]))
            if not sample_ms:
                per_draw()
                r.synchronize()
            tp = time_steps(stream, flush, per_draw_steps, per_draw)
            per_draw_ms[key(c)] = round(sum(tp) / len(tp), 3)
        w, h = (int(x) for x in best["bin"].split("x"))
        r.set_raster_config(w, h, bool(best["hiz"]))
    r.synchronize()
    mb = sum(tb) / len(tb)
    mp = min(per_draw_ms.values()) if per_draw_ms else float("nan")
    per_step = {k: v // steps if k != "texture_levels_mask" else v for k, v in cnt.items()}
    return b, db, {
        "config": {"draws": b.n, "triangles_log_uniform": [params["tri_min"], params["tri_max"]],
                   "triangles": int(b.tris.sum()), "viewport_sides": [128, 256, 384, 512],
                   "atlas_pages": b.pages, "page": b.page_size, "texture": "256^2 RGBA8 per draw, bilinear"},
        "batched_ms_per_step": round(mb, 3), "per_draw_ms_per_step": round(mp, 3) if per_draw_steps else None,
        "per_draw_ms_by_config": per_draw_ms or None,
        "per_draw_pick": ({"sample_draws": pick_sample, "sample_ms_by_config": sample_ms,
                           "how": "per-draw configurations compared on a seeded sample of draws (median of 3); "
                                  "the faster one timed on all draws"} if sample_ms else None),
        "speedup_vs_per_draw": round(mp / mb, 2) if per_draw_steps else None,
        "draws_per_s": round(b.n / (mb * 1e-3), 1), "per_draw_draws_per_s": round(b.n / (mp * 1e-3), 1) if per_draw_steps else None,
        "gfrag_passed_per_s": round(per_step["fragments_passed"] / (mb * 1e-3) / 1e9, 3),
        "gfrag_tested_per_s": round(per_step["fragments_tested"] / (mb * 1e-3) / 1e9, 3),
        "tested_how": "samples tested against depth, including those of whole triangles the hierarchical depth "
                      "rejection counts from their span rows without expanding them (the oracle's count)",
        "mtri_per_s": round(per_step["triangles_in"] / (mb * 1e-3) / 1e6, 2),
        "gpu_launches_per_step": launches / steps, "steps": steps, "per_draw_steps": per_draw_steps,
        "counters_per_step": per_step, "raster_config": tuned,
    }


def measure_adjoint(r, stream, flush, dev, workload, steps=3, warmup=2, views=256):
    """Forward and adjoint times of one adjoint workload, through the same
    DrawSet calls the autograd function makes (no torch autograd overhead):
    forward = clear + draw(s); adjoint = zero gradients + adjoint draw(s) for
    a fixed dL/dcolour."""
    import numpy as np
    import torch
    from swiftshader_gb300 import abi, adjoint, scenes
    if workload == "sphere":
        scene_list = [scenes.scene_sphere_fp32()]
        desc = ("20k-triangle uv-sphere (100x100 segments), 512^2 RGBA32F, 1024^2 RGBA32F texture bilinear "
                "CLAMP, colour = texel x vertex colour, depth LESS; L2 loss gradient")
    else:
        rng = np.random.Generator(np.random.PCG64(0x53570004))
        mesh = scenes.uv_sphere(rng, 250, 200, noise_sigma=0.02)
        levels = scenes.float_mip_chain(rng.uniform(0.0, 1.0, (2048, 2048, 4)), np.float16)
        scene_list = [scenes.scene_sphere_views(v, mesh=mesh, levels=levels) for v in range(views)]
        for sc in scene_list:
            sc.samples = 4
        desc = ("%d views of a 100k-triangle uv-sphere with radial N(0, 0.02^2) noise, cameras on a radius-3 "
                "sphere, 512^2 4x MSAA RGBA16F, 2048^2 RGBA16F mip chain trilinear, premultiplied OVER, depth "
                "LESS; all views as one batch forward and one batch adjoint" % views)
    sc0 = scene_list[0]
    verts = torch.from_numpy(np.ascontiguousarray(sc0.vertices, np.float32)).to(dev)
    tdt = torch.float16 if sc0.texture_format == abi.FORMAT_R16G16B16A16_SFLOAT else torch.float32
    tex = [torch.from_numpy(np.ascontiguousarray(l)).to(dev).to(tdt) for l in sc0.texture_levels]
    ds = adjoint.DrawSet(scene_list, verts, tex)
    ds.forward(r)
    torch.cuda.synchronize()
    g = (2.0 * (ds.colors() - 0.25)).contiguous()  # dL/dcolour of an L2 loss against a grey target
    for _ in range(warmup):
        ds.forward(r)
        ds.adjoint(r, g)
    r.synchronize()
    r.reset_counters()
    tf = time_steps(stream, flush, steps, lambda: ds.forward(r))
    ta = time_steps(stream, flush, steps, lambda: ds.adjoint(r, g))
    r.synchronize()
    cnt = r.counters()
    mf, ma = sum(tf) / len(tf), sum(ta) / len(ta)
    return {"config": {"workload": desc, "views": len(scene_list), "triangles_per_view": sc0.tri_count},
            "forward_ms": round(mf, 3), "adjoint_ms": round(ma, 3), "adjoint_over_forward": round(ma / mf, 3),
            "adjoint_fragments_per_step": cnt["adjoint_fragments"] // steps,
            "adjoint_depth_mismatch": cnt["adjoint_depth_mismatch"], "adjoint_list_overflow": cnt["adjoint_list_overflow"],
            "steps": steps}


def run_adjoint(args):
    """--workload sphere|views: forward and adjoint of one adjoint workload
    as the headline line (metric: adjoint ms per step; the forward beside)."""
    import torch
    from swiftshader_gb300 import Renderer
    world, rank, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    r = Renderer(local, stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    res = measure_adjoint(r, stream, flush, dev, args.workload, steps=args.steps, warmup=args.warmup, views=args.views)
    clk = clocks.stop()
    if rank != 0:
        return
    line = {
        "metric": "adjoint ms/step", "value": res["adjoint_ms"], "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["adjoint_ms"], "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (fp64 geometry in the adjoint)", "data": "synthetic (seeded generator)",
        "config": res["config"], "adjoint": res, "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_blitter(args):
    """--workload blitter: the clear / resolve / mip-chain timings alone, as
    their own line (metric: GB/s of the mip chain, the others beside)."""
    import torch
    from swiftshader_gb300 import Renderer
    world, rank, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    r = Renderer(local, stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    res = measure_blitter(r, stream, flush, dev, steps=args.steps, warmup=args.warmup)
    clk = clocks.stop()
    if rank != 0:
        return
    mip = res["mip_chain_rgba8"]
    line = {
        "metric": "GB/s", "value": mip["achieved_gbs"], "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mip["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8 / f16 / f32 texels", "data": "synthetic (seeded generator)",
        "config": {"workload": WORKLOADS["blitter"]},
        "l2": "flushed before every timed step (256 MiB write)",
        "step_how": "the two Blitter clears (swgb_clear, a second context on its own stream, after the previous "
                    "frame's raster) and one swgb_draw whose raster stage waits for them "
                    "(swgb_draw_args.raster_wait_event); the step's end event follows both",
        "blitter": res, "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_batch(args):
    """--workload batch: the full 4096-draw atlas workload as the headline."""
    import numpy as np
    import torch
    from swiftshader_gb300 import Renderer
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    r = Renderer(local, stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    params = dict(BATCH_FULL, n_draws=args.batch_draws, tri_max=args.batch_tri_max)
    b, db, res = measure_batch(r, stream, flush, params, args.steps, args.warmup,
                               0 if args.no_per_draw else 1, dev, world, rank, tune=not args.no_autotune)
    clk = clocks.stop()
    # kernel-level timing: the batch as direct launches (timing disables the graph)
    r.set_kernel_timing(True)
    r.kernel_times()
    db.clear()
    db.draw_batch(r)
    r.synchronize()
    kt = r.kernel_times()
    r.set_kernel_timing(False)
    # end to end: vertices + textures host->device, atlas back, inside the timed region
    pin = lambda arr: torch.from_numpy(np.ascontiguousarray(arr)).pin_memory()
    h_vert, h_tex = pin(b.vertices), pin(b.textures)
    h_color = torch.empty(db.color.shape, dtype=db.color.dtype).pin_memory()
    h_depth = torch.empty(db.depth.shape, dtype=db.depth.dtype).pin_memory()
    h2d = h_vert.numel() * 4 + h_tex.numel()
    d2h = h_color.numel() + h_depth.numel() * 4

    def e2e_step():
        db.vertices.copy_(h_vert, non_blocking=True)
        db.textures.copy_(h_tex, non_blocking=True)
        db.clear()
        db.draw_batch(r)
        h_color.copy_(db.color, non_blocking=True)
        h_depth.copy_(db.depth, non_blocking=True)

    e2e_step()
    e2e_steps = max(1, min(args.steps, 3))
    te = time_steps(stream, flush, e2e_steps, e2e_step)
    mb = res["batched_ms_per_step"]
    me = sum(te) / len(te)
    mb, me = max_over_ranks([mb, me], dev)
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    rast_ms, rast_n = kt.get("raster", (0.0, 0))
    rast_avg = rast_ms / max(1, rast_n)
    rbytes = batch_raster_bytes(b, res["counters_per_step"])
    peak, peak_kind = measured_peaks()
    achieved = rbytes / (rast_avg * 1e-3) / 1e9 if rast_avg > 0 else 0.0
    total = params["n_draws"]
    line = {
        "metric": "draws/s", "value": round(total / (mb * 1e-3), 1), "unit": "draws/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(mb, 3), "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "f32 + int32 fixed point (RGBA8 / D32F out)",
        "data": "synthetic (seeded generator, swiftshader_gb300.scenes.scene_batch)",
        "config": {"workload": WORKLOADS["batch"] if params == BATCH_FULL else
                   "%d independent draws, triangle counts log-uniform in [%d, %d], otherwise as the 4096-draw atlas "
                   "workload" % (params["n_draws"], params["tri_min"], params["tri_max"])},
        "l2": "flushed before every timed step (256 MiB write)",
        "step_how": "the two Blitter clears (swgb_clear, a second context on its own stream, after the previous "
                    "frame's raster) and one swgb_draw whose raster stage waits for them "
                    "(swgb_draw_args.raster_wait_event); the step's end event follows both",
        "parallelism": ("draws split over ranks, longest-processing-time-first on triangles x viewport "
                        "area; no collective") if world > 1 else "single GPU",
        "batched": res,
        "kernels": {k: {"avg_ms": v[0] / max(1, v[1]), "launches": v[1]} for k, v in kt.items()},
        "roofline": {"kernel": "k_raster_batch", "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "algorithmic_bytes_per_launch": rbytes, "traffic": None},
        "e2e": {"value": round(total / (me * 1e-3), 1), "unit": "draws/s", "ms_per_step": round(me, 3),
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(round(res["gpu_launches_per_step"] * args.steps)),
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_batch(b, bounded_s=args.cpu_seconds)
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


_TIMING_BUILD = {}


def oracle_timing_build(oracle, scene, threads):
    """Whether to time the oracle's timing build: the same restatement with
    the FPU's flush-to-zero mode set through fenv.h (as the reference's worker
    threads set it) instead of flushing every operand in software, built -O3.
    It is used only when its frame of 'scene' equals the checker build's, bit
    for bit; returns (use it, note for the sample text)."""
    import numpy as np
    if "ok" not in _TIMING_BUILD:
        try:
            c1, d1, n1 = oracle.render(scene, threads, timing=True)
            c0, d0, n0 = oracle.render(scene, threads)
            ok = c0.tobytes() == c1.tobytes() and np.asarray(d0).tobytes() == np.asarray(d1).tobytes() and n0 == n1
            _TIMING_BUILD["ok"] = ok
            _TIMING_BUILD["note"] = ("timing build of the port (FPU flush-to-zero mode, -O3; its frame equals the "
                                     "checker build's)" if ok else "checker build of the port (the timing build's "
                                     "frame differed)")
        except Exception as e:  # noqa: BLE001 - any failure means: time the checker build
            _TIMING_BUILD["ok"] = False
            _TIMING_BUILD["note"] = "checker build of the port (timing build unavailable: %s)" % e
    return _TIMING_BUILD["ok"], _TIMING_BUILD["note"]


def cpu_baseline_batch(b, bounded_s=12.0, threads=None):
    """Oracle on a seeded random sample of the batch's draws, scaled to the
    whole batch by fragment work (triangles x viewport area)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    threads = threads or os.cpu_count() or 1
    order = np.random.Generator(np.random.PCG64(7)).permutation(b.n)
    cost = b.tris.astype(np.float64) * b.sides.astype(np.float64) ** 2
    fast, note = oracle_timing_build(oracle, b.draw_scene(int(order[0])), threads)
    done, work, t0 = 0, 0.0, time.perf_counter()
    for i in order:
        oracle.render(b.draw_scene(int(i)), threads, timing=fast)
        done += 1
        work += cost[i]
        if time.perf_counter() - t0 >= bounded_s:
            break
    dt = time.perf_counter() - t0
    est = dt * cost.sum() / work
    return {"value": round(b.n / est, 3), "unit": "draws/s", "cores": threads, "kind": "port",
            "sample": "%d of %d draws (seeded random order), %.1f s, scaled to the batch by triangles x viewport "
                      "area; %s; %s" % (done, b.n, dt, platform.machine(), note)}


def cpu_baseline(args, scene, bounded_s=12.0, threads=None):
    """Times the oracle (CPU restatement of the reference path) on host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    threads = threads or os.cpu_count() or 1
    fast, note = oracle_timing_build(oracle, scene, threads)
    frames, frags, t0 = 0, 0, time.perf_counter()
    while True:
        _, _, cnt = oracle.render(scene, threads, timing=fast)
        frames += 1
        frags += cnt["fragments_passed"]
        if time.perf_counter() - t0 >= bounded_s:
            break
    dt = time.perf_counter() - t0
    return {"value": round(frags / dt / 1e9, 5), "unit": "Gfrag/s", "cores": threads, "kind": "port",
            "sample": "%d full frame(s) of the same workload, %.1f s, %s; %s" % (
                frames, dt, platform.machine(), note)}


def run_reference(args):
    world, rank, local = dist_env()
    if rank != 0:
        return
    if args.workload in ("sphere", "views"):
        print(json.dumps({"impl": "reference", "unavailable": "the reference draw path has no backward pass"}), flush=True)
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    if args.workload == "blitter":
        run_reference_blitter(args, oracle)
        return
    scene = make_scene(args.workload)
    threads = os.cpu_count() or 1
    if args.workload == "batch":
        return run_reference_batch(args, scene, world, threads)
    fast, note = oracle_timing_build(oracle, scene, threads)
    for _ in range(args.warmup):
        oracle.render(scene, threads, timing=fast)
    t = []
    frags = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, _, cnt = oracle.render(scene, threads, timing=fast)
        t.append(time.perf_counter() - t0)
        frags += cnt["fragments_passed"]
    ms = 1e3 * sum(t) / len(t)
    value = frags / sum(t) / 1e9
    line = {
        "impl": "reference",
        "metric": "Gfrag/s", "value": round(value, 5), "unit": "Gfrag/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 + int32 fixed point (RGBA8 / D32F out)",
        "data": "synthetic (seeded generator, swiftshader_gb300.scenes)",
        "config": {"workload": WORKLOADS[args.workload]},
        "parallelism": "host threads",
        "value_counts": "fragments passed (F_p: written after the depth test) per second",
        "cpu_baseline": {"value": round(value, 5), "unit": "Gfrag/s", "cores": threads, "kind": "port",
                         "sample": "one full frame per step; the CPU restatement of the reference draw path "
                                   "(the reference's JIT builds only for x86-64 here), %s; %s" % (platform.machine(), note)},
        "e2e": {"value": round(value, 5), "unit": "Gfrag/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference_blitter(args, oracle):
    """Reference arm of --workload blitter: the oracle's Blitter restatement
    (one host thread) building the mip chain of a 2048^2 RGBA8 texture, a
    bounded sample of the 8192^2 chain; GB/s of the same algorithmic bytes."""
    import numpy as np
    from swiftshader_gb300 import abi
    levels, size = [], 2048
    rng = np.random.default_rng(9)
    while True:
        levels.append(np.zeros((size, size, 4), np.uint8))
        if size == 1:
            break
        size //= 2
    levels[0][:] = rng.integers(0, 256, size=levels[0].shape, dtype=np.uint8)
    nbytes = sum(a.nbytes for a in levels[:-1]) + sum(a.nbytes for a in levels[1:])
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        for a, c in zip(levels[:-1], levels[1:]):
            oracle.blit(a, abi.FORMAT_R8G8B8A8_UNORM, c, abi.FORMAT_R8G8B8A8_UNORM, (0, 0, a.shape[1], a.shape[0]),
                        (0, 0, c.shape[1], c.shape[0]), abi.FILTER_LINEAR)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    ms = statistics.median(times) * 1e3
    v = round(nbytes / (ms * 1e-3) / 1e9, 3)
    sample = "12-level LINEAR mip chain of a 2048^2 RGBA8 texture (bounded sample of the 8192^2 chain)"
    line = {"impl": "reference", "metric": "GB/s", "value": v, "unit": "GB/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "config": {"workload": WORKLOADS["blitter"]},
            "cpu_baseline": {"value": v, "unit": "GB/s", "cores": 1, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_batch(args, b, world, threads):
    """Reference arm of the batch workload: every step times the oracle on a
    bounded sample of draws, scaled to the whole batch."""
    per_step = max(2.0, min(10.0, 150.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_baseline_batch(b, bounded_s=per_step, threads=threads)
    vals = [cpu_baseline_batch(b, bounded_s=per_step, threads=threads) for _ in range(args.steps)]
    value = statistics.mean(v["value"] for v in vals)
    line = {
        "impl": "reference",
        "metric": "draws/s", "value": round(value, 3), "unit": "draws/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * b.n / value, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 + int32 fixed point (RGBA8 / D32F out)",
        "data": "synthetic (seeded generator, swiftshader_gb300.scenes.scene_batch)",
        "config": {"workload": WORKLOADS["batch"]},
        "parallelism": "host threads",
        "cpu_baseline": {"value": round(value, 3), "unit": "draws/s", "cores": threads, "kind": "port",
                         "sample": "per step: " + vals[-1]["sample"]},
        "e2e": {"value": round(value, 3), "unit": "draws/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-vs-per-draw sample")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint / forward timings")
    ap.add_argument("--no-blitter", action="store_true", help="skip the clear / resolve / mip-chain timings")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default raster configuration (16x16 bins, hiz on)")
    ap.add_argument("--raster-config", default=None, help="fix the raster configuration, e.g. 16x16:0 (bins, hiz); no autotuning")
    ap.add_argument("--batch-draws", type=int, default=BATCH_FULL["n_draws"], help="--workload batch: draws")
    ap.add_argument("--batch-tri-max", type=int, default=BATCH_FULL["tri_max"], help="--workload batch: largest draw")
    ap.add_argument("--no-per-draw", action="store_true", help="--workload batch: skip the per-draw comparison")
    ap.add_argument("--views", type=int, default=256, help="--workload views: views")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload in ("sphere", "views"):
        run_adjoint(args)
    elif args.workload == "blitter":
        run_blitter(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
