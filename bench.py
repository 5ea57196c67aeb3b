"""Benchmark of the GB300 draw path.

Default workload (one JSON line): the instanced scene at 1920x1080 - the
64x32 UV sphere drawn as 1024 instances with per-instance model matrices,
Blinn-Phong with 4 point lights and a 1024^2 RGBA8 noise texture, RGBA8
colour + float32 depth. One step = one frame: clear + draw_instanced.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c2|c1|c3|c4]
  python bench.py --impl reference ...   # the CPU restatement of the reference path

Metric: frames/s (whole job, all ranks). value = device-timed frames with
inputs resident in HBM; L2 is flushed (a 256 MiB write) between timed frames.
e2e = the same frames through the C ABI from pinned host buffers: per frame
the uniform block and instance matrices are uploaded, the frame is drawn and
the colour attachment is read back to pinned host memory.
"""
import argparse
import atexit
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/s at 1080p, batched vs per-draw GPU (exact coverage); adjoint ms/frame"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    p.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "sg"])
    p.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-render timing")
    p.add_argument("--no-extra", action="store_true", help="default workload only: skip the c3 and c4 sub-objects")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-sample-seconds", type=float, default=15.0)
    p.add_argument("--ref-seconds", type=float, default=0.0,
                   help="reference arm: time full frames for about this long (median) instead of --steps")
    p.add_argument("--tile", default="auto", help="screen tile WxH (8x8 .. 64x64) or auto (autotuner)")
    p.add_argument("--raster", default="auto", choices=["auto", "tiled", "untiled"],
                   help="order-free launches: the autotuner's pick (with --tile auto; tiled with a fixed tile), on "
                        "screen tiles, or untiled")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


SCENE_GRAPH_KW = dict(width=3840, height=2160, groups=32, per_group=8, seed=21, tex_size=512, lon=64, lat=32)


def max_over_ranks(value, world, device="cuda"):
    """The largest of a per-rank float over the process group (the slowest
    replica's time); the value itself on one rank."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, steps, seconds):
    """Whole-job frames/s of `world` replicas that each drew `steps` frames,
    timed by the slowest one."""
    return world * steps / seconds


def usable_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline_subprocess(workload, seconds):
    """The oracle port timed in a fresh process (no CUDA context; the GPU
    process's CPU affinity can be narrower than the host's), through the
    reference arm bounded to about `seconds` of full frames."""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--workload", workload,
           "--steps", "1", "--warmup", "1", "--ref-seconds", str(seconds)]
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600 + 20 * seconds, env=env)
    if res.returncode != 0:
        raise RuntimeError(f"cpu baseline failed: {res.stderr[-2000:]}")
    line = json.loads(res.stdout.strip().splitlines()[-1])
    return line["cpu_baseline"]


def workload_config(name):
    from softlight_gb300 import scenes as S
    if name == "c1":
        return S.build_c1, {}, {"workload": "single UV sphere 64x32 (4096 tris), Lambert, 256^2 checker", "resolution": "640x480"}
    if name == "c2":
        return S.build_c2, {}, {"workload": "instanced UV sphere 64x32 x 1024 instances (4.19M tris), Blinn-Phong 4 point lights, 1024^2 RGBA8 noise texture",
                                 "resolution": "1920x1080", "instances": 1024}
    if name == "c3":
        return S.build_c3, {}, {"workload": "2M-triangle soup, 30% back-facing, 10% near-plane clipped, alpha blend, 2048^2 texture",
                                 "resolution": "1920x1080"}
    if name == "sg":
        return S.build_scene_graph, dict(SCENE_GRAPH_KW), {"workload": "scene graph 32x8 mesh nodes, 3840x2160, 512^2 textures, "
                                                                  "64x32 meshes, 40-degree cull frustum", "resolution": "3840x2160"}
    if name == "c5":
        return S.build_c5, {}, {"workload": "10k-triangle noise-displaced sphere, float32 vertex colours x 256^2 float32 texture, "
                                             "visibility map recorded", "resolution": "512x512"}
    return S.build_c4, {}, {"workload": "256 uneven meshes (12..65k tris), per-draw 512^2 textures, Lambert+ambient, one batched launch",
                             "resolution": "3840x2160", "draws": 256}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms; only the
    samples taken inside the timed windows (begin() .. end()) count."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []      # (perf_counter, line)
        self.windows = []    # (t0, t1)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            atexit.register(self._stop)
            # the first sample takes a moment: start timing once it arrived
            t_end = time.perf_counter() + 3.0
            while not self.lines and time.perf_counter() < t_end and self.proc.poll() is None:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def begin(self):
        self.windows.append([time.perf_counter(), None])

    def end(self):
        if self.windows and self.windows[-1][1] is None:
            self.windows[-1][1] = time.perf_counter()

    def _stop(self):
        if self.proc and self.proc.poll() is None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.05)     # the sample covering the end of the last window
            self._stop()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, ln in self.lines:
            if not any(t0 <= t <= (t1 if t1 is not None else t) for t0, t1 in self.windows):
                continue
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm),
                "interval_ms": 20}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def cpu_calibration(workload):
    """The port's speed relative to the reference's own sources built here
    (portable branches, same thread count), from profiles/cpu_calibration.json."""
    path = os.path.join(ROOT, "profiles", "cpu_calibration.json")
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        d = json.load(fh)
    r = d.get("port_over_reference", {}).get(workload)
    if r is None:
        return None
    return {"port_over_reference_speed": r, "threads": d.get("threads"), "host": d.get("host"),
            "reference_build": d.get("reference_build"), "source": "profiles/cpu_calibration.json"}


def kernel_sources_digest():
    """SHA-256 (16 hex digits) of the sources the draw-path kernels are built
    from (softlight_gb300/csrc and include), to tell whether a recorded ncu
    figure still describes the kernels that run."""
    import hashlib
    h = hashlib.sha256()
    for d in (os.path.join(ROOT, "softlight_gb300", "csrc"), os.path.join(ROOT, "include")):
        for f in sorted(os.listdir(d)):
            with open(os.path.join(d, f), "rb") as fh:
                h.update(f.encode() + b"\0" + fh.read())
    return h.hexdigest()[:16]


def profiled_traffic(workload, kernel):
    """DRAM bytes per launch of `kernel` at `workload` from an ncu capture
    (profiles/traffic.json), with where it came from; None when no capture
    exists or the kernel sources changed since the capture."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None, "no ncu capture recorded"
    with open(path) as fh:
        d = json.load(fh)
    entry = d.get(workload, {}).get(kernel)
    if entry is None:
        return None, f"no ncu capture of {kernel} at this workload"
    if isinstance(entry, dict):
        if entry.get("sources") != kernel_sources_digest():
            return None, f"ncu capture {entry.get('capture')} is of other kernel sources ({entry.get('sources')})"
        return entry["bytes"], f"ncu capture {entry.get('capture')} (dram__bytes_read.sum + dram__bytes_write.sum), kernel sources {entry['sources']}"
    return None, "ncu capture without a kernel-source digest"


def run_reference(args):
    """--impl reference: the reference path's CPU restatement on all host cores."""
    rank, world, _ = dist_env()
    if world > 1 and rank != 0:
        return
    builder, kwargs, cfg = workload_config(args.workload)
    import oracle
    threads = usable_cores()
    ctx = oracle.Context(num_threads=threads)
    scene = builder(ctx, **kwargs)
    for _ in range(args.warmup):
        scene.render()
    if args.ref_seconds > 0:
        times = []
        t_end = time.perf_counter() + args.ref_seconds
        while (time.perf_counter() < t_end or len(times) < 2) and len(times) < 50:
            t0 = time.perf_counter()
            scene.render()
            times.append(time.perf_counter() - t0)
        fps = 1.0 / statistics.median(times)
        sample = f"{len(times)} full frames, median"
    else:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            scene.render()
        fps = args.steps / (time.perf_counter() - t0)
        sample = "full frames, mean over the timed steps"
    _, frags = oracle.last_stats(ctx)
    line = {"impl": "reference", "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / fps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": threads, "kind": "port",
                             "sample": sample + "; reference sources cannot be shipped to this host, so the oracle port "
                                                "(CPU restatement of the reference's portable path) is timed",
                             "fragments_per_frame": frags, "mfragments_per_s": fps * frags / 1e6,
                             "calibration": cpu_calibration(args.workload)},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def scene_graph_timing(sg, torch, flush, steps, warmup, cpu_seconds):
    """Scene graph at 2160p: 32 groups x 8 mesh nodes (+ grandchildren and
    late children; 64x32 spheres, tori, grids; 512^2 textures), three
    transforms changed per frame, culled against a 40-degree frustum. A frame
    is clear + transform changes + update + draw list. Device time with CUDA
    events after an L2 flush; host wall time per frame (the host side of the
    producer, its per-draw validation included); the oracle port on all host
    cores for the same frames."""
    from softlight_gb300 import scenes as S
    kw = dict(SCENE_GRAPH_KW)
    ctx = sg.Context()
    s = S.build_scene_graph(ctx, **kw)
    ctx.set_tile_size(16, 16)
    stream = torch.cuda.ExternalStream(ctx.stream_handle())
    for _ in range(max(3, warmup)):
        s.render()
    ctx.finish()
    dev = []
    for i in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xFF)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        s.render()
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        dev.append(e0.elapsed_time(e1))
    ctx.finish()
    t0 = time.perf_counter()
    for _ in range(steps):
        s.render()
    ctx.finish()
    host_ms = (time.perf_counter() - t0) * 1000.0 / steps
    draws = len(s.read_models())
    ctx.close()
    out = {"workload": "scene graph 32x8 mesh nodes, 3840x2160, 512^2 textures, 64x32 meshes, 40-degree cull frustum",
           "nodes": draws, "triangles_submitted": s.num_triangles,
           "device_ms": statistics.median(dev), "frames_per_s": 1000.0 / statistics.median(dev),
           "wall_ms": host_ms, "wall_frames_per_s": 1000.0 / host_ms, "launches_per_frame": 10}
    if cpu_seconds > 0:
        out["cpu_baseline"] = cpu_baseline_subprocess("sg", cpu_seconds)
    return out


def adjoint_timing(sg, torch, flush, steps, warmup):
    """Differentiable render (512x512, 10k-triangle displaced sphere, vertex
    colours x 256^2 float texture): device time of the forward (clear + exact
    draw recording the visibility map + model image) and of the adjoint
    (gradient buffers zeroed + adjoint kernel), each frame timed with CUDA
    events on the context's stream after an L2 flush."""
    from softlight_gb300 import scenes as S
    ctx = sg.Context()
    s = S.build_c5(ctx)
    tw, th, vb = ctx.autotune([sg.api.DrawCmd(s.mesh, 1, s.shader)], s.fbo, s.clear_color, s.clear_depth)
    stream = torch.cuda.ExternalStream(ctx.stream_handle())
    img = torch.empty(s.height, s.width, 4, device="cuda")
    target = torch.rand(s.height, s.width, 4, device="cuda", generator=torch.Generator("cuda").manual_seed(5))
    nv = s.pos.shape[0]
    dvert = torch.zeros(nv * 9, device="cuda")
    dtex = torch.zeros(s.tex.size, device="cuda")
    d_img = torch.empty_like(img)

    def forward():
        s.render()
        ctx.diff_shade(s.mesh, s.shader, s.fbo, img.data_ptr(), img.numel())

    def backward():
        with torch.cuda.stream(stream):
            dvert.zero_()
            dtex.zero_()
        ctx.draw_adjoint(s.mesh, s.shader, s.fbo, d_img.data_ptr(), d_img.numel(), dvert.data_ptr(), dvert.numel(),
                         dtex.data_ptr(), dtex.numel())

    def timed(fn, k):
        out = []
        for i in range(k):
            with torch.cuda.stream(stream):
                flush.fill_(i & 0xFF)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            fn()
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            out.append(e0.elapsed_time(e1))
        return out

    for _ in range(max(3, warmup)):
        forward()
    ctx.finish()
    with torch.cuda.stream(stream):
        d_img.copy_(2.0 * (img - target))
    for _ in range(max(3, warmup)):
        backward()
    ctx.finish()
    f_ms = statistics.median(timed(forward, steps))
    b_ms = statistics.median(timed(backward, steps))
    ctx.close()
    return {"workload": "differentiable render 512x512: 10k-triangle noise-displaced sphere, float32 vertex colours "
                        "x 256^2 float32 RGBA texture, L2 image loss",
            "unit": "ms/frame", "forward_ms": f_ms, "adjoint_ms": b_ms, "adjoint_over_forward": b_ms / f_ms,
            "forward": "clear + exact draw recording the visibility map + model image (slg_diff_shade)",
            "adjoint": "gradient buffers zeroed + slg_draw_adjoint (forward recomputed per pixel)",
            "tile": f"{tw}x{th}", "vertex_block": vb, "l2": "flushed before each timed frame"}


def launches_per_frame(scene, tile):
    """Kernels one frame launches (counted from the launch sequence, matched
    against the ncu launch lists in profiles/): two clears, then per draw
    launch the vertex cache (indexed draws of 64K or more triangles),
    vs_setup, clip and the launch mark, plus the path's tile-list and raster
    kernels: untiled order-free raster + resolve + counter reset; tiled
    order-free tile scan + fill + raster; blended with key-order lists (grids
    of at most 4 096 tiles) bin numbering (3) + count + chunk scan + tile
    scan + fill + raster, else tile scan + fill + tile sort + raster."""
    from softlight_gb300 import api as A
    tw, th = tile
    tiles = -(-scene.width // tw) * -(-scene.height // th)
    # order-free untiled: raster + resolve + counter reset; on tiles: tile
    # scan + fill + raster (three either way)
    path = (8 if tiles <= 4096 else 4) if scene.blending else 3
    per_launch = 3 + path

    def cache(tris, indexed):
        return 1 if indexed and tris >= 65536 else 0
    if scene.batched:
        indexed = any(m.mode == A.RENDER_MODE_INDEXED_TRIANGLES for (m, _, _) in scene.draws)
        return 2 + per_launch + cache(scene.num_triangles, indexed)
    total = 2
    for (m, n, _) in scene.draws:
        tris = n * (m.elementEnd - m.elementBegin) // 3
        total += per_launch + cache(tris, m.mode == A.RENDER_MODE_INDEXED_TRIANGLES)
    return total


def time_workload(name, args, sg, torch, flush, world, local, rank, clocks=None, cpu_seconds=0.0):
    """Times one workload: `args.steps` frames with CUDA events on the
    context's stream after an L2 flush each, per-stage times, the same
    frames issued one draw per launch for batched scenes, and the frames end
    to end through the C ABI from pinned host buffers. Returns a dict of the
    figures; clocks, when given, samples nvidia-smi during the timed frames."""
    import numpy as np
    builder, kwargs, cfg = workload_config(name)
    ctx = sg.Context()
    scene = builder(ctx, **kwargs)
    stream = torch.cuda.ExternalStream(ctx.stream_handle())
    cmds = [sg.api.DrawCmd(m, n, sh) for (m, n, sh) in scene.draws]
    if args.raster != "auto":
        ctx.set_raster_mode(2 if args.raster == "tiled" else 3)
    if args.tile == "auto":
        tw, th, vb = ctx.autotune(cmds, scene.fbo, scene.clear_color, scene.clear_depth)
    else:
        tw, th = (int(v) for v in args.tile.split("x"))
        vb = 128
        ctx.set_tile_size(tw, th)
    untiled = ctx.untiled_raster()
    if scene.batched:
        ctx.set_batch_graphs(True)

    def timed_frames(k, profile):
        """k frames, each timed with CUDA events on the context's stream,
        L2 flushed before each; optional per-stage event times."""
        ctx.profile_stages(profile)
        ms, stages = [], []
        for i in range(k):
            with torch.cuda.stream(stream):
                flush.fill_(i & 0xFF)
                ev0 = torch.cuda.Event(enable_timing=True)
                ev1 = torch.cuda.Event(enable_timing=True)
                ev0.record(stream)
            scene.render()
            with torch.cuda.stream(stream):
                ev1.record(stream)
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
            if profile:
                stages.append(ctx.stage_times())
        ctx.finish()
        ctx.profile_stages(False)
        return ms, stages

    for _ in range(max(3, args.warmup)):
        scene.render()
    ctx.finish()

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    # clocks are sampled over the timed frames, the stage-timed ones and the
    # end-to-end frames below
    if clocks is not None:
        clocks.__enter__()
        clocks.begin()
    step_ms, _ = timed_frames(args.steps, False)
    _, stage_ms = timed_frames(max(3, min(args.steps, 10)), True)
    if clocks is not None:
        clocks.end()
    torch.cuda.synchronize()
    total_ms = max_over_ranks(sum(step_ms), world)
    fps = replica_throughput(world, args.steps, total_ms / 1000.0)
    out = {"workload": cfg["workload"], "config": cfg, "value": fps, "unit": "frames/s", "ms_per_step": total_ms / args.steps,
           "tile": f"{tw}x{th}", "vertex_block": vb, "batched_graph": bool(scene.batched),
           "order_free_raster": "untiled" if untiled else "tiles",
           "triangles_per_frame": scene.num_triangles,
           "launches_per_frame": launches_per_frame(scene, (tw, th))}

    if scene.batched:
        # the same frames issued as one slg_draw call per mesh
        scene.batched = False
        for _ in range(2):
            scene.render()
        pd_ms, _ = timed_frames(args.steps, False)
        scene.batched = True
        out["per_draw"] = {"value": args.steps / (sum(pd_ms) / 1000.0), "unit": "frames/s",
                           "launches_per_frame": 2 + 6 * len(scene.draws),
                           "batched_speedup": (sum(pd_ms) / max(total_ms, 1e-9))}

    # end to end through the C ABI with pinned host buffers: every uniform
    # block of the frame (one slg_ubo_assign_many call), the instance
    # matrices, the frame, and the colour attachment read back
    h2d = 0
    ubo_ids = [u for u, _ in scene.frame_ubos]
    nbytes = max(len(b) for _, b in scene.frame_ubos)
    ubo_host = torch.zeros(len(ubo_ids), nbytes, dtype=torch.uint8, pin_memory=True).numpy()
    for k, (_, b) in enumerate(scene.frame_ubos):
        ubo_host[k, :len(b)] = np.frombuffer(b, dtype=np.uint8)
    h2d += ubo_host.nbytes
    inst = getattr(scene, "instance_matrices", None)
    if inst is not None:
        inst_host = torch.empty(inst[1].nbytes, dtype=torch.uint8, pin_memory=True).numpy()
        inst_host[:] = inst[1].view(np.uint8).reshape(-1)
        h2d += inst_host.nbytes
    color_bytes = scene.height * scene.width * sg.api.BYTES_PER_COLOR[scene.color_type]
    color_host = torch.empty(color_bytes, dtype=torch.uint8, pin_memory=True).numpy()

    def read_color():
        ctx.texture_read(scene.color_tex, (color_bytes,), np.uint8, out=color_host)
    for _ in range(2):
        scene.render()
        read_color()
    if world > 1:
        torch.distributed.barrier()
    if clocks is not None:
        clocks.begin()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.ubo_assign_many(ubo_ids, ubo_host)
        if inst is not None:
            ctx.vbo_assign(inst[0], inst_host)
        scene.render()
        read_color()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    if clocks is not None:
        clocks.end()
        clocks.__exit__(None, None, None)
    out["e2e"] = {"value": replica_throughput(world, args.steps, e2e_s), "unit": "frames/s", "h2d_bytes_per_step": h2d,
                  "d2h_bytes_per_step": color_bytes}

    # roofline of the dominant stage
    stages = np.asarray(stage_ms)
    mean_stage = stages.mean(0)
    names = ["vs_setup", "tile_scan", "bin_fill", "raster"]
    geo = scene.geometry_bytes
    frame_bytes = geo + scene.texture_bytes + scene.framebuffer_bytes()
    if untiled and not scene.blending:
        # the untiled raster's walk runs inside vs_setup_kernel and its
        # resolve in the raster stage: one kernel group over both stages,
        # with the raster's bytes and the geometry
        kernel = "vs_setup+raster"
        kernel_ms = float(mean_stage[0] + mean_stage[3])
        algo_bytes = frame_bytes
    else:
        dom = int(np.argmax(mean_stage))
        kernel = names[dom]
        kernel_ms = float(mean_stage[dom])
        algo_bytes = {"vs_setup": geo, "tile_scan": 0, "bin_fill": 0, "raster": scene.texture_bytes + scene.framebuffer_bytes()}[kernel]
    peak, peak_kind = measured_peaks()
    achieved = algo_bytes / (kernel_ms / 1000.0) / 1e9
    traffic, traffic_note = profiled_traffic(name, kernel)
    out["roofline"] = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                       "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic, "traffic_source": traffic_note,
                       "algorithmic_bytes": algo_bytes, "kernel_ms": kernel_ms,
                       "stage_ms": {n: float(v) for n, v in zip(names, mean_stage)},
                       "frame_algorithmic_bytes": frame_bytes,
                       "frame_frac": frame_bytes / (total_ms / args.steps / 1000.0) / 1e9 / peak}
    ctx.close()

    if rank == 0 and world == 1 and cpu_seconds > 0:
        cpu = cpu_baseline_subprocess(name, cpu_seconds)
        out["cpu_baseline"] = cpu
        frags = cpu.get("fragments_per_frame")
        if frags:
            out["fragments_per_frame"] = frags
            out["mfragments_per_s"] = fps * frags / 1e6
            out["mfragments_source"] = ("fragments passing the depth test per frame in the reference's sequential "
                                        "model (oracle count of the same frame; the GPU frame is bit-exact to it)")
    return out


def run_gpu(args):
    import torch
    import softlight_gb300 as sg

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    if args.workload == "sg":
        raise SystemExit("the scene-graph workload is timed inside the default run (its \"scene_graph\" key); "
                         "--workload sg is for --impl reference")
    sg.build()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    cpu_s = 0.0 if args.no_cpu_baseline else args.cpu_sample_seconds
    clocks = ClockSampler(local)
    head = time_workload(args.workload, args, sg, torch, flush, world, local, rank, clocks=clocks,
                         cpu_seconds=cpu_s if rank == 0 and world == 1 else 0.0)
    extra = {}
    if args.workload == "c2" and not args.no_extra:
        # the hard 1080p configuration (2M blended soup) and the batched 2160p
        # scene, each with its own CPU baseline
        for name in ("c3", "c4"):
            extra[name] = time_workload(name, args, sg, torch, flush, world, local, rank,
                                        cpu_seconds=min(cpu_s, 10.0) if rank == 0 and world == 1 else 0.0)

    if rank == 0:
        cfg = dict(head["config"])
        cfg.update({"l2": "flushed between timed frames (256 MiB write)", "tile": head["tile"],
                    "vertex_block": head["vertex_block"], "tuned": args.tile == "auto", "batched_graph": head["batched_graph"],
                    "order_free_raster": head["order_free_raster"], "triangles_per_frame": head["triangles_per_frame"]})
        line = {"metric": METRIC, "value": head["value"], "unit": "frames/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": cfg, "e2e": head["e2e"], "roofline": head["roofline"],
                "cpu_baseline": head.get("cpu_baseline"), "clocks": clocks.summary(),
                "gpu_launches": args.steps * head["launches_per_frame"]}
        for k in ("fragments_per_frame", "mfragments_per_s", "mfragments_source", "per_draw"):
            if k in head:
                line[k] = head[k]
        for name, d in extra.items():
            d = dict(d)
            d.pop("config", None)
            line[name] = d
        if not args.no_adjoint and world == 1:
            line["adjoint"] = adjoint_timing(sg, torch, flush, max(args.steps, 5), args.warmup)
            line["scene_graph"] = scene_graph_timing(sg, torch, flush, max(args.steps, 5), args.warmup,
                                                     0 if args.no_cpu_baseline else min(10.0, args.cpu_sample_seconds))
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
