#!/usr/bin/env python3
"""Benchmark of the dependency-tracked radiance cache on GB300.

Workload: the reference's headline timing case (cuda/poc_gpu.cu `timing` mode, published as
reference/cuda_rtx4060/timing_1M.jsonl) on the reference's own timing scene
cuda/scenes/scene_scale_1M.bin (1,082,802 cache points, 58 triangles, 3 point lights, 5 states
switched every 60 frames; shipped gzip-compressed in tests/golden/), method "v4-A2C suivi 1/4"
(adaptive ray allocation, dependency masks on a 8 x 4 x 4 transit grid tracked one frame in
four, verified dormant-light memory, history ramp).  A seeded stand-in room of the same size
(render_engine_gb300/scene.py: box_room) is measured the same way as a second line.

One step = one frame of the whole cache (trace + update of every cache point, plus the
event kernels when the state changes).  With fewer than 120 timed frames the timed window is
centred on the first state change (frame 60): the frames before the warm-up run untimed, so
that both arms time an event frame and the verification frames after it.  Timed frames are
separated by an L2 flush (a 512 MB write) and timed with CUDA events on the stream the
kernels run on.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference runs the reference's own kernels (the unmodified cuda/poc_gpu.cu compiled
for sm_103a into oracle/_ref/, driven by oracle/refrun.cpp) on the same scene, method and
frames, timed the same way.
"""
from __future__ import annotations

import argparse
import gzip
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/s and Mrays/s at 1080p, 1M cache pts; 30-frame post-event luma err % vs FP64"
POINTS = 1_082_802
METHOD = "v4-A2C suivi 1/4"
FRAMES_PER_STATE = 60
PUBLISHED_FPS = 1000.0 / 1.44806   # timing_1M.jsonl:10 (RTX 4060): trace+decide+update+swap = 1.448 ms
SCENE_1M = os.path.join(ROOT, "tests", "golden", "scene_scale_1M.bin.gz")
POST_FRAMES, PRE_FRAMES = 30, 20     # the reference's post / pre windows (poc_gpu.cu:1428-1429)


def _json_default(o):
    """numpy scalars (a bool or a float that came from an array) as Python values."""
    if hasattr(o, "item"):
        return o.item()
    raise TypeError("not JSON serializable: %r" % (o,))


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--points", type=int, default=POINTS)
    ap.add_argument("--method", default=METHOD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-frames", type=int, default=12)
    ap.add_argument("--profile", choices=["frame", "street", "hashgrid", "mlp", "adjoint", "taa", "paths"], default=None,
                    help="no timing: run --steps frames of state 0 of the headline scene (frame), three resolve "
                         "passes of the hash-grid table (hashgrid), two inference and training passes of the MLP "
                         "(mlp) or one 16-sweep adjoint of a 16-light room of --points points (adjoint), --steps "
                         "frames of the taa mode (taa), --steps camera-path passes at --width x --height (paths) "
                         "or --steps frames of state 0 of the prepared street workload (street; --ray-queue: "
                         "through the ray queue), for an ncu capture, and exit")
    ap.add_argument("--ray-queue", action="store_true")
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    return ap.parse_args()


def profile_run(args):
    """The small, untimed workloads the committed ncu summaries were captured on."""
    import torch
    from render_engine_gb300 import methods as M
    from render_engine_gb300 import native as N
    from render_engine_gb300 import scene as S
    if args.profile == "frame":
        ctx = N.Context()
        ctx.load_bytes(headline_scene(args.points)[0])
        ctx.begin(M.by_name(M.timing_methods(), args.method), 0, 11)
        for _ in range(args.steps):
            ctx.frame(0)
        ctx.sync()
        ctx.close()
        return
    if args.profile == "street":
        ctx = N.Context(flags=N.FLAG_RAY_QUEUE if args.ray_queue else 0, expect_lights=SCALE_CONFIGS["street"]["lamps"])
        ctx.load_bytes(scale_scene("street"))
        ctx.begin(M.by_name(M.timing_methods(), SCALE_CONFIGS["street"]["method"]), 0, 11)
        for _ in range(args.steps):
            ctx.frame(0)
        ctx.sync()
        ctx.close()
        return
    if args.profile == "mlp":
        mlp_bench(torch.cuda.current_stream(), reps=2)
        torch.cuda.synchronize()
        return
    if args.profile == "paths":
        paths_bench(reps=args.steps, warm=0, width=args.width, height=args.height)
        torch.cuda.synchronize()
        return
    if args.profile == "taa":
        ctx = N.Context()
        ctx.load_bytes(taa_scene(args.points))
        ctx.taa_begin(0.1, 1.0, 2, 0, 5000)
        for f in range(args.steps):
            ctx.taa_frame(taa_state(f), want_err=True)
        ctx.close()
        return
    if args.profile == "adjoint":
        import numpy as np
        ctx = N.Context()
        info = ctx.load_bytes(S.write(S.box_room(points=args.points, seed=0, lights=16)))
        w = np.full(info["np"], 1.0 / info["np"], np.float32)
        ctx.adjoint(0, w, K=16, seed=5, iterations=16)
        ctx.close()
        return
    from render_engine_gb300 import hashgrid as H
    cap, live = 1 << 24, 1 << 23
    hg = H.HashGrid(H.make_config(capacity=cap, cell=0.02, max_depth=4, acc_frames=64, stale_frames=1000, tracing_distance=50.0))
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    pos = torch.rand(live, 3, device="cuda", generator=g) * torch.tensor([8.0, 4.0, 3.0], device="cuda")
    nrm = torch.randn(live, 3, device="cuda", generator=g)
    rgb = torch.rand(live, 3, device="cuda", generator=g)
    entry = torch.empty(live, dtype=torch.int32, device="cuda")
    hg.insert(pos, nrm, entry)
    for _ in range(3):
        hg.accumulate(entry, rgb)
        hg.resolve()
    torch.cuda.synchronize()
    hg.close()


def street_scene(points: int):
    """Format-3 street: ground, 40 buildings with facades subdivided into 0.58 m cells
    (about 200 k triangles, median-split tree), three lamp-post lights, the movable cube."""
    from render_engine_gb300 import scene as S
    return S.street_scene(points=points, buildings=40, facade_cell=0.58, size=200.0)


# The at-scale workloads: seeded procedural meshes made into format-3 scenes by the library's
# GPU preparation (rc_prep_mesh_params, linear BVH, cell-grid cache points, lamps and cube placed
# by probe rays), without references (timing only).  Both arms load the same scene file.
SCALE_CONFIGS = {
    "street": {"mesh": dict(kind="street", buildings=40, seed=0, facade_cell=0.58, size=200.0), "points": 530_000,
               "lamps": 8, "method": "v4-A2C suivi 1/4",
               "desc": "procedural street (ground + 40 buildings 5-30 m tall, facades in 0.58 m cells: 199,346 triangles), "
                       "8 lamp lights, ~530 k cache points"},
    "city": {"mesh": dict(kind="city", buildings=400, seed=0, facade_cell=1.6), "points": 1_000_000, "lamps": 32,
             "method": "v3 complet",
             "desc": "procedural city (400 buildings 5-60 m tall on a 20 x 20 block grid, facades in 1.6 m cells: ~1 M triangles), "
                     "32 lamp lights, ~1 M cache points; a method without dormant-light memory (the reference's per-point stale "
                     "mask holds 8 lights)"},
}


def scale_scene(name: str) -> bytes:
    """The prepared scene of an at-scale workload, cached on the machine's temporary directory
    (the two arms run as separate processes)."""
    import tempfile
    cfg = SCALE_CONFIGS[name]
    d = os.path.join(tempfile.gettempdir(), "rc_bench_scenes")
    os.makedirs(d, exist_ok=True)
    key = "%s_%d_%d" % (name, cfg["points"], cfg["lamps"])
    path = os.path.join(d, key + ".bin")
    if not os.path.exists(path):
        from render_engine_gb300 import native as N
        from render_engine_gb300 import scene as S
        m = dict(cfg["mesh"])
        kind = m.pop("kind")
        V, alb, ds = S.street_mesh(**m) if kind == "street" else S.city_mesh(**m)
        mesh = os.path.join(d, key + ".msh")
        with open(mesh, "wb") as f:
            f.write(S.write_msh1(V, alb, ds))
        ctx = N.Context()
        ctx.prep_mesh(mesh, path + ".tmp", points=cfg["points"], lamps=cfg["lamps"], ref_iterations=-1)
        ctx.close()
        os.replace(path + ".tmp", path)
    return open(path, "rb").read()


def sequence(n: int, ns: int = 5) -> list[int]:
    return [(f // FRAMES_PER_STATE) % ns for f in range(n)]


def window_start(warmup: int, steps: int) -> int:
    """First timed frame.  Fewer than 120 timed frames are centred on the first state change
    (frame 60), so that the window holds an event frame and the verification frames after it;
    the frames before the warm-up run untimed.  Longer runs start right after the warm-up."""
    return max(warmup, FRAMES_PER_STATE - steps // 2)


def headline_scene(points: int) -> tuple[bytes, str]:
    """The reference's own 1,082,802-point timing scene when it is present and the size asked
    for, else the seeded stand-in room of that size."""
    from render_engine_gb300 import scene as S
    if points == POINTS and os.path.exists(SCENE_1M):
        return gzip.decompress(open(SCENE_1M, "rb").read()), \
            "the reference's timing scene cuda/scenes/scene_scale_1M.bin (1082802 cache points, 58 triangles, 3 point lights, 5 states)"
    return S.write(S.box_room(points=points, seed=0)), \
        "seeded stand-in for the reference's scene_scale_1M.bin (box room, %d cache points, 62 triangles, 3 point lights, 5 states)" % points


class Clocks:
    """nvidia-smi sampling during the timed region (every 200 ms)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.p = None
        self.device = device
        self.t0 = time.perf_counter()
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        # at least one sampling period after the start (a short timed region would end before the
        # first sample); the GPU idles meanwhile, so the samples taken then are marked idle
        rest = 0.45 - (time.perf_counter() - self.t0)
        if rest > 0:
            time.sleep(rest)
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic() -> float | None:
    """DRAM bytes of one launch of the fused frame kernel (a tracked frame of the headline scene)
    from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "k_frame_fused_scene_scale_1m.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def algorithmic_bytes(np_: int, tracked: bool, ramp: bool) -> float:
    """Bytes one fused frame kernel must move for Np points (each array touched once):
    reads P 16, N 16, n 4, own cache 16, gathered albedo+direct light 16 and cache 16 at the
    hit points; writes cache 16, n 4; ramp: age read+write 8; tracked frames: shadow-voxel
    mask gather 16 and dependency-mask read 16 + write 16."""
    b = 16 + 16 + 4 + 16 + 16 + 16 + 16 + 4
    if ramp:
        b += 8
    if tracked:
        b += 48
    return float(np_) * b


def max_over_ranks(x: float, dist, device) -> float:
    """The slowest rank's value (the timed region ends when every replica has finished)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, max_ms: float) -> float:
    """Units all replicas processed per second of the slowest replica's timed region."""
    return units_per_rank * world / (max_ms * 1e-3)


def setup_dist(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    return world, rank, local, dist


def time_frames(ctx, method, seq, s0, args, stream, flush, dist=None):
    """Frames [0, s0 - W) untimed, W warm-up frames, then the timed frames [s0, s0 + K), each
    after an L2 flush, between CUDA events on the library's stream.  Returns per-frame times
    and the kind of each timed frame (event: the state changed; fused: one fused kernel;
    split: trace and update as separate kernels)."""
    import torch
    from render_engine_gb300 import native as N
    # every state built before the frames (as the reference's load does): no build shares the GPU
    # with a timed frame
    ctx.build_states()
    ctx.begin(method, seq[0], 11)
    for f in range(s0):
        ctx.frame(seq[f])
    torch.cuda.synchronize()
    K = args.steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    fused, kinds, tracked = [], [], []
    l0 = ctx.stats()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(torch.cuda.current_device())
    wall0 = time.perf_counter()
    for k in range(K):
        f = s0 + k
        flush.zero_()
        starts[k].record(stream)
        ctx.frame(seq[f])
        ends[k].record(stream)
        nk = ctx.scalar(N.S_LAST_FRAME_KERNELS)
        fu = ctx.scalar(N.S_LAST_FRAME_FUSED) == 1
        fused.append(fu and nk == 1)   # exactly one launch: the roofline's kernel
        kinds.append("event" if seq[f] != seq[f - 1] else ("fused" if fu else "split"))
        tracked.append(f % method.track_every == 0)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    st = ctx.stats()
    ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    return {"ms": ms, "fused": fused, "kinds": kinds, "tracked": tracked, "rays": st["rays"] - l0["rays"],
            "launches": st["launches"] - l0["launches"], "wall_s": wall, "clocks": clk}


def kinds_table(ms, kinds):
    return {kd: {"frames": sum(1 for x in kinds if x == kd),
                 "mean_ms": sum(m for m, x in zip(ms, kinds) if x == kd) / max(1, sum(1 for x in kinds if x == kd))}
            for kd in sorted(set(kinds) | {"event"})}


def run_ours(args, world, rank, local, dist):
    import torch

    from render_engine_gb300 import methods as M
    from render_engine_gb300 import native as N
    from render_engine_gb300 import scene as S

    torch.cuda.set_device(local)
    # a dedicated stream: the library's kernels, the L2 flush and the timing events all go on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    data, scene_desc = headline_scene(args.points)
    method = M.by_name(M.timing_methods(), args.method)
    s0 = window_start(args.warmup, args.steps)
    seq = sequence(s0 + args.steps)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    ctx = N.Context(device=local, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    tl = time.perf_counter()
    info = ctx.load_bytes(data)
    ctx.sync()
    first_load_ms = (time.perf_counter() - tl) * 1e3
    t = time_frames(ctx, method, seq, s0, args, stream, flush, dist)
    ms, fused, tracked = t["ms"], t["fused"], t["tracked"]
    total_ms = sum(ms)
    if dist:
        total_ms = max_over_ranks(total_ms, dist, "cuda")
        dist.barrier()
    # the 1920x1080 image pass of the same cache (one primary ray per pixel), timed the same way
    cam = N.camera(eye=(0.4, 0.4, 1.7), at=(7.6, 3.6, 0.8), fov_y_deg=75.0, width=1920, height=1080)
    state_now = seq[-1]
    ctx.render(state_now, cam, copy=False)
    nimg = 20
    cams = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nimg)]
    for e0, e1 in cams:
        flush.zero_()
        e0.record(stream)
        ctx.render(state_now, cam, copy=False)
        e1.record(stream)
    torch.cuda.synchronize()
    camera_ms = sum(e0.elapsed_time(e1) for e0, e1 in cams) / nimg
    frames = args.steps * world
    rays = t["rays"]
    np_ = info["np"]
    # dominant kernel: frames that are exactly one fused launch
    fk = [m for m, fu in zip(ms, fused) if fu]
    fk_bytes = [algorithmic_bytes(np_, tr, method.ramp) for fu, tr in zip(fused, tracked) if fu]
    kern_ms = sum(fk) / max(len(fk), 1)
    kern_bytes = sum(fk_bytes) / max(len(fk_bytes), 1)
    peak, peak_kind = measured_peaks()
    achieved = kern_bytes / (kern_ms * 1e-3) / 1e9 if fk else None
    traffic = profile_traffic()
    out = {
        "frames_per_s": whole_job_rate(args.steps, world, total_ms),
        "ms_per_step": total_ms / args.steps,
        "mrays_per_s": rays * world / (total_ms * 1e-3) / 1e6,
        "cache_updates_per_s": np_ * frames / (total_ms * 1e-3),
        "rays_per_frame": rays / args.steps,
        "launches": t["launches"],
        "wall_s": t["wall_s"],
        "clocks": t["clocks"],
        "scene": scene_desc,
        "window": {"first_timed_frame": s0, "untimed_lead_in_frames": s0 - args.warmup, "state_changes_timed":
                   sum(1 for f in range(s0, s0 + args.steps) if seq[f] != seq[f - 1])},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None, "traffic": traffic,
                     "kernel": "rc::k_frame<3,4,DEPS,FUSED=true>", "kernel_ms": kern_ms, "kernel_launches": len(fk),
                     "peak_source": peak_kind, "traffic_of": "one tracked frame (ncu, profiles/k_frame_fused_scene_scale_1m.md)"},
        "np": np_,
        "nt": info["nt"],
        "frame_kinds_ms": kinds_table(ms, t["kinds"]),
        "frame_1080p": {"cache_ms": total_ms / args.steps, "image_ms": camera_ms,
                        "frames_per_s": 1000.0 / (total_ms / args.steps + camera_ms),
                        "mrays_per_s": (rays / args.steps + 1920 * 1080) / ((total_ms / args.steps + camera_ms) * 1e-3) / 1e6,
                        "note": "cache-point frame + one primary ray per pixel at 1920x1080 shaded from the cache"},
    }
    ctx.close()
    # three end-to-end runs, the median reported (each maps no new memory unless the pool could
    # not reuse a freed block in time: the spread is in `runs`)
    e2e_runs = sorted((e2e_run(data, method, seq, local, stream, world) for _ in range(3)), key=lambda r: r["value"])
    out["e2e"] = dict(e2e_runs[1])
    out["e2e"]["runs"] = [round(r["value"], 1) for r in e2e_runs]
    out["e2e"]["first_load_in_process_ms"] = first_load_ms
    # the seeded stand-in room of the same size, the same frames
    if args.points == POINTS and os.path.exists(SCENE_1M):
        c2 = N.Context(device=local, stream=stream.cuda_stream)
        c2.load_bytes(S.write(S.box_room(points=args.points, seed=0)))
        t2 = time_frames(c2, method, seq, s0, args, stream, flush)
        c2.close()
        out["standin_room"] = {"scene": "seeded box room (render_engine_gb300/scene.py: box_room, %d points, 62 triangles)" % args.points,
                               "frames_per_s": args.steps / (sum(t2["ms"]) * 1e-3), "ms_per_step": sum(t2["ms"]) / args.steps,
                               "frame_kinds_ms": kinds_table(t2["ms"], t2["kinds"]), "clocks": t2["clocks"]}
    del flush
    out["quality"], refs = quality(data, method, local, stream)
    out["learned_cache"] = learned_bench(data, refs, local)
    out["hashgrid"] = hashgrid_bench(stream, peak)
    out["mlp"] = mlp_bench(stream)
    out["adjoint"] = adjoint_bench(peak)
    out["taa"] = taa_bench()
    out["camera_paths"] = paths_bench()
    for name in SCALE_CONFIGS:
        out[name] = scale_line_ours(name, args, local)
    return out, data, method, refs


def scale_line_ours(name, args, local):
    """An at-scale workload timed like the headline: the same window of frames around the first
    state change, L2 flushed between frames, CUDA events on the library's stream, clocks
    sampled.  The city line adds the 3840 x 2160 image pass from its cache."""
    import numpy as np
    import torch
    from render_engine_gb300 import methods as M
    from render_engine_gb300 import native as N
    cfg = SCALE_CONFIGS[name]
    data = scale_scene(name)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    method = M.by_name(M.timing_methods(), cfg["method"])
    s0 = window_start(args.warmup, args.steps)
    seq = sequence(s0 + args.steps)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    ctx = N.Context(device=local, stream=stream.cuda_stream, expect_lights=cfg["lamps"])
    info = ctx.load_bytes(data)
    t = time_frames(ctx, method, seq, s0, args, stream, flush)
    total = sum(t["ms"])
    out = {"scene": cfg["desc"], "triangles": info["nst"], "cache_points": info["np"], "lights": info["nl"],
           "method": cfg["method"], "frames_per_s": args.steps / (total * 1e-3), "ms_per_step": total / args.steps,
           "mrays_per_s": t["rays"] / (total * 1e-3) / 1e6, "frame_kinds_ms": kinds_table(t["ms"], t["kinds"]),
           "clocks": t["clocks"], "bvh_nodes": info["nnodes"]}
    if name == "city":
        lo = np.frombuffer(data, np.float32, count=3, offset=32)   # the scene box's lower corner
        cam = N.camera(eye=(float(lo[0]) * 0.9, float(lo[1]) * 0.9, 120.0), at=(0.0, 0.0, 0.0), fov_y_deg=60.0,
                       width=3840, height=2160)
        ctx.render(seq[-1], cam, copy=False)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(10)]
        for e0, e1 in ev:
            flush.zero_()
            e0.record(stream)
            ctx.render(seq[-1], cam, copy=False)
            e1.record(stream)
        torch.cuda.synchronize()
        out["image_3840x2160_ms"] = sum(a.elapsed_time(b) for a, b in ev) / len(ev)
    ctx.close()
    del flush
    return out


def e2e_run(data, method, seq, local, stream, world):
    """End to end through the C ABI from host memory: the scene upload from a pinned buffer and
    its load, the run's frames from frame 0 through the last timed frame, and the cache read
    back into pinned memory, all inside one host-clock interval.  Measured in a process that has
    run the library before (the device memory pool keeps the pages an earlier context mapped, as
    in a renderer that loads scene after scene); the first load of the process, which maps them,
    is reported beside it."""
    import torch
    from render_engine_gb300 import native as N
    from render_engine_gb300 import scene as S
    host = torch.frombuffer(bytearray(data), dtype=torch.uint8).pin_memory()
    hdr = S.header(data)
    lc_host = torch.empty(hdr["nl"] * hdr["np"], dtype=torch.float32).pin_memory()
    # RC_FLAG_LOAD_ASYNC: the pinned buffer stays alive until the final sync, so the states after
    # the first keep streaming in on the second stream while the first frames run
    ctx = N.Context(device=local, stream=stream.cuda_stream, flags=N.FLAG_LOAD_ASYNC)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    # the load returns once the global arrays and state 0 are on the device and checked; the other
    # states' copies and the state builds run on the context's second stream behind it, and each
    # frame waits (on the device) only for its own state's build, as a caller that does not
    # synchronise sees it
    ctx.load_bytes(host.numpy())
    t1 = time.perf_counter()
    ctx.begin(method, seq[0], 11)
    for s in seq:
        ctx.frame(s)
    lc = ctx.array(N.A_LC, out=lc_host.numpy())
    ctx.sync()
    t2 = time.perf_counter()
    ctx.close()
    nf = len(seq)
    return {"value": nf * world / (t2 - t0), "unit": "frames/s", "h2d_bytes_per_step": len(data) / nf,
            "d2h_bytes_per_step": lc.nbytes / nf, "frames": nf, "load_ms": (t1 - t0) * 1e3, "frames_ms": (t2 - t1) * 1e3,
            "includes": "scene upload from pinned host memory (RC_FLAG_LOAD_ASYNC: states 1-4 stream in behind the load) + load "
                        "(returns when state 0 and the global arrays are checked) + the state builds (second stream) + frames "
                        "0-%d + final cache download" % (nf - 1)}


def quality(data, method, local, stream):
    """The metric's error part over the reference's whole timing sequence (5 states x 60
    frames, 4 state changes), whatever the number of timed steps: the per-frame luminance error
    sqrt(sum (est - ref)^2 / n) / (sum ref / n) of the reference (poc_gpu.cu:683-696, 1005-1010)
    against converged references, averaged over the 30 frames after each change
    (poc_gpu.cu:1428-1429) and the 20 before it, over all valid points (as the reference reports
    it) and over the event region: the valid points whose reference changes by more than 5 %
    between the two states, |new - old| / (old + 0.01) > 0.05 (the two upper recon categories,
    poc_gpu.cu:1520-1526).  The scene carries no references, so they are computed first on the
    GPU by the stochastic Jacobi of the reference's scene preparation (rc_reference_build); the
    CPU leg checks them against the FP64 path tracer.  The event-region sums come from
    rc_error_sums_noalloc on the run's own cache buffer after each frame."""
    import math
    import numpy as np
    import torch
    from render_engine_gb300 import native as N
    q = N.Context(device=local, stream=stream.cuda_stream)
    info = q.load_bytes(data)
    np_, nl, ns = info["np"], info["nl"], info["ns"]
    t0 = time.perf_counter()
    noise, iters = q.build_reference()
    tref = time.perf_counter() - t0
    refs = [q.state_array(k, N.SA_REF) for k in range(ns)]
    valid = [q.state_array(k, N.SA_VALID) for k in range(ns)]
    pw = [q.state_array(k, N.SA_PW) for k in range(ns)]
    seq = sequence(ns * FRAMES_PER_STATE, ns)
    events = [f for f in range(1, len(seq)) if seq[f] != seq[f - 1]]
    dev = torch.device("cuda", local)
    region = {}
    for e in events:
        a, b = seq[e - 1], seq[e]
        rel = np.abs(refs[b] - refs[a]).astype(np.float64) / (refs[a].astype(np.float64) + 1e-2)
        mask = (valid[b] != 0) & (rel > 0.05)
        region[e] = (torch.from_numpy(mask.astype(np.uint8)).to(dev), torch.from_numpy(refs[b]).to(dev), int(mask.sum()))
    out3 = torch.zeros((len(events) * POST_FRAMES, 3), dtype=torch.float64, device=dev)
    lc_stride = (nl + 3) // 4 * 4
    q.begin(method, seq[0], 11)
    slot = 0
    for f, s in enumerate(seq):
        q.frame(s, want_err=True)
        e = max([x for x in events if x <= f], default=None)
        if e is not None and f < e + POST_FRAMES:
            m, r, _ = region[e]
            N.error_sums_noalloc(q.device_ptr(N.A_LC), lc_stride, nl, q.scalar(N.S_DORMANT), r.data_ptr(), m.data_ptr(), np_,
                                 out3[slot].data_ptr(), stream.cuda_stream)
            slot += 1
    errs = [float(x) for x in q.errors()]
    sums = out3.cpu().numpy()
    q.close()
    post = [statistics.mean(errs[e:e + POST_FRAMES]) for e in events]
    pre = [statistics.mean(errs[e - PRE_FRAMES:e]) for e in events]
    post_region = []
    for k, e in enumerate(events):
        v = []
        for j in range(POST_FRAMES):
            d2, rs, cnt = sums[k * POST_FRAMES + j]
            v.append(math.sqrt(d2 / cnt) / (rs / cnt) if cnt > 0 and rs > 0 else 0.0)
        post_region.append(statistics.mean(v))
    res = {"luma_err_post_event_pct": 100 * statistics.mean(post), "luma_err_pre_event_pct": 100 * statistics.mean(pre),
           "luma_err_post_event_region_pct": 100 * statistics.mean(post_region),
           "per_event": [{"frame": e, "from": seq[e - 1], "to": seq[e], "region_points": region[e][2],
                          "post_pct": 100 * p, "post_region_pct": 100 * pr, "pre_pct": 100 * pe}
                         for e, p, pr, pe in zip(events, post, post_region, pre)],
           "events": len(events), "frames": len(seq), "reference_noise": [float(x) for x in noise],
           "reference_iterations": [int(x) for x in iters], "reference_build_s": tref,
           "note": "references from the GPU stochastic Jacobi of the reference's scene preparation (K=32, two chains, 3 % noise "
                   "target); their gap to the FP64 path tracer is measured by the CPU leg (fp64_reference_check)"}
    return res, {"refs": refs, "valid": valid, "pw": pw}


def learned_bench(data, refs, local, batch=1 << 16):
    """The learned cache (render_engine_gb300/learned.py: the network trained online every frame on
    the tracer's one-bounce estimates, 2^16 samples per step, loss-scaled, and served as the
    cache) against the reference's cache methods over the whole timing sequence (5 states x 60
    frames, 4 state changes): the dependency-tracked `v4-A2C suivi 1/4`, the plain `Classique 1.0x`
    and the SHaRC-style hash-grid cache `SHaRC responsive 1.0x`, the cache the learned one is held against: the 30-frame post-event luminance error over all
    valid points and over the event region (as the quality leg), and each method's frame ms (CUDA
    events around each frame's work; for the learned cache inference + frame + training step).
    The per-point caches run at 1, 2, 4, 8 and 16 rays per point (the hash-grid cache at 32 too), so
    that one of them spends at least the learned cache's time per frame.  The per-point caches start from the converged cache of the
    first state, as the reference's runs do (the references' per-light warm start written into the
    scene); the network runs 120 frames of its own online training in the first state before the
    sequence (training it on that warm start first was measured worse: 46-49 % before events).
    Four training steps of 2^16 samples per frame, lr 7e-3, eight more steps in each of the 10
    frames after a state change (of 2-8 steps, lr 5e-3-2e-2, 0-16 extra steps for 5-30 frames,
    the lowest post-event error on this scene below 1 ms a frame).  frame_ms is the mean over
    frames 5.. of the sequence (event frames and the learned cache's extra steps included),
    frame_ms_median the median."""
    import math
    import numpy as np
    import torch
    from render_engine_gb300 import learned as LC
    from render_engine_gb300 import methods as M
    from render_engine_gb300 import native as N
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dev = torch.device("cuda", local)
    hdr = __import__("render_engine_gb300.scene", fromlist=["header"]).header(data)
    np_, nl, ns = hdr["np"], hdr["nl"], hdr["ns"]
    seq = sequence(ns * FRAMES_PER_STATE, ns)
    events = [f for f in range(1, len(seq)) if seq[f] != seq[f - 1]]
    ref_d = [torch.from_numpy(r).to(dev) for r in refs["refs"]]
    val_d = [torch.from_numpy(v.astype(np.uint8)).to(dev) for v in refs["valid"]]
    reg_d = {}
    for e in events:
        a, b = seq[e - 1], seq[e]
        rel = np.abs(refs["refs"][b] - refs["refs"][a]).astype(np.float64) / (refs["refs"][a].astype(np.float64) + 1e-2)
        reg_d[e] = torch.from_numpy(((refs["valid"][b] != 0) & (rel > 0.05)).astype(np.uint8)).to(dev)
    lcs = (nl + 3) // 4 * 4
    warm = 120
    from render_engine_gb300 import scene as S
    sc = S.read(data)
    for k, st in enumerate(sc.states):
        st.ref, st.valid, st.Pw = refs["refs"][k], refs["valid"][k].astype(np.uint8), refs["pw"][k].reshape(np_, nl)
    data = S.write(sc)     # the scene with its references and warm start

    def run(step, ctx, dormant_of):
        sums = torch.zeros((len(seq), 2, 3), dtype=torch.float64, device=dev)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in seq]
        for f, s in enumerate(seq):
            ev[f][0].record(stream)
            served = step(f, s)     # the cache's values for frame f are in the context's buffer
            ev[f][1].record(stream)
            e = max([x for x in events if x <= f], default=None)
            N.error_sums_noalloc(served, lcs, nl, dormant_of(), ref_d[s].data_ptr(), val_d[s].data_ptr(), np_,
                                 sums[f, 0].data_ptr(), stream.cuda_stream)
            if e is not None and f < e + POST_FRAMES:
                N.error_sums_noalloc(served, lcs, nl, dormant_of(), ref_d[s].data_ptr(), reg_d[e].data_ptr(), np_,
                                     sums[f, 1].data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        h = sums.cpu().numpy()
        ms = [a.elapsed_time(b) for a, b in ev]
        err = lambda x: math.sqrt(x[0] / x[2]) / (x[1] / x[2]) if x[2] > 0 and x[1] > 0 else 0.0
        post = statistics.mean(statistics.mean(err(h[f, 0]) for f in range(e, e + POST_FRAMES)) for e in events)
        post_r = statistics.mean(statistics.mean(err(h[f, 1]) for f in range(e, e + POST_FRAMES)) for e in events)
        pre = statistics.mean(statistics.mean(err(h[f, 0]) for f in range(e - PRE_FRAMES, e)) for e in events)
        return {"post_event_err_pct": 100 * post, "post_event_region_err_pct": 100 * post_r, "pre_event_err_pct": 100 * pre,
                "frame_ms": statistics.mean(ms[5:]), "frame_ms_median": statistics.median(ms[5:])}

    out = {}
    ctx = N.Context(device=local, stream=stream.cuda_stream)
    ctx.load_bytes(data)
    steps_per_frame, event_steps, event_frames, lr = 4, 8, 10, 7e-3
    lc = LC.LearnedCache(ctx, data, stream.cuda_stream, batch=batch, lr=lr, seed=1, steps_per_frame=steps_per_frame,
                         event_steps=event_steps, event_frames=event_frames)
    ctx.build_states()
    ctx.sync()
    lc.begin(seq[0], 11)
    for _ in range(warm):
        lc.frame(seq[0])
    pending = {}

    def learned_step(f, s):
        if f > 0:
            lc.frame(pending["s"], predicted=True)   # finish the previous frame: trace, gather, train
        lc.predict(s)
        pending["s"] = s
        return ctx.device_ptr(N.A_LC)

    r = run(learned_step, ctx, lambda: 0)
    scale, steps, skipped = lc.mlp.loss_scale()
    lc.close()
    ctx.close()
    r.update({"loss_scale": scale, "train_steps": steps, "skipped_steps": skipped, "batch": batch, "steps_per_frame": steps_per_frame,
              "event_steps": event_steps, "event_frames": event_frames, "lr": lr, "warm_frames": warm,
              "note": "frame_ms = training step of the previous frame + inference of this one (the served values) + the rest "
                      "of the frame loop"})
    out["learned"] = r
    for name in ("v4-A2C suivi 1/4", "Classique 1.0x", "SHaRC responsive 1.0x"):
        for rays in (1.0, 2.0, 4.0, 8.0, 16.0) + ((32.0,) if name.startswith("SHaRC") else ()):
            m = M.by_name(M.timing_methods(), name).replace(rays=rays)
            c = N.Context(device=local, stream=stream.cuda_stream)
            c.load_bytes(data)
            c.build_states()
            c.sync()
            c.begin(m, seq[0], 11)

            def cache_step(f, s, c=c):
                c.frame(s)
                return c.device_ptr(N.A_LC)

            out["%s x%g" % (name, rays)] = run(cache_step, c, lambda c=c: c.scalar(N.S_DORMANT))
            c.close()
    best = None
    for k, v in out.items():
        if k != "learned" and v["frame_ms"] >= out["learned"]["frame_ms"]:
            if best is None or v["post_event_err_pct"] < out[best]["post_event_err_pct"]:
                best = k
    out["per_point_cache_at_equal_or_more_ms"] = best
    # the comparison the learned cache is held to: the SHaRC-style hash-grid cache (bench B's "SHaRC
    # responsive": spatial-hash cache points, running mean reset where a light's contribution
    # changes) at the cheapest ray budget whose frame costs at least the learned cache's
    sharc = sorted((v["frame_ms"], k) for k, v in out.items() if k.startswith("SHaRC") and isinstance(v, dict))
    ref_k = next((k for ms, k in sharc if ms >= out["learned"]["frame_ms"]), sharc[-1][1] if sharc else None)
    if ref_k is not None:
        out["vs_hash_grid"] = {"method": ref_k, "frame_ms": out[ref_k]["frame_ms"],
                                  "post_event_err_pct": out[ref_k]["post_event_err_pct"],
                                  "hash_grid_frame_ms_ge_learned": bool(out[ref_k]["frame_ms"] >= out["learned"]["frame_ms"]),
                                  "learned_post_event_le_hash_grid": bool(out["learned"]["post_event_err_pct"] <= out[ref_k]["post_event_err_pct"])}
    return out


def hashgrid_bench(stream, peak, capacity=1 << 24, live=1 << 23, npaths=1 << 20, reps=10):
    """Secondary lines: the hash-grid cache with dependency masks (include/rc_hashgrid.h).

    resolve: one pass over a 2^24-entry table with about 2^23 live entries that all received
    samples this frame (each pass preceded, untimed, by the accumulation that refills them); it
    reads every slot's key (8 B) and, for a live entry only, its accumulation 16 B, resolved 16 B
    and two mask banks 32 B, and writes its accumulation and resolved words (32 B): the HBM
    roofline over those necessary bytes.
    mark: dependency marking of 2^20 random paths of 1-5 bounces in the zone box."""
    import numpy as np
    import torch
    from render_engine_gb300 import hashgrid as H

    cfg = H.make_config(capacity=capacity, cell=0.02, max_depth=4, acc_frames=64, stale_frames=1000,
                        tracing_distance=50.0, stream=stream.cuda_stream)
    hg = H.HashGrid(cfg)
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    pos = torch.rand(live, 3, device="cuda", generator=g) * torch.tensor([8.0, 4.0, 3.0], device="cuda")
    nrm = torch.randn(live, 3, device="cuda", generator=g)
    rgb = torch.rand(live, 3, device="cuda", generator=g)
    entry = torch.empty(live, dtype=torch.int32, device="cuda")
    hg.insert(pos, nrm, entry)
    hg.accumulate(entry, rgb)
    hg.resolve()
    keys = np.frombuffer(hg.download(H.A_KEYS).tobytes(), np.uint64)
    nlive = int(((keys != 0) & (keys != H.EVICTED)).sum())
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in evs:
        hg.accumulate(entry, rgb)
        e0.record(stream)
        hg.resolve()
        e1.record(stream)
    torch.cuda.synchronize()
    res_ms = sum(a.elapsed_time(b) for a, b in evs) / reps
    # necessary bytes: every slot's key; the accumulation, resolved radiance and two mask banks
    # (64 B) of each live entry; its accumulation and resolved words written (32 B)
    res_bytes = 8.0 * capacity + 64.0 * nlive + 32.0 * nlive
    # path batch
    rng = np.random.default_rng(8)
    lens = rng.integers(1, 6, npaths)
    start = np.zeros(npaths + 1, np.int32)
    start[1:] = np.cumsum(lens)
    n = int(start[-1])
    v = np.zeros(n, H.VERTEX_DTYPE)
    v["origin"] = rng.uniform([0, 0, 0], [8, 4, 3], (n, 3))
    v["hit"] = rng.uniform([0, 0, 0], [8, 4, 3], (n, 3))
    d = rng.normal(size=(n, 3))
    v["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    t = rng.normal(size=(n, 3))
    v["to_light"] = t / np.linalg.norm(t, axis=1, keepdims=True)
    v["light_dist"] = rng.uniform(0.5, 10.0, n)
    v["light_index"] = rng.integers(-1, 8, n)
    v["entry"] = entry.cpu().numpy().view(np.uint32)[rng.integers(0, live, n)]
    v["flags"] = np.where(rng.random(n) < 0.5, H.LIGHT_VISIBLE, 0) | np.where(rng.random(n) < 0.1, H.MISS, 0)
    dv = torch.from_numpy(v.view(np.uint8)).cuda()
    ds = torch.from_numpy(start).cuda()
    hg.mark_paths(dv, ds, npaths)
    evm = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
    for e0, e1 in evm:
        e0.record(stream)
        hg.mark_paths(dv, ds, npaths)
        e1.record(stream)
    torch.cuda.synchronize()
    mark_ms = sum(a.elapsed_time(b) for a, b in evm) / len(evm)
    hg.close()
    achieved = res_bytes / (res_ms * 1e-3) / 1e9
    return {"resolve": {"entries": capacity, "live_entries": nlive, "ms": res_ms, "entries_per_s": capacity / (res_ms * 1e-3),
                        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                                     "algorithmic_bytes": res_bytes}},
            "mark_paths": {"paths": npaths, "vertices": n, "ms": mark_ms, "vertices_per_s": n / (mark_ms * 1e-3)}}


def paths_bench(reps=10, points=1_082_802, warm=3, width=1920, height=1080):
    """Secondary line: the 1080p camera-path pass feeding the hash-grid cache (rc_hg_camera_paths):
    1920 x 1080 paths with 2 bounces through the 1.08 M-point room, the room's 3 point lights
    plus a 1 x 1 m rectangle light and a sun, one light sample and shadow ray per vertex; 2^22
    entries, dependency marking and 128^3 per-voxel light masks.  CUDA events on the cache's
    stream around each pass (trace, insert, accumulate, mark, voxels)."""
    import torch
    from render_engine_gb300 import hashgrid as H
    from render_engine_gb300 import native as N
    from render_engine_gb300 import scene as S
    st = torch.cuda.Stream()
    ctx = N.Context(stream=st.cuda_stream)
    ctx.load_bytes(S.write(S.box_room(points=points, seed=0)))
    cfg = H.make_config(zone_lo=(0, 0, 0), zone_hi=(8, 4, 3), cell=0.05, capacity=1 << 22, max_depth=4, tracing_distance=50.0,
                        stream=st.cuda_stream)
    hg = H.HashGrid(cfg)
    hg.voxels_init(128)
    cam = N.camera((0.5, 0.5, 1.6), (6.0, 3.0, 1.0), width=width, height=height, fov_y_deg=75.0)
    area = ((3.5, 1.5, 2.95), (1.0, 0.0, 0.0), (0.0, -1.0, 0.0), (4.0, 3.5, 3.0))
    sun = ((0.3, 0.2, 1.0), (0.5, 0.5, 0.45))
    img = torch.zeros(width * height * 3, device="cuda")
    for f in range(warm):
        hg.begin_frame(f, 16)
        hg.camera_paths(ctx, 0, H.path_params(cam, bounces=2, seed=1, frame=f, area=area, sun=sun), img)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for k in range(reps):
        hg.begin_frame(3 + k, 16)
        ev[k][0].record(st)
        hg.camera_paths(ctx, 0, H.path_params(cam, bounces=2, seed=1, frame=3 + k, area=area, sun=sun), img)
        ev[k][1].record(st)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / reps
    a = H.camera_arrays(ctx)
    verts = a["vertices"]
    used = int(a["len"].sum())
    hg.close()
    ctx.close()
    rays = used + int(((verts["light_index"] >= 0)).sum())   # path rays + shadow rays of the last pass
    return {"width": width, "height": height, "bounces": 2, "ms": ms, "paths_per_s": width * height / (ms * 1e-3),
            "rays_per_pass": rays, "mrays_per_s": rays / (ms * 1e-3) / 1e6, "voxel_res": 128, "capacity": 1 << 22}


def taa_scene(points: int) -> bytes:
    """The room with stand-in references (1.0 everywhere, all points valid) so that the taa mode
    runs: its cost does not depend on the reference values."""
    import numpy as np
    from render_engine_gb300 import scene as S
    sc = S.box_room(points=points, seed=0)
    n = len(sc.A)
    for st in sc.states:
        st.ref = np.ones(n, np.float32)
        st.valid = np.ones(n, np.uint8)
        st.Pw = np.zeros((n, len(sc.L)), np.float32)
    return S.write(sc)


def taa_state(f: int) -> int:
    return (f // 50) % 5


def taa_bench(frames=200, warm=10, points=1_082_802):
    """Secondary line: the taa mode (rc_taa_frame, dependency mask, alpha 0.1, clamp 1) on the
    1.08 M-point room, each frame with its error read back as the reference's run_taa_mode does;
    wall-clock frames/s over 200 frames with 4 events."""
    from render_engine_gb300 import native as N
    ctx = N.Context()
    ctx.load_bytes(taa_scene(points))
    ctx.taa_begin(0.1, 1.0, 2, 0, 5000)
    for f in range(warm):
        ctx.taa_frame(0, want_err=True)
    t0 = time.perf_counter()
    for f in range(frames):
        ctx.taa_frame(taa_state(f), want_err=True)
    dt = time.perf_counter() - t0
    ctx.close()
    return {"points": points, "frames": frames, "frames_per_s": frames / dt, "ms_per_frame": dt * 1e3 / frames,
            "method": "TAA + masque dependances"}


def adjoint_bench(peak, points=1_082_802, lights=16, K=16):
    """Secondary line: dJ/dE for all 16 lights of a 1.08 M-point room (rc_adjoint): K frozen rays
    per point, the transposed ray lists, 64 forward + 64 adjoint Jacobi sweeps, the FP64
    gradient.  The unit-emission direct light of the state is built by the first call and kept
    by the context (it depends on neither the weights nor the seed): `first_call_ms` includes
    it and the buffer allocation, `ms` is a later call.  A sweep pair's time is
    (t(64) - t(16)) / 48 from two calls; its algorithmic HBM
    bytes: the hit list and the transposed source list (4 B per ray each), offsets, weights and
    the two iterates (about 24 B per point); the gathers of the iterates stay in L2 (4 MB)."""
    import numpy as np
    from render_engine_gb300 import native as N
    from render_engine_gb300 import scene as S
    ctx = N.Context()
    info = ctx.load_bytes(S.write(S.box_room(points=points, seed=0, lights=lights)))
    rng = np.random.default_rng(1)
    w = np.zeros(info["np"], np.float32)
    w[rng.choice(info["np"], 4096, replace=False)] = 1.0 / 4096
    t0 = time.perf_counter()
    ctx.adjoint(0, w, K=K, seed=5, iterations=64)   # first call: allocation, unit-emission build
    first_ms = (time.perf_counter() - t0) * 1e3
    t = {}
    for it in (16, 64):
        t0 = time.perf_counter()
        g, res = ctx.adjoint(0, w, K=K, seed=5, iterations=it)
        t[it] = (time.perf_counter() - t0) * 1e3
    ctx.close()
    pair_ms = (t[64] - t[16]) / 48
    counted = res["rays"] - res["back"]
    pair_bytes = 4.0 * res["rays"] + 4.0 * counted + 24.0 * info["np"]
    gbs = pair_bytes / (pair_ms * 1e-3) / 1e9 if pair_ms > 0 else None
    return {"points": info["np"], "lights": lights, "rays_per_point": K, "iterations": 64, "ms": t[64], "first_call_ms": first_ms,
            "sweep_pair_ms": pair_ms, "J_rel_linearity_gap": abs(res["J_grad"] - res["J"]) / abs(res["J"]),
            "fwd_change": res["fwd_change"], "adj_change": res["adj_change"],
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak if gbs else None,
                         "bytes_per_sweep_pair": pair_bytes}}


def mlp_bench(stream, npoints=1_082_802, batch=1 << 16, reps=10):
    """Secondary lines: the learned radiance cache on the tensor cores (include/rc_mlp.h).

    infer: the network's 3 outputs for 1,082,802 points (one per cache point of the room);
    train: one Adam step on 2^16 samples (forward, backward, gradient sum, update).
    Algorithmic FLOPs per query: 2 x (168 x 64 + 3 x 64 x 64 + 64 x 3) = 46,464 (forward),
    3x that per training sample, against the measured bf16 tensor peak (burst)."""
    import torch
    from render_engine_gb300 import mlp as MLP

    if stream.cuda_stream == 0:   # a null handle would make the library use a stream of its own
        stream = torch.cuda.Stream()
    g = torch.Generator(device="cuda")
    g.manual_seed(11)
    P = (torch.rand(npoints, 4, device="cuda", generator=g) * torch.tensor([8.0, 4.0, 3.0, 0.0], device="cuda")).contiguous()
    N = torch.randn(npoints, 4, device="cuda", generator=g)
    N[:, :3] /= N[:, :3].norm(dim=1, keepdim=True)
    N = N.contiguous()
    aux = torch.rand(npoints, 4, device="cuda", generator=g).contiguous()
    target = torch.rand(npoints, 3, device="cuda", generator=g).contiguous()
    out = torch.empty(npoints, 3, device="cuda")
    net = MLP.Mlp(n_out=3, lr=1e-2, max_batch=batch, stream=stream.cuda_stream)
    idx = torch.randint(0, npoints, (batch,), device="cuda", generator=g, dtype=torch.int32)
    net.infer(P, N, aux, out)
    net.train(P, N, aux, target, idx=idx)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(2 * reps)]
    for k in range(reps):
        ev[k][0].record(stream)
        net.infer(P, N, aux, out)
        ev[k][1].record(stream)
    for k in range(reps):
        ev[reps + k][0].record(stream)
        net.train(P, N, aux, target, idx=idx)
        ev[reps + k][1].record(stream)
    torch.cuda.synchronize()
    inf_ms = sum(a.elapsed_time(b) for a, b in ev[:reps]) / reps
    tr_ms = sum(a.elapsed_time(b) for a, b in ev[reps:]) / reps
    flops = 2.0 * (168 * 64 + 3 * 64 * 64 + 64 * 3)
    flags = net.error_flags()
    net.close()
    peak = tensor_peak()
    inf_tf = npoints * flops / (inf_ms * 1e-3) / 1e12
    tr_tf = batch * 3 * flops / (tr_ms * 1e-3) / 1e12
    return {"infer": {"queries": npoints, "ms": inf_ms, "queries_per_s": npoints / (inf_ms * 1e-3),
                      "roofline": {"bound": "tensor", "achieved": inf_tf, "peak": peak, "unit": "TFLOP/s", "frac": inf_tf / peak}},
            "train_step": {"samples": batch, "ms": tr_ms, "samples_per_s": batch / (tr_ms * 1e-3),
                           "roofline": {"bound": "tensor", "achieved": tr_tf, "peak": peak, "unit": "TFLOP/s", "frac": tr_tf / peak}},
            "error_flags": flags}


def tensor_peak() -> float:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["bf16_tflops"])
    return 1900.0


def cpu_model() -> str:
    """The host CPU's model name (lscpu), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "unknown"


def cpu_baseline(args, data, method, refs):
    """The CPU leg: the oracle (plain-C restatement, OpenMP on all host cores) timed on the first
    frames of the same workload, and the checker of the GPU references the quality leg used:
    the oracle's FP64 path tracer at 128 sampled valid points per state (16,384 paths each)
    against the GPU's stochastic-Jacobi values there."""
    import numpy as np
    from oracle import pyoracle as po
    cores = os.cpu_count() or 1
    po.set_threads(cores)
    sc = po.Scene(data=data)
    sc.build()
    run = po.Run(sc)
    seq = sequence(args.cpu_frames)
    run.begin(method, seq[0], 11)
    t = time.perf_counter()
    for s in seq:
        run.frame(s)
    dt = time.perf_counter() - t
    out = {"value": args.cpu_frames / dt, "unit": "frames/s", "cores": cores, "cpu_model": cpu_model(), "kind": "port",
           "sample": "frames 0-%d of the same sequence at full size (%d points), C restatement with OpenMP" % (args.cpu_frames - 1, sc.Np)}
    if refs is not None:
        rng = np.random.default_rng(31)
        t = time.perf_counter()
        gaps, z2, worst = [], [], []
        for si, (ref, val) in enumerate(zip(refs["refs"], refs["valid"])):
            ok = np.flatnonzero((val != 0) & (ref > 0))
            pts = ok[rng.choice(len(ok), min(128, len(ok)), replace=False)]
            m, se = sc.path_trace(si, pts, paths=16384, min_bounces=3, seed=50 + si)
            r = ref[pts].astype(np.float64)
            gaps.append(float((r - m).mean() / m.mean()))
            z = (r - m) / np.sqrt(se ** 2 + (0.03 * r) ** 2 + (0.01 * float(ref[ok].mean())) ** 2)
            z2.append(float((z ** 2).mean()))
            w = int(np.argmax(np.abs(z)))
            worst.append({"point": int(pts[w]), "gpu": float(r[w]), "fp64": float(m[w]), "fp64_se": float(se[w]), "z": float(z[w])})
        out["fp64_reference_check"] = {
            "points_per_state": 128, "paths_per_point": 16384, "seconds": time.perf_counter() - t,
            "mean_rel_gap_per_state": gaps, "mean_abs_rel_gap_pct": 100 * float(np.mean(np.abs(gaps))),
            "z2_per_state": z2, "worst_per_state": worst,
            "note": "GPU FP32 stochastic-Jacobi references minus the FP64 path tracer, relative to the latter's mean; z2 = "
                    "mean squared difference over the path tracer's standard error, the references' 3 % noise target and 1 % of the "
                    "mean reference"}
    return out


def run_reference(args, world, rank, local, dist):
    import torch

    from oracle import pyref
    from render_engine_gb300 import methods as M

    if not pyref.available(3):
        return None, "reference kernels not built (oracle/_ref/ref_l3.cubin missing: needs the reference checkout at build time)"
    torch.cuda.set_device(local)
    torch.cuda.init()
    data, scene_desc = headline_scene(args.points)
    method = M.by_name(M.timing_methods(), args.method)
    ref = pyref.RefRunner(3, data)
    s0 = window_start(args.warmup, args.steps)
    seq = sequence(s0 + args.steps)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    ref.begin(method, seq[0], 11)
    for f in range(s0):
        ref.frame(seq[f])
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = Clocks(local)
    for k in range(args.steps):
        flush.zero_()
        starts[k].record(stream)
        ref.frame(seq[s0 + k])
        ends[k].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    kinds = ["event" if seq[s0 + k] != seq[s0 + k - 1] else "other" for k in range(args.steps)]
    total_ms = sum(ms)
    # the reference's own timing-mode figures (per-frame events, one sync per frame)
    import numpy as np
    tm = np.zeros(5)
    ref.begin(method, seq[0], 12)
    nf = min(args.steps, 5 * FRAMES_PER_STATE)
    for f in range(nf):
        ref.frame(seq[f], timers=tm)
    ref.close()
    # the taa mode with the reference's own kernels, as taa_bench times the product's
    rt = pyref.RefRunner(3, taa_scene(args.points))
    rt.taa_begin(0.1, 1.0, 2, 0, 5000)
    for f in range(10):
        rt.taa_frame(0)
    t0 = time.perf_counter()
    for f in range(200):
        rt.taa_frame(taa_state(f))
    dt = time.perf_counter() - t0
    rt.close()
    return {"frames_per_s": args.steps / (total_ms * 1e-3), "ms_per_step": total_ms / args.steps, "clocks": clk,
            "scene": scene_desc, "frame_kinds_ms": kinds_table(ms, kinds),
            "window": {"first_timed_frame": s0, "untimed_lead_in_frames": s0 - args.warmup},
            "timing_mode": {"trace": tm[1] / nf, "decide": tm[2] / nf, "update": tm[3] / nf, "swap": tm[0] / nf,
                            "event_total": tm[4]},
            "street": scale_line_reference("street", args),
            "city": scale_line_reference("city", args),
            "taa": {"points": args.points, "frames": 200, "frames_per_s": 200 / dt, "ms_per_frame": dt * 1e3 / 200,
                    "method": "TAA + masque dependances"}}, None


def scale_line_reference(name, args):
    """The reference's own kernels on an at-scale workload, timed as scale_line_ours times ours."""
    import torch
    from oracle import pyref
    from render_engine_gb300 import methods as M
    cfg = SCALE_CONFIGS[name]
    if not pyref.available(cfg["lamps"]):
        return {"unavailable": "reference kernels for %d lights not built" % cfg["lamps"]}
    data = scale_scene(name)
    method = M.by_name(M.timing_methods(), cfg["method"])
    ref = pyref.RefRunner(cfg["lamps"], data)
    s0 = window_start(args.warmup, args.steps)
    seq = sequence(s0 + args.steps)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    ref.begin(method, seq[0], 11)
    for f in range(s0):
        ref.frame(seq[f])
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = Clocks(torch.cuda.current_device())
    for k, (e0, e1) in enumerate(ev):
        flush.zero_()
        e0.record(stream)
        ref.frame(seq[s0 + k])
        e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ref.close()
    ms = [a.elapsed_time(b) for a, b in ev]
    kinds = ["event" if seq[s0 + k] != seq[s0 + k - 1] else "other" for k in range(args.steps)]
    return {"scene": cfg["desc"], "method": cfg["method"], "frames_per_s": args.steps / (sum(ms) * 1e-3),
            "ms_per_step": sum(ms) / args.steps, "frame_kinds_ms": kinds_table(ms, kinds), "clocks": clk}


def main():
    args = parse()
    if args.profile:
        profile_run(args)
        return
    world, rank, local, dist = setup_dist(args)
    s0 = window_start(args.warmup, args.steps)
    config = {"workload": "dependency-tracked radiance cache, %s, the reference's scene_scale_1M timing case (%d cache points, "
                          "3 point lights, 5 states x %d frames with events), one frame per step" % (args.method, args.points, FRAMES_PER_STATE),
              "method": args.method, "cache_points": args.points, "transit_grid": "8x4x4 (128-bit dependency masks)",
              "l2": "flushed between timed frames (512 MB write); per-frame working set ~140 MB",
              "window": "timed frames %d-%d of the state sequence (state changes every %d frames); frames before the warm-up run untimed"
                        % (s0, s0 + args.steps - 1, FRAMES_PER_STATE),
              "parallelism": "replicas" if world > 1 else "single GPU"}
    if args.impl == "reference":
        if rank != 0:
            return
        res, why = run_reference(args, 1, 0, local, None)
        if res is None:
            print(json.dumps({"impl": "reference", "unavailable": why}))
            return
        config["scene"] = res["scene"]
        line = {"metric": METRIC, "value": res["frames_per_s"], "unit": "frames/s", "n_gpus": 1, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": res["frames_per_s"] / PUBLISHED_FPS, "dtype": "f32", "data": "the reference's own scene file",
                "config": config, "impl": "reference", "clocks": res["clocks"], "frame_kinds_ms": res["frame_kinds_ms"],
                "window": res["window"], "reference_timing_mode_ms": res["timing_mode"], "taa": res["taa"],
                "street": res["street"], "city": res["city"],
                "cpu_baseline": {"value": res["frames_per_s"], "unit": "frames/s", "cores": 1, "kind": "reference",
                                 "sample": "the reference's own kernels (cuda/poc_gpu.cu for sm_103a) on the GB300, driven by one host thread; "
                                           "the reference has no CPU implementation of this path"},
                "e2e": {"value": res["frames_per_s"], "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line, default=_json_default))
        return
    res, data, method, refs = run_ours(args, world, rank, local, dist)
    if rank != 0:
        return
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args, data, method, refs)
        if "fp64_reference_check" in cpu:
            res["quality"]["reference_vs_fp64_gap_pct"] = cpu["fp64_reference_check"]["mean_abs_rel_gap_pct"]
    config["scene"] = res["scene"]
    line = {"metric": METRIC, "value": res["frames_per_s"], "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": res["frames_per_s"] / PUBLISHED_FPS, "dtype": "f32", "data": "the reference's own scene file",
            "config": config, "window": res["window"],
            "mrays_per_s": res["mrays_per_s"], "cache_updates_per_s": res["cache_updates_per_s"],
            "rays_per_frame": res["rays_per_frame"], "frame_kinds_ms": res["frame_kinds_ms"], "frame_1080p": res["frame_1080p"],
            "clocks": res["clocks"], "e2e": res["e2e"], "gpu_launches": res["launches"], "roofline": res["roofline"],
            "cpu_baseline": cpu, "quality": res["quality"], "standin_room": res.get("standin_room"), "hashgrid": res["hashgrid"],
            "mlp": res["mlp"], "adjoint": res["adjoint"], "taa": res["taa"], "camera_paths": res["camera_paths"],
            "street": res["street"], "city": res["city"], "learned_cache": res["learned_cache"]}
    print(json.dumps(line, default=_json_default))


if __name__ == "__main__":
    main()
