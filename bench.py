"""Benchmark: INSTA deformation + render hot path on GB300.

Workload (one step = one frame): the 512x512 single-frame render of a tracked
FLAME-topology-scale mesh -- device LBVH rebuild of the frame, occupancy bitfield
from the mesh (cells within 1.5 cm), ray march with exponential stepping, per-sample
canonical map, 16-level hash encode, density + colour MLPs (tcgen05), compositing.
Metric: network samples per second (deform + encode + MLP), whole job.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

For N > 1 (launched by torchrun) every rank renders its own frames (replicas, no
data-path collective); value = all ranks' samples / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "samples/s (deform+encode+MLP)"
UNIT = "samples/s"
WIDTH = HEIGHT = 512   # --width overrides (small cases for profiling)
RADIUS = 0.015
CONE = 1.0 / 256.0
L2_FLUSH_BYTES = 512 << 20
SETTLE_S = 0.5   # untimed steps before the warm-up, long enough for the SM clock to ramp
# DRAM bytes (read + write) of the deform+encode stage per 512x512 frame (nearest_stage_kernel and
# map_encode_kernel, two rounds each), from an ncu capture of this workload's kernels
TRAFFIC_PER_FRAME = 431_540_000
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12
FIELD = "benchmark"   # --field: the benchmark's 16 x 2 field, or INSTA's shipped 16 x 8 one


def field_config():
    from insta_gb300 import synthetic as S
    return S.FieldConfig() if FIELD == "benchmark" else S.insta_field_config()


def hash_bytes_per_sample(fc) -> int:
    """Hash-grid gathers: levels x 8 corners x features x 2 B (FP16)."""
    return fc.n_levels * 8 * fc.n_features * 2


def deform_encode_bytes_per_sample(fc) -> int:
    """Algorithmic bytes per sample of the dominant stage (deform + encode): the hash gathers +
    sample record, ray direction and ray index in + the encoded operand row (hash features,
    expression dims, 16 SH, FP16) and (dt, depth) out.  652 B for the benchmark field."""
    return hash_bytes_per_sample(fc) + 16 + 16 + 4 + (fc.n_levels * fc.n_features + fc.n_extra + 16) * 2 + 8


def mlp_flop_per_sample(fc) -> int:
    """Unpadded MLP FLOP per sample: 18,816 for the benchmark field (32-64-16 / 32-64-64-3)."""
    n_in = fc.n_levels * fc.n_features + fc.n_extra
    macs = n_in * 64 + 64 * 64 * (fc.density_layers - 1) + 64 * 16 + 32 * 64 + 64 * 64 * (fc.rgb_layers - 1) + 64 * 3
    return 2 * macs


def field_label(fc) -> str:
    if FIELD == "benchmark":
        return "16-level hash grid T=2^19, MLPs 32-64-16 / 32-64-64-3"
    n_in = fc.n_levels * fc.n_features + fc.n_extra
    return (f"INSTA's shipped field: {fc.n_levels}-level hash grid x {fc.n_features} features T=2^{fc.log2_table} + "
            f"{fc.n_extra} expression dims, MLPs {n_in}-64x{fc.density_layers}-16 / 32-64x{fc.rgb_layers}-3")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(rank: int):
    from insta_gb300 import synthetic as S
    av = S.make_avatar(0)
    fc = field_config()
    params = S.field_params(fc, seed=0)
    frames = [av.frame(av.frame_coeffs(1000 * rank + k)) for k in range(4)]
    cams = [S.camera(yaw, width=WIDTH, height=HEIGHT) for yaw in (0.0, -8.0, 8.0, 15.0)]
    return av, fc, params, frames, cams


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append((time.perf_counter(), parts))

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self, t0=None, t1=None):
        """Samples taken in [t0, t1] (perf_counter): the loaded window."""
        rows = [r for t, r in self.rows if (t0 is None or t >= t0) and (t1 is None or t <= t1)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_render_rate(av, fc, params, frame, cam_focal, rows: int, threads: int | None = None):
    """The CPU restatement of the path timed on the host cores for `rows` image rows."""
    from oracle import oracle as O
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    cam, focal = cam_focal
    can = O.build_triangles(av.canonical, None, av.faces, av.mask)
    t0 = time.perf_counter()
    dtr = O.build_triangles(frame, av.canonical, av.faces, av.mask)
    adj = O.adjacency(av.faces, av.n_verts)
    bvh = O.Bvh(dtr)
    bits = O.occupancy(dtr, RADIUS)
    setup = time.perf_counter() - t0
    d = O.Deformation(dtr, can, adj, bvh)
    rc = O.render_cfg(WIDTH, HEIGHT, focal, cam, av.render_aabb(), cone_angle=CONE)
    r0 = (HEIGHT - rows) // 2
    t0 = time.perf_counter()
    _, _, _, total = O.render(rc, d, bits, fc, params, rows=(r0, r0 + rows))
    dt = time.perf_counter() - t0
    return total, dt, setup, O.num_threads()


def run_reference(args, rank, world):
    """The reference arm: the path's CPU restatement on the host cores (the reference's own
    CUDA path cannot be built: its tiny-cuda-nn and Eigen submodules are empty)."""
    if rank != 0:
        return
    av, fc, params, frames, cams = workload(0)
    rows = 32
    for _ in range(args.warmup):
        cpu_render_rate(av, fc, params, frames[0], cams[0], 8)
    tot_s, tot_t = 0, 0.0
    threads = 1
    for k in range(args.steps):
        s, t, _, threads = cpu_render_rate(av, fc, params, frames[k % len(frames)], cams[k % len(cams)], rows)
        tot_s += s
        tot_t += t
    value = tot_s / tot_t
    sample = f"{rows} central rows of the {WIDTH}x{HEIGHT} frame per step (encode+MLP+deform+march+composite), OpenMP"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * tot_t / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 geometry / fp16 mlp", "data": "synthetic", "impl": "reference",
            "config": {"workload": f"render {WIDTH}x{HEIGHT}, 1 avatar, 10240-triangle tracked mesh, {field_label(fc)}",
                       "global_batch": 1, "parallelism": "cpu"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def combine_ranks(dist, dev_t, e2e_t, samples, e2e_samples, device):
    """Replicas: the job's time is the slowest rank's (max), its work the sum over ranks."""
    import torch
    t = torch.tensor([dev_t, e2e_t, float(samples), float(e2e_samples)], dtype=torch.float64, device=device)
    times, work = t[:2].clone(), t[2:].clone()
    dist.all_reduce(times, op=dist.ReduceOp.MAX)
    dist.all_reduce(work, op=dist.ReduceOp.SUM)
    return float(times[0]), float(times[1]), float(work[0]), float(work[1])


def run_ours(args, rank, world, local):
    import torch
    from insta_gb300 import abi

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    av, fc, params, frames, cams = workload(rank)
    stream = torch.cuda.Stream()
    ctx = abi.Context(local, stream=stream.cuda_stream)
    ctx.canonical_set(0, av.canonical, av.faces, av.mask)
    ctx.params_load(0, fc, params)
    apply_tuning(ctx, args)
    frames_dev = [torch.from_numpy(f).cuda() for f in frames]
    rgba = torch.empty((HEIGHT * WIDTH, 4), dtype=torch.float32, device="cuda")
    depth = torch.empty(HEIGHT * WIDTH, dtype=torch.float32, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    reqs = [ctx.render_desc(0, 0, WIDTH, HEIGHT, c[1], c[0], cone_angle=CONE) for c in cams]

    # Double-buffered frames: step k renders frame slot k % 2 (uploaded during step k - 1) and
    # uploads the next frame (LBVH rebuild + occupancy) into the other slot on the library's side
    # stream, where it overlaps this render.  Every step still does one upload and one render.
    counter = {"k": 0}

    def upload_next(k, src):
        ctx.frame_upload_async(0, (k + 1) % 2, src[(k + 1) % len(src)], RADIUS)

    def step(_k, src=None):
        k = counter["k"]
        counter["k"] += 1
        src = src if src is not None else frames_dev
        if k == 0:   # prime the first slot
            ctx.frame_upload_async(0, 0, src[0], RADIUS)
        upload_next(k, src)
        req = reqs[k % len(reqs)]
        req.frame = k % 2
        ctx.render(req, rgba, depth)
        # the step ends when both its render and the next frame's upload are done, so the timed
        # interval holds the work of both streams
        ctx.frame_wait(0, (k + 1) % 2)
        return k

    tuning_note = None
    if args.autotune:   # untimed: the library's autotuner picks the launch shapes on this frame
        ctx.frame_upload(0, 0, frames[0])
        ctx.occupancy_from_mesh(0, 0, RADIUS)
        tuned, tuned_ms = ctx.autotune([reqs[0]], repeats=3)
        tuning_note = {"autotuned": tuned, "ms_per_frame_at_tuning": tuned_ms}
    if args.stage_timing:   # every render with per-stage events: host-driven rounds (for kernel-level profiles)
        ctx.stats_enable(True)
    clocks = ClockSampler(local).__enter__()
    with torch.cuda.stream(stream):
        # settle: untimed steps for SETTLE_S so the SM clock has left its idle state before the
        # W warm-up steps and the timed ones (the clock samples below cover this window too)
        t_load0 = time.perf_counter()
        while time.perf_counter() - t_load0 < SETTLE_S:
            step(0)
            ctx.sync()
        for k in range(args.warmup):
            step(k)
        ctx.sync()
        samples_per_frame = [0] * len(reqs)
        for k in range(len(reqs)):
            kk = step(k)
            samples_per_frame[kk % len(reqs)] = ctx.render_samples()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        total_samples = 0
        # the timed steps run the library's default path: the render's rounds as one CUDA-graph
        # launch each; the launch count covers the kernels those graphs ran
        ctx.stats(reset=True)
        t_wall0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            kk = step(k)
            ev[k][1].record(stream)
            total_samples += samples_per_frame[kk % len(reqs)]
        stream.synchronize()
        t_wall = time.perf_counter() - t_wall0
        clocks.__exit__()
        clock_summary = clocks.summary(t_load0, t_wall0 + t_wall + 0.25)
        step_ms = [a.elapsed_time(b) for a, b in ev]
        launches = ctx.stats(reset=True)["kernel_launches"]
        # per-stage device time (untimed pass, same frames and kernels): with stage timing on the
        # library records CUDA events around each stage and drives the rounds from the host
        ctx.stats_enable(True)
        ctx.stats(reset=True)
        for k in range(args.steps):
            flush.zero_()
            step(k)
        stream.synchronize()
        stages = ctx.stats(reset=True)
        ctx.stats_enable(False)
        ctx.sync()
        # end to end through the C ABI with host buffers: H2D of the frame's vertices, D2H of RGBA +
        # depth.  insta_render_async copies each frame back on the library's copy stream into one
        # of two page-locked host buffer pairs while the next frame renders; the clock stops after
        # the last copy has landed.
        host_out = [(torch.empty((HEIGHT * WIDTH, 4), dtype=torch.float32).pin_memory(),
                     torch.empty(HEIGHT * WIDTH, dtype=torch.float32).pin_memory()) for _ in range(2)]
        host_frames = [torch.from_numpy(f).pin_memory() for f in frames]
        e2e_samples = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_np = [f.numpy() for f in host_frames]
        for k in range(args.steps):
            kk = counter["k"]
            counter["k"] += 1
            upload_next(kk, host_np)
            req = reqs[kk % len(reqs)]
            req.frame = kk % 2
            ctx.render_async(req, host_out[k % 2][0].numpy(), host_out[k % 2][1].numpy())
            ctx.frame_wait(0, (kk + 1) % 2)
            e2e_samples += samples_per_frame[kk % len(reqs)]
        ctx.sync()
        e2e_t = time.perf_counter() - t0

    dev_t = sum(step_ms) / 1000.0
    if dist:
        dev_t, e2e_t, total_samples, e2e_samples = combine_ranks(dist, dev_t, e2e_t, total_samples, e2e_samples, "cuda")
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    value = total_samples / dev_t
    mean_samples = statistics.mean(samples_per_frame)
    stage_ms = {k: v / args.steps for k, v in stages["stage_ms"].items() if stages["stage_calls"][k]}
    # deform + encode = the nearest-triangle walk (its own stage) + the map and hash encode
    near_s = stage_ms.get("nearest", 0.0) / 1000.0
    de_s = near_s + stage_ms.get("deform_encode", 0.0) / 1000.0
    mlp_s = stage_ms["mlp"] / 1000.0
    de_bytes, mlp_flop = deform_encode_bytes_per_sample(fc), mlp_flop_per_sample(fc)
    achieved = mean_samples * de_bytes / de_s / 1e9
    # the walk's FP32 work from its counters (the stage-timing pass): 4 child boxes per inner node
    # for all 32 lanes at 12 FLOP, 15 FLOP per bounding-disk test, 60 per exact triangle test
    walk = stages["walk"]
    walk_flop = (walk["inner_nodes"] * 4 * 32 * 12 + walk["bound_tests"] * 15 + walk["exact_tests"] * 60) / args.steps
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    tflops_peak = peaks.get("bf16_tflops", 1900.0)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * dev_t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32 geometry / fp16 mlp", "data": "synthetic",
        "config": {"workload": f"render {WIDTH}x{HEIGHT}, 1 avatar, 10240-triangle tracked mesh rebuilt per frame, "
                               f"occupancy from mesh (1.5 cm), {field_label(fc)}",
                   "global_batch": world, "samples_per_frame": mean_samples, "parallelism": f"replicas x{world}",
                   "l2": "flushed (512 MiB write) between timed steps", "frames_per_s": args.steps * world / dev_t,
                   "settle_s": SETTLE_S,
                   "render_loop": "host-driven rounds with per-stage events" if args.stage_timing else
                                  "one CUDA-graph launch per frame (conditional while node over the rounds)"},
        "roofline": {"bound": "hbm", "kernel": "deform+encode stage (nearest_stage_kernel + map_encode_kernel)",
                     "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": TRAFFIC_PER_FRAME if WIDTH == 512 and FIELD == "benchmark" else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the stage's launches for one "
                                       "512x512 frame, captured separately (not measured in this run)",
                     "basis": f"{de_bytes} B per sample ({hash_bytes_per_sample(fc)} B hash gathers + stream in/out) "
                              f"x samples per frame / deform_encode stage time per frame (CUDA events); per frame = "
                              f"its 2 launches, for achieved and traffic alike",
                     "peak_source": "MEASURED_PEAKS.json (of measured)" if peaks else "fallback"},
        "roofline_fp32": {"kernel": "nearest_stage_kernel (warp-cooperative exact nearest triangle)",
                          "achieved": walk_flop / near_s / 1e12 if near_s else None, "peak": FP32_PEAK_TFLOPS, "unit": "TFLOP/s",
                          "frac": walk_flop / near_s / 1e12 / FP32_PEAK_TFLOPS if near_s else None,
                          "peak_source": "nominal (152 SMs x 128 FP32 lanes x 2 x 2.07 GHz)",
                          "per_warp_walk": {"inner_nodes": walk["inner_nodes"] / max(walk["warps"], 1),
                                            "leaves": walk["leaves"] / max(walk["warps"], 1)},
                          "per_sample": {"bound_tests": walk["bound_tests"] / args.steps / mean_samples,
                                         "exact_tests": walk["exact_tests"] / args.steps / mean_samples}},
        "roofline_tensor": {"kernel": "mlp256_kernel", "achieved": mean_samples * mlp_flop / mlp_s / 1e12,
                            "peak": tflops_peak, "unit": "TFLOP/s", "flop_per_sample": mlp_flop,
                            "frac": mean_samples * mlp_flop / mlp_s / 1e12 / tflops_peak},
        "stage_ms_per_frame": stage_ms,
        "e2e": {"value": e2e_samples / e2e_t, "unit": UNIT, "h2d_bytes_per_step": int(av.n_verts * 12),
                "d2h_bytes_per_step": int(WIDTH * HEIGHT * 20)},
        "gpu_launches": launches,
        "clocks": clock_summary,
        "wall_s_timed": t_wall,
        "tuning": dict(ctx.tuning_get(), **(tuning_note or {})),
    }
    if not args.no_cpu_baseline:
        s, t, _, threads = cpu_render_rate(av, fc, params, frames[0], cams[0], 24)
        line["cpu_baseline"] = {"value": s / t, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"24 central rows of the {WIDTH}x{HEIGHT} frame, CPU restatement, OpenMP"}
    print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


def run_batch64(args):
    """Batched expressions: one avatar, 64 tracked frames (own LBVH each, one build launch), each
    rendered at 512x512 with its own camera yaw in [-30, 30] degrees, all rays in one wavefront.
    One step = upload of the 64 frames + their occupancy + the batched render."""
    import torch
    from insta_gb300 import abi, synthetic as S
    n = args.batch
    av = S.make_avatar(0)
    fc = S.FieldConfig()
    ctx = abi.Context(0)
    ctx.canonical_set(0, av.canonical, av.faces, av.mask)
    ctx.params_load(0, fc, S.field_params(fc, seed=0))
    rng = np.random.default_rng(3)
    frames = [torch.from_numpy(av.frame(av.frame_coeffs(k))).cuda() for k in range(n)]
    yaws = rng.uniform(-30.0, 30.0, n)
    reqs, outs = [], []
    for k in range(n):
        cam, focal = S.camera(float(yaws[k]), width=WIDTH, height=HEIGHT)
        reqs.append(ctx.render_desc(0, k, WIDTH, HEIGHT, focal, cam, cone_angle=CONE))
        outs.append((torch.empty((WIDTH * HEIGHT, 4), device="cuda"), torch.empty(WIDTH * HEIGHT, device="cuda")))
    ids = list(range(n))

    def step():
        ctx.frame_upload_batch(0, ids, frames)
        for k in ids:
            ctx.occupancy_from_mesh(0, k, RADIUS)
        ctx.render_batch(reqs, [o[0] for o in outs], [o[1] for o in outs])

    for _ in range(args.warmup):
        step()
    ctx.sync()
    samples = ctx.render_samples()
    ctx.stats(reset=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):   # the batched render's rounds: one CUDA-graph launch per batch
        step()
    ctx.sync()
    dt = (time.perf_counter() - t0) / args.steps
    launches = ctx.stats(reset=True)["kernel_launches"] / args.steps
    ctx.stats_enable(True)        # stage breakdown (host-driven rounds, same kernels), untimed
    for _ in range(args.steps):
        step()
    ctx.sync()
    st = ctx.stats(reset=True)
    ctx.stats_enable(False)
    # the same frames one at a time (plain path)
    t1 = time.perf_counter()
    for k in ids:
        ctx.frame_upload(0, k, frames[k])
        ctx.occupancy_from_mesh(0, k, RADIUS)
        ctx.render(reqs[k], outs[k][0], outs[k][1])
    ctx.sync()
    plain = time.perf_counter() - t1
    line = {"workload": f"batch of {n} expressions x {WIDTH}x{HEIGHT}", "samples_per_batch": samples,
            "ms_per_batch": dt * 1e3, "frames_per_s": n / dt, "samples_per_s": samples / dt,
            "plain_frames_per_s": n / plain, "speedup_vs_plain": plain / dt, "kernel_launches_per_batch": launches,
            "stage_ms_per_batch": {k: v / args.steps for k, v in st["stage_ms"].items() if st["stage_calls"][k]}}
    print(json.dumps(line), flush=True)
    ctx.close()


def apply_tuning(ctx, args):
    """--tune k=v,...: the render wavefront's launch shapes through insta_tuning_set."""
    if args.tune:
        kv = dict(item.split("=") for item in args.tune.split(",") if item)
        ctx.tuning_set(**{k: int(v) for k, v in kv.items()})


def run_map(args):
    """Plain canonical mapping: 1,048,576 points uniform in a 1 cm shell around the deformed
    surface (area-weighted surface point + normal offset U(-5, 5) mm) -> nearest triangle id
    (bit-exact) + canonical xyz, through insta_canonical_map_soa.  Device time from the library's
    stage events; e2e adds the pinned H2D of the points and the D2H of ids + canonical xyz."""
    import torch
    from insta_gb300 import abi, synthetic as S
    from oracle import oracle as O
    n = 1 << 20
    av = S.make_avatar(0)
    frame = av.frame(av.frame_coeffs(0))
    pts = S.shell_points(frame, av.faces, n, seed=0, half_width=5e-3)
    stream = torch.cuda.Stream()
    ctx = abi.Context(0, stream=stream.cuda_stream)
    ctx.canonical_set(0, av.canonical, av.faces, av.mask)
    ctx.frame_upload(0, 0, frame)
    d_pts = torch.from_numpy(pts).cuda()
    idx = torch.empty(n, dtype=torch.int32, device="cuda")
    can = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    with torch.cuda.stream(stream):
        for _ in range(max(3, args.warmup)):
            ctx.canonical_map_soa(0, 0, d_pts, n, idx, can)
        ctx.sync()
        ctx.stats(reset=True)
        ctx.stats_enable(True)
        for _ in range(args.steps):
            flush.zero_()
            ctx.canonical_map_soa(0, 0, d_pts, n, idx, can)
        ctx.sync()
        st = ctx.stats(reset=True)
        ctx.stats_enable(False)
        dev_ms = st["stage_ms"]["canonical_map"] / st["stage_calls"]["canonical_map"]
        # the same points as NerfCoordinate records through the render_deformed hook (frame 0)
        rec = np.zeros((n, 11), np.float32)
        rec[:, :3] = pts
        rec[:, 8:11] = 0.5
        d_rec0 = torch.from_numpy(rec).cuda()
        d_rec = torch.empty_like(d_rec0)
        for _ in range(3):
            d_rec.copy_(d_rec0)
            ctx.canonical_map(0, 0, d_rec, 11, 0, n)
        ctx.sync()
        ctx.stats(reset=True)
        ctx.stats_enable(True)
        for _ in range(args.steps):
            d_rec.copy_(d_rec0)
            ctx.canonical_map(0, 0, d_rec, 11, 0, n)
        ctx.sync()
        st = ctx.stats(reset=True)
        ctx.stats_enable(False)
        coords_ms = st["stage_ms"]["canonical_map"] / st["stage_calls"]["canonical_map"]
        h_pts = torch.from_numpy(pts).pin_memory()
        h_idx = torch.empty(n, dtype=torch.int32).pin_memory()
        h_can = torch.empty((n, 3), dtype=torch.float32).pin_memory()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            d_pts.copy_(h_pts, non_blocking=True)
            ctx.canonical_map_soa(0, 0, d_pts, n, idx, can)
            h_idx.copy_(idx, non_blocking=True)
            h_can.copy_(can, non_blocking=True)
        stream.synchronize()
        e2e_s = (time.perf_counter() - t0) / args.steps
    dtr = O.build_triangles(frame, av.canonical, av.faces, av.mask)
    bvh = O.Bvh(dtr)
    ref_ids, _ = bvh.nearest(pts[:65536])
    assert (h_idx.numpy()[:65536] == ref_ids).all(), "canonical map ids differ from the oracle"
    line = {"workload": "canonical map, 1,048,576 points in a 1 cm shell, 10,240-triangle frame",
            "points_per_s": n / (dev_ms / 1e3), "ms_per_call": dev_ms, "launches_per_call": 6,
            "records_ms_per_call": coords_ms, "records_per_s": n / (coords_ms / 1e3),
            "e2e": {"points_per_s": n / e2e_s, "h2d_bytes": n * 12, "d2h_bytes": n * 16}}
    if not args.no_cpu_baseline:
        m = 1 << 16
        d = O.Deformation(dtr, O.build_triangles(av.canonical, None, av.faces, av.mask), O.adjacency(av.faces, av.n_verts), bvh)
        t0 = time.perf_counter()
        d.map_soa(pts[:m])
        t = time.perf_counter() - t0
        line["cpu_baseline"] = {"points_per_s": m / t, "cores": O.num_threads(), "kind": "port",
                                "sample": f"first {m} points, oracle map_soa (BVH nearest + map), OpenMP"}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_grid(args):
    """Density-grid maintenance (update_density_grid_nerf with the random-frame warp) at the sizes
    training_prep_nerf uses with 2 cascades: the first 256 steps take 128^3 x 2 uniform samples,
    later steps 128^3 / 4 x 2 uniform + as many non-uniform.  8 tracked frames to pick from; the
    bench field (16-level hash grid, 32-64-16 / 32-64-64-3 MLPs).  Device time from the library's
    stage events (the update, then the bitfield of frame 0)."""
    import torch
    from insta_gb300 import abi, synthetic as S
    from oracle import oracle as O
    av = S.make_avatar(0)
    fc = S.FieldConfig()
    ctx = abi.Context(0)
    ctx.canonical_set(0, av.canonical, av.faces, av.mask)
    for k in range(8):
        ctx.frame_upload(0, k, av.frame(av.frame_coeffs(k)))
    ctx.params_load(0, fc, S.field_params(fc, seed=0))
    n_casc = 2
    ctx.density_grid_reset(0, n_casc, None)
    grid_rng = O.Pcg32.seeded(1337)
    warp_rng = O.Pcg32.seeded(42)
    out = {}
    for name, (nu, nn) in {"early (128^3 x 2 uniform)": (128 ** 3 * n_casc, 0),
                           "later (128^3/4 x 2 uniform + non-uniform)": (128 ** 3 // 4 * n_casc, 128 ** 3 // 4 * n_casc)}.items():
        desc = abi.DensityUpdateDesc()
        desc.decay, desc.n_uniform, desc.n_nonuniform, desc.n_cascades = 0.95, nu, nn, n_casc
        desc.aabb_max[:] = [1.0, 1.0, 1.0]
        desc.grid_rng = abi.Pcg32State(grid_rng.state, grid_rng.inc)
        desc.warp_rng = abi.Pcg32State(warp_rng.state, warp_rng.inc)
        desc.n_frames, desc.bitfield_frame = 8, 0
        for _ in range(max(3, args.warmup)):
            ctx.density_grid_update(0, desc)
        ctx.sync()
        ctx.stats(reset=True)
        ctx.stats_enable(True)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ctx.density_grid_update(0, desc)
        ctx.sync()
        wall = (time.perf_counter() - t0) / args.steps
        st = ctx.stats(reset=True)
        ctx.stats_enable(False)
        dev = st["stage_ms"]["occupancy"] / args.steps
        out[name] = {"samples": nu + nn, "ms_per_update": dev, "wall_ms_per_update": wall * 1e3,
                     "samples_per_s": (nu + nn) / (dev / 1e3)}
    print(json.dumps({"workload": "density-grid update, 2 cascades, 8 frames", "results": out}), flush=True)
    ctx.close()


def run_train(args):
    """One training step of the field (Testbed::train_nerf_step as insta_gb300.train.TrainStep
    runs it): 4096 rays per batch through the tracked frame's occupancy, the field evaluated on
    every march sample, the loss over the rays, backward over the 2^18-sample compacted batch
    (rollover-filled), Adam.  The bench field with 16 expression dims.  Device time per stage
    from the library's events, wall time per step with the step's one counter read-back."""
    import torch
    from insta_gb300 import abi, synthetic as S
    from insta_gb300.train import TrainConfig, TrainStep
    av = S.make_avatar(0)
    fc = S.FieldConfig(n_extra=16) if FIELD == "benchmark" else S.insta_field_config()
    ctx = abi.Context(0)
    ctx.canonical_set(0, av.canonical, av.faces, av.mask)
    ctx.frame_upload(0, 0, av.frame(av.frame_coeffs(0)))
    ctx.occupancy_from_mesh(0, 0, 0.015)
    ctx.params_load(0, fc, S.field_params(fc, seed=0))
    cfg = TrainConfig(n_rays_per_batch=4096, target_batch_size=1 << 18, max_samples=1 << 20, tf32=args.train_math != "fp32",
                      tcgen05=args.train_math == "tcgen05")
    ts = TrainStep(ctx, 0, fc, cfg)
    rng = np.random.default_rng(0)
    n = cfg.n_rays_per_batch

    def batch():
        c0 = np.array([0.5, 0.5, 0.5], np.float32)
        u = rng.normal(size=(n, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        org = c0 + u * 0.9
        tgt = c0 + rng.normal(0, 0.05, (n, 3))
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        return (dev(np.concatenate([org, tgt - org], 1).astype(np.float32)), dev(np.zeros(n, np.int32)),
                dev(rng.random(n).astype(np.float32)), dev(rng.uniform(0, 1, (n, 4)).astype(np.float32)),
                dev(rng.uniform(0, 1, (n, 3)).astype(np.float32)), dev(rng.uniform(-1, 1, (1, 16)).astype(np.float32)))

    batches = [batch() for _ in range(4)]

    def step(k):
        r, img, rnd, tgt, bg, ex = batches[k % len(batches)]
        return ts.step(0, r, img, rnd, tgt, background=bg, extra=ex, n_images=1)

    for k in range(max(3, args.warmup)):
        step(k)
    ctx.sync()
    ctx.stats(reset=True)
    ctx.stats_enable(True)
    samples = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        samples += step(k)["samples"]
    ctx.sync()
    wall = (time.perf_counter() - t0) / args.steps
    st = ctx.stats(reset=True)
    ctx.stats_enable(False)
    stage = {k: v / args.steps for k, v in st["stage_ms"].items() if v > 0}
    dev_ms = sum(stage.values())
    line = {"workload": "training step: 4096 rays, 2^18-sample batch, " + ("field with 16 expression dims" if FIELD == "benchmark" else field_label(fc)),
            "train_math": {"tcgen05": "tcgen05 kernel: FP16 operands, FP32 accumulation in TMEM",
                           "tf32": "TF32 tensor-core layer products (cuBLAS), FP32 accumulation",
                           "fp32": "FP32 layer products (cuBLAS)"}["tcgen05" if ts.tcgen05 else ("fp32" if args.train_math == "fp32" else "tf32")],
            "ms_per_step_device": dev_ms, "ms_per_step_wall": wall * 1e3, "stage_ms_per_step": stage,
            "march_samples_per_step": samples / args.steps,
            "trained_samples_per_s_device": cfg.target_batch_size / (dev_ms / 1e3),
            "rays_per_s_wall": n / wall}
    if not args.no_cpu_baseline:
        # the CPU restatement of the loss and the field backward on a bounded slice of one step
        from oracle import oracle as O
        torch.cuda.synchronize()
        ctx.sync()
        n_cpu = 4096
        co = ts.coords_out[:n_cpu].cpu().numpy()
        dl = ts.dloss[:n_cpu].cpu().numpy()
        params = S.field_params(fc, seed=0)
        t0 = time.perf_counter()
        O.field_backward(fc, params, co, dl)
        t_bwd = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n_cpu / t_bwd, "unit": "trained samples/s", "cores": 1, "kind": "port",
                                "sample": f"FP64 field forward+backward of {n_cpu} compacted samples of the step"}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_raycast(args):
    """raycast_flame of the 10,240-triangle tracked frame at 512^2 and 1024^2 (closest hit over the
    frame's LBVH + shading).  Device time from the library's stage events; the CPU restatement
    (brute-force closest hit) is timed on 8 image rows."""
    import torch
    from insta_gb300 import abi, synthetic as S
    from oracle import oracle as O
    av = S.make_avatar(0)
    frame = av.frame(av.frame_coeffs(0))
    ctx = abi.Context(0)
    ctx.canonical_set(0, av.canonical, av.faces, av.mask)
    ctx.frame_upload(0, 0, frame)
    out = {}
    for w in (512, 1024):
        cam, focal = S.camera(0.0, width=w, height=w)
        req = ctx.render_desc(0, 0, w, w, focal, cam)
        rgba = torch.zeros((w * w, 4), device="cuda")
        depth = torch.zeros(w * w, device="cuda")
        for _ in range(max(3, args.warmup)):
            ctx.raycast(req, rgba, depth)
        ctx.sync()
        ctx.stats(reset=True)
        ctx.stats_enable(True)
        for _ in range(args.steps):
            ctx.raycast(req, rgba, depth)
        ctx.sync()
        st = ctx.stats(reset=True)
        ctx.stats_enable(False)
        ms = st["stage_ms"]["raycast"] / args.steps
        out[f"{w}x{w}"] = {"ms_per_frame": ms, "rays_per_s": w * w / (ms / 1e3)}
    line = {"workload": "raycast of the tracked frame (10,240 triangles)", "results": out}
    if not args.no_cpu_baseline:
        tris = O.build_triangles(frame, av.canonical, av.faces, av.mask)
        cam, focal = S.camera(0.0, width=512, height=8)
        rc = O.render_cfg(512, 8, focal, cam, av.render_aabb())
        t0 = time.perf_counter()
        O.raycast(rc, tris, O.mesh_centroid(av.canonical))
        t = time.perf_counter() - t0
        line["cpu_baseline"] = {"rays_per_s": 512 * 8 / t, "cores": O.num_threads(), "kind": "port",
                                "sample": "512 x 8 rays, brute-force closest hit, OpenMP"}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_serve(args):
    """Served mixed stream: 8 resident avatars, Poisson arrivals, each request a fresh expression
    (its own frame upload, LBVH, occupancy) at a resolution drawn from {256, 512, 768, 1024}^2.

    * plain: the single-frame path served for real -- one request at a time in arrival order
      (frame upload + occupancy + insta_render, FP32 geometry / FP16 MLPs), each latency measured
      from its arrival to the end of its render;
    * batched: the request loop (insta_server_*: continuous batching, rounds as CUDA-graph launches
      between admission points, launch shapes from insta_autotune) with BF16 MLPs (hash features
      FP16, geometry FP32), submissions paced to the same arrival times.
    Both arms also run a saturating burst (every request of a 2-second slice submitted at once) for
    their capacity in frames/s."""
    from insta_gb300 import abi, synthetic as S
    rng = np.random.default_rng(17)
    ctx = abi.Context(0, budget_bytes=40 << 30)
    fc = S.FieldConfig()
    avs, params = [], []
    for aid in range(8):
        av = S.make_avatar(aid)
        ctx.canonical_set(aid, av.canonical, av.faces, av.mask)
        params.append(S.field_params(fc, seed=aid))
        avs.append(av)
    n = int(args.rate * args.duration)
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, n))
    sizes = rng.choice([256, 512, 768, 1024], n)
    reqs = []
    for k in range(n):
        aid = int(rng.integers(0, 8))
        w = int(sizes[k])
        cam, focal = S.camera(float(rng.uniform(-30, 30)), width=w, height=w)
        coeffs = rng.normal(0.0, 0.3, avs[aid].basis.shape[0])
        reqs.append((ctx.render_desc(aid, -1, w, w, focal, cam, cone_angle=CONE), avs[aid].frame(coeffs)))
    import torch
    # page-locked host outputs for both arms (a serving front end hands out such buffers)
    pool = {w: [(torch.empty((w * w, 4), dtype=torch.float32).pin_memory().numpy(),
                 torch.empty(w * w, dtype=torch.float32).pin_memory().numpy()) for _ in range(48)] for w in (256, 512, 768, 1024)}
    n_burst = min(n, int(2.0 * args.rate))

    def plain_one(k):
        r, v = reqs[k]
        o = pool[r.width][k % 48]
        ctx.frame_upload(r.avatar, 0, v)
        ctx.occupancy_from_mesh(r.avatar, 0, RADIUS)
        r.frame = 0
        ctx.render(r, o[0], o[1])      # host outputs: returns with the frame in host memory
        r.frame = -1

    # ---- plain arm (FP16 MLPs)
    for aid in range(8):
        ctx.params_load(aid, fc, params[aid], precision=abi.PRECISION_FP16)
    for k in range(3):
        plain_one(k)
    ctx.sync()
    t0 = time.perf_counter()
    for k in range(n_burst):
        plain_one(k)
    plain_capacity = n_burst / (time.perf_counter() - t0)
    plain_lat = np.zeros(n)
    t_start = time.perf_counter()
    for k in range(n):
        now = time.perf_counter() - t_start
        if now < arrivals[k]:
            time.sleep(arrivals[k] - now)
        plain_one(k)
        plain_lat[k] = (time.perf_counter() - t_start - arrivals[k]) * 1e3
    plain_span = time.perf_counter() - t_start

    # ---- batched arm (BF16 MLPs, the request loop)
    for aid in range(8):
        ctx.params_load(aid, fc, params[aid], precision=abi.PRECISION_BF16)
    ctx.frame_upload(0, 0, avs[0].frame(avs[0].frame_coeffs(0)))
    ctx.occupancy_from_mesh(0, 0, RADIUS)
    cam, focal = S.camera(0.0, width=512, height=512)
    tuned, _ = ctx.autotune([ctx.render_desc(0, 0, 512, 512, focal, cam, cone_angle=CONE)], repeats=3)
    ctx.sync()

    def serve(order_arrivals, count):
        srv = abi.Server(ctx, max_inflight=args.slots, max_inflight_pixels=args.slot_pixels, rounds_per_launch=2,
                         round_samples=args.round_samples)
        tickets = []
        t_s = time.perf_counter()
        for k in range(count):
            if order_arrivals is not None:
                while time.perf_counter() - t_s < order_arrivals[k]:
                    time.sleep(0.0002)
            r, v = reqs[k]
            o = pool[r.width][k % 48]
            if k >= 48:
                srv.wait(tickets[k - 48])   # the output buffer's previous request is done
            tickets.append(srv.submit(r, v, o[0], o[1]))
        states = [srv.wait(t) for t in tickets]
        t_e = time.perf_counter()
        lat = np.array([srv.poll(t)[1] for t in tickets])
        srv.close()
        return states, lat, t_e - t_s

    serve(None, min(64, n))                          # warm-up: graph instantiation, buffers
    _, _, burst_t = serve(None, n_burst)
    batched_capacity = n_burst / burst_t
    states, lat, span = serve(arrivals, n)
    ok = sum(1 for x in states if x == abi.REQ_DONE)
    px = float(np.mean(sizes.astype(np.float64) ** 2))
    line = {"workload": f"served stream: 8 avatars, Poisson {args.rate} req/s over {args.duration} s, "
                        f"sizes {{256,512,768,1024}}^2 (mean {px:.0f} px), fresh expression per request",
            "requests": n, "done": ok,
            "batched": {"precision": "bf16 mlp, fp16 hash features, fp32 geometry",
                        "capacity_frames_per_s": batched_capacity, "frames_per_s": ok / span,
                        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                        "p99_512_ms": float(np.percentile(lat[sizes == 512], 99)),
                        "slots": args.slots, "slot_pixels": args.slot_pixels, "rounds_per_launch": 2,
                        "round_samples": args.round_samples or (32 << 20), "tuning": tuned},
            "plain": {"precision": "fp16 mlp, fp32 geometry", "capacity_frames_per_s": plain_capacity, "frames_per_s": n / plain_span,
                      "p50_ms": float(np.percentile(plain_lat, 50)), "p99_ms": float(np.percentile(plain_lat, 99)),
                      "p99_512_ms": float(np.percentile(plain_lat[sizes == 512], 99))},
            "capacity_ratio": batched_capacity / plain_capacity,
            "burst_requests": n_burst}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_precision(args):
    """Precision variants of the 1024x1024 render: MLPs in FP16 (plain), BF16 and FP8 E4M3 (per-layer
    weight scale), FP32 accumulation; geometry FP32.  Reports per variant: device time per frame,
    pixel error and PSNR against the host FP64 oracle on a band of central rows, PSNR against the
    plain path, network-output error against the FP64 oracle on random field coordinates, and the
    canonical-coordinate error of the map against the FP64 oracle."""
    import torch
    from insta_gb300 import abi, synthetic as S
    from oracle import oracle as O
    W = H = args.width if args.width != 512 else 1024
    av = S.make_avatar(0)
    fc = S.FieldConfig()
    params = S.field_params(fc, seed=0)
    frame = av.frame(av.frame_coeffs(0))
    ctx = abi.Context(0)
    apply_tuning(ctx, args)
    ctx.canonical_set(0, av.canonical, av.faces, av.mask)
    ctx.frame_upload(0, 0, frame)
    ctx.occupancy_from_mesh(0, 0, RADIUS)
    cam, focal = S.camera(0.0, width=W, height=H)
    req = ctx.render_desc(0, 0, W, H, focal, cam, cone_angle=CONE)
    # FP64 oracle references
    can = O.build_triangles(av.canonical, None, av.faces, av.mask)
    dtr = O.build_triangles(frame, av.canonical, av.faces, av.mask)
    adj = O.adjacency(av.faces, av.n_verts)
    bvh = O.Bvh(dtr)
    bits = O.occupancy(dtr, RADIUS)
    d64 = O.Deformation(dtr, can, adj, bvh, fp64=True)
    rc = O.render_cfg(W, H, focal, cam, av.render_aabb(), cone_angle=CONE)
    r0, r1 = H // 2 - args.rows // 2, H // 2 + args.rows // 2
    ref64, _, _, _ = O.render(rc, d64, bits, fc, params, rows=(r0, r1), fp64=True)
    rng = np.random.default_rng(5)
    coords = np.zeros((1 << 16, 11), np.float32)
    coords[:, :3] = rng.uniform(0.38, 0.62, (len(coords), 3))
    dirs = rng.normal(size=(len(coords), 3))
    coords[:, 8:11] = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True) + 1) * 0.5
    field64 = O.field_eval(fc, params, coords, fp64=True)
    pts = S.shell_points(frame, av.faces, 1 << 18, seed=3)
    _, can64 = d64.map_soa(pts)
    idx = torch.empty(len(pts), dtype=torch.int32, device="cuda")
    canon = torch.empty((len(pts), 3), device="cuda")
    ctx.canonical_map_soa(0, 0, torch.from_numpy(pts).cuda(), len(pts), idx, canon)
    ctx.sync()
    diag = float(np.linalg.norm(av.canonical.max(0) - av.canonical.min(0)))
    canon_err = float(np.abs(canon.cpu().numpy().astype(np.float64) - can64).max()) / diag
    rgba = torch.empty((W * H, 4), device="cuda")
    depth = torch.empty(W * H, device="cuda")
    out = {"workload": f"precision variants, render {W}x{H}", "canonical_err_over_diag": canon_err,
           "oracle_rows": [r0, r1], "variants": {}}
    plain = None
    for name, prec in (("fp16", abi.PRECISION_FP16), ("bf16", abi.PRECISION_BF16), ("fp8_e4m3", abi.PRECISION_FP8)):
        ctx.params_load(0, fc, params, precision=prec)
        for _ in range(args.warmup):
            ctx.render(req, rgba, depth)
        ctx.sync()
        ctx.stats(reset=True)
        ctx.stats_enable(True)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ctx.render(req, rgba, depth)
        ctx.sync()
        ms = (time.perf_counter() - t0) / args.steps * 1e3
        st = ctx.stats(reset=True)
        ctx.stats_enable(False)
        img = rgba.cpu().numpy()
        band = img.reshape(H, W, 4)[r0:r1].reshape(-1, 4)
        if plain is None:
            plain = img.copy()
        fo = torch.zeros((len(coords), 4), device="cuda")
        ctx.field_eval(0, torch.from_numpy(coords).cuda(), 11, len(coords), fo)
        ctx.sync()
        fe = np.abs(fo.cpu().numpy().astype(np.float64) - field64)
        mse = float(np.mean((band.astype(np.float64) - ref64) ** 2))
        mse_plain = float(np.mean((img.astype(np.float64) - plain) ** 2))
        out["variants"][name] = {
            "ms_per_frame": ms, "mlp_ms": st["stage_ms"]["mlp"] / args.steps,
            "pixel_max_abs_err_vs_fp64": float(np.abs(band - ref64).max()),
            "psnr_vs_fp64_oracle": 10 * math.log10(1.0 / mse) if mse > 0 else float("inf"),
            "psnr_vs_plain": 10 * math.log10(1.0 / mse_plain) if mse_plain > 0 else float("inf"),
            "field_mean_abs_err_vs_fp64": float(fe.mean()), "field_max_abs_err_vs_fp64": float(fe.max()),
            "density_max_abs_err_vs_fp64": float(fe[:, 3].max())}
    print(json.dumps(out), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--stage-timing", action="store_true",
                    help="per-stage CUDA events on every render (host-driven rounds instead of the CUDA-graph loop; "
                         "for kernel-level profiles)")
    ap.add_argument("--width", type=int, default=512, help="square render size (512 = the benchmark workload)")
    ap.add_argument("--workload", choices=["render", "batch", "serve", "precision", "map", "grid", "raycast", "train"], default="render",
                    help="render: the benchmark line; batch: 64 expressions in one wavefront; serve: request stream; "
                         "precision: FP16 / BF16 / FP8 MLPs at 1024x1024 against the FP64 oracle; "
                         "map: canonical mapping of 1M shell points; grid: density-grid update; raycast: mesh raycast")
    ap.add_argument("--rows", type=int, default=16, help="precision: image rows rendered by the FP64 oracle")
    ap.add_argument("--tune", default="", help="launch shapes, e.g. max_steps_per_round=16,bvh_top_nodes=21 (insta_tuning_set)")
    ap.add_argument("--autotune", action="store_true", help="render: run insta_autotune on the frame before the warm-up")
    ap.add_argument("--train-math", choices=["tcgen05", "tf32", "fp32"], default="tcgen05", help="train: the backward's layer products")
    ap.add_argument("--field", choices=["benchmark", "insta"], default="benchmark",
                    help="render / reference arm: the benchmark's 16 x 2 field or INSTA's shipped 16 x 8 one (16 expression dims)")
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--rate", type=float, default=240.0)
    ap.add_argument("--duration", type=float, default=30.0)
    ap.add_argument("--slots", type=int, default=16)
    ap.add_argument("--slot-pixels", type=int, default=6 << 20)
    ap.add_argument("--round-samples", type=int, default=0, help="served stream: samples per round at most (0 = 2^25)")
    args = ap.parse_args()
    global WIDTH, HEIGHT, FIELD
    WIDTH = HEIGHT = args.width
    FIELD = args.field
    if args.workload == "batch":
        return run_batch64(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "precision":
        return run_precision(args)
    if args.workload == "map":
        return run_map(args)
    if args.workload == "grid":
        return run_grid(args)
    if args.workload == "train":
        return run_train(args)
    if args.workload == "raycast":
        return run_raycast(args)
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
