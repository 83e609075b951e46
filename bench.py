"""Benchmark: aggregate fused frames/s and per-frame latency of the served
(batched) path against the plain one-session-at-a-time path, on one GB300.

A step (tick) fuses one 640x480 frame for every concurrent session: ingest and
pyramids, coarse-to-fine ICP + photometric tracking, block allocation,
visible-block enumeration, TSDF/colour integration, z-range tiles, raycast and
the post-raycast pyramid (System::process_images of the reference,
src/system.cpp:40-114), all sessions in the same launches replayed from a CUDA
graph.  Inputs are seeded synthetic RGB-D frames of the reference's camera
shape (the reference measures on a live camera; no dataset is available).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--sessions S] [--impl reference]

Prints one JSON line.  With torchrun (N > 1) every rank serves its own
sessions (replicas, no collective on the data path); rank 0 prints.
"""
from __future__ import annotations

import argparse
import gc
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

METRIC = "aggregate fused frames/s + p99 frame latency: served vs plain, same GPU & err"
UNIT = "frames/s"
W, H = 640, 480
VOXELS = (0.005, 0.006, 0.008, 0.01)  # served sessions draw voxel sizes of 5-10 mm
# voxel layouts: gbf_voxel_layout value and storage
LAYOUTS = {"half": (1, "fp16 sdf + binary16 weight + rgba8 (8 B/voxel)"),
           "snorm": (2, "int16 sdf (rounded) + binary16 weight + rgba8 (8 B/voxel)"),
           "ref": (0, "int16 sdf (truncated) + f32 weight + rgba8 (12 B/voxel)")}
LAYOUT = "snorm"  # the 8-byte layout within the 1e-3 x truncation TSDF error goal (HALF's fp16 step is not)
PREC_FRAMES = 20  # frames of the precision check (tracking loop and mapping at ground-truth poses)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--sessions", type=int, default=64)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-frames", type=int, default=0,
                    help="timed frames per plain session (0 = as many as the timed ticks)")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--groups", type=int, default=2, help="concurrent session groups per tick (with --no-autotune)")
    ap.add_argument("--no-autotune", action="store_true", help="fixed launch shape instead of the batch's tuner")
    ap.add_argument("--tune-ticks", type=int, default=6, help="timed ticks per tuner candidate")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--serve-seconds", type=float, default=40.0,
                    help="wall-clock seconds of the continuous-batching serving run (0: skip)")
    ap.add_argument("--layout", default="snorm", choices=sorted(LAYOUTS), help="voxel storage of every session")
    ap.add_argument("--precision-frames", type=int, default=PREC_FRAMES,
                    help="frames of the precision check against the FP64 oracle (0: skip)")
    ap.add_argument("--workload", default="served", choices=["served", "mixed", "scale", "precision"],
                    help="mixed: sessions of three resolutions and three voxel sizes in one batch "
                         "(served vs plain only; prints its own line); scale: the large-map "
                         "configuration as one plain session, phase by phase")
    ap.add_argument("--scale-frames", type=int, default=2000, help="frames of the scale workload")
    ap.add_argument("--precision-track", type=int, default=2000, help="tracked frames of the precision workload")
    return ap.parse_args()


# ----------------------------------------------------------------------------- setup

def session_config(L, i: int):
    v = VOXELS[i % len(VOXELS)]
    tau = min(max(3.0 * v, 0.02), 0.03)
    return L.default_config(voxel_size=v, truncation=tau, zmin_update=0.3, zmax_update=4.0, zmin_raycast=0.3,
                            zmax_raycast=4.0, num_buckets=1 << 19, num_blocks=1 << 18, voxel_layout=LAYOUTS[LAYOUT][0],
                            num_levels=3, max_iterations=[10, 5, 3, 3, 3], max_probe=256)


def workload_config(sessions: int) -> dict:
    """The served workload both arms report."""
    return {"workload": f"served: {sessions} concurrent 640x480 sessions per GPU, one frame each per tick",
            "sessions_per_gpu": sessions, "voxel_m": list(VOXELS), "truncation": "clip(3*voxel, 2 cm, 3 cm)",
            "voxel_layout": LAYOUTS[LAYOUT][1], "pool_blocks": 1 << 18,
            "hash_slots": 1 << 19, "pyramid": "3 levels 10/5/3"}


def tune_launch_shape(L, K, S, frames, poses0, per_candidate, make=None):
    """The batch tuner's search for this workload's shape, run on throwaway
    sessions of the same configurations over the first frames, so that the
    measured batches settle from the process-wide table at their first tick.
    make(i) builds session i (default: the served workload's)."""
    import torch
    L.autotune_forget()
    ss = [make(i) if make else L.System(K, session_config(L, i)) for i in range(S)]
    for i, s in enumerate(ss):
        s.set_pose(poses0[i])
    b = L.FusionBatch(S)
    for i, s in enumerate(ss):
        b.set(i, s)
    b.autotune(True, per_candidate)
    active, k = [True] * S, 0
    while b.tuning()["state"] != "settled" and k < frames[0][0].shape[0]:
        for i in range(S):
            b.set_inputs(i, frames[i][0][k].data_ptr(), frames[i][1][k].data_ptr())
        b.process(active)
        k += 1
    t = b.tuning()
    t["ticks"] = k
    b.close()
    del ss
    torch.cuda.synchronize()
    return t


def launch_shape(batch, args, tuned):
    if tuned is None:
        batch.set_groups(args.groups)
    else:
        batch.autotune(True, args.tune_ticks)


def shape_report(batch, tuned, args, unsettled=None):
    t = batch.tuning()
    if tuned is None:
        return {"autotune": False, **t["chosen"], **({"note": unsettled} if unsettled else {})}
    return {"autotune": True, "settled_from_table": t["from_table"], "groups": t["chosen"]["groups"],
            "stagger": t["chosen"]["stagger"], "ray_tile_w": t["chosen"]["ray_tile_w"],
            "tuning_ticks": tuned["ticks"], "ticks_per_candidate": tuned["ticks_per_candidate"],
            "candidates_ms": [[c["groups"], c["stagger"], c["ray_tile_w"], round(c["median_ms"], 3)]
                              for c in tuned["tried"]],
            "candidate_fields": ["groups", "stagger", "ray_tile_w", "median tick ms"]}


def intrinsics(L):
    return L.IntrinsicMatrix(W, H, 525.0, 525.0, 319.5, 239.5)


def render_frames(L, K, seeds, n_frames):
    """Device-resident frames [session][frame] -> (depth u16, rgb8) tensors."""
    import torch
    frames = []
    poses = []
    for seed in seeds:
        sc = L.SynthScene(seed=seed)
        d = torch.empty((n_frames, H, W), dtype=torch.uint16, device="cuda")
        c = torch.empty((n_frames, H, W, 3), dtype=torch.uint8, device="cuda")
        for k in range(n_frames):
            sc.render_into(K, k, d[k].data_ptr(), c[k].data_ptr())
        frames.append((d, c))
        poses.append(sc.pose(0))
        sc.close()
    torch.cuda.synchronize()
    return frames, poses


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons during the timed region.

    The sampler starts before the region and waits (at most 5 s) for its first
    reading, so that the region is covered from its start; every line is
    stamped when it arrives, and the summary keeps the lines stamped between
    start() and stop() (the nearest one when the region is shorter than the
    sampling period)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 100

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines: list[tuple[float, str]] = []
        self.first = threading.Event()
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self.first.wait(timeout=5.0)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))
            self.first.set()

    def start(self):
        self.t0 = time.perf_counter()

    def stop(self):
        self.t1 = time.perf_counter()
        # one more period, so that a reading taken just before stop() has arrived
        time.sleep(self.PERIOD_MS / 1e3)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        t0 = self.t0 if self.t0 is not None else float("-inf")
        t1 = self.t1 if self.t1 is not None else float("inf")
        inside = [ln for t, ln in self.lines if t0 <= t <= t1 + self.PERIOD_MS / 1e3]
        if not inside and self.lines:
            mid = 0.5 * (self.t0 + self.t1) if self.t0 is not None and self.t1 is not None else self.lines[-1][0]
            inside = [min(self.lines, key=lambda tl: abs(tl[0] - mid))[1]]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in inside:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unsampled"], "samples": 0}
        load = [x for x in sm if x > 0.5 * max(sm)] or sm
        out = {"sm_mhz": statistics.median(load), "sm_max_mhz": mx, "reasons": sorted(reasons),
               "samples": len(sm), "period_ms": self.PERIOD_MS}
        if self.t0 is not None and self.t1 is not None:
            out["region_s"] = round(self.t1 - self.t0, 3)
        return out


# DRAM bytes one pixel-iteration of the ICP + photometric reduction moves, from
# one ncu capture of a level-0 launch over 4 sessions (105.50 MB for 1,228,800
# pixel-iterations, dram__bytes_read.sum + dram__bytes_write.sum): the roofline's traffic
REDUCE_DRAM_BYTES_PER_PIXEL_ITER = (102.178048e6 + 3.364608e6) / 1228800
# DRAM bytes per raycast pixel, from one ncu capture of the SNORM raycast over 4
# sessions with maps of 96 fused frames (81.94 MB read + 12.55 MB written for
# 4 x 307,200 pixels; same counters), and its issue-active fraction there.  The
# bytes depend on the maps the rays cross, so scaling by pixels is an estimate.
RAYCAST_DRAM_BYTES_PER_PIXEL = (81.93536e6 + 12.553472e6) / (4 * 307200)
RAYCAST_ISSUE_ACTIVE = 0.744


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def work_counters(sessions) -> tuple[int, int]:
    """Cumulative (pixel-iterations, integrated blocks) summed over sessions."""
    pi = ib = 0
    for s in sessions:
        st = s.stats()
        pi += st.pixel_iterations
        ib += st.integrated_blocks
    return pi, ib


def kernel_bytes(L, sessions, phase: str, K, d_pixel_iters: int, d_blocks: int, ticks: int) -> float:
    """Algorithmic bytes per tick of the phase's kernel, from the work the
    sessions actually did during the timed ticks (iterations that the
    reference's early-exit rules skipped read nothing)."""
    P = K.width * K.height
    sv = 12 if sessions[0].cfg.voxel_layout == L.VOXEL_REF else 8
    if phase == "integrate":
        # voxel read-modify-write of every visible block + per-pixel depth/weight and colour
        return (2.0 * sv * 512 * d_blocks + len(sessions) * ticks * P * (8 + 4)) / ticks
    # fused ICP + photometric rows: reference vertex+normal (32 B) and intensity (4 B),
    # current vertex+normal (32 B) and intensity + gradients (12 B) per pixel-iteration
    return 80.0 * d_pixel_iters / ticks


# ----------------------------------------------------------------------------- replicas

def replica_seeds(rank: int, sessions: int) -> list[int]:
    """Sessions are independent replicas: rank r serves its own seeded sessions."""
    return [1000 * rank + s for s in range(sessions)]


def max_over_ranks(ms: float, dist=None, device="cpu") -> float:
    """Whole-job time = the slowest rank's timed region."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(sessions_per_rank: int, world: int, steps: int, total_ms: float) -> float:
    return sessions_per_rank * world * steps / (total_ms / 1e3)


# ----------------------------------------------------------------------------- CPU

def cpu_mix(L, K, warmup: int, steps: int, seconds: float | None = None, threads: int | None = None,
            precision: str = "f32"):
    """The FP32 oracle (the reference's kernel bodies restated in C, OpenMP over
    pixels and blocks) on this machine's host cores: one CPU session per voxel
    size of the served mix, `warmup` untimed frames each, then frames timed
    round-robin over the sessions -- `steps` of them, or as many as fit in
    `seconds`.  Returns (per-frame seconds, sessions, threads)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    O.build()
    threads = threads or os.cpu_count() or 1
    n_mix = len(VOXELS)
    per = warmup + (steps + n_mix - 1) // n_mix
    mix = []
    for i in range(n_mix):
        fr = host_frames(L, K, per, seed=i)
        sysm = O.OracleSystem(O.config_from(session_config(L, i), threads=threads), O.intrinsics_from(K), precision)
        sysm.set_pose(fr[0][2])
        for k in range(warmup):
            sysm.process(fr[k][0], fr[k][1])
        mix.append((sysm, fr))
    t = []
    t_start = time.perf_counter()
    for k in range(steps):
        sysm, fr = mix[k % n_mix]
        d, c, _ = fr[warmup + k // n_mix]
        t0 = time.perf_counter()
        sysm.process(d, c)
        t.append(time.perf_counter() - t0)
        if seconds is not None and time.perf_counter() - t_start > seconds and len(t) >= n_mix:
            break
    return t, n_mix, threads


def cpu_sample_text(n: int, n_mix: int, threads: int) -> str:
    return (f"{n} 640x480 frames round-robin over {n_mix} sessions (voxel "
            f"{', '.join(f'{x * 1000:.0f}' for x in VOXELS[:n_mix])} mm) after warm-up frames, FP32 oracle "
            f"restating the reference kernels, {threads} threads")


def cpu_model() -> str:
    """The host CPU as /proc/cpuinfo names it (x86: model name; Arm: implementer and part)."""
    info = {}
    try:
        for line in open("/proc/cpuinfo"):
            k, _, v = line.partition(":")
            info.setdefault(k.strip(), v.strip())
    except OSError:
        pass
    if "model name" in info:
        return info["model name"]
    if "CPU part" in info:
        return f"{os.uname().machine}, CPU implementer {info.get('CPU implementer', '?')} part {info['CPU part']}"
    return os.uname().machine


def cpu_baseline(L, K, seconds: float, warmup: int):
    """All host threads on the bounded sample, one thread on a third of it, and
    the FP64 oracle (the error reference, not a baseline) on all threads."""
    t, n_mix, threads = cpu_mix(L, K, warmup, 256, seconds)
    t1, _, _ = cpu_mix(L, K, min(warmup, 2), 256, seconds / 3, threads=1)
    t64, _, _ = cpu_mix(L, K, min(warmup, 2), 256, seconds / 3, precision="f64")
    return {"value": len(t) / sum(t), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": cpu_sample_text(len(t), n_mix, threads) + f", {sum(t):.1f} s",
            "cpu": cpu_model(), "nproc": os.cpu_count(),
            "single_thread": {"value": len(t1) / sum(t1), "unit": UNIT, "cores": 1,
                              "sample": cpu_sample_text(len(t1), n_mix, 1) + f", {sum(t1):.1f} s"},
            "fp64_oracle": {"value": len(t64) / sum(t64), "unit": UNIT, "cores": threads,
                            "sample": cpu_sample_text(len(t64), n_mix, threads).replace("FP32", "FP64")
                            + f", {sum(t64):.1f} s; the error reference, timed for the record"}}


def precision_gpu(L, K, cfg, fr):
    """The GPU side of the precision check on one session's frames `fr`
    (depth u16, rgb, ground-truth pose): the tracking loop (System, the plain
    path, whose results the served batch reproduces bit for bit), and the
    normal-weighted mapping at the ground-truth poses with each frame's own
    normal map, raycast at the last pose."""
    import torch
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    s = L.System(K, cfg)
    s.set_pose(fr[0][2])
    poses = []
    for d, c, _ in fr:
        s.process_images(cu(d), cu(c))
        poses.append(s.get_camera_pose())
    s.close()
    t, m, nmaps = L.DenseTracking(K, cfg), L.DenseMapping(K, cfg), []
    for d, c, T in fr:
        dm = cu(d.astype(np.float32) * np.float32(0.001))
        t.set_current(dm, cu(c))
        n = t.get_image(0, 1, 0)  # the frame's level-0 normals (from the filtered depth, as System fuses)
        m.update(dm, cu(c), T, normal=n)
        nmaps.append(n.cpu().numpy())
    vm = torch.full((K.height, K.width, 4), float("nan"), dtype=torch.float32, device="cuda")
    m.raycast(vm, fr[-1][2])
    out = {"poses": np.array(poses), "map": m.export(), "vmap": vm.cpu().numpy(), "nmaps": nmaps}
    m.close()
    t.close()
    return out


def precision_check(L, K, cfg, fr, g, threads):
    """CPU leg: the FP64 oracle (double arithmetic, unquantised voxels) on the
    same frames, as the checker of the GPU results `g`: pose drift of the
    tracking loop, TSDF error of the ground-truth-pose map (sdf in units of
    the truncation distance, voxels observed in both maps), raycast depth of
    that map at the last pose (rays on the same surface, |dz| < truncation),
    and the tracking loop's trajectory error against the ground truth."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    O.build()
    oc, ok = O.config_from(cfg, threads=threads), O.intrinsics_from(K)
    t0 = time.perf_counter()
    osys = O.OracleSystem(oc, ok, "f64")
    osys.set_pose(fr[0][2])
    op = []
    for d, c, _ in fr:
        osys.process(d, c)
        op.append(osys.pose())
    op = np.array(op)
    gp = g["poses"]
    om = O.OracleMap(oc, ok, "f64")
    for (d, c, T), n in zip(fr, g["nmaps"]):
        om.fuse(d.astype(np.float32) * np.float32(0.001), c, T, nmap=n)
    gcoord, gs, gw, _ = g["map"]
    oc_, os_, ow, _ = om.export()
    key = lambda a: a[:, 0].astype(np.int64) * (1 << 42) + a[:, 1].astype(np.int64) * (1 << 21) + a[:, 2]
    gk, okk = key(gcoord.astype(np.int64) + (1 << 20)), key(oc_.astype(np.int64) + (1 << 20))
    common, gi, oi = np.intersect1d(gk, okk, return_indices=True)
    gs, gw, os_, ow = gs[gi], gw[gi], os_[oi], ow[oi]
    both = (gw > 0) & (ow > 0)
    err = np.abs(gs[both] - os_[both]).astype(np.float64)
    ov = om.raycast(fr[-1][2])
    gv = g["vmap"]
    gh, oh = ~np.isnan(gv[..., 2]), ~np.isnan(ov[..., 2])
    dz = np.abs(gv[..., 2][gh & oh] - ov[..., 2][gh & oh]).astype(np.float64)
    same = dz < cfg.truncation
    truth = np.array([T for _, _, T in fr])
    ate = np.sqrt(np.mean(np.sum((gp[:, :3, 3] - truth[:, :3, 3]) ** 2, axis=1)))
    return {
        "reference": "FP64 oracle (double arithmetic, unquantised voxels) on the host cores",
        "session": f"{len(fr)} frames of served session 0 (640x480, voxel {cfg.voxel_size * 1e3:.0f} mm, "
                   f"truncation {cfg.truncation * 1e3:.0f} mm, {LAYOUTS[LAYOUT][1]})",
        "pose_drift_mm": float(np.abs(gp[:, :3, 3] - op[:, :3, 3]).max() * 1e3),
        "pose_drift_goal_mm": 1.0,
        "tsdf_err_over_tau": {"p99.9": float(np.quantile(err, 0.999)), "mean": float(err.mean()),
                              "max": float(err.max()), "voxels": int(both.sum()),
                              "above_1e-3": int(np.sum(err > 1e-3)), "goal_p99.9": 1e-3,
                              "basis": "normal-weighted updates at the ground-truth poses, voxels observed in both "
                                       "maps; sdf is stored in units of the truncation distance"},
        "raycast_depth_mm": {"same_surface_rms": float(np.sqrt(np.mean(dz[same] ** 2)) * 1e3),
                             "p99": float(np.quantile(dz[same], 0.99) * 1e3), "rays": int(same.sum()),
                             "other_surface": int(np.sum(~same)), "hit_masks_differing": int(np.sum(gh != oh))},
        "ate_vs_ground_truth_mm": float(ate * 1e3),
        "oracle_seconds": round(time.perf_counter() - t0, 1),
    }


def host_frames(L, K, n, seed=0):
    import torch
    sc = L.SynthScene(seed=seed)
    out = []
    for k in range(n):
        d, c = sc.render(K, k)
        torch.cuda.synchronize()
        out.append((d.cpu().numpy(), c.cpu().numpy(), sc.pose(k)))
    return out


# the served configuration: Poisson arrivals at 4/s, up to 64 concurrent 640x480
# sessions at 30 fps for 300-3000 frames, voxel sizes of 5-10 mm, admission by
# device memory under a 150 GB budget
SERVE_VOXELS_MM = (5, 6, 7, 8, 9, 10)
SERVE_SCENES = 16        # distinct synthetic rooms the cameras film
SERVE_SWEEP = 120        # frames of a room's pre-rendered sweep, played back and forth


def serve_pool(v_mm: int) -> int:
    """Block pool of a session: a 4x4x3 m room's surfaces at v mm, with room to spare."""
    return 1 << 20 if v_mm < 6 else (1 << 19 if v_mm < 8 else 1 << 18)


def serve_config(L, v_mm: int):
    v = v_mm / 1000.0
    pool = serve_pool(v_mm)
    return L.default_config(voxel_size=v, truncation=min(max(3.0 * v, 0.02), 0.03), zmin_update=0.3,
                            zmax_update=4.0, zmin_raycast=0.3, zmax_raycast=4.0, num_buckets=2 * pool,
                            num_blocks=pool, voxel_layout=LAYOUTS[LAYOUT][0], num_levels=3,
                            max_iterations=[10, 5, 3, 3, 3], max_probe=256)


def serve_run(L, K, seconds: float, groups: int, stream, rate: float = 4.0, slots: int = 64,
              budget: int = 150 * (1 << 30), seed: int = 12345):
    """Config-5 serving, continuous batching (libfusion_gb300/serving.py), in
    real time for `seconds`: requests arrive as a Poisson process of `rate`/s,
    each a camera streaming 640x480 frames at 30 fps for 300-3000 frames with
    a voxel size of 5-10 mm; a request is admitted when one of `slots` batch
    slots is free and its session arena fits the device budget
    (gbf_session_bytes), its camera then streams, every tick fuses one frame of
    each session whose next frame has arrived, and a session is evicted after
    its last frame (its arena cached for reuse).  The cameras film
    SERVE_SCENES synthetic rooms whose frames are rendered beforehand (a sweep
    of SERVE_SWEEP frames played forwards and backwards, a continuous camera
    motion), so no rendering competes with the server for the GPU."""
    import torch
    from libfusion_gb300.serving import ArenaCache, Request, Server
    rng = np.random.default_rng(seed)
    sweep = []
    for i in range(SERVE_SCENES):
        sc = L.SynthScene(seed=70000 + i)
        d = torch.empty((SERVE_SWEEP, H, W), dtype=torch.uint16, device="cuda")
        c = torch.empty((SERVE_SWEEP, H, W, 3), dtype=torch.uint8, device="cuda")
        for k in range(SERVE_SWEEP):
            sc.render_into(K, k, d[k].data_ptr(), c[k].data_ptr())
        sweep.append((d, c, sc.pose(0)))
        sc.close()
    torch.cuda.synchronize()

    def source(scene):
        d, c, _ = sweep[scene]
        period = 2 * SERVE_SWEEP - 2

        def frame(k):
            j = k % period
            j = j if j < SERVE_SWEEP else period - j
            return d[j].data_ptr(), c[j].data_ptr()
        return frame

    cfgs = {v: serve_config(L, v) for v in SERVE_VOXELS_MM}
    nbytes = {v: L.session_bytes(cfgs[v], K) for v in SERVE_VOXELS_MM}
    reqs, t, sid = [], 0.0, 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        v = int(rng.choice(SERVE_VOXELS_MM))
        scene = sid % SERVE_SCENES
        reqs.append(Request(sid=sid, arrival=t, frames=int(rng.integers(300, 3001)), key=(v,), nbytes=nbytes[v],
                            pose0=sweep[scene][2], source=source(scene)))
        sid += 1
    batch = L.FusionBatch(slots)
    batch.reserve(K, cfgs[min(SERVE_VOXELS_MM)], slots)  # the largest session: the tick's shape never changes
    batch.set_groups(groups)
    cache = ArenaCache(budget, make=lambda key: L.System(K, cfgs[key[0]]), destroy=lambda s: s.close(),
                       reset=lambda s: s.reset(stream))
    srv = Server(batch, slots, cache, set_pose=lambda s, T: s.set_pose(T, stream), stream=stream)
    for r in reqs:
        srv.submit(r)
    srv.run(seconds)
    rep = srv.report()
    rep["graphs_captured"] = batch.captures()  # 2 (one per tick parity): admissions never re-capture
    for slot, x in enumerate(srv.live):
        if x is not None:
            batch.set(slot, None)
            x.session.close()
    batch.close()
    cache.close()
    del sweep
    torch.cuda.synchronize()
    rep["model"] = (f"Poisson arrivals {rate}/s for {seconds:.0f} s of wall time, up to {slots} concurrent 640x480 "
                    f"sessions, cameras at 30 fps for 300-3000 frames, voxel {SERVE_VOXELS_MM[0]}-"
                    f"{SERVE_VOXELS_MM[-1]} mm (block pools of 2^18-2^20), admitted when a slot is free and the "
                    f"session's arena fits the {budget / (1 << 30):.0f} GiB budget, evicted after the last frame; "
                    "latency from a frame's capture (admission + index / 30 fps) to its pose on the host")
    rep["session_bytes_by_voxel_mm"] = {str(v): nbytes[v] for v in SERVE_VOXELS_MM}
    rep["graph_shape_reserved"] = f"{slots} slots of the largest session (pool {serve_pool(min(SERVE_VOXELS_MM))})"
    return rep


# ----------------------------------------------------------------------------- arms

def run_reference(args):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import libfusion_gb300 as L
    from libfusion_gb300 import build as B
    B.build()
    K = intrinsics(L)
    t, n_mix, threads = cpu_mix(L, K, args.warmup, args.steps)
    total = sum(t)
    v = args.steps / total
    lat = sorted(x * 1e3 for x in t)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(workload_config(args.sessions),
                       sample=f"the CPU path (FP32 oracle restating the reference kernels, {threads} host threads) "
                              f"processes frames one at a time: a step is one 640x480 frame, round-robin over "
                              f"{n_mix} sessions with the served mix's voxel sizes",
                       inputs="seeded synthetic RGB-D (sphere-traced SDF room)"),
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": cpu_sample_text(args.steps, n_mix, threads)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import libfusion_gb300 as L
    from libfusion_gb300 import build as B
    if rank == 0:
        B.build()
    if world > 1:
        dist.barrier()
    K = intrinsics(L)
    S = args.sessions
    steps, warm = args.steps, args.warmup
    n_phase = min(steps, 8)
    nfr = warm + steps + n_phase
    # the tuner's search: 10 candidates, each timed for --tune-ticks ticks after
    # one untimed tick, plus the two ticks in flight at every switch
    n_tune = 0 if args.no_autotune else 10 * (args.tune_ticks + 3) + 10

    # admission: every session's device bytes under a 150 GB budget per GPU
    budget = 150 * (1 << 30)
    need = sum(L.session_bytes(session_config(L, i), K) for i in range(S))
    if need > budget:
        raise SystemExit(f"{S} sessions need {need/2**30:.1f} GiB > 150 GiB budget")

    frames, poses0 = render_frames(L, K, replica_seeds(rank, S), max(nfr, n_tune))
    tuned = None if args.no_autotune else tune_launch_shape(L, K, S, frames, poses0, args.tune_ticks)
    unsettled = None
    if tuned is not None and tuned["state"] != "settled":  # fall back to the fixed shape
        unsettled = f"the launch-shape search did not settle in {tuned['ticks']} ticks; --groups {args.groups} used"
        tuned = None
    sessions = []
    for i in range(S):
        s = L.System(K, session_config(L, i))
        s.set_pose(poses0[i])
        sessions.append(s)
    batch = L.FusionBatch(S)
    for i, s in enumerate(sessions):
        batch.set(i, s)
    launch_shape(batch, args, tuned)
    active = [True] * S
    use_graph = not args.no_graph
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    def tick(k, graph=None):
        for i in range(S):
            d, c = frames[i]
            batch.set_inputs(i, d[k].data_ptr(), c[k].data_ptr())
        batch.process(active, use_graph=use_graph if graph is None else graph)

    for k in range(warm):
        tick(k)
    torch.cuda.synchronize()
    kpt = batch.kernels_per_tick()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    # the timed loops run with Python's garbage collector paused (as timeit does):
    # a collection pass in the host loop would stall the submission of ticks
    gc.collect()
    gc.disable()
    try:
        with ClockSampler(local) as clocks:
            clocks.start()
            t_wall = time.perf_counter()
            for k in range(steps):
                ev[k][0].record(stream)
                tick(warm + k)
                ev[k][1].record(stream)
            torch.cuda.synchronize()
            t_wall = time.perf_counter() - t_wall
            clocks.stop()
    finally:
        gc.enable()
    if world > 1:
        dist.barrier()
    tick_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = ev[0][0].elapsed_time(ev[-1][1])
    total_ms = max_over_ranks(total_ms, dist, "cuda")
    value = aggregate_rate(S, world, steps, total_ms)
    lat = sorted(tick_ms)
    p = lambda q: lat[min(len(lat) - 1, int(math.ceil(q * len(lat))) - 1)]

    # ---- per-phase kernel times: the same ticks launched directly on the stream
    # with CUDA events at the phase boundaries (a second timed region, no graph)
    batch.flush()  # the staggered group's owed second halves, before the counters are read
    pi0, ib0 = work_counters(sessions)
    batch.set_timing(True)
    for k in range(n_phase):
        tick(warm + steps + k, graph=False)
    phases = batch.phase_ms()
    pi1, ib1 = work_counters(sessions)
    batch.set_timing(False)
    torch.cuda.synchronize()

    status = [s.stats() for s in sessions]
    bad = [i for i, st in enumerate(status) if st.status & ~L.FLAG_TRACK_FAILED]
    failed = sum(1 for st in status if st.status & L.FLAG_TRACK_FAILED)


    # roofline of the dominant kernel phase: algorithmic bytes of the work the
    # phase's launches did, over their CUDA-event time (the mean launch)
    dom = max(("integrate", "track"), key=lambda n: phases[n])
    peak, peak_kind = measured_peaks()
    bytes_step = kernel_bytes(L, sessions, dom, K, pi1 - pi0, ib1 - ib0, phases["ticks"])
    n_launch = 1 if dom == "integrate" else sum(sessions[0].cfg.max_iterations[l] for l in range(3))
    achieved = bytes_step / (phases[dom] / 1e3) / 1e9
    pix_iter = (pi1 - pi0) / phases["ticks"]
    traffic = REDUCE_DRAM_BYTES_PER_PIXEL_ITER * pix_iter / n_launch if dom == "track" else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": "integrate_kernel" if dom == "integrate" else "gn_reduce_kernel",
                "launches_per_step": n_launch, "peak_source": f"{peak_kind} hbm_gbs",
                "algorithmic_bytes_per_launch": bytes_step / n_launch, "algorithmic_bytes_per_step": bytes_step,
                "traffic_basis": "ncu dram__bytes_read.sum + dram__bytes_write.sum of a level-0 launch at 4 "
                                 "sessions: 85.9 B per pixel-iteration, "
                                 "times this run's pixel-iterations per launch" if traffic is not None else None,
                "work_per_step": {"pixel_iterations": pix_iter, "integrated_blocks": (ib1 - ib0) / phases["ticks"]},
                "timing": f"CUDA events around the phase over {phases['ticks']} ticks on the launching stream",
                "why_this_kernel": "the raycast (39% of launch time against the reduction's 27% and its step's "
                                   "4% in an ncu launch list of the 64-session tick) is bound by instruction "
                                   "issue, not HBM "
                                   "(74% issue active, DRAM 3.8% in its ncu capture at 4 sessions), so its "
                                   "figures are under 'march'; the HBM roofline is given for the memory-bound phase",
                "march_ms_per_step": phases["march"]}
    px_step = sum(s.K.width * s.K.height for s in sessions)
    march_bytes = RAYCAST_DRAM_BYTES_PER_PIXEL * px_step
    roofline["march"] = {
        "kernel": "raycast_kernel", "bound": "issue", "ms_per_step": phases["march"],
        "issue_active_ncu": RAYCAST_ISSUE_ACTIVE,
        "dram_bytes_per_step_est": march_bytes,
        "dram_gbs_est": march_bytes / (phases["march"] / 1e3) / 1e9,
        "dram_frac_est": march_bytes / (phases["march"] / 1e3) / 1e9 / peak,
        "basis": "DRAM bytes per pixel from one ncu capture of the raycast at 4 sessions, times this "
                 "run's raycast pixels, over the phase's CUDA-event time; issue activity from the same capture"}

    # ---- end to end through the public API with host buffers (pinned): the same
    # frames as the timed ticks, after the same warm-up frames (untimed).  Each
    # tick's frames are staged into the batch's double-buffered inputs on a copy
    # stream (overlapping the previous tick) and every tick's per-slot results
    # (poses, tracking flags) are read back one tick behind.
    n_e2e = min(steps, 30)  # about 0.35 s of host wall clock at 64 sessions
    # the timed batch is done: its report first, then its sessions' memory goes
    # back before the end-to-end leg builds its own (at 128 sessions both sets
    # would not fit together)
    shape = shape_report(batch, tuned, args, unsettled)
    batch.close()
    for s in sessions:
        s.close()
    del sessions
    torch.cuda.synchronize()
    host = [(frames[i][0][:warm + n_e2e].cpu().pin_memory(), frames[i][1][:warm + n_e2e].cpu().pin_memory())
            for i in range(S)]
    e2e_sessions = [L.System(K, session_config(L, i)) for i in range(S)]
    for i, s in enumerate(e2e_sessions):
        s.set_pose(poses0[i])
    eb = L.FusionBatch(S)
    for i, s in enumerate(e2e_sessions):
        eb.set(i, s)
    launch_shape(eb, args, tuned)
    copy = torch.cuda.Stream()
    got = []

    def e2e_tick(k, first):
        for i in range(S):
            eb.stage(i, host[i][0][k], host[i][1][k], stream=copy)
        eb.process(active, use_graph=use_graph, stream=stream)
        if k > first:
            got.append(eb.results(back=1))  # the previous tick's poses on the host

    for k in range(warm):
        e2e_tick(k, 0)
    eb.results(back=0)
    torch.cuda.synchronize()
    got.clear()
    gc.collect()
    gc.disable()
    try:
        with ClockSampler(local) as e2e_clocks:
            e2e_clocks.start()
            t_e2e = time.perf_counter()
            for k in range(warm, warm + n_e2e):
                e2e_tick(k, warm)
            got.append(eb.results(back=0))
            t_e2e = time.perf_counter() - t_e2e
            e2e_clocks.stop()
    finally:
        gc.enable()
    assert len(got) == n_e2e
    e2e = {"value": S * world * n_e2e / t_e2e, "unit": UNIT, "h2d_bytes_per_step": S * W * H * 5,
           "d2h_bytes_per_step": S * 144, "steps": n_e2e, "clocks": e2e_clocks.summary(),
           "note": f"frames {warm}..{warm + n_e2e - 1} of every session after {warm} untimed warm-up frames; "
                   "host wall clock from the first staging copy to the last tick's results on the host"}
    eb.close()
    del e2e_sessions
    e2e_pose = {}  # (session, frames processed) -> pose after the served tick
    for poses_k, _, _, fidx in got:
        for i in range(S):
            e2e_pose[(i, int(fidx[i]))] = poses_k[i]

    # ---- plain path: one session at a time, one frame at a time, pose read back per frame
    plain_sessions = [L.System(K, session_config(L, i)) for i in range(min(S, 8))]
    for i, s in enumerate(plain_sessions):
        s.set_pose(poses0[i])
    per = max(1, min(args.plain_frames or steps, nfr - warm))
    plat = []
    plain_pose = {}
    for k in range(warm):  # the served sessions' warm-up frames, untimed
        for i, s in enumerate(plain_sessions):
            d, c = frames[i]
            s.process_images(d[k], c[k])
    torch.cuda.synchronize()
    tp = time.perf_counter()
    for k in range(per):
        for i, s in enumerate(plain_sessions):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            d, c = frames[i]
            s.process_images(d[warm + k], c[warm + k])
            b.record(stream)
            plain_pose[(i, warm + k + 1)] = s.get_pose()
            plat.append(a.elapsed_time(b))
    torch.cuda.synchronize()
    tp = time.perf_counter() - tp
    nplain_done = per * len(plain_sessions)
    plain_fps = nplain_done / tp
    plat.sort()
    plain = {"value": plain_fps, "unit": UNIT, "frames": nplain_done, "sessions": len(plain_sessions),
             "p50_ms": plat[len(plat) // 2], "p99_ms": plat[min(len(plat) - 1, int(0.99 * len(plat)))],
             "path": "gbf_process_frame per session, direct launches, pose read back per frame",
             "frame_indices": f"{warm}..{warm + per - 1} after {warm} untimed warm-up frames"}
    del plain_sessions
    # the same sessions' poses after the same frames, served (in the batch of S) and plain
    both = sorted(set(e2e_pose) & set(plain_pose))
    diffs = [float(np.abs(e2e_pose[k] - plain_pose[k]).max()) for k in both]
    same_results = {"compared": len(both), "max_abs_pose_diff": max(diffs) if diffs else None,
                    "bit_identical": bool(diffs) and all(np.array_equal(e2e_pose[k], plain_pose[k]) for k in both),
                    "basis": "camera->world pose of each of the first sessions after the same frame, from the "
                             "pipelined batch of all sessions (e2e leg) and from the plain one-session path"}

    # config-5 serving in real time, every other leg's sessions released
    torch.cuda.synchronize()
    serving = serve_run(L, K, args.serve_seconds, shape.get("groups") or args.groups, stream) \
        if args.serve_seconds > 0 else None

    prec_frames = host_frames(L, K, args.precision_frames, seed=replica_seeds(rank, S)[0]) \
        if args.precision_frames > 0 and rank == 0 else None
    prec_gpu = precision_gpu(L, K, session_config(L, 0), prec_frames) if prec_frames else None

    if rank != 0:
        return
    cpu = cpu_baseline(L, K, args.cpu_seconds, warm)
    # the CPU leg also runs the FP64 oracle as the checker of the GPU's results
    precision = precision_check(L, K, session_config(L, 0), prec_frames, prec_gpu, os.cpu_count() or 1) \
        if prec_gpu else None
    clk = clocks.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": warm,
        "ms_per_step": total_ms / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": dict(workload_config(S), graph=use_graph, launch_shape=shape,
                       l2="working set per tick (voxel pools, 64 x 640x480 pyramids) far above the 129 MB L2; no flush",
                       inputs="seeded synthetic RGB-D (sphere-traced SDF room, depth noise model) resident in HBM"),
        "latency_ms": {"p50": p(0.50), "p95": p(0.95), "p99": p(0.99), "basis": "tick duration (every session's "
                       "frame arrives at the tick start)"},
        "plain": plain, "served_vs_plain": value / plain_fps, "served_vs_plain_results": same_results,
        "serving": serving,
        "phases_ms": {k: v for k, v in phases.items()},
        "precision": precision,
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": kpt * steps,
        "clocks": clk, "tracking_failures": failed, "sessions_with_errors": bad,
        "wall_s": t_wall,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# the mixed workload: resolutions and voxel sizes cycled over the sessions
MIXED_SIZES = ((320, 240), (640, 480), (1280, 720))
MIXED_VOXELS = (0.004, 0.008, 0.016)


def mixed_room(i):
    """Session i's synthetic room, from 3x3x2.5 m to 10x10x3 m (a golden-ratio
    sequence over the sessions), the camera circling at 3/8 of the side."""
    u = (i * 0.6180339887) % 1.0
    side = 3.0 + 7.0 * u
    return dict(seed=1000 + i, room=(side, side, 2.5 + 0.5 * u), radius=min(max(0.375 * side, 1.1), 3.5))


def mixed_session(L, i):
    """(intrinsics, config) of session i of the mixed workload."""
    w, h = MIXED_SIZES[i % len(MIXED_SIZES)]
    v = MIXED_VOXELS[(i // len(MIXED_SIZES)) % len(MIXED_VOXELS)]
    s = w / 640.0
    K = L.IntrinsicMatrix(w, h, 525.0 * s, 525.0 * s, (w - 1) / 2.0, (h - 1) / 2.0)
    cfg = L.default_config(voxel_size=v, truncation=min(max(3.0 * v, 0.02), 0.05), zmin_update=0.3,
                           zmax_update=4.0, zmin_raycast=0.3, zmax_raycast=4.0, num_buckets=1 << 19,
                           num_blocks=1 << 18, voxel_layout=LAYOUTS[LAYOUT][0], num_levels=3,
                           max_iterations=[10, 5, 3, 3, 3], max_probe=256)
    return K, cfg


def run_mixed(args):
    """Sessions of 320x240, 640x480 and 1280x720 with 4, 8 and 16 mm voxels in
    one batch (every launch sized for the largest), against the same sessions
    one at a time.  Frames per second count frames of every size alike."""
    import torch
    import libfusion_gb300 as L
    from libfusion_gb300 import build as B
    B.build()
    S, steps, warm = args.sessions, args.steps, args.warmup
    spec = [mixed_session(L, i) for i in range(S)]
    n_tune = 0 if args.no_autotune else 10 * (args.tune_ticks + 3) + 10
    nfr = max(warm + steps, n_tune)
    frames, poses0 = [], []
    for i, (K, _) in enumerate(spec):
        sc = L.SynthScene(**mixed_room(i))
        d = torch.empty((nfr, K.height, K.width), dtype=torch.uint16, device="cuda")
        c = torch.empty((nfr, K.height, K.width, 3), dtype=torch.uint8, device="cuda")
        for k in range(nfr):
            sc.render_into(K, k, d[k].data_ptr(), c[k].data_ptr())
        frames.append((d, c))
        poses0.append(sc.pose(0))
        sc.close()
    torch.cuda.synchronize()
    make = lambda i: L.System(*spec[i])
    tuned = None if args.no_autotune else tune_launch_shape(L, None, S, frames, poses0, args.tune_ticks, make)
    if tuned is not None and tuned["state"] != "settled":
        tuned = None
    sessions = [make(i) for i in range(S)]
    for s, p in zip(sessions, poses0):
        s.set_pose(p)
    batch = L.FusionBatch(S)
    for i, s in enumerate(sessions):
        batch.set(i, s)
    launch_shape(batch, args, tuned)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    active = [True] * S

    def tick(k):
        for i in range(S):
            batch.set_inputs(i, frames[i][0][k].data_ptr(), frames[i][1][k].data_ptr())
        batch.process(active)

    for k in range(warm):
        tick(k)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with ClockSampler(torch.cuda.current_device()) as clocks:
        clocks.start()
        for k in range(steps):
            ev[k][0].record(stream)
            tick(warm + k)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        clocks.stop()
    tick_ms = sorted(a.elapsed_time(b) for a, b in ev)
    total_ms = ev[0][0].elapsed_time(ev[-1][1])
    value = S * steps / (total_ms / 1e3)
    shape = shape_report(batch, tuned, args)
    batch.close()
    del sessions
    # the same sessions one at a time, one frame at a time, pose read back per frame
    plain_s = [make(i) for i in range(S)]
    for s, p in zip(plain_s, poses0):
        s.set_pose(p)
    for k in range(warm):
        for i, s in enumerate(plain_s):
            s.process_images(frames[i][0][k], frames[i][1][k])
    torch.cuda.synchronize()
    per = min(steps, args.plain_frames or steps)
    t0 = time.perf_counter()
    for k in range(per):
        for i, s in enumerate(plain_s):
            s.process_images(frames[i][0][warm + k], frames[i][1][warm + k])
            s.get_pose()
    torch.cuda.synchronize()
    plain = S * per / (time.perf_counter() - t0)
    p = lambda q: tick_ms[min(len(tick_ms) - 1, int(math.ceil(q * len(tick_ms))) - 1)]
    print(json.dumps({
        "metric": METRIC, "workload": "mixed", "value": value, "unit": UNIT, "n_gpus": 1, "steps": steps,
        "warmup": warm, "ms_per_step": total_ms / steps, "higher_is_better": True,
        "config": {"workload": f"{S} sessions per tick: resolutions {['%dx%d' % s for s in MIXED_SIZES]} and voxels "
                               f"{[f'{v * 1000:.0f} mm' for v in MIXED_VOXELS]} cycled over the sessions, "
                               f"rooms from 3x3x2.5 to 10x10x3 m",
                   "voxel_layout": LAYOUTS[LAYOUT][1], "launch_shape": shape},
        "latency_ms": {"p50": p(0.5), "p99": p(0.99)}, "clocks": clocks.summary(),
        "plain": {"value": plain, "unit": UNIT, "frames": S * per}, "served_vs_plain": value / plain,
    }), flush=True)


# the large-map configuration: 8x8x3 m room, 20 spheres, 12 boxes, figure-eight at 0.5 m/s and 30 fps
SCALE_SCENE = dict(trajectory=1, room=(8, 8, 3), n_spheres=20, n_boxes=12, radius=2.5, speed=0.5, fps=30, seed=2)
SCALE_MESH_EVERY = 100


def scale_config(L):
    return L.default_config(voxel_size=0.005, truncation=0.02, zmin_update=0.3, zmax_update=4.0, zmin_raycast=0.3,
                            zmax_raycast=4.0, num_buckets=1 << 21, num_blocks=1 << 20,
                            voxel_layout=LAYOUTS[LAYOUT][0], num_levels=3, max_iterations=[10, 5, 3, 3, 3],
                            w_rgb=0.1, max_probe=1024, motion_prior=1)


def phase_bytes(phase: str, P: int, levels: int, s_v: int, d: dict) -> float | None:
    """Algorithmic bytes of one frame's phase (the kernels' own reads and
    writes, each byte once): d holds the frame's work counters."""
    Pl = [P >> (2 * l) for l in range(levels)]
    if phase == "ingest":   # u16 depth + rgb8 in; depth, intensity out; pyramids; per level vmap, nmap, gradients
        return 5 * P + 8 * P + sum(8 * (Pl[l - 1] + Pl[l]) for l in range(1, levels)) + sum(48 * x for x in Pl)
    if phase == "track":    # reference vmap+nmap+I, current vmap+nmap+I+gradients per pixel-iteration
        return 80.0 * d["pixel_iterations"]
    if phase == "alloc_visible":  # depth in; per allocated block its record; the visible list out (lower bound)
        return 4 * P + 20.0 * d["allocated_blocks"] + 4.0 * d["visible_blocks"]
    if phase == "integrate":  # voxel read-modify-write of every visible block + depth, normal, colour per pixel
        return 2.0 * s_v * 512 * d["integrated_blocks"] + 23 * P
    if phase == "zrange":
        return 20.0 * d["visible_blocks"] + 8 * (P // 64)
    if phase == "post":     # vertex maps halved per level, normals recomputed per level
        return sum(16 * (Pl[l - 1] + Pl[l]) for l in range(1, levels)) + sum(32 * x for x in Pl)
    return None             # the march: bound by instruction issue, its voxel fetches depend on the rays


def run_scale(args):
    """The large-map configuration as a plain single session: 640x480 frames
    along the figure-eight, 5 mm voxels, 2 cm truncation, 2^21 hash slots and a
    2^20-block pool, photometric weight 0.1, marching cubes every 100 frames.
    Pass 1 times every frame (gbf_process_frame, CUDA events on the stream) and
    every mesh extraction; pass 2 runs the same frames as a batch of one with
    CUDA events at the phase boundaries, for each phase's time and HBM rate."""
    import torch
    import libfusion_gb300 as L
    from libfusion_gb300 import build as B
    B.build()
    K = intrinsics(L)
    cfg = scale_config(L)
    n = args.scale_frames
    P = W * H
    s_v = 12 if cfg.voxel_layout == L.VOXEL_REF else 8
    sc = L.SynthScene(**SCALE_SCENE)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    bufs = [(torch.empty((H, W), dtype=torch.uint16, device="cuda"),
             torch.empty((H, W, 3), dtype=torch.uint8, device="cuda")) for _ in range(2)]
    max_tris = 1 << 26  # 2.4 GB of vertices: the 2000-frame map meshes to over 2^25 triangles
    vtx = torch.empty((max_tris, 3, 3), dtype=torch.float32, device="cuda")
    truth = [sc.pose(k) for k in range(n)]

    def render(k):
        d, c = bufs[k & 1]
        sc.render_into(K, k, d.data_ptr(), c.data_ptr(), stream=stream)
        return d, c

    # pass 1: the plain path, frame by frame
    s = L.System(K, cfg)
    s.set_pose(truth[0])
    frame_ms, mesh_ms, tris, poses, failed = [], [], [], [], 0
    for k in range(args.warmup):  # untimed warm-up on a throwaway session
        w = L.System(K, cfg)
        w.set_pose(truth[0])
        w.process_images(*render(k), stream=stream)
        w.close()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clocks:
        clocks.start()
        for k in range(n):
            d, c = render(k)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            s.process_images(d, c, stream=stream)
            b.record(stream)
            frame_ms.append((a, b))
            if (k + 1) % SCALE_MESH_EVERY == 0:
                a2, b2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a2.record(stream)
                tris.append(s.fetch_mesh_vertex_only(vtx, stream=stream))
                b2.record(stream)
                mesh_ms.append((a2, b2))
            poses.append(s.get_camera_pose(stream=stream))
            failed += 0 if s.stats(stream=stream).track.success else 1
        torch.cuda.synchronize()
        clocks.stop()
    frame_ms = [a.elapsed_time(b) for a, b in frame_ms]
    mesh_ms = [a.elapsed_time(b) for a, b in mesh_ms]
    st = s.stats()
    # block garbage collection on the full map: the blocks farther than 3 m from
    # the last camera pruned on the stream (gbf_map_prune_async), timed by events
    a3, b3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a3.record(stream)
    s.prune_async(center=poses[-1][:3, 3], radius=3.0, stream=stream)
    b3.record(stream)
    torch.cuda.synchronize()
    collection = {"kind": "gbf_map_prune_async, blocks farther than 3 m from the last camera",
                  "blocks_before": st.allocated_blocks, "blocks_after": s.stats().allocated_blocks,
                  "ms": a3.elapsed_time(b3)}
    # evict to host and resume: the pruned session snapshotted into pinned host
    # memory and restored into a fresh session (host wall clock, both synchronise)
    nb = s.snapshot_bytes()
    host = torch.empty(nb, dtype=torch.uint8, pin_memory=True).numpy()
    t0 = time.perf_counter()
    s.snapshot(out=host)
    t1 = time.perf_counter()
    r = L.System(K, cfg)
    t2 = time.perf_counter()
    r.restore(host)
    t3 = time.perf_counter()
    snapshot = {"blocks": s.stats().allocated_blocks, "bytes": nb, "snapshot_ms": (t1 - t0) * 1e3,
                "restore_ms": (t3 - t2) * 1e3, "snapshot_gbs": nb / (t1 - t0) / 1e9,
                "restore_gbs": nb / (t3 - t2) / 1e9, "host_memory": "pinned",
                "same_pose": bool(np.array_equal(r.get_camera_pose(), s.get_camera_pose()))}
    r.close()
    del host
    s.close()
    total_ms = sum(frame_ms) + sum(mesh_ms)
    poses = np.array(poses)
    tr = np.array(truth)
    err = np.linalg.norm(poses[:, :3, 3] - tr[:, :3, 3], axis=1)

    # pass 2: the same frames as a batch of one, phase by phase
    s2 = L.System(K, cfg)
    s2.set_pose(truth[0])
    b1 = L.FusionBatch(1)
    b1.set(0, s2)
    b1.set_groups(1)
    b1.set_timing(True)
    acc = {k: 0.0 for k in L.FusionBatch.PHASES}
    work = {"pixel_iterations": 0, "integrated_blocks": 0, "allocated_blocks": 0, "visible_blocks": 0}
    byt = {k: 0.0 for k in L.FusionBatch.PHASES}
    prev = s2.stats()
    for k in range(n):
        d, c = render(k)
        b1.set_inputs(0, d.data_ptr(), c.data_ptr())
        b1.process([True], use_graph=False, stream=stream)
        cur = s2.stats(stream=stream)
        dd = {"pixel_iterations": cur.pixel_iterations - prev.pixel_iterations,
              "integrated_blocks": cur.integrated_blocks - prev.integrated_blocks,
              "allocated_blocks": cur.allocated_blocks, "visible_blocks": cur.visible_blocks}
        for ph in byt:
            x = phase_bytes(ph, P, cfg.num_levels, s_v, dd)
            if x is not None:
                byt[ph] += x
        for key in work:
            work[key] += dd[key]
        prev = cur
    ph = b1.phase_ms()
    b1.close()
    s2.close()
    peak, peak_kind = measured_peaks()
    phases = {}
    for name in L.FusionBatch.PHASES:
        ms = ph[name]
        entry = {"ms_per_frame": ms}
        if byt[name] > 0:
            gbs = byt[name] / n / (ms / 1e3) / 1e9
            entry.update({"algorithmic_bytes_per_frame": byt[name] / n, "gbs": gbs, "hbm_frac": gbs / peak})
        else:
            entry["bound"] = "instruction issue (voxel fetches depend on the rays; no algorithmic byte count)"
        phases[name] = entry
    mesh_bytes = [s_v * 512.0 * st.allocated_blocks + 36.0 * t for t in tris]
    phases["mesh"] = {"ms_per_extraction": statistics.mean(mesh_ms) if mesh_ms else None,
                      "extractions": len(mesh_ms), "triangles_last": tris[-1] if tris else 0,
                      "gbs": (statistics.mean(mesh_bytes) / (statistics.mean(mesh_ms) / 1e3) / 1e9) if mesh_ms else None}
    if mesh_ms:
        phases["mesh"]["hbm_frac"] = phases["mesh"]["gbs"] / peak
    lat = sorted(frame_ms)
    q = lambda f: lat[min(len(lat) - 1, int(math.ceil(f * len(lat))) - 1)]
    print(json.dumps({
        "metric": METRIC, "workload": "scale", "value": n / (total_ms / 1e3), "unit": UNIT, "n_gpus": 1,
        "steps": n, "warmup": args.warmup, "ms_per_step": total_ms / n, "higher_is_better": True,
        "config": {"workload": f"plain single session at scale: {n} frames of 640x480 along a figure-eight "
                               f"(0.5 m/s, 30 fps) in an 8x8x3 m room with 20 spheres and 12 boxes",
                   "voxel_m": cfg.voxel_size, "truncation_m": cfg.truncation, "hash_slots": 1 << 21,
                   "pool_blocks": 1 << 20, "voxel_layout": LAYOUTS[LAYOUT][1], "w_icp": cfg.w_icp,
                   "w_rgb": cfg.w_rgb, "pyramid": "3 levels 10/5/3", "mesh_every": SCALE_MESH_EVERY,
                   "motion_prior": "constant velocity: each frame's tracking starts from the last frame's motion "
                                   "(at 16.7 mm per frame the reference's no-motion start is beyond its 1 cm ICP "
                                   "gate; over 2000 frames it lost the camera from frame 1274 in a measured run)"},
        "latency_ms": {"p50": q(0.5), "p99": q(0.99), "basis": "CUDA events around each frame's gbf_process_frame"},
        "mesh_ms_total": sum(mesh_ms),
        "phases": phases, "peak_gbs": peak, "peak_source": f"{peak_kind} hbm_gbs",
        "work_per_frame": {k: v / n for k, v in work.items() if k in ("pixel_iterations", "integrated_blocks")},
        "map": {"allocated_blocks": st.allocated_blocks, "status": st.status},
        "collection": collection,
        "snapshot": snapshot,
        "tracking": {"failed_frames": failed, "ate_vs_ground_truth_mm": float(np.sqrt(np.mean(err ** 2)) * 1e3),
                     "max_error_mm": float(err.max() * 1e3)},
        "clocks": clocks.summary(),
    }), flush=True)


def precision_config(L, layout: int):
    """Config 1's map: 1 cm voxels, 3 cm truncation, 2^18 slots, 2^17-block pool."""
    return L.default_config(voxel_size=0.01, truncation=0.03, zmin_update=0.3, zmax_update=4.0, zmin_raycast=0.3,
                            zmax_raycast=4.0, num_buckets=1 << 18, num_blocks=1 << 17, voxel_layout=layout,
                            num_levels=3, max_iterations=[10, 5, 3, 3, 3], max_probe=256)


def trajectory_errors(poses, truth) -> dict:
    """ATE (RMS of the camera position error) and RPE (RMS of the frame-to-frame
    relative pose error: translation, rotation angle) against `truth`."""
    P, T = np.asarray(poses), np.asarray(truth)
    ate = np.sqrt(np.mean(np.sum((P[:, :3, 3] - T[:, :3, 3]) ** 2, axis=1)))
    dt, dr = [], []
    for k in range(1, len(P)):
        e = np.linalg.inv(np.linalg.inv(T[k - 1]) @ T[k]) @ (np.linalg.inv(P[k - 1]) @ P[k])
        dt.append(np.linalg.norm(e[:3, 3]))
        dr.append(np.degrees(np.arccos(np.clip((np.trace(e[:3, :3]) - 1) / 2, -1, 1))))
    return {"ate_mm": float(ate * 1e3), "rpe_mm": float(np.sqrt(np.mean(np.square(dt))) * 1e3),
            "rpe_deg": float(np.sqrt(np.mean(np.square(dr)))), "max_error_mm":
            float(np.max(np.linalg.norm(P[:, :3, 3] - T[:, :3, 3], axis=1)) * 1e3)}


def run_precision(args):
    """Config 3: the precision form of config 1 (the 4x4x3 m room, circle
    path, 640x480), every voxel layout on the GPU against the FP64 oracle (the
    checker, on the host cores).  The tracking loop runs --precision-track
    frames (2000) on the GPU in each layout and in the FP64 oracle: trajectory
    error against the ground truth (ATE, RPE), pose drift against the FP64
    loop, tracking failures.  The map: --precision-frames frames fused at the
    ground-truth poses with the normal-weighted update, then TSDF error, raycast
    depth and the mesh's symmetric Chamfer distance against the FP64 map."""
    import torch
    import libfusion_gb300 as L
    from libfusion_gb300 import build as B
    B.build()
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    O.build()
    from scipy.spatial import cKDTree
    K = intrinsics(L)
    n_track, n_map = args.precision_track, max(args.precision_frames, 2)
    sc = L.SynthScene(seed=0)
    truth = [sc.pose(k) for k in range(n_track)]
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    threads = os.cpu_count() or 1
    out = {"layouts": {}}
    # ---- tracking loop, 2000 frames: GPU per layout, then the FP64 oracle on the same frames
    fp64 = O.OracleSystem(O.config_from(precision_config(L, 0), threads=threads), O.intrinsics_from(K), "f64")
    fp64.set_pose(truth[0])
    gpu = {name: L.System(K, precision_config(L, LAYOUTS[name][0])) for name in LAYOUTS}
    for s in gpu.values():
        s.set_pose(truth[0])
    gp = {name: [] for name in LAYOUTS}
    gfail = {name: 0 for name in LAYOUTS}
    op, ofail = [], 0
    t0 = time.perf_counter()
    t_oracle = 0.0
    for k in range(n_track):
        d, c = sc.render(K, k)
        for name, s in gpu.items():
            s.process_images(d, c)
            gp[name].append(s.get_camera_pose())
            gfail[name] += 0 if s.stats().track.success else 1
        dh, ch = d.cpu().numpy(), c.cpu().numpy()
        ta = time.perf_counter()
        fp64.process(dh, ch)
        t_oracle += time.perf_counter() - ta
        op.append(fp64.pose())
        ofail += 0 if fp64.last_result().success else 1
    op = np.array(op)
    out["fp64_oracle_tracking"] = dict(trajectory_errors(op, truth), failed_frames=ofail)
    for name in LAYOUTS:
        P = np.array(gp[name])
        out["layouts"][name] = {"storage": LAYOUTS[name][1],
                                "tracking": dict(trajectory_errors(P, truth), failed_frames=gfail[name],
                                                 drift_vs_fp64_max_mm=float(np.abs(P[:, :3, 3] - op[:, :3, 3]).max()
                                                                            * 1e3))}
        gpu[name].close()
    # ---- the map at the ground-truth poses (System's normal-weighted update)
    om = O.OracleMap(O.config_from(precision_config(L, 0), threads=threads), O.intrinsics_from(K), "f64")
    t = L.DenseTracking(K, precision_config(L, 0))
    maps = {name: L.DenseMapping(K, precision_config(L, LAYOUTS[name][0])) for name in LAYOUTS}
    for k in range(n_map):
        d, c = sc.render(K, k)
        dm = (d.float() * np.float32(0.001)).contiguous()
        t.set_current(dm, c)
        n = t.get_image(0, 1, 0)
        for m in maps.values():
            m.update(dm, c, truth[k], normal=n)
        om.fuse(dm.cpu().numpy(), c.cpu().numpy(), truth[k], nmap=n.cpu().numpy())
    T = truth[n_map - 1]
    ov = om.raycast(T)
    oc, osd, ow, _ = om.export()
    okey = {tuple(x): i for i, x in enumerate(oc.tolist())}
    ovtx, _ = om.mesh(0, 1 << 23)
    otree = cKDTree(ovtx.reshape(-1, 3).astype(np.float64))
    for name, m in maps.items():
        gcoord, gs, gw, _ = m.export()
        gi, oi = [], []
        for i, x in enumerate(gcoord.tolist()):
            j = okey.get(tuple(x))
            if j is not None:
                gi.append(i)
                oi.append(j)
        a, b, wa, wb = gs[gi], osd[oi], gw[gi], ow[oi]
        both = (wa > 0) & (wb > 0)
        err = np.abs(a[both] - b[both]).astype(np.float64)
        vm = torch.full((K.height, K.width, 4), float("nan"), dtype=torch.float32, device="cuda")
        m.raycast(vm, T)
        gv = vm.cpu().numpy()
        gh, oh = ~np.isnan(gv[..., 2]), ~np.isnan(ov[..., 2])
        dz = np.abs(gv[..., 2][gh & oh] - ov[..., 2][gh & oh]).astype(np.float64)
        same = dz < 0.03
        vtx = torch.zeros((len(ovtx) + (1 << 16), 3, 3), dtype=torch.float32, device="cuda")
        nt = m.fetch_mesh_vertex_only(vtx)
        gpts = vtx[:nt].cpu().numpy().reshape(-1, 3).astype(np.float64)
        d1, _ = otree.query(gpts)
        d2, _ = cKDTree(gpts).query(otree.data)
        out["layouts"][name]["map"] = {
            "tsdf_err_over_tau": {"p99.9": float(np.quantile(err, 0.999)), "mean": float(err.mean()),
                                  "max": float(err.max()), "voxels": int(both.sum())},
            "raycast_depth_mm": {"same_surface_rms": float(np.sqrt(np.mean(dz[same] ** 2)) * 1e3),
                                 "p99": float(np.quantile(dz[same], 0.99) * 1e3),
                                 "hit_masks_differing": int(np.sum(gh != oh)), "other_surface": int(np.sum(~same))},
            "mesh": {"triangles": int(nt), "fp64_triangles": int(len(ovtx)),
                     "chamfer_mm": float((d1.mean() + d2.mean()) / 2 * 1e3),
                     "hausdorff_mm": float(max(d1.max(), d2.max()) * 1e3)}}
        m.close()
    t.close()
    sc.close()
    print(json.dumps({
        "metric": METRIC, "workload": "precision", "unit": "mm / fraction of truncation",
        "config": {"workload": f"config-1 room (4x4x3 m, 6 spheres, 4 boxes, seed 0), circle path, 640x480: "
                               f"{n_track} tracked frames, map of {n_map} frames at the ground-truth poses",
                   "voxel_m": 0.01, "truncation_m": 0.03, "pyramid": "3 levels 10/5/3",
                   "reference": "FP64 oracle (double arithmetic, unquantised voxels), host cores"},
        "goals": {"pose_drift_mm": 1.0, "tsdf_p99.9_over_tau": 1e-3},
        **out, "oracle_seconds": round(t_oracle, 1), "wall_s": round(time.perf_counter() - t0, 1),
    }), flush=True)


def main():
    global LAYOUT
    args = parse()
    LAYOUT = args.layout
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "mixed":
        run_mixed(args)
    elif args.workload == "scale":
        run_scale(args)
    elif args.workload == "precision":
        run_precision(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
