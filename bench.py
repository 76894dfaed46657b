#!/usr/bin/env python
"""Benchmark of the GB300 SVO / brick ray caster (one JSON line on rank 0).

Default workload: the large plain SVO scene - a depth-11 (2048^3) seeded
value-noise terrain with 10k floating cubes, 1920x1080 primary rays plus one
hard-shadow ray per hit.  A step is one frame (primary + shadow rays) through
the persistent SVO kernel; `value` counts primary and shadow rays.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config cfg2]
  python bench.py --impl reference ...   (CPU reference arm)

Timing: each step is bracketed by CUDA events on the launching stream; an
L2 flush (write of a 256 MiB buffer, larger than the 129 MB L2) runs between
steps outside the events.  The K steps sit between barrier + synchronize.
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "yoxel-voxel_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Mrays/s on 1 GB300: plain vs persistent-batched, and fwd+bwd at stated error"
UNIT = "Mrays/s"
LIGHT = (np.array([0.3, 0.5, 0.8]) / np.linalg.norm([0.3, 0.5, 0.8])).astype(np.float32)


def camera():
    d = np.array([1.0, 0.7, 0.5])
    d /= np.linalg.norm(d)
    return (0.5 + 1.5 * d).astype(np.float32), (-d).astype(np.float32)


CONFIGS = {
    "cfg1": dict(kind="svo", scene=("spheres", dict(depth=8, n_spheres=200, rmin=4.0,
                                                    rmax=24.0, seed=1234)),
                 width=512, height=512, shadows=False,
                 workload="200 seeded spheres in 256^3 (SVO depth 8), 512x512 FP32 primary "
                          "rays, Lambert, one directional light"),
    "cfg2": dict(kind="svo", scene=("terrain", dict(depth=11, n_cubes=10000, cube_min=2,
                                                    cube_max=16, seed=1234)),
                 width=1920, height=1080, shadows=True,
                 workload="2048^3 (SVO depth 11) seeded 6-octave value-noise terrain + 10k "
                          "floating cubes, 1920x1080 FP32 primary rays + 1 hard-shadow ray "
                          "per hit"),
}


# --------------------------------------------------------------------- utils
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
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
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        top = max(sm)
        loaded = [s for s in sm if s >= 0.5 * top] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profile_traffic(name):
    """DRAM bytes per launch recorded from an ncu capture in profiles/<name>.md
    (line `traffic_bytes_per_launch: N`), or None."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    if not os.path.exists(p):
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", open(p).read())
    return float(m.group(1)) if m else None


def make_scene(cfg):
    import yoxel
    kind, kw = cfg["scene"]
    if kind == "spheres":
        return yoxel.SVOScene.spheres(**kw)
    return yoxel.SVOScene.terrain(**kw)


# --------------------------------------------------------------- CPU oracle
def cpu_svo(cfg, scene, width, height, threads, min_seconds=0.0, max_runs=1):
    """Times the FP32 oracle (restatement of the reference CPU renderer) on
    `threads` host threads.  Returns (Mrays/s, seconds per run, rays per run)."""
    from oracle import pyoracle
    pos, view = camera()
    runs, t_tot, rays = 0, 0.0, 0
    while runs < max_runs and (runs == 0 or t_tot < min_seconds):
        t0 = time.perf_counter()
        o = pyoracle.svo_render(scene.nodes_u32, scene.root, scene.attrs_u8, pos, view,
                                [0, 0, 1], 60.0, width, height, LIGHT,
                                shadows=cfg["shadows"], threads=threads)
        t_tot += time.perf_counter() - t0
        runs += 1
        hits = int((o["hit"] != 0xFFFFFFFF).sum())
        rays = width * height + (hits if cfg["shadows"] else 0)
    return rays * runs / t_tot / 1e6, t_tot / runs, rays


# ------------------------------------------------------------------- arms
def run_reference(args, cfg):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    scene = make_scene(cfg)
    # each step: the same view at half the resolution per axis (1/4 of rays)
    w, h = cfg["width"] // 2, cfg["height"] // 2
    for _ in range(args.warmup):
        cpu_svo(cfg, scene, w, h, threads)
    vals, secs = [], []
    rays = 0
    for _ in range(args.steps):
        v, s, rays = cpu_svo(cfg, scene, w, h, threads)
        vals.append(v)
        secs.append(s)
    value = rays * len(secs) / sum(secs) / 1e6
    sample = (f"{w}x{h} frame of the same scene and camera per step ({rays} rays incl. "
              f"shadow rays)")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT,
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * sum(secs) / len(secs), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": cfg["workload"], "config": args.config},
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "reference CPU renderer (cell/ppu_renderer.cpp) cannot be compiled here "
                "(missing cpp/ headers, Boost, libspe2); the FP32 C restatement of it is timed",
    }
    print(json.dumps(line), flush=True)


def run_svo(args, cfg):
    import torch
    import yoxel
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize()

    t_scene = time.perf_counter()
    scene = make_scene(cfg)
    t_scene = time.perf_counter() - t_scene
    pos, view = camera()
    w, h = cfg["width"], cfg["height"]
    npix = w * h
    r = yoxel.Renderer()
    r.SetScene(scene)
    r.SetViewPos(pos)
    r.SetViewDir(view)
    r.SetViewUp([0, 0, 1])
    r.SetResolution(w, h)
    r.SetFOV(60.0)
    r.SetLight(LIGHT, 0.15, 0.85, cfg["shadows"])
    dev_nodes, dev_bytes = r.device_scene_info()

    # algorithmic bytes of this frame: 40 B per node dereference (RecTrace
    # calls reaching cell/ppu_renderer.cpp:23) of primary and shadow rays,
    # + 8 B per pixel (RGBA8 + hit id) + 8 B leaf attribute per hit
    o = r.render_outputs()
    F = int(o["fetches"].to(torch.int64).sum())
    Fs = int(o["shadow_fetches"].to(torch.int64).sum())
    hits = int(o["stats"]["hits"])
    del o
    shadow_rays = hits if cfg["shadows"] else 0
    rays = npix + shadow_rays
    alg_bytes = 40 * F + 40 * Fs + 8 * npix + 8 * hits

    rgba = torch.empty((h, w), dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        flush.fill_(1)
        r.render_async(rgba=rgba, stream=stream)
    r.frame_stats()
    barrier()

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.4)
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(1)
        evs[i][0].record(stream)
        r.render_async(rgba=rgba, stream=stream)
        evs[i][1].record(stream)
    barrier()
    wall = time.perf_counter() - t0
    st = r.frame_stats()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    dev_s = sum(step_ms) / 1000.0

    # warm-L2 steady state (no flush between frames), for reference
    ew = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    ew[0].record(stream)
    for _ in range(args.steps):
        r.render_async(rgba=rgba, stream=stream)
    ew[1].record(stream)
    torch.cuda.synchronize()
    warm_ms = ew[0].elapsed_time(ew[1]) / args.steps
    clocks = sampler.stop()

    # end to end through the C ABI with a pinned host frame buffer
    host = torch.empty((h, w), dtype=torch.int32, pin_memory=True)
    import ctypes as C
    from yoxel import _lib as L
    for _ in range(2):
        L.check(L.lib.yv_render_frame(r.handle, C.c_void_p(host.data_ptr()), None,
                                      C.c_void_p(stream.cuda_stream)), "render_frame")
    barrier()
    te = time.perf_counter()
    for _ in range(args.steps):
        L.check(L.lib.yv_render_frame(r.handle, C.c_void_p(host.data_ptr()), None,
                                      C.c_void_p(stream.cuda_stream)), "render_frame")
    barrier()
    e2e_s = (time.perf_counter() - te) / args.steps

    # max over ranks
    tot = torch.tensor([dev_s, e2e_s], dtype=torch.float64, device="cuda")
    if pg is not None:
        pg.all_reduce(tot, op=pg.ReduceOp.MAX)
    dev_s, e2e_s = float(tot[0]), float(tot[1])
    if rank != 0:
        if pg is not None:
            pg.destroy_process_group()
        return

    mean_step_s = dev_s / args.steps
    value = rays * args.steps * ws / dev_s / 1e6
    peaks, peak_kind = measured_peaks()
    achieved = alg_bytes / mean_step_s / 1e9
    traffic = profile_traffic(f"svo_frame_{args.config}")
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(mean_step_s * 1000, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": cfg["workload"], "config": args.config,
                   "primary_rays_per_step": npix, "shadow_rays_per_step": shadow_rays,
                   "scene_nodes": dev_nodes, "scene_device_bytes": dev_bytes,
                   "l2": "flushed between steps (256 MiB write); scene > L2",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
        "primary_mrays_s": round(npix * args.steps * ws / dev_s / 1e6, 3),
        "warm_l2_mrays_s": round(rays * ws / (warm_ms / 1000) / 1e6, 3),
        "wall_s_timed_region": round(wall, 4),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2),
                     "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "traffic": traffic, "peak_source": peak_kind,
                     "algorithmic_bytes_per_step": alg_bytes,
                     "bytes_per_ray": round(alg_bytes / rays, 2),
                     "mean_node_fetches_primary": round(F / npix, 3),
                     "mean_node_fetches_shadow": round(Fs / max(1, shadow_rays), 3)},
        "e2e": {"value": round(rays / e2e_s / 1e6, 3), "unit": UNIT,
                "h2d_bytes_per_step": 40, "d2h_bytes_per_step": npix * 4 + 32,
                "path": "yv_render_frame (C ABI) into pinned host memory, synchronous"},
        "gpu_launches": int(st["launches"]) * args.steps,
        "clocks": clocks,
        "scene_build_s": round(t_scene, 2),
    }
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sw, sh = w // 4, h // 4
        v, s, rr = cpu_svo(cfg, scene, sw, sh, threads, min_seconds=10.0, max_runs=50)
        v1, s1, rr1 = cpu_svo(cfg, scene, w // 16, h // 16, 1)
        line["cpu_baseline"] = {
            "value": round(v, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{sw}x{sh} frame of the same scene and camera ({rr} rays incl. shadow "
                      f"rays), repeated for >=10 s; FP32 C restatement of cell/ppu_renderer.cpp",
            "single_thread_value": round(v1, 4)}
    print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="yoxel", choices=["yoxel", "reference"])
    ap.add_argument("--config", default="cfg2", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    cfg = CONFIGS[args.config]
    import importlib.util
    spec = importlib.util.spec_from_file_location("_gentry", os.path.join(ROOT, "__graft_entry__.py"))
    ge = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ge)
    ge.build()
    if args.impl == "reference":
        return run_reference(args, cfg)
    if cfg["kind"] == "svo":
        return run_svo(args, cfg)
    raise SystemExit(f"unknown workload kind {cfg['kind']}")


if __name__ == "__main__":
    main()
