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
import math
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
# brick pool formats (include/yv_c_api.h YV_PRECISION_*)
POOL_FORMATS = {0: "fp16 density + RGBA8 albedo", 1: "fp32 density + fp32 RGB albedo",
                2: "packed float4 (r, g, b, density)",
                3: "packed 8 B (fp16 density, RGB8)"}
SEED = 1234  # default seed of every synthetic workload
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
    "lod": dict(kind="svo", scene=("terrain", dict(depth=11, n_cubes=10000, cube_min=2,
                                                   cube_max=16, seed=1234)),
                width=1920, height=1080, shadows=True, detail=4.0,
                workload="cfg2 (2048^3 terrain, 1920x1080 + 1 hard-shadow ray per hit) with "
                         "level-of-detail data and the cut-off at detail coefficient 4 "
                         "(subtrees under 2 pixels: side < t * 4 * radians(30) / 1920)"),
    "cfg3": dict(kind="brick", levels=3, width=1024, height=1024, alpha_scale=1.0,
                 step_vox=0.5, precision=3,
                 workload="N=4 brick tree, 3 grid levels + 8^3 bricks = 512^3, fp16 density "
                          "(4-octave noise - 0.4, empty bricks culled, ~20% occupancy) + uint8 "
                          "RGB albedo packed 8 B per lattice point, 1024x1024 rays, 0.5-voxel steps, trilinear, "
                          "front-to-back, early exit at T<0.01"),
    "cfg4": dict(kind="train", levels=2, cams=64, width=256, height=256, alpha_scale=1.0,
                 step_vox=0.5,
                 workload="differentiable 128^3 brick volume (fp32 density + fp32 RGB albedo), "
                          "64 cameras on a sphere at 256x256, L2 loss to images of the volume "
                          "+ N(0,0.1) noise; forward + re-marching adjoint (value = fwd+bwd)"),
    "build": dict(kind="build", depth=10, spheres=200, seed=1234,
                  workload="GPU SVO build from a dense 1024^3 float32 density grid (union of "
                           "200 seeded sphere distance fields, iso 0): surface-voxel leaves, "
                           "canonical breadth-first pool straight into the renderer layout"),
    "vbuild": dict(kind="vbuild", levels=3, precision=3, seed=1234,
                   workload="GPU brick-volume build from a dense 513^3 float32 lattice (4 "
                            "seeded sinusoid products - 0.4, clamped to [0, 1]): mark, N=4 tree, "
                            "pack into the 8-byte fp16+RGB8 device pool, rebuilt in place every "
                            "step (BrickPool::Update)"),
    "dynsync": dict(kind="dynsync", depth=8, edits=1000, seed=1234,
                    workload="editable SVO (200 seeded spheres in 256^3): 1000 random voxel "
                             "edits per step, then a sync of the changed 256-node pages into "
                             "the device mirror and one 512x512 frame traced from it"),
    "ssna": dict(kind="ssna", scene=("terrain", dict(depth=11, n_cubes=10000, cube_min=2,
                                                     cube_max=16, seed=1234)),
                 width=1920, height=1080, passes=5,
                 workload="cfg2 scene and camera (2048^3 SVO terrain), 1920x1080: unlit trace "
                          "(albedo, hit distance, leaf normal), view depth, 5 depth-limited 5x5 "
                          "blur passes (voxel 1/2048), depth normals, Phong with one point light "
                          "at the eye"),
    "cfg5": dict(kind="batch", n=32, precision=3,
                 workload="32 seeded scenes (cfg1-type SVO or cfg3-type fp16 bricks), depth "
                          "6..11, resolution 128^2..1024^2, one persistent launch from a global "
                          "ray queue replayed from a CUDA graph (value) vs 32 per-scene launches"),
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


ARM_PARTS = {0xd0c: "Neoverse-N1", 0xd40: "Neoverse-V1", 0xd49: "Neoverse-N2",
             0xd4f: "Neoverse-V2", 0xd84: "Neoverse-V3", 0xd8e: "Neoverse-N3"}


def cpu_model():
    """Host CPU name and core count: x86 "model name", or the Arm part
    number of /proc/cpuinfo named (0xd4f = Neoverse-V2)."""
    name = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k, _, v = line.partition(":")
                k, v = k.strip(), v.strip()
                if k == "model name" and name is None:
                    name = v
                elif k == "CPU part" and name is None:
                    try:
                        part = int(v, 16)
                        name = ARM_PARTS.get(part, f"Arm part {v}")
                    except ValueError:
                        name = v
    except OSError:
        pass
    if name is None:
        import platform
        name = platform.processor() or platform.machine()
    return f"{name} x {os.cpu_count() or 1} cores"


def profile_traffic(name):
    """DRAM bytes per launch recorded from an ncu capture in profiles/<name>.md
    (line `traffic_bytes_per_launch: N`), or None."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    if not os.path.exists(p):
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", open(p).read())
    return float(m.group(1)) if m else None


def profile_l2(name):
    """L2 traffic of the kernel from profiles/<name>.md (lines
    `l2_bytes_per_launch: N`, `l2_pct_of_peak: P`, from lts__t_sectors of the
    capture), or None."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    if not os.path.exists(p):
        return None
    txt = open(p).read()
    m = re.search(r"l2_bytes_per_launch:\s*([0-9.eE+]+)", txt)
    if not m:
        return None
    out = {"bytes_per_launch": float(m.group(1))}
    m = re.search(r"l2_pct_of_peak:\s*([0-9.]+)", txt)
    if m:
        out["pct_of_peak_sector_rate"] = float(m.group(1))
    out["source"] = f"ncu --set full capture (lts__t_sectors.sum x 32 B), profiles/{name}.md"
    return out


def profile_issue(name):
    """Issue-side figures of the kernel from profiles/<name>.md (lines
    `issue_active_pct: X`, `thread_inst_per_unit: Y (unit)`,
    `simd_efficiency_pct: Z`), or None: the traversal kernels are bound by
    instruction issue, so these say more than the bandwidth fraction."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    if not os.path.exists(p):
        return None
    txt = open(p).read()
    out = {}
    for key in ("issue_active_pct", "simd_efficiency_pct"):
        m = re.search(key + r":\s*([0-9.]+)", txt)
        if m:
            out[key] = float(m.group(1))
    m = re.search(r"thread_inst_per_unit:\s*([0-9.]+)\s*\(([^)]*)\)", txt)
    if m:
        out["thread_instructions_per_unit"] = float(m.group(1))
        out["unit"] = m.group(2)
    if out:
        out["source"] = f"ncu --set full capture, profiles/{name}.md"
    return out or None


def cfg_seed(cfg):
    """The workload's scene seed (1234 unless --seed set another)."""
    if "scene" in cfg:
        return cfg["scene"][1]["seed"]
    return cfg.get("seed", SEED)


def with_seed(cfg, seed):
    """A copy of cfg whose scene, volume or batch specs use `seed`."""
    import copy
    c = copy.deepcopy(cfg)
    if "scene" in c:
        c["scene"][1]["seed"] = seed
    else:
        c["seed"] = seed
    return c


def make_scene(cfg):
    import yoxel
    kind, kw = cfg["scene"]
    if kind == "spheres":
        s = yoxel.SVOScene.spheres(**kw)
    else:
        s = yoxel.SVOScene.terrain(**kw)
    if cfg.get("detail"):
        s.build_lod()
    return s


# --------------------------------------------------------------- CPU oracle
def cpu_svo(cfg, scene, width, height, threads, min_seconds=0.0, max_runs=1, lod_coef=0.0):
    """Times the FP32 oracle (restatement of the reference CPU renderer) on
    `threads` host threads.  Returns (Mrays/s, seconds per run, rays per run).
    lod_coef: the level-of-detail cut-off of the full-size frame."""
    from oracle import pyoracle
    pos, view = camera()
    runs, t_tot, rays = 0, 0.0, 0
    while runs < max_runs and (runs == 0 or t_tot < min_seconds):
        t0 = time.perf_counter()
        o = pyoracle.svo_render(scene.nodes_u32, scene.root, scene.attrs_u8, pos, view,
                                [0, 0, 1], 60.0, width, height, LIGHT,
                                shadows=cfg["shadows"], threads=threads, lod_coef=lod_coef)
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
    if cfg["kind"] not in ("svo", "brick"):
        print(json.dumps({"impl": "reference", "unavailable":
                          f"{args.config}: the reference has no CPU form of this workload"}))
        return
    # each step: the same frame as the GPU arm (all its primary and shadow
    # rays)
    w, h = cfg["width"], cfg["height"]
    if cfg["kind"] == "svo":
        scene = make_scene(cfg)
        # the cut-off of the full-size frame (detail * radians(fov / 2) / width)
        lod = (float(np.float32(cfg["detail"] * 60.0 * (math.pi / 360.0) / cfg["width"]))
               if cfg.get("detail") else 0.0)
        step = lambda: cpu_svo(cfg, scene, w, h, threads, lod_coef=lod)
    else:
        import yoxel
        from oracle import pyoracle
        vol = yoxel.BrickVolume.noise(cfg["levels"], 0.4, 1.4, cfg_seed(cfg))
        den = vol.density.astype(np.float16).astype(np.float32)
        alb = vol.albedo_u8.astype(np.float32) * np.float32(1.0 / 255.0)
        pos, view = camera()

        def step():
            t0 = time.perf_counter()
            pyoracle.brick_render_f32_mt(vol.grids, den, alb, vol.levels, pos, view, (0, 0, 1),
                                         60.0, w, h, cfg["alpha_scale"], cfg["step_vox"],
                                         threads=threads)
            s = time.perf_counter() - t0
            return w * h / s / 1e6, s, w * h
    for _ in range(args.warmup):
        step()
    vals, secs = [], []
    rays = 0
    for _ in range(args.steps):
        v, s, rays = step()
        vals.append(v)
        secs.append(s)
    value = rays * len(secs) / sum(secs) / 1e6
    sample = (f"the {w}x{h} frame of the same scene and camera per step ({rays} rays incl. "
              f"shadow rays), as the GPU arm traces it")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT,
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * sum(secs) / len(secs), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": cfg["workload"], "config": args.config, "seed": cfg_seed(cfg)},
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "the FP32 C restatement of the reference CPU renderer (cell/ppu_renderer.cpp) "
                "on all host cores in row-interleaved threads; the reference renderer itself, "
                "compiled from its sources with stand-ins for its missing headers "
                "(oracle/build_ref.py), returns the same hits, t and fetch counts bit for bit "
                "(tests/test_ref_pin.py) but its sources are not on this machine",
        "cpu_model": cpu_model(),
    }
    print(json.dumps(line), flush=True)


def run_svo(args, cfg):
    """SVO frame (cfg1 / cfg2 / lod).  With N > 1 ranks the one frame is
    sharded: rank r traces its contiguous range of 8x4-pixel tiles (ranges of
    equal node-fetch cost, yoxel.parallel.partition_tiles over the per-tile
    fetches of a first frame), the tile split of the reference's threaded
    renderer (cell/ppu_renderer.cpp:121-144); no collective on the data path.
    `value` = the frame's rays / the slowest rank's time (strong scaling)."""
    import torch
    import yoxel
    from yoxel import parallel as P
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
    r.SetDetailCoef(cfg.get("detail", 0.0))
    lod_coef = r.lod_coef() if cfg.get("detail") else 0.0
    dev_nodes, dev_bytes = r.device_scene_info()

    # algorithmic bytes of this frame: 40 B per node dereference (RecTrace
    # calls reaching cell/ppu_renderer.cpp:23) of primary and shadow rays,
    # + 8 B per pixel (RGBA8 + hit id) + 8 B leaf attribute per hit
    o = r.render_outputs()
    F = int(o["fetches"].to(torch.int64).sum())
    Fs = int(o["shadow_fetches"].to(torch.int64).sum())
    hits = int(o["stats"]["hits"])
    shadow_rays = hits if cfg["shadows"] else 0
    rays = npix + shadow_rays
    alg_bytes = 40 * F + 40 * Fs + 8 * npix + 8 * hits
    # this rank's tiles (all of them on one GPU) and its share of the bytes
    tx, ty = r.tile_count()
    if ws > 1:
        fcost = (o["fetches"].to(torch.int64) + o["shadow_fetches"].to(torch.int64)).cpu()
        ranges = P.partition_tiles(P.tile_costs(fcost.numpy(), w, h), ws)
        tb, te = ranges[rank]
        y0, y1 = P.tile_rows((tb, te), w, h)
        mask = torch.zeros((ty * 4, tx * 8), dtype=torch.bool)
        for t in range(tb, te):
            mask[(t // tx) * 4:(t // tx) * 4 + 4, (t % tx) * 8:(t % tx) * 8 + 8] = True
        mask = mask[:h, :w].cuda()
        hitm = (o["hit"] != -1) & mask
        my_bytes = (40 * int(o["fetches"].to(torch.int64)[mask].sum()) +
                    40 * int(o["shadow_fetches"].to(torch.int64)[mask].sum()) +
                    8 * int(mask.sum()) + 8 * int(hitm.sum()))
    else:
        tb, te, y0, y1 = 0, tx * ty, 0, h
        my_bytes = alg_bytes
    del o

    rgba = torch.empty((h, w), dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def frame():
        if ws > 1:
            r.render_tiles(tb, te, rgba=rgba, stream=stream)
        else:
            r.render_async(rgba=rgba, stream=stream)

    for _ in range(args.warmup):
        flush.fill_(1)
        frame()
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
        frame()
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
        frame()
    ew[1].record(stream)
    torch.cuda.synchronize()
    warm_ms = ew[0].elapsed_time(ew[1]) / args.steps
    clocks = sampler.stop()

    # end to end through the C ABI with a pinned host frame buffer: one
    # GPU renders the whole frame with yv_render_frame (synchronous, frame
    # read back); sharded, each rank renders its tiles and reads back the
    # rows that hold them
    host = torch.empty((h, w), dtype=torch.int32, pin_memory=True)
    import ctypes as C
    from yoxel import _lib as L

    def e2e_frame():
        if ws > 1:
            r.render_tiles(tb, te, rgba=rgba, stream=stream)
            if y1 > y0:
                host[y0:y1].copy_(rgba[y0:y1], non_blocking=True)
            r.frame_stats()
        else:
            L.check(L.lib.yv_render_frame(r.handle, C.c_void_p(host.data_ptr()), None,
                                          C.c_void_p(stream.cuda_stream)), "render_frame")

    for _ in range(2):
        e2e_frame()
    barrier()
    te_ = time.perf_counter()
    for _ in range(args.steps):
        e2e_frame()
    barrier()
    e2e_s = (time.perf_counter() - te_) / args.steps
    d2h = (y1 - y0) * w * 4 + 32

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
    value = rays * args.steps / dev_s / 1e6
    peaks, peak_kind = measured_peaks()
    achieved = my_bytes / mean_step_s / 1e9
    traffic = profile_traffic(f"svo_frame_{args.config}") if ws == 1 else None
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(mean_step_s * 1000, 4), "higher_is_better": True,
        "scaling": "strong" if ws > 1 else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": cfg["workload"], "config": args.config, "seed": cfg_seed(cfg),
                   "primary_rays_per_step": npix, "shadow_rays_per_step": shadow_rays,
                   "scene_nodes": dev_nodes, "scene_device_bytes": dev_bytes,
                   "l2": "flushed between steps (256 MiB write); scene > L2",
                   "parallelism": (f"one frame sharded into {ws} tile ranges of equal node-fetch "
                                   f"cost (rank 0: tiles {tb}-{te} of {tx * ty})" if ws > 1
                                   else "single GPU")},
        "primary_mrays_s": round(npix * args.steps / dev_s / 1e6, 3),
        "warm_l2_mrays_s": round(rays / (warm_ms / 1000) / 1e6, 3),
        "wall_s_timed_region": round(wall, 4),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2),
                     "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "traffic": traffic, "peak_source": peak_kind,
                     "traffic_source": (f"ncu capture of one launch (dram__bytes_read.sum + "
                                        f"dram__bytes_write.sum), profiles/svo_frame_"
                                        f"{args.config}.md" if traffic else None),
                     "kernel": "svo_frame_kernel",
                     "algorithmic_bytes_per_step": my_bytes,
                     "bytes_per_ray": round(alg_bytes / rays, 2),
                     "mean_node_fetches_primary": round(F / npix, 3),
                     "mean_node_fetches_shadow": round(Fs / max(1, shadow_rays), 3)},
        "e2e": {"value": round(rays / e2e_s / 1e6, 3), "unit": UNIT,
                "h2d_bytes_per_step": 40, "d2h_bytes_per_step": d2h,
                "path": ("yv_render_frame (C ABI) into pinned host memory, synchronous"
                         if ws == 1 else "yv_render_frame_tiles (C ABI) per rank, its rows "
                         "read back into pinned host memory, synchronous")},
        "gpu_launches": int(st["launches"]) * args.steps,
        "clocks": clocks,
        "scene_build_s": round(t_scene, 2),
    }
    issue = profile_issue(f"svo_frame_{args.config}")
    if issue and ws == 1:
        line["roofline"]["issue"] = issue
        line["roofline"]["l2"] = profile_l2(f"svo_frame_{args.config}")
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sw, sh = w // 4, h // 4
        v, s_, rr = cpu_svo(cfg, scene, sw, sh, threads, min_seconds=10.0, max_runs=100000,
                            lod_coef=lod_coef)
        v1, s1, rr1 = cpu_svo(cfg, scene, w // 16, h // 16, 1, lod_coef=lod_coef)
        v4, s4, rr4 = cpu_svo(cfg, scene, w // 8, h // 8, 4, lod_coef=lod_coef)
        runs = max(1, int(round(10.0 / s_))) if s_ > 0 else 1
        line["cpu_baseline"] = {
            "value": round(v, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{sw}x{sh} frame of the same scene and camera ({rr} rays incl. shadow "
                      f"rays), repeated for >= 10 s (~{runs} frames); the FP32 C "
                      f"restatement of cell/ppu_renderer.cpp, which reproduces the reference "
                      f"renderer compiled from its sources bit for bit (tests/test_ref_pin.py)",
            "single_thread_value": round(v1, 4),
            "four_thread_value": round(v4, 4),
            "cpu_model": cpu_model()}
    print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


def _timed_steps(torch, steps, fn, flush=None, stream=None):
    """Per-step CUDA-event times (ms) of fn(), flush() between steps outside
    the events; bracketed by synchronize."""
    stream = stream or torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(steps)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(steps):
        if flush is not None:
            flush()
        evs[i][0].record(stream)
        fn()
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    return [a.elapsed_time(b) for a, b in evs], wall


def _base_line(args, cfg, value, ms, dtype):
    ws, _, _ = dist_env()
    return {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic",
            "config": {"workload": cfg["workload"], "config": args.config,
                       "seed": cfg_seed(cfg), "l2": "flushed between steps (256 MiB write)"}}


def run_brick(args, cfg):
    """cfg3: plain brick march, fp16 pool.  Under torchrun (N > 1) the frame
    is split into warp-tile ranges of near-equal sample count (the samples
    of a first frame; yoxel.parallel.partition_volume_tiles), each rank
    renders its range (yv_volume_render_tiles), and `value` = the frame's
    rays / the slowest rank's time (strong scaling); no collective on the
    data path."""
    import torch
    import yoxel
    from yoxel import parallel as P
    from yoxel import workloads as W
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
    vol = yoxel.BrickVolume.noise(cfg["levels"], 0.4, 1.4, cfg_seed(cfg))
    t_scene = time.perf_counter() - t_scene
    prec = cfg["precision"] if args.precision is None else args.precision
    gv = vol.upload(prec)
    desc = gv.desc()
    pos, view = W.camera()
    cam = [(pos, view, (0, 0, 1), 60.0)]
    w, h = cfg["width"], cfg["height"]
    rays = w * h
    ns = torch.zeros((1, h, w), dtype=torch.int32, device="cuda")
    nb = torch.zeros((1, h, w), dtype=torch.int32, device="cuda")
    out = yoxel.render_volume(desc, cam, w, h, cfg["alpha_scale"], cfg["step_vox"],
                              samples=ns, bricks=nb)
    S, B = int(ns.to(torch.int64).sum()), int(nb.to(torch.int64).sum())
    # 8 trilinear corners x (density + RGB) per sample - 2 + 3 B for the fp16
    # formats, 4 + 12 B for fp32 - 4 B per tree level per occupied brick
    # entered, 16 B RGBA fp32 out
    per_corner = 5 if prec in (0, 3) else 16
    alg = 8 * per_corner * S + 4 * cfg["levels"] * B + 16 * rays
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    y0, y1 = 0, h
    if ws > 1:
        # this rank's squares of warp tiles and the pixel rows they hold
        ranges = P.partition_volume_tiles(P.volume_tile_costs(ns.cpu().numpy(), w, h), ws)
        tb, te_t = ranges[rank]
        if te_t > tb:
            y0, y1 = P.volume_tile_rows((tb, te_t), w, h)
        share = float(ns[:, y0:y1].to(torch.int64).sum()) / max(1, S)
        alg = int(alg * share)  # this rank's part of the bytes (rows it covers)
        fn = lambda: yoxel.render_volume_tiles(desc, cam, w, h, tb, te_t, out,
                                               cfg["alpha_scale"], cfg["step_vox"])
    else:
        fn = lambda: yoxel.render_volume(desc, cam, w, h, cfg["alpha_scale"],
                                         cfg["step_vox"], out=out)
    for _ in range(args.warmup):
        flush.fill_(1)
        fn()
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.4)
    barrier()
    ms, wall = _timed_steps(torch, args.steps, fn, lambda: flush.fill_(1))
    barrier()
    clocks = sampler.stop()
    mean_ms = sum(ms) / len(ms)
    host = torch.empty((1, h, w, 4), dtype=torch.float32, pin_memory=True)
    torch.cuda.synchronize()
    barrier()
    te = time.perf_counter()
    for _ in range(args.steps):
        fn()
        host[:, y0:y1].copy_(out[:, y0:y1])  # synchronous D2H into pinned memory
    barrier()
    e2e_s = (time.perf_counter() - te) / args.steps
    my_ms = mean_ms
    if pg is not None:
        tot = torch.tensor([mean_ms, e2e_s], dtype=torch.float64, device="cuda")
        pg.all_reduce(tot, op=pg.ReduceOp.MAX)
        mean_ms, e2e_s = float(tot[0]), float(tot[1])
        if rank != 0:
            pg.destroy_process_group()
            return
    peaks, kind = measured_peaks()
    achieved = alg / (my_ms / 1e3) / 1e9
    line = _base_line(args, cfg, rays / (mean_ms / 1e3) / 1e6, mean_ms,
                      "f32 (fp16 storage)" if prec in (0, 3) else "f32")
    line["config"].update(volume_bricks=vol.nbricks, occupancy=round(vol.occupancy, 4),
                          mean_samples_per_ray=round(S / rays, 2),
                          pool_format=POOL_FORMATS[prec])
    if ws > 1:
        line["scaling"] = "strong"
        line["config"]["parallelism"] = (f"one frame split into {ws} warp-tile ranges of "
                                         f"near-equal samples (rank 0: tiles {tb}..{te_t})")
    line.update({
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "traffic": profile_traffic("volume_forward_cfg3"), "peak_source": kind,
                     "traffic_source": "ncu capture of one launch (dram__bytes_read.sum + "
                                       "dram__bytes_write.sum), profiles/volume_forward_cfg3.md",
                     "algorithmic_bytes_per_step": alg,
                     "issue": profile_issue("volume_forward_cfg3"),
                     "l2": profile_l2("volume_forward_cfg3")},
        "e2e": {"value": round(rays / e2e_s / 1e6, 3), "unit": UNIT, "h2d_bytes_per_step": 40,
                "d2h_bytes_per_step": (y1 - y0) * w * 16,
                "path": ("yoxel.render_volume + copy into pinned host memory" if ws == 1 else
                         "yoxel.render_volume_tiles per rank, its rows copied into pinned "
                         "host memory")},
        "gpu_launches": args.steps, "clocks": clocks, "wall_s_timed_region": round(wall, 4),
        "scene_build_s": round(t_scene, 2)})
    if not args.no_cpu_baseline and ws == 1:
        from oracle import pyoracle
        den = vol.density.astype(np.float16 if prec in (0, 3) else np.float32)
        den = den.astype(np.float32)
        alb = vol.albedo_u8.astype(np.float32) * np.float32(1.0 / 255.0)
        threads = os.cpu_count() or 1
        sw, sh = w // 4, h // 4
        t0, runs = time.perf_counter(), 0
        while runs == 0 or time.perf_counter() - t0 < 10.0:
            pyoracle.brick_render_f32_mt(vol.grids, den, alb, vol.levels, pos, view, (0, 0, 1),
                                         60.0, sw, sh, cfg["alpha_scale"], cfg["step_vox"],
                                         threads=threads)
            runs += 1
        v = sw * sh * runs / (time.perf_counter() - t0) / 1e6
        line["cpu_baseline"] = {"value": round(v, 4), "unit": UNIT, "cores": threads,
                                "kind": "port",
                                "sample": f"{sw}x{sh} frame of the same volume and camera, "
                                          f"repeated {runs}x (>= 10 s); FP32 C restatement of "
                                          "reaction/trace/trace.cu castRay over the ntree pool",
                                "cpu_model": cpu_model()}
    print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


def run_train(args, cfg):
    """cfg4: differentiable volume, forward + adjoint.  Under torchrun
    (N > 1): data parallel over the cameras (yoxel.parallel.partition_cameras),
    each step ending in the exchange step - a sum all-reduce of the density
    and albedo gradients (yoxel.parallel.sum_gradients) - inside the timed
    region; `value` = all cameras' rays / the slowest rank's step (strong
    scaling)."""
    import torch
    import yoxel
    from yoxel import parallel as P
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    from yoxel import workloads as W
    vol, tv, tgt_d, tgt_a, cam_list = W.cfg4_problem(cfg["levels"], cfg["cams"], cfg_seed(cfg))
    c0, c1 = P.partition_cameras(len(cam_list), ws)[rank]
    cams = yoxel.cameras(cam_list[c0:c1])  # this rank's cameras (all of them on one GPU)
    ncam = c1 - c0
    w, h = cfg["width"], cfg["height"]
    a_s, st = cfg["alpha_scale"], cfg["step_vox"]
    target = yoxel.render_volume(yoxel.torch_desc(tv, tgt_d, tgt_a), cams, w, h, a_s, st)
    rays = cfg["cams"] * w * h
    density = tv["density"].clone().requires_grad_(True)
    albedo = tv["albedo"].clone().requires_grad_(True)

    def fwd_bwd():
        density.grad = None
        albedo.grad = None
        rgba = yoxel.volume_march(density, albedo, tv, cams, w, h, a_s, st)
        loss = ((rgba - target) ** 2).sum()
        loss.backward()
        if pg is not None:
            P.sum_gradients([density.grad, albedo.grad])  # the exchange step
        return loss

    fwd_out = torch.empty((ncam, h, w, 4), dtype=torch.float32, device="cuda")
    # forward-only and adjoint-only legs read the same packed float4 pool
    # that volume_march builds each step
    packed = yoxel.pack_volume(density.detach(), albedo.detach())
    desc = yoxel.torch_desc(tv, packed=packed)

    def fwd():
        yoxel.render_volume(desc, cams, w, h, a_s, st, out=fwd_out)

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        fwd_bwd()
        fwd()
    ns = torch.zeros((ncam, h, w), dtype=torch.int32, device="cuda")
    yoxel.render_volume(desc, cams, w, h, a_s, st, out=fwd_out, samples=ns)
    S = int(ns.to(torch.int64).sum())
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.4)
    if pg is not None:
        pg.barrier()
    ms_fb, wall = _timed_steps(torch, args.steps, fwd_bwd, lambda: flush.fill_(1))
    ms_f, _ = _timed_steps(torch, args.steps, fwd, lambda: flush.fill_(1))
    # the adjoint kernel alone (dominant kernel of the step)
    grad = torch.randn(fwd_out.shape, device="cuda")
    gd = torch.zeros_like(tv["density"])
    ga = torch.zeros_like(tv["albedo"])
    ms_b, _ = _timed_steps(torch, args.steps,
                           lambda: yoxel.volume_backward(desc, cams, w, h, fwd_out, grad, gd, ga,
                                                         a_s, st, fold=False),
                           lambda: flush.fill_(1))
    clocks = sampler.stop()
    fb = sum(ms_fb) / len(ms_fb)
    f = sum(ms_f) / len(ms_f)
    b = sum(ms_b) / len(ms_b)
    b_mine = b
    if pg is not None:
        tot = torch.tensor([fb, f, b], dtype=torch.float64, device="cuda")
        pg.all_reduce(tot, op=pg.ReduceOp.MAX)
        fb, f, b = (float(x) for x in tot)
    peaks, kind = measured_peaks()
    # adjoint bytes: replay of the fp32 forward reads (8 x (4 + 12) B per
    # sample) + the same again as gradient atomics + 32 B/ray (rgba, dL/drgba)
    alg_b = 2 * 128 * S + 32 * ncam * w * h  # this rank's launch
    achieved = alg_b / (b_mine / 1e3) / 1e9
    line = _base_line(args, cfg, rays / (fb / 1e3) / 1e6, fb, "f32")
    if ws > 1:
        line["scaling"] = "strong"
        line["config"]["parallelism"] = (f"data parallel over the {cfg['cams']} cameras on "
                                         f"{ws} GPUs, gradient sum all-reduce each step")
    line["config"].update(rays_per_step=rays, mean_samples_per_ray=round(S / rays, 2),
                          bricks=vol.nbricks)
    line.update({
        "forward_mrays_s": round(rays / (f / 1e3) / 1e6, 3),
        "fwd_bwd_over_fwd": round(f / fb, 4),
        "backward_kernel_ms": round(b, 4),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "traffic": profile_traffic("volume_backward_cfg4"), "peak_source": kind,
                     "traffic_source": "ncu capture of one launch (dram__bytes_read.sum + "
                                       "dram__bytes_write.sum), profiles/volume_backward_cfg4.md",
                     "kernel": "volume_backward_kernel", "algorithmic_bytes_per_launch": alg_b,
                     "note": "the replay reads and the gradient atomics are served by L1/L2 "
                             "(the 29 MB gradient scratch stays in L2), so the algorithmic "
                             "bytes exceed what HBM could move in the time (frac > 1) while "
                             "DRAM moves only `traffic`: the kernel is bound by load latency "
                             "and L2 atomic requests, not HBM",
                     "issue": profile_issue("volume_backward_cfg4"),
                     "l2": profile_l2("volume_backward_cfg4")},
        "gradient_check": "GPU adjoint vs FP64 adjoint / naive PyTorch marcher / FP64 central "
                          "differences: rel. error <= 1e-4 (tests/test_volume_gpu.py)",
        # per fwd+bwd step: pack, forward, adjoint, unpack, 2 x (fold gather +
        # scatter); the loss and its gradient are torch's own kernels
        "gpu_launches": args.steps * (6 + 2 * -(-ncam // 64)),
        "clocks": clocks, "wall_s_timed_region": round(wall, 4)})
    host = torch.empty((), dtype=torch.float32, pin_memory=True)
    torch.cuda.synchronize()
    if pg is not None:
        pg.barrier()
    te = time.perf_counter()
    for _ in range(args.steps):
        loss = fwd_bwd()
        host.copy_(loss.detach())  # D2H of the step's loss
    e2e = (time.perf_counter() - te) / args.steps
    if pg is not None:
        t = torch.tensor([e2e], dtype=torch.float64, device="cuda")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        e2e = float(t[0])
        if rank != 0:
            pg.destroy_process_group()
            return
    line["e2e"] = {"value": round(rays / e2e / 1e6, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 4,
                   "path": "yoxel.volume_march + L2 loss + backward, loss read on the host"
                           + (" (each rank its cameras, gradient all-reduce)" if ws > 1 else "")}
    print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


def run_batch(args, cfg):
    """cfg5: batched persistent launch vs per-scene launches.  Under torchrun
    (N > 1) the scenes are split across the ranks (largest-first greedy on
    pixels, a brick pixel weighing 4; yoxel.parallel.partition_scenes), each
    rank batches its own, and `value` = all scenes' rays / the slowest rank's
    batch (strong scaling); no collective on the data path."""
    import torch
    import yoxel
    from yoxel import autotune
    from yoxel import parallel as P
    from yoxel import workloads as W
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    all_specs = W.cfg5_specs(cfg_seed(cfg), cfg["n"])
    all_rays = sum(sp["res"] ** 2 for sp in all_specs)
    specs = all_specs
    if ws > 1:
        costs = [sp["res"] ** 2 * (4 if sp["kind"] != "svo" else 1) for sp in all_specs]
        specs = [all_specs[i] for i in P.partition_scenes(costs, ws)[rank]]
    prec = cfg["precision"] if args.precision is None else args.precision
    t_scene = time.perf_counter()
    batch, items = W.cfg5_batch(specs, prec)
    rays = 0
    alg = 0      # algorithmic bytes of one batch (SVO: 40 B/fetch + 8 B/pixel + 8 B/hit;
    outs = []    # bricks: 8 corners x format bytes per sample + refs + 16 B/pixel)
    for it in items:
        res = it["res"]
        if it["kind"] == "svo":
            # algorithmic bytes of this scene from its own counters (one render)
            o = it["renderer"].render_outputs()
            alg += (40 * int(o["fetches"].to(torch.int64).sum()) + 8 * res * res +
                    8 * int(o["stats"]["hits"]))
            del o
        else:
            ns = torch.zeros((1, res, res), dtype=torch.int32, device="cuda")
            nb = torch.zeros((1, res, res), dtype=torch.int32, device="cuda")
            gv = it["gpu_volume"]
            yoxel.render_volume(gv.desc(), [it["cam"]], res, res, samples=ns, bricks=nb)
            per_corner = 5 if prec in (0, 3) else 16
            alg += (8 * per_corner * int(ns.to(torch.int64).sum()) +
                    4 * it["volume"].levels * int(nb.to(torch.int64).sum()) + 16 * res * res)
            del ns, nb
        outs.append(it["out"])
        rays += res * res
    t_scene = time.perf_counter() - t_scene
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    best, _ = autotune.tune_batch(batch, f"cfg5-{cfg['n']}" + (f"-r{rank}of{ws}" if ws > 1 else ""),
                                  reps=2, flush=lambda: flush.fill_(1))
    for _ in range(args.warmup):
        batch.render(graph=True)
        batch.render_separate()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.4)
    if pg is not None:
        pg.barrier()
    ms_b, wall = _timed_steps(torch, args.steps, lambda: batch.render(graph=True),
                              lambda: flush.fill_(1))
    ms_s, _ = _timed_steps(torch, args.steps, batch.render_separate, lambda: flush.fill_(1))
    ms_p, _ = _timed_steps(torch, args.steps, lambda: batch.render(graph=False),
                           lambda: flush.fill_(1))
    clocks = sampler.stop()
    tb, ts, tp = (sum(x) / len(x) for x in (ms_b, ms_s, ms_p))
    # end to end: the graph replay plus the device-to-host copy of every
    # frame of the batch into pinned memory, synchronous per step
    hosts = [torch.empty(o.shape, dtype=o.dtype, pin_memory=True) for o in outs]
    d2h = sum(o.numel() * o.element_size() for o in outs)
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(args.steps):
        batch.render(graph=True)
        for hst, o in zip(hosts, outs):
            hst.copy_(o, non_blocking=True)
        torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - te) / args.steps
    peaks, kind = measured_peaks()
    achieved = alg / (tb / 1e3) / 1e9  # this rank's batch
    if pg is not None:
        tot = torch.tensor([tb, ts, tp, e2e_s], dtype=torch.float64, device="cuda")
        pg.all_reduce(tot, op=pg.ReduceOp.MAX)
        tb, ts, tp, e2e_s = (float(x) for x in tot)
        if rank != 0:
            pg.destroy_process_group()
            return
    rays = all_rays
    line = _base_line(args, cfg, rays / (tb / 1e3) / 1e6, tb, "f32")
    if ws > 1:
        line["scaling"] = "strong"
        line["config"]["parallelism"] = (f"the {len(all_specs)} scenes split across {ws} GPUs "
                                         f"(rank 0: {len(specs)} scenes)")
    line["config"].update(scenes=len(specs), rays_per_step=rays,
                          svo_scenes=sum(1 for s in specs if s["kind"] == "svo"),
                          launch_config=best)
    line.update({
        "separate_launches_mrays_s": round(rays / (ts / 1e3) / 1e6, 3),
        "persistent_without_graph_mrays_s": round(rays / (tp / 1e3) / 1e6, 3),
        "speedup_vs_separate": round(ts / tb, 3),
        "gpu_launches": args.steps, "clocks": clocks, "wall_s_timed_region": round(wall, 4),
        "scene_build_s": round(t_scene, 2),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "traffic": None, "peak_source": kind, "kernel": "batch_kernel",
                     "algorithmic_bytes_per_launch": alg},
        "e2e": {"value": round(rays / e2e_s / 1e6, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": d2h,
                "path": "yoxel.Batch.render (CUDA graph replay) + copy of all frames into "
                        "pinned host memory; scenes and cameras resident on the device"}})
    print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


def sphere_density(torch, G, n, seed, device):
    """(G, G, G) float32 [z, y, x]: max over n seeded spheres of (r - |p - c|),
    in voxel units, built slab by slab on `device`."""
    rng = np.random.default_rng(seed)
    c = torch.tensor(rng.uniform(0, G, (n, 3)), dtype=torch.float32, device=device)
    r = torch.tensor(rng.uniform(G / 64, G / 8, n), dtype=torch.float32, device=device)
    ax = torch.arange(G, dtype=torch.float32, device=device)
    out = torch.empty((G, G, G), dtype=torch.float32, device=device)
    zs = max(1, (1 << 24) // (G * G))
    for z0 in range(0, G, zs):
        z = ax[z0:z0 + zs].view(-1, 1, 1)
        acc = torch.full((z.shape[0], G, G), -1e9, dtype=torch.float32, device=device)
        for i in range(n):
            d = torch.sqrt((ax.view(1, 1, -1) - c[i, 0]) ** 2 + (ax.view(1, -1, 1) - c[i, 1]) ** 2
                           + (z - c[i, 2]) ** 2)
            torch.maximum(acc, r[i] - d, out=acc)
        out[z0:z0 + zs] = acc
    return out


def run_build(args, cfg):
    """GPU SVO build from a dense grid, Mvoxels/s of grid processed."""
    import torch
    import yoxel
    torch.cuda.set_device(dist_env()[2])
    depth = cfg["depth"]
    G = 1 << depth
    dens = sphere_density(torch, G, cfg["spheres"], cfg["seed"], "cuda")
    torch.cuda.synchronize()
    r = yoxel.Renderer()
    fn = lambda: r.SetSceneDense(dens, depth, 0.0)
    for _ in range(args.warmup):
        fn()
    torch.cuda.synchronize()
    nn, nbytes = r.device_scene_info()
    s = yoxel.SVOScene.build_dense(dens, depth, 0.0)
    na = s.attr_count
    sampler = ClockSampler(dist_env()[2])
    sampler.start()
    time.sleep(0.4)
    ms, wall = _timed_steps(torch, args.steps, fn)
    clocks = sampler.stop()
    mean_ms = sum(ms) / len(ms)
    vox = G ** 3
    # density read once + node records (32 B + 4 B id) + shading records (16 B)
    alg = 4 * vox + 36 * nn + 16 * na
    peaks, kind = measured_peaks()
    achieved = alg / (mean_ms / 1e3) / 1e9
    line = _base_line(args, cfg, vox / (mean_ms / 1e3) / 1e6, mean_ms, "f32 density, u32 pool")
    line["metric"] = "Mvoxels/s of dense grid turned into a device SVO on 1 GB300"
    line["unit"] = "Mvoxels/s"
    line["config"].update(grid=f"{G}^3", nodes=nn, leaves=na, l2="grid (4 GiB) > L2")
    # end to end: host density (pinned) -> device, build, pool copied back to the host
    host = torch.empty(dens.shape, dtype=torch.float32, pin_memory=True)
    host.copy_(dens)
    dev = torch.empty_like(dens)
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(max(1, args.steps // 4)):
        dev.copy_(host, non_blocking=True)
        s2 = yoxel.SVOScene.build_dense(dev, depth, 0.0)
        del s2
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - te) / max(1, args.steps // 4)
    line.update({
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "traffic": None, "peak_source": kind, "kernel": "dense build (all passes)",
                     "algorithmic_bytes_per_step": alg},
        "e2e": {"value": round(vox / e2e_s / 1e6, 3), "unit": "Mvoxels/s",
                "h2d_bytes_per_step": 4 * vox, "d2h_bytes_per_step": 40 * nn + 8 * na,
                "path": "density from pinned host memory, yoxel.SVOScene.build_dense (pool "
                        "copied back into a host container)"},
        # 67 kernels per 1024^3 build (the ncu launch list of the same command)
        "gpu_launches": args.steps * 67,
        "gpu_launches_source": "ncu launch list, profiles/svo_build_dense_1024.md",
        "clocks": clocks, "wall_s_timed_region": round(wall, 4)})
    if not args.no_cpu_baseline:
        from oracle import pyoracle
        sd = 8
        small = sphere_density(torch, 1 << sd, cfg["spheres"], cfg["seed"], "cuda").cpu().numpy()
        t0, runs = time.perf_counter(), 0
        while runs == 0 or (time.perf_counter() - t0 < 10.0 and runs < 20):
            pyoracle.svo_build_dense(small, sd, 0.0)
            runs += 1
        v = (1 << sd) ** 3 * runs / (time.perf_counter() - t0) / 1e6
        line["cpu_baseline"] = {"value": round(v, 3), "unit": "Mvoxels/s", "cores": 1,
                                "kind": "port",
                                "sample": f"the same field at 256^3, built {runs}x by the C "
                                          "oracle (recursive region build + breadth-first "
                                          "renumbering)"}
    print(json.dumps(line), flush=True)


def wave_lattice(torch, n, seed, device):
    """(n, n, n) float32 [z, y, x]: clamp(sum of 4 seeded sinusoid products
    - 0.4, 0, 1)."""
    rng = np.random.default_rng(seed)
    ax = torch.arange(n, dtype=torch.float32, device=device) / n
    acc = torch.zeros((n, n, n), dtype=torch.float32, device=device)
    for _ in range(4):
        f = rng.uniform(2, 9, 3)
        p = rng.uniform(0, 6.28, 3)
        acc += (torch.sin(ax.view(-1, 1, 1) * float(f[2]) + float(p[2])) *
                torch.sin(ax.view(1, -1, 1) * float(f[1]) + float(p[1])) *
                torch.sin(ax.view(1, 1, -1) * float(f[0]) + float(p[0])))
    return (acc * 0.5 - 0.4).clamp_(0, 1)


def run_vbuild(args, cfg):
    """GPU brick-volume build from a dense lattice, Mvoxels/s of lattice."""
    import torch
    import yoxel
    torch.cuda.set_device(dist_env()[2])
    levels = cfg["levels"]
    n = 8 * 4 ** levels + 1
    lat = wave_lattice(torch, n, cfg["seed"], "cuda")
    torch.cuda.synchronize()
    # BrickPool::Update: the pool is rebuilt in place every step
    vol = yoxel.VolumeGPU.from_dense(lat, levels, cfg["precision"])

    def fn():
        vol.rebuild_dense(lat, levels)

    for _ in range(args.warmup):
        fn()
    torch.cuda.synchronize()
    host = yoxel.BrickVolume.build_dense(lat, levels)
    nb = host.nbricks
    sampler = ClockSampler(dist_env()[2])
    sampler.start()
    time.sleep(0.4)
    ms, wall = _timed_steps(torch, args.steps, fn)
    clocks = sampler.stop()
    mean_ms = sum(ms) / len(ms)
    vox = n ** 3
    # lattice read once + the 8-byte pool + grid refs
    alg = 4 * vox + 8 * 729 * nb + 256 * host.ngrids
    peaks, kind = measured_peaks()
    achieved = alg / (mean_ms / 1e3) / 1e9
    line = _base_line(args, cfg, vox / (mean_ms / 1e3) / 1e6, mean_ms, "f32 lattice, fp16+RGB8 pool")
    line["metric"] = "Mvoxels/s of dense lattice turned into a device brick pool on 1 GB300"
    line["unit"] = "Mvoxels/s"
    line["config"].update(lattice=f"{n}^3", bricks=nb, occupancy=round(host.occupancy, 4),
                          l2="lattice (540 MB) > L2")
    # end to end: lattice from pinned host memory, build, pool copied to the host
    hl = torch.empty(lat.shape, dtype=torch.float32, pin_memory=True)
    hl.copy_(lat)
    dev = torch.empty_like(lat)
    torch.cuda.synchronize()
    te = time.perf_counter()
    reps = max(1, args.steps // 4)
    for _ in range(reps):
        dev.copy_(hl, non_blocking=True)
        v2 = yoxel.BrickVolume.build_dense(dev, levels)
        del v2
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - te) / reps
    line.update({
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "traffic": None, "peak_source": kind, "kernel": "volume build (all passes)",
                     "algorithmic_bytes_per_step": alg},
        "e2e": {"value": round(vox / e2e_s / 1e6, 3), "unit": "Mvoxels/s",
                "h2d_bytes_per_step": 4 * vox, "d2h_bytes_per_step": 4 * 729 * nb * 4,
                "path": "lattice from pinned host memory, yoxel.BrickVolume.build_dense (pool "
                        "copied back into a host container)"},
        # 21 kernels per 513^3 rebuild (the ncu launch list of the same command)
        "gpu_launches": args.steps * 21,
        "gpu_launches_source": "ncu launch list, profiles/volume_build_dense_513.md",
        "clocks": clocks, "wall_s_timed_region": round(wall, 4)})
    if not args.no_cpu_baseline:
        cpu = lat.cpu().numpy()
        t0 = time.perf_counter()
        v = yoxel.BrickVolume.from_dense(levels, cpu)
        dt = time.perf_counter() - t0
        assert v.nbricks == nb
        line["cpu_baseline"] = {"value": round(vox / dt / 1e6, 3), "unit": "Mvoxels/s",
                                "cores": 1, "kind": "port",
                                "sample": f"the same {n}^3 lattice built once by the host "
                                          "RangeBuilder restatement (yv_volume_from_dense)"}
    print(json.dumps(line), flush=True)


def run_dynsync(args, cfg):
    """Incremental device sync of an edited SVO: frames per second of the
    edit -> sync -> trace loop and the bytes each sync moves."""
    import torch
    import yoxel
    torch.cuda.set_device(dist_env()[2])
    depth = cfg["depth"]
    scene = yoxel.SVOScene.spheres(depth, 200, 4.0, 24.0, cfg["seed"])
    dyn = yoxel.DynamicSVO(scene.node_count + 64 * cfg["edits"] * (args.steps + args.warmup + 4),
                           scene.attr_count + 2 * cfg["edits"] * (args.steps + args.warmup + 4))
    dyn.load(scene)
    full_bytes = dyn.transfer_bytes()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dyn.sync()
    torch.cuda.synchronize()
    full_ms = (time.perf_counter() - t0) * 1e3
    rng = np.random.default_rng(cfg["seed"])
    G = 1 << depth
    pos, view = camera()
    w = h = 512

    def edits():
        for _ in range(cfg["edits"]):
            x, y, z = (int(v) for v in rng.integers(0, G, 3))
            if rng.random() < 0.5:
                dyn.set_voxel(depth, x, y, z, rgb=(255, 128, 0))
            else:
                dyn.set_voxel(depth, x, y, z, None)

    for _ in range(args.warmup):
        edits()
        dyn.sync()
        dyn.render(pos, view, (0, 0, 1), 60.0, w, h, LIGHT)
    torch.cuda.synchronize()
    sync_ms, moved, frame_ms = [], [], []
    for _ in range(args.steps):
        edits()
        moved.append(dyn.transfer_bytes())
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        c = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ts = time.perf_counter()
        a.record()
        dyn.sync()
        b.record()
        dyn.render(pos, view, (0, 0, 1), 60.0, w, h, LIGHT)
        c.record()
        torch.cuda.synchronize()
        sync_ms.append((time.perf_counter() - ts) * 1e3)
        frame_ms.append(b.elapsed_time(c))
    mean_sync = sum(sync_ms) / len(sync_ms)
    mean_frame = sum(frame_ms) / len(frame_ms)
    step_ms = mean_sync + mean_frame
    # the frame kernel's algorithmic bytes: 40 B per node dereference, 8 B
    # per pixel (RGBA8 + hit id), 8 B leaf attribute per hit
    fo = dyn.render(pos, view, (0, 0, 1), 60.0, w, h, LIGHT)
    torch.cuda.synchronize()
    F = int(fo["fetches"].to(torch.int64).sum())
    hits = int((fo["hit"] != -1).sum())
    frame_bytes = 40 * F + 8 * w * h + 8 * hits
    peaks, kind = measured_peaks()
    achieved = frame_bytes / (mean_frame / 1e3) / 1e9
    line = _base_line(args, cfg, (w * h) / (step_ms / 1e3) / 1e6, step_ms, "f32")
    line["metric"] = "Mrays/s of the edit-sync-trace loop on 1 GB300"
    line["config"].update(scene_nodes=scene.node_count, edits_per_step=cfg["edits"])
    line.update({
        "sync_ms_host_wall": round(mean_sync, 4), "frame_ms": round(mean_frame, 4),
        "bytes_per_sync": int(sum(moved) / len(moved)), "full_upload_bytes": full_bytes,
        "full_sync_ms": round(full_ms, 3),
        "roofline": {"bound": "hbm", "kernel": "svo_frame_kernel (caller pool: the mirror)",
                     "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": None,
                     "peak_source": kind, "algorithmic_bytes_per_frame": frame_bytes,
                     "note": "the sync moves its pages host to device; the frame reads the "
                             "mirror"},
        # per step: one page scatter per array (nodes, attributes) + the frame
        "e2e": None, "gpu_launches": 3 * args.steps})
    print(json.dumps(line), flush=True)


def run_ssna(args, cfg):
    """Screen-space normal approximation frame (trace + post passes): pixels
    per second of the whole frame; the post chain timed against the unlit
    trace alone."""
    import ctypes as C

    import torch
    import yoxel
    from yoxel import _lib as L
    torch.cuda.set_device(dist_env()[2])
    scene = make_scene(cfg)
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
    r.SetLight(LIGHT, 1.0, 0.0, False)
    p = r.ssna_params()
    p.blur_passes = cfg["passes"]
    dev = torch.device("cuda", torch.cuda.current_device())
    rgba = torch.empty((h, w), dtype=torch.int32, device=dev)
    alb = torch.empty((h, w), dtype=torch.int32, device=dev)
    ht = torch.empty((h, w), dtype=torch.float32, device=dev)
    nrm = torch.empty((h, w, 3), dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()

    def frame():
        r.render_ssna(p, rgba=rgba, stream=stream)

    def unlit():
        r.render_async(rgba=alb, hit_t=ht, normal=nrm, stream=stream)

    for _ in range(args.warmup):
        frame()
        unlit()
    st = r.frame_stats()
    sampler = ClockSampler(dist_env()[2])
    sampler.start()
    time.sleep(0.4)
    ms, wall = _timed_steps(torch, args.steps, frame, flush=lambda: flush.fill_(1))
    ms_trace, _ = _timed_steps(torch, args.steps, unlit, flush=lambda: flush.fill_(1))
    clocks = sampler.stop()
    st = r.frame_stats()
    mean = sum(ms) / len(ms)
    mean_trace = sum(ms_trace) / len(ms_trace)
    post_ms = max(mean - mean_trace, 1e-6)
    # algorithmic bytes of the post chain per pixel: depth (albedo + t in, z
    # out: 12), each blur pass (z in + out: 8), shading (albedo, z, stored
    # normal in, rgba out: 24)
    post_bytes = npix * (12 + 8 * cfg["passes"] + 24)
    peaks, peak_kind = measured_peaks()
    achieved = post_bytes / (post_ms / 1e3) / 1e9

    # end to end: yv_render_ssna + the frame read back into pinned memory
    host = torch.empty((h, w), dtype=torch.int32, pin_memory=True)
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(args.steps):
        frame()
        host.copy_(rgba, non_blocking=True)
        stream.synchronize()
    e2e_s = (time.perf_counter() - te) / args.steps
    r.frame_stats()

    line = _base_line(args, cfg, npix / (mean / 1e3) / 1e6, mean, "f32")
    line["metric"] = "Mpixels/s of the SSNA frame (trace + post passes) on 1 GB300"
    line["unit"] = "Mpixels/s"
    line["config"].update(pixels=npix, blur_passes=cfg["passes"])
    line.update({
        "unlit_trace_ms": round(mean_trace, 4), "post_chain_ms": round(post_ms, 4),
        "post_chain_mpix_s": round(npix / (post_ms / 1e3) / 1e6, 2),
        "wall_s_timed_region": round(wall, 4),
        "roofline": {"bound": "hbm", "kernel": "post chain (depth + blur passes + shade)",
                     "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": None,
                     "peak_source": peak_kind, "algorithmic_bytes_per_step": post_bytes,
                     "note": "the 8 MB depth buffers stay in L2 between passes"},
        "e2e": {"value": round(npix / e2e_s / 1e6, 3), "unit": "Mpixels/s",
                "h2d_bytes_per_step": C.sizeof(L.SsnaParams),
                "d2h_bytes_per_step": npix * 4,
                "path": "yv_render_ssna (C ABI) + frame copy into pinned host memory"},
        "gpu_launches": (int(st["launches"]) + 2 + cfg["passes"]) * args.steps,
        "clocks": clocks})
    if not args.no_cpu_baseline:
        from oracle import ssna as O
        r.render_async(rgba=alb, hit_t=ht, normal=nrm, stream=stream)
        r.frame_stats()
        sw, sh = w // 4, h // 4
        y0, x0 = (h - sh) // 2, (w - sw) // 2
        a_np = alb.cpu().numpy().view(np.uint32)[y0:y0 + sh, x0:x0 + sw]
        t_np = ht.cpu().numpy()[y0:y0 + sh, x0:x0 + sw]
        n_np = nrm.cpu().numpy()[y0:y0 + sh, x0:x0 + sw]
        d0, du, dv = r.ray_basis()
        d0 = (d0 + du * np.float32(x0) + dv * np.float32(y0)).astype(np.float32)
        lt = p.lights[0]
        light = dict(pos=list(lt.pos), diffuse=list(lt.diffuse), specular=list(lt.specular),
                     attenuation=list(lt.attenuation))
        runs, tc = 0, time.perf_counter()
        while True:
            O.ssna_frame(a_np, t_np, n_np, pos, d0, du, dv, 60.0, passes=cfg["passes"],
                         lights=[light])
            runs += 1
            if time.perf_counter() - tc > 10.0 or runs >= 200:
                break
        cpu_s = (time.perf_counter() - tc) / runs
        line["cpu_baseline"] = {
            "value": round(sw * sh / cpu_s / 1e6, 4), "unit": "Mpixels/s", "cores": 1,
            "kind": "port",
            "sample": f"post chain only on the central {sw}x{sh} crop of the device's unlit "
                      f"trace, numpy FP32 restatement, {runs} runs"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="yoxel", choices=["yoxel", "reference"])
    ap.add_argument("--config", default="cfg2", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", type=int, default=None, choices=[0, 1, 2, 3],
                    help="brick pool format for the brick workload (default: the config's)")
    ap.add_argument("--seed", type=int, default=SEED,
                    help="seed of the synthetic scene, volume or batch (default 1234; other "
                         "seeds give the run-to-run variance over scenes)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    cfg = with_seed(CONFIGS[args.config], args.seed)
    import importlib.util
    spec = importlib.util.spec_from_file_location("_gentry", os.path.join(ROOT, "__graft_entry__.py"))
    ge = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ge)
    ge.build()
    if args.impl == "reference":
        return run_reference(args, cfg)
    if cfg["kind"] == "svo":
        return run_svo(args, cfg)
    if cfg["kind"] == "brick":
        return run_brick(args, cfg)
    if cfg["kind"] == "train":
        return run_train(args, cfg)
    if cfg["kind"] == "batch":
        return run_batch(args, cfg)
    if dist_env()[0] > 1:
        # the multi-GPU forms: one frame split by tile ranges (SVO and brick
        # frames), data-parallel training, a batch split by scenes; the
        # builders and the edit loop run on one GPU
        raise SystemExit(f"--gpus > 1 runs the frame, training and batch workloads (cfg1-5, "
                         f"lod); run {args.config} on one GPU")
    if cfg["kind"] == "build":
        return run_build(args, cfg)
    if cfg["kind"] == "vbuild":
        return run_vbuild(args, cfg)
    if cfg["kind"] == "dynsync":
        return run_dynsync(args, cfg)
    if cfg["kind"] == "ssna":
        return run_ssna(args, cfg)
    raise SystemExit(f"unknown workload kind {cfg['kind']}")


if __name__ == "__main__":
    main()
