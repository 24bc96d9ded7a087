#!/usr/bin/env python3
"""Benchmark of the GB300 path-tracer hot path: Mpaths/s on the mid scene.

Workload (one step = one full frame): 1,000,010 triangles (400 seeded UV spheres of 2,500
triangles on a 20 x 20 ground quad), 60/30/10 % Lambertian / modified Phong / dielectric,
4 quad lights, SAH kd-tree with Milton's defaults except the traversal cost (the renderer's
default, MGPU_KD_COST_TRAVERSAL = 3; the CPU baseline builds Milton's own), 1024 x 1024 pixels x
64 spp = 67,108,864 paths, max depth 8, Russian roulette from depth 3, noDirectSamples 1.

Printed JSON line (rank 0):
  value       Mpaths/s with the scene resident in HBM (device-timed, max over ranks)
  e2e         the same through the public API with host buffers: per step the scene upload
              (host -> device), the render and the film read-back (device -> host)
  roofline    the dominant kernel's algorithmic bytes (traversal counters x bytes per node,
              leaf reference and triangle) over its CUDA-event time, against the measured
              HBM copy bandwidth
  cpu_baseline  the FP64 oracle (port of Milton's PathTracer) on a bounded pixel subset

`--impl reference` times the CPU implementation of the path -- the FP64 oracle port of Milton's
PathTracer (Milton's renderer needs Boost, Qt 4 and OpenGL and does not build here; its kd-tree and
triangle code do, and pin the oracle's intersections) -- on the same bounded sample of the same
workload as the cpu_baseline leg, with every host thread, and prints its own line.

Other workloads (`--workload`): plain (the CPU-runnable 256 x 256 x 16 spp frame, same line
format, CPU baseline over the whole frame), batched (64 scenes rendered one by one and as one
batch) and serving (a Poisson request stream through the render service, p50/p99 latency).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mpaths/s at 1 GB300 at fixed RMSE vs FP64 ref; served p50/p99 latency"
UNIT = "Mpaths/s"
SEED = 0
# The frame workloads: mid (the benchmark line) and plain (the CPU-runnable configuration).
CONFIGS = {
    "mid": dict(scene="mid", width=1024, height=1024, spp=64, max_depth=8, rr_start=3,
                cpu_rows=(496, 528),  # the bounded CPU sample: 32 rows of the frame, every pass
                hispp_rows=(508, 512), hispp_spp=1024,  # the FP64 high-spp image of the parity check
                workload=("mid: 1,000,010 triangles (400 seeded UV spheres x 2,500 tris on a 20x20 ground quad), "
                          "60/30/10% Lambertian/modified-Phong/dielectric(IOR 1.5), 4 quad lights, SAH kd-tree "
                          "(Milton's parameters, traversal cost 3; the CPU baseline: Milton's, cost 1), "
                          "1024x1024 px, 64 spp, max depth 8, RR from depth 3, fp32")),
    "plain": dict(scene="plain", width=256, height=256, spp=16, max_depth=5, rr_start=3,
                  cpu_rows=(0, 256),  # the whole frame
                  hispp_rows=(120, 136), hispp_spp=1024,
                  workload=("plain: closed box of 5 quads + 2 rotated boxes (34 triangles), one 0.25-area quad "
                            "light of radiance 15, Lambertian albedos U[0.2, 0.8], 256x256 px, 16 spp, max depth 5, "
                            "RR from depth 3, 40 degree pinhole, fp32")),
}
CFG = CONFIGS["mid"]
W_IMG = H_IMG = CFG["width"]
SPP = CFG["spp"]
MAX_DEPTH = CFG["max_depth"]
RR_START = CFG["rr_start"]
WORKLOAD = CFG["workload"]
CPU_ROWS = CFG["cpu_rows"]


def _use_config(name: str) -> None:
    """Points the frame-workload constants at CONFIGS[name]."""
    global CFG, W_IMG, H_IMG, SPP, MAX_DEPTH, RR_START, WORKLOAD, CPU_ROWS
    CFG = CONFIGS[name]
    W_IMG, H_IMG, SPP = CFG["width"], CFG["height"], CFG["spp"]
    MAX_DEPTH, RR_START, WORKLOAD, CPU_ROWS = CFG["max_depth"], CFG["rr_start"], CFG["workload"], CFG["cpu_rows"]


def _frame_scene():
    from milton_gb300 import scenegen
    return scenegen.mid(SEED) if CFG["scene"] == "mid" else scenegen.plain(SEED)


def _peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def _l2_read_peak() -> float:
    """GB/s of reading an L2-resident 32 MiB buffer 400 times in one launch with L2-only loads
    (mgpu_measure_read_bandwidth), best of 3: the denominator of the traversal kernels' L2
    roofline, whose working set is served from L2."""
    from milton_gb300 import pathtracer as pt
    return max(pt.measure_read_bandwidth(32 << 20, 400) for _ in range(3))


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


L2_NOTE = "a 256 MiB buffer (larger than the 129 MB L2) is written before every step"
# The CPU sample (cpu_baseline leg and the reference arm) uses its own seed, independent of the
# GPU frame's, so that its image also serves the z-test on per-pixel means.
CPU_SEED = SEED + 1
HISPP_SEED = SEED + 2


def _config(ws: int) -> dict:
    """The workload description, identical in both arms' lines."""
    return {"workload": WORKLOAD, "l2": L2_NOTE,
            "parallelism": f"replicas x{ws} (independent sample streams, no collective in the step)"}


def _cpu_sample_text(threads: int) -> str:
    return (f"rows {CPU_ROWS[0]}-{CPU_ROWS[1] - 1} of the {CFG['scene']} frame ({CPU_ROWS[1] - CPU_ROWS[0]} x {W_IMG} "
            f"px x {SPP} spp = {W_IMG * (CPU_ROWS[1] - CPU_ROWS[0]) * SPP} paths), FP64 oracle port of Milton's "
            f"PathTracer, {threads} threads, work handed out in 32-pixel spans")


def _cpu_sample(scene, tree=None, threads=None, per_path=False):
    """Times the oracle (FP64 restatement of Milton's PathTracer) on the bounded pixel subset
    CPU_ROWS, every sample pass, seed CPU_SEED."""
    from oracle import pyoracle
    t0 = time.perf_counter()
    tree = tree or pyoracle.Tree(scene.tri_v)
    build_s = time.perf_counter() - t0
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    mean, paths, st = pyoracle.render(scene, tree, W_IMG, H_IMG, SPP, max_depth=MAX_DEPTH, rr_start=RR_START,
                                      seed=CPU_SEED, rows=CPU_ROWS, threads=threads, per_path=per_path)
    dt = time.perf_counter() - t0
    n = W_IMG * (CPU_ROWS[1] - CPU_ROWS[0]) * SPP
    return dict(mpaths=n / dt / 1e6, seconds=dt, paths=n, threads=threads, build_s=build_s, mean=mean,
                per_path=paths, stats=st, tree=tree)


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    scene = _frame_scene()
    from oracle import pyoracle
    tree = pyoracle.Tree(scene.tri_v)
    threads = os.cpu_count() or 1
    times = []
    paths_per_step = 0
    for k in range(args.warmup + args.steps):
        r = _cpu_sample(scene, tree=tree, threads=threads)
        paths_per_step = r["paths"]
        if k >= args.warmup:
            times.append(r["seconds"])
    total = sum(times)
    value = paths_per_step * len(times) / total / 1e6
    sample = "each step: " + _cpu_sample_text(threads)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": _config(ws),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _luminance(x):
    return x.mean(axis=-1)


def _image_parity(scene, dscene, tree, W, H, spp, depth, rr, rows_z, rows_hi, hispp_spp, pt, torch, film=None,
                  img=None, oracle_band=None, ns=4, camera=None, stream=0):
    """Parity of a rendered image against the FP64 oracle (rank 0, after the timed region):
      path_agreement   per-path radiance, GPU vs oracle with the same seed and counter RNG, on
                       rows_z at the first ns passes (within 1e-4 + 2e-3 relative)
      z                per-pixel mean luminance of the GPU image (seed SEED, all spp passes)
                       against the oracle's (seed CPU_SEED, independent) on rows_z: z = difference
                       / standard error; z_frac = fraction of pixels with |z| > 4
      rmse_*_vs_fp64_hispp  RMSE of the GPU image and of the oracle image, both at spp, against an
                       FP64 oracle image of rows_hi at hispp_spp passes (seed HISPP_SEED)
    film / img: the GPU film and its mean when the caller already rendered them (else rendered
    here); oracle_band: the oracle's rows_z render (mean, per_path) when already made."""
    import numpy as np
    from oracle import pyoracle
    r0, r1 = rows_z
    h0, h1 = rows_hi
    assert r0 <= h0 and h1 <= r1
    kw = {} if camera is None else {"camera": camera}
    if film is None:
        film = pt.Film(W, H)
        pt.render(dscene, pt.RenderSettings(W, H, spp, max_depth=depth, rr_start_depth=rr, seed=SEED, stream_id=stream),
                  film, **kw)
        img = film.mean()
    # same-sample per-path agreement
    out = torch.zeros((W * H * ns, 4), dtype=torch.float32, device="cuda")
    pf = pt.Film(W, H)
    pt.render(dscene, pt.RenderSettings(W, H, spp, sample_count=ns, max_depth=depth, rr_start_depth=rr, seed=SEED,
                                        stream_id=stream), pf, path_out=out, **kw)
    torch.cuda.synchronize()
    pg = out.cpu().numpy().reshape(H, W, ns, 4)[r0:r1, ..., :3].astype(np.float64)
    del out
    pf.close()
    oscene = scene if camera is None else _with_camera(scene, camera)
    _, po, _ = pyoracle.render(oscene, tree, W, H, spp, sample_count=ns, max_depth=depth, rr_start=rr, seed=SEED,
                               stream=stream, rows=rows_z, per_path=True)
    close = np.abs(pg - po) <= 1e-4 + 2e-3 * np.maximum(np.abs(pg), np.abs(po))
    agree = float(np.all(close, axis=-1).mean())
    # z-test on per-pixel mean luminance, independent seeds
    if oracle_band is None:
        m, pp, _ = pyoracle.render(oscene, tree, W, H, spp, max_depth=depth, rr_start=rr, seed=CPU_SEED, rows=rows_z,
                                   per_path=True)
        oracle_band = {"mean": m, "per_path": pp}
    raw = film.raw()[:, r0:r1].astype(np.float64)  # [0]: sum rgb, count; [1]: compensation rgb, sum of lum^2
    n_g = raw[0, ..., 3]
    m_g = _luminance(img[r0:r1])
    v_g = np.maximum(raw[1, ..., 3] / n_g - m_g ** 2, 0.0) * n_g / np.maximum(n_g - 1, 1)
    lo = _luminance(oracle_band["per_path"])  # (rows, W, spp)
    n_o = lo.shape[-1]
    m_o = lo.mean(-1)
    v_o = lo.var(-1, ddof=1) if n_o > 1 else np.zeros_like(m_o)
    se = np.sqrt(v_g / n_g + v_o / n_o)
    with np.errstate(divide="ignore", invalid="ignore"):
        z = np.where(se > 0, (m_g - m_o) / se, 0.0)
    z_frac = float((np.abs(z) > 4).mean())
    # FP64 high-spp image of a few rows
    t0 = time.perf_counter()
    hi, _, _ = pyoracle.render(oscene, tree, W, H, hispp_spp, max_depth=depth, rr_start=rr, seed=HISPP_SEED,
                               rows=rows_hi)
    hi_s = time.perf_counter() - t0
    rmse_g = float(np.sqrt(((img[h0:h1] - hi) ** 2).mean()))
    rmse_o = float(np.sqrt(((oracle_band["mean"][h0 - r0:h1 - r0] - hi) ** 2).mean()))
    return {"path_agreement": agree, "path_agreement_sample": f"rows {r0}-{r1 - 1}, first {ns} of {spp} passes, "
                                                             f"same seed ({W * (r1 - r0) * ns} paths)",
            "z_frac": z_frac, "z_abs_mean": float(np.abs(z).mean()),
            "z_sample": f"rows {r0}-{r1 - 1}, {spp} spp, GPU seed vs an independent oracle seed",
            "rmse_gpu_vs_fp64_hispp": rmse_g, "rmse_oracle_vs_fp64_hispp": rmse_o,
            "rmse_gpu_over_oracle": rmse_g / rmse_o if rmse_o > 0 else None,
            "hispp": f"FP64 oracle, rows {h0}-{h1 - 1}, {hispp_spp} spp, {hi_s:.1f} s",
            "image_mean_gpu": float(img[h0:h1].mean()), "image_mean_fp64_hispp": float(hi.mean())}


def _with_camera(scene, camera):
    import copy
    s2 = copy.copy(scene)
    s2.camera = camera
    return s2


def _frame_parity(scene, dscene, film, img, cpu, pt, torch):
    """The benchmark frame's parity (_image_parity) on the CPU-baseline rows, reusing the
    cpu_baseline leg's oracle render as the independent-seed image."""
    return _image_parity(scene, dscene, cpu["tree"], W_IMG, H_IMG, SPP, MAX_DEPTH, RR_START, CPU_ROWS,
                         CFG["hispp_rows"], CFG["hispp_spp"], pt, torch, film=film, img=img,
                         oracle_band={"mean": cpu["mean"], "per_path": cpu["per_path"]})


def _hit_parity(scene, dscene, tree, n, pt, torch):
    """Closest-hit primitive ids of the GPU against the oracle's kd traversal on n camera rays and
    n rays from random points of the scene's box; a mismatch counts as a tie when the oracle's
    brute force finds the two nearest hits within 1e-6 relative t, or the GPU's t within 1e-6 of
    the oracle's (at most 64 mismatches are classified by brute force)."""
    import numpy as np
    from oracle import pyoracle
    sys.path.insert(0, str(ROOT / "tests"))
    from raygen import camera_rays, classify, sphere_rays
    lo, hi = scene.tri_v.reshape(-1, 3).min(0), scene.tri_v.reshape(-1, 3).max(0)
    rays = np.concatenate([camera_rays(scene.camera, n, 41), sphere_rays(lo, hi, n, 42)])
    h = pt.trace_closest(dscene, torch.from_numpy(rays).cuda())
    torch.cuda.synchronize()
    h = h.cpu().numpy()
    pg, tg = h[:, 1].view(np.int32).astype(np.int64), h[:, 0].astype(np.float64)
    t0 = time.perf_counter()
    to, po, _, _ = pyoracle.trace_closest(tree, scene.tri_v, scene.tri_flags, rays)
    bad = np.nonzero(pg != po)[0]
    classified = bad[:64]
    t2 = np.full(len(rays), np.inf)
    if classified.size:
        _, _, t2b, _ = pyoracle.trace_closest(None, scene.tri_v, scene.tri_flags, rays[classified])
        t2[classified] = t2b
    r = classify(po[classified], to[classified], t2[classified], pg[classified], tg[classified]) \
        if classified.size else {"ties": 0, "mismatches": 0}
    both = (po >= 0) & (pg == po)
    rel = np.abs(tg[both] - to[both]) / np.maximum(to[both], 1e-30)
    return {"rays": int(len(rays)), "identical_ids": int((pg == po).sum()), "differing": int(bad.size),
            "of_which_ties": int(r["ties"]), "of_which_mismatches": int(r["mismatches"]),
            "classified": int(classified.size), "t_rel_err_mean": float(rel.mean()) if rel.size else 0.0,
            "t_abs_err_max_over_max_t_1": float((np.abs(tg[both] - to[both]) / np.maximum(to[both], 1.0)).max())
            if rel.size else 0.0, "oracle_s": round(time.perf_counter() - t0, 1)}


def run_ours(args):
    import numpy as np
    import torch

    from milton_gb300 import pathtracer as pt
    from milton_gb300 import scenegen

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    stream = torch.cuda.current_stream()

    scene = _frame_scene()
    t0 = time.perf_counter()
    accel = pt.Accel(scene)
    build_s = time.perf_counter() - t0
    kst = accel.stats()
    dscene = pt.DeviceScene(scene, accel)
    film = pt.Film(W_IMG, H_IMG)
    # every rank renders its own independent replica of the frame (stream_id = rank)
    settings = pt.RenderSettings(W_IMG, H_IMG, SPP, max_depth=MAX_DEPTH, rr_start_depth=RR_START, seed=SEED,
                                 stream_id=rank)

    # traversal counters on a 4-spp slice of the same frame (untimed): bytes per ray
    cfilm = pt.Film(W_IMG, H_IMG)
    cnt = pt.render_counted(dscene, pt.RenderSettings(W_IMG, H_IMG, SPP, sample_count=4, max_depth=MAX_DEPTH,
                                                      rr_start_depth=RR_START, seed=SEED, stream_id=rank), cfilm)
    cfilm.close()

    def per_ray(prefix, out_bytes):
        n = max(cnt[prefix + "_rays"], 1)
        nodes, refs, tris = cnt[prefix + "_nodes"] / n, cnt[prefix + "_refs"] / n, cnt[prefix + "_tris"] / n
        return dict(nodes=nodes, refs=refs, tris=tris, bytes=32 + out_bytes + 16 * nodes + 4 * refs + 48 * tris)

    ext_ray = per_ray("ext", 16)
    sh_ray = per_ray("sh", 4)

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > 129 MB L2

    def step():
        flush.fill_(1.0)
        film.clear(stream)
        pt.render(dscene, settings, film, stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    clocks = Clocks(dev)
    pt.profile_enable(True)
    launches0 = pt.launch_count()
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    launches = pt.launch_count() - launches0
    prof = pt.profile_read()
    pt.profile_enable(False)
    stats = pt.render_stats()  # of the last step
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    paths_per_step = W_IMG * H_IMG * SPP
    value = paths_per_step * ws * args.steps / (ms / 1e3) / 1e6

    # end to end through the public API with host buffers
    h2d = 0
    d2h = W_IMG * H_IMG * 3 * 8  # the per-pixel FP64 means (mgpu_film_read)

    def e2e_step():
        ds = pt.DeviceScene(scene, accel, stream=stream)
        nbytes = ds.nbytes
        f = pt.Film(W_IMG, H_IMG, stream=stream)
        pt.render(ds, settings, f, stream=stream)
        mean = f.mean(stream)
        f.close()
        ds.close()
        return nbytes, mean

    for _ in range(min(args.warmup, 2)):  # untimed, as the device-timed steps have theirs
        e2e_step()
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        h2d, img = e2e_step()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if ws > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = paths_per_step * ws * args.steps / e2e_s / 1e6

    # once through the renderer object a Milton host drives (Renderer::init: kd build and upload;
    # render; the finalized output read back), so the host kd build is inside the time
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ptr = pt.PathTracer(props={"noSuperSamples": SPP, "maxDepth": MAX_DEPTH, "rrStartDepth": RR_START,
                               "seed": SEED})
    ptr.set_scene(scene)
    ptr.set_output(W_IMG, H_IMG)
    ptr.init()
    ptr.render(stream=stream)
    ptr.output()
    init_s = time.perf_counter() - t0
    e2e_init = {"value": paths_per_step / init_s / 1e6, "unit": UNIT, "seconds": round(init_s, 3),
                "what": "one frame through PathTracer init (host kd build + upload) + render + output read"}
    del ptr

    # roofline of the dominant kernel
    peaks = _peaks()
    ext_ms, ext_n = prof["extend"]
    sh_ms, sh_n = prof["shadow"]
    ext_rays_total = stats["extension_rays"] * args.steps
    sh_rays_total = stats["shadow_rays"] * args.steps
    kern = {"extend": (ext_ms, ext_n, ext_rays_total * ext_ray["bytes"]),
            "shadow": (sh_ms, sh_n, sh_rays_total * sh_ray["bytes"])}
    dom = max(kern, key=lambda k: kern[k][0])
    kms, kn, kbytes = kern[dom]
    achieved = (kbytes / max(kn, 1)) / ((kms / max(kn, 1)) / 1e3) / 1e9
    # DRAM traffic per launch: the ncu capture of the same kernel on the small case gives DRAM
    # bytes per ray (profiles/traffic_per_ray.json); scaled here by the rays of an average launch
    traffic = None
    l2 = None
    tfile = ROOT / "profiles" / "traffic_per_ray.json"
    if tfile.exists():
        tr = json.loads(tfile.read_text()).get(dom, {})
        per_ray = tr.get("dram_bytes_per_ray")
        rays_total = ext_rays_total if dom == "extend" else sh_rays_total
        if per_ray:
            traffic = per_ray * rays_total / max(kn, 1)
        # the L2 roofline: the kernel's L2 traffic (ncu lts__t_bytes per ray of the same kernel on
        # the small case, times the rays of an average launch) over its launch time, against the
        # measured copy bandwidth of an L2-resident buffer
        l2_per_ray = tr.get("l2_bytes_per_ray")
        if l2_per_ray:
            l2_peak = _l2_read_peak()
            l2_ach = (l2_per_ray * rays_total / max(kn, 1)) / ((kms / max(kn, 1)) / 1e3) / 1e9
            l2 = {"achieved": l2_ach, "peak": l2_peak, "unit": "GB/s", "frac": l2_ach / l2_peak,
                  "bytes_per_ray": l2_per_ray, "peak_source": "measured: reads of a 32 MiB L2-resident buffer, one launch"}

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded scene generator, no external assets)",
        "config": _config(ws),
        "details": {"paths_per_step": paths_per_step,
                    "wave_paths": "automatic (up to 2^26 paths per wave, workspace within 40 GB)",
                    "kd_build_s": round(build_s, 3), "kd_nodes": kst["node_pairs"], "kd_refs": kst["refs"],
                    "rays_per_path": (stats["extension_rays"] + stats["shadow_rays"]) / paths_per_step,
                    "mrays_per_s": value * (stats["extension_rays"] + stats["shadow_rays"]) / paths_per_step},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "e2e_with_init": e2e_init,
        "gpu_launches": int(launches),
        "kernels_ms": {k: round(v[0], 3) for k, v in prof.items()},
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                     "peak_source": peaks["source"] + " copy bandwidth",
                     "bytes_per_ray": {"extend": ext_ray, "shadow": sh_ray}, "l2": l2},
        "clocks": clk,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = _cpu_sample(scene, per_path=True)
        out["cpu_baseline"] = {"value": cpu["mpaths"], "unit": UNIT, "cores": cpu["threads"], "kind": "port",
                               "sample": _cpu_sample_text(cpu["threads"]), "seconds": round(cpu["seconds"], 2)}
        out["parity"] = _frame_parity(scene, dscene, film, img, cpu, pt, torch)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_batched(args):
    """Batched configuration: 64 seeded scenes of uneven size, 128^2-1024^2, 16 spp each.
    Times the same requests rendered one after another with mgpu_render (plain) and together in
    one autotuned, graph-captured batch."""
    import torch

    from milton_gb300 import autotune
    from milton_gb300 import pathtracer as pt
    from milton_gb300 import workloads
    torch.cuda.set_device(0)
    specs = workloads.batched_specs(SEED)
    reqs = []
    t0 = time.perf_counter()
    for k, sp in enumerate(specs):
        s = workloads.build_scene(sp)
        ds = pt.DeviceScene(s, pt.Accel(s))
        reqs.append((ds, pt.RenderSettings(sp["width"], sp["height"], sp["spp"], max_depth=MAX_DEPTH,
                                           rr_start_depth=RR_START, seed=SEED, stream_id=k)))
    setup_s = time.perf_counter() - t0
    films = [pt.Film(st.width, st.height) for _, st in reqs]
    paths = sum(st.width * st.height * st.spp for _, st in reqs)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    def plain():
        for (ds, st), f in zip(reqs, films):
            f.clear()
            pt.render(ds, st, f)

    ms_plain = timed(plain)
    tuned = autotune.tune(reqs)
    batch = pt.Batch(wave_paths=tuned["wave_paths"], use_graph=True)
    for (ds, st), f in zip(reqs, films):
        batch.add(ds, st, f)

    def batched():
        for f in films:
            f.clear()
        batch.render()

    ms_batch = timed(batched)
    tris = sum(ds.scene.ntri for ds, _ in reqs)
    parity = None
    if not args.no_parity:
        # one representative request (median triangle count among the frames of at most 512
        # pixels a side) as the batch left it, against the FP64 oracle
        from oracle import pyoracle
        cand = sorted((ds.scene.ntri, k) for k, (ds, st) in enumerate(reqs) if st.width <= 512)
        k = cand[len(cand) // 2][1]
        ds, st = reqs[k]
        f = films[k]
        mid_row = st.height // 2
        parity = {"request": k, "triangles": ds.scene.ntri, "size": [st.width, st.height], "spp": st.spp}
        parity.update(_image_parity(ds.scene, ds, pyoracle.Tree(ds.scene.tri_v), st.width, st.height, st.spp,
                                    MAX_DEPTH, RR_START, (mid_row - 8, mid_row + 8), (mid_row - 1, mid_row + 1), 1024,
                                    pt, torch, film=f, img=f.mean(), stream=k))
    out = {"metric": METRIC, "workload": "batched", "value": paths / ms_batch / 1e3, "unit": UNIT,
           "plain_value": paths / ms_plain / 1e3, "batched_over_plain": ms_plain / ms_batch,
           "ms_per_step": ms_batch, "plain_ms_per_step": ms_plain, "steps": args.steps, "warmup": args.warmup,
           "config": {"scenes": len(reqs), "triangles": tris, "paths_per_step": paths,
                      "setup_s": round(setup_s, 1), "autotuned": tuned}, "parity": parity}
    print(json.dumps(out), flush=True)
    return 0


def run_serving(args):
    """Serving configuration: a Poisson request stream (200 req/s) over 8 resident scenes of
    10k-2M triangles, resolutions {256, 512, 1024, 2048}^2, target spp {1, 16, 64, 256}, each
    job refined progressively until its film's error estimate is at most 0.01 (or the target
    spp), admitted by a 120 GB budget.  Reports throughput and p50/p99 time-to-target, and
    times the same jobs (same final sample counts, hence the same images) rendered one after
    another with mgpu_render (plain)."""
    import numpy as np
    import torch

    from milton_gb300 import pathtracer as pt
    from milton_gb300 import workloads
    from milton_gb300.serving import Server, ServerSettings, latency_summary, replay
    torch.cuda.set_device(0)
    specs, reqs = workloads.serving_requests(SEED, n=args.requests, rate=args.rate)
    t0 = time.perf_counter()
    scenes = [workloads.build_scene(sp) for sp in specs]
    gen_s = time.perf_counter() - t0
    settings = ServerSettings(hbm_budget=120_000_000_000, tick_paths=args.tick_paths, use_graph=args.graph,
                              policy=args.policy)
    srv = Server(settings)
    ids = [srv.add_scene(s) for s in scenes]
    t0 = time.perf_counter()
    for i in ids:
        srv.prefetch(i)
    srv.wait_builds()
    build_s = time.perf_counter() - t0
    target_rmse = 0.01

    def make_job(r):
        st = pt.RenderSettings(r["width"], r["height"], min(r["spp"], 16), max_depth=MAX_DEPTH,
                               rr_start_depth=RR_START, seed=r["seed"], stream_id=r["id"])
        cam = workloads.request_camera(scenes[r["scene"]].camera, r["seed"])
        return ids[r["scene"]], st, cam, r["spp"], target_rmse

    # warm-up: every scene uploaded and the wave workspace allocated before the clock starts
    warm = [dict(id=10_000 + k, arrival=0.0, scene=k, width=256, height=256, spp=1, seed=k)
            for k in range(len(scenes))]
    replay(srv, warm, make_job)
    s0 = srv.stats()
    check_ids = {r["id"] for r in reqs[:4]}
    served_imgs = {}

    def on_done(r, jid, info):
        if r["id"] in check_ids:
            served_imgs[r["id"]] = srv.read(jid)

    clocks = Clocks(0)
    clocks.start()
    infos, t_start = replay(srv, reqs, on_done=on_done, make_job=make_job)
    clk = clocks.stop()
    s1 = srv.stats()
    paths = s1["paths"] - s0["paths"]
    busy = s1["render_seconds"] - s0["render_seconds"]
    t_end = max(v["t_done"] for v in infos.values())
    lat = latency_summary(infos)
    srv.close()

    # plain: the same jobs, one after another, each alone with mgpu_render
    dscenes = [pt.DeviceScene(s, pt.Accel(s)) for s in scenes]
    jobs = []
    for r in reqs:
        info = infos[r["id"]]
        sid, st, cam, _, _ = make_job(r)
        st.sample_count = info["spp_done"]
        jobs.append((r, st, cam))
    films = {}
    for r, st, cam in jobs:
        if (st.width, st.height) not in films:
            films[(st.width, st.height)] = pt.Film(st.width, st.height)
    same = []
    for r, st, cam in jobs:  # warm-up and image check
        if r["id"] in check_ids:
            f = films[(st.width, st.height)]
            f.clear()
            pt.render(dscenes[r["scene"]], st, f, camera=cam)
            same.append(bool(np.array_equal(f.mean(), served_imgs[r["id"]])))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for r, st, cam in jobs:
        f = films[(st.width, st.height)]
        f.clear()
        pt.render(dscenes[r["scene"]], st, f, camera=cam)
    e1.record()
    torch.cuda.synchronize()
    plain_s = e0.elapsed_time(e1) / 1e3
    stop_rule = None
    if not args.no_parity:
        # the stop rule against an FP64 image: for up to three jobs that stopped at their error
        # target (the smallest frames on the smallest scenes), the luminance RMSE of the served
        # image against a 1024-spp FP64 oracle image of 8 rows, beside the film's estimate
        import numpy as np
        from oracle import pyoracle
        done_early = [r for r in reqs if infos[r["id"]]["reached_target"] and r["width"] <= 512]
        done_early.sort(key=lambda r: (scenes[r["scene"]].ntri, r["width"]))
        trees = {}
        stop_rule = []
        for r in done_early[:3]:
            info = infos[r["id"]]
            sid, st, cam, _, _ = make_job(r)
            st.sample_count = info["spp_done"]
            f = films[(st.width, st.height)]
            f.clear()
            pt.render(dscenes[r["scene"]], st, f, camera=cam)  # the served image (equal to it, checked above)
            img = f.mean()
            if r["scene"] not in trees:
                trees[r["scene"]] = pyoracle.Tree(scenes[r["scene"]].tri_v)
            h0 = st.height // 2 - 4
            t0 = time.perf_counter()
            hi, _, _ = pyoracle.render(_with_camera(scenes[r["scene"]], cam), trees[r["scene"]], st.width, st.height,
                                       1024, max_depth=MAX_DEPTH, rr_start=RR_START, seed=HISPP_SEED, rows=(h0, h0 + 8))
            rm = float(np.sqrt(((_luminance(img[h0:h0 + 8]) - _luminance(hi)) ** 2).mean()))
            stop_rule.append({"request": r["id"], "size": st.width, "triangles": scenes[r["scene"]].ntri,
                              "spp_done": info["spp_done"], "target_rmse": target_rmse,
                              "estimated_rmse": info["rmse"], "rmse_vs_fp64_1024spp_8_rows": rm,
                              "oracle_s": round(time.perf_counter() - t0, 1)})
    spp_hist = {}
    for v in infos.values():
        spp_hist[v["spp_done"]] = spp_hist.get(v["spp_done"], 0) + 1
    out = {"metric": METRIC, "workload": "serving", "value": paths / busy / 1e6, "unit": UNIT,
           "wall_value": paths / (t_end - t_start) / 1e6, "plain_value": paths / plain_s / 1e6,
           "served_over_plain": plain_s / busy, "latency": lat, "images_equal_plain": same,
           "stop_rule_vs_fp64": stop_rule,
           "clocks": clk,
           "config": {"requests": len(reqs), "rate_per_s": args.rate, "scenes": len(scenes),
                      "triangles": [s.ntri for s in scenes], "target_rmse": target_rmse,
                      "hbm_budget": settings.hbm_budget, "tick_paths": settings.tick_paths,
                      "use_graph": settings.use_graph, "policy": settings.policy, "paths": paths,
                      "busy_s": round(busy, 3),
                      "wall_s": round(t_end - t_start, 3), "plain_s": round(plain_s, 3),
                      "peak_resident_bytes": s1["peak_resident_bytes"], "ticks": s1["ticks"] - s0["ticks"],
                      "spp_done_histogram": {str(k): v for k, v in sorted(spp_hist.items())},
                      "scene_gen_s": round(gen_s, 1), "kd_build_s": round(build_s, 1)}}
    print(json.dumps(out), flush=True)
    return 0


def run_large(args):
    """Large configuration: ~20 M triangles (fBm terrain + 2,000 copied spheres), 16 quad
    lights, 2048 x 2048 x 128 spp, depth 16.  A step renders 16 of the 128 sample passes
    (33,554,432 paths); the full frame is 8 steps.  The kd-tree is built with kdMaxDepth 32:
    Milton's default 24 suits scenes of ~10^5 triangles and leaves 15 triangles per leaf here
    (measured 26.7 vs 41.5 Mpaths/s)."""
    import torch

    from milton_gb300 import pathtracer as pt
    from milton_gb300 import scenegen
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    scene = scenegen.large(SEED)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    kd_depth = 32
    accel = pt.Accel(scene, pt.KdSettings(max_depth=kd_depth))
    build_s = time.perf_counter() - t0
    kst = accel.stats()
    dscene = pt.DeviceScene(scene, accel)
    W = H = 2048
    spp, per_step, depth = 128, 16, 16
    film = pt.Film(W, H)
    stream = torch.cuda.current_stream()
    k = [0]

    def step():
        s0 = (k[0] * per_step) % spp
        k[0] += 1
        pt.render(dscene, pt.RenderSettings(W, H, spp, sample_begin=s0, sample_count=per_step, max_depth=depth,
                                            rr_start_depth=RR_START, seed=SEED), film, stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    pt.profile_enable(True)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    prof = pt.profile_read()
    pt.profile_enable(False)
    stats = pt.render_stats()
    ms = e0.elapsed_time(e1) / args.steps
    paths = W * H * per_step
    out = {"metric": METRIC, "workload": "large", "value": paths / ms / 1e3, "unit": UNIT, "ms_per_step": ms,
           "full_frame_s": ms * spp / per_step / 1e3, "steps": args.steps, "warmup": args.warmup,
           "mrays_per_s": (stats["extension_rays"] + stats["shadow_rays"]) / ms / 1e3,
           "kernels_ms": {k_: round(v[0], 3) for k_, v in prof.items()}, "clocks": clk,
           "config": {"triangles": scene.ntri, "lights": len(scene.lights), "width": W, "height": H, "spp": spp,
                      "passes_per_step": per_step, "max_depth": depth, "rr_start": RR_START,
                      "scene_gen_s": round(gen_s, 1), "kd_build_s": round(build_s, 1),
                      "kd_max_depth_param": kd_depth, "kd_node_pairs": kst["node_pairs"], "kd_refs": kst["refs"],
                      "kd_leaf_depth_max": kst["max_depth"],
                      "device_scene_bytes": dscene.nbytes,
                      "cpu_baseline": "not run here: the mid line carries the CPU baseline"}}
    if not args.no_parity:
        # parity against the FP64 oracle, which traverses the product's tree read from its
        # serialisation (node-for-node the tree its own restated build gives, tests/test_kdtree.py;
        # that build takes minutes at 20 M triangles)
        from oracle import pyoracle
        t0 = time.perf_counter()
        tree = pyoracle.Tree.from_serial(scene.tri_v, *accel.serialize())
        out["parity"] = {"hit_ids": _hit_parity(scene, dscene, tree, 1 << 15, pt, torch),
                         "oracle_tree": "the product's tree from its serialisation",
                         "oracle_tree_s": round(time.perf_counter() - t0, 1)}
        out["parity"].update(_image_parity(scene, dscene, tree, W, H, spp, depth, RR_START, (1020, 1024), (1022, 1023),
                                           512, pt, torch, ns=1))
    print(json.dumps(out), flush=True)
    return 0


def run_profile_case(args):
    """Small case for ncu captures: the mid scene (~143 MB resident, larger than the 129 MB
    L2) at 512 x 512 x 4 spp = 1,048,576 paths per frame, two frames."""
    import torch

    from milton_gb300 import pathtracer as pt
    from milton_gb300 import scenegen
    for kv in args.tune:  # knobs of the captured kernels, e.g. --tune smem_stack=4
        k, v = kv.split("=")
        pt.tune(k, int(v))
    s = scenegen.mid(SEED)
    ds = pt.DeviceScene(s, pt.Accel(s))
    film = pt.Film(512, 512)
    st = pt.RenderSettings(512, 512, 4, max_depth=MAX_DEPTH, rr_start_depth=RR_START, seed=SEED)
    for _ in range(2):
        pt.render(ds, st, film)
    torch.cuda.synchronize()
    ext, sh = pt.wave_queues(MAX_DEPTH)
    print(json.dumps({"profile_case": "mid 512x512x4spp x2", **pt.render_stats(),
                      "extension_rays_per_bounce": ext.tolist(), "shadow_rays_per_bounce": sh.tolist()}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="batched / serving / large: skip the FP64 parity check")
    ap.add_argument("--profile-case", action="store_true", help="small two-frame case for ncu captures")
    ap.add_argument("--tune", action="append", default=[], metavar="KEY=VALUE",
                    help="profile case: a tuning knob (mgpu_tune_set) to set first; repeatable")
    ap.add_argument("--workload", default="mid", choices=["mid", "plain", "batched", "serving", "large"],
                    help="mid (default, the benchmark line), plain (the CPU-runnable frame), batched (64 scenes, "
                         "batch vs one-by-one) or serving (Poisson request stream through the render service)")
    ap.add_argument("--requests", type=int, default=200, help="serving: requests in the stream")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: arrivals per second")
    ap.add_argument("--tick-paths", type=int, default=1 << 26, help="serving: paths per scheduling tick")
    ap.add_argument("--graph", type=int, default=0, help="serving: capture each tick in a CUDA graph")
    ap.add_argument("--policy", default="rotate", choices=["fair", "oldest", "rotate"],
                    help="serving: tick scheduling policy")
    args = ap.parse_args()
    if args.profile_case:
        return run_profile_case(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "large":
        args.warmup = max(args.warmup, 3)
        return run_large(args)
    if args.workload == "batched":
        if args.warmup < 3:
            args.warmup = 3
        return run_batched(args)
    if args.warmup < 3:
        args.warmup = 3
    _use_config("plain" if args.workload == "plain" else "mid")
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
