#!/usr/bin/env python3
"""Benchmark: BVH closest-hit traversal throughput (Mrays/s) on the 1,310,720-triangle
displaced icosphere with 2^23 rays, on one GB300 per rank.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one closest-hit pass (ckr_trace_closest) over the 2^23-ray batch
(4,194,304 primary rays of a 2048x2048 pinhole camera at distance 3 + 4,194,304
incoherent rays, origins uniform in the mesh AABB, directions uniform, seed 7), inputs
resident in HBM.  `e2e` is the same metric through ckr_trace_closest_host with pinned
host buffers (ray upload and hit download inside the timed region).  Rank 0 prints one
JSON line.  Under torchrun each rank traces its own copy of the batch (weak scaling, no
data-path collective).  `--impl reference` times the reference's CPU traversal
(BvhAccel::intersectT) on the host cores: its FP64 restatement in oracle/, on inputs made
by the oracle's own generator (that process never loads libckr.so), the full batch per
step unless the run would exceed a few minutes.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mrays/s at 1.3M tris; relMSE at equal time, learned vs plain MIS, 1 GB300"
UNIT = "Mrays/s"
NRAYS_HALF = 4194304
WORKLOAD = ("bvh-traversal: displaced icosphere (8 subdivisions, 1,310,720 tris, value-noise amp 0.05, "
            "6 octaves), 2^23 rays = 4,194,304 primary (2048x2048 pinhole, distance 3, 40 deg) + "
            "4,194,304 incoherent (uniform in AABB, uniform directions, seed 7); closest-hit")


def make_workload():
    from chakumrender_gb300 import ckr

    tri = ckr.icosphere(8, 0.05, 6, 1)
    lo, hi = tri.reshape(-1, 3).min(0), tri.reshape(-1, 3).max(0)
    primary = ckr.rays_pinhole([0, 0, 3], [0, 0, 0], [0, 1, 0], 40.0, 2048, 2048)
    incoh = ckr.rays_incoherent(lo, hi, 7, NRAYS_HALF, 0.05, 2.0)
    closest = np.concatenate([primary, incoh])
    anyhit = closest.copy()
    closest[:, 7] = 1e30
    return tri, closest, anyhit


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profile():
    """Per-launch DRAM bytes of the closest-hit kernel from the committed ncu summary."""
    f = ROOT / "profiles" / "trace_closest_icosphere_1310720.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.strip().startswith("dram_bytes_per_launch"):
            try:
                return float(line.split("=")[1].split()[0])
            except (IndexError, ValueError):
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def build_oracle_only():
    """Compiles oracle/liboracle.so (the FP64 C restatement) with make, without
    importing the package, so that a process which only times the CPU port never
    loads libckr.so."""
    r = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), f"-j{min(16, os.cpu_count() or 4)}", "all"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise SystemExit(f"oracle build failed:\n{r.stdout}\n{r.stderr}")


def make_workload_oracle():
    """The same inputs as make_workload(), generated by the oracle's C restatement
    (byte-identical to ckr_workload_*, checked by tests/test_workloads.py)."""
    import oracle as O

    tri = O.icosphere(8, 0.05, 6, 1)
    lo, hi = tri.reshape(-1, 3).min(0), tri.reshape(-1, 3).max(0)
    primary = O.rays_pinhole([0, 0, 3], [0, 0, 0], [0, 1, 0], 40.0, 2048, 2048)
    incoh = O.rays_incoherent(lo, hi, 7, NRAYS_HALF, 0.05, 2.0)
    closest = np.concatenate([primary, incoh])
    closest[:, 7] = 1e30
    return tri, closest


def bench_config(n_rays: int, ntri: int, world: int) -> dict:
    """The workload's config; identical in both arms."""
    return {"workload": WORKLOAD, "rays_per_step": n_rays, "triangles": ntri,
            "l2": "inputs larger than L2 (rays 256 MiB), no flush", "parallelism": f"replica x{world}"}


REF_BUDGET_S = 180.0  # whole --impl reference run (warm-up + timed steps)


def run_reference(args, rank, world):
    """CPU arm: the reference's closest-hit traversal (BvhAccel::intersectT over its
    midpoint BVH, src/bvhAccel.cpp:13-249) on all host cores, as the oracle's FP64
    restatement (the reference's own objects are x86 builds from sources that are not
    on the GPU host).  Inputs come from the oracle's generator: this process loads
    only oracle/liboracle.so.  Each step traces the full 2^23-ray batch unless the
    projected run exceeds REF_BUDGET_S, in which case later steps trace a stride
    sample (reported in config and cpu_baseline)."""
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    build_oracle_only()
    import oracle as O

    tri, closest = make_workload_oracle()
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    ob = O.OracleBvh(tri)
    build_s = time.perf_counter() - t0
    n = len(closest)
    t0 = time.perf_counter()
    ob.closest(closest, threads=cores)  # first warm-up step, full batch
    t_full = time.perf_counter() - t0
    total = args.warmup + args.steps
    rays = closest
    if t_full * total > REF_BUDGET_S:
        stride = 1
        while t_full / stride * (total - 1) + t_full > REF_BUDGET_S:
            stride *= 2
        rays = np.ascontiguousarray(closest[::stride])
    times = []
    for k in range(1, total):
        t0 = time.perf_counter()
        ob.closest(rays, threads=cores)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
    if args.warmup == 0:
        times.insert(0, t_full)
    m = len(rays)
    full = m == n
    sample = ("full 2^23-ray batch every step" if full else
              f"{m} rays per step (stride-{n // m} sample of the 2^23-ray batch; the full batch took {t_full:.2f} s)")
    mrays = m * len(times) / sum(times) / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": round(mrays, 4), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sum(times) / len(times), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(n if full else m, len(tri), world),
            "structure": {"bvh": f"the reference's midpoint BVH, one triangle per leaf ({ob.node_count()} nodes)",
                          "bvh_build_s": round(build_s, 3)},
            "cpu_baseline": {"value": round(mrays, 4), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample + "; FP64 restatement of BvhAccel::intersectT, inputs from the "
                                                "oracle's generator"},
            "e2e": {"value": round(mrays, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline(tri, closest):
    """The oracle port of the reference traversal on the host cores over the full
    2^23-ray batch (one pass, about 1.5 s on 16 cores), with per-ray node and
    triangle counts of the reference's midpoint BVH."""
    sys.path.insert(0, str(ROOT / "oracle"))
    build_oracle_only()
    import oracle as O

    cores = os.cpu_count() or 1
    ob = O.OracleBvh(tri)
    n = len(closest)
    t0 = time.perf_counter()
    _, _, nv, nt = ob.closest(closest, threads=cores, counts=True)
    dt = time.perf_counter() - t0
    half = n // 2
    return ({"value": round(n / dt / 1e6, 4), "unit": UNIT, "cores": cores, "kind": "port",
             "sample": f"the full {n}-ray batch, one pass, FP64 restatement of BvhAccel::intersectT over the "
                       f"reference's midpoint BVH (with per-ray visit counters)"},
            {"primary": [float(nv[:half].mean()), float(nt[:half].mean())],
             "incoherent": [float(nv[half:].mean()), float(nt[half:].mean())]})


def bench_box_render(torch, steps: int):
    """Box scene (unit cube, 10 walls, ceiling quad light, GGX + Phong spheres), 256x256,
    16 spp, max depth 4, MIS light+BRDF, Russian roulette 0.3, seed 1: the wavefront path
    tracer.  Returns samples/s and Mrays/s (closest-hit + shadow rays)."""
    from chakumrender_gb300 import scene as S

    sd = S.load_xml(S.SCENES / "box.xml")
    cam = sd.camera
    cfg = S.render_cfg(shader=S.SHADER_PATH, spp=16, max_depth=4, n_light=1, n_brdf=1, rr_prob=0.3, seed=1)
    scene = S.RenderScene(sd)
    rgb = torch.empty((cam.height, cam.width, 3), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(2):
        scene.render(cam, cfg, rgb.data_ptr(), None, stream.cuda_stream)
    torch.cuda.synchronize()
    scene.ray_stats(reset=True)
    k = max(3, min(steps, 20))
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(k):
        scene.render(cam, cfg, rgb.data_ptr(), None, stream.cuda_stream)
    b.record(stream)
    torch.cuda.synchronize()
    sec = a.elapsed_time(b) / 1e3
    closest, shadow = scene.ray_stats(reset=True)
    samples = cam.width * cam.height * cfg.spp * k
    pixels = cam.width * cam.height * k
    nbytes = box_state_bytes(samples, closest, shadow, pixels)
    peak, peak_kind = peaks()
    return {"workload": "box scene 256x256, 16 spp, depth 4, MIS (1 light + 1 BRDF sample), RR 0.3",
            "ms_per_frame": round(1e3 * sec / k, 3), "samples_per_s": round(samples / sec, 1),
            "mrays_per_s": round((closest + shadow) / sec / 1e6, 2),
            "rays_per_sample": round((closest + shadow) / samples, 3),
            "roofline": {"bound": "hbm", "bytes_per_sample": round(nbytes / samples, 1),
                         "achieved": round(nbytes / sec / 1e9, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(nbytes / sec / 1e9 / peak, 4), "peak_kind": peak_kind,
                         "counted": "wavefront state moved between kernels (BOX_STATE_BYTES); the 13-triangle "
                                    "scene itself stays in L1/L2"}}


# Bytes the box render's wavefront stages must move through global memory, from the
# layout of the path state (csrc/wavefront.cuh): a camera path writes ray_o, ray_d,
# beta, meta (16 B each) and its queue entry (4 B); a closest-hit ray reads its queue
# entry and ray (36 B) and writes id + t (8 B); its shading reads queue entry, id,
# meta, ray, beta, t and the triangle's normal/material word (92 B); a continuation
# writes the path state and queue entry again (68 B); a shadow ray is written and read
# once (sh_o, sh_d, sh_c 16 B each + pixel 4 B) and, unoccluded, adds 3 doubles to its
# pixel (24 B read + 24 B written); per pixel the sums are cleared (24 B), read (24 B)
# and the image written (12 B).
BOX_STATE_BYTES = {"camera_path": 68, "closest_ray": 36 + 8 + 92, "continuation": 68, "shadow_ray": 52 + 52 + 48,
                   "pixel": 24 + 24 + 12}


def box_state_bytes(paths, closest, shadow, pixels):
    B = BOX_STATE_BYTES
    return (paths * B["camera_path"] + closest * B["closest_ray"] + (closest - paths) * B["continuation"]
            + shadow * B["shadow_ray"] + pixels * B["pixel"])


# FP32 operations of LTC shading per pixel and emitter triangle, counted from the
# formulas of getLightAnalytic / getLightAnalyticDiffuse (src/lightSources_CV.cpp:221-333)
# for a triangle wholly above the horizon (a clipped one does more), a fused
# multiply-add counted as two: specular lobe 3 x (v - x) 9, 3 x Minv v 45, 3
# normalisations 24, 3 edge integrals (z of the cross product 3, cos 5, clamp 2,
# (1 - c)(1 + c) 3, theta / sin theta 1) 42, sum 3 -> 126; cosine lobe (v - x) 9, 3
# normalisations 24, 3 dots with n 15, 3 edge integrals (cross 9, dot with n 5, the
# same 11, product 1) 78, sum 3 -> 129; radiance weights 12.  Transcendentals (acos,
# sqrt, rsqrt, divide) per triangle: 30.  Per pixel once: the table lookup and the
# world-space Minv (about 90).
LTC_FLOP_PER_PIXEL_TRI = 126 + 129 + 12
LTC_SFU_PER_PIXEL_TRI = 30
LTC_FLOP_PER_PIXEL = 90
# FP32 peak, nominal: 152 SMs x 128 FP32 lanes x 2 (FMA) x 2.07 GHz.
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def bench_ltc(torch, steps: int):
    """LTC shading of a 1024x1024 G-buffer lit by 8 quad lights (16 emitter triangles)."""
    from chakumrender_gb300 import ckr

    n = 1024 * 1024
    g = torch.from_numpy(ckr.gbuffer(2, n)).cuda()
    lt, lc = ckr.quad_lights(3, 8)
    dt, dc = torch.from_numpy(lt).cuda(), torch.from_numpy(lc).cuda()
    out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(3):
        ckr.ltc_shade(g.data_ptr(), n, dt.data_ptr(), dc.data_ptr(), len(lt), out.data_ptr(), stream.cuda_stream)
    k = max(3, min(steps, 50))
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(k):
        ckr.ltc_shade(g.data_ptr(), n, dt.data_ptr(), dc.data_ptr(), len(lt), out.data_ptr(), stream.cuda_stream)
    b.record(stream)
    torch.cuda.synchronize()
    sec = a.elapsed_time(b) / 1e3 / k
    # Against the 4096-spp Monte Carlo reference of the same integral (FP64 sums).
    ltc = out.double()
    mc = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    mc2 = torch.empty_like(mc)
    a.record(stream)
    ckr.ltc_mc(g.data_ptr(), n, dt.data_ptr(), dc.data_ptr(), len(lt), 4096, 1, False, mc.data_ptr(),
               stream.cuda_stream)
    b.record(stream)
    ckr.ltc_mc(g.data_ptr(), n, dt.data_ptr(), dc.data_ptr(), len(lt), 4096, 2, False, mc2.data_ptr(),
               stream.cuda_stream)
    torch.cuda.synchronize()
    mc_ms = a.elapsed_time(b)

    def rel_mse(x, y):
        return float(((x - y) ** 2 / (y * y + 1e-2)).mean())

    mc_f = torch.empty_like(mc)
    ckr.ltc_mc(g.data_ptr(), n, dt.data_ptr(), dc.data_ptr(), len(lt), 4096, 1, True, mc_f.data_ptr(),
               stream.cuda_stream)
    torch.cuda.synchronize()
    ntri = lt.reshape(-1, 9).shape[0]
    flop = n * (LTC_FLOP_PER_PIXEL + ntri * LTC_FLOP_PER_PIXEL_TRI)
    return {"workload": "LTC shading, 1024x1024 G-buffer, 8 quad lights", "ms_per_frame": round(1e3 * sec, 4),
            "mpixels_per_s": round(n / sec / 1e6, 1), "io_gb_per_s": round(n * 60 / sec / 1e9, 1),
            "roofline": {"bound": "fp32 alu", "flop_per_pixel": LTC_FLOP_PER_PIXEL + ntri * LTC_FLOP_PER_PIXEL_TRI,
                         "emitter_triangles": ntri, "achieved": round(flop / sec / 1e12, 3),
                         "peak": round(FP32_PEAK_TFLOPS, 1), "unit": "TFLOP/s",
                         "frac": round(flop / sec / 1e12 / FP32_PEAK_TFLOPS, 4), "peak_kind": "nominal",
                         "sfu_per_pixel": ntri * LTC_SFU_PER_PIXEL_TRI},
            "vs_mc_4096spp": {"relmse_ltc_vs_mc": round(rel_mse(ltc, mc), 6),
                              "relmse_ltc_vs_mc_with_fresnel": round(rel_mse(ltc, mc_f), 6),
                              "relmse_mc_seed_to_seed": round(rel_mse(mc2, mc), 7),
                              "mc_ms": round(mc_ms, 2)}}


def bench_manylight(torch):
    """The many-light scene (1,310,720-triangle displaced icosphere, GGX roughness
    uniform per triangle in [0.1, 0.8], 10^3 room, 4,096 emissive triangles in 64
    clusters), 1920x1080, 64 spp, max depth 6, one-sample NEE path tracer.  Plain =
    lights chosen in proportion to power; learned = the proposal network (BF16
    tensor-core MLP, defensive 0.2, Adam lr 1e-3 as the workload specifies) trained
    online from scratch inside the timed frame (cold) or carried over from one
    earlier frame (warm); the learned frame gets the spp that fit in the plain
    frame's time.

    relMSE is over the whole frame against an FP64-accumulated reference rendered as
    two independent halves of 1,024 spp: with ref = (h1 + h2) / 2 and the per-pixel
    estimate (h1 - h2)^2 / 4 of the reference's own variance subtracted,
    mean(((img - ref)^2 - (h1 - h2)^2 / 4) / (ref^2 + 1e-2)) is an unbiased estimate
    of the relMSE against the converged image.  The earlier metric (a 320x180 window
    against 16,384 spp) is reported beside it, as is Adam lr 3e-3."""
    from chakumrender_gb300 import scene as S
    from chakumrender_gb300.proposal import Proposal

    W, H, SPP, DEPTH = 1920, 1080, 64, 6
    X0, Y0, CW, CH = 800, 300, 320, 180  # window (x from the left, y from the bottom)
    sd = S.manylight_scene(S.manylight_spec(width=W, height=H))
    scene = S.RenderScene(sd)
    cam = sd.camera
    win = S.Camera()
    cx, cy, d = np.array(cam.cx, float), np.array(cam.cy, float), np.array(cam.dir, float)
    nd = d + cx * ((X0 + CW / 2) / W - .5) + cy * ((Y0 + CH / 2) / H - .5)
    for k in range(3):
        win.pos[k], win.dir[k], win.cx[k], win.cy[k] = cam.pos[k], nd[k], cx[k] * CW / W, cy[k] * CH / H
    win.width, win.height = CW, CH
    rgb = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    acc = torch.empty((H, W, 3), dtype=torch.float64, device="cuda")
    wrgb = torch.empty((CH, CW, 3), dtype=torch.float32, device="cuda")

    def timed(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t

    cfg = lambda spp, seed: S.render_cfg(shader=S.SHADER_PATH_NEE, spp=spp, max_depth=DEPTH, seed=seed)
    ref_sec = timed(lambda: scene.render(win, cfg(16384, 1000), wrgb.data_ptr()))
    wref = wrgb.double().cpu().numpy()
    REF_HALF = 1024
    halves = []
    t_ref = 0.0
    for seed in (2000, 2001):
        t_ref += timed(lambda: scene.render(cam, cfg(REF_HALF, seed), rgb.data_ptr(), acc.data_ptr()))
        halves.append(acc.cpu().numpy() / REF_HALF)  # FP64 per-pixel sums
    fref = 0.5 * (halves[0] + halves[1])
    fnoise = 0.25 * (halves[0] - halves[1]) ** 2
    fden = fref * fref + 1e-2

    def rel_mse():
        img = rgb.double().cpu().numpy()
        full = float(np.mean(((img - fref) ** 2 - fnoise) / fden))
        w = img[H - Y0 - CH:H - Y0, X0:X0 + CW]
        return full, float(np.mean((w - wref) ** 2 / (wref * wref + 1e-2)))

    scene.render(cam, cfg(SPP, 1), rgb.data_ptr())  # warm-up
    scene.ray_stats(reset=True)
    t_plain = timed(lambda: scene.render(cam, cfg(SPP, 2), rgb.data_ptr()))
    closest, shadow = scene.ray_stats(reset=True)
    e_plain = rel_mse()

    def learned_runs(lr):
        opts = dict(minibatch=4096, max_steps=1000, lr=lr, batch=262144)
        cold = Proposal(scene, seed=1, **opts)
        t_c64 = timed(lambda: cold.render(cam, cfg(SPP, 3), rgb.data_ptr()))
        e_c64 = rel_mse()
        spp_c = max(2, int(SPP * t_plain / t_c64))
        cold2 = Proposal(scene, seed=2, **opts)
        t_c = timed(lambda: cold2.render(cam, cfg(spp_c, 4), rgb.data_ptr()))
        e_c = rel_mse()
        st, steps, loss = cold2.status()
        if st != 0:
            raise RuntimeError(f"proposal network error {st}")
        cold.set_training(False)  # warm: the network of the first learned frame, frozen
        t_w64 = timed(lambda: cold.render(cam, cfg(SPP, 5), rgb.data_ptr()))
        e_w64 = rel_mse()
        spp_w = max(2, int(SPP * t_plain / t_w64))
        t_w = timed(lambda: cold.render(cam, cfg(spp_w, 6), rgb.data_ptr()))
        e_w = rel_mse()
        return {"cold_64spp": {"sec": round(t_c64, 4), "relmse": round(e_c64[0], 5),
                               "relmse_window": round(e_c64[1], 5)},
                "cold_equal_time": {"spp": spp_c, "sec": round(t_c, 4), "relmse": round(e_c[0], 5),
                                    "relmse_window": round(e_c[1], 5), "adam_steps": steps,
                                    "last_loss": round(loss, 4)},
                "warm_64spp": {"sec": round(t_w64, 4), "relmse": round(e_w64[0], 5),
                               "relmse_window": round(e_w64[1], 5)},
                "warm_equal_time": {"spp": spp_w, "sec": round(t_w, 4), "relmse": round(e_w[0], 5),
                                    "relmse_window": round(e_w[1], 5)},
                "relmse_ratio_plain_over_learned_equal_time": {
                    "cold": round(e_plain[0] / e_c[0], 3), "warm": round(e_plain[0] / e_w[0], 3),
                    "cold_window": round(e_plain[1] / e_c[1], 3), "warm_window": round(e_plain[1] / e_w[1], 3)},
                "relmse_ratio_plain_over_learned_64spp": {"cold": round(e_plain[0] / e_c64[0], 3),
                                                          "warm": round(e_plain[0] / e_w64[0], 3)}}

    main_run = learned_runs(1e-3)
    alt_run = learned_runs(3e-3)
    samples = W * H * SPP
    out = {"workload": "many-light: 1,310,720-tri GGX icosphere in a 10^3 room, 4,096 emitters in 64 clusters, "
                       "1920x1080, 64 spp, depth 6, one-sample NEE",
           "plain": {"spp": SPP, "sec": round(t_plain, 4), "relmse": round(e_plain[0], 5),
                     "relmse_window": round(e_plain[1], 5), "samples_per_s": round(samples / t_plain, 1),
                     "mrays_per_s": round((closest + shadow) / t_plain / 1e6, 1)},
           "learned": main_run,
           "relmse_ratio_plain_over_learned_equal_time": main_run["relmse_ratio_plain_over_learned_equal_time"],
           "learned_lr_3e-3": alt_run,
           "reference": {"full_frame": {"spp": 2 * REF_HALF, "halves": 2, "sec": round(t_ref, 2),
                                        "accumulation": "fp64", "correction": "(h1 - h2)^2 / 4 subtracted"},
                         "window": {"spp": 16384, "window": [X0, Y0, CW, CH], "sec": round(ref_sec, 2)}},
           "proposal": {"minibatch": 4096, "batch": 262144, "max_steps": 1000, "defensive": 0.2, "lr": 1e-3}}
    return out


def bench_batch(torch, njobs=64, sizes=(256, 512, 768, 1024), spps=(4, 16, 64)):
    """Box-scene jobs (random sphere BRDFs GGX/Beckmann/Phong with roughness in
    [0.05, 0.9], camera yaw in [-30, 30] degrees, square resolution from `sizes`, spp
    from `spps`, depth from {3, 6}), path tracer with MIS: one pass replayed from a
    CUDA graph (renderer, block size and paths in flight from the autotuner) against
    the same jobs rendered one after another with the same renderer (a launch per
    job), against one ckr_render call per job (the wavefront renderer), and against
    the whole batch in the wavefront renderer (block 128, 2^21 paths per wave)."""
    from chakumrender_gb300 import scene as S
    from chakumrender_gb300.batch import Batch, BatchTuning, Job, box_jobs

    sd = S.load_xml(S.SCENES / "box.xml")
    params, mats = box_jobs(sd, njobs=njobs, seed=4, sizes=sizes, spps=spps)
    outs = [torch.empty((p["cam"].height, p["cam"].width, 3), dtype=torch.float32, device="cuda") for p in params]
    jobs = [Job(p["cam"], p["spp"], p["max_depth"], p["seed"], p["material_set"], 0, o.data_ptr())
            for p, o in zip(params, outs)]
    scene = S.RenderScene(sd)
    t0 = time.perf_counter()
    b = Batch(scene, jobs, materials=mats, shader=S.SHADER_PATH)
    create_s = time.perf_counter() - t0
    paths, launches = b.stats()
    tune = b.tuning()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    s = torch.cuda.current_stream()
    b.render(s.cuda_stream)
    b.render_sequential(s.cuda_stream)
    ev[0].record(s)
    b.render(s.cuda_stream)
    ev[1].record(s)
    b.render_sequential(s.cuda_stream)
    ev[2].record(s)
    torch.cuda.synchronize()
    t_graph = ev[0].elapsed_time(ev[1]) / 1e3
    t_seq = ev[1].elapsed_time(ev[2]) / 1e3
    # One ckr_render call per job through the public entry point (a scene per
    # material set; the second of two passes is timed).
    scenes = [S.RenderScene(S.SceneData(sd.tri9, sd.tri_mat, sd.sph4, sd.sph_mat,
                                        [S.Material.from_buffer_copy(mats[j * sd.nmat + k]) for k in range(sd.nmat)],
                                        [sd.lights[k] for k in range(sd.nlights)])) for j in range(len(params))]
    cfgs = [S.render_cfg(shader=S.SHADER_PATH, spp=p["spp"], max_depth=p["max_depth"], n_light=1, n_brdf=1,
                         rr_prob=0.3, seed=p["seed"]) for p in params]
    for rep in range(2):
        ev[2].record(s)
        for sc, p, c, o in zip(scenes, params, cfgs, outs):
            sc.render(p["cam"], c, o.data_ptr(), None, s.cuda_stream)
        ev[3].record(s)
        torch.cuda.synchronize()
    t_api = ev[2].elapsed_time(ev[3]) / 1e3
    # The same batch in the wavefront renderer, for comparison.
    bw = Batch(scene, jobs, materials=mats, shader=S.SHADER_PATH, tuning=BatchTuning(128, 1 << 21, 0.0, 0, 0))
    _, launches_w = bw.stats()
    bw.render(s.cuda_stream)
    ev[2].record(s)
    bw.render(s.cuda_stream)
    ev[3].record(s)
    torch.cuda.synchronize()
    t_wave = ev[2].elapsed_time(ev[3]) / 1e3
    del bw
    return {"workload": (f"{njobs} box-scene jobs, random sphere BRDFs and yaw, {min(sizes)}^2..{max(sizes)}^2, "
                         f"{'/'.join(map(str, spps))} spp, depth 3/6, path tracer with MIS"),
            "samples": paths, "graph_launches": launches,
            "batched_graph": {"sec": round(t_graph, 4), "samples_per_s": round(paths / t_graph, 1)},
            "sequential_per_job": {"sec": round(t_seq, 4), "samples_per_s": round(paths / t_seq, 1)},
            "one_ckr_render_per_job": {"sec": round(t_api, 4), "samples_per_s": round(paths / t_api, 1)},
            "wavefront_batch_graph": {"sec": round(t_wave, 4), "samples_per_s": round(paths / t_wave, 1),
                                      "graph_launches": launches_w},
            "speedup": round(t_seq / t_graph, 3),
            "speedup_vs_ckr_render_per_job": round(t_api / t_graph, 3),
            "autotuner": {"renderer": "persistent" if tune.mode == 1 else "wavefront", "block": tune.block,
                          "paths_in_flight" if tune.mode == 1 else "wave": tune.wave,
                          "candidates": tune.candidates, "reduced_batch_ms": round(tune.ms, 3)},
            "create_and_capture_s": round(create_s, 2)}


def cpu_side_baselines(tri_unused=None):
    """FP64 restatements of the reference on the host cores for the box render
    (path tracer, 64x64 x 16 spp sample) and LTC shading (65,536 pixels)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    from chakumrender_gb300 import ckr
    from chakumrender_gb300 import scene as S

    cores = os.cpu_count() or 1
    sd = S.load_xml(S.SCENES / "box.xml")
    cam = sd.camera
    cam.width = cam.height = 64
    cfg = S.render_cfg(shader=S.SHADER_PATH, spp=16, max_depth=4, n_light=1, n_brdf=1, rr_prob=0.3, seed=1)
    t0 = time.perf_counter()
    O.render(sd, cam, cfg, threads=cores)
    box = 64 * 64 * 16 / (time.perf_counter() - t0)
    g = ckr.gbuffer(2, 65536)
    lt, lc = ckr.quad_lights(3, 8)
    m = np.zeros(len(g), dtype=O.MATERIAL)
    m["brdf"], m["alpha"], m["spec"], m["int_ior"], m["ext_ior"] = 2, g[:, 3], g[:, 11], 1.5, 1.0
    t0 = time.perf_counter()
    O.ltc_shade_batch(m, g[:, 0:3], g[:, 4:7], g[:, 8:11], lt, lc, threads=cores)
    ltc = 65536 / (time.perf_counter() - t0)
    return {"box_samples_per_s": round(box, 1), "ltc_mpixels_per_s": round(ltc / 1e6, 4), "cores": cores,
            "kind": "port"}


def case_manylight_learned():
    """Small case of the many-light workload for profilers: 640x360, 16 spp, depth 6,
    one learned render training for 40 Adam steps (minibatch 16384)."""
    import torch
    from chakumrender_gb300 import build
    from chakumrender_gb300 import scene as S
    from chakumrender_gb300.proposal import Proposal

    build.build_library()
    sd = S.manylight_scene(S.manylight_spec(width=640, height=360))
    scene = S.RenderScene(sd)
    rgb = torch.empty((360, 640, 3), dtype=torch.float32, device="cuda")
    prop = Proposal(scene, seed=1, minibatch=16384, max_steps=40)
    prop.render(sd.camera, S.render_cfg(shader=S.SHADER_PATH_NEE, spp=16, max_depth=6, seed=10), rgb.data_ptr())
    torch.cuda.synchronize()
    st = prop.status()[0]
    if st != 0:
        raise SystemExit(f"proposal error {st}")


def case_manylight_split():
    """One frozen learned render and one plain render of the many-light workload at
    640x360, 16 spp, depth 6 (after a 200-step training render), for launch lists."""
    import torch
    from chakumrender_gb300 import build
    from chakumrender_gb300 import scene as S
    from chakumrender_gb300.proposal import Proposal

    build.build_library()
    sd = S.manylight_scene(S.manylight_spec(width=640, height=360))
    scene = S.RenderScene(sd)
    cam = sd.camera
    rgb = torch.empty((360, 640, 3), dtype=torch.float32, device="cuda")
    prop = Proposal(scene, seed=1, minibatch=16384, max_steps=200)
    cfg = lambda seed: S.render_cfg(shader=S.SHADER_PATH_NEE, spp=16, max_depth=6, seed=seed)
    prop.render(cam, cfg(10), rgb.data_ptr())
    prop.set_training(False)
    prop.render(cam, cfg(11), rgb.data_ptr())
    scene.render(cam, cfg(1), rgb.data_ptr())
    torch.cuda.synchronize()


def case_trace():
    """The traversal workload (2^23 rays over the 1.3M-triangle icosphere, 0.4 GB on
    the device) for profilers: two closest-hit launches, then two any-hit launches."""
    import torch
    from chakumrender_gb300 import build
    from chakumrender_gb300 import ckr

    build.build_library()
    tri, closest, anyhit = make_workload()
    scene = ckr.Scene(tri)
    n = len(closest)
    s = torch.cuda.current_stream().cuda_stream
    d_rays, d_any = torch.from_numpy(closest).cuda(), torch.from_numpy(anyhit).cuda()
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    ts = torch.empty(n, dtype=torch.float32, device="cuda")
    occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    for _ in range(2):
        scene.trace_closest(d_rays.data_ptr(), n, ids.data_ptr(), ts.data_ptr(), s)
    for _ in range(2):
        scene.trace_any(d_any.data_ptr(), n, occ.data_ptr(), s)
    if scene.check_device(s) != 0:
        raise SystemExit("device status error")


def case_ltc():
    """LTC shading of the 1024x1024 G-buffer with 8 quad lights, three launches, for
    profilers."""
    import torch
    from chakumrender_gb300 import build
    from chakumrender_gb300 import ckr

    build.build_library()
    n = 1024 * 1024
    g = torch.from_numpy(ckr.gbuffer(2, n)).cuda()
    lt, lc = ckr.quad_lights(3, 8)
    dt, dc = torch.from_numpy(lt).cuda(), torch.from_numpy(lc).cuda()
    out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    for _ in range(3):
        ckr.ltc_shade(g.data_ptr(), n, dt.data_ptr(), dc.data_ptr(), len(lt), out.data_ptr(), s)
    torch.cuda.synchronize()


def case_ltc_mc():
    """The Monte Carlo reference of the LTC integral on 65,536 pixels of the same
    G-buffer, 4,096 samples per pixel, once, for profilers."""
    import torch
    from chakumrender_gb300 import build
    from chakumrender_gb300 import ckr

    build.build_library()
    n = 65536
    g = torch.from_numpy(ckr.gbuffer(2, n)).cuda()
    lt, lc = ckr.quad_lights(3, 8)
    dt, dc = torch.from_numpy(lt).cuda(), torch.from_numpy(lc).cuda()
    out = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    ckr.ltc_mc(g.data_ptr(), n, dt.data_ptr(), dc.data_ptr(), len(lt), 4096, 9, 0, out.data_ptr(),
               torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()


def case_box():
    """The box render of the benchmark (256x256, 16 spp, depth 4, MIS 1 + 1), three
    frames, for profilers."""
    import torch
    from chakumrender_gb300 import build
    from chakumrender_gb300 import scene as S

    build.build_library()
    sd = S.load_xml(S.SCENES / "box.xml")
    cam = sd.camera
    cfg = S.render_cfg(shader=S.SHADER_PATH, spp=16, max_depth=4, n_light=1, n_brdf=1, rr_prob=0.3, seed=1)
    scene = S.RenderScene(sd)
    rgb = torch.empty((cam.height, cam.width, 3), dtype=torch.float32, device="cuda")
    for _ in range(3):
        scene.render(cam, cfg, rgb.data_ptr())
    torch.cuda.synchronize()


def case_batch():
    """The batched-jobs workload alone (64 box jobs, and 512 small ones); prints its
    JSON (for profilers and for tuning the batch renderers)."""
    import torch
    from chakumrender_gb300 import build

    build.build_library()
    out = {"batch": bench_batch(torch), "batch_small": bench_batch(torch, njobs=512, sizes=(32, 48, 64),
                                                                    spps=(1, 2, 4))}
    print(json.dumps(out), flush=True)


def case_batch_persistent():
    """16 box-scene jobs of 256x256 at 4 spp rendered twice by the persistent batch
    renderer (forced: block 64, 77,824 paths in flight), for profilers."""
    import torch
    from chakumrender_gb300 import build
    from chakumrender_gb300 import scene as S
    from chakumrender_gb300.batch import Batch, BatchTuning, Job, box_jobs

    build.build_library()
    sd = S.load_xml(S.SCENES / "box.xml")
    params, mats = box_jobs(sd, njobs=16, seed=4, sizes=(256,), spps=(4,))
    outs = [torch.empty((p["cam"].height, p["cam"].width, 3), dtype=torch.float32, device="cuda") for p in params]
    jobs = [Job(p["cam"], p["spp"], p["max_depth"], p["seed"], p["material_set"], 0, o.data_ptr())
            for p, o in zip(params, outs)]
    b = Batch(S.RenderScene(sd), jobs, materials=mats, shader=S.SHADER_PATH,
              tuning=BatchTuning(64, 77824, 0.0, 0, 1))
    for _ in range(2):
        b.render()
    torch.cuda.synchronize()


CASES = {"batch": case_batch, "batch-persistent": case_batch_persistent, "manylight-learned": case_manylight_learned, "manylight-split": case_manylight_split, "trace": case_trace,
         "ltc": case_ltc, "ltc-mc": case_ltc_mc, "box": case_box}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--leaf", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--case", default=None, choices=sorted(CASES),
                    help="run one small workload and exit (for profiling; prints nothing to parse)")
    args = ap.parse_args()
    if args.case:
        return CASES[args.case]()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from chakumrender_gb300 import build

    build.build_library()
    from chakumrender_gb300 import ckr

    tri, closest, anyhit = make_workload()
    scene = ckr.Scene(tri, max_leaf_size=args.leaf)
    info = scene.info()
    n = len(closest)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    d_rays = torch.from_numpy(closest).cuda()
    d_any = torch.from_numpy(anyhit).cuda()
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    ts = torch.empty(n, dtype=torch.float32, device="cuda")
    occ = torch.empty(n, dtype=torch.uint8, device="cuda")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        scene.trace_closest(d_rays.data_ptr(), n, ids.data_ptr(), ts.data_ptr(), sh)
    torch.cuda.synchronize()
    if scene.check_device(sh) != 0:
        raise SystemExit("device status error during warm-up")

    # Device-resident throughput: K steps, each bracketed by CUDA events on the launch stream.
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        barrier()
        t0 = time.perf_counter()
        for k in range(args.steps):
            ev[k][0].record(stream)
            scene.trace_closest(d_rays.data_ptr(), n, ids.data_ptr(), ts.data_ptr(), sh)
            ev[k][1].record(stream)
        barrier()
        wall = time.perf_counter() - t0
    clocks = clk.summary()
    kernel_ms = [a.elapsed_time(b) for a, b in ev]
    step_ms = sum(kernel_ms) / len(kernel_ms)
    t_max = torch.tensor([wall], dtype=torch.float64, device="cuda")
    if dist is not None:
        dist.all_reduce(t_max, op=dist.ReduceOp.MAX)
    total_rays = n * args.steps * world
    value = total_rays / float(t_max.item()) / 1e6

    # Any-hit pass (reported alongside).
    for _ in range(2):
        scene.trace_any(d_any.data_ptr(), n, occ.data_ptr(), sh)
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0.record(stream)
    for _ in range(args.steps):
        scene.trace_any(d_any.data_ptr(), n, occ.data_ptr(), sh)
    a1.record(stream)
    torch.cuda.synchronize()
    any_mrays = n * args.steps / (a0.elapsed_time(a1) / 1e3) / 1e6

    # End to end through the host-buffer C ABI (pinned buffers, copies inside the timed region).
    h_rays = torch.from_numpy(closest).pin_memory()
    h_ids = torch.empty(n, dtype=torch.int32).pin_memory()
    h_t = torch.empty(n, dtype=torch.float32).pin_memory()
    L = ckr.lib()
    for _ in range(2):
        ckr.check(L.ckr_trace_closest_host(scene.handle, h_rays.data_ptr(), n, h_ids.data_ptr(), h_t.data_ptr(), sh),
                  "e2e warm-up")
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ckr.check(L.ckr_trace_closest_host(scene.handle, h_rays.data_ptr(), n, h_ids.data_ptr(), h_t.data_ptr(), sh),
                  "e2e")
    barrier()
    e2e_wall = torch.tensor([time.perf_counter() - t0], dtype=torch.float64, device="cuda")
    if dist is not None:
        dist.all_reduce(e2e_wall, op=dist.ReduceOp.MAX)
    e2e = n * args.steps * world / float(e2e_wall.item()) / 1e6

    if rank != 0:
        dist.destroy_process_group()
        return

    # Roofline: algorithmic bytes per ray from the replayed node/triangle counts
    # (80-byte wide nodes, 36 bytes of vertices per triangle).  The kernel also reads
    # 32 bytes of precomputed slot bits per node visit (derived from the node's meta
    # bytes); being redundant, they are left out of the algorithmic bytes.
    sample = np.ascontiguousarray(closest[::16])
    mean_nodes, mean_tris = scene.stats(sample)
    bytes_per_ray = 32 + 8 + 80 * mean_nodes + 36 * mean_tris
    achieved = n * bytes_per_ray / (step_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic = traffic_from_profile()
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(step_ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(n, int(info.ntri), world),
        "structure": {"bvh": (f"binned SAH to single triangles ({info.nnodes_binary} binary nodes), SAH-optimal "
                              f"collapse to 8-wide nodes with 8-bit quantised boxes and leaves <= "
                              f"{min(args.leaf, 3)}: {info.nnodes} wide nodes, depth {info.max_depth}"),
                      "bvh_build_ms": round(info.build_ms, 1)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                     "bytes_per_ray": round(bytes_per_ray, 1), "mean_wide_nodes": round(mean_nodes, 2),
                     "mean_tris": round(mean_tris, 3),
                     "not_counted": "32 B of precomputed slot bits read per node visit"},
        "e2e": {"value": round(e2e, 3), "unit": UNIT, "h2d_bytes_per_step": n * 32, "d2h_bytes_per_step": n * 8},
        "gpu_launches": args.steps,
        "any_hit_mrays": round(any_mrays, 3),
        "kernel_ms_min_max": [round(min(kernel_ms), 4), round(max(kernel_ms), 4)],
        "clocks": clocks,
    }
    line["box_render"] = bench_box_render(torch, args.steps)
    line["ltc_shade"] = bench_ltc(torch, args.steps)
    line["manylight"] = bench_manylight(torch)
    line["batch"] = bench_batch(torch)
    # Many small jobs: launch-bound when each is rendered on its own.
    line["batch_small"] = bench_batch(torch, njobs=512, sizes=(32, 48, 64), spps=(1, 2, 4))
    if not args.no_cpu_baseline:
        cb, ref_counts = cpu_baseline(tri, closest)
        line["cpu_baseline"] = cb
        line["roofline"]["reference_bvh_counts"] = ref_counts
        line["cpu_baseline_other"] = cpu_side_baselines()
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
