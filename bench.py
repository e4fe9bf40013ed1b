"""Benchmark of the CRaystal hot path on GB300.

Workload (the ray-cast microbenchmark): 1,048,576 random FP32 triangles
(centroids U[0,1]^3, edges N(0, 0.01) per component), binned-SAH BVH with 32
bins built on the GPU, 16,777,216 rays from the sphere of radius 2 towards
U[0,1]^3 (tmin 1e-4, tmax inf), closest hit (prim, t, u, v) per ray.  One
step = one closest-hit pass over the 16M rays.

  value : Mrays/s with rays and hits resident in HBM (cr_trace_closest_device),
          CUDA events on the launching stream.
  e2e   : Mrays/s through cr_trace_closest with pinned host buffers; every step
          moves the 512 MiB of rays in and the 256 MiB of hits out (the
          library has the GPU read and write pinned arrays in place).
  roofline : algorithmic bytes per ray counted by the oracle on the
          reference BVH (32 B ray + 16 B hit + 24 B per child box tested +
          48 B per triangle tested + 4 B per leaf-map read) over the kernel's
          measured time, against the measured HBM copy bandwidth.
  cpu_baseline : the oracle (a CPU restatement of the reference path; the
          reference itself cannot be built) on all host cores, on a sample of
          the same rays.

--impl reference times that CPU path on its own (the reference arm).
Under torchrun (N > 1) every rank runs its own replica (the path does not
need to exchange data); value sums the rays of all ranks over the slowest
rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_TRIS = 1 << 20
N_RAYS = 1 << 24  # --rays / --tris shrink the workload for profiler captures
TRI_SEED, RAY_SEED = 0, 1
METRIC = "Mrays/s (closest-hit ray cast, 1M triangles, 16M rays)"
WORKLOAD = "raycast_1M_tris_16M_rays"


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def slowest_rank_ms(ms, world, device):
    """The timed region of the slowest rank (max over ranks), as every rank
    times its own replica between barriers."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def tensor_peak():
    """Dense bf16 tensor-core throughput (TFLOP/s), burst, and its source."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


def fp32_peak_tflops(torch):
    """FP32 FMA throughput measured here: cuBLAS SGEMM 8192^3 with TF32 off,
    best of 5 (CUDA events)."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    g = torch.Generator(device="cuda").manual_seed(0)
    a = torch.randn(n, n, device="cuda", generator=g)
    b = torch.randn(n, n, device="cuda", generator=g)
    c = a @ b
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b, c
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo) and core count."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                name = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if name is None:
        try:
            with open("/proc/cpuinfo") as f:
                for line in f:
                    if line.lower().startswith("model name"):
                        name = line.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    import platform
    return {"model": name or platform.machine(), "nproc": os.cpu_count()}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def algorithmic_bytes_per_ray(flat, rays_sample, threads):
    """Oracle counts on the reference BVH (independent of the GPU's tree)."""
    import oracle
    osc = oracle.OracleScene(flat)
    _, _, c = osc.trace_closest(rays_sample, threads=threads, counters=True)
    n = c["rays"]
    per = {"boxes": c["boxes"] / n, "tris": c["tris"] / n, "map_reads": c["map_reads"] / n}
    bpr = 32 + 16 + 24 * per["boxes"] + 48 * per["tris"] + 4 * per["map_reads"]
    return bpr, per, osc


def cpu_baseline(osc, rays, threads, target_s=6.0):
    """Times the oracle's closest-hit traversal on a bounded sample."""
    probe = rays[: 1 << 16]
    t0 = time.perf_counter()
    osc.trace_closest(probe, threads=threads)
    rate = len(probe) / max(time.perf_counter() - t0, 1e-6)
    n = int(min(len(rays), max(1 << 18, rate * target_s)))
    n -= n % 1024
    sample = rays[:n]
    t0 = time.perf_counter()
    osc.trace_closest(sample, threads=threads)
    dt = time.perf_counter() - t0
    return n / dt / 1e6, n, dt


def read_bandwidth_gbs(nbytes, passes):
    """Device read bandwidth of a buffer of nbytes, read `passes` times
    (cr_device_read_bandwidth: 16-byte loads cached in L2 only, CUDA events)."""
    import ctypes
    from craystal_gb300._lib import check, load
    v = ctypes.c_double()
    check(load().cr_device_read_bandwidth(int(nbytes), int(passes), ctypes.byref(v)))
    return float(v.value)


def l2_peak_gbs():
    """L2 read bandwidth: best of 3 runs of 40 passes over 64 MiB (resident
    in the 129 MB L2); beside it the HBM read bandwidth over 4 GiB."""
    l2 = max(read_bandwidth_gbs(64 << 20, 40) for _ in range(3))
    hbm = max(read_bandwidth_gbs(4 << 30, 3) for _ in range(2))
    return l2, hbm


def two_level_extra(torch, sc, d_rays, n, ref_hits, one_level_ms, reps=5):
    """The same cast with the two-level step (cr_scene_set_traversal): two
    binary levels of a node group per step.  Device time per launch beside
    the one-level step's, and whether every hit is the same bit for bit."""
    import craystal_gb300 as cg
    out_hits = torch.empty(n * 16, dtype=torch.uint8, device=d_rays.device)
    s = torch.cuda.current_stream()
    sc.set_traversal("two_level")
    try:
        for _ in range(2):
            sc.trace_closest_device(d_rays.data_ptr(), n, out_hits.data_ptr(), s.cuda_stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            sc.trace_closest_device(d_rays.data_ptr(), n, out_hits.data_ptr(), s.cuda_stream)
        e1.record(s)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / reps
    finally:
        sc.set_traversal("one_level")
    hits = out_hits.cpu().numpy().view(cg.HIT_DTYPE)
    return {"ms_per_launch": round(ms, 3), "Mrays_s": round(n / ms / 1e3, 1),
            "one_level_ms_per_launch": round(one_level_ms, 3), "two_over_one_time": round(ms / one_level_ms, 3),
            "hits_equal_one_level": bool(np.array_equal(hits.view(np.uint32), ref_hits.view(np.uint32)))}


def hbm_raycast_extra(torch, n_tris=1 << 23, n_rays=1 << 24, reps=5, with_oracle=True):
    """The ray cast on a scene far larger than L2: 8,388,608 random triangles
    (the C2 distribution, seed 2), 16,777,216 rays (seed 3).  Nodes and
    triangle blocks take about 0.6 GB, so node and triangle loads are served
    from HBM.  Device time per launch (CUDA events), algorithmic bytes per
    ray from the oracle's counts on the reference tree, fractions of the
    measured HBM and L2 peaks, DRAM traffic from the committed ncu summary of
    this workload, and bit-exact hits on a sample of rays."""
    from craystal_gb300 import scenes
    from craystal_gb300.api import Scene, flatten_scene
    import craystal_gb300 as cg
    data = scenes.random_triangle_scene(n_tris, seed=2)
    sc = Scene(data)
    st = sc.bvh_stats()
    rays = scenes.random_rays(n_rays, seed=3)
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_hits = torch.empty(n_rays * 16, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    for _ in range(2):
        sc.trace_closest_device(d_rays.data_ptr(), n_rays, d_hits.data_ptr(), s.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        sc.trace_closest_device(d_rays.data_ptr(), n_rays, d_hits.data_ptr(), s.cuda_stream)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    out = {"config": f"{n_tris} random triangles (C2 distribution), {n_rays} rays, closest hit",
           "bvh_device_mib": round(st["device_bytes"] / 2 ** 20, 1), "ms_per_launch": round(ms, 3),
           "Mrays_s": round(n_rays / ms / 1e3, 1)}
    out["two_level_traversal"] = two_level_extra(torch, sc, d_rays, n_rays, d_hits.cpu().numpy(), ms)
    if with_oracle:
        import oracle
        threads = oracle.hardware_threads()
        sample = 1 << 18
        bpr, per, osc = algorithmic_bytes_per_ray(flatten_scene(data), rays[:sample], threads)
        oh, ties = osc.trace_closest(rays[:sample], threads=threads)
        gh = d_hits[: sample * 16].cpu().numpy().view(cg.HIT_DTYPE)
        hit = oh["prim"] != cg.CR_MISS
        same = (gh["prim"] == oh["prim"]) & (~hit | (gh.view(np.uint32).reshape(-1, 4)[:, 1:] ==
                                                      oh.view(np.uint32).reshape(-1, 4)[:, 1:]).all(1))
        del osc
        achieved = bpr * n_rays / (ms * 1e-3) / 1e9
        peak, src = peaks()
        out.update({"bytes_per_ray": round(bpr, 1), "per_ray": {k: round(v, 2) for k, v in per.items()},
                    "achieved_gbs": round(achieved, 1), "hbm_peak_gbs": peak,
                    "algorithmic_frac_of_hbm": round(achieved / peak, 4),
                    "hits_checked": sample, "hits_bit_exact": int((same | ties).sum()), "ties": int(ties.sum())})
        prof = os.path.join(ROOT, "profiles", "trace_closest_raycast_hbm8m.json")
        if os.path.exists(prof):
            with open(prof) as f:
                p = json.load(f)
            per_launch = p["dram_bytes_per_launch_capture"] * n_rays / p["capture_rays"]
            out["dram"] = {"bytes_per_launch": round(per_launch), "gbs": round(per_launch / (ms * 1e-3) / 1e9, 1),
                           "frac_of_hbm": round(per_launch / (ms * 1e-3) / 1e9 / peak, 4),
                           "source": "profiles/trace_closest_raycast_hbm8m.json, scaled by rays"}
    sc.close()
    return out


def traffic_from_profile():
    """DRAM bytes per launch of the trace kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "trace_closest_raycast.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        p = json.load(f)
    return p.get("dram_bytes_per_launch_full_size")


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    from craystal_gb300 import scenes
    from craystal_gb300.api import flatten_scene
    threads = oracle.hardware_threads()
    osc = oracle.OracleScene(flatten_scene(scenes.random_triangle_scene(N_TRIS, TRI_SEED)))
    sample = 1 << 20
    rays = scenes.random_rays(sample * 2, RAY_SEED)
    for i in range(args.warmup):
        osc.trace_closest(rays[(i % 2) * sample:(i % 2 + 1) * sample], threads=threads)
    t0 = time.perf_counter()
    for i in range(args.steps):
        osc.trace_closest(rays[(i % 2) * sample:(i % 2 + 1) * sample], threads=threads)
    dt = time.perf_counter() - t0
    v = sample * args.steps / dt / 1e6
    out = {"metric": METRIC, "value": round(v, 3), "unit": "Mrays/s", "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * dt / args.steps, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded)",
           "config": {"workload": WORKLOAD, "triangles": N_TRIS, "rays": N_RAYS,
                      "step_sample_rays": sample, "bvh": "binned SAH, 32 bins (reference CPU build)"},
           "cpu_baseline": {"value": round(v, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                            "sample": f"{sample} of the {N_RAYS} rays per step", "cpu": cpu_model()},
           "e2e": {"value": round(v, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def cornell_extra(torch):
    """The plain path tracer on the procedural Cornell box, 256x256, 16 spp,
    max depth 8, NEE + MIS, hero-wavelength spectral (the C1 config) and RGB,
    plus RGB at the reference's effective settings (max depth 10), on the
    default (wavefront) schedule: Mpaths/s and Mrays/s; beside it the
    reference's own path tracer restated in CUDA and the CPU oracle's path
    tracer on all host cores (RGB, a bounded number of samples)."""
    from craystal_gb300 import scenes
    from craystal_gb300.api import PathTraceIntegrator, Scene, flatten_scene
    data, cam = scenes.cornell_box(seed=0, width=256, height=256)
    sc = Scene(data)
    sc.setCamera(cam)
    cfg = PathTraceIntegrator.Configs(maxDepth=8, rrThreshold=0.05, useMIS=True)
    spp, reps = 16, 5
    s = torch.cuda.current_stream()
    out = {"config": "cornell 256x256, 16 spp, max depth 8, NEE+MIS, default schedule (wavefront)"}
    # compat: the reference's effective settings (its Configs never reach the
    # kernel, so it always runs max depth 10, rr 0.05)
    for label, spectral, compat in (("spectral", True, False), ("rgb", False, False),
                                    ("rgb_compat_depth10", False, True)):
        integ = PathTraceIntegrator(cfg, compat=compat, spectral=spectral)
        integ.dispatch(sc, spp, readback=False)
        torch.cuda.synchronize()
        sc.film_clear()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for r in range(reps):
            integ.dispatch(sc, spp, first_sample=r * spp, stream=s.cuda_stream, readback=False)
        e1.record(s)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        rays = sc.render_ray_count()
        paths = 256 * 256 * spp * reps
        out[label] = {"Mpaths_s": round(paths / ms / 1e3, 2), "Mrays_s": round(rays / ms / 1e3, 2),
                      "ms_per_16spp": round(ms / reps, 3), "rays_per_path": round(rays / paths, 3)}
    # the reference's own path tracer restated (W x H grid of 16 x 16 blocks, a launch and a
    # device sync per sample, 36-byte nodes, closest-hit shadow rays, atomic film); RGB
    from baseline.restated import RestatedPathTracer
    ref = RestatedPathTracer(sc, flatten_scene(data))
    ref.render(cam, 2, max_depth=8, rr_threshold=0.05)
    torch.cuda.synchronize()
    t = time.perf_counter()
    _, ref_rays = ref.render(cam, spp, max_depth=8, rr_threshold=0.05)
    ref_s = time.perf_counter() - t
    out["restated_reference_path_tracer"] = {
        "Mpaths_s": round(256 * 256 * spp / ref_s / 1e6, 2), "Mrays_s": round(ref_rays / ref_s / 1e6, 2),
        "ms_per_16spp": round(ref_s * 1e3, 3)}
    out["speedup_over_restated_reference_rgb"] = round(out["rgb"]["Mpaths_s"] /
                                                       out["restated_reference_path_tracer"]["Mpaths_s"], 2)
    torch.cuda.synchronize()
    t = time.perf_counter()
    _, ref_rays = ref.render(cam, spp, max_depth=10, rr_threshold=0.05)
    ref_s = time.perf_counter() - t
    out["restated_reference_path_tracer_depth10"] = {
        "Mpaths_s": round(256 * 256 * spp / ref_s / 1e6, 2), "Mrays_s": round(ref_rays / ref_s / 1e6, 2),
        "ms_per_16spp": round(ref_s * 1e3, 3)}
    out["speedup_over_restated_reference_compat"] = round(
        out["rgb_compat_depth10"]["Mpaths_s"] / out["restated_reference_path_tracer_depth10"]["Mpaths_s"], 2)
    # the CPU oracle's path tracer, all host threads, a bounded sample of spp
    import oracle
    threads = oracle.hardware_threads()
    osc = oracle.OracleScene(flatten_scene(data))
    oc = oracle.make_camera(cam.posW, cam.target, cam.up, cam.fovY, 256, 256)
    t = time.perf_counter()
    _, orays = osc.render(oc, 8, 0.05, True, spp=1, threads=threads)
    one = time.perf_counter() - t
    cpu_spp = max(1, min(16, int(8.0 / max(one, 1e-3))))
    t = time.perf_counter()
    _, orays = osc.render(oc, 8, 0.05, True, spp=cpu_spp, first_sample=1, threads=threads)
    cpu_s = time.perf_counter() - t
    out["cpu_oracle"] = {"Mpaths_s": round(256 * 256 * cpu_spp / cpu_s / 1e6, 3),
                         "Mrays_s": round(orays / cpu_s / 1e6, 3), "threads": threads, "spp": cpu_spp}
    return out


def rel_mse(img, ref):
    """mean((I - R)^2 / (R^2 + 1e-2)) over pixels and channels, in FP64."""
    img = np.nan_to_num(np.asarray(img, np.float64))
    ref = np.nan_to_num(np.asarray(ref, np.float64))
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


def gpu_film_1spp(integ, sc):
    """The GPU film of one sample per pixel at sample index 0."""
    sc.film_clear()
    integ.dispatch(sc, 1, first_sample=0, readback=False)
    return sc.film_read()


def crop_parity(integ, sc, orgb, ow, rows, film=None):
    """Equal-seed comparison of a full GPU render at 1 spp (sample index 0)
    with the oracle's 1-spp render of rows [rows) (FP64 film): relMSE on the
    rows whose filter footprint lies inside the band, and the two films'
    mean radiance there."""
    r0, r1 = rows
    rgb, w = film if film is not None else gpu_film_1spp(integ, sc)
    band = slice(r0 + 1, r1 - 1)
    g = rgb[band] / w[band][..., None]
    o = orgb[band] / ow[band][..., None]
    return {"rows": [r0 + 1, r1 - 1], "spp": 1, "relmse_vs_oracle_equal_seed": rel_mse(g, o),
            "mean_gpu": [round(float(x), 5) for x in np.nanmean(g, axis=(0, 1))],
            "mean_oracle": [round(float(x), 5) for x in np.nanmean(o, axis=(0, 1))],
            "weight_max_rel_diff": float(np.max(np.abs(w[band] - ow[band]) / np.maximum(ow[band], 1e-12)))}


def c1_parity_extra(torch, chunks=128, chunk_spp=512, crop=(120, 136), crop_spp=4096):
    """Parity of the plain path tracer at the C1 configuration (Cornell box,
    256x256, 16 spp, max depth 8, rr 0.05, NEE + MIS):
      - equal seed: the GPU's 16-spp image against the oracle's (same sample
        indices 0..15), RGB and spectral;
      - a 65,536-spp reference from the GPU plain tracer, `chunks` renders of
        `chunk_spp` spp whose films are summed in FP64 on the host (sample
        indices from 1,000,000 on, disjoint from the images compared with it),
        spot-checked on rows [crop) against the oracle at `crop_spp` spp with
        its FP64 film;
      - the relMSE of the GPU's and the oracle's 16-spp images against that
        reference."""
    import oracle
    from craystal_gb300 import scenes
    from craystal_gb300.api import PathTraceIntegrator, Scene, flatten_scene
    data, cam = scenes.cornell_box(seed=0, width=256, height=256)
    sc = Scene(data)
    sc.setCamera(cam)
    cfg = PathTraceIntegrator.Configs(maxDepth=8, rrThreshold=0.05, useMIS=True)
    threads = oracle.hardware_threads()
    osc = oracle.OracleScene(flatten_scene(data))
    oc = oracle.make_camera(cam.posW, cam.target, cam.up, cam.fovY, 256, 256)
    out = {"config": "cornell 256x256, 16 spp, max depth 8, rr 0.05, NEE+MIS; relMSE = mean((I-R)^2/(R^2+1e-2))"}
    imgs = {}
    for label, spectral in (("rgb", False), ("spectral", True)):
        integ = PathTraceIntegrator(cfg, compat=False, spectral=spectral)
        sc.film_clear()
        integ.dispatch(sc, 16, readback=False)
        rgb, w = sc.film_read()
        img = rgb / w[..., None]
        (orgb, ow), _ = osc.render(oc, 8, 0.05, True, spp=16, threads=threads, spectral=spectral)
        oimg = orgb / ow[..., None]
        imgs[label] = (img, oimg)
        out[f"equal_seed_relmse_{label}"] = rel_mse(img, oimg)
    # the 65,536-spp reference: FP64 sum of the GPU films
    integ = PathTraceIntegrator(cfg, compat=False)
    acc = np.zeros((256, 256, 3))
    accw = np.zeros((256, 256))
    torch.cuda.synchronize()
    t = time.perf_counter()
    for k in range(chunks):
        sc.film_clear()
        integ.dispatch(sc, chunk_spp, first_sample=1_000_000 + chunk_spp * k, readback=False)
        rgb, w = sc.film_read()
        acc += rgb
        accw += w
    ref_s = time.perf_counter() - t
    ref = acc / accw[..., None]
    # spot check: the oracle's own FP64 film at crop_spp on a band of rows
    r0, r1 = crop
    t = time.perf_counter()
    (orgb, ow), _ = osc.render(oc, 8, 0.05, True, spp=crop_spp, first_sample=50_000_000, rows=(r0, r1),
                               threads=threads)
    crop_s = time.perf_counter() - t
    band = slice(r0 + 1, r1 - 1)  # rows whose filter footprint lies inside the rendered band
    ocrop = orgb[band] / ow[band][..., None]
    img, oimg = imgs["rgb"]
    out["reference"] = {"spp": chunks * chunk_spp, "film": "FP64 sum of GPU plain-tracer films",
                        "render_s": round(ref_s, 2)}
    out["reference_spot_check"] = {
        "rows": [r0 + 1, r1 - 1], "oracle_spp": crop_spp, "oracle_s": round(crop_s, 2),
        "relmse_reference_vs_oracle": rel_mse(ref[band], ocrop),
        "relmse_oracle_16spp_vs_oracle": rel_mse(oimg[band], ocrop),
        "note": "the oracle band's own noise at its spp is about 16/oracle_spp of its 16-spp error"}
    out["relmse_vs_reference_16spp"] = {"gpu": rel_mse(img, ref), "oracle": rel_mse(oimg, ref),
                                        "gpu_spectral": rel_mse(imgs["spectral"][0], ref),
                                        "oracle_spectral": rel_mse(imgs["spectral"][1], ref)}
    sc.close()
    return out


def c3_plain_extra(torch):
    """The radiance-cache config's scene rendered plain once, 1920x1080 at 64
    spp (after a 1-spp warm-up): the command its per-bounce launch list is
    taken from."""
    from craystal_gb300 import scenes
    from craystal_gb300.api import PathTraceIntegrator, Scene
    cfg = PathTraceIntegrator.Configs(maxDepth=16, rrThreshold=0.05, useMIS=True)
    plain = PathTraceIntegrator(cfg, compat=False)
    data, cam, env, sph = scenes.cache_scene(seed=0, width=1920, height=1080)
    sc = Scene(data)
    sc.setCamera(cam)
    sc.set_environment(env)
    sc.set_sphere_lights(sph)
    plain.dispatch(sc, 1, readback=False)
    sc.film_clear()
    torch.cuda.synchronize()
    t = time.perf_counter()
    plain.dispatch(sc, 64, readback=False)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    return {"config": "8 displaced icospheres (2.6M tris), 1920x1080, 64 spp, depth 16, plain", "s": round(dt, 4),
            "Mpaths_s": round(1920 * 1080 * 64 / dt / 1e6, 1), "rays": int(sc.render_ray_count())}


def c3_cached_frames_extra(torch, frames=32):
    """Cached frames of the radiance-cache config alone (1920x1080, depth 16,
    2^16 training records per frame), after 16 warm-up frames: ms per frame,
    the command the cached frames' launch list is taken from."""
    from craystal_gb300 import scenes
    from craystal_gb300.api import CachedPathTraceIntegrator, PathTraceIntegrator, RadianceCache, Scene
    cfg = PathTraceIntegrator.Configs(maxDepth=16, rrThreshold=0.05, useMIS=True)
    data, cam, env, sph = scenes.cache_scene(seed=0, width=1920, height=1080)
    sc = Scene(data)
    sc.setCamera(cam)
    sc.set_environment(env)
    sc.set_sphere_lights(sph)
    integ = CachedPathTraceIntegrator(cfg, train_samples=1 << 16, cache=RadianceCache(seed=1))
    integ.dispatch(sc, 16, first_sample=2_000_000, readback=False)
    torch.cuda.synchronize()
    t = time.perf_counter()
    integ.dispatch(sc, frames, first_sample=3_000_000, readback=False)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    return {"config": "8 displaced icospheres (2.6M tris), 1920x1080, depth 16, cached frames, 2^16 records",
            "frames": frames, "ms_per_cached_frame": round(1e3 * dt / frames, 3),
            "train_every_reached": int(integ.stats.last_train_every)}


def c3_extra(torch, res=(1920, 1080), budgets=(16, 64), trials=5):
    """The radiance-cache config: 8 displaced icospheres (2.6M triangles),
    Principled materials, constant environment 0.5 and one sphere light, max
    depth 16, 1920x1080.  Plain throughput at 64 spp; equal-seed parity of a
    64-row band against the oracle; the equal-time cache comparison
    (reference: 4096 spp of the plain tracer, FP64 film sum, with its own
    noise estimated from its two halves; the cache trained from scratch
    inside its time on 2^16 path-suffix records per frame, the configured
    batch, and beside it on 8,192; `trials` independent trials per budget)."""
    from craystal_gb300 import scenes
    from craystal_gb300.api import CachedPathTraceIntegrator, PathTraceIntegrator, RadianceCache, Scene
    cfg = PathTraceIntegrator.Configs(maxDepth=16, rrThreshold=0.05, useMIS=True)
    plain = PathTraceIntegrator(cfg, compat=False)

    def timed(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t

    data, cam, env, sph = scenes.cache_scene(seed=0, width=1920, height=1080)
    sc = Scene(data)
    sc.setCamera(cam)
    sc.set_environment(env)
    sc.set_sphere_lights(sph)
    plain.dispatch(sc, 1, readback=False)
    sc.film_clear()
    dt = timed(lambda: plain.dispatch(sc, 64, readback=False))
    rays = sc.render_ray_count()
    out = {"config": "8 displaced icospheres (2.6M tris), Principled, env 0.5 + sphere light, depth 16",
           "plain_1080p_64spp": {"s": round(dt, 3), "Mpaths_s": round(1920 * 1080 * 64 / dt / 1e6, 1),
                                 "Mrays_s": round(rays / dt / 1e6, 1), "triangles": int(sc.n_tris)}}
    # the CPU oracle on all host threads: a crop of the 64 rows at the image
    # centre at 1 spp, scaled linearly to the full 1920x1080 x 64 spp render
    import oracle
    from craystal_gb300.api import flatten_scene
    threads = oracle.hardware_threads()
    osc = oracle.OracleScene(flatten_scene(data))
    osc.set_lights(env, sph)
    oc = oracle.make_camera(cam.posW, cam.target, cam.up, cam.fovY, 1920, 1080)
    t = time.perf_counter()
    (orgb, ow), orays = osc.render(oc, 16, 0.05, True, spp=1, rows=(508, 572), threads=threads)
    cpu_s = time.perf_counter() - t
    cpu_rate = 1920 * 64 / cpu_s
    out["cpu_oracle"] = {"Mpaths_s": round(cpu_rate / 1e6, 4), "Mrays_s": round(orays / cpu_s / 1e6, 4),
                         "threads": threads, "sample": "rows 508-571 at 1 spp",
                         "projected_1080p_64spp_s": round(1920 * 1080 * 64 / cpu_rate, 1)}
    del osc
    # parity at this configuration: the GPU's 1-spp render at the same sample
    # index (0) against the oracle's band, on the rows whose filter footprint
    # lies inside it
    out["parity"] = crop_parity(plain, sc, orgb, ow, (508, 572))
    w, h = res
    cam.setSensor(type(cam.sensor)((w, h)))
    sc.setCamera(cam)
    acc_half = [np.zeros((h, w, 3)), np.zeros((h, w, 3))]
    accw_half = [np.zeros((h, w)), np.zeros((h, w))]
    for k in range(8):
        sc.film_clear()
        plain.dispatch(sc, 512, first_sample=1_000_000 + 512 * k, readback=False)
        rgb, wt = sc.film_read()
        acc_half[k % 2] += rgb
        accw_half[k % 2] += wt
    acc = acc_half[0] + acc_half[1]
    accw = accw_half[0] + accw_half[1]
    ref = acc / accw[..., None]

    def rel_mse(rgb, wt):
        img = np.nan_to_num((rgb / wt[..., None]).astype(np.float64))
        return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))

    # the reference's own noise: the relMSE of one half of it against the other,
    # halved again (each half carries twice the full reference's variance)
    half_a = acc_half[0] / accw_half[0][..., None]
    half_b = acc_half[1] / accw_half[1][..., None]
    ref_noise = 0.25 * float(np.mean((half_a - half_b) ** 2 / (ref ** 2 + 1e-2)))
    for label, samples in (("equal_time", 1 << 16), ("equal_time_8192_records", 8192)):
        probe = CachedPathTraceIntegrator(cfg, train_samples=samples, cache=RadianceCache(seed=1))
        probe.dispatch(sc, 16, first_sample=2_000_000, readback=False)
        t_frame = timed(lambda: probe.dispatch(sc, 32, first_sample=3_000_000, readback=False)) / 32
        rows = equal_time_trials(sc, cfg, plain, rel_mse, timed, t_frame, budgets, trials=trials,
                                 train_samples=samples)
        out[label] = {"resolution": [w, h], "reference_spp": 4096, "reference_noise_relmse": round(ref_noise, 6),
                      "train_samples_per_frame": samples, "ms_per_cached_frame": round(t_frame * 1e3, 3),
                      "train_every": "adaptive", "train_every_reached": int(probe.stats.last_train_every),
                      "trials_per_budget": trials, "budgets": rows}
    sc.close()
    return out


def mlp_extra(torch):
    """The radiance-cache network alone on device buffers (the calls the
    cached integrator makes per frame): inference of 4,194,304 queries
    (inputs and outputs larger than L2) and one Adam training step on 65,536
    records, CUDA events on the launching stream.  FLOPs: 2 x 27,840 (the
    weights) per query forward; 3x that per training record (forward, data
    gradient, weight gradient).  Peak: the measured dense bf16 tensor-core
    rate (FP16 runs at the same rate)."""
    from craystal_gb300.api import RadianceCache
    net = RadianceCache(seed=3)
    n_inf, n_tr = 1 << 22, 1 << 16
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand((n_inf, 7), device="cuda", generator=g)
    y = torch.empty((n_inf, 3), device="cuda")
    t = torch.rand((n_tr, 3), device="cuda", generator=g)
    s = torch.cuda.current_stream()

    def ev_ms(fn, reps):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            fn()
        e1.record(s)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    ms_inf = ev_ms(lambda: net.infer_device(x.data_ptr(), n_inf, y.data_ptr(), s.cuda_stream), 20)
    ms_tr = ev_ms(lambda: net.train_step_device(x.data_ptr(), t.data_ptr(), n_tr, s.cuda_stream), 20)
    net.close()
    peak, src = tensor_peak()
    f = 2 * 27840
    inf_tf = f * n_inf / (ms_inf * 1e-3) / 1e12
    tr_tf = 3 * f * n_tr / (ms_tr * 1e-3) / 1e12
    return {"inference": {"queries": n_inf, "ms": round(ms_inf, 4), "Mqueries_s": round(n_inf / ms_inf / 1e3, 1),
                          "tflops": round(inf_tf, 1), "frac": round(inf_tf / peak, 4)},
            "train_step": {"records": n_tr, "ms": round(ms_tr, 4), "tflops": round(tr_tf, 1),
                           "frac": round(tr_tf / peak, 4)},
            "peak_tflops": peak, "peak_source": f"{src} dense bf16 (burst)",
            "instruction": {"inference": "tcgen05.mma kind::f16, M128, TMEM accumulators, weights by cp.async.bulk",
                            "training": "tcgen05.mma kind::f16, M128: forward, backward data gradients and "
                                        "MN-major weight gradients accumulated in TMEM over each CTA's tiles"}}


def wavefront_extra(torch):
    """The two schedules of the plain path tracer on the same paths: the
    megakernel (one thread per pixel, all bounces in registers) and the
    wavefront variant (extend, sort by material, shade per bounce).  Scenes:
    the Cornell box 256x256 and a 500k-triangle box-clutter scene 512x512,
    16 spp, max depth 10, NEE + MIS."""
    from craystal_gb300 import scenes
    from craystal_gb300.api import PathTraceIntegrator, Scene
    out = {}
    for name, (data, cam) in (("cornell_256", scenes.cornell_box(seed=0, width=256, height=256)),
                              ("box_clutter_500k_512", scenes.box_clutter(3, 500000, 512, 512))):
        sc = Scene(data)
        sc.setCamera(cam)
        cfg = PathTraceIntegrator.Configs(maxDepth=10, rrThreshold=0.05, useMIS=True)
        row = {}
        for label, wf in (("megakernel", False), ("wavefront", True)):
            integ = PathTraceIntegrator(cfg, compat=False, wavefront=wf)
            integ.dispatch(sc, 4, readback=False)
            torch.cuda.synchronize()
            sc.film_clear()
            t = time.perf_counter()
            integ.dispatch(sc, 16, readback=False)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t
            paths = cam.sensor.size[0] * cam.sensor.size[1] * 16
            row[label] = {"ms": round(dt * 1e3, 2), "Mpaths_s": round(paths / dt / 1e6, 2),
                          "Mrays_s": round(sc.render_ray_count() / dt / 1e6, 1)}
        row["wavefront_over_megakernel_time"] = round(row["wavefront"]["ms"] / row["megakernel"]["ms"], 3)
        out[name] = row
        sc.close()
    return out


def large_scene_extra(torch, spp=32, with_cache=True):
    """The large workload: a 4096 x 4096 fBm heightfield (33.5M triangles)
    plus 10k boxes, Principled materials, a sun sphere light and a constant
    sky, rendered at 3840 x 2160, 32 spp, max depth 12, NEE + MIS, on the
    wavefront schedule; with the host generation time, the GPU BVH build
    time and the device memory the scene and its render hold."""
    from craystal_gb300 import scenes
    from craystal_gb300.api import PathTraceIntegrator, Scene
    t = time.perf_counter()
    data, cam, env, sun = scenes.large_terrain_scene()
    gen_s = time.perf_counter() - t
    torch.cuda.synchronize()
    free0, total = torch.cuda.mem_get_info()
    t = time.perf_counter()
    sc = Scene(data)
    sc.setCamera(cam)
    sc.set_environment(env)
    sc.set_sphere_lights(sun)
    torch.cuda.synchronize()
    create_s = time.perf_counter() - t
    st = sc.bvh_stats()
    n_tris = sc.n_tris
    from craystal_gb300.api import flatten_scene
    flat = flatten_scene(data)
    del data
    integ = PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=12, rrThreshold=0.05, useMIS=True), compat=False)
    integ.dispatch(sc, 1, readback=False)  # allocates the path state
    torch.cuda.synchronize()
    sc.film_clear()
    t = time.perf_counter()
    integ.dispatch(sc, spp, readback=False)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    free1, _ = torch.cuda.mem_get_info()
    rays = sc.render_ray_count()
    rgb, w = sc.film_read()
    # for parity below: the 1-spp film at sample index 0 and the GPU's tree
    film1 = gpu_film_1spp(integ, sc)
    gnodes, gmap = sc.bvh_export()
    cached = c5_cache_equal_time(torch, sc, integ) if with_cache else None
    paths = 3840 * 2160 * spp
    out = {"config": "terrain 4096^2 (fBm, 6 octaves) + 10k boxes, 3840x2160, 32 spp, depth 12, sun + sky",
           "triangles": int(n_tris), "host_generation_s": round(gen_s, 2), "scene_create_s": round(create_s, 2),
           "gpu_bvh_build_ms": round(st["build_ms"], 1), "bvh_device_mib": round(st["device_bytes"] / 2 ** 20, 1),
           "device_gib_held": round((free0 - free1) / 2 ** 30, 2), "render_s": round(dt, 3),
           "Mpaths_s": round(paths / dt / 1e6, 1), "Mrays_s": round(rays / dt / 1e6, 1),
           "rays_per_path": round(rays / paths, 3),
           "mean_rgb": [round(float(x), 4) for x in np.nanmean(rgb / w[..., None], axis=(0, 1))]}
    sc.close()
    # the CPU oracle on all host threads: its own BVH build, then a crop of the
    # 16 rows at the image centre at 1 spp, scaled linearly to the full render
    import oracle
    threads = oracle.hardware_threads()
    t = time.perf_counter()
    osc = oracle.OracleScene(flat)
    build_s = time.perf_counter() - t
    del flat
    out["tree_vs_oracle"] = compare_trees(gnodes, gmap, *osc.bvh_export())
    del gnodes, gmap
    osc.set_lights(env, sun)
    oc = oracle.make_camera(cam.posW, cam.target, cam.up, cam.fovY, 3840, 2160)
    t = time.perf_counter()
    (orgb, ow), orays = osc.render(oc, 12, 0.05, True, spp=1, rows=(1072, 1088), threads=threads)
    cpu_s = time.perf_counter() - t
    cpu_rate = 3840 * 16 / cpu_s
    out["cpu_oracle"] = {"bvh_build_s": round(build_s, 1), "Mpaths_s": round(cpu_rate / 1e6, 4),
                         "Mrays_s": round(orays / cpu_s / 1e6, 4), "threads": threads,
                         "sample": "rows 1072-1087 at 1 spp",
                         "projected_render_s": round(paths / cpu_rate, 1)}
    del osc
    out["parity"] = crop_parity(None, None, orgb, ow, (1072, 1088), film=film1)
    if cached is not None:
        out["radiance_cache_equal_time"] = cached
    return out


def c5_cache_equal_time(torch, sc, plain, rows=(824, 1336), ref_chunks=16, ref_spp=32, budgets=(32,), trials=3):
    """The radiance cache on the large scene at full resolution (3840x2160,
    depth 12): at equal time with the plain tracer's 32-spp render, relMSE
    on a 512-row band at the image centre against a plain reference of
    ref_chunks x ref_spp spp (FP64 film sum), whose own noise is estimated
    from its two halves.  The cache trains from scratch inside its time on
    2^16 path-suffix records per frame."""
    from craystal_gb300.api import CachedPathTraceIntegrator, RadianceCache
    cfg = plain.configs
    r0, r1 = rows
    halves = [[0.0, 0.0], [0.0, 0.0]]
    for k in range(ref_chunks):
        sc.film_clear()
        plain.dispatch(sc, ref_spp, first_sample=1_000_000 + ref_spp * k, readback=False)
        rgb, w = sc.film_read()
        h = halves[k % 2]
        h[0] = h[0] + rgb[r0:r1].astype(np.float64)
        h[1] = h[1] + w[r0:r1].astype(np.float64)
    ref = (halves[0][0] + halves[1][0]) / (halves[0][1] + halves[1][1])[..., None]
    ha = halves[0][0] / halves[0][1][..., None]
    hb = halves[1][0] / halves[1][1][..., None]
    ref_noise = 0.25 * float(np.mean((ha - hb) ** 2 / (ref ** 2 + 1e-2)))

    def crop_rel_mse(rgb, w):
        img = np.nan_to_num((rgb[r0:r1] / w[r0:r1][..., None]).astype(np.float64))
        return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))

    def timed(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t

    samples = 1 << 16
    probe = CachedPathTraceIntegrator(cfg, train_samples=samples, cache=RadianceCache(seed=1))
    probe.dispatch(sc, 8, first_sample=2_000_000, readback=False)
    t_frame = timed(lambda: probe.dispatch(sc, 16, first_sample=3_000_000, readback=False)) / 16
    rows_out = equal_time_trials(sc, cfg, plain, crop_rel_mse, timed, t_frame, budgets, trials=trials,
                                 train_samples=samples)
    return {"resolution": [3840, 2160], "crop_rows": [r0, r1], "reference_spp": ref_chunks * ref_spp,
            "reference_noise_relmse": round(ref_noise, 6), "train_samples_per_frame": samples,
            "ms_per_cached_frame": round(t_frame * 1e3, 3), "train_every_reached": int(probe.stats.last_train_every),
            "budgets": rows_out}


def compare_trees(gnodes, gmap, onodes, omap):
    """The GPU's tree against the oracle's (the reference's host build), both
    in the reference layout: node count, every box as bits, topology, and
    the set of triangles in every leaf (slot order inside a leaf may differ,
    since the builders partition in different orders)."""
    out = {"nodes_gpu": int(len(gnodes)), "nodes_oracle": int(len(onodes))}
    same_size = len(gnodes) == len(onodes) and len(gmap) == len(omap)
    boxes = same_size and (np.array_equal(gnodes["bmin"].view(np.uint32), onodes["bmin"].view(np.uint32)) and
                           np.array_equal(gnodes["bmax"].view(np.uint32), onodes["bmax"].view(np.uint32)))
    topo = same_size and (np.array_equal(gnodes["is_leaf"], onodes["is_leaf"]) and
                          np.array_equal(gnodes["a"], onodes["a"]) and np.array_equal(gnodes["b"], onodes["b"]))
    leaves_same = False
    if topo:
        lf = gnodes[gnodes["is_leaf"] == 1]
        starts, counts = lf["a"].astype(np.int64), lf["b"].astype(np.int64)
        # the slots of every leaf, leaf after leaf, tagged with the leaf's number
        within = np.arange(counts.sum()) - np.repeat(np.cumsum(counts) - counts, counts)
        slots = np.repeat(starts, counts) + within
        leaf = np.repeat(np.arange(len(lf), dtype=np.int64), counts)
        if len(slots) == len(gmap) and len(np.unique(slots)) == len(gmap):
            g = np.sort(leaf << 32 | gmap[slots].astype(np.int64))
            o = np.sort(leaf << 32 | omap[slots].astype(np.int64))
            leaves_same = bool(np.array_equal(g, o))
    out.update({"boxes_bit_equal": bool(boxes), "topology_equal": bool(topo), "leaf_sets_equal": leaves_same,
                "tree_equal": bool(boxes and topo and leaves_same)})
    return out


def cache_frames_extra(torch, res=512, frames=32):
    """The cached integrator's frames alone (Cornell res x res, max depth 8,
    NEE + MIS, training every frame) after 16 warm-up frames: ms per frame
    and per plain sample of the same image, for profiling."""
    from craystal_gb300 import scenes
    from craystal_gb300.api import CachedPathTraceIntegrator, PathTraceIntegrator, Scene
    data, cam = scenes.cornell_box(seed=0, width=res, height=res)
    sc = Scene(data)
    sc.setCamera(cam)
    cfg = PathTraceIntegrator.Configs(maxDepth=8, rrThreshold=0.05, useMIS=True)
    integ = CachedPathTraceIntegrator(cfg)
    integ.dispatch(sc, 16, first_sample=5_000_000, readback=False)
    plain = PathTraceIntegrator(cfg, compat=False)
    plain.dispatch(sc, 4, readback=False)
    torch.cuda.synchronize()
    t = time.perf_counter()
    integ.dispatch(sc, frames, readback=False)
    torch.cuda.synchronize()
    tc = time.perf_counter() - t
    t = time.perf_counter()
    plain.dispatch(sc, frames, readback=False)
    torch.cuda.synchronize()
    tp = time.perf_counter() - t
    return {"config": f"cornell {res}x{res}, max depth 8", "frames": frames,
            "cache_ms_per_frame": round(1e3 * tc / frames, 3), "plain_ms_per_spp": round(1e3 * tp / frames, 3)}


def equal_time_trials(sc, cfg, plain, rel_mse, timed, t_frame, budgets, trials=3, train_every=0,
                      train_samples=8192):
    """Per budget (plain spp): `trials` independent pairs of (plain render,
    fresh cache trained and rendering inside the plain render's time) on
    disjoint sample indices and network seeds; relMSE is heavy-tailed
    (rare bright paths), so every trial and the median ratio are reported."""
    from craystal_gb300.api import CachedPathTraceIntegrator, RadianceCache
    rows = []
    for spp in budgets:
        trials_out = []
        for k in range(trials):
            sc.film_clear()
            t_plain = timed(lambda: plain.dispatch(sc, spp, first_sample=10_000_000 * (k + 1), readback=False))
            e_plain = rel_mse(*sc.film_read())
            frames = max(1, int(t_plain / t_frame))
            integ = CachedPathTraceIntegrator(cfg, train_every=train_every, train_samples=train_samples,
                                              cache=RadianceCache(seed=k))
            sc.film_clear()
            t_cache = timed(lambda: integ.dispatch(sc, frames, first_sample=50_000_000 + 10_000_000 * k,
                                                   readback=False))
            e_cache = rel_mse(*sc.film_read())
            trials_out.append({"plain_s": round(t_plain, 4), "plain_relmse": round(e_plain, 5), "cache_frames": frames,
                               "cache_s": round(t_cache, 4), "cache_relmse": round(e_cache, 5),
                               "ratio": round(e_plain / e_cache, 3)})
        ratios = sorted(t["ratio"] for t in trials_out)
        rows.append({"plain_spp": spp, "median_ratio_plain_over_cache": ratios[len(ratios) // 2],
                     "trials": trials_out})
    return rows


def cache_extra(torch, res=512, budgets=(64, 256, 1024)):
    """Equal-time relMSE of the radiance-cache integrator against the plain
    path tracer on the Cornell box (res x res, max depth 8, NEE + MIS), both
    on the default (wavefront) schedule.  The reference is the plain tracer
    at 16384 spp with its films of 512-spp passes summed in FP64.  For each
    budget the plain tracer renders that many spp in time T; a fresh cache
    (untrained network) then renders, trains and renders as many frames (1
    spp each) as fit in T, its training included."""
    from craystal_gb300 import scenes
    from craystal_gb300.api import CachedPathTraceIntegrator, PathTraceIntegrator, RadianceCache, Scene
    data, cam = scenes.cornell_box(seed=0, width=res, height=res)
    sc = Scene(data)
    sc.setCamera(cam)
    cfg = PathTraceIntegrator.Configs(maxDepth=8, rrThreshold=0.05, useMIS=True)
    plain = PathTraceIntegrator(cfg, compat=False)
    acc = np.zeros((res, res, 3))
    accw = np.zeros((res, res))
    for k in range(32):
        sc.film_clear()
        plain.dispatch(sc, 512, first_sample=1_000_000 + 512 * k, readback=False)
        rgb, w = sc.film_read()
        acc += rgb
        accw += w
    ref = acc / accw[..., None]

    def rel_mse(rgb, w):
        img = np.nan_to_num((rgb / w[..., None]).astype(np.float64))
        return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))

    def timed(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t

    # cost of a cached frame, from a separate cache
    probe = CachedPathTraceIntegrator(cfg, cache=RadianceCache(seed=1))
    probe.dispatch(sc, 16, first_sample=2_000_000, readback=False)
    t_frame = timed(lambda: probe.dispatch(sc, 32, first_sample=3_000_000, readback=False)) / 32
    rows = equal_time_trials(sc, cfg, plain, rel_mse, timed, t_frame, budgets)
    return {"config": f"cornell {res}x{res}, max depth 8, NEE+MIS; reference 16384 spp plain, FP64 film sum; "
                      "cache trained from scratch inside its time; 3 independent trials per budget",
            "ms_per_cached_frame": round(t_frame * 1e3, 3), "train_every": "adaptive",
            "train_every_reached": int(probe.stats.last_train_every), "query_vertex": 1, "budgets": rows}


def batch_extra(torch, n_scenes=64):
    """The batched workload: 64 random-box-clutter scenes (triangles
    log-uniform 10k-500k, resolution from {128..1024}^2, spp log-uniform 4-256,
    depth 8-16) replayed from captured CUDA graphs on the schedule the
    autotuner picks on a 1/16-spp probe of the same batch (persistent
    megakernel or many-scene wavefront); compared with the same renders
    dispatched scene by scene."""
    from craystal_gb300 import scenes
    from craystal_gb300.api import BatchRenderer, PathTraceIntegrator, Scene
    params = scenes.batch_workload(n_scenes)
    scs, integs = [], []
    for p in params:
        data, cam = scenes.box_clutter(p["seed"], p["tris"], p["res"], p["res"])
        sc = Scene(data)
        sc.setCamera(cam)
        scs.append(sc)
        integs.append(PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=p["depth"], rrThreshold=0.05),
                                          compat=False))
    probe = BatchRenderer(scs, integs, [max(1, p["spp"] // 16) for p in params])
    tune = probe.autotune()
    probe.close()
    b = BatchRenderer(scs, integs, [p["spp"] for p in params])
    b.set_tuning(tune["best"]["tile"], tune["best"]["spp_per_item"], wave_log2=tune["best"]["wave_log2"])

    def timed(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t

    b.render()  # builds the work list and the graph
    for sc in scs:
        sc.film_clear()
    t_batch = timed(b.render)
    rays = sum(sc.render_ray_count() for sc in scs)
    # the scenes whose reference is cheap (resolution <= 256) carry the error comparison
    small = [i for i, p in enumerate(params) if p["res"] <= 256]
    plain_films = {i: scs[i].film_read() for i in small}
    # one untimed sample per scene first, so that per-scene dispatch is timed
    # with its path-state buffers already allocated, as the batch's are
    for sc, integ in zip(scs, integs):
        integ.dispatch(sc, 1, first_sample=1 << 30, readback=False)
    for sc in scs:
        sc.film_clear()
    t_seq = timed(lambda: [integ.dispatch(sc, p["spp"], readback=False) for sc, integ, p in zip(scs, integs, params)])
    paths = sum(p["res"] ** 2 * p["spp"] for p in params)
    out = {"config": f"{n_scenes} box-clutter scenes from captured CUDA graphs",
           "triangles": int(sum(sc.n_tris for sc in scs)), "paths": int(paths), "rays": int(rays),
           "batched_s": round(t_batch, 3), "batched_Mpaths_s": round(paths / t_batch / 1e6, 1),
           "batched_Mrays_s": round(rays / t_batch / 1e6, 1), "per_scene_dispatch_s": round(t_seq, 3),
           "speedup_vs_per_scene": round(t_seq / t_batch, 3), "tuning": tune["best"]}
    out["radiance_cache"] = batch_cached_extra(torch, b, scs, integs, params, small, plain_films, timed, t_batch)
    out["breakdown"] = batch_breakdown(torch, scs, integs, params, tune["best"], t_batch, timed)
    return out


def batch_breakdown(torch, scs, integs, params, tuning, t_batch, timed):
    """Where the batched workload's time goes.  Every scene dispatched alone
    (synchronised) gives its own time; the scenes with at least one wave of
    paths (2^wave_log2) render on their own waves inside the batch too, so
    only the rest can gain from sharing waves, which bounds the batch's
    speed-up over per-scene dispatch (Amdahl).  The shared part's own
    speed-up is their summed per-scene time against the batch time left
    after the own-wave scenes.  Beside it, the reference's dispatch
    structure (Core/Integrator.cu:246-259: one launch and one device
    synchronisation per sample per scene) run with this library's kernels."""
    wave = 1 << tuning["wave_log2"] if tuning.get("wave_log2") else None
    per = []
    for sc, integ, p in zip(scs, integs, params):
        sc.film_clear()
        per.append(timed(lambda: integ.dispatch(sc, p["spp"], readback=False)))
    per = np.array(per)
    paths = np.array([p["res"] ** 2 * p["spp"] for p in params], dtype=np.float64)
    own = paths >= wave if wave else np.zeros(len(params), bool)
    t_own, t_shared_seq = float(per[own].sum()), float(per[~own].sum())
    classes = {}
    for r in sorted({p["res"] for p in params}):
        m = np.array([p["res"] == r for p in params])
        classes[str(r)] = {"scenes": int(m.sum()), "paths_share": round(float(paths[m].sum() / paths.sum()), 4),
                           "time_share": round(float(per[m].sum() / per.sum()), 4),
                           "Mpaths_s": round(float(paths[m].sum() / per[m].sum() / 1e6), 1)}

    def per_spp():
        for sc, integ, p in zip(scs, integs, params):
            for k in range(p["spp"]):
                integ.dispatch(sc, 1, first_sample=k, readback=False)
                torch.cuda.synchronize()

    for sc in scs:
        sc.film_clear()
    t_spp = timed(per_spp)
    t_shared_batch = max(t_batch - t_own, 1e-9)
    return {"per_scene_sum_s": round(float(per.sum()), 3), "by_resolution": classes,
            "own_wave_scenes": int(own.sum()), "own_wave_paths_share": round(float(paths[own].sum() / paths.sum()), 4),
            "own_wave_time_s": round(t_own, 3), "shared_scenes_per_scene_s": round(t_shared_seq, 4),
            "shared_scenes_in_batch_s": round(t_shared_batch, 4),
            "shared_part_speedup": round(t_shared_seq / t_shared_batch, 2),
            "amdahl_bound_vs_per_scene": round(float(per.sum()) / t_own, 3) if t_own > 0 else None,
            "per_spp_dispatch_s": round(t_spp, 3), "speedup_vs_per_spp_dispatch": round(t_spp / t_batch, 2)}


def batch_cached_extra(torch, b, scs, integs, params, small, plain_films, timed, t_plain, ref_mult=8):
    """The radiance-cache form of the batched workload: every scene renders
    its spp as cached frames (one sample per pixel each) with a network of
    its own, trained from scratch during the render, all scenes advancing
    wave by wave together on their own streams (cr_batch_render_cached).
    Beside the time, each scene with resolution <= 256 is checked against
    its own plain reference (ref_mult x its spp, FP64 film): relMSE of its
    cached film and of its plain batched film at the same spp."""
    from craystal_gb300.api import RadianceCache
    caches = [RadianceCache(seed=100 + i) for i in range(len(scs))]
    for sc in scs:
        sc.film_clear()
    t_cached = timed(lambda: b.render_cached(caches))
    cached_films = {i: scs[i].film_read() for i in small}
    ratios, rows = [], []
    for i in small:
        sc, p = scs[i], params[i]
        sc.film_clear()
        integs[i].dispatch(sc, ref_mult * p["spp"], first_sample=1_000_000, readback=False)
        rgb, w = sc.film_read()
        ref = rgb.astype(np.float64) / w.astype(np.float64)[..., None]
        e = {}
        for label, (frgb, fw) in (("plain", plain_films[i]), ("cached", cached_films[i])):
            e[label] = rel_mse(frgb / fw[..., None], ref)
        ratios.append(e["plain"] / e["cached"])
        rows.append({"scene": i, "res": p["res"], "spp": p["spp"], "plain_relmse": round(e["plain"], 5),
                     "cached_relmse": round(e["cached"], 5)})
    for c in caches:
        c.close()
    ratios.sort()
    return {"cached_s": round(t_cached, 3), "plain_batched_s": round(t_plain, 3),
            "time_ratio_cached_over_plain": round(t_cached / t_plain, 3), "frames_per_scene": "its spp",
            "checked_scenes": len(small), "reference": f"plain, {ref_mult}x each scene's spp, FP64 film",
            "median_relmse_ratio_plain_over_cached": round(ratios[len(ratios) // 2], 3) if ratios else None,
            "scenes": rows}


def restated_reference_extra(torch, sc, flat, d_rays, n, d_hits_ours, reps=3):
    """The reference's own traversal restated in CUDA (baseline/restated:
    36-byte variant nodes, per-box division, 64-entry local stack, indexed
    vertex fetches, default FMA contraction) on the same rays and the same
    reference-layout tree: its Mrays/s and how many of its hits equal ours."""
    from baseline.restated import RestatedTraversal
    ref = RestatedTraversal(sc, flat)
    out = torch.empty(n * 16, dtype=torch.uint8, device=d_rays.device)
    s = torch.cuda.current_stream()
    ref.trace_closest_device(d_rays.data_ptr(), n, out.data_ptr(), s.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        ref.trace_closest_device(d_rays.data_ptr(), n, out.data_ptr(), s.cuda_stream)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    a = out.view(torch.int32).view(-1, 4).cpu().numpy()
    b = d_hits_ours.view(torch.int32).view(-1, 4).cpu().numpy()
    return {"kernel": "restated BVHData::intersect, one thread per ray", "ms_per_launch": round(ms, 3),
            "Mrays_s": round(n / ms / 1e3, 2), "prim_equal_fraction": round(float((a[:, 0] == b[:, 0]).mean()), 6),
            "bit_equal_fraction": round(float((a == b).all(axis=1).mean()), 6)}


def run_ours(args):
    import torch
    import torch.distributed as dist
    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    import craystal_gb300 as cg
    from craystal_gb300 import scenes
    from craystal_gb300.api import Scene, flatten_scene
    cg.load().cr_set_device(local)

    data = scenes.random_triangle_scene(N_TRIS, TRI_SEED)
    t0 = time.perf_counter()
    sc = Scene(data)
    build_wall = time.perf_counter() - t0
    st = sc.bvh_stats()
    sc.set_traversal(args.traversal)
    rays = scenes.random_rays(N_RAYS, RAY_SEED)
    raw = torch.from_numpy(rays.view(np.uint8))
    d_rays = raw.to(f"cuda:{local}")
    d_hits = torch.empty(N_RAYS * 16, dtype=torch.uint8, device=f"cuda:{local}")
    s = torch.cuda.current_stream()

    def step():
        sc.trace_closest_device(d_rays.data_ptr(), N_RAYS, d_hits.data_ptr(), s.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    launches0 = cg.kernel_launch_count()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(args.steps):
        step()
    e1.record(s)
    e1.synchronize()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = cg.kernel_launch_count() - launches0
    clk = clocks.stop()
    ms = slowest_rank_ms(ms, world, f"cuda:{local}")
    value = N_RAYS * args.steps * world / (ms * 1e-3) / 1e6
    kernel_ms = ms / args.steps  # one launch per step

    # e2e: host buffers through the C ABI, host<->device transfers inside the timed region
    # (pinned arrays: the library has the GPU read and write them in place)
    pin_r = torch.empty(N_RAYS * 32, dtype=torch.uint8).pin_memory()
    pin_r.numpy()[:] = rays.view(np.uint8)
    pin_h = torch.empty(N_RAYS * 16, dtype=torch.uint8).pin_memory()
    from craystal_gb300._lib import check, load
    lib = load()
    rp, hp = pin_r.data_ptr(), pin_h.data_ptr()
    check(lib.cr_trace_closest(sc.handle, rp, N_RAYS, hp))
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        check(lib.cr_trace_closest(sc.handle, rp, N_RAYS, hp))
    e2e_s = slowest_rank_ms((time.perf_counter() - t0) * 1e3, world, f"cuda:{local}") * 1e-3
    e2e = N_RAYS * e2e_steps * world / e2e_s / 1e6
    # the host-path result is the device-path result
    hits_host = pin_h.numpy().view(cg.HIT_DTYPE)
    hits_dev = d_hits.cpu().numpy().view(cg.HIT_DTYPE)
    same = bool(np.array_equal(hits_host.view(np.uint32), hits_dev.view(np.uint32)))

    extra = {"bvh": {"nodes": st["node_count"], "leaves": st["leaf_count"], "max_depth": st["max_depth"],
                     "gpu_build_ms": round(st["build_ms"], 2), "scene_create_wall_s": round(build_wall, 3),
                     "device_mib": round(st["device_bytes"] / 2 ** 20, 1)},
             "host_path_matches_device_path": same,
             "hit_fraction": round(float((hits_dev["prim"] != cg.CR_MISS).mean()), 4)}
    if not args.skip_extra and world == 1:
        extra["two_level_traversal"] = two_level_extra(torch, sc, d_rays, N_RAYS, hits_dev, kernel_ms)
    # the extras are single-GPU configurations (and time the CPU oracle on the
    # host's cores): a replica run under torchrun measures the ray cast only
    if not args.skip_extra and world == 1:
        extra["restated_reference_kernel"] = restated_reference_extra(torch, sc, flatten_scene(data), d_rays, N_RAYS,
                                                                      d_hits)
        extra["path_tracer"] = cornell_extra(torch)
        extra["c1_parity"] = c1_parity_extra(torch)
        extra["wavefront_vs_megakernel"] = wavefront_extra(torch)
        extra["radiance_cache_network"] = mlp_extra(torch)
        extra["radiance_cache_equal_time"] = cache_extra(torch, args.cache_res)
        extra["radiance_cache_scene"] = c3_extra(torch)
        extra["batched_scenes"] = batch_extra(torch, args.batch_scenes)
        extra["large_scene"] = large_scene_extra(torch)

    out = {"metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
           "config": {"workload": WORKLOAD, "triangles": N_TRIS, "rays_per_step": N_RAYS,
                      "parallelism": "replicas" if world > 1 else "single", "bvh": "GPU binned SAH, 32 bins",
                      "l2": "inputs larger than L2 (512 MiB of rays per step)"},
             "e2e": {"value": round(e2e, 2), "unit": "Mrays/s", "h2d_bytes_per_step": N_RAYS * 32,
                     "d2h_bytes_per_step": N_RAYS * 16},
             "gpu_launches": int(launches), "clocks": clk, "extra": extra}

    if rank == 0:
        import oracle
        threads = oracle.hardware_threads()
        flat = flatten_scene(data)
        bpr, per, osc = algorithmic_bytes_per_ray(flat, rays[: 1 << 18], threads)
        achieved = bpr * N_RAYS / (kernel_ms * 1e-3) / 1e9
        peak, src = peaks()
        traffic = traffic_from_profile()
        out["roofline"] = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                           "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": src,
                           "kernel": "kTraceDyn<closest>", "kernel_ms": round(kernel_ms, 4),
                           "bytes_per_ray": round(bpr, 1),
                           "per_ray": {k: round(v, 2) for k, v in per.items()},
                           "note": f"of {src}; per-ray counts from the oracle on 262144 rays"}
        # the same counts as FP32 work: 24 flops per box test, 50 per Moller-Trumbore test
        fpr = 24 * per["boxes"] + 50 * per["tris"]
        fp32_peak = fp32_peak_tflops(torch)
        fp32 = fpr * N_RAYS / (kernel_ms * 1e-3) / 1e12
        out["roofline"]["fp32"] = {"achieved": round(fp32, 2), "peak": round(fp32_peak, 1), "unit": "TFLOP/s",
                                   "frac": round(fp32 / fp32_peak, 4), "flops_per_ray": round(fpr, 1),
                                   "peak_source": "measured here: cuBLAS SGEMM 8192^3, TF32 off"}
        prof = os.path.join(ROOT, "profiles", "trace_closest_raycast.json")
        if os.path.exists(prof):
            with open(prof) as f:
                out["roofline"]["l2_hit_rate_pct"] = json.load(f).get("l2_hit_rate_pct")
        # the scene (72 MiB) is L2-resident: the bound is L2 bandwidth; frac
        # stays the fraction of the measured HBM copy peak
        l2, hbm_read = l2_peak_gbs()
        out["roofline"]["bound"] = "l2"
        out["roofline"]["l2_peak"] = {"value": round(l2, 1), "unit": "GB/s",
                                      "source": "measured here: cr_device_read_bandwidth, 64 MiB x 40 passes"}
        out["roofline"]["l2_frac"] = round(achieved / l2, 4)
        out["roofline"]["hbm_read_gbs_measured_here"] = round(hbm_read, 1)
        if world == 1 and not args.skip_extra:
            out["roofline"]["hbm_resident"] = hbm_raycast_extra(torch, with_oracle=not args.skip_cpu)
        if not args.skip_cpu:
            v, n, dt = cpu_baseline(osc, rays, threads)
            out["cpu_baseline"] = {"value": round(v, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                                   "sample": f"first {n} of the {N_RAYS} rays ({dt:.1f} s wall)",
                                   "cpu": cpu_model()}
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def run_only(args):
    import torch
    torch.cuda.set_device(0)
    import craystal_gb300 as cg
    cg.load().cr_set_device(0)
    if args.only == "path_tracer":
        r = cornell_extra(torch)
    elif args.only == "c1_parity":
        r = c1_parity_extra(torch)
    elif args.only == "wavefront":
        r = wavefront_extra(torch)
    elif args.only == "radiance_cache":
        r = cache_extra(torch, args.cache_res)
    elif args.only == "cache_frames":
        r = cache_frames_extra(torch, args.cache_res)
    elif args.only == "large_scene":
        r = large_scene_extra(torch)
    elif args.only == "radiance_cache_network":
        r = mlp_extra(torch)
    elif args.only == "radiance_cache_scene":
        r = c3_extra(torch)
    elif args.only == "radiance_cache_scene_plain":
        r = c3_plain_extra(torch)
    elif args.only == "radiance_cache_scene_frames":
        r = c3_cached_frames_extra(torch)
    elif args.only == "hbm_raycast":
        r = hbm_raycast_extra(torch, n_rays=args.hbm_rays, with_oracle=not args.skip_cpu)
        l2, hbm_read = l2_peak_gbs()
        r["l2_peak_gbs"], r["hbm_read_gbs"] = round(l2, 1), round(hbm_read, 1)
    else:
        r = batch_extra(torch, args.batch_scenes)
    print(json.dumps({args.only: r}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU baseline leg")
    ap.add_argument("--skip-extra", action="store_true", help="omit the path-tracer figures")
    ap.add_argument("--rays", type=int, default=N_RAYS, help="rays per step (profiling a smaller case)")
    ap.add_argument("--tris", type=int, default=N_TRIS, help="triangles (profiling a smaller case)")
    ap.add_argument("--hbm-rays", type=int, default=1 << 24, help="rays of the HBM-resident ray cast")
    ap.add_argument("--traversal", choices=["one_level", "two_level"], default="one_level",
                    help="traversal step of the headline ray cast (profiling the two-level step)")
    ap.add_argument("--only", choices=["path_tracer", "c1_parity", "hbm_raycast", "wavefront", "radiance_cache", "cache_frames", "batched_scenes",
                                       "large_scene", "radiance_cache_scene", "radiance_cache_scene_plain",
                                       "radiance_cache_scene_frames", "radiance_cache_network"],
                    help="run one secondary workload alone and print its figures (profiling)")
    ap.add_argument("--cache-res", type=int, default=512, help="radiance-cache workload resolution")
    ap.add_argument("--batch-scenes", type=int, default=64, help="scenes in the batched workload")
    args = ap.parse_args()
    globals()["N_RAYS"], globals()["N_TRIS"] = args.rays, args.tris
    if args.warmup < 3:
        args.warmup = 3
    if args.only:
        run_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
