#!/usr/bin/env python
"""Benchmark: renderer::pt on the plain drop-in workload, on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl lmgpu|reference]

Workload (one step = one full render): the displaced-sphere scene of lightmetrica.synthetic
(40 icospheres at subdivision 6 on a 512 x 512-quad ground: 3,801,100 triangles; 50 % diffuse,
30 % GGX glossy, 20 % dielectric; 6 area lights + constant environment), 1920 x 1080, 64 spp,
max path length 10 (max_verts = 11), MIS, pixel sampling, fp32. Synthetic seeded data stands in
for the reference's external scenes.

Metric: Mrays/s = every traced segment (extension + shadow rays) / device time of the render,
timed with CUDA events on the launching stream. `e2e` is the same metric through the public
`lightmetrica` API (renderer.render() + film.buffer(): host parameters in, the film copied back to
host memory every step). The scene (BVH, triangles, shading data: well above the 129 MB L2)
stays resident; L2 is also flushed between timed steps with a 256 MB write.

More legs (rank 0), each a key of the same JSON line:

* raycast -- the plain drop-in workload's probe: 2^24 uniform-sphere rays from one point inside the
  scene, closest hit through lmgpu_accel_intersect_device (CUDA events) and end to end through
  lmgpu_accel_intersect; every hit checked against the fp32 oracle (bit-exact count, exact-t ties)
  and the fp64 oracle timed on 2^21 of the rays as the CPU baseline.
* frame_vs_golden -- the timed 1920x1080 frame, box-filtered 4x4, against the oracle's 4096-spp
  480x270 image of the same camera (tests/golden/spheres480_ref_4k.npz): its relative MSE beside
  what an unbiased render predicts.
* batched -- 256 procedural jobs (lightmetrica.synthetic.batch_jobs: random-triangle scenes of
  1k-200k triangles, 64^2-512^2, 4-64 spp, path length 6-12), rendered job by job with
  renderer::pt and then all at once through the shared wavefront (queue size autotuned on a
  32-job probe). jobs/s = jobs / wall-clock seconds (host overhead included); the images of the
  two forms are compared (same random streams, so the same estimate up to fp32 summation order).
* batched_to_error -- the same 256 jobs at equal relative MSE: each renders until its film's
  reference-free error estimate is at or below --target-rel-mse (1e-3), at most 4096 spp; plain
  job by job (renderer::pt's 'error' scheduler) against the shared wavefront
  (BatchRenderer.render_to_error); the estimate is checked against the true relative MSE of the
  smallest jobs (16k-spp GPU references).
* instanced -- renderer::pt through the two-level accel on lightmetrica.synthetic.instanced_scene:
  64 instances of a 499k-triangle displaced mesh (32M triangles effective, 1.5M stored), a
  1024x512 procedural HDR environment and 16 area lights, 4096x2160, path length 16.
* served_stress (and served_stress_150gb) -- the heavy-tailed mix of the instanced configuration:
  1 request in 10 renders the instanced scene at 4096x2160 (1-4 spp), the rest batched-workload
  scenes, through a RenderServer that builds scenes on admission under a 1.5 GB HBM budget, so
  memory admission, eviction and rebuilds are exercised (bounded to 300 requests); the second
  key runs the same mix under the served configuration's 150 GB budget.
* served -- a Poisson stream of --served-requests requests (300 by default; the configuration
  names 5000, which at the target error would take over 15 minutes) over the same scenes at 80 %
  of the batched capacity at the target error, through RenderServer under a 150 GB HBM budget:
  new images render to the target error (time-to-target is read at the server's error check,
  not extrapolated), 30 % of requests are +16 spp refinements of finished films; p50/p99 of
  time-to-first-image (first complete sample pass), time-to-done and time-to-target.

--impl reference times the CPU restatement of the reference's path (fp64 accel::sahbvh +
renderer::pt with std::mt19937 per thread under OpenMP, all host cores) on a bounded sample of
the same workload: one full-frame render at 1 spp per step. The reference itself cannot be built
here (glm, nlohmann_json, cereal, stb are absent), so the restatement stands in for it.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "lightmetrica-v3_gb300"))

METRIC = "Mrays/s (renderer::pt, all traced segments)"
W_PX, H_PX, SPP, MAX_VERTS = 1920, 1080, 64, 11
SEED_SCENE, SEED_RENDER = 7, 12345
NODE_BYTES, TRI_BYTES = 80, 48


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None

    def __enter__(self):
        try:
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap")
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def build_scene():
    import lightmetrica as lm
    from lightmetrica import synthetic as syn
    lm.init()
    scene, film, info = syn.spheres_scene(seed=SEED_SCENE, w=W_PX, h=H_PX)
    return lm, scene, film, info


def _apply_overrides(args) -> None:
    """--width/--height/--spp shrink the frame for profiling captures (same scene)."""
    global W_PX, H_PX, SPP
    W_PX = args.width or W_PX
    H_PX = args.height or H_PX
    SPP = args.spp or SPP


def cpu_port(scene, spp: int, threads: int = 0):
    """Times the CPU restatement (fp64, reference RNG stream) on one render of `spp`."""
    from oracle import oracle as O
    S = O.from_lm_scene(scene, double=True)
    S.build(nthreads=threads)
    return S


def aggregate_ranks(dist, seconds: float, rays: int, device: str = "cuda") -> tuple[float, int]:
    """Replicas (one job per GPU, no data-path collective): the job's time is the slowest rank's
    and its work the rays of every rank. dist None: one process."""
    if dist is None:
        return seconds, rays
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    n = torch.tensor([rays], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(t.item()), int(n.item())


def replica_seed(rank: int, k: int) -> int:
    """Render seed of step k on a rank: each replica renders its own samples."""
    return SEED_RENDER + k + 100_003 * rank


def golden_check(img) -> dict | None:
    """The rendered 1920x1080 frame box-filtered 4x4 (= the same camera's 480x270 image at 16x the
    spp) against the committed 4096-spp oracle image tests/golden/spheres480_ref_4k.npz: relative
    MSE sum((x - ref)^2) / sum(ref^2), and what an unbiased render predicts from the golden's
    recorded per-sample variance."""
    import numpy as np
    g = os.path.join(ROOT, "tests", "golden", "spheres480_ref_4k")
    if (W_PX, H_PX) != (1920, 1080) or not os.path.exists(g + ".npz") or img is None or img.shape[:2] != (H_PX, W_PX):
        return None
    ref = np.load(g + ".npz")["img"].astype(np.float64)
    meta = json.load(open(g + ".json"))
    low = img.astype(np.float64).reshape(270, 4, 480, 4, 3).mean(axis=(1, 3))
    e = float(np.sum((low - ref) ** 2) / np.sum(ref ** 2))
    spp = SPP * 16
    pred = meta["sum_var"] * (1.0 / spp + 1.0 / meta["spp"]) / meta["sum_img2"]
    return {"rel_mse": e, "predicted_unbiased": pred, "golden": "spheres480_ref_4k (oracle fp64, 4096 spp, 480x270)",
            "filter": "4x4 box: the frame's 480x270 image at 16x its spp"}


def workload_config(info: dict, ws: int) -> dict:
    """The `config` both arms report: the plain drop-in workload one step renders."""
    return {"workload": f"renderer::pt, displaced spheres ({info['triangles']} tris), {W_PX}x{H_PX}, "
                        f"{SPP} spp, max path length {MAX_VERTS - 1}, MIS",
            "triangles": info["triangles"], "spp": SPP, "max_verts": MAX_VERTS,
            "l2": "inputs larger than L2 (scene resident) and a 256 MB L2 flush between steps",
            "parallelism": "replicas" if ws > 1 else "single GPU"}


def run_reference(args) -> None:
    ws, rank, _ = _dist()
    if rank != 0:
        return
    from oracle import oracle as O
    from lightmetrica import synthetic as syn  # data only: the reference arm loads no GPU library
    parts = syn.spheres_parts(seed=SEED_SCENE, w=W_PX, h=H_PX)
    info = parts["info"]
    S = O.from_parts(parts, double=True)
    S.build()
    cores = O.max_threads()
    for _ in range(args.warmup):
        S.render_pt(W_PX, H_PX, 1, MAX_VERTS, seed=SEED_RENDER, rng="mt19937")
    rays = 0
    secs = 0.0
    for k in range(args.steps):
        _, _, r, s = S.render_pt(W_PX, H_PX, 1, MAX_VERTS, seed=SEED_RENDER + k, rng="mt19937")
        rays += r
        secs += s
    v = rays / secs / 1e6
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": workload_config(info, 1),
           "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": cores, "kind": "port",
                            "sample": f"each step renders 1 of the workload's {SPP} samples per pixel: {W_PX}x{H_PX} "
                                      f"at 1 spp ({W_PX * H_PX} paths), {args.steps} steps; Mrays/s counts every "
                                      f"traced segment, as the GPU arm does"},
           "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "build_seconds": S.build_seconds}
    print(json.dumps(out))


def run_gpu(args) -> None:
    import ctypes as C

    ws, rank, local = _dist()
    import lightmetrica as lm_mod
    from lightmetrica import _native as N
    N.check(N.lib().lmgpu_set_device(local))
    dist = None
    if ws > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(local)
        td.init_process_group("nccl")
        dist = td
    lm, scene, film, info = build_scene()
    t0 = time.perf_counter()
    scene.build()
    build_s = time.perf_counter() - t0
    acc = scene.accel().stats()
    # the same triangles through the GPU builder (timed apart; the frame renders on the host tree)
    gpu_acc = lm.load_accel("bench_ploc_accel", "sahbvh", builder="ploc")
    gpu_acc.build_triangles(scene.flattened()["positions"])
    gpu_build = gpu_acc.stats()
    gpu_acc._release()
    L = N.lib()

    def params(spp, seed, instrument=0):
        p = N.PTParams()
        p.spp = spp
        p.max_verts = MAX_VERTS
        p.seed = seed
        p.sampling_mode = 2
        p.primary_mode = 0
        p.instrument = instrument
        p.wave_paths = args.wave
        return p

    # instrumented (untimed) pass: node / triangle visits per ray for the roofline's byte count
    st = N.RenderStats()
    N.check(L.lmgpu_render_pt(scene._h, film._h, C.byref(params(4, 1, 1)), None, C.byref(st)))
    counts = {"ext_nodes": st.ext_nodes, "ext_tris": st.ext_tris, "shadow_nodes": st.shadow_nodes,
              "shadow_tris": st.shadow_tris}

    # L2 flush buffer (256 MB)
    flush = C.c_void_p()
    cudart = _cudart()
    assert cudart.cudaMalloc(C.byref(flush), 256 << 20) == 0

    def flush_l2():
        cudart.cudaMemset(flush, 0, 256 << 20)

    for k in range(args.warmup):
        N.check(L.lmgpu_render_pt(scene._h, film._h, C.byref(params(SPP, SEED_RENDER + 1000 + k)), None, None))
    cudart.cudaDeviceSynchronize()

    tot = {"rays": 0, "ext": 0, "sh": 0, "ms": 0.0, "ext_ms": 0.0, "shade_ms": 0.0, "shadow_ms": 0.0, "gen_ms": 0.0,
           "ext_launches": 0, "sh_launches": 0}
    with ClockSampler(local) as clk:
        if dist:
            dist.barrier()
        for k in range(args.steps):
            flush_l2()
            cudart.cudaDeviceSynchronize()
            s = N.RenderStats()
            N.check(L.lmgpu_render_pt(scene._h, film._h, C.byref(params(SPP, replica_seed(rank, k))), None, C.byref(s)))
            tot["rays"] += s.rays
            tot["ext"] += s.extension_rays
            tot["sh"] += s.shadow_rays
            tot["ms"] += s.elapsed_ms
            tot["ext_ms"] += s.extend_ms
            tot["shade_ms"] += s.shade_ms
            tot["shadow_ms"] += s.shadow_ms
            tot["gen_ms"] += s.generate_ms
            tot["ext_launches"] += s.extend_launches
            tot["sh_launches"] += s.shadow_launches
        cudart.cudaDeviceSynchronize()
        if dist:
            dist.barrier()
    clocks = clk.summary()

    # e2e through the public API: renderer.render() + film.buffer() per step
    r = lm.load_renderer("renderer", "pt", scene=scene, output=film, max_verts=MAX_VERTS, seed=SEED_RENDER,
                         sampling_mode="mis", scheduler="sample", spp=SPP, wave_paths=args.wave)
    e2e_rays, e2e_s = 0, 0.0
    img = film.buffer_f32()
    if not args.skip_e2e:
        r.render()
        film.buffer()
        for k in range(max(1, args.steps)):
            t = time.perf_counter()
            out = r.render()
            img = film.buffer_f32()
            e2e_s += time.perf_counter() - t
            e2e_rays += out["rays"]
    d2h = img.nbytes
    h2d = C.sizeof(N.PTParams)
    frame_check = golden_check(img)

    sec, rays_all = aggregate_ranks(dist, tot["ms"] / 1e3, tot["rays"])
    value = rays_all / sec / 1e6

    # roofline of the dominant kernel
    peaks = _peaks()
    kern = {"extend": tot["ext_ms"], "shade": tot["shade_ms"], "shadow": tot["shadow_ms"], "generate": tot["gen_ms"]}
    dom = max(kern, key=kern.get)
    b_ext = 32 + 16 + NODE_BYTES * counts["ext_nodes"] + TRI_BYTES * counts["ext_tris"]
    b_sh = 48 + NODE_BYTES * counts["shadow_nodes"] + TRI_BYTES * counts["shadow_tris"]
    if dom == "extend":
        bytes_total, launches = tot["ext"] * b_ext, tot["ext_launches"]
    elif dom == "shadow":
        bytes_total, launches = tot["sh"] * b_sh, tot["sh_launches"]
    else:
        # per extension-ray hit: ray+state read 88 B, next ray+state written 88 B, shading record 96 B,
        # shadow ray written 48 B
        bytes_total, launches = tot["ext"] * (88 + 88 + 96 + 48), tot["ext_launches"]
    achieved = bytes_total / (kern[dom] / 1e3) / 1e9
    # L2 read bandwidth (64 MB buffer, below the 129 MB L2): the node arrays of this scene fit in L2
    l2 = C.c_double()
    N.check(L.lmgpu_probe_l2_bandwidth(64 << 20, 20, C.byref(l2)))
    # DRAM traffic per launch of the dominant kernel: bytes per traced ray from an ncu capture of
    # every launch of that kernel in one step (profiles/traffic_per_ray.json) times the rays one
    # launch of this run traces on average
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic_per_ray.json")
    if os.path.exists(tf) and dom in ("extend", "shadow"):
        per_ray = json.load(open(tf)).get(dom)
        if per_ray:
            n_rays, n_launch = (tot["ext"], tot["ext_launches"]) if dom == "extend" else (tot["sh"], tot["sh_launches"])
            traffic = per_ray * n_rays / max(1, n_launch)
    cpu = None
    S = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O
        S = cpu_port(scene, 1)
        _, _, crays, csec = S.render_pt(W_PX, H_PX, 1, MAX_VERTS, seed=SEED_RENDER, rng="mt19937")
        cpu = {"value": crays / csec / 1e6, "unit": "Mrays/s", "cores": O.max_threads(), "kind": "port",
               "sample": f"{W_PX}x{H_PX} at 1 spp ({W_PX * H_PX} paths, {crays} rays, {csec:.1f} s)",
               "build_seconds": S.build_seconds}

    # kernels per step: every chunk of the shared wavefront launches extend, shade, shadow, plan and
    # generate once per bounce iteration; one film resolve per render
    launches_per_step = 5 * tot["ext_launches"] / max(1, args.steps) + 1
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sec / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(info, ws),
            "rays_per_step": tot["rays"] / max(1, args.steps),
            "extension_rays_per_step": tot["ext"] / max(1, args.steps),
            "shadow_rays_per_step": tot["sh"] / max(1, args.steps),
            "kernel_ms_per_step": {k: v / max(1, args.steps) for k, v in kern.items()},
            "e2e": {"value": e2e_rays / e2e_s / 1e6 if e2e_s > 0 else None, "unit": "Mrays/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                         # what limits it: the counters (profiles/k_pt_extend_small.md) show issue slots
                         # busy and node reads served by L2, not DRAM bandwidth
                         "limiter": "instruction issue and latency; nodes and triangles L2-resident" if dom in (
                             "extend", "shadow") else "dependent gathers (latency)",
                         "frac_dram": (traffic * launches / (kern[dom] / 1e3) / 1e9 / peaks["hbm_gbs"]
                                       if traffic else None),
                         "l2_peak_gbs": l2.value, "frac_l2": achieved / l2.value,
                         "traffic": traffic, "bytes_per_ray": {"extend": b_ext, "shadow": b_sh},
                         "launches": launches, **counts},
            "cpu_baseline": cpu,
            "frame_vs_golden": frame_check,
            "gpu_launches": int(launches_per_step * args.steps),
            "clocks": clocks,
            "accel": {"nodes": acc["num_nodes"], "depth": acc["max_depth"], "build_seconds": acc["build_seconds"],
                      "scene_build_seconds": build_s, "sah_cost": acc["sah_cost"], "builder": "host SAH",
                      "gpu_builder": {"build_seconds": gpu_build["build_seconds"], "nodes": gpu_build["num_nodes"],
                                      "depth": gpu_build["max_depth"], "sah_cost": gpu_build["sah_cost"]}},
        }
        if not args.no_batched:
            out["batched"], ctx = run_batched(lm, args)
            if args.target_rel_mse > 0:
                out["batched_to_error"] = run_batched_to_error(lm, args, ctx)
                ctx["capacity_to_error"] = out["batched_to_error"]["batched"]["jobs_per_s"]
            if args.served_requests > 0:
                out["served"] = run_served(lm, args, ctx)
            if args.stress_requests > 0:
                out["served_stress"] = run_served_stress(lm, args, ctx)
                # the same mix at the served configuration's 150 GB budget: nothing is evicted
                out["served_stress_150gb"] = run_served_stress(lm, args, ctx, budget_bytes=150 * 10**9)
        if args.raycast:
            out["raycast"] = run_raycast(lm, scene, args, cpu_scene=S if not args.no_cpu else None)
        if args.lt_paths > 0:
            out["lt"] = run_lt(lm, scene, film, args)
        if args.bdpt_samples > 0:
            out["bdpt"] = run_bdpt(lm, scene, film, args)
        if args.instanced_spp > 0:
            out["instanced"] = run_instanced(lm, args)
        print(json.dumps(out))
    cudart.cudaFree(flush)
    if dist:
        dist.destroy_process_group()


def _batched_scenes(lm, n_jobs: int):
    from lightmetrica import synthetic as syn
    jobs = syn.batch_jobs(n_jobs)
    scenes = []
    t = time.perf_counter()
    accel_s = {"sah": 0.0, "ploc": 0.0}
    for i, j in enumerate(jobs):
        s, f = syn.triangles_scene(j["scene_seed"], j["tris"], j["res"], j["res"], prefix=f"batch{i}_")
        s.build()
        accel_s["sah"] += s.accel().stats()["build_seconds"]
        g = lm.load_accel(f"batch{i}_ploc", "sahbvh", builder="ploc")
        g.build_triangles(s.flattened()["positions"])
        accel_s["ploc"] += g.stats()["build_seconds"]
        g._release()
        scenes.append((s, f))
    _batched_scenes.accel_seconds = accel_s
    return jobs, scenes, time.perf_counter() - t


def run_batched(lm, args) -> tuple[dict, dict]:
    """Plain job-by-job renderer::pt vs the shared wavefront on the batched workload, after the
    autotuner has chosen queue size, launch shape, shade-kernel split and node width on a 32-job
    probe (both forms then run with its choices)."""
    import numpy as np
    from lightmetrica.autotune import tune
    from lightmetrica.serving import BatchRenderer
    jobs, scenes, build_s = _batched_scenes(lm, args.batched_jobs)
    paths = sum(j["res"] ** 2 * j["spp"] for j in jobs)
    s0, f0 = scenes[0]
    lm.load_renderer("batch_warm", "pt", scene=s0, output=f0, max_verts=7, seed=1, spp=2, scheduler="sample").render()
    probe_films = [lm.load_film(f"batch_probe{i}", "bitmap", w=j["res"], h=j["res"]) for i, j in enumerate(jobs[:32])]
    probe = [dict(scene=s, film=f2, max_verts=j["max_verts"], spp=j["spp"], seed=j["seed"])
             for j, (s, _), f2 in zip(jobs, scenes, probe_films)]
    t = time.perf_counter()
    chosen, tune_times = tune(probe, rebuild=lambda: [s.build() for s, _ in scenes[:len(probe)]])
    tune_s = time.perf_counter() - t
    if chosen.get("node_width", 8) != 8:
        for s, _ in scenes[len(probe):]:
            s.build()
    queue = chosen["queue_paths"]
    # plain: one renderer::pt per job, in order
    t = time.perf_counter()
    plain_rays = 0
    for i, (j, (s, f)) in enumerate(zip(jobs, scenes)):
        r = lm.load_renderer(f"batch_r{i}", "pt", scene=s, output=f, max_verts=j["max_verts"], seed=j["seed"],
                             spp=j["spp"], scheduler="sample")
        plain_rays += r.render()["rays"]
    plain_s = time.perf_counter() - t
    plain_imgs = [f.buffer_f32().copy() for _, f in scenes]
    films = [lm.load_film(f"batch_out{i}", "bitmap", w=j["res"], h=j["res"]) for i, j in enumerate(jobs)]
    spec = [dict(scene=s, film=f2, max_verts=j["max_verts"], spp=j["spp"], seed=j["seed"])
            for j, (s, _), f2 in zip(jobs, scenes, films)]
    b = BatchRenderer(queue_paths=queue)
    b.submit(s0, films[0], max_verts=7, spp=1, seed=0)
    b.run(0)
    b.reset()
    t = time.perf_counter()
    b.render(spec)
    batch_s = time.perf_counter() - t
    st = b.stats()
    b.close()
    diff = 0.0
    for f2, a in zip(films, plain_imgs):
        diff = max(diff, float(np.max(np.abs(f2.buffer_f32() - a))) / (float(np.max(np.abs(a))) + 1e-12))
    out = {
        "workload": f"{len(jobs)} random-triangle scenes ({sum(j['tris'] for j in jobs)} triangles in all, 1k-200k "
                    f"log-uniform), 64^2-512^2, spp 4-64, path length 6-12, MIS; {paths} paths",
        "jobs": len(jobs), "paths": paths,
        "plain": {"jobs_per_s": len(jobs) / plain_s, "seconds": plain_s, "Mrays_per_s": plain_rays / plain_s / 1e6},
        "batched": {"jobs_per_s": len(jobs) / batch_s, "seconds": batch_s, "Mrays_per_s": st["rays"] / batch_s / 1e6,
                    "device_ms": st["device_ms"], "queue_paths": queue},
        "speedup": plain_s / batch_s,
        "autotune": {"chosen": chosen, "seconds_per_candidate": {k: {str(c): v for c, v in d.items()}
                                                                 for k, d in tune_times.items()},
                     "tuning_seconds": tune_s, "probe": f"the first {len(probe)} jobs, wall clock per render"},
        "max_rel_image_diff": diff,
        "timing": "wall clock around all jobs (host overhead included); scene builds excluded",
        "scene_build_seconds": build_s,
        "accel_build_seconds": {"host_sah": _batched_scenes.accel_seconds["sah"],
                                "gpu_ploc": _batched_scenes.accel_seconds["ploc"],
                                "note": "all 256 scenes' trees (the timed renders use the host builder's)"},
    }
    return out, {"jobs": jobs, "scenes": scenes, "queue": queue, "capacity": len(jobs) / batch_s,
                 "paths_per_s": paths / batch_s}


def run_batched_to_error(lm, args, ctx) -> dict:
    """The batched workload at equal relative MSE: every job renders until its film's rel-MSE
    estimate (even / odd passes, eps 0.01) is at or below args.target_rel_mse, at most
    args.error_budget_spp samples per pixel. Plain: renderer::pt job by job with the 'error'
    scheduler (a round of 8 spp, then rounds sized from the estimate, each a full render call).
    Batched: BatchRenderer.render_to_error, every job in one shared wavefront (a job that reaches
    its round's count is checked and raised while the others keep the queue full). The estimate
    is checked against the true relative MSE on the smallest jobs, against GPU renders of 16k spp."""
    import numpy as np
    from lightmetrica import _native as N
    from lightmetrica.serving import BatchRenderer
    import ctypes as C
    jobs, scenes = ctx["jobs"], ctx["scenes"]
    target, budget = args.target_rel_mse, args.error_budget_spp
    # plain, job by job
    plain = []
    t = time.perf_counter()
    for i, (j, (s, f)) in enumerate(zip(jobs, scenes)):
        r = lm.load_renderer(f"err_r{i}", "pt", scene=s, output=f, max_verts=j["max_verts"], seed=j["seed"],
                             scheduler="error", target_rel_mse=target, spp=budget)
        out = r.render()
        plain.append({"spp": r.last_spp, "rel_mse": r.last_rel_mse, "rays": out["rays"]})
    plain_s = time.perf_counter() - t
    # batched
    films = [lm.load_film(f"err_out{i}", "bitmap", w=j["res"], h=j["res"]) for i, j in enumerate(jobs)]
    spec = [dict(scene=s, film=f2, max_verts=j["max_verts"], spp=budget, seed=j["seed"])
            for j, (s, _), f2 in zip(jobs, scenes, films)]
    b = BatchRenderer(queue_paths=ctx["queue"])
    t = time.perf_counter()
    res = b.render_to_error(spec, target)
    batch_s = time.perf_counter() - t
    st = b.stats()
    b.close()
    # the estimate against the true relative MSE on the eight smallest jobs (16k-spp GPU reference)
    small = sorted(range(len(jobs)), key=lambda i: (jobs[i]["res"], jobs[i]["tris"]))[:8]
    checks = []
    L = N.lib()
    for i in small:
        j = jobs[i]
        s, _ = scenes[i]
        ref_f = lm.load_film(f"err_ref{i}", "bitmap", w=j["res"], h=j["res"])
        p = N.PTParams()
        p.spp, p.max_verts, p.seed, p.sampling_mode = 16384, j["max_verts"], j["seed"] + 99991, 2
        N.check(L.lmgpu_render_pt(s._h, ref_f._h, C.byref(p), None, None))
        ref = ref_f.buffer_f32().astype(np.float64)
        for form, img, est in (("plain", scenes[i][1].buffer_f32(), plain[i]["rel_mse"]),
                               ("batched", films[i].buffer_f32(), res[i]["rel_mse"])):
            true = float(np.mean((img.astype(np.float64) - ref) ** 2 / (ref * ref + 1e-2)))
            checks.append({"job": i, "form": form, "res": j["res"], "estimate": est, "true_vs_16k": true})
        ref_f._release()
    pe = [p["rel_mse"] for p in plain]
    be = [r["rel_mse"] for r in res]
    return {
        "workload": f"the batched workload's {len(jobs)} jobs, each rendered until its relative-MSE estimate <= "
                    f"{target:g} (at most {budget} spp)",
        "target_rel_mse": target,
        "plain": {"jobs_per_s": len(jobs) / plain_s, "seconds": plain_s,
                  "Mrays_per_s": sum(p["rays"] for p in plain) / plain_s / 1e6,
                  "reached": float(np.mean([e <= target for e in pe])), "rel_mse_mean": float(np.mean(pe)),
                  "spp_p50": float(np.median([p["spp"] for p in plain]))},
        "batched": {"jobs_per_s": len(jobs) / batch_s, "seconds": batch_s, "Mrays_per_s": st["rays"] / batch_s / 1e6,
                    "reached": float(np.mean([e <= target for e in be])), "rel_mse_mean": float(np.mean(be)),
                    "spp_p50": float(np.median([r["spp"] for r in res])),
                    "rounds_mean": float(np.mean([r["rounds"] for r in res])), "queue_paths": ctx["queue"]},
        "speedup": plain_s / batch_s,
        "estimate_vs_true": checks,
        "timing": "wall clock around all jobs (host overhead, error checks and rounds included); scene builds excluded",
    }


def run_served(lm, args, ctx) -> dict:
    """Poisson request stream through RenderServer at 80 % of the measured batched capacity."""
    from lightmetrica import synthetic as syn
    from lightmetrica.serving import RenderServer, Request
    scenes = ctx["scenes"]
    target = args.target_rel_mse if args.target_rel_mse > 0 else None
    rate = 0.8 * (ctx.get("capacity_to_error") if target else ctx["capacity"])
    reqs = syn.served_requests(args.served_requests, rate=rate, n_scenes=len(scenes))
    srv = RenderServer(lambda k: scenes[k][0], hbm_budget=150 * 10**9, queue_paths=args.served_queue, max_inflight=1024)
    srv.owns_scenes = False
    t0 = srv.clock()
    i, n = 0, len(reqs)
    while i < n or not srv.idle():
        now = srv.clock() - t0
        while i < n and reqs[i]["arrival"] <= now:
            q = reqs[i]
            # new images render to the target error (at most error_budget_spp); refinements add
            # 16 spp to a finished film
            new_image = q["refine"] is None and target is not None
            srv.submit(Request(rid=q["rid"], arrival=t0 + q["arrival"], scene_key=q["scene"], w=q["res"], h=q["res"],
                               spp=args.error_budget_spp if new_image else q["spp"], max_verts=q["max_verts"],
                               seed=q["seed"], refine=q["refine"], target=target if new_image else None))
            i += 1
        if srv.idle() and i < n:
            time.sleep(max(0.0, reqs[i]["arrival"] - (srv.clock() - t0)))
            continue
        srv.step()
    total = srv.clock() - t0
    lat = srv.latencies()
    st = srv.batch.stats()
    srv.close()
    return {"queue_paths": args.served_queue,
            "workload": f"{n} requests, Poisson at {rate:.1f}/s (80 % of the batched capacity"
                        f"{' at the target error' if target else ''}), {sum(1 for q in reqs if q['refine'] is not None)} "
                        f"refinements (+16 spp on a finished film), the others new images rendered "
                        + (f"to rel-MSE {target:g} (at most {args.error_budget_spp} spp)" if target else "at 4-64 spp")
                        + ", scenes of the batched workload, 150 GB HBM budget",
            "requests": n, "rate_per_s": rate, "seconds": total, "jobs_per_s": n / total,
            "Mrays_per_s": st["rays"] / total / 1e6,
            "ttfi_p50_s": lat["ttfi_p50"], "ttfi_p99_s": lat["ttfi_p99"],
            "done_p50_s": lat["done_p50"], "done_p99_s": lat["done_p99"], "evictions": lat["evictions"],
            "peak_resident_bytes": srv.peak_resident_bytes,
            **{k: v for k, v in lat.items() if k.startswith(("rel_mse", "target_", "reached_target", "time_to_target"))}}


def run_served_stress(lm, args, ctx, budget_bytes: int | None = None) -> dict:
    """Heavy-tailed served mix: 1 request in 10 renders the instanced scene at 4096x2160 (path
    length 16, 1-4 spp), the rest batched-workload scenes (the first 32 of the mix), under a small
    HBM budget, so admission waits for memory and idle scenes are evicted and rebuilt. Scenes are
    built on admission and released on eviction by the server; films are released when done."""
    import numpy as np
    from lightmetrica import synthetic as syn
    from lightmetrica.serving import RenderServer, Request
    jobs = ctx["jobs"]
    rng = np.random.default_rng(99)
    reqs = []
    for i in range(args.stress_requests):
        if rng.random() < 0.1:
            reqs.append({"key": "inst", "w": 4096, "h": 2160, "spp": int(rng.integers(1, 5)), "max_verts": 17})
        else:
            r = int(rng.choice(syn.BATCH_RESOLUTIONS))
            reqs.append({"key": int(rng.integers(0, 32)), "w": r, "h": r, "spp": int(rng.integers(4, 65)),
                         "max_verts": int(rng.integers(6, 13)) + 1})
        reqs[-1]["seed"] = int(rng.integers(0, 2**31))
    mean_paths = float(np.mean([q["w"] * q["h"] * q["spp"] for q in reqs]))
    rate = 0.8 * ctx["paths_per_s"] / mean_paths
    t = 0.0
    for q in reqs:
        t += rng.exponential(1.0 / rate)
        q["arrival"] = t

    def make_scene(key):
        if key == "inst":
            s, _, _ = syn.instanced_scene(prefix="stress_inst_")
        else:
            j = jobs[key]
            s, _ = syn.triangles_scene(j["scene_seed"], j["tris"], 64, 64, prefix=f"stress{key}_")
        s._accel.builder = args.served_builder  # built on admission: the GPU builder by default
        s.build()
        return s
    budget = (args.stress_budget_mb << 20) if budget_bytes is None else budget_bytes
    srv = RenderServer(make_scene, hbm_budget=budget, queue_paths=args.served_queue, max_inflight=256)
    t0 = srv.clock()
    i, n, released = 0, len(reqs), 0
    while i < n or not srv.idle():
        now = srv.clock() - t0
        while i < n and reqs[i]["arrival"] <= now:
            q = reqs[i]
            srv.submit(Request(rid=i, arrival=t0 + q["arrival"], scene_key=q["key"], w=q["w"], h=q["h"], spp=q["spp"],
                               max_verts=q["max_verts"], seed=q["seed"]))
            i += 1
        if srv.idle() and i < n:
            time.sleep(max(0.0, reqs[i]["arrival"] - (srv.clock() - t0)))
            continue
        srv.step()
        for r in srv.finished[released:]:
            srv.release(r.rid)
        released = len(srv.finished)
    total = srv.clock() - t0
    lat = srv.latencies()
    inst = [r for r in srv.finished if r.scene_key == "inst"]
    small = [r for r in srv.finished if r.scene_key != "inst"]
    pct = lambda xs, p: float(np.percentile(xs, p)) if xs else None  # noqa: E731
    st = srv.batch.stats()
    srv.close()
    return {"queue_paths": args.served_queue,
            "workload": f"{n} requests, Poisson at {rate:.1f}/s (80 % of the measured path throughput for this mix), "
                        f"{len(inst)} instanced 4096x2160 jobs (1-4 spp, length 16) among batched-workload jobs on 32 "
                        f"scenes; {budget >> 20} MB HBM budget; scenes built on admission "
                        f"({'GPU PLOC' if args.served_builder == 'ploc' else 'host SAH'} builder)",
            "requests": n, "seconds": total, "jobs_per_s": n / total, "Mrays_per_s": st["rays"] / total / 1e6,
            "ttfi_p50_s": lat["ttfi_p50"], "ttfi_p99_s": lat["ttfi_p99"], "done_p50_s": lat["done_p50"],
            "done_p99_s": lat["done_p99"],
            "instanced_done_p50_s": pct([r.done - r.arrival for r in inst], 50),
            "small_done_p99_s": pct([r.done - r.arrival for r in small], 99),
            "evictions": srv.evictions, "scene_builds": srv.scene_builds,
            "scene_build_seconds": srv.scene_build_seconds, "peak_resident_bytes": srv.peak_resident_bytes,
            "budget_bytes": budget,
            **{k: v for k, v in lat.items() if k.startswith("rel_mse")}}


def run_instanced(lm, args) -> dict:
    """renderer::pt on the instanced stress scene (two-level accel), one frame per step."""
    import ctypes as C
    import numpy as np
    from lightmetrica import _native as N
    from lightmetrica import synthetic as syn
    scene, film, info = syn.instanced_scene(prefix="c5_")
    t = time.perf_counter()
    scene.build()
    build_s = time.perf_counter() - t
    acc = scene.accel().stats()
    sb = C.c_int64()
    N.check(N.lib().lmgpu_scene_device_bytes(scene._h, C.byref(sb)))
    L = N.lib()

    def params(spp, seed):
        p = N.PTParams()
        p.spp, p.max_verts, p.seed, p.sampling_mode, p.primary_mode = spp, 17, seed, 2, 0
        return p
    N.check(L.lmgpu_render_pt(scene._h, film._h, C.byref(params(1, 1)), None, None))
    best = None
    for k in range(2):
        st = N.RenderStats()
        N.check(L.lmgpu_render_pt(scene._h, film._h, C.byref(params(args.instanced_spp, 100 + k)), None, C.byref(st)))
        if best is None or st.elapsed_ms < best.elapsed_ms:
            best = st
    stored = int(np.sum(np.diff(scene.flattened()["blas_offsets"]))) if "blas_offsets" in scene.flattened() else info["triangles"]
    # a flattened build stores every instanced triangle (48 B in the tree + 96 B of shading data) and
    # about as many nodes per triangle as the BLAS have
    flat_est = info["triangles"] * (TRI_BYTES + 96) + info["triangles"] * acc["num_nodes"] / max(1, stored) * NODE_BYTES
    return {"workload": f"{info['instances']} instances of a {info['mesh_triangles']}-triangle displaced mesh "
                        f"({info['triangles']} triangles effective, {stored} stored), 1024x512 env + 16 area lights, "
                        f"4096x2160, {args.instanced_spp} spp, path length 16, MIS",
            "Mrays_per_s": best.rays / best.elapsed_ms / 1e3, "ms_per_frame": best.elapsed_ms, "rays": best.rays,
            "instances": acc["num_instances"], "accel_device_bytes": acc["device_bytes"],
            "scene_device_bytes": int(sb.value), "flattened_bytes_estimate": int(flat_est),
            "build_seconds": build_s}


def run_raycast(lm, scene, args, cpu_scene=None) -> dict:
    """The raycast probe of the plain drop-in workload: 2^24 uniform-sphere rays from one point
    inside the displaced-sphere scene, closest hit through lmgpu_accel_intersect_device (the batched
    Accel::intersect), device buffers, CUDA events on the launching stream; `e2e` through
    lmgpu_accel_intersect (host rays in, host hits out) from pinned host memory, with the pageable
    figure beside it. Every hit of one pass is then checked
    against the fp32 oracle (bit-exact index, t, u, v; exact-t ties counted), and the fp64 oracle
    (the reference's precision) is timed on a bounded subsample as the CPU baseline."""
    import ctypes as C
    import numpy as np
    from lightmetrica import _native as N
    from lightmetrica import synthetic as syn
    L = N.lib()
    rt = _cudart()
    acc = scene.accel()
    rays = syn.sphere_rays(syn.RAYCAST_PROBE_RAYS, syn.RAYCAST_PROBE_ORIGIN, seed=syn.RAYCAST_PROBE_SEED)
    n = len(rays)
    d_rays, d_hits = C.c_void_p(), C.c_void_p()
    assert rt.cudaMalloc(C.byref(d_rays), rays.nbytes) == 0
    assert rt.cudaMalloc(C.byref(d_hits), n * 16) == 0
    flush = C.c_void_p()
    assert rt.cudaMalloc(C.byref(flush), 256 << 20) == 0
    try:
        assert rt.cudaMemcpy(d_rays, rays.ctypes.data, rays.nbytes, 1) == 0
        mn, mt = C.c_double(), C.c_double()
        N.check(L.lmgpu_accel_trace_counts(acc._h, d_rays, n, 0, 64, C.byref(mn), C.byref(mt)))
        e0, e1 = C.c_void_p(), C.c_void_p()
        rt.cudaEventCreate(C.byref(e0))
        rt.cudaEventCreate(C.byref(e1))
        for _ in range(max(3, args.warmup)):
            N.check(L.lmgpu_accel_intersect_device(acc._h, d_rays, n, d_hits, None))
        rt.cudaDeviceSynchronize()
        times = []
        for _ in range(max(1, args.steps)):
            rt.cudaMemset(flush, 0, 256 << 20)
            rt.cudaDeviceSynchronize()
            rt.cudaEventRecord(e0, None)
            N.check(L.lmgpu_accel_intersect_device(acc._h, d_rays, n, d_hits, None))
            rt.cudaEventRecord(e1, None)
            rt.cudaEventSynchronize(e1)
            ms = C.c_float()
            rt.cudaEventElapsedTime(C.byref(ms), e0, e1)
            times.append(ms.value)
        rt.cudaEventDestroy(e0)
        rt.cudaEventDestroy(e1)
        hits = np.zeros(n, dtype=[("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<i4")])
        assert rt.cudaMemcpy(hits.ctypes.data, d_hits, n * 16, 2) == 0
    finally:
        rt.cudaFree(d_rays)
        rt.cudaFree(d_hits)
        rt.cudaFree(flush)
    # end to end: host rays in, host hits out, through the C-ABI (Accel::intersect over host
    # buffers): from pinned host memory, as a caller streaming rays would hold them, and, for
    # comparison, from ordinary (pageable) numpy arrays
    e2e, e2e_pageable = [], []
    h_rays, h_hits = C.c_void_p(), C.c_void_p()
    assert rt.cudaMallocHost(C.byref(h_rays), rays.nbytes) == 0
    assert rt.cudaMallocHost(C.byref(h_hits), n * 16) == 0
    try:
        C.memmove(h_rays, rays.ctypes.data, rays.nbytes)
        N.check(L.lmgpu_accel_intersect(acc._h, C.cast(h_rays, C.POINTER(C.c_float)), n, C.cast(h_hits, C.POINTER(N.Hit))))
        for _ in range(max(1, min(3, args.steps))):
            t = time.perf_counter()
            N.check(L.lmgpu_accel_intersect(acc._h, C.cast(h_rays, C.POINTER(C.c_float)), n, C.cast(h_hits, C.POINTER(N.Hit))))
            e2e.append(time.perf_counter() - t)
        hits_pinned = np.frombuffer((C.c_char * (n * 16)).from_address(h_hits.value), dtype=hits.dtype).copy()
        assert np.array_equal(hits_pinned, hits), "hits through host buffers differ from the device-buffer pass"
    finally:
        rt.cudaFreeHost(h_rays)
        rt.cudaFreeHost(h_hits)
    for _ in range(max(1, min(3, args.steps))):
        t = time.perf_counter()
        acc.intersect_batch(rays)
        e2e_pageable.append(time.perf_counter() - t)
    ms = statistics.median(times)
    b_ray = 32 + 16 + NODE_BYTES * mn.value + TRI_BYTES * mt.value
    peaks = _peaks()
    achieved = n * b_ray / (ms / 1e3) / 1e9
    out = {"workload": f"{n} uniform-sphere rays from {list(syn.RAYCAST_PROBE_ORIGIN)} in the displaced-sphere scene "
                       f"({acc.stats()['num_tris']} triangles), closest hit, tmin 1e-3, tmax 1e10",
           "Mrays_per_s": n / ms / 1e3, "ms_median": ms, "ms_all": times,
           "e2e": {"value": n / statistics.median(e2e) / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": rays.nbytes,
                   "d2h_bytes_per_step": n * 16, "host_memory": "pinned",
                   "pageable_value": n / statistics.median(e2e_pageable) / 1e6},
           "hit_fraction": float((hits["prim"] >= 0).mean()),
           "roofline": {"bound": "issue/latency (L2-resident nodes)", "achieved": achieved, "unit": "GB/s",
                        "peak": peaks["hbm_gbs"], "frac": achieved / peaks["hbm_gbs"], "bytes_per_ray": b_ray,
                        "nodes_per_ray": mn.value, "tris_per_ray": mt.value}}
    if cpu_scene is not None:
        from oracle import oracle as O
        # checker: every GPU hit against the fp32 restatement (not timed)
        S32 = O.from_lm_scene(scene, double=False)
        S32.build(robust=True)
        t32, uv32, id32, _ = S32.intersect(rays, refine_t=True)
        tri32 = S32.triangles()
        del S32
        g = hits["prim"].astype(np.int64)
        same = g == id32
        hit = same & (g >= 0)
        exact = same & (~hit | ((hits["t"] == t32.astype(np.float32)) & (hits["u"] == uv32[:, 0].astype(np.float32))
                                & (hits["v"] == uv32[:, 1].astype(np.float32))))
        cand = np.nonzero(~same & (g >= 0) & (id32 >= 0))[0]
        ties = 0
        if len(cand):
            ties = int(np.sum(O.mt32(rays[cand], tri32, g[cand]) == O.mt32(rays[cand], tri32, id32[cand])))
        out["check_fp32_oracle"] = {"rays": n, "bit_exact": int(exact.sum()), "exact_t_ties": ties,
                                    "mismatches": int(n - exact.sum() - ties)}
        # CPU baseline: the fp64 restatement of accel_sahbvh.cpp on a bounded subsample
        sub = rays[: 1 << 21]
        _, _, _, csec = cpu_scene.intersect(sub)
        out["cpu_baseline"] = {"value": len(sub) / csec / 1e6, "unit": "Mrays/s", "cores": O.max_threads(),
                               "kind": "port", "sample": f"first {len(sub)} of the probe's rays, fp64 accel::sahbvh "
                                                         f"restatement ({csec:.2f} s)"}
    return out


def run_lt(lm, scene, film, args) -> dict:
    """renderer::lt on the headline scene (already built): args.lt_paths light paths per frame,
    device-timed with CUDA events; end to end through RendererLT.render() + film.buffer(); and the
    oracle's light tracer (fp64, the reference's std::mt19937 stream) on a bounded sample."""
    import ctypes as C
    from lightmetrica import _native as N
    L = N.lib()

    def frame(seed):
        p = N.LTParams()
        p.num_samples, p.first_path, p.max_verts, p.seed = args.lt_paths, 0, MAX_VERTS, seed
        st = N.RenderStats()
        N.check(L.lmgpu_render_lt(scene._h, film._h, C.byref(p), None, C.byref(st)))
        return st
    frame(1)
    runs = [frame(200 + k) for k in range(3)]
    ms = sorted(r.elapsed_ms for r in runs)
    rays = sum(r.rays for r in runs)
    value = rays / sum(r.elapsed_ms for r in runs) / 1e3
    r = lm.load_renderer("lt_bench", "lt", scene=scene, output=film, max_verts=MAX_VERTS, seed=7, scheduler="sample",
                         num_samples=args.lt_paths)
    r.render()
    e2e_rays, e2e_s = 0, 0.0
    for _ in range(3):
        t = time.perf_counter()
        out = r.render()
        film.buffer_f32()
        e2e_s += time.perf_counter() - t
        e2e_rays += out["rays"]
    res = {"workload": f"renderer::lt on the headline scene ({W_PX}x{H_PX} film), {args.lt_paths} light paths per frame, "
                       f"max path length {MAX_VERTS - 1}",
           "Mrays_per_s": value, "ms_per_frame_median": ms[1], "rays_per_frame": rays / len(runs),
           "extension_rays_per_frame": sum(r.extension_rays for r in runs) / len(runs),
           "camera_connections_per_frame": sum(r.shadow_rays for r in runs) / len(runs),
           "kernel_ms_per_frame": {"extend": sum(r.extend_ms for r in runs) / len(runs),
                                   "shade": sum(r.shade_ms for r in runs) / len(runs),
                                   "shadow": sum(r.shadow_ms for r in runs) / len(runs),
                                   "generate": sum(r.generate_ms for r in runs) / len(runs)},
           "e2e_Mrays_per_s": e2e_rays / e2e_s / 1e6}
    if not args.no_cpu:
        from oracle import oracle as O
        S = cpu_port(scene, 1)
        n = 1 << 21
        _, crays, csec = S.render_lt(W_PX, H_PX, n, MAX_VERTS, seed=7, rng="mt19937")
        res["cpu_baseline"] = {"value": crays / csec / 1e6, "unit": "Mrays/s", "cores": O.max_threads(), "kind": "port",
                               "sample": f"{n} light paths ({crays} rays, {csec:.1f} s)"}
    return res


def run_bdpt(lm, scene, film, args) -> dict:
    """renderer::bdpt on the headline scene (already built): args.bdpt_samples samples per frame
    (one eye and one light subpath each), device-timed with CUDA events; end to end through
    RendererBDPT.render() + film.buffer(); and the oracle's BDPT (fp64, the reference's
    std::mt19937 stream) on a bounded sample."""
    import ctypes as C
    from lightmetrica import _native as N
    L = N.lib()

    def frame(seed):
        p = N.BDPTParams()
        p.num_samples, p.first_path, p.min_verts, p.max_verts, p.seed = args.bdpt_samples, 0, 2, MAX_VERTS, seed
        st = N.RenderStats()
        N.check(L.lmgpu_render_bdpt(scene._h, film._h, C.byref(p), None, C.byref(st)))
        return st
    frame(1)
    runs = [frame(300 + k) for k in range(3)]
    ms = sorted(r.elapsed_ms for r in runs)
    rays = sum(r.rays for r in runs)
    r = lm.load_renderer("bdpt_bench", "bdpt", scene=scene, output=film, max_verts=MAX_VERTS, seed=7, scheduler="sample",
                         num_samples=args.bdpt_samples)
    r.render()
    e2e_rays, e2e_s = 0, 0.0
    for _ in range(3):
        t = time.perf_counter()
        out = r.render()
        film.buffer_f32()
        e2e_s += time.perf_counter() - t
        e2e_rays += out["rays"]
    res = {"workload": f"renderer::bdpt on the headline scene ({W_PX}x{H_PX} film), {args.bdpt_samples} samples per frame, "
                       f"subpaths of up to {MAX_VERTS} vertices, every strategy with s + t <= {MAX_VERTS}",
           "Mrays_per_s": rays / sum(r.elapsed_ms for r in runs) / 1e3, "ms_per_frame_median": ms[1],
           "samples_per_s": args.bdpt_samples / (ms[1] / 1e3),
           "rays_per_frame": rays / len(runs),
           "subpath_rays_per_frame": sum(r.extension_rays for r in runs) / len(runs),
           "connection_rays_per_frame": sum(r.shadow_rays for r in runs) / len(runs),
           "kernel_ms_per_frame": {"extend": sum(r.extend_ms for r in runs) / len(runs),
                                   "shade_and_connect": sum(r.shade_ms for r in runs) / len(runs),
                                   "shadow": sum(r.shadow_ms for r in runs) / len(runs),
                                   "generate": sum(r.generate_ms for r in runs) / len(runs)},
           "e2e_Mrays_per_s": e2e_rays / e2e_s / 1e6}
    if not args.no_cpu:
        from oracle import oracle as O
        S = cpu_port(scene, 1)
        n = 1 << 17
        _, crays, csec = S.render_bdpt(W_PX, H_PX, n, MAX_VERTS, seed=7, rng="mt19937")
        res["cpu_baseline"] = {"value": crays / csec / 1e6, "unit": "Mrays/s", "cores": O.max_threads(), "kind": "port",
                               "samples_per_s": n / csec, "sample": f"{n} samples ({crays} rays, {csec:.1f} s)"}
    return res


def _cudart():
    import ctypes as C
    import glob
    cands = ["libcudart.so", "libcudart.so.13"] + sorted(glob.glob("/usr/local/cuda*/lib64/libcudart.so*"))
    for c in cands:
        try:
            lib = C.CDLL(c)
            lib.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
            lib.cudaMemset.argtypes = [C.c_void_p, C.c_int, C.c_size_t]
            lib.cudaFree.argtypes = [C.c_void_p]
            lib.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
            lib.cudaEventCreate.argtypes = [C.POINTER(C.c_void_p)]
            lib.cudaEventRecord.argtypes = [C.c_void_p, C.c_void_p]
            lib.cudaEventSynchronize.argtypes = [C.c_void_p]
            lib.cudaEventDestroy.argtypes = [C.c_void_p]
            lib.cudaEventElapsedTime.argtypes = [C.POINTER(C.c_float), C.c_void_p, C.c_void_p]
            lib.cudaMallocHost.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
            lib.cudaFreeHost.argtypes = [C.c_void_p]
            return lib
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="lmgpu", choices=["lmgpu", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--skip-e2e", action="store_true", help="skip the end-to-end API pass (profiling runs)")
    ap.add_argument("--width", type=int, default=0)
    ap.add_argument("--height", type=int, default=0)
    ap.add_argument("--spp", type=int, default=0)
    ap.add_argument("--wave", type=int, default=0, help="paths in flight per wave (0 = library default)")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched and served legs")
    ap.add_argument("--raycast", type=int, default=1, help="1: the 2^24-ray raycast probe leg (0 skips it)")
    ap.add_argument("--target-rel-mse", type=float, default=1e-3,
                    help="relative MSE the batched_to_error and served legs render to (0 skips batched_to_error)")
    ap.add_argument("--error-budget-spp", type=int, default=4096, help="most spp a job may take to reach the target")
    ap.add_argument("--served-builder", default="ploc", choices=["sah", "ploc"],
                    help="BVH builder of the scenes the served_stress legs build on admission")
    ap.add_argument("--batched-jobs", type=int, default=256)
    ap.add_argument("--served-requests", type=int, default=300,
                    help="requests of the served leg (0 skips it); new images render to the target error")
    ap.add_argument("--instanced-spp", type=int, default=4, help="spp of the instanced leg (0 skips it)")
    ap.add_argument("--stress-requests", type=int, default=300, help="requests of the served stress leg (0 skips it)")
    ap.add_argument("--served-queue", type=int, default=1 << 22,
                    help="paths in flight of the served legs (smaller than the batched optimum: less queueing delay)")
    ap.add_argument("--stress-budget-mb", type=int, default=1536)
    ap.add_argument("--lt-paths", type=int, default=1 << 24, help="light paths per frame of the renderer::lt leg (0 skips it)")
    ap.add_argument("--bdpt-samples", type=int, default=1 << 22, help="samples per frame of the renderer::bdpt leg (0 skips it)")
    args = ap.parse_args()
    _apply_overrides(args)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
