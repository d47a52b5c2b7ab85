"""Benchmark: plain `path` tracer on the many-spheres stress scene.

Workload: 10,000 icospheres (subdivision 2, 3.2 M triangles) with lognormal
radii, 40/30/20/10 diffuse / rough_metal / rough_glass / disney, constant sky
plus 20 sphere emitters; 1920x1080, max depth 16, Russian roulette from 3.
One step = one sample per pixel over the whole frame (2,073,600 samples).

Reported:
* value  -- samples/s with the scene resident in HBM, device-timed with CUDA
  events on the library's stream over K steps (one job of K samples/pixel);
* e2e    -- the same metric through the public C ABI with host buffers: each
  step submits a 1-spp job, waits, and copies the film to pinned host memory;
* roofline -- the dominant kernel (BVH8 closest-hit traversal, `extend`):
  algorithmic bytes per launch (queue entry + ray + hit record + 80 B per node
  visited + 48 B per primitive tested) / its average launch time, against the
  measured HBM copy bandwidth;
* cpu_baseline -- the CPU oracle (C++ restatement of the reference's path
  loop with a SAH BVH) on this host's cores, on a bounded row sample.

`--impl reference` times that CPU implementation alone on the same workload
(the reference itself needs Embree/oneTBB/Eigen, which are not available).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H = 1920, 1080
MAX_DEPTH = 16
# DRAM bytes (read + written) per closest-hit ray of KExtend on this scene, from one ncu capture of the 16
# launches of one timed wave of this bench (16 samples of the 1080p frame, tuned launch parameters): 31.85 GB
# for 110.9 M closest-hit rays (290.0 B with 4-sample waves). The algorithmic bytes per ray are ~7x larger:
# L1/L2 serve the rest.
EXTEND_DRAM_BYTES_PER_RAY = 287.3
# Issue-side counters of a bounce-1 launch (ncu --set full, 1080p frame, 1-sample waves): the kernel's limiter.
EXTEND_ISSUE = {"lanes_active_per_warp_inst": 16.51, "issue_active_pct": 76.8, "alu_pipe_pct": 65.6,
                "fma_pipe_pct": 30.5}
BYTES_QUEUE, BYTES_RAY, BYTES_HIT, BYTES_NODE, BYTES_PRIM = 4, 32, 32, 80, 48


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def make_scene(tmp, n_spheres=10000, width=W, height=H, seed=2):
    from radiantiumplusplus_gb300 import scenes
    sc, assets = scenes.many_spheres(n_spheres=n_spheres, width=width, height=height, spp=1, max_depth=MAX_DEPTH,
                                     seed=seed)
    return scenes.write_scene(tmp, sc, assets)


def cpu_baseline(scene_path, row_step=8, min_s=10.0):
    """Times the CPU oracle with all host threads on successive 1-spp passes over rows [0, H) step `row_step`
    (sample 0, 1, ...) until at least `min_s` seconds of work are timed."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    o = oracle_lib.OracleScene.from_file(scene_path)
    threads = os.cpu_count() or 1
    n, rays, dt, passes = 0, 0, 0.0, 0
    while dt < min_s and passes < 256:
        t0 = time.perf_counter()
        _, stats = o.render(rows=(0, o.height, row_step), samples=(passes, passes + 1), threads=threads)
        dt += time.perf_counter() - t0
        n += int(stats[2])
        rays += int(stats[0] + stats[1])
        passes += 1
    o.close()
    return {"value": n / dt, "unit": "samples/s", "cores": threads, "kind": "port",
            "sample": "%d one-sample passes over rows 0..%d step %d of the %dx%d many-spheres frame (%d samples, "
                      "%.1f s)" % (passes, o.height, row_step, o.width, o.height, n, dt),
            "mrays_per_s": rays / dt / 1e6}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(world, v):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, world, rank):
    if rank != 0:
        return
    with tempfile.TemporaryDirectory(prefix="rad_bench_") as tmp:
        path = make_scene(tmp)
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_lib
        o = oracle_lib.OracleScene.from_file(path)
        threads = os.cpu_count() or 1
        # the same sample as the GPU arm's cpu_baseline: one-sample passes over every 4th row
        row_step = args.cpu_row_step
        for _ in range(args.warmup):
            o.render(rows=(0, H, row_step * 4), samples=(0, 1), threads=threads)
        n_tot, t_tot = 0, 0.0
        for k in range(args.steps):
            t0 = time.perf_counter()
            _, st = o.render(rows=(k % row_step, H, row_step), samples=(k // row_step, k // row_step + 1),
                             threads=threads)
            t_tot += time.perf_counter() - t0
            n_tot += int(st[2])
        value = n_tot / t_tot
        line = {"impl": "reference", "metric": "samples/s (path, many-spheres 1920x1080, depth 16)", "value": value,
                "unit": "samples/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000 * t_tot / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
                "config": {"workload": "many_spheres_1080p", "spheres": 10000, "triangles": 3200000, "emitters": 20,
                           "width": W, "height": H, "max_depth": MAX_DEPTH, "rr_depth": 3,
                           "sample_per_step": "1/%d of the rows, one sample" % row_step},
                "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads, "kind": "port",
                                 "sample": "per step a one-sample pass over every %d-th row of the frame (%d samples, "
                                           "%.1f s over %d steps)" % (row_step, n_tot, t_tot, args.steps)},
                "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import numpy as np
    import torch
    import radiantiumplusplus_gb300 as rad

    torch.cuda.set_device(local)
    rad.init({"device": local, "max_paths": args.max_paths})
    hbm_peak, peak_src = _peaks()
    with tempfile.TemporaryDirectory(prefix="rad_bench_") as tmp:
        path = make_scene(tmp, seed=2)
        t0 = time.perf_counter()
        scene = rad.Scene.from_file(path)
        load_s = time.perf_counter() - t0
        spp_step = args.spp_per_step
        # launch parameters of the traversal kernels for this scene (rad_autotune, not timed)
        tune = scene.autotune() if not args.no_tune else {"refill_busy": 20, "blocks_per_sm": 8, "leaf_frac8": 4,
                                                             "shade_block": 128,
                                                             "best_ms": 0.0, "default_ms": 0.0}
        # traversal statistics for the roofline's algorithmic bytes (not timed)
        j = scene.submit(spp=1, first_sample=10_000, count_traversal=True)
        j.wait()
        cs = j.stats()
        j.close()
        nodes_per_ray = cs["trav_nodes_closest"] / max(1, cs["rays_closest"])
        prims_per_ray = cs["trav_prims_closest"] / max(1, cs["rays_closest"])
        # warm-up
        # warm-up: at least 8 samples, so that its waves hold as many samples as the timed job's
        # (their CUDA graphs are captured here, outside the timed region)
        j = scene.submit(spp=max(8, args.warmup) * spp_step, first_sample=20_000)
        j.wait()
        j.close()
        # ---- device-timed value: one job of K samples per pixel, events on the library stream
        clocks = ClockSampler(local)
        barrier(world)
        torch.cuda.synchronize()
        clocks.start()
        job = scene.submit(spp=args.steps * spp_step, first_sample=0)
        job.wait()
        torch.cuda.synchronize()
        barrier(world)
        st = job.stats()
        job.close()
        # per-kernel breakdown (events around every launch, so no graph replay): one more step, not timed
        pj = scene.submit(spp=max(2, spp_step), first_sample=40_000, profile=True)
        pj.wait()
        pst = pj.stats()
        pj.close()
        gpu_s = allreduce_max(world, st["gpu_ms"] / 1000.0)
        samples = st["samples"] * world
        value = samples / gpu_s
        mrays = (st["rays_closest"] + st["rays_shadow"]) * world / gpu_s / 1e6
        # ---- e2e through the C ABI with host buffers: per step submit a job of the step's samples, wait,
        # film -> pinned host
        pinned = torch.empty((H, W, 3), dtype=torch.float32, pin_memory=True)
        host_film = pinned.numpy()
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.steps):
            jj = scene.submit(spp=spp_step, first_sample=30_000 + k)
            jj.wait()
            jj.film(out=host_film)
            jj.close()
        torch.cuda.synchronize()
        e2e_s = allreduce_max(world, time.perf_counter() - t0)
        barrier(world)
        clk = clocks.stop()  # sampled through both timed regions (and the profiled step between them)
        e2e_value = args.steps * W * H * spp_step * world / e2e_s
        # ---- roofline for the dominant kernel
        kern = {"extend": pst["ms_extend"], "shade": pst["ms_shade"], "shadow": pst["ms_shadow"],
                "generate": pst["ms_generate"], "accumulate": pst["ms_accumulate"]}
        dominant = max(kern, key=kern.get)
        n_ext = max(1, pst["n_extend"])
        ext_bytes = pst["rays_closest"] * (BYTES_QUEUE + BYTES_RAY + BYTES_HIT + nodes_per_ray * BYTES_NODE
                                           + prims_per_ray * BYTES_PRIM)
        ext_launch_ms = pst["ms_extend"] / n_ext
        achieved = (ext_bytes / n_ext) / (ext_launch_ms / 1000.0) / 1e9 if ext_launch_ms > 0 else 0.0
        traffic = EXTEND_DRAM_BYTES_PER_RAY * pst["rays_closest"] / n_ext
        dram_gbs = traffic / (ext_launch_ms / 1000.0) / 1e9 if ext_launch_ms > 0 else 0.0
        cpu = None
        if rank == 0 and world == 1 and not args.no_cpu:
            cpu = cpu_baseline(path, row_step=args.cpu_row_step)
        scene.close()
    line = {
        "metric": "samples/s (path, many-spheres 1920x1080, depth 16)",
        "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * gpu_s / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": "many_spheres_1080p", "spheres": 10000, "triangles": 3200000, "emitters": 20,
                   "width": W, "height": H, "spp_per_step": spp_step, "max_depth": MAX_DEPTH, "rr_depth": 3,
                   "parallelism": "replicas" if world > 1 else "single_gpu",
                   "l2": "inputs larger than L2: resident scene + path state > 129 MB",
                   "max_paths": args.max_paths,
                   "scene_load_s": round(load_s, 3),
                   "autotune": {"refill_busy": tune["refill_busy"], "blocks_per_sm": tune["blocks_per_sm"],
                                "shade_block": tune["shade_block"],
                                "leaf_frac8": tune["leaf_frac8"],
                                "wave_ms_tuned": round(tune["best_ms"], 3),
                                "wave_ms_default": round(tune["default_ms"], 3)}},
        "mrays_per_s": mrays,
        "rays_per_sample": (st["rays_closest"] + st["rays_shadow"]) / max(1, st["samples"]),
        "gpu_launches": st["kernel_launches"],
        "kernel_ms_profiled_step": {k: round(v, 3) for k, v in kern.items()},
        "roofline": {"bound": "hbm", "kernel": "extend (BVH8 closest hit)", "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum over the 16 launches of "
                                       "one timed wave (287.3 B per closest-hit ray) x closest-hit rays per launch",
                     "achieved_is": "algorithmic bytes (nodes, primitives, ray, hit) per launch / launch time; "
                                    "mostly served by L1/L2",
                     "dram_gbs": dram_gbs, "dram_frac": dram_gbs / hbm_peak,
                     "limiter": "instruction issue (ALU pipe), not HBM: see issue",
                     "issue": dict(EXTEND_ISSUE, simt_efficiency=EXTEND_ISSUE["lanes_active_per_warp_inst"] / 32.0,
                                   source="ncu --set full, bounce-1 launch, 1080p frame of this scene"),
                     "peak_source": peak_src, "dominant_kernel_by_time": dominant,
                     "nodes_per_ray": nodes_per_ray, "prims_per_ray": prims_per_ray,
                     "bytes_per_ray": BYTES_QUEUE + BYTES_RAY + BYTES_HIT + nodes_per_ray * BYTES_NODE
                     + prims_per_ray * BYTES_PRIM},
        "e2e": {"value": e2e_value, "unit": "samples/s", "h2d_bytes_per_step": 16,
                "d2h_bytes_per_step": W * H * 3 * 4},
        "clocks": clk,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_volume(args, world, rank, local):
    """Volumetric scene (vol_path): fBm density grid in a rough-dielectric box, 1024x1024, depth 32."""
    import torch
    import radiantiumplusplus_gb300 as rad
    from radiantiumplusplus_gb300 import scenes
    torch.cuda.set_device(local)
    # waves of max_paths paths (samples of whole pixel rows): up to 16 samples of the 1024^2 frame per wave
    rad.init({"device": local, "max_paths": args.vol_max_paths})
    res = args.vol_res
    with tempfile.TemporaryDirectory(prefix="rad_bench_vol_") as tmp:
        sc, assets = scenes.volume_box(width=res, height=res, spp=1, max_depth=32, grid=args.vol_grid)
        path = scenes.write_scene(tmp, sc, assets)
        scene = rad.Scene.from_file(path)
        # lane top-up threshold and blocks per SM of the wavefront's part kernels (rad_autotune, not timed)
        tune = scene.autotune() if not args.no_tune else None
        j = scene.submit(spp=args.warmup, first_sample=20_000)
        j.wait()
        j.close()
        clocks = ClockSampler(local)
        torch.cuda.synchronize()
        clocks.start()
        fast = dict(vol_fp16=True)
        j = scene.submit(spp=args.warmup, first_sample=30_000, **fast)
        j.wait()
        j.close()
        job = scene.submit(spp=args.steps, profile=True, **fast)
        job.wait()
        torch.cuda.synchronize()
        clk = clocks.stop()
        st = job.stats()
        job.close()
        # the unbiased-depth estimator with the global and with the 16^3-brick majorants,
        # and the reference's algorithm with the fp32 grid, on the same frame
        jg = scene.submit(spp=max(1, args.steps // 4), profile=True, vol_real_depth=True, vol_fp16=True)
        jg.wait()
        st_glob = jg.stats()
        jg.close()
        jb = scene.submit(spp=max(1, args.steps // 4), profile=True, vol_bricks=True, vol_fp16=True)
        jb.wait()
        st_brk = jb.stats()
        jb.close()
        jr = scene.submit(spp=max(1, args.steps // 4), profile=True)
        jr.wait()
        st_ref = jr.stats()
        jr.close()
        # the same frame on the persistent single-kernel schedule (warp-voted loop parts)
        jp = scene.submit(spp=args.steps, profile=True, vol_persistent=True, **fast)
        jp.wait()
        st_per = jp.stats()
        jp.close()
        value = st["samples"] / (st["gpu_ms"] / 1000.0)
        cpu = None
        if rank == 0 and not args.no_cpu:
            sys.path.insert(0, os.path.join(ROOT, "tests"))
            import oracle_lib
            o = oracle_lib.OracleScene.from_file(path)
            # successive samples of every 16th row until at least 10 s of CPU work are timed
            n_cpu, dt, s = 0, 0.0, 0
            while dt < 10.0 and s < 4096:
                t0 = time.perf_counter()
                _, cs = o.render(rows=(s % 16, res, 16), samples=(s // 16, s // 16 + 1), threads=os.cpu_count() or 1)
                dt += time.perf_counter() - t0
                n_cpu += int(cs[2])
                s += 1
            cpu = {"value": n_cpu / dt, "unit": "samples/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": "%d passes over every 16th row of the %dx%d volume frame, 1 spp each (%d samples, %.1f s)"
                             % (s, res, res, n_cpu, dt)}
        scene.close()
    line = {"metric": "samples/s (vol_path, fBm volume %dx%d, depth 32)" % (res, res), "value": value,
            "unit": "samples/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": st["gpu_ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fBm grid)",
            "config": {"workload": "volume_box", "width": res, "height": res, "grid": args.vol_grid,
                       "max_paths": args.vol_max_paths,
                       "max_depth": 32, "rr_depth": 5, "sigma_t_scale": 20, "albedo": 0.9, "hg_g": 0.6,
                       "autotune": None if tune is None else
                       {"refill_busy": tune["refill_busy"], "blocks_per_sm": tune["blocks_per_sm"],
                        "vol_chunk": tune["vol_chunk"], "wave_ms_tuned": round(tune["best_ms"], 3),
                        "wave_ms_default": round(tune["default_ms"], 3)}},
            "mrays_per_s": (st["rays_closest"] + st["rays_shadow"]) / (st["gpu_ms"] / 1000.0) / 1e6,
            "gpu_launches": st["kernel_launches"], "kernel_ms": {"vol_path": st["ms_volpath"]}, "clocks": clk,
            "mode": "the reference's delta tracking (global majorant, null collisions counted as depth) on the "
                    "fp16 grid (RAD_JOB_VOL_FP16)",
            "schedule": "per-event wavefront (a kernel per loop part over queues; state in HBM between parts)",
            "persistent_kernel": {"samples_per_s": st_per["samples"] / (st_per["gpu_ms"] / 1000.0),
                                  "gpu_launches": st_per["kernel_launches"],
                                  "schedule": "one persistent kernel, lanes vote on the loop part each warp step"},
            "unbiased_depth": {"global_majorant_samples_per_s": st_glob["samples"] / (st_glob["gpu_ms"] / 1000.0),
                               "brick_majorants_samples_per_s": st_brk["samples"] / (st_brk["gpu_ms"] / 1000.0),
                               "brick_mrays_per_s": (st_brk["rays_closest"] + st_brk["rays_shadow"])
                               / (st_brk["gpu_ms"] / 1000.0) / 1e6},
            "reference_algorithm_fp32": {"mode": "global majorant, fp32 grid, null collisions counted as depth",
                                    "spp": st_ref["samples"] // (res * res),
                                    "samples_per_s": st_ref["samples"] / (st_ref["gpu_ms"] / 1000.0),
                                    "mrays_per_s": (st_ref["rays_closest"] + st_ref["rays_shadow"])
                                    / (st_ref["gpu_ms"] / 1000.0) / 1e6}}
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)


def run_renderers(args, world, rank, local):
    """The other renderers on the many-spheres 1080p frame: bdpt (the line's value), particle_tracer and ao,
    each one job of `steps` whole-frame passes timed on the device, and the CPU oracle of each on a bounded
    sample with all host threads."""
    import torch
    import radiantiumplusplus_gb300 as rad
    from radiantiumplusplus_gb300 import scenes
    torch.cuda.set_device(local)
    rad.init({"device": local, "max_paths": args.renderers_max_paths, "bdpt_scratch_bytes": args.bdpt_scratch})
    Wr, Hr = args.renderers_res
    npix = Wr * Hr
    out = {}
    clk = None
    with tempfile.TemporaryDirectory(prefix="rad_bench_r_") as tmp:
        sc, assets = scenes.many_spheres(n_spheres=10000, width=Wr, height=Hr, spp=1, max_depth=MAX_DEPTH, seed=2)
        for name, renderer in (("bdpt", {"type": "bdpt", "max_depth": args.bdpt_depth}),
                               ("particle_tracer", {"type": "particle_tracer", "max_depth": MAX_DEPTH}),
                               ("ao", {"type": "ao"})):
            sc["renderer"] = renderer
            d = os.path.join(tmp, name)
            path = scenes.write_scene(d, sc, assets)
            scene = rad.Scene.from_file(path)
            per = npix  # samples (light paths for particle_tracer) per whole-frame pass
            j = scene.submit(spp=max(1, args.warmup) * (per if name == "particle_tracer" else 1), first_sample=20_000)
            j.wait()
            j.close()
            clocks = ClockSampler(local) if name == "bdpt" else None
            torch.cuda.synchronize()
            if clocks:
                clocks.start()
            job = scene.submit(spp=args.steps * (per if name == "particle_tracer" else 1), profile=True)
            job.wait()
            torch.cuda.synchronize()
            if clocks:
                clk = clocks.stop()
            st = job.stats()
            job.close()
            r = {"samples_per_s": st["samples"] / (st["gpu_ms"] / 1000.0), "gpu_ms": st["gpu_ms"],
                 "samples": st["samples"], "gpu_launches": st["kernel_launches"],
                 "unit": "light paths/s" if name == "particle_tracer" else "samples/s",
                 # profiled stage times (events around every launch); bdpt: generate = subpath starts,
                 # extend = closest-hit bounces, shade = walks + connections, shadow = visibility rays
                 "kernel_ms": {k: round(st["ms_" + k], 3) for k in
                               ("generate", "extend", "shade", "shadow", "accumulate", "volpath")}}
            if rank == 0 and not args.no_cpu:
                sys.path.insert(0, os.path.join(ROOT, "tests"))
                import oracle_lib
                o = oracle_lib.OracleScene.from_file(path)
                threads = os.cpu_count() or 1
                t0 = time.perf_counter()
                if name == "bdpt":
                    _, n = o.render_bdpt(rows=(0, Hr, args.bdpt_cpu_row_step), samples=(0, 1), threads=threads,
                                         count=True)
                    what = "rows 0..%d step %d at 1 spp" % (Hr, args.bdpt_cpu_row_step)
                elif name == "particle_tracer":
                    n = 2_000_000
                    o.render_particle(spp=npix, first=0, count=n, threads=threads)
                    what = "%d light paths of a %d-path frame" % (n, npix)
                else:
                    _, cs = o.render(rows=(0, Hr, 16), samples=(0, 1), threads=threads)
                    n = int(cs[2])
                    what = "rows 0..%d step 16 at 1 spp" % Hr
                dt = time.perf_counter() - t0
                r["cpu_baseline"] = {"value": n / dt, "unit": r["unit"], "cores": threads, "kind": "port",
                                     "sample": "%s (%d, %.1f s)" % (what, n, dt)}
                o.close()
            scene.close()
            out[name] = r
    b = out["bdpt"]
    line = {"metric": "samples/s (bdpt, many-spheres %dx%d, depth %d)" % (Wr, Hr, args.bdpt_depth),
            "value": b["samples_per_s"], "unit": "samples/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": b["gpu_ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": "many_spheres_renderers", "spheres": 10000, "triangles": 3200000,
                       "max_paths": args.renderers_max_paths, "bdpt_scratch_bytes": args.bdpt_scratch,
                       "width": Wr, "height": Hr, "bdpt_max_depth": args.bdpt_depth, "bdpt_rr_depth": 5,
                       "particle_max_depth": MAX_DEPTH, "l2": "inputs larger than L2: resident scene > 129 MB"},
            "gpu_launches": b["gpu_launches"], "clocks": clk, "renderers": out}
    if "cpu_baseline" in b:
        line["cpu_baseline"] = b["cpu_baseline"]
    print(json.dumps(line), flush=True)


def run_guided(args, world, rank, local):
    """Learned proposal vs plain BSDF sampling on the guided room (the sphere field in
    a closed room lit only through a ceiling opening), depth 16. The reference is a
    plain (BSDF-sampled) render of --guided-ref-spp samples per pixel, on the frame
    of --guided-res (a reduced frame by default, so that the plain reference
    converges within minutes). relMSE = mean over pixel channels of
    (x - ref)^2 / (ref^2 + 1e-2 mean(ref)^2); MSE is reported beside it. The
    guided job (fresh network, training in its first quarter of samples) runs at
    increasing spp until it reaches the plain job's 64-spp relMSE, and the
    wall-time ratio is reported. Every run has its own seed."""
    import numpy as np
    import torch
    import radiantiumplusplus_gb300 as rad
    from radiantiumplusplus_gb300 import scenes
    torch.cuda.set_device(local)
    rad.init({"device": local, "max_paths": args.guided_max_paths})
    Wg, Hg = args.guided_res
    with tempfile.TemporaryDirectory(prefix="rad_bench_guided_") as tmp:
        sc, assets = scenes.guided_room(n_spheres=args.guided_spheres, width=Wg, height=Hg, spp=64, max_depth=16)
        path = scenes.write_scene(tmp, sc, assets)
        scene = rad.Scene.from_file(path)
        gcfg = dict({"log2_table": 19}, **json.loads(args.guided_config))
        # Reference: the plain tracer at many samples per pixel
        j = scene.submit(spp=args.guided_ref_spp, seed=777)
        j.wait()
        ref = j.film().astype(np.float64)
        j.close()
        eps = 1e-2 * ref.mean() ** 2

        def relmse(film):
            d2 = (film.astype(np.float64) - ref) ** 2
            e = (d2 / (ref ** 2 + eps)).mean(axis=2).ravel()
            srt = np.sort(e)
            return (float(e.mean()), float(srt[:int(0.99 * srt.size)].mean()), float(np.median(e)),
                    float(d2.mean()))

        seeds = iter(range(100, 10000))

        def timed(spp, guide):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            j = scene.submit(spp=spp, seed=next(seeds), guide=guide)
            j.wait()
            dt = time.perf_counter() - t0
            st = j.stats()
            f = j.film()
            j.close()
            return dt, st, f

        timed(64, False)  # warm-up: the timed plain job's wave graphs (64 samples a wave) and allocations
        scene.guide_enable(gcfg)
        timed(4, True)
        clocks = ClockSampler(local)
        clocks.start()
        tp, stp, fp = timed(64, False)
        ep = relmse(fp)
        runs = []
        reached = None
        for spp in args.guided_spp:
            scene.guide_enable(gcfg)  # fresh network: training is part of the time
            tg, stg, fg = timed(spp, True)
            eg = relmse(fg)
            runs.append({"spp": spp, "wall_s": tg, "relmse": eg[0], "relmse_trim1": eg[1], "relmse_median": eg[2],
                         "mse": eg[3], "mean_over_ref": float(fg.mean() / ref.mean()),
                         "train_steps": stg["guide_train_steps"], "records": stg["guide_records"],
                         "samples_per_s": stg["samples"] / tg,
                         "mrays_per_s": (stg["rays_closest"] + stg["rays_shadow"]) / tg / 1e6})
            if reached is None and eg[0] <= ep[0]:
                reached = runs[-1]
        clk = clocks.stop()
        scene.close()
    line = {"metric": "wall-time ratio guided/plain at plain 64-spp relMSE (guided room %dx%d, depth 16)" % (Wg, Hg),
            "value": (reached["wall_s"] / tp) if reached else None, "unit": "ratio", "n_gpus": 1,
            "steps": 1, "warmup": 1, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (guide network fp16 weights, fp32 accumulation)", "data": "synthetic (seeded generator)",
            "config": {"workload": "guided_room", "spheres": args.guided_spheres, "width": Wg, "height": Hg,
                       "max_paths": args.guided_max_paths,
                       "max_depth": 16, "room": 200, "opening": 5, "irradiance": 1000,
                       "reference": "plain render, %d spp" % args.guided_ref_spp, "ref_mean": float(ref.mean()),
                       "relmse_eps": eps,
                       "guide": dict({"levels": 16, "mlp": "3x64", "lobes": 8}, **gcfg)},
            "plain": {"spp": 64, "wall_s": tp, "relmse": ep[0], "relmse_trim1": ep[1], "relmse_median": ep[2],
                      "mse": ep[3],
                      "mean_over_ref": float(fp.mean() / ref.mean()),
                      "samples_per_s": stp["samples"] / tp,
                      "mrays_per_s": (stp["rays_closest"] + stp["rays_shadow"]) / tp / 1e6},
            "guided": runs, "clocks": clk}
    print(json.dumps(line), flush=True)


def _serving_pool(rng, n_scenes):
    """Resident scenes of the serving mix: many-spheres scenes with sphere counts
    lognormal between 32 and 10,000 (10 k - 3.2 M triangles), frames cycling
    through 256^2, 512^2, 1280x720 and 1920x1080, depth uniform in 8..16."""
    import numpy as np
    res = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]
    pool = []
    for k in range(n_scenes):
        n = int(np.clip(np.exp(rng.normal(np.log(600.0), 1.3)), 32, 10000))
        w, h = res[k % 4]
        pool.append((n, w, h, int(rng.integers(8, 17))))
    return pool


def run_serving(args, world, rank, local):
    """Serving loop (continuous batching): Poisson arrivals of jobs over resident
    scenes, offered at fractions of the measured peak throughput; per load, the
    throughput and the p50 / p99 of job latency (submit to completion) and of
    stretch (latency / the job's time alone on the GPU)."""
    import numpy as np
    import torch
    import radiantiumplusplus_gb300 as rad
    from radiantiumplusplus_gb300 import scenes
    torch.cuda.set_device(local)
    rad.init({"device": local})
    rng = np.random.default_rng(4)
    pool = _serving_pool(rng, args.serving_scenes)
    with tempfile.TemporaryDirectory(prefix="rad_bench_srv_") as tmp:
        loaded = []
        for k, (n, w, h, depth) in enumerate(pool):
            sc, assets = scenes.many_spheres(n_spheres=n, n_emitters=8, width=w, height=h, spp=1, max_depth=depth,
                                             seed=40 + k, extent=100.0 * (n / 10000.0) ** (1 / 3))
            path = scenes.write_scene(os.path.join(tmp, "s%d" % k), sc, assets)
            loaded.append(rad.Scene.from_file(path))
        # each scene alone: samples/s of a job of ~40 M samples (device-timed), and the
        # fixed cost of a job through the API (latency of 1-spp jobs minus their GPU time)
        alone, fixed_ms = [], []
        for sc in loaded:
            spp = max(1, int(4e7 / (sc.width * sc.height)))
            j = sc.submit(spp=spp)
            j.wait()
            st = j.stats()
            j.close()
            alone.append(st["samples"] / max(1e-6, st["gpu_ms"] / 1000.0))
            lat1 = []
            for _ in range(5):
                j = sc.submit(spp=1)
                j.wait()
                st = j.stats()
                j.close()
                lat1.append(st["queue_ms"] + st["wall_ms"] - 1000.0 * st["samples"] / alone[-1])
            fixed_ms.append(max(0.0, float(np.median(lat1))))

        def draw(n, r):
            picks = r.integers(0, len(loaded), n)
            spps = np.exp(r.uniform(np.log(args.spp_min), np.log(args.spp_max), n)).astype(int)
            return picks, spps

        # mean samples per job of the distribution: mean frame x mean of log-uniform spp
        lo, hi = float(args.spp_min), float(args.spp_max)
        mean_spp = (hi - lo) / np.log(hi / lo) if hi > lo else lo
        mean_samples = float(np.mean([sc.width * sc.height for sc in loaded])) * mean_spp

        def run(jobs_spec, arrivals):
            submitted = []
            t0 = time.perf_counter()
            for a, (k, spp) in zip(arrivals, jobs_spec):
                delay = t0 + a - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                submitted.append((loaded[k].submit(spp=int(spp)), k))
            lat, stretch, stretch_e2e, samples, mixed = [], [], [], 0, 0
            for j, k in submitted:
                j.wait()
                st = j.stats()
                l_ms = st["queue_ms"] + st["wall_ms"]
                lat.append(l_ms)
                samples += st["samples"]
                mixed += st["mixed_waves"] > 0
                gpu_alone = 1000.0 * st["samples"] / alone[k]
                stretch.append(l_ms / gpu_alone)
                stretch_e2e.append(l_ms / (gpu_alone + fixed_ms[k]))
                j.close()
            return (time.perf_counter() - t0, np.array(lat), np.array(stretch), np.array(stretch_e2e), samples,
                    mixed)

        # peak: a burst of jobs submitted at once
        picks, spps = draw(args.serving_burst, np.random.default_rng(5))
        span, _, _, _, samples, _ = run(list(zip(picks, spps)), np.zeros(len(picks)))
        peak = samples / span
        results = []
        for load, policy in args.serving_loads:
            cfg = {"share_exponent": 1.0 if policy == "size" else 0.0,
                   "deadline_ns_per_sample": float(policy[3:]) if policy.startswith("edf") else 0.0,
                   "slowdown_ns_per_sample": float(policy[4:]) if policy.startswith("slow") else 0.0}
            rad.init(cfg)
            lam = load * peak / mean_samples
            r = np.random.default_rng(1000 + int(round(load * 1000)))  # the same jobs for every policy at a load
            picks, spps = draw(args.serving_jobs, r)
            arrivals = np.cumsum(r.exponential(1.0 / lam, len(picks)))
            span, lat, stretch, st_e2e, samples, mixed = run(list(zip(picks, spps)), arrivals)
            results.append({"offered_load": load, "policy": policy, "rate_jobs_per_s": lam,
                            "jobs": len(picks), "jobs_in_mixed_waves": int(mixed),
                            "offered_samples_per_s": samples / arrivals[-1],
                            "throughput_samples_per_s": samples / span,
                            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                            "p99_over_p50": float(np.percentile(lat, 99) / np.percentile(lat, 50)),
                            "stretch_p50": float(np.percentile(stretch, 50)),
                            "stretch_p99": float(np.percentile(stretch, 99)),
                            "stretch_p99_over_p50": float(np.percentile(stretch, 99) / np.percentile(stretch, 50)),
                            "stretch_e2e_p50": float(np.percentile(st_e2e, 50)),
                            "stretch_e2e_p99": float(np.percentile(st_e2e, 99)),
                            "stretch_e2e_p99_over_p50": float(np.percentile(st_e2e, 99) / np.percentile(st_e2e, 50))})
        rad.init({"share_exponent": 0.0, "deadline_ns_per_sample": 0.0, "slowdown_ns_per_sample": 0.0})
        for sc in loaded:
            sc.close()
    line = {"metric": "serving: throughput and p50/p99 job latency (Poisson arrivals, continuous batching)",
            "value": peak, "unit": "samples/s", "n_gpus": 1, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded many-spheres generator)",
            "config": {"workload": "serving_mix", "scenes": [{"spheres": n, "triangles": 320 * n, "width": w,
                                                              "height": h, "max_depth": d} for n, w, h, d in pool],
                       "spp": "log-uniform [%d, %d]" % (args.spp_min, args.spp_max),
                       "mean_samples_per_job": mean_samples, "peak_from_burst_of": args.serving_burst,
                       "budget_bytes": 150e9},
            "alone_samples_per_s": alone, "fixed_ms_per_job": fixed_ms,
            "policies": {"fair": "equal path-slot shares in mixed waves (processor sharing)",
                         "size": "shares in proportion to the work left",
                         "edfN": "earliest deadline first, deadline = submit + N ns x samples",
                         "slowN": "highest slowdown first, slowdown = age / (N ns x samples + 20 ms)"},
            "sweep": results}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--cpu-row-step", type=int, default=4)
    ap.add_argument("--workload", default="many_spheres",
                    choices=["many_spheres", "volume", "serving", "guided", "renderers"])
    ap.add_argument("--bdpt-depth", type=int, default=MAX_DEPTH, help="renderers: bdpt max_depth")
    ap.add_argument("--renderers-res", type=int, nargs=2, default=[W, H], help="renderers: frame size")
    ap.add_argument("--bdpt-cpu-row-step", type=int, default=8, help="renderers: oracle bdpt row sample")
    ap.add_argument("--renderers-max-paths", type=int, default=1 << 24, help="renderers: rad_init max_paths")
    ap.add_argument("--bdpt-scratch", type=int, default=32 << 30, help="renderers: rad_init bdpt_scratch_bytes")
    ap.add_argument("--guided-res", type=int, nargs=2, default=[240, 135])
    ap.add_argument("--guided-spheres", type=int, default=10000)
    ap.add_argument("--guided-ref-spp", type=int, default=1 << 20)
    ap.add_argument("--guided-spp", type=int, nargs="+", default=[8, 16, 24, 32, 48, 64])
    ap.add_argument("--guided-config", default="{}", help="JSON of rad_guide_enable settings for the guided jobs")
    ap.add_argument("--guided-max-paths", type=int, default=1 << 21, help="guided workload: rad_init max_paths")
    ap.add_argument("--no-tune", action="store_true", help="skip rad_autotune (keeps launch indices fixed for ncu)")
    ap.add_argument("--vol-res", type=int, default=1024)
    ap.add_argument("--max-paths", type=int, default=1 << 25,
                    help="path workload: paths per wave (rad_init max_paths; 2^25 = 16 samples of 1080p)")
    ap.add_argument("--spp-per-step", type=int, default=16,
                    help="path workload: samples per pixel of one step (one job of the e2e loop)")
    ap.add_argument("--vol-max-paths", type=int, default=1 << 24,
                    help="volume workload: paths per wave (rad_init max_paths)")
    ap.add_argument("--vol-grid", type=int, default=256)
    ap.add_argument("--serving-scenes", type=int, default=16, help="serving: resident scenes")
    ap.add_argument("--serving-jobs", type=int, default=120, help="serving: jobs per load point")
    ap.add_argument("--serving-burst", type=int, default=40, help="serving: jobs of the peak-throughput burst")
    ap.add_argument("--serving-loads", type=lambda t: (float(t.split(":")[0]), t.split(":")[1]), nargs="+",
                    default=[(0.5, "fair"), (0.8, "fair"), (0.8, "edf20"), (1.0, "fair")],
                    help="serving: offered load (fraction of peak):policy (fair | size | edfN | slowN) pairs")
    ap.add_argument("--spp-min", type=int, default=16)
    ap.add_argument("--spp-max", type=int, default=1024)
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "volume":
        run_volume(args, world, rank, local)
    elif args.workload == "guided":
        run_guided(args, world, rank, local)
    elif args.workload == "serving":
        run_serving(args, world, rank, local)
    elif args.workload == "renderers":
        run_renderers(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
