"""Benchmark: M path samples/s of the GB300 renderer core on the 1080p triangle-mesh workload.

One step = one dfpt_render call of --spp-per-step passes (default 64) over the whole 1920x1080
image; a pass is one sample per pixel, the unit of the reference's Kernel.execute
(DayflowerApplication.java:853), so the default 4 timed steps render the 256 spp of the
triangle-mesh configuration. Inside a call, the passes run `wide_samples` at a time through the
wave kernels (same samples, same film and image as pass-by-pass rendering, tested); the autotuner
picks up to 64 passes per wave (133 M path slots). The workload
is mesh_scene: an fBm-displaced geodesic icosphere (200,000 triangles, 4 Lambertian/Phong regions)
over a 512x512 fBm heightfield (522,242 triangles), BVHs built by the restated reference builder,
depth 8, ACES; seeded synthetic data (the reference publishes no scenes).

  value : device-resident throughput (scene uploaded once, per-step CUDA events on the handle's
          stream, L2 flushed between steps with a 256 MiB write);
  e2e   : the same metric through the C-ABI as the reference's render loop uses it
          (dfpt_set_camera from host memory, dfpt_render, dfpt_read_bgra8 into host memory);
  frame_loop : the interactive loop of DayflowerApplication (one pass per dfpt_render call, the
          image read back every frame), M samples/s on the host clock;
  roofline : the dominant kernel (closest-hit traversal), algorithmic bytes per closest-hit
          segment = nodes*32 + triangles*48 + 64 with the mean visit counts of closest-hit
          segments from the GPU's own counters over a step (the CPU restatement's counts on its
          sample reported beside them), against the L2-resident read bandwidth measured in the
          same run (the records live in L2); the HBM copy rate of MEASURED_PEAKS.json and the
          DRAM traffic of one ncu capture are reported beside it;
  cpu_baseline : the oracle's strict-FP32 restatement of the reference kernel on all host cores,
          over a bounded band of rows (the reference's Java thread-pool path needs a JVM).
--impl reference times that CPU restatement alone on the same workload, config and metric; it
reads the workload file that build() wrote (dfpt.workloads), so its process maps only the oracle.
Multi-GPU: pixels are independent, so N ranks render N replicas (weak scaling, no collective on
the data path); value sums the ranks' samples over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import math
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "dayflower-path-tracer_gb300"))
sys.path.insert(0, str(ROOT))

METRIC = "M path samples/s @1080p"
UNIT = "M samples/s"
# Measured DRAM bytes (read + write) per closest-hit segment of the traversal kernel on
# mesh_scene: one ncu capture of the traversal kernel at 960x540.
TRACE_DRAM_BYTES_PER_SEGMENT = 65.5


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--spp-per-step", type=int, default=64, help="passes (1 spp each) per step: one dfpt_render call")
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="dfpt", choices=["dfpt", "reference"])
    ap.add_argument("--workload", default="mesh_scene", choices=["mesh_scene", "sphere_scene", "instances_scene"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-scenes leg")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the inverse-rendering leg")
    ap.add_argument("--adjoint-iters", type=int, default=10)
    ap.add_argument("--trace-config", type=int, default=-1, help="fixed traversal configuration (skips the autotuner)")
    ap.add_argument("--set-tuning", action="append", default=[], metavar="KEY=VALUE",
                    help="a dfpt_set_tuning key applied after the traversal configuration is chosen (repeatable)")
    ap.add_argument("--wide", type=int, default=0, help="fixed passes per wave (skips that tuner)")
    ap.add_argument("--shadow-defer", type=int, default=-1, help="with --wide: 1 one shadow launch per wave, 0 per bounce")
    return ap.parse_args()


def build_workload(name, width, height):
    """(scene, sky, params struct, (w, h), meta, source) from the workload file `build()` wrote
    (read with numpy alone: the process maps no GPU library for it), else generated here."""
    from dfpt import workloads

    path = workloads.cache_path(name, width, height)
    source = "workload file"
    if not path.exists():
        path = workloads.prepare(name, width, height)  # generator + libdfpt's scene compiler
        source = "generated in this process"
    scene, sky, params, size, meta = workloads.load(path)
    return scene, sky, params, size, meta, source


TONE_MAPPERS = {1: "ACES (modified filmic)", 2: "Reinhard", 3: "Reinhard modified 1", 4: "Reinhard modified 2"}
EXTENSIONS = {
    "mesh_scene": "Phong regions with exponents U(10,200) (extension records)",
    "instances_scene": "500 area-light triangle primitives, emission U(1,20) (extension records)",
    "sphere_scene": "none",
}


def workload_config(name, w, h, scene, params, world=1):
    """The workload as both arms name it (same keys and values on the GPU and CPU reference arms)."""
    return {"workload": f"{name} {w}x{h}", "triangles": int(scene.triangles.size // 12),
            "primitives": int(scene.primitive_count), "depth_max": int(params.pt_ray_depth_maximum),
            "russian_roulette_from": int(params.pt_ray_depth_russian_roulette),
            "tone_mapper": TONE_MAPPERS.get(int(params.tone_mapper_type), str(params.tone_mapper_type)),
            "extensions": EXTENSIONS.get(name, "none"), "spp_per_pass": 1, "parallelism": f"replicas x{world}"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device_index=0):
        self.rows = []
        self.proc = None
        self.device_index = device_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device_index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        import statistics

        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, nm in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def cpu_baseline(scene, sky, p, width, height, seconds, threads=0):
    """Times the oracle's strict-FP32 restatement on a band of rows sized to ~`seconds`."""
    from oracle import oracle

    threads = threads or os.cpu_count() or 1
    rows = max(1, threads // 2)
    t0 = time.perf_counter()
    out = oracle.render(scene, sky, p, width, height, passes=1, precision=32, threads=threads, rows=(0, rows))
    dt = time.perf_counter() - t0
    target = min(height, max(rows, int(rows * seconds / max(dt, 1e-3))))
    r0 = max(0, height // 2 - target // 2)
    passes = 1
    for _ in range(3):
        t0 = time.perf_counter()
        out = oracle.render(scene, sky, p, width, height, passes=passes, precision=32, threads=threads,
                            rows=(r0, r0 + target))
        dt = time.perf_counter() - t0
        # A whole frame that takes well under `seconds` is rendered for more passes (1 spp each).
        if target < height or dt >= 0.5 * seconds or passes >= 256:
            break
        passes = min(256, int(math.ceil(passes * seconds / max(dt, 1e-3))))
    samples = target * width * passes
    c = out["counters"].astype(float)
    segs = c[0] + c[1]
    return {
        "value": samples / dt / 1e6,
        "unit": UNIT,
        "cores": threads,
        "kind": "port",
        "sample": f"rows {r0}..{r0 + target} of {width}x{height}, {passes} pass(es) of 1 spp, strict FP32 restatement, "
                  f"{threads} threads, {dt:.1f} s",
        "segments_per_sample": segs / samples,
        "nodes_per_segment": c[2] / max(segs, 1),
        "tris_per_segment": c[3] / max(segs, 1),
        "closest_nodes_per_segment": c[4] / max(c[0], 1),
        "closest_tris_per_segment": c[5] / max(c[0], 1),
        "closest_per_sample": c[0] / samples,
    }


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    scene, sky, p, (w, h), meta, source = build_workload(args.workload, args.width, args.height)
    from oracle import oracle

    threads = os.cpu_count() or 1
    # Each step renders a band of rows sized so the whole run stays within a few minutes.
    band = max(1, threads // 2)
    t0 = time.perf_counter()
    oracle.render(scene, sky, p, w, h, passes=1, precision=32, threads=threads, rows=(0, band))
    per_row = (time.perf_counter() - t0) / band
    budget = 120.0 / max(1, args.steps + args.warmup)
    band = int(min(h, max(band, budget / max(per_row, 1e-6))))
    for i in range(args.warmup):
        oracle.render(scene, sky, p, w, h, passes=1, precision=32, threads=threads, rows=(0, band), pass_begin=i)
    total, samples = 0.0, 0
    for i in range(args.steps):
        r0 = (i * band) % max(1, h - band)
        t0 = time.perf_counter()
        oracle.render(scene, sky, p, w, h, passes=1, precision=32, threads=threads, rows=(r0, r0 + band), pass_begin=i)
        total += time.perf_counter() - t0
        samples += band * w
    value = samples / total / 1e6
    with open("/proc/self/maps") as f:
        maps = f.read()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": workload_config(args.workload, w, h, scene, p, args.gpus),
        "step": {"rows": band, "passes": 1, "samples": band * w},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{band} rows x {w} px x 1 pass per step, strict FP32 restatement of "
                                   "GPURendererKernel.run on all host threads (the reference's Java thread-pool "
                                   "path is unavailable: no JVM)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "workload_source": source, "gpu_library_mapped": "libdfpt" in maps,
    }
    print(json.dumps(line), flush=True)


def batch_leg(args, stream, torch, barrier, dist, world):
    """Batched rendering: `--batch-scenes` seeded scenes (triangles log-uniform in [1k, 500k],
    resolutions {256^2, 512^2, 1024^2}, spp {16, 64, 256}) rendered to their full sample counts
    (a) by one BatchRenderer - one launch per stage per wave, a replayed CUDA graph, wave capacity
    and traversal configuration picked by the autotuner - and (b) as sequential single-scene
    renders (one RendererKernel per scene, spp passes each, one stream). Scenes are uploaded and
    graphs built before either timed region; each region is bracketed by CUDA events."""
    import numpy as np
    from dfpt import synthetic
    from dfpt.autotune import tune_batch
    from dfpt.batch import BatchRenderer
    from dfpt.kernel import RendererKernel

    t0 = time.perf_counter()
    work = synthetic.batch_workload(seed=5, count=args.batch_scenes)
    build_s = time.perf_counter() - t0
    samples = sum(x["width"] * x["height"] * x["spp"] for x in work)

    def timed(fn):
        with torch.cuda.stream(stream):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        fn()
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3

    b = BatchRenderer()
    b.set_stream(stream.cuda_stream)
    for x in work:
        b.add(x["scene"], x["width"], x["height"], x["spp"], x["sky"], x["params"])
    tuning = tune_batch(b)
    launches0 = b.launch_count()
    barrier()
    batch_s = timed(b.render)
    barrier()
    batch_launches = b.launch_count() - launches0

    # Sequential single-scene renders, (a) pass by pass (the plain kernel: one launch sequence per
    # pass) and (b) with the handle's wide passes (8 passes per wave).
    handles = []
    for x in work:
        k = RendererKernel(x["scene"], x["sky"], x["params"])
        k.update(x["width"], x["height"])
        k.set_stream(stream.cuda_stream)
        k.set_tuning("trace_config", tuning["best"]["trace_config"])
        k.set_tuning("wide_samples", 1)
        k.execute(2)  # builds the pass graph
        handles.append(k)
    torch.cuda.synchronize()

    def sequential():
        for k, x in zip(handles, work):
            k.clear()
            k.execute(x["spp"])

    barrier()
    seq_s = timed(sequential)
    barrier()
    for k in handles:
        k.set_tuning("wide_samples", 8)
        k.set_tuning("shadow_defer", tuning["best"].get("shadow_defer", 0))  # the batch's shadow schedule
        k.execute(9)  # builds the wave graph
    torch.cuda.synchronize()
    barrier()
    seq_wide_s = timed(sequential)
    barrier()
    for k in handles:
        k.dispose()
    # The batch reproduces the single-scene films (same paths, same Kahan order per pixel): fresh
    # handles (pass index from 0, as the batch's sample index) on a sample of the scenes.
    worst = 0.0
    for i in range(0, len(work), max(1, len(work) // 8)):
        x = work[i]
        k = RendererKernel(x["scene"], x["sky"], x["params"])
        k.update(x["width"], x["height"])
        k.execute(x["spp"])
        fs, ns = k.film()
        k.dispose()
        fb, nb = b.film(i)
        if not np.array_equal(nb, ns):
            worst = float("inf")
            break
        worst = max(worst, float(np.max(np.abs(fb - fs) / (np.abs(fs) + 1e-3))))
    b.dispose()
    if dist is not None:
        t = torch.tensor([batch_s, seq_s, seq_wide_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        batch_s, seq_s, seq_wide_s = (float(v) for v in t.tolist())
    n = len(work)
    return {
        "metric": "scenes/s", "value": world * n / batch_s, "sequential_value": world * n / seq_s,
        "speedup_vs_sequential": seq_s / batch_s, "samples": samples,
        "sequential_wide_value": world * n / seq_wide_s, "speedup_vs_sequential_wide": seq_wide_s / batch_s,
        "sequential": "64 RendererKernel handles on one stream, clear + dfpt_render(spp) each: pass by pass "
                      "(wide_samples 1, the plain kernel) and with 8-pass waves and the batch's shadow schedule "
                      "(sequential_wide_*)",
        "m_samples_per_s": world * samples / batch_s / 1e6, "sequential_m_samples_per_s": world * samples / seq_s / 1e6,
        "batch_s": batch_s, "sequential_s": seq_s, "gpu_launches": int(batch_launches),
        "triangles_total": sum(x["triangles"] for x in work), "scenes": n, "scene_build_s": round(build_s, 1),
        "tuning": tuning["best"], "film_max_rel_diff_vs_sequential": worst,
        "workload": "batch_workload seed 5: tris log-uniform [1k,500k], res {256,512,1024}^2, spp {16,64,256}, depth 5",
    }


def adjoint_leg(args, torch, barrier, dist, world):
    """Inverse rendering at 512x512, 16 spp per iteration: 256 spheres on a plane under a Perez sky;
    the target is rendered at the true albedos U(0.1, 0.9)^3 and turbidity 3, the optimisation
    starts at albedo 0.5 and turbidity 2. One iteration = dfpt_diff_forward (16 spp, image to host)
    + FP64 L2 loss + dfpt_diff_backward (replay, gradients to host) + a normalised gradient step;
    timed on the host clock around the whole iteration. t_fwd is the forward alone."""
    import numpy as np
    from dfpt import synthetic
    from dfpt.diff import DiffRenderer
    from dfpt.kernel import RendererKernel
    from dfpt.scene import SkyState

    cs, params, (w, h), truth, start = synthetic.inverse_scene(seed=6, width=512, height=512, count=256)
    k = RendererKernel(cs, SkyState(truth["sun_direction"], truth["turbidity"]), params)
    k.update(w, h)
    from dfpt.autotune import tune_trace

    tuning = tune_trace(k, passes=4, warmup=1)
    d = DiffRenderer(k)
    spp = 16
    target = d.forward(truth["albedo"], None, truth["phong_exponent"], truth["turbidity"], truth["sun_direction"], 256).astype(np.float64)
    albedo = start["albedo"].astype(np.float64).copy()
    turb = float(start["turbidity"])
    expo, sun = start["phong_exponent"], start["sun_direction"]

    target32 = target.astype(np.float32)

    def step(update=True):
        # Residual in FP32 (the image's precision), the loss reduced in FP64, dL/dimage = 2 r.
        r = d.forward(albedo, None, expo, turb, sun, spp) - target32
        r64 = r.reshape(-1).astype(np.float64)
        loss = float(r64 @ r64)
        r *= 2.0
        g = d.backward(r)
        return loss, g

    for _ in range(2):  # warm-up: graphs, buffers
        step()
    barrier()
    fw = []
    for _ in range(3):
        t0 = time.perf_counter()
        d.forward(albedo, None, expo, turb, sun, spp)
        fw.append(time.perf_counter() - t0)
    t_fwd = min(fw)
    losses, iters = [], []
    for _ in range(args.adjoint_iters):
        t0 = time.perf_counter()
        loss, g = step()
        ga = g["albedo"]
        albedo[1:] -= 0.05 * ga[1:] / (np.abs(ga[1:]).max() + 1e-30)
        np.clip(albedo, 0.01, 1.0, out=albedo)
        turb = float(np.clip(turb - 0.1 * np.sign(g["turbidity"]), 1.5, 8.0))
        iters.append(time.perf_counter() - t0)
        losses.append(loss)
    barrier()
    t_adj = float(np.median(iters))
    # Finite-difference checks at the start point. The loss is linearised at a 64-spp start image
    # (weights W = 2 (img - target), the same for every seed), so adjoint and central difference
    # estimate the same derivative of sum(W * E[img]). Each seed renders the pair with common random
    # numbers (fresh handles: the same pass indices). As configured (Russian roulette from depth 3:
    # its albedo-dependent decisions make a single seed's difference jump) over `seeds` seeds, with
    # the standard error of the mean per-seed gap; the Phong exponent's adjoint is a score-function
    # estimate (a different estimator of the same derivative), so it needs the seeds too. With
    # roulette off, albedo and turbidity on one seed (the estimator is smooth in them).
    a0 = start["albedo"].astype(np.float64)
    t0_ = float(start["turbidity"])
    sun0 = np.asarray(start["sun_direction"], np.float64)
    hstep = 1e-3

    def render(prm, theta, n_spp):
        k2 = RendererKernel(cs, SkyState(truth["sun_direction"], truth["turbidity"]), prm)
        k2.update(w, h)
        img = DiffRenderer(k2).forward(theta["albedo"], None, theta["exponent"], theta["turbidity"], theta["sun"], n_spp)
        k2.dispose()
        return img.astype(np.float64)

    theta0 = {"albedo": a0, "exponent": expo.astype(np.float64), "turbidity": t0_, "sun": sun0}
    kp = RendererKernel(cs, SkyState(truth["sun_direction"], truth["turbidity"]), dict(params, seed=77))
    kp.update(w, h)
    dp_ = DiffRenderer(kp)
    wgt = 2.0 * (dp_.forward(theta0["albedo"], None, theta0["exponent"], t0_, sun0, 64).astype(np.float64) - target)
    # The Phong sphere checked is the one with the largest exponent gradient in this pilot (seed 77,
    # independent of the checked seeds); every 4th sphere (primitives 4, 8, ...) is Phong.
    pilot = np.abs(dp_.backward(wgt.astype(np.float32))["phong_exponent"])
    kp.dispose()
    phong = np.arange(4, pilot.size, 4)
    phong_prim = int(phong[np.argmax(pilot[phong])])

    def shifted(key, idx, dv):
        t = {kk: (v.copy() if isinstance(v, np.ndarray) else v) for kk, v in theta0.items()}
        if key == "turbidity":
            t[key] = t[key] + dv
        else:
            t[key][idx] += dv
        return t

    checks = [("albedo[1,0]", "albedo", (1, 0), hstep), ("albedo[17,1]", "albedo", (17, 1), hstep),
              ("albedo[100,2]", "albedo", (100, 2), hstep), ("albedo[200,0]", "albedo", (200, 0), hstep),
              ("turbidity", "turbidity", None, hstep)]
    more = [(f"phong_exponent[{phong_prim}]", "exponent", phong_prim, 1.0)] + \
           [(f"sun_direction[{j}]", "sun", j, hstep) for j in range(3)]

    def fd_check(prm, items, seeds):
        per = {name: ([], []) for name, *_ in items}
        for sd in range(seeds):
            ps = dict(prm, seed=1000 + sd)
            kk = RendererKernel(cs, SkyState(truth["sun_direction"], truth["turbidity"]), ps)
            kk.update(w, h)
            dd = DiffRenderer(kk)
            dd.forward(theta0["albedo"], None, theta0["exponent"], theta0["turbidity"], theta0["sun"], spp)
            g = dd.backward(wgt.astype(np.float32))
            kk.dispose()
            adj = {"albedo": g["albedo"], "exponent": g["phong_exponent"], "turbidity": g["turbidity"], "sun": g["sun_direction"]}
            for name, key, idx, hh in items:
                plus = float(np.sum(wgt * render(ps, shifted(key, idx, hh), spp)))
                minus = float(np.sum(wgt * render(ps, shifted(key, idx, -hh), spp)))
                per[name][0].append(float(adj[key] if idx is None else adj[key][idx]))
                per[name][1].append((plus - minus) / (2 * hh))
        out = {}
        for name, (av, fv) in per.items():
            av, fv = np.asarray(av), np.asarray(fv)
            gap = fv - av
            se = float(gap.std(ddof=1) / np.sqrt(len(gap))) if len(gap) > 1 else 0.0
            rel = abs(float(av.mean() - fv.mean())) / max(abs(float(fv.mean())), 1e-30)
            out[name] = {"adjoint": float(av.mean()), "fd": float(fv.mean()), "rel_err": rel, "se": se,
                         "within": bool(rel <= 0.02 or abs(float(gap.mean())) <= 3 * se), "seeds": len(gap)}
        return out

    fd = fd_check(params, checks + more, seeds=8)
    fd_no_rr = fd_check(dict(params, pt_ray_depth_russian_roulette=params["pt_ray_depth_maximum"] + 1), checks, seeds=1)
    k.dispose()
    return {
        "metric": "adjoint iters/s", "value": world / t_adj, "unit": "iters/s", "t_adj_s": t_adj, "t_fwd_s": t_fwd,
        "t_adj_over_t_fwd": t_adj / t_fwd, "spp_per_iter": spp, "resolution": [w, h], "primitives": int(cs.primitives.size // 3),
        "loss_first": losses[0], "loss_last": losses[-1], "iters": len(losses),
        "fd_check": fd, "fd_check_no_russian_roulette": fd_no_rr, "fd_step": hstep, "fd_step_phong_exponent": 1.0,
        "fd_note": "mean over seeds of adjoint and central difference (common random numbers per seed); se = standard "
                   "error of the mean per-seed gap; within = rel_err <= 0.02 or |gap| <= 3 se",
        "trace_config": tuning["best"], "primitive_culling": tuning.get("primitive_culling", 0),
        "culling_ms_per_pass": {str(kk): round(v, 3) for kk, v in tuning.get("culling_ms_per_pass", {}).items()},
        "workload": "inverse_scene seed 6: 256 spheres (every 4th Phong) on a plane, Perez sky; albedo U(0.1,0.9)^3, T 3 -> start 0.5, T 2",
        "timing": "host clock around forward + FP64 loss + backward + update (C-ABI, host buffers)",
    }


def l2_read_peak(torch, stream):
    """The L2-resident read roof: dfpt_probe_read_bandwidth over buffers of 24-64 MiB (smaller than
    L2), the best of three runs per size, on the bench's stream."""
    from dfpt import _lib as dlib

    lib = dlib.load()
    best, per_size = 0.0, {}
    for mib in (24, 48, 64):
        buf = torch.ones(mib * (1 << 20) // 4, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        g = C.c_double()
        runs = []
        for _ in range(3):
            dlib.check(lib.dfpt_probe_read_bandwidth(C.c_void_p(buf.data_ptr()), buf.numel() * 4, 200,
                                                     C.c_void_p(stream.cuda_stream), C.byref(g)))
            runs.append(g.value)
        per_size[str(mib)] = round(max(runs), 1)
        best = max(best, max(runs))
        del buf
    return best, per_size


def frame_loop(k, cam, host_img, frames, warmup, barrier):
    """The reference's interactive render loop (DayflowerApplication.java:853-855): per frame
    dfpt_set_camera from host memory, dfpt_render of ONE pass (1 spp) and dfpt_read_bgra8 into host
    memory. Host clock around `frames` frames; M samples/s of the whole image."""
    import torch

    for _ in range(warmup):
        k.update_camera(cam)
        k.execute(1)
        k.get(host_img)
    barrier()
    torch.cuda.nvtx.range_push("frame_loop")  # lets a profiler take the frames' kernels alone
    t0 = time.perf_counter()
    for _ in range(frames):
        k.update_camera(cam)
        k.execute(1)
        k.get(host_img)
    barrier()
    dt = time.perf_counter() - t0
    torch.cuda.nvtx.range_pop()
    return dt


def frame_kernels(k, frames=8):
    """Per-kernel milliseconds of one frame (1-pass calls with an event between kernels)."""
    k.set_profiling(True)
    tot = {}
    for _ in range(frames):
        k.execute(1)
        k.synchronize()
        for kk, (ms, n) in k.read_profile().items():
            tot[kk] = tot.get(kk, 0.0) + ms / frames
    k.set_profiling(False)
    return {kk: round(v, 4) for kk, v in tot.items() if v > 0}


# ncu figures of the closest-hit traversal kernel on mesh_scene (960x540, a 16-pass wave, pixel-major
# slots, configuration 17; one --set full capture of the timed step's bounces 0 and 1): active lanes
# per issued instruction, the fraction of cycles with an instruction issued, and warps active (of
# the SM's maximum; the register limit allows 0.625).
TRACE_NCU = {"config": 17, "lanes_per_instruction": {"bounce0": 17.5, "bounce1": 9.4}, "issue_active": [0.756, 0.710],
             "warps_active": [0.618, 0.578]}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    from dfpt.kernel import RendererKernel
    from dfpt import _lib as dlib
    from dfpt import workloads

    def l2_reset():
        # Persisting L2 lines survive a plain flush: return them to normal too.
        dlib.check(dlib.load().dfpt_l2_reset())

    t_build = time.perf_counter()
    scene, sky, pstruct, (w, h), meta, source = build_workload(args.workload, args.width, args.height)
    params = workloads.params_to_dict(pstruct)
    t_build = time.perf_counter() - t_build
    k = RendererKernel(scene, sky, params)
    k.update(w, h)
    k.set_seed(0x5EED0000 + rank)
    stream = torch.cuda.Stream()
    k.set_stream(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    n_pix = w * h

    # Warm-up (graphs built here), then the launch configuration is autotuned on this scene
    # (outside the timed region): passes per wave, primitive culling, L2 residency, traversal kernel.
    S = args.spp_per_step
    k.execute(S)
    k.synchronize()
    from dfpt.autotune import tune_trace, tune_wide

    if args.wide > 0:
        k.set_tuning("wide_samples", args.wide)
        if args.shadow_defer >= 0:
            k.set_tuning("shadow_defer", args.shadow_defer)
        wide = {"best": args.wide, "ms_per_step": {}, "shadow_defer": k.get_tuning("shadow_defer")}
    else:
        wide = tune_wide(k, passes=S)
    if args.trace_config >= 0:
        k.set_tuning("trace_config", args.trace_config)
        tuning = {"best": args.trace_config, "ms_per_pass": {}}
    else:
        tuning = tune_trace(k, passes=S, warmup=1)
    for kv in args.set_tuning:
        key, val = kv.split("=", 1)
        k.set_tuning(key, int(val))
    for _ in range(args.warmup):
        k.execute(S)
    k.synchronize()

    # Timed region: one dfpt_render call of S passes per step (waves of wide passes + the last
    # pass, replayed graphs), per-step events on the handle's stream, L2 flushed between steps.
    sampler = ClockSampler(local)
    launches0 = k.launch_count()
    barrier()
    sampler.start()
    step_ms = []
    torch.cuda.nvtx.range_push("timed_steps")  # lets a profiler take the timed steps' kernels alone
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            l2_reset()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        k.execute(S)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    torch.cuda.nvtx.range_pop()
    barrier()
    clocks = sampler.stop()
    launches = k.launch_count() - launches0
    total_s = sum(step_ms) / 1e3
    if dist is not None:
        t = torch.tensor([total_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())
    value = world * n_pix * S * args.steps / total_s / 1e6

    # The same steps with an event between kernels (direct launches): per-kernel times, and the
    # closest-hit traversal time for the roofline.
    k.set_profiling(True)
    trace_ms, trace_n, kind_ms, prof_ms = 0.0, 0, {}, []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            l2_reset()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        k.execute(S)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        prof_ms.append(e0.elapsed_time(e1))
        prof = k.read_profile()
        trace_ms += prof["trace"][0]
        trace_n += prof["trace"][1]
        for kk, (ms, n) in prof.items():
            a = kind_ms.setdefault(kk, [0.0, 0])
            a[0] += ms
            a[1] += n
    k.set_profiling(False)

    # Traversal counters over one extra step (not timed): segments per step.
    k.set_counting(True)
    k.execute(S)
    k.synchronize()
    cnt = k.counters().astype(float)
    k.set_counting(False)

    # End to end through the C-ABI with host buffers (camera in, BGRA8 out), the render loop of
    # DayflowerApplication.java:832-877.
    cam = torch.from_numpy(np.ascontiguousarray(scene.camera.copy())).pin_memory().numpy()
    host_img = torch.empty(n_pix * 4, dtype=torch.uint8).pin_memory().numpy()  # pinned host buffers
    # Untimed warm-up steps: the counting step above changed the pass graphs, which are rebuilt here.
    for _ in range(args.warmup):
        k.update_camera(cam)
        k.execute(S)
        k.get(host_img)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        k.update_camera(cam)
        k.execute(S)
        k.get(host_img)
    barrier()
    e2e_s = time.perf_counter() - t0
    # The interactive loop: one pass per call, as many frames as one step has passes (the tail
    # launch for one-pass calls picked first, outside the timed frames).
    from dfpt.autotune import tune_frame

    main_config = k.get_tuning("trace_config")
    frame_tuning = tune_frame(k, configs=tuple(dict.fromkeys((main_config, 16, 17))))
    k_pixel_tiles = k.get_tuning("pixel_tiles")
    fl_s = frame_loop(k, cam, host_img, S, max(3, args.warmup), barrier)
    fl_kernels = frame_kernels(k)
    if dist is not None:
        t = torch.tensor([e2e_s, fl_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s, fl_s = (float(v) for v in t.tolist())
    e2e_value = world * n_pix * S * args.steps / e2e_s / 1e6
    fl_value = world * n_pix * S / fl_s / 1e6
    # The main handle's waves (up to 64 passes of 1080p with every bounce's shadow rays queued)
    # hold most of the device memory: release it before the other legs create their handles.
    k.dispose()
    del flush
    l2_peak, l2_sizes = l2_read_peak(torch, stream)

    batched = None
    if not args.no_batch:
        batched = batch_leg(args, stream, torch, barrier, dist, world)
    adjoint = None
    if not args.no_adjoint:
        adjoint = adjoint_leg(args, torch, barrier, dist, world)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(scene, sky, pstruct, w, h, args.cpu_seconds)

    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm = peaks.get("hbm_gbs")
    hbm_note = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    closest_segments = cnt[0]
    # Visits per closest-hit segment, the timed kernel's work: the GPU's own counters over a step.
    # Without primitive culling they equal the reference algorithm's (the CPU restatement's counts
    # on its sample are reported beside them); with culling the GPU skips primitives the reference
    # tests, and the roofline counts only the work done.
    nodes_per_seg = cnt[4] / max(cnt[0], 1)
    tris_per_seg = cnt[5] / max(cnt[0], 1)
    bytes_per_seg = nodes_per_seg * 32 + tris_per_seg * 48 + 64
    oracle_bytes_per_seg = (cpu["closest_nodes_per_segment"] * 32 + cpu["closest_tris_per_segment"] * 48 + 64) if cpu else None
    # Closest-hit segments of one step (counters over a step) x algorithmic bytes per segment,
    # over the closest-hit traversal time of a step (events inside the profiled loop).
    avg_trace_ms = trace_ms / max(trace_n, 1)
    trace_ms_per_step = trace_ms / args.steps
    launches_per_step = max(trace_n / args.steps, 1)
    achieved = closest_segments * bytes_per_seg / (trace_ms_per_step / 1e3) / 1e9
    # DRAM bytes per launch: ncu's dram__bytes_read.sum + dram__bytes_write.sum per closest-hit
    # segment of the mesh_scene traversal at 960x540 (one ncu capture), scaled by this run's
    # segments per launch (the traffic grows with the rays of a launch).
    traffic = None
    if args.workload == "mesh_scene" and TRACE_DRAM_BYTES_PER_SEGMENT:
        traffic = TRACE_DRAM_BYTES_PER_SEGMENT * closest_segments / launches_per_step
    dram_gbs = traffic / (avg_trace_ms / 1e3) / 1e9 if traffic else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_s / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": workload_config(args.workload, w, h, scene, pstruct, world),
        "step": {"passes": S, "spp_total": S * args.steps, "samples": n_pix * S,
                 "l2": "flushed between steps (256 MiB write)"},
        "tuning": {"wide_samples": wide["best"], "wide_ms_per_step": wide["ms_per_step"],
                   "ray_sort": wide.get("ray_sort"), "sort_ms_per_step": wide.get("sort_ms_per_step"),
                   "shadow_defer": wide.get("shadow_defer"), "defer_ms_per_step": wide.get("defer_ms_per_step"),
                   "trace_config": tuning["best"], "primitive_culling": tuning.get("primitive_culling", 0),
                   "l2_persist": tuning.get("l2_persist", 0),
                   "l2_ms_per_pass": {str(kk): round(v, 3) for kk, v in tuning.get("l2_ms_per_pass", {}).items()},
                   "culling_ms_per_pass": {str(kk): round(v, 3) for kk, v in tuning.get("culling_ms_per_pass", {}).items()},
                   "trace_config_ms": {str(kk): round(v, 3) for kk, v in tuning["ms_per_pass"].items()},
                   "set_tuning": args.set_tuning},
        "workload_source": source, "scene_build_s": round(t_build, 1),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 19 * 4, "d2h_bytes_per_step": n_pix * 4,
                "loop": "dfpt_set_camera(pinned host) + dfpt_render(S passes) + dfpt_read_bgra8(pinned host) per step"},
        "frame_loop": {"value": fl_value, "unit": UNIT, "frames": S, "ms_per_frame": fl_s / S * 1e3,
                       "fraction_of_value": fl_value / value, "tail_bounce": frame_tuning["tail_bounce"],
                       "tail_ms_per_frame": {str(t): round(v, 3) for t, v in frame_tuning["ms_per_frame"].items()},
                       "trace_config": frame_tuning["trace_config"],
                       "config_ms_per_frame": {str(c): round(v, 3) for c, v in frame_tuning["config_ms_per_frame"].items()},
                       "tail_blocks": frame_tuning["tail_blocks"],
                       "tail_blocks_ms_per_frame": {str(t): round(v, 3) for t, v in frame_tuning["tail_blocks_ms_per_frame"].items()},
                       "shadow_sort": frame_tuning["pass_shadow_sort"],
                       "shadow_sort_ms_per_frame": {str(t): round(v, 3) for t, v in frame_tuning["shadow_sort_ms_per_frame"].items()},
                       "ray_sort": frame_tuning["pass_ray_sort"],
                       "ray_sort_ms_per_frame": {str(t): round(v, 3) for t, v in frame_tuning["ray_sort_ms_per_frame"].items()},
                       "pixel_tiles": k_pixel_tiles, "kernels_ms_per_frame": fl_kernels,
                       "loop": "per frame: dfpt_set_camera(pinned host) + dfpt_render(1 pass) + dfpt_read_bgra8(pinned host), "
                               "as DayflowerApplication's execute/get loop"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "l2", "achieved": achieved, "peak": l2_peak, "unit": "GB/s", "frac": achieved / l2_peak,
                     "traffic": traffic,
                     "peak_source": "measured in this run: L2-resident 16-byte ld.global.cg read stream "
                                    "(dfpt_probe_read_bandwidth, best of 24/48/64 MiB buffers)",
                     "peak_by_buffer_mib": l2_sizes,
                     "kernel": "k_trace<closest>", "avg_launch_ms": avg_trace_ms,
                     "note": "algorithmic bytes = node and triangle records per closest-hit segment; the records are "
                             "L2-resident, so the roof is L2 read bandwidth; DRAM carries the rays (traffic)",
                     "hbm": {"peak": hbm, "peak_source": hbm_note, "dram_gbs": dram_gbs,
                             "dram_frac": dram_gbs / hbm if dram_gbs else None,
                             "algorithmic_frac": achieved / hbm},
                     "ncu": TRACE_NCU,
                     "bytes_per_segment": bytes_per_seg, "oracle_bytes_per_segment": oracle_bytes_per_seg,
                     "nodes_per_segment": nodes_per_seg, "triangles_per_segment": tris_per_seg,
                     "segments_per_launch": closest_segments / launches_per_step,
                     "segments_per_step": closest_segments},
        "kernels_ms_per_step": {kk: round(v[0] / args.steps, 4) for kk, v in kind_ms.items() if v[1]},
        "ms_per_step_profiled": sum(prof_ms) / len(prof_ms),
        "clocks": clocks,
    }
    if cpu:
        line["cpu_baseline"] = {k2: cpu[k2] for k2 in ("value", "unit", "cores", "kind", "sample")}
    if batched:
        line["batched"] = batched
    if adjoint:
        line["adjoint"] = adjoint
    line["rays_per_s"] = (cnt[0] + cnt[1]) * world / (total_s / args.steps)  # segments of one step / step time
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
