"""Launch-configuration autotuner for the traversal kernels.

Every traversal configuration (walk variant x block size x resident blocks per SM, see
TRACE_CONFIGS in csrc/dfpt_kernels.cuh) visits the same BVH nodes in the same order, so the choice
only changes speed. The tuner times a few passes of the handle's own scene per configuration with
CUDA events on the handle's stream and keeps the fastest.
"""
from __future__ import annotations

import time


def tune_trace(kernel, passes: int = 4, warmup: int = 1, verbose: bool = False) -> dict:
    """Times each configuration on `kernel` (a RendererKernel after update()); sets the best one.
    Scenes with enough bounded primitives first get their primitive-culling mode picked (0 the
    reference's full loop, 1 a world-box test per primitive, 2 candidates from a BVH over the
    boxes; all three give the same hits)."""
    culling = {}
    kernel.set_tuning("primitive_culling", 1)
    if kernel.get_tuning("primitive_culling") == 1:
        for mode in (0, 1, 2):
            kernel.set_tuning("primitive_culling", mode)
            kernel.execute(warmup)
            kernel.synchronize()
            t0 = time.perf_counter()
            kernel.execute(passes)
            kernel.synchronize()
            culling[mode] = (time.perf_counter() - t0) / passes * 1e3
            if verbose:
                print(f"primitive_culling {mode}: {culling[mode]:.3f} ms/pass", flush=True)
        kernel.set_tuning("primitive_culling", min(culling, key=culling.get))
    # L2 residency of the traversal records on or off.
    l2 = {}
    for mode in (1, 0):
        kernel.set_tuning("l2_persist", mode)
        kernel.execute(warmup)
        kernel.synchronize()
        t0 = time.perf_counter()
        kernel.execute(passes)
        kernel.synchronize()
        l2[mode] = (time.perf_counter() - t0) / passes * 1e3
        if verbose:
            print(f"l2_persist {mode}: {l2[mode]:.3f} ms/pass", flush=True)
    kernel.set_tuning("l2_persist", min(l2, key=l2.get))
    n = kernel.get_tuning("trace_configs")
    results = {}
    for cfg in range(n):
        kernel.set_tuning("trace_config", cfg)
        kernel.execute(warmup)
        kernel.synchronize()
        t0 = time.perf_counter()
        kernel.execute(passes)
        kernel.synchronize()
        results[cfg] = (time.perf_counter() - t0) / passes * 1e3
        if verbose:
            print(f"trace_config {cfg}: {results[cfg]:.3f} ms/pass", flush=True)
    best = min(results, key=results.get)
    kernel.set_tuning("trace_config", best)
    out = {"best": best, "ms_per_pass": results, "l2_persist": kernel.get_tuning("l2_persist"), "l2_ms_per_pass": l2}
    if culling:
        out["primitive_culling"] = kernel.get_tuning("primitive_culling")
        out["culling_ms_per_pass"] = culling
    return out


def tune_batch(batch, capacities=(1 << 22, 1 << 23, 1 << 24, 1 << 25, 1 << 26), configs=None, window: int | None = None,
               verbose: bool = False) -> dict:
    """Picks the batch's wave capacity (queue depth) and traversal configuration (block size x
    resident blocks x walk variant) by timing the same window of the batch's own samples with
    each candidate. The walks' stack depth is fixed (the threaded walks keep none; the pair walks
    keep 8 entries and fall back to the threaded records when those run out), so it is not a
    candidate. Leaves the films cleared and the best candidate set."""
    total = batch.total_samples
    if configs is None:
        # The per-lane walks at 4 and 3 blocks per SM, the lane-refill walk and the pair walks: the
        # warp-synchronous walk (4-6) maps to the per-lane walk in a batch, and the 6-8 block
        # configurations (11-14) spill and lose on every workload measured.
        configs = [c for c in (0, 1, 2, 3, 9, 15, 16, 17) if c < batch.get_tuning("trace_configs")]
    results = {}
    # One window of the batch's sample sequence for every candidate, so the rates compare.
    span = int(min(total, window if window is not None else 2 * max(capacities)))
    first = max(0, (total - span) // 2)
    for cap in capacities:
        cap = int(min(cap, total))
        batch.set_tuning("wave_capacity", max(cap, 1024))
        for cfg in configs:
            batch.set_tuning("trace_config", cfg)
            batch.clear()
            batch.render_range(first, min(span, cap))  # warm-up (graph build, caches)
            batch.synchronize()
            t0 = time.perf_counter()
            batch.render_range(first, span)
            batch.synchronize()
            dt = time.perf_counter() - t0
            results[(cap, cfg)] = span / dt / 1e6
            if verbose:
                print(f"wave_capacity {cap} trace_config {cfg}: {results[(cap, cfg)]:.1f} M samples/s", flush=True)
        if cap >= total:
            break
    best = max(results, key=results.get)
    batch.set_tuning("wave_capacity", max(best[0], 1024))
    batch.set_tuning("trace_config", best[1])
    # Ray binning on or off at the best point (results[best] was measured with the default, on).
    sort = {1: results[best]}
    batch.set_tuning("ray_sort", 0)
    batch.clear()
    batch.render_range(first, min(span, best[0]))
    batch.synchronize()
    t0 = time.perf_counter()
    batch.render_range(first, span)
    batch.synchronize()
    sort[0] = span / (time.perf_counter() - t0) / 1e6
    batch.set_tuning("ray_sort", max(sort, key=sort.get))
    # Sun shadow rays per bounce or all bounces' in one launch (the queue then holds depth x as many).
    defer = {0: sort[max(sort, key=sort.get)]}
    batch.set_tuning("shadow_defer", 1)
    batch.clear()
    batch.render_range(first, min(span, best[0]))
    batch.synchronize()
    t0 = time.perf_counter()
    batch.render_range(first, span)
    batch.synchronize()
    defer[1] = span / (time.perf_counter() - t0) / 1e6
    batch.set_tuning("shadow_defer", max(defer, key=defer.get))
    batch.clear()
    return {"best": {"wave_capacity": best[0], "trace_config": best[1], "ray_sort": max(sort, key=sort.get),
                     "shadow_defer": max(defer, key=defer.get)},
            "m_samples_per_s": {f"{k[0]}/{k[1]}": round(v, 2) for k, v in results.items()},
            "ray_sort_m_samples_per_s": {str(k): round(v, 2) for k, v in sort.items()},
            "shadow_defer_m_samples_per_s": {str(k): round(v, 2) for k, v in defer.items()}}


def tune_wide(kernel, passes: int = 16, candidates=(1, 4, 8, 16, 32, 64), verbose: bool = False) -> dict:
    """Picks how many passes run per wave in dfpt_render (1 = one pass at a time) by timing
    `passes` passes per candidate (those up to `passes`) on the handle's own scene; every choice
    gives the same film."""
    results = {}
    for k in [c for c in candidates if c <= max(1, passes)]:
        kernel.set_tuning("wide_samples", k)
        kernel.execute(passes)
        kernel.synchronize()
        t0 = time.perf_counter()
        kernel.execute(passes)
        kernel.synchronize()
        results[k] = (time.perf_counter() - t0) * 1e3
        if verbose:
            print(f"wide_samples {k}: {results[k]:.3f} ms / {passes} passes", flush=True)
    best = min(results, key=results.get)
    kernel.set_tuning("wide_samples", best)
    sort = {}
    if best > 1:
        for mode in (1, 0):
            kernel.set_tuning("ray_sort", mode)
            kernel.execute(passes)
            kernel.synchronize()
            t0 = time.perf_counter()
            kernel.execute(passes)
            kernel.synchronize()
            sort[mode] = (time.perf_counter() - t0) * 1e3
        kernel.set_tuning("ray_sort", min(sort, key=sort.get))
    defer = {}
    if best > 1:
        # One shadow launch per wave needs a queue of depth x the slots: try it where memory allows.
        for mode in (0, 1):
            try:
                kernel.set_tuning("shadow_defer", mode)
                kernel.execute(passes)
                kernel.synchronize()
            except Exception:
                continue
            t0 = time.perf_counter()
            kernel.execute(passes)
            kernel.synchronize()
            defer[mode] = (time.perf_counter() - t0) * 1e3
        kernel.set_tuning("shadow_defer", min(defer, key=defer.get) if defer else 0)
    return {"best": best, "ms_per_step": {str(k): round(v, 3) for k, v in results.items()},
            "ray_sort": kernel.get_tuning("ray_sort"), "sort_ms_per_step": {str(k): round(v, 3) for k, v in sort.items()},
            "shadow_defer": kernel.get_tuning("shadow_defer"), "defer_ms_per_step": {str(k): round(v, 3) for k, v in defer.items()}}


def tune_frame(kernel, frames: int = 16, candidates=(-1, 0, 1, 2, 3, 4), blocks=(2, 3, 4), ray_sort=(0, 9, 12, 15),
               configs=None, culling: bool = False, verbose: bool = False) -> dict:
    """Picks the launch structure of one-pass calls (the interactive frame loop), as dfpt_tune_frame
    does in the C-ABI: with `culling`, first the primitive culling mode (scenes with enough bounded
    primitives; every mode gives the same hits); then times `frames`
    calls of dfpt_render(1) per `tail_bounce` candidate (-1 = a launch per bounce) and per
    `tail_blocks` (resident blocks of the tail kernel) - for each traversal configuration in
    `configs` when given (the primary rays', shadow rays' and tail's walk), else the handle's - and
    sets the fastest, then keeps or
    drops the binning of the shadow rays (`pass_shadow_sort`: its scan has a fixed cost that small
    frames may not earn back), then picks the binning of bounce 1's rays (`pass_ray_sort`: 0 =
    none, else the origin grid's bits) and times the tail candidates once more with it. Every
    choice gives each path the same steps; only the launch structure and the processing order
    change."""
    def frame_ms():
        kernel.execute(1)
        kernel.synchronize()
        t0 = time.perf_counter()
        for _ in range(frames):
            kernel.execute(1)
        kernel.synchronize()
        return (time.perf_counter() - t0) / frames * 1e3

    def sweep_tail():
        table = {}
        for b in blocks:
            kernel.set_tuning("tail_blocks", b)
            for t in candidates:
                if t < 0 and b != blocks[0]:
                    table[(b, t)] = table[(blocks[0], t)]  # no tail launch: the blocks do not matter
                    continue
                kernel.set_tuning("tail_bounce", t)
                table[(b, t)] = frame_ms()
                if verbose:
                    print(f"tail_blocks {b} tail_bounce {t}: {table[(b, t)]:.3f} ms/frame", flush=True)
        b, t = min(table, key=table.get)
        kernel.set_tuning("tail_blocks", b)
        kernel.set_tuning("tail_bounce", t)
        return table, b, t

    cull = {}
    if culling:
        mode0 = kernel.get_tuning("primitive_culling")
        kernel.set_tuning("primitive_culling", 1)
        if kernel.get_tuning("primitive_culling") == 1:
            for mode in (0, 1, 2):
                kernel.set_tuning("primitive_culling", mode)
                cull[mode] = frame_ms()
            kernel.set_tuning("primitive_culling", min(cull, key=cull.get))
        else:
            kernel.set_tuning("primitive_culling", mode0)
    if configs:
        per_config = {}
        for cfg in configs:
            kernel.set_tuning("trace_config", cfg)
            t_cfg, b_cfg, best_cfg = sweep_tail()
            per_config[cfg] = (t_cfg[(b_cfg, best_cfg)], t_cfg, b_cfg, best_cfg)
        cfg = min(per_config, key=lambda c: per_config[c][0])
        kernel.set_tuning("trace_config", cfg)
        _, table, tb_blocks, best = per_config[cfg]
        kernel.set_tuning("tail_blocks", tb_blocks)
        kernel.set_tuning("tail_bounce", best)
    else:
        per_config = {}
        table, tb_blocks, best = sweep_tail()
    sort = {kernel.get_tuning("pass_shadow_sort"): table[(tb_blocks, best)]}
    other = 1 - next(iter(sort))
    kernel.set_tuning("pass_shadow_sort", other)
    sort[other] = frame_ms()
    kernel.set_tuning("pass_shadow_sort", min(sort, key=sort.get))
    rays = {}
    # Bounce 1's rays are binned between bounce 0's shading and their traversal: not with a tail
    # launch that starts at the camera rays.
    for bits in ray_sort if best != 0 else (0,):
        kernel.set_tuning("pass_ray_sort", bits)
        rays[bits] = frame_ms()
        if verbose:
            print(f"pass_ray_sort {bits}: {rays[bits]:.3f} ms/frame", flush=True)
    bits = min(rays, key=rays.get)
    kernel.set_tuning("pass_ray_sort", bits)
    if bits:
        # The tail may start elsewhere once bounce 1's rays arrive in bin order.
        table, tb_blocks, best = sweep_tail()
        if best == 0:
            bits = 0
            kernel.set_tuning("pass_ray_sort", 0)
    return {"primitive_culling": kernel.get_tuning("primitive_culling") if culling else None, "culling_ms_per_frame": cull,
            "trace_config": kernel.get_tuning("trace_config"),
            "config_ms_per_frame": {c: v[0] for c, v in per_config.items()},
            "tail_bounce": best, "tail_blocks": tb_blocks,
            "ms_per_frame": {t: table[(tb_blocks, t)] for t in candidates},
            "tail_blocks_ms_per_frame": {b: min(table[(b, t)] for t in candidates) for b in blocks},
            "pass_shadow_sort": min(sort, key=sort.get), "shadow_sort_ms_per_frame": sort,
            "pass_ray_sort": bits, "ray_sort_ms_per_frame": rays}
