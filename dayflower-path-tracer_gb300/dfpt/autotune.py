"""Launch-configuration autotuner for the traversal kernels.

Every traversal configuration (walk variant x block size x resident blocks per SM, see
TRACE_CONFIGS in csrc/dfpt_kernels.cuh) visits the same BVH nodes in the same order, so the choice
only changes speed. The tuner times a few passes of the handle's own scene per configuration with
CUDA events on the handle's stream and keeps the fastest.
"""
from __future__ import annotations

import time


def tune_trace(kernel, passes: int = 4, warmup: int = 1, verbose: bool = False) -> dict:
    """Times each configuration on `kernel` (a RendererKernel after update()); sets the best one."""
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
    return {"best": best, "ms_per_pass": results}
