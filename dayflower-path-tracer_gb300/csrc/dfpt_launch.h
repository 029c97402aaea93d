// dfpt_launch.h - the interface between the host API and a compiled kernel set.
#pragma once

#include <cuda_runtime.h>

#include "dfpt_device_types.h"

// Traversal configuration a handle or batch starts with (the compact pair walk).
#define DFPT_DEFAULT_TRACE_CONFIG 16

struct LaunchCtx {
    const DevScene* scene;
    const DevParams* params;  // device pointer
    const DevPass* pass;
    cudaStream_t stream;
    int grid, grid_trace, grid_simple;
    int trace_config;  // index into the kernel set's traversal configurations
    const DevBatch* batch = nullptr;  // batch launches only
    int tail_blocks = 2;              // resident blocks per SM the tail kernel is compiled for (2-4)
};

struct KernelSet {
    void (*camera)(const LaunchCtx&);
    void (*trace_closest)(const LaunchCtx&, int bounce);
    void (*shade)(const LaunchCtx&, int bounce);
    void (*shadow)(const LaunchCtx&, int bounce);
    void (*final_)(const LaunchCtx&, int bounce);
    void (*tail)(const LaunchCtx&, int first_bounce, int bounces) = nullptr;  // bounces first .. bounces-1 + the final any-hit
    void (*simple)(const LaunchCtx&);
    void (*wireframe)(const LaunchCtx&);
    void (*film)(const LaunchCtx&);
    void (*end_pass)(const LaunchCtx&);
    int (*sort_shadow)(const LaunchCtx&, const DevPass& to) = nullptr;  // plain passes: bins the deferred shadow rays
    int (*sort_rays)(const LaunchCtx&, int bounce, const DevPass& to) = nullptr;  // plain passes: bins a bounce's rays
    void (*film_mean)(const LaunchCtx&, double* out3);
    void (*film_average)(const LaunchCtx&, float* rgb, int* samples);
    void (*init_tables)(cudaStream_t, const int* perm256, const float* grad36);
    void (*occupancy)(int sms, int& grid, int& grid_trace, int& grid_simple);
    int (*trace_grid)(int config, int sms);
    // Shared-memory carveout preference (percent of the maximum, -1 the driver's choice) of the
    // closest-hit traversal kernels of one configuration.
    void (*trace_carveout)(int config, int percent);
    int trace_configs;
    // Batch stages (the fast kernel set only; null elsewhere). The int is the bounce where it applies.
    void (*b_camera)(const LaunchCtx&, int) = nullptr;
    void (*b_trace_closest)(const LaunchCtx&, int) = nullptr;
    void (*b_shade)(const LaunchCtx&, int) = nullptr;
    void (*b_shadow)(const LaunchCtx&, int) = nullptr;
    void (*b_final)(const LaunchCtx&, int) = nullptr;
    void (*b_wave)(const LaunchCtx&, int) = nullptr;
    void (*b_film)(const LaunchCtx&, int) = nullptr;
    void (*b_resolve)(const LaunchCtx&, int) = nullptr;
    void (*b_end)(const LaunchCtx&, int) = nullptr;
    int (*b_sort)(const LaunchCtx&, int bounce, bool counted) = nullptr;  // ray binning (sorted queues); kernels launched
    int (*b_sort_shadow)(const LaunchCtx&, const DevPass& to) = nullptr;   // shadow-ray binning into to.s_*
    void (*b_shadow_reset)(const LaunchCtx&, int) = nullptr;               // empties the shadow queue
    // Path-replay adjoint (the fast kernel set only).
    void (*shade_adj)(const LaunchCtx&, int bounce) = nullptr;
    void (*final_adj)(const LaunchCtx&, int bounce) = nullptr;
    void (*b_shade_adj)(const LaunchCtx&, int bounce) = nullptr;  // the replay in waves (one scene)
    void (*b_final_adj)(const LaunchCtx&, int bounce) = nullptr;
    void (*diff_reduce)(const LaunchCtx&, const double* rows, int n_rows, int row_len, double* out) = nullptr;
};

namespace dfpt_fast { KernelSet kernel_set(); }
namespace dfpt_strict { KernelSet kernel_set(); }
namespace dfpt_wide { KernelSet kernel_set(); }  // batch stages over one scene (waves of passes)
