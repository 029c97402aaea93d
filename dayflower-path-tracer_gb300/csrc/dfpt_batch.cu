// dfpt_batch.cu - many scenes rendered by one set of launches per wave (C-ABI dfpt_batch_*).
//
// The reference renders one scene per GPURendererKernel; a batch holds many compiled scenes, each
// with its own resolution, sample count, camera, sky and renderer settings, resident in HBM at once.
// All samples of all scenes form one global sequence (scene-major, then sample, then pixel). A wave
// takes `wave_capacity` consecutive samples of it - one path slot each, whatever scenes they belong
// to - and runs the path tracer's stages over them, one launch per stage:
//   wave table -> camera -> [trace closest -> shade -> sun shadow rays] x depth -> final any-hit ->
//   film -> advance
// (with shadow_defer, every bounce's sun shadow rays wait in one queue and go in one launch after
// the final any-hit), captured once as a CUDA graph and replayed per wave. A pixel's samples enter its film in sample
// order, so each scene's film is the one a single-scene handle gives after `spp` passes with the
// same seed (the path tracer's counter-based RNG is keyed by pixel and sample, not by launch).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "dfpt.h"
#include "dfpt_internal.h"
#include "dfpt_launch.h"
#include "dfpt_store.h"

struct dfpt_batch {
    std::vector<std::unique_ptr<SceneStore>> stores;
    std::vector<dfpt_params> params;
    std::vector<dfpt_sky> skies;
    std::vector<DevParams> dev_params;
    std::vector<int> width, height, spp;
    std::vector<long long> sample_begin{0}, film_begin{0};
    int depth = -1;
    bool any_sun = false;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sms = 0;
    KernelSet ks{};
    // Scene tables on the device (rebuilt after dfpt_batch_add).
    bool tables_valid = false;
    DevBuf<DevScene> d_scenes;
    DevBuf<DevParams> d_params, d_run;
    DevBuf<long long> d_sample_begin, d_film_begin, d_wave_base, d_wave_tab;
    DevBuf<int> d_wave_entries;
    // Wave buffers (path slots) and films.
    long long capacity_request = 1ll << 23;
    int capacity = 0;         // slots allocated
    size_t shadow_slots = 0;  // deferred shadow queue entries allocated
    DevBuf<float4> q_o0, q_o1, q_d0, q_d1, s_o, s_d, s_c, throughput, film_sum, film_comp;  // throughput: throughput + radiance records (PSI)
    DevBuf<int4> q_hit, slot_key;
    DevBuf<uint64_t> rng;
    DevBuf<int> pixel_flags, counts, pass_index, film_n;
    DevBuf<unsigned long long> stats;
    DevBuf<uint8_t> bgra;
    DevPass pass{};
    DevBatch Q{};
    LaunchCtx ctx{};
    int trace_config = DFPT_DEFAULT_TRACE_CONFIG;
    bool shadow_defer = false;  // every bounce's sun shadow rays traced in one launch after the last
    bool use_graph = true;
    cudaGraphExec_t graph_exec = nullptr;
    bool graph_valid = false;
    int graph_kernels = 0;
    uint64_t launches = 0;
    long long range_host[4] = {0, 0, 0, -1};  // wave base, range end, pass of sample 0, clear sample
    // Ray binning between bounces and before the shadow launch (same scheme as wide passes).
    bool ray_sort = true;
    DevBuf<int> sort_bins;
    DevBuf<float4> s2_o, s2_d, s2_c;
    DevPass pass_shadow{};
    LaunchCtx ctx_shadow{};
};

namespace {

void batch_release_buffers(dfpt_batch* b) {
    DevBuf<float4>* f4[] = {&b->q_o0, &b->q_o1, &b->q_d0, &b->q_d1, &b->s_o, &b->s_d, &b->s_c, &b->throughput};
    for (auto* x : f4) x->release();
    b->q_hit.release();
    b->slot_key.release();
    b->rng.release();
    b->pixel_flags.release();
    b->s2_o.release(); b->s2_d.release(); b->s2_c.release();
    b->capacity = 0;
    b->shadow_slots = 0;
}

void batch_release(dfpt_batch* b) {
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    b->graph_exec = nullptr;
    for (auto& s : b->stores) s->release();
    b->stores.clear();
    batch_release_buffers(b);
    b->film_sum.release(); b->film_comp.release(); b->film_n.release(); b->bgra.release();
    b->counts.release(); b->pass_index.release(); b->stats.release();
    b->d_scenes.release(); b->d_params.release(); b->d_run.release();
    b->d_sample_begin.release(); b->d_film_begin.release(); b->d_wave_base.release(); b->d_wave_tab.release();
    b->d_wave_entries.release();
    b->sort_bins.release();
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    b->stream = nullptr;
}

long long total_samples(const dfpt_batch* b) { return b->sample_begin.back(); }

// Scene tables, films and wave buffers for the current scene list and wave capacity.
int batch_prepare(dfpt_batch* b) {
    const int n = (int)b->stores.size();
    if (n == 0) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "the batch has no scenes");
    cudaStream_t st = b->stream;
    if (!b->tables_valid) {
        std::vector<DevScene> scenes(n);
        for (int i = 0; i < n; ++i) scenes[i] = b->stores[i]->scene;
        CUDA_TRY(upload(b->d_scenes, scenes, st));
        CUDA_TRY(upload(b->d_params, b->dev_params, st));
        CUDA_TRY(upload(b->d_sample_begin, b->sample_begin, st));
        CUDA_TRY(upload(b->d_film_begin, b->film_begin, st));
        std::vector<DevParams> run(1);
        std::memset(run.data(), 0, sizeof(DevParams));
        CUDA_TRY(upload(b->d_run, run, st));
        b->d_wave_tab.release();
        CUDA_TRY(b->d_wave_tab.alloc(4 * ((size_t)n + 1)));
        if (!b->d_wave_base.p) CUDA_TRY(b->d_wave_base.alloc(4));
        if (!b->d_wave_entries.p) CUDA_TRY(b->d_wave_entries.alloc(1));
        if (!b->counts.p) CUDA_TRY(b->counts.alloc(DFPT_COUNTS_SIZE));
        if (!b->pass_index.p) CUDA_TRY(b->pass_index.alloc(1));
        if (!b->stats.p) CUDA_TRY(b->stats.alloc(6));
        CUDA_TRY(cudaMemsetAsync(b->pass_index.p, 0, sizeof(int), st));
        CUDA_TRY(cudaMemsetAsync(b->stats.p, 0, 6 * sizeof(unsigned long long), st));
        const size_t pixels = (size_t)b->film_begin.back();
        b->film_sum.release(); b->film_comp.release(); b->film_n.release(); b->bgra.release();
        CUDA_TRY(b->film_sum.alloc(pixels));
        CUDA_TRY(b->film_comp.alloc(pixels));
        CUDA_TRY(b->film_n.alloc(pixels));
        CUDA_TRY(b->bgra.alloc(pixels * 4));
        CUDA_TRY(cudaMemsetAsync(b->film_sum.p, 0, pixels * sizeof(float4), st));
        CUDA_TRY(cudaMemsetAsync(b->film_comp.p, 0, pixels * sizeof(float4), st));
        CUDA_TRY(cudaMemsetAsync(b->film_n.p, 0, pixels * sizeof(int), st));
        CUDA_TRY(cudaMemsetAsync(b->bgra.p, 0, pixels * 4, st));
        b->tables_valid = true;
        b->graph_valid = false;
    }
    const long long want = std::min<long long>(b->capacity_request, total_samples(b));
    const int cap = (int)std::max<long long>(want, 1);
    // One bounce of shadow rays (traced before the next bounce), or every bounce's when deferred.
    const size_t shadow = (size_t)cap * (size_t)(b->shadow_defer ? std::max(b->depth, 1) : 1);
    if (cap != b->capacity || shadow != b->shadow_slots) {
        batch_release_buffers(b);
        const size_t c = (size_t)cap;
        CUDA_TRY(b->q_o0.alloc(c)); CUDA_TRY(b->q_o1.alloc(c)); CUDA_TRY(b->q_d0.alloc(c)); CUDA_TRY(b->q_d1.alloc(c));
        CUDA_TRY(b->q_hit.alloc(c)); CUDA_TRY(b->slot_key.alloc(c));
        CUDA_TRY(b->throughput.alloc(2 * c)); CUDA_TRY(b->rng.alloc(c)); CUDA_TRY(b->pixel_flags.alloc(c));
        // Each path leaves at most one sun shadow ray per bounce.
        CUDA_TRY(b->s_o.alloc(shadow)); CUDA_TRY(b->s_d.alloc(shadow)); CUDA_TRY(b->s_c.alloc(shadow));
        b->capacity = cap;
        b->shadow_slots = shadow;
        b->graph_valid = false;
    }
    DevPass& B = b->pass;
    B = DevPass{};
    B.n_pixels = b->capacity;
    B.q_o[0] = b->q_o0.p; B.q_o[1] = b->q_o1.p; B.q_d[0] = b->q_d0.p; B.q_d[1] = b->q_d1.p;
    B.q_hit = b->q_hit.p; B.s_o = b->s_o.p; B.s_d = b->s_d.p; B.s_c = b->s_c.p;
    B.throughput = b->throughput.p; B.radiance = b->throughput.p + 1; B.rng = b->rng.p; B.pixel_flags = b->pixel_flags.p;
    B.counts = b->counts.p; B.stats = b->stats.p; B.pass_index = b->pass_index.p;
    B.film_sum = b->film_sum.p; B.film_comp = b->film_comp.p; B.film_n = b->film_n.p; B.bgra = b->bgra.p;
    B.sorted_queues = (b->ray_sort && b->ks.b_sort) ? 1 : 0;
    if (B.sorted_queues) {
        if (!b->sort_bins.p) {
            // Offsets, then the ray and the shadow-ray counts (zero at rest).
            CUDA_TRY(b->sort_bins.alloc(3 * DFPT_SORT_BINS + DFPT_SORT_CHUNKS));
            CUDA_TRY(cudaMemsetAsync(b->sort_bins.p, 0, (3 * DFPT_SORT_BINS + DFPT_SORT_CHUNKS) * sizeof(int), b->stream));
        }
        if (!b->s2_o.p) {
            CUDA_TRY(b->s2_o.alloc(b->shadow_slots));
            CUDA_TRY(b->s2_d.alloc(b->shadow_slots));
            CUDA_TRY(b->s2_c.alloc(b->shadow_slots));
        }
    }
    B.sort_bins = b->sort_bins.p;
    B.sort_count = b->sort_bins.p ? b->sort_bins.p + DFPT_SORT_BINS : nullptr;
    B.sort_count_shadow = b->sort_bins.p ? b->sort_bins.p + 2 * DFPT_SORT_BINS : nullptr;
    B.sort_partials = b->sort_bins.p ? b->sort_bins.p + 3 * DFPT_SORT_BINS : nullptr;
    b->pass_shadow = B;
    if (B.sorted_queues) {
        b->pass_shadow.s_o = b->s2_o.p;
        b->pass_shadow.s_d = b->s2_d.p;
        b->pass_shadow.s_c = b->s2_c.p;
    }
    DevBatch& Q = b->Q;
    Q.scenes = b->d_scenes.p;
    Q.params = b->d_params.p;
    Q.sample_begin = b->d_sample_begin.p;
    Q.film_begin = b->d_film_begin.p;
    Q.n_scenes = n;
    Q.capacity = b->capacity;
    Q.total = total_samples(b);
    Q.wave_base = b->d_wave_base.p;
    Q.slot_key = b->slot_key.p;
    Q.wave_tab = b->d_wave_tab.p;
    Q.wave_entries = b->d_wave_entries.p;
    LaunchCtx& c = b->ctx;
    c.scene = nullptr;
    c.params = b->d_run.p;
    c.pass = &b->pass;
    c.batch = &b->Q;
    c.stream = b->stream;
    b->ks.occupancy(b->sms, c.grid, c.grid_trace, c.grid_simple);
    c.trace_config = b->trace_config;
    c.grid_trace = b->ks.trace_grid(b->trace_config, b->sms);
    b->ctx_shadow = c;
    b->ctx_shadow.pass = &b->pass_shadow;
    return DFPT_OK;
}

// One wave on the batch stream; returns the number of kernels launched.
int issue_wave(dfpt_batch* b) {
    const KernelSet& K = b->ks;
    const LaunchCtx& c = b->ctx;
    int k = 0;
    cudaMemsetAsync(b->counts.p, 0, DFPT_COUNTS_SIZE * sizeof(int), b->stream);
    K.b_wave(c, 0); ++k;
    K.b_camera(c, 0); ++k;
    // Sun shadow rays: after each bounce's shading, or (shadow_defer) all bounces' in one launch
    // after the last bounce; they only add to their paths' radiance.
    auto shadows = [&]() {
        if (!b->any_sun) return;
        if (b->pass.sorted_queues) {
            k += K.b_sort_shadow(c, b->pass_shadow);
            K.b_shadow(b->ctx_shadow, 0); ++k;
        } else {
            K.b_shadow(c, 0); ++k;
        }
        K.b_shadow_reset(c, 0); ++k;
    };
    for (int i = 0; i < b->depth; ++i) {
        K.b_trace_closest(c, i); ++k;
        K.b_shade(c, i); ++k;
        if (b->pass.sorted_queues) k += K.b_sort(c, i, true);
        if (!b->shadow_defer) shadows();
    }
    K.b_final(c, b->depth); ++k;
    if (b->shadow_defer) shadows();
    K.b_film(c, 0); ++k;
    K.b_end(c, 0); ++k;
    return k;
}

int batch_graph(dfpt_batch* b) {
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    b->graph_exec = nullptr;
    b->graph_valid = false;
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const int k = issue_wave(b);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return dfpt_fail(DFPT_ERR_CUDA, "batch graph capture failed: %s", cudaGetErrorString(e));
    }
    e = cudaGraphInstantiate(&b->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        b->graph_exec = nullptr;
        return dfpt_fail(DFPT_ERR_CUDA, "batch graph instantiate failed: %s", cudaGetErrorString(e));
    }
    b->graph_kernels = k;
    b->graph_valid = true;
    return DFPT_OK;
}

}  // namespace

extern "C" {

int dfpt_batch_create(dfpt_batch** out) {
    if (!out) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    auto b = std::make_unique<dfpt_batch>();
    b->ks = dfpt_fast::kernel_set();
    if (!b->ks.b_camera) return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "kernel set has no batch stages");
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) {
        (void)cudaGetLastError();
        return dfpt_fail(DFPT_ERR_CUDA, "CUDA device unavailable: %s", cudaGetErrorString(ce));
    }
    b->own_stream = true;
    int r = noise_tables_init(b->ks, b->stream);
    if (r) { batch_release(b.get()); return r; }
    *out = b.release();
    return DFPT_OK;
}

int dfpt_batch_destroy(dfpt_batch* b) {
    if (!b) return DFPT_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    batch_release(b);
    delete b;
    return DFPT_OK;
}

int dfpt_batch_add(dfpt_batch* b, const dfpt_scene_desc* sd, const dfpt_sky* sky, const dfpt_params* p, int32_t width,
                   int32_t height, int32_t spp, int32_t* index) {
    if (!b || !sd || !sky || !p) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (width <= 0 || height <= 0 || (int64_t)width * (int64_t)height > (1ll << 28))
        return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "resolution %d x %d is not supported", width, height);
    if (spp < 1) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "spp %d < 1", spp);
    if (p->renderer_type != DFPT_RENDERER_PATH_TRACER) return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "a batch renders with the path tracer only");
    if (p->rng_kind != DFPT_RNG_COUNTER) return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "a batch keys its samples with the counter-based RNG");
    if (p->wireframes == 1) return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "no wireframe overlay in a batch");
    const int depth = std::min(std::max(p->pt_ray_depth_maximum, 1), DFPT_MAX_DEPTH);
    if (b->depth >= 0 && depth != b->depth)
        return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "every scene of a batch has the same maximum depth (%d, got %d)", b->depth, depth);
    const long long samples = (long long)width * height * spp;
    if (total_samples(b) + samples > (1ll << 50)) return dfpt_fail(DFPT_ERR_NOT_SUPPORTED, "batch too large");
    auto st = std::make_unique<SceneStore>();
    int r = scene_load(sd, *st);
    if (r) return r;
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    r = scene_upload(*st, b->stream);
    if (r) { st->release(); return r; }
    DevParams d;
    dev_params_fill(d, *p, *sky, st->host.camera.data(), width, height);
    b->stores.push_back(std::move(st));
    b->params.push_back(*p);
    b->skies.push_back(*sky);
    b->dev_params.push_back(d);
    b->width.push_back(width);
    b->height.push_back(height);
    b->spp.push_back(spp);
    b->sample_begin.push_back(total_samples(b) + samples);
    b->film_begin.push_back(b->film_begin.back() + (long long)width * height);
    b->depth = depth;
    b->any_sun = b->any_sun || sky->is_sun_active == 1;
    b->tables_valid = false;
    b->graph_valid = false;
    if (index) *index = (int32_t)b->stores.size() - 1;
    return DFPT_OK;
}

int dfpt_batch_set_stream(dfpt_batch* b, void* stream) {
    if (!b) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "batch == NULL");
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    if (b->own_stream) cudaStreamDestroy(b->stream);
    b->own_stream = false;
    b->stream = (cudaStream_t)stream;
    if (!b->stream) {
        CUDA_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
        b->own_stream = true;
    }
    b->ctx.stream = b->stream;
    b->graph_valid = false;
    return DFPT_OK;
}

int dfpt_batch_set_tuning(dfpt_batch* b, const char* key, int64_t value) {
    if (!b || !key) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    const std::string k(key);
    if (k == "wave_capacity") {
        if (value < 1024 || value > (1ll << 27)) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "wave_capacity %lld outside [1024, 2^27]", (long long)value);
        b->capacity_request = value;
    } else if (k == "trace_config") {
        if (value < 0 || value >= b->ks.trace_configs) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "trace_config %lld outside [0, %d)", (long long)value, b->ks.trace_configs);
        b->trace_config = (int)value;
    } else if (k == "graphs") {
        b->use_graph = value != 0;
    } else if (k == "ray_sort") {
        b->ray_sort = value != 0;
    } else if (k == "shadow_defer") {
        b->shadow_defer = value != 0;
    } else {
        return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "unknown tuning key '%s'", key);
    }
    b->graph_valid = false;
    return DFPT_OK;
}

int dfpt_batch_get_tuning(dfpt_batch* b, const char* key, int64_t* value) {
    if (!b || !key || !value) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    const std::string k(key);
    if (k == "wave_capacity") *value = b->capacity_request;
    else if (k == "trace_config") *value = b->trace_config;
    else if (k == "trace_configs") *value = b->ks.trace_configs;
    else if (k == "graphs") *value = b->use_graph ? 1 : 0;
    else if (k == "ray_sort") *value = b->ray_sort ? 1 : 0;
    else if (k == "shadow_defer") *value = b->shadow_defer ? 1 : 0;
    else if (k == "scenes") *value = (int64_t)b->stores.size();
    else if (k == "total_samples") *value = total_samples(b);
    else if (k == "depth") *value = b->depth;
    else return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "unknown tuning key '%s'", key);
    return DFPT_OK;
}

int dfpt_batch_clear(dfpt_batch* b) {
    if (!b) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "batch == NULL");
    int r = batch_prepare(b);
    if (r) return r;
    const size_t pixels = (size_t)b->film_begin.back();
    CUDA_TRY(cudaMemsetAsync(b->film_sum.p, 0, pixels * sizeof(float4), b->stream));
    CUDA_TRY(cudaMemsetAsync(b->film_comp.p, 0, pixels * sizeof(float4), b->stream));
    CUDA_TRY(cudaMemsetAsync(b->film_n.p, 0, pixels * sizeof(int), b->stream));
    return DFPT_OK;
}

int dfpt_batch_render_range(dfpt_batch* b, int64_t first_sample, int64_t count) {
    if (!b) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "batch == NULL");
    int r = batch_prepare(b);
    if (r) return r;
    const long long total = total_samples(b);
    if (first_sample < 0 || count < 0 || first_sample > total) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "sample range outside the batch");
    if (count > total - first_sample) count = total - first_sample;
    if (count == 0) return DFPT_OK;
    b->range_host[0] = first_sample;
    b->range_host[1] = first_sample + count;
    CUDA_TRY(cudaMemcpyAsync(b->d_wave_base.p, b->range_host, 4 * sizeof(long long), cudaMemcpyHostToDevice, b->stream));
    const long long waves = (count + b->capacity - 1) / b->capacity;
    if (b->use_graph) {
        if (!b->graph_valid) {
            r = batch_graph(b);
            if (r) return r;
        }
        for (long long w = 0; w < waves; ++w) {
            CUDA_TRY(cudaGraphLaunch(b->graph_exec, b->stream));
            b->launches += (uint64_t)b->graph_kernels;
        }
    } else {
        for (long long w = 0; w < waves; ++w) b->launches += (uint64_t)issue_wave(b);
        CUDA_TRY(cudaGetLastError());
    }
    return DFPT_OK;
}

int dfpt_batch_resolve(dfpt_batch* b) {
    if (!b) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "batch == NULL");
    int r = batch_prepare(b);
    if (r) return r;
    b->ks.b_resolve(b->ctx, 0);
    b->launches += 1;
    CUDA_TRY(cudaGetLastError());
    return DFPT_OK;
}

int dfpt_batch_render(dfpt_batch* b) {
    int r = dfpt_batch_clear(b);
    if (!r) r = dfpt_batch_render_range(b, 0, total_samples(b));
    if (!r) r = dfpt_batch_resolve(b);
    return r;
}

int dfpt_batch_synchronize(dfpt_batch* b) {
    if (!b) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "batch == NULL");
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    return DFPT_OK;
}

int dfpt_batch_read_film(dfpt_batch* b, int32_t index, float* rgb, int32_t* samples) {
    if (!b || (!rgb && !samples)) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (index < 0 || index >= (int32_t)b->stores.size()) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "scene index %d out of range", index);
    if (!b->tables_valid) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "the batch has not rendered since its last change");
    const size_t n = (size_t)b->width[index] * (size_t)b->height[index];
    const size_t f0 = (size_t)b->film_begin[index];
    std::vector<float4> sum(n);
    std::vector<int> cnt(n);
    CUDA_TRY(cudaMemcpyAsync(sum.data(), b->film_sum.p + f0, n * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(cudaMemcpyAsync(cnt.data(), b->film_n.p + f0, n * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    for (size_t i = 0; i < n; ++i) {
        const float inv = cnt[i] > 0 ? 1.0f / (float)cnt[i] : 0.0f;
        if (rgb) { rgb[3 * i] = sum[i].x * inv; rgb[3 * i + 1] = sum[i].y * inv; rgb[3 * i + 2] = sum[i].z * inv; }
        if (samples) samples[i] = cnt[i];
    }
    return DFPT_OK;
}

int dfpt_batch_read_bgra8(dfpt_batch* b, int32_t index, uint8_t* out) {
    if (!b || !out) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (index < 0 || index >= (int32_t)b->stores.size()) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "scene index %d out of range", index);
    if (!b->tables_valid) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "the batch has not rendered since its last change");
    const size_t n = (size_t)b->width[index] * (size_t)b->height[index];
    CUDA_TRY(cudaMemcpyAsync(out, b->bgra.p + 4 * (size_t)b->film_begin[index], n * 4, cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    return DFPT_OK;
}

int dfpt_batch_launch_count(dfpt_batch* b, uint64_t* launches) {
    if (!b || !launches) return dfpt_fail(DFPT_ERR_INVALID_ARGUMENT, "NULL argument");
    *launches = b->launches;
    return DFPT_OK;
}

}  // extern "C"
