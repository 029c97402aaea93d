/*
 * dfpt.h - C-ABI of the GB300 renderer core.
 *
 * The core replaces Aparapi's Kernel.execute/put/get for Dayflower's renderer kernel
 * (src/main/java/org/dayflower/pathtracer/kernel/GPURendererKernel.java) and keeps its data
 * contract: the compiled-scene float/int arrays produced by SceneCompiler
 * (src/main/java/org/dayflower/pathtracer/scene/compiler/SceneCompiler.java:79-188) are passed
 * in unchanged, as plain pointers and element counts, and uploaded to the device once.
 *
 * Conventions
 *  - Every entry point returns DFPT_OK (0) or a negative DFPT_ERR_* code; dfpt_last_error()
 *    returns a message for the last failure on the calling thread.
 *  - All buffers are host memory owned by the caller unless the name says "device".
 *  - A handle is not thread-safe; use one handle per host thread / CUDA stream.
 *  - Offsets inside the scene arrays are element offsets, exactly as the reference writes them.
 */
#ifndef DFPT_H
#define DFPT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DFPT_OK 0
#define DFPT_ERR_INVALID_ARGUMENT (-1)  /* IllegalArgumentException in the reference */
#define DFPT_ERR_CUDA (-2)
#define DFPT_ERR_OUT_OF_MEMORY (-3)
#define DFPT_ERR_INVALID_SCENE (-4)     /* offsets that point outside their arrays */
#define DFPT_ERR_TIMEOUT (-5)           /* a bounded device-side wait gave up */
#define DFPT_ERR_NOT_SUPPORTED (-6)

/* Renderer, tone mapper and shader enums: AbstractRendererKernel.java:40-105. */
#define DFPT_RENDERER_AMBIENT_OCCLUSION 1
#define DFPT_RENDERER_PATH_TRACER 2
#define DFPT_RENDERER_RAY_CASTER 3
#define DFPT_RENDERER_RAY_MARCHER 4
#define DFPT_RENDERER_RAY_TRACER 5
#define DFPT_RENDERER_SURFACE_NORMALS 6
#define DFPT_SHADER_FLAT 1
#define DFPT_SHADER_GOURAUD 2
#define DFPT_TONE_MAPPER_FILMIC_CURVE_ACES_MODIFIED 1
#define DFPT_TONE_MAPPER_REINHARD 2
#define DFPT_TONE_MAPPER_REINHARD_MODIFIED_1 3
#define DFPT_TONE_MAPPER_REINHARD_MODIFIED_2 4

/* Random number streams. DFPT_RNG_COUNTER is the counter-based Philox4x32-10 stream keyed by
 * (seed, pixel) and counted by (pass, bounce, slot); DFPT_RNG_LCG is the reference's per-pixel
 * 48-bit LCG (AbstractKernel.java:1101-1110) seeded from dfpt_params.seed. */
#define DFPT_RNG_COUNTER 0
#define DFPT_RNG_LCG 1

/* The 14 compiled-scene arrays plus the camera, as CompiledScene holds them
 * (CompiledScene.java:55-71). Counts are element counts (floats or ints), not bytes. */
typedef struct dfpt_scene_desc {
    const float* point2fs;                    int64_t point2fs_count;
    const float* point3fs;                    int64_t point3fs_count;
    const float* vector3fs;                   int64_t vector3fs_count;
    const int32_t* planes;                    int64_t planes_count;
    const float* spheres;                     int64_t spheres_count;
    const float* terrains;                    int64_t terrains_count;
    const int32_t* triangles;                 int64_t triangles_count;
    const int32_t* bounding_volume_hierarchies; int64_t bounding_volume_hierarchies_count;
    const float* textures;                    int64_t textures_count;
    const float* surfaces;                    int64_t surfaces_count;
    const int32_t* primitives;                int64_t primitives_count;
    const float* primitives_object_to_world;  int64_t primitives_object_to_world_count;
    const float* primitives_world_to_object;  int64_t primitives_world_to_object_count;
    const float* camera;                      int64_t camera_count; /* 19 floats, Camera.java:87-222 */
    /* Optional per-primitive extension records: 4 floats per primitive {Phong exponent, emission
     * scale r, g, b}; NULL and 0 when absent (a zero-initialised descriptor has none). They have no
     * counterpart in the compiled arrays: PhongMaterial's exponent is dropped by the compiler
     * (PhongMaterial.java:39-58, SceneCompiler.java:760-768; the kernel uses 50, GRK:3524) and
     * colours are packed to 8 bits clamped to [0, 1] (ConstantTexture.java:150-155). The path tracer
     * (and its adjoint) uses a primitive's exponent for its Phong lobe and multiplies its emission
     * texture's colour by the scale (HDR emitters). Absent: exponent 50, scale 1. Exponents must be
     * finite and in [0, 1e6], scales finite and >= 0. */
    const float* primitive_extensions;        int64_t primitive_extensions_count;
} dfpt_scene_desc;

/* Sun and sky state: the scalars and arrays GPURendererKernel copies from Sky
 * (GPURendererKernel.java:201-233, Sky.java:295-333). */
typedef struct dfpt_sky {
    double perez_relative_luminance[5];
    double perez_x[5];
    double perez_y[5];
    double zenith_relative_luminance;
    double zenith_x;
    double zenith_y;
    float theta;
    float orthonormal_basis_u[3];
    float orthonormal_basis_v[3];
    float orthonormal_basis_w[3];
    float sun_direction[3];        /* sun direction in the sky basis */
    float sun_direction_world[3];
    float sun_origin[3];
    int32_t is_sky_active;
    int32_t is_sun_active;
} dfpt_sky;

/* The renderer knobs of AbstractRendererKernel (setters at AbstractRendererKernel.java:383-580)
 * and the global noise knobs of AbstractKernel (AbstractKernel.java:250-288). */
typedef struct dfpt_params {
    int32_t renderer_type;
    int32_t tone_mapper_type;
    int32_t shader_type;
    int32_t normal_mapping;             /* BOOLEAN_TRUE/FALSE */
    int32_t wireframes;                 /* BOOLEAN_TRUE/FALSE */
    int32_t pt_ray_depth_maximum;
    int32_t pt_ray_depth_russian_roulette;
    float tone_mapper_exposure;
    float ao_maximum_distance;
    float global_amplitude;
    float global_frequency;
    float global_gain;
    float global_lacunarity;
    int32_t global_octaves;
    int32_t selected_primitive_offset;  /* -1 = no selection */
    int32_t rng_kind;                   /* DFPT_RNG_* */
    uint64_t seed;
} dfpt_params;

typedef struct dfpt_handle dfpt_handle;

/* Defaults of AbstractRendererKernel's constructor (AbstractRendererKernel.java:171-184). */
void dfpt_params_default(dfpt_params* params);

/* Replaces new GPURendererKernel(sceneLoader) + update(w, h, bytes, localSize) + the 19 put()
 * calls of GPURendererKernel.update (GPURendererKernel.java:166-234, 411-449): validates the
 * arrays, uploads them once and allocates the film for width x height pixels.
 * Returns DFPT_ERR_INVALID_ARGUMENT for non-positive sizes (AbstractImageKernel.java:146-148). */
int dfpt_create(const dfpt_scene_desc* scene, const dfpt_sky* sky, int32_t width, int32_t height,
                dfpt_handle** out_handle);

/* Replaces Kernel.dispose (DayflowerApplication.java:502). */
int dfpt_destroy(dfpt_handle* handle);

/* Issues all device work of the handle on this CUDA stream (a cudaStream_t); 0 = legacy stream. */
int dfpt_set_stream(dfpt_handle* handle, void* cuda_stream);

/* Replaces updateCamera() (GPURendererKernel.java:455-461): uploads the 19-float camera. */
int dfpt_set_camera(dfpt_handle* handle, const float* camera19);

/* Replaces updatePrimitives() (GPURendererKernel.java:467-521): 16 floats per primitive each. */
int dfpt_set_transforms(dfpt_handle* handle, const float* object_to_world,
                        const float* world_to_object, int32_t primitive_count);

/* Replaces togglePrimitiveMaterial()'s put(surfaces) (GPURendererKernel.java:314-342). */
int dfpt_set_surfaces(dfpt_handle* handle, const float* surfaces, int64_t surfaces_count);

/* Replaces updateSunAndSky() and toggleSky/toggleSun (GPURendererKernel.java:375-397, 527-569). */
int dfpt_set_sky(dfpt_handle* handle, const dfpt_sky* sky);

/* Replaces the AbstractRendererKernel setters; takes effect at the next pass. */
int dfpt_set_params(dfpt_handle* handle, const dfpt_params* params);

/* Replaces clear() (AbstractImageKernel.java:119-121): the next pass replaces the film. */
int dfpt_clear(dfpt_handle* handle);

/* Replaces kernel.execute(range) + kernel.clearFilmFlags() (DayflowerApplication.java:853-854):
 * renders `passes` passes of one sample per pixel each, accumulates the film and resolves
 * the BGRA8 image and the primitive-offset buffer. Asynchronous on the handle's stream. */
int dfpt_render(dfpt_handle* handle, int32_t passes);

/* Waits for the handle's stream. */
int dfpt_synchronize(dfpt_handle* handle);

/* Replaces kernel.get(byte[]) (DayflowerApplication.java:855): width*height*4 bytes, B,G,R,A. */
int dfpt_read_bgra8(dfpt_handle* handle, uint8_t* bgra);

/* The film: running-average linear radiance (width*height*3 floats, filmData of
 * AbstractImageKernel.java:333-359) and samples per pixel (filmDataSamples). Either may be NULL. */
int dfpt_read_film(dfpt_handle* handle, float* rgb, int32_t* samples);

/* Mean linear radiance of the film, reduced in FP64 on the device. */
int dfpt_read_film_mean(dfpt_handle* handle, double* mean_rgb3);

/* dfpt_film_mean_noalloc has no counterpart in the reference. It is the allocation-free variant of
 * dfpt_read_film_mean for callers that cannot allocate device memory when they need the mean: a
 * frame loop that must not call cudaMalloc/cudaFree once running (allocation can synchronise the
 * device and stall the loop), or a host whose device memory belongs to another allocator (a
 * JVM-side pool, an engine's frame allocator). The caller passes the film (pixel_count x 3 floats,
 * linear RGB) and the output (3 doubles, the FP64 mean per channel), both in device memory; the
 * result is written asynchronously on `cuda_stream` (a cudaStream_t, NULL = legacy stream).
 * Scratch: a fixed device array of DFPT_NOALLOC_MAX_BLOCKS x 3 doubles (24 KiB) that every GPU
 * which loads this library holds until the process exits. The first call on a device looks up
 * that array's device address (cudaGetSymbolAddress), so make the first call on each device
 * before any stream capture. Every call shares the array: calls that overlap on the GPU race.
 * pixel_count outside 1..DFPT_NOALLOC_MAX_PIXELS returns DFPT_ERR_INVALID_ARGUMENT. */
#define DFPT_NOALLOC_MAX_BLOCKS 1024
#define DFPT_NOALLOC_MAX_PIXELS (1ll << 28)
int dfpt_film_mean_noalloc(const float* device_rgb, int64_t pixel_count, double* device_mean3, void* cuda_stream);

/* Replaces get(primitiveOffsets) of togglePrimitiveSelection (GPURendererKernel.java:351-369). */
int dfpt_read_primitive_offsets(dfpt_handle* handle, int32_t* primitive_offsets);

/* The primary-ray hit record of the last pass (hit record of GPURendererKernel.java:79-94):
 * primitive offset, shape type, shape offset, distance (INFINITY=100000 on a miss) and the
 * world-space shading normal (3 floats per pixel). Any pointer may be NULL. */
int dfpt_read_hits(dfpt_handle* handle, int32_t* primitive_offset, int32_t* shape_type,
                   int32_t* shape_offset, float* distance, float* normal3);

/* Ray-segment counters of the last dfpt_render call: closest-hit segments, any-hit segments,
 * BVH nodes visited and triangles tested (summed over all segments), then the nodes and the
 * triangles of the closest-hit segments alone. */
int dfpt_read_counters(dfpt_handle* handle, uint64_t* counters6);
/* Enables (1) or disables (0, the default) the traversal counters; counting costs atomics. */
int dfpt_set_counting(dfpt_handle* handle, int32_t enabled);

/* Per-kernel timing of the last dfpt_render call: when enabled, passes are issued as direct
 * launches with a CUDA event between kernels (no graph), and dfpt_read_profile returns, per kernel
 * kind (0 camera, 1 trace closest, 2 shade, 3 shadow, 4 final any-hit, 5 per-pixel modes,
 * 6 wireframe, 7 film, 8 end of pass, 9 ray binning), the milliseconds and the launch count. */
int dfpt_set_profiling(dfpt_handle* handle, int32_t enabled);
int dfpt_read_profile(dfpt_handle* handle, double* ms_by_kind10, int32_t* launches_by_kind10);

/* Launch tuning (no reference counterpart; results never depend on it). Keys:
 *   "trace_config"      traversal kernel configuration (walk variant x block size x resident
 *                       blocks per SM, 0..N-1, N readable as "trace_configs"); every configuration
 *                       visits the same nodes in the same order (default 16: the compact pair
 *                       walk for closest hits, the autotuner's usual pick);
 *   "shadow_config"     the configuration of the sun shadow-ray (any-hit) launches; -1 (default)
 *                       the trace_config's (any hit is the same hit-or-miss in every walk order);
 *   "pair_stack"        stack entries of the compact pair walk (1..8, default 8); fewer entries
 *                       take its overflow path more often (same hits; a rejected node may then be
 *                       counted twice by the visit counters);
 *   "trace_carveout"    shared-memory carveout preference of the current configuration's
 *                       closest-hit kernels (percent, -1 the driver's choice; process-wide);
 *   "primitive_culling" 0 the reference's full primitive loop, 1 a padded world-box test per
 *                       primitive, 2 candidates from a BVH over those boxes, tested in primitive
 *                       order (scenes with fewer than 8 bounded primitives always use 0);
 *   "l2_persist"        1 (default) keeps the BVH nodes and triangles L2-persistent through an
 *                       access-policy window on the handle's stream; 0 turns it off;
 *   "wide_samples"      passes per wave when dfpt_render renders several passes (1..64, default
 *                       8; 1 renders pass by pass); the film is the same either way;
 *   "pixel_tiles"       1 (default) runs a plain pass's queue slots over 8 x 4 pixel tiles (a warp's
 *                       primary rays leave a compact block of pixels; width a multiple of 8, height
 *                       of 4, counter-based RNG, path tracer without wireframes), 0 in row order;
 *   "tail_bounce"       t >= 0: a plain pass runs bounces t .. depth-1 and the final any-hit of each
 *                       path in one launch (same steps per path; t = 0 includes the camera rays'
 *                       traversal and shading); -1 (default) a launch per bounce;
 *   "tail_blocks"       2 (default), 3 or 4: resident blocks of 256 threads per SM the tail launch
 *                       is compiled for (fewer registers per thread, more warps) when it walks with
 *                       the compact pair walk (configurations 16 and 17) in the fast kernel set; other
 *                       walks and the strict set use 2;
 *   "pass_shadow_sort"  1 (default): a plain pass bins its deferred sun shadow rays by origin cell
 *                       before their launch (processing order only; a second copy of the shadow
 *                       queue); 0 in queue order;
 *   "pass_ray_sort"     0 (default): a plain pass traces bounce 1's rays in queue order; 3, 6, 9,
 *                       12 or 15: in bins of a 6 x 4 x 4 cube-map direction over an origin grid of
 *                       that many bits (processing order only; a second copy of bounce 1's queue);
 *   "ray_sort"       1 (default) bins rays by direction and origin cell between the bounces of
 *                       wide passes (processing order only);
 *   "shadow_sort"       with ray_sort, 1 (default) also bins the sun shadow rays by origin cell
 *                       before their launch;
 *   "shadow_defer"      0 (default) traces each bounce's sun shadow rays after its shading in wide
 *                       passes; 1 traces all bounces' at once after the last (faster, but the
 *                       shadow queue holds depth x as many rays). */
int dfpt_set_tuning(dfpt_handle* handle, const char* key, int32_t value);
int dfpt_get_tuning(dfpt_handle* handle, const char* key, int32_t* value);

/* Picks the launch structure of one-pass dfpt_render calls - the interactive frame loop of
 * DayflowerApplication (execute() + get() per frame) - for this handle's scene, size and knobs:
 * times `frames` (1..1024) one-pass renders per candidate with CUDA events on the handle's stream
 * and sets the fastest "primitive_culling" (0..2, scenes with enough bounded primitives),
 * "trace_config" (the handle's, 16 or 17), "tail_bounce" (-1..4), "tail_blocks" (2..4) and
 * "pass_shadow_sort". It renders about 45 x (frames + 1) passes, then puts
 * back the film, image, selection buffer, per-pixel random states, primary-hit records, counters
 * and pass counter as they were: only the tuning changes. `ms_per_frame` (may be NULL) receives
 * the chosen structure's device time per frame (0 for the renderers with one kernel per pass,
 * which have nothing to tune). Not during a differentiable forward. Allocates a temporary copy
 * of those buffers (about 80 bytes per pixel). */
int dfpt_tune_frame(dfpt_handle* handle, int32_t frames, float* ms_per_frame);
/* Measurement hook (no reference counterpart): returns every persisting L2 line of this process
 * to normal, as a benchmark's L2 flush between timed steps must. */
int dfpt_l2_reset(void);
/* Measurement hook (no reference counterpart): the read bandwidth, in GB/s, of streaming the
 * caller's device buffer (`bytes`: at least 1 MiB, a multiple of 16; 16-byte aligned) `repeats`
 * times through L2 only (16-byte ld.global.cg loads), timed with CUDA events on `stream` (NULL: the
 * legacy default stream) after one untimed pass that brings it into L2. With a buffer smaller than
 * L2 this is the roof of kernels whose working set is L2-resident, as the closest-hit traversal's
 * BVH and triangle records are. */
int dfpt_probe_read_bandwidth(const void* device_buffer, int64_t bytes, int32_t repeats, void* stream, double* gbs);

/* Number of kernels the handle launched since it was created (for launch accounting). */
int dfpt_launch_count(dfpt_handle* handle, uint64_t* launches);

/* Message of the last failed call on this thread ("" if none). */
const char* dfpt_last_error(void);

/* ---------------------------------------------------------------------------------------------
 * Scene compiler (host only). Restates SceneCompiler.compile (SceneCompiler.java:79-188) and the
 * BVH builder (BoundingVolumeHierarchy.java:118-157, 805-986) so callers without a JVM can build
 * the same arrays. A scene is described by flat records and compiled into a dfpt_compiled. */

#define DFPT_SHAPE_PLANE 1
#define DFPT_SHAPE_SPHERE 2
#define DFPT_SHAPE_TERRAIN 3
#define DFPT_SHAPE_TRIANGLE 4
#define DFPT_SHAPE_TRIANGLE_MESH 5
#define DFPT_MATERIAL_CLEAR_COAT 1
#define DFPT_MATERIAL_GLASS 2
#define DFPT_MATERIAL_LAMBERTIAN 3
#define DFPT_MATERIAL_PHONG 4
#define DFPT_MATERIAL_REFLECTION 5
#define DFPT_TEXTURE_BLEND 1
#define DFPT_TEXTURE_BULLSEYE 2
#define DFPT_TEXTURE_CHECKERBOARD 3
#define DFPT_TEXTURE_CONSTANT 4
#define DFPT_TEXTURE_FBM 5
#define DFPT_TEXTURE_IMAGE 6
#define DFPT_TEXTURE_SURFACE_NORMAL 7
#define DFPT_TEXTURE_UV 8

typedef struct dfpt_scene_builder dfpt_scene_builder;
typedef struct dfpt_compiled dfpt_compiled;

int dfpt_builder_create(dfpt_scene_builder** out_builder);
int dfpt_builder_destroy(dfpt_scene_builder* builder);
/* Adds a texture record exactly as Texture.toArray() lays it out (type, size, ...); Blend
 * textures give the builder indices of their two textures in slots 2 and 3. Returns the index. */
int dfpt_builder_add_texture(dfpt_scene_builder* builder, const float* record, int32_t count);
/* Adds a Surface (Surface.java:33-63); texture arguments are builder texture indices. */
int dfpt_builder_add_surface(dfpt_scene_builder* builder, int32_t material, int32_t albedo,
                             int32_t emission, int32_t normal, float noise_amount, float noise_scale);
/* Adds a shape; params: plane a,b,c (9); sphere position + radius (4); terrain 5 floats. */
int dfpt_builder_add_shape(dfpt_scene_builder* builder, int32_t shape_type, const float* params);
/* Adds a triangle mesh (or a single triangle when triangle_count == 1 and as_mesh == 0).
 * Per vertex: position 3, normal 3, uv 2, tangent 3 (11 floats); indices 3 per triangle. */
int dfpt_builder_add_mesh(dfpt_scene_builder* builder, const float* vertices11, int64_t vertex_count,
                          const int32_t* indices, int64_t triangle_count, int32_t as_mesh);
/* Adds a Primitive with a Transform (position 3, quaternion x,y,z,w 4, scale 3). */
int dfpt_builder_add_primitive(dfpt_scene_builder* builder, int32_t shape, int32_t surface,
                               const float* transform10);
/* Camera: eye, look-at point, field of view X in degrees, resolution, aperture, focal distance,
 * lens (1 thin, 2 fisheye). */
int dfpt_builder_set_camera(dfpt_scene_builder* builder, const float* eye3, const float* look_at3,
                            float field_of_view_x, float resolution_x, float resolution_y,
                            float aperture_radius, float focal_distance, int32_t lens);
/* Compiles; threads <= 0 uses all cores for the BVH sweeps (results do not depend on it). */
int dfpt_builder_compile(dfpt_scene_builder* builder, int32_t threads, dfpt_compiled** out_compiled);
int dfpt_compiled_destroy(dfpt_compiled* compiled);
/* Points desc at the compiled arrays (valid until dfpt_compiled_destroy). */
int dfpt_compiled_describe(const dfpt_compiled* compiled, dfpt_scene_desc* desc);

/* Sky.set(sunDirectionWorld, turbidity) (Sky.java:295-333). */
int dfpt_sky_set(dfpt_sky* sky, const float* sun_direction_world3, float turbidity);

/* ---------------------------------------------------------------------------------------------
 * Differentiable rendering. No counterpart in the reference (its kernel only renders). A forward /
 * backward pair over one handle: dfpt_diff_forward renders `spp` path-traced samples per pixel
 * with per-primitive parameters and a sky given by (turbidity, sun direction) - Sky.set
 * (Sky.java:295-333) - and keeps per sample only the path radiance and its sun-visibility bits;
 * dfpt_diff_backward replays every path from its RNG key (path-replay backpropagation) and
 * returns d(loss)/d(parameters) for a given d(loss)/d(image). Needs the path tracer and the
 * counter-based RNG. Gradients hold Russian roulette's survival probability and the sun shadow
 * rays' visibility fixed (no derivative of shadow boundaries); the Phong exponent's gradient is the
 * score of the lobe density (n+1) cos^n the sample was drawn from. */
typedef struct dfpt_diff_params {
    const float* albedo;         /* 3 per primitive: multiplies the albedo texture color (NULL: 1) */
    const float* emission;       /* 3 per primitive: added to the emission texture color (NULL: 0) */
    const float* phong_exponent; /* 1 per primitive, > -1 (NULL: 50, the reference's constant) */
    float turbidity;             /* Perez turbidity, > 0 */
    float sun_direction[3];      /* world-space sun direction (normalised inside, as Sky.set) */
} dfpt_diff_params;

/* Clears the film, renders spp passes with the parameters (the handle keeps using them until
 * dfpt_diff_end) and, if image_rgb != NULL, writes the film average (3 floats per pixel). */
int dfpt_diff_forward(dfpt_handle* handle, const dfpt_diff_params* params, int32_t spp, float* image_rgb);
/* dloss_dimage: 3 floats per pixel. Outputs (each may be NULL): grad_albedo and grad_emission
 * 3 per primitive, grad_phong_exponent 1 per primitive, grad_sky 4 = d/d(turbidity, sun x, y, z). */
int dfpt_diff_backward(dfpt_handle* handle, const float* dloss_dimage, double* grad_albedo, double* grad_emission,
                       double* grad_phong_exponent, double* grad_sky);
/* Leaves differentiable mode: shading uses the textures alone again; the records are freed. */
int dfpt_diff_end(dfpt_handle* handle);

/* ---------------------------------------------------------------------------------------------
 * Batched rendering. No counterpart in the reference, which renders one scene per
 * GPURendererKernel (one AbstractRendererKernel per DayflowerApplication window). A batch holds
 * many compiled scenes resident at once, each with its own resolution, samples per pixel, camera,
 * sky and dfpt_params (path tracer only, counter-based RNG, no wireframes, one maximum depth for
 * the whole batch). dfpt_batch_render renders every scene to its sample count in waves of
 * `wave_capacity` samples, one launch per stage per wave (a replayed CUDA graph); each scene's
 * film then equals what dfpt_create + dfpt_render(spp) gives for that scene with the same seed. */
typedef struct dfpt_batch dfpt_batch;

int dfpt_batch_create(dfpt_batch** out);
int dfpt_batch_destroy(dfpt_batch* batch);
/* Validates and uploads one scene (the checks of dfpt_create); *index receives its index. */
int dfpt_batch_add(dfpt_batch* batch, const dfpt_scene_desc* scene, const dfpt_sky* sky,
                   const dfpt_params* params, int32_t width, int32_t height, int32_t spp, int32_t* index);
int dfpt_batch_set_stream(dfpt_batch* batch, void* cuda_stream);
/* Keys: "wave_capacity" (path slots per wave, 1024..2^27), "trace_config" (traversal launch
 * configuration, as dfpt_set_tuning), "graphs" (0/1), "ray_sort" (0/1), "shadow_defer" (0: each
 * bounce's sun shadow rays traced before the next bounce; 1: all bounces' in one launch after the
 * last, with a shadow queue of depth x wave_capacity entries). Read-only for get: "trace_configs",
 * "scenes", "total_samples", "depth". */
int dfpt_batch_set_tuning(dfpt_batch* batch, const char* key, int64_t value);
int dfpt_batch_get_tuning(dfpt_batch* batch, const char* key, int64_t* value);
/* Clears every film, renders all samples of all scenes, tone maps the images (asynchronous). */
int dfpt_batch_render(dfpt_batch* batch);
/* Pieces of dfpt_batch_render: zero the films; render the waves covering global samples
 * [first_sample, first_sample + count) (scene-major order); tone map the films. */
int dfpt_batch_clear(dfpt_batch* batch);
int dfpt_batch_render_range(dfpt_batch* batch, int64_t first_sample, int64_t count);
int dfpt_batch_resolve(dfpt_batch* batch);
int dfpt_batch_synchronize(dfpt_batch* batch);
/* One scene's film average (rgb, 3 floats per pixel) and sample counts, as dfpt_read_film. */
int dfpt_batch_read_film(dfpt_batch* batch, int32_t index, float* rgb, int32_t* samples);
int dfpt_batch_read_bgra8(dfpt_batch* batch, int32_t index, uint8_t* bgra);
int dfpt_batch_launch_count(dfpt_batch* batch, uint64_t* launches);

#ifdef __cplusplus
}
#endif

#endif /* DFPT_H */
