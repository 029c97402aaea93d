// dfpt_device_types.h - device-side views of the scene, the parameters and the pass buffers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dfpt.h"

// The uploaded scene. The reference's arrays are kept as they are (shading reads them through
// the same element offsets); the traversal reads the derived, 16-byte aligned records below.
struct DevScene {
    const float* point2fs;
    const float* point3fs;
    const float* vector3fs;
    const int* planes;
    const float* spheres;
    const float* terrains;
    const int* triangles;
    const float* textures;
    const float* surfaces;
    const int* primitives;
    const float* o2w;  // 16 floats per primitive, row-major
    const float* w2o;
    const float* camera;
    int primitive_count;
    int textures_count;
    // Derived records.
    const int4* prim_info;  // {shape type, shape offset, surface offset, record index}
    const float4* nodes;    // 2 per BVH node: {min.xyz, next}, {max.xyz, first triangle or -1}
    const float4* tris;     // 3 per triangle: {a.xyz, triangle offset}, {b-a, last-in-leaf}, {c-a, leaf node index}
    const float4* pairs;    // 4 per BVH node, filled for inner nodes N: the boxes of children L = N + 1 and
                            // R = next(L): {L.min.xyz, L.max.x}, {L.max.yz, R.min.xy}, {R.min.z, R.max.xyz},
                            // {L first triangle, R first triangle, R index, 0} (-1 inner, -2 empty leaf)
    int use_pairs;          // 1: every mesh BVH is a full binary tree, so pair records describe the walk;
                            // 2: the same, and no leaf is empty (the compact pair walk's condition)
    int pair_stack;         // entries of the compact pair walk's stack in use (1..8; 8 unless a test lowers it)
    const float4* shade_tris;  // per triangle (triangle offset / 12), the values surface() reads, copied from
                               // point3fs / point2fs / vector3fs: {a.xyz, b.x}, {b.yz, c.xy}, {c.z, uva.xy, uvb.x},
                               // {uvb.y, uvc.xy, na.x}, {na.yz, nb.xy}, {nb.z, nc.xyz}, {tga.xyz, tgb.x},
                               // {tgb.yz, tgc.xy}, {tgc.z, 0, 0, 0}; null when some triangle offset is not a
                               // multiple of 12 (surface() then follows the reference's indices)
    const float4* prim_ext; // per primitive {Phong exponent, emission scale r, g, b}; null when absent
    const float4* sphere4;  // {position.xyz, radius} per sphere record
    const float4* plane_a;  // point A per plane record
    const float4* plane_n;  // surface normal per plane record
    // Primitive culling (scenes with many primitives): a BVH over padded world-space bounds of
    // the bounded primitives, and the unbounded ones (planes, terrains) that every ray tests.
    int use_culling;          // 0: the full primitive loop; 1: the loop with a world-box test per
                              // primitive; 2: the candidates collected from the culling BVH
    const float4* cull_nodes; // 2 per node: {lo.xyz, left child or -(first + 1) for a leaf}, {hi.xyz, right child or count}
    const int* cull_prims;    // leaf primitive lists, ascending within a leaf
    const int* always;        // unbounded primitives, ascending
    int always_count;
    const float4* prim_box;   // 2 per primitive: padded world bounds lo, hi (unbounded: -/+inf)
    float4 bounds_lo, bounds_hi;  // union of the bounded primitives' world boxes (ray binning grid)
};
#define DFPT_CULL_CANDIDATES 16  // candidates a ray collects before falling back to the full loop
#define DFPT_CULL_STACK 32

// Renderer parameters and derived per-scene constants, in device memory (read through __ldg) so
// captured CUDA graphs stay valid when they change.
struct DevParams {
    int renderer_type;
    int tone_mapper_type;
    int shader_type;
    int normal_mapping;
    int wireframes;
    int depth_max;
    int depth_rr;
    float exposure;
    float ao_max_distance;
    float g_amplitude, g_frequency, g_gain, g_lacunarity;
    int g_octaves;
    int selected_primitive_offset;
    int rng_kind;
    uint32_t seed_lo, seed_hi;
    int width, height;
    int record_hits;
    int counting;
    int clear_pass;  // the film is replaced (not averaged) on this pass index
    int pixel_tiles; // plain passes: queue slot i holds a pixel of an 8 x 4 tile (pixel_of_slot)
    // Sky (float copies of the Perez model; den_l is the theta0-only denominator).
    float sky_u[3], sky_v[3], sky_w[3];
    float sun_dir[3], sun_dir_world[3], sun_origin[3];
    float theta;
    int sky_active, sun_active;
    float perez_l[5], perez_x[5], perez_y[5];
    float zenith_l, zenith_x, zenith_y;
    float den_l;        // (1 + l0 e^l1)(1 + l2 e^(l3 theta0) + l4 cos^2 theta0)
    float den_x_a, den_y_a;  // 1 + x0 e^x1, 1 + y0 e^y1
    float cos_theta0;
    // Camera constants computed once on the host with java.lang.Math semantics (double math,
    // rounded to float): tan(fovX/2), tan(-fovY/2) (GPURendererKernel.java:603-605) and the
    // wireframe threshold cos(PI/2/4096) (GPURendererKernel.java:2933-2934).
    float fov_tan_x, fov_tan_y;
    float wire_cos;
    // sRGB redo-gamma constants (RGBColorSpace.SRGB).
    float cs_break, cs_gamma, cs_slope, cs_slope_match, cs_segment;
    // Differentiable rendering (dfpt_diff_*): per-primitive parameters and replay bookkeeping.
    int diff;                     // 1: shading reads the per-primitive parameters below
    int diff_pass0, diff_spp;     // the forward's first pass index and sample count
    const float4* diff_albedo;    // per primitive {r, g, b, 0}: multiplies the albedo texture color
    const float4* diff_emission;  // per primitive: added to the emission texture color
    const float* diff_exponent;   // per primitive Phong exponent (the reference fixes 50)
    const float* diff_sky_tan;    // [DFPT_SKY_FIELDS][4]: d(field)/d(turbidity, sun x, sun y, sun z)
};

// Sky fields the sky and sun code reads, in the order of the tangent table above.
enum {
    SKY_SUN_DIR = 0, SKY_PEREZ_L = 3, SKY_PEREZ_X = 8, SKY_PEREZ_Y = 13, SKY_ZENITH_L = 18, SKY_ZENITH_X = 19,
    SKY_ZENITH_Y = 20, SKY_DEN_L = 21, SKY_DEN_X_A = 22, SKY_DEN_Y_A = 23, SKY_COS_THETA0 = 24, SKY_SUN_ORIGIN = 25,
    SKY_SUN_DIR_WORLD = 28, DFPT_SKY_FIELDS = 31
};
#define DFPT_DIFF_PER_PRIM 7  // gradient entries per primitive: albedo rgb, emission rgb, exponent
#define DFPT_DIFF_GLOBAL 4    // turbidity, sun direction x, y, z

// Wavefront buffers of one handle. Queue entries are SoA float4 records.
// Index of a path's record in DevPass::throughput / DevPass::radiance (2 float4 per path).
#define PSI(i) (2 * (size_t)(i))

struct DevPass {
    int n_pixels;
    float4* q_o[2];       // {origin.xyz, path id}
    float4* q_d[2];       // {direction.xyz, 0}
    int4* q_hit;          // {t bits, primitive index, shape type, shape offset}
    float4* s_o;          // shadow rays {origin.xyz, path id}
    float4* s_d;          // {direction.xyz, 0}
    float4* s_c;          // pending sun contribution {rgb, 0}
    float4* throughput;   // per path, index PSI(path): one 32-byte record holds a path's throughput
    float4* radiance;     // and radiance (radiance = throughput + 1), read and written together
    uint64_t* rng;        // per pixel: LCG state or draw counter
    int* pixel_flags;     // bit 0: film set to black this pass
    float4* primary_o;    // primary rays (wireframe overlay)
    float4* primary_d;
    int* counts;          // [0..31] ray queue counts per bounce, [32] deferred shadow rays, [64..95] work fetch
    unsigned long long* stats;  // closest, any, nodes, triangles
    int* pass_index;      // device pass counter
    // Film (Kahan-compensated sums), image and selection buffers.
    float4* film_sum;
    float4* film_comp;
    int* film_n;
    uint8_t* bgra;
    int* primitive_offsets;
    // Primary hit record (optional).
    int* hit_prim_offset;
    int* hit_shape_type;
    int* hit_shape_offset;
    float* hit_distance;
    float* hit_normal;
    // Differentiable rendering.
    int* vis;                  // per path: bit b = the sun shadow ray of bounce b was unoccluded
    float4* diff_L;            // [sample][pixel] path radiance of the forward's samples
    int* diff_vis;             // [sample][pixel] the forward's visibility bits
    const float4* diff_dldi;   // per pixel dLoss/dImage (rgb)
    double* diff_rows;         // per block of the adjoint kernels: gradient partials
    int diff_row_len;          // primitives x 7 + 4
    // Ray binning between bounces (wide passes): with sorted_queues set, shading writes queue 1,
    // the binning pass moves it to queue 0 in bin order, and every bounce reads queue 0.
    int sorted_queues;
    int* sort_bins;            // DFPT_SORT_BINS exclusive offsets (scan output, scatter cursors)
    int* sort_count;           // DFPT_SORT_BINS ray counts of the next bounce; zero at rest (the scan clears them)
    int* sort_count_shadow;    // the same for the sun shadow rays
    int* sort_partials;        // DFPT_SORT_CHUNKS chunk sums of the scan
    int sort_ray_bits;         // plain passes: origin-grid bits of the bounce rays' bins (plain_ray_bin)
};
// Bins: waves of several scenes use 3 bits of scene (within a wave) x a 6 x 4 x 4 cube-map
// direction bin (7 bits) x 12 bits of origin cell (bounce rays), or 3 bits of scene x 18 bits of
// cell (shadow rays); waves of one scene use a direction bin (DFPT_RAY_DIR_RES) over an origin grid
// of DFPT_RAY_CELL_BITS bits (bounce rays) or a grid of DFPT_SHADOW_CELL_BITS bits (shadow rays),
// multiples of 3 (an equal split over the axes). Every key stays below DFPT_SORT_BINS (2^22 with
// these settings). The scan runs over DFPT_SORT_CHUNKS chunks of 1024 bins.
#ifndef DFPT_RAY_CELL_BITS
#define DFPT_RAY_CELL_BITS 15
#endif
#ifndef DFPT_SHADOW_CELL_BITS
#define DFPT_SHADOW_CELL_BITS 21
#endif
#ifndef DFPT_RAY_DIR_RES
#define DFPT_RAY_DIR_RES 4  // 0: direction octant (3 bits); n: cube-map bins, 6 x n x n directions
#endif
#ifndef DFPT_BATCH_DIR_BINS
#define DFPT_BATCH_DIR_BINS 1  // waves of several scenes: 1 cube-map 6 x 4 x 4 direction bins, 0 the octant
#endif
#define DFPT_RAY_DIR_COUNT (DFPT_RAY_DIR_RES ? 6 * DFPT_RAY_DIR_RES * DFPT_RAY_DIR_RES : 8)
#define DFPT_RAY_DIR_BITS (DFPT_RAY_DIR_COUNT <= 8 ? 3 : DFPT_RAY_DIR_COUNT <= 16 ? 4 : DFPT_RAY_DIR_COUNT <= 32 ? 5 : \
                           DFPT_RAY_DIR_COUNT <= 64 ? 6 : DFPT_RAY_DIR_COUNT <= 128 ? 7 : DFPT_RAY_DIR_COUNT <= 256 ? 8 : 9)
#define DFPT_SORT_BITS (DFPT_RAY_CELL_BITS + DFPT_RAY_DIR_BITS > DFPT_SHADOW_CELL_BITS ? DFPT_RAY_CELL_BITS + DFPT_RAY_DIR_BITS : DFPT_SHADOW_CELL_BITS)
#define DFPT_SORT_BINS (1 << (DFPT_SORT_BITS < 22 ? 22 : DFPT_SORT_BITS))  // several scenes: up to 22 bits
#define DFPT_SORT_CHUNKS (DFPT_SORT_BINS / 1024)

// Many scenes rendered by one set of launches. Every scene's samples form one global sequence
// (scene-major, then sample, then pixel); a wave takes `capacity` consecutive samples of it, one
// path slot each. Queue entries carry their scene in the direction's w.
struct DevBatch {
    const DevScene* scenes;           // [n_scenes]
    const DevParams* params;          // [n_scenes]
    const long long* sample_begin;    // [n_scenes + 1] first global sample of each scene
    const long long* film_begin;      // [n_scenes + 1] first film pixel of each scene
    int n_scenes;
    int capacity;                     // path slots per wave
    long long total;                  // samples of all scenes
    long long* wave_base;             // device: [0] global sample of slot 0 of the current wave,
                                      // [1] end of the sample range being rendered, [2] RNG pass
                                      // index of sample 0, [3] sample whose film update replaces
                                      // the pixel (-1: none), [4] RNG pass whose first hits fill
                                      // the selection buffer (one-scene waves; -1: none)
    int4* slot_key;                   // per slot {scene, pixel, RNG pass index, 0}
    long long* wave_tab;              // per scene in the wave {scene, local begin, local end, film-task prefix}
    int* wave_entries;                // entries in wave_tab
};

#define DFPT_COUNTS_SHADOW 32
#define DFPT_COUNTS_FETCH 64  // [64..95]: work-fetch counters of the traversal launches
#define DFPT_MAX_DEPTH 30
#define DFPT_COUNTS_SIZE 128
