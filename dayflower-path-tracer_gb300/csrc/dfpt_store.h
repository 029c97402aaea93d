// dfpt_store.h - host-side pieces shared by the single-scene handle (dfpt_api.cu) and the batch
// (dfpt_batch.cu): device buffers, the validated compiled scene resident in HBM, and the packing
// of renderer parameters into the device record.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "dfpt.h"
#include "dfpt_device_types.h"
#include "dfpt_internal.h"
#include "dfpt_launch.h"

#define CUDA_TRY(expr)                                                                          \
    do {                                                                                        \
        cudaError_t e_ = (expr);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            (void)cudaGetLastError();                                                           \
            return dfpt_fail(e_ == cudaErrorMemoryAllocation ? DFPT_ERR_OUT_OF_MEMORY : DFPT_ERR_CUDA, \
                             "%s: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__); \
        }                                                                                       \
    } while (0)

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count) {
        n = count;
        return cudaMalloc((void**)&p, (count ? count : 1) * sizeof(T));
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

template <typename T>
cudaError_t upload(DevBuf<T>& b, const std::vector<T>& v, cudaStream_t s) {
    if (!b.p || b.n != v.size()) {
        b.release();
        cudaError_t e = b.alloc(v.size());
        if (e != cudaSuccess) return e;
    }
    return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

// The 14 compiled-scene arrays as the caller passed them (CompiledScene.java:55-71).
struct HostScene {
    std::vector<float> point2fs, point3fs, vector3fs, spheres, terrains, textures, surfaces, o2w, w2o, camera;
    std::vector<int> planes, triangles, bvh, primitives;
    std::vector<float4> prim_ext;  // optional extension records, one per primitive (empty: none)
};

// Traversal records derived from the arrays at upload (16-byte aligned, see build_derived).
struct Derived {
    std::vector<int4> prim_info;
    std::vector<float4> nodes, tris, sphere4, plane_a, plane_n;
    // Primitive culling (see build_culling): BVH nodes, leaf lists, unbounded primitives, boxes.
    std::vector<float4> cull_nodes, prim_box;
    std::vector<int> cull_prims, always;
    int bounded = 0;  // primitives with a world box
    float4 bounds_lo = make_float4(-1.0e4f, -1.0e4f, -1.0e4f, 0), bounds_hi = make_float4(1.0e4f, 1.0e4f, 1.0e4f, 0);
};

// One validated compiled scene: the host copy, its device arrays and the kernel-side view.
struct SceneStore {
    HostScene host;
    Derived derived;  // emptied once uploaded
    DevBuf<float> point2fs, point3fs, vector3fs, spheres, terrains, textures, surfaces, o2w, w2o, camera;
    DevBuf<int> planes, triangles, primitives;
    DevBuf<int4> prim_info;
    DevBuf<float4> trav;  // BVH nodes then triangles, one allocation (one L2 persistence window)
    DevBuf<float4> pairs;  // per node: the children's boxes (pair records, see DevScene::pairs)
    DevBuf<float4> shade_tris;  // per triangle: the vertex values shading reads (see DevScene::shade_tris)
    size_t trav_nodes = 0;  // float4 records of nodes at the start of trav
    DevBuf<float4> sphere4, plane_a, plane_n, prim_ext;
    DevBuf<float4> cull_nodes, prim_box;
    DevBuf<int> cull_prims, always;
    std::vector<float> obj_box;      // object-space bound per primitive (culling rebuilds)
    bool culling_available = false;  // enough bounded primitives for culling to pay
    int culling_wanted = 1;          // 0 none, 1 box test per primitive, 2 BVH candidates
    DevScene scene{};
    void release();
};

// Copies and validates `sd` (every offset the kernels follow) and derives the traversal records.
int scene_load(const dfpt_scene_desc* sd, SceneStore& st);
// Uploads a loaded scene to the device on `s` and fills `st.scene`.
int scene_upload(SceneStore& st, cudaStream_t s);
// Selects the primitive culling mode in st.scene (0 none, 1 box test, 2 BVH candidates; 0 when
// the scene has too few bounded primitives).
void scene_set_culling(SceneStore& st, int mode);
// Rebuilds the culling structure after the world-to-object matrices changed.
int scene_rebuild_culling(SceneStore& st, cudaStream_t s);
int culling_upload(SceneStore& st, const Derived& d, cudaStream_t s);
// Packs parameters, sky and camera into the device record (host-computed tangents and constants).
void dev_params_fill(DevParams& d, const dfpt_params& p, const dfpt_sky& k, const float* camera19, int width, int height);
// Loads the simplex noise tables into the kernel set's device copies.
int noise_tables_init(const KernelSet& ks, cudaStream_t s);
