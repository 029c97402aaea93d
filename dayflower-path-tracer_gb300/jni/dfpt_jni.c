/*
 * dfpt_jni.c - the native half of org.dayflower.pathtracer.kernel.CudaRendererKernel: each native
 * method of that class forwards to one or two calls of the C-ABI in dfpt.h.
 *
 * Java arrays are read in place (GetPrimitiveArrayCritical): the core copies what it keeps to the
 * GPU before the call returns, and writes images and offsets straight into the caller's array. No
 * other JNI call is made while an array is held. Every failure of the core becomes a Java
 * exception carrying dfpt_last_error()'s message:
 *   DFPT_ERR_INVALID_ARGUMENT, DFPT_ERR_INVALID_SCENE -> IllegalArgumentException
 *   DFPT_ERR_OUT_OF_MEMORY                           -> OutOfMemoryError
 *   any other code (CUDA error, timeout, unsupported) -> IllegalStateException
 * and a null array throws NullPointerException, as Objects.requireNonNull does in the reference.
 *
 * The jlong handle is a pointer to a jni_kernel: the core's handle plus the parameters last handed
 * to it, so that execute(), which passes the renderer knobs every frame, uploads them only when one
 * changed (dfpt_set_params rebuilds the pass graphs).
 */
#include <jni.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "dfpt.h"

typedef struct jni_kernel {
    dfpt_handle* handle;
    dfpt_params params;
    int64_t pixels;  /* width x height of the film */
} jni_kernel;

static jni_kernel* kernel_of(jlong h) { return (jni_kernel*)(intptr_t)h; }

static void throw_class(JNIEnv* env, const char* cls, const char* msg) {
    jclass c = (*env)->FindClass(env, cls);
    if (c) (*env)->ThrowNew(env, c, msg);
}

/* Throws for a negative return code; returns 1 if it threw. */
static int throw_if(JNIEnv* env, int rc) {
    if (rc >= 0) return 0;
    const char* msg = dfpt_last_error();
    if (rc == DFPT_ERR_INVALID_ARGUMENT || rc == DFPT_ERR_INVALID_SCENE)
        throw_class(env, "java/lang/IllegalArgumentException", msg);
    else if (rc == DFPT_ERR_OUT_OF_MEMORY)
        throw_class(env, "java/lang/OutOfMemoryError", msg);
    else
        throw_class(env, "java/lang/IllegalStateException", msg);
    return 1;
}

static int need_handle(JNIEnv* env, jlong h) {
    if (h != 0 && kernel_of(h)->handle) return 1;
    throw_class(env, "java/lang/IllegalStateException", "the kernel has no scene on the GPU (update() not called, or disposed)");
    return 0;
}

/* Null checks of the arrays a native method takes, before any of them is held. */
static int need_arrays(JNIEnv* env, const jarray* arrays, const char* const* names, int n) {
    for (int i = 0; i < n; ++i) {
        if (!arrays[i]) {
            char msg[96];
            strcpy(msg, names[i]);
            strcat(msg, " == null");
            throw_class(env, "java/lang/NullPointerException", msg);
            return 0;
        }
    }
    return 1;
}

/* dfpt_sky from CudaRendererKernel.skyDoubles (18), skyFloats (19) and the flag bits. */
static int fill_sky(JNIEnv* env, dfpt_sky* sky, jdoubleArray sd, jfloatArray sf, jint flags) {
    if ((*env)->GetArrayLength(env, sd) != 18 || (*env)->GetArrayLength(env, sf) != 19) {
        throw_class(env, "java/lang/IllegalArgumentException", "sky arrays must hold 18 doubles and 19 floats");
        return 0;
    }
    double d[18];
    float f[19];
    (*env)->GetDoubleArrayRegion(env, sd, 0, 18, d);
    (*env)->GetFloatArrayRegion(env, sf, 0, 19, f);
    memset(sky, 0, sizeof(*sky));
    memcpy(sky->perez_relative_luminance, d, 5 * sizeof(double));
    memcpy(sky->perez_x, d + 5, 5 * sizeof(double));
    memcpy(sky->perez_y, d + 10, 5 * sizeof(double));
    sky->zenith_relative_luminance = d[15];
    sky->zenith_x = d[16];
    sky->zenith_y = d[17];
    sky->theta = f[0];
    memcpy(sky->orthonormal_basis_u, f + 1, 3 * sizeof(float));
    memcpy(sky->orthonormal_basis_v, f + 4, 3 * sizeof(float));
    memcpy(sky->orthonormal_basis_w, f + 7, 3 * sizeof(float));
    memcpy(sky->sun_direction, f + 10, 3 * sizeof(float));
    memcpy(sky->sun_direction_world, f + 13, 3 * sizeof(float));
    memcpy(sky->sun_origin, f + 16, 3 * sizeof(float));
    sky->is_sky_active = (flags & 1) ? 1 : 0;
    sky->is_sun_active = (flags & 2) ? 1 : 0;
    return 1;
}

#define SCENE_ARRAYS 14

JNIEXPORT jlong JNICALL Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_nativeCreate(
    JNIEnv* env, jclass cls, jfloatArray point2fs, jfloatArray point3fs, jfloatArray vector3fs, jintArray planes,
    jfloatArray spheres, jfloatArray terrains, jintArray triangles, jintArray bvh, jfloatArray textures,
    jfloatArray surfaces, jintArray primitives, jfloatArray o2w, jfloatArray w2o, jfloatArray camera,
    jdoubleArray sky_d, jfloatArray sky_f, jint sky_flags, jint width, jint height, jlong seed) {
    (void)cls;
    static const char* const names[SCENE_ARRAYS + 2] = {
        "point2Fs", "point3Fs", "vector3Fs", "planes", "spheres", "terrains", "triangles",
        "boundingVolumeHierarchies", "textures", "surfaces", "primitives", "primitivesObjectToWorld",
        "primitivesWorldToObject", "camera", "skyDoubles", "skyFloats"};
    const jarray arrays[SCENE_ARRAYS + 2] = {point2fs, point3fs, vector3fs, planes, spheres, terrains, triangles, bvh,
                                             textures, surfaces, primitives, o2w, w2o, camera, sky_d, sky_f};
    if (!need_arrays(env, arrays, names, SCENE_ARRAYS + 2)) return 0;
    dfpt_sky sky;
    if (!fill_sky(env, &sky, sky_d, sky_f, sky_flags)) return 0;
    jni_kernel* k = (jni_kernel*)calloc(1, sizeof(jni_kernel));
    if (!k) {
        throw_class(env, "java/lang/OutOfMemoryError", "jni_kernel");
        return 0;
    }
    jsize len[SCENE_ARRAYS];
    for (int i = 0; i < SCENE_ARRAYS; ++i) len[i] = (*env)->GetArrayLength(env, arrays[i]);
    /* Held together (nested critical sections); dfpt_create copies them to the GPU and returns. */
    void* p[SCENE_ARRAYS] = {0};
    int held = 0;
    for (; held < SCENE_ARRAYS; ++held) {
        p[held] = (*env)->GetPrimitiveArrayCritical(env, arrays[held], NULL);
        if (!p[held]) break;
    }
    int rc = DFPT_ERR_OUT_OF_MEMORY;
    if (held == SCENE_ARRAYS) {
        dfpt_scene_desc d;
        memset(&d, 0, sizeof(d));
        d.point2fs = (const float*)p[0];                      d.point2fs_count = len[0];
        d.point3fs = (const float*)p[1];                      d.point3fs_count = len[1];
        d.vector3fs = (const float*)p[2];                     d.vector3fs_count = len[2];
        d.planes = (const int32_t*)p[3];                      d.planes_count = len[3];
        d.spheres = (const float*)p[4];                       d.spheres_count = len[4];
        d.terrains = (const float*)p[5];                      d.terrains_count = len[5];
        d.triangles = (const int32_t*)p[6];                   d.triangles_count = len[6];
        d.bounding_volume_hierarchies = (const int32_t*)p[7]; d.bounding_volume_hierarchies_count = len[7];
        d.textures = (const float*)p[8];                      d.textures_count = len[8];
        d.surfaces = (const float*)p[9];                      d.surfaces_count = len[9];
        d.primitives = (const int32_t*)p[10];                 d.primitives_count = len[10];
        d.primitives_object_to_world = (const float*)p[11];   d.primitives_object_to_world_count = len[11];
        d.primitives_world_to_object = (const float*)p[12];   d.primitives_world_to_object_count = len[12];
        d.camera = (const float*)p[13];                       d.camera_count = len[13];
        rc = dfpt_create(&d, &sky, width, height, &k->handle);
        k->pixels = (int64_t)width * height;
    }
    for (int i = held - 1; i >= 0; --i) (*env)->ReleasePrimitiveArrayCritical(env, arrays[i], p[i], JNI_ABORT);
    if (held != SCENE_ARRAYS) {
        free(k);
        throw_class(env, "java/lang/OutOfMemoryError", "could not pin the compiled-scene arrays");
        return 0;
    }
    if (!rc) {
        /* The reference seeds every pass from ThreadLocalRandom (AbstractKernel.java:1148-1156); the
         * core's counter-based stream takes the caller's seed. */
        dfpt_params_default(&k->params);
        k->params.seed = (uint64_t)seed;
        k->params.rng_kind = DFPT_RNG_COUNTER;
        rc = dfpt_set_params(k->handle, &k->params);
    }
    if (rc) {
        if (k->handle) dfpt_destroy(k->handle);
        free(k);
        throw_if(env, rc);
        return 0;
    }
    return (jlong)(intptr_t)k;
}

JNIEXPORT void JNICALL Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_nativeDestroy(JNIEnv* env, jclass cls, jlong h) {
    (void)cls;
    if (h == 0) return;
    jni_kernel* k = kernel_of(h);
    int rc = k->handle ? dfpt_destroy(k->handle) : DFPT_OK;
    free(k);
    throw_if(env, rc);
}

/* ints: renderer type, tone mapper, shader, normal mapping, wireframes, path depth maximum, Russian
 * roulette depth, global octaves, selected primitive offset; floats: tone-mapper exposure, AO
 * maximum distance, global amplitude, frequency, gain, lacunarity. */
JNIEXPORT void JNICALL Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_nativeSetParams(
    JNIEnv* env, jclass cls, jlong h, jintArray ints, jfloatArray floats) {
    (void)cls;
    static const char* const names[2] = {"paramInts", "paramFloats"};
    const jarray arrays[2] = {ints, floats};
    if (!need_handle(env, h) || !need_arrays(env, arrays, names, 2)) return;
    if ((*env)->GetArrayLength(env, ints) != 9 || (*env)->GetArrayLength(env, floats) != 6) {
        throw_class(env, "java/lang/IllegalArgumentException", "params must hold 9 ints and 6 floats");
        return;
    }
    jint i[9];
    jfloat f[6];
    (*env)->GetIntArrayRegion(env, ints, 0, 9, i);
    (*env)->GetFloatArrayRegion(env, floats, 0, 6, f);
    jni_kernel* k = kernel_of(h);
    dfpt_params p = k->params;
    p.renderer_type = i[0];
    p.tone_mapper_type = i[1];
    p.shader_type = i[2];
    p.normal_mapping = i[3];
    p.wireframes = i[4];
    p.pt_ray_depth_maximum = i[5];
    p.pt_ray_depth_russian_roulette = i[6];
    p.global_octaves = i[7];
    p.selected_primitive_offset = i[8];
    p.tone_mapper_exposure = f[0];
    p.ao_maximum_distance = f[1];
    p.global_amplitude = f[2];
    p.global_frequency = f[3];
    p.global_gain = f[4];
    p.global_lacunarity = f[5];
    if (memcmp(&p, &k->params, sizeof(p)) == 0) return;
    if (throw_if(env, dfpt_set_params(k->handle, &p))) return;
    k->params = p;
}

JNIEXPORT void JNICALL Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_nativeClear(JNIEnv* env, jclass cls, jlong h) {
    (void)cls;
    if (!need_handle(env, h)) return;
    throw_if(env, dfpt_clear(kernel_of(h)->handle));
}

JNIEXPORT void JNICALL Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_nativeRender(JNIEnv* env, jclass cls, jlong h, jint passes) {
    (void)cls;
    if (!need_handle(env, h)) return;
    throw_if(env, dfpt_render(kernel_of(h)->handle, passes));
}

/* The frame loop's launch structure for this kernel's scene and size (dfpt_tune_frame); the film,
 * image and random streams are left as they were. */
JNIEXPORT void JNICALL Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_nativeTuneFrame(JNIEnv* env, jclass cls, jlong h, jint frames) {
    (void)cls;
    if (!need_handle(env, h)) return;
    throw_if(env, dfpt_tune_frame(kernel_of(h)->handle, frames, NULL));
}

/* The array must hold width x height x 4 bytes of the size given to nativeCreate. */
JNIEXPORT void JNICALL Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_nativeReadBgra8(JNIEnv* env, jclass cls, jlong h, jbyteArray out) {
    (void)cls;
    static const char* const names[1] = {"bgra"};
    const jarray arrays[1] = {out};
    if (!need_handle(env, h) || !need_arrays(env, arrays, names, 1)) return;
    if ((int64_t)(*env)->GetArrayLength(env, out) != kernel_of(h)->pixels * 4) {
        throw_class(env, "java/lang/IllegalArgumentException", "bgra.length != resolutionX * resolutionY * 4");
        return;
    }
    void* p = (*env)->GetPrimitiveArrayCritical(env, out, NULL);
    if (!p) {
        throw_class(env, "java/lang/OutOfMemoryError", "could not pin the image array");
        return;
    }
    int rc = dfpt_read_bgra8(kernel_of(h)->handle, (uint8_t*)p);
    (*env)->ReleasePrimitiveArrayCritical(env, out, p, 0);
    throw_if(env, rc);
}

JNIEXPORT void JNICALL Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_nativeReadPrimitiveOffsets(JNIEnv* env, jclass cls, jlong h, jintArray out) {
    (void)cls;
    static const char* const names[1] = {"primitiveOffsets"};
    const jarray arrays[1] = {out};
    if (!need_handle(env, h) || !need_arrays(env, arrays, names, 1)) return;
    if ((int64_t)(*env)->GetArrayLength(env, out) != kernel_of(h)->pixels) {
        throw_class(env, "java/lang/IllegalArgumentException", "primitiveOffsets.length != resolutionX * resolutionY");
        return;
    }
    void* p = (*env)->GetPrimitiveArrayCritical(env, out, NULL);
    if (!p) {
        throw_class(env, "java/lang/OutOfMemoryError", "could not pin the offsets array");
        return;
    }
    int rc = dfpt_read_primitive_offsets(kernel_of(h)->handle, (int32_t*)p);
    (*env)->ReleasePrimitiveArrayCritical(env, out, p, 0);
    throw_if(env, rc);
}

JNIEXPORT void JNICALL Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_nativeSetCamera(JNIEnv* env, jclass cls, jlong h, jfloatArray camera) {
    (void)cls;
    static const char* const names[1] = {"camera"};
    const jarray arrays[1] = {camera};
    if (!need_handle(env, h) || !need_arrays(env, arrays, names, 1)) return;
    if ((*env)->GetArrayLength(env, camera) < 19) {
        throw_class(env, "java/lang/IllegalArgumentException", "camera.length < 19");
        return;
    }
    jfloat c[19];
    (*env)->GetFloatArrayRegion(env, camera, 0, 19, c);
    throw_if(env, dfpt_set_camera(kernel_of(h)->handle, c));
}

JNIEXPORT void JNICALL Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_nativeSetTransforms(
    JNIEnv* env, jclass cls, jlong h, jfloatArray o2w, jfloatArray w2o, jint count) {
    (void)cls;
    static const char* const names[2] = {"objectToWorld", "worldToObject"};
    const jarray arrays[2] = {o2w, w2o};
    if (!need_handle(env, h) || !need_arrays(env, arrays, names, 2)) return;
    if (count < 0 || (int64_t)(*env)->GetArrayLength(env, o2w) < (int64_t)count * 16 ||
        (int64_t)(*env)->GetArrayLength(env, w2o) < (int64_t)count * 16) {
        throw_class(env, "java/lang/IllegalArgumentException", "matrix arrays shorter than primitiveCount * 16");
        return;
    }
    void* a = (*env)->GetPrimitiveArrayCritical(env, o2w, NULL);
    void* b = a ? (*env)->GetPrimitiveArrayCritical(env, w2o, NULL) : NULL;
    int rc = (a && b) ? dfpt_set_transforms(kernel_of(h)->handle, (const float*)a, (const float*)b, count) : DFPT_ERR_OUT_OF_MEMORY;
    if (b) (*env)->ReleasePrimitiveArrayCritical(env, w2o, b, JNI_ABORT);
    if (a) (*env)->ReleasePrimitiveArrayCritical(env, o2w, a, JNI_ABORT);
    if (!(a && b)) {
        throw_class(env, "java/lang/OutOfMemoryError", "could not pin the matrix arrays");
        return;
    }
    throw_if(env, rc);
}

JNIEXPORT void JNICALL Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_nativeSetSurfaces(JNIEnv* env, jclass cls, jlong h, jfloatArray surfaces) {
    (void)cls;
    static const char* const names[1] = {"surfaces"};
    const jarray arrays[1] = {surfaces};
    if (!need_handle(env, h) || !need_arrays(env, arrays, names, 1)) return;
    const jsize n = (*env)->GetArrayLength(env, surfaces);
    void* p = (*env)->GetPrimitiveArrayCritical(env, surfaces, NULL);
    if (!p) {
        throw_class(env, "java/lang/OutOfMemoryError", "could not pin the surfaces array");
        return;
    }
    int rc = dfpt_set_surfaces(kernel_of(h)->handle, (const float*)p, n);
    (*env)->ReleasePrimitiveArrayCritical(env, surfaces, p, JNI_ABORT);
    throw_if(env, rc);
}

JNIEXPORT void JNICALL Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_nativeSetSky(
    JNIEnv* env, jclass cls, jlong h, jdoubleArray sky_d, jfloatArray sky_f, jint flags) {
    (void)cls;
    static const char* const names[2] = {"skyDoubles", "skyFloats"};
    const jarray arrays[2] = {sky_d, sky_f};
    if (!need_handle(env, h) || !need_arrays(env, arrays, names, 2)) return;
    dfpt_sky sky;
    if (!fill_sky(env, &sky, sky_d, sky_f, flags)) return;
    throw_if(env, dfpt_set_sky(kernel_of(h)->handle, &sky));
}
