/*
 * A fake JNIEnv for testing dayflower-path-tracer_gb300/jni/dfpt_jni.c without a JVM (tests only).
 *
 * Java arrays are stand-ins that point at the caller's memory (no copy), so the test sees what the
 * shim writes. The environment records the last exception thrown (class and message) and checks
 * the rule of JNI's critical sections: between GetPrimitiveArrayCritical and the matching release
 * no other JNI call may be made. A call that breaks it, a release of an array that is not held and
 * a critical section left open at the end of a native call are counted as violations.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "jni.h"

struct _jobject {
    int is_class;
    jsize length;
    void* data;
    int element_size;
    char name[64];
};

static char g_exception_class[64];
static char g_exception_message[512];
static int g_critical_depth;
static int g_violations;

static void note_call(void) {
    if (g_critical_depth > 0) ++g_violations;
}

static jclass JNICALL fake_find_class(JNIEnv* env, const char* name) {
    (void)env;
    note_call();
    jclass c = (jclass)calloc(1, sizeof(struct _jobject));
    c->is_class = 1;
    snprintf(c->name, sizeof(c->name), "%s", name);
    return c;  /* leaked: a test makes a handful */
}

static jint JNICALL fake_throw_new(JNIEnv* env, jclass clazz, const char* msg) {
    (void)env;
    note_call();
    snprintf(g_exception_class, sizeof(g_exception_class), "%s", clazz->name);
    snprintf(g_exception_message, sizeof(g_exception_message), "%s", msg ? msg : "");
    return 0;
}

static jsize JNICALL fake_get_array_length(JNIEnv* env, jarray a) {
    (void)env;
    note_call();
    return a->length;
}

static void region(jarray a, jsize start, jsize len, void* buf) {
    note_call();
    if (start < 0 || len < 0 || start + len > a->length) {
        ++g_violations;  /* the JVM throws ArrayIndexOutOfBoundsException */
        return;
    }
    memcpy(buf, (char*)a->data + (size_t)start * a->element_size, (size_t)len * a->element_size);
}

static void JNICALL fake_get_int_region(JNIEnv* env, jintArray a, jsize s, jsize n, jint* buf) { (void)env; region(a, s, n, buf); }
static void JNICALL fake_get_float_region(JNIEnv* env, jfloatArray a, jsize s, jsize n, jfloat* buf) { (void)env; region(a, s, n, buf); }
static void JNICALL fake_get_double_region(JNIEnv* env, jdoubleArray a, jsize s, jsize n, jdouble* buf) { (void)env; region(a, s, n, buf); }

static void* JNICALL fake_get_critical(JNIEnv* env, jarray a, jboolean* is_copy) {
    (void)env;
    if (is_copy) *is_copy = 0;
    ++g_critical_depth;
    return a->data;
}

static void JNICALL fake_release_critical(JNIEnv* env, jarray a, void* p, jint mode) {
    (void)env;
    (void)mode;
    if (g_critical_depth <= 0 || p != a->data) ++g_violations;
    else --g_critical_depth;
}

static const struct JNINativeInterface_ g_table = {
    fake_find_class, fake_throw_new, fake_get_array_length, fake_get_int_region,
    fake_get_float_region, fake_get_double_region, fake_get_critical, fake_release_critical,
};
static JNIEnv g_env = &g_table;

/* ---- exported to the test (ctypes) ---- */

JNIEXPORT JNIEnv* fake_env(void) { return &g_env; }

/* A Java array of `length` elements of `element_size` bytes over the caller's memory. */
JNIEXPORT jarray fake_array(void* data, jsize length, int element_size) {
    jarray a = (jarray)calloc(1, sizeof(struct _jobject));
    a->length = length;
    a->data = data;
    a->element_size = element_size;
    return a;
}

JNIEXPORT void fake_free(jarray a) { free(a); }

/* Clears the recorded exception and counters before a native call. */
JNIEXPORT void fake_reset(void) {
    g_exception_class[0] = 0;
    g_exception_message[0] = 0;
    g_critical_depth = 0;
    g_violations = 0;
}

JNIEXPORT const char* fake_exception_class(void) { return g_exception_class; }
JNIEXPORT const char* fake_exception_message(void) { return g_exception_message; }

/* Violations of the critical-section rule so far, counting a section still open. */
JNIEXPORT int fake_violations(void) { return g_violations + (g_critical_depth != 0); }
