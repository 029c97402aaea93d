/*
 * A stand-in for a JDK's jni.h, for tests only: neither image of this project has a JDK. It
 * declares the JNI types by their sizes in the JNI specification and a JNIEnv whose function table
 * holds only the entries dayflower-path-tracer_gb300/jni/dfpt_jni.c calls, under their JNI names
 * and signatures, so that the shim's source compiles unchanged against either header. The table's
 * layout is not the JVM's: a library built against this header runs only with the fake JNIEnv of
 * tests/jni/fake_env.c.
 */
#ifndef DFPT_TEST_JNI_H
#define DFPT_TEST_JNI_H

#include <stdint.h>

#define JNIEXPORT __attribute__((visibility("default")))
#define JNICALL
#define JNI_COMMIT 1
#define JNI_ABORT 2

typedef uint8_t jboolean;
typedef int8_t jbyte;
typedef int32_t jint;
typedef int64_t jlong;
typedef float jfloat;
typedef double jdouble;
typedef jint jsize;

struct _jobject;
typedef struct _jobject* jobject;
typedef jobject jclass;
typedef jobject jthrowable;
typedef jobject jarray;
typedef jarray jbyteArray;
typedef jarray jintArray;
typedef jarray jfloatArray;
typedef jarray jdoubleArray;

struct JNINativeInterface_;
typedef const struct JNINativeInterface_* JNIEnv;

struct JNINativeInterface_ {
    jclass (JNICALL* FindClass)(JNIEnv* env, const char* name);
    jint (JNICALL* ThrowNew)(JNIEnv* env, jclass clazz, const char* msg);
    jsize (JNICALL* GetArrayLength)(JNIEnv* env, jarray array);
    void (JNICALL* GetIntArrayRegion)(JNIEnv* env, jintArray array, jsize start, jsize len, jint* buf);
    void (JNICALL* GetFloatArrayRegion)(JNIEnv* env, jfloatArray array, jsize start, jsize len, jfloat* buf);
    void (JNICALL* GetDoubleArrayRegion)(JNIEnv* env, jdoubleArray array, jsize start, jsize len, jdouble* buf);
    void* (JNICALL* GetPrimitiveArrayCritical)(JNIEnv* env, jarray array, jboolean* isCopy);
    void (JNICALL* ReleasePrimitiveArrayCritical)(JNIEnv* env, jarray array, void* carray, jint mode);
};

#endif
