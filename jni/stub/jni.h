/*
 * jni.h -- a minimal, project-written stand-in for the JDK's jni.h, enough to
 * compile jni/imfcs_jni.c without a JDK (this image has none) and to drive it
 * from a mock JNIEnv in the tests.
 *
 * Types follow the JNI specification's primitive and reference types; the
 * function table lists the slots of the specification's "Interface Function
 * Table" by index (0-3 reserved, GetVersion = 4, ..., GetObjectRefType =
 * 232).  Only the functions the shim calls are typed; every other slot is an
 * untyped placeholder, and static assertions pin the typed ones to their
 * indices.  Build the shim that a JVM loads against the JDK's own jni.h.
 */
#ifndef IMFCS_JNI_STUB_H
#define IMFCS_JNI_STUB_H

#include <stddef.h>
#include <stdint.h>

#define JNIEXPORT __attribute__((visibility("default")))
#define JNIIMPORT
#define JNICALL

typedef int32_t jint;
typedef int64_t jlong;
typedef int8_t jbyte;
typedef uint8_t jboolean;
typedef uint16_t jchar;
typedef int16_t jshort;
typedef float jfloat;
typedef double jdouble;
typedef jint jsize;

struct _jobject;
typedef struct _jobject *jobject;
typedef jobject jclass;
typedef jobject jthrowable;
typedef jobject jstring;
typedef jobject jarray;
typedef jarray jbooleanArray;
typedef jarray jbyteArray;
typedef jarray jcharArray;
typedef jarray jshortArray;
typedef jarray jintArray;
typedef jarray jlongArray;
typedef jarray jfloatArray;
typedef jarray jdoubleArray;
typedef jarray jobjectArray;

struct _jfieldID;
typedef struct _jfieldID *jfieldID;

#define JNI_FALSE 0
#define JNI_TRUE 1
#define JNI_OK 0
#define JNI_COMMIT 1
#define JNI_ABORT 2

struct JNINativeInterface_;
typedef const struct JNINativeInterface_ *JNIEnv;

struct JNINativeInterface_ {
    void *reserved0, *reserved1, *reserved2, *reserved3;                       /* 0-3 */
    jint(JNICALL *GetVersion)(JNIEnv *env);                                    /* 4 */
    void *DefineClass;                                                         /* 5 */
    jclass(JNICALL *FindClass)(JNIEnv *env, const char *name);                 /* 6 */
    void *slots_7_13[7];                                                       /* 7-13 */
    jint(JNICALL *ThrowNew)(JNIEnv *env, jclass clazz, const char *msg);       /* 14 */
    jthrowable(JNICALL *ExceptionOccurred)(JNIEnv *env);                       /* 15 */
    void *slots_16_30[15];                                                     /* 16-30 */
    jclass(JNICALL *GetObjectClass)(JNIEnv *env, jobject obj);                 /* 31 */
    void *slots_32_93[62];                                                     /* 32-93 */
    jfieldID(JNICALL *GetFieldID)(JNIEnv *env, jclass clazz, const char *name, const char *sig); /* 94 */
    void *GetObjectField;                                                      /* 95 */
    jboolean(JNICALL *GetBooleanField)(JNIEnv *env, jobject obj, jfieldID f);  /* 96 */
    void *slots_97_99[3];                                                      /* 97-99 */
    jint(JNICALL *GetIntField)(JNIEnv *env, jobject obj, jfieldID f);          /* 100 */
    void *slots_101_102[2];                                                    /* 101-102 */
    jdouble(JNICALL *GetDoubleField)(JNIEnv *env, jobject obj, jfieldID f);    /* 103 */
    void *slots_104_166[63];                                                   /* 104-166 */
    jstring(JNICALL *NewStringUTF)(JNIEnv *env, const char *utf);              /* 167 */
    void *slots_168_178[11];                                                   /* 168-178 */
    jintArray(JNICALL *NewIntArray)(JNIEnv *env, jsize len);                   /* 179 */
    void *slots_180_186[7];                                                    /* 180-186 */
    jint *(JNICALL *GetIntArrayElements)(JNIEnv *env, jintArray a, jboolean *is_copy);       /* 187 */
    void *GetLongArrayElements;                                                /* 188 */
    jfloat *(JNICALL *GetFloatArrayElements)(JNIEnv *env, jfloatArray a, jboolean *is_copy); /* 189 */
    jdouble *(JNICALL *GetDoubleArrayElements)(JNIEnv *env, jdoubleArray a, jboolean *is_copy); /* 190 */
    void *slots_191_194[4];                                                    /* 191-194 */
    void(JNICALL *ReleaseIntArrayElements)(JNIEnv *env, jintArray a, jint *e, jint mode);       /* 195 */
    void *ReleaseLongArrayElements;                                            /* 196 */
    void(JNICALL *ReleaseFloatArrayElements)(JNIEnv *env, jfloatArray a, jfloat *e, jint mode); /* 197 */
    void(JNICALL *ReleaseDoubleArrayElements)(JNIEnv *env, jdoubleArray a, jdouble *e, jint mode); /* 198 */
    void *slots_199_210[12];                                                   /* 199-210 */
    void(JNICALL *SetIntArrayRegion)(JNIEnv *env, jintArray a, jsize start, jsize len, const jint *buf); /* 211 */
    void *slots_212_229[18];                                                   /* 212-229 */
    void *(JNICALL *GetDirectBufferAddress)(JNIEnv *env, jobject buf);         /* 230 */
    void *slots_231_232[2];                                                    /* 231-232 */
};

#define IMFCS_JNI_SLOT(m, i) \
    _Static_assert(offsetof(struct JNINativeInterface_, m) == (i) * sizeof(void *), #m " slot")
IMFCS_JNI_SLOT(GetVersion, 4);
IMFCS_JNI_SLOT(FindClass, 6);
IMFCS_JNI_SLOT(ThrowNew, 14);
IMFCS_JNI_SLOT(ExceptionOccurred, 15);
IMFCS_JNI_SLOT(GetObjectClass, 31);
IMFCS_JNI_SLOT(GetFieldID, 94);
IMFCS_JNI_SLOT(GetBooleanField, 96);
IMFCS_JNI_SLOT(GetIntField, 100);
IMFCS_JNI_SLOT(GetDoubleField, 103);
IMFCS_JNI_SLOT(NewStringUTF, 167);
IMFCS_JNI_SLOT(NewIntArray, 179);
IMFCS_JNI_SLOT(GetIntArrayElements, 187);
IMFCS_JNI_SLOT(GetFloatArrayElements, 189);
IMFCS_JNI_SLOT(GetDoubleArrayElements, 190);
IMFCS_JNI_SLOT(ReleaseIntArrayElements, 195);
IMFCS_JNI_SLOT(ReleaseFloatArrayElements, 197);
IMFCS_JNI_SLOT(ReleaseDoubleArrayElements, 198);
IMFCS_JNI_SLOT(SetIntArrayRegion, 211);
IMFCS_JNI_SLOT(GetDirectBufferAddress, 230);
_Static_assert(sizeof(struct JNINativeInterface_) == 233 * sizeof(void *), "233 slots");
#undef IMFCS_JNI_SLOT

#endif
