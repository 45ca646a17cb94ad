/*
 * mock_jni.c -- a mock JNIEnv for driving jni/imfcs_jni.c from the tests:
 * just enough of a JVM (classes, strings, primitive arrays, direct buffers,
 * an object with named int/double/boolean fields, pending exceptions) behind
 * the function table of jni/stub/jni.h.
 *
 * Arrays behave like a copying JVM: Get<T>ArrayElements returns a fresh copy,
 * Release<T>ArrayElements copies it back for mode 0 / JNI_COMMIT and discards
 * it for JNI_ABORT, so a shim that releases an output with the wrong mode is
 * caught.  Objects are never freed (the tests are short-lived).
 */
#include <jni.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum { K_CLASS = 1, K_STRING, K_FLOAT_ARRAY, K_DOUBLE_ARRAY, K_INT_ARRAY, K_DIRECT, K_FIELDS };

#define MAX_FIELDS 40
struct _jobject {
    int kind;
    void *data;        /* arrays: the caller's memory; direct: the address */
    int len, elem;     /* arrays: length, element size */
    char str[512];     /* strings, class names */
    int nf;            /* K_FIELDS */
    char fname[MAX_FIELDS][32];
    char fsig[MAX_FIELDS];
    double fval[MAX_FIELDS];
};

struct _jfieldID {
    char name[32];
    char sig;
};

static char g_exception[1100];
static int g_exceptions;
static int g_release[3];     /* releases by mode 0, JNI_COMMIT, JNI_ABORT */
static int g_bad_field;      /* GetFieldID / Get<T>Field on a missing or mistyped field */
static struct _jobject g_class = {K_CLASS};

static jobject new_obj(int kind)
{
    jobject o = (jobject)calloc(1, sizeof(struct _jobject));
    o->kind = kind;
    return o;
}

static jint JNICALL m_GetVersion(JNIEnv *env) { (void)env; return 0x00010008; }
static jclass JNICALL m_FindClass(JNIEnv *env, const char *name)
{
    (void)env;
    jobject c = new_obj(K_CLASS);
    snprintf(c->str, sizeof(c->str), "%s", name);
    return c;
}
static jint JNICALL m_ThrowNew(JNIEnv *env, jclass cls, const char *msg)
{
    (void)env;
    snprintf(g_exception, sizeof(g_exception), "%s: %s", cls ? cls->str : "?", msg ? msg : "");
    g_exceptions++;
    return 0;
}
static jthrowable JNICALL m_ExceptionOccurred(JNIEnv *env) { (void)env; return g_exceptions ? &g_class : NULL; }
static jclass JNICALL m_GetObjectClass(JNIEnv *env, jobject o) { (void)env; (void)o; return &g_class; }
static jfieldID JNICALL m_GetFieldID(JNIEnv *env, jclass c, const char *name, const char *sig)
{
    (void)env;
    (void)c;
    jfieldID f = (jfieldID)calloc(1, sizeof(struct _jfieldID));
    snprintf(f->name, sizeof(f->name), "%s", name);
    f->sig = sig[0];
    return f;
}
static double field(jobject o, jfieldID f, char sig)
{
    if (!o || o->kind != K_FIELDS || !f || f->sig != sig) { g_bad_field++; return 0; }
    for (int i = 0; i < o->nf; i++)
        if (!strcmp(o->fname[i], f->name)) {
            if (o->fsig[i] != sig) { g_bad_field++; return 0; }
            return o->fval[i];
        }
    g_bad_field++;
    return 0;
}
static jboolean JNICALL m_GetBooleanField(JNIEnv *env, jobject o, jfieldID f)
{
    (void)env;
    return field(o, f, 'Z') != 0 ? JNI_TRUE : JNI_FALSE;
}
static jint JNICALL m_GetIntField(JNIEnv *env, jobject o, jfieldID f) { (void)env; return (jint)field(o, f, 'I'); }
static jdouble JNICALL m_GetDoubleField(JNIEnv *env, jobject o, jfieldID f) { (void)env; return field(o, f, 'D'); }
static jstring JNICALL m_NewStringUTF(JNIEnv *env, const char *s)
{
    (void)env;
    jobject o = new_obj(K_STRING);
    snprintf(o->str, sizeof(o->str), "%s", s ? s : "");
    return o;
}
static jintArray JNICALL m_NewIntArray(JNIEnv *env, jsize n)
{
    (void)env;
    jobject o = new_obj(K_INT_ARRAY);
    o->data = calloc(n > 0 ? n : 1, sizeof(jint));
    o->len = n;
    o->elem = sizeof(jint);
    return o;
}
static void *get_elems(jobject a, int kind, jboolean *is_copy)
{
    if (!a || a->kind != kind) return NULL;
    void *p = malloc((size_t)(a->len > 0 ? a->len : 1) * a->elem);
    memcpy(p, a->data, (size_t)a->len * a->elem);
    if (is_copy) *is_copy = JNI_TRUE;
    return p;
}
static void release_elems(jobject a, void *p, jint mode)
{
    if (!a || !p) return;
    if (mode == 0 || mode == JNI_COMMIT) memcpy(a->data, p, (size_t)a->len * a->elem);
    if (mode >= 0 && mode <= 2) g_release[mode]++;
    if (mode != JNI_COMMIT) free(p);
}
static jint *JNICALL m_GetIntArrayElements(JNIEnv *e, jintArray a, jboolean *c)
{
    (void)e;
    return (jint *)get_elems(a, K_INT_ARRAY, c);
}
static jfloat *JNICALL m_GetFloatArrayElements(JNIEnv *e, jfloatArray a, jboolean *c)
{
    (void)e;
    return (jfloat *)get_elems(a, K_FLOAT_ARRAY, c);
}
static jdouble *JNICALL m_GetDoubleArrayElements(JNIEnv *e, jdoubleArray a, jboolean *c)
{
    (void)e;
    return (jdouble *)get_elems(a, K_DOUBLE_ARRAY, c);
}
static void JNICALL m_ReleaseIntArrayElements(JNIEnv *e, jintArray a, jint *p, jint m) { (void)e; release_elems(a, p, m); }
static void JNICALL m_ReleaseFloatArrayElements(JNIEnv *e, jfloatArray a, jfloat *p, jint m) { (void)e; release_elems(a, p, m); }
static void JNICALL m_ReleaseDoubleArrayElements(JNIEnv *e, jdoubleArray a, jdouble *p, jint m) { (void)e; release_elems(a, p, m); }
static void JNICALL m_SetIntArrayRegion(JNIEnv *e, jintArray a, jsize start, jsize n, const jint *buf)
{
    (void)e;
    if (a && a->kind == K_INT_ARRAY && start >= 0 && start + n <= a->len) memcpy((jint *)a->data + start, buf, n * sizeof(jint));
}
static void *JNICALL m_GetDirectBufferAddress(JNIEnv *e, jobject b)
{
    (void)e;
    return (b && b->kind == K_DIRECT) ? b->data : NULL;
}

static struct JNINativeInterface_ g_table;
static JNIEnv g_env;

/* ---- test-side helpers (called through ctypes) ---- */
JNIEXPORT JNIEnv *mock_env(void)
{
    memset(&g_table, 0, sizeof(g_table));
    g_table.GetVersion = m_GetVersion;
    g_table.FindClass = m_FindClass;
    g_table.ThrowNew = m_ThrowNew;
    g_table.ExceptionOccurred = m_ExceptionOccurred;
    g_table.GetObjectClass = m_GetObjectClass;
    g_table.GetFieldID = m_GetFieldID;
    g_table.GetBooleanField = m_GetBooleanField;
    g_table.GetIntField = m_GetIntField;
    g_table.GetDoubleField = m_GetDoubleField;
    g_table.NewStringUTF = m_NewStringUTF;
    g_table.NewIntArray = m_NewIntArray;
    g_table.GetIntArrayElements = m_GetIntArrayElements;
    g_table.GetFloatArrayElements = m_GetFloatArrayElements;
    g_table.GetDoubleArrayElements = m_GetDoubleArrayElements;
    g_table.ReleaseIntArrayElements = m_ReleaseIntArrayElements;
    g_table.ReleaseFloatArrayElements = m_ReleaseFloatArrayElements;
    g_table.ReleaseDoubleArrayElements = m_ReleaseDoubleArrayElements;
    g_table.SetIntArrayRegion = m_SetIntArrayRegion;
    g_table.GetDirectBufferAddress = m_GetDirectBufferAddress;
    g_env = &g_table;
    return &g_env;
}
static jobject wrap(int kind, void *p, int n, int elem)
{
    jobject o = new_obj(kind);
    o->data = p;
    o->len = n;
    o->elem = elem;
    return o;
}
JNIEXPORT jobject mock_float_array(float *p, int n) { return wrap(K_FLOAT_ARRAY, p, n, sizeof(float)); }
JNIEXPORT jobject mock_double_array(double *p, int n) { return wrap(K_DOUBLE_ARRAY, p, n, sizeof(double)); }
JNIEXPORT jobject mock_int_array(int *p, int n) { return wrap(K_INT_ARRAY, p, n, sizeof(int)); }
JNIEXPORT jobject mock_direct(void *p) { return wrap(K_DIRECT, p, 0, 1); }
JNIEXPORT jobject mock_object(void) { return new_obj(K_FIELDS); }
JNIEXPORT int mock_set_field(jobject o, const char *name, char sig, double v)
{
    if (!o || o->kind != K_FIELDS || o->nf >= MAX_FIELDS) return 1;
    snprintf(o->fname[o->nf], sizeof(o->fname[0]), "%s", name);
    o->fsig[o->nf] = sig;
    o->fval[o->nf] = v;
    o->nf++;
    return 0;
}
JNIEXPORT const char *mock_string(jobject o) { return (o && o->kind == K_STRING) ? o->str : NULL; }
JNIEXPORT int mock_int_array_len(jobject o) { return (o && o->kind == K_INT_ARRAY) ? o->len : -1; }
JNIEXPORT const int *mock_int_array_data(jobject o) { return (o && o->kind == K_INT_ARRAY) ? (const int *)o->data : NULL; }
JNIEXPORT const char *mock_exception(void) { return g_exceptions ? g_exception : NULL; }
JNIEXPORT int mock_release_count(int mode) { return (mode >= 0 && mode <= 2) ? g_release[mode] : -1; }
JNIEXPORT int mock_bad_fields(void) { return g_bad_field; }
JNIEXPORT void mock_reset(void)
{
    g_exception[0] = 0;
    g_exceptions = 0;
    g_bad_field = 0;
    memset(g_release, 0, sizeof(g_release));
}
