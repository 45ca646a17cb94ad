/*
 * imfcs_jni.c -- the JNI shim: the natives of gpufitImFCS.GpufitImFCS
 * (GpufitImFCS.java:323-538) forwarded to libimfcs_gb300.so's C ABI.  Built
 * as libagpufit.so, the name GpufitImFCS.java:46-201 loads, it replaces the
 * reference's JNI layer (agpufitjni.cu:91-170 declarations, 4614-5831
 * bodies) without any change on the Java side.
 *
 *   cc -O2 -shared -fPIC -I$JAVA_HOME/include -I$JAVA_HOME/include/linux \
 *      -I include jni/imfcs_jni.c -L imaging_fcs_1_52_gb300 -limfcs_gb300 \
 *      -Wl,-rpath,'$ORIGIN' -o libagpufit.so
 *
 * (the tests build it against jni/stub/jni.h and a mock JNIEnv instead).
 *
 * Buffers: fit() takes direct NIO buffers (GetDirectBufferAddress, NULL for a
 * null buffer, like agpufitjni.cu:4592-4605); the other natives take Java
 * arrays, pinned or copied with Get<T>ArrayElements and released with mode 0
 * (copy back) for outputs and JNI_ABORT for inputs.  A failing call throws
 * java.lang.Exception with the library's last error, where the reference
 * throws from its catch blocks; fit() returns 0 or -1 (Gpufit's
 * ReturnState), which GpufitImFCS.fit turns into its RuntimeException.
 */
#include <jni.h>

#include "imfcs_gb300.h"

/* GpufitImFCS.ACFParameters (GpufitImFCS.java:453-486) -> the C struct; the
 * two boolean fields become 0 / 1. */
static void read_params(JNIEnv *env, jobject o, imfcs_acf_parameters *p)
{
    jclass c = (*env)->GetObjectClass(env, o);
#define I(f) p->f = (*env)->GetIntField(env, o, (*env)->GetFieldID(env, c, #f, "I"))
#define D(f) p->f = (*env)->GetDoubleField(env, o, (*env)->GetFieldID(env, c, #f, "D"))
#define Z(f) p->f = (*env)->GetBooleanField(env, o, (*env)->GetFieldID(env, c, #f, "Z")) ? 1 : 0
    I(width); I(height); I(win_star); I(hin_star); I(w_temp); I(h_temp); I(pixbinX); I(pixbinY);
    I(binningX); I(binningY); I(firstframe); I(lastframe); I(framediff); I(cfXDistance);
    I(cfYDistance); D(correlatorp); D(correlatorq); D(frametime); I(background); D(mtab1);
    D(mtabchanumminus1); D(sampchanumminus1); I(chanum); Z(isNBcalculation); Z(bleachcorr_gpu);
    I(bleachcorr_order); I(nopit); I(ave);
#undef I
#undef D
#undef Z
}

static void throw_last(JNIEnv *env)
{
    (*env)->ThrowNew(env, (*env)->FindClass(env, "java/lang/Exception"), imfcs_get_last_error());
}

static void *buffer_address(JNIEnv *env, jobject b) { return b ? (*env)->GetDirectBufferAddress(env, b) : NULL; }

/* GpufitImFCS.fit (GpufitImFCS.java:323) -> imfcs_fit */
JNIEXPORT jint JNICALL Java_gpufitImFCS_GpufitImFCS_fit(JNIEnv *env, jclass cls, jint nfits, jint npts, jobject data,
                                                        jobject weights, jint model, jobject init, jfloat tol,
                                                        jint maxit, jint ncoef, jobject to_fit, jint estimator,
                                                        jint user_info_size, jobject user_info, jobject out_par,
                                                        jobject out_states, jobject out_chi2, jobject out_iter)
{
    (void)cls;
    int rc = imfcs_fit(nfits, npts, (const float *)buffer_address(env, data), (const float *)buffer_address(env, weights),
                       model, (const float *)buffer_address(env, init), tol, maxit, ncoef,
                       (const int *)buffer_address(env, to_fit), estimator, (size_t)user_info_size,
                       buffer_address(env, user_info), (float *)buffer_address(env, out_par),
                       (int *)buffer_address(env, out_states), (float *)buffer_address(env, out_chi2),
                       (int *)buffer_address(env, out_iter));
    return rc == 0 ? 0 : -1;
}

/* GpufitImFCS.getLastError (GpufitImFCS.java:382) */
JNIEXPORT jstring JNICALL Java_gpufitImFCS_GpufitImFCS_getLastError(JNIEnv *env, jclass cls)
{
    (void)cls;
    return (*env)->NewStringUTF(env, imfcs_get_last_error());
}

/* GpufitImFCS.isCudaAvailableInt (GpufitImFCS.java:389) */
JNIEXPORT jboolean JNICALL Java_gpufitImFCS_GpufitImFCS_isCudaAvailableInt(JNIEnv *env, jclass cls)
{
    (void)env;
    (void)cls;
    return imfcs_is_cuda_available() ? JNI_TRUE : JNI_FALSE;
}

/* GpufitImFCS.getCudaVersionAsArray (GpufitImFCS.java:403); null on failure */
JNIEXPORT jintArray JNICALL Java_gpufitImFCS_GpufitImFCS_getCudaVersionAsArray(JNIEnv *env, jclass cls)
{
    (void)cls;
    jint v[2];
    int rt = 0, dr = 0;
    if (imfcs_get_cuda_version(&rt, &dr)) return NULL;
    v[0] = rt;
    v[1] = dr;
    jintArray a = (*env)->NewIntArray(env, 2);
    if (a) (*env)->SetIntArrayRegion(env, a, 0, 2, v);
    return a;
}

/* GpufitImFCS.resetGPU / resetDevice (GpufitImFCS.java:491, 538): frees the
 * library's cached buffers; the shared device itself is never reset. */
JNIEXPORT void JNICALL Java_gpufitImFCS_GpufitImFCS_resetGPU(JNIEnv *env, jclass cls)
{
    (void)cls;
    if (imfcs_reset_gpu()) throw_last(env);
}

JNIEXPORT void JNICALL Java_gpufitImFCS_GpufitImFCS_resetDevice(JNIEnv *env, jclass cls)
{
    (void)cls;
    if (imfcs_reset_gpu()) throw_last(env);
}

#define ARR(T, a) ((a) ? (*env)->Get##T##ArrayElements(env, (a), NULL) : NULL)
#define REL(T, a, p, mode)                                          \
    do {                                                            \
        if ((a) && (p)) (*env)->Release##T##ArrayElements(env, (a), (p), (mode)); \
    } while (0)

/* GpufitImFCS.calcBinning (GpufitImFCS.java:520) */
JNIEXPORT void JNICALL Java_gpufitImFCS_GpufitImFCS_calcBinning(JNIEnv *env, jclass cls, jfloatArray in,
                                                                jfloatArray out, jobject prm)
{
    (void)cls;
    imfcs_acf_parameters p;
    read_params(env, prm, &p);
    jfloat *i = ARR(Float, in), *o = ARR(Float, out);
    int rc = imfcs_calc_binning(i, o, &p);
    REL(Float, in, i, JNI_ABORT);
    REL(Float, out, o, rc ? JNI_ABORT : 0);
    if (rc) throw_last(env);
}

/* GpufitImFCS.calcDataBleachCorrection (GpufitImFCS.java:501) */
JNIEXPORT void JNICALL Java_gpufitImFCS_GpufitImFCS_calcDataBleachCorrection(JNIEnv *env, jclass cls,
                                                                             jfloatArray px, jfloatArray out,
                                                                             jobject prm)
{
    (void)cls;
    imfcs_acf_parameters p;
    read_params(env, prm, &p);
    jfloat *i = ARR(Float, px), *o = ARR(Float, out);
    int rc = imfcs_calc_data_bleach_correction(i, o, &p);
    REL(Float, px, i, JNI_ABORT);
    REL(Float, out, o, rc ? JNI_ABORT : 0);
    if (rc) throw_last(env);
}

/* GpufitImFCS.isBinningMemorySufficient (GpufitImFCS.java:510) */
JNIEXPORT jboolean JNICALL Java_gpufitImFCS_GpufitImFCS_isBinningMemorySufficient(JNIEnv *env, jclass cls,
                                                                                  jobject prm)
{
    (void)cls;
    imfcs_acf_parameters p;
    read_params(env, prm, &p);
    return imfcs_is_binning_memory_sufficient(&p) ? JNI_TRUE : JNI_FALSE;
}

/* GpufitImFCS.isACFmemorySufficient (GpufitImFCS.java:531) */
JNIEXPORT jboolean JNICALL Java_gpufitImFCS_GpufitImFCS_isACFmemorySufficient(JNIEnv *env, jclass cls, jobject prm)
{
    (void)cls;
    imfcs_acf_parameters p;
    read_params(env, prm, &p);
    return imfcs_is_acf_memory_sufficient(&p) ? JNI_TRUE : JNI_FALSE;
}

/* GpufitImFCS.calcACF (GpufitImFCS.java:533-536); the bleach-correction
 * coefficients are read only when bleachcorr_gpu is set. */
JNIEXPORT void JNICALL Java_gpufitImFCS_GpufitImFCS_calcACF(JNIEnv *env, jclass cls, jfloatArray px, jdoubleArray acf,
                                                            jdoubleArray var, jdoubleArray nbm, jdoubleArray nbc,
                                                            jdoubleArray blk, jdoubleArray bcp, jdoubleArray samp,
                                                            jintArray lag, jobject prm)
{
    (void)cls;
    imfcs_acf_parameters p;
    read_params(env, prm, &p);
    jfloat *i = ARR(Float, px);
    jdouble *a = ARR(Double, acf), *v = ARR(Double, var), *m = ARR(Double, nbm), *n = ARR(Double, nbc),
            *b = ARR(Double, blk), *q = p.bleachcorr_gpu ? ARR(Double, bcp) : NULL, *s = ARR(Double, samp);
    jint *l = ARR(Int, lag);
    int rc = imfcs_calc_acf(i, a, v, m, n, b, q, s, l, &p);
    const jint out_mode = rc ? JNI_ABORT : 0;
    REL(Float, px, i, JNI_ABORT);
    REL(Double, acf, a, out_mode);
    REL(Double, var, v, out_mode);
    REL(Double, nbm, m, out_mode);
    REL(Double, nbc, n, out_mode);
    REL(Double, blk, b, out_mode);
    REL(Double, bcp, q, JNI_ABORT);
    REL(Double, samp, s, out_mode);
    REL(Int, lag, l, out_mode);
    if (rc) throw_last(env);
}
