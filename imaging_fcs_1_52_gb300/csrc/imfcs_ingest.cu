// imfcs_ingest.cu -- stack ingest and background-file statistics.
//
// TIFF: the plugin reads its stacks through ImageJ (getVoxels,
// Imaging_FCS_1_52.java:14791, and GPU_get_pixels 14913-14983, which copy
// every frame into a Java float array before the JNI call).  Here a uint16
// TIFF stack goes from the file to device memory as uint16: the reader
// parses baseline TIFF (either byte order, uncompressed, one 16-bit sample
// per pixel, one IFD per frame with any number of strips) and ImageJ's
// layout for stacks written as one IFD plus "images=N" in the image
// description (frames stored contiguously after the first), and copies a
// frame range to a host buffer or, through two pinned staging buffers used
// in turn, to the device (the file read of one chunk overlaps the copy of
// the previous one).
//
// Background statistics: loadBGRFile (java:6988-7103) over a background
// stack of the image's size -- per-pixel mean and variance over all frames,
// the lag-1 covariance with the means of frames 1..f-1 and 2..f, and the
// row and column means.  The Java accumulates pixel values, squares and
// lag-1 products in double; they are integers below 2^53, so the GPU sums
// them exactly in 64-bit integers and finishes with the same FP64
// operations (no contraction), in the same order for the row and column
// means, so the results are identical to the Java's.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/types.h>

#include <algorithm>
#include <string>
#include <vector>

#include "imfcs_gb300.h"
#include "imfcs_host.h"

using namespace imfcs;

#define CK(call)                                                        \
    do {                                                                \
        cudaError_t _e = (call);                                        \
        if (_e != cudaSuccess) { set_error(cuda_msg(_e, #call)); return 1; } \
    } while (0)

// ---------------------------------------------------------------------------
// TIFF reader (host).
// ---------------------------------------------------------------------------
struct TiffStrip {
    uint64_t offset, bytes;
};

struct imfcs_tiff {
    FILE *f = nullptr;
    bool swap = false;                       // file byte order differs from the host's
    int width = 0, height = 0, frames = 0;
    std::vector<std::vector<TiffStrip>> strips;   // per IFD frame
    bool contiguous = false;                 // ImageJ: frames after the first IFD's data
    uint64_t base = 0;                       // contiguous: offset of frame 0
    uint16_t *pinned[2] = {nullptr, nullptr};
    size_t pinned_bytes = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done[2] = {};
    ~imfcs_tiff()
    {
        if (stream) cudaStreamSynchronize(stream);
        for (int i = 0; i < 2; i++) {
            if (pinned[i]) cudaFreeHost(pinned[i]);
            if (done[i]) cudaEventDestroy(done[i]);
        }
        if (stream) cudaStreamDestroy(stream);
        if (f) fclose(f);
    }
};

static bool host_little_endian()
{
    const uint16_t v = 1;
    unsigned char c;
    memcpy(&c, &v, 1);
    return c == 1;
}

static uint16_t bswap16(uint16_t v) { return (uint16_t)((v >> 8) | (v << 8)); }
static uint32_t bswap32(uint32_t v)
{
    return (v >> 24) | ((v >> 8) & 0xff00u) | ((v << 8) & 0xff0000u) | (v << 24);
}

static bool rd(imfcs_tiff *t, uint64_t off, void *dst, size_t n)
{
    if (fseeko(t->f, (off_t)off, SEEK_SET) != 0) return false;
    return fread(dst, 1, n, t->f) == n;
}

static bool rd16(imfcs_tiff *t, uint64_t off, uint16_t &v)
{
    if (!rd(t, off, &v, 2)) return false;
    if (t->swap) v = bswap16(v);
    return true;
}

static bool rd32(imfcs_tiff *t, uint64_t off, uint32_t &v)
{
    if (!rd(t, off, &v, 4)) return false;
    if (t->swap) v = bswap32(v);
    return true;
}

// The values of a SHORT or LONG entry (inline when they fit in 4 bytes).
static bool entry_values(imfcs_tiff *t, uint64_t entry, uint16_t type, uint32_t count, std::vector<uint64_t> &out)
{
    const int sz = type == 3 ? 2 : (type == 4 ? 4 : 0);
    if (!sz) return false;
    uint64_t at = entry + 8;
    if ((uint64_t)sz * count > 4) {
        uint32_t o;
        if (!rd32(t, entry + 8, o)) return false;
        at = o;
    }
    out.resize(count);
    for (uint32_t i = 0; i < count; i++) {
        if (sz == 2) {
            uint16_t v;
            if (!rd16(t, at + 2 * (uint64_t)i, v)) return false;
            out[i] = v;
        } else {
            uint32_t v;
            if (!rd32(t, at + 4 * (uint64_t)i, v)) return false;
            out[i] = v;
        }
    }
    return true;
}

static int tiff_fail(imfcs_tiff *t, const std::string &m)
{
    delete t;
    set_error(m);
    return 1;
}

extern "C" int imfcs_tiff_open(const char *path, imfcs_tiff **out, int *width, int *height, int *frames)
{
    if (!out || !path) { set_error("null argument"); return 1; }
    *out = nullptr;
    imfcs_tiff *t = new imfcs_tiff();
    t->f = fopen(path, "rb");
    if (!t->f) return tiff_fail(t, std::string("cannot open ") + path);
    unsigned char hdr[8];
    if (fread(hdr, 1, 8, t->f) != 8) return tiff_fail(t, "not a TIFF file (short header)");
    bool file_le;
    if (hdr[0] == 'I' && hdr[1] == 'I') file_le = true;
    else if (hdr[0] == 'M' && hdr[1] == 'M') file_le = false;
    else return tiff_fail(t, "not a TIFF file");
    t->swap = file_le != host_little_endian();
    uint16_t magic;
    if (!rd16(t, 2, magic)) return tiff_fail(t, "not a TIFF file");
    if (magic == 43) return tiff_fail(t, "BigTIFF is not supported");
    if (magic != 42) return tiff_fail(t, "not a TIFF file");
    uint32_t ifd;
    if (!rd32(t, 4, ifd)) return tiff_fail(t, "not a TIFF file");
    long images = 0;
    int nifd = 0;
    while (ifd != 0) {
        if (++nifd > 10000000) return tiff_fail(t, "TIFF: too many IFDs");
        uint16_t n;
        if (!rd16(t, ifd, n)) return tiff_fail(t, "TIFF: truncated IFD");
        uint64_t w = 0, h = 0, bps = 1, spp = 1, comp = 1, fmt = 1;
        std::vector<uint64_t> offs, cnts;
        for (int e = 0; e < n; e++) {
            const uint64_t ent = (uint64_t)ifd + 2 + 12 * (uint64_t)e;
            uint16_t tag, type;
            uint32_t count;
            if (!rd16(t, ent, tag) || !rd16(t, ent + 2, type) || !rd32(t, ent + 4, count))
                return tiff_fail(t, "TIFF: truncated IFD entry");
            std::vector<uint64_t> v;
            if (tag == 270 && nifd == 1 && type == 2 && count <= (1u << 20)) {
                // ImageJ's description: "ImageJ=...\nimages=N\n..."
                uint32_t o = 0;
                std::string d(count, '\0');
                if (count > 4) {
                    if (!rd32(t, ent + 8, o) || !rd(t, o, &d[0], count)) return tiff_fail(t, "TIFF: bad description");
                } else if (!rd(t, ent + 8, &d[0], count)) {
                    return tiff_fail(t, "TIFF: bad description");
                }
                const size_t p = d.find("images=");
                if (d.compare(0, 7, "ImageJ=") == 0 && p != std::string::npos) images = atol(d.c_str() + p + 7);
                continue;
            }
            if (tag != 256 && tag != 257 && tag != 258 && tag != 259 && tag != 273 && tag != 277 && tag != 279 &&
                tag != 339)
                continue;
            if (!entry_values(t, ent, type, count, v) || v.empty()) return tiff_fail(t, "TIFF: bad entry");
            switch (tag) {
            case 256: w = v[0]; break;
            case 257: h = v[0]; break;
            case 258: bps = v[0]; break;
            case 259: comp = v[0]; break;
            case 273: offs = v; break;
            case 277: spp = v[0]; break;
            case 279: cnts = v; break;
            case 339: fmt = v[0]; break;
            }
        }
        if (bps != 16 || spp != 1) return tiff_fail(t, "TIFF: only 16-bit single-channel images are supported");
        if (comp != 1) return tiff_fail(t, "TIFF: compressed images are not supported");
        if (fmt != 1) return tiff_fail(t, "TIFF: only unsigned integer samples are supported");
        if (w == 0 || h == 0 || w > 65535 || h > 65535 || offs.empty() || offs.size() != cnts.size())
            return tiff_fail(t, "TIFF: bad image geometry or strips");
        if (nifd == 1) {
            t->width = (int)w;
            t->height = (int)h;
        } else if ((int)w != t->width || (int)h != t->height) {
            return tiff_fail(t, "TIFF: frames of different sizes");
        }
        std::vector<TiffStrip> st(offs.size());
        uint64_t total = 0;
        for (size_t i = 0; i < offs.size(); i++) {
            st[i] = {offs[i], cnts[i]};
            total += cnts[i];
        }
        if (total != 2 * w * h) return tiff_fail(t, "TIFF: strip sizes do not match the frame size");
        t->strips.push_back(st);
        uint32_t next;
        if (!rd32(t, (uint64_t)ifd + 2 + 12 * (uint64_t)n, next)) return tiff_fail(t, "TIFF: truncated IFD");
        ifd = next;
    }
    t->frames = (int)t->strips.size();
    if (images > t->frames) {
        // ImageJ stack written as one IFD: contiguous frames from the first
        // frame's (single, contiguous) data
        const auto &s0 = t->strips[0];
        for (size_t i = 1; i < s0.size(); i++)
            if (s0[i].offset != s0[i - 1].offset + s0[i - 1].bytes)
                return tiff_fail(t, "TIFF: ImageJ stack with non-contiguous first frame");
        t->contiguous = true;
        t->base = s0[0].offset;
        t->frames = (int)images;
        const uint64_t need = t->base + 2ull * t->width * t->height * (uint64_t)images;
        if (fseeko(t->f, 0, SEEK_END) != 0 || (uint64_t)ftello(t->f) < need)
            return tiff_fail(t, "TIFF: file shorter than its ImageJ stack");
    }
    *out = t;
    if (width) *width = t->width;
    if (height) *height = t->height;
    if (frames) *frames = t->frames;
    return 0;
}

// Frames [first, first + count) into host memory (native byte order).
static int tiff_read_frames(imfcs_tiff *t, int first, int count, uint16_t *dst)
{
    const size_t fpx = (size_t)t->width * t->height;
    if (t->contiguous) {
        if (!rd(t, t->base + 2 * fpx * (uint64_t)first, dst, 2 * fpx * (size_t)count)) {
            set_error("TIFF: read failed");
            return 1;
        }
    } else {
        for (int k = 0; k < count; k++) {
            unsigned char *p = (unsigned char *)(dst + fpx * k);
            for (const auto &s : t->strips[first + k]) {
                if (!rd(t, s.offset, p, s.bytes)) { set_error("TIFF: read failed"); return 1; }
                p += s.bytes;
            }
        }
    }
    if (t->swap) {
        const size_t n = fpx * (size_t)count;
        for (size_t i = 0; i < n; i++) dst[i] = bswap16(dst[i]);
    }
    return 0;
}

extern "C" int imfcs_tiff_read(imfcs_tiff *t, int first, int count, uint16_t *host_out)
{
    if (!t || !host_out) { set_error("null argument"); return 1; }
    if (first < 0 || count < 0 || first + count > t->frames) { set_error("TIFF: frame range outside the stack"); return 1; }
    return tiff_read_frames(t, first, count, host_out);
}

extern "C" int imfcs_tiff_read_device(imfcs_tiff *t, int first, int count, uint16_t *dev_out, void *stream)
{
    if (!t || !dev_out) { set_error("null argument"); return 1; }
    if (first < 0 || count < 0 || first + count > t->frames) { set_error("TIFF: frame range outside the stack"); return 1; }
    const size_t fbytes = 2 * (size_t)t->width * t->height;
    const size_t chunk_bytes = 64ull << 20;
    const int chunk = (int)std::max<size_t>(1, chunk_bytes / fbytes);
    if (!t->pinned[0]) {
        t->pinned_bytes = fbytes * chunk;
        for (int i = 0; i < 2; i++) {
            CK(cudaHostAlloc((void **)&t->pinned[i], t->pinned_bytes, cudaHostAllocDefault));
            CK(cudaEventCreateWithFlags(&t->done[i], cudaEventDisableTiming));
        }
        CK(cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking));
    }
    cudaStream_t s = (cudaStream_t)stream;
    int b = 0;
    for (int k0 = 0; k0 < count; k0 += chunk, b ^= 1) {
        const int n = std::min(chunk, count - k0);
        CK(cudaEventSynchronize(t->done[b]));   // the copy that last read this buffer
        if (tiff_read_frames(t, first + k0, n, t->pinned[b])) return 1;
        CK(cudaMemcpyAsync((char *)dev_out + fbytes * k0, t->pinned[b], fbytes * n, cudaMemcpyHostToDevice,
                           t->stream));
        CK(cudaEventRecord(t->done[b], t->stream));
    }
    // the caller's stream sees the frames
    CK(cudaEventRecord(t->done[b], t->stream));
    CK(cudaStreamWaitEvent(s, t->done[b], 0));
    return 0;
}

extern "C" int imfcs_tiff_close(imfcs_tiff *t)
{
    delete t;
    return 0;
}

// ---------------------------------------------------------------------------
// Background statistics (loadBGRFile).
// ---------------------------------------------------------------------------
// One thread per pixel: exact integer sums over the frames.
__global__ void bg_pixel_kernel(const uint16_t *st, int npx, int frames, double *mean, double *var, double *covar)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npx) return;
    unsigned long long s = 0, s2 = 0, sxy = 0;
    unsigned int prev = st[p];
    s = prev;
    s2 = (unsigned long long)prev * prev;
    for (int t = 1; t < frames; t++) {
        const unsigned int v = st[(size_t)t * npx + p];
        s += v;
        s2 += (unsigned long long)v * v;
        sxy += (unsigned long long)prev * v;
        prev = v;
    }
    const unsigned int first = st[p], last = prev;
    const double f = (double)frames, f1 = (double)(frames - 1);
    // java:7079-7083: means of frames 1..f-1 and 2..f, covariance
    const double m1 = __ddiv_rn((double)(s - last), f1), m2 = __ddiv_rn((double)(s - first), f1);
    if (covar) covar[p] = __dsub_rn(__ddiv_rn((double)sxy, f1), __dmul_rn(m1, m2));
    // java:7098-7103: mean and variance over all frames
    const double m = __ddiv_rn((double)s, f);
    if (mean) mean[p] = m;
    if (var) var[p] = __dsub_rn(__ddiv_rn((double)s2, f), __dmul_rn(m, m));
}

// Per frame, exact integer sums of each row (rs[t][h]) and each column
// (cs[t][w]).
__global__ void bg_line_sums_kernel(const uint16_t *st, int w, int h, int frames, long long *rs, long long *cs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = blockIdx.y;
    if (t >= frames) return;
    const uint16_t *fr = st + (size_t)t * w * h;
    if (i < h) {
        long long a = 0;
        for (int x = 0; x < w; x++) a += fr[(size_t)i * w + x];
        rs[(size_t)t * h + i] = a;
    } else if (i < h + w) {
        const int x = i - h;
        long long a = 0;
        for (int y = 0; y < h; y++) a += fr[(size_t)y * w + x];
        cs[(size_t)t * w + x] = a;
    }
}

// java:7038-7058: mean[l] = sum over frames, in frame order, of
// line_sum / (len * frames), in FP64.
__global__ void bg_line_means_kernel(const long long *sums, int nlines, int frames, int len, double *out)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nlines) return;
    const double d = (double)(len * frames);
    double acc = 0.0;
    for (int t = 0; t < frames; t++) acc = __dadd_rn(acc, __ddiv_rn((double)sums[(size_t)t * nlines + l], d));
    out[l] = acc;
}

extern "C" int imfcs_background_stats(const uint16_t *dev_stack, int width, int height, int frames,
                                      double *mean, double *var, double *covar, double *row_mean,
                                      double *col_mean, void *stream)
{
    if (!dev_stack || width <= 0 || height <= 0 || frames < 2) {
        set_error("background statistics need a stack of at least two frames");
        return 1;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int npx = width * height;
    if (mean || var || covar)
        bg_pixel_kernel<<<(npx + 255) / 256, 256, 0, s>>>(dev_stack, npx, frames, mean, var, covar);
    CK(cudaGetLastError());
    if (row_mean || col_mean) {
        long long *sums = nullptr;
        CK(cudaMallocAsync((void **)&sums, sizeof(long long) * (size_t)frames * (width + height), s));
        long long *rs = sums, *cs = sums + (size_t)frames * height;
        const dim3 g((width + height + 127) / 128, frames);
        bg_line_sums_kernel<<<g, 128, 0, s>>>(dev_stack, width, height, frames, rs, cs);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess && row_mean) {
            bg_line_means_kernel<<<(height + 63) / 64, 64, 0, s>>>(rs, height, frames, width, row_mean);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess && col_mean) {
            bg_line_means_kernel<<<(width + 63) / 64, 64, 0, s>>>(cs, width, frames, height, col_mean);
            e = cudaGetLastError();
        }
        cudaError_t e2 = cudaFreeAsync(sums, s);
        if (e == cudaSuccess) e = e2;
        if (e != cudaSuccess) { set_error(cuda_msg(e, "background line means")); return 1; }
    }
    return 0;
}
