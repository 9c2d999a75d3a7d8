// lyap_capi.cu -- the C ABI (include/lyap_gb300.h): argument checking, error
// reporting, scratch management and the host-buffer wrappers.  Nothing here
// exits the process (the reference's helper_cuda checks do); every failure
// returns a negative LYAP_ERR_* code and leaves a message for
// lyap_last_error_string().
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "lyap_device.cuh"
#include "lyap_gb300.h"
#include "lyap_internal.h"
#include "lyap_jit.h"

namespace lyapgb {

static thread_local char g_err[512] = "";

int set_error(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int cuda_error(cudaError_t e, const char *what)
{
    int code = LYAP_ERR_CUDA;
    if (e == cudaErrorMemoryAllocation) code = LYAP_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice ||
        e == cudaErrorInvalidDevice)
        code = LYAP_ERR_NO_DEVICE;
    return set_error(code, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

// Scratch and the host-buffer calls' device copies come from a stream-ordered
// memory pool the library creates per device, which keeps up to
// LYAP_POOL_KEEP_MB (default 1024) MiB of freed memory between calls.  The
// device's default pool keeps nothing: every stream synchronisation hands
// its memory back, and the next call maps it again (for lyap_render_host at
// 1080p, 92 MB per call) while the GPU waits.  Without a pool of its own
// (creation failed) the library allocates from the default pool.
static uint64_t pool_keep_bytes()
{
    const char *v = getenv("LYAP_POOL_KEEP_MB");
    if (v && *v) {
        char *end = nullptr;
        const unsigned long long mb = strtoull(v, &end, 10);
        if (end && *end == '\0') return (uint64_t)mb << 20;
    }
    return (uint64_t)1024 << 20;
}

cudaError_t scratch_alloc(void **p, size_t bytes, cudaStream_t s)
{
    static std::mutex mu;
    static cudaMemPool_t pools[64];
    static bool tried[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaMallocAsync(p, bytes, s);
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!tried[dev]) {
            tried[dev] = true;
            cudaMemPoolProps props;
            memset(&props, 0, sizeof(props));
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            cudaMemPool_t created = nullptr;
            if (cudaMemPoolCreate(&created, &props) == cudaSuccess) {
                uint64_t keep = pool_keep_bytes();
                cudaMemPoolSetAttribute(created, cudaMemPoolAttrReleaseThreshold, &keep);
                pools[dev] = created;
            } else {
                (void)cudaGetLastError();   // not sticky: fall back to the default pool
            }
        }
        pool = pools[dev];
    }
    if (!pool) return cudaMallocAsync(p, bytes, s);
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

static int check_params(const LyapParams *prm, const char *fn)
{
    if (!prm) return set_error(LYAP_ERR_INVALID_ARG, "%s: null params", fn);
    return LYAP_OK;
}

static int check_seq_len(size_t seq_len, const char *fn)
{
    if (seq_len < 2 || seq_len > LYAP_MAX_SEQ_LEN)
        return set_error(LYAP_ERR_SEQUENCE, "%s: seq_len %zu outside [2, %d] (entries incl. the -1)", fn, seq_len,
                         LYAP_MAX_SEQ_LEN);
    return LYAP_OK;
}

static int check_host_seq(const int32_t *seq, size_t seq_len, const char *fn)
{
    if (!seq) return set_error(LYAP_ERR_INVALID_ARG, "%s: null sequence", fn);
    int rc = check_seq_len(seq_len, fn);
    if (rc) return rc;
    for (size_t i = 0; i + 1 < seq_len; i++)
        if (seq[i] < 0 || seq[i] > 3)
            return set_error(LYAP_ERR_SEQUENCE, "%s: symbol %d at %zu is not 0..3", fn, seq[i], i);
    if (seq[seq_len - 1] != -1) return set_error(LYAP_ERR_SEQUENCE, "%s: sequence is not -1 terminated", fn);
    return LYAP_OK;
}

// the proposal fields exist only in the full-size struct
const LyapNet *ext_proposal(const LyapRenderExt *ext)
{
    return (ext && ext->size == sizeof(LyapRenderExt)) ? ext->proposal : nullptr;
}

static int check_ext_render(const LyapRenderExt *ext, const LyapParams *prm, const char *fn)
{
    if (!ext) return LYAP_OK;
    if (ext->size != sizeof(LyapRenderExt) && ext->size != offsetof(LyapRenderExt, proposal))
        return set_error(LYAP_ERR_INVALID_ARG, "%s: LyapRenderExt.size is %u, expected %zu (or %zu)", fn, ext->size,
                         sizeof(LyapRenderExt), offsetof(LyapRenderExt, proposal));
    if (const LyapNet *net = ext_proposal(ext)) {
        if (net->magic != LYAP_NET_MAGIC || net->version != LYAP_NET_VERSION)
            return set_error(LYAP_ERR_INVALID_ARG, "%s: proposal is not a LyapNet (magic %08x, version %u)", fn,
                             net->magic, net->version);
        for (int k = 0; k < 3; k++)
            if (!(net->hi[k] > net->lo[k]))
                return set_error(LYAP_ERR_INVALID_ARG, "%s: proposal net has an empty box on axis %d", fn, k);
        if (!std::isfinite(ext->proposal_margin) || ext->proposal_margin < 0.0f)
            return set_error(LYAP_ERR_INVALID_ARG, "%s: proposal_margin must be finite and >= 0", fn);
        if (ext->proposal_grid == 1 || ext->proposal_grid > 512)
            return set_error(LYAP_ERR_INVALID_ARG, "%s: proposal_grid %u outside 2..512", fn, ext->proposal_grid);
        if (ext->proposal_segment > 64)
            return set_error(LYAP_ERR_INVALID_ARG, "%s: proposal_segment %u > 64", fn, ext->proposal_segment);
        if (ext->proposal_dilate > 1)
            return set_error(LYAP_ERR_INVALID_ARG, "%s: proposal_dilate must be 0 or 1", fn);
        if (prm->jitter != 0.0f || prm->nearMultiplier != 1.0f)
            return set_error(LYAP_ERR_INVALID_ARG,
                             "%s: the proposal needs a fixed step (jitter 0, nearMultiplier 1)", fn);
    }
    if (ext->variant > LYAP_VARIANT_PRODUCT) return set_error(LYAP_ERR_INVALID_ARG, "%s: unknown variant %u", fn, ext->variant);
    if (ext->light_model > LYAP_LIGHT_DIRECTIONAL)
        return set_error(LYAP_ERR_INVALID_ARG, "%s: unknown light model %u", fn, ext->light_model);
    if (ext->threads_per_block && (ext->threads_per_block % 32 || ext->threads_per_block > 128))
        return set_error(LYAP_ERR_INVALID_ARG, "%s: threads_per_block must be a multiple of 32, at most 128", fn);
    return LYAP_OK;
}

static int check_ext_volume(const LyapVolumeExt *ext, const char *fn)
{
    if (!ext) return LYAP_OK;
    if (ext->size != sizeof(LyapVolumeExt))
        return set_error(LYAP_ERR_INVALID_ARG, "%s: LyapVolumeExt.size is %u, expected %zu", fn, ext->size,
                         sizeof(LyapVolumeExt));
    if (ext->variant > LYAP_VARIANT_PRODUCT) return set_error(LYAP_ERR_INVALID_ARG, "%s: unknown variant %u", fn, ext->variant);
    if (ext->threads_per_block && (ext->threads_per_block % 32 || ext->threads_per_block > 256))
        return set_error(LYAP_ERR_INVALID_ARG, "%s: threads_per_block must be a multiple of 32, at most 256", fn);
    return LYAP_OK;
}

int check_render_args(const LyapCam *cam, const LyapParams *prm, const void *seq, size_t seq_len,
                             const void *lights, uint32_t n_lights, const void *rgba, const void *points,
                             uint32_t width, uint32_t height, const LyapRenderExt *ext, const char *fn)
{
    if (!cam) return set_error(LYAP_ERR_INVALID_ARG, "%s: null camera", fn);
    int rc = check_params(prm, fn);
    if (rc) return rc;
    if (!seq) return set_error(LYAP_ERR_INVALID_ARG, "%s: null sequence", fn);
    if ((rc = check_seq_len(seq_len, fn))) return rc;
    if (n_lights > LYAP_MAX_LIGHTS) return set_error(LYAP_ERR_INVALID_ARG, "%s: %u lights > %d", fn, n_lights, LYAP_MAX_LIGHTS);
    if (n_lights && !lights) return set_error(LYAP_ERR_INVALID_ARG, "%s: null lights", fn);
    if (!rgba) return set_error(LYAP_ERR_INVALID_ARG, "%s: null rgba output", fn);
    if (!points) return set_error(LYAP_ERR_INVALID_ARG, "%s: null points output", fn);
    if (width == 0 || height == 0) return set_error(LYAP_ERR_INVALID_ARG, "%s: zero image size %ux%u", fn, width, height);
    if ((uint64_t)width * height > LYAP_MAX_PIXELS)
        return set_error(LYAP_ERR_INVALID_ARG, "%s: %ux%u exceeds %llu pixels", fn, width, height,
                         (unsigned long long)LYAP_MAX_PIXELS);
    return check_ext_render(ext, prm, fn);
}

RenderJob make_job(const LyapCam *cam, const LyapParams *prm, const int32_t *d_seq, size_t seq_len,
                          const LyapLight *d_lights, uint32_t n_lights, RGBA *d_rgba, LyapPoint *d_points,
                          uint32_t width, uint32_t height, const LyapRenderExt *ext)
{
    RenderJob job;
    memset(&job, 0, sizeof(job));
    job.cam = *cam;
    job.prm = *prm;
    job.seq = d_seq;
    job.lights = d_lights;
    job.rgba = d_rgba;
    job.points = d_points;
    job.counts = ext ? ext->d_counts : nullptr;
    job.seq_period = (uint32_t)(seq_len - 1);
    job.n_lights = n_lights;
    job.width = width;
    job.height = height;
    job.light_model = ext ? ext->light_model : LYAP_LIGHT_SPOT;
    job.flags = ext ? ext->flags : 0u;
    return job;
}

}  // namespace lyapgb

using namespace lyapgb;

extern "C" {

int lyap_abi_version(void) { return LYAP_ABI_VERSION; }

const char *lyap_version(void) { return "lyapunov3d_gb300 " LYAP_VERSION_STRING " (sm_103a)"; }

const char *lyap_last_error_string(void) { return g_err; }

const char *lyap_status_string(int code)
{
    switch (code) {
    case LYAP_OK: return "ok";
    case LYAP_ERR_INVALID_ARG: return "invalid argument";
    case LYAP_ERR_SEQUENCE: return "bad sequence";
    case LYAP_ERR_CUDA: return "CUDA error";
    case LYAP_ERR_NO_DEVICE: return "no usable sm_103 device";
    case LYAP_ERR_OUT_OF_MEMORY: return "out of device memory";
    case LYAP_ERR_CAPACITY: return "output buffer too small";
    case LYAP_ERR_JIT: return "specialised kernel unavailable";
    default: return "unknown status";
    }
}

int lyap_render(const LyapCam *cam, const LyapParams *prm, const int32_t *d_seq, size_t seq_len,
                const LyapLight *d_lights, uint32_t n_lights, RGBA *d_rgba, LyapPoint *d_points, uint32_t width,
                uint32_t height, const LyapRenderExt *ext, void *stream)
{
    int rc = check_render_args(cam, prm, d_seq, seq_len, d_lights, n_lights, d_rgba, d_points, width, height, ext,
                               "lyap_render");
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    RenderJob job = make_job(cam, prm, d_seq, seq_len, d_lights, n_lights, d_rgba, d_points, width, height, ext);
    // the learned proposal's grid over the net's box: built on this stream on
    // first use (then cached per device and net), read by the march
    if (const LyapNet *net = ext_proposal(ext)) {
        const uint32_t n = ext->proposal_grid ? ext->proposal_grid : LYAP_PROPOSAL_GRID_DEFAULT;
        const uint32_t seg = ext->proposal_segment ? ext->proposal_segment : 8u;
        const float tau = prm->opaqueThreshold + ext->proposal_margin;
        const uint32_t *bits = nullptr;
        cudaError_t ge = proposal_bits(*net, n, ext->proposal_dilate, tau, &bits, ext->d_stats, s);
        if (ge != cudaSuccess) return cuda_error(ge, "lyap_render: proposal grid");
        job.prop.bits = bits;
        job.prop.n = n;
        job.prop.run = seg - 1;
        for (int k = 0; k < 3; k++) {
            job.prop.lo[k] = net->lo[k];
            job.prop.scale[k] = (float)n / (net->hi[k] - net->lo[k]);
        }
        job.prop.tau = tau;
        const uint64_t words = ((uint64_t)n * n * n + 31) / 32;
        job.prop.smem_words = words * 4 <= LYAP_PROPOSAL_SMEM_MAX ? (uint32_t)words : 0u;
    }
    // scratch, stream-ordered so concurrent calls on different streams each
    // get their own: a 256-byte header (the queue's counter, the ray list's
    // length), the list of rays that meet the box (ray_list); with FP64
    // bisection also the per-pixel crossing brackets and the list of pixels
    // that crossed (scratch of the two passes)
    const bool bisect = ext && (ext->flags & LYAP_FLAG_BISECT_F64);
    const size_t npix = (size_t)width * height;
    const size_t bisect_bytes = bisect ? 256 + (((npix + 1) * sizeof(uint32_t) + 255) & ~(size_t)255) +
                                             npix * 2 * sizeof(float)
                                       : 256;
    const size_t list_off = (bisect_bytes + 255) & ~(size_t)255;
    const size_t scratch = list_off + npix * sizeof(RayEntry);
    uint32_t *d_counter = nullptr;
    cudaError_t e = scratch_alloc((void **)&d_counter, scratch, s);
    if (e != cudaSuccess) return cuda_error(e, "lyap_render: scratch allocation");
    e = cudaMemsetAsync(d_counter, 0, 2 * sizeof(uint32_t), s);
    job.list = reinterpret_cast<RayEntry *>(reinterpret_cast<char *>(d_counter) + list_off);
    job.list_count = d_counter + 1;
    if (e == cudaSuccess)
        e = launch_ray_list(job, const_cast<RayEntry *>(job.list), d_counter + 1, ext ? ext->d_stats : nullptr, s);
    if (e == cudaSuccess && bisect) {
        char *base = reinterpret_cast<char *>(d_counter);
        job.hits = reinterpret_cast<uint32_t *>(base + 256);
        job.bracket = reinterpret_cast<float *>(base + 256 + (((npix + 1) * sizeof(uint32_t) + 255) & ~(size_t)255));
        e = cudaMemsetAsync(job.hits, 0, sizeof(uint32_t), s);
    }
    if (e == cudaSuccess) {
        const uint32_t variant = ext ? ext->variant : LYAP_VARIANT_PLAIN;
        const uint32_t flags = ext ? ext->flags : 0u;
        bool launched = false;
        if (ext && ext->h_seq && !(flags & LYAP_FLAG_NO_JIT)) {
            std::string why;
            cudaError_t le = cudaSuccess;
            if (jit_launch_render(job, variant, ext->h_seq, d_counter, ext->d_stats, ext->blocks_per_sm,
                                  ext->threads_per_block, s, &le, &why)) {
                e = le;
                launched = true;
            } else if (flags & LYAP_FLAG_REQUIRE_JIT) {
                cudaFreeAsync(d_counter, s);
                return set_error(LYAP_ERR_JIT, "lyap_render: specialised kernel unavailable: %s", why.c_str());
            }
        } else if (flags & LYAP_FLAG_REQUIRE_JIT) {
            cudaFreeAsync(d_counter, s);
            return set_error(LYAP_ERR_JIT, "lyap_render: LYAP_FLAG_REQUIRE_JIT needs ext->h_seq");
        }
        if (!launched)
            e = launch_render(job, variant, d_counter, ext ? ext->d_stats : nullptr, ext ? ext->blocks_per_sm : 0,
                              ext ? ext->threads_per_block : 0, s);
        if (e == cudaSuccess && bisect)
            e = launch_bisect(job, variant, ext->bisect_halvings ? ext->bisect_halvings : 20u, ext->d_stats, s);
    }
    cudaError_t e2 = cudaFreeAsync(d_counter, s);
    if (e != cudaSuccess) return cuda_error(e, "lyap_render: launch");
    if (e2 != cudaSuccess) return cuda_error(e2, "lyap_render: scratch release");
    return LYAP_OK;
}

int lyap_volume(float *d_out, uint32_t nx, uint32_t ny, uint32_t nz, const float *lo, const float *hi,
                const LyapParams *prm, const int32_t *d_seq, size_t seq_len, const LyapVolumeExt *ext, void *stream)
{
    int rc = check_params(prm, "lyap_volume");
    if (rc) return rc;
    if (!d_out) return set_error(LYAP_ERR_INVALID_ARG, "lyap_volume: null output");
    if (!d_seq) return set_error(LYAP_ERR_INVALID_ARG, "lyap_volume: null sequence");
    if ((rc = check_seq_len(seq_len, "lyap_volume"))) return rc;
    if (nx == 0 || ny == 0 || nz == 0) return set_error(LYAP_ERR_INVALID_ARG, "lyap_volume: zero dimension");
    if ((uint64_t)nx * ny * nz > LYAP_MAX_VOXELS)
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_volume: %ux%ux%u exceeds %llu voxels", nx, ny, nz,
                         (unsigned long long)LYAP_MAX_VOXELS);
    if ((rc = check_ext_volume(ext, "lyap_volume"))) return rc;
    VolumeJob job;
    memset(&job, 0, sizeof(job));
    job.out = d_out;
    job.seq = d_seq;
    job.prm = *prm;
    job.seq_period = (uint32_t)(seq_len - 1);
    job.nx = nx;
    job.ny = ny;
    job.nz = nz;
    for (int k = 0; k < 3; k++) {
        job.lo[k] = lo ? lo[k] : 0.0f;   // kernel.cu:527-529: [0, 4) when not given
        job.hi[k] = hi ? hi[k] : 4.0f;
    }
    const uint32_t variant = ext ? ext->variant : LYAP_VARIANT_PLAIN;
    const uint32_t flags = ext ? ext->flags : 0u;
    cudaError_t e = cudaSuccess;
    bool launched = false;
    if (ext && ext->h_seq && !(flags & LYAP_FLAG_NO_JIT)) {
        std::string why;
        if (jit_launch_volume(job, variant, ext->h_seq, ext->d_stats, ext->blocks_per_sm, ext->threads_per_block,
                              (cudaStream_t)stream, &e, &why))
            launched = true;
        else if (flags & LYAP_FLAG_REQUIRE_JIT)
            return set_error(LYAP_ERR_JIT, "lyap_volume: specialised kernel unavailable: %s", why.c_str());
    } else if (flags & LYAP_FLAG_REQUIRE_JIT) {
        return set_error(LYAP_ERR_JIT, "lyap_volume: LYAP_FLAG_REQUIRE_JIT needs ext->h_seq");
    }
    if (!launched)
        e = launch_volume(job, variant, ext ? ext->d_stats : nullptr, ext ? ext->blocks_per_sm : 0,
                          ext ? ext->threads_per_block : 0, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_error(e, "lyap_volume: launch");
    return LYAP_OK;
}

}  // extern "C"

namespace {

// The device address of a host output buffer the kernels can store into
// directly, or null.  Page-locked host memory that the runtime has mapped into
// the device's address space (allocated with cudaHostAlloc / cudaMallocHost,
// or registered with cudaHostRegister) has one; the runtime reports it for the
// first and the last byte of the range, which must lie in the same mapping.
// On Grace-Blackwell the volume sweep's coalesced streaming stores then reach
// host memory over NVLink-C2C while it runs, and no download follows (512^3:
// 18.0 ms per call instead of 20.8 with the staging copy).  Pageable memory,
// and anything the runtime cannot describe, takes the staging copy.
void *mapped_host_view(void *host, size_t bytes)
{
    if (!host || bytes == 0) return nullptr;
    cudaPointerAttributes a, b;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    if (cudaPointerGetAttributes(&b, static_cast<char *>(host) + bytes - 1) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    if (b.type != cudaMemoryTypeHost || !b.devicePointer ||
        static_cast<char *>(b.devicePointer) - static_cast<char *>(a.devicePointer) != (ptrdiff_t)(bytes - 1))
        return nullptr;
    return a.devicePointer;
}

}  // namespace

extern "C" {

int lyap_render_host(const LyapCam *cam, const LyapParams *prm, const int32_t *seq, size_t seq_len,
                     const LyapLight *lights, uint32_t n_lights, RGBA *rgba, LyapPoint *points, uint32_t width,
                     uint32_t height, const LyapRenderExt *ext, void *stream)
{
    int rc = check_render_args(cam, prm, seq, seq_len, lights, n_lights, rgba, (void *)1, width, height, ext,
                               "lyap_render_host");
    if (rc) return rc;
    if ((rc = check_host_seq(seq, seq_len, "lyap_render_host"))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t npix = (size_t)width * height;
    const size_t seq_b = seq_len * sizeof(int32_t), light_b = (size_t)n_lights * sizeof(LyapLight);
    const size_t rgba_b = npix * sizeof(RGBA), pts_b = npix * sizeof(LyapPoint);
    // one device block: [seq | lights | rgba | points], 256-byte aligned parts.
    // The outputs are always staged in device memory and downloaded in one
    // copy each, page-locked or not: the render finishes pixels in scattered
    // order, and storing them straight into mapped host memory over
    // NVLink-C2C made the 1080p frame 1.8 ms slower than the 83 MB download.
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t off_l = up(seq_b), off_r = off_l + up(light_b), off_p = off_r + up(rgba_b);
    const size_t total = off_p + up(pts_b);
    char *dev = nullptr;
    cudaError_t e = scratch_alloc((void **)&dev, total, s);
    if (e != cudaSuccess) return cuda_error(e, "lyap_render_host: device buffers");
    e = cudaMemcpyAsync(dev, seq, seq_b, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && light_b) e = cudaMemcpyAsync(dev + off_l, lights, light_b, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        // the sequence is on the host here: hand it on for the specialised kernels
        LyapRenderExt x;
        memset(&x, 0, sizeof(x));
        if (ext) memcpy(&x, ext, ext->size);   // a short (older) struct: the rest stays zero
        x.size = sizeof(x);
        if (!x.h_seq) x.h_seq = seq;
        rc = lyap_render(cam, prm, (const int32_t *)dev, seq_len, (const LyapLight *)(dev + off_l), n_lights,
                         (RGBA *)(dev + off_r), (LyapPoint *)(dev + off_p), width, height, &x, stream);
        if (rc) {
            cudaFreeAsync(dev, s);
            return rc;
        }
        e = cudaMemcpyAsync(rgba, dev + off_r, rgba_b, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && points) e = cudaMemcpyAsync(points, dev + off_p, pts_b, cudaMemcpyDeviceToHost, s);
    }
    cudaError_t e2 = cudaFreeAsync(dev, s);
    cudaError_t e3 = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_error(e, "lyap_render_host: copies");
    if (e2 != cudaSuccess) return cuda_error(e2, "lyap_render_host: release");
    if (e3 != cudaSuccess) return cuda_error(e3, "lyap_render_host: synchronize");
    return LYAP_OK;
}

int lyap_volume_host(float *out, uint32_t nx, uint32_t ny, uint32_t nz, const float *lo, const float *hi,
                     const LyapParams *prm, const int32_t *seq, size_t seq_len, const LyapVolumeExt *ext,
                     void *stream)
{
    int rc = check_host_seq(seq, seq_len, "lyap_volume_host");
    if (rc) return rc;
    if (!out) return set_error(LYAP_ERR_INVALID_ARG, "lyap_volume_host: null output");
    if (nx == 0 || ny == 0 || nz == 0) return set_error(LYAP_ERR_INVALID_ARG, "lyap_volume_host: zero dimension");
    if ((uint64_t)nx * ny * nz > LYAP_MAX_VOXELS)
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_volume_host: %ux%ux%u exceeds %llu voxels", nx, ny, nz,
                         (unsigned long long)LYAP_MAX_VOXELS);
    cudaStream_t s = (cudaStream_t)stream;
    const size_t out_b = (size_t)nx * ny * nz * sizeof(float);
    // an output in mapped page-locked host memory is written in place
    float *out_direct = static_cast<float *>(mapped_host_view(out, out_b));
    const size_t seq_off = out_direct ? 0 : (out_b + 255) & ~(size_t)255;
    char *dev = nullptr;
    cudaError_t e = scratch_alloc((void **)&dev, seq_off + seq_len * sizeof(int32_t), s);
    if (e != cudaSuccess) return cuda_error(e, "lyap_volume_host: device buffers");
    e = cudaMemcpyAsync(dev + seq_off, seq, seq_len * sizeof(int32_t), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        LyapVolumeExt x;
        if (ext) {
            x = *ext;
        } else {
            memset(&x, 0, sizeof(x));
            x.size = sizeof(x);
        }
        if (!x.h_seq) x.h_seq = seq;
        rc = lyap_volume(out_direct ? out_direct : (float *)dev, nx, ny, nz, lo, hi, prm,
                         (const int32_t *)(dev + seq_off), seq_len, &x, stream);
        if (rc) {
            cudaFreeAsync(dev, s);
            return rc;
        }
        if (!out_direct) e = cudaMemcpyAsync(out, dev, out_b, cudaMemcpyDeviceToHost, s);
    }
    cudaError_t e2 = cudaFreeAsync(dev, s);
    cudaError_t e3 = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_error(e, "lyap_volume_host: copies");
    if (e2 != cudaSuccess) return cuda_error(e2, "lyap_volume_host: release");
    if (e3 != cudaSuccess) return cuda_error(e3, "lyap_volume_host: synchronize");
    return LYAP_OK;
}

}  // extern "C"
