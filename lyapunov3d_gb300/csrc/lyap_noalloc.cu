// lyap_noalloc.cu -- lyap_render_noalloc: the raymarch entry point for callers
// that must not allocate device memory.
//
// Who needs it: callers that cannot or must not allocate device memory on
// each call -- processes on devices or drivers without stream-ordered memory
// pools (cudaDevAttrMemoryPoolsSupported = 0, e.g. some virtualised GPUs),
// where lyap_render's stream-ordered allocation fails; applications that own every
// device allocation (a fixed memory budget or their own allocator) and
// forbid libraries from allocating; render loops that must not risk an
// allocation failing or blocking mid-frame when device memory runs out.
// lyap_render allocates its scratch (the pixel queue's counter and the list
// of rays that meet the box) from a stream-ordered memory pool on every call;
// this variant walks every pixel instead of a list and takes the counter
// from a small array in the library's own device memory, which exists for as
// long as the library is loaded.
//
// The scratch: g_render_noalloc_scratch, LYAP_NOALLOC_SCRATCH_BYTES (256)
// bytes per device that loads the library, of which one call uses 4 bytes
// (one 32-bit counter, reset to zero on the call's stream before the launch).
// Because every call shares the array, calls whose work overlaps on the GPU
// (different streams, or different host threads) race on the counter and
// produce wrong images; serialise them.  The counter's range also bounds the
// image: at most LYAP_MAX_PIXELS pixels.
//
// Set-up: host code cannot use the array's name as a device address (on the
// host it names a stand-in object), so the first call on each device asks
// the runtime for the address with cudaGetSymbolAddress while that device is
// current and caches it for the life of the process (a cudaDeviceReset
// destroys the context it belongs to: do not call this after one).  Make
// that first call before any stream capture.
//
// Kernels: always the precompiled ones.  The run-time specialised kernels
// are loaded into the context with cudaLibraryLoadData, which allocates, so
// ext->h_seq is ignored here and LYAP_FLAG_REQUIRE_JIT is refused.
// Nothing here calls cudaMalloc, cudaFree or any allocating routine.
#include <cuda_runtime.h>

#include <mutex>

#include "lyap_device.cuh"
#include "lyap_internal.h"

using namespace lyapgb;

namespace {

constexpr int kMaxDevices = 64;
constexpr size_t kScratchWords = LYAP_NOALLOC_SCRATCH_BYTES / sizeof(unsigned int);
constexpr size_t kWordsPerCall = 1;   // the pixel-queue counter
static_assert(kWordsPerCall <= kScratchWords, "noalloc scratch too small");

static __device__ __align__(256) unsigned int g_render_noalloc_scratch[kScratchWords];

std::mutex g_mu;
unsigned int *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch on the current device (set up once per device).
int scratch_address(unsigned int **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "lyap_render_noalloc: current device");
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(LYAP_ERR_NO_DEVICE, "lyap_render_noalloc: device %d beyond the %d supported", dev,
                         kMaxDevices);
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_render_noalloc_scratch);
        if (e != cudaSuccess) return cuda_error(e, "lyap_render_noalloc: scratch set-up (cudaGetSymbolAddress)");
        g_scratch_addr[dev] = static_cast<unsigned int *>(p);
    }
    *out = g_scratch_addr[dev];
    return LYAP_OK;
}

}  // namespace

extern "C" int lyap_render_noalloc(const LyapCam *cam, const LyapParams *prm, const int32_t *d_seq, size_t seq_len,
                                   const LyapLight *d_lights, uint32_t n_lights, RGBA *d_rgba, LyapPoint *d_points,
                                   uint32_t width, uint32_t height, const LyapRenderExt *ext, void *stream)
{
    int rc = check_render_args(cam, prm, d_seq, seq_len, d_lights, n_lights, d_rgba, d_points, width, height, ext,
                               "lyap_render_noalloc");
    if (rc) return rc;
    if (ext_proposal(ext))
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_render_noalloc: the learned proposal needs scratch memory; "
                                               "use lyap_render");
    if (ext && (ext->flags & LYAP_FLAG_REQUIRE_JIT))
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_render_noalloc: always runs the precompiled kernels "
                                               "(loading a specialised kernel allocates); drop LYAP_FLAG_REQUIRE_JIT "
                                               "or use lyap_render");
    if (ext && (ext->flags & LYAP_FLAG_BISECT_F64))
        return set_error(LYAP_ERR_INVALID_ARG,
                         "lyap_render_noalloc: LYAP_FLAG_BISECT_F64 needs per-pixel scratch; use lyap_render");
    unsigned int *scratch = nullptr;
    if ((rc = scratch_address(&scratch))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    RenderJob job = make_job(cam, prm, d_seq, seq_len, d_lights, n_lights, d_rgba, d_points, width, height, ext);
    // the queue counter must start at zero; the previous call left its final count
    cudaError_t e = cudaMemsetAsync(scratch, 0, kWordsPerCall * sizeof(unsigned int), s);
    if (e != cudaSuccess) return cuda_error(e, "lyap_render_noalloc: scratch reset");
    e = launch_render(job, ext ? ext->variant : LYAP_VARIANT_PLAIN, scratch, ext ? ext->d_stats : nullptr,
                      ext ? ext->blocks_per_sm : 0, ext ? ext->threads_per_block : 0, s);
    if (e != cudaSuccess) return cuda_error(e, "lyap_render_noalloc: launch");
    return LYAP_OK;
}
