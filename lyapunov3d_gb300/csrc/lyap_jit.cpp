// lyap_jit.cpp -- run-time specialisation of the kernels to one sequence.
//
// The lambda loop picks r for each step from {x, y, z, d} by the sequence
// symbol.  Compiled for "any sequence" (RuntimeLambda) those picks are
// per-sample registers (up to 3 per period position); compiled with the
// symbols as template constants (ConstLambda) they vanish, which frees the
// registers for more resident warps and, in the volume sweep, for several
// independent samples per thread.  When the caller hands the host copy of
// the sequence (LyapRenderExt/LyapVolumeExt.h_seq, or the *_host entry
// points), this file compiles lyap_kernels.cuh for that sequence with NVRTC
// (loaded with dlopen: the library itself does not depend on it), loads the
// cubin with the runtime's library API and launches it.  Compiled kernels
// are cached per (sequence, settle mod period) for the life of the process.
// Anything missing (NVRTC not installed, a period the specialisation does
// not cover, a compile error) sends the call to the precompiled kernels,
// which compute the same bits; LYAP_FLAG_REQUIRE_JIT turns that into an
// error, LYAP_FLAG_NO_JIT or LYAP_JIT=0 in the environment skip this path.
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "lyap_internal.h"
#include "lyap_jit.h"

namespace lyapgb {

// embedded copies of the device headers (generated at build time)
extern const int kJitHeaderCount;
extern const char *const kJitHeaderNames[];
extern const char *const kJitHeaderSources[];

namespace {

struct Nvrtc {
    void *handle = nullptr;
    decltype(&::nvrtcCreateProgram) create = nullptr;
    decltype(&::nvrtcCompileProgram) compile = nullptr;
    decltype(&::nvrtcDestroyProgram) destroy = nullptr;
    decltype(&::nvrtcGetCUBINSize) cubin_size = nullptr;
    decltype(&::nvrtcGetCUBIN) cubin = nullptr;
    decltype(&::nvrtcGetProgramLogSize) log_size = nullptr;
    decltype(&::nvrtcGetProgramLog) log = nullptr;
    decltype(&::nvrtcAddNameExpression) add_name = nullptr;
    decltype(&::nvrtcGetLoweredName) lowered = nullptr;
    decltype(&::nvrtcGetErrorString) err = nullptr;
    std::string why;   // reason it is unavailable

    bool load()
    {
        const char *names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                               "/usr/local/cuda/lib64/libnvrtc.so"};
        for (const char *n : names) {
            handle = dlopen(n, RTLD_NOW | RTLD_LOCAL);
            if (handle) break;
        }
        if (!handle) {
            why = "libnvrtc.so.13 not found";
            return false;
        }
#define LYAP_SYM(field, name)                                        \
    field = reinterpret_cast<decltype(field)>(dlsym(handle, #name)); \
    if (!field) {                                                    \
        why = "libnvrtc lacks " #name;                               \
        return false;                                                \
    }
        LYAP_SYM(create, nvrtcCreateProgram)
        LYAP_SYM(compile, nvrtcCompileProgram)
        LYAP_SYM(destroy, nvrtcDestroyProgram)
        LYAP_SYM(cubin_size, nvrtcGetCUBINSize)
        LYAP_SYM(cubin, nvrtcGetCUBIN)
        LYAP_SYM(log_size, nvrtcGetProgramLogSize)
        LYAP_SYM(log, nvrtcGetProgramLog)
        LYAP_SYM(add_name, nvrtcAddNameExpression)
        LYAP_SYM(lowered, nvrtcGetLoweredName)
        LYAP_SYM(err, nvrtcGetErrorString)
#undef LYAP_SYM
        return true;
    }
};

// One compiled specialisation: the render and volume kernels of both lambda
// forms (kind KIND_RENDER); the render kernels with the learned proposal,
// render_persistent<Lam, true> (KIND_PROPOSAL, compiled on the first render
// with a proposal); or the batch kernel of one lambda form, render_batch<Lam>
// (KIND_BATCH + form, compiled for the requests of a batch that share one
// sequence; a batch compiles several in parallel threads).
struct Entry {
    std::once_flag once;   // the compile, done once outside the cache's lock
    bool done = false;     // the compile has finished (read and written under g_mu)
    bool ok = false;
    std::string error;
    cudaLibrary_t lib = nullptr;
    cudaKernel_t render[2] = {nullptr, nullptr};   // [mode]
    cudaKernel_t volume[2] = {nullptr, nullptr};
    int render_blocks_per_sm[2][64] = {};   // per lambda form and device
    std::string log;
    double compile_ms = 0;
};

std::mutex g_mu;
Nvrtc g_nvrtc;
int g_nvrtc_state = 0;   // 0 unknown, 1 loaded, -1 unavailable
std::map<std::string, std::unique_ptr<Entry>> g_cache;
unsigned long g_compiles = 0, g_launches = 0;

bool jit_disabled_by_env()
{
    const char *v = getenv("LYAP_JIT");
    return v && (strcmp(v, "0") == 0 || strcmp(v, "off") == 0);
}

// Resident render blocks per SM the specialised kernel is compiled for (its
// register cap, blocks of jit_render_threads threads);
// LYAP_JIT_RENDER_BLOCKS=1..16 overrides the default.
// the lambda forms (the kernels' MODE_PLAIN / MODE_PRODUCT; e->render[mode])
constexpr uint32_t kModePlain = 0, kModeProduct = 1;

// paired rounds in the specialised render of lambda form `mode`: environment
// LYAP_JIT_PAIRS=0/1 overrides the default for both forms
int jit_render_pairs(uint32_t mode)
{
    const char *v = getenv("LYAP_JIT_PAIRS");
    if (v && (v[0] == '0' || v[0] == '1')) return v[0] - '0';
    return mode == kModeProduct ? LYAP_JIT_RENDER_PAIRS_PRODUCT : LYAP_JIT_RENDER_PAIRS_PLAIN;
}

int jit_render_min_blocks(uint32_t mode)
{
    const char *v = getenv("LYAP_JIT_RENDER_BLOCKS");
    if (v) {
        const int n = atoi(v);
        if (n >= 1 && n <= 16) return n;
    }
    return jit_render_pairs(mode) ? LYAP_JIT_RENDER_MIN_BLOCKS_PAIRS : LYAP_JIT_RENDER_MIN_BLOCKS;
}

// threads per block of the specialised render of lambda form `mode`
int jit_render_threads(uint32_t mode)
{
    return jit_render_pairs(mode) ? LYAP_JIT_RENDER_THREADS_PAIRS : LYAP_JIT_RENDER_THREADS;
}

std::string hex64(uint64_t v)
{
    char b[32];
    snprintf(b, sizeof(b), "0x%llxull", (unsigned long long)v);
    return b;
}

// Template arguments of one specialisation: period L, words of the settle
// and accumulation symbol tables, OA = settle mod L.
struct Spec {
    int L;
    uint32_t oA;
    uint64_t s0, s1, a0, a1;
};

Spec make_spec(const int32_t *h_seq, uint32_t L, uint32_t settle)
{
    Spec s{(int)L, settle % L, 0, 0, 0, 0};
    for (uint32_t j = 0; j < L; j++) {
        const uint64_t sym = (uint64_t)(h_seq[j] & 3);
        const uint64_t asym = (uint64_t)(h_seq[(s.oA + j) % L] & 3);
        if (j < 32) {
            s.s0 |= sym << (2 * j);
            s.a0 |= asym << (2 * j);
        } else {
            s.s1 |= sym << (2 * (j - 32));
            s.a1 |= asym << (2 * (j - 32));
        }
    }
    return s;
}

std::string lam_type(const Spec &s, int mode)
{
    const std::string L = std::to_string(s.L);
    return "lyapgb::ConstLambda<" + std::to_string(mode) + "u, " + std::to_string(s.oA) + "u, lyapgb::CSeq<" + L +
           ", " + hex64(s.s0) + ", " + hex64(s.s1) + ">, lyapgb::CSeq<" + L + ", " + hex64(s.a0) + ", " +
           hex64(s.a1) + ">>";
}

// KIND_BATCH + mode: the batch kernel of lambda form `mode` only
constexpr int KIND_RENDER = 0, KIND_PROPOSAL = 1, KIND_BATCH = 2;

void compile_entry(Entry &e, const Spec &s, int kind)
{
    Nvrtc &N = g_nvrtc;
    // each kernel's name expression and where its handle goes
    std::vector<std::string> names;
    std::vector<cudaKernel_t *> slots;
    for (int mode = 0; mode < 2; mode++) {
        if (kind == KIND_PROPOSAL) {
            names.push_back("&lyapgb::render_persistent<" + lam_type(s, mode) + ", true>");
            slots.push_back(&e.render[mode]);
        } else if (kind >= KIND_BATCH) {
            if (mode != kind - KIND_BATCH) continue;
            names.push_back("&lyapgb::render_batch<" + lam_type(s, mode) + ">");
            slots.push_back(&e.render[mode]);
        } else {
            names.push_back("&lyapgb::render_persistent<" + lam_type(s, mode) + ">");
            slots.push_back(&e.render[mode]);
            names.push_back("&lyapgb::volume_sweep<" + lam_type(s, mode) + ", " +
                            std::to_string(LYAP_JIT_VOLUME_K) + ">");
            slots.push_back(&e.volume[mode]);
        }
    }
    const char *src = "#include \"lyap_kernels.cuh\"\n";
    nvrtcProgram prog = nullptr;
    nvrtcResult r = N.create(&prog, src, "lyap_jit.cu", kJitHeaderCount, kJitHeaderSources, kJitHeaderNames);
    if (r != NVRTC_SUCCESS) {
        e.error = std::string("nvrtcCreateProgram: ") + N.err(r);
        return;
    }
    for (auto &n : names) N.add_name(prog, n.c_str());
    const std::string rmin0 = "-DLYAP_RENDER_MIN_BLOCKS_PLAIN=" + std::to_string(jit_render_min_blocks(kModePlain));
    const std::string rmin1 =
        "-DLYAP_RENDER_MIN_BLOCKS_PRODUCT=" + std::to_string(jit_render_min_blocks(kModeProduct));
    const std::string vmin = "-DLYAP_VOLUME_MIN_BLOCKS=" + std::to_string(LYAP_JIT_VOLUME_MIN_BLOCKS);
    const std::string pairs0 = "-DLYAP_RENDER_PAIRS_PLAIN=" + std::to_string(jit_render_pairs(kModePlain));
    const std::string pairs1 = "-DLYAP_RENDER_PAIRS_PRODUCT=" + std::to_string(jit_render_pairs(kModeProduct));
    const std::string rthr0 = "-DLYAP_RENDER_THREADS_PLAIN=" + std::to_string(jit_render_threads(kModePlain));
    const std::string rthr1 = "-DLYAP_RENDER_THREADS_PRODUCT=" + std::to_string(jit_render_threads(kModeProduct));
    const char *opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-fmad=false", "-lineinfo",
                          "--ptxas-options=-v", rmin0.c_str(), rmin1.c_str(), vmin.c_str(), pairs0.c_str(),
                          pairs1.c_str(), rthr0.c_str(), rthr1.c_str()};
    r = N.compile(prog, (int)(sizeof(opts) / sizeof(opts[0])), opts);
    size_t ls = 0;
    N.log_size(prog, &ls);
    if (ls > 1) {
        e.log.resize(ls);
        N.log(prog, &e.log[0]);
    }
    if (r != NVRTC_SUCCESS) {
        e.error = std::string("nvrtcCompileProgram: ") + N.err(r) + "\n" + e.log.substr(0, 2000);
        N.destroy(&prog);
        return;
    }
    size_t cs = 0;
    N.cubin_size(prog, &cs);
    std::vector<char> cubin(cs);
    N.cubin(prog, cubin.data());
    std::vector<std::string> lowered;
    for (auto &n : names) {
        const char *ln = nullptr;
        if (N.lowered(prog, n.c_str(), &ln) != NVRTC_SUCCESS || !ln) {
            e.error = "nvrtcGetLoweredName failed for " + n;
            N.destroy(&prog);
            return;
        }
        lowered.push_back(ln);
    }
    N.destroy(&prog);
    cudaError_t ce = cudaLibraryLoadData(&e.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (ce != cudaSuccess) {
        e.error = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(ce);
        return;
    }
    for (size_t i = 0; i < names.size(); i++) {
        ce = cudaLibraryGetKernel(slots[i], e.lib, lowered[i].c_str());
        if (ce != cudaSuccess) {
            e.error = std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(ce);
            return;
        }
    }
    e.ok = true;
}

// The cached specialisation for this sequence, compiling it on first use.
// Returns null (with *why set) when the path is unavailable.
Entry *get_entry(const int32_t *h_seq, uint32_t L, uint32_t settle, std::string *why, int kind = KIND_RENDER)
{
    if (jit_disabled_by_env()) {
        *why = "disabled by LYAP_JIT=0";
        return nullptr;
    }
    if (L == 0 || L > LYAP_JIT_MAX_PERIOD) {
        *why = "period " + std::to_string(L) + " outside 1.." + std::to_string(LYAP_JIT_MAX_PERIOD);
        return nullptr;
    }
    for (uint32_t j = 0; j < L; j++)
        if (h_seq[j] < 0 || h_seq[j] > 3) {
            *why = "sequence symbol out of range";
            return nullptr;
        }
    if (h_seq[L] != -1) {
        *why = "host sequence is not -1 terminated at seq_len - 1";
        return nullptr;
    }
    const Spec s = make_spec(h_seq, L, settle);
    const std::string key = lam_type(s, 9) + (kind == KIND_PROPOSAL ? "|proposal"
                                              : kind >= KIND_BATCH ? "|batch" + std::to_string(kind - KIND_BATCH)
                                                                   : "");
    Entry *e = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (g_nvrtc_state == 0) g_nvrtc_state = g_nvrtc.load() ? 1 : -1;
        if (g_nvrtc_state < 0) {
            *why = "NVRTC unavailable: " + g_nvrtc.why;
            return nullptr;
        }
        auto it = g_cache.find(key);
        if (it == g_cache.end()) it = g_cache.emplace(key, std::unique_ptr<Entry>(new Entry())).first;
        e = it->second.get();   // entries are never removed: the pointer stays valid
    }
    // compiled outside the lock, so that different sequences compile in
    // parallel; callers of the same entry wait for its one compile
    std::call_once(e->once, [&] {
        compile_entry(*e, s, kind);
        std::lock_guard<std::mutex> lock(g_mu);
        e->done = true;
        g_compiles++;
    });
    if (!e->ok) {
        *why = e->error;
        return nullptr;
    }
    return e;
}

}  // namespace

int jit_launch_render(const RenderJob &job, uint32_t mode, const int32_t *h_seq, uint32_t *d_work_counter,
                      unsigned long long *d_stats, uint32_t blocks_per_sm, uint32_t threads, cudaStream_t stream,
                      cudaError_t *launch_err, std::string *why)
{
    const bool prop = job.prop.bits != nullptr;
    const uint32_t smem = proposal_smem_bytes(job);
    Entry *e = get_entry(h_seq, job.seq_period, job.prm.settle, why, prop ? KIND_PROPOSAL : KIND_RENDER);
    if (!e) return 0;
    const int sms = device_sm_count();
    if (sms <= 0) {
        *why = "no device";
        return 0;
    }
    if (threads == 0) threads = (uint32_t)jit_render_threads(mode);
    if (blocks_per_sm == 0) {
        int dev = 0, nb = 0;
        cudaGetDevice(&dev);
        {
            std::lock_guard<std::mutex> lock(g_mu);
            int &cached = e->render_blocks_per_sm[mode & 1u][dev & 63];
            if (!cached || smem) {
                if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void *)e->render[mode], (int)threads,
                                                                  smem) != cudaSuccess || nb <= 0)
                    nb = jit_render_min_blocks(mode);
                if (!smem) cached = nb;
            }
            if (!smem) nb = cached;
        }
        blocks_per_sm = (uint32_t)nb;
    }
    const uint32_t grid = (uint32_t)sms * blocks_per_sm;
    RenderJob j = job;
    void *args[] = {&j, &d_work_counter, &d_stats};
    *launch_err = cudaLaunchKernel((const void *)e->render[mode], dim3(grid), dim3(threads), args, smem, stream);
    {
        std::lock_guard<std::mutex> lock(g_mu);
        g_launches++;
    }
    return 1;
}

int jit_batch_kernel(const int32_t *h_seq, uint32_t L, uint32_t settle, uint32_t mode, cudaKernel_t *kernel,
                     std::string *why)
{
    Entry *e = get_entry(h_seq, L, settle, why, KIND_BATCH + (int)(mode & 1u));
    if (!e) return 0;
    *kernel = e->render[mode & 1u];
    return 1;
}

int jit_launch_volume(const VolumeJob &job, uint32_t mode, const int32_t *h_seq, unsigned long long *d_stats,
                      uint32_t blocks_per_sm, uint32_t threads, cudaStream_t stream, cudaError_t *launch_err,
                      std::string *why)
{
    Entry *e = get_entry(h_seq, job.seq_period, job.prm.settle, why);
    if (!e) return 0;
    const int sms = device_sm_count();
    if (sms <= 0) {
        *why = "no device";
        return 0;
    }
    if (threads == 0) threads = LYAP_VOLUME_THREADS_JIT;
    if (blocks_per_sm == 0) blocks_per_sm = LYAP_JIT_VOLUME_MIN_BLOCKS;
    const uint64_t total = (uint64_t)job.nx * job.ny * job.nz;
    const uint64_t per_block = (uint64_t)threads * LYAP_JIT_VOLUME_K;
    uint64_t grid = (uint64_t)sms * blocks_per_sm;
    const uint64_t need = (total + per_block - 1) / per_block;
    if (need < grid) grid = need;
    if (grid == 0) {
        *launch_err = cudaSuccess;
        return 1;
    }
    VolumeJob j = job;
    void *args[] = {&j, &d_stats};
    *launch_err = cudaLaunchKernel((const void *)e->volume[mode], dim3((uint32_t)grid), dim3(threads), args, 0, stream);
    {
        std::lock_guard<std::mutex> lock(g_mu);
        g_launches++;
    }
    return 1;
}

}  // namespace lyapgb

extern "C" int lyap_jit_info(char *buf, size_t cap)
{
    using namespace lyapgb;
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_nvrtc_state == 0) g_nvrtc_state = g_nvrtc.load() ? 1 : -1;
    std::string s = std::string("nvrtc=") + (g_nvrtc_state > 0 ? "loaded" : ("unavailable (" + g_nvrtc.why + ")")) +
                    " env=" + (jit_disabled_by_env() ? "off" : "on") + " compiled=" + std::to_string(g_compiles) +
                    " launches=" + std::to_string(g_launches) + " cached=" + std::to_string(g_cache.size());
    for (auto &kv : g_cache)
        if (kv.second->done && !kv.second->ok) s += "\nerror: " + kv.second->error.substr(0, 400);
    if (buf && cap) {
        strncpy(buf, s.c_str(), cap - 1);
        buf[cap - 1] = 0;
    }
    return g_nvrtc_state > 0 ? 1 : 0;
}
