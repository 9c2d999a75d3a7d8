// lyap_batch.cu -- many render requests in one launch (persistent warps over
// a device work queue), captured in a CUDA graph, launch shape picked by an
// autotuner.
//
// The reference renders one frame per launch (lyap_interactive.cu:711); a
// sweep of frames (scale.pl) is a loop of whole program runs.  Here a batch
// of requests -- each with its own camera, parameters, sequence, lights,
// image size and iteration counts -- is cut into chunks of tiles, the
// chunks are ordered longest-job-first (estimated cost: pixels x (settle +
// accum) x depth), and persistent warps take chunks from a global counter.
// A warp renders one request at a time (its lambda loop must be uniform), so
// it continues with the next chunk while that belongs to the same request
// and otherwise lets its rays run out -- idle lanes speculate for the rays
// still running (sample_round) -- before switching (render_batch,
// lyap_kernels.cuh).  When every request has the same sequence (and settle
// count mod its period) -- the frames of an animation of one field -- the
// kernel is compiled for that sequence at run time (ConstLambda, paired
// rounds; LYAP_FLAG_NO_JIT in the options keeps the library's kernel).
//
// Autotuner: the tile shape (32x1, 8x4, 16x16), the tiles per chunk (1, 4)
// and the resident blocks per SM (3, 4) are timed on every 8th chunk of the
// batch itself and the fastest kept; the whole launch (counter reset +
// kernel) is then captured once in a graph that lyap_batch_run replays.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include <string>

#include "lyap_internal.h"
#include "lyap_jit.h"
#include "lyap_kernels.cuh"

namespace lyapgb {

}  // namespace lyapgb

using namespace lyapgb;

struct LyapBatch {
    int device = 0;
    uint32_t n_jobs = 0, mode = 0;
    RenderJob *d_jobs = nullptr;
    uint32_t *d_counter = nullptr;
    unsigned long long *d_stats = nullptr;
    std::vector<RenderJob> jobs;
    std::vector<double> cost;
    // chosen launch shape and its chunk list
    uint32_t tile_w = 16, tile_h = 16, tiles_per_chunk = 1, blocks_per_sm = 3, threads = 128;
    uint32_t *d_chunks = nullptr;   // chunk_job then chunk_tile
    uint32_t n_chunks = 0;
    cudaKernel_t jit_kernel = nullptr;   // the kernel compiled for the batch's one sequence, if any
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    LyapBatchInfo info;
};

namespace {

void build_chunks(const LyapBatch &b, uint32_t tw, uint32_t th, uint32_t tpc, uint32_t sample_every,
                  std::vector<uint32_t> &cj, std::vector<uint32_t> &ct)
{
    std::vector<uint32_t> order(b.n_jobs);
    for (uint32_t i = 0; i < b.n_jobs; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t c) { return b.cost[a] > b.cost[c]; });
    cj.clear();
    ct.clear();
    uint64_t k = 0;
    for (uint32_t j : order) {
        const RenderJob &J = b.jobs[j];
        const uint32_t tiles = ((J.width + tw - 1) / tw) * ((J.height + th - 1) / th);
        for (uint32_t t = 0; t < tiles; t += tpc, k++) {
            if (sample_every > 1 && (k % sample_every) != 0) continue;
            cj.push_back(j);
            ct.push_back(t);
        }
    }
}

cudaError_t upload_chunks(LyapBatch &b, const std::vector<uint32_t> &cj, const std::vector<uint32_t> &ct,
                          cudaStream_t s)
{
    if (b.d_chunks) cudaFreeAsync(b.d_chunks, s);
    b.d_chunks = nullptr;
    b.n_chunks = (uint32_t)cj.size();
    cudaError_t e = cudaMallocAsync((void **)&b.d_chunks, sizeof(uint32_t) * 2 * (cj.size() + 1), s);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(b.d_chunks, cj.data(), sizeof(uint32_t) * cj.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b.d_chunks + cj.size(), ct.data(), sizeof(uint32_t) * ct.size(), cudaMemcpyHostToDevice, s);
    return e;
}

cudaError_t launch_batch(const LyapBatch &b, uint32_t tw, uint32_t th, uint32_t tpc, uint32_t bps, const uint32_t *chunks,
                         uint32_t n_chunks, unsigned long long *stats, cudaStream_t s)
{
    BatchTables tb;
    tb.jobs = b.d_jobs;
    tb.chunk_job = chunks;
    tb.chunk_tile = chunks + n_chunks;
    tb.n_chunks = n_chunks;
    tb.tile_w = tw;
    tb.tile_h = th;
    tb.tiles_per_chunk = tpc;
    const int sms = device_sm_count();
    if (sms <= 0) return cudaErrorNoDevice;
    cudaError_t e = cudaMemsetAsync(b.d_counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    const uint32_t grid = (uint32_t)sms * bps;
    if (b.jit_kernel) {
        uint32_t *counter = b.d_counter;
        void *args[] = {&tb, &counter, &stats};
        return cudaLaunchKernel((const void *)b.jit_kernel, dim3(grid), dim3(b.threads), args, 0, s);
    }
    if (b.mode == MODE_PRODUCT)
        render_batch<RuntimeLambda<MODE_PRODUCT>><<<grid, b.threads, 0, s>>>(tb, b.d_counter, stats);
    else
        render_batch<RuntimeLambda<MODE_PLAIN>><<<grid, b.threads, 0, s>>>(tb, b.d_counter, stats);
    return cudaGetLastError();
}

void destroy(LyapBatch *b)
{
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d_chunks) cudaFree(b->d_chunks);
    if (b->d_jobs) cudaFree(b->d_jobs);
    if (b->d_counter) cudaFree(b->d_counter);
    delete b;
}

}  // namespace

extern "C" {

int lyap_batch_create(const LyapRequest *reqs, uint32_t n, const LyapBatchOptions *opt, LyapBatch **out)
{
    if (!reqs || !out || n == 0) return set_error(LYAP_ERR_INVALID_ARG, "lyap_batch_create: no requests");
    if (opt && opt->size != sizeof(LyapBatchOptions))
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_batch_create: LyapBatchOptions.size is %u, expected %zu",
                         opt->size, sizeof(LyapBatchOptions));
    if (opt && opt->variant > LYAP_VARIANT_PRODUCT)
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_batch_create: unknown variant %u", opt->variant);
    *out = nullptr;
    LyapBatch *b = new (std::nothrow) LyapBatch();
    if (!b) return set_error(LYAP_ERR_OUT_OF_MEMORY, "lyap_batch_create: host allocation");
    memset(&b->info, 0, sizeof(b->info));
    b->n_jobs = n;
    b->mode = opt ? opt->variant : LYAP_VARIANT_PLAIN;
    b->d_stats = opt ? opt->d_stats : nullptr;
    cudaGetDevice(&b->device);
    b->jobs.resize(n);
    b->cost.resize(n);
    for (uint32_t i = 0; i < n; i++) {
        const LyapRequest &q = reqs[i];
        char fn[64];
        snprintf(fn, sizeof(fn), "lyap_batch_create: request %u", i);
        LyapRenderExt x;
        memset(&x, 0, sizeof(x));
        x.size = sizeof(x);
        x.light_model = q.light_model;
        x.flags = q.flags & LYAP_FLAG_NO_SPECULATION;
        x.d_counts = q.d_counts;
        int rc = check_render_args(&q.cam, &q.prm, q.d_seq, q.seq_len, q.d_lights, q.n_lights, q.d_rgba, q.d_points,
                                   q.width, q.height, &x, fn);
        if (rc) {
            delete b;
            return rc;
        }
        b->jobs[i] = make_job(&q.cam, &q.prm, q.d_seq, q.seq_len, q.d_lights, q.n_lights, q.d_rgba, q.d_points,
                              q.width, q.height, &x);
        b->cost[i] = (double)q.width * q.height * ((double)q.prm.settle + q.prm.accum) *
                     (q.prm.depth > 1.0f ? (double)q.prm.depth : 1.0);
    }
    cudaStream_t s = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_jobs, sizeof(RenderJob) * n);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_counter, 256);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_jobs, b->jobs.data(), sizeof(RenderJob) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        if (s) cudaStreamDestroy(s);
        destroy(b);
        return cuda_error(e, "lyap_batch_create: device tables");
    }
    // one sequence for every request (same symbols, same settle count mod its
    // period): the batch kernel compiled for it
    if (!(opt && (opt->flags & LYAP_FLAG_NO_JIT))) {
        std::vector<int32_t> first, cur;
        bool same = true;
        for (uint32_t i = 0; i < n && same && e == cudaSuccess; i++) {
            cur.resize(reqs[i].seq_len);
            e = cudaMemcpy(cur.data(), reqs[i].d_seq, reqs[i].seq_len * sizeof(int32_t), cudaMemcpyDeviceToHost);
            if (i == 0)
                first = cur;
            else
                same = cur == first && (reqs[i].prm.settle % (uint32_t)(cur.size() - 1)) ==
                                           (reqs[0].prm.settle % (uint32_t)(first.size() - 1));
        }
        if (e == cudaSuccess && same && !first.empty()) {
            std::string why;
            cudaKernel_t k = nullptr;
            if (jit_batch_kernel(first.data(), (uint32_t)first.size() - 1, reqs[0].prm.settle, b->mode, &k, &why))
                b->jit_kernel = k;
        }
        if (e != cudaSuccess) {
            cudaStreamDestroy(s);
            destroy(b);
            return cuda_error(e, "lyap_batch_create: reading the sequences");
        }
    }
    struct Cand {
        uint32_t tw, th, tpc, bps;
    };
    std::vector<Cand> cands;
    const bool tune = !opt || opt->autotune;
    if (tune) {
        const uint32_t shapes[3][2] = {{32, 1}, {8, 4}, {16, 16}};
        for (auto &sh : shapes)
            for (uint32_t tpc : {1u, 4u})
                for (uint32_t bps : {3u, 4u}) cands.push_back(Cand{sh[0], sh[1], tpc, bps});
    } else {
        cands.push_back(Cand{opt->tile_w ? opt->tile_w : 16u, opt->tile_h ? opt->tile_h : 16u,
                             opt->tiles_per_chunk ? opt->tiles_per_chunk : 1u, opt->blocks_per_sm ? opt->blocks_per_sm : 3u});
    }
    std::vector<uint32_t> cj, ct;
    size_t best = 0;
    float best_ms = -1.0f;
    if (cands.size() > 1) {
        // time each candidate on every 8th chunk of the batch
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        for (size_t i = 0; i < cands.size() && e == cudaSuccess; i++) {
            const Cand &c = cands[i];
            build_chunks(*b, c.tw, c.th, c.tpc, 8, cj, ct);
            e = upload_chunks(*b, cj, ct, s);
            if (e != cudaSuccess) break;
            cudaEventRecord(e0, s);
            e = launch_batch(*b, c.tw, c.th, c.tpc, c.bps, b->d_chunks, b->n_chunks, nullptr, s);
            cudaEventRecord(e1, s);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (i < 16) b->info.tuned_ms[i] = ms;
            if (best_ms < 0 || ms < best_ms) {
                best_ms = ms;
                best = i;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        b->info.candidates = (uint32_t)cands.size();
    }
    if (e == cudaSuccess) {
        const Cand &c = cands[best];
        b->tile_w = c.tw;
        b->tile_h = c.th;
        b->tiles_per_chunk = c.tpc;
        b->blocks_per_sm = c.bps;
        build_chunks(*b, c.tw, c.th, c.tpc, 1, cj, ct);
        e = upload_chunks(*b, cj, ct, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    // capture the launch (counter reset + kernel) once; lyap_batch_run replays it
    if (e == cudaSuccess) e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t le = launch_batch(*b, b->tile_w, b->tile_h, b->tiles_per_chunk, b->blocks_per_sm, b->d_chunks,
                                      b->n_chunks, b->d_stats, s);
        e = cudaStreamEndCapture(s, &b->graph);
        if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) {
        destroy(b);
        return cuda_error(e, "lyap_batch_create");
    }
    b->info.size = sizeof(LyapBatchInfo);
    b->info.requests = n;
    b->info.chunks = b->n_chunks;
    b->info.tile_w = b->tile_w;
    b->info.tile_h = b->tile_h;
    b->info.tiles_per_chunk = b->tiles_per_chunk;
    b->info.blocks_per_sm = b->blocks_per_sm;
    b->info.threads_per_block = b->threads;
    b->info.specialised = b->jit_kernel ? 1u : 0u;
    *out = b;
    return LYAP_OK;
}

int lyap_batch_run(LyapBatch *b, void *stream)
{
    if (!b || !b->exec) return set_error(LYAP_ERR_INVALID_ARG, "lyap_batch_run: no batch");
    cudaError_t e = cudaGraphLaunch(b->exec, (cudaStream_t)stream);
    return e == cudaSuccess ? LYAP_OK : cuda_error(e, "lyap_batch_run");
}

int lyap_batch_info(const LyapBatch *b, LyapBatchInfo *info)
{
    if (!b || !info) return set_error(LYAP_ERR_INVALID_ARG, "lyap_batch_info: null pointer");
    *info = b->info;
    return LYAP_OK;
}

int lyap_batch_destroy(LyapBatch *b)
{
    if (!b) return LYAP_OK;
    destroy(b);
    return LYAP_OK;
}

}  // extern "C"
