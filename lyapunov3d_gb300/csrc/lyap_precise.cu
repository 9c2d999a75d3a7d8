// lyap_precise.cu -- the precision form's FP64 parts and lambda at points.
//
//  * bisect_pass: second pass of a LYAP_FLAG_BISECT_F64 render.  The first
//    pass (render_persistent in bracket mode) stops every ray at its first
//    sample at or below the opaque threshold and records [t of the previous
//    sample, t of that sample].  Here each crossing is halved n times with
//    lambda in double (lambda_f64) on P(t) = C + V t evaluated in double;
//    the surface point is P at the near end of the final interval's "at or
//    below" side, its normal comes from six FP32 samples (the render's form)
//    at +-dt*gradient, and it is shaded.  One thread per crossing: every
//    thread runs the same FP64 loop, so the warp stays converged.
//  * points_lambda: lyap4d (kernel.cu:108) at caller-given points, in any of
//    the three forms, x fastest in a grid-stride loop.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lyap_internal.h"
#include "lyap_kernels.cuh"

namespace lyapgb {

__global__ void __launch_bounds__(128) bisect_pass(const __grid_constant__ RenderJob job, uint32_t mode,
                                                    uint32_t halvings, unsigned long long *__restrict__ stats)
{
    const RuntimeLambda<MODE_PLAIN> lam_plain(job.seq, job.seq_period, job.prm);
    const RuntimeLambda<MODE_PRODUCT> lam_prod(job.seq, job.seq_period, job.prm);
    const CamRays cr = cam_rays(job.cam);
    const uint32_t count = job.hits[0];
    LaneStats st = {};
    const uint32_t stride = gridDim.x * blockDim.x;
    // every thread of a warp runs the same number of iterations (idle ones on a dummy crossing)
    const uint32_t rounds = (count + stride - 1) / stride;
    for (uint32_t it = 0; it < rounds; it++) {
        const uint32_t i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        const bool real = i < count;
        const uint32_t pix = real ? job.hits[1 + i] : job.hits[1];
        const uint32_t sx = pix % job.width, sy = pix / job.width;
        Ray r;
        ray_init(r, cr, job.prm, sx, sy);   // the ray's direction, exactly as the march had it
        const double Cx = cr.C.x, Cy = cr.C.y, Cz = cr.C.z;
        const double Vx = r.V.x, Vy = r.V.y, Vz = r.V.z;
        const double opaque = (double)job.prm.opaqueThreshold;
        double lo = job.bracket[2 * (size_t)pix + 0], hi = job.bracket[2 * (size_t)pix + 1];
        const float step = (float)(hi - lo);
        SeqInfo si = lam_plain.si;
        uint32_t nh = 0;
        if (lo < hi) {
            for (uint32_t n = 0; n < halvings; n++) {
                const double mid = 0.5 * (lo + hi);
                const double l64 = lambda_f64(Cx + Vx * mid, Cy + Vy * mid, Cz + Vz * mid, si);
                if (l64 > opaque) lo = mid;   // NaN counts as "at or below" (a hit), as the march does
                else hi = mid;
                nh++;
            }
        }
        // the surface point, rounded to float, and the double lambda there
        V3 P = v3((float)(Cx + Vx * hi), (float)(Cy + Vy * hi), (float)(Cz + Vz * hi));
        const double lP = lambda_f64(P.x, P.y, P.z, si);
        // normal: six samples of the render's form at +-mag (kernel.cu:456-473)
        const float dt = (step > 0.0f) ? step : r.dt;
        const float mag = dt * job.prm.gradient;
        float ls[6];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            V3 Q = P;
            if (k == 0) Q.x = Q.x - mag;
            else if (k == 1) Q.x = Q.x + mag;
            else if (k == 2) Q.y = Q.y - mag;
            else if (k == 3) Q.y = Q.y + mag;
            else if (k == 4) Q.z = Q.z - mag;
            else Q.z = Q.z + mag;
            bool sk, fb;
            ls[k] = (mode == MODE_PRODUCT) ? lam_prod(Q.x, Q.y, Q.z, sk, fb) : lam_plain(Q.x, Q.y, Q.z, sk, fb);
            if (real) {
                st.samples += 1;
                st.skipped += sk ? 1u : 0u;
                st.fallback += fb ? 1u : 0u;
            }
        }
        if (!real) continue;
        const LyapPoint &prov = job.points[pix];
        Ray out;
        out.P = P;
        out.N = normalized(v3(ls[1] - ls[0], ls[3] - ls[2], ls[5] - ls[4]));
        out.a = prov.a;
        out.c = prov.c;
        out.l = (float)lP;
        out.nm = job.counts ? job.counts[3 * (size_t)pix + 0] : 0u;
        out.nh = nh;
        st.hone += nh;
        LaneStats dummy = {};
        finish_pixel(job.rgba, job.points, job.counts, pix, out, true, cr.C, job.lights, job.n_lights,
                     job.light_model, dummy);
        st.normal += 6;
        st.hits += 1;
    }
    if (stats) {
        const uint32_t mask = __activemask();
        const uint32_t v[5] = {st.samples, st.skipped, st.hone, st.normal, st.hits};
        const int slot[5] = {LYAP_STAT_SAMPLES, LYAP_STAT_SKIPPED, LYAP_STAT_HONE, LYAP_STAT_NORMAL, LYAP_STAT_HITS};
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const uint32_t s = __reduce_add_sync(mask, v[k]);
            if ((threadIdx.x & 31u) == (uint32_t)(__ffs(mask) - 1) && s) atomicAdd(stats + slot[k], (unsigned long long)s);
        }
    }
}

__global__ void __launch_bounds__(256) points_lambda(const float *__restrict__ xyz, size_t n, const int32_t *seq,
                                                      uint32_t period, LyapParams prm, uint32_t form, void *out)
{
    const RuntimeLambda<MODE_PLAIN> lam_plain(seq, period, prm);
    const RuntimeLambda<MODE_PRODUCT> lam_prod(seq, period, prm);
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t rounds = (n + stride - 1) / stride;
    for (size_t it = 0; it < rounds; it++) {
        const size_t i = it * stride + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
        const size_t j = i < n ? i : n - 1;
        const float x = xyz[3 * j], y = xyz[3 * j + 1], z = xyz[3 * j + 2];
        bool sk, fb;
        if (form == LYAP_FORM_F64) {
            const double v = lambda_f64(x, y, z, lam_plain.si);
            if (i < n) static_cast<double *>(out)[i] = v;
        } else {
            const float v = (form == LYAP_VARIANT_PRODUCT) ? lam_prod(x, y, z, sk, fb) : lam_plain(x, y, z, sk, fb);
            if (i < n) static_cast<float *>(out)[i] = v;
        }
    }
}

cudaError_t launch_bisect(const RenderJob &job, uint32_t mode, uint32_t halvings, unsigned long long *d_stats,
                          cudaStream_t stream)
{
    const int sms = device_sm_count();
    if (sms <= 0) return cudaErrorNoDevice;
    bisect_pass<<<(uint32_t)sms * 4, 128, 0, stream>>>(job, mode, halvings, d_stats);
    return cudaGetLastError();
}

}  // namespace lyapgb

using namespace lyapgb;

extern "C" int lyap_lambda_points(const float *d_xyz, size_t n, const LyapParams *prm, const int32_t *d_seq,
                                  size_t seq_len, uint32_t form, void *d_out, void *stream)
{
    if (!d_xyz || !prm || !d_seq || !d_out) return set_error(LYAP_ERR_INVALID_ARG, "lyap_lambda_points: null pointer");
    if (seq_len < 2 || seq_len > LYAP_MAX_SEQ_LEN)
        return set_error(LYAP_ERR_SEQUENCE, "lyap_lambda_points: seq_len %zu outside [2, %d]", seq_len,
                         LYAP_MAX_SEQ_LEN);
    if (form > LYAP_FORM_F64) return set_error(LYAP_ERR_INVALID_ARG, "lyap_lambda_points: unknown form %u", form);
    if (n == 0) return LYAP_OK;
    const int sms = device_sm_count();
    if (sms <= 0) return cuda_error(cudaErrorNoDevice, "lyap_lambda_points");
    const size_t threads = 256;
    size_t grid = (n + threads - 1) / threads;
    const size_t cap = (size_t)sms * 8;
    if (grid > cap) grid = cap;
    points_lambda<<<(uint32_t)grid, (uint32_t)threads, 0, (cudaStream_t)stream>>>(
        d_xyz, n, d_seq, (uint32_t)(seq_len - 1), *prm, form, d_out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LYAP_OK : cuda_error(e, "lyap_lambda_points: launch");
}
