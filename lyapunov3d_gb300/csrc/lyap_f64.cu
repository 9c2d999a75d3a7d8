// lyap_f64.cu -- the DOUBLE_REALS render mode (structs.hpp:10-14 with Real =
// double): kernel_calc_render / raymarch / shade (kernel.cu:25-516) with
// every Real in double, on the double structs (LyapCamD, LyapParamsD,
// LyapLightD, LyapPointD).  One thread per pixel over a grid-stride loop:
// FP64 is this GPU's slow path, so the mode is for precision work, not
// throughput.  lambda is lambda_f64_core: the reference's double orbit, the
// log sum as a renormalised double product (within ~1e-13 relative of one
// log per step).  shade keeps the reference's float powf (kernel.cu:81) and
// its double log of c (VEC3::logf with T = double).
#include <cuda_runtime.h>

#include "lyap_device.cuh"
#include "lyap_internal.h"

namespace lyapgb {

struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 d3(double x, double y, double z) { return D3{x, y, z}; }
__device__ __forceinline__ D3 d3(const LyapVecD &v) { return D3{v.x, v.y, v.z}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ D3 operator*(D3 a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ D3 operator/(D3 a, double s) { return d3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// vec3.hpp:127-154 with T = double
__device__ __forceinline__ D3 dnormalized(D3 a)
{
    const double mag2 = a.x * a.x + a.y * a.y + a.z * a.z;
    if (mag2 < 1e-12) return d3(0, 0, 0);
    if (mag2 == 1.0f || (mag2 > (1.0f - 1e-12) && mag2 < (1.0f + 1e-12))) return a;
    return a / sqrt(mag2);
}
__device__ __forceinline__ double dclamp01(double v) { return v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v); }

struct RenderJobD {
    LyapCamD cam;
    LyapParamsD prm;
    const int32_t *seq;
    const LyapLightD *lights;
    RGBA *rgba;
    LyapPointD *points;
    uint32_t *counts;
    uint32_t seq_period, n_lights, width, height, light_model;
};

// raymarch (kernel.cu:156-486), Real = double; 0 on a hit
__device__ int raymarch_d(LyapPointD &pt, uint32_t sx, uint32_t sy, const RenderJobD &job, uint32_t cnt[3])
{
    const LyapCamD &cam = job.cam;
    const LyapParamsD &prm = job.prm;
    auto lam = [&](D3 P) {
        return lambda_f64_core(P.x, P.y, P.z, prm.d, job.seq, job.seq_period, prm.settle, prm.accum);
    };
    uint32_t nm = 0, nh = 0, nn = 0;
    cnt[0] = cnt[1] = cnt[2] = 0;
    D3 V = (d3(cam.S0) + d3(cam.SDX) * (double)sx) + d3(cam.SDY) * (double)sy;
    V = dnormalized(V);
    V = V / cam.M;
    const double LMIN = prm.lMin, LMAX = prm.lMax;
    const double INF = __longlong_as_double(0x7ff0000000000000ll);
    const double QNAN = __longlong_as_double(0x7ff8000000000000ll);
    const D3 C = d3(cam.C);
    double ts[6];
    ts[0] = (V.x != 0.0f) ? ((LMIN - C.x) / V.x) : INF;
    ts[1] = (V.x != 0.0f) ? ((LMAX - C.x) / V.x) : INF;
    ts[2] = (V.y != 0.0f) ? ((LMIN - C.y) / V.y) : INF;
    ts[3] = (V.y != 0.0f) ? ((LMAX - C.y) / V.y) : INF;
    ts[4] = (V.z != 0.0f) ? ((LMIN - C.z) / V.z) : INF;
    ts[5] = (V.z != 0.0f) ? ((LMAX - C.z) / V.z) : INF;
    for (int k = 0; k < 6; k++) {
        if (ts[k] != INF) {
            const D3 P = C + V * ts[k];
            const double u = (k < 2) ? P.y : P.x;
            const double w = (k < 4) ? P.z : P.y;
            if (u < LMIN || u > LMAX || w < LMIN || w > LMAX) ts[k] = QNAN;
        }
    }
    int i0 = -1, i1 = -1;
    double t0 = 3.40282347e+38F, t1 = 0;
    for (int k = 0; k < 6; k++) {
        if (isfinite(ts[k])) {
            if (i0 == -1 || ts[k] < t0) t0 = ts[i0 = k];
            if (i1 == -1 || ts[k] > t1) t1 = ts[i1 = k];
        }
    }
    if (i0 == -1 && i1 == -1) return 1;
    if (i1 == -1 || i0 == i1) {
        t1 = t0;
        t0 = 0;
    }
    if (t0 < 0) t0 = 0;
    double t = t0;
    D3 P = C + V * t;
    double a = 0, c = 0;
    double Fdt = (prm.stepMethod == 1) ? (t1 - t0) / prm.depth : sqrt(V.x * V.x + V.y * V.y + V.z * V.z) / prm.depth;
    double dt = Fdt;
    const double Ndt = dt / prm.nearMultiplier;
    bool near = false;
    const double dmin = Fdt < Ndt ? Fdt : Ndt;
    const double capd = ceil((t1 - t0) / dmin * 1.001) + 16.0;
    const uint32_t cap = (capd > 0.0 && capd < (double)MARCH_MAX) ? (uint32_t)capd : MARCH_MAX;
    double l = lam(P);
    nm++;
    while (l > prm.opaqueThreshold) {
        if (nm >= cap) {
            cnt[0] = nm;
            return 1;
        }
        double step = dt;
        if (prm.jitter != 0.0) {
            double jit = l - trunc(l);
            jit = (jit < 0) ? 1.0 - jit * prm.jitter : 1.0 + jit * prm.jitter;
            if (isfinite(jit)) step = dt * jit;
        }
        t += step;
        P = P + V * step;
        if (t > t1) {
            cnt[0] = nm;
            return 1;
        }
        l = lam(P);
        nm++;
        if (l > prm.chaosThreshold) c += l;
        else if (l > prm.opaqueThreshold) a += l;
        if (l <= prm.nearThreshold && !near) {
            near = true;
            dt = Ndt;
        } else if (l > prm.nearThreshold && near) {
            near = false;
            dt = Fdt;
        }
    }
    if (t > t1) {
        cnt[0] = nm;
        return 1;
    }
    // honing (kernel.cu:402-441)
    int sign = 0;
    double Qdt = dt * -0.5f;
    D3 QdV = V * Qdt;
    const double Qt1 = t, Qt0 = t - dt, min_Qdt = dt / prm.refine;
    while (t <= Qt1 && t >= Qt0 && (Qdt <= -min_Qdt || Qdt >= min_Qdt) && nh < HONE_CAP) {
        t += Qdt;
        P = P + QdV;
        l = lam(P);
        nh++;
        if (l == prm.opaqueThreshold) break;
        const int osign = sign;
        sign = (l < prm.opaqueThreshold) ? 0 : 1;
        if (sign != osign) {
            Qdt *= -0.5f;
            QdV = QdV * -0.5f;
        }
    }
    // normal (kernel.cu:456-473)
    const double mag = dt * prm.gradient;
    double ls[6];
    for (int k = 0; k < 6; k++) {
        D3 Q = P;
        if (k == 0) Q.x -= mag;
        else if (k == 1) Q.x += mag;
        else if (k == 2) Q.y -= mag;
        else if (k == 3) Q.y += mag;
        else if (k == 4) Q.z -= mag;
        else Q.z += mag;
        ls[k] = lam(Q);
        nn++;
    }
    const D3 N = dnormalized(d3(ls[1] - ls[0], ls[3] - ls[2], ls[5] - ls[4]));
    pt.P = LyapVecD{P.x, P.y, P.z};
    pt.N = LyapVecD{N.x, N.y, N.z};
    pt.a = a;
    pt.c = c;
    pt.l = l;
    cnt[0] = nm;
    cnt[1] = nh;
    cnt[2] = nn;
    return 0;
}

struct C4D {
    double x, y, z, w;
};
__device__ __forceinline__ C4D cd(const LyapColorD &c) { return C4D{c.x, c.y, c.z, c.w}; }
__device__ __forceinline__ C4D operator+(C4D a, C4D b) { return C4D{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
__device__ __forceinline__ C4D operator*(C4D a, double s) { return C4D{a.x * s, a.y * s, a.z * s, a.w * s}; }

// shade (kernel.cu:25-106), Real = double
__device__ C4D shade_d(const LyapPointD &pt, const RenderJobD &job)
{
    C4D color{0, 0, 0, 0};
    if (isnan(pt.a)) return color;
    const D3 P = d3(pt.P), N = d3(pt.N);
    for (uint32_t li = 0; li < job.n_lights; li++) {
        const LyapLightD &L = job.lights[li];
        C4D phong;
        if (job.light_model == LYAP_LIGHT_DIRECTIONAL) {
            const double i = dclamp01(ddot(N, d3(0, 0, 0) - d3(L.V)));
            phong = cd(L.diffuseColor) * (i * L.diffusePower) + cd(L.ambient);
        } else {
            const D3 camV = d3(job.cam.C) - P;
            D3 lightV = d3(L.C) - P;
            const double lightD2 = lightV.x * lightV.x + lightV.y * lightV.y + lightV.z * lightV.z;
            lightV = dnormalized(lightV);
            double i = ddot(lightV, N);
            double j = -ddot(lightV, d3(L.V));
            if (j > L.lightOuterCone) {
                i = dclamp01(i);
                const C4D diffuse = cd(L.diffuseColor) * (i * L.diffusePower);
                const D3 halfV = dnormalized(camV + lightV);
                i = dclamp01(ddot(N, halfV));
                i = powf((float)i, (float)L.specularHardness);
                const C4D specular = cd(L.specularColor) * (i * L.specularPower);
                phong = (specular + diffuse) * (L.lightRange / lightD2);
                if (j < L.lightInnerCone) phong = phong * ((j - L.lightOuterCone) / (L.lightInnerCone - L.lightOuterCone));
                phong = phong + cd(L.ambient);
            } else {
                phong = cd(L.ambient);
            }
        }
        if (pt.c > 0.0) phong = phong + cd(L.chaosColor) * (0.1125 / log(pt.c));
        color = color + phong;
    }
    return color;
}

__device__ __forceinline__ unsigned char to_byte_d(double ch)
{
    const double v = 255.0 * ch;   // color.hpp:171-174, saturated
    if (!(v > 0.0)) return 0;
    if (v >= 255.0) return 255;
    return (unsigned char)v;
}

__global__ void __launch_bounds__(128) render_f64(const __grid_constant__ RenderJobD job)
{
    const uint64_t npix = (uint64_t)job.width * job.height;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t sx = (uint32_t)(p % job.width), sy = (uint32_t)(p / job.width);
        LyapPointD pt;
        uint32_t cnt[3];
        const bool hit = raymarch_d(pt, sx, sy, job, cnt) == 0;
        if (!hit) {
            double *f = reinterpret_cast<double *>(&pt);
            for (int k = 0; k < 9; k++) f[k] = __longlong_as_double(-1ll);
        }
        job.points[p] = pt;
        uint32_t px = 0;
        if (hit) {
            const C4D col = shade_d(pt, job);
            px = (uint32_t)to_byte_d(col.x) | ((uint32_t)to_byte_d(col.y) << 8) |
                 ((uint32_t)to_byte_d(col.z) << 16) | ((uint32_t)to_byte_d(col.w) << 24);
        }
        reinterpret_cast<uint32_t *>(job.rgba)[p] = px;
        if (job.counts) {
            job.counts[3 * p + 0] = cnt[0];
            job.counts[3 * p + 1] = cnt[1];
            job.counts[3 * p + 2] = cnt[2];
        }
    }
}

}  // namespace lyapgb

using namespace lyapgb;

extern "C" int lyap_render_d(const LyapCamD *cam, const LyapParamsD *prm, const int32_t *d_seq, size_t seq_len,
                             const LyapLightD *d_lights, uint32_t n_lights, RGBA *d_rgba, LyapPointD *d_points,
                             uint32_t width, uint32_t height, uint32_t light_model, uint32_t *d_counts, void *stream)
{
    const char *fn = "lyap_render_d";
    if (!cam || !prm || !d_seq || !d_rgba || !d_points || (n_lights && !d_lights))
        return set_error(LYAP_ERR_INVALID_ARG, "%s: null pointer", fn);
    if (seq_len < 2 || seq_len > LYAP_MAX_SEQ_LEN)
        return set_error(LYAP_ERR_SEQUENCE, "%s: seq_len %zu outside [2, %d]", fn, seq_len, LYAP_MAX_SEQ_LEN);
    if (n_lights > LYAP_MAX_LIGHTS) return set_error(LYAP_ERR_INVALID_ARG, "%s: %u lights", fn, n_lights);
    if (width == 0 || height == 0 || (uint64_t)width * height > LYAP_MAX_PIXELS)
        return set_error(LYAP_ERR_INVALID_ARG, "%s: image size %ux%u", fn, width, height);
    if (light_model > LYAP_LIGHT_DIRECTIONAL) return set_error(LYAP_ERR_INVALID_ARG, "%s: light model %u", fn, light_model);
    const int sms = device_sm_count();
    if (sms <= 0) return cuda_error(cudaErrorNoDevice, fn);
    RenderJobD job;
    job.cam = *cam;
    job.prm = *prm;
    job.seq = d_seq;
    job.lights = d_lights;
    job.rgba = d_rgba;
    job.points = d_points;
    job.counts = d_counts;
    job.seq_period = (uint32_t)(seq_len - 1);
    job.n_lights = n_lights;
    job.width = width;
    job.height = height;
    job.light_model = light_model;
    const uint64_t npix = (uint64_t)width * height;
    const uint64_t want = (npix + 127) / 128, cap = (uint64_t)sms * 16;
    render_f64<<<(uint32_t)(want < cap ? want : cap), 128, 0, (cudaStream_t)stream>>>(job);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LYAP_OK : cuda_error(e, fn);
}
