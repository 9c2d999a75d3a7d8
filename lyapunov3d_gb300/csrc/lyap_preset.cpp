// lyap_preset.cpp -- the reference's parameter preset (params_init,
// params.cu:21-114) and the camera path of its animation driver (scale.pl),
// for both Real widths (float and the DOUBLE_REALS build).  Results are
// bit-identical to the reference's host build: every expression keeps the
// operand types the reference's source gives it (float Real arithmetic,
// promotion to double where a double literal or QUAT_PI enters, the float or
// double libm function QUAT<T>::sin/cos/acos call) and this file is compiled
// with -ffp-contract=off.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "lyap_gb300.h"
#include "lyap_internal.h"

namespace {

// quat.hpp:12-13 and vec3.hpp:10
constexpr double QUAT_EPS = 1e-6;
constexpr double QUAT_PI_D = 3.14159265358979323846264338327950288;
constexpr double VEC_EPS = 1e-12;

template <class T>
struct V {
    T x, y, z;
};
template <class T>
struct Q {
    T x, y, z, w;
};

template <class T> T m_sin(T a) { return std::sin(a); }
template <class T> T m_cos(T a) { return std::cos(a); }
template <class T> T m_acos(T a) { return std::acos(a); }
template <class T> T m_sqrt(T a) { return std::sqrt(a); }

// VEC3::normalize / normalized (vec3.hpp:127-154)
template <class T>
void vnormalize(V<T> &v)
{
    T mag2 = v.x * v.x + v.y * v.y + v.z * v.z;
    if (mag2 < VEC_EPS) {
        v.x = v.y = v.z = 0;
    } else if (mag2 == 1.0f || (mag2 > (1.0f - VEC_EPS) && mag2 < (1.0f + VEC_EPS))) {
    } else {
        mag2 = m_sqrt(mag2);
        v.x /= mag2;
        v.y /= mag2;
        v.z /= mag2;
    }
}
template <class T>
V<T> vnormalized(V<T> v)
{
    const T mag2 = v.x * v.x + v.y * v.y + v.z * v.z;
    if (mag2 < VEC_EPS) return V<T>{0, 0, 0};
    if (mag2 == 1.0f || (mag2 > (1.0f - VEC_EPS) && mag2 < (1.0f + VEC_EPS))) return v;
    const T m = m_sqrt(mag2);
    return V<T>{v.x / m, v.y / m, v.z / m};
}
// VEC3 operator* (vec3.hpp:112-115): the cross product
template <class T>
V<T> cross(const V<T> &a, const V<T> &b)
{
    return V<T>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T>
T vdot(const V<T> &a, const V<T> &b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}

// QUAT::normalize (quat.hpp:147-165): scales by |q| (not 1/|q|)
template <class T>
void qnormalize(Q<T> &q)
{
    T mag2 = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    if (mag2 < QUAT_EPS) {
        q.x = q.y = q.z = 0;
        q.w = 1.0;
    } else if (mag2 == 1.0f || (mag2 > (1.0f - QUAT_EPS) && mag2 < (1.0f + QUAT_EPS))) {
    } else {
        mag2 = m_sqrt(mag2);
        q.x *= mag2;
        q.y *= mag2;
        q.z *= mag2;
        q.w *= mag2;
    }
}

// QUAT(axis, ang, inDegrees) (quat.hpp:227-238): the degree conversion runs
// in double (QUAT_PI is double) and is stored back into the Real angle
template <class T>
Q<T> quat_axis_angle(const V<T> &axis, T ang, bool in_degrees)
{
    ang = in_degrees ? (ang * QUAT_PI_D / 360.0f) : (ang * 0.5f);
    const T s = m_sin(ang);
    Q<T> q{axis.x * s, axis.y * s, axis.z * s, m_cos(ang)};
    qnormalize(q);
    return q;
}

// QUAT::nlerp (quat.hpp:172-192)
template <class T>
Q<T> nlerp(const Q<T> &a, const Q<T> &b, T t)
{
    if (t == 0.0 || (t < QUAT_EPS)) return a;
    if (t == 1.0f || (t > 1.0f - QUAT_EPS)) return b;
    const T dot = a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
    const T tA = dot >= 0 ? t : -t;
    const T tI = 1.0f - t;
    Q<T> r{a.x * tI + b.x * tA, a.y * tI + b.y * tA, a.z * tI + b.z * tA, a.w * tI + b.w * tA};
    qnormalize(r);
    return r;
}

// QUAT::transform (quat.hpp:279-284)
template <class T>
V<T> transform(const Q<T> &q, const V<T> &v)
{
    const T x = q.x, y = q.y, z = q.z, w = q.w;
    return V<T>{w * w * v.x + 2 * y * w * v.z - 2 * z * w * v.y + x * x * v.x + 2 * y * x * v.y + 2 * z * x * v.z -
                    z * z * v.x - y * y * v.x,
                2 * x * y * v.x + y * y * v.y + 2 * z * y * v.z + 2 * w * z * v.x - z * z * v.y + w * w * v.y -
                    2 * x * w * v.z - x * x * v.y,
                2 * x * z * v.x + 2 * y * z * v.y + z * z * v.z - 2 * w * y * v.x - y * y * v.z + 2 * w * x * v.y -
                    x * x * v.z + w * w * v.z};
}

// QUAT(p, q, scale) (quat.hpp:194-220): the rotation taking p towards q;
// ang*0.5*scale is a double expression handed to the Real sin/cos
template <class T>
Q<T> quat_between(const V<T> &p, const V<T> &q, T scale)
{
    T cosa = vdot(p, q);
    if (cosa < -1.0) cosa = -1.0;
    else if (cosa > 1.0) cosa = 1.0;
    if (cosa == 0 || (cosa >= -QUAT_EPS && cosa <= QUAT_EPS)) return Q<T>{0, 0, 0, 1.0};
    const T ang = m_acos(cosa);
    const V<T> axis = cross(p, q);
    const T sinang1 = m_sin((T)(ang * 0.5 * scale)) / m_sin(ang);
    return Q<T>{axis.x * sinang1, axis.y * sinang1, axis.z * sinang1, m_cos((T)(ang * 0.5 * scale))};
}

// The /*startcalc*/ block of params.cu:41-60 with the interpolation value i
// (params.cu has i = 1; scale.pl substitutes its eased value): the camera
// swings between two orientations 40 degrees apart about `up` while moving
// from (4,4,4) towards (3.1, 3.1, 3.1).
template <class T, class Cam>
void startcalc(double i_nlerp, double i_pos, Cam *cam)
{
    const V<T> dir{4, 4, 4};
    V<T> side{-4, 4, 4};
    vnormalize(side);
    V<T> up = cross(side, vnormalized(dir));
    vnormalize(up);
    const Q<T> rot0 = quat_axis_angle(up, (T)-20, true);
    const Q<T> rot1 = quat_axis_angle(up, (T)20, true);
    const Q<T> nrot = nlerp(rot0, rot1, (T)i_nlerp);
    V<T> nd = vnormalized(transform(nrot, dir));
    const T m1 = (T)-1.0;
    nd = V<T>{nd.x * m1, nd.y * m1, nd.z * m1};
    const V<T> c{(T)(4.0 - 0.9 * i_pos), (T)(4.0 - 0.9 * i_pos), (T)(4.0 - 0.9 * i_pos)};
    cam->C.x = c.x - nd.x;
    cam->C.y = c.y - nd.y;
    cam->C.z = c.z - nd.z;
    const Q<T> q = quat_between(V<T>{0, 0, 1}, nd, (T)1.0);
    cam->Q.x = q.x;
    cam->Q.y = q.y;
    cam->Q.z = q.z;
    cam->Q.w = q.w;
}

template <class T, class Prm, class Cam, class Light>
void params_init_t(Prm *prm, Cam *cam, Light *lights, uint32_t light_cap, uint32_t *n_lights)
{
    if (prm) {
        std::memset(prm, 0, sizeof(*prm));
        prm->d = (T)2.1;
        prm->settle = 18;
        prm->accum = 1008;
        prm->stepMethod = 2;
        prm->nearThreshold = (T)-1.0;
        prm->nearMultiplier = (T)2.0;
        prm->opaqueThreshold = (T)-0.75;
        prm->chaosThreshold = (T)-0.5;
        prm->depth = (T)4096u;   // res (params.cu:15)
        prm->jitter = (T)0.5;
        prm->refine = (T)32;
        prm->gradient = (T)0.01;
        prm->lMin = (T)0.0;
        prm->lMax = (T)4.0;
    }
    if (cam) {
        std::memset(cam, 0, sizeof(*cam));
        startcalc<T>(1.0, 1.0, cam);
        cam->M = (T)0.45;
    }
    if (lights && light_cap >= 1) {
        // the branch params_init takes (params.cu:95-110): one spot light
        Light &L = lights[0];
        std::memset(&L, 0, sizeof(L));
        L.C.x = (T)6.0f;
        L.C.y = (T)5.0f;
        L.C.z = (T)3.0f;
        L.Q.x = (T)0.710595f;
        L.Q.y = (T)0.282082f;
        L.Q.z = (T)-0.512168f;
        L.Q.w = (T)0.391368f;
        L.M = (T)0.500000;
        L.lightInnerCone = (T)0.904535f;
        L.lightOuterCone = (T)0.816497f;
        L.lightRange = (T)1.0;
        L.ambient.x = (T)0.1;
        L.diffuseColor.x = (T)1.0;
        L.diffuseColor.y = (T)0.25;
        L.diffuseColor.z = (T)0.125;
        L.diffuseColor.w = (T)1;
        L.diffusePower = (T)10.0;
        L.specularColor.x = L.specularColor.y = L.specularColor.z = L.specularColor.w = (T)1.0;
        L.specularPower = (T)10.0;
        L.specularHardness = (T)10.0;
    }
    if (n_lights) *n_lights = 1;
}

const char *const kPresetSeq = "BCABA";   // params.cu:39

int preset_common(char *seq, size_t seq_cap, uint32_t *width, uint32_t *height, uint32_t light_cap,
                  const void *lights, const char *fn)
{
    if (lights && light_cap < 1) return lyapgb::set_error(LYAP_ERR_CAPACITY, "%s: light_cap 0", fn);
    if (seq) {
        const size_t n = std::strlen(kPresetSeq) + 1;
        if (seq_cap < n) return lyapgb::set_error(LYAP_ERR_CAPACITY, "%s: sequence buffer holds %zu bytes", fn, seq_cap);
        std::memcpy(seq, kPresetSeq, n);
    }
    if (width) *width = 3840;   // default_imageWidth / Height (params.cu:17-18)
    if (height) *height = 2160;
    return LYAP_OK;
}

// scale.pl prints the eased value into params.cu with Perl's default
// number formatting (15 significant digits); the compiler reads that text
double as_source_literal(double i)
{
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.15g", i);
    return std::strtod(buf, nullptr);
}

// scene_cam_recalculate / scene_lights_recalculate (scene.cu:20-63) for the
// DOUBLE_REALS structs; the float forms live in lyap_scene.cpp
template <class T, class Cam>
void cam_recalc_t(Cam *cam)
{
    const T M = cam->M;
    Q<T> q{cam->Q.x, cam->Q.y, cam->Q.z, cam->Q.w};
    const V<T> Vv = vnormalized(transform(q, V<T>{0, 0, 1}));
    cam->V.x = Vv.x;
    cam->V.y = Vv.y;
    cam->V.z = Vv.z;
    const V<T> s0 = transform(q, V<T>{-M, -M, 1});
    cam->S0.x = s0.x;
    cam->S0.y = s0.y;
    cam->S0.z = s0.z;
    cam->lightInnerCone = vdot(Vv, vnormalized(transform(q, V<T>{-M, -M, (T)1.5})));
    cam->lightOuterCone = vdot(Vv, vnormalized(transform(q, V<T>{-M, -M, 1})));
    const V<T> dx = transform(q, V<T>{2 * M / (T)cam->renderWidth, 0, 0});
    const V<T> dy = transform(q, V<T>{0, 2 * M / (T)cam->renderHeight, 0});
    cam->SDX.x = dx.x;
    cam->SDX.y = dx.y;
    cam->SDX.z = dx.z;
    cam->SDY.x = dy.x;
    cam->SDY.y = dy.y;
    cam->SDY.z = dy.z;
}

}  // namespace

extern "C" {

int lyap_cam_recalculate_d(LyapCamD *cam, uint32_t tw, uint32_t th, uint32_t td)
{
    if (!cam) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_cam_recalculate_d: null camera");
    const uint32_t den = td > 0 ? td : cam->renderDenominator;
    if (den == 0) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_cam_recalculate_d: renderDenominator is 0");
    if (cam->M < 1e-6) cam->M = 1e-6;
    Q<double> q{cam->Q.x, cam->Q.y, cam->Q.z, cam->Q.w};
    qnormalize(q);
    cam->Q.x = q.x;
    cam->Q.y = q.y;
    cam->Q.z = q.z;
    cam->Q.w = q.w;
    if (td > 0) cam->renderDenominator = td;
    if (tw > 0) {
        cam->textureWidth = tw;
        cam->renderWidth = cam->textureWidth / cam->renderDenominator;
    }
    if (th > 0) {
        cam->textureHeight = th;
        cam->renderHeight = cam->textureHeight / cam->renderDenominator;
    }
    if (cam->renderWidth == 0 || cam->renderHeight == 0)
        return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_cam_recalculate_d: zero render size");
    cam_recalc_t<double>(cam);
    return LYAP_OK;
}

int lyap_lights_recalculate_d(LyapLightD *lights, size_t n)
{
    if (n && !lights) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_lights_recalculate_d: null lights");
    for (size_t l = 0; l < n; l++) {
        LyapLightD &L = lights[l];
        const Q<double> q{L.Q.x, L.Q.y, L.Q.z, L.Q.w};   // not normalised (scene.cu:20-29)
        const V<double> Vv = vnormalized(transform(q, V<double>{0, 0, 1}));
        L.V.x = Vv.x;
        L.V.y = Vv.y;
        L.V.z = Vv.z;
        L.lightInnerCone = vdot(Vv, vnormalized(transform(q, V<double>{-L.M, -L.M, 1.5})));
        L.lightOuterCone = vdot(Vv, vnormalized(transform(q, V<double>{-L.M, -L.M, 1})));
    }
    return LYAP_OK;
}


int lyap_params_init(LyapParams *prm, LyapCam *cam, LyapLight *lights, uint32_t light_cap, uint32_t *n_lights,
                     char *seq, size_t seq_cap, uint32_t *width, uint32_t *height)
{
    int rc = preset_common(seq, seq_cap, width, height, light_cap, lights, "lyap_params_init");
    if (rc) return rc;
    params_init_t<float>(prm, cam, lights, light_cap, n_lights);
    return LYAP_OK;
}

int lyap_params_init_d(LyapParamsD *prm, LyapCamD *cam, LyapLightD *lights, uint32_t light_cap, uint32_t *n_lights,
                       char *seq, size_t seq_cap, uint32_t *width, uint32_t *height)
{
    int rc = preset_common(seq, seq_cap, width, height, light_cap, lights, "lyap_params_init_d");
    if (rc) return rc;
    params_init_t<double>(prm, cam, lights, light_cap, n_lights);
    return LYAP_OK;
}

double lyap_ease_in_out_quart(double t, double b, double c, double d)
{
    // scale.pl:5-11 (despite its name, a quadratic ease in and out)
    t /= d / 2;
    if (t < 1) return c / 2 * t * t + b;
    t--;
    return -c / 2 * (t * (t - 2) - 1) + b;
}

int lyap_anim_camera(double i, LyapCam *cam)
{
    if (!cam) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_anim_camera: null camera");
    const double v = as_source_literal(i);
    startcalc<float>(v, v, cam);
    return LYAP_OK;
}

int lyap_anim_camera_d(double i, LyapCamD *cam)
{
    if (!cam) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_anim_camera_d: null camera");
    const double v = as_source_literal(i);
    startcalc<double>(v, v, cam);
    return LYAP_OK;
}

}  // extern "C"
