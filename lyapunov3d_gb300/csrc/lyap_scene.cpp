// lyap_scene.cpp -- the host scene helpers the reference runs before each
// launch (scene.hpp:11-15): sequence parsing, camera basis and spot-light
// cones.  Results are bit-identical to the reference's host build: every
// expression keeps the reference's operand types (a double literal there
// promotes the expression to double here too) and this file is compiled
// with -ffp-contract=off so nothing is fused.
#include <cmath>
#include <cstddef>
#include <cstdint>

#include "lyap_gb300.h"
#include "lyap_internal.h"

namespace {

struct Vec {
    float x, y, z;
    Vec() : x(0), y(0), z(0) {}
    Vec(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit Vec(const LyapVec &v) : x(v.x), y(v.y), z(v.z) {}
    LyapVec abi() const { return LyapVec{x, y, z}; }
};

inline Vec operator/(const Vec &a, float d) { return Vec(a.x / d, a.y / d, a.z / d); }
inline float dot(const Vec &a, const Vec &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// vec3.hpp:127-139
inline Vec normalized(const Vec &a)
{
    float mag2 = a.x * a.x + a.y * a.y + a.z * a.z;
    if (mag2 < 1e-12) return Vec();
    if (mag2 == 1.0f || (mag2 > (1.0f - 1e-12) && mag2 < (1.0f + 1e-12))) return a;
    return a / std::sqrt(mag2);
}

// QUAT::transform (quat.hpp:279-284); this term order is the one whose
// float rounding the reference's cameras carry.
inline Vec rotate(const LyapQuat &q, const Vec &v)
{
    const float x = q.x, y = q.y, z = q.z, w = q.w;
    return Vec(w * w * v.x + 2 * y * w * v.z - 2 * z * w * v.y + x * x * v.x + 2 * y * x * v.y + 2 * z * x * v.z -
                   z * z * v.x - y * y * v.x,
               2 * x * y * v.x + y * y * v.y + 2 * z * y * v.z + 2 * w * z * v.x - z * z * v.y + w * w * v.y -
                   2 * x * w * v.z - x * x * v.y,
               2 * x * z * v.x + 2 * y * z * v.y + z * z * v.z - 2 * w * y * v.x - y * y * v.z + 2 * w * x * v.y -
                   x * x * v.z + w * w * v.z);
}

// QUAT::normalize (quat.hpp:147-165).  It scales by |q| where a division
// is meant; unit quaternions leave it a no-op, others come out scaled by
// |q| as in the reference.
inline void quat_normalize(LyapQuat &q)
{
    float mag2 = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    if (mag2 < 1e-6) {
        q.x = q.y = q.z = 0;
        q.w = 1.0;
    } else if (mag2 == 1.0f || (mag2 > (1.0f - 1e-6) && mag2 < (1.0f + 1e-6))) {
        // unchanged
    } else {
        mag2 = std::sqrt(mag2);
        q.x *= mag2;
        q.y *= mag2;
        q.z *= mag2;
        q.w *= mag2;
    }
}

// The spot cone of a camera/light: cos of the angle between the axis V and
// the direction through screen corner (-M, -M, k).
inline float cone(const LyapQuat &q, const Vec &axis, float M, double k)
{
    return dot(axis, normalized(rotate(q, Vec(-M, -M, (float)k))));
}

}  // namespace

extern "C" {

int lyap_seq_parse(const char *str, int32_t *out, size_t cap, size_t *len)
{
    if (!str || !out || !len) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_seq_parse: null pointer");
    // scene.cu:69-108: A-D (any case) append symbols 0-3; a digit k appends k
    // more copies of the last letter (B before any letter); -1 terminates.
    size_t n = 0;
    int32_t last = 1;
    const unsigned char *p = reinterpret_cast<const unsigned char *>(str);
    do {
        const unsigned ch = *p;
        int reps;
        if (ch >= '1' && ch <= '9') {
            reps = (int)(ch - '0');
        } else if ((ch | 0x20u) >= 'a' && (ch | 0x20u) <= 'd') {
            last = (int32_t)((ch | 0x20u) - 'a');
            reps = 1;
        } else {
            return lyapgb::set_error(LYAP_ERR_SEQUENCE, "lyap_seq_parse: bad sequence letter '%c' (0x%02x) at %zu",
                                     ch >= 32 && ch < 127 ? (char)ch : '?', ch,
                                     (size_t)(p - reinterpret_cast<const unsigned char *>(str)));
        }
        for (int k = 0; k < reps; k++) {
            if (n + 1 >= cap) return lyapgb::set_error(LYAP_ERR_CAPACITY, "lyap_seq_parse: output holds %zu entries", cap);
            out[n++] = last;
        }
    } while (*(++p));
    if (n + 1 > cap) return lyapgb::set_error(LYAP_ERR_CAPACITY, "lyap_seq_parse: output holds %zu entries", cap);
    out[n++] = -1;
    *len = n;
    return LYAP_OK;
}

int lyap_cam_recalculate(LyapCam *cam, uint32_t tw, uint32_t th, uint32_t td)
{
    if (!cam) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_cam_recalculate: null camera");
    const uint32_t den = td > 0 ? td : cam->renderDenominator;
    if (den == 0) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_cam_recalculate: renderDenominator is 0");
    // scene.cu:31-63
    if (cam->M < 1e-6) cam->M = 1e-6;
    quat_normalize(cam->Q);
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
        return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_cam_recalculate: zero render size");
    const float M = cam->M;
    const Vec V = normalized(rotate(cam->Q, Vec(0, 0, 1)));
    cam->V = V.abi();
    cam->S0 = rotate(cam->Q, Vec(-M, -M, 1)).abi();
    cam->lightInnerCone = cone(cam->Q, V, M, 1.5);
    cam->lightOuterCone = cone(cam->Q, V, M, 1);
    cam->SDX = rotate(cam->Q, Vec(2 * M / (float)cam->renderWidth, 0, 0)).abi();
    cam->SDY = rotate(cam->Q, Vec(0, 2 * M / (float)cam->renderHeight, 0)).abi();
    return LYAP_OK;
}

int lyap_lights_recalculate(LyapLight *lights, size_t n)
{
    if (n && !lights) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_lights_recalculate: null lights");
    // scene.cu:20-29 (the light's quaternion is not normalised)
    for (size_t l = 0; l < n; l++) {
        LyapLight &L = lights[l];
        const Vec V = normalized(rotate(L.Q, Vec(0, 0, 1)));
        L.V = V.abi();
        L.lightInnerCone = cone(L.Q, V, L.M, 1.5);
        L.lightOuterCone = cone(L.Q, V, L.M, 1);
    }
    return LYAP_OK;
}

}  // extern "C"
