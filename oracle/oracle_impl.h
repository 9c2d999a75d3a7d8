/*
 * oracle_impl.h -- body of the oracle restatement, included twice by
 * lyap_oracle.c: once with R = float (the reference's default build) and
 * once with R = double (its DOUBLE_REALS build, structs.hpp:10-13).
 * TEST INFRASTRUCTURE ONLY (see lyap_oracle.h).
 *
 * Every expression keeps the reference's operand types and evaluation order,
 * because bit-exact agreement with the reference's host build is the pin:
 * a literal such as 1.0 or 0.0 in the reference promotes a float expression
 * to double there, and it does so here too.  Compiled with
 * -ffp-contract=off so no multiply-add is fused.
 *
 * Macros supplied by the includer:
 *   R, SFX(name), RLOG, RSQRT, RSIN, RCOS, RACOS,
 *   VEC, QUAT, COLOR, CAM, LIGHT, PARAMS, POINT, LAMBDA(P, d) (lambda call)
 */

#define VEC_EPSILON (1e-12)   /* vec3.hpp:10 */
#define QUAT_EPSILON (1e-6)   /* quat.hpp:12 */

/* ---- VEC3 (vec3.hpp:30-154) -------------------------------------------- */
static inline VEC SFX(v3)(R x, R y, R z) { VEC v; v.x = x; v.y = y; v.z = z; return v; }
static inline VEC SFX(vadd)(VEC a, VEC b) { return SFX(v3)(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline VEC SFX(vsub)(VEC a, VEC b) { return SFX(v3)(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline VEC SFX(vscale)(VEC a, R s) { return SFX(v3)(a.x * s, a.y * s, a.z * s); }
static inline VEC SFX(vdiv)(VEC a, R d) { return SFX(v3)(a.x / d, a.y / d, a.z / d); }
static inline R SFX(vdot)(VEC a, VEC b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline R SFX(vmag2)(VEC a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline R SFX(vmag)(VEC a) { return RSQRT(a.x * a.x + a.y * a.y + a.z * a.z); }

/* normalize()/normalized(): zero below 1e-12, untouched when |v|^2 is 1
 * within 1e-12 (only exactly 1 in float), else divided by |v|. */
static inline VEC SFX(vnormalized)(VEC a)
{
    R mag2 = a.x * a.x + a.y * a.y + a.z * a.z;
    if (mag2 < VEC_EPSILON)
        return SFX(v3)(0, 0, 0);
    else if (mag2 == 1.0f || (mag2 > (1.0f - VEC_EPSILON) && mag2 < (1.0f + VEC_EPSILON)))
        return a;
    else
        return SFX(vdiv)(a, RSQRT(mag2));
}

/* VEC3::clamp(T) (vec3.hpp:190-193): the conditional is evaluated in double. */
static inline R SFX(clamp01)(R that) { return that < 0.0 ? 0.0 : that > 1.0 ? 1.0 : that; }

/* ---- COLOR (color.hpp:320-395) ----------------------------------------- */
static inline COLOR SFX(c4)(R x, R y, R z, R w) { COLOR c; c.x = x; c.y = y; c.z = z; c.w = w; return c; }
static inline COLOR SFX(cadd)(COLOR a, COLOR b) { return SFX(c4)(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline COLOR SFX(cscale)(COLOR a, R s) { return SFX(c4)(a.x * s, a.y * s, a.z * s, a.w * s); }

/* ---- QUAT (quat.hpp:147-284) ------------------------------------------- */
/* normalize() multiplies by |q| where a divide is meant (quat.hpp:159-163,
 * hazard H9); kept, because unit quaternions make it inert. */
static inline void SFX(qnormalize)(QUAT *q)
{
    R mag2 = q->x * q->x + q->y * q->y + q->z * q->z + q->w * q->w;
    if (mag2 < QUAT_EPSILON) {
        q->x = q->y = q->z = 0;
        q->w = 1.0;
    } else if (mag2 == 1.0f || (mag2 > (1.0f - QUAT_EPSILON) && mag2 < (1.0f + QUAT_EPSILON))) {
        /* unchanged */
    } else {
        mag2 = RSQRT(mag2);
        q->x *= mag2;
        q->y *= mag2;
        q->z *= mag2;
        q->w *= mag2;
    }
}

/* QUAT::transform (quat.hpp:279-284), term order kept for bit-exactness. */
static inline VEC SFX(qtransform)(QUAT q, VEC v)
{
    R x = q.x, y = q.y, z = q.z, w = q.w;
    return SFX(v3)(
        w*w*v.x + 2*y*w*v.z - 2*z*w*v.y + x*x*v.x + 2*y*x*v.y + 2*z*x*v.z - z*z*v.x - y*y*v.x,
        2*x*y*v.x + y*y*v.y + 2*z*y*v.z + 2*w*z*v.x - z*z*v.y + w*w*v.y - 2*x*w*v.z - x*x*v.y,
        2*x*z*v.x + 2*y*z*v.y + z*z*v.z - 2*w*y*v.x - y*y*v.z + 2*w*x*v.y - x*x*v.z + w*w*v.z);
}

/* ---- scene.cu:20-63 ----------------------------------------------------- */
void SFX(orc_lights_recalculate_impl)(LIGHT *lights, size_t n)
{
    for (size_t l = 0; l < n; l++) {
        LIGHT *L = &lights[l];
        L->V = SFX(vnormalized)(SFX(qtransform)(L->Q, SFX(v3)(0, 0, 1)));
        L->lightInnerCone = SFX(vdot)(L->V, SFX(vnormalized)(SFX(qtransform)(L->Q, SFX(v3)(-L->M, -L->M, 1.5))));
        L->lightOuterCone = SFX(vdot)(L->V, SFX(vnormalized)(SFX(qtransform)(L->Q, SFX(v3)(-L->M, -L->M, 1))));
    }
}

void SFX(orc_cam_recalculate_impl)(CAM *cam, uint32_t tw, uint32_t th, uint32_t td)
{
    if (cam->M < 1e-6)
        cam->M = 1e-6;
    SFX(qnormalize)(&cam->Q);
    if (td > 0)
        cam->renderDenominator = td;
    if (tw > 0) {
        cam->textureWidth = tw;
        cam->renderWidth = cam->textureWidth / cam->renderDenominator;
    }
    if (th > 0) {
        cam->textureHeight = th;
        cam->renderHeight = cam->textureHeight / cam->renderDenominator;
    }
    cam->V = SFX(vnormalized)(SFX(qtransform)(cam->Q, SFX(v3)(0, 0, 1)));
    cam->S0 = SFX(qtransform)(cam->Q, SFX(v3)(-cam->M, -cam->M, 1));
    cam->lightInnerCone = SFX(vdot)(cam->V, SFX(vnormalized)(SFX(qtransform)(cam->Q, SFX(v3)(-cam->M, -cam->M, 1.5))));
    cam->lightOuterCone = SFX(vdot)(cam->V, SFX(vnormalized)(SFX(qtransform)(cam->Q, SFX(v3)(-cam->M, -cam->M, 1))));
    VEC SX = SFX(v3)(2 * cam->M / (R)cam->renderWidth, 0, 0);
    cam->SDX = SFX(qtransform)(cam->Q, SX);
    VEC SY = SFX(v3)(0, 2 * cam->M / (R)cam->renderHeight, 0);
    cam->SDY = SFX(qtransform)(cam->Q, SY);
}

/* ---- raymarch (kernel.cu:156-486) --------------------------------------- */
/* prop (float instantiation only; NULL = the reference's march): the
 * product's learned-proposal march, restated for its own parity check --
 * after every march step, a run of up to prop->run positions whose grid
 * cell holds a value >= prop->tau is skipped (never the last position before
 * t1 or the cap); the position after the run is evaluated and confirms it
 * when its lambda is above prop->tau, else every position from the run's
 * first through the confirming one is evaluated exactly.  counts[0] is then
 * the evaluated march samples; pcounts (may be NULL) receives the skipped
 * positions and the rewound runs. */
int SFX(orc_raymarch_impl)(int mode, POINT *point, uint32_t sx, uint32_t sy,
                           const CAM *cam, const PARAMS *prm,
                           const int32_t *seq, uint32_t *counts,
                           const OrcProposal *prop, uint32_t *pcounts)
{
    uint32_t nm = 0, nh = 0, nn = 0;
    uint32_t ns = 0, nrew = 0, noskip = 0;   /* proposal: skipped, rewound, exact until */
    (void)mode;
    if (counts) counts[0] = counts[1] = counts[2] = 0;
    if (pcounts) pcounts[0] = pcounts[1] = 0;
#define ORC_COUNTS() do { if (counts) { counts[0] = nm - ns; counts[1] = nh; counts[2] = nn; } \
                          if (pcounts) { pcounts[0] = ns; pcounts[1] = nrew; } } while (0)

    VEC V = SFX(vadd)(SFX(vadd)(cam->S0, SFX(vscale)(cam->SDX, (R)sx)), SFX(vscale)(cam->SDY, (R)sy));
    V = SFX(vnormalized)(V);
    V = SFX(vdiv)(V, cam->M);

    /* H5: the box is [lMin, lMax]^3, in double like the 0.0 / 4.0 literals. */
    const double LMIN = (double)prm->lMin, LMAX = (double)prm->lMax;

    VEC P, N;
    R a, c, l, t;
    R t0 = 3.40282347e+38F, t1 = 0;
    R ts[6];
    ts[0] = (V.x != 0.0f) ? ((LMIN - cam->C.x) / V.x) : INFINITY;
    ts[1] = (V.x != 0.0f) ? ((LMAX - cam->C.x) / V.x) : INFINITY;
    ts[2] = (V.y != 0.0f) ? ((LMIN - cam->C.y) / V.y) : INFINITY;
    ts[3] = (V.y != 0.0f) ? ((LMAX - cam->C.y) / V.y) : INFINITY;
    ts[4] = (V.z != 0.0f) ? ((LMIN - cam->C.z) / V.z) : INFINITY;
    ts[5] = (V.z != 0.0f) ? ((LMAX - cam->C.z) / V.z) : INFINITY;

    /* Drop plane hits outside the other two axes' extent (kernel.cu:204-244). */
    for (int k = 0; k < 6; k++) {
        if (ts[k] != INFINITY) {
            P = SFX(vadd)(cam->C, SFX(vscale)(V, ts[k]));
            R u, w;
            if (k < 2)      { u = P.y; w = P.z; }
            else if (k < 4) { u = P.x; w = P.z; }
            else            { u = P.x; w = P.y; }
            if (u < LMIN || u > LMAX || w < LMIN || w > LMAX)
                ts[k] = NAN;
        }
    }

    int i0 = -1, i1 = -1;
    for (int k = 0; k < 6; k++) {
        if (isfinite(ts[k])) {
            if (i0 == -1 || ts[k] < t0) t0 = ts[i0 = k];
            if (i1 == -1 || ts[k] > t1) t1 = ts[i1 = k];
        }
    }
    if (i0 == -1 && i1 == -1)
        return 1;
    else if (i1 == -1 || i0 == i1) {
        i1 = i0;
        t1 = t0;
        i0 = 0;
        t0 = 0;
    }
    if (t0 < 0)
        t0 = 0;

    t = t0;
    P = SFX(vadd)(cam->C, SFX(vscale)(V, t));
    a = 0;
    c = 0;

    R dt, Ndt, Fdt;
    switch (prm->stepMethod) {
    case 1:
        Fdt = (t1 - t0) / prm->depth;
        break;
    case 2:
    default:
        Fdt = SFX(vmag)(V) / prm->depth;
    }
    dt = Fdt;
    Ndt = dt / prm->nearMultiplier;
    int near = 0;

    /* Bound on march samples: every step is at least min(Fdt, Ndt) long, so
     * a ray leaves [t0, t1] well within this many; a non-positive or NaN
     * step gives the global bound ORC_MARCH_MAX. */
    R dmin = Fdt < Ndt ? Fdt : Ndt;
    double capd = ceil((double)(t1 - t0) / (double)dmin * 1.001) + 16.0;
    uint32_t cap = (capd > 0.0 && capd < (double)ORC_MARCH_MAX) ? (uint32_t)capd : ORC_MARCH_MAX;

    l = LAMBDA(P, prm->d); nm++;

    while (l > prm->opaqueThreshold) {
        if (nm >= cap) {
            ORC_COUNTS();
            return 1;
        }
        if (prm->jitter != 0.0) {
            R jit = l - trunc(l);
            if (jit < 0)
                jit = 1.0 - jit * prm->jitter;
            else
                jit = 1.0 + jit * prm->jitter;
            if (isfinite(jit)) {
                t += dt * jit;
                P = SFX(vadd)(P, SFX(vscale)(V, dt * jit));
            } else {
                t += dt;
                P = SFX(vadd)(P, SFX(vscale)(V, dt));
            }
        } else {
            t += dt;
            P = SFX(vadd)(P, SFX(vscale)(V, dt));
        }
        if (t > t1) {
            ORC_COUNTS();
            return 1;
        }
        if (prop && nm >= noskip) {
            uint32_t k = 0;
            VEC Q = P;
            R tq = t;
            while (k < prop->run && nm + k + 1 < cap && orc_prop_skippable(prop, (float)Q.x, (float)Q.y, (float)Q.z)) {
                R tn = tq + dt;
                if (tn > t1) break;
                tq = tn;
                Q = SFX(vadd)(Q, SFX(vscale)(V, dt));
                k++;
            }
            if (k) {
                R lc = LAMBDA(Q, prm->d);
                if (lc > prop->tau) {
                    /* confirmed: the run is skipped, lc is the march sample at Q */
                    P = Q;
                    t = tq;
                    nm += k;
                    ns += k;
                    l = lc;
                    nm++;
                    if (l > prm->chaosThreshold)
                        c += l;
                    else if (l > prm->opaqueThreshold)
                        a += l;
                    continue;
                }
                /* rewound: march exactly through the confirming position */
                noskip = nm + k + 1;
                nrew++;
            }
        }
        l = LAMBDA(P, prm->d); nm++;
        if (l > prm->chaosThreshold)
            c += l;
        else if (l > prm->opaqueThreshold)
            a += l;
        if (l <= prm->nearThreshold && !near) {
            near = 1;
            dt = Ndt;
        } else if (l > prm->nearThreshold && near) {
            near = 0;
            dt = Fdt;
        }
    }
    if (t > t1) {
        ORC_COUNTS();
        return 1;
    }

    /* Honing (kernel.cu:402-441): back and forth at halving speed. */
    int sign = 0, osign;
    R Qdt = dt * -0.5f;
    VEC QdV = SFX(vscale)(V, Qdt);
    R Qt1 = t;
    R Qt0 = t - dt;
    R min_Qdt = dt / prm->refine;
    while (t <= Qt1 && t >= Qt0 && (Qdt <= -min_Qdt || Qdt >= min_Qdt) && nh < ORC_HONE_CAP) {
        t += Qdt;
        P = SFX(vadd)(P, QdV);
        l = LAMBDA(P, prm->d); nh++;
        if (l == prm->opaqueThreshold)
            break;
        osign = sign;
        sign = (l < prm->opaqueThreshold) ? 0 : 1;
        if (sign != osign) {
            Qdt *= -0.5f;
            QdV = SFX(vscale)(QdV, -0.5f);
        }
    }

    /* Normal from six central-difference samples (kernel.cu:456-473). */
    R mag = dt * prm->gradient;
    VEC Ps[6];
    for (int k = 0; k < 6; k++) Ps[k] = P;
    Ps[0].x -= mag;
    Ps[1].x += mag;
    Ps[2].y -= mag;
    Ps[3].y += mag;
    Ps[4].z -= mag;
    Ps[5].z += mag;
    R ls[6];
    for (int k = 0; k < 6; k++) {
        ls[k] = LAMBDA(Ps[k], prm->d);
        nn++;
    }
    N.x = ls[1] - ls[0];
    N.y = ls[3] - ls[2];
    N.z = ls[5] - ls[4];
    N = SFX(vnormalized)(N);

    point->P = P;
    point->N = N;
    point->a = a;
    point->c = c;
    point->l = l;
    ORC_COUNTS();
    return 0;
#undef ORC_COUNTS
}
