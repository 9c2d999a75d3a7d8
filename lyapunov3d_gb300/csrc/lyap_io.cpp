// lyap_io.cpp -- the reference front-ends' output files, headless: the PPM
// image and the raw LyapPoint dump of lyap_interactive.cu (save_ppm :570,
// save_points :617) and the raw float volume of lyap_calculate.cu (:84-86),
// with the reference's file-name convention.  Host code only.
#include <cstdio>
#include <cstring>

#include "lyap_gb300.h"
#include "lyap_internal.h"

namespace {

int write_all(const char *path, const void *data, size_t bytes, const char *fn)
{
    FILE *f = std::fopen(path, "wb");
    if (!f) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "%s: cannot open %s", fn, path);
    const size_t w = bytes ? std::fwrite(data, bytes, 1, f) : 1;
    const int c = std::fclose(f);
    if (w != 1 || c != 0) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "%s: write to %s failed", fn, path);
    return LYAP_OK;
}

}  // namespace

extern "C" {

int lyap_write_ppm(const char *path, const RGBA *rgba, uint32_t width, uint32_t height, int binary)
{
    const char *fn = "lyap_write_ppm";
    if (!path || !rgba) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "%s: null pointer", fn);
    if (width == 0 || height == 0) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "%s: empty image", fn);
    FILE *f = std::fopen(path, "wb");
    if (!f) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "%s: cannot open %s", fn, path);
    const size_t n = (size_t)width * height;
    int ok = 1;
    if (binary) {
        // P6 (an extension): the same pixels, one byte per channel
        ok = std::fprintf(f, "P6\n%u %u\n255\n", width, height) > 0;
        unsigned char buf[3 * 1024];
        for (size_t i = 0; i < n && ok;) {
            size_t k = 0;
            for (; k < 1024 && i < n; k++, i++) {
                buf[3 * k] = rgba[i].r;
                buf[3 * k + 1] = rgba[i].g;
                buf[3 * k + 2] = rgba[i].b;
            }
            ok = std::fwrite(buf, 3 * k, 1, f) == 1;
        }
    } else {
        // P3 exactly as save_ppm writes it: header, then "%3d %3d %3d " per
        // pixel in memory order (row 0 first), then one newline
        ok = std::fprintf(f, "P3\n%d %d\n%d\n", (int)width, (int)height, 255) > 0;
        for (size_t i = 0; i < n && ok; i++) ok = std::fprintf(f, "%3d %3d %3d ", rgba[i].r, rgba[i].g, rgba[i].b) > 0;
        if (ok) ok = std::fprintf(f, "\n") > 0;
    }
    const int c = std::fclose(f);
    if (!ok || c != 0) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "%s: write to %s failed", fn, path);
    return LYAP_OK;
}

int lyap_write_points(const char *path, const LyapPoint *points, size_t n)
{
    if (!path || (!points && n)) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_write_points: null pointer");
    return write_all(path, points, n * sizeof(LyapPoint), "lyap_write_points");
}

int lyap_write_exps(const char *path, const float *values, size_t n)
{
    if (!path || (!values && n)) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "lyap_write_exps: null pointer");
    return write_all(path, values, n * sizeof(float), "lyap_write_exps");
}

int lyap_output_name(char *buf, size_t cap, const char *kind, long stamp, uint32_t width, uint32_t height,
                     const char *seq, const LyapCam *cam, const LyapParams *prm, uint32_t elapsed_s, const char *ext)
{
    const char *fn = "lyap_output_name";
    if (!buf || !kind || !seq || !cam || !prm || !ext) return lyapgb::set_error(LYAP_ERR_INVALID_ARG, "%s: null pointer", fn);
    // lyap_interactive.cu:576-596: the leaf (at most 255 characters), then
    // "_time=<h>h<mm>m<ss>s" and the extension (timer_stop's split, :562-567)
    char leaf[256];
    std::snprintf(leaf, 255, "%s_%ld_%dx%d_%s_cx=%.8g_cy=%.8g_cz=%.8g_step=%d_D=%g_i=%d,%d_d=%d_j=%g_r=%d_ot=%g", kind,
                  stamp, (int)width, (int)height, seq, cam->C.x, cam->C.y, cam->C.z, (int)prm->stepMethod, prm->d,
                  (int)prm->settle, (int)prm->accum, (int)(unsigned int)prm->depth, prm->jitter,
                  (int)(unsigned int)prm->refine, prm->opaqueThreshold);
    // the time suffix goes through the reference's two 255-byte buffers
    char fmt[256], name[256];
    std::snprintf(fmt, 255, "%s_time=%%dh%%02dm%%02ds.%s", leaf, ext);
    const unsigned h = elapsed_s / 3600u, m = (elapsed_s / 60u) % 60u, s = elapsed_s % 60u;
    std::snprintf(name, 255, fmt, (int)h, (int)m, (int)s);
    const size_t need = std::strlen(name) + 1;
    if (need > cap) return lyapgb::set_error(LYAP_ERR_CAPACITY, "%s: name needs %zu bytes, buffer holds %zu", fn, need, cap);
    std::memcpy(buf, name, need);
    return LYAP_OK;
}

}  // extern "C"
