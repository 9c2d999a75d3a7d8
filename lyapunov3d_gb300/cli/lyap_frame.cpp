// lyap_frame -- one frame of the reference's render front-end
// (lyap_interactive.cu:696-741, which renders a single frame and exits),
// headless: the params_init preset (params.cu:21-114), camera and lights
// prepared as scene_cam_recalculate / scene_lights_recalculate do, one
// render through the C ABI, then the PPM image and the LyapPoint dump under
// the reference's file names (save_ppm / save_points, :570-652).
//
//   lyap_frame [--width W] [--height H] [--seq STR] [--variant plain|product]
//              [--binary] [--no-points] [--out-dir DIR] [--directional]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "lyap_gb300.h"

static int fail(const char *what)
{
    std::fprintf(stderr, "lyap_frame: %s: %s\n", what, lyap_last_error_string());
    return 1;
}

int main(int argc, char **argv)
{
    LyapParams prm;
    LyapCam cam;
    LyapLight lights[LYAP_MAX_LIGHTS];
    uint32_t n_lights = 0, width = 0, height = 0;
    char preset_seq[64];
    if (lyap_params_init(&prm, &cam, lights, LYAP_MAX_LIGHTS, &n_lights, preset_seq, sizeof(preset_seq), &width,
                         &height))
        return fail("params_init");
    std::string seq_str = preset_seq, out_dir = ".";
    uint32_t variant = LYAP_VARIANT_PLAIN, light_model = LYAP_LIGHT_SPOT;
    bool binary = false, points = true;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        const char *v = (i + 1 < argc) ? argv[i + 1] : nullptr;
        if (a == "--width" && v) { width = (uint32_t)std::strtoul(v, nullptr, 10); i++; }
        else if (a == "--height" && v) { height = (uint32_t)std::strtoul(v, nullptr, 10); i++; }
        else if (a == "--seq" && v) { seq_str = v; i++; }
        else if (a == "--variant" && v) { variant = std::strcmp(v, "product") == 0 ? LYAP_VARIANT_PRODUCT : LYAP_VARIANT_PLAIN; i++; }
        else if (a == "--out-dir" && v) { out_dir = v; i++; }
        else if (a == "--binary") binary = true;
        else if (a == "--no-points") points = false;
        else if (a == "--directional") light_model = LYAP_LIGHT_DIRECTIONAL;
        else {
            std::fprintf(stderr, "usage: lyap_frame [--width W] [--height H] [--seq STR] [--variant plain|product] "
                                 "[--binary] [--no-points] [--out-dir DIR] [--directional]\n");
            return 2;
        }
    }
    std::vector<int32_t> seq(LYAP_MAX_SEQ_LEN);
    size_t seq_len = 0;
    if (lyap_seq_parse(seq_str.c_str(), seq.data(), seq.size(), &seq_len)) return fail("sequence");
    if (lyap_cam_recalculate(&cam, width, height, 1)) return fail("camera");
    if (lyap_lights_recalculate(lights, n_lights)) return fail("lights");
    const size_t npix = (size_t)width * height;
    std::vector<RGBA> rgba(npix);
    std::vector<LyapPoint> pts(points ? npix : 0);
    LyapRenderExt ext;
    std::memset(&ext, 0, sizeof(ext));
    ext.size = sizeof(ext);
    ext.variant = variant;
    ext.light_model = light_model;
    const long stamp = (long)std::time(nullptr);   // timer_start (lyap_interactive.cu:554)
    const auto t0 = std::chrono::steady_clock::now();
    if (lyap_render_host(&cam, &prm, seq.data(), seq_len, lights, n_lights, rgba.data(), points ? pts.data() : nullptr,
                         width, height, &ext, nullptr))
        return fail("render");
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const uint32_t elapsed = (uint32_t)(std::time(nullptr) - stamp);
    char name[512];
    if (lyap_output_name(name, sizeof(name), "Render", stamp, width, height, seq_str.c_str(), &cam, &prm, elapsed,
                         "ppm"))
        return fail("name");
    std::string path = out_dir + "/" + name;
    if (lyap_write_ppm(path.c_str(), rgba.data(), width, height, binary ? 1 : 0)) return fail("ppm");
    std::printf("%s\n", path.c_str());
    if (points) {
        if (lyap_output_name(name, sizeof(name), "Points", stamp, width, height, seq_str.c_str(), &cam, &prm, elapsed,
                             "raw"))
            return fail("name");
        path = out_dir + "/" + name;
        if (lyap_write_points(path.c_str(), pts.data(), npix)) return fail("points");
        std::printf("%s\n", path.c_str());
    }
    std::printf("rendered %ux%u in %.3f s\n", width, height, secs);
    return 0;
}
