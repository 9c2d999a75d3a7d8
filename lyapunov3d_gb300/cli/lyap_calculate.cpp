// lyap_calculate -- the reference's headless volume front-end
// (lyap_calculate.cu:58-119) over the C ABI: the params_init preset, lambda
// at every voxel of an N^3 grid over [0, 4) (kernel_calc_volume's
// coordinates, kernel.cu:518-532), the floats written x-fastest to exps.raw.
//
//   lyap_calculate [--n N] [--seq STR] [--variant plain|product] [--out PATH]
//                  [--lo X --hi X]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "lyap_gb300.h"

static int fail(const char *what)
{
    std::fprintf(stderr, "lyap_calculate: %s: %s\n", what, lyap_last_error_string());
    return 1;
}

int main(int argc, char **argv)
{
    uint32_t n = 512;   // volumeWidth (lyap_calculate.cu:19)
    std::string out = "exps.raw", seq_override;
    uint32_t variant = LYAP_VARIANT_PLAIN;
    bool have_box = false;
    float lo = 0.0f, hi = 4.0f;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        const char *v = (i + 1 < argc) ? argv[i + 1] : nullptr;
        if (a == "--n" && v) { n = (uint32_t)std::strtoul(v, nullptr, 10); i++; }
        else if (a == "--out" && v) { out = v; i++; }
        else if (a == "--seq" && v) { seq_override = v; i++; }
        else if (a == "--variant" && v) { variant = std::strcmp(v, "product") == 0 ? LYAP_VARIANT_PRODUCT : LYAP_VARIANT_PLAIN; i++; }
        else if (a == "--lo" && v) { lo = std::strtof(v, nullptr); have_box = true; i++; }
        else if (a == "--hi" && v) { hi = std::strtof(v, nullptr); have_box = true; i++; }
        else {
            std::fprintf(stderr, "usage: lyap_calculate [--n N] [--seq STR] [--variant plain|product] [--out PATH] "
                                 "[--lo X --hi X]\n");
            return 2;
        }
    }
    LyapParams prm;
    char preset_seq[64];
    if (lyap_params_init(&prm, nullptr, nullptr, 0, nullptr, preset_seq, sizeof(preset_seq), nullptr, nullptr))
        return fail("params_init");
    const std::string seq_str = seq_override.empty() ? std::string(preset_seq) : seq_override;
    std::vector<int32_t> seq(LYAP_MAX_SEQ_LEN);
    size_t seq_len = 0;
    if (lyap_seq_parse(seq_str.c_str(), seq.data(), seq.size(), &seq_len)) return fail("sequence");
    const size_t count = (size_t)n * n * n;
    std::vector<float> exps(count);
    LyapVolumeExt ext;
    std::memset(&ext, 0, sizeof(ext));
    ext.size = sizeof(ext);
    ext.variant = variant;
    const float lo3[3] = {lo, lo, lo}, hi3[3] = {hi, hi, hi};
    if (lyap_volume_host(exps.data(), n, n, n, have_box ? lo3 : nullptr, have_box ? hi3 : nullptr, &prm, seq.data(),
                         seq_len, &ext, nullptr))
        return fail("volume");
    std::printf("Points size = %zu\n", count * sizeof(float));
    if (lyap_write_exps(out.c_str(), exps.data(), count)) return fail("write");
    std::printf("wrote %s (%ux%ux%u float32, x fastest)\n", out.c_str(), n, n, n);
    return 0;
}
