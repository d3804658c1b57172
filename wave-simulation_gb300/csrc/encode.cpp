// encode.cpp — source encoding: the shots of an acquisition regrouped into
// NumShotDomains super-shots, Sources::calcSourceSettingsEncode
// (Acquisition/Sources.cpp:569-660) for time-domain modelling
// (gradientDomain = 0). One source row per shot, as the reference assumes.
// Mode 1 assigns the first NumShotDomains shots to super-shots 1.. in order and
// every later shot to a random super-shot that is not yet full, then flips
// the sign of each shot's amplitude at random; mode 2 deals the shots out in
// turn; mode 3 gives each super-shot a contiguous run of shots. Super-shot k
// (0-based) is numbered NumShotDomains * 10^4 + 1 + k. The random numbers are
// the C library's rand() after srand(seed), as in the reference, so a seed
// reproduces the reference's assignment on the same C library.
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "wave_internal.h"

extern "C" int wave_encode_sources(int mode, int num_domains, unsigned int seed, int n, const int* shot_no, const float* amp,
                                   int* shot_no_out, float* amp_out)
{
    if (mode < 1 || mode > 3 || num_domains < 1 || n < 1 || !shot_no || !amp || !shot_no_out || !amp_out) {
        wave::set_global_error("wave_encode_sources: invalid arguments (mode 1..3, num_domains >= 1, n >= 1)");
        return WAVE_ERR_ARG;
    }
    if (n < num_domains) {
        wave::set_global_error("wave_encode_sources: numshots = " + std::to_string(n) + " < NumShotDomains = " + std::to_string(num_domains));
        return WAVE_ERR_ARG;
    }
    const int perSuper = static_cast<int>(std::ceil(static_cast<float>(n) / num_domains));
    const double base = num_domains * 1e4 + 1;
    for (int i = 0; i < n; ++i) amp_out[i] = amp[i];
    std::srand(seed);
    std::vector<int> history(num_domains, 0);
    if (mode == 1) {
        for (int i = 0; i < n; ++i) {
            int k;
            if (i < num_domains) {
                k = i;
            } else {
                k = std::rand() % num_domains;
                while (history[k] >= perSuper) k = std::rand() % num_domains;
            }
            ++history[k];
            shot_no_out[i] = static_cast<int>(base + k);
        }
        for (int i = 0; i < n; ++i) {
            const int s = std::rand() % 2;
            amp_out[i] *= s > 0 ? 1.0f : -1.0f;
        }
    } else if (mode == 2) {
        for (int i = 0; i < n; ++i) shot_no_out[i] = static_cast<int>(base + i % num_domains);
    } else {
        for (int i = 0; i < n; ++i) shot_no_out[i] = static_cast<int>(base + i / perSuper);
    }
    (void)shot_no;
    return WAVE_OK;
}
