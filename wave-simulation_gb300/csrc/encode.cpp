// encode.cpp — source encoding: the shots of an acquisition regrouped into
// NumShotDomains super-shots, Sources::calcSourceSettingsEncode
// (Acquisition/Sources.cpp:569-660) for time-domain modelling
// (gradientDomain = 0) and frequency-domain modelling (gradientDomain != 0,
// where every shot of a super-shot is given its own frequency of the
// encoding's frequency list). One source row per shot, as the reference
// assumes.
// Mode 1 assigns the first NumShotDomains shots to super-shots 1.. in order and
// every later shot to a random super-shot that is not yet full, then flips
// the sign of each shot's amplitude at random; mode 2 deals the shots out in
// turn; mode 3 gives each super-shot a contiguous run of shots. Super-shot k
// (0-based) is numbered NumShotDomains * 10^4 + 1 + k. The random numbers are
// the C library's rand() after srand(seed), as in the reference, so a seed
// reproduces the reference's assignment on the same C library.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "wave_internal.h"

namespace {

// the super-shot assignment of the time-domain encoding with the rand() stream
// already seeded; returns shots per super-shot
int assign(int mode, int num_domains, int n, const float* amp, int* shot_no_out, float* amp_out)
{
    const int perSuper = static_cast<int>(std::ceil(static_cast<float>(n) / num_domains));
    const double base = num_domains * 1e4 + 1;
    for (int i = 0; i < n; ++i) amp_out[i] = amp[i];
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
    return perSuper;
}

bool check_args(const char* who, int mode, int num_domains, int n, const void* a, const void* b, const void* c)
{
    if (mode < 1 || mode > 3 || num_domains < 1 || n < 1 || !a || !b || !c) {
        wave::set_global_error(std::string(who) + ": invalid arguments (mode 1..3, num_domains >= 1, n >= 1)");
        return false;
    }
    if (n < num_domains) {
        wave::set_global_error(std::string(who) + ": numshots = " + std::to_string(n) + " < NumShotDomains = " +
                               std::to_string(num_domains));
        return false;
    }
    return true;
}

// the frequency list of the frequency-domain encoding (Sources.cpp:587-611):
// df = 1 / (nFFT DT) with nFFT the next power of two of NT - 1
// (Common::calcNextPowTwo), indices ceil(fc / df); encoded shots take every
// second frequency from an even first index, unencoded ones every frequency of
// the widened band [ceil(fc1 index / 2), 2 fc2 index]
std::vector<float> frequency_list(bool encoded, float fc1, float fc2, float T, float DT, float cpmlFc)
{
    if (fc2 == 0.0f) fc2 = cpmlFc * 2.0f;
    const int NT = static_cast<int>(static_cast<double>(T / DT) + 0.5);   // (T / DT) + 0.5 as in Sources.cpp:592
    float e = std::log(static_cast<float>(NT - 1));
    e /= std::log(2.0);
    e = std::ceil(e);
    const int nFFT = static_cast<int>(std::pow(2.0f, e));
    const float df = 1.0f / (static_cast<float>(nFFT) * DT);
    int i1 = static_cast<int>(std::ceil(fc1 / df)), i2 = static_cast<int>(std::ceil(fc2 / df));
    int n;
    float step;
    if (!encoded) {
        i1 = static_cast<int>(std::ceil(static_cast<float>(i1) / 2.0f));
        i2 *= 2;
        if (i1 == 0) i1 = 1;
        n = static_cast<int>(std::ceil(static_cast<float>(i2 - i1 + 1)));
        step = df;
    } else {
        if (i1 == 0) i1 = 2;
        if (i1 % 2 == 1) i1 += 1;
        n = static_cast<int>(std::ceil(static_cast<float>(i2 - i1 + 1) / 2.0f));
        step = 2.0f * df;
    }
    std::vector<float> f(n > 0 ? n : 0);
    const float start = static_cast<float>(i1) * df;
    for (int k = 0; k < n; ++k) f[k] = start + static_cast<float>(k) * step;
    return f;
}

} // namespace

extern "C" int wave_encode_sources(int mode, int num_domains, unsigned int seed, int n, const int* shot_no, const float* amp,
                                   int* shot_no_out, float* amp_out)
{
    if (!check_args("wave_encode_sources", mode, num_domains, n, shot_no, amp, shot_no_out) || !amp_out) {
        if (!amp_out) wave::set_global_error("wave_encode_sources: invalid arguments (amp_out)");
        return WAVE_ERR_ARG;
    }
    std::srand(seed);
    assign(mode, num_domains, n, amp, shot_no_out, amp_out);
    return WAVE_OK;
}

extern "C" int wave_encode_frequencies(int encoded, double fc1, double fc2, double T, double DT, double cpml_fc, float* freqs,
                                       int cap, int* nfreq)
{
    if (!nfreq || DT <= 0.0 || T <= DT) {
        wave::set_global_error("wave_encode_frequencies: invalid arguments");
        return WAVE_ERR_ARG;
    }
    const std::vector<float> f = frequency_list(encoded != 0, static_cast<float>(fc1), static_cast<float>(fc2), static_cast<float>(T),
                                                static_cast<float>(DT), static_cast<float>(cpml_fc));
    *nfreq = static_cast<int>(f.size());
    if (freqs)
        for (int k = 0; k < std::min(cap, *nfreq); ++k) freqs[k] = f[k];
    return WAVE_OK;
}

extern "C" int wave_encode_sources_frequency(int mode, int num_domains, unsigned int seed, int n, const float* amp, double fc1,
                                             double fc2, double T, double DT, double cpml_fc, int* shot_no_out, float* amp_out,
                                             float* fc_out)
{
    if (!check_args("wave_encode_sources_frequency", mode, num_domains, n, amp, shot_no_out, amp_out) || !fc_out || DT <= 0.0 ||
        T <= DT) {
        if (!fc_out || DT <= 0.0 || T <= DT) wave::set_global_error("wave_encode_sources_frequency: invalid arguments");
        return WAVE_ERR_ARG;
    }
    const std::vector<float> f = frequency_list(true, static_cast<float>(fc1), static_cast<float>(fc2), static_cast<float>(T),
                                                static_cast<float>(DT), static_cast<float>(cpml_fc));
    const int nf = static_cast<int>(f.size());
    const int perSuper = static_cast<int>(std::ceil(static_cast<float>(n) / num_domains));
    if (nf < perSuper) {
        wave::set_global_error("wave_encode_sources_frequency: the number of frequencies (" + std::to_string(nf) +
                               ") is less than the shots per super-shot (" + std::to_string(perSuper) + ")");
        return WAVE_ERR_ARG;
    }
    std::srand(seed);
    assign(mode, num_domains, n, amp, shot_no_out, amp_out);
    // super-shots in order of first appearance; each of its shots a distinct
    // random frequency of the list (Sources.cpp:641-660), continuing the stream
    std::vector<int> order;
    for (int i = 0; i < n; ++i)
        if (std::find(order.begin(), order.end(), shot_no_out[i]) == order.end()) order.push_back(shot_no_out[i]);
    for (int k = 0; k < std::min(num_domains, static_cast<int>(order.size())); ++k) {
        std::vector<int> used(nf, 0);
        for (int i = 0; i < n; ++i) {
            if (shot_no_out[i] != order[k]) continue;
            int j = std::rand() % nf;
            while (used[j] > 0) j = std::rand() % nf;
            ++used[j];
            fc_out[i] = f[j];
        }
    }
    return WAVE_OK;
}
