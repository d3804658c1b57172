// trace.cpp — the switch, the domain and the region names of trace.h.
#include "trace.h"

#include <cstdlib>
#include <cstring>

namespace wave {

bool trace_enabled()
{
    static const bool on = [] {
        const char* v = std::getenv("WAVE_TRACE");
        return !(v && std::strcmp(v, "0") == 0);
    }();
    return on;
}

nvtxDomainHandle_t trace_domain()
{
    static const nvtxDomainHandle_t d = nvtxDomainCreateA("WAVE");
    return d;
}

namespace {
// equation names in WAVE_EQ_* order, as the reference's region names spell them
const char* const kEq[] = {"acoustic", "elastic", "viscoelastic", "sh", "viscosh", "tmem", "emem", "viscotmem", "viscoemem"};
constexpr int kNumEq = sizeof(kEq) / sizeof(kEq[0]);

struct Names {
    char init[2][kNumEq][48];
    char step[2][kNumEq][48];
    Names()
    {
        for (int d = 0; d < 2; ++d)
            for (int e = 0; e < kNumEq; ++e) {
                const char* dim = d == 0 ? "2D" : "3D";
                std::strcpy(init[d][e], "ForwardSolver.init");
                std::strcat(init[d][e], dim);
                std::strcat(init[d][e], kEq[e]);
                std::strcpy(step[d][e], "ForwardSolver.timestep");
                std::strcat(step[d][e], dim);
                std::strcat(step[d][e], kEq[e]);
            }
    }
};
const Names& names()
{
    static const Names n;
    return n;
}
} // namespace

const char* trace_init_name(int dimension, int equation)
{
    if (equation < 0 || equation >= kNumEq) return "ForwardSolver.init";
    return names().init[dimension == 3 ? 1 : 0][equation];
}

const char* trace_timestep_name(int dimension, int equation)
{
    if (equation < 0 || equation >= kNumEq) return "ForwardSolver.timestep";
    return names().step[dimension == 3 ? 1 : 0][equation];
}

} // namespace wave
