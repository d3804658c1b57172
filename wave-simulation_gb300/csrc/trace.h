// trace.h — NVTX ranges around the library's phases, the counterpart of the
// reference's SCAI_REGION markers (ForwardSolver2Delastic.cpp:121 and the
// other ForwardSolver*::run bodies, Simulation.cpp:446 timeLoop). The ranges
// live in the "WAVE" domain, so a profiler can select them (e.g. ncu --nvtx
// --nvtx-include "WAVE@WAVE-Simulation.timeLoop/"). NVTX calls return at once
// when no profiler is attached; WAVE_TRACE=0 in the environment turns them off
// entirely (the reference switches its regions with SCAI_TRACE).
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace wave {

// true unless WAVE_TRACE is set to "0" (read once)
bool trace_enabled();
nvtxDomainHandle_t trace_domain();

// an NVTX push/pop range in the WAVE domain for the lifetime of the object
class TraceRange {
public:
    explicit TraceRange(const char* name) : on_(trace_enabled()) { push(name); }
    ~TraceRange()
    {
        if (on_) nvtxDomainRangePop(trace_domain());
    }
    // ends this range and opens the next phase's in its place
    void next(const char* name)
    {
        if (!on_) return;
        nvtxDomainRangePop(trace_domain());
        push(name);
    }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;

private:
    void push(const char* name)
    {
        if (!on_) return;
        nvtxEventAttributes_t a{};
        a.version = NVTX_VERSION;
        a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
        a.messageType = NVTX_MESSAGE_TYPE_ASCII;
        a.message.ascii = name;
        nvtxDomainRangePushEx(trace_domain(), &a);
    }
    bool on_;
};

// "ForwardSolver.init<dim><equation>" / "ForwardSolver.timestep<dim><equation>"
// names of a configuration, as the reference's solvers call their regions
const char* trace_init_name(int dimension, int equation);
const char* trace_timestep_name(int dimension, int equation);

} // namespace wave
