// forward_solver.hpp — C++ host mirror of the reference's ForwardSolver plugin
// over the C ABI of include/wave.h. Header-only; link against libwavegpu.so.
//
// Mirrors (src/ForwardSolver/ForwardSolver.hpp:25-70, ForwardSolverFactory.cpp:4-67):
//   Factory<float>::Create(dimension, type)          -> wave::gpu::Factory::Create
//   initForwardSolver(config, derivatives, ...)      -> initForwardSolver(wave_config)
//   prepareForModelling(model, DT)                   -> prepareForModelling(Model)
//   run(receiver, sources, model, wavefield, derivatives, t) -> run(t) / run(t0, t1)
//   resetCPML()                                      -> resetCPML()
// Errors are thrown as wave::gpu::Error, as the reference throws
// COMMON_THROWEXCEPTION / SCAI_ASSERT_ERROR.
#pragma once

#include <algorithm>
#include <cctype>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/wave.h"

namespace wave {
namespace gpu {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(const wave_handle* h, int rc)
{
    if (rc != WAVE_OK) throw Error(rc, wave_last_error(h));
}

// Material arrays in the reference's index order (x fastest, then z, then y).
struct Model {
    std::vector<float> rho, vp, vs, taup, taus;         // seismic
    std::vector<float> eps_r, sigma, mu_r;              // EM
    std::vector<float> tau_eps, tau_sigma;              // visco-EM relaxation (tauEpsilon, tauSigmar)
};

// Acquisition in the reference's terms: 1-D grid indices, component types
// (1=P 2=VX 3=VY 4=VZ; EM 1=EZ 2=EX 3=EY 4=HZ) and source signals (ns x NT).
struct Acquisition {
    std::vector<int64_t> index;
    std::vector<int> type;
    std::vector<float> signals;
};

class ForwardSolver {
  public:
    ForwardSolver(std::string dimension, std::string type) : dim_(std::move(dimension)), type_(std::move(type)) {}
    ~ForwardSolver()
    {
        if (h_) wave_solver_destroy(h_);
    }
    ForwardSolver(const ForwardSolver&) = delete;
    ForwardSolver& operator=(const ForwardSolver&) = delete;

    // The configuration must describe the equation this solver was created
    // for (ForwardSolverFactory.cpp:4-67 picks the class from the same keys).
    void initForwardSolver(const wave_config& cfg)
    {
        const int dim = dim_ == "3d" ? 3 : 2;
        if (cfg.dimension != dim || cfg.equation != equation_of(type_))
            throw Error(WAVE_ERR_ARG, "configuration (dimension " + std::to_string(cfg.dimension) + ", equation " +
                                          std::to_string(cfg.equation) + ") does not match the solver created as " + dim_ +
                                          " " + type_);
        if (h_) wave_solver_destroy(h_);
        h_ = nullptr;
        check(nullptr, wave_solver_create(&cfg, &h_));
        check(h_, wave_get_nt(h_, &nt_));
        cfg_ = cfg;
    }

    void prepareForModelling(const Model& m)
    {
        int64_t npts = 0;
        check(nullptr, wave_grid_num_points(&cfg_, &npts));
        const size_t n = static_cast<size_t>(npts);
        auto p = [](const std::vector<float>& v) { return v.empty() ? nullptr : v.data(); };
        if (cfg_.equation >= WAVE_EQ_TMEM)
            check(h_, wave_set_model_em(h_, p(m.eps_r), p(m.sigma), p(m.mu_r), p(m.tau_eps), p(m.tau_sigma), n, WAVE_MEM_HOST));
        else
            check(h_, wave_set_model(h_, p(m.rho), p(m.vp), p(m.vs), p(m.taup), p(m.taus), n, WAVE_MEM_HOST));
    }

    void setSources(const Acquisition& a)
    {
        check(h_, wave_set_sources(h_, static_cast<int>(a.index.size()), a.index.data(), a.type.data(), a.signals.data(),
                                   WAVE_MEM_HOST));
    }
    void setReceivers(const Acquisition& a)
    {
        nrec_ = static_cast<int>(a.index.size());
        check(h_, wave_set_receivers(h_, nrec_, a.index.data(), a.type.data()));
    }

    // one time step, as ForwardSolver::run(..., t)
    void run(int t) { check(h_, wave_solver_step(h_, t, t + 1)); }
    // the whole loop t0..t1-1 as one captured CUDA graph
    void run(int t0, int t1) { check(h_, wave_solver_step(h_, t0, t1)); }

    void resetCPML() { check(h_, wave_solver_reset(h_)); }

    std::vector<float> seismograms()
    {
        std::vector<float> out(static_cast<size_t>(nrec_) * nt_);
        check(h_, wave_get_seismograms(h_, out.data(), out.size(), WAVE_MEM_HOST));
        return out;
    }

    bool isFinite()
    {
        int rc = wave_check_finite(h_);
        if (rc == WAVE_ERR_NONFINITE) return false;
        check(h_, rc);
        return true;
    }

    // ForwardSolver::estimateMemory (ForwardSolver.hpp:46): the handle's device memory in MB, measured
    double estimateMemory()
    {
        int64_t b = 0;
        check(h_, wave_device_bytes(h_, &b));
        return static_cast<double>(b) / (1024.0 * 1024.0);
    }

    int NT() const { return nt_; }
    wave_handle* handle() { return h_; }

    // factory key -> WAVE_EQ_* (the order of wave.h's equation enumeration)
    static int equation_of(const std::string& type)
    {
        static const char* keys[] = {"acoustic", "elastic", "viscoelastic", "sh", "viscosh",
                                     "tmem", "emem", "viscotmem", "viscoemem"};
        for (int k = 0; k < 9; ++k)
            if (type == keys[k]) return k;
        return -1;
    }

  private:
    std::string dim_, type_;
    wave_handle* h_ = nullptr;
    wave_config cfg_{};
    int nt_ = 0, nrec_ = 0;
};

struct Factory {
    static std::unique_ptr<ForwardSolver> Create(std::string dimension, std::string type)
    {
        auto lower = [](std::string s) {
            std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return static_cast<char>(std::tolower(c)); });
            return s;
        };
        dimension = lower(dimension);
        type = lower(type);
        if (dimension != "2d" && dimension != "3d") throw Error(WAVE_ERR_ARG, "Unkown dimension");
        static const char* types[] = {"acoustic", "elastic", "viscoelastic", "sh", "viscosh",
                                      "tmem", "emem", "viscotmem", "viscoemem"};
        if (std::find(std::begin(types), std::end(types), type) == std::end(types)) throw Error(WAVE_ERR_ARG, "Unkown type");
        return std::unique_ptr<ForwardSolver>(new ForwardSolver(dimension, type));
    }
};

} // namespace gpu
} // namespace wave
