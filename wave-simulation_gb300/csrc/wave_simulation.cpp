// wave_simulation.cpp — command-line driver that runs a reference parameter
// file end to end on the GPU solver, the way Simulation.cpp:36-570 does for the
// reference: read the configuration, build the model (homogeneous from the
// velocityP/velocityS/rho keys, or MatrixMarket files <ModelFilename>.<p>.mtx
// for ModelRead=1, FileFormat=1), loop over the shots of <SourceFilename>.txt,
// generate the wavelets, run the time loop, normalise the traces
// (normalizeTraces 0-4), resample them to seismoDT and write
// <SeismogramFilename>.shot_<n>.<c>.mtx (SeismogramFormat 1) or .su (4), as
// Simulation.cpp:521-531 does.
//
//   wave_simulation <parameter file>
#include <cstdio>
#include <ctime>
#include <fstream>
#include <iostream>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "forward_solver.hpp"

namespace {

std::map<std::string, std::string> read_keys(const std::string& path)
{
    std::map<std::string, std::string> m;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        size_t end = line.size(), c = line.find('#');
        if (c != std::string::npos) {
            if (c == 0) continue;
            end = c;
        }
        size_t e = line.find('=');
        if (e == std::string::npos) continue;
        std::string k = line.substr(0, e);
        for (auto& ch : k) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
        m[k] = line.substr(e + 1, end > e ? end - e - 1 : 0);
    }
    return m;
}

template <class T>
T key(const std::map<std::string, std::string>& m, const char* k, T def)
{
    std::string kk(k);
    for (auto& ch : kk) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
    auto it = m.find(kk);
    if (it == m.end()) return def;
    std::istringstream in(it->second);
    T v = def;
    in >> v;
    return in.fail() ? def : v;
}

std::vector<float> read_mtx_vector(const std::string& path, size_t n)
{
    int64_t rows = 0, cols = 0;
    wave::gpu::check(nullptr, wave_read_mtx(path.c_str(), nullptr, 0, &rows, &cols));
    if (static_cast<size_t>(rows * cols) != n) throw wave::gpu::Error(WAVE_ERR_IO, path + ": wrong number of values");
    std::vector<float> v(n);
    wave::gpu::check(nullptr, wave_read_mtx(path.c_str(), v.data(), static_cast<int64_t>(n), &rows, &cols));
    return v;
}

// wavefields written for snapType 1 / 2 (/ 4 for 2-D acoustic), as the
// Wavefields*::write functions name them (Wavefields2Delastic.cpp:62-72, ...)
std::vector<std::string> snapshot_fields(int eq, bool is3d, int snapType)
{
    const bool em = eq >= WAVE_EQ_TMEM;
    if (em) {
        // snapType 4 / 5 of TMz add the decomposition parts (Wavefields2Dtmem.cpp:88-96)
        if (eq == WAVE_EQ_TMEM && snapType == 4) return {"EZ", "EZ.up", "EZ.down"};
        if (eq == WAVE_EQ_TMEM && snapType == 5) return {"EZ", "EZ.left", "EZ.right"};
        if (eq == WAVE_EQ_TMEM || eq == WAVE_EQ_VISCOTMEM) return snapType == 1 ? std::vector<std::string>{"HX", "HY"} : std::vector<std::string>{"EZ"};
        if (!is3d) return snapType == 1 ? std::vector<std::string>{"HZ"} : std::vector<std::string>{"EX", "EY"};
        return snapType == 1 ? std::vector<std::string>{"HX", "HY", "HZ"} : std::vector<std::string>{"EX", "EY", "EZ"};
    }
    if (eq == WAVE_EQ_SH || eq == WAVE_EQ_VISCOSH) return snapType == 1 ? std::vector<std::string>{"VZ"} : std::vector<std::string>{"Sxz", "Syz"};
    std::vector<std::string> v = is3d ? std::vector<std::string>{"VX", "VY", "VZ"} : std::vector<std::string>{"VX", "VY"};
    if (eq == WAVE_EQ_ACOUSTIC) {
        if (snapType == 1) return v;
        if (snapType == 2) return {"P"};
        // snapType 4 / 5 add the decomposition parts (Wavefields2Dacoustic.cpp:86-107)
        if (snapType == 4 && !is3d) return {"P", "VX", "VY", "P.up", "P.down", "VX.up", "VX.down", "VY.up", "VY.down"};
        if (snapType == 5 && !is3d) return {"P", "VX", "VY", "P.left", "P.right", "VX.left", "VX.right", "VY.left", "VY.right"};
        return {};
    }
    if (snapType == 1) return v;
    if (snapType == 2) return is3d ? std::vector<std::string>{"Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz"} : std::vector<std::string>{"Sxx", "Syy", "Sxy"};
    return {};
}

} // namespace

int main(int argc, char** argv)
{
    if (argc != 2) {
        std::cerr << "usage: wave_simulation <parameter file>\n";
        return 2;
    }
    try {
        wave_config cfg;
        wave::gpu::check(nullptr, wave_config_from_file(argv[1], &cfg));
        auto keys = read_keys(argv[1]);
        const std::string dir = [&] {
            std::string p(argv[1]);
            size_t s = p.find_last_of('/');
            return s == std::string::npos ? std::string(".") : p.substr(0, s);
        }();
        // grid points: NX*NY*NZ, or the variable grid's (Coordinates.cpp:119-245)
        int64_t npts = 0;
        wave::gpu::check(nullptr, wave_grid_num_points(&cfg, &npts));
        const size_t n = static_cast<size_t>(npts);
        const bool layered = cfg.useVariableGrid || cfg.useVariableFDoperators;
        const size_t nRegular = static_cast<size_t>(cfg.NX * cfg.NY * (cfg.dimension == 3 ? cfg.NZ : 1));
        // a regular-grid model onto the grid's points (Acoustic.cpp:180-200:
        // each point takes the value at its fine-grid coordinate)
        std::vector<int64_t> gx, gy, gz;
        if (layered) {
            gx.resize(n); gy.resize(n); gz.resize(n);
            wave::gpu::check(nullptr, wave_grid_coordinates(&cfg, gx.data(), gy.data(), gz.data(), npts, nullptr));
        }
        auto onto_grid = [&](std::vector<float> v) {
            if (!layered) return v;
            std::vector<float> out(n);
            const int64_t NZr = cfg.dimension == 3 ? cfg.NZ : 1;
            for (size_t i = 0; i < n; ++i) out[i] = v[static_cast<size_t>(gx[i] + gz[i] * cfg.NX + gy[i] * cfg.NX * NZr)];
            return out;
        };
        auto grid_index = [&](long long x, long long y, long long z) {
            int64_t idx = 0;
            wave::gpu::check(nullptr, wave_grid_index(&cfg, x, y, z, &idx));
            return static_cast<long long>(idx);
        };
        wave::gpu::Model model;
        const bool em = cfg.equation >= WAVE_EQ_TMEM;
        const std::string mf = key<std::string>(keys, "ModelFilename", "model/model");
        if (key<int>(keys, "ModelRead", 0) == 1) {
            if (key<int>(keys, "FileFormat", 1) != 1)
                throw wave::gpu::Error(WAVE_ERR_UNSUPPORTED, "model files: only FileFormat=1 (MatrixMarket) is readable here; lmf/frv are LAMA formats");
            auto rd = [&](const char* p) { return onto_grid(read_mtx_vector(dir + "/../" + mf + "." + p + ".mtx", nRegular)); };
            if (em) {
                model.eps_r = rd("epsilonr"); model.sigma = rd("sigma"); model.mu_r = rd("mur");
                // ViscoTMEM.cpp:320-329 / ViscoEMEM: the relaxation times' files
                if (cfg.equation == WAVE_EQ_VISCOTMEM || cfg.equation == WAVE_EQ_VISCOEMEM) {
                    model.tau_sigma = rd("tauSigmar");
                    model.tau_eps = rd("tauEpsilon");
                }
            }
            else {
                model.rho = rd("density");
                if (cfg.equation != WAVE_EQ_SH && cfg.equation != WAVE_EQ_VISCOSH) model.vp = rd("vp");
                if (cfg.equation != WAVE_EQ_ACOUSTIC) model.vs = rd("vs");
                if (cfg.equation == WAVE_EQ_VISCOELASTIC) model.taup = rd("tauP");
                if (cfg.equation == WAVE_EQ_VISCOELASTIC || cfg.equation == WAVE_EQ_VISCOSH) model.taus = rd("tauS");
            }
        } else if (em) {
            model.eps_r.assign(n, key<float>(keys, "epsilonr", 1.0f));
            model.sigma.assign(n, key<float>(keys, "sigma", 0.0f));
            model.mu_r.assign(n, key<float>(keys, "mur", 1.0f));
            // ViscoTMEM.cpp:206 / ViscoEMEM.cpp:192: homogeneous relaxation times from the keys
            if (cfg.equation == WAVE_EQ_VISCOTMEM || cfg.equation == WAVE_EQ_VISCOEMEM) {
                model.tau_sigma.assign(n, key<float>(keys, "tauSigmar", 0.0f));
                model.tau_eps.assign(n, key<float>(keys, "tauEpsilon", 0.0f));
            }
        } else {
            model.rho.assign(n, key<float>(keys, "rho", 1000.0f));
            model.vp.assign(n, key<float>(keys, "velocityP", 0.0f));
            model.vs.assign(n, key<float>(keys, "velocityS", 0.0f));
            model.taup.assign(n, key<float>(keys, "tauP", 0.0f));
            model.taus.assign(n, key<float>(keys, "tauS", 0.0f));
        }
        // acquisition (AcquisitionSettings.hpp:55-109; receivers: x y z type)
        struct Src { int no, x, y, z, type, wtype, shape; double fc, amp, ts; };
        std::vector<Src> srcs;
        {
            std::ifstream f(dir + "/../" + key<std::string>(keys, "SourceFilename", "") + ".txt");
            std::string line;
            while (std::getline(f, line)) {
                if (line.empty() || line[0] == '#') continue;
                std::istringstream in(line);
                Src s;
                if (in >> s.no >> s.x >> s.y >> s.z >> s.type >> s.wtype >> s.shape >> s.fc >> s.amp >> s.ts) srcs.push_back(s);
            }
        }
        wave::gpu::Acquisition rec;
        {
            std::ifstream f(dir + "/../" + key<std::string>(keys, "ReceiverFilename", "") + ".txt");
            std::string line;
            while (std::getline(f, line)) {
                if (line.empty() || line[0] == '#') continue;
                std::istringstream in(line);
                long long x, y, z;
                int t;
                if (in >> x >> y >> z >> t) {
                    rec.index.push_back(grid_index(x, y, z));
                    rec.type.push_back(t);
                }
            }
        }
        if (srcs.empty() || rec.index.empty()) throw wave::gpu::Error(WAVE_ERR_IO, "no sources or receivers read");
        const std::string eqname[] = {"acoustic", "elastic", "viscoelastic", "sh", "viscosh", "tmem", "emem", "viscotmem", "viscoemem"};
        auto solver = wave::gpu::Factory::Create(cfg.dimension == 3 ? "3D" : "2D", eqname[cfg.equation]);
        solver->initForwardSolver(cfg);
        // wavefield decomposition (Simulation.cpp:316, 457-461)
        const int decomposition = key<int>(keys, "decomposeWavefieldType", 0);
        if (decomposition != 0) wave::gpu::check(solver->handle(), wave_set_decomposition(solver->handle(), decomposition));
        solver->prepareForModelling(model);
        solver->setReceivers(rec);
        const int nt = solver->NT();
        // source encoding into NumShotDomains super-shots (Simulation.cpp:255-266,
        // Sources.cpp:569-660); seeded with time(0) as in the reference unless
        // the key seedtime is given
        const int encodeMode = key<int>(keys, "useSourceEncode", 0);
        if (encodeMode != 0) {
            const int domains = key<int>(keys, "NumShotDomains", 1);
            const unsigned seed = static_cast<unsigned>(key<long long>(keys, "seedtime", static_cast<long long>(std::time(nullptr))));
            std::vector<int> no(srcs.size()), noOut(srcs.size());
            std::vector<float> amp(srcs.size()), ampOut(srcs.size());
            for (size_t i = 0; i < srcs.size(); ++i) { no[i] = srcs[i].no; amp[i] = static_cast<float>(srcs[i].amp); }
            if (key<int>(keys, "gradientDomain", 0) != 0) {
                // frequency domain: each shot of a super-shot gets its own frequency
                // of the band [fc1, fc2] as a synthetic sin wavelet (shape 9)
                std::vector<float> fc(srcs.size());
                wave::gpu::check(nullptr, wave_encode_sources_frequency(encodeMode, domains, seed, static_cast<int>(srcs.size()), amp.data(),
                                                                        key<double>(keys, "fc1", 0.0), key<double>(keys, "fc2", 0.0), cfg.T,
                                                                        cfg.DT, cfg.CenterFrequencyCPML, noOut.data(), ampOut.data(),
                                                                        fc.data()));
                for (size_t i = 0; i < srcs.size(); ++i) { srcs[i].wtype = 1; srcs[i].shape = 9; srcs[i].fc = fc[i]; }
            } else {
                wave::gpu::check(nullptr, wave_encode_sources(encodeMode, domains, seed, static_cast<int>(srcs.size()), no.data(), amp.data(),
                                                              noOut.data(), ampOut.data()));
            }
            for (size_t i = 0; i < srcs.size(); ++i) { srcs[i].no = noOut[i]; srcs[i].amp = ampOut[i]; }
        }
        std::set<int> shots;
        for (auto& s : srcs) shots.insert(s.no);
        const char* names[2][4] = {{"p", "vx", "vy", "vz"}, {"ez", "ex", "ey", "hz"}};
        const int normalize = key<int>(keys, "normalizeTraces", 0);
        const double seismoDT = key<double>(keys, "seismoDT", cfg.DT);
        const int format = key<int>(keys, "SeismogramFormat", 1);
        if (normalize < 0 || normalize > 4) throw wave::gpu::Error(WAVE_ERR_ARG, "normalizeTraces must be 0-4");
        const int snapType = key<int>(keys, "snapType", 0);
        if (snapType < 0 || snapType > 5) throw wave::gpu::Error(WAVE_ERR_ARG, "Invalid snapType.");
        const int instantaneous = key<int>(keys, "outputInstantaneous", 0);
        if (format != 1 && format != 4) throw wave::gpu::Error(WAVE_ERR_UNSUPPORTED, "SeismogramFormat: 1 (mtx) and 4 (su) are written here");
        for (int shot : shots) {
            wave::gpu::Acquisition src;
            for (auto& s : srcs) {
                if (s.no != shot) continue;
                src.index.push_back(grid_index(s.x, s.y, s.z));
                src.type.push_back(s.type);
                std::vector<float> w(nt);
                wave::gpu::check(nullptr, wave_wavelet(s.shape, nt, cfg.DT, s.fc, s.amp, s.ts, w.data()));
                src.signals.insert(src.signals.end(), w.begin(), w.end());
            }
            solver->resetCPML();
            solver->setSources(src);
            // time loop with snapshots after the steps tFirst, tFirst + tinc, ... <= tLast (Simulation.cpp:468-475)
            int t = 0;
            if (snapType > 0) {
                const int t1 = static_cast<int>(key<double>(keys, "tFirstSnapshot", 0.0) / cfg.DT + 0.5);
                const int t2 = static_cast<int>(key<double>(keys, "tlastSnapshot", 0.0) / cfg.DT + 0.5);
                int inc = static_cast<int>(key<double>(keys, "tincSnapshot", cfg.DT) / cfg.DT + 0.5);
                if (inc < 1) inc = 1;
                const std::string wbase = dir + "/../" + key<std::string>(keys, "WavefieldFileName", "wavefields/wavefield") + ".shot_" + std::to_string(shot);
                const size_t npts = n;
                for (int ts = t1; ts <= t2 && ts < nt; ts += inc) {
                    solver->run(t, ts + 1);
                    t = ts + 1;
                    const std::string step = std::to_string(ts);
                    if (snapType == 3) {
                        std::vector<float> curl(npts), div(npts);
                        wave::gpu::check(solver->handle(), wave_get_curl_div(solver->handle(), curl.data(), div.data(), WAVE_MEM_HOST));
                        const bool big = cfg.dimension == 3;
                        wave::gpu::check(nullptr, wave_write_mtx((wbase + (big ? ".CURL." : ".curl.") + step + ".mtx").c_str(), curl.data(), static_cast<int64_t>(npts), 1));
                        wave::gpu::check(nullptr, wave_write_mtx((wbase + (big ? ".DIV." : ".div.") + step + ".mtx").c_str(), div.data(), static_cast<int64_t>(npts), 1));
                    } else {
                        std::vector<float> f(npts);
                        for (const auto& name : snapshot_fields(cfg.equation, cfg.dimension == 3, snapType)) {
                            // decomposition parts of another (or no) decomposition type are zero, as in the reference
                            const bool part = name.find('.') != std::string::npos;
                            const bool have = !part || (snapType == 4 && decomposition == 1) || (snapType == 5 && decomposition == 2);
                            if (have) wave::gpu::check(solver->handle(), wave_get_field(solver->handle(), name.c_str(), f.data(), WAVE_MEM_HOST));
                            else std::fill(f.begin(), f.end(), 0.0f);
                            wave::gpu::check(nullptr, wave_write_mtx((wbase + "." + name + "." + step + ".mtx").c_str(), f.data(), static_cast<int64_t>(npts), 1));
                        }
                    }
                }
            }
            solver->run(t, nt);
            auto seis = solver->seismograms();
            if (!solver->isFinite()) throw wave::gpu::Error(WAVE_ERR_NONFINITE, "Infinite or NaN value in seismogram or/and velocity wavefield!");
            for (int type = 1; type <= 4; ++type) {
                std::vector<float> part;
                int ntr = 0;
                for (size_t r = 0; r < rec.type.size(); ++r)
                    if (rec.type[r] == type) {
                        part.insert(part.end(), seis.begin() + r * nt, seis.begin() + (r + 1) * nt);
                        ++ntr;
                    }
                if (!ntr) continue;
                // Seismogram::normalizeTrace, then the resampling of Seismogram::write
                int64_t ntOut = 0;
                wave::gpu::check(nullptr, wave_resample_traces(nullptr, ntr, nt, cfg.DT, seismoDT, nullptr, &ntOut, WAVE_MEM_HOST));
                const std::string base = dir + "/../" + key<std::string>(keys, "SeismogramFilename", "seismogram") + ".shot_" +
                                         std::to_string(shot) + "." + names[em ? 1 : 0][type - 1];
                if (normalize == 3) {
                    // Simulation.cpp:521-524: the inverse AGC (window from CenterFrequencyCPML) is written
                    // resampled as <seismogram>.<component>.inverseAGC.mtx, then normalizeTrace(3)
                    std::vector<float> inv(part.size()), invOut(static_cast<size_t>(ntr) * ntOut);
                    wave::gpu::check(nullptr, wave_agc_normalize_traces(part.data(), ntr, nt, cfg.DT, cfg.CenterFrequencyCPML, inv.data(),
                                                                        WAVE_MEM_HOST));
                    wave::gpu::check(nullptr, wave_resample_traces(inv.data(), ntr, nt, cfg.DT, seismoDT, invOut.data(), &ntOut, WAVE_MEM_HOST));
                    wave::gpu::check(nullptr, wave_write_mtx((base + ".inverseAGC.mtx").c_str(), invOut.data(), ntr, ntOut));
                } else {
                    wave::gpu::check(nullptr, wave_normalize_traces(part.data(), ntr, nt, normalize, WAVE_MEM_HOST));
                }
                std::vector<float> out(static_cast<size_t>(ntr) * ntOut);
                wave::gpu::check(nullptr, wave_resample_traces(part.data(), ntr, nt, cfg.DT, seismoDT, out.data(), &ntOut, WAVE_MEM_HOST));
                if (format == 4) {
                    std::vector<int64_t> ridx;
                    for (size_t r = 0; r < rec.type.size(); ++r)
                        if (rec.type[r] == type) ridx.push_back(rec.index[r]);
                    wave::gpu::check(nullptr, wave_write_su((base + ".su").c_str(), out.data(), ntr, ntOut, seismoDT > 0 ? seismoDT : cfg.DT,
                                                           ridx.data(), src.index.empty() ? 0 : src.index[0], cfg.NX, cfg.NY,
                                                           cfg.dimension == 3 ? cfg.NZ : 1, cfg.DH));
                } else {
                    wave::gpu::check(nullptr, wave_write_mtx((base + ".mtx").c_str(), out.data(), ntr, ntOut));
                }
                // Seismogram::write: envelope or instantaneous phase of the written traces (Seismogram.cpp:127-145)
                if ((instantaneous == 1 || instantaneous == 2) && ntOut >= 2) {
                    std::string suffix = ".envelope";
                    if (instantaneous == 1) wave::gpu::check(nullptr, wave_envelope(out.data(), ntr, ntOut, WAVE_MEM_HOST));
                    else {
                        wave::gpu::check(nullptr, wave_instantaneous_phase(out.data(), ntr, ntOut, 2, WAVE_MEM_HOST));
                        suffix = ".instantaneousPhase";
                    }
                    if (format == 4) {
                        std::vector<int64_t> ridx;
                        for (size_t r = 0; r < rec.type.size(); ++r)
                            if (rec.type[r] == type) ridx.push_back(rec.index[r]);
                        wave::gpu::check(nullptr, wave_write_su((base + suffix + ".su").c_str(), out.data(), ntr, ntOut, seismoDT > 0 ? seismoDT : cfg.DT,
                                                               ridx.data(), src.index.empty() ? 0 : src.index[0], cfg.NX, cfg.NY,
                                                               cfg.dimension == 3 ? cfg.NZ : 1, cfg.DH));
                    } else {
                        wave::gpu::check(nullptr, wave_write_mtx((base + suffix + ".mtx").c_str(), out.data(), ntr, ntOut));
                    }
                }
            }
            std::cout << "shot " << shot << ": " << nt << " time steps done\n";
        }
    } catch (wave::gpu::Error& e) {
        std::cerr << "wave_simulation: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
