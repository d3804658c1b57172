// refcpu_capi.cpp — TEST INFRASTRUCTURE ONLY (the oracle).
// C entry points over refcpu::Sim<float> (stand-in for the reference's FP32
// CPU run) and refcpu::Sim<double> (FP64 oracle), loaded with ctypes by the
// tests and by bench.py's CPU-baseline leg.
#include <cstring>
#include <exception>
#include <string>
#include <type_traits>

#include "refcpu.hpp"
#include "adjoint_impl.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

struct Handle {
    int is_double;
    void* sim;
};

template <class T>
refcpu::Model<T> make_model(const wave_config* c, const T* const* arr)
{
    // arr: rho, vp, vs, taup, taus, eps_r, sigma, mu_r, tau_eps, tau_sigma (any may be NULL)
    const refcpu::idx_t N = c->NX * c->NY * (c->dimension == 2 ? 1 : c->NZ);
    refcpu::Model<T> m;
    auto cp = [&](const T* p, std::vector<T>& v) { if (p) v.assign(p, p + N); };
    cp(arr[0], m.rho); cp(arr[1], m.vp); cp(arr[2], m.vs); cp(arr[3], m.taup); cp(arr[4], m.taus);
    cp(arr[5], m.eps_r); cp(arr[6], m.sigma); cp(arr[7], m.mu_r); cp(arr[8], m.tau_eps); cp(arr[9], m.tau_sigma);
    return m;
}

template <class T>
void* create(const wave_config* c, const T* const* arr, int nsrc, const int64_t* sidx, const int* stype,
             const T* signals, int nrec, const int64_t* ridx, const int* rtype)
{
    auto* s = new refcpu::Sim<T>();
    s->src.idx.assign(sidx, sidx + nsrc);
    s->src.type.assign(stype, stype + nsrc);
    s->rec.idx.assign(ridx, ridx + nrec);
    s->rec.type.assign(rtype, rtype + nrec);
    s->setup(*c, make_model<T>(c, arr));
    s->signals.assign(signals, signals + static_cast<size_t>(nsrc) * s->NT);
    return s;
}

} // namespace

extern "C" {

const char* refcpu_last_error() { return g_err.c_str(); }

int refcpu_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

void* refcpu_create_f32(const wave_config* c, const float* const* model, int nsrc, const int64_t* sidx,
                        const int* stype, const float* signals, int nrec, const int64_t* ridx, const int* rtype)
{
    try {
        auto* h = new Handle{0, create<float>(c, model, nsrc, sidx, stype, signals, nrec, ridx, rtype)};
        return h;
    } catch (std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void* refcpu_create_f64(const wave_config* c, const double* const* model, int nsrc, const int64_t* sidx,
                        const int* stype, const double* signals, int nrec, const int64_t* ridx, const int* rtype)
{
    try {
        auto* h = new Handle{1, create<double>(c, model, nsrc, sidx, stype, signals, nrec, ridx, rtype)};
        return h;
    } catch (std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

int refcpu_nt(void* hv)
{
    auto* h = static_cast<Handle*>(hv);
    return h->is_double ? static_cast<refcpu::Sim<double>*>(h->sim)->NT : static_cast<refcpu::Sim<float>*>(h->sim)->NT;
}

// Runs steps t in [t0, t1); copy_state mirrors the per-step state copy of
// Simulation.cpp:450 (on for the timed CPU baseline). Returns wall seconds via *sec.
int refcpu_step(void* hv, int t0, int t1, int copy_state, double* sec)
{
    auto* h = static_cast<Handle*>(hv);
    try {
        auto t_start = std::chrono::steady_clock::now();
        if (h->is_double) {
            auto* s = static_cast<refcpu::Sim<double>*>(h->sim);
            s->copyStateEachStep = copy_state != 0;
            for (int t = t0; t < t1; ++t) s->step(t);
        } else {
            auto* s = static_cast<refcpu::Sim<float>*>(h->sim);
            s->copyStateEachStep = copy_state != 0;
            for (int t = t0; t < t1; ++t) s->step(t);
        }
        auto t_end = std::chrono::steady_clock::now();
        if (sec) *sec = std::chrono::duration<double>(t_end - t_start).count();
        return 0;
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// Copies the seismograms (nrec x NT, row-major) as double.
int refcpu_seismograms(void* hv, double* out)
{
    auto* h = static_cast<Handle*>(hv);
    if (h->is_double) {
        auto* s = static_cast<refcpu::Sim<double>*>(h->sim);
        std::copy(s->seis.begin(), s->seis.end(), out);
    } else {
        auto* s = static_cast<refcpu::Sim<float>*>(h->sim);
        std::copy(s->seis.begin(), s->seis.end(), out);
    }
    return 0;
}

// snapType 3 curl and div energies as double (elastic equations)
int refcpu_curl_div(void* hv, double* curl, double* div)
{
    auto* h = static_cast<Handle*>(hv);
    auto run = [&](auto* s) -> int {
        using T = typename std::decay_t<decltype(s->M)>::value_type;
        std::vector<T> c, d;
        s->curlDiv(c, d);
        std::copy(c.begin(), c.end(), curl);
        std::copy(d.begin(), d.end(), div);
        return 0;
    };
    try {
        if (h->is_double) return run(static_cast<refcpu::Sim<double>*>(h->sim));
        return run(static_cast<refcpu::Sim<float>*>(h->sim));
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// Copies a named wavefield ("vx", "sxx", "p", "ez", ... or "rxx0" for memory
// variable 0) as double. Returns 1 if the field does not exist.
int refcpu_field(void* hv, const char* name, double* out)
{
    auto* h = static_cast<Handle*>(hv);
    auto grab = [&](auto* s) -> int {
        std::string n(name);
        if (s->F.count(n)) {
            std::copy(s->F[n].begin(), s->F[n].end(), out);
            return 0;
        }
        if (n.size() > 1 && isdigit(static_cast<unsigned char>(n.back()))) {
            std::string base = n.substr(0, n.size() - 1);
            int l = n.back() - '0';
            if (s->R.count(base) && l < static_cast<int>(s->R[base].size())) {
                std::copy(s->R[base][l].begin(), s->R[base][l].end(), out);
                return 0;
            }
        }
        return 1;
    };
    if (h->is_double) return grab(static_cast<refcpu::Sim<double>*>(h->sim));
    return grab(static_cast<refcpu::Sim<float>*>(h->sim));
}

// Gradient of J = 1/2 sum (d - dobs)^2 with respect to vp, vs, rho for a 2-D
// or 3-D elastic or a 2-D visco-elastic simulation (adjoint_impl.hpp; the
// relaxation times held fixed), in the handle's value type; dobs is
// nrec x NT. The model arrays are the ones the handle was created with. The
// handle's state is left at the end of the forward run. Returns the misfit
// through *misfit; 0 on success.
int refcpu_adjoint_elastic2d(void* hv, const double* vp, const double* vs, const double* rho, const double* dobs, int K,
                             double* misfit, double* gvp, double* gvs, double* grho)
{
    auto* h = static_cast<Handle*>(hv);
    auto run = [&](auto* s) -> int {
        using T = typename std::decay_t<decltype(s->M)>::value_type;
        const size_t N = s->g.N(), nd = s->rec.idx.size() * static_cast<size_t>(s->NT);
        std::vector<T> P(vp, vp + N), S(vs, vs + N), R(rho, rho + N), D(dobs, dobs + nd), a(N), b(N), c(N);
        if (s->is3d) {
            refcpu::ElasticAdjoint3D<T> adj(*s);
            *misfit = adj.run(P, S, R, D.data(), K, a.data(), b.data(), c.data());
        } else {
            refcpu::ElasticAdjoint2D<T> adj(*s);
            *misfit = adj.run(P, S, R, D.data(), K, a.data(), b.data(), c.data());
        }
        std::copy(a.begin(), a.end(), gvp);
        std::copy(b.begin(), b.end(), gvs);
        std::copy(c.begin(), c.end(), grho);
        return 0;
    };
    try {
        if (K < 1) throw std::invalid_argument("checkpoint interval must be >= 1");
        if (h->is_double) return run(static_cast<refcpu::Sim<double>*>(h->sim));
        return run(static_cast<refcpu::Sim<float>*>(h->sim));
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// The same for an acoustic simulation (2-D or 3-D): gradients with respect to
// vp and rho (adjoint_impl.hpp, AcousticAdjoint).
int refcpu_adjoint_acoustic(void* hv, const double* vp, const double* rho, const double* dobs, int K, double* misfit, double* gvp,
                            double* grho)
{
    auto* h = static_cast<Handle*>(hv);
    auto run = [&](auto* s) -> int {
        using T = typename std::decay_t<decltype(s->M)>::value_type;
        const size_t N = s->g.N(), nd = s->rec.idx.size() * static_cast<size_t>(s->NT);
        std::vector<T> P(vp, vp + N), R(rho, rho + N), D(dobs, dobs + nd), a(N), b(N);
        refcpu::AcousticAdjoint<T> adj(*s);
        *misfit = adj.run(P, R, D.data(), K, a.data(), b.data());
        std::copy(a.begin(), a.end(), gvp);
        std::copy(b.begin(), b.end(), grho);
        return 0;
    };
    try {
        if (K < 1) throw std::invalid_argument("checkpoint interval must be >= 1");
        if (h->is_double) return run(static_cast<refcpu::Sim<double>*>(h->sim));
        return run(static_cast<refcpu::Sim<float>*>(h->sim));
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// The same for a 2-D SH simulation (vz receivers): gradients with respect to
// vs and rho (adjoint_impl.hpp, SHAdjoint2D).
int refcpu_adjoint_sh(void* hv, const double* vs, const double* rho, const double* dobs, int K, double* misfit, double* gvs,
                      double* grho)
{
    auto* h = static_cast<Handle*>(hv);
    auto run = [&](auto* s) -> int {
        using T = typename std::decay_t<decltype(s->M)>::value_type;
        const size_t N = s->g.N(), nd = s->rec.idx.size() * static_cast<size_t>(s->NT);
        std::vector<T> S(vs, vs + N), R(rho, rho + N), D(dobs, dobs + nd), a(N), b(N);
        refcpu::SHAdjoint2D<T> adj(*s);
        *misfit = adj.run(S, R, D.data(), K, a.data(), b.data());
        std::copy(a.begin(), a.end(), gvs);
        std::copy(b.begin(), b.end(), grho);
        return 0;
    };
    try {
        if (K < 1) throw std::invalid_argument("checkpoint interval must be >= 1");
        if (h->is_double) return run(static_cast<refcpu::Sim<double>*>(h->sim));
        return run(static_cast<refcpu::Sim<float>*>(h->sim));
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// The same for a lossless 2-D TMz simulation (Ez receivers) or a lossless 2-D
// TEz one (Ex, Ey, Hz receivers): gradients with respect to eps_r, sigma and
// mu_r (adjoint_impl.hpp, TMAdjoint2D / TEAdjoint2D).
int refcpu_adjoint_tmz(void* hv, const double* epsr, const double* sigma, const double* mur, const double* dobs, int K,
                       double* misfit, double* geps, double* gsig, double* gmu)
{
    auto* h = static_cast<Handle*>(hv);
    auto run = [&](auto* s) -> int {
        using T = typename std::decay_t<decltype(s->M)>::value_type;
        const size_t N = s->g.N(), nd = s->rec.idx.size() * static_cast<size_t>(s->NT);
        std::vector<T> E(epsr, epsr + N), S(sigma, sigma + N), U(mur, mur + N), D(dobs, dobs + nd), a(N), b(N), c(N);
        if ((s->eq == WAVE_EQ_EMEM || s->eq == WAVE_EQ_VISCOEMEM) && s->is3d) {
            refcpu::EM3Adjoint<T> adj(*s);
            *misfit = adj.run(E, S, U, D.data(), K, a.data(), b.data(), c.data());
        } else if (s->eq == WAVE_EQ_EMEM || s->eq == WAVE_EQ_VISCOEMEM) {
            refcpu::TEAdjoint2D<T> adj(*s);
            *misfit = adj.run(E, S, U, D.data(), K, a.data(), b.data(), c.data());
        } else {
            refcpu::TMAdjoint2D<T> adj(*s);
            *misfit = adj.run(E, S, U, D.data(), K, a.data(), b.data(), c.data());
        }
        std::copy(a.begin(), a.end(), geps);
        std::copy(b.begin(), b.end(), gsig);
        std::copy(c.begin(), c.end(), gmu);
        return 0;
    };
    try {
        if (K < 1) throw std::invalid_argument("checkpoint interval must be >= 1");
        if (h->is_double) return run(static_cast<refcpu::Sim<double>*>(h->sim));
        return run(static_cast<refcpu::Sim<float>*>(h->sim));
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

void refcpu_destroy(void* hv)
{
    auto* h = static_cast<Handle*>(hv);
    if (!h) return;
    if (h->is_double) delete static_cast<refcpu::Sim<double>*>(h->sim);
    else delete static_cast<refcpu::Sim<float>*>(h->sim);
    delete h;
}

} // extern "C"
