// C ABI of the 3D Cartesian run (mag3d_*, include/mag2d_gpu.h).
#include <cstring>
#include <memory>
#include <new>
#include <string>

#include "mag2d_gpu.h"
#include "sim3d.hpp"

namespace mag {
void set_last_error(const std::string& msg);
}

struct mag3d_sim {
    std::unique_ptr<mag::Sim3D> s;
};

namespace {

template <class F>
int guarded3(F&& f)
{
    try {
        return f();
    } catch (const mag::Error& e) {
        mag::set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        mag::set_last_error("out of host memory");
        return MAG_ENOMEM;
    } catch (const std::exception& e) {
        mag::set_last_error(e.what());
        return MAG_EINVAL;
    }
}

mag::Sim3D& sim_of(mag3d_sim* h, int species = 0)
{
    if (!h || !h->s) throw mag::Error(MAG_EINVAL, "null 3D simulation handle");
    if (species < 0 || species >= (int)h->s->sp.size()) throw mag::Error(MAG_EINVAL, "species index out of range");
    return *h->s;
}

int status3(mag::Sim3D& s)
{
    const int e = s.sync();
    if (e == 0) return MAG_OK;
    mag::set_last_error(e == -5 ? "a bounded device-side wait gave up in the 3D solve" : "device error " + std::to_string(e));
    return e;
}

}  // namespace

extern "C" {

int mag3d_create(const char* config_path, const char* species_conf_path, const mag_opts* opts, mag3d_sim** out)
{
    return guarded3([&]() {
        if (!config_path || !species_conf_path || !out) throw mag::Error(MAG_EINVAL, "null argument");
        *out = nullptr;
        mag::SimOptions o;
        if (opts) {
            o.device = opts->device;
            o.seed = opts->seed;
            o.poisson_tol = opts->poisson_tol;
            o.poisson_max_iter = opts->poisson_max_iter;
            o.capacity_hint = opts->capacity_hint;
        }
        auto h = std::make_unique<mag3d_sim>();
        h->s = std::make_unique<mag::Sim3D>(config_path, species_conf_path, o);
        *out = h.release();
        return MAG_OK;
    });
}

void mag3d_destroy(mag3d_sim* sim) { delete sim; }

int mag3d_grid(mag3d_sim* sim, int* dims, double* spacing)
{
    return guarded3([&]() {
        mag::Sim3D& s = sim_of(sim);
        if (dims) {
            dims[0] = s.nx;
            dims[1] = s.ny;
            dims[2] = s.nz;
        }
        if (spacing) {
            spacing[0] = s.dx;
            spacing[1] = s.dy;
            spacing[2] = s.dz;
        }
        return (int)s.sp.size();
    });
}

int mag3d_set_particles(mag3d_sim* sim, int species, int64_t n, const double* x, const double* y, const double* z,
                        const double* vx, const double* vy, const double* vz)
{
    return guarded3([&]() {
        mag::Sim3D& s = sim_of(sim, species);
        if (n < 0 || (n > 0 && (!x || !y || !z || !vx || !vy || !vz))) throw mag::Error(MAG_EINVAL, "bad particle arrays");
        s.set_particles(species, n, x, y, z, vx, vy, vz);
        return status3(s);
    });
}

int mag3d_get_particles(mag3d_sim* sim, int species, int64_t cap, double* x, double* y, double* z, double* vx,
                        double* vy, double* vz, uint32_t* id, int64_t* n_out)
{
    return guarded3([&]() {
        mag::Sim3D& s = sim_of(sim, species);
        int64_t n = 0;
        s.get_particles(species, cap, x, y, z, vx, vy, vz, id, &n);
        if (n_out) *n_out = n;
        return status3(s);
    });
}

int mag3d_advance_init(mag3d_sim* sim)
{
    return guarded3([&]() {
        mag::Sim3D& s = sim_of(sim);
        s.advance_init();
        return status3(s);
    });
}

int mag3d_advance(mag3d_sim* sim, uint64_t nsteps)
{
    return guarded3([&]() {
        sim_of(sim).advance(nsteps);
        return MAG_OK;
    });
}

int mag3d_solve(mag3d_sim* sim, const double* rho, mag_solve_info* info)
{
    return guarded3([&]() {
        mag::Sim3D& s = sim_of(sim);
        const mag::SolveStatus st = s.solve(rho);
        if (info) {
            info->iterations = st.iterations;
            info->residual = st.residual;
            info->status = st.converged ? MAG_OK : MAG_ENOTCONV;
            info->levels = 1;
        }
        return st.converged ? MAG_OK : MAG_ENOTCONV;
    });
}

int mag3d_get_field(mag3d_sim* sim, int which, double* out)
{
    return guarded3([&]() {
        mag::Sim3D& s = sim_of(sim);
        if (!out) throw mag::Error(MAG_EINVAL, "null output");
        const int w = which == MAG_U ? 0 : which == MAG_RHO ? 2 : which == MAG_MASK ? 3 : -1;
        if (w < 0) throw mag::Error(MAG_EINVAL, "3D field: MAG_U, MAG_RHO or MAG_MASK");
        s.get_field(w, out);
        return status3(s);
    });
}

int mag3d_get_rho_fixed(mag3d_sim* sim, int species, int64_t* out)
{
    return guarded3([&]() {
        mag::Sim3D& s = sim_of(sim, species);
        if (!out) throw mag::Error(MAG_EINVAL, "null output");
        s.get_rho_fixed(species, out);
        return MAG_OK;
    });
}

int mag3d_diag(mag3d_sim* sim, int species, mag_diag_out* out)
{
    return guarded3([&]() {
        mag::Sim3D& s = sim_of(sim, species);
        if (!out) throw mag::Error(MAG_EINVAL, "null output");
        std::memset(out, 0, sizeof *out);
        double e2 = 0;
        unsigned long long n = 0;
        if (s.sp[species].n_slots > 0) s.energy(species, e2, n);
        const mag::SpeciesState& S = s.sp[species];
        out->n_live = (int64_t)n;
        out->mean_energy_eV = n ? e2 / (double)n * S.prm.mass * 0.5 / mag::kQe : 0.0;
        out->total_charge = (double)n * S.prm.charge * s.p.macroparticle_factor;
        const mag::Counters c = s.counters(species);
        out->collisions = (int64_t)c.ncoll;
        out->null_collisions = (int64_t)c.nnull;
        out->removed = (int64_t)c.removed;
        out->particle_steps = (int64_t)c.live_sum;
        out->niter = (int64_t)S.niter;
        return status3(s);
    });
}

int64_t mag3d_kernel_launches(mag3d_sim* sim) { return sim && sim->s ? sim->s->launches : 0; }

}  // extern "C"
