// C ABI of libmag2d_gpu.so (include/mag2d_gpu.h).  Every entry point catches
// C++ exceptions and turns them into a status code plus mag_last_error().
#include "mag2d_gpu.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "adjoint.hpp"
#include "batch.hpp"
#include "particle_io.hpp"
#include "sim.hpp"

// A handle owns its Sim, or borrows one that a batch owns.
struct SimRelease {
    bool owned = true;
    void operator()(mag::Sim* p) const
    {
        if (owned) delete p;
    }
};

struct mag_sim {
    std::unique_ptr<mag::Sim, SimRelease> s;
};

struct mag_batch {
    std::unique_ptr<mag::Batch> b;
    std::vector<std::unique_ptr<mag_sim>> views;
};

namespace {

thread_local std::string g_last_error;

template <class F>
int guarded(F&& f)
{
    try {
        return f();
    } catch (const mag::Error& e) {
        g_last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_last_error = "out of host memory";
        return MAG_ENOMEM;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return MAG_EINVAL;
    }
}

int check_species(mag_sim* sim, int s)
{
    if (!sim || !sim->s) throw mag::Error(MAG_EINVAL, "null simulation handle");
    if (s < 0 || s >= (int)sim->s->sp.size()) throw mag::Error(MAG_EINVAL, "species index out of range");
    return 0;
}

int status_of(int e)
{
    if (e == 0) return MAG_OK;
    switch (e) {
    case -4: g_last_error = "Poisson solve did not reach its tolerance"; break;
    case -5: g_last_error = "a bounded device-side wait gave up"; break;
    case -3: g_last_error = "particle or node index outside the grid"; break;
    default: g_last_error = "device error " + std::to_string(e); break;
    }
    return e;
}

int device_status(mag_sim* sim) { return status_of(sim->s->sync()); }

}  // namespace

namespace mag {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace mag

extern "C" {

const char* mag_last_error(void) { return g_last_error.c_str(); }

const char* mag_version(void) { return "mag2d_gb300 0.1 (sm_103a)"; }

int mag_create(const char* config_path, const char* species_conf_path, const char* initscript_path,
               const mag_opts* opts, mag_sim** out)
{
    return guarded([&]() {
        if (!config_path || !species_conf_path || !out) throw mag::Error(MAG_EINVAL, "null argument");
        mag::SimOptions o;
        if (opts) {
            o.device = opts->device;
            o.seed = opts->seed;
            o.sort_interval = opts->sort_interval;
            o.poisson_tol = opts->poisson_tol;
            o.poisson_max_iter = opts->poisson_max_iter;
            o.capacity_hint = opts->capacity_hint;
            o.push_vec = opts->push_vec;
            o.direct_solve = opts->direct_solve;
            o.max_fused_steps = opts->max_fused_steps;
            o.multigrid_fp64 = opts->multigrid_fp64;
        }
        auto h = std::make_unique<mag_sim>();
        h->s = std::unique_ptr<mag::Sim, SimRelease>(new mag::Sim(config_path, species_conf_path, o), SimRelease{true});
        if (initscript_path && *initscript_path) h->s->run_initscript(initscript_path);
        *out = h.release();
        return MAG_OK;
    });
}

void mag_destroy(mag_sim* sim)
{
    if (sim && sim->s && !sim->s.get_deleter().owned) return;  // a batch's borrowed instance
    delete sim;
}

int mag_run_initscript(mag_sim* sim, const char* path)
{
    return guarded([&]() {
        check_species(sim, 0);
        sim->s->run_initscript(path);
        return MAG_OK;
    });
}

int mag_advance_init(mag_sim* sim)
{
    return guarded([&]() {
        check_species(sim, 0);
        sim->s->advance_init();
        return MAG_OK;
    });
}

int mag_advance_init_ex(mag_sim* sim, int deposit)
{
    return guarded([&]() {
        check_species(sim, 0);
        sim->s->advance_init(deposit != 0);
        return MAG_OK;
    });
}

int mag_advance(mag_sim* sim, uint64_t nsteps)
{
    return guarded([&]() {
        check_species(sim, 0);
        sim->s->advance(nsteps);
        return MAG_OK;
    });
}

int mag_advance_timed(mag_sim* sim, uint64_t nsteps, double* ms_out)
{
    return guarded([&]() {
        check_species(sim, 0);
        sim->s->advance_timed(nsteps, ms_out);
        return device_status(sim);
    });
}

int mag_sync(mag_sim* sim)
{
    return guarded([&]() {
        check_species(sim, 0);
        return device_status(sim);
    });
}

int mag_grid(mag_sim* sim, int* nx, int* nz, double* dx, double* dz, double* x_min, double* z_min)
{
    return guarded([&]() {
        check_species(sim, 0);
        mag::Sim& s = *sim->s;
        if (nx) *nx = s.nx;
        if (nz) *nz = s.nz;
        if (dx) *dx = s.dx;
        if (dz) *dz = s.dz;
        if (x_min) *x_min = s.x0;
        if (z_min) *z_min = s.z0;
        return MAG_OK;
    });
}

int mag_n_species(mag_sim* sim)
{
    return guarded([&]() {
        check_species(sim, 0);
        return (int)sim->s->sp.size();
    });
}

int mag_species(mag_sim* sim, int species, mag_species_info* out)
{
    return guarded([&]() {
        check_species(sim, species);
        mag::Sim& s = *sim->s;
        const mag::SpeciesState& S = s.sp[species];
        std::memset(out, 0, sizeof *out);
        std::strncpy(out->name, S.prm.name.c_str(), sizeof out->name - 1);
        out->type = S.prm.type;
        out->mass = S.prm.mass;
        out->charge = S.prm.charge;
        out->dt = S.prm.dt;
        out->density = S.prm.density;
        out->temperature = S.prm.temperature;
        out->E_max = S.E_max;
        out->v_max = S.v_max;
        out->lifetime = S.lifetime;
        out->capacity = S.cap;
        if (S.n_slots > 0) {
            double e2;
            unsigned long long n;
            s.energy(species, e2, n);
            out->n_live = (int64_t)n;
        }
        out->niter = s.niter(species);
        return MAG_OK;
    });
}

int mag_get_field(mag_sim* sim, int which, double* host_out)
{
    return guarded([&]() {
        check_species(sim, 0);
        sim->s->get_field(which, host_out);
        return MAG_OK;
    });
}

int mag_get_face_field(mag_sim* sim, int component, float* host_out)
{
    return guarded([&]() {
        check_species(sim, 0);
        if (!host_out || (component != 0 && component != 1)) throw mag::Error(MAG_EINVAL, "face field: component 0 or 1");
        sim->s->get_faces(component, host_out);
        return MAG_OK;
    });
}

int mag_set_field(mag_sim* sim, int which, const double* host_in)
{
    return guarded([&]() {
        check_species(sim, 0);
        sim->s->set_field(which, host_in);
        return MAG_OK;
    });
}

int mag_field_solve(mag_sim* sim, mag_solve_info* info)
{
    return guarded([&]() {
        check_species(sim, 0);
        mag::SolveStatus st = sim->s->field_solve();
        int rc = device_status(sim);
        if (info) {
            info->iterations = st.iterations;
            info->residual = st.residual;
            info->status = st.converged ? MAG_OK : MAG_ENOTCONV;
            info->levels = sim->s->solver_levels();
        }
        return rc;
    });
}

int mag_solve_status(mag_sim* sim, mag_solve_info* info)
{
    return guarded([&]() {
        check_species(sim, 0);
        if (!info) throw mag::Error(MAG_EINVAL, "null argument");
        int rc = device_status(sim);  // synchronises and refreshes the last solve's status
        const mag::SolveStatus st = sim->s->last_solve;
        info->iterations = st.iterations;
        info->residual = st.residual;
        info->status = st.converged ? MAG_OK : MAG_ENOTCONV;
        info->levels = sim->s->solver_levels();
        return rc;
    });
}

int mag_solve_phase_times(mag_sim* sim, double* ms_out, int cap)
{
    return guarded([&]() {
        check_species(sim, 0);
        if (!ms_out || cap <= 0) throw mag::Error(MAG_EINVAL, "null argument");
        return sim->s->solve_phase_times(ms_out, cap);
    });
}

int mag_get_particles(mag_sim* sim, int species, int64_t cap, double* x, double* z, double* vx, double* vy,
                      double* vz, uint32_t* id, int64_t* n_out)
{
    return guarded([&]() {
        check_species(sim, species);
        int64_t n = 0;
        sim->s->get_particles(species, cap, x, z, vx, vy, vz, id, &n);
        if (n_out) *n_out = n;
        return device_status(sim);
    });
}

int mag_set_particles(mag_sim* sim, int species, int64_t n, const double* x, const double* z, const double* vx,
                      const double* vy, const double* vz)
{
    return guarded([&]() {
        check_species(sim, species);
        if (n < 0) throw mag::Error(MAG_EINVAL, "negative particle count");
        sim->s->set_particles(species, n, x, z, vx, vy, vz);
        return MAG_OK;
    });
}

int mag_diag(mag_sim* sim, int species, mag_diag_out* out)
{
    return guarded([&]() {
        check_species(sim, species);
        mag::Sim& s = *sim->s;
        const mag::SpeciesState& S = s.sp[species];
        std::memset(out, 0, sizeof *out);
        double e2 = 0;
        unsigned long long n = 0;
        mag::Counters c{};
        const int err = s.diag(species, e2, n, c);
        out->n_live = (int64_t)n;
        out->mean_energy_eV = n ? e2 / (double)n * S.prm.mass * 0.5 / mag::kQe : 0.0;
        out->total_charge = (double)n * S.prm.charge * s.p.macroparticle_factor;
        out->collisions = (int64_t)c.ncoll;
        out->null_collisions = (int64_t)c.nnull;
        out->removed = (int64_t)c.removed;
        out->particle_steps = (int64_t)c.live_sum;
        out->niter = s.niter(species);
        return status_of(err);
    });
}

int mag_get_rho_fixed(mag_sim* sim, int species, int64_t* host_out)
{
    return guarded([&]() {
        check_species(sim, species);
        sim->s->get_rho_fixed(species, host_out);
        return MAG_OK;
    });
}

void* mag_rho_fixed_ptr(mag_sim* sim, int species)
{
    if (!sim || !sim->s || species < 0 || species >= (int)sim->s->sp.size()) return nullptr;
    return sim->s->sp[species].rho.p;
}

int mag_set_rho_fixed(mag_sim* sim, int species, const int64_t* host_in)
{
    return guarded([&]() {
        check_species(sim, species);
        if (!host_in) throw mag::Error(MAG_EINVAL, "null input");
        sim->s->set_rho_fixed(species, host_in);
        return MAG_OK;
    });
}

int mag_deposit(mag_sim* sim)
{
    return guarded([&]() {
        check_species(sim, 0);
        sim->s->deposit_all();
        return device_status(sim);
    });
}

int mag_config_param(const char* config_path, const char* key, double* value)
{
    return guarded([&]() {
        const mag::Param p = mag::make_param(mag::KeyValueConfig::from_file(config_path));
        const std::string k = key;
        const std::map<std::string, double> v = {
            {"x_max", p.x_max}, {"y_max", p.y_max}, {"z_max", p.z_max}, {"x_sampl", (double)p.x_sampl},
            {"z_sampl", (double)p.z_sampl}, {"n_particles_total", p.n_particles_total},
            {"density_total", p.density_total}, {"pressure", p.pressure},
            {"neutral_temperature", p.neutral_temperature}, {"probe_radius", p.probe_radius},
            {"u_probe", p.u_probe}, {"extern_field", p.extern_field}, {"Br", p.Br}, {"Bz", p.Bz}, {"Bt", p.Bt},
            {"rf_amplitude", p.rf_amplitude}, {"rf_U0", p.rf_U0}, {"rf_omega", p.rf_omega},
            {"macroparticle_factor", p.macroparticle_factor}, {"dx", p.dx}, {"dz", p.dz}, {"idx", p.idx},
            {"idz", p.idz}, {"V", p.V}, {"dV", p.dV}, {"dy", p.dy}, {"neutral_density", p.neutral_density},
            {"coord", (double)p.coord}, {"boundary", (double)p.boundary}, {"geometry", (double)p.geometry},
            {"selfconsistent", (double)p.selfconsistent}, {"rf", (double)p.rf},
            {"electric_field_from_file", (double)p.electric_field_from_file},
            {"magnetic_field_const", (double)p.magnetic_field_const}, {"niter", (double)p.niter},
            {"t_print", (double)p.t_print}, {"t_dist_sample", (double)p.t_dist_sample},
            {"t_equilib", (double)p.t_equilib}, {"mover", (double)p.mover}};
        auto it = v.find(k);
        if (it == v.end()) throw mag::Error(MAG_EINVAL, "unknown Param key " + k);
        *value = it->second;
        return MAG_OK;
    });
}

int mag_config_geometry(const char* config_path, int64_t cap, int8_t* mask, double* voltage, int* nx, int* nz)
{
    return guarded([&]() {
        const mag::Param p = mag::make_param(mag::KeyValueConfig::from_file(config_path));
        std::vector<int8_t> m;
        std::vector<double> v;
        mag::build_geometry(p, m, v);
        if (nx) *nx = p.x_sampl;
        if (nz) *nz = p.z_sampl;
        if ((int64_t)m.size() > cap) throw mag::Error(MAG_EINVAL, "output arrays too small");
        if (mask) std::copy(m.begin(), m.end(), mask);
        if (voltage) std::copy(v.begin(), v.end(), voltage);
        return MAG_OK;
    });
}

int mag_config_species(const char* config_path, const char* species_conf_path, int index, mag_species_info* out,
                       double* rates_out)
{
    return guarded([&]() {
        (void)config_path;
        std::vector<mag::SpeciesParams> sp;
        std::vector<mag::InteractionParams> in;
        mag::parse_species_conf(species_conf_path, sp, in);
        if (index < 0 || index >= (int)sp.size()) throw mag::Error(MAG_EINVAL, "species index out of range");
        std::vector<double> rates;
        double lifetime;
        mag::species_rates(sp, in, index, rates, lifetime);
        const mag::SpeciesParams& S = sp[index];
        if (out) {
            std::memset(out, 0, sizeof *out);
            std::strncpy(out->name, S.name.c_str(), sizeof out->name - 1);
            out->type = S.type;
            out->mass = S.mass;
            out->charge = S.charge;
            out->dt = S.dt;
            out->density = S.density;
            out->temperature = S.temperature;
            out->E_max = S.E_max > 0. ? S.E_max : S.temperature * mag::kKB / mag::kQe * 10.0;
            out->v_max = std::sqrt(2.0 * mag::kKB * S.temperature / S.mass);
            out->lifetime = lifetime;
        }
        if (rates_out) std::copy(rates.begin(), rates.end(), rates_out);
        return (int)sp.size();
    });
}

void* mag_stream(mag_sim* sim) { return sim && sim->s ? (void*)sim->s->stream : nullptr; }

int64_t mag_kernel_launches(mag_sim* sim) { return sim && sim->s ? sim->s->launches : 0; }

int mag_dist_reset(mag_sim* sim)
{
    return guarded([&]() {
        check_species(sim, 0);
        sim->s->dist_reset();
        return device_status(sim);
    });
}

int mag_dist_sample(mag_sim* sim)
{
    return guarded([&]() {
        check_species(sim, 0);
        sim->s->dist_sample();
        return MAG_OK;
    });
}

int mag_dist_samples(mag_sim* sim)
{
    return guarded([&]() {
        check_species(sim, 0);
        return sim->s->dist_samples();
    });
}

int mag_energy_dist(mag_sim* sim, int species, int cap, double* centers, double* values, double* stats)
{
    return guarded([&]() {
        check_species(sim, species);
        std::vector<double> pos, val;
        double st[4];
        sim->s->energy_dist(species, pos, val, st);
        if ((int)pos.size() > cap && (centers || values)) throw mag::Error(MAG_EINVAL, "output arrays too small");
        if (centers) std::copy(pos.begin(), pos.end(), centers);
        if (values) std::copy(val.begin(), val.end(), values);
        if (stats) std::copy(st, st + 4, stats);
        return (int)pos.size();
    });
}

int mag_get_average(mag_sim* sim, int which, double* host_out)
{
    return guarded([&]() {
        check_species(sim, 0);
        if (!host_out) throw mag::Error(MAG_EINVAL, "null output");
        if (sim->s->dist_samples() <= 0) throw mag::Error(MAG_EINVAL, "no samples (call mag_dist_sample first)");
        sim->s->average(which, host_out);
        return device_status(sim);
    });
}

int mag_print_distribution(mag_sim* sim, const char* dir)
{
    return guarded([&]() {
        check_species(sim, 0);
        if (!dir) throw mag::Error(MAG_EINVAL, "null directory");
        sim->s->print_distribution(dir);
        return device_status(sim);
    });
}

int mag_print_trace(mag_sim* sim, const char* dir)
{
    return guarded([&]() {
        check_species(sim, 0);
        if (!dir) throw mag::Error(MAG_EINVAL, "null directory");
        sim->s->print_trace(dir);
        return device_status(sim);
    });
}

int mag_print_field(mag_sim* sim, const char* path)
{
    return guarded([&]() {
        check_species(sim, 0);
        if (!path) throw mag::Error(MAG_EINVAL, "null path");
        sim->s->print_field(path);
        return device_status(sim);
    });
}

int mag_species_save(mag_sim* sim, int species, const char* path)
{
    return guarded([&]() {
        check_species(sim, species);
        if (!path) throw mag::Error(MAG_EINVAL, "null path");
        sim->s->save_species(species, path);
        return device_status(sim);
    });
}

int mag_set_electrode_voltages(mag_sim* sim, const double* v, int64_t n)
{
    return guarded([&]() {
        check_species(sim, 0);
        if (!v || n < 0) throw mag::Error(MAG_EINVAL, "null or negative voltage array");
        sim->s->set_voltages(v, (size_t)n);
        return device_status(sim);
    });
}

int mag_n_live(mag_sim* sim, int species, int64_t* n_out)
{
    return guarded([&]() {
        check_species(sim, species);
        if (!n_out) throw mag::Error(MAG_EINVAL, "null output");
        double e2 = 0;
        unsigned long long n = 0;
        if (sim->s->sp[species].n_slots > 0) sim->s->energy(species, e2, n);
        *n_out = (int64_t)n;
        return device_status(sim);
    });
}

int mag_get_particles_aos(mag_sim* sim, int species, int64_t cap, void* records, int64_t* n_out)
{
    return guarded([&]() {
        check_species(sim, species);
        if (!records && cap > 0) throw mag::Error(MAG_EINVAL, "null output");
        const int64_t n = std::max<int64_t>(0, std::min<int64_t>(cap, sim->s->sp[species].n_slots));
        std::vector<double> x(n), z(n), vx(n), vy(n), vz(n);
        int64_t m = 0;
        sim->s->get_particles(species, n, x.data(), z.data(), vx.data(), vy.data(), vz.data(), nullptr, &m);
        unsigned char* out = static_cast<unsigned char*>(records);
        for (int64_t k = 0; k < m; ++k) {
            unsigned char* r = out + 64 * k;
            std::memset(r, 0, 64);
            const double d[7] = {x[k], 0.0, z[k], vx[k], vy[k], vz[k], 0.0};
            std::memcpy(r, d, sizeof d);  // empty = false, padding zero
        }
        if (n_out) *n_out = m;
        return device_status(sim);
    });
}

int mag_source_refresh(mag_sim* sim, int factor)
{
    return guarded([&]() {
        check_species(sim, 0);
        if (!sim->s->p.use_source) throw mag::Error(MAG_EINVAL, "mag_source_refresh: the config does not set use_source");
        sim->s->source_refresh(factor);
        return device_status(sim);
    });
}

int mag_source_save(mag_sim* sim, int species, const char* path)
{
    return guarded([&]() {
        check_species(sim, species);
        if (!path) throw mag::Error(MAG_EINVAL, "null path");
        sim->s->source_save(species, path);
        return device_status(sim);
    });
}

int mag_source_load(mag_sim* sim, int species, const char* path)
{
    return guarded([&]() {
        check_species(sim, species);
        if (!path) throw mag::Error(MAG_EINVAL, "null path");
        if (!sim->s->source_load(species, path)) throw mag::Error(MAG_EIO, std::string("cannot open ") + path);
        return device_status(sim);
    });
}

int mag_source_info(mag_sim* sim, int species, int64_t* n_box, int64_t* injected, int64_t* dropped)
{
    return guarded([&]() {
        check_species(sim, species);
        mag::Sim& s = *sim->s;
        const mag::SourceState& Q = s.src[species];
        unsigned long long d = 0;
        if (Q.dropped.p) {
            MAG_CK(cudaStreamSynchronize(s.stream));
            MAG_CK(cudaMemcpy(&d, Q.dropped.p, sizeof d, cudaMemcpyDeviceToHost));
        }
        if (n_box) *n_box = Q.n;
        if (injected) *injected = (int64_t)Q.injected;
        if (dropped) *dropped = (int64_t)d;
        return device_status(sim);
    });
}

int mag_species_load(mag_sim* sim, int species, const char* path)
{
    return guarded([&]() {
        check_species(sim, species);
        if (!path) throw mag::Error(MAG_EINVAL, "null path");
        sim->s->load_species(species, path);
        return device_status(sim);
    });
}

int mag_particle_file_read(const char* path, int64_t cap, double* x, double* y, double* z, double* vx, double* vy,
                           double* vz, double* time_to_death, int64_t* n_out, int64_t* total_out)
{
    return guarded([&]() {
        if (!path) throw mag::Error(MAG_EINVAL, "null path");
        const mag::ParticleFile f = mag::read_particle_file(path);
        const int64_t n = (int64_t)f.x.size();
        if (n_out) *n_out = n;
        if (total_out) *total_out = f.total;
        if (n > cap && (x || y || z || vx || vy || vz || time_to_death))
            throw mag::Error(MAG_EINVAL, "output arrays too small");
        auto put = [&](double* o, const std::vector<double>& v) {
            if (o) std::copy(v.begin(), v.end(), o);
        };
        put(x, f.x);
        put(y, f.y);
        put(z, f.z);
        put(vx, f.vx);
        put(vy, f.vy);
        put(vz, f.vz);
        put(time_to_death, f.ttd);
        return MAG_OK;
    });
}

int mag_particle_file_write(const char* path, int64_t total, int64_t n, const double* x, const double* y,
                            const double* z, const double* vx, const double* vy, const double* vz,
                            const double* time_to_death)
{
    return guarded([&]() {
        if (!path || n < 0 || (n > 0 && (!x || !z || !vx || !vy || !vz)))
            throw mag::Error(MAG_EINVAL, "invalid arguments");
        mag::ParticleFile f;
        f.total = (int32_t)std::max(total, n);
        f.x.assign(x, x + n);
        f.z.assign(z, z + n);
        f.vx.assign(vx, vx + n);
        f.vy.assign(vy, vy + n);
        f.vz.assign(vz, vz + n);
        if (y) f.y.assign(y, y + n);
        else f.y.assign(n, 0.0);
        if (time_to_death) f.ttd.assign(time_to_death, time_to_death + n);
        else f.ttd.assign(n, 0.0);
        mag::write_particle_file(path, f);
        return MAG_OK;
    });
}

int mag_adjoint_run(mag_sim* sim, const mag_adj_cfg* cfg, double* grad_out, mag_adj_out* out)
{
    return guarded([&]() {
        check_species(sim, 0);
        if (!cfg || (cfg->n_voltage_keys > 0 && !cfg->voltage_keys) || cfg->n_voltage_keys < 0)
            throw mag::Error(MAG_EINVAL, "invalid adjoint configuration");
        mag::AdjointConfig c;
        c.nsteps = cfg->nsteps;
        c.checkpoint = cfg->checkpoint > 0 ? cfg->checkpoint : 100;
        for (int q = 0; q < cfg->n_voltage_keys; ++q) {
            if (!cfg->voltage_keys[q]) throw mag::Error(MAG_EINVAL, "null voltage key");
            c.voltage_keys.push_back(cfg->voltage_keys[q]);
        }
        c.grad_b = cfg->grad_b != 0;
        c.w_energy = cfg->w_energy;
        c.w_lost = cfg->w_lost;
        const mag::AdjointResult r = mag::Adjoint::run(*sim->s, c);
        if (grad_out) std::copy(r.grad.begin(), r.grad.end(), grad_out);
        if (out) {
            out->loss = r.loss;
            out->mean_energy_eV = r.mean_energy_eV;
            out->lost_fraction = r.lost_fraction;
            out->n0 = r.n0;
            out->n_live = r.n_live;
        }
        return device_status(sim);
    });
}

int mag_batch_create(int n, const mag_instance_desc* desc, const mag_opts* opts, mag_batch** out)
{
    return guarded([&]() {
        if (n <= 0 || !desc || !out) throw mag::Error(MAG_EINVAL, "invalid arguments");
        mag::SimOptions o;
        if (opts) {
            o.device = opts->device;
            o.sort_interval = opts->sort_interval;
            o.poisson_tol = opts->poisson_tol;
            o.poisson_max_iter = opts->poisson_max_iter;
            o.capacity_hint = opts->capacity_hint;
            o.push_vec = opts->push_vec;
        }
        std::vector<mag::BatchInstanceDesc> d((size_t)n);
        for (int i = 0; i < n; ++i) {
            if (!desc[i].config_path || !desc[i].species_conf_path)
                throw mag::Error(MAG_EINVAL, "instance " + std::to_string(i) + ": null path");
            d[i].config = desc[i].config_path;
            d[i].species_conf = desc[i].species_conf_path;
            d[i].initscript = desc[i].initscript_path ? desc[i].initscript_path : "";
            d[i].seed = desc[i].seed;
        }
        auto h = std::make_unique<mag_batch>();
        h->b = std::make_unique<mag::Batch>(d, o);
        h->views.resize((size_t)n);
        *out = h.release();
        return MAG_OK;
    });
}

void mag_batch_destroy(mag_batch* b) { delete b; }

static mag::Batch& batch_of(mag_batch* b)
{
    if (!b || !b->b) throw mag::Error(MAG_EINVAL, "null batch handle");
    return *b->b;
}

int mag_batch_size(mag_batch* b)
{
    return guarded([&]() { return batch_of(b).size(); });
}

int mag_batch_advance_init(mag_batch* b)
{
    return guarded([&]() {
        batch_of(b).advance_init();
        return MAG_OK;
    });
}

int mag_batch_advance(mag_batch* b, uint64_t nsteps)
{
    return guarded([&]() {
        batch_of(b).advance(nsteps);
        return MAG_OK;
    });
}

int mag_batch_tune(mag_batch* b, int steps_per_trial, mag_batch_tuning* out)
{
    return guarded([&]() {
        const mag::BatchTuning t = batch_of(b).tune(steps_per_trial);
        if (out) {
            out->push_vec = t.push_vec;
            out->solve_threads = t.solve_threads;
            out->sort_interval = t.sort_interval;
            out->ms_per_step = t.ms_per_step;
        }
        return MAG_OK;
    });
}

int mag_batch_set_graph(mag_batch* b, int enabled)
{
    return guarded([&]() {
        batch_of(b).use_graph = enabled != 0;
        return MAG_OK;
    });
}

int mag_batch_sync(mag_batch* b)
{
    return guarded([&]() {
        const int e = batch_of(b).sync();
        if (e) g_last_error = "device error " + std::to_string(e) + " in a batched instance";
        return e;
    });
}

int mag_batch_instance(mag_batch* b, int i, mag_sim** out)
{
    return guarded([&]() {
        mag::Batch& B = batch_of(b);
        if (i < 0 || i >= B.size() || !out) throw mag::Error(MAG_EINVAL, "instance index out of range");
        if (!b->views[i]) {
            b->views[i] = std::make_unique<mag_sim>();
            b->views[i]->s = std::unique_ptr<mag::Sim, SimRelease>(&B.instance(i), SimRelease{false});
        }
        *out = b->views[i].get();
        return MAG_OK;
    });
}

void* mag_batch_stream(mag_batch* b) { return (b && b->b) ? (void*)b->b->stream : nullptr; }

int64_t mag_batch_kernel_launches(mag_batch* b)
{
    if (!b || !b->b) return 0;
    int64_t n = b->b->launches;
    for (int i = 0; i < b->b->size(); ++i) n += b->b->instance(i).launches;
    return n;
}

}  // extern "C"
