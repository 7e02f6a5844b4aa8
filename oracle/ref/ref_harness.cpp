// C-callable harness around the reference's own Pic<D> (test infrastructure).
//
// This file is compiled together with the reference's unmodified sources
// (src/pic.cpp is included below, the other src/*.cpp files are compiled as
// separate units) by oracle/Makefile into oracle/_ref/libmag2d_ref.so.  It
// replaces the reference's main() (src/test.cpp:18-97, src/test_MCC.cpp:18-90)
// with C entry points so tests can drive the reference step by step:
//   construction      test.cpp:24-50 (Param, Pic<D>)
//   seeding           test_MCC.cpp:148 (rnd.initialize_seed)
//   run_initscript    pic.cpp:241-328
//   advance_init      pic.cpp:359-384
//   advance           pic.cpp:330-358
// Nothing in the product links this library.
#include "particles.hpp"

#include <chrono>
#include <cstring>
#include <stdexcept>
#include <string>

// The reference declares these Species<CYLINDRICAL> members
// (particles.hpp:293-295, 311) but never defines them, so a Pic<CYLINDRICAL>
// does not link as shipped.  They are defined here to fail the same way an
// initscript using them would fail to build in the reference.
template <>
void Species<CYLINDRICAL>::add_particles_everywhere(int)
{
    throw std::runtime_error("add_particles_everywhere is not defined for CYLINDRICAL in the reference\n");
}
template <>
void Species<CYLINDRICAL>::add_particles_bessel(int, double, double, double)
{
    throw std::runtime_error("add_particles_bessel is not defined for CYLINDRICAL in the reference\n");
}
template <>
void Species<CYLINDRICAL>::add_particles_on_disk(int, double, double, double)
{
    throw std::runtime_error("add_particles_on_disk is not defined for CYLINDRICAL in the reference\n");
}
template <>
void Species<CYLINDRICAL>::source()
{
    throw std::runtime_error("source is not defined for CYLINDRICAL in the reference\n");
}

#include "pic.cpp"

namespace {

thread_local std::string g_err;

struct RefSim {
    GetPot* config = nullptr;
    Param* param = nullptr;
    Pic<CARTESIAN>* cart = nullptr;
    Pic<CYLINDRICAL>* cyl = nullptr;
    ~RefSim()
    {
        delete cart;
        delete cyl;
        delete param;
        delete config;
    }
};

template <class F>
int guard(F&& f)
{
    try {
        return f();
    } catch (std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

// Apply f to whichever Pic<D> the simulation holds.
template <class F>
int with_pic(void* h, F&& f)
{
    RefSim* s = static_cast<RefSim*>(h);
    return guard([&]() { return s->cart ? f(*s->cart) : f(*s->cyl); });
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

void* ref_create(const char* config_path, const char* species_conf, const char* output_dir, unsigned seed)
{
    RefSim* s = new RefSim;
    int rc = guard([&]() {
        s->config = new GetPot(config_path);
        s->param = new Param(*s->config);
        s->param->species_conf_file = species_conf;
        s->param->output_dir = output_dir;
        s->param->do_plot = false;  // the gnuplot pipe is out of scope
        if (s->param->coord == CYLINDRICAL) {
            s->cyl = new Pic<CYLINDRICAL>(*s->param);
            s->cyl->rnd.initialize_seed(seed);
        } else {
            s->cart = new Pic<CARTESIAN>(*s->param);
            s->cart->rnd.initialize_seed(seed);
        }
        return 0;
    });
    if (rc != 0) {
        delete s;
        return nullptr;
    }
    return s;
}

void ref_destroy(void* h) { delete static_cast<RefSim*>(h); }

int ref_seed(void* h, unsigned seed)
{
    return with_pic(h, [&](auto& p) { p.rnd.initialize_seed(seed); return 0; });
}

int ref_coord(void* h) { return static_cast<RefSim*>(h)->cyl ? 1 : 0; }

// out[0..11] = dx, dz, x_min, z_min, x_max, z_max, V, dV, dy, macroparticle_factor,
//              eps_0, q_e ; dims[0..1] = rows (x), columns (z) of field.u
int ref_grid(void* h, int* dims, double* out)
{
    RefSim* s = static_cast<RefSim*>(h);
    return with_pic(h, [&](auto& p) {
        Field2D& u = p.field.u;
        dims[0] = u.jmax;
        dims[1] = u.lmax;
        Param& q = *s->param;
        double v[12] = {u.GetDx(), u.GetDy(), q.x_min, q.z_min, q.x_max, q.z_max,
                        q.V, q.dV, q.dy, q.macroparticle_factor, q.eps_0, q.q_e};
        std::memcpy(out, v, sizeof v);
        return 0;
    });
}

int ref_n_species(void* h)
{
    return with_pic(h, [&](auto& p) { return (int)p.speclist.size(); });
}

// out[0..10] = mass, charge, dt, density, temperature, lifetime, E_max, v_max,
//              slots, live, niter
int ref_species(void* h, int sp, char* name, int namelen, double* out)
{
    return with_pic(h, [&](auto& p) {
        BaseSpecies* b = p.speclist[sp];
        std::strncpy(name, b->name.c_str(), namelen - 1);
        name[namelen - 1] = 0;
        double v[11] = {b->mass, b->charge, b->dt, b->density, b->temperature, b->lifetime,
                        b->E_max, b->v_max, (double)b->particles.size(), (double)b->n_particles(),
                        (double)p.speclist[sp]->t / (b->dt > 0 ? b->dt : 1.0)};
        std::memcpy(out, v, sizeof v);
        return 0;
    });
}

int ref_rates(void* h, int sp, double* out)
{
    return with_pic(h, [&](auto& p) {
        BaseSpecies* b = p.speclist[sp];
        for (size_t i = 0; i < b->rates_by_species.size(); ++i) out[i] = b->rates_by_species[i];
        return (int)b->rates_by_species.size();
    });
}

// sigma_v of every interaction of species sp with target species tgt, at the
// relative speeds v[0..n).  out is laid out [interaction][n].
int ref_sigma_v(void* h, int sp, int tgt, int n, const double* v, double* out)
{
    return with_pic(h, [&](auto& p) {
        BaseSpecies* b = p.speclist[sp];
        std::vector<Interaction*>& ints = b->interactions_by_species[tgt];
        for (size_t k = 0; k < ints.size(); ++k)
            for (int i = 0; i < n; ++i) out[k * n + i] = ints[k]->sigma_v(v[i]);
        return (int)ints.size();
    });
}

int ref_run_initscript(void* h, const char* path)
{
    return with_pic(h, [&](auto& p) { p.run_initscript(path); return 0; });
}

// Replace the particles of species sp by n particles.  Slot i holds input i.
int ref_set_particles(void* h, int sp, int n, const double* x, const double* z,
                      const double* vx, const double* vy, const double* vz)
{
    return with_pic(h, [&](auto& p) {
        BaseSpecies* b = p.speclist[sp];
        if (!b->particles.empty())
            throw std::runtime_error("ref_set_particles: species already holds particles\n");
        // grow to exactly n slots through the reference's own free list
        // (particles.hpp:223-249, particles.cpp:95-107)
        b->resize(n);
        for (int k = 0; k < n; ++k) b->insert();
        for (int i = 0; i < n; ++i) {
            t_particle& q = b->particles[i];
            q.x = x[i];
            q.y = 0.0;
            q.z = z[i];
            q.vx = vx[i];
            q.vy = vy[i];
            q.vz = vz[i];
            q.time_to_death = 0.0;
            q.empty = false;
        }
        return 0;
    });
}

// All slots of species sp: out[slot*8 + {0..7}] = x, y, z, vx, vy, vz, time_to_death, empty
int ref_get_particles(void* h, int sp, double* out)
{
    return with_pic(h, [&](auto& p) {
        BaseSpecies* b = p.speclist[sp];
        for (size_t i = 0; i < b->particles.size(); ++i) {
            const t_particle& q = b->particles[i];
            double* o = out + 8 * i;
            o[0] = q.x; o[1] = q.y; o[2] = q.z; o[3] = q.vx; o[4] = q.vy; o[5] = q.vz;
            o[6] = q.time_to_death; o[7] = q.empty ? 1.0 : 0.0;
        }
        return (int)b->particles.size();
    });
}

// BaseSpecies::save / load (src/particles.cpp:32-93) of species sp
int ref_save(void* h, int sp, const char* path)
{
    return with_pic(h, [&](auto& p) { p.speclist[sp]->save(path); return 0; });
}

int ref_load(void* h, int sp, const char* path)
{
    return with_pic(h, [&](auto& p) { p.speclist[sp]->load(path); return (int)p.speclist[sp]->particles.size(); });
}

// The driver's source refresh after advance_init (src/test.cpp:56-59):
// Species::source5_refresh(factor) of every species
int ref_source_refresh(void* h, int factor)
{
    RefSim* s = static_cast<RefSim*>(h);
    return guard([&]() {
        if (!s->cart) throw std::runtime_error("source5_refresh is defined for CARTESIAN only in the reference\n");
        for (size_t i = 0; i < s->cart->speclist.size(); ++i)
            if (s->cart->speclist[i]->particle) s->cart->speclist[i]->source5_refresh(factor);
        return 0;
    });
}

// BaseSpecies::source5_save (src/particles.cpp:109-120) of species sp
int ref_source_save(void* h, int sp, const char* path)
{
    return with_pic(h, [&](auto& p) { p.speclist[sp]->source5_save(path); return 0; });
}

// live particles of species sp (non-empty slots)
int ref_n_live(void* h, int sp)
{
    return with_pic(h, [&](auto& p) {
        int n = 0;
        for (const t_particle& q : p.speclist[sp]->particles) n += q.empty ? 0 : 1;
        return n;
    });
}

int ref_advance_init(void* h)
{
    return with_pic(h, [&](auto& p) { p.advance_init(); return 0; });
}

int ref_advance(void* h, int nsteps)
{
    return with_pic(h, [&](auto& p) { for (int i = 0; i < nsteps; ++i) p.advance(); return 0; });
}

// Wall time of nsteps calls of Pic::advance (the std::chrono pattern of a
// driver loop; init and I/O excluded).
double ref_time_advance(void* h, int nsteps)
{
    double secs = -1.0;
    with_pic(h, [&](auto& p) {
        auto t0 = std::chrono::steady_clock::now();
        for (int i = 0; i < nsteps; ++i) p.advance();
        secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return 0;
    });
    return secs;
}

// which: 0 u, 1 uRF, 2 field.rho, 3 mask, 4 voltage, 5 species-0 rho ... (5+s)
int ref_get_field(void* h, int which, double* out)
{
    return with_pic(h, [&](auto& p) {
        if (which <= 2 || which >= 5) {
            Field2D* f = which == 0 ? &p.field.u : which == 1 ? &p.field.uRF
                       : which == 2 ? &p.field.rho : &p.speclist[which - 5]->rho;
            for (int i = 0; i < f->jmax; ++i)
                for (int j = 0; j < f->lmax; ++j) out[(size_t)i * f->lmax + j] = (*f)[i][j];
            return f->jmax * f->lmax;
        }
        t_grid& g = p.field.grid;
        for (int i = 0; i < g.M; ++i)
            for (int j = 0; j < g.N; ++j)
                out[(size_t)i * g.N + j] = which == 3 ? (double)g.mask[i][j] : g.voltage[i][j];
        return g.M * g.N;
    });
}

// Fields::boundary_solve (fields.cpp:278-312) on a caller-given rho.
int ref_solve(void* h, const double* rho, double* u)
{
    return with_pic(h, [&](auto& p) {
        Field2D& r = p.field.rho;
        for (int i = 0; i < r.jmax; ++i)
            for (int j = 0; j < r.lmax; ++j) r[i][j] = rho[(size_t)i * r.lmax + j];
        p.field.boundary_solve();
        for (int i = 0; i < r.jmax; ++i)
            for (int j = 0; j < r.lmax; ++j) u[(size_t)i * r.lmax + j] = p.field.u[i][j];
        p.field.reset();
        return 0;
    });
}

// Fields::u_smooth() with its default arguments (fields.cpp:28-111) applied to
// a caller-given potential; field.u is restored afterwards.
int ref_u_smooth(void* h, const double* u_in, double* u_out)
{
    return with_pic(h, [&](auto& p) {
        Field2D& u = p.field.u;
        std::vector<double> keep((size_t)u.jmax * u.lmax);
        for (int i = 0; i < u.jmax; ++i)
            for (int j = 0; j < u.lmax; ++j) {
                keep[(size_t)i * u.lmax + j] = u[i][j];
                u[i][j] = u_in[(size_t)i * u.lmax + j];
            }
        p.field.u_smooth();
        for (int i = 0; i < u.jmax; ++i)
            for (int j = 0; j < u.lmax; ++j) {
                u_out[(size_t)i * u.lmax + j] = u[i][j];
                u[i][j] = keep[(size_t)i * u.lmax + j];
            }
        return 0;
    });
}

// Field2D::grad of u (which=0) or uRF (which=1) at n points (Field2D.hpp:80-168)
int ref_grad(void* h, int which, int n, const double* x, const double* z, double* gx, double* gz)
{
    return with_pic(h, [&](auto& p) {
        Field2D& f = which == 0 ? p.field.u : p.field.uRF;
        for (int i = 0; i < n; ++i) f.grad(x[i], z[i], gx[i], gz[i]);
        return 0;
    });
}

// Draws from the reference's t_random (src/random.cpp): kind 0 uni, 1 rnor,
// 2 rexp, 3 iuni, 4 rot(1, x, y, z) -> 3 values, 5 deflect(arg) of (1,0,0) -> 3 values
int ref_rng(void* h, int kind, int n, double arg, double* out)
{
    return with_pic(h, [&](auto& p) {
        t_random& r = p.rnd;
        for (int i = 0; i < n; ++i) {
            if (kind == 0) out[i] = r.uni();
            else if (kind == 1) out[i] = r.rnor();
            else if (kind == 2) out[i] = r.rexp();
            else if (kind == 3) out[i] = (double)r.iuni();
            else if (kind == 4) r.rot(1.0, out[3 * i], out[3 * i + 1], out[3 * i + 2]);
            else {
                double x = 1.0, y = 0.0, z = 0.0;
                r.deflect(arg, x, y, z);
                out[3 * i] = x; out[3 * i + 1] = y; out[3 * i + 2] = z;
            }
        }
        return n;
    });
}

}  // extern "C"
