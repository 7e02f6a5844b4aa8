/* mag2d_gpu — GB300 (sm_103a) implementation of the mag2d PIC-MCC time step.
 *
 * C ABI of libmag2d_gpu.so.  Plain pointers and sizes only; every call returns
 * an int status (MAG_OK = 0, negative on error) and mag_last_error() gives the
 * message of the last failing call on the calling thread.  No C++ exception
 * crosses this boundary.
 *
 * The reference (rouckas/mag2d) has no plugin or FFI layer: its time loop is a
 * C++ driver (src/test.cpp:18-97) that builds a Param from config.txt, a
 * Pic<D> from it, runs the initscript, advance_init() and then advance() once
 * per iteration.  Each entry point below replaces one of those C++ calls; the
 * comment names the reference interface (file:line) it stands in for.
 *
 * Threading: one mag_sim per host thread.  Device memory belongs to the
 * handle; every host buffer passed in or out is owned by the caller.  All work
 * of a handle runs in order on the handle's own CUDA stream.
 */
#ifndef MAG2D_GPU_H
#define MAG2D_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MAG_OK = 0,
    MAG_EINVAL = -1,     /* bad argument or configuration (Param / config_parse errors) */
    MAG_ECUDA = -2,      /* CUDA runtime error */
    MAG_ERANGE = -3,     /* particle or node index outside the grid (Field2D range checks) */
    MAG_ENOTCONV = -4,   /* Poisson solve did not reach its tolerance */
    MAG_ETIMEOUT = -5,   /* a bounded device-side wait gave up */
    MAG_EIO = -6,        /* file could not be read */
    MAG_ENOMEM = -7
};

/* Field selectors for mag_get_field / mag_set_field (Fields members, src/fields.hpp:187-222) */
enum {
    MAG_U = 0,        /* electrostatic potential u [V] */
    MAG_URF = 1,      /* RF unit potential uRF [V per V of rf_amplitude] */
    MAG_RHO = 2,      /* field.rho: summed species charge per node [C], as deposited */
    MAG_MASK = 3,     /* t_grid::mask: FIXED=0, FIXED_RF=1, FREE=2, BOUNDARY=3 */
    MAG_VOLTAGE = 4,  /* t_grid::voltage [V] */
    MAG_SPECIES_RHO = 5 /* + species index: BaseSpecies::rho [C] */
};

typedef struct mag_sim mag_sim;

typedef struct {
    int device;            /* CUDA device ordinal */
    uint64_t seed;         /* Philox key of every random draw */
    int sort_interval;     /* counting sort of particles by cell every N steps (0 = 20, < 0 = never) */
    double poisson_tol;    /* Jacobi-scaled residual / max|u| at which the solve stops (0 = 1e-12) */
    int poisson_max_iter;  /* outer refinement iterations before MAG_ENOTCONV (0 = 200) */
    int64_t capacity_hint; /* particle slots to reserve per species (0 = grow as needed) */
    int push_vec;          /* consecutive slots per thread of the particle kernel: 1, 2 or 4 (0 = 4 for
                              species of at least 4e6 slots, else 2); results do not depend on it */
    int direct_solve;      /* self-consistent Poisson solves by the precomputed inverse of the operator
                              (built at the first solve): 0 = for grids up to 20000 nodes, 1 = also
                              larger ones up to the one-block size, -1 = always multigrid */
    int max_fused_steps;   /* where particles are independent over several steps (no self-consistent
                              field, collision targets without particles), up to this many steps run
                              as one particle launch, with results identical to single steps
                              (0 = 64, 1 = never) */
    int multigrid_fp64;    /* 1: multigrid Poisson solves with every level in FP64 (no FP32 V-cycle), for
                              grids up to 70000 nodes; slower, kept to time the FP32 multigrid with FP64
                              refinement against (0 = FP32 multigrid + FP64 refinement) */
} mag_opts;

typedef struct {
    char name[64];
    int type;              /* SpeciesType: NEUTRAL=0, ELECTRON=1, ION=2 (src/parser.hpp:14) */
    double mass, charge, dt, density, temperature, E_max, v_max, lifetime;
    int64_t n_live;        /* BaseSpecies::n_particles (src/particles.hpp:248) */
    int64_t capacity;
    uint64_t niter;        /* steps this species has advanced */
} mag_species_info;

typedef struct {
    int64_t n_live;
    double mean_energy_eV;   /* mean (vx^2+vy^2+vz^2) m / 2 / q_e over live particles (FP64) */
    double total_charge;     /* n_live * charge * macroparticle factor of the deposit [C] */
    int64_t collisions;      /* real (non-null) collisions since creation */
    int64_t null_collisions; /* candidates that the null-collision test rejected */
    int64_t removed;         /* particles removed at the boundary since creation */
    int64_t particle_steps;  /* sum over completed steps of the live particles after the step */
    uint64_t niter;          /* completed steps of this species */
} mag_diag_out;

typedef struct {
    int iterations;          /* outer FP64 refinement iterations of the last solve */
    double residual;         /* Jacobi-scaled residual / max|u| after the last solve */
    int status;              /* MAG_OK or MAG_ENOTCONV */
    int levels;              /* multigrid levels (1 = plain red-black SOR) */
} mag_solve_info;

const char* mag_last_error(void);

/* Library version string. */
const char* mag_version(void);

/* Param(GetPot&) + Pic<D>(param) + run_initscript (src/test.cpp:24-53,
 * src/param.cpp:12-143, src/pic.cpp:127-189, :241-328).  initscript may be
 * NULL.  opts may be NULL for defaults. */
int mag_create(const char* config_path, const char* species_conf_path, const char* initscript_path,
               const mag_opts* opts, mag_sim** out);
void mag_destroy(mag_sim* sim);

/* Pic::run_initscript (src/pic.cpp:241-328) */
int mag_run_initscript(mag_sim* sim, const char* initscript_path);

/* Pic::advance_init (src/pic.cpp:359-384) */
int mag_advance_init(mag_sim* sim);
/* the same; deposit = 0 solves from the species' fixed-point deposits as they
 * are (set by mag_set_rho_fixed, e.g. summed over the processes of a particle
 * decomposition) instead of depositing the handle's own particles first */
int mag_advance_init_ex(mag_sim* sim, int deposit);

/* nsteps calls of Pic::advance (src/pic.cpp:330-358).  Asynchronous: returns
 * once the work is queued; errors found on the device are reported by the
 * next synchronising call (mag_sync, getters). */
int mag_advance(mag_sim* sim, uint64_t nsteps);

/* mag_advance with CUDA events recorded on the handle's stream between the
 * kernels of every step; ms_out[0..3] receive the summed device time of the
 * particle sort (every sort_interval steps), the Poisson solve, the particle
 * kernels and the collision kernels (timed after all particle kernels, so
 * without their overlap).  Fused steps (mag_opts.max_fused_steps) count their
 * launch, collisions included, as particle time.  Synchronises. */
int mag_advance_timed(mag_sim* sim, uint64_t nsteps, double* ms_out);

/* Wait for queued work and report any device-side error flag. */
int mag_sync(mag_sim* sim);

/* Grid of field u (Field2D::GetDx/GetDy/GetXMin..., src/Field2D.hpp:32-37). */
int mag_grid(mag_sim* sim, int* nx, int* nz, double* dx, double* dz, double* x_min, double* z_min);

int mag_n_species(mag_sim* sim);
int mag_species(mag_sim* sim, int species, mag_species_info* out);

/* Copy a field to host (Field2D data, row-major, z fastest; x_sampl*z_sampl doubles). */
int mag_get_field(mag_sim* sim, int which, double* host_out);
/* Overwrite u, uRF or rho from host doubles (e.g. for a solve of a given rho). */
int mag_set_field(mag_sim* sim, int which, const double* host_in);
/* Copy the face field E = -grad u that the particle kernel reads (Field2D::grad,
 * src/Field2D.hpp, staggered differences; FP32 [V/m]): component 0 = Ex on
 * (x_sampl+1)*z_sampl faces, 1 = Ez on x_sampl*(z_sampl+1) faces, row-major.
 * After u is set by hand (mag_set_field) the faces follow at the next solve. */
int mag_get_face_field(mag_sim* sim, int component, float* host_out);

/* Fields::boundary_solve (src/fields.cpp:278-312): solve for u from the current
 * rho (MAG_RHO) exactly as a self-consistent step does. */
int mag_field_solve(mag_sim* sim, mag_solve_info* info);

/* Status of the most recent Poisson solve (the one of the last self-consistent
 * step, or of mag_field_solve): outer FP64 refinement iterations, final
 * residual, convergence.  Synchronises.  No reference counterpart (UMFPACK's
 * direct solve has no iteration count). */
int mag_solve_status(mag_sim* sim, mag_solve_info* info);

/* Phase times of the multigrid Poisson solve (the time spent inside
 * Fields::boundary_solve, src/fields.cpp:278-312, by part).  The first call
 * switches the timing on for every later solve of the handle (thread 0 of
 * block 0 reads the GPU's global timer after each grid-wide barrier; cost:
 * one memset per solve) and returns zeros.  Later calls return the times of
 * the most recent multigrid solve in ms (solves by the precomputed inverse
 * are not timed):
 *   [0] start (extrapolated start, right-hand side)  [1] FP64 residuals with
 *   their max reductions  [2 + l] down part of level l (smoothing, residual,
 *   restriction; l < 12)  [14] the coarse levels run by block 0, or the
 *   coarsest solve  [15 + l] up part of level l (prolongation, smoothing; on
 *   level 0 also the update of u)  [27] face field  [28] whole solve.
 * Writes min(cap, 29) values; returns that number. */
int mag_solve_phase_times(mag_sim* sim, double* ms_out, int cap);

/* Live particles of a species as SoA doubles in SI units (the t_particle
 * fields x, z, vx, vy, vz of src/particles.hpp:26-33) plus a persistent id.
 * Any pointer may be NULL.  *n_out receives the number written (<= cap). */
int mag_get_particles(mag_sim* sim, int species, int64_t cap, double* x, double* z, double* vx,
                      double* vy, double* vz, uint32_t* id, int64_t* n_out);
/* Replace the particles of a species (ids 0..n-1 in input order). */
int mag_set_particles(mag_sim* sim, int species, int64_t n, const double* x, const double* z,
                      const double* vx, const double* vy, const double* vz);

/* Diagnostics of one species (BaseSpecies::print_status, src/particles.cpp:367-375). */
int mag_diag(mag_sim* sim, int species, mag_diag_out* out);

/* Fixed-point charge accumulator of a species: int64 per node, each live
 * particle contributing exactly 2^40 split over its four CIC nodes
 * (Field2D::accumulate weights, src/Field2D.hpp:45-62, quantised to 2^-20 per
 * axis).  Reflects the deposit of the last step. */
int mag_get_rho_fixed(mag_sim* sim, int species, int64_t* host_out);

/* Particle decomposition of one instance over several processes (one GPU
 * each, every one with the full grid): after each mag_advance(sim, 1) every
 * process sums the species' fixed-point deposits over all processes (an
 * integer all-reduce, so the sum is bit-identical in any order) and writes
 * the total back before the next step's Poisson solve.  mag_rho_fixed_ptr
 * gives the device array (nx*nz int64, on the handle's stream) for an
 * in-place device all-reduce; mag_set_rho_fixed writes it from the host.  No
 * reference counterpart (the reference runs on one core). */
void* mag_rho_fixed_ptr(mag_sim* sim, int species);
int mag_set_rho_fixed(mag_sim* sim, int species, const int64_t* host_in);

/* Recompute the fixed-point deposit of the current particles of every species
 * (Species::accumulate, src/particles.hpp:358-367) without moving them. */
int mag_deposit(mag_sim* sim);

/* ---- host-only inspection (no GPU needed) -------------------------------- */

/* A value of the Param built from config_path (src/param.cpp:12-143), by key:
 * the config keys (x_max, z_max, x_sampl, z_sampl, extern_field, rf_omega,
 * macroparticle_factor, Br, Bz, Bt, ...), the derived dx, dz, idx, idz, V, dV,
 * dy, neutral_density, and the enumerations coord, boundary, geometry,
 * selfconsistent, rf, electric_field_from_file as numbers. */
int mag_config_param(const char* config_path, const char* key, double* value);

/* t_grid mask and voltage of the config's geometry (src/fields.cpp:374-868).
 * cap = capacity of the output arrays in nodes; *nx, *nz receive the grid. */
int mag_config_geometry(const char* config_path, int64_t cap, int8_t* mask, double* voltage, int* nx, int* nz);

/* Species 'index' of species_conf_path as parsed (src/parser.cpp:25-147), with
 * its null-collision rates against every species (rates_out, n_species
 * doubles) and lifetime (BaseSpecies::lifetime_init, src/particles.cpp:142-206).
 * Returns the number of species. */
int mag_config_species(const char* config_path, const char* species_conf_path, int index,
                       mag_species_info* out, double* rates_out);

/* ---- allocation-free Poisson solve ------------------------------------------
 *
 * No counterpart in the reference.  Fields::boundary_solve (src/fields.cpp:278-312)
 * as a stateless call that allocates no device memory, for callers that cannot
 * call cudaMalloc: code running under a fixed, pre-reserved device-memory budget
 * or a caching allocator it does not own, or calling from a context where a
 * device allocation would synchronise the device.  The caller owns rho_dev and
 * u_dev (device memory, nx*nz doubles, z fastest); u_dev holds the initial guess
 * on entry (zeros are fine) and the potential on return.  mask_host and
 * voltage_host are host arrays (t_grid::mask / voltage).  coord: 0 Cartesian,
 * 1 cylindrical; dV is used by the Cartesian scaling, macroparticle_factor by
 * the cylindrical one.  stream may be NULL (default stream).  With info != NULL
 * the call waits for the solve and reports it (info->status MAG_OK,
 * MAG_ENOTCONV or MAG_ETIMEOUT, also the return value).  With info == NULL it
 * returns once the work is queued and gives no report of the solve at all;
 * voltage_host is then still being copied, so page-locked voltage_host memory
 * must stay valid until the stream has reached the solve.
 *
 * Working memory is one static device array of 4 MiB that every GPU loading the
 * library holds until exit; grids above 257 x 257 nodes are rejected with
 * MAG_EINVAL.  The first call on a device looks up the array's device address
 * with that device current and keeps it for the process; the kept address
 * does not survive cudaDeviceReset.  All
 * calls share the array and it keeps the last call's contents: calls that
 * overlap on the GPU race. */
int mag_poisson_solve_noalloc(int coord, int nx, int nz, double dx, double dz, double macroparticle_factor,
                              double dV, const int8_t* mask_host, const double* voltage_host,
                              const double* rho_dev, double* u_dev, double tol, int max_iter, void* stream,
                              mag_solve_info* info);

/* Device stream of the handle (a cudaStream_t) so callers can order their own
 * work and timing events with the simulation's. */
void* mag_stream(mag_sim* sim);

/* Number of kernel launches the handle has issued since creation. */
int64_t mag_kernel_launches(mag_sim* sim);

/* ---- Sampled distributions ------------------------------------------------
 * Pic::dist_reset / dist_sample (src/pic.cpp:412-428): each sample adds every
 * species' kinetic-energy histogram (Histogram of 200 bins over [0, E_max],
 * src/particles.hpp:169, filled as energy_dist_compute does) and its charge
 * deposit (rhoAverage), and the potential (uAvg).  Computed on the GPU. */
int mag_dist_reset(mag_sim* sim);
int mag_dist_sample(mag_sim* sim);
int mag_dist_samples(mag_sim* sim);  /* samples since the last reset, or < 0 on error */
/* Histogram::print values of species s: bin centres and data / norm; stats =
 * n_val, sum, n_val_tot, sum_tot (mean = sum / n_val, mean_tot = sum_tot /
 * n_val_tot).  Arrays of cap >= 200 entries (any may be NULL).  Returns the
 * number of bins or a negative status. */
int mag_energy_dist(mag_sim* sim, int species, int cap, double* centers, double* values, double* stats);
/* The average over the samples of MAG_U (uAvg) or MAG_SPECIES_RHO + s (rhoAverage) */
int mag_get_average(mag_sim* sim, int which, double* host_out);
/* BaseSpecies::print_distribution files <dir>/<name>_energy_dist.dat and
 * <name>_rho.dat, and Fields::u_print (potential.dat) at path */
int mag_print_distribution(mag_sim* sim, const char* dir);
int mag_print_field(mag_sim* sim, const char* path);
/* Pic::print_trace (src/pic.cpp:446-451, TrackedParticle::print,
 * src/particles.cpp:12-17): for every particle an initscript added with
 * add_tracked_particle, one line "x z vx vz vy" (10 significant digits) is
 * appended to <dir>/<species>_traj_<slot>.dat, slot being the particle's
 * index when it was added; a handle's first call truncates the file (the
 * reference opens it when the particle is added).  A removed particle gets
 * no line (the reference prints its stale slot). */
int mag_print_trace(mag_sim* sim, const char* dir);

/* ---- Particle files ---------------------------------------------------------
 * BaseSpecies::save / load (src/particles.cpp:32-93): int32 slot count, int32
 * live count, then one 64-byte t_particle record (doubles x, y, z, vx, vy, vz,
 * time_to_death; bool empty; padding) per live particle.  Loading replaces the
 * species' particles; positions outside the domain are redrawn uniformly in
 * it.  A config with particle_reload = 1 loads every species from
 * <particle_reload_dir>/particles_<name>.dat at mag_create (src/pic.cpp:138-146). */
/* Electrode voltages (t_grid::voltage, x_sampl * z_sampl values; only the
 * FIXED and FIXED_RF nodes' entries are used).  The RF Laplace solution and,
 * without a self-consistent field, the static potential are solved again as
 * in the Pic constructor (src/pic.cpp:170-186); a self-consistent run solves
 * with them from its next step.  Not with electric_field_from_file. */
int mag_set_electrode_voltages(mag_sim* sim, const double* v, int64_t n);

/* Live particles of a species (BaseSpecies::n_particles, src/particles.hpp:248). */
int mag_n_live(mag_sim* sim, int species, int64_t* n_out);

/* Live particles as 64-byte t_particle records (src/particles.hpp:26-33:
 * doubles x, y, z, vx, vy, vz, time_to_death, bool empty = false, padding),
 * at most cap records, in slot order. */
int mag_get_particles_aos(mag_sim* sim, int species, int64_t cap, void* records, int64_t* n_out);

int mag_species_save(mag_sim* sim, int species, const char* path);
int mag_species_load(mag_sim* sim, int species, const char* path);

/* Particle source of a Cartesian run with use_source = 1
 * (Species<CARTESIAN>::source5_refresh / source, src/particles.cpp:1052-1226).
 * mag_advance_init refreshes the source boxes with src_fact, as the
 * reference's driver does after advance_init (src/test.cpp:56-59);
 * mag_source_refresh redraws them with another factor.  Every step, after a
 * species' push, its box particles fly in the external field (with the
 * species' background collisions) and each crossing of a box face appends a
 * copy entering the domain through the opposite face at a random tile.
 * save / load: the source5 file (int32 count, then 64-byte t_particle
 * records, src/particles.cpp:109-140); load returns MAG_EIO when the file
 * cannot be opened (the reference warns and continues).  A config with
 * particle_reload = 1 and use_source = 1 loads
 * <particle_reload_dir>/particles_source_<name>.dat at mag_create.
 * mag_source_info: box particles, copies appended so far, copies dropped
 * (more than 4 face crossings of one box particle in one step). */
int mag_source_refresh(mag_sim* sim, int factor);
int mag_source_save(mag_sim* sim, int species, const char* path);
int mag_source_load(mag_sim* sim, int species, const char* path);
int mag_source_info(mag_sim* sim, int species, int64_t* n_box, int64_t* injected, int64_t* dropped);
/* Host-only reading and writing of that file.  read: n_out = live records,
 * total_out = the slot count of the header; arrays of at least cap entries
 * (any may be NULL).  write: y and time_to_death may be NULL (zeros). */
int mag_particle_file_read(const char* path, int64_t cap, double* x, double* y, double* z, double* vx, double* vy,
                           double* vz, double* time_to_death, int64_t* n_out, int64_t* total_out);
int mag_particle_file_write(const char* path, int64_t total, int64_t n, const double* x, const double* y,
                            const double* z, const double* vx, const double* vy, const double* vz,
                            const double* time_to_death);

/* ---- Adjoint gradients ------------------------------------------------------
 * Gradient of a trap diagnostic after nsteps steps,
 *   L = w_energy * mean over live particles of m vz^2 / 2 [eV]
 *     + w_lost * (particles lost) / (particles at the start),
 * with respect to electrode voltages (config keys such as u_segment_3 or
 * u_endcap; the geometry is linear in them) and the constant magnetic field,
 * by a hand-written adjoint of the collisionless step (push, gather, deposit,
 * Poisson), checkpointed every `checkpoint` steps and recomputed in between.
 * The handle must be fresh: particles loaded, mag_advance_init not yet called;
 * the call runs advance_init and the nsteps forward steps itself and leaves
 * the handle at the end of them.  Requires collisions off, constant B and no
 * RF.  No reference counterpart (the reference computes no derivatives). */
typedef struct {
    uint64_t nsteps;
    int checkpoint;                 /* steps between checkpoints (0 = 100) */
    int n_voltage_keys;
    const char* const* voltage_keys;
    int grad_b;                     /* 1: append d L / d(Br, Bt, Bz) */
    double w_energy, w_lost;
} mag_adj_cfg;

typedef struct {
    double loss, mean_energy_eV, lost_fraction;
    int64_t n0, n_live;
} mag_adj_out;

/* grad_out: n_voltage_keys (+ 3 with grad_b) doubles */
int mag_adjoint_run(mag_sim* sim, const mag_adj_cfg* cfg, double* grad_out, mag_adj_out* out);

/* ---- Batched instances ----------------------------------------------------
 * Many independent simulations (each one the Pic of its own config.txt,
 * species_conf and initscript, as src/test.cpp builds it, with its own seed)
 * advanced together: each step issues one Poisson launch with a block per
 * self-consistent instance, one particle launch over every instance's
 * particles and one collision launch, replayed from a captured CUDA graph
 * between particle sorts.  No reference counterpart: the reference runs one
 * Pic per process (the drive_*.py sweeps).  Instances keep the reference's
 * step semantics; with several moving species per instance the collision
 * scatter of all species follows the push of all species. */
typedef struct mag_batch mag_batch;

typedef struct {
    const char* config_path;
    const char* species_conf_path;
    const char* initscript_path;   /* may be NULL */
    uint64_t seed;
} mag_instance_desc;

typedef struct {
    int push_vec;        /* slots per thread of the particle kernel */
    int solve_threads;   /* threads of each instance's solve block */
    int sort_interval;   /* steps between particle sorts */
    double ms_per_step;  /* device time per step measured with these parameters */
} mag_batch_tuning;

/* opts: device, sort_interval, poisson_tol, poisson_max_iter, push_vec apply to
 * every instance (seed comes from each descriptor); opts may be NULL. */
int mag_batch_create(int n, const mag_instance_desc* desc, const mag_opts* opts, mag_batch** out);
void mag_batch_destroy(mag_batch* b);
int mag_batch_size(mag_batch* b);
/* Pic::advance_init of every instance */
int mag_batch_advance_init(mag_batch* b);
/* nsteps steps of every instance; asynchronous like mag_advance */
int mag_batch_advance(mag_batch* b, uint64_t nsteps);
/* The batch's own autotuner: times candidate launch parameters on
 * steps_per_trial real steps each (the instances advance; no parameter changes
 * any result) and keeps the fastest.  out may be NULL. */
int mag_batch_tune(mag_batch* b, int steps_per_trial, mag_batch_tuning* out);
/* 0: every step is issued as separate launches; 1 (default): steps between
 * sorts are replayed from a captured CUDA graph */
int mag_batch_set_graph(mag_batch* b, int enabled);
/* wait for queued work; first device error of any instance */
int mag_batch_sync(mag_batch* b);
/* Borrowed handle of instance i for the single-instance getters (mag_diag,
 * mag_get_field, mag_get_particles, ...).  It must not be advanced on its own
 * and stays valid until mag_batch_destroy; mag_destroy on it is a no-op. */
int mag_batch_instance(mag_batch* b, int i, mag_sim** out);
/* Device stream of the batch (a cudaStream_t) */
void* mag_batch_stream(mag_batch* b);
int64_t mag_batch_kernel_launches(mag_batch* b);

/* ---- 3D Cartesian run (coord = CARTESIAN3D) --------------------------------
 * ElMag3D + Species<CARTESIAN3D> (src/fields3d.cpp:1-101, src/species3d.cpp:3-94,
 * src/Field3D.hpp:40-163), whose prototype code does not build as shipped;
 * these entry points follow its mathematics: the box faces fixed at 0 V and
 * the centre node (the "Quadrupole" electrode) at 1 V; -lap(u) = rho / eps0
 * on the 7-point grid with its spacings (rho = deposited charge x
 * macroparticle_factor / cell volume); E = -grad u by Field3D's staggered
 * differences; the leapfrog Boris step with constant B (Br, Bt, Bz as
 * Bx, By, Bz), FREE or PERIODIC boundary, the 8-corner is_free test, the
 * trilinear deposit and the null-collision MCC of the 2D path.  Grids are
 * x_sampl x y_sampl x z_sampl nodes, index (i ny + j) nz + k.
 * mag3d_grid returns the number of species; dims = nx, ny, nz; spacing =
 * dx, dy, dz.  mag3d_solve: ElMag3D::solve of the given charge density
 * [C/m^3] (or of the deposits when rho is NULL), conjugate gradients to
 * poisson_tol (relative residual).  mag3d_get_field: MAG_U, MAG_RHO (charge
 * per node [C] as deposited), MAG_MASK (0 fixed, -1 electrode, 2 free).
 * mag_opts fields used: device, seed, poisson_tol, poisson_max_iter,
 * capacity_hint. */
typedef struct mag3d_sim mag3d_sim;
int mag3d_create(const char* config_path, const char* species_conf_path, const mag_opts* opts, mag3d_sim** out);
void mag3d_destroy(mag3d_sim* sim);
int mag3d_grid(mag3d_sim* sim, int* dims, double* spacing);
int mag3d_set_particles(mag3d_sim* sim, int species, int64_t n, const double* x, const double* y, const double* z,
                        const double* vx, const double* vy, const double* vz);
int mag3d_get_particles(mag3d_sim* sim, int species, int64_t cap, double* x, double* y, double* z, double* vx,
                        double* vy, double* vz, uint32_t* id, int64_t* n_out);
int mag3d_advance_init(mag3d_sim* sim);
int mag3d_advance(mag3d_sim* sim, uint64_t nsteps);
int mag3d_solve(mag3d_sim* sim, const double* rho, mag_solve_info* info);
int mag3d_get_field(mag3d_sim* sim, int which, double* out);
int mag3d_get_rho_fixed(mag3d_sim* sim, int species, int64_t* out);
int mag3d_diag(mag3d_sim* sim, int species, mag_diag_out* out);
int64_t mag3d_kernel_launches(mag3d_sim* sim);

#ifdef __cplusplus
}
#endif
#endif
