/* CPU oracle for the mag2d PIC-MCC step — TEST INFRASTRUCTURE ONLY.
 *
 * A restatement, in our own code, of the reference's time step in FP64 with
 * the reference's own random number generator (SHR3 + ziggurat), so that the
 * same inputs and seed give the same particle states bit for bit.  It is the
 * checker for the GPU library: only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load it.  The product never does.
 *
 * Every function cites the reference file:line it follows (paths relative to
 * the reference project root).
 */
#ifndef MAG2D_ORACLE_H
#define MAG2D_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

/* Param (src/param.cpp:12-143) fields the step reads. */
typedef struct {
    int coord;            /* 0 CARTESIAN, 1 CYLINDRICAL */
    int x_sampl, z_sampl; /* grid nodes along x (rows) and z (columns) */
    double x_max, z_max, y_max;
    double n_particles_total, density_total, macroparticle_factor;
    double extern_field;
    int geometry_empty;   /* geometry == EMPTY (fields.hpp:256) */
    int selfconsistent, rf, electric_field_from_file;
    double rf_amplitude, rf_omega, rf_U0;
    int boundary;         /* 0 FREE, 1 PERIODIC */
    int magnetic_field_const;
    double Br, Bz, Bt;
    int mover;            /* 0 ADVANCE_BORIS, 1 ADVANCE_MULTICOLL (param.cpp mover) */
    int u_smooth;         /* Fields::u_smooth after each self-consistent solve (param.cpp:53) */
} orc_config;

enum { ORC_ELASTIC = 0, ORC_LANGEVIN = 1, ORC_CX = 2, ORC_COULOMB = 3, ORC_SUPERELASTIC = 4 };
enum { ORC_U = 0, ORC_URF = 1, ORC_RHO = 2, ORC_MASK = 3, ORC_VOLTAGE = 4, ORC_SPECIES_RHO = 5 };

const char* orc_last_error(void);

orc_sim* orc_create(const orc_config* cfg, const signed char* mask, const double* voltage);
void orc_destroy(orc_sim* s);
int orc_add_species(orc_sim* s, const char* name, double mass, double charge, double dt,
                    double density, double temperature, double E_max);
int orc_add_interaction(orc_sim* s, int primary, int secondary, int type, double DE_eV,
                        double rate, double cutoff, int n_table, const double* E_eV,
                        const double* sigma);
/* electric_field_from_file (src/pic.cpp:154-177): u (and uRF when rf) on their own grid */
int orc_set_loaded_fields(orc_sim* s, int nx, int nz, double dx, double dz, double xmin,
                          double zmin, const double* u, const double* uRF);
/* Magnetic field tables (src/fields.cpp:870-959) on their own grid */
int orc_set_bfield(orc_sim* s, int nx, int nz, double dx, double dz, double xmin, double zmin,
                   const double* Br, const double* Bz);
/* Pic constructor tail: lifetimes, matrix factorisation, initial field solves */
int orc_init(orc_sim* s);
int orc_seed(orc_sim* s, uint32_t seed);
int orc_run_initscript(orc_sim* s, const char* path);
int orc_set_particles(orc_sim* s, int sp, int n, const double* x, const double* z,
                      const double* vx, const double* vy, const double* vz);
int orc_n_slots(orc_sim* s, int sp);
int orc_n_live(orc_sim* s, int sp);
int orc_get_particles(orc_sim* s, int sp, double* out8);
int orc_advance_init(orc_sim* s);
int orc_advance(orc_sim* s, int nsteps);
double orc_time_advance(orc_sim* s, int nsteps);
int orc_get_field(orc_sim* s, int which, double* out);
int orc_field_shape(orc_sim* s, int which, int* nx, int* nz);
int orc_solve(orc_sim* s, const double* rho, double* u);
int orc_grad(orc_sim* s, int which, int n, const double* x, const double* z, double* gx, double* gz);
int orc_species_info(orc_sim* s, int sp, double* out11);
int orc_rates(orc_sim* s, int sp, double* out);
int orc_sigma_v(orc_sim* s, int sp, int tgt, int n, const double* v, double* out);
/* kind: 0 uni, 1 rnor, 2 rexp, 3 iuni, 4 rot(1,...) x3, 5 deflect(angle=arg) of (1,0,0) x3 */
int orc_rng(orc_sim* s, int kind, int n, double arg, double* out);
/* Collision counter: number of scatter() calls per species since creation */
int64_t orc_collisions(orc_sim* s, int sp);
/* collisions that selected an interaction (the candidates minus the null collisions) */
int64_t orc_real_collisions(orc_sim* s, int sp);

/* Fixed-point CIC deposit (Field2D.hpp:45-62 with quantised weights): a
 * particle at fixed-point grid position (xf, zf) -- cells times 2^20 -- in
 * cell i = xf >> 20, j = zf >> 20 (clamped to the last cell) adds
 * (2^20-U)(2^20-V), U(2^20-V), (2^20-U)V, UV to the four corners of the cell,
 * U = xf - i*2^20, V = zf - j*2^20.  acc is nx*nz int64 (row-major, z
 * fastest), accumulated into.  Particles with alive[i]==0 are skipped.
 * Returns the number deposited. */
/* Fields::u_smooth (fields.cpp:28-111) with its defaults (no symmetry
 * averaging, no radius): out = the 3x3 smoothing of in on rows 1..nx-2,
 * columns 1..nz-1, in elsewhere.  Neighbours are read by row-major flat index,
 * so column nz wraps to column 0 of the next row, as in the reference; the one
 * read past the array (row nx-2, column nz-1, its +1/+1 neighbour) reads 0. */
void orc_u_smooth(int nx, int nz, const double* in, double* out);

int64_t orc_deposit_fixed(int nx, int nz, int64_t n, const uint32_t* xf, const uint32_t* zf,
                          const uint8_t* alive, int64_t* acc);

#ifdef __cplusplus
}
#endif
#endif
