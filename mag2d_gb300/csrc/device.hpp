// Data shared between the host orchestration and the sm_103a kernels.
//
// HBM layout of one species (SoA, one array per component, length = slots):
//   x, z   uint32  position in cells of the field grid as fixed point with
//                  kFracBits fractional bits: x = round((x_SI - x_min)/dx * 2^20).
//                  The cell index is x >> 20 and the CIC fraction (x & 0xFFFFF)
//                  is exact; resolution 2^-20 cell everywhere on grids up to
//                  4095 cells per axis.  A removed particle holds x = kDead.
//   vx, vy, vz float  velocity [m/s]; (vx, vy, vz) = (radial/x, azimuthal/y, axial/z)
//                  as in t_particle (src/particles.hpp:26-33)
//   id     uint32  persistent particle id (key of its random stream)
// Fields live on node grids of nx*nz points, row-major with z fastest
// (Array2D, src/Array.hpp:14-23).  The electric field is kept on cell faces:
//   Exf[(nx+1)*nz]  -du/dx between nodes i-1 and i, with the end faces repeated
//   Ezf[nx*(nz+1)]  -du/dz between nodes j-1 and j
// which makes the staggered gradient of Field2D::grad (src/Field2D.hpp:80-168)
// a plain bilinear interpolation of four face values per component.
#pragma once
#include <vector_types.h>

#include <cstdint>

namespace mag {

constexpr int kMaxSpecies = 16;
constexpr int kMaxInteractions = 64;
constexpr int kMaxLevels = 12;
constexpr long long kSingleBlockNodes = 70000;  // grids up to this size run on one block
constexpr long long kSingleBlockLevel = 4096;   // levels of a multi-block solve up to this size run on block 0
// tile phases of a multi-block solve: halo rings around a tile's interior (the
// four colour passes of a phase plus two) and shared bytes per region node
// (FP32 correction, FP32 right-hand side / residual, one flag byte; on the
// Galerkin levels also the 9 operator planes and the inverse diagonal)
constexpr int kTileHalo = 6;
constexpr int kTileNodeBytes = 9;
constexpr int kTileNodeBytesGalerkin = 49;
// phase times of one solve (mag_solve_phase_times): start and right-hand side,
// FP64 residual with its reduction, the down part of each level, the coarse
// part run by block 0 (or the coarsest solve), the up part of each level, the
// face field, and the whole solve
constexpr int kPhaseStart = 0, kPhaseResidual = 1, kPhaseDown = 2, kPhaseCoarse = 2 + 12, kPhaseUp = 3 + 12,
              kPhaseFaces = 3 + 24, kPhaseTotal = 4 + 24, kSolvePhases = 5 + 24;
constexpr long long kGreenMaxNodes = 20000;     // grids up to this size solve by the precomputed inverse
constexpr int kFracBits = 20;      // fixed-point fraction of a cell in the positions
constexpr int kDepositShift = 20;  // CIC weights quantised to 2^-20 per axis (= kFracBits)
constexpr uint32_t kFracMask = (1u << kFracBits) - 1u;
constexpr uint32_t kDead = 0xFFFFFFFFu;
constexpr int kMaxCellsPerAxis = 4095;
constexpr int64_t kSlotAlign = 64;  // particle arrays hold a multiple of this many slots (vector access)
constexpr int64_t kScrambledSortMin = 4000000;  // slots from which scrambled input takes the three-pass sort

// CollType of the species_conf INTERACTION blocks (src/parser.hpp:15)
enum CollType { ELASTIC = 0, LANGEVIN = 1, CX = 2, COULOMB = 3, SUPERELASTIC = 4 };

// Per-species counters.  The particle kernel of launch i adds to slot i & 1
// of the per-step counters; the next launch's first thread folds slot
// (i - 1) & 1 into the running totals and clears it, so no kernel has to find
// out which of its blocks finished last.  Host reads add the slot of the last
// launch, which no kernel has folded yet.
struct Counters {
    unsigned long long live_par[2];   // live particles after the step of that launch parity
    unsigned long long ncand_par[2];  // collision candidates listed by the step of that parity
    unsigned long long live_sum;      // sum over folded steps of live particles
    unsigned long long removed;       // particles removed at the boundary
    unsigned long long ncoll;         // real collisions
    unsigned long long nnull;         // null collisions
    unsigned long long partner_miss;
    unsigned long long slots;         // slots in use on the device (shrinks when a sort compacts)
    int error;                        // first device error code (0 = none)
    int pad;
};

// Null-collision tables of one species (device copy), shared by the inline
// collision path of the particle kernel and the candidate-list kernel.
struct InterDev;
struct MccSpecies {
    double mass, inv_lifetime;
    int nsp;
    double rates[kMaxSpecies];
    double t_mass[kMaxSpecies], t_density[kMaxSpecies], t_sigma_v[kMaxSpecies];
    int inter_begin[kMaxSpecies], inter_end[kMaxSpecies];
    const InterDev* inter;
    const double* tables;
};

struct PushArgs {
    uint32_t *x, *z;
    float *vx, *vy, *vz;
    const uint32_t* id;
    int64_t n;                 // slots (upper bound; the live range may be shorter after a sort)
    const unsigned long long* n_dev;  // current slot count on the device (null: use n)
    int nx, nz;
    uint32_t xmaxf, zmaxf;     // domain extent in fixed point
    int periodic;
    int check_mask;            // kill particles in cells with no FREE corner (t_grid::is_free)
    const int8_t* mask;        // nx*nz
    const uint8_t* cellfree;   // (nx-1)*(nz-1): 1 when one of the cell's four nodes is FREE
    // electric field: 0 uniform (0, extern_ez), 1 from u faces, 2 from (u, uRF) face pairs
    int emode;
    const float* Exf;
    const float* Ezf;
    const float2* Exf2;
    const float2* Ezf2;
    float extern_ez;
    float phase;                   // rf_amplitude cos(mod(rf_omega niter dt, 1e7 pi)) + rf_U0 (fields.hpp:135-145)
    uint64_t step;                 // this species' step counter (niter), the counter of its random streams
    // magnetic field: constant Boris vectors, or tables Br/Bz (Field2D::interpolate)
    int has_b;                     // 0: B = 0 everywhere, the rotation is the identity
    int btab;
    // t = q B dt / 2m and s = 2 t / (1 + t^2), each as a float pair hi + lo (lo
    // the FP32 rounding remainder of the FP64 value), so that the rotation angle
    // carries no systematic FP32 rounding from one step to the next
    float tx, ty, tz, sx, sy, sz;
    float tlx, tly, tlz, slx, sly, slz;
    const float* Br;
    const float* Bz;
    int bnx, bnz;
    float b_x0, b_z0, b_ix, b_iz;  // table index = (x_cells*dx + x_min - b_xmin) * b_idx
    float gdx, gdz, gx0, gz0;      // field grid dx, dz, x_min, z_min (for tables)
    float q_dt_2m;                 // charge*dt/(2*mass)
    float hq;                      // charge/mass*dt/2
    float cx, cz;                  // dt/dx, dt/dz (cells per m/s)
    unsigned long long* rho;       // fixed-point deposit (nx*nz) or null
    uint32_t coll_threshold;       // collision probability * 2^32 (0: no test)
    uint32_t* cand;                // candidate slots (run by k_collide)
    float4* cand_rec;              // candidate (vx, vy, vz, id bits) after the push
    const MccSpecies* mcc;
    uint64_t seed;
    uint32_t species;
    Counters* cnt;
    int slot;                      // parity of this launch (Counters::live_par, ncand_par)
    int fold_slot;                 // slot of the previous launch to fold into the totals, or -1
};

struct InterDev {
    int type;          // CollType
    int target;        // secondary species index
    double DE;         // [J]
    double rate;       // RATE (LANGEVIN: already times cutoff^2)
    double cutoff;
    double mu;         // reduced mass
    int tab_off, tab_n;
    double coul_lambda_D, coul_q1q2;
};

struct CollideArgs {
    float *vx, *vy, *vz;
    const uint32_t* cand;
    const float4* cand_rec;    // (vx, vy, vz, id bits) of each candidate after the push
    const InterDev* inter;     // the whole interaction list (MccSpecies::inter) and its tables,
    int n_inter;               // staged in shared memory by the kernel
    const double* tables;
    int n_tables;
    Counters* cnt;
    int slot;                  // parity of the particle kernel launch whose candidates these are
    const MccSpecies* mcc;
    int t_has_slots[kMaxSpecies];
    int any_target_slots;      // some target species holds particles (partner = random particle)
    const uint32_t* t_x[kMaxSpecies];
    float* t_vx[kMaxSpecies];
    float* t_vy[kMaxSpecies];
    float* t_vz[kMaxSpecies];
    int64_t t_n[kMaxSpecies];
    uint64_t seed;
    uint32_t species;
    uint64_t step;
};

struct SortArgs {
    const uint32_t *x, *z;
    const float *vx, *vy, *vz;
    const uint32_t* id;
    uint32_t *ox, *oz;
    float *ovx, *ovy, *ovz;
    uint32_t* oid;
    int64_t n;
    int nx, nz;
    int si, sj, nzk;         // sort key of cell (i, j): (i >> si) * nzk + (j >> sj)
    long long ncells;        // number of keys: ((nx-2 >> si) + 1) * nzk
    uint32_t* count;         // ncells, zero on entry and on exit
    uint32_t* offset;        // ncells + 1
    uint32_t* blocksum;      // ceil(ncells/1024)
    Counters* cnt;
};

// Source box particles of one species (use_source): positions in the box
// [0, bx) x [0, bz) (FP64), velocities FP32, and per particle the copies of a
// step (count, records of x, z, vx, vy, vz relative to the domain origin).
constexpr int kMaxInject = 4;
struct SourceArgs {
    double* x;
    double* z;
    float* vx;
    float* vy;
    float* vz;
    int64_t n;
    int* count;
    double* rec;
    unsigned long long* dropped;
    Counters* cnt;
    double bx, bz, lx, lz, dt;
    float hq, ez, tx, ty, tz, sx, sy, sz, prob;
    int coll, factor;
    uint32_t species;
    uint64_t seed, step;
};
// where the copies of a step go: the species' arrays from slot base on
struct SourceAppend {
    uint32_t* x;
    uint32_t* z;
    float* vx;
    float* vy;
    float* vz;
    uint32_t* id;
    unsigned long long* rho;  // deposit (self-consistent runs) or null
    int64_t base;
    uint32_t next_id;
    int nx, nz;
    double dx, dz;
};

// Box and cell sizes for converting physical positions to fixed point.
struct SetParticlesGeom {
    double x0, xmax, z0, zmax, dx, dz;
};
// FP64 particle columns x, z, vx, vy, vz as the kernel reads them: a device
// staging copy, or the caller's page-locked host arrays read in place
struct ParticleColumns {
    const double* v[5];
};

// Steps of one fused particle launch: their number and the RF factor of each
// (rf_amplitude cos(...) + rf_U0 at the species' step counter + k).
constexpr int kMaxFusedSteps = 64;
struct FusedSteps {
    float phase[kMaxFusedSteps];
    int nsteps;
    int pad;
};

// Direct solve with the precomputed inverse G (nn x nn, column-major by
// right-hand-side node); u_vac (nullable) is the stored potential of the
// Dirichlet values of the solve's voltages; list_j and list_b hold nn entries
// (the compacted right-hand side, tile by tile of 1024 nodes), tile_count one
// per tile, part nchunks * nn.
constexpr int kGreenMaxChunks = 32;
constexpr int kGreenMaxTiles = (int)((kSingleBlockNodes + 1023) / 1024);
struct GreenArgs {
    const double* G;
    const double* u_vac;
    int* tile_count;
    int* list_j;
    double* list_b;
    double* part;
    int nchunks;
    // rows != null: compute only the free nodes within two nodes of a charged
    // one (rows / row_count in the list's tile layout, charged: one byte per node)
    int* rows;
    int* row_count;
    uint8_t* charged;
};

struct SolveStatus {
    int iterations;
    int converged;
    double residual;
    int aborted;
    int pad;
};

// Device status of an instance gathered by one kernel into page-locked host
// memory: the error flag, the last solve's status and every species' counters
struct StatusSources {
    const int* err;
    const SolveStatus* st;
    const Counters* cnt[kMaxSpecies];
    int nsp;
    const double* energy;  // optional: sum of v^2 and (as bits) the live count
};
struct StatusHost {
    int err;
    int pad;
    SolveStatus st;
    Counters c[kMaxSpecies];
    double sum_v2;
    unsigned long long n_live;
};

// ---- the 3D Cartesian path ------------------------------------------------
constexpr int kDeposit3Bits = 14;  // 3D CIC weights quantised to 2^-14 per axis (2^42 per particle)

struct Push3Args {
    uint32_t* x;
    uint32_t* y;
    uint32_t* z;
    float* vx;
    float* vy;
    float* vz;
    uint32_t* id;
    int64_t n;
    int nx, ny, nz;
    uint32_t xmaxf, ymaxf, zmaxf;
    int periodic, init, has_b;
    const uint8_t* cellfree;  // (nx-1)(ny-1)(nz-1): the cell has a FREE corner
    const float* Exf;         // (nx+1) ny nz
    const float* Eyf;         // nx (ny+1) nz
    const float* Ezf;         // nx ny (nz+1)
    float hq, tx, ty, tz, sx, sy, sz;
    float cx, cy, cz;         // dt / dx, dt / dy, dt / dz
    unsigned long long* rho;  // deposit (self-consistent runs) or null
    uint32_t coll_threshold;
    uint32_t species;
    uint64_t seed, step;
    uint32_t* cand;
    float4* cand_rec;
    Counters* cnt;
    int slot, fold_slot;
};

struct Set3Geom {
    double xmax, ymax, zmax, dx, dy, dz;
};

struct Solve3Args {
    int nx, ny, nz, nsp;
    const int8_t* mask;  // nonzero: fixed (Dirichlet) node
    const double* voltage;
    double *u, *b, *r, *p, *qv, *part;
    const unsigned long long* rho_fixed[kMaxSpecies];
    double rho_weight[kMaxSpecies];  // charge * 2^-42
    const double* rho64;             // charge density [C/m^3] instead of the deposits, or null
    double rho_scale;                // macroparticle_factor / (dV eps0), or 1 / eps0 with rho64
    double ix2, iy2, iz2;            // 1 / h^2 per axis
    double tol;
    int max_iter, clear_rho;
    unsigned* bar;
    int* err;
    SolveStatus* status;
};

// State of the grid barrier of a cooperative solve (zeroed before each
// launch): the monotonic arrival counter and the abort flag a block sets when
// its bounded wait gives up.
struct GridBarrier {
    unsigned int count;
    unsigned int abort;
    unsigned int pad[2];
};

// Magic numbers of an unsigned division by a divisor fixed for a whole pass
// (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994, figure 4.1): n / d = (t + ((n - t) >> 1)) >> (l - 1)
// with t = umulhi(m, n), exact for every 32-bit n.  Setting them up takes a
// 64-bit division, so the host does it once per level.
struct DivMagic {
    unsigned d, m;
    int l;
};
__host__ __device__ inline DivMagic div_magic(unsigned d)
{
    DivMagic r{d, 0u, 0};
    if (d > 1) {
        int l = 0;
        while (l < 32 && (1ull << l) < d) ++l;  // ceil(log2 d)
        r.l = l;
        r.m = (unsigned)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    }
    return r;
}

struct MGLevelDev {
    int nx, nz;
    DivMagic dz, dhz;       // divisions by nz and by (nz + 1) / 2
    float* e;               // correction
    float* r;               // right-hand side of the correction equation
    float* t;               // residual scratch
    const float* coef;      // 9 planes of nx*nz (levels >= 1), plane k = (di+1)*3 + (dj+1)
    const float* inv_diag;  // levels >= 1
    int ti, tj;             // multi-block solves: interior size of this level's tiles (0: not tiled)
    // divisions of a tile's loops, for the interior tiles [0] and the last
    // column of tiles [1]: by the region width, by its half, by the interior width
    DivMagic tw[2], th[2], tn[2];
    int staged;             // Galerkin levels of a tiled solve: 1 = tiles stage the operator in shared memory,
                            // 0 = the passes read it from global memory (larger tiles)
    int cmode;              // coarsening to the next level: 0 both directions, 1 x only, 2 z only
};

struct SolveArgs {
    int coord;              // 0 Cartesian, 1 cylindrical
    int nx, nz;
    double dx, dz;
    const int8_t* mask;
    const double* voltage;
    double* u;              // FP64 solution (in/out, warm start)
    double* b;              // FP64 right-hand side (scratch)
    int rf_solve;           // boundary_solve_rf: FIXED -> 0, FIXED_RF -> voltage
    int rho_src;            // 0 none, 1 fixed-point species accumulators, 2 FP64 array, 3 unit right-hand side
    double* u_prev;         // non-null: start from u <- 2 u - u_prev on the free nodes (u_prev <- u) ...
    int* u_prev_valid;      // ... once *u_prev_valid is set (the first solve only records u_prev and sets it)
    long long unit_node;    // rho_src 3: b = 1 at this node, 0 elsewhere (columns of the inverse)
    const unsigned long long* rho_fixed[kMaxSpecies];
    double rho_weight[kMaxSpecies];  // charge * 2^-40
    int nsp;
    const double* rho64;
    int clear_rho;
    double mpf, dV;         // macroparticle_factor, cell volume (Cartesian scaling)
    const double* st64;     // fine stencil per row i: (w, e, c, 1/c), FP64 (4 * nx)
    const double* rscale;   // right-hand-side scaling of rho per row i (nx), or null: computed per node
    double idx, idz;        // 1 / dx, 1 / dz
    const float* st32;      // the same in FP32 for the smoother
    double k2;              // s/n coefficient of the fine stencil
    int nlev;
    int l_single;           // multi-block solves: first level run by block 0 alone (0: none)
    int tiled;              // multi-block solves: levels above l_single run as tile phases (dynamic shared memory)
    int coarse_staged;      // tiled solves: block 0 runs the levels from l_single down in shared memory
    const float* coarse_inv;  // dense inverse of the coarsest level, column-major (null: smooth it)
    const float* coarse_inv_rows;  // multi-block solves: the same inverse row-major, applied by every block
    int coarse_grid;          // 1: the coarsest level is l_single and all blocks solve it with coarse_inv_rows
    MGLevelDev lev[kMaxLevels];
    int nu1, nu2, ncoarse;
    float omega;            // SOR factor for the one-level smoother
    double tol;
    int max_outer;
    float* Exf;             // faces of -grad u (may be null)
    float* Ezf;
    double* red;            // reduction scratch (8 doubles: FP64 residual passes, then updated residuals)
    GridBarrier* bar;
    SolveStatus* status;
    int* err;
    double* prof;           // phase times of the solve [ns] (kSolvePhases slots), or null
};

// FP64 multigrid levels (the all-FP64 solver option): the same hierarchy and
// Galerkin operators as the FP32 levels, every array in FP64
struct MG64Level {
    int nx, nz, cmode;
    double *e, *r, *t;
    const double* coef;      // 9 planes (levels >= 1)
    const double* inv_diag;  // levels >= 1
};
struct MG64Args {
    MG64Level lev[kMaxLevels];
    const double* coarse_inv;  // dense inverse of the coarsest level, column-major (null: smooth it)
};

// bytes of the argument copy in front of block 0's staged coarse levels (16-byte aligned)
constexpr size_t kStagedArgsBytes = (sizeof(SolveArgs) + 15) & ~(size_t)15;

// Adjoint of one particle step (or of the leapfrog start) for every particle
// of a species: the state before the step, the removal marker after it, and
// the adjoints of the state after the step, overwritten with those before it.
// Positions in cells, velocities in m/s.
struct AdjPushArgs {
    const uint32_t *x0, *z0;
    const float *vx0, *vy0, *vz0;
    const uint32_t* x1;     // state after the step (kDead: removed during it); null for the start
    int64_t n;
    float *lr, *lz, *lvx, *lvy, *lvz;
    float* lExf;            // adjoints of the face fields of this step, accumulated
    float* lEzf;
    double* lB;             // d loss / d(Br, Bt, Bz), accumulated
    int init;               // 1: the leapfrog start (backward half rotation and half kick, no move)
};

}  // namespace mag
