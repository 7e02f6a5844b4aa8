// Host-callable launchers of the sm_103a kernels.  Each returns the number of
// kernel launches it issued on the given stream.
#pragma once
#include <cuda_runtime.h>

#include "device.hpp"

namespace mag {

// particle step (init: leapfrog start).  vec = slots per thread (1, 2 or 4);
// sm_count = multiprocessors of the device (sizes the persistent grid)
int launch_push(const PushArgs& a, int coord, bool init, int vec, int sm_count, cudaStream_t s);
// batched particle step: nitems work items (one species of one instance each)
// with the same coord / field mode / B flag; d_chunk_off = first chunk of each
// item (nitems + 1 entries), chunks of push_batch_chunk(vec) slots
int push_batch_chunk(int vec);
// adjoint of the particle step (or of the leapfrog start) of one species;
// field mode 1 (potential faces) or 0 (uniform field)
int launch_adj_push(const PushArgs& a, const AdjPushArgs& d, int coord, cudaStream_t s);
// adjoint helpers of the self-consistent step (adjoint_kernels.cu)
int launch_adj_faces(int nx, int nz, double dx, double dz, const float* lExf, const float* lEzf, double* g,
                     cudaStream_t s);
int launch_adj_rhs(int nx, int nz, const int8_t* mask, const double* g, const double* w_scale, double* rho,
                   cudaStream_t s);
int launch_adj_post(int nx, int nz, const int8_t* mask, const double* x, const double* w, const double* scale,
                    double* y, double* lrho, cudaStream_t s);
int launch_adj_dirichlet(int nx, int nz, const int8_t* mask, const double* g, const double* y, const double* st64,
                         double k2, const double* basis, int nparam, double* grad, cudaStream_t s);
int launch_adj_deposit(const uint32_t* x, const uint32_t* z, int64_t n, int nx, int nz, const double* lrho,
                       double charge, float* lr, float* lz, cudaStream_t s);
int launch_adj_loss(const uint32_t* x, const float* vz, int64_t n, double half_m_eV, double* out_e,
                    unsigned long long* out_n, cudaStream_t s);
int launch_adj_seed(const uint32_t* x, const float* vz, int64_t n, double coef, float* lr, float* lz, float* lvx,
                    float* lvy, float* lvz, cudaStream_t s);
int launch_push_batch(const PushArgs* d_args, const unsigned* d_chunk_off, int nitems, int coord, int emode,
                      bool has_b, int vec, int sm_count, cudaStream_t s);
// fs.nsteps steps of one species in one launch (k_push_fused); c supplies the
// species' collision data when its collision test is on
int launch_push_fused(const PushArgs& a, const CollideArgs& c, const FusedSteps& fs, int coord, int sm_count,
                      cudaStream_t s);
// particle source (use_source): box refresh, a step of the box particles with
// the scan of their copies (offs, total), and the append of the copies
int launch_source_refresh(const SourceArgs& a, float vsig, cudaStream_t s);
int launch_source_step(const SourceArgs& a, const CollideArgs& c, int* offs, long long* total, cudaStream_t s);
int launch_source_append(const SourceArgs& a, const int* offs, const SourceAppend& t, cudaStream_t s);
// the 3D Cartesian path
int launch_push3d(const Push3Args& a, int sm_count, cudaStream_t s);
int launch_deposit3d(const Push3Args& a, cudaStream_t s);
int launch_faces3d(const double* u, int nx, int ny, int nz, double dx, double dy, double dz, float* Exf, float* Eyf,
                   float* Ezf, cudaStream_t s);
int launch_set_particles3d(const double* staged, int64_t n, const Set3Geom& g, uint32_t* x, uint32_t* y, uint32_t* z,
                           float* vx, float* vy, float* vz, uint32_t* id, cudaStream_t s);
int solve3d_blocks(int sm_count);
int launch_solve3d(const Solve3Args& a, int nblocks, cudaStream_t s);
int launch_deposit(const PushArgs& a, cudaStream_t s);
int launch_collide(const CollideArgs& a, int grid, cudaStream_t s);
// ADVANCE_MULTICOLL step of one species (multicoll.cu); ttd = time to the next
// collision per slot (FP64); qm = charge / mass
int launch_multicoll(const PushArgs& a, const CollideArgs& c, double* ttd, double dt, double lifetime, double qm,
                     cudaStream_t s);
int launch_init_ttd(double* ttd, const uint32_t* id, int64_t first, int64_t n, double lifetime, uint64_t seed,
                    uint32_t species, uint64_t step, cudaStream_t s);
// candidate lists of nitems work items (one block each); max_tables = the
// largest cross-section table size among them (shared-memory staging)
int launch_collide_batch(const CollideArgs* d_args, int nitems, int max_tables, cudaStream_t s);
// counting sort by cell with compaction; n_src = slots of the source arrays
int launch_sort(const SortArgs& a, long long n_src, cudaStream_t s);
// whole FP64-refined multigrid solve in one kernel; nblocks > 1 uses a
// cooperative launch with a bounded grid barrier, smem bytes of dynamic
// shared memory per block for the tile phases (a.tiled)
int launch_solve(const SolveArgs& a, int nblocks, cudaStream_t s, size_t smem = 0);
// blocks of 1024 threads a cooperative launch of the solve can have with smem
// bytes of dynamic shared memory (1 when the device cannot launch cooperatively)
int solve_max_blocks(int sm_count, size_t smem = 0);
// n independent single-block solves, arguments in device memory (one block of
// 'threads' threads each; grids up to kSingleBlockNodes nodes)
int launch_solve_batch(const SolveArgs* d_args, int n, int threads, cudaStream_t s);
// the all-FP64 multigrid solve of one grid of at most kSingleBlockNodes nodes (one block)
int launch_solve64(const SolveArgs& a, const MG64Args& g, cudaStream_t s);
int launch_faces(const double* u, int nx, int nz, double dx, double dz, float* Exf, float* Ezf, cudaStream_t s);
// Fields::u_smooth(): u = the smoothing of t, a copy of u (nx*nz each)
int launch_u_smooth(const double* t, double* u, int nx, int nz, cudaStream_t s);
// direct solve u = G b' with the precomputed inverse G (nn x nn, column j =
// response to a unit right-hand side at node j); bprime (nn) and part
// (nchunks x nn) are scratch; writes the faces when a.Exf is set
int green_chunks(long long nn, int sm_count);
// Direct solve with the precomputed inverse (GreenArgs).
int launch_green_solve(const SolveArgs& a, const GreenArgs& g, cudaStream_t s);
// the product (and sum) of the last right-hand side again, every node or the
// rows of g (the solve's list must be unchanged since)
int launch_green_product(const SolveArgs& a, const GreenArgs& g, bool partial, cudaStream_t s);
int launch_load_disk(uint32_t* x, uint32_t* z, float* vx, float* vy, float* vz, uint32_t* id, int64_t n,
                     uint32_t id0, int kind, double cx, double cz, double radius, double zlo, double zhi,
                     double x0, double z0, double dx, double dz, double xmax, double zmax, double vsig,
                     uint64_t seed, uint32_t species, int coord, cudaStream_t s);
int launch_interleave(const float* a, const float* b, float2* out, long long n, cudaStream_t s);
int launch_fill_u32(uint32_t* p, uint32_t v0, int64_t n, cudaStream_t s);
// staged = x, z, vx, vy, vz of n particles (FP64, one array after the other)
int launch_set_particles(const ParticleColumns& staged, int64_t n, const SetParticlesGeom& g, uint32_t* x, uint32_t* z,
                         float* vx, float* vy, float* vz, uint32_t* id, cudaStream_t s);
// error flag, solve status and counters into out (device address of
// page-locked host memory)
int launch_gather_status(const StatusSources& src, StatusHost* out, cudaStream_t s);
// the records of the live particles whose ids are want[0..nwant) (tracked particles)
int launch_find_ids(const uint32_t* id, const uint32_t* x, const uint32_t* z, const float* vx, const float* vy,
                    const float* vz, int64_t n, const uint32_t* want, int nwant, uint32_t* rec, cudaStream_t s);
int launch_energy(const uint32_t* x, const float* vx, const float* vy, const float* vz, int64_t n,
                  double* out_sum_v2, unsigned long long* out_n, cudaStream_t s);
// energy histogram of the live particles (Histogram::add), bins += counts,
// stats += (n_val, sum, n_val_tot, sum_tot)
int launch_energy_hist(const uint32_t* x, const float* vx, const float* vy, const float* vz, int64_t n, double mass,
                       double qe, double emin, double emax, int nbins, unsigned long long* bins, double* stats,
                       cudaStream_t s);
int launch_axpy_i64(double* acc, const unsigned long long* src, double w, long long n, cudaStream_t s);
int launch_axpy_f64(double* acc, const double* src, double w, long long n, cudaStream_t s);

}  // namespace mag
