// Host-callable launchers of the sm_103a kernels.  Each returns the number of
// kernel launches it issued on the given stream.
#pragma once
#include <cuda_runtime.h>

#include "device.hpp"

namespace mag {

// particle step (init: leapfrog start).  vec = slots per thread (1, 2 or 4);
// sm_count = multiprocessors of the device (sizes the persistent grid)
int launch_push(const PushArgs& a, int coord, bool init, int vec, int sm_count, cudaStream_t s);
int launch_deposit(const PushArgs& a, cudaStream_t s);
int launch_collide(const CollideArgs& a, int grid, cudaStream_t s);
// counting sort by cell with compaction; n_src = slots of the source arrays
int launch_sort(const SortArgs& a, long long n_src, cudaStream_t s);
// whole FP64-refined multigrid solve in one kernel; nblocks > 1 uses a
// cooperative launch with a bounded grid barrier
int launch_solve(const SolveArgs& a, int nblocks, cudaStream_t s);
// blocks of 1024 threads a cooperative launch of the solve can have (1 when
// the device cannot launch cooperatively)
int solve_max_blocks(int sm_count);
int launch_faces(const double* u, int nx, int nz, double dx, double dz, float* Exf, float* Ezf, cudaStream_t s);
int launch_load_disk(uint32_t* x, uint32_t* z, float* vx, float* vy, float* vz, uint32_t* id, int64_t n,
                     uint32_t id0, int kind, double cx, double cz, double radius, double zlo, double zhi,
                     double x0, double z0, double dx, double dz, double xmax, double zmax, double vsig,
                     uint64_t seed, uint32_t species, int coord, cudaStream_t s);
int launch_interleave(const float* a, const float* b, float2* out, long long n, cudaStream_t s);
int launch_fill_u32(uint32_t* p, uint32_t v0, int64_t n, cudaStream_t s);
int launch_energy(const uint32_t* x, const float* vx, const float* vy, const float* vz, int64_t n,
                  double* out_sum_v2, unsigned long long* out_n, cudaStream_t s);

}  // namespace mag
