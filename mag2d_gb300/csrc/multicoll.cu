// Event-driven mover ADVANCE_MULTICOLL (Species<CARTESIAN>::advance_multicoll,
// src/particles.cpp:812-859) followed by advance_boundary: every particle
// flies freely in the constant external field until its time to the next
// collision, is scattered there (BaseSpecies::scatter, null collisions
// included) and draws a new exponential time lifetime * rexp, until the step
// dt is used up; the rest of the step is a free flight.  The time to the next
// collision is kept per particle in FP64, as in the reference.  The reference
// requires zero B, a constant external field (selfconsistent = 0, geometry
// EMPTY) and Cartesian coordinates; so does this kernel.
#include <algorithm>

#include "device.hpp"
#include "kernels.hpp"
#include "mcc_device.cuh"

namespace mag {

namespace {

constexpr int kMaxEventsPerStep = 1 << 20;  // bound of the event loop of one particle in one step

__device__ __forceinline__ bool move_fixed(uint32_t& x, double cells, uint32_t maxf, bool periodic)
{
    const double one = (double)(1u << kFracBits);
    const double v = fmin(fmax(cells * one, -1.0e9), 1.0e9);
    const long long d = __double2ll_rn(v);
    const long long p = (long long)x + d;
    if (p >= 0 && p <= (long long)maxf) {
        x = (uint32_t)p;
        return true;
    }
    if (!periodic || maxf == 0) return false;
    long long q = p % (long long)maxf;
    if (q < 0) q += maxf;
    x = (uint32_t)q;
    return true;
}

// a = push arguments of the step (field mode 0: E = (0, extern_ez)); c = the
// species' collision arguments with every target a background (no partners)
__global__ void __launch_bounds__(128) k_multicoll(const __grid_constant__ PushArgs a,
                                                   const __grid_constant__ CollideArgs c, double* __restrict__ ttd,
                                                   double dt, double lifetime, double qm)
{
    __shared__ MccStage st;
    extern __shared__ double s_tab[];
    double* tab = c.n_tables <= kStageTables ? s_tab : nullptr;
    mcc_stage(c, st, tab);
    __syncthreads();
    if (threadIdx.x == 0) mcc_stage_pointers(c, st, tab);
    __syncthreads();
    const double ax = 0.0, az = (double)a.extern_ez * qm;  // Fields::E of the EMPTY geometry
    unsigned live = 0, removed = 0, ncoll = 0, nnull = 0;
    bool overflow = false;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < a.n; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t x = a.x[k];
        if (x == kDead) continue;
        uint32_t z = a.z[k];
        const uint32_t id = a.id[k];
        double vx = a.vx[k], vy = a.vy[k], vz = a.vz[k];
        double t = ttd[k], local = 0.0, dxm = 0.0, dzm = 0.0;
        Stream rs(a.seed, a.species, id, TAG_MULTICOLL, a.step);
        int events = 0;
        while (local + t < dt) {
            if (++events > kMaxEventsPerStep) {
                overflow = true;
                break;
            }
            vx += ax * t;
            vz += az * t;
            dxm += (vx + 0.5 * ax * t) * t;
            dzm += (vz + 0.5 * az * t) * t;
            local += t;
            float fvx = (float)vx, fvy = (float)vy, fvz = (float)vz;
            const int r = scatter_background(st.m, rs, fvx, fvy, fvz);
            if (r == MCC_HIT) {
                vx = fvx;
                vy = fvy;
                vz = fvz;
                ++ncoll;
            } else {
                ++nnull;
            }
            t = lifetime * -log(rs.uni());  // rexp
        }
        const double rem = dt - local;
        vx += ax * rem;
        vz += az * rem;
        dxm += (vx + 0.5 * ax * rem) * rem;
        dzm += (vz + 0.5 * az * rem) * rem;
        t -= rem;
        // advance_boundary (src/particles.hpp:370-411) on the step's total displacement
        bool alive = move_fixed(x, dxm / a.gdx, a.xmaxf, a.periodic) && move_fixed(z, dzm / a.gdz, a.zmaxf, a.periodic);
        if (alive && a.check_mask) {
            const int ic = min((int)(x >> kFracBits), a.nx - 2), jc = min((int)(z >> kFracBits), a.nz - 2);
            alive = a.cellfree[(size_t)ic * (a.nz - 1) + jc] != 0;
        }
        a.x[k] = alive ? x : kDead;
        a.z[k] = z;
        a.vx[k] = (float)vx;
        a.vy[k] = (float)vy;
        a.vz[k] = (float)vz;
        ttd[k] = t;
        live += alive;
        removed += !alive;
    }
    const unsigned full = 0xffffffffu;
    live = __reduce_add_sync(full, live);
    removed = __reduce_add_sync(full, removed);
    ncoll = __reduce_add_sync(full, ncoll);
    nnull = __reduce_add_sync(full, nnull);
    if ((threadIdx.x & 31) == 0) {
        if (live) atomicAdd(&a.cnt->live_par[a.slot], (unsigned long long)live);
        if (removed) atomicAdd(&a.cnt->removed, (unsigned long long)removed);
        if (ncoll) atomicAdd(&a.cnt->ncoll, (unsigned long long)ncoll);
        if (nnull) atomicAdd(&a.cnt->nnull, (unsigned long long)nnull);
    }
    if (overflow) atomicCAS(&a.cnt->error, 0, -5);
    if (a.fold_slot >= 0 && blockIdx.x == 0 && threadIdx.x == 0) {
        // fold the previous launch's counts (no other block touches that slot)
        Counters* cn = a.cnt;
        cn->live_sum += cn->live_par[a.fold_slot];
        cn->live_par[a.fold_slot] = 0;
        cn->ncand_par[a.fold_slot] = 0;
    }
}

// time to the first collision of particles [first, first + n): lifetime * rexp
__global__ void k_init_ttd(double* ttd, const uint32_t* id, int64_t first, int64_t n, double lifetime, uint64_t seed,
                           uint32_t species, uint64_t step)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        Stream rs(seed, species, id[first + k], TAG_TTD, step);
        ttd[first + k] = lifetime * -log(rs.uni());
    }
}

}  // namespace

int launch_multicoll(const PushArgs& a, const CollideArgs& c, double* ttd, double dt, double lifetime, double qm,
                     cudaStream_t s)
{
    if (a.n == 0) return 0;
    const size_t smem = c.n_tables <= kStageTables ? (size_t)c.n_tables * sizeof(double) : 0;
    const unsigned grid = (unsigned)std::min<int64_t>((a.n + 127) / 128, 152 * 8);
    k_multicoll<<<grid, 128, smem, s>>>(a, c, ttd, dt, lifetime, qm);
    return 1;
}

int launch_init_ttd(double* ttd, const uint32_t* id, int64_t first, int64_t n, double lifetime, uint64_t seed,
                    uint32_t species, uint64_t step, cudaStream_t s)
{
    if (n <= 0) return 0;
    k_init_ttd<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 8), 256, 0, s>>>(ttd, id, first, n, lifetime,
                                                                                    seed, species, step);
    return 1;
}

}  // namespace mag
