// Null-collision Monte Carlo collisions of the particles that the particle
// kernel listed as candidates (BaseSpecies::scatter, src/particles.cpp:208-365):
// the target species by the null-collision rates, the partner velocity from a
// Maxwellian background (rndv, src/particles.hpp:188-192) or from a random
// live particle of the target species (random_particle, :207-217; COULOMB
// also updates the partner), the interaction by sigma_v * density, and the
// velocity update of its type.  Arithmetic is FP32 (see mcc_device.cuh).
//
// The last block to finish closes the step of the species: it moves the live
// count into the running totals, clears the candidate counter and advances
// the species step counter (Species::advance niter++, src/particles.hpp:347).
#include "device.hpp"
#include "kernels.hpp"
#include "mcc_device.cuh"

namespace mag {

namespace {

__global__ void __launch_bounds__(128) k_collide(const CollideArgs a)
{
    __shared__ unsigned long long s_coll, s_null, s_miss;
    if (threadIdx.x == 0) {
        s_coll = 0;
        s_null = 0;
        s_miss = 0;
    }
    __syncthreads();
    const MccSpecies& m = *a.mcc;
    const unsigned long long ncand = *((volatile unsigned long long*)&a.cnt->ncand);
    const uint64_t step = a.step;
    for (unsigned long long c = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncand;
         c += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t p = a.cand[c];
        const uint32_t pid = a.id[p];
        Stream rs(a.seed, a.species, pid, TAG_COLLIDE, step);
        float vx = a.vx[p], vy = a.vy[p], vz = a.vz[p];
        const int s = mcc_pick_target(m, rs);
        float vr2, vz2, vt2;
        int partner = -1;
        if (!a.t_has_slots[s]) {
            const float sig = (float)m.t_sigma_v[s];
            vr2 = rs.normalf() * sig;
            vz2 = rs.normalf() * sig;
            vt2 = rs.normalf() * sig;
        } else {
            Stream ps(a.seed, a.species, pid, TAG_PARTNER, step);
            const int64_t nt = a.t_n[s];
            for (int tries = 0; tries < 256 && nt > 0; ++tries) {
                const uint64_t hi = ps.next();
                const int64_t q = (int64_t)(((hi << 32) | ps.next()) % (uint64_t)nt);
                if (a.t_x[s][q] != kDead) {  // any live particle, itself included (random_particle)
                    partner = (int)q;
                    break;
                }
            }
            if (partner < 0) {
                atomicAdd(&s_miss, 1ull);
                continue;
            }
            vr2 = a.t_vx[s][partner];
            vz2 = a.t_vz[s][partner];
            vt2 = a.t_vy[s][partner];
        }
        bool pu;
        float pvx, pvy, pvz;
        const int r = mcc_collide(m, s, rs, vx, vy, vz, vr2, vz2, vt2, pu, pvx, pvy, pvz);
        if (r != MCC_HIT) {
            atomicAdd(&s_null, 1ull);
            continue;
        }
        a.vx[p] = vx;
        a.vy[p] = vy;
        a.vz[p] = vz;
        if (pu && partner >= 0) {
            a.t_vx[s][partner] = pvx;
            a.t_vy[s][partner] = pvy;
            a.t_vz[s][partner] = pvz;
        }
        atomicAdd(&s_coll, 1ull);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_coll) atomicAdd(&a.cnt->ncoll, s_coll);
        if (s_null) atomicAdd(&a.cnt->nnull, s_null);
        if (s_miss) atomicAdd(&a.cnt->partner_miss, s_miss);
        __threadfence();
        const unsigned long long ticket = atomicAdd(&a.cnt->done_blocks, 1ull);
        if (ticket == gridDim.x - 1) {
            __threadfence();
            Counters* c = a.cnt;
            const unsigned long long live = *((volatile unsigned long long*)&c->live_step);
            c->live_last = live;
            c->live_sum += live;
            c->live_step = 0;
            c->ncand = 0;
            c->done_blocks = 0;
            c->niter += 1;
            __threadfence();
        }
    }
}

}  // namespace

int launch_collide(const CollideArgs& a, int grid, cudaStream_t s)
{
    k_collide<<<grid < 1 ? 1 : grid, 128, 0, s>>>(a);
    return 1;
}

}  // namespace mag
