// Null-collision Monte Carlo collisions of the particles that the particle
// kernel listed as candidates (BaseSpecies::scatter, src/particles.cpp:208-365):
// the target species by the null-collision rates, the partner velocity from a
// Maxwellian background (rndv, src/particles.hpp:188-192) or from a random
// live particle of the target species (random_particle, :207-217; COULOMB
// also updates the partner), the interaction by sigma_v * density, and the
// velocity update of its type.  Arithmetic is FP32 (see mcc_device.cuh).
//
// Counters of collisions, null collisions and partner misses are added per
// block; the candidate count of the step is folded by the next particle kernel.
#include "device.hpp"
#include "kernels.hpp"
#include "mcc_device.cuh"

namespace mag {

namespace {

// Launched with programmatic stream serialisation after the particle kernel:
// the species' collision data are staged in shared memory while the particle
// kernel finishes, and griddepcontrol.wait orders every access to its results.
__global__ void __launch_bounds__(128) k_collide(const __grid_constant__ CollideArgs a)
{
    __shared__ unsigned long long s_cnt[3];
    __shared__ MccStage st;
    extern __shared__ double s_tab[];
    double* tab = a.n_tables <= kStageTables ? s_tab : nullptr;
    mcc_stage(a, st, tab);
    if (threadIdx.x < 3) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    if (threadIdx.x == 0) mcc_stage_pointers(a, st, tab);
    asm volatile("griddepcontrol.wait;" ::: "memory");
    __syncthreads();
    const unsigned long long ncand = __ldcg(&a.cnt->ncand_par[a.slot]);
    unsigned long long nc = 0, nn = 0, nm = 0;
    for (unsigned long long c = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncand;
         c += (unsigned long long)gridDim.x * blockDim.x) {
        const int r = collide_one(a, st.m, c);
        nc += r == MCC_HIT;
        nn += r == MCC_NULL;
        nm += r == MCC_NOPARTNER;
    }
    if (nc) atomicAdd(&s_cnt[0], nc);
    if (nn) atomicAdd(&s_cnt[1], nn);
    if (nm) atomicAdd(&s_cnt[2], nm);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_cnt[0]) atomicAdd(&a.cnt->ncoll, s_cnt[0]);
        if (s_cnt[1]) atomicAdd(&a.cnt->nnull, s_cnt[1]);
        if (s_cnt[2]) atomicAdd(&a.cnt->partner_miss, s_cnt[2]);
    }
}

// Collisions of many instances in one launch (batched runs): block b runs
// the candidate list of work item b (one colliding species of one instance).
__global__ void __launch_bounds__(128) k_collide_batch(const CollideArgs* __restrict__ args)
{
    __shared__ __align__(16) unsigned char raw[sizeof(CollideArgs)];
    __shared__ unsigned long long s_cnt[3];
    __shared__ MccStage st;
    extern __shared__ double s_tab[];
    static_assert(sizeof(CollideArgs) % 8 == 0, "word copy");
    {
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(args + blockIdx.x);
        unsigned long long* dst = reinterpret_cast<unsigned long long*>(raw);
        for (int w = threadIdx.x; w < (int)(sizeof(CollideArgs) / 8); w += blockDim.x) dst[w] = src[w];
    }
    if (threadIdx.x < 3) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    const CollideArgs& a = *reinterpret_cast<const CollideArgs*>(raw);
    double* tab = a.n_tables <= kStageTables ? s_tab : nullptr;
    mcc_stage(a, st, tab);
    __syncthreads();
    if (threadIdx.x == 0) mcc_stage_pointers(a, st, tab);
    __syncthreads();
    const unsigned long long ncand = __ldcg(&a.cnt->ncand_par[a.slot]);
    unsigned long long nc = 0, nn = 0, nm = 0;
    for (unsigned long long c = threadIdx.x; c < ncand; c += blockDim.x) {
        const int r = collide_one(a, st.m, c);
        nc += r == MCC_HIT;
        nn += r == MCC_NULL;
        nm += r == MCC_NOPARTNER;
    }
    if (nc) atomicAdd(&s_cnt[0], nc);
    if (nn) atomicAdd(&s_cnt[1], nn);
    if (nm) atomicAdd(&s_cnt[2], nm);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_cnt[0]) atomicAdd(&a.cnt->ncoll, s_cnt[0]);
        if (s_cnt[1]) atomicAdd(&a.cnt->nnull, s_cnt[1]);
        if (s_cnt[2]) atomicAdd(&a.cnt->partner_miss, s_cnt[2]);
    }
}

}  // namespace

int launch_collide_batch(const CollideArgs* d_args, int nitems, int max_tables, cudaStream_t s)
{
    if (nitems <= 0) return 0;
    const size_t smem = max_tables <= kStageTables ? (size_t)max_tables * sizeof(double) : 0;
    k_collide_batch<<<nitems, 128, smem, s>>>(d_args);
    return 1;
}

int launch_collide(const CollideArgs& a, int grid, cudaStream_t s)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(grid < 1 ? 1 : grid));
    cfg.blockDim = dim3(128);
    cfg.dynamicSmemBytes = a.n_tables <= kStageTables ? (size_t)a.n_tables * sizeof(double) : 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_collide, a);
    return 1;
}

}  // namespace mag
