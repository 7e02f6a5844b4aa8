// Counting sort of a species' particles by cell every sort_interval steps,
// with compaction of removed particles.  After a sort, consecutive threads of the particle kernel touch the
// same few cells, so the field gather and the deposit atomics hit L1/L2
// instead of scattering over the grid.  The order inside a cell is not
// deterministic; nothing depends on it (random streams are keyed by particle
// id, the deposit is an integer sum).
//
//   k_cell_count   count[cell] += 1 per live particle
//   k_scan_*       offset = exclusive prefix sum of count (3-phase block scan)
//   k_cell_scatter position = offset[cell] + (atomicSub(count[cell]) - 1);
//                  count returns to zero for the next sort
// Invariant kept for all other kernels: every slot below the host's slot
// count holds a live particle or the removed marker.
#include "device.hpp"
#include "kernels.hpp"

namespace mag {

namespace {

__device__ __forceinline__ int cell_of(uint32_t x, uint32_t z, int nx, int nz)
{
    const int i = min((int)(x >> kFracBits), nx - 2);
    const int j = min((int)(z >> kFracBits), nz - 2);
    return i * (nz - 1) + j;
}

// Runs of consecutive lanes with the same cell (c < 0: no particle): the
// lane's run head and, for a head, the run's length.  Particles sorted a few
// steps ago arrive in such runs; a cell that occurs in two runs of a warp is
// simply counted twice.
struct LaneRun {
    int head, len;
    bool is_head;
};
__device__ __forceinline__ LaneRun lane_run(int c, int lane)
{
    const int cprev = __shfl_up_sync(0xffffffffu, c, 1);
    const bool h = lane == 0 || cprev != c;
    const unsigned heads = __ballot_sync(0xffffffffu, h);
    const unsigned upto = lane == 31 ? 0xffffffffu : (2u << lane) - 1u;  // lanes <= lane
    const unsigned after = heads & ~upto;
    LaneRun r;
    r.head = 31 - __clz(heads & upto);
    r.len = (after ? __ffs(after) - 1 : 32) - lane;
    r.is_head = h;
    return r;
}

// Each run of a warp's particles in one cell adds to its counter once.
__global__ void k_cell_count(const SortArgs a)
{
    const long long n = a.n;
    const int lane = threadIdx.x & 31;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += (long long)gridDim.x * blockDim.x) {
        const long long k = base + threadIdx.x;
        const uint32_t x = k < n ? a.x[k] : kDead;
        const bool valid = x != kDead;
        const int c = valid ? cell_of(x, a.z[k], a.nx, a.nz) : -1;
        const LaneRun r = lane_run(c, lane);
        if (valid && r.is_head) atomicAdd(&a.count[c], (unsigned)r.len);
    }
}

// exclusive scan of one 1024-element chunk per block; returns the block total
__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t& excl)
{
    __shared__ uint32_t warp_tot[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint32_t t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0u;
        uint32_t ti = t;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, ti, o);
            if (lane >= o) ti += u;
        }
        warp_tot[lane] = ti - t;  // exclusive warp offsets
    }
    __syncthreads();
    excl = warp_tot[w] + inc - v;
    // block total = last thread's inclusive value
    __shared__ uint32_t total;
    if (threadIdx.x == blockDim.x - 1) total = excl + v;
    __syncthreads();
    const uint32_t t = total;
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(1024) k_scan_local(const SortArgs a)
{
    const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
    const uint32_t v = i < a.ncells ? a.count[i] : 0u;
    uint32_t excl;
    const uint32_t tot = block_exclusive_scan(v, excl);
    if (i < a.ncells) a.offset[i] = excl;
    if (threadIdx.x == 0) a.blocksum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_top(const SortArgs a, int nblocks)
{
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nblocks; base += 1024) {
        const int i = base + threadIdx.x;
        const uint32_t v = i < nblocks ? a.blocksum[i] : 0u;
        uint32_t excl;
        const uint32_t tot = block_exclusive_scan(v, excl);
        if (i < nblocks) a.blocksum[i] = excl + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.offset[a.ncells] = carry;
        a.cnt->slots = carry;
    }
}

__global__ void __launch_bounds__(1024) k_scan_add(const SortArgs a)
{
    const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
    if (i < a.ncells) a.offset[i] += a.blocksum[blockIdx.x];
}

// Every slot k >= total of the destination is marked removed, so all slots
// below the host's slot count are either live or removed in both buffers.
// Each thread moves SP particles per pass: all their loads and all their
// counter atomics are issued before any result is used, so the atomic round
// trips overlap.
constexpr int SP = 2;
__global__ void __launch_bounds__(256) k_cell_scatter(const SortArgs a, long long n_src)
{
    const long long total = __ldg(&a.offset[a.ncells]);
    const int lane = threadIdx.x & 31;
    const long long span = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n_src; base += SP * span) {
        uint32_t x[SP], z[SP], id[SP];
        float vx[SP], vy[SP], vz[SP];
        long long k[SP];
        int c[SP];
        LaneRun run[SP];
        uint32_t old[SP];
#pragma unroll
        for (int q = 0; q < SP; ++q) {
            k[q] = base + q * span + threadIdx.x;
            const bool in = k[q] < n_src;
            if (in && k[q] >= total) a.ox[k[q]] = kDead;
            x[q] = in ? a.x[k[q]] : kDead;
            z[q] = in ? a.z[k[q]] : 0u;
            vx[q] = in ? a.vx[k[q]] : 0.f;
            vy[q] = in ? a.vy[k[q]] : 0.f;
            vz[q] = in ? a.vz[k[q]] : 0.f;
            id[q] = in ? a.id[k[q]] : 0u;
        }
#pragma unroll
        for (int q = 0; q < SP; ++q) {
            // one atomic per run of equal cells in the warp; lanes take the slots below the old count
            const bool valid = x[q] != kDead;
            c[q] = valid ? cell_of(x[q], z[q], a.nx, a.nz) : -1;
            run[q] = lane_run(c[q], lane);
            old[q] = 0;
            if (valid && run[q].is_head) old[q] = atomicSub(&a.count[c[q]], (unsigned)run[q].len);
        }
#pragma unroll
        for (int q = 0; q < SP; ++q) {
            const uint32_t o = __shfl_sync(0xffffffffu, old[q], run[q].head);
            if (x[q] == kDead) continue;
            const uint32_t rank = (uint32_t)(lane - run[q].head);
            const uint32_t pos = __ldg(&a.offset[c[q]]) + o - 1u - rank;
            a.ox[pos] = x[q];
            a.oz[pos] = z[q];
            a.ovx[pos] = vx[q];
            a.ovy[pos] = vy[q];
            a.ovz[pos] = vz[q];
            a.oid[pos] = id[q];
        }
    }
}

}  // namespace

int launch_sort(const SortArgs& a, long long n_src, cudaStream_t s)
{
    if (a.n == 0) return 0;
    const int grid = (int)std::min<long long>((a.n + 255) / 256, 152 * 16);
    k_cell_count<<<grid, 256, 0, s>>>(a);
    const int nb = (int)((a.ncells + 1023) / 1024);
    k_scan_local<<<nb, 1024, 0, s>>>(a);
    k_scan_top<<<1, 1024, 0, s>>>(a, nb);
    k_scan_add<<<nb, 1024, 0, s>>>(a);
    k_cell_scatter<<<(int)std::min<long long>((n_src + 2 * 256 - 1) / (2 * 256), 152 * 8), 256, 0, s>>>(a, n_src);
    return 5;
}

}  // namespace mag
