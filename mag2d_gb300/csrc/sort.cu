// Counting sort of a species' particles by cell every sort_interval steps,
// with compaction of removed particles.  After a sort, consecutive threads of the particle kernel touch the
// same few cells, so the field gather and the deposit atomics hit L1/L2
// instead of scattering over the grid.  The order inside a cell is not
// deterministic; nothing depends on it (random streams are keyed by particle
// id, the deposit is an integer sum).
//
// One call sorts by a key of the cell: the cell index, or the index of a block
// of 2^si x 2^sj cells (the host sorts scrambled slots by coarse blocks first).
// Both passes of a call work on chunks of consecutive slots per block.  The
// slots were sorted a few steps ago (or by a coarser key), so a chunk holds a
// few hundred distinct keys; a shared-memory table of the chunk's keys turns
// the per-particle global atomics into one per (chunk, key), and the scatter
// stages the chunk in shared memory and writes it grouped by key, so each
// key's particles of the chunk leave as one contiguous run of stores.
//
//   k_cell_count   count[key] += particles of the chunk with the key
//   k_scan_*       offset = exclusive prefix sum of count (3-phase block scan)
//   k_cell_scatter each (chunk, key) reserves its run below the key's
//                  remaining count (atomicSub); count returns to zero for the
//                  next sort
// Invariant kept for all other kernels: every slot below the host's slot
// count holds a live particle or the removed marker.
#include <algorithm>

#include "bulk.cuh"
#include "device.hpp"
#include "kernels.hpp"

namespace mag {

namespace {

// sort key of the particle's cell (the cell index itself when si = sj = 0)
__device__ __forceinline__ int key_of(uint32_t x, uint32_t z, const SortArgs& a)
{
    const int i = min((int)(x >> kFracBits), a.nx - 2);
    const int j = min((int)(z >> kFracBits), a.nz - 2);
    return (i >> a.si) * a.nzk + (j >> a.sj);
}

// Runs of consecutive lanes with the same key (c < 0: no particle): the
// lane's run head and, for a head, the run's length.  Particles sorted a few
// steps ago arrive in such runs; a key that occurs in two runs of a warp is
// simply looked up twice.
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

// Chunks and the chunk's table of cells.  A table has twice as many entries
// as a chunk has particles, so it is at most half full and a probe sequence
// always reaches the cell's entry or a free one.
constexpr uint32_t kNoCell = 0xFFFFFFFFu;

// A table entry: .x the cell (kNoCell: free), .y the chunk's particles in it;
// the scatter later overwrites them with the run's first destination slot and
// its place in the chunk's output order.
//
// Entry of cell c in a table of 2^TBITS entries (inserted if absent): linear
// probing from a multiplicative hash, entries claimed with atomicCAS.  An
// entry never changes its cell within a chunk, so a read that sees another
// cell moves on.
template <int TBITS>
__device__ __forceinline__ int table_entry(uint2* tab, uint32_t c)
{
    constexpr int kSize = 1 << TBITS;
    uint32_t h = (c * 2654435761u) >> (32 - TBITS);
    for (int probe = 0; probe < kSize; ++probe) {
        const uint32_t k = *(volatile uint32_t*)&tab[h].x;
        if (k == c) return (int)h;
        if (k == kNoCell) {
            const uint32_t prev = atomicCAS(&tab[h].x, kNoCell, c);
            if (prev == kNoCell || prev == c) return (int)h;
        }
        h = (h + 1) & (kSize - 1);
    }
    return -1;  // unreachable: at most half of the entries are taken
}

// Entry of every live particle of one pass of a chunk and its rank among the
// chunk's particles of that cell: the head of each run of equal cells in the
// warp looks the cell up once and adds the run's length to the entry's count.
// Returns (rank << TBITS) | entry, or kNoCell for no particle.
template <int TBITS>
__device__ __forceinline__ uint32_t chunk_rank(uint2* tab, int c, int lane)
{
    const LaneRun r = lane_run(c, lane);
    uint32_t e = 0, r0 = 0;
    if (c >= 0 && r.is_head) {
        e = (uint32_t)table_entry<TBITS>(tab, (uint32_t)c);
        r0 = atomicAdd(&tab[e].y, (unsigned)r.len);
    }
    e = __shfl_sync(0xffffffffu, e, r.head);
    r0 = __shfl_sync(0xffffffffu, r0, r.head);
    return c < 0 ? kNoCell : ((r0 + (uint32_t)(lane - r.head)) << TBITS) | e;
}

constexpr int kCountChunk = 2048, kCountTableBits = 12, kCountTable = 1 << kCountTableBits;
constexpr int kCountThreads = 256, kCountPer = kCountChunk / kCountThreads;
static_assert(kCountTable >= 2 * kCountChunk, "cell table must stay at most half full");

// count[cell] += the chunk's particles in the cell, one atomic per (chunk, cell).
__global__ void __launch_bounds__(kCountThreads) k_cell_count(const SortArgs a)
{
    __shared__ uint2 tab[kCountTable];
    for (int t = threadIdx.x; t < kCountTable; t += kCountThreads) tab[t] = make_uint2(kNoCell, 0u);
    __syncthreads();
    const long long n = a.n;
    const int lane = threadIdx.x & 31;
    for (long long base = (long long)blockIdx.x * kCountChunk; base < n; base += (long long)gridDim.x * kCountChunk) {
        uint32_t x[kCountPer], z[kCountPer];
#pragma unroll
        for (int q = 0; q < kCountPer; ++q) {
            const long long k = base + q * kCountThreads + threadIdx.x;
            x[q] = k < n ? a.x[k] : kDead;
            z[q] = k < n ? a.z[k] : 0u;
        }
#pragma unroll
        for (int q = 0; q < kCountPer; ++q)
            chunk_rank<kCountTableBits>(tab, x[q] != kDead ? key_of(x[q], z[q], a) : -1, lane);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < kCountTable / kCountThreads; ++i) {
            const int t = i * kCountThreads + threadIdx.x;
            const uint2 en = tab[t];
            if (en.x != kNoCell) {
                atomicAdd(&a.count[en.x], en.y);
                tab[t] = make_uint2(kNoCell, 0u);
            }
        }
        __syncthreads();
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
//
// Persistent blocks, each over the chunks blockIdx.x + i * gridDim.x.  The
// six state arrays of a chunk are contiguous ranges of the source buffers;
// they arrive in shared memory by bulk asynchronous copies NB chunks ahead,
// so the block always has NB - 1 chunks of loads in flight while it works on
// one.  Per chunk: (1) each particle finds its entry and rank in the chunk's
// cell table; (2) each entry reserves its run of the cell's destination slots
// with one atomicSub and gets a place in the chunk's output order (entries
// in thread order, a block scan of their counts); (3) the output order is
// written as a permutation of the staged particles; (4) consecutive threads
// store consecutive particles of the output order, so each cell's run leaves
// as contiguous stores.
template <int THREADS, int CHUNK, int TBITS, int NB>
struct Scatter {
    static constexpr int kChunk = CHUNK, kTableBits = TBITS, kTable = 1 << TBITS, kIdxBits = 11;
    static constexpr int kPer = kChunk / THREADS, kEntries = kTable / THREADS;
    static constexpr size_t kStageBytes = (size_t)kChunk * 6 * sizeof(uint32_t);
    static constexpr size_t kSmem = NB * kStageBytes + kTable * sizeof(uint2) + kChunk * sizeof(uint32_t) + NB * 8;
    static_assert(kChunk % THREADS == 0 && kTable % THREADS == 0, "whole passes");
    static_assert(kTable >= 2 * kChunk, "cell table must stay at most half full");
    static_assert(kChunk <= (1 << kIdxBits) && kChunk % 4 == 0, "staged index fits the permutation entry; 16-byte copies");
};

template <int THREADS, int CHUNK, int TBITS, int NB>
__global__ void __launch_bounds__(THREADS) k_cell_scatter(const SortArgs a, long long n_src)
{
    using S = Scatter<THREADS, CHUNK, TBITS, NB>;
    constexpr int kChunk = S::kChunk, kTable = S::kTable, kTB = S::kTableBits, kIB = S::kIdxBits;
    extern __shared__ uint4 sort_smem[];
    uint32_t* stage = reinterpret_cast<uint32_t*>(sort_smem);          // NB x 6 arrays of kChunk
    uint2* tab = reinterpret_cast<uint2*>(stage + NB * 6 * kChunk);     // kTable entries
    uint32_t* perm = reinterpret_cast<uint32_t*>(tab + kTable);         // (entry << kIB) | staged index
    uint64_t* bar = reinterpret_cast<uint64_t*>(perm + kChunk);         // NB barriers

    const long long nchunks = (n_src + kChunk - 1) / kChunk;
    const long long mine_n = blockIdx.x < nchunks ? (nchunks - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    // chunk i of this block into stage buffer i % NB; one arrival (with the byte count) per fill
    auto fill = [&](long long i) {
        const long long base = ((long long)blockIdx.x + i * gridDim.x) * kChunk;
        const long long cnt = n_src - base < kChunk ? n_src - base : kChunk;
        const uint32_t bytes = (uint32_t)((cnt + 3) & ~3ll) * sizeof(uint32_t);  // slots come in multiples of 64
        uint32_t* st = stage + (i % NB) * 6 * kChunk;
        uint64_t* b = bar + (i % NB);
        mbar_arrive_expect_tx(b, 6 * bytes);
        bulk_load(st + 0 * kChunk, a.x + base, bytes, b);
        bulk_load(st + 1 * kChunk, a.z + base, bytes, b);
        bulk_load(st + 2 * kChunk, a.vx + base, bytes, b);
        bulk_load(st + 3 * kChunk, a.vy + base, bytes, b);
        bulk_load(st + 4 * kChunk, a.vz + base, bytes, b);
        bulk_load(st + 5 * kChunk, a.id + base, bytes, b);
    };
    for (int t = threadIdx.x; t < kTable; t += THREADS) tab[t] = make_uint2(kNoCell, 0u);
    if (threadIdx.x == 0) {
        for (int s = 0; s < NB; ++s) mbar_init(bar + s, 1);
        mbar_init_fence();
        for (long long i = 0; i < NB && i < mine_n; ++i) fill(i);
    }
    __syncthreads();
    const long long total = __ldg(&a.offset[a.ncells]);
    const int lane = threadIdx.x & 31;
    for (long long i = 0; i < mine_n; ++i) {
        const long long base = ((long long)blockIdx.x + i * gridDim.x) * kChunk;
        const uint32_t* st = stage + (i % NB) * 6 * kChunk;
        const bool landed = mbar_wait_bounded(bar + (i % NB), (uint32_t)((i / NB) & 1));
        if (__syncthreads_or(!landed)) {
            // a copy did not complete: report it, give the copies in flight a bounded wait, stop
            if (threadIdx.x == 0) {
                atomicCAS(&a.cnt->error, 0, -5);
                for (long long k = i; k < i + NB && k < mine_n; ++k) mbar_wait_bounded(bar + (k % NB), (uint32_t)((k / NB) & 1));
            }
            return;
        }
        // (1)
        uint32_t er[S::kPer];
#pragma unroll
        for (int q = 0; q < S::kPer; ++q) {
            const int j = q * THREADS + threadIdx.x;
            const long long k = base + j;
            const uint32_t x = k < n_src ? st[j] : kDead;
            if (k < n_src && k >= total) a.ox[k] = kDead;
            er[q] = chunk_rank<kTB>(tab, x != kDead ? key_of(x, st[kChunk + j], a) : -1, lane);
        }
        __syncthreads();
        // (2) this thread's entries t = e * THREADS + threadIdx.x
        uint2 en[S::kEntries];
        uint32_t old[S::kEntries], off[S::kEntries];
        uint32_t mine = 0;
#pragma unroll
        for (int e = 0; e < S::kEntries; ++e) {
            en[e] = tab[e * THREADS + threadIdx.x];
            mine += en[e].y;
        }
#pragma unroll
        for (int e = 0; e < S::kEntries; ++e) {
            old[e] = en[e].x != kNoCell ? atomicSub(&a.count[en[e].x], en[e].y) : 0u;
            off[e] = en[e].x != kNoCell ? __ldg(&a.offset[en[e].x]) : 0u;
        }
        uint32_t at;
        const uint32_t staged = block_exclusive_scan(mine, at);
#pragma unroll
        for (int e = 0; e < S::kEntries; ++e) {
            if (en[e].x != kNoCell) {
                tab[e * THREADS + threadIdx.x] = make_uint2(off[e] + old[e] - en[e].y, at);
                at += en[e].y;
            }
        }
        __syncthreads();
        // (3)
#pragma unroll
        for (int q = 0; q < S::kPer; ++q) {
            if (er[q] == kNoCell) continue;
            const uint32_t e = er[q] & (kTable - 1), r = er[q] >> kTB;
            perm[tab[e].y + r] = (e << kIB) | (uint32_t)(q * THREADS + threadIdx.x);
        }
        __syncthreads();
        // (4)
        for (uint32_t j = threadIdx.x; j < staged; j += THREADS) {
            const uint32_t p = perm[j];
            const uint32_t s = p & ((1u << kIB) - 1);
            const uint2 t = tab[p >> kIB];
            const uint32_t d = t.x + (j - t.y);
            a.ox[d] = st[s];
            a.oz[d] = st[kChunk + s];
            a.ovx[d] = __uint_as_float(st[2 * kChunk + s]);
            a.ovy[d] = __uint_as_float(st[3 * kChunk + s]);
            a.ovz[d] = __uint_as_float(st[4 * kChunk + s]);
            a.oid[d] = st[5 * kChunk + s];
        }
        __syncthreads();
        // the buffer and the table are free: refill the buffer NB chunks ahead, clear the table
        if (threadIdx.x == 0 && i + NB < mine_n) {
            async_proxy_fence();
            fill(i + NB);
        }
#pragma unroll
        for (int e = 0; e < S::kEntries; ++e) tab[e * THREADS + threadIdx.x] = make_uint2(kNoCell, 0u);
        __syncthreads();
    }
}

// two blocks per SM, so that one block's stores overlap the other's table and
// atomic phases
constexpr int kScatterThreads = 512, kScatterChunk = 1536, kScatterTableBits = 12, kScatterStages = 2;
using ScatterCfg = Scatter<kScatterThreads, kScatterChunk, kScatterTableBits, kScatterStages>;
#define SCATTER_KERNEL k_cell_scatter<kScatterThreads, kScatterChunk, kScatterTableBits, kScatterStages>

int blocks_per_sm(const void* f, int threads, size_t smem)
{
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f, threads, smem) != cudaSuccess || b < 1) b = 1;
    return b;
}

}  // namespace

int launch_sort(const SortArgs& a, long long n_src, cudaStream_t s)
{
    if (a.n == 0) return 0;
    // resident blocks of each chunk kernel, found once per process
    struct Grid {
        long long count, scatter;
    };
    static const Grid g = [] {
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(SCATTER_KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ScatterCfg::kSmem);
        return Grid{(long long)sms * blocks_per_sm((const void*)k_cell_count, kCountThreads, 0),
                    (long long)sms * blocks_per_sm((const void*)SCATTER_KERNEL, kScatterThreads, ScatterCfg::kSmem)};
    }();
    k_cell_count<<<(int)std::min<long long>((a.n + kCountChunk - 1) / kCountChunk, g.count), kCountThreads, 0, s>>>(a);
    const int nb = (int)((a.ncells + 1023) / 1024);
    k_scan_local<<<nb, 1024, 0, s>>>(a);
    k_scan_top<<<1, 1024, 0, s>>>(a, nb);
    k_scan_add<<<nb, 1024, 0, s>>>(a);
    SCATTER_KERNEL<<<(int)std::min<long long>((n_src + ScatterCfg::kChunk - 1) / ScatterCfg::kChunk, g.scatter),
                     kScatterThreads, ScatterCfg::kSmem, s>>>(a, n_src);
    return 5;
}

}  // namespace mag
