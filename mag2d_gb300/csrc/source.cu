// Particle source of a Cartesian run (use_source = 1): Species<CARTESIAN>::
// source5_refresh and source (src/particles.cpp:1052-1082, :1165-1226).
//
// Each species keeps a small periodic source box of size (Lx / f, Lz / f)
// (f = src_fact) filled with N / f thermal particles, N = density * V.  Every
// step the box particles fly in the external field (Boris, extern_field along
// z, constant B) with the species' null-collision test against the
// background targets; a particle leaving the box through a face is wrapped
// back into it, and a copy enters the domain through the opposite face of the
// domain, at a random one of the f tiles along that face.  The copies are
// appended to the species after the step's push, in the order of the box
// particles (a scan of per-particle counts), and deposit their charge.
//
// Random variates come from Philox streams keyed by (seed, species, box
// particle, step) instead of the reference's global generator and rand().
#include <algorithm>

#include "device.hpp"
#include "kernels.hpp"
#include "mcc_device.cuh"

namespace mag {

namespace {

// Boris step of the reference's Cartesian mover with the external field only
// (advance_boris with extern_fields = true, src/particles.cpp:924-995): half
// acceleration, rotation with (t, s), half acceleration.  (x, y, z) carry
// (r, theta, z) ~ (x, z, y) as in the reference.
__device__ __forceinline__ void boris_extern(float& vx, float& vy, float& vz, float hq, float ez, float tx, float ty,
                                             float tz, float sx, float sy, float sz)
{
    vz = fmaf(ez, hq, vz);
    const float vpr = vx - vy * tz + vz * ty;
    const float vpz = vz - vx * ty + vy * tx;
    const float vpt = vy - vz * tx + vx * tz;
    vx = vx - vpt * sz + vpz * sy;
    vy = vy - vpz * sx + vpr * sz;
    vz = vz - vpr * sy + vpt * sx;
    vz = fmaf(ez, hq, vz);
}

// source5_refresh: positions uniform in the box, velocities rnor v_max / sqrt 2
// per component (vx, vz, vy in the reference's order), then the leapfrog start
// (advance_boris_init with the external field: half backward rotation, half
// backward acceleration; a.hq and a.t*/a.s* hold the backward values).
__global__ void k_source_refresh(const SourceArgs a, float vsig)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        Stream rs(a.seed, a.species, (uint32_t)i, TAG_SOURCE_INIT, 0);
        a.x[i] = a.bx * rs.uni();
        a.z[i] = a.bz * rs.uni();
        float vx = rs.normalf() * vsig;
        float vz = rs.normalf() * vsig;
        float vy = rs.normalf() * vsig;
        const float vpr = vx - vy * a.tz + vz * a.ty;
        const float vpz = vz - vx * a.ty + vy * a.tx;
        const float vpt = vy - vz * a.tx + vx * a.tz;
        vx = vx - vpt * a.sz + vpz * a.sy;
        vy = vy - vpz * a.sx + vpr * a.sz;
        vz = vz - vpr * a.sy + vpt * a.sx;
        vz = fmaf(a.ez, a.hq, vz);
        a.vx[i] = vx;
        a.vy[i] = vy;
        a.vz[i] = vz;
    }
}

// One step of the box particles and their crossings (source()).  count[i]
// receives the number of copies particle i makes (at most kMaxInject are
// kept; more are counted in *dropped), rec[i][c] = (x, z, vx, vy, vz) of copy
// c in domain coordinates relative to the domain's origin.
__global__ void __launch_bounds__(128) k_source_step(const __grid_constant__ SourceArgs a,
                                                     const __grid_constant__ CollideArgs c)
{
    __shared__ MccStage st;
    extern __shared__ double s_tab[];
    if (a.coll) {
        double* tab = c.n_tables <= kStageTables ? s_tab : nullptr;
        mcc_stage(c, st, tab);
        __syncthreads();
        if (threadIdx.x == 0) mcc_stage_pointers(c, st, tab);
    }
    __syncthreads();
    unsigned ncoll = 0, nnull = 0, dropped = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        double x = a.x[i], z = a.z[i];
        float vx = a.vx[i], vy = a.vy[i], vz = a.vz[i];
        boris_extern(vx, vy, vz, a.hq, a.ez, a.tx, a.ty, a.tz, a.sx, a.sy, a.sz);
        x += (double)vx * a.dt;
        z += (double)vz * a.dt;
        Stream rs(a.seed, a.species, (uint32_t)i, TAG_SOURCE, a.step);
        if (a.coll && rs.unif() < a.prob) {
            const int r = scatter_background(st.m, rs, vx, vy, vz);
            ncoll += r == MCC_HIT;
            nnull += r != MCC_HIT;
        }
        Stream tile(a.seed, a.species, (uint32_t)i, TAG_SOURCE_TILE, a.step);
        int cnt = 0;
        double* rec = a.rec + (size_t)i * kMaxInject * 5;
        auto inject = [&](double px, double pz) {
            if (cnt < kMaxInject) {
                double* r = rec + cnt * 5;
                r[0] = px;
                r[1] = pz;
                r[2] = vx;
                r[3] = vy;
                r[4] = vz;
            }
            ++cnt;
        };
        // a box particle crosses a face at most a few times per step; a wild
        // velocity is wrapped without copies after kMaxInject crossings
        if (x > a.bx) {
            for (int q = 0; x > a.bx; ++q) {
                if (q >= kMaxInject) {
                    x -= a.bx * floor(x / a.bx);
                    break;
                }
                x -= a.bx;
                inject(x, z + (double)(tile.next() % a.factor) * a.bz);
            }
        } else if (x < 0.0) {
            for (int q = 0; x < 0.0; ++q) {
                if (q >= kMaxInject) {
                    x -= a.bx * floor(x / a.bx);
                    break;
                }
                inject(x + a.lx, z + (double)(tile.next() % a.factor) * a.bz);
                x += a.bx;
            }
        }
        if (z > a.bz) {
            for (int q = 0; z > a.bz; ++q) {
                if (q >= kMaxInject) {
                    z -= a.bz * floor(z / a.bz);
                    break;
                }
                z -= a.bz;
                inject(x + (double)(tile.next() % a.factor) * a.bx, z);
            }
        } else if (z < 0.0) {
            for (int q = 0; z < 0.0; ++q) {
                if (q >= kMaxInject) {
                    z -= a.bz * floor(z / a.bz);
                    break;
                }
                inject(x + (double)(tile.next() % a.factor) * a.bx, z + a.lz);
                z += a.bz;
            }
        }
        a.x[i] = x;
        a.z[i] = z;
        a.vx[i] = vx;
        a.vy[i] = vy;
        a.vz[i] = vz;
        a.count[i] = min(cnt, kMaxInject);
        dropped += cnt > kMaxInject ? (unsigned)(cnt - kMaxInject) : 0u;
    }
    const unsigned full = 0xffffffffu;
    ncoll = __reduce_add_sync(full, ncoll);
    nnull = __reduce_add_sync(full, nnull);
    dropped = __reduce_add_sync(full, dropped);
    if ((threadIdx.x & 31) == 0) {
        if (ncoll) atomicAdd(&a.cnt->ncoll, (unsigned long long)ncoll);
        if (nnull) atomicAdd(&a.cnt->nnull, (unsigned long long)nnull);
        if (dropped) atomicAdd(a.dropped, (unsigned long long)dropped);
    }
}

// Exclusive scan of count[0..n) in place (one block), the sum to *total.
__global__ void __launch_bounds__(1024) k_source_scan(int* count, int64_t n, long long* total)
{
    __shared__ long long wsum[32];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t base = 0; base < n; base += blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const long long v = i < n ? count[i] : 0;
        long long inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        long long before = carry;
        for (int w = 0; w < warp; ++w) before += wsum[w];
        if (i < n) count[i] = (int)(before + inc - v);
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + inc;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// Copies of box particle i go to slots base + offs[i] + c with ids
// next_id + offs[i] + c; a copy outside the open domain is a removed slot
// (the reference inserts and removes it), one inside deposits its charge.
__global__ void k_source_append(const SourceArgs a, const int* __restrict__ offs, const int* __restrict__ count_in,
                                SourceAppend t)
{
    const double one = (double)(1u << kFracBits);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        const int m = count_in[i];
        for (int c = 0; c < m; ++c) {
            const double* r = a.rec + ((size_t)i * kMaxInject + c) * 5;
            const int64_t k = t.base + offs[i] + c;
            const double px = r[0], pz = r[1];
            const bool inside = px > 0.0 && px < a.lx && pz > 0.0 && pz < a.lz;
            uint32_t fx = kDead, fz = 0;
            if (inside) {
                fx = (uint32_t)__double2ll_rn(__dmul_rn(__ddiv_rn(px, t.dx), one));
                fz = (uint32_t)__double2ll_rn(__dmul_rn(__ddiv_rn(pz, t.dz), one));
                if (t.rho) {
                    const int ic = min((int)(fx >> kFracBits), t.nx - 2);
                    const int jc = min((int)(fz >> kFracBits), t.nz - 2);
                    const unsigned long long o = 1ull << kDepositShift;
                    const unsigned long long U = fx - ((uint32_t)ic << kFracBits);
                    const unsigned long long V = fz - ((uint32_t)jc << kFracBits);
                    unsigned long long* r0 = t.rho + (size_t)ic * t.nz + jc;
                    atomicAdd(r0, (o - U) * (o - V));
                    atomicAdd(r0 + t.nz, U * (o - V));
                    atomicAdd(r0 + 1, (o - U) * V);
                    atomicAdd(r0 + t.nz + 1, U * V);
                }
            }
            t.x[k] = fx;
            t.z[k] = fz;
            t.vx[k] = (float)r[2];
            t.vy[k] = (float)r[3];
            t.vz[k] = (float)r[4];
            t.id[k] = t.next_id + (uint32_t)(offs[i] + c);
        }
    }
}

unsigned grid_of(int64_t n, int threads) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 152 * 8)); }

}  // namespace

int launch_source_refresh(const SourceArgs& a, float vsig, cudaStream_t s)
{
    if (a.n == 0) return 0;
    k_source_refresh<<<grid_of(a.n, 256), 256, 0, s>>>(a, vsig);
    return 1;
}

int launch_source_step(const SourceArgs& a, const CollideArgs& c, int* offs, long long* total, cudaStream_t s)
{
    if (a.n == 0) return 0;
    const size_t smem = a.coll && c.n_tables <= kStageTables ? (size_t)c.n_tables * sizeof(double) : 0;
    k_source_step<<<grid_of(a.n, 128), 128, smem, s>>>(a, c);
    cudaMemcpyAsync(offs, a.count, (size_t)a.n * sizeof(int), cudaMemcpyDeviceToDevice, s);
    k_source_scan<<<1, 1024, 0, s>>>(offs, a.n, total);
    return 2;
}

int launch_source_append(const SourceArgs& a, const int* offs, const SourceAppend& t, cudaStream_t s)
{
    if (a.n == 0) return 0;
    k_source_append<<<grid_of(a.n, 256), 256, 0, s>>>(a, offs, a.count, t);
    return 1;
}

}  // namespace mag
