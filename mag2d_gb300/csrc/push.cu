// Particle step kernel: field gather, Boris push, collision test, boundary,
// mask test and fixed-point charge deposit, fused into one pass over the SoA.
//
// Replaces, per particle, the loop bodies of
//   Species<CYLINDRICAL>::advance_boris   src/particles.cpp:539-621
//   Species<CARTESIAN>::advance_boris     src/particles.cpp:924-995
//   Fields::E / Fields::B                 src/fields.hpp:124-177
//   Species::advance_boundary             src/particles.hpp:370-411
//   t_grid::is_free                       src/fields.hpp:94-101
//   Field2D::accumulate                   src/Field2D.hpp:45-62
// Scattering changes only velocities, so boundary and deposit, which read
// positions only, give the same result as in the reference's order.
//
// HBM traffic per live particle and step: read x, z, vx, vy, vz (20 B) and,
// when collisions are on, id (4 B); write x, z, vx, vy, vz (20 B).  Field
// faces, mask and the charge grid are small and stay in L1/L2 when the
// particles are sorted by cell.
#include "device.hpp"
#include "kernels.hpp"
#include "philox.hpp"

namespace mag {

namespace {

constexpr float kInvOne = 1.0f / (float)(1u << kFracBits);
constexpr float kOne = (float)(1u << kFracBits);
constexpr uint32_t kHalf = 1u << (kFracBits - 1);

__device__ __forceinline__ float frac(uint32_t v) { return (float)(v & kFracMask) * kInvOne; }

__device__ __forceinline__ float bilerp(const float* __restrict__ f, int stride, int i, int j, float fx, float fz)
{
    const float* p = f + (size_t)i * stride + j;
    const float a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + stride), d = __ldg(p + stride + 1);
    return (1.f - fx) * ((1.f - fz) * a + fz * b) + fx * ((1.f - fz) * c + fz * d);
}

__device__ __forceinline__ float2 bilerp2(const float2* __restrict__ f, int stride, int i, int j, float fx, float fz)
{
    const float2* p = f + (size_t)i * stride + j;
    const float2 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + stride), d = __ldg(p + stride + 1);
    const float w00 = (1.f - fx) * (1.f - fz), w01 = (1.f - fx) * fz, w10 = fx * (1.f - fz), w11 = fx * fz;
    return make_float2(w00 * a.x + w01 * b.x + w10 * c.x + w11 * d.x, w00 * a.y + w01 * b.y + w10 * c.y + w11 * d.y);
}

// Stencil of Field2D::grad at fixed-point position (x, z): the x component
// interpolates faces (ix, ix+1) x (jz, jz+1) around the rounded x, the z
// component faces (iz, iz+1) x (jz2, jz2+1) around the rounded z.
struct GatherIdx {
    int ix, jz, iz, jz2;
    float fx, fz, gx, gz;
};
__device__ __forceinline__ GatherIdx gather_idx(uint32_t x, uint32_t z, int nx, int nz)
{
    GatherIdx g;
    const uint32_t xr = x + kHalf, zr = z + kHalf;
    g.ix = min((int)(xr >> kFracBits), nx - 1);
    g.fx = frac(xr);
    g.jz = min((int)(z >> kFracBits), nz - 2);
    g.fz = (float)(z - ((uint32_t)g.jz << kFracBits)) * kInvOne;
    g.iz = min((int)(x >> kFracBits), nx - 2);
    g.gx = (float)(x - ((uint32_t)g.iz << kFracBits)) * kInvOne;
    g.jz2 = min((int)(zr >> kFracBits), nz - 1);
    g.gz = frac(zr);
    return g;
}

// Field2D::interpolate of a B table at physical position (x, z)
__device__ __forceinline__ float table_interp(const float* __restrict__ t, int bnx, int bnz, float xi, float zi)
{
    const int i = max(0, min((int)xi, bnx - 2));
    const int j = max(0, min((int)zi, bnz - 2));
    return bilerp(t, bnz, i, j, xi - (float)i, zi - (float)j);
}

template <int EMODE>
__device__ __forceinline__ void gather_E(const PushArgs& a, uint32_t x, uint32_t z, float phase, float& ex, float& ez)
{
    if (EMODE == 0) {
        ex = 0.f;
        ez = a.extern_ez;
        return;
    }
    const GatherIdx g = gather_idx(x, z, a.nx, a.nz);
    if (EMODE == 1) {
        ex = bilerp(a.Exf, a.nz, g.ix, g.jz, g.fx, g.fz);
        ez = bilerp(a.Ezf, a.nz + 1, g.iz, g.jz2, g.gx, g.gz);
    } else {
        const float2 px = bilerp2(a.Exf2, a.nz, g.ix, g.jz, g.fx, g.fz);
        const float2 pz = bilerp2(a.Ezf2, a.nz + 1, g.iz, g.jz2, g.gx, g.gz);
        ex = px.x + phase * px.y;
        ez = pz.x + phase * pz.y;
    }
}

__device__ __forceinline__ void boris_vectors(const PushArgs& a, uint32_t x, uint32_t z, float& tx, float& ty,
                                              float& tz, float& sx, float& sy, float& sz)
{
    tx = a.tx, ty = a.ty, tz = a.tz, sx = a.sx, sy = a.sy, sz = a.sz;
    if (a.btab) {
        const float xc = (float)(x >> kFracBits) + frac(x), zc = (float)(z >> kFracBits) + frac(z);
        const float xi = (xc * a.gdx + a.gx0 - a.b_x0) * a.b_ix;
        const float zi = (zc * a.gdz + a.gz0 - a.b_z0) * a.b_iz;
        tx = table_interp(a.Br, a.bnx, a.bnz, xi, zi) * a.q_dt_2m;
        tz = table_interp(a.Bz, a.bnx, a.bnz, xi, zi) * a.q_dt_2m;
        ty = 0.f;
        const float f = 2.f / (1.f + tx * tx + ty * ty + tz * tz);
        sx = tx * f;
        sy = ty * f;
        sz = tz * f;
    }
}

template <int COORD>
__device__ __forceinline__ void rotate(float& vx, float& vy, float& vz, float tx, float ty, float tz, float sx,
                                       float sy, float sz)
{
    if (COORD == 1) {  // (r, theta, z) orientation, particles.cpp:581-592
        const float vpr = vx + vy * tz - vz * ty;
        const float vpt = vy + vz * tx - vx * tz;
        const float vpz = vz + vx * ty - vy * tx;
        vx += vpt * sz - vpz * sy;
        vy += vpz * sx - vpr * sz;
        vz += vpr * sy - vpt * sx;
    } else {  // (x, y, z) ~ (r, z, theta), particles.cpp:968-979
        const float vpr = vx - vy * tz + vz * ty;
        const float vpz = vz - vx * ty + vy * tx;
        const float vpt = vy - vz * tx + vx * tz;
        vx += -vpt * sz + vpz * sy;
        vy += -vpz * sx + vpr * sz;
        vz += -vpr * sy + vpt * sx;
    }
}

// Move a fixed-point coordinate by d fixed-point units; false when it leaves
// [0, maxf] (advance_boundary, FREE), or wrapped into [0, maxf) (PERIODIC).
__device__ __forceinline__ bool move_coord(uint32_t& x, int d, uint32_t maxf, bool periodic)
{
    const uint32_t nx = x + (uint32_t)d;
    const bool out = d >= 0 ? (nx < x || nx > maxf) : (nx > x);
    if (!out) {
        x = nx;
        return true;
    }
    if (!periodic || maxf == 0) return false;
    long long p = (long long)x + d;  // rare path
    p %= (long long)maxf;
    if (p < 0) p += maxf;
    x = (uint32_t)p;
    return true;
}

// displacement in fixed-point units, clamped so that a wild value is simply "out"
__device__ __forceinline__ int to_fixed_disp(float cells)
{
    const float v = fminf(fmaxf(cells * kOne, -1.0e9f), 1.0e9f);
    return __float2int_rn(v);
}

__device__ __forceinline__ void close_step_if_last(Counters* c, unsigned long long coll, unsigned long long nnull)
{
    // one thread per block; the last block to arrive finishes the step
    if (coll) atomicAdd(&c->ncoll, coll);
    if (nnull) atomicAdd(&c->nnull, nnull);
    __threadfence();
    const unsigned long long ticket = atomicAdd(&c->done_blocks, 1ull);
    if (ticket == gridDim.x - 1) {
        __threadfence();
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

// One particle of the step.  Returns the new state through the references;
// alive / removed / candidate flags drive the counters.
template <int COORD, int EMODE>
__device__ __forceinline__ void step_particle(const PushArgs& a, int64_t k, uint32_t& x, uint32_t& z, float& vx,
                                              float& vy, float& vz, bool& alive, bool& cand)
{
    float ex, ez;
    gather_E<EMODE>(a, x, z, a.phase, ex, ez);
    float tx, ty, tz, sx, sy, sz;
    boris_vectors(a, x, z, tx, ty, tz, sx, sy, sz);
    // half acceleration, Boris rotation (Birdsall & Langdon), half acceleration
    vx += ex * a.hq;
    vz += ez * a.hq;
    rotate<COORD>(vx, vy, vz, tx, ty, tz, sx, sy, sz);
    vx += ex * a.hq;
    vz += ez * a.hq;
    int dpx;
    const float dz = vz * a.cz;
    if (COORD == 1) {
        // push in the local Cartesian frame, map back to r and rotate v (Birdsall p. 338);
        // dr = r' - r = (2 r a + a^2 + b^2) / (r' + r) keeps the fixed-point r exact
        const float r = (float)(x >> kFracBits) + frac(x);
        const float ax = vx * a.cx, by = vy * a.cx;
        const float x2 = r + ax;
        const float rn = sqrtf(x2 * x2 + by * by);
        const float den = rn + r;
        const float dr = den > 0.f ? (ax * (r + x2) + by * by) / den : 0.f;
        float sa = 0.f, ca = 1.f;
        if (rn != 0.f) {
            const float ir = 1.f / rn;
            sa = by * ir;
            ca = x2 * ir;
        }
        const float t0 = vx;
        vx = ca * vx + sa * vy;
        vy = -sa * t0 + ca * vy;
        dpx = to_fixed_disp(dr);
        alive = isfinite(dr);
    } else {
        const float dx = vx * a.cx;
        dpx = to_fixed_disp(dx);
        alive = isfinite(dx);
    }
    alive = alive && isfinite(dz);
    // boundary (advance_boundary): outside the box -> removed, or wrapped if PERIODIC
    alive = alive && move_coord(x, dpx, a.xmaxf, a.periodic) && move_coord(z, to_fixed_disp(dz), a.zmaxf, a.periodic);
    cand = false;
    if (!alive) return;
    const int ic = min((int)(x >> kFracBits), a.nx - 2);
    const int jc = min((int)(z >> kFracBits), a.nz - 2);
    if (a.check_mask) {
        const int8_t* m = a.mask + (size_t)ic * a.nz + jc;
        const bool fr = m[0] == 2 || m[a.nz] == 2 || m[1] == 2 || m[a.nz + 1] == 2;  // FREE
        if (!fr) {
            alive = false;
            return;
        }
    }
    if (a.rho != nullptr) {
        const unsigned long long one = 1ull << kDepositShift;
        const unsigned long long U = x - ((uint32_t)ic << kFracBits);
        const unsigned long long V = z - ((uint32_t)jc << kFracBits);
        unsigned long long* r0 = a.rho + (size_t)ic * a.nz + jc;
        atomicAdd(r0, (one - U) * (one - V));
        atomicAdd(r0 + a.nz, U * (one - V));
        atomicAdd(r0 + 1, (one - U) * V);
        atomicAdd(r0 + a.nz + 1, U * V);
    }
    if (a.coll_threshold != 0u) cand = collision_test_u32(a.seed, a.species, a.id[k], a.step) < a.coll_threshold;
}

__device__ __forceinline__ void append_candidate(const PushArgs& a, bool cand, int64_t k)
{
    const unsigned full = 0xffffffffu;
    const unsigned cand_mask = __ballot_sync(full, cand);
    if (cand_mask) {
        const int lane = threadIdx.x & 31;
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&a.cnt->ncand, (unsigned long long)__popc(cand_mask));
        base = __shfl_sync(full, base, 0);
        if (cand) a.cand[base + __popc(cand_mask & ((1u << lane) - 1u))] = (uint32_t)k;
    }
}

// Persistent grid-stride kernel, two particles per thread and iteration (two
// independent load streams in flight), counters kept in registers and added
// once per warp at the end.  Collision candidates go to a compacted list that
// k_collide processes; without collisions this kernel closes the step.
template <int COORD, int EMODE>
__global__ void __launch_bounds__(256, 4) k_push(const PushArgs a)
{
    const int64_t n = a.n;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned live = 0, removed = 0;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += 2 * stride) {
        const int64_t k0 = base + threadIdx.x, k1 = k0 + stride;
        uint32_t x0 = k0 < n ? a.x[k0] : kDead, x1 = k1 < n ? a.x[k1] : kDead;
        uint32_t z0 = 0, z1 = 0;
        float vx0 = 0.f, vy0 = 0.f, vz0 = 0.f, vx1 = 0.f, vy1 = 0.f, vz1 = 0.f;
        if (x0 != kDead) {
            z0 = a.z[k0];
            vx0 = a.vx[k0];
            vy0 = a.vy[k0];
            vz0 = a.vz[k0];
        }
        if (x1 != kDead) {
            z1 = a.z[k1];
            vx1 = a.vx[k1];
            vy1 = a.vy[k1];
            vz1 = a.vz[k1];
        }
        bool al0 = false, c0 = false, al1 = false, c1 = false;
        if (x0 != kDead) {
            step_particle<COORD, EMODE>(a, k0, x0, z0, vx0, vy0, vz0, al0, c0);
            a.x[k0] = al0 ? x0 : kDead;
            a.z[k0] = z0;
            a.vx[k0] = vx0;
            a.vy[k0] = vy0;
            a.vz[k0] = vz0;
            live += al0;
            removed += !al0;
        }
        if (x1 != kDead) {
            step_particle<COORD, EMODE>(a, k1, x1, z1, vx1, vy1, vz1, al1, c1);
            a.x[k1] = al1 ? x1 : kDead;
            a.z[k1] = z1;
            a.vx[k1] = vx1;
            a.vy[k1] = vy1;
            a.vz[k1] = vz1;
            live += al1;
            removed += !al1;
        }
        if (a.coll_threshold != 0u) {
            append_candidate(a, c0, k0);
            append_candidate(a, c1, k1);
        }
    }
    const unsigned full = 0xffffffffu;
    live = __reduce_add_sync(full, live);
    removed = __reduce_add_sync(full, removed);
    if ((threadIdx.x & 31) == 0) {
        if (live) atomicAdd(&a.cnt->live_step, (unsigned long long)live);
        if (removed) atomicAdd(&a.cnt->removed, (unsigned long long)removed);
    }
    if (a.close_step) {
        __syncthreads();
        if (threadIdx.x == 0) close_step_if_last(a.cnt, 0, 0);
    }
}

// Leapfrog start (advance_boris_init, src/particles.cpp:623-679, :997-1050):
// a backward half rotation and a backward half acceleration, no move.  The
// caller passes the half-angle backward rotation vectors and hq = -q/m dt/2.
template <int COORD, int EMODE>
__global__ void __launch_bounds__(256) k_push_init(const PushArgs a)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n) return;
    const uint32_t x = a.x[k];
    if (x == kDead) return;
    const uint32_t z = a.z[k];
    float vx = a.vx[k], vy = a.vy[k], vz = a.vz[k];
    float ex, ez;
    gather_E<EMODE>(a, x, z, a.phase, ex, ez);
    float tx, ty, tz, sx, sy, sz;
    boris_vectors(a, x, z, tx, ty, tz, sx, sy, sz);
    rotate<COORD>(vx, vy, vz, tx, ty, tz, sx, sy, sz);
    vx += ex * a.hq;
    vz += ez * a.hq;
    a.vx[k] = vx;
    a.vy[k] = vy;
    a.vz[k] = vz;
}

// Species::accumulate (src/particles.hpp:358-367) into the fixed-point grid
__global__ void __launch_bounds__(256) k_deposit(const PushArgs a)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n) return;
    const uint32_t x = a.x[k];
    if (x == kDead) return;
    const uint32_t z = a.z[k];
    const int ic = min((int)(x >> kFracBits), a.nx - 2);
    const int jc = min((int)(z >> kFracBits), a.nz - 2);
    const unsigned long long one = 1ull << kDepositShift;
    const unsigned long long U = x - ((uint32_t)ic << kFracBits);
    const unsigned long long V = z - ((uint32_t)jc << kFracBits);
    unsigned long long* r0 = a.rho + (size_t)ic * a.nz + jc;
    atomicAdd(r0, (one - U) * (one - V));
    atomicAdd(r0 + a.nz, U * (one - V));
    atomicAdd(r0 + 1, (one - U) * V);
    atomicAdd(r0 + a.nz + 1, U * V);
}

template <int COORD>
void launch_push_t(const PushArgs& a, cudaStream_t s, bool init)
{
    const unsigned grid = (unsigned)((a.n + 255) / 256);
    if (grid == 0) return;
    // the step kernel runs a persistent grid: at most 8 blocks per SM of the 152
    const unsigned pgrid = (unsigned)std::min<int64_t>((a.n + 511) / 512, 152 * 8);
    switch (a.emode) {
    case 0: init ? k_push_init<COORD, 0><<<grid, 256, 0, s>>>(a) : k_push<COORD, 0><<<pgrid, 256, 0, s>>>(a); break;
    case 1: init ? k_push_init<COORD, 1><<<grid, 256, 0, s>>>(a) : k_push<COORD, 1><<<pgrid, 256, 0, s>>>(a); break;
    default: init ? k_push_init<COORD, 2><<<grid, 256, 0, s>>>(a) : k_push<COORD, 2><<<pgrid, 256, 0, s>>>(a); break;
    }
}

}  // namespace

int launch_push(const PushArgs& a, int coord, bool init, cudaStream_t s)
{
    if (a.n == 0) return 0;
    if (coord == 1) launch_push_t<1>(a, s, init);
    else launch_push_t<0>(a, s, init);
    return 1;
}

int launch_deposit(const PushArgs& a, cudaStream_t s)
{
    if (a.n == 0) return 0;
    k_deposit<<<(unsigned)((a.n + 255) / 256), 256, 0, s>>>(a);
    return 1;
}

}  // namespace mag
