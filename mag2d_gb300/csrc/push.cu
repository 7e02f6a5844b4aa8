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
#include <algorithm>

#include "device.hpp"
#include "kernels.hpp"
#include "mcc_device.cuh"
#include "philox.hpp"

namespace mag {

namespace {

constexpr float kInvOne = 1.0f / (float)(1u << kFracBits);
constexpr float kOne = (float)(1u << kFracBits);
constexpr uint32_t kHalf = 1u << (kFracBits - 1);

// Explicitly rounded arithmetic: a product that is added is an fmaf, every
// other product and sum is rounded on its own (__fmul_rn, __fadd_rn, which the
// compiler never contracts).  Every instantiation of the step (slots per
// thread, field and B variants) then produces the same bits per particle.
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }

__device__ __forceinline__ float frac(uint32_t v) { return mul((float)(v & kFracMask), kInvOne); }
__device__ __forceinline__ float cells(uint32_t v) { return add((float)(v >> kFracBits), frac(v)); }

// (1-fx) ((1-fz) a + fz b) + fx ((1-fz) c + fz d)
__device__ __forceinline__ float lerp4(float a, float b, float c, float d, float fx, float fz)
{
    const float ofz = sub(1.f, fz);
    const float lo = fmaf(fz, b, mul(ofz, a)), hi = fmaf(fz, d, mul(ofz, c));
    return fmaf(fx, hi, mul(sub(1.f, fx), lo));
}

__device__ __forceinline__ float bilerp(const float* __restrict__ f, int stride, int i, int j, float fx, float fz)
{
    const float* p = f + (size_t)i * stride + j;
    const float a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + stride), d = __ldg(p + stride + 1);
    return lerp4(a, b, c, d, fx, fz);
}

__device__ __forceinline__ float2 bilerp2(const float2* __restrict__ f, int stride, int i, int j, float fx, float fz)
{
    const float2* p = f + (size_t)i * stride + j;
    const float2 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + stride), d = __ldg(p + stride + 1);
    return make_float2(lerp4(a.x, b.x, c.x, d.x, fx, fz), lerp4(a.y, b.y, c.y, d.y, fx, fz));
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
    g.fz = mul((float)(z - ((uint32_t)g.jz << kFracBits)), kInvOne);
    g.iz = min((int)(x >> kFracBits), nx - 2);
    g.gx = mul((float)(x - ((uint32_t)g.iz << kFracBits)), kInvOne);
    g.jz2 = min((int)(zr >> kFracBits), nz - 1);
    g.gz = frac(zr);
    return g;
}

// Field2D::interpolate of a B table at physical position (x, z)
__device__ __forceinline__ float table_interp(const float* __restrict__ t, int bnx, int bnz, float xi, float zi)
{
    const int i = max(0, min((int)xi, bnx - 2));
    const int j = max(0, min((int)zi, bnz - 2));
    return bilerp(t, bnz, i, j, sub(xi, (float)i), sub(zi, (float)j));
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
        ex = fmaf(phase, px.y, px.x);
        ez = fmaf(phase, pz.y, pz.x);
    }
}

// Boris vectors t and s at (x, z) as hi + lo float pairs: the constants of a
// uniform B, or the table values (whose lo parts are zero).
struct BorisVec {
    float tx, ty, tz, sx, sy, sz;
    float tlx, tly, tlz, slx, sly, slz;
};
__device__ __forceinline__ BorisVec boris_vectors(const PushArgs& a, uint32_t x, uint32_t z)
{
    BorisVec b{a.tx, a.ty, a.tz, a.sx, a.sy, a.sz, a.tlx, a.tly, a.tlz, a.slx, a.sly, a.slz};
    if (a.btab) {
        const float xi = mul(sub(fmaf(cells(x), a.gdx, a.gx0), a.b_x0), a.b_ix);
        const float zi = mul(sub(fmaf(cells(z), a.gdz, a.gz0), a.b_z0), a.b_iz);
        b.tx = mul(table_interp(a.Br, a.bnx, a.bnz, xi, zi), a.q_dt_2m);
        b.tz = mul(table_interp(a.Bz, a.bnx, a.bnz, xi, zi), a.q_dt_2m);
        b.ty = 0.f;
        const float f = __fdiv_rn(2.f, fmaf(b.tz, b.tz, fmaf(b.tx, b.tx, 1.f)));
        b.sx = mul(b.tx, f);
        b.sy = 0.f;
        b.sz = mul(b.tz, f);
        b.tlx = b.tly = b.tlz = b.slx = b.sly = b.slz = 0.f;
    }
    return b;
}

// v' = v + v x t, v+ = v + v' x s in the orientation of each coordinate
// system.  Each component is the FP32 sum of the hi-part terms plus the
// separately summed lo-part terms, so the only rounding left is that of the
// arithmetic itself, which does not repeat identically from step to step.
// rot_term = v + (p q - r s) with the lo parts ql, sl of q and s
__device__ __forceinline__ float rot_term(float v, float p, float q, float r, float s, float ql, float sl)
{
    return add(fmaf(-r, s, fmaf(p, q, v)), fmaf(-r, sl, mul(p, ql)));
}
template <int COORD>
__device__ __forceinline__ void rotate(float& vx, float& vy, float& vz, const BorisVec& b)
{
    if (COORD == 1) {  // (r, theta, z) orientation, particles.cpp:581-592
        const float vpr = rot_term(vx, vy, b.tz, vz, b.ty, b.tlz, b.tly);
        const float vpt = rot_term(vy, vz, b.tx, vx, b.tz, b.tlx, b.tlz);
        const float vpz = rot_term(vz, vx, b.ty, vy, b.tx, b.tly, b.tlx);
        vx = rot_term(vx, vpt, b.sz, vpz, b.sy, b.slz, b.sly);
        vy = rot_term(vy, vpz, b.sx, vpr, b.sz, b.slx, b.slz);
        vz = rot_term(vz, vpr, b.sy, vpt, b.sx, b.sly, b.slx);
    } else {  // (x, y, z) ~ (r, z, theta), particles.cpp:968-979
        const float vpr = rot_term(vx, vz, b.ty, vy, b.tz, b.tly, b.tlz);
        const float vpz = rot_term(vz, vy, b.tx, vx, b.ty, b.tlx, b.tly);
        const float vpt = rot_term(vy, vx, b.tz, vz, b.tx, b.tlz, b.tlx);
        vx = rot_term(vx, vpz, b.sy, vpt, b.sz, b.sly, b.slz);
        vy = rot_term(vy, vpr, b.sz, vpz, b.sx, b.slz, b.slx);
        vz = rot_term(vz, vpt, b.sx, vpr, b.sy, b.slx, b.sly);
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
__device__ __forceinline__ int to_fixed_disp(float c)
{
    const float v = fminf(fmaxf(mul(c, kOne), -1.0e9f), 1.0e9f);
    return __float2int_rn(v);
}

// The four CIC corner weights of fractions U, V (2^-20 cell units, at most
// 2^20): products of two 21-bit numbers, each one 32 x 32 -> 64 multiply.
__device__ __forceinline__ void cic_weights(uint32_t U, uint32_t V, unsigned long long (&w)[4])
{
    const uint32_t one = 1u << kDepositShift;
    const uint32_t oU = one - U, oV = one - V;
    w[0] = (unsigned long long)oU * oV;
    w[1] = (unsigned long long)U * oV;
    w[2] = (unsigned long long)oU * V;
    w[3] = (unsigned long long)U * V;
}

// One particle of the step, in registers.  Returns alive (false: removed at
// the boundary or in a closed cell) and cand (the collision test fired).
// CIC deposit of one particle into the fixed-point grid (Field2D::accumulate):
// four int64 corner weights summing to 2^40.
struct GlobalDeposit {
    unsigned long long* rho;
    int nz;
    __device__ __forceinline__ void add(int ic, int jc, unsigned long long U, unsigned long long V) const
    {
        unsigned long long w[4];
        cic_weights((uint32_t)U, (uint32_t)V, w);
        unsigned long long* r0 = rho + (size_t)ic * nz + jc;
        atomicAdd(r0, w[0]);
        atomicAdd(r0 + nz, w[1]);
        atomicAdd(r0 + 1, w[2]);
        atomicAdd(r0 + nz + 1, w[3]);
    }
};

// The same into a block's shared tile of kTileRows x kTileCols nodes whose
// first node is (ai, aj); weights are kept as two 32-bit sums of their low and
// high 20 bits (a tile receives at most 2^11 particles between flushes, so
// neither sum overflows).  A particle whose corners fall outside the tile goes
// to the grid directly.  Integer sums make the result the same either way.
constexpr int kTileRows = 6, kTileCols = 40;
// Lanes add into kTileCopies interleaved copies of the tile (copy lane % 8,
// offset by one bank each), so sorted particles of one cell in a warp
// serialise 8 ways less on the same shared address; the flush adds the copies.
constexpr int kTileCopies = 8, kTileStride = kTileRows * kTileCols + 1;
struct TileDeposit {
    unsigned* lo;  // copy c of node t at c * kTileStride + t
    unsigned* hi;
    int ai, aj;
    GlobalDeposit g;
    __device__ __forceinline__ void add(int ic, int jc, unsigned long long U, unsigned long long V) const
    {
        const int r = ic - ai, c = jc - aj;
        if ((unsigned)r > (unsigned)(kTileRows - 2) || (unsigned)c > (unsigned)(kTileCols - 2)) {
            g.add(ic, jc, U, V);
            return;
        }
        unsigned long long w[4];
        cic_weights((uint32_t)U, (uint32_t)V, w);
        const int cp = (threadIdx.x & (kTileCopies - 1)) * kTileStride;
        const int t[4] = {cp + r * kTileCols + c, cp + (r + 1) * kTileCols + c, cp + r * kTileCols + c + 1,
                          cp + (r + 1) * kTileCols + c + 1};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            atomicAdd(lo + t[q], (unsigned)(w[q] & 0xFFFFFu));
            atomicAdd(hi + t[q], (unsigned)(w[q] >> 20));
        }
    }
};

// no deposit (runs without a self-consistent field)
struct NoDeposit {
    __device__ __forceinline__ void add(int, int, unsigned long long, unsigned long long) const {}
};

// step: the species' step counter; phase: the RF factor of that step; dep:
// where the charge of the new position goes when a.rho is set.
template <int COORD, int EMODE, bool BFIELD, class Dep>
__device__ __forceinline__ void step_particle(const PushArgs& a, uint32_t& x, uint32_t& z, float& vx, float& vy,
                                              float& vz, uint32_t id, uint64_t step, float phase, bool& alive,
                                              bool& cand, const Dep& dep)
{
    // the test uses only (seed, species, id, step): computed first, off the dependency chain
    cand = a.coll_threshold != 0u && collision_test_u32(a.seed, a.species, id, step) < a.coll_threshold;
    float ex, ez;
    gather_E<EMODE>(a, x, z, phase, ex, ez);
    // half acceleration, Boris rotation (Birdsall & Langdon), half acceleration
    vx = fmaf(ex, a.hq, vx);
    vz = fmaf(ez, a.hq, vz);
    if (BFIELD) {
        rotate<COORD>(vx, vy, vz, boris_vectors(a, x, z));
    }
    vx = fmaf(ex, a.hq, vx);
    vz = fmaf(ez, a.hq, vz);
    int dpx;
    const float dz = mul(vz, a.cz);
    if (COORD == 1) {
        // push in the local Cartesian frame, map back to r and rotate v (Birdsall p. 338);
        // dr = r' - r = (2 r a + a^2 + b^2) / (r' + r) keeps the fixed-point r exact
        const float r = cells(x);
        const float ax = mul(vx, a.cx), by = mul(vy, a.cx);
        const float x2 = add(r, ax);
        const float b2 = mul(by, by);
        const float rn = __fsqrt_rn(fmaf(x2, x2, b2));
        const float den = add(rn, r);
        const float dr = den > 0.f ? __fdiv_rn(fmaf(ax, add(r, x2), b2), den) : 0.f;
        float sa = 0.f, ca = 1.f;
        if (rn != 0.f) {
            const float ir = __fdiv_rn(1.f, rn);
            sa = mul(by, ir);
            ca = mul(x2, ir);
        }
        const float t0 = vx;
        vx = fmaf(sa, vy, mul(ca, vx));
        vy = fmaf(-sa, t0, mul(ca, vy));
        dpx = to_fixed_disp(dr);
        alive = isfinite(dr);
    } else {
        const float dx = mul(vx, a.cx);
        dpx = to_fixed_disp(dx);
        alive = isfinite(dx);
    }
    alive = alive && isfinite(dz);
    // boundary (advance_boundary): outside the box -> removed, or wrapped if PERIODIC
    alive = alive && move_coord(x, dpx, a.xmaxf, a.periodic) && move_coord(z, to_fixed_disp(dz), a.zmaxf, a.periodic);
    if (!alive) {
        cand = false;
        return;
    }
    const int ic = min((int)(x >> kFracBits), a.nx - 2);
    const int jc = min((int)(z >> kFracBits), a.nz - 2);
    // t_grid::is_free: at least one FREE corner, precomputed per cell
    if (a.check_mask && __ldg(a.cellfree + (size_t)ic * (a.nz - 1) + jc) == 0) {
        alive = false;
        cand = false;
        return;
    }
    if (a.rho != nullptr)
        dep.add(ic, jc, x - ((uint32_t)ic << kFracBits), z - ((uint32_t)jc << kFracBits));
}

// Warp-aggregated append of a collision candidate: slot index and a record
// of (vx, vy, vz, id) after the push, so that k_collide needs one load per
// candidate.
__device__ __forceinline__ void append_candidate(const PushArgs& a, bool cand, int64_t k, float vx, float vy,
                                                 float vz, uint32_t id)
{
    const unsigned full = 0xffffffffu;
    const unsigned cand_mask = __ballot_sync(full, cand);
    if (cand_mask) {
        const int lane = threadIdx.x & 31;
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&a.cnt->ncand_par[a.slot], (unsigned long long)__popc(cand_mask));
        base = __shfl_sync(full, base, 0);
        if (cand) {
            const unsigned long long c = base + __popc(cand_mask & ((1u << lane) - 1u));
            a.cand[c] = (uint32_t)k;
            a.cand_rec[c] = make_float4(vx, vy, vz, __uint_as_float(id));
        }
    }
}

// VEC consecutive slots as one vector access (slots are allocated in
// multiples of kSlotAlign, so a group never runs past the arrays).
template <int VEC> struct Vec;
template <> struct Vec<1> {
    using U = uint32_t;
    using F = float;
    static __device__ __forceinline__ U ldu(const uint32_t* p, int64_t g) { return __ldcs(p + g); }
    static __device__ __forceinline__ F ldf(const float* p, int64_t g) { return __ldcs(p + g); }
    static __device__ __forceinline__ void stu(uint32_t* p, int64_t g, U v) { __stcs(p + g, v); }
    static __device__ __forceinline__ void stf(float* p, int64_t g, F v) { __stcs(p + g, v); }
    static __device__ __forceinline__ uint32_t& at(U& v, int) { return v; }
    static __device__ __forceinline__ float& at(F& v, int) { return v; }
};
template <> struct Vec<2> {
    using U = uint2;
    using F = float2;
    static __device__ __forceinline__ U ldu(const uint32_t* p, int64_t g) { return __ldcs((const uint2*)p + g); }
    static __device__ __forceinline__ F ldf(const float* p, int64_t g) { return __ldcs((const float2*)p + g); }
    static __device__ __forceinline__ void stu(uint32_t* p, int64_t g, U v) { __stcs((uint2*)p + g, v); }
    static __device__ __forceinline__ void stf(float* p, int64_t g, F v) { __stcs((float2*)p + g, v); }
    static __device__ __forceinline__ uint32_t& at(U& v, int j) { return j == 0 ? v.x : v.y; }
    static __device__ __forceinline__ float& at(F& v, int j) { return j == 0 ? v.x : v.y; }
};
template <> struct Vec<4> {
    using U = uint4;
    using F = float4;
    static __device__ __forceinline__ U ldu(const uint32_t* p, int64_t g) { return __ldcs((const uint4*)p + g); }
    static __device__ __forceinline__ F ldf(const float* p, int64_t g) { return __ldcs((const float4*)p + g); }
    static __device__ __forceinline__ void stu(uint32_t* p, int64_t g, U v) { __stcs((uint4*)p + g, v); }
    static __device__ __forceinline__ void stf(float* p, int64_t g, F v) { __stcs((float4*)p + g, v); }
    static __device__ __forceinline__ uint32_t& at(U& v, int j)
    {
        return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w;
    }
    static __device__ __forceinline__ float& at(F& v, int j) { return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w; }
};

// blocks of 256 per SM the register budget is set for: the 4-slot kernel fits
// 63 registers without spills, and 4 blocks (32 warps) issue faster than 3 at
// 80 registers (1e8 electrons: 1.57 against 1.61 ms; 5 blocks spill)
template <int VEC> constexpr int push_min_blocks() { return VEC == 4 ? 4 : VEC == 2 ? 3 : 4; }
// the batched kernel keeps the earlier budget (its 4-slot variant would spill at 64 registers)
template <int VEC> constexpr int batch_min_blocks() { return VEC == 4 ? 2 : VEC == 2 ? 3 : 4; }

// Persistent grid-stride kernel over groups of VEC consecutive slots: every
// load of a group (x, z, vx, vy, vz and, with collisions, id) is issued before
// any of its results is used, as streaming (evict-first) vector accesses, so
// that each thread keeps 20-24 VEC bytes in flight and the field faces stay in
// L1.  Collision candidates go to a compacted list (slot and post-push
// velocity and id) for k_collide, which runs the scatter of each
// (BaseSpecies::scatter after the push, as Species::advance does).  Counters
// are reduced per warp and added once at the end; thread 0 of block 0 first
// folds the previous launch's per-step counters into the totals.
template <int COORD, int EMODE, bool BFIELD, int VEC>
__global__ void __launch_bounds__(256, push_min_blocks<VEC>()) k_push(const __grid_constant__ PushArgs a)
{
    using V = Vec<VEC>;
    // launched with programmatic serialisation: everything of the previous
    // kernel is visible after this wait
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // a dependent k_collide may be scheduled and stage its tables now; it
    // waits for this whole grid before it reads any result
    asm volatile("griddepcontrol.launch_dependents;");
    if (a.fold_slot >= 0 && blockIdx.x == 0 && threadIdx.x == 0) {
        Counters* c = a.cnt;
        c->live_sum += c->live_par[a.fold_slot];
        c->live_par[a.fold_slot] = 0;
        c->ncand_par[a.fold_slot] = 0;
    }
    const int64_t n = a.n;
    const int64_t ngroups = (n + VEC - 1) / VEC;
    // each block takes one contiguous range of groups: particles sorted by
    // cell then keep a block's field faces and deposit nodes local (L1, L2)
    const int64_t per_block = ((ngroups + gridDim.x - 1) / gridDim.x + blockDim.x - 1) / blockDim.x * blockDim.x;
    const int64_t gbeg = (int64_t)blockIdx.x * per_block, gend = min(ngroups, gbeg + per_block);
    const bool coll = a.coll_threshold != 0u;
    // the deposit of a chunk (blockDim x VEC consecutive slots, sorted by
    // cell) goes to a shared tile anchored near the chunk's first particle,
    // which is added to the grid once per chunk
    __shared__ unsigned t_lo[kTileCopies * kTileStride], t_hi[kTileCopies * kTileStride];
    __shared__ int anchor[2][2];
    const bool tiled = a.rho != nullptr;
    if (tiled) {
        for (int t = threadIdx.x; t < kTileCopies * kTileStride; t += blockDim.x) t_lo[t] = t_hi[t] = 0u;
        if (threadIdx.x == 0) anchor[1][0] = anchor[1][1] = 0;
    }
    unsigned live = 0, removed = 0;
    int par = 0;
    for (int64_t g0 = gbeg; g0 < gend; g0 += blockDim.x, par ^= 1) {
        const int64_t g = g0 + threadIdx.x;
        const bool act = g < gend;
        typename V::U X{}, Z{}, ID{};
        typename V::F VX{}, VY{}, VZ{};
        if (act) {
            X = V::ldu(a.x, g);
            Z = V::ldu(a.z, g);
            VX = V::ldf(a.vx, g);
            VY = V::ldf(a.vy, g);
            VZ = V::ldf(a.vz, g);
            if (coll) ID = V::ldu(a.id, g);
        }
        TileDeposit dep{t_lo, t_hi, 0, 0, GlobalDeposit{a.rho, a.nz}};
        if (tiled) {
            if (threadIdx.x == 0) {
                const uint32_t x0 = V::at(X, 0), z0 = V::at(Z, 0);
                if (act && x0 != kDead) {
                    anchor[par][0] = min((int)(x0 >> kFracBits), a.nx - 2) - 2;
                    anchor[par][1] = min((int)(z0 >> kFracBits), a.nz - 2) - kTileCols / 4;
                } else {
                    anchor[par][0] = anchor[par ^ 1][0];
                    anchor[par][1] = anchor[par ^ 1][1];
                }
            }
            __syncthreads();
            dep.ai = anchor[par][0];
            dep.aj = anchor[par][1];
        }
        bool cand[VEC];
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            cand[j] = false;
            const int64_t k = g * VEC + j;
            uint32_t& x = V::at(X, j);
            if (!act || k >= n || x == kDead) continue;
            bool al;
            step_particle<COORD, EMODE, BFIELD, TileDeposit>(a, x, V::at(Z, j), V::at(VX, j), V::at(VY, j),
                                                             V::at(VZ, j), V::at(ID, j), a.step, a.phase, al,
                                                             cand[j], dep);
            if (!al) x = kDead;
            live += al;
            removed += !al;
        }
        if (tiled) {
            __syncthreads();
            for (int t = threadIdx.x; t < kTileRows * kTileCols; t += blockDim.x) {
                unsigned long long sum = 0;
#pragma unroll
                for (int c = 0; c < kTileCopies; ++c) {
                    const int q = c * kTileStride + t;
                    sum += ((unsigned long long)t_hi[q] << 20) + t_lo[q];
                    t_lo[q] = t_hi[q] = 0u;
                }
                if (sum) {
                    const int i = dep.ai + t / kTileCols, jj = dep.aj + t % kTileCols;
                    atomicAdd(a.rho + (size_t)i * a.nz + jj, sum);
                }
            }
        }
        if (act) {
            V::stu(a.x, g, X);
            V::stu(a.z, g, Z);
            V::stf(a.vx, g, VX);
            V::stf(a.vy, g, VY);
            V::stf(a.vz, g, VZ);
        }
        if (coll) {
#pragma unroll
            for (int j = 0; j < VEC; ++j)
                append_candidate(a, cand[j], g * VEC + j, V::at(VX, j), V::at(VY, j), V::at(VZ, j), V::at(ID, j));
        }
    }
    const unsigned full = 0xffffffffu;
    live = __reduce_add_sync(full, live);
    removed = __reduce_add_sync(full, removed);
    if ((threadIdx.x & 31) == 0) {
        if (live) atomicAdd(&a.cnt->live_par[a.slot], (unsigned long long)live);
        if (removed) atomicAdd(&a.cnt->removed, (unsigned long long)removed);
    }
}

// Several steps of one species in one launch, for runs whose particles do not
// interact within those steps: no self-consistent field (the field is the
// static plus RF one, or the uniform external one), no sort in between, and
// collision targets that are Maxwellian backgrounds only.  Every particle is
// then independent of the others, and its state stays in registers for all
// steps: step k is step_particle with the species' step counter step0 + k and
// that step's RF factor, and a fired collision test is scattered at once with
// the same random stream k_collide would use (collide_background), so the
// result is bit-identical to the same steps launched one by one.
// (inlined, with no address-taken arguments: as a call it made the loop keep
// its values in callee-saved registers, 80 of them with spills around the
// call, and the fused launch ran 9 % slower on the 22-pole workload)
struct ScatterOut {
    int r;
    float vx, vy, vz;
};
__device__ __forceinline__ ScatterOut fused_scatter(const MccSpecies& m, uint64_t seed, uint32_t species, uint32_t id,
                                                 uint64_t step, float vx0, float vy0, float vz0)
{
    ScatterOut o{0, vx0, vy0, vz0};
    o.r = collide_background(m, seed, species, id, step, o.vx, o.vy, o.vz);
    if (o.r != MCC_HIT) {
        o.vx = vx0;
        o.vy = vy0;
        o.vz = vz0;
    }
    return o;
}

template <int COORD, int EMODE, bool BFIELD>
__global__ void __launch_bounds__(256, 3) k_push_fused(const __grid_constant__ PushArgs a,
                                                    const __grid_constant__ CollideArgs c,
                                                    const __grid_constant__ FusedSteps fs)
{
    __shared__ MccStage st;
    extern __shared__ double s_tab[];
    const bool coll = a.coll_threshold != 0u;
    if (coll) {
        double* tab = c.n_tables <= kStageTables ? s_tab : nullptr;
        mcc_stage(c, st, tab);
        __syncthreads();
        if (threadIdx.x == 0) mcc_stage_pointers(c, st, tab);
    }
    __syncthreads();
    // launched with programmatic serialisation: the collision tables (set-up
    // data) are staged while the previous kernel finishes; its results are
    // read only after this wait
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (a.fold_slot >= 0 && blockIdx.x == 0 && threadIdx.x == 0) {
        Counters* cn = a.cnt;
        cn->live_sum += cn->live_par[a.fold_slot];
        cn->live_par[a.fold_slot] = 0;
        cn->ncand_par[a.fold_slot] = 0;
    }
    const int K = fs.nsteps;
    unsigned live = 0, removed = 0, ncoll = 0, nnull = 0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < a.n; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t x = __ldcs(a.x + k);
        if (x == kDead) continue;
        uint32_t z = __ldcs(a.z + k);
        float vx = __ldcs(a.vx + k), vy = __ldcs(a.vy + k), vz = __ldcs(a.vz + k);
        const uint32_t id = coll ? __ldcs(a.id + k) : 0u;
#pragma unroll 1
        for (int q = 0; q < K; ++q) {
            bool al, cand;
            step_particle<COORD, EMODE, BFIELD, NoDeposit>(a, x, z, vx, vy, vz, id, a.step + q, fs.phase[q], al, cand,
                                                           NoDeposit{});
            if (!al) {
                x = kDead;
                ++removed;
                break;
            }
            ++live;
            if (cand) {
                const ScatterOut o = fused_scatter(st.m, a.seed, a.species, id, a.step + q, vx, vy, vz);
                vx = o.vx;
                vy = o.vy;
                vz = o.vz;
                ncoll += o.r == MCC_HIT;
                nnull += o.r != MCC_HIT;
            }
        }
        __stcs(a.x + k, x);
        __stcs(a.z + k, z);
        __stcs(a.vx + k, vx);
        __stcs(a.vy + k, vy);
        __stcs(a.vz + k, vz);
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
}

// Particle step of many independent instances in one launch (batched runs).
// Work item i is one species of one instance (arguments args[i]); its slots
// are cut into chunks of kBatchIters x 256 x VEC slots and chunk_off[i] is the
// first chunk of item i (chunk_off[nitems] = all chunks).  A persistent grid
// takes chunks in turn; the block stages the item's arguments in shared memory
// and runs the loop body of k_push over the chunk.
constexpr int kBatchIters = 4;

template <int COORD, int EMODE, bool BFIELD, int VEC>
__global__ void __launch_bounds__(256, batch_min_blocks<VEC>())
    k_push_batch(const PushArgs* __restrict__ args, const unsigned* __restrict__ chunk_off, int nitems)
{
    using V = Vec<VEC>;
    __shared__ __align__(16) unsigned char raw[sizeof(PushArgs)];
    __shared__ int s_item;
    static_assert(sizeof(PushArgs) % 8 == 0, "word copy");
    const PushArgs& a = *reinterpret_cast<const PushArgs*>(raw);
    const unsigned nchunks = chunk_off[nitems];
    const unsigned full = 0xffffffffu;
    for (unsigned c = blockIdx.x; c < nchunks; c += gridDim.x) {
        __syncthreads();  // the previous chunk is done with the staged arguments
        if (threadIdx.x == 0) {
            int lo = 0, hi = nitems - 1;  // last item whose first chunk is <= c
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (chunk_off[mid] <= c) lo = mid;
                else hi = mid - 1;
            }
            s_item = lo;
        }
        __syncthreads();
        const int item = s_item;
        {
            const unsigned long long* src = reinterpret_cast<const unsigned long long*>(args + item);
            unsigned long long* dst = reinterpret_cast<unsigned long long*>(raw);
            for (int w = threadIdx.x; w < (int)(sizeof(PushArgs) / 8); w += blockDim.x) dst[w] = src[w];
        }
        __syncthreads();
        const unsigned first = chunk_off[item];
        if (c == first && a.fold_slot >= 0 && threadIdx.x == 0) {
            Counters* cn = a.cnt;
            cn->live_sum += cn->live_par[a.fold_slot];
            cn->live_par[a.fold_slot] = 0;
            cn->ncand_par[a.fold_slot] = 0;
        }
        const int64_t n = a.n;
        const int64_t ngroups = (n + VEC - 1) / VEC;
        const bool coll = a.coll_threshold != 0u;
        unsigned live = 0, removed = 0;
        const int64_t g0 = (int64_t)(c - first) * kBatchIters * blockDim.x;
#pragma unroll 1
        for (int it = 0; it < kBatchIters; ++it) {
            const int64_t g = g0 + (int64_t)it * blockDim.x + threadIdx.x;
            if (g - threadIdx.x >= ngroups) break;
            const bool act = g < ngroups;
            typename V::U X{}, Z{}, ID{};
            typename V::F VX{}, VY{}, VZ{};
            if (act) {
                X = V::ldu(a.x, g);
                Z = V::ldu(a.z, g);
                VX = V::ldf(a.vx, g);
                VY = V::ldf(a.vy, g);
                VZ = V::ldf(a.vz, g);
                if (coll) ID = V::ldu(a.id, g);
            }
            bool cand[VEC];
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                cand[j] = false;
                const int64_t k = g * VEC + j;
                uint32_t& x = V::at(X, j);
                if (!act || k >= n || x == kDead) continue;
                bool al;
                step_particle<COORD, EMODE, BFIELD, GlobalDeposit>(a, x, V::at(Z, j), V::at(VX, j), V::at(VY, j),
                                                                   V::at(VZ, j), V::at(ID, j), a.step, a.phase, al,
                                                                   cand[j], GlobalDeposit{a.rho, a.nz});
                if (!al) x = kDead;
                live += al;
                removed += !al;
            }
            if (act) {
                V::stu(a.x, g, X);
                V::stu(a.z, g, Z);
                V::stf(a.vx, g, VX);
                V::stf(a.vy, g, VY);
                V::stf(a.vz, g, VZ);
            }
            if (coll) {
#pragma unroll
                for (int j = 0; j < VEC; ++j)
                    append_candidate(a, cand[j], g * VEC + j, V::at(VX, j), V::at(VY, j), V::at(VZ, j),
                                     V::at(ID, j));
            }
        }
        live = __reduce_add_sync(full, live);
        removed = __reduce_add_sync(full, removed);
        if ((threadIdx.x & 31) == 0) {
            if (live) atomicAdd(&a.cnt->live_par[a.slot], (unsigned long long)live);
            if (removed) atomicAdd(&a.cnt->removed, (unsigned long long)removed);
        }
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
    rotate<COORD>(vx, vy, vz, boris_vectors(a, x, z));
    vx = fmaf(ex, a.hq, vx);
    vz = fmaf(ez, a.hq, vz);
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

// Persistent launch: as many blocks as fit on the device at once (occupancy of
// this instantiation x SMs), reduced so that every thread runs the same number
// of grid-stride iterations.
template <int COORD, int EMODE, bool BFIELD, int VEC>
void launch_step(const PushArgs& a, int sm_count, cudaStream_t s)
{
    static int per_sm = 0;  // resident blocks per SM of this instantiation
    if (per_sm == 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_push<COORD, EMODE, BFIELD, VEC>, 256, 0) !=
                cudaSuccess ||
            b < 1)
            b = 1;
        per_sm = b;
    }
    const int64_t groups = (a.n + VEC - 1) / VEC;
    const int64_t resident = (int64_t)per_sm * std::max(sm_count, 1);
    const int64_t needed = (groups + 255) / 256;
    const int64_t iters = (needed + resident - 1) / resident;
    const unsigned grid = (unsigned)std::max<int64_t>(1, (needed + iters - 1) / iters);
    // programmatic stream serialisation: the blocks are scheduled while the
    // previous kernel (the face field of the solve) finishes, and wait for it
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_push<COORD, EMODE, BFIELD, VEC>, a);
}

template <int COORD, int EMODE, bool BFIELD>
void launch_step_vec(const PushArgs& a, int vec, int sm_count, cudaStream_t s)
{
    switch (vec) {
    case 1: launch_step<COORD, EMODE, BFIELD, 1>(a, sm_count, s); break;
    case 2: launch_step<COORD, EMODE, BFIELD, 2>(a, sm_count, s); break;
    default: launch_step<COORD, EMODE, BFIELD, 4>(a, sm_count, s); break;
    }
}

template <int COORD, int EMODE>
void launch_push_e(const PushArgs& a, bool init, int vec, int sm_count, cudaStream_t s)
{
    if (init) {
        k_push_init<COORD, EMODE><<<(unsigned)((a.n + 255) / 256), 256, 0, s>>>(a);
        return;
    }
    if (a.has_b) launch_step_vec<COORD, EMODE, true>(a, vec, sm_count, s);
    else launch_step_vec<COORD, EMODE, false>(a, vec, sm_count, s);
}

template <int COORD>
void launch_push_t(const PushArgs& a, bool init, int vec, int sm_count, cudaStream_t s)
{
    switch (a.emode) {
    case 0: launch_push_e<COORD, 0>(a, init, vec, sm_count, s); break;
    case 1: launch_push_e<COORD, 1>(a, init, vec, sm_count, s); break;
    default: launch_push_e<COORD, 2>(a, init, vec, sm_count, s); break;
    }
}

template <int COORD, int EMODE, bool BFIELD>
void launch_fused_t(const PushArgs& a, const CollideArgs& c, const FusedSteps& fs, int sm_count, cudaStream_t s)
{
    static int per_sm = 0;
    const size_t smem = a.coll_threshold != 0u && c.n_tables <= kStageTables ? (size_t)c.n_tables * sizeof(double) : 0;
    if (per_sm == 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_push_fused<COORD, EMODE, BFIELD>, 256,
                                                          kStageTables * sizeof(double)) != cudaSuccess ||
            b < 1)
            b = 1;
        per_sm = b;
    }
    const int64_t needed = (a.n + 255) / 256;
    const int64_t resident = (int64_t)per_sm * std::max(sm_count, 1);
    const int64_t iters = (needed + resident - 1) / resident;
    const unsigned grid = (unsigned)std::max<int64_t>(1, (needed + iters - 1) / iters);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_push_fused<COORD, EMODE, BFIELD>, a, c, fs);
}

template <int COORD, int EMODE>
void launch_fused_e(const PushArgs& a, const CollideArgs& c, const FusedSteps& fs, int sm_count, cudaStream_t s)
{
    if (a.has_b) launch_fused_t<COORD, EMODE, true>(a, c, fs, sm_count, s);
    else launch_fused_t<COORD, EMODE, false>(a, c, fs, sm_count, s);
}

template <int COORD>
void launch_fused_c(const PushArgs& a, const CollideArgs& c, const FusedSteps& fs, int sm_count, cudaStream_t s)
{
    switch (a.emode) {
    case 0: launch_fused_e<COORD, 0>(a, c, fs, sm_count, s); break;
    case 1: launch_fused_e<COORD, 1>(a, c, fs, sm_count, s); break;
    default: launch_fused_e<COORD, 2>(a, c, fs, sm_count, s); break;
    }
}

// ---- adjoint of the particle step ----------------------------------------
//
// Reverse-mode derivative of step_particle (collisionless, constant B, field
// from the potential faces) and of the leapfrog start, for the adjoint runs.
// The forward quantities are recomputed from the stored state before the
// step; positions are continuous in the derivative (the fixed-point rounding
// of a move passes the adjoint through unchanged).  Derivatives are FP32.

struct Vec3 {
    float x, y, z;
};
__device__ __forceinline__ Vec3 cross3(Vec3 a, Vec3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ Vec3 add3(Vec3 a, Vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ Vec3 scale3(float k, Vec3 a) { return {k * a.x, k * a.y, k * a.z}; }
__device__ __forceinline__ float dot3(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// field at the particle with its derivatives in cells, and the stencil for the adjoint scatter
struct GatherD {
    GatherIdx g;
    float ex, ez, dex_dr, dex_dz, dez_dr, dez_dz;
};
template <int EMODE>
__device__ __forceinline__ GatherD gather_E_d(const PushArgs& a, uint32_t x, uint32_t z)
{
    GatherD G{};
    if (EMODE == 0) {
        G.ez = a.extern_ez;
        return G;
    }
    G.g = gather_idx(x, z, a.nx, a.nz);
    const GatherIdx& g = G.g;
    {
        const float* p = a.Exf + (size_t)g.ix * a.nz + g.jz;
        const float A = p[0], B = p[1], C = p[a.nz], D = p[a.nz + 1];
        G.ex = lerp4(A, B, C, D, g.fx, g.fz);
        G.dex_dr = (1.f - g.fz) * (C - A) + g.fz * (D - B);
        G.dex_dz = (1.f - g.fx) * (B - A) + g.fx * (D - C);
    }
    {
        const int st = a.nz + 1;
        const float* p = a.Ezf + (size_t)g.iz * st + g.jz2;
        const float A = p[0], B = p[1], C = p[st], D = p[st + 1];
        G.ez = lerp4(A, B, C, D, g.gx, g.gz);
        G.dez_dr = (1.f - g.gz) * (C - A) + g.gz * (D - B);
        G.dez_dz = (1.f - g.gx) * (B - A) + g.gx * (D - C);
    }
    return G;
}

template <int EMODE>
__device__ __forceinline__ void scatter_lE(const PushArgs& a, const AdjPushArgs& d, const GatherIdx& g, float lex,
                                           float lez)
{
    if (EMODE == 0) return;
    float* p = d.lExf + (size_t)g.ix * a.nz + g.jz;
    atomicAdd(p, (1.f - g.fx) * (1.f - g.fz) * lex);
    atomicAdd(p + 1, (1.f - g.fx) * g.fz * lex);
    atomicAdd(p + a.nz, g.fx * (1.f - g.fz) * lex);
    atomicAdd(p + a.nz + 1, g.fx * g.fz * lex);
    const int st = a.nz + 1;
    float* q = d.lEzf + (size_t)g.iz * st + g.jz2;
    atomicAdd(q, (1.f - g.gx) * (1.f - g.gz) * lez);
    atomicAdd(q + 1, (1.f - g.gx) * g.gz * lez);
    atomicAdd(q + st, g.gx * (1.f - g.gz) * lez);
    atomicAdd(q + st + 1, g.gx * g.gz * lez);
}

template <int COORD, int EMODE>
__global__ void __launch_bounds__(256) k_adj_push(const __grid_constant__ PushArgs a,
                                                  const __grid_constant__ AdjPushArgs d)
{
    const float sg = COORD == 1 ? 1.f : -1.f;  // p = v + sg v x t, v' = v + sg p x s (rotate<COORD>)
    const Vec3 t{a.tx, a.ty, a.tz}, s{a.sx, a.sy, a.sz};
    float lb0 = 0.f, lb1 = 0.f, lb2 = 0.f;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < d.n; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t x = d.x0[k];
        if (x == kDead) continue;
        if (!d.init && d.x1[k] == kDead) {  // removed during the step: the loss no longer depends on it
            d.lr[k] = d.lz[k] = d.lvx[k] = d.lvy[k] = d.lvz[k] = 0.f;
            continue;
        }
        const uint32_t z = d.z0[k];
        const Vec3 v{d.vx0[k], d.vy0[k], d.vz0[k]};
        const GatherD G = gather_E_d<EMODE>(a, x, z);
        float lr = d.lr[k], lz = d.lz[k];
        Vec3 lv{d.lvx[k], d.lvy[k], d.lvz[k]};
        float lex = 0.f, lez = 0.f;
        Vec3 v1 = v;
        if (!d.init) {
            v1.x += a.hq * G.ex;
            v1.z += a.hq * G.ez;
        }
        const Vec3 p = add3(v1, scale3(sg, cross3(v1, t)));
        Vec3 l2;  // adjoint of the rotated velocity
        if (d.init) {
            // v0 = rot(v_in) + hq E: no move
            l2 = lv;
            lex += a.hq * lv.x;
            lez += a.hq * lv.z;
        } else {
            const Vec3 v2 = add3(v1, scale3(sg, cross3(p, s)));
            Vec3 v3 = v2;
            v3.x += a.hq * G.ex;
            v3.z += a.hq * G.ez;
            Vec3 l3;
            if (COORD == 1) {
                const float r = cells(x);
                const float ax = v3.x * a.cx, by = v3.y * a.cx;
                const float x2 = r + ax;
                const float rn = sqrtf(x2 * x2 + by * by);
                float ca = 1.f, sa = 0.f, ir3 = 0.f;
                if (rn > 0.f) {
                    ca = x2 / rn;
                    sa = by / rn;
                    ir3 = 1.f / (rn * rn * rn);
                }
                // outputs: r' = rn, z' = z + v3z cz, v4 = (ca v3x + sa v3y, -sa v3x + ca v3y, v3z)
                const float lca = v3.x * lv.x + v3.y * lv.y, lsa = v3.y * lv.x - v3.x * lv.y;
                l3.x = ca * lv.x - sa * lv.y;
                l3.y = sa * lv.x + ca * lv.y;
                l3.z = lv.z + lz * a.cz;
                const float lx2 = lr * ca + (lca * by * by - lsa * by * x2) * ir3;
                const float lby = lr * sa + (-lca * x2 * by + lsa * x2 * x2) * ir3;
                lr = lx2;
                l3.x += lx2 * a.cx;
                l3.y += lby * a.cx;
            } else {
                // outputs: x' = x + v3x cx, z' = z + v3z cz, v3
                l3.x = lv.x + lr * a.cx;
                l3.y = lv.y;
                l3.z = lv.z + lz * a.cz;
            }
            l2 = l3;
            lex += a.hq * l3.x;
            lez += a.hq * l3.z;
        }
        // rotation: v2 = v1 + sg p x s, p = v1 + sg v1 x t
        const Vec3 lp = scale3(sg, cross3(s, l2));
        Vec3 lv1 = add3(add3(l2, lp), scale3(sg, cross3(t, lp)));
        const Vec3 ls = scale3(sg, cross3(l2, p));
        Vec3 lt = scale3(sg, cross3(lp, v1));
        const float f = 2.f / (1.f + dot3(t, t));
        lt = add3(lt, add3(scale3(f, ls), scale3(-f * f * dot3(ls, t), t)));
        lb0 += a.q_dt_2m * lt.x;
        lb1 += a.q_dt_2m * lt.y;
        lb2 += a.q_dt_2m * lt.z;
        if (!d.init) {
            lex += a.hq * lv1.x;
            lez += a.hq * lv1.z;
        }
        // gather: E depends on the position before the step
        lr += lex * G.dex_dr + lez * G.dez_dr;
        lz += lex * G.dex_dz + lez * G.dez_dz;
        scatter_lE<EMODE>(a, d, G.g, lex, lez);
        d.lr[k] = lr;
        d.lz[k] = lz;
        d.lvx[k] = lv1.x;
        d.lvy[k] = lv1.y;
        d.lvz[k] = lv1.z;
    }
    const unsigned full = 0xffffffffu;
    for (int o = 16; o > 0; o >>= 1) {
        lb0 += __shfl_xor_sync(full, lb0, o);
        lb1 += __shfl_xor_sync(full, lb1, o);
        lb2 += __shfl_xor_sync(full, lb2, o);
    }
    if ((threadIdx.x & 31) == 0 && d.lB) {
        atomicAdd(&d.lB[0], (double)lb0);
        atomicAdd(&d.lB[1], (double)lb1);
        atomicAdd(&d.lB[2], (double)lb2);
    }
}

template <int COORD, int EMODE, bool BFIELD, int VEC>
void launch_batch_t(const PushArgs* d_args, const unsigned* d_chunk_off, int nitems, int sm_count, cudaStream_t s)
{
    static int per_sm = 0;
    if (per_sm == 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_push_batch<COORD, EMODE, BFIELD, VEC>, 256, 0) !=
                cudaSuccess ||
            b < 1)
            b = 1;
        per_sm = b;
    }
    k_push_batch<COORD, EMODE, BFIELD, VEC><<<per_sm * std::max(sm_count, 1), 256, 0, s>>>(d_args, d_chunk_off, nitems);
}

template <int COORD, int EMODE, bool BFIELD>
void launch_batch_v(const PushArgs* d_args, const unsigned* d_off, int nitems, int vec, int sm, cudaStream_t s)
{
    switch (vec) {
    case 1: launch_batch_t<COORD, EMODE, BFIELD, 1>(d_args, d_off, nitems, sm, s); break;
    case 2: launch_batch_t<COORD, EMODE, BFIELD, 2>(d_args, d_off, nitems, sm, s); break;
    default: launch_batch_t<COORD, EMODE, BFIELD, 4>(d_args, d_off, nitems, sm, s); break;
    }
}

template <int COORD, int EMODE>
void launch_batch_b(const PushArgs* d_args, const unsigned* d_off, int nitems, bool has_b, int vec, int sm,
                    cudaStream_t s)
{
    if (has_b) launch_batch_v<COORD, EMODE, true>(d_args, d_off, nitems, vec, sm, s);
    else launch_batch_v<COORD, EMODE, false>(d_args, d_off, nitems, vec, sm, s);
}

template <int COORD>
void launch_batch_e(const PushArgs* d_args, const unsigned* d_off, int nitems, int emode, bool has_b, int vec,
                    int sm, cudaStream_t s)
{
    switch (emode) {
    case 0: launch_batch_b<COORD, 0>(d_args, d_off, nitems, has_b, vec, sm, s); break;
    case 1: launch_batch_b<COORD, 1>(d_args, d_off, nitems, has_b, vec, sm, s); break;
    default: launch_batch_b<COORD, 2>(d_args, d_off, nitems, has_b, vec, sm, s); break;
    }
}

}  // namespace

int push_batch_chunk(int vec) { return kBatchIters * 256 * vec; }

int launch_push_batch(const PushArgs* d_args, const unsigned* d_chunk_off, int nitems, int coord, int emode,
                      bool has_b, int vec, int sm_count, cudaStream_t s)
{
    if (nitems <= 0) return 0;
    if (coord == 1) launch_batch_e<1>(d_args, d_chunk_off, nitems, emode, has_b, vec, sm_count, s);
    else launch_batch_e<0>(d_args, d_chunk_off, nitems, emode, has_b, vec, sm_count, s);
    return 1;
}

int launch_adj_push(const PushArgs& a, const AdjPushArgs& d, int coord, cudaStream_t s)
{
    if (d.n == 0) return 0;
    const unsigned grid = (unsigned)std::min<int64_t>((d.n + 255) / 256, 152 * 8);
    const int em = a.emode == 0 ? 0 : 1;
    if (coord == 1) {
        if (em == 0) k_adj_push<1, 0><<<grid, 256, 0, s>>>(a, d);
        else k_adj_push<1, 1><<<grid, 256, 0, s>>>(a, d);
    } else {
        if (em == 0) k_adj_push<0, 0><<<grid, 256, 0, s>>>(a, d);
        else k_adj_push<0, 1><<<grid, 256, 0, s>>>(a, d);
    }
    return 1;
}

int launch_push(const PushArgs& a, int coord, bool init, int vec, int sm_count, cudaStream_t s)
{
    if (a.n == 0) return 0;
    if (coord == 1) launch_push_t<1>(a, init, vec, sm_count, s);
    else launch_push_t<0>(a, init, vec, sm_count, s);
    return 1;
}

int launch_push_fused(const PushArgs& a, const CollideArgs& c, const FusedSteps& fs, int coord, int sm_count,
                      cudaStream_t s)
{
    if (a.n == 0 || fs.nsteps <= 0) return 0;
    if (coord == 1) launch_fused_c<1>(a, c, fs, sm_count, s);
    else launch_fused_c<0>(a, c, fs, sm_count, s);
    return 1;
}

int launch_deposit(const PushArgs& a, cudaStream_t s)
{
    if (a.n == 0) return 0;
    k_deposit<<<(unsigned)((a.n + 255) / 256), 256, 0, s>>>(a);
    return 1;
}

}  // namespace mag
