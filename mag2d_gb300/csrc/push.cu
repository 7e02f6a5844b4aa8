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
// The scatter itself (uni() < prob -> BaseSpecies::scatter) is deferred to
// the collide kernel through a compacted candidate list; scattering changes
// only velocities, so boundary and deposit, which read positions only, give
// the same result as in the reference's order.
//
// HBM traffic per live particle and step: read x, z, vx, vy, vz (20 B) and,
// when collisions are on, id (4 B); write x, z, vx, vy, vz (20 B).  Field
// faces, mask and the charge grid are small and stay in L2.
#include "device.hpp"
#include "kernels.hpp"
#include "philox.hpp"

namespace mag {

namespace {

__device__ __forceinline__ float bilerp(const float* __restrict__ f, int stride, int i, int j, float fx, float fz)
{
    const float* p = f + (size_t)i * stride + j;
    const float a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + stride), d = __ldg(p + stride + 1);
    return (1.f - fx) * ((1.f - fz) * a + fz * b) + fx * ((1.f - fz) * c + fz * d);
}

// E at grid position (xg, zg) from face arrays (Field2D::grad with the sign of Fields::E)
__device__ __forceinline__ void gather_faces(const float* __restrict__ Exf, const float* __restrict__ Ezf, int nx,
                                             int nz, float xg, float zg, float& ex, float& ez)
{
    int ix = (int)(xg + 0.5f);
    ix = max(0, min(ix, nx - 1));
    int jz = max(0, min((int)zg, nz - 2));
    ex = bilerp(Exf, nz, ix, jz, xg + 0.5f - (float)ix, zg - (float)jz);
    int ix2 = max(0, min((int)xg, nx - 2));
    int jz2 = (int)(zg + 0.5f);
    jz2 = max(0, min(jz2, nz - 1));
    ez = bilerp(Ezf, nz + 1, ix2, jz2, xg - (float)ix2, zg + 0.5f - (float)jz2);
}

// Field2D::interpolate of a B table at physical position (x, z)
__device__ __forceinline__ float table_interp(const float* __restrict__ t, int bnx, int bnz, float xi, float zi)
{
    int i = max(0, min((int)xi, bnx - 2));
    int j = max(0, min((int)zi, bnz - 2));
    return bilerp(t, bnz, i, j, xi - (float)i, zi - (float)j);
}

__device__ __forceinline__ double mod_phase(double x, double y)  // src/mymath.cpp:62-67
{
    if (x >= 0.0 && x <= y) return x;
    return x - y * (double)(int)(x / y) + (x < 0 ? y : 0);
}

template <int COORD, int EMODE>
__global__ void __launch_bounds__(256) k_push(const PushArgs a)
{
    __shared__ float s_phase;
    if (EMODE == 2) {
        if (threadIdx.x == 0) {
            const double t = (double)a.cnt->niter * a.dt;
            s_phase = (float)(a.rf_amp * cos(mod_phase(a.rf_omega * t, 10000000 * M_PI)) + a.rf_U0);
        }
        __syncthreads();
    }
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in_range = k < a.n;
    float xg = in_range ? a.x[k] : kDeadX;
    const bool was_alive = xg >= 0.f;
    bool alive = was_alive;
    bool cand = false;
    if (was_alive) {
        float zg = a.z[k];
        float vx = a.vx[k], vy = a.vy[k], vz = a.vz[k];
        float ex, ez;
        if (EMODE == 0) {
            ex = 0.f;
            ez = a.extern_ez;
        } else {
            gather_faces(a.Exf, a.Ezf, a.nx, a.nz, xg, zg, ex, ez);
            if (EMODE == 2) {
                float rx, rz;
                gather_faces(a.Exf_rf, a.Ezf_rf, a.nx, a.nz, xg, zg, rx, rz);
                ex += s_phase * rx;
                ez += s_phase * rz;
            }
        }
        float tx = a.tx, ty = a.ty, tz = a.tz, sx = a.sx, sy = a.sy, sz = a.sz;
        if (a.btab) {
            const float xi = (xg * a.gdx + a.gx0 - a.b_x0) * a.b_ix;
            const float zi = (zg * a.gdz + a.gz0 - a.b_z0) * a.b_iz;
            tx = table_interp(a.Br, a.bnx, a.bnz, xi, zi) * a.q_dt_2m;
            tz = table_interp(a.Bz, a.bnx, a.bnz, xi, zi) * a.q_dt_2m;
            ty = 0.f;
            const float f = 2.f / (1.f + tx * tx + ty * ty + tz * tz);
            sx = tx * f;
            sy = ty * f;
            sz = tz * f;
        }
        // half acceleration, Boris rotation (Birdsall & Langdon), half acceleration
        vx += ex * a.hq;
        vz += ez * a.hq;
        if (COORD == 1) {
            const float vpr = vx + vy * tz - vz * ty;
            const float vpt = vy + vz * tx - vx * tz;
            const float vpz = vz + vx * ty - vy * tx;
            vx += vpt * sz - vpz * sy;
            vy += vpz * sx - vpr * sz;
            vz += vpr * sy - vpt * sx;
        } else {
            const float vpr = vx - vy * tz + vz * ty;
            const float vpz = vz - vx * ty + vy * tx;
            const float vpt = vy - vz * tx + vx * tz;
            vx += -vpt * sz + vpz * sy;
            vy += -vpz * sx + vpr * sz;
            vz += -vpr * sy + vpt * sx;
        }
        vx += ex * a.hq;
        vz += ez * a.hq;
        if (COORD == 1) {
            // push in the local Cartesian frame, map back to r and rotate v (Birdsall p. 338)
            const float x2 = xg + vx * a.cx;
            const float y2 = vy * a.cx;
            const float r = sqrtf(x2 * x2 + y2 * y2);
            zg += vz * a.cz;
            float sa = 0.f, ca = 1.f;
            if (r != 0.f) {
                const float ir = 1.f / r;
                sa = y2 * ir;
                ca = x2 * ir;
            }
            const float t0 = vx;
            vx = ca * vx + sa * vy;
            vy = -sa * t0 + ca * vy;
            xg = r;
        } else {
            xg += vx * a.cx;
            zg += vz * a.cz;
        }
        // boundary (advance_boundary): outside the box -> removed, or wrapped if PERIODIC
        if (!(xg >= 0.f && xg <= a.xmaxg && zg >= 0.f && zg <= a.zmaxg)) {
            if (a.periodic && isfinite(xg) && isfinite(zg)) {
                xg = fmodf(xg, a.xmaxg);
                if (xg < 0.f) xg += a.xmaxg;
                zg = fmodf(zg, a.zmaxg);
                if (zg < 0.f) zg += a.zmaxg;
            } else {
                alive = false;
            }
        }
        int ic = 0, jc = 0;
        if (alive) {
            ic = min((int)xg, a.nx - 2);
            jc = min((int)zg, a.nz - 2);
        }
        if (alive && a.check_mask) {
            const int8_t* m = a.mask + (size_t)ic * a.nz + jc;
            const bool fr = m[0] == 2 || m[a.nz] == 2 || m[1] == 2 || m[a.nz + 1] == 2;  // FREE
            if (!fr) alive = false;
        }
        if (alive && a.rho != nullptr) {
            const unsigned long long one = 1ull << kDepositShift;
            const unsigned long long U = (unsigned long long)((xg - (float)ic) * (float)(1 << kDepositShift));
            const unsigned long long V = (unsigned long long)((zg - (float)jc) * (float)(1 << kDepositShift));
            unsigned long long* r0 = a.rho + (size_t)ic * a.nz + jc;
            atomicAdd(r0, (one - U) * (one - V));
            atomicAdd(r0 + a.nz, U * (one - V));
            atomicAdd(r0 + 1, (one - U) * V);
            atomicAdd(r0 + a.nz + 1, U * V);
        }
        if (alive && a.coll_threshold != 0u) {
            const U4 r = draw(a.seed, a.species, a.id[k], a.cnt->niter, TAG_COLLIDE_TEST, 0);
            cand = r.x < a.coll_threshold;
        }
        a.x[k] = alive ? xg : kDeadX;
        a.z[k] = zg;
        a.vx[k] = vx;
        a.vy[k] = vy;
        a.vz[k] = vz;
    }
    // warp-aggregated counters and candidate append
    const unsigned full = 0xffffffffu;
    const unsigned live_mask = __ballot_sync(full, alive);
    const unsigned rem_mask = __ballot_sync(full, was_alive && !alive);
    const unsigned cand_mask = __ballot_sync(full, cand);
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        if (live_mask) atomicAdd(&a.cnt->live_step, (unsigned long long)__popc(live_mask));
        if (rem_mask) atomicAdd(&a.cnt->removed, (unsigned long long)__popc(rem_mask));
    }
    if (cand_mask) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&a.cnt->ncand, (unsigned long long)__popc(cand_mask));
        base = __shfl_sync(full, base, 0);
        if (cand) a.cand[base + __popc(cand_mask & ((1u << lane) - 1u))] = (uint32_t)k;
    }
}

// Leapfrog start (advance_boris_init, src/particles.cpp:623-679, :997-1050):
// a backward half rotation and a backward half acceleration, no move.
template <int COORD, int EMODE>
__global__ void __launch_bounds__(256) k_push_init(const PushArgs a)
{
    __shared__ float s_phase;
    if (EMODE == 2) {
        if (threadIdx.x == 0) {
            const double t = (double)a.cnt->niter * a.dt;
            s_phase = (float)(a.rf_amp * cos(mod_phase(a.rf_omega * t, 10000000 * M_PI)) + a.rf_U0);
        }
        __syncthreads();
    }
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n) return;
    const float xg = a.x[k];
    if (!(xg >= 0.f)) return;
    const float zg = a.z[k];
    float vx = a.vx[k], vy = a.vy[k], vz = a.vz[k];
    float ex, ez;
    if (EMODE == 0) {
        ex = 0.f;
        ez = a.extern_ez;
    } else {
        gather_faces(a.Exf, a.Ezf, a.nx, a.nz, xg, zg, ex, ez);
        if (EMODE == 2) {
            float rx, rz;
            gather_faces(a.Exf_rf, a.Ezf_rf, a.nx, a.nz, xg, zg, rx, rz);
            ex += s_phase * rx;
            ez += s_phase * rz;
        }
    }
    // here (tx..sz) hold the half-angle backward rotation vectors and hq = -q/m*dt/2
    float tx = a.tx, ty = a.ty, tz = a.tz, sx = a.sx, sy = a.sy, sz = a.sz;
    if (a.btab) {
        const float xi = (xg * a.gdx + a.gx0 - a.b_x0) * a.b_ix;
        const float zi = (zg * a.gdz + a.gz0 - a.b_z0) * a.b_iz;
        tx = table_interp(a.Br, a.bnx, a.bnz, xi, zi) * a.q_dt_2m;
        tz = table_interp(a.Bz, a.bnx, a.bnz, xi, zi) * a.q_dt_2m;
        ty = 0.f;
        const float f = 2.f / (1.f + tx * tx + ty * ty + tz * tz);
        sx = tx * f;
        sy = ty * f;
        sz = tz * f;
    }
    if (COORD == 1) {
        const float vpr = vx + vy * tz - vz * ty;
        const float vpt = vy + vz * tx - vx * tz;
        const float vpz = vz + vx * ty - vy * tx;
        vx += vpt * sz - vpz * sy;
        vy += vpz * sx - vpr * sz;
        vz += vpr * sy - vpt * sx;
    } else {
        const float vpr = vx - vy * tz + vz * ty;
        const float vpz = vz - vx * ty + vy * tx;
        const float vpt = vy - vz * tx + vx * tz;
        vx += -vpt * sz + vpz * sy;
        vy += -vpz * sx + vpr * sz;
        vz += -vpr * sy + vpt * sx;
    }
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
    const float xg = a.x[k];
    if (!(xg >= 0.f)) return;
    const float zg = a.z[k];
    const int ic = max(0, min((int)xg, a.nx - 2));
    const int jc = max(0, min((int)zg, a.nz - 2));
    const unsigned long long one = 1ull << kDepositShift;
    const unsigned long long U = (unsigned long long)((xg - (float)ic) * (float)(1 << kDepositShift));
    const unsigned long long V = (unsigned long long)((zg - (float)jc) * (float)(1 << kDepositShift));
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
    switch (a.emode) {
    case 0: init ? k_push_init<COORD, 0><<<grid, 256, 0, s>>>(a) : k_push<COORD, 0><<<grid, 256, 0, s>>>(a); break;
    case 1: init ? k_push_init<COORD, 1><<<grid, 256, 0, s>>>(a) : k_push<COORD, 1><<<grid, 256, 0, s>>>(a); break;
    default: init ? k_push_init<COORD, 2><<<grid, 256, 0, s>>>(a) : k_push<COORD, 2><<<grid, 256, 0, s>>>(a); break;
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
