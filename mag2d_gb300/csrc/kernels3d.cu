// The 3D Cartesian path (Species<CARTESIAN3D>::advance, src/species3d.cpp:3-94;
// Field3D accumulate / grad, src/Field3D.hpp:40-163; the 7-point Poisson
// problem of src/fields3d.cpp:35-101).
//
// Layout: nodes (i, j, k) at (i ny + j) nz + k (z fastest, Array3D's order);
// positions fixed point like the 2D path (cells x 2^20 per axis); the charge
// of a particle is split over the 8 corners of its cell with 14-bit weights
// per axis (2^42 per particle, so an int64 node holds 2^21 particles); face
// fields Exf (nx+1) ny nz, Eyf nx (ny+1) nz, Ezf nx ny (nz+1) hold the
// staggered differences of Field3D::grad_component, the end faces repeating
// the last interior one.
#include <algorithm>

#include "device.hpp"
#include "kernels.hpp"
#include "philox.hpp"

namespace mag {

namespace {

constexpr float kInv = 1.0f / (float)(1u << kFracBits);
constexpr uint32_t kHalfCell = 1u << (kFracBits - 1);

__device__ __forceinline__ float fracf(uint32_t v) { return (float)(v & kFracMask) * kInv; }

// trilinear interpolation of f at corner (i, j, k) with strides (si, sj, 1)
__device__ __forceinline__ float trilerp(const float* __restrict__ f, long long si, long long sj, int i, int j, int k,
                                         float fx, float fy, float fz)
{
    const float* p = f + i * si + j * sj + k;
    const float c000 = __ldg(p), c001 = __ldg(p + 1), c010 = __ldg(p + sj), c011 = __ldg(p + sj + 1);
    const float c100 = __ldg(p + si), c101 = __ldg(p + si + 1), c110 = __ldg(p + si + sj),
                c111 = __ldg(p + si + sj + 1);
    const float c00 = c000 + fz * (c001 - c000), c01 = c010 + fz * (c011 - c010);
    const float c10 = c100 + fz * (c101 - c100), c11 = c110 + fz * (c111 - c110);
    const float c0 = c00 + fy * (c01 - c00), c1 = c10 + fy * (c11 - c10);
    return c0 + fx * (c1 - c0);
}

__device__ __forceinline__ void cell_of(uint32_t v, int n, int& c, float& f)
{
    c = min((int)(v >> kFracBits), n - 2);
    f = (float)(v - ((uint32_t)c << kFracBits)) * kInv;
}

__device__ __forceinline__ void face_of(uint32_t v, int n, int& c, float& f)
{
    const uint32_t r = v + kHalfCell;
    c = min((int)(r >> kFracBits), n - 1);
    f = fracf(r);
}

// E = -grad u at the particle (Field3D::grad with the staggered differences)
__device__ __forceinline__ void gather3(const Push3Args& a, uint32_t x, uint32_t y, uint32_t z, float& ex, float& ey,
                                        float& ez)
{
    int ic, jc, kc, ir, jr, kr;
    float fx, fy, fz, gx, gy, gz;
    cell_of(x, a.nx, ic, fx);
    cell_of(y, a.ny, jc, fy);
    cell_of(z, a.nz, kc, fz);
    face_of(x, a.nx, ir, gx);
    face_of(y, a.ny, jr, gy);
    face_of(z, a.nz, kr, gz);
    const long long ny = a.ny, nz = a.nz;
    ex = trilerp(a.Exf, ny * nz, nz, ir, jc, kc, gx, fy, fz);
    ey = trilerp(a.Eyf, (ny + 1) * nz, nz, ic, jr, kc, fx, gy, fz);
    ez = trilerp(a.Ezf, ny * (nz + 1), nz + 1, ic, jc, kr, fx, fy, gz);
}

__device__ __forceinline__ bool move3(uint32_t& v, float cells, uint32_t maxf, bool periodic)
{
    const float c = fminf(fmaxf(cells * (float)(1u << kFracBits), -1.0e9f), 1.0e9f);
    const int d = __float2int_rn(c);
    const uint32_t nv = v + (uint32_t)d;
    const bool out = d >= 0 ? (nv < v || nv > maxf) : (nv > v);
    if (!out) {
        v = nv;
        return true;
    }
    if (!periodic || maxf == 0) return false;
    long long q = ((long long)v + d) % (long long)maxf;
    if (q < 0) q += maxf;
    v = (uint32_t)q;
    return true;
}

__device__ __forceinline__ void deposit3(unsigned long long* rho, int ny, int nz, uint32_t x, uint32_t y, uint32_t z,
                                         int ic, int jc, int kc)
{
    const int sh = kFracBits - kDeposit3Bits;
    const unsigned long long one = 1ull << kDeposit3Bits;
    const unsigned long long U = (x - ((uint32_t)ic << kFracBits)) >> sh;
    const unsigned long long V = (y - ((uint32_t)jc << kFracBits)) >> sh;
    const unsigned long long W = (z - ((uint32_t)kc << kFracBits)) >> sh;
    const long long sj = nz, si = (long long)ny * nz;
    unsigned long long* r = rho + ic * si + jc * sj + kc;
    atomicAdd(r, (one - U) * (one - V) * (one - W));
    atomicAdd(r + si, U * (one - V) * (one - W));
    atomicAdd(r + sj, (one - U) * V * (one - W));
    atomicAdd(r + si + sj, U * V * (one - W));
    atomicAdd(r + 1, (one - U) * (one - V) * W);
    atomicAdd(r + si + 1, U * (one - V) * W);
    atomicAdd(r + sj + 1, (one - U) * V * W);
    atomicAdd(r + si + sj + 1, U * V * W);
}

// Boris rotation v += v' x s with v' = v + v x t (Birdsall & Langdon)
__device__ __forceinline__ void rotate3(const Push3Args& a, float& vx, float& vy, float& vz)
{
    const float px = vx + (vy * a.tz - vz * a.ty);
    const float py = vy + (vz * a.tx - vx * a.tz);
    const float pz = vz + (vx * a.ty - vy * a.tx);
    vx += py * a.sz - pz * a.sy;
    vy += pz * a.sx - px * a.sz;
    vz += px * a.sy - py * a.sx;
}

// One step of every particle: gather, half acceleration, rotation, half
// acceleration, move, boundary (FREE: removed outside [0, max]; PERIODIC:
// wrapped), cell test (t_grid::is_free: a FREE corner), deposit, collision
// test with the candidate list of the 2D path.
__global__ void __launch_bounds__(256) k_push3d(const __grid_constant__ Push3Args a)
{
    asm volatile("griddepcontrol.launch_dependents;");
    if (a.fold_slot >= 0 && blockIdx.x == 0 && threadIdx.x == 0) {
        Counters* c = a.cnt;
        c->live_sum += c->live_par[a.fold_slot];
        c->live_par[a.fold_slot] = 0;
        c->ncand_par[a.fold_slot] = 0;
    }
    unsigned live = 0, removed = 0;
    const unsigned full = 0xffffffffu;
    for (int64_t k0 = (int64_t)blockIdx.x * blockDim.x; k0 < a.n; k0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = k0 + threadIdx.x;
        bool cand = false;
        float vx = 0.f, vy = 0.f, vz = 0.f;
        uint32_t id = 0;
        if (k < a.n) {
            uint32_t x = a.x[k];
            if (x != kDead) {
                uint32_t y = a.y[k], z = a.z[k];
                vx = a.vx[k];
                vy = a.vy[k];
                vz = a.vz[k];
                id = a.id[k];
                cand = a.coll_threshold != 0u && collision_test_u32(a.seed, a.species, id, a.step) < a.coll_threshold;
                if (!a.init) {
                    float ex, ey, ez;
                    gather3(a, x, y, z, ex, ey, ez);
                    vx = fmaf(ex, a.hq, vx);
                    vy = fmaf(ey, a.hq, vy);
                    vz = fmaf(ez, a.hq, vz);
                    if (a.has_b) rotate3(a, vx, vy, vz);
                    vx = fmaf(ex, a.hq, vx);
                    vy = fmaf(ey, a.hq, vy);
                    vz = fmaf(ez, a.hq, vz);
                    bool alive = isfinite(vx) && isfinite(vy) && isfinite(vz);
                    alive = alive && move3(x, vx * a.cx, a.xmaxf, a.periodic) &&
                            move3(y, vy * a.cy, a.ymaxf, a.periodic) && move3(z, vz * a.cz, a.zmaxf, a.periodic);
                    int ic = 0, jc = 0, kc = 0;
                    if (alive) {
                        ic = min((int)(x >> kFracBits), a.nx - 2);
                        jc = min((int)(y >> kFracBits), a.ny - 2);
                        kc = min((int)(z >> kFracBits), a.nz - 2);
                        alive = a.cellfree[((size_t)ic * (a.ny - 1) + jc) * (a.nz - 1) + kc] != 0;
                    }
                    if (alive && a.rho) deposit3(a.rho, a.ny, a.nz, x, y, z, ic, jc, kc);
                    if (!alive) {
                        x = kDead;
                        cand = false;
                    }
                    a.x[k] = x;
                    a.y[k] = y;
                    a.z[k] = z;
                    live += alive;
                    removed += !alive;
                } else {
                    // leapfrog start: half backward rotation, half backward acceleration
                    float ex, ey, ez;
                    gather3(a, x, y, z, ex, ey, ez);
                    if (a.has_b) rotate3(a, vx, vy, vz);
                    vx = fmaf(ex, a.hq, vx);
                    vy = fmaf(ey, a.hq, vy);
                    vz = fmaf(ez, a.hq, vz);
                    cand = false;
                }
                a.vx[k] = vx;
                a.vy[k] = vy;
                a.vz[k] = vz;
            }
        }
        const unsigned m = __ballot_sync(full, cand);
        if (m) {
            const int lane = threadIdx.x & 31;
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(&a.cnt->ncand_par[a.slot], (unsigned long long)__popc(m));
            base = __shfl_sync(full, base, 0);
            if (cand) {
                const unsigned long long c = base + __popc(m & ((1u << lane) - 1u));
                a.cand[c] = (uint32_t)k;
                a.cand_rec[c] = make_float4(vx, vy, vz, __uint_as_float(id));
            }
        }
    }
    if (a.init) return;
    live = __reduce_add_sync(full, live);
    removed = __reduce_add_sync(full, removed);
    if ((threadIdx.x & 31) == 0) {
        if (live) atomicAdd(&a.cnt->live_par[a.slot], (unsigned long long)live);
        if (removed) atomicAdd(&a.cnt->removed, (unsigned long long)removed);
    }
}

__global__ void k_deposit3d(const Push3Args a)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < a.n; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t x = a.x[k];
        if (x == kDead) continue;
        const uint32_t y = a.y[k], z = a.z[k];
        deposit3(a.rho, a.ny, a.nz, x, y, z, min((int)(x >> kFracBits), a.nx - 2), min((int)(y >> kFracBits), a.ny - 2),
                 min((int)(z >> kFracBits), a.nz - 2));
    }
}

__global__ void k_faces3d(const double* __restrict__ u, int nx, int ny, int nz, double idx, double idy, double idz,
                          float* Exf, float* Eyf, float* Ezf)
{
    const long long n1 = (long long)(nx + 1) * ny * nz, n2 = (long long)nx * (ny + 1) * nz,
                    n3 = (long long)nx * ny * (nz + 1);
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n1 + n2 + n3;
         q += (long long)gridDim.x * blockDim.x) {
        if (q < n1) {
            const long long k = q % nz, t = q / nz, j = t % ny;
            int r = (int)(t / ny);
            r = r < 1 ? 1 : (r > nx - 1 ? nx - 1 : r);
            const long long c = ((long long)r * ny + j) * nz + k, b = c - (long long)ny * nz;
            Exf[q] = (float)(-(u[c] - u[b]) * idx);
        } else if (q < n1 + n2) {
            const long long p = q - n1;
            const long long k = p % nz, t = p / nz, i = t / (ny + 1);
            int r = (int)(t % (ny + 1));
            r = r < 1 ? 1 : (r > ny - 1 ? ny - 1 : r);
            const long long c = (i * ny + r) * nz + k, b = c - nz;
            Eyf[p] = (float)(-(u[c] - u[b]) * idy);
        } else {
            const long long p = q - n1 - n2;
            int r = (int)(p % (nz + 1));
            const long long t = p / (nz + 1);
            r = r < 1 ? 1 : (r > nz - 1 ? nz - 1 : r);
            const long long c = t * nz + r, b = c - 1;
            Ezf[p] = (float)(-(u[c] - u[b]) * idz);
        }
    }
}

__global__ void k_set_particles3d(const double* __restrict__ in, int64_t n, Set3Geom g, uint32_t* x, uint32_t* y,
                                  uint32_t* z, float* vx, float* vy, float* vz, uint32_t* id)
{
    const double one = (double)(1u << kFracBits);
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const double px = in[k], py = in[n + k], pz = in[2 * n + k];
        const bool inside = px >= 0.0 && px <= g.xmax && py >= 0.0 && py <= g.ymax && pz >= 0.0 && pz <= g.zmax;
        x[k] = inside ? (uint32_t)__double2ll_rn(__dmul_rn(__ddiv_rn(px, g.dx), one)) : kDead;
        y[k] = inside ? (uint32_t)__double2ll_rn(__dmul_rn(__ddiv_rn(py, g.dy), one)) : 0u;
        z[k] = inside ? (uint32_t)__double2ll_rn(__dmul_rn(__ddiv_rn(pz, g.dz), one)) : 0u;
        vx[k] = (float)in[3 * n + k];
        vy[k] = (float)in[4 * n + k];
        vz[k] = (float)in[5 * n + k];
        id[k] = (uint32_t)k;
    }
}

// ---- Poisson: conjugate gradients on the free nodes ----------------------
//
// (A u)_f = sum over axes (2 u_f - u_+ - u_-) / h^2, b_f = rho_f / eps0 + the
// fixed neighbours' values / h^2; A is symmetric positive definite on the
// free nodes.  One cooperative launch: every block keeps its part of the
// vectors, dot products are per-block partial sums added in block order
// after a grid barrier (deterministic), and the barrier's wait is bounded.

__device__ bool grid3_sync(unsigned* bar, unsigned nblocks, int* err)
{
    __syncthreads();
    __shared__ bool ok;
    if (threadIdx.x == 0) {
        ok = true;
        volatile unsigned* gen = bar + 1;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(bar, 1u) == nblocks - 1) {
            bar[0] = 0;
            __threadfence();
            atomicAdd((unsigned*)gen, 1u);
        } else {
            long long spins = 0;
            while (*gen == g) {
                if (++spins > (1ll << 26)) {  // another block never arrived
                    atomicCAS(err, 0, -5);
                    ok = false;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok;
}

__device__ double block_sum(double v, double* sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    __syncthreads();
    return s;  // valid in thread 0
}

// sum of part[0..nb) in a fixed order, broadcast to the block
__device__ double grid_total(const double* part, int nb, double* sh)
{
    __shared__ double tot;
    double v = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) v += ((volatile const double*)part)[b];
    const double s = block_sum(v, sh);
    if (threadIdx.x == 0) tot = s;
    __syncthreads();
    return tot;
}

__device__ __forceinline__ double apply_A(const Solve3Args& a, const double* __restrict__ v, long long q)
{
    const int k = (int)(q % a.nz);
    const long long t = q / a.nz;
    const int j = (int)(t % a.ny), i = (int)(t / a.ny);
    const long long si = (long long)a.ny * a.nz, sj = a.nz;
    double acc = 2.0 * (a.ix2 + a.iy2 + a.iz2) * v[q];
    // fixed nodes hold 0 in the search vectors, so they drop out
    if (i > 0) acc -= a.ix2 * v[q - si];
    if (i < a.nx - 1) acc -= a.ix2 * v[q + si];
    if (j > 0) acc -= a.iy2 * v[q - sj];
    if (j < a.ny - 1) acc -= a.iy2 * v[q + sj];
    if (k > 0) acc -= a.iz2 * v[q - 1];
    if (k < a.nz - 1) acc -= a.iz2 * v[q + 1];
    return acc;
}

__global__ void __launch_bounds__(256) k_solve3d(const __grid_constant__ Solve3Args a)
{
    __shared__ double sh[32];
    const long long nn = (long long)a.nx * a.ny * a.nz;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nb = gridDim.x;
    const long long si = (long long)a.ny * a.nz, sj = a.nz;
    // b, Dirichlet values, r = b - A u (u: previous solution on free nodes)
    for (long long q = t0; q < nn; q += stride) {
        const bool fixed = a.mask[q] != 0;
        if (fixed) a.u[q] = a.voltage[q];
        double rho = 0.0;
        if (a.rho64) {
            rho = a.rho64[q];
        } else {
            for (int s = 0; s < a.nsp; ++s) rho += a.rho_weight[s] * (double)a.rho_fixed[s][q];
        }
        a.b[q] = fixed ? 0.0 : rho * a.rho_scale;
        if (a.clear_rho && !a.rho64)
            for (int s = 0; s < a.nsp; ++s) ((unsigned long long*)a.rho_fixed[s])[q] = 0ull;
    }
    if (!grid3_sync(a.bar, nb, a.err)) return;
    double lr = 0.0, lb = 0.0;
    for (long long q = t0; q < nn; q += stride) {
        if (a.mask[q] != 0) {
            a.r[q] = 0.0;
            a.p[q] = 0.0;
            continue;
        }
        const int k = (int)(q % a.nz);
        const long long t = q / a.nz;
        const int j = (int)(t % a.ny), i = (int)(t / a.ny);
        // fixed neighbours move to the right-hand side; free ones use u
        double bq = a.b[q], au = 2.0 * (a.ix2 + a.iy2 + a.iz2) * a.u[q];
        auto nbr = [&](bool in, long long d, double w) {
            if (!in) return;
            if (a.mask[q + d] != 0) bq += w * a.u[q + d];
            else au -= w * a.u[q + d];
        };
        nbr(i > 0, -si, a.ix2);
        nbr(i < a.nx - 1, si, a.ix2);
        nbr(j > 0, -sj, a.iy2);
        nbr(j < a.ny - 1, sj, a.iy2);
        nbr(k > 0, -1, a.iz2);
        nbr(k < a.nz - 1, 1, a.iz2);
        const double r = bq - au;
        a.r[q] = r;
        a.p[q] = r;
        lr += r * r;
        lb += bq * bq;
    }
    double s = block_sum(lr, sh);
    const double s2 = block_sum(lb, sh);
    if (threadIdx.x == 0) {
        a.part[blockIdx.x] = s;
        a.part[nb + blockIdx.x] = s2;
    }
    if (!grid3_sync(a.bar, nb, a.err)) return;
    double rr = grid_total(a.part, nb, sh);
    const double bb = grid_total(a.part + nb, nb, sh);
    const double stop = a.tol * a.tol * fmax(bb, 1e-300);
    int it = 0;
    bool conv = rr <= stop;
    for (; !conv && it < a.max_iter; ++it) {
        double lpq = 0.0;
        for (long long q = t0; q < nn; q += stride) {
            if (a.mask[q] != 0) {
                a.qv[q] = 0.0;
                continue;
            }
            const double qq = apply_A(a, a.p, q);
            a.qv[q] = qq;
            lpq += a.p[q] * qq;
        }
        s = block_sum(lpq, sh);
        if (threadIdx.x == 0) a.part[2 * nb + (it & 1) * nb + blockIdx.x] = s;
        if (!grid3_sync(a.bar, nb, a.err)) return;
        const double pq = grid_total(a.part + 2 * nb + (it & 1) * nb, nb, sh);
        const double alpha = pq != 0.0 ? rr / pq : 0.0;
        double lrr = 0.0;
        for (long long q = t0; q < nn; q += stride) {
            if (a.mask[q] != 0) continue;
            a.u[q] += alpha * a.p[q];
            const double r = a.r[q] - alpha * a.qv[q];
            a.r[q] = r;
            lrr += r * r;
        }
        s = block_sum(lrr, sh);
        if (threadIdx.x == 0) a.part[4 * nb + (it & 1) * nb + blockIdx.x] = s;
        if (!grid3_sync(a.bar, nb, a.err)) return;
        const double rr_new = grid_total(a.part + 4 * nb + (it & 1) * nb, nb, sh);
        const double beta = rr != 0.0 ? rr_new / rr : 0.0;
        rr = rr_new;
        conv = rr <= stop;
        for (long long q = t0; q < nn; q += stride)
            if (a.mask[q] == 0) a.p[q] = a.r[q] + beta * a.p[q];
        if (!grid3_sync(a.bar, nb, a.err)) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.status->iterations = it;
        a.status->residual = bb > 0.0 ? sqrt(rr / bb) : 0.0;
        a.status->converged = conv ? 1 : 0;
        a.status->aborted = 0;
    }
}

unsigned grid_n(long long n) { return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 8)); }

}  // namespace

int launch_push3d(const Push3Args& a, int sm_count, cudaStream_t s)
{
    if (a.n == 0) return 0;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((a.n + 255) / 256, (int64_t)sm_count * 8));
    k_push3d<<<grid, 256, 0, s>>>(a);
    return 1;
}

int launch_deposit3d(const Push3Args& a, cudaStream_t s)
{
    if (a.n == 0) return 0;
    k_deposit3d<<<grid_n(a.n), 256, 0, s>>>(a);
    return 1;
}

int launch_faces3d(const double* u, int nx, int ny, int nz, double dx, double dy, double dz, float* Exf, float* Eyf,
                   float* Ezf, cudaStream_t s)
{
    const long long n = (long long)(nx + 1) * ny * nz + (long long)nx * (ny + 1) * nz + (long long)nx * ny * (nz + 1);
    k_faces3d<<<grid_n(n), 256, 0, s>>>(u, nx, ny, nz, 1.0 / dx, 1.0 / dy, 1.0 / dz, Exf, Eyf, Ezf);
    return 1;
}

int launch_set_particles3d(const double* staged, int64_t n, const Set3Geom& g, uint32_t* x, uint32_t* y, uint32_t* z,
                           float* vx, float* vy, float* vz, uint32_t* id, cudaStream_t s)
{
    if (n == 0) return 0;
    k_set_particles3d<<<grid_n(n), 256, 0, s>>>(staged, n, g, x, y, z, vx, vy, vz, id);
    return 1;
}

int solve3d_blocks(int sm_count)
{
    int per_sm = 0, coop = 0, dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve3d, 256, 0) != cudaSuccess || per_sm < 1) return 1;
    return std::min(per_sm, 2) * sm_count;
}

int launch_solve3d(const Solve3Args& a, int nblocks, cudaStream_t s)
{
    void* args[] = {(void*)&a};
    cudaLaunchCooperativeKernel((const void*)k_solve3d, dim3((unsigned)std::max(nblocks, 1)), dim3(256), args, 0, s);
    return 1;
}

}  // namespace mag
