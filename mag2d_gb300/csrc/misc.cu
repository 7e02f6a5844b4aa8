// Small kernels: particle loaders of the initscript, fills and reductions.
#include "device.hpp"
#include "kernels.hpp"
#include "philox.hpp"

namespace mag {

namespace {

constexpr double kPi = 3.14159265358979323846;

struct LoadArgs {
    uint32_t *x, *z;
    float *vx, *vy, *vz;
    uint32_t* id;
    int64_t n;
    uint32_t id0;
    int kind;  // 0 disk, 1 everywhere, 2 bessel, 3 cylinder (r-z)
    double cx, cz, radius, zlo, zhi, x0, z0, dx, dz, xmax, zmax, vsig;
    uint64_t seed;
    uint32_t species;
};

struct LStream {
    uint64_t seed;
    uint32_t sp, id;
    uint32_t blk = 0;
    U4 buf;
    int pos = 4;
    __device__ double uni()
    {
        if (pos >= 4) {
            buf = draw(seed, sp, id, 0, TAG_LOAD, blk++);
            pos = 0;
        }
        const uint32_t a = pos == 0 ? buf.x : buf.z;
        const uint32_t b = pos == 0 ? buf.y : buf.w;
        pos += 2;
        return u01d(a, b);
    }
    __device__ double normal()
    {
        const double u1 = 1.0 - uni(), u2 = uni();
        return sqrt(-2.0 * log(u1)) * cos(2.0 * kPi * u2);
    }
};

// Species::add_particles_on_disk / _everywhere / _bessel (src/particles.cpp:685-749)
// with Philox draws; kind 3 (uniform in a cylinder r < radius, zlo < z < zhi,
// r = radius * sqrt(u)) is the r-z loader the reference leaves undefined.
__global__ void k_load(const LoadArgs a)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n) return;
    const uint32_t pid = a.id0 + (uint32_t)k;
    LStream r{a.seed, a.species, pid};
    double x = 0, z = 0;
    bool ok = true;
    if (a.kind == 0) {
        double px, py;
        int t = 0;
        do {
            px = r.uni() - 0.5;
            py = r.uni() - 0.5;
        } while (px * px + py * py > 0.25 && ++t < 200);
        x = px * 2 * a.radius + a.cx;
        z = py * 2 * a.radius + a.cz;
    } else if (a.kind == 1) {
        x = a.x0 + (a.xmax - a.x0) * r.uni();
        z = a.z0 + (a.zmax - a.z0) * r.uni();
    } else if (a.kind == 2) {
        const double root = 2.404825557695773;
        double px, py, rr;
        int t = 0;
        do {
            px = r.uni() * 2 - 1.0;
            py = r.uni() * 2 - 1.0;
            rr = sqrt(px * px + py * py);
        } while ((rr > 1.0 || r.uni() > j0(rr * root)) && ++t < 400);
        x = px * a.radius + a.cx;
        z = py * a.radius + a.cz;
    } else {
        x = a.radius * sqrt(r.uni());
        z = a.zlo + (a.zhi - a.zlo) * r.uni();
    }
    if (x < a.x0 || x > a.xmax || z < a.z0 || z > a.zmax) ok = false;
    const double fx = rint((x - a.x0) / a.dx * (double)(1u << kFracBits));
    const double fz = rint((z - a.z0) / a.dz * (double)(1u << kFracBits));
    a.x[k] = ok ? (uint32_t)fx : kDead;
    a.z[k] = ok ? (uint32_t)fz : 0u;
    a.vx[k] = (float)(r.normal() * a.vsig);
    a.vz[k] = (float)(r.normal() * a.vsig);
    a.vy[k] = (float)(r.normal() * a.vsig);
    a.id[k] = pid;
}

__global__ void k_fill_u32(uint32_t* p, uint32_t v0, int64_t n)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        p[k] = v0 + (uint32_t)k;
}

// Host particle arrays (FP64, staged in device memory or read in place from
// page-locked host memory) to the SoA state: fixed-point positions
// llrint((x - x0) / dx * 2^20) (outside the box: removed), FP32 velocities,
// ids 0..n-1
__global__ void k_set_particles(ParticleColumns in, int64_t n, SetParticlesGeom g, uint32_t* __restrict__ x,
                                uint32_t* __restrict__ z, float* __restrict__ vx, float* __restrict__ vy,
                                float* __restrict__ vz, uint32_t* __restrict__ id)
{
    const double one = (double)(1u << kFracBits);
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const double px = in.v[0][k], pz = in.v[1][k];
        const bool inside = px >= g.x0 && px <= g.xmax && pz >= g.z0 && pz <= g.zmax;
        x[k] = inside ? (uint32_t)__double2ll_rn(__dmul_rn(__ddiv_rn(__dsub_rn(px, g.x0), g.dx), one)) : kDead;
        z[k] = inside ? (uint32_t)__double2ll_rn(__dmul_rn(__ddiv_rn(__dsub_rn(pz, g.z0), g.dz), one)) : 0u;
        vx[k] = (float)in.v[2][k];
        vy[k] = (float)in.v[3][k];
        vz[k] = (float)in.v[4][k];
        id[k] = (uint32_t)k;
    }
}

// sum of v^2 over live particles (FP64) and their count: per-thread partial
// sums, a block reduction in shared memory, one atomic per block
__global__ void __launch_bounds__(256) k_energy(const uint32_t* x, const float* vx, const float* vy, const float* vz,
                                                int64_t n, double* sum, unsigned long long* cnt)
{
    __shared__ double ss[8];
    __shared__ unsigned long long sc[8];
    double s = 0.0;
    unsigned long long c = 0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        if (x[k] == kDead) continue;
        const float a = vx[k], b = vy[k], d = vz[k];
        s += (double)fmaf(a, a, fmaf(b, b, d * d));
        ++c;
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        ss[w] = s;
        sc[w] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        unsigned long long u = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            t += ss[i];
            u += sc[i];
        }
        if (u) {
            atomicAdd(sum, t);
            atomicAdd(cnt, u);
        }
    }
}

// Histogram::add (src/histogram.cpp:22-35) of the kinetic energies [eV] of the
// live particles (BaseSpecies::energy_dist_compute, src/particles.cpp:412-418),
// in the reference's operation order: bins counted in shared memory; stats =
// n_val, sum, n_val_tot, sum_tot
__global__ void __launch_bounds__(256) k_energy_hist(const uint32_t* x, const float* vx, const float* vy,
                                                     const float* vz, int64_t n, double mass, double qe, double emin,
                                                     double emax, int nbins, unsigned long long* bins, double* stats)
{
    extern __shared__ unsigned int sbin[];
    __shared__ double s_sum[8], s_tot[8];
    __shared__ unsigned long long s_nv[8], s_nt[8];
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) sbin[i] = 0;
    __syncthreads();
    double sum = 0.0, tot = 0.0;
    unsigned long long nv = 0, nt = 0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        if (x[k] == kDead) continue;
        const double a = vx[k], b = vy[k], d = vz[k];
        const double f = (a * a + d * d + b * b) * mass * 0.5 / qe;  // operation order of the reference
        if (f < emax && f > emin) {
            atomicAdd(&sbin[min((int)((f - emin) * nbins / (emax - emin)), nbins - 1)], 1u);
            ++nv;
            sum += f;
        }
        ++nt;
        tot += f;
    }
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        tot += __shfl_xor_sync(0xffffffffu, tot, o);
        nv += __shfl_xor_sync(0xffffffffu, nv, o);
        nt += __shfl_xor_sync(0xffffffffu, nt, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_sum[w] = sum;
        s_tot[w] = tot;
        s_nv[w] = nv;
        s_nt[w] = nt;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nbins; i += blockDim.x)
        if (sbin[i]) atomicAdd(&bins[i], (unsigned long long)sbin[i]);
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        unsigned long long c = 0, d = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            a += s_sum[i];
            b += s_tot[i];
            c += s_nv[i];
            d += s_nt[i];
        }
        if (d) {
            atomicAdd(&stats[0], (double)c);
            atomicAdd(&stats[1], a);
            atomicAdd(&stats[2], (double)d);
            atomicAdd(&stats[3], b);
        }
    }
}

// acc[k] += w * src[k] (averaged fields: Field2D::add of rhoAverage / uAvg)
__global__ void k_axpy_i64(double* acc, const unsigned long long* src, double w, long long n)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        acc[k] += w * (double)(long long)src[k];
}
__global__ void k_axpy_f64(double* acc, const double* src, double w, long long n)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        acc[k] += w * src[k];
}

__global__ void k_interleave(const float* a, const float* b, float2* out, long long n)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        out[k] = make_float2(a[k], b[k]);
}

}  // namespace

int launch_interleave(const float* a, const float* b, float2* out, long long n, cudaStream_t s)
{
    if (n == 0) return 0;
    k_interleave<<<(unsigned)std::min<long long>((n + 255) / 256, 152 * 8), 256, 0, s>>>(a, b, out, n);
    return 1;
}

int launch_load_disk(uint32_t* x, uint32_t* z, float* vx, float* vy, float* vz, uint32_t* id, int64_t n, uint32_t id0,
                     int kind, double cx, double cz, double radius, double zlo, double zhi, double x0, double z0,
                     double dx, double dz, double xmax, double zmax, double vsig, uint64_t seed, uint32_t species,
                     int, cudaStream_t s)
{
    if (n == 0) return 0;
    LoadArgs a{x, z, vx, vy, vz, id, n, id0, kind, cx, cz, radius, zlo, zhi, x0, z0, dx, dz, xmax, zmax, vsig, seed, species};
    k_load<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return 1;
}

int launch_fill_u32(uint32_t* p, uint32_t v0, int64_t n, cudaStream_t s)
{
    if (n == 0) return 0;
    k_fill_u32<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(p, v0, n);
    return 1;
}

int launch_set_particles(const ParticleColumns& staged, int64_t n, const SetParticlesGeom& g, uint32_t* x, uint32_t* z,
                         float* vx, float* vy, float* vz, uint32_t* id, cudaStream_t s)
{
    if (n == 0) return 0;
    k_set_particles<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(staged, n, g, x, z, vx, vy,
                                                                                          vz, id);
    return 1;
}

// rec[6 w ..]: found flag, x, z (fixed point), vx, vy, vz (FP32 bits) of the
// live particle with id want[w]
__global__ void k_find_ids(const uint32_t* __restrict__ id, const uint32_t* __restrict__ x,
                           const uint32_t* __restrict__ z, const float* __restrict__ vx, const float* __restrict__ vy,
                           const float* __restrict__ vz, int64_t n, const uint32_t* __restrict__ want, int nwant,
                           uint32_t* __restrict__ rec)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        if (x[k] == kDead) continue;
        const uint32_t pid = id[k];
        for (int w = 0; w < nwant; ++w)
            if (want[w] == pid) {
                uint32_t* r = rec + 6 * w;
                r[0] = 1u;
                r[1] = x[k];
                r[2] = z[k];
                r[3] = __float_as_uint(vx[k]);
                r[4] = __float_as_uint(vy[k]);
                r[5] = __float_as_uint(vz[k]);
            }
    }
}

int launch_find_ids(const uint32_t* id, const uint32_t* x, const uint32_t* z, const float* vx, const float* vy,
                    const float* vz, int64_t n, const uint32_t* want, int nwant, uint32_t* rec, cudaStream_t s)
{
    if (n == 0 || nwant == 0) return 0;
    k_find_ids<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 8), 256, 0, s>>>(id, x, z, vx, vy, vz, n, want,
                                                                                      nwant, rec);
    return 1;
}

__global__ void k_gather_status(StatusSources src, StatusHost* out)
{
    if (threadIdx.x == 0) {
        out->err = *src.err;
        out->st = *src.st;
        if (src.energy) {
            out->sum_v2 = src.energy[0];
            out->n_live = reinterpret_cast<const unsigned long long*>(src.energy)[1];
        }
    }
    for (int s = threadIdx.x; s < src.nsp; s += blockDim.x)
        if (src.cnt[s]) out->c[s] = *src.cnt[s];
}

int launch_gather_status(const StatusSources& src, StatusHost* out, cudaStream_t s)
{
    k_gather_status<<<1, 32, 0, s>>>(src, out);
    return 1;
}

int launch_energy(const uint32_t* x, const float* vx, const float* vy, const float* vz, int64_t n, double* out_sum_v2,
                  unsigned long long* out_n, cudaStream_t s)
{
    if (n == 0) return 0;
    k_energy<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 4), 256, 0, s>>>(x, vx, vy, vz, n, out_sum_v2, out_n);
    return 1;
}

int launch_energy_hist(const uint32_t* x, const float* vx, const float* vy, const float* vz, int64_t n, double mass,
                       double qe, double emin, double emax, int nbins, unsigned long long* bins, double* stats,
                       cudaStream_t s)
{
    if (n == 0) return 0;
    k_energy_hist<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 4), 256, (size_t)nbins * 4, s>>>(
        x, vx, vy, vz, n, mass, qe, emin, emax, nbins, bins, stats);
    return 1;
}

int launch_axpy_i64(double* acc, const unsigned long long* src, double w, long long n, cudaStream_t s)
{
    k_axpy_i64<<<(unsigned)std::min<long long>((n + 255) / 256, 152 * 8), 256, 0, s>>>(acc, src, w, n);
    return 1;
}

int launch_axpy_f64(double* acc, const double* src, double w, long long n, cudaStream_t s)
{
    k_axpy_f64<<<(unsigned)std::min<long long>((n + 255) / 256, 152 * 8), 256, 0, s>>>(acc, src, w, n);
    return 1;
}

}  // namespace mag
