// Null-collision Monte Carlo collisions of the particles that the push kernel
// listed as candidates (BaseSpecies::scatter, src/particles.cpp:208-365).
//
// Per candidate: pick the target species by the null-collision rates
// (:211-222), take the partner velocity from a Maxwellian of the target
// (rndv, src/particles.hpp:188-192) or from a random live target particle
// (random_particle, :207-217), pick the interaction by sigma_v * density
// (:245-258, sigma_v src/particles.hpp:61-70, vec_interpolate
// src/tabulate.cpp:89-141) and apply ELASTIC / COULOMB / SUPERELASTIC / CX /
// LANGEVIN (:266-360).  Candidates are few (collision probability per step is
// small), so the arithmetic here is FP64.  All random numbers come from the
// Philox stream of (species, particle id, step).
//
// The last block to finish also closes the step for this species: it moves
// the live count of the step into the running totals, clears the candidate
// counter and advances the species step counter (Species::advance niter++,
// src/particles.hpp:347).
#include "device.hpp"
#include "kernels.hpp"
#include "philox.hpp"

namespace mag {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kQe = 1.602189e-19;
constexpr double kEps0d = 8.854187817e-12;

struct Stream {
    uint64_t seed;
    uint32_t sp, id, tag;
    uint64_t step;
    uint32_t blk = 0;
    U4 buf;
    int pos = 4;
    __device__ uint32_t next()
    {
        if (pos == 4) {
            buf = draw(seed, sp, id, step, tag, blk++);
            pos = 0;
        }
        const uint32_t v = pos == 0 ? buf.x : pos == 1 ? buf.y : pos == 2 ? buf.z : buf.w;
        ++pos;
        return v;
    }
    __device__ double uni()
    {
        const uint32_t a = next();
        const uint32_t b = next();
        return u01d(a, b);
    }
    __device__ double normal()  // Box-Muller
    {
        const double u1 = 1.0 - uni(), u2 = uni();
        return sqrt(-2.0 * log(u1)) * cos(2.0 * kPi * u2);
    }
};

__device__ double table_lookup(const double* E, const double* S, int n, double x)
{
    if (x >= E[n - 1]) return S[n - 1];
    if (x <= E[0]) return S[0];
    int j1 = 0, j2 = n - 1;
    while (j2 - j1 > 1) {
        const int j3 = (j1 + j2) / 2;
        if (x < E[j3]) j2 = j3;
        else j1 = j3;
    }
    const double w = (x - E[j1]) / (E[j2] - E[j1]);
    return S[j1] * (1 - w) + S[j2] * w;
}

__device__ double sigma_v(const InterDev& in, const double* tables, double v)
{
    const double EeV = 0.5 * in.mu * v * v / kQe;
    if (in.type == COULOMB) {  // Interaction::coulomb_sigma, src/particles.cpp:19-26
        const double E = EeV * kQe;
        const double Lambda = in.coul_q1q2 / (4 * kPi * kEps0d * E);
        return kPi * Lambda * Lambda * log(in.coul_lambda_D / Lambda) * v;
    }
    if (in.tab_n > 0) {
        const double* E = tables + in.tab_off;
        return table_lookup(E, E + in.tab_n, in.tab_n, EeV) * v;
    }
    return in.rate;
}

// isotropic vector of length len (t_random::rot, src/random.cpp:103-115)
__device__ void rot(Stream& r, double len, double& x, double& y, double& z)
{
    const double cs = 1.0 - 2.0 * r.uni();
    x = len * cs;
    const double sn = sqrt(fmax(0.0, 1.0 - cs * cs));
    double sp, cp;
    sincos(2.0 * kPi * r.uni(), &sp, &cp);
    y = len * sn * sp;
    z = len * sn * cp;
}

// rotation of (x, y, z) by 'angle' about a random axis normal to it
// (t_random::deflect, src/random.cpp:133-175)
__device__ void deflect(Stream& r, double angle, double& x, double& y, double& z)
{
    const double len = tan(angle / 2.0);
    double x1, y1, z1;
    rot(r, len, x1, y1, z1);
    double tx = y * z1 - z * y1, ty = z * x1 - x * z1, tz = x * y1 - y * x1;
    double tmp = len / sqrt(tx * tx + ty * ty + tz * tz);
    tx *= tmp;
    ty *= tmp;
    tz *= tmp;
    const double xp = x - y * tz + z * ty;
    const double yp = y - z * tx + x * tz;
    const double zp = z - x * ty + y * tx;
    tmp = 2.0 / (1 + len * len);
    x1 = tx * tmp;
    y1 = ty * tmp;
    z1 = tz * tmp;
    x += -yp * z1 + zp * y1;
    y += -zp * x1 + xp * z1;
    z += -xp * y1 + yp * x1;
}

// complete elliptic integral of the first kind K(k) by the arithmetic-geometric
// mean: K(k) = pi / (2 AGM(1, sqrt(1 - k^2)))
__device__ double ellint_K(double k)
{
    double a = 1.0, b = sqrt(fmax(0.0, 1.0 - k * k));
    for (int i = 0; i < 40 && fabs(a - b) > 1e-16 * a; ++i) {
        const double an = 0.5 * (a + b);
        b = sqrt(a * b);
        a = an;
    }
    return kPi / (2.0 * a);
}

__global__ void __launch_bounds__(128) k_collide(const CollideArgs a)
{
    __shared__ unsigned long long s_coll, s_null, s_miss;
    if (threadIdx.x == 0) {
        s_coll = 0;
        s_null = 0;
        s_miss = 0;
    }
    __syncthreads();
    const unsigned long long ncand = *((volatile unsigned long long*)&a.cnt->ncand);
    const uint64_t step = a.cnt->niter;
    for (unsigned long long c = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncand;
         c += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t p = a.cand[c];
        const uint32_t pid = a.id[p];
        Stream rs{a.seed, a.species, pid, TAG_COLLIDE, step};
        double vx = a.vx[p], vy = a.vy[p], vz = a.vz[p];
        // target species (null-collision rates)
        const double gamma = rs.uni() * a.inv_lifetime;
        double acc = 0.0;
        int s;
        for (s = 0; s < a.nsp - 1; ++s) {
            acc += a.rates[s];
            if (acc > gamma) break;
        }
        double vr2, vz2, vt2;
        int partner = -1;
        if (!a.t_has_slots[s]) {
            const double sig = a.t_sigma_v[s];
            vr2 = rs.normal() * sig;
            vz2 = rs.normal() * sig;
            vt2 = rs.normal() * sig;
        } else {
            Stream ps{a.seed, a.species, pid, TAG_PARTNER, step};
            const int64_t nt = a.t_n[s];
            for (int tries = 0; tries < 256 && nt > 0; ++tries) {
                const int64_t q = (int64_t)(((uint64_t)ps.next() << 32 | ps.next()) % (uint64_t)nt);
                if (a.t_x[s][q] >= 0.f) {  // any live particle, itself included (random_particle)
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
        const double dvx = vx - vr2, dvz = vz - vz2, dvt = vy - vt2;
        const double v_rel = sqrt(dvx * dvx + dvz * dvz + dvt * dvt);
        const double m2 = a.t_mass[s];
        const double g2 = rs.uni() * a.rates[s];
        acc = 0.0;
        int hit = -1;
        for (int q = a.inter_begin[s]; q < a.inter_end[s]; ++q) {
            acc += sigma_v(a.inter[q], a.tables, v_rel) * a.t_density[s];
            if (acc > g2) {
                hit = q;
                break;
            }
        }
        if (hit < 0) {
            atomicAdd(&s_null, 1ull);
            continue;
        }
        const InterDev in = a.inter[hit];
        const double mass = a.mass;
        const double tmp = 1.0 / (mass + m2);
        switch (in.type) {
        case SUPERELASTIC: {
            const double E = 0.5 * in.mu * v_rel * v_rel + in.DE;
            const double vr = sqrt(2 * E / in.mu);
            double rx, rz, ry;
            rot(rs, vr, rx, rz, ry);
            vx = (rx * m2 + vx * mass + vr2 * m2) * tmp;
            vz = (ry * m2 + vz * mass + vz2 * m2) * tmp;
            vy = (rz * m2 + vy * mass + vt2 * m2) * tmp;
        } break;
        case COULOMB:
        case ELASTIC: {
            const double cx = (vx * mass + vr2 * m2) * tmp;
            const double cz = (vz * mass + vz2 * m2) * tmp;
            const double cy = (vy * mass + vt2 * m2) * tmp;
            double rx, ry, rz;
            rot(rs, v_rel, rx, ry, rz);
            vx = rx * m2 * tmp + cx;
            vz = rz * m2 * tmp + cz;
            vy = ry * m2 * tmp + cy;
            if (in.type == COULOMB && partner >= 0) {
                a.t_vx[s][partner] = (float)(-rx * mass * tmp + cx);
                a.t_vz[s][partner] = (float)(-rz * mass * tmp + cz);
                a.t_vy[s][partner] = (float)(-ry * mass * tmp + cy);
            }
        } break;
        case CX:
            vx = vr2;
            vz = vz2;
            vy = vt2;
            break;
        case LANGEVIN: {
            double v1x = (vx - vr2) * m2 * tmp;
            double v1y = (vz - vz2) * m2 * tmp;
            double v1z = (vy - vt2) * m2 * tmp;
            const double beta = sqrt(rs.uni()) * in.cutoff;
            if (beta > 1.0) {  // Nanbu & Kitatani, J. Phys. D 28 (1995) 324
                const double b2 = beta * beta;
                const double tt = sqrt(b2 * b2 - 1.0);
                const double xi0 = sqrt(b2 - tt), xi1 = sqrt(b2 + tt);
                const double theta = ellint_K(xi0 / xi1) * 1.41421356237309504880 * beta / xi1;
                deflect(rs, kPi - 2 * theta, v1x, v1y, v1z);
            } else {
                const double len = sqrt(v1x * v1x + v1y * v1y + v1z * v1z);
                rot(rs, len, v1x, v1y, v1z);
            }
            vx = v1x + (vx * mass + vr2 * m2) * tmp;
            vz = v1y + (vz * mass + vz2 * m2) * tmp;
            vy = v1z + (vy * mass + vt2 * m2) * tmp;
        } break;
        default:
            break;
        }
        a.vx[p] = (float)vx;
        a.vy[p] = (float)vy;
        a.vz[p] = (float)vz;
        atomicAdd(&s_coll, 1ull);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_coll) atomicAdd(&a.cnt->ncoll, s_coll);
        if (s_null) atomicAdd(&a.cnt->nnull, s_null);
        if (s_miss) atomicAdd(&a.cnt->partner_miss, s_miss);
        __threadfence();
        const unsigned long long ticket = atomicAdd(&a.cnt->done_blocks, 1ull);
        if (ticket == gridDim.x - 1) {  // last block closes the step
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
