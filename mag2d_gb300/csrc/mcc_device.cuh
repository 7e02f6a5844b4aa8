// Device side of BaseSpecies::scatter (src/particles.cpp:208-365), shared by
// the inline collision path of the particle kernel and the candidate-list
// collision kernel.  Random variates come from the Philox stream of the
// colliding particle; velocity algebra is FP64, variates FP32.
#pragma once
#include "device.hpp"
#include "philox.hpp"

namespace mag {

constexpr double kPiD = 3.14159265358979323846;
constexpr double kQeD = 1.602189e-19;
constexpr double kEps0D = 8.854187817e-12;

struct Stream {
    uint64_t seed;
    uint32_t sp, id, tag;
    uint64_t step;
    uint32_t blk = 0;
    U4 buf;
    int pos = 4;
    __device__ Stream(uint64_t s, uint32_t p, uint32_t i, uint32_t t, uint64_t st)
        : seed(s), sp(p), id(i), tag(t), step(st)
    {
    }
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
    __device__ double uni() { return (double)next() * (1.0 / 4294967296.0) + (0.5 / 4294967296.0); }  // (0,1)
    __device__ float unif() { return ((float)(next() >> 8) + 0.5f) * (1.0f / 16777216.0f); }        // (0,1)
    __device__ float normalf()  // Box-Muller in FP32
    {
        const float u1 = unif(), u2 = unif();
        return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
    }
};

__device__ inline double mcc_table(const double* E, const double* S, int n, double x)
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

// Interaction::sigma_v (src/particles.hpp:61-70)
__device__ inline double mcc_sigma_v(const InterDev& in, const double* tables, double v)
{
    const double EeV = 0.5 * in.mu * v * v / kQeD;
    if (in.type == COULOMB) {  // Interaction::coulomb_sigma, src/particles.cpp:19-26
        const double E = EeV * kQeD;
        const double Lambda = in.coul_q1q2 / (4 * kPiD * kEps0D * E);
        return kPiD * Lambda * Lambda * log(in.coul_lambda_D / Lambda) * v;
    }
    if (in.tab_n > 0) {
        const double* E = tables + in.tab_off;
        return mcc_table(E, E + in.tab_n, in.tab_n, EeV) * v;
    }
    return in.rate;
}

// isotropic vector of length len (t_random::rot, src/random.cpp:103-115)
__device__ inline void mcc_rot(Stream& r, double len, double& x, double& y, double& z)
{
    const float cs = 1.0f - 2.0f * r.unif();
    const float sn = sqrtf(fmaxf(0.0f, 1.0f - cs * cs));
    float sp, cp;
    sincospif(2.0f * r.unif(), &sp, &cp);
    x = len * cs;
    y = len * (double)(sn * sp);
    z = len * (double)(sn * cp);
}

// rotation of (x, y, z) by 'angle' about a random axis normal to it (t_random::deflect, src/random.cpp:133-175)
__device__ inline void mcc_deflect(Stream& r, double angle, double& x, double& y, double& z)
{
    const double len = tan(angle / 2.0);
    double x1, y1, z1;
    mcc_rot(r, len, x1, y1, z1);
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
// mean (Gauss): K(k) = pi / (2 AGM(1, sqrt(1 - k^2)))
__device__ inline double mcc_ellint_K(double k)
{
    double a = 1.0, b = sqrt(fmax(0.0, 1.0 - k * k));
    for (int i = 0; i < 40 && fabs(a - b) > 1e-16 * a; ++i) {
        const double an = 0.5 * (a + b);
        b = sqrt(a * b);
        a = an;
    }
    return kPiD / (2.0 * a);
}

enum { MCC_NULL = 0, MCC_HIT = 1, MCC_NOPARTNER = 2 };

// Target species by the null-collision rates (particles.cpp:211-222).
__device__ inline int mcc_pick_target(const MccSpecies& m, Stream& rs)
{
    const double gamma = rs.uni() * m.inv_lifetime;
    double acc = 0.0;
    int s;
    for (s = 0; s < m.nsp - 1; ++s) {
        acc += m.rates[s];
        if (acc > gamma) break;
    }
    return s;
}

// Everything of scatter() after the partner velocity (vr2, vz2, vt2) of
// target species s is known (particles.cpp:241-360).  Updates (vx, vy, vz);
// for COULOMB also returns the partner's new velocity in (pvx, pvy, pvz).
__device__ inline int mcc_collide(const MccSpecies& m, int s, Stream& rs, double& vx, double& vy, double& vz,
                                  double vr2, double vz2, double vt2, bool& partner_update, double& pvx,
                                  double& pvy, double& pvz)
{
    partner_update = false;
    const double dvx = vx - vr2, dvz = vz - vz2, dvt = vy - vt2;
    const double v_rel = sqrt(dvx * dvx + dvz * dvz + dvt * dvt);
    const double m2 = m.t_mass[s];
    const double g2 = rs.uni() * m.rates[s];
    double acc = 0.0;
    int hit = -1;
    for (int q = m.inter_begin[s]; q < m.inter_end[s]; ++q) {
        acc += mcc_sigma_v(m.inter[q], m.tables, v_rel) * m.t_density[s];
        if (acc > g2) {
            hit = q;
            break;
        }
    }
    if (hit < 0) return MCC_NULL;
    const InterDev in = m.inter[hit];
    const double mass = m.mass;
    const double tmp = 1.0 / (mass + m2);
    switch (in.type) {
    case SUPERELASTIC: {
        const double E = 0.5 * in.mu * v_rel * v_rel + in.DE;
        const double vr = sqrt(2 * E / in.mu);
        double rx, rz, ry;
        mcc_rot(rs, vr, rx, rz, ry);
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
        mcc_rot(rs, v_rel, rx, ry, rz);
        vx = rx * m2 * tmp + cx;
        vz = rz * m2 * tmp + cz;
        vy = ry * m2 * tmp + cy;
        if (in.type == COULOMB) {
            partner_update = true;
            pvx = -rx * mass * tmp + cx;
            pvz = -rz * mass * tmp + cz;
            pvy = -ry * mass * tmp + cy;
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
            const double theta = mcc_ellint_K(xi0 / xi1) * 1.41421356237309504880 * beta / xi1;
            mcc_deflect(rs, kPiD - 2 * theta, v1x, v1y, v1z);
        } else {
            const double len = sqrt(v1x * v1x + v1y * v1y + v1z * v1z);
            mcc_rot(rs, len, v1x, v1y, v1z);
        }
        vx = v1x + (vx * mass + vr2 * m2) * tmp;
        vz = v1y + (vz * mass + vz2 * m2) * tmp;
        vy = v1z + (vy * mass + vt2 * m2) * tmp;
    } break;
    default:
        break;
    }
    return MCC_HIT;
}

}  // namespace mag
