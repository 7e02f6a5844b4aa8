// Device side of BaseSpecies::scatter (src/particles.cpp:208-365) for the
// candidate-list collision kernel.  Random variates come from the Philox
// stream of the colliding particle.  The arithmetic is FP32 (GB300 runs FP64
// at 1/64 of the FP32 rate, and MCC parity is statistical); only the Coulomb
// cross section, whose charge products sit near the FP32 range limit, is FP64.
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

__device__ inline float mcc_table(const double* E, const double* S, int n, float x)
{
    if (x >= (float)E[n - 1]) return (float)S[n - 1];
    if (x <= (float)E[0]) return (float)S[0];
    int j1 = 0, j2 = n - 1;
    while (j2 - j1 > 1) {
        const int j3 = (j1 + j2) / 2;
        if (x < (float)E[j3]) j2 = j3;
        else j1 = j3;
    }
    const float e1 = (float)E[j1], e2 = (float)E[j2];
    const float w = (x - e1) / (e2 - e1);
    return (float)S[j1] * (1.f - w) + (float)S[j2] * w;
}

// Interaction::sigma_v (src/particles.hpp:61-70)
__device__ inline float mcc_sigma_v(const InterDev& in, const double* tables, float v)
{
    if (in.type == COULOMB) {  // Interaction::coulomb_sigma, src/particles.cpp:19-26
        const double vd = v;
        const double E = 0.5 * in.mu * vd * vd;
        const double Lambda = in.coul_q1q2 / (4 * kPiD * kEps0D * E);
        return (float)(kPiD * Lambda * Lambda * log(in.coul_lambda_D / Lambda) * vd);
    }
    const float EeV = (float)(0.5 * in.mu / kQeD) * v * v;
    if (in.tab_n > 0) {
        const double* E = tables + in.tab_off;
        return mcc_table(E, E + in.tab_n, in.tab_n, EeV) * v;
    }
    return (float)in.rate;
}

// isotropic vector of length len (t_random::rot, src/random.cpp:103-115)
__device__ inline void mcc_rot(Stream& r, float len, float& x, float& y, float& z)
{
    const float cs = 1.0f - 2.0f * r.unif();
    const float sn = sqrtf(fmaxf(0.0f, 1.0f - cs * cs));
    float sp, cp;
    sincospif(2.0f * r.unif(), &sp, &cp);
    x = len * cs;
    y = len * sn * sp;
    z = len * sn * cp;
}

// rotation of (x, y, z) by 'angle' about a random axis normal to it (t_random::deflect, src/random.cpp:133-175)
__device__ inline void mcc_deflect(Stream& r, float angle, float& x, float& y, float& z)
{
    const float len = tanf(angle / 2.0f);
    float x1, y1, z1;
    mcc_rot(r, len, x1, y1, z1);
    float tx = y * z1 - z * y1, ty = z * x1 - x * z1, tz = x * y1 - y * x1;
    float tmp = len / sqrtf(tx * tx + ty * ty + tz * tz);
    tx *= tmp;
    ty *= tmp;
    tz *= tmp;
    const float xp = x - y * tz + z * ty;
    const float yp = y - z * tx + x * tz;
    const float zp = z - x * ty + y * tx;
    tmp = 2.0f / (1 + len * len);
    x1 = tx * tmp;
    y1 = ty * tmp;
    z1 = tz * tmp;
    x += -yp * z1 + zp * y1;
    y += -zp * x1 + xp * z1;
    z += -xp * y1 + yp * x1;
}

// complete elliptic integral of the first kind K(k) by the arithmetic-geometric
// mean (Gauss): K(k) = pi / (2 AGM(1, sqrt(1 - k^2)))
__device__ inline float mcc_ellint_K(float k)
{
    float a = 1.0f, b = sqrtf(fmaxf(0.0f, 1.0f - k * k));
    for (int i = 0; i < 30 && fabsf(a - b) > 1e-7f * a; ++i) {
        const float an = 0.5f * (a + b);
        b = sqrtf(a * b);
        a = an;
    }
    return 3.14159265358979f / (2.0f * a);
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
__device__ inline int mcc_collide(const MccSpecies& m, int s, Stream& rs, float& vx, float& vy, float& vz,
                                  float vr2, float vz2, float vt2, bool& partner_update, float& pvx, float& pvy,
                                  float& pvz)
{
    partner_update = false;
    const float dvx = vx - vr2, dvz = vz - vz2, dvt = vy - vt2;
    const float v_rel = sqrtf(dvx * dvx + dvz * dvz + dvt * dvt);
    const float m2 = (float)(m.t_mass[s] / m.mass);  // masses relative to the primary's
    const float g2 = (float)(rs.uni() * m.rates[s]);
    const float dens = (float)m.t_density[s];
    float acc = 0.0f;
    int hit = -1;
    for (int q = m.inter_begin[s]; q < m.inter_end[s]; ++q) {
        acc += mcc_sigma_v(m.inter[q], m.tables, v_rel) * dens;
        if (acc > g2) {
            hit = q;
            break;
        }
    }
    if (hit < 0) return MCC_NULL;
    const InterDev in = m.inter[hit];
    const float mass = 1.0f;
    const float tmp = 1.0f / (mass + m2);
    switch (in.type) {
    case SUPERELASTIC: {
        const double E = 0.5 * in.mu * (double)v_rel * v_rel + in.DE;
        const float vr = (float)sqrt(2 * E / in.mu);
        float rx, rz, ry;
        mcc_rot(rs, vr, rx, rz, ry);
        vx = (rx * m2 + vx * mass + vr2 * m2) * tmp;
        vz = (ry * m2 + vz * mass + vz2 * m2) * tmp;
        vy = (rz * m2 + vy * mass + vt2 * m2) * tmp;
    } break;
    case COULOMB:
    case ELASTIC: {
        const float cx = (vx * mass + vr2 * m2) * tmp;
        const float cz = (vz * mass + vz2 * m2) * tmp;
        const float cy = (vy * mass + vt2 * m2) * tmp;
        float rx, ry, rz;
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
        float v1x = (vx - vr2) * m2 * tmp;
        float v1y = (vz - vz2) * m2 * tmp;
        float v1z = (vy - vt2) * m2 * tmp;
        const float beta = sqrtf(rs.unif()) * (float)in.cutoff;
        if (beta > 1.0f) {  // Nanbu & Kitatani, J. Phys. D 28 (1995) 324
            const float b2 = beta * beta;
            const float tt = sqrtf(b2 * b2 - 1.0f);
            const float xi0 = sqrtf(b2 - tt), xi1 = sqrtf(b2 + tt);
            const float theta = mcc_ellint_K(xi0 / xi1) * 1.41421356f * beta / xi1;
            mcc_deflect(rs, 3.14159265358979f - 2 * theta, v1x, v1y, v1z);
        } else {
            const float len = sqrtf(v1x * v1x + v1y * v1y + v1z * v1z);
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

// Shared-memory copy of a species' MCC data (MccSpecies and the interaction
// list) and, when small enough, its cross-section tables.
constexpr int kStageTables = 4096;  // table doubles staged in shared memory (32 KB)

struct MccStage {
    MccSpecies m;
    InterDev inter[kMaxInteractions];
};

// Block-wide copy into shared memory; the caller synchronises the block,
// calls mcc_stage_pointers from one thread, and synchronises again.
__device__ inline void mcc_stage(const CollideArgs& a, MccStage& st, double* s_tab)
{
    static_assert(sizeof(MccSpecies) % 8 == 0 && sizeof(InterDev) % 8 == 0, "word copies");
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(a.mcc);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&st.m);
    for (int w = threadIdx.x; w < (int)(sizeof(MccSpecies) / 8); w += blockDim.x) dst[w] = src[w];
    const int ni = min(a.n_inter, kMaxInteractions);
    src = reinterpret_cast<const unsigned long long*>(a.inter);
    dst = reinterpret_cast<unsigned long long*>(st.inter);
    for (int w = threadIdx.x; w < ni * (int)(sizeof(InterDev) / 8); w += blockDim.x) dst[w] = src[w];
    if (s_tab && a.n_tables <= kStageTables)
        for (int w = threadIdx.x; w < a.n_tables; w += blockDim.x) s_tab[w] = a.tables[w];
}

__device__ inline void mcc_stage_pointers(const CollideArgs& a, MccStage& st, double* s_tab)
{
    st.m.inter = st.inter;
    if (s_tab && a.n_tables <= kStageTables) st.m.tables = s_tab;
}

// Scatter of one particle against a target drawn from the null-collision
// rates, when every target species is a Maxwellian background (no particles):
// the partner velocity is rndv (src/particles.hpp:188-192).  Updates
// (vx, vy, vz); returns MCC_HIT or MCC_NULL.  Draws from rs.
static __device__ __forceinline__ int scatter_background(const MccSpecies& m, Stream& rs, float& vx, float& vy,
                                                         float& vz)
{
    const int s = mcc_pick_target(m, rs);
    const float sig = (float)m.t_sigma_v[s];
    const float vr2 = rs.normalf() * sig;
    const float vz2 = rs.normalf() * sig;
    const float vt2 = rs.normalf() * sig;
    bool pu;
    float pvx, pvy, pvz;
    return mcc_collide(m, s, rs, vx, vy, vz, vr2, vz2, vt2, pu, pvx, pvy, pvz);
}

// the same with the particle's own stream of the step
static __device__ __forceinline__ int collide_background(const MccSpecies& m, uint64_t seed, uint32_t species,
                                                         uint32_t pid, uint64_t step, float& vx, float& vy, float& vz)
{
    Stream rs(seed, species, pid, TAG_COLLIDE, step);
    return scatter_background(m, rs, vx, vy, vz);
}

// One candidate c of the list: the whole of BaseSpecies::scatter for it.
// Returns MCC_HIT, MCC_NULL or MCC_NOPARTNER.  The list and the particle
// arrays are read through L2 (ld.global.cg): the kernel that wrote them may
// still have been running when this one started (programmatic launch).
static __device__ __noinline__ int collide_one(const CollideArgs& a, const MccSpecies& m, unsigned long long c)
{
    const uint32_t p = __ldcg(a.cand + c);
    const float4 rec = __ldcg(a.cand_rec + c);
    const uint32_t pid = __float_as_uint(rec.w);
    float vx = rec.x, vy = rec.y, vz = rec.z;
    int r;
    int64_t partner = -1;
    int s = 0;
    bool pu = false;
    float pvx = 0.f, pvy = 0.f, pvz = 0.f;
    if (!a.any_target_slots) {
        r = collide_background(m, a.seed, a.species, pid, a.step, vx, vy, vz);
    } else {
        Stream rs(a.seed, a.species, pid, TAG_COLLIDE, a.step);
        s = mcc_pick_target(m, rs);
        float vr2, vz2, vt2;
        if (!a.t_has_slots[s]) {
            const float sig = (float)m.t_sigma_v[s];
            vr2 = rs.normalf() * sig;
            vz2 = rs.normalf() * sig;
            vt2 = rs.normalf() * sig;
        } else {
            Stream ps(a.seed, a.species, pid, TAG_PARTNER, a.step);
            const int64_t nt = a.t_n[s];
            for (int tries = 0; tries < 256 && nt > 0; ++tries) {
                const uint64_t hi = ps.next();
                const int64_t q = (int64_t)(((hi << 32) | ps.next()) % (uint64_t)nt);
                if (__ldcg(a.t_x[s] + q) != kDead) {  // any live particle, itself included (random_particle)
                    partner = q;
                    break;
                }
            }
            if (partner < 0) return MCC_NOPARTNER;
            vr2 = __ldcg(a.t_vx[s] + partner);
            vz2 = __ldcg(a.t_vz[s] + partner);
            vt2 = __ldcg(a.t_vy[s] + partner);
        }
        r = mcc_collide(m, s, rs, vx, vy, vz, vr2, vz2, vt2, pu, pvx, pvy, pvz);
    }
    if (r != MCC_HIT) return MCC_NULL;
    a.vx[p] = vx;
    a.vy[p] = vy;
    a.vz[p] = vz;
    if (pu && partner >= 0) {
        a.t_vx[s][partner] = pvx;
        a.t_vy[s][partner] = pvy;
        a.t_vz[s][partner] = pvz;
    }
    return MCC_HIT;
}

}  // namespace mag
