// CPU oracle for the mag2d PIC-MCC step — TEST INFRASTRUCTURE ONLY.
// See mag2d_oracle.h.  Our own restatement of the reference algorithm in FP64;
// the reference's floating-point operations are kept in the same order and the
// same types (including the float-valued uni()/rnor()/rexp()) so that results
// agree bit for bit when both are compiled without FMA contraction.
#include "mag2d_oracle.h"

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;

const double kEps0 = 8.854187817e-12;  // src/param.cpp:8
const double kKB = 1.380662e-23;       // src/param.cpp:9
const double kQe = 1.602189e-19;       // src/param.cpp:10

enum { FIXED = 0, FIXED_RF = 1, FREE = 2, BOUNDARY = 3 };  // src/fields.hpp:20

inline double sqr(double x) { return x * x; }

// mod() of src/mymath.cpp:62-67
inline double mod(double x, double y)
{
    if (x >= 0.0 && x <= y) return x;
    return x - y * int(x / y) + (x < 0 ? y : 0);
}

// ---------------------------------------------------------------------------
// Random numbers: Marsaglia's SHR3 with the Marsaglia-Tsang ziggurat method
// (J. Stat. Software 5(8), 2000), as used by src/random.cpp:19-336.  Types
// follow the reference: uni() is float, rnor()/rexp() are float.
// ---------------------------------------------------------------------------
struct Rng {
    uint32_t jsr = 123456789, jz = 0, iz = 0;
    int32_t hz = 0;
    uint32_t kn[128], ke[256];
    float wn[128], fn[128], we[256], fe[256];

    Rng() { tables(); seed((uint32_t)0); }

    uint32_t shr3()  // random.cpp:33-36
    {
        jz = jsr;
        jsr ^= (jsr << 13);
        jsr ^= (jsr >> 17);
        jsr ^= (jsr << 5);
        return jz + jsr;
    }
    uint32_t iuni() { return shr3(); }
    float uni() { return (float)(.5 + (double)(int32_t)iuni() * 2.3283064365386963e-10); }  // :42

    void seed(uint32_t s)  // random.cpp:200-208: three draws feed the unused MWC/CONG state
    {
        jsr = 123456789;
        jsr ^= s;
        shr3();
        shr3();
        shr3();
    }

    float rnor()  // random.cpp:49-52
    {
        hz = (int32_t)iuni();
        iz = (uint32_t)hz & 127;
        uint32_t ahz = hz < 0 ? (uint32_t)(-(int64_t)hz) : (uint32_t)hz;
        if (ahz < kn[iz]) return (float)hz * wn[iz];
        return nfix();
    }
    float rexp()  // random.cpp:54-57
    {
        jz = iuni();
        iz = jz & 255;
        if (jz < ke[iz]) return (float)jz * we[iz];
        return efix();
    }
    float nfix()  // random.cpp:294-318
    {
        const float r = 3.442620f;
        float x, y;
        for (;;) {
            x = (float)hz * wn[iz];
            if (iz == 0) {
                do {
                    x = (float)(-logf(uni()) * 0.2904764);
                    y = -logf(uni());
                } while (y + y < x * x);
                return (hz > 0) ? r + x : -r - x;
            }
            if (fn[iz] + uni() * (fn[iz - 1] - fn[iz]) < exp(-.5 * x * x)) return x;
            hz = (int32_t)shr3();
            iz = (uint32_t)hz & 127;
            if (std::fabs((double)hz) < (double)kn[iz]) return (float)hz * wn[iz];
        }
    }
    float efix()  // random.cpp:322-335
    {
        float x;
        for (;;) {
            if (iz == 0) return (float)(7.69711 - logf(uni()));
            x = (float)jz * we[iz];
            if (fe[iz] + uni() * (fe[iz - 1] - fe[iz]) < expf(-x)) return x;
            jz = shr3();
            iz = jz & 255;
            if (jz < ke[iz]) return (float)jz * we[iz];
        }
    }
    void tables()  // random.cpp:211-244, constants of the published method
    {
        const double m1 = 2147483648.0, m2 = 4294967296.;
        double dn = 3.442619855899, tn = dn, vn = 9.91256303526217e-3, q;
        double de = 7.697117470131487, te = de, ve = 3.949659822581572e-3;
        q = vn / exp(-.5 * dn * dn);
        kn[0] = (uint32_t)((dn / q) * m1);
        kn[1] = 0;
        wn[0] = (float)(q / m1);
        wn[127] = (float)(dn / m1);
        fn[0] = 1.f;
        fn[127] = (float)exp(-.5 * dn * dn);
        for (int i = 126; i >= 1; i--) {
            dn = sqrt(-2. * log(vn / dn + exp(-.5 * dn * dn)));
            kn[i + 1] = (uint32_t)((dn / tn) * m1);
            tn = dn;
            fn[i] = (float)exp(-.5 * dn * dn);
            wn[i] = (float)(dn / m1);
        }
        q = ve / exp(-de);
        ke[0] = (uint32_t)((de / q) * m2);
        ke[1] = 0;
        we[0] = (float)(q / m2);
        we[255] = (float)(de / m2);
        fe[0] = 1.f;
        fe[255] = (float)exp(-de);
        for (int i = 254; i >= 1; i--) {
            de = -log(ve / de + exp(-de));
            ke[i + 1] = (uint32_t)((de / te) * m2);
            te = de;
            fe[i] = (float)exp(-de);
            we[i] = (float)(de / m2);
        }
    }
    // isotropic direction of length len (random.cpp:103-115)
    void rot(double len, double& x, double& y, double& z)
    {
        double cs = (float)(1.0f - 2.0f * uni());
        x = len * cs;
        cs = sqrt(1 - sqr(cs));
        double sp, cp;
        sincos(2 * M_PI * uni(), &sp, &cp);
        y = len * cs * sp;
        z = len * cs * cp;
    }
    void rot(double& x, double& y, double& z)  // random.cpp:117-131
    {
        double len = sqrt(sqr(x) + sqr(y) + sqr(z));
        rot(len, x, y, z);
    }
    // rotation of (x,y,z) by 'angle' about a random axis (random.cpp:133-175)
    void deflect(double angle, double& x, double& y, double& z)
    {
        double len = tan(angle / 2.0);
        double x1, y1, z1;
        double tmp = (float)(1.0f - 2.0f * uni());
        x1 = len * tmp;
        tmp = sqrt(1 - sqr(tmp));
        double sp, cp;
        sincos(2 * M_PI * uni(), &sp, &cp);
        y1 = len * tmp * sp;
        z1 = len * tmp * cp;
        double tx = y * z1 - z * y1;
        double ty = z * x1 - x * z1;
        double tz = x * y1 - y * x1;
        tmp = len / sqrt(sqr(tx) + sqr(ty) + sqr(tz));
        tx *= tmp;
        ty *= tmp;
        tz *= tmp;
        double xp = x - y * tz + z * ty;
        double yp = y - z * tx + x * tz;
        double zp = z - x * ty + y * tx;
        tmp = 2.0 / (1 + len * len);
        x1 = tx * tmp;
        y1 = ty * tmp;
        z1 = tz * tmp;
        x += -yp * z1 + zp * y1;
        y += -zp * x1 + xp * z1;
        z += -xp * y1 + yp * x1;
    }
    double radius() { return (double)sqrtf(uni()); }  // random.cpp:177
};

// ---------------------------------------------------------------------------
// 2D node field (src/Field2D.hpp:14-168), row-major with z fastest.
// ---------------------------------------------------------------------------
struct Field {
    int jmax = 0, lmax = 0;
    double dx = 0, dy = 0, idx = 0, idy = 0, xmin = 0, ymin = 0;
    std::vector<double> d;

    void resize(int nx, int nz, double _dx, double _dy, double _xmin = 0, double _ymin = 0)
    {
        jmax = nx;
        lmax = nz;
        dx = _dx;
        dy = _dy;
        idx = 1. / dx;
        idy = 1. / dy;
        xmin = _xmin;
        ymin = _ymin;
        d.assign((size_t)nx * nz, 0.0);
    }
    double& at(int i, int j) { return d[(size_t)i * lmax + j]; }
    double at(int i, int j) const { return d[(size_t)i * lmax + j]; }
    void reset() { std::fill(d.begin(), d.end(), 0.0); }

    void accumulate(double charge, double x, double y)  // Field2D.hpp:45-62
    {
        x -= xmin;
        y -= ymin;
        int i = (int)(x * idx);
        int j = (int)(y * idy);
        double u = x * idx - i;
        double v = y * idy - j;
        if (i < 0 || i > jmax - 1 || j < 0 || j > lmax - 1)
            throw std::runtime_error("Field2D::accumulate() outside of range\n");
        at(i, j) += (1 - u) * (1 - v) * charge;
        at(i + 1, j) += u * (1 - v) * charge;
        at(i, j + 1) += (1 - u) * v * charge;
        at(i + 1, j + 1) += u * v * charge;
    }

    double interpolate(double x, double y) const  // Field2D.hpp:64-78
    {
        x -= xmin;
        y -= ymin;
        int i = (int)(x * idx);
        int j = (int)(y * idy);
        double u = x * idx - i;
        double v = y * idy - j;
        if (i < 0 || i > jmax - 1 || j < 0 || j > lmax - 1)
            throw std::runtime_error("Field2D::interpolate() outside of range\n");
        return (1 - u) * (1 - v) * at(i, j) + u * (1 - v) * at(i + 1, j) + (1 - u) * v * at(i, j + 1) +
               u * v * at(i + 1, j + 1);
    }

    // staggered-difference gradient, bilinearly interpolated (Field2D.hpp:80-168)
    void grad(double x, double y, double& gx, double& gy) const
    {
        int i, j;
        double g1, g2, g3, g4, fx, fy;
        x -= xmin;
        y -= ymin;
        i = (int)(x * idx + 0.5);
        j = (int)(y * idy);
        j = std::min(j, lmax - 2);
        if (i > 0 && i < jmax - 1) {
            g1 = (at(i, j) - at(i - 1, j)) * idx;
            g2 = (at(i, j + 1) - at(i - 1, j + 1)) * idx;
            g3 = (at(i + 1, j + 1) - at(i, j + 1)) * idx;
            g4 = (at(i + 1, j) - at(i, j)) * idx;
            fx = x * idx - i + .5;
            fy = y * idy - j;
            gx = g1 * (1 - fx) * (1 - fy) + g2 * (1 - fx) * fy + g3 * fx * fy + g4 * fx * (1 - fy);
        } else if (i == jmax - 1) {
            g1 = (at(i, j) - at(i - 1, j)) * idx;
            g2 = (at(i, j + 1) - at(i - 1, j + 1)) * idx;
            fy = y * idy - j;
            gx = g1 * (1 - fy) + g2 * fy;
        } else if (i == 0) {
            g3 = (at(i + 1, j + 1) - at(i, j + 1)) * idx;
            g4 = (at(i + 1, j) - at(i, j)) * idx;
            fy = y * idy - j;
            gx = g3 * fy + g4 * (1 - fy);
        }
        i = (int)(x * idx);
        j = (int)(y * idy + 0.5);
        i = std::min(i, jmax - 2);
        if (j > 0 && j < lmax - 1) {
            g1 = (at(i, j) - at(i, j - 1)) * idy;
            g2 = (at(i + 1, j) - at(i + 1, j - 1)) * idy;
            g3 = (at(i + 1, j + 1) - at(i + 1, j)) * idy;
            g4 = (at(i, j + 1) - at(i, j)) * idy;
            fx = x * idx - i;
            fy = y * idy - j + 0.5;
            gy = g1 * (1 - fx) * (1 - fy) + g2 * (1 - fy) * fx + g3 * fx * fy + g4 * fy * (1 - fx);
        } else if (j == lmax - 1) {
            g1 = (at(i, j) - at(i, j - 1)) * idy;
            g2 = (at(i + 1, j) - at(i + 1, j - 1)) * idy;
            fx = x * idx - i;
            gy = g1 * (1 - fx) + g2 * fx;
        } else if (j == 0) {
            g3 = (at(i + 1, j + 1) - at(i + 1, j)) * idy;
            g4 = (at(i, j + 1) - at(i, j)) * idy;
            fx = x * idx - i;
            gy = g3 * fx + g4 * (1 - fx);
        }
    }
};

struct Particle {
    double x, y, z, vx, vy, vz, ttd;
    bool empty;
};

struct Species;

// Interaction (src/particles.hpp:49-92, :415-433; src/particles.cpp:19-26)
struct Interaction {
    int type;
    double DE, rate, cutoff;
    Species* primary;
    Species* secondary;
    std::vector<double> tE, tS;  // vec_interpolate table (src/tabulate.cpp:89-141)
    double table(double x) const
    {
        const int n = (int)tE.size();
        if (x >= tE[n - 1]) return tS[n - 1];
        if (x <= tE[0]) return tS[0];
        int j1 = 0, j2 = n - 1, j3;
        while ((j2 - j1) > 1) {
            j3 = (j1 + j2) / 2;
            if (x < tE[j3]) j2 = j3;
            else j1 = j3;
        }
        double w = (x - tE[j1]) / (tE[j2] - tE[j1]);
        return tS[j1] * (1 - w) + tS[j2] * w;
    }
    double mu() const;
    double EeV(double v) const { return 0.5 * mu() * v * v / kQe; }
    double E(double v) const { return 0.5 * mu() * v * v; }
    double v_rel(double e) const { return sqrt(2 * e / mu()); }
    double coulomb_sigma(double e) const;
    double sigma_v(double v) const
    {
        if (type == ORC_COULOMB) return coulomb_sigma(EeV(v)) * v;
        if (!tE.empty()) return table(EeV(v)) * v;
        return rate;
    }
};

struct Species {
    std::string name;
    double mass, charge, dt, density, temperature, E_max, v_max, lifetime, t;
    unsigned long niter = 0;
    int64_t ncoll = 0;  // candidates (null collisions included)
    int64_t nreal = 0;  // collisions that selected an interaction
    std::vector<Particle> p;
    std::vector<int> freelist;  // BaseSpecies::empty (particles.hpp:100)
    Field rho;
    std::vector<Interaction*> interactions;
    std::vector<std::vector<Interaction*>> by_species;
    std::vector<double> rates;
    std::vector<Species*> speclist;

    double veV(double e) const { return sqrt(e * kQe / mass * 2.0); }
    int n_particles() const { return (int)(p.size() - freelist.size()); }
    void resize(unsigned n)  // particles.cpp:95-107
    {
        unsigned old = (unsigned)p.size();
        if (n > old) {
            p.resize(n);
            for (unsigned i = old; i < n; i++) {
                p[i].empty = true;
                freelist.push_back((int)i);
            }
        }
    }
    int insert()  // particles.hpp:237-247
    {
        if (freelist.empty()) resize(int(p.size() * 1.1) + 1);
        int k = freelist.back();
        if (p[k].empty == false) throw std::runtime_error("error inserting particle");
        freelist.pop_back();
        p[k].empty = false;
        return k;
    }
    void remove(int n)  // particles.hpp:223-232
    {
        if (p[n].empty) throw std::runtime_error("removing empty particle from " + name);
        p[n].empty = true;
        freelist.push_back(n);
    }
};

double Interaction::mu() const { return primary->mass * secondary->mass / (primary->mass + secondary->mass); }

double Interaction::coulomb_sigma(double e) const  // particles.cpp:19-26
{
    e *= kQe;
    double lambda_D = sqrt(kEps0 * kKB * primary->temperature /
                           (primary->density * primary->charge * primary->charge));
    double Lambda = primary->charge * secondary->charge / (4 * M_PI * kEps0 * e);
    return M_PI * Lambda * Lambda * log(lambda_D / Lambda);
}

// Fields::u_smooth (fields.cpp:28-111) with its default arguments: the 3x3
// weights 1, 1/2 (edges), 1/4 (corners) summed in the reference's order and
// divided by 4, from a copy of the input.  The reference indexes uTmp[i][j+1]
// up to j+1 = lmax on one contiguous allocation (Array.hpp:19-22), i.e. the
// flat index i*lmax+j+1, which is column 0 of row i+1; the single read one
// past the array (i = jmax-2, j = lmax-1, neighbour i+1, j+1) is taken as 0.
void smooth_flat(int nx, int nz, const double* t, double* out)
{
    const long long n = (long long)nx * nz;
    for (long long k = 0; k < n; ++k) out[k] = t[k];
    auto at = [&](long long f) { return f < n ? t[f] : 0.0; };
    for (int i = 1; i < nx - 1; i++)
        for (int j = 1; j <= nz - 1; j++) {
            const long long f = (long long)i * nz + j;
            double sum = at(f) + at(f - nz) * 0.5 + at(f + nz) * 0.5 + at(f - 1) * 0.5 + at(f + 1) * 0.5 +
                         at(f - nz - 1) * 0.25 + at(f + nz - 1) * 0.25 + at(f - nz + 1) * 0.25 +
                         at(f + nz + 1) * 0.25;
            out[f] = sum / 4.0;
        }
}

}  // namespace

struct orc_sim {
    orc_config c;
    // derived Param values (param.cpp:209-225)
    double dx, dz, idx, idz, V, dV, dy, x_min = 0, z_min = 0, x_max, z_max;
    std::vector<signed char> mask;
    std::vector<double> voltage;
    Field u, uRF, rho, Bra, Bza;
    bool have_bfield = false;
    // banded LU of the row-stencil operator (fields.cpp:136-276 solved with UMFPACK_At)
    int n = 0, bw = 0;
    std::vector<double> lu;
    bool factored = false;
    Rng rnd;
    std::vector<Species*> sp;
    std::vector<Interaction*> ints;
    unsigned long iter = 0;

    ~orc_sim()
    {
        for (Species* s : sp) delete s;
        for (Interaction* i : ints) delete i;
    }
    double& L(int r, int c) { return lu[(size_t)r * (2 * bw + 1) + (c - r + bw)]; }

    bool is_free(double r, double z) const  // fields.hpp:94-101
    {
        int i = (int)(r * idx);
        int j = (int)(z * idz);
        const int N = c.z_sampl;
        return mask[(size_t)i * N + j] == FREE || mask[(size_t)(i + 1) * N + j] == FREE ||
               mask[(size_t)i * N + j + 1] == FREE || mask[(size_t)(i + 1) * N + j + 1] == FREE;
    }

    void E(double x, double y, double& gx, double& gy, double time) const  // fields.hpp:124-150
    {
        if (c.geometry_empty && !c.selfconsistent) {
            gx = 0.;
            gy = c.extern_field;
            return;
        }
        u.grad(x, y, gx, gy);
        if (c.rf) {
            double rx, ry;
            uRF.grad(x, y, rx, ry);
            double phase = mod(c.rf_omega * time, 10000000 * M_PI);
            phase = c.rf_amplitude * cos(phase) + c.rf_U0;
            gx += rx * phase;
            gy += ry * phase;
        }
        gx = -gx;
        gy = -gy;
    }
    void B(double x, double y, double& br, double& bz, double& bt) const  // fields.hpp:152-177
    {
        if (c.magnetic_field_const) {
            br = c.Br;
            bz = c.Bz;
            bt = c.Bt;
        } else {
            br = Bra.interpolate(x, y);
            bz = Bza.interpolate(x, y);
            bt = 0.00;
        }
    }

    // Matrix assembly (fields.cpp:136-259) as the row stencil that UMFPACK_At solves,
    // then a banded LU factorisation without pivoting.
    void factor()
    {
        const int M = c.x_sampl, N = c.z_sampl;
        n = M * N;
        bw = N;
        lu.assign((size_t)n * (2 * bw + 1), 0.0);
        for (int i = 0; i < M; i++)
            for (int j = 0; j < N; j++) {
                const int k = j + N * i;
                const signed char m = mask[k];
                if (m == FIXED || m == FIXED_RF) {
                    L(k, k) += 1;
                } else if (c.coord == 1 && i == 0 && j > 0 && j < N - 1) {
                    double k2 = 1.0 / (dz * dz);
                    double k3 = 1.0 / (dx * dx * 0.25);
                    L(k, k - 1) += k2;
                    L(k, k) += -2.0 * k2 - k3;
                    L(k, k + 1) += k2;
                    L(k, k + N) += k3;
                } else if (c.coord == 1) {
                    double k1 = (i - 0.5) / (dx * dx * i);
                    double k2 = 1.0 / (dz * dz);
                    double k3 = (i + 0.5) / (dx * dx * i);
                    L(k, k - N) += k1;
                    L(k, k - 1) += k2;
                    L(k, k) += -2.0 * k2 - k1 - k3;
                    L(k, k + 1) += k2;
                    L(k, k + N) += k3;
                } else {
                    L(k, k - N) += 1.0;
                    L(k, k - 1) += 1.0;
                    L(k, k) += -4;
                    L(k, k + 1) += 1.0;
                    L(k, k + N) += 1.0;
                }
            }
        for (int k = 0; k < n; ++k) {
            const double piv = L(k, k);
            const int rmax = k + bw < n - 1 ? k + bw : n - 1;
            for (int r = k + 1; r <= rmax; ++r) {
                double& lrk = L(r, k);
                if (lrk == 0.0) continue;
                lrk /= piv;
                const double m = lrk;
                for (int cc = k + 1; cc <= rmax; ++cc) L(r, cc) -= m * L(k, cc);
            }
        }
        factored = true;
    }
    void lu_solve(const double* b, double* x)
    {
        std::vector<double> y(b, b + n);
        for (int r = 0; r < n; ++r) {
            const int c0 = r - bw > 0 ? r - bw : 0;
            double acc = y[r];
            for (int cc = c0; cc < r; ++cc) acc -= L(r, cc) * y[cc];
            y[r] = acc;
        }
        for (int r = n - 1; r >= 0; --r) {
            const int c1 = r + bw < n - 1 ? r + bw : n - 1;
            double acc = y[r];
            for (int cc = r + 1; cc <= c1; ++cc) acc -= L(r, cc) * x[cc];
            x[r] = acc / L(r, r);
        }
    }
    // Fields::boundary_solve / boundary_solve_rf (fields.cpp:278-348)
    void boundary_solve(bool rf_solve)
    {
        if (!factored) factor();
        const int M = c.x_sampl, N = c.z_sampl;
        for (int i = 0; i < M; i++)
            for (int j = 0; j < N; j++) {
                const size_t k = (size_t)i * N + j;
                const signed char m = mask[k];
                double& r = rho.d[k];
                if (m == FIXED) r = rf_solve ? 0 : voltage[k];
                else if (m == FIXED_RF) r = rf_solve ? voltage[k] : 0;
                else if (c.coord == 1) {
                    if (i > 0) r *= -1.0 / kEps0 / (M_PI * dx * dx * 2.0 * i * dz) * c.macroparticle_factor;
                    else r *= -1.0 / kEps0 / (M_PI * dx * dx * 0.25 * dz) * c.macroparticle_factor;
                } else
                    r *= -sqr(dx) / kEps0 / dV;
            }
        lu_solve(rho.d.data(), rf_solve ? uRF.d.data() : u.d.data());
    }

    // Fields::u_smooth() as Pic::advance / advance_init call it (pic.cpp:336, 372)
    void smooth_u()
    {
        const std::vector<double> t = u.d;
        smooth_flat(u.jmax, u.lmax, t.data(), u.d.data());
    }

    // BaseSpecies::scatter (particles.cpp:208-365)
    void scatter(Species& s, Particle& q)
    {
        s.ncoll++;
        double gamma = rnd.uni() / s.lifetime;
        double tmp = 0.0;
        size_t specid;
        for (specid = 0; specid < s.rates.size() - 1; specid++) {
            tmp += s.rates[specid];
            if (tmp > gamma) break;
        }
        Species& t = *s.speclist[specid];
        double vr2, vz2, vt2;
        Particle* partner = nullptr;
        if (t.p.size() == 0) {  // rndv (particles.hpp:188-192)
            vr2 = rnd.rnor() * t.v_max * M_SQRT1_2;
            vz2 = rnd.rnor() * t.v_max * M_SQRT1_2;
            vt2 = rnd.rnor() * t.v_max * M_SQRT1_2;
        } else {  // random_particle (particles.hpp:207-217)
            int i = rnd.iuni() % t.p.size();
            while (t.p[i].empty) i = rnd.iuni() % t.p.size();
            partner = &t.p[i];
            vr2 = partner->vx;
            vz2 = partner->vz;
            vt2 = partner->vy;
        }
        double v_rel = sqrt(sqr(q.vx - vr2) + sqr(q.vz - vz2) + sqr(q.vy - vt2));
        double m2 = t.mass;
        gamma = rnd.uni() * s.rates[specid];
        tmp = 0.0;
        std::vector<Interaction*>& list = s.by_species[specid];
        size_t intid;
        for (intid = 0; intid < list.size(); intid++) {
            tmp += list[intid]->sigma_v(v_rel) * t.density;
            if (tmp > gamma) break;
        }
        if (intid == list.size()) return;  // null collision
        s.nreal++;
        Interaction* in = list[intid];
        const double mass = s.mass;
        tmp = 1.0 / (mass + m2);
        switch (in->type) {
        case ORC_SUPERELASTIC: {
            double e = in->E(v_rel) + in->DE;
            double vr = in->v_rel(e);
            double rx, rz, ry;
            rnd.rot(vr, rx, rz, ry);
            q.vx = (rx * m2 + q.vx * mass + vr2 * m2) * tmp;
            q.vz = (ry * m2 + q.vz * mass + vz2 * m2) * tmp;
            q.vy = (rz * m2 + q.vy * mass + vt2 * m2) * tmp;
        } break;
        case ORC_COULOMB:
        case ORC_ELASTIC: {
            double cx = (q.vx * mass + vr2 * m2) * tmp;
            double cz = (q.vz * mass + vz2 * m2) * tmp;
            double cy = (q.vy * mass + vt2 * m2) * tmp;
            double rx, ry, rz;
            rnd.rot(v_rel, rx, ry, rz);
            q.vx = rx * m2 * tmp + cx;
            q.vz = rz * m2 * tmp + cz;
            q.vy = ry * m2 * tmp + cy;
            if (in->type == ORC_COULOMB && partner) {
                partner->vx = -rx * mass * tmp + cx;
                partner->vz = -rz * mass * tmp + cz;
                partner->vy = -ry * mass * tmp + cy;
            }
        } break;
        case ORC_CX:
            q.vx = vr2;
            q.vz = vz2;
            q.vy = vt2;
            break;
        case ORC_LANGEVIN: {
            double v1x = (q.vx - vr2) * m2 * tmp;
            double v1y = (q.vz - vz2) * m2 * tmp;
            double v1z = (q.vy - vt2) * m2 * tmp;
            double beta = rnd.radius() * in->cutoff;
            if (beta > 1.0) {  // Nanbu & Kitatani, J. Phys. D 28 (1995) 324
                double tt = sqrt(beta * beta * beta * beta - 1.0);
                double xi0 = sqrt(beta * beta - tt);
                double xi1 = sqrt(beta * beta + tt);
                double zeta = xi0 / xi1;
                double theta = std::comp_ellint_1(zeta) * M_SQRT2 * beta / xi1;
                double chi = M_PI - 2 * theta;
                rnd.deflect(chi, v1x, v1y, v1z);
            } else {
                rnd.rot(v1x, v1y, v1z);
            }
            q.vx = v1x + (q.vx * mass + vr2 * m2) * tmp;
            q.vz = v1y + (q.vz * mass + vz2 * m2) * tmp;
            q.vy = v1z + (q.vy * mass + vt2 * m2) * tmp;
        } break;
        default:
            throw std::runtime_error("scatter: interaction type not implemented\n");
        }
    }

    // Species<CYLINDRICAL>::advance_boris (particles.cpp:539-621)
    void boris_cyl(Species& s)
    {
        double fr = 0, fz = c.extern_field;
        double Bx = c.Br, Bz = c.Bz, By = c.Bt;
        const double qmdt = s.charge / s.mass * s.dt;
        const double prob = 1.0 - exp(-s.dt / s.lifetime);
        for (size_t k = 0; k < s.p.size(); ++k) {
            Particle& I = s.p[k];
            if (I.empty) continue;
            E(I.x, I.z, fr, fz, s.niter * s.dt);
            B(I.x, I.z, Bx, Bz, By);
            I.vx += fr * qmdt / 2.0;
            I.vz += fz * qmdt / 2.0;
            double tmp = s.charge * s.dt / (2.0 * s.mass);
            double tx = Bx * tmp, ty = By * tmp, tz = Bz * tmp;
            double vpr = I.vx + I.vy * tz - I.vz * ty;
            double vpt = I.vy + I.vz * tx - I.vx * tz;
            double vpz = I.vz + I.vx * ty - I.vy * tx;
            tmp = 2.0 / (1 + sqr(tx) + sqr(ty) + sqr(tz));
            double sx = tx * tmp, sy = ty * tmp, sz = tz * tmp;
            I.vx = I.vx + vpt * sz - vpz * sy;
            I.vy = I.vy + vpz * sx - vpr * sz;
            I.vz = I.vz + vpr * sy - vpt * sx;
            I.vx += fr * qmdt / 2.0;
            I.vz += fz * qmdt / 2.0;
            double x2 = I.x + I.vx * s.dt;
            double y2 = I.vy * s.dt;
            I.x = sqrt(sqr(x2) + sqr(y2));
            I.z += I.vz * s.dt;
            double sa = y2 / I.x, ca = x2 / I.x;
            if (I.x == 0) {
                sa = 0;
                ca = 1;
            }
            tmp = I.vx;
            I.vx = ca * I.vx + sa * I.vy;
            I.vy = -sa * tmp + ca * I.vy;
            if (rnd.uni() < prob) scatter(s, I);
        }
    }
    // Species<CARTESIAN>::advance_boris (particles.cpp:924-995)
    void boris_cart(Species& s)
    {
        double fx = 0, fz = c.extern_field;
        double Bx = c.Br, Bz = c.Bz, By = c.Bt;
        const double qmdt = s.charge / s.mass * s.dt;
        const double prob = 1.0 - exp(-s.dt / s.lifetime);
        for (size_t k = 0; k < s.p.size(); ++k) {
            Particle& I = s.p[k];
            if (I.empty) continue;
            E(I.x, I.z, fx, fz, s.niter * s.dt);
            B(I.x, I.z, Bx, Bz, By);
            I.vx += fx * qmdt / 2.0;
            I.vz += fz * qmdt / 2.0;
            double tmp = s.charge * s.dt / (2.0 * s.mass);
            double tx = Bx * tmp, ty = By * tmp, tz = Bz * tmp;
            double vpr = I.vx - I.vy * tz + I.vz * ty;
            double vpz = I.vz - I.vx * ty + I.vy * tx;
            double vpt = I.vy - I.vz * tx + I.vx * tz;
            tmp = 2.0 / (1 + sqr(tx) + sqr(ty) + sqr(tz));
            double sx = tx * tmp, sy = ty * tmp, sz = tz * tmp;
            I.vx = I.vx - vpt * sz + vpz * sy;
            I.vy = I.vy - vpz * sx + vpr * sz;
            I.vz = I.vz - vpr * sy + vpt * sx;
            I.vx += fx * qmdt / 2.0;
            I.vz += fz * qmdt / 2.0;
            I.x += I.vx * s.dt;
            I.z += I.vz * s.dt;
            if (rnd.uni() < prob) scatter(s, I);
        }
    }
    // advance_boris_init, cylindrical (particles.cpp:623-679) and Cartesian (:997-1050)
    void boris_init(Species& s)
    {
        double fx = 0, fz = c.extern_field;
        double Bx = c.Br, Bz = c.Bz, By = c.Bt;
        const double qmdt = c.coord == 1 ? -1.0 * s.charge / s.mass * s.dt : -s.charge / s.mass * s.dt;
        for (size_t k = 0; k < s.p.size(); ++k) {
            Particle& I = s.p[k];
            if (I.empty) continue;
            E(I.x, I.z, fx, fz, s.niter * s.dt);
            B(I.x, I.z, Bx, Bz, By);
            double tmp = -0.5 * s.charge * s.dt / (2.0 * s.mass);
            double tx = Bx * tmp, ty = By * tmp, tz = Bz * tmp;
            if (c.coord == 1) {
                double vpr = I.vx + I.vy * tz - I.vz * ty;
                double vpt = I.vy + I.vz * tx - I.vx * tz;
                double vpz = I.vz + I.vx * ty - I.vy * tx;
                tmp = 2.0 / (1 + sqr(tx) + sqr(ty) + sqr(tz));
                double sx = tx * tmp, sy = ty * tmp, sz = tz * tmp;
                I.vx = I.vx + vpt * sz - vpz * sy;
                I.vy = I.vy + vpz * sx - vpr * sz;
                I.vz = I.vz + vpr * sy - vpt * sx;
            } else {
                double vpr = I.vx - I.vy * tz + I.vz * ty;
                double vpz = I.vz - I.vx * ty + I.vy * tx;
                double vpt = I.vy - I.vz * tx + I.vx * tz;
                tmp = 2.0 / (1 + sqr(tx) + sqr(ty) + sqr(tz));
                double sx = tx * tmp, sy = ty * tmp, sz = tz * tmp;
                I.vx = I.vx - vpt * sz + vpz * sy;
                I.vy = I.vy - vpz * sx + vpr * sz;
                I.vz = I.vz - vpr * sy + vpt * sx;
            }
            I.vx += fx * qmdt / 2.0;
            I.vz += fz * qmdt / 2.0;
        }
    }
    // Species::advance_boundary (particles.hpp:370-411)
    void boundary(Species& s)
    {
        for (size_t k = 0; k < s.p.size(); ++k) {
            Particle& I = s.p[k];
            if (I.empty) continue;
            if (I.x < x_min || I.x > x_max || I.z < z_min || I.z > z_max) {
                if (c.boundary == 0) {
                    s.remove((int)k);
                    continue;
                } else {
                    I.x = fmod(I.x, x_max);
                    if (I.x < 0) I.x += x_max;
                    I.z = fmod(I.z, z_max);
                    if (I.z < 0) I.z += z_max;
                }
            }
            if (!c.electric_field_from_file) {
                if (!is_free(I.x, I.z)) {
                    s.remove((int)k);
                    continue;
                }
            }
            if (c.selfconsistent) s.rho.accumulate(s.charge, I.x, I.z);
        }
    }
    // Pic::advance (pic.cpp:330-358)
    void advance()
    {
        if (c.selfconsistent) {
            boundary_solve(false);
            if (c.u_smooth) smooth_u();
            rho.reset();
            for (Species* s : sp)
                if (s->n_particles() > 0) s->rho.reset();
        }
        for (Species* s : sp) {
            if (c.mover == 1) multicoll(*s);
            else if (c.coord == 1) boris_cyl(*s);
            else boris_cart(*s);
            boundary(*s);
            s->niter++;
            s->t += s->dt;
        }
        for (Species* s : sp)
            if (c.selfconsistent) add_rho(*s);
        iter++;
    }
    // Species<CARTESIAN>::advance_multicoll (particles.cpp:812-859): free flight in
    // the constant external field to time_to_death, scatter, redraw; the rest of
    // dt in free flight (the reference also counts niter and t here, and again in
    // Species::advance)
    void multicoll(Species& s)
    {
        const double fx = 0.0, fz = c.extern_field;  // Fields::E of the EMPTY geometry (fields.hpp:126-131)
        const double qm = s.charge / s.mass;
        const double dt = s.dt;
        for (Particle& I : s.p) {
            if (I.empty) continue;
            double local_time = 0.;
            double ttd;
            while (local_time + I.ttd < dt) {
                ttd = I.ttd;
                I.vx += fx * qm * ttd;
                I.vz += fz * qm * ttd;
                I.x += (I.vx + 0.5 * fx * qm * ttd) * ttd;
                I.z += (I.vz + 0.5 * fz * qm * ttd) * ttd;
                local_time += I.ttd;
                scatter(s, I);
                I.ttd = s.lifetime * rnd.rexp();
            }
            ttd = dt - local_time;
            I.vx += fx * qm * ttd;
            I.vz += fz * qm * ttd;
            I.x += (I.vx + 0.5 * fx * qm * ttd) * ttd;
            I.z += (I.vz + 0.5 * fz * qm * ttd) * ttd;
            I.ttd -= ttd;
        }
        s.niter++;
        s.t += dt;
    }
    void add_rho(Species& s)
    {
        for (size_t k = 0; k < rho.d.size(); ++k) rho.d[k] += s.rho.d[k];
    }
    // Pic::advance_init (pic.cpp:359-384)
    void advance_init()
    {
        if (c.selfconsistent) {
            for (Species* s : sp)
                if (s->n_particles() > 0) {
                    for (Particle& I : s->p)  // Species::accumulate (particles.hpp:358-367)
                        if (!I.empty) s->rho.accumulate(s->charge, I.x, I.z);
                    add_rho(*s);
                }
            boundary_solve(false);
            if (c.u_smooth) smooth_u();
            rho.reset();
            for (Species* s : sp)
                if (s->n_particles() > 0) add_rho(*s);
        }
        if (c.mover != 1)  // ADVANCE_MULTICOLL has no leapfrog start (particles.cpp:805-806)
            for (Species* s : sp) boris_init(*s);
    }
    // svmax_find (particles.cpp:190-206)
    static double svmax_find(const std::vector<Interaction*>& list, double vmax)
    {
        const int samples = 1000;
        double dv = vmax / samples, svmax = 0.0;
        for (double v = 0; v < vmax; v += dv) {
            double sv = 0;
            for (Interaction* in : list) sv += in->sigma_v(v);
            if (std::isnan(sv)) continue;
            if (sv > svmax) svmax = sv;
        }
        return svmax;
    }
    // lifetime_init (particles.cpp:142-170)
    void lifetime_init(Species& s)
    {
        double rate = 0;
        for (size_t i = 0; i < s.rates.size(); i++) {
            s.rates[i] = svmax_find(s.by_species[i], s.veV(s.E_max)) * s.speclist[i]->density;
            rate += s.rates[i];
        }
        s.lifetime = rate > 0.0 ? 1.0 / rate : INFINITY;
        for (Particle& I : s.p)
            if (!I.empty) I.ttd = rnd.rexp() * s.lifetime;
    }

    // initscript loaders, Cartesian (particles.cpp:685-749) and tracked particles (particles.hpp:297-309)
    void add_on_disk(Species& s, int np, double cx, double cy, double radius)
    {
        if (c.coord == 1) throw std::runtime_error("add_particles_on_disk is not defined for CYLINDRICAL in the reference\n");
        for (int i = 0; i < np; i++) {
            double x, y;
            do {
                x = (rnd.uni() - 0.5);
                y = (rnd.uni() - 0.5);
            } while (sqr(x) + sqr(y) > 0.25);
            x = x * 2 * radius + cx;
            y = y * 2 * radius + cy;
            if (x < x_min || x > x_max || y < z_min || y > z_max) continue;
            int ii = s.insert();
            Particle& q = s.p[ii];
            q.x = x;
            q.z = y;
            q.vx = rnd.rnor() * s.v_max * M_SQRT1_2;
            q.vz = rnd.rnor() * s.v_max * M_SQRT1_2;
            q.vy = rnd.rnor() * s.v_max * M_SQRT1_2;
        }
    }
    void add_everywhere(Species& s, int np)
    {
        if (c.coord == 1) throw std::runtime_error("add_particles_everywhere is not defined for CYLINDRICAL in the reference\n");
        for (int i = 0; i < np; i++) {
            int ii = s.insert();
            Particle& q = s.p[ii];
            q.x = (x_max - x_min) * (rnd.uni()) + x_min;
            q.y = (c.y_max - 0.0) * (rnd.uni()) + 0.0;
            q.z = (z_max - z_min) * (rnd.uni()) + z_min;
            q.vx = rnd.rnor() * s.v_max / (M_SQRT2);
            q.vy = rnd.rnor() * s.v_max / (M_SQRT2);
            q.vz = rnd.rnor() * s.v_max / (M_SQRT2);
            q.ttd = rnd.rexp() * s.lifetime;
        }
    }
    void add_bessel(Species& s, int np, double cx, double cy, double radius)
    {
        if (c.coord == 1) throw std::runtime_error("add_particles_bessel is not defined for CYLINDRICAL in the reference\n");
        for (int i = 0; i < np; i++) {
            double x, y, r = 0;
            const double bessel_root = 2.404825557695773;
            do {
                x = (double)(rnd.uni() * 2) - 1.0;
                y = (double)(rnd.uni() * 2) - 1.0;
                r = sqrt(sqr(x) + sqr(y));
            } while (r > 1.0 || rnd.uni() > std::cyl_bessel_j(0.0, r * bessel_root));
            x = x * radius + cx;
            y = y * radius + cy;
            if (x < x_min || x > x_max || y < z_min || y > z_max) continue;
            int ii = s.insert();
            Particle& q = s.p[ii];
            q.x = x;
            q.z = y;
            q.vx = rnd.rnor() * s.v_max * M_SQRT1_2;
            q.vz = rnd.rnor() * s.v_max * M_SQRT1_2;
            q.vy = rnd.rnor() * s.v_max * M_SQRT1_2;
        }
    }
    void add_tracked(Species& s, double x, double y, double vx, double vy, double vz)
    {
        int ii = s.insert();
        Particle& q = s.p[ii];
        q.x = x;
        q.z = y;
        q.y = 0;
        q.vx = vx;
        q.vy = vz;
        q.vz = vy;
    }
    // Pic::run_initscript (pic.cpp:241-328)
    void run_initscript(const char* path)
    {
        std::map<std::string, int> index;
        for (size_t i = 0; i < sp.size(); ++i) index[sp[i]->name] = (int)i;
        std::ifstream fr(path);
        std::string line;
        auto species = [&](const std::string& name) -> Species& {
            if (index.find(name) == index.end())
                throw std::runtime_error("Pic::run_initscript: unrecognized species type \"" + name + "\"\n");
            return *sp[index[name]];
        };
        auto num = [](const std::string& t) {
            std::istringstream is(t);
            double v;
            if (!(is >> v)) throw std::runtime_error("string2: error converting string " + t + " to T\n");
            return v;
        };
        auto inum = [](const std::string& t) {
            std::istringstream is(t);
            int v;
            if (!(is >> v)) throw std::runtime_error("string2: error converting string " + t + " to T\n");
            return v;
        };
        while (fr.good()) {
            std::getline(fr, line);
            if (!line.empty() && line[0] == '#') continue;
            std::istringstream is(line);
            std::vector<std::string> t;
            std::string tok;
            while (is >> tok) t.push_back(tok);
            if (t.empty()) continue;
            auto need = [&](size_t k) {
                if (t.size() != k)
                    throw std::runtime_error("Pic::run_initscript: wrong number of parameters (" +
                                             std::to_string(t.size()) + ") to " + t[0] + "\n");
            };
            if (t[0] == "add_particles_bessel") {
                need(6);
                add_bessel(species(t[1]), inum(t[2]), num(t[3]), num(t[4]), num(t[5]));
            }
            if (t[0] == "add_particles_everywhere") {
                need(3);
                add_everywhere(species(t[1]), inum(t[2]));
            }
            if (t[0] == "add_particles_on_disk") {
                need(6);
                add_on_disk(species(t[1]), inum(t[2]), num(t[3]), num(t[4]), num(t[5]));
            } else if (t[0] == "add_tracked_particle") {
                need(7);
                add_tracked(species(t[1]), num(t[2]), num(t[3]), num(t[4]), num(t[5]), num(t[6]));
            }
        }
    }
};

namespace {
template <class F>
int guard(F&& f)
{
    try {
        return f();
    } catch (std::exception& e) {
        g_err = e.what();
        return -1;
    }
}
}  // namespace

extern "C" {

const char* orc_last_error(void) { return g_err.c_str(); }

orc_sim* orc_create(const orc_config* cfg, const signed char* mask, const double* voltage)
{
    orc_sim* s = new orc_sim;
    s->c = *cfg;
    const orc_config& c = s->c;
    s->x_max = c.x_max;
    s->z_max = c.z_max;
    s->dx = c.x_max / (c.x_sampl - 1);  // param.cpp:209-225
    s->dz = c.z_max / (c.z_sampl - 1);
    s->idx = 1.0 / s->dx;
    s->idz = 1.0 / s->dz;
    s->V = c.n_particles_total / c.density_total;
    s->dV = s->V / ((c.x_sampl - 1) * (c.z_sampl - 1));
    s->dy = s->dV / (s->dx * s->dz);
    if (c.coord == 1) s->dy = 2 * M_PI / c.macroparticle_factor;
    const size_t nn = (size_t)c.x_sampl * c.z_sampl;
    s->mask.assign(mask, mask + nn);
    s->voltage.assign(voltage, voltage + nn);
    s->u.resize(c.x_sampl, c.z_sampl, s->dx, s->dz);
    s->uRF.resize(c.x_sampl, c.z_sampl, s->dx, s->dz);
    s->rho.resize(c.x_sampl, c.z_sampl, s->dx, s->dz);
    return s;
}

void orc_destroy(orc_sim* s) { delete s; }

int orc_add_species(orc_sim* s, const char* name, double mass, double charge, double dt, double density,
                    double temperature, double E_max)
{
    Species* p = new Species;
    p->name = name;
    p->mass = mass;
    p->charge = charge;
    p->dt = dt;
    p->density = density;
    p->temperature = temperature;
    // BaseSpecies constructor (particles.hpp:152-183)
    p->E_max = E_max > 0. ? E_max : temperature * kKB / kQe * 10.0;
    p->lifetime = INFINITY;
    p->t = 0;
    p->v_max = sqrt(2.0 * kKB * temperature / mass);
    p->rho.resize(s->c.x_sampl, s->c.z_sampl, s->dx, s->dz);
    s->sp.push_back(p);
    return (int)s->sp.size() - 1;
}

int orc_add_interaction(orc_sim* s, int primary, int secondary, int type, double DE_eV, double rate,
                        double cutoff, int n_table, const double* E_eV, const double* sigma)
{
    Interaction* in = new Interaction;
    in->type = type;
    in->DE = DE_eV * kQe;
    in->rate = rate;
    in->cutoff = cutoff;
    in->tE.assign(E_eV, E_eV + n_table);
    in->tS.assign(sigma, sigma + n_table);
    if (type == ORC_LANGEVIN) in->rate *= sqr(cutoff);
    in->primary = s->sp[primary];
    in->secondary = s->sp[secondary];
    s->ints.push_back(in);
    return (int)s->ints.size() - 1;
}

int orc_set_loaded_fields(orc_sim* s, int nx, int nz, double dx, double dz, double xmin, double zmin,
                          const double* u, const double* uRF)
{
    return guard([&]() {
        s->u.resize(nx, nz, dx, dz, xmin, zmin);
        std::copy(u, u + (size_t)nx * nz, s->u.d.begin());
        if (s->c.rf && uRF) {
            s->uRF.resize(nx, nz, dx, dz, xmin, zmin);
            std::copy(uRF, uRF + (size_t)nx * nz, s->uRF.d.begin());
        }
        s->rho.resize(nx, nz, dx, dz, xmin, zmin);
        s->x_max = xmin + (nx - 1) * dx;
        s->x_min = xmin;
        s->z_max = zmin + (nz - 1) * dz;
        s->z_min = zmin;
        for (Species* p : s->sp) p->rho.resize(nx, nz, dx, dz, xmin, zmin);
        return 0;
    });
}

int orc_set_bfield(orc_sim* s, int nx, int nz, double dx, double dz, double xmin, double zmin,
                   const double* Br, const double* Bz)
{
    s->Bra.resize(nx, nz, dx, dz, xmin, zmin);
    s->Bza.resize(nx, nz, dx, dz, xmin, zmin);
    std::copy(Br, Br + (size_t)nx * nz, s->Bra.d.begin());
    std::copy(Bz, Bz + (size_t)nx * nz, s->Bza.d.begin());
    s->have_bfield = true;
    return 0;
}

int orc_init(orc_sim* s)
{
    return guard([&]() {
        // Speclist (pic.cpp:27-80): interactions by target species, then lifetimes
        const size_t ns = s->sp.size();
        for (Species* p : s->sp) {
            p->speclist = s->sp;
            p->by_species.assign(ns, {});
            p->rates.assign(ns, 0.0);
        }
        for (Interaction* in : s->ints) {
            in->primary->interactions.push_back(in);
            size_t k = 0;
            while (s->sp[k] != in->secondary) ++k;
            in->primary->by_species[k].push_back(in);
        }
        for (Species* p : s->sp) s->lifetime_init(*p);
        // Pic constructor (pic.cpp:127-189)
        if (!s->c.electric_field_from_file) {
            s->boundary_solve(true);
            if (!s->c.selfconsistent) {
                s->boundary_solve(false);
                s->rho.reset();
            }
        }
        s->rho.reset();
        return 0;
    });
}

int orc_seed(orc_sim* s, uint32_t seed)
{
    s->rnd.seed(seed);
    return 0;
}

int orc_run_initscript(orc_sim* s, const char* path)
{
    return guard([&]() { s->run_initscript(path); return 0; });
}

int orc_set_particles(orc_sim* s, int sp, int n, const double* x, const double* z, const double* vx,
                      const double* vy, const double* vz)
{
    return guard([&]() {
        Species& p = *s->sp[sp];
        if (!p.p.empty()) throw std::runtime_error("orc_set_particles: species already holds particles\n");
        p.resize(n);
        for (int k = 0; k < n; ++k) p.insert();
        for (int i = 0; i < n; ++i) {
            Particle& q = p.p[i];
            q.x = x[i];
            q.y = 0.0;
            q.z = z[i];
            q.vx = vx[i];
            q.vy = vy[i];
            q.vz = vz[i];
            q.ttd = 0.0;
            q.empty = false;
        }
        return 0;
    });
}

int orc_n_slots(orc_sim* s, int sp) { return (int)s->sp[sp]->p.size(); }
int orc_n_live(orc_sim* s, int sp) { return s->sp[sp]->n_particles(); }

int orc_get_particles(orc_sim* s, int sp, double* out)
{
    const Species& p = *s->sp[sp];
    for (size_t i = 0; i < p.p.size(); ++i) {
        const Particle& q = p.p[i];
        double* o = out + 8 * i;
        o[0] = q.x; o[1] = q.y; o[2] = q.z; o[3] = q.vx; o[4] = q.vy; o[5] = q.vz;
        o[6] = q.ttd; o[7] = q.empty ? 1.0 : 0.0;
    }
    return (int)p.p.size();
}

int orc_advance_init(orc_sim* s)
{
    return guard([&]() { s->advance_init(); return 0; });
}

int orc_advance(orc_sim* s, int nsteps)
{
    return guard([&]() {
        for (int i = 0; i < nsteps; ++i) s->advance();
        return 0;
    });
}

double orc_time_advance(orc_sim* s, int nsteps)
{
    auto t0 = std::chrono::steady_clock::now();
    if (orc_advance(s, nsteps) != 0) return -1.0;
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

int orc_field_shape(orc_sim* s, int which, int* nx, int* nz)
{
    if (which == ORC_MASK || which == ORC_VOLTAGE) {
        *nx = s->c.x_sampl;
        *nz = s->c.z_sampl;
        return 0;
    }
    const Field& f = which == ORC_U ? s->u : which == ORC_URF ? s->uRF : which == ORC_RHO ? s->rho
                                                              : s->sp[which - ORC_SPECIES_RHO]->rho;
    *nx = f.jmax;
    *nz = f.lmax;
    return 0;
}

int orc_get_field(orc_sim* s, int which, double* out)
{
    if (which == ORC_MASK) {
        for (size_t k = 0; k < s->mask.size(); ++k) out[k] = (double)s->mask[k];
        return (int)s->mask.size();
    }
    if (which == ORC_VOLTAGE) {
        std::copy(s->voltage.begin(), s->voltage.end(), out);
        return (int)s->voltage.size();
    }
    const Field& f = which == ORC_U ? s->u : which == ORC_URF ? s->uRF : which == ORC_RHO ? s->rho
                                                              : s->sp[which - ORC_SPECIES_RHO]->rho;
    std::copy(f.d.begin(), f.d.end(), out);
    return (int)f.d.size();
}

int orc_solve(orc_sim* s, const double* rho, double* u)
{
    return guard([&]() {
        std::copy(rho, rho + s->rho.d.size(), s->rho.d.begin());
        s->boundary_solve(false);
        std::copy(s->u.d.begin(), s->u.d.end(), u);
        s->rho.reset();
        return 0;
    });
}

int orc_grad(orc_sim* s, int which, int n, const double* x, const double* z, double* gx, double* gz)
{
    const Field& f = which == 0 ? s->u : s->uRF;
    for (int i = 0; i < n; ++i) f.grad(x[i], z[i], gx[i], gz[i]);
    return 0;
}

int orc_species_info(orc_sim* s, int sp, double* out)
{
    const Species& p = *s->sp[sp];
    double v[11] = {p.mass, p.charge, p.dt, p.density, p.temperature, p.lifetime, p.E_max, p.v_max,
                    (double)p.p.size(), (double)p.n_particles(), (double)p.niter};
    std::memcpy(out, v, sizeof v);
    return 0;
}

int orc_rates(orc_sim* s, int sp, double* out)
{
    const Species& p = *s->sp[sp];
    std::copy(p.rates.begin(), p.rates.end(), out);
    return (int)p.rates.size();
}

int orc_sigma_v(orc_sim* s, int sp, int tgt, int n, const double* v, double* out)
{
    const std::vector<Interaction*>& l = s->sp[sp]->by_species[tgt];
    for (size_t k = 0; k < l.size(); ++k)
        for (int i = 0; i < n; ++i) out[k * n + i] = l[k]->sigma_v(v[i]);
    return (int)l.size();
}

int orc_rng(orc_sim* s, int kind, int n, double arg, double* out)
{
    Rng& r = s->rnd;
    for (int i = 0; i < n; ++i) {
        switch (kind) {
        case 0: out[i] = r.uni(); break;
        case 1: out[i] = r.rnor(); break;
        case 2: out[i] = r.rexp(); break;
        case 3: out[i] = (double)r.iuni(); break;
        case 4: r.rot(1.0, out[3 * i], out[3 * i + 1], out[3 * i + 2]); break;
        case 5: {
            double x = 1.0, y = 0.0, z = 0.0;
            r.deflect(arg, x, y, z);
            out[3 * i] = x;
            out[3 * i + 1] = y;
            out[3 * i + 2] = z;
        } break;
        default: return -1;
        }
    }
    return n;
}

int64_t orc_collisions(orc_sim* s, int sp) { return s->sp[sp]->ncoll; }
int64_t orc_real_collisions(orc_sim* s, int sp) { return s->sp[sp]->nreal; }

void orc_u_smooth(int nx, int nz, const double* in, double* out)
{
    const std::vector<double> t(in, in + (size_t)nx * nz);
    smooth_flat(nx, nz, t.data(), out);
}

int64_t orc_deposit_fixed(int nx, int nz, int64_t n, const uint32_t* xf, const uint32_t* zf, const uint8_t* alive,
                          int64_t* acc)
{
    const int64_t one = (int64_t)1 << 20;
    int64_t cnt = 0;
    for (int64_t k = 0; k < n; ++k) {
        if (alive && !alive[k]) continue;
        int i = (int)(xf[k] >> 20), j = (int)(zf[k] >> 20);
        if (i > nx - 2) i = nx - 2;  // a particle on the last node line
        if (j > nz - 2) j = nz - 2;
        const int64_t U = (int64_t)xf[k] - ((int64_t)i << 20);
        const int64_t V = (int64_t)zf[k] - ((int64_t)j << 20);
        const size_t b = (size_t)i * nz + j;
        acc[b] += (one - U) * (one - V);
        acc[b + nz] += U * (one - V);
        acc[b + 1] += (one - U) * V;
        acc[b + nz + 1] += U * V;
        ++cnt;
    }
    return cnt;
}

}  // extern "C"
