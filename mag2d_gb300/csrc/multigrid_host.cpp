// Host set-up of the multigrid hierarchy (see multigrid_host.hpp).
#include "multigrid_host.hpp"

#include <cmath>
#include <utility>

namespace mag {

namespace {
bool fixed_node(int8_t m) { return m == 0 || m == 1; }  // FIXED, FIXED_RF
}  // namespace


void fine_operator(int coord, int nx, int nz, double dx, double dz, const std::vector<int8_t>& mask,
                   std::vector<double>& A)
{
    const size_t n = (size_t)nx * nz;
    A.assign(9 * n, 0.0);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j) {
            const size_t k = (size_t)i * nz + j;
            if (fixed_node(mask[k])) {
                A[4 * n + k] = 1.0;
                continue;
            }
            double w, e, s, nn, c;
            if (coord == 1) {
                const double k2 = 1.0 / (dz * dz);
                if (i == 0) {
                    const double k3 = 1.0 / (dx * dx * 0.25);
                    w = 0.0; e = k3; s = k2; nn = k2; c = -2.0 * k2 - k3;
                } else {
                    const double k1 = (i - 0.5) / (dx * dx * i), k3 = (i + 0.5) / (dx * dx * i);
                    w = k1; e = k3; s = k2; nn = k2; c = -2.0 * k2 - k1 - k3;
                }
            } else {
                w = e = s = nn = 1.0;
                c = -4.0;
            }
            A[4 * n + k] = c;
            if (i > 0 && !fixed_node(mask[k - nz])) A[(size_t)plane(-1, 0) * n + k] = w;
            if (i < nx - 1 && !fixed_node(mask[k + nz])) A[(size_t)plane(1, 0) * n + k] = e;
            if (j > 0 && !fixed_node(mask[k - 1])) A[(size_t)plane(0, -1) * n + k] = s;
            if (j < nz - 1 && !fixed_node(mask[k + 1])) A[(size_t)plane(0, 1) * n + k] = nn;
        }
}

void galerkin(int nxf, int nzf, const std::vector<double>& Af, const std::vector<char>& fixed_f, int mode, int& nxc,
              int& nzc, std::vector<double>& Ac)
{
    // coarse node (J0, J1) sits on fine node (sx J0, sz J1); the interpolation
    // reaches rx (rz) fine nodes either side in a coarsened direction, none in
    // a kept one
    const int sx = mode == kCoarsenZ ? 1 : 2, sz = mode == kCoarsenX ? 1 : 2;
    const int rx = sx - 1, rz = sz - 1;
    nxc = sx == 2 ? (nxf - 1) / 2 + 1 : nxf;
    nzc = sz == 2 ? (nzf - 1) / 2 + 1 : nzf;
    const size_t nf = (size_t)nxf * nzf, nc = (size_t)nxc * nzc;
    Ac.assign(9 * nc, 0.0);
    auto pw = [](int a) { return a == 0 ? 1.0 : 0.5; };
    for (int J0 = 0; J0 < nxc; ++J0)
        for (int J1 = 0; J1 < nzc; ++J1) {
            double v[3][3] = {{0}};  // P e_J on the fine nodes around (sx J0, sz J1)
            for (int a = -rx; a <= rx; ++a)
                for (int b = -rz; b <= rz; ++b) {
                    const int i = sx * J0 + a, j = sz * J1 + b;
                    if (i < 0 || i >= nxf || j < 0 || j >= nzf) continue;
                    if (fixed_f[(size_t)i * nzf + j]) continue;
                    v[a + 1][b + 1] = pw(a) * pw(b);
                }
            double w[5][5] = {{0}};  // A P e_J on the fine nodes within reach + 1
            for (int a = -rx - 1; a <= rx + 1; ++a)
                for (int b = -rz - 1; b <= rz + 1; ++b) {
                    const int i = sx * J0 + a, j = sz * J1 + b;
                    if (i < 0 || i >= nxf || j < 0 || j >= nzf) continue;
                    const size_t f = (size_t)i * nzf + j;
                    double acc = 0.0;
                    for (int di = -1; di <= 1; ++di)
                        for (int dj = -1; dj <= 1; ++dj) {
                            const int ga = a + di, gb = b + dj;
                            if (ga < -1 || ga > 1 || gb < -1 || gb > 1) continue;
                            const double vv = v[ga + 1][gb + 1];
                            if (vv == 0.0) continue;
                            acc += Af[(size_t)plane(di, dj) * nf + f] * vv;
                        }
                    w[a + 2][b + 2] = acc;
                }
            for (int I0 = J0 - 1; I0 <= J0 + 1; ++I0)
                for (int I1 = J1 - 1; I1 <= J1 + 1; ++I1) {
                    if (I0 < 0 || I0 >= nxc || I1 < 0 || I1 >= nzc) continue;
                    double acc = 0.0;
                    for (int a = -rx; a <= rx; ++a)
                        for (int b = -rz; b <= rz; ++b) {
                            const int i = sx * I0 + a, j = sz * I1 + b;
                            if (i < 0 || i >= nxf || j < 0 || j >= nzf) continue;
                            if (fixed_f[(size_t)i * nzf + j]) continue;
                            const int wa = i - sx * J0, wb = j - sz * J1;
                            if (wa < -rx - 1 || wa > rx + 1 || wb < -rz - 1 || wb > rz + 1) continue;
                            acc += pw(a) * pw(b) * w[wa + 2][wb + 2];
                        }
                    Ac[(size_t)plane(J0 - I0, J1 - I1) * nc + (size_t)I0 * nzc + I1] = acc;
                }
        }
    for (size_t k = 0; k < nc; ++k)
        if (Ac[4 * nc + k] == 0.0) {
            for (int q = 0; q < 9; ++q) Ac[q * nc + k] = 0.0;
            Ac[4 * nc + k] = 1.0;
        }
}

void multigrid_levels(int nx, int nz, double couple_ratio, int max_levels, std::vector<int>& lnx, std::vector<int>& lnz,
                      std::vector<int>& lmode, long long coarse_max)
{
    lnx.assign(1, nx);
    lnz.assign(1, nz);
    lmode.assign(1, kCoarsenFull);
    double ratio = couple_ratio;  // x couplings / z couplings of the current level
    while ((int)lnx.size() < max_levels && (long long)lnx.back() * lnz.back() > coarse_max) {
        const int x = lnx.back(), z = lnz.back();
        const bool cx = (x - 1) % 2 == 0 && x >= 5, cz = (z - 1) % 2 == 0 && z >= 5;
        int mode;
        if (ratio >= kSemiCoarsenRatio && cx) mode = kCoarsenX;       // strong x couplings: halve x only
        else if (ratio <= 1.0 / kSemiCoarsenRatio && cz) mode = kCoarsenZ;
        else if (cx && cz) mode = kCoarsenFull;
        else break;
        lnx.push_back(mode == kCoarsenZ ? x : (x - 1) / 2 + 1);
        lnz.push_back(mode == kCoarsenX ? z : (z - 1) / 2 + 1);
        lmode.push_back(mode);
        if (mode == kCoarsenX) ratio /= 4.0;  // the x spacing doubles
        if (mode == kCoarsenZ) ratio *= 4.0;
    }
}

void fine_stencil_table(int coord, int nx, double dx, double dz, std::vector<double>& st, double& k2)
{
    st.assign(4 * (size_t)nx, 0.0);
    k2 = coord == 1 ? 1.0 / (dz * dz) : 1.0;
    for (int i = 0; i < nx; ++i) {
        double w, e, c;
        if (coord != 1) {
            w = 1.0;
            e = 1.0;
            c = -4.0;
        } else if (i == 0) {
            const double k3 = 1.0 / (dx * dx * 0.25);
            w = 0.0;
            e = k3;
            c = -2.0 * k2 - k3;
        } else {
            const double k1 = (i - 0.5) / (dx * dx * i), k3 = (i + 0.5) / (dx * dx * i);
            w = k1;
            e = k3;
            c = -2.0 * k2 - k1 - k3;
        }
        st[4 * i] = w;
        st[4 * i + 1] = e;
        st[4 * i + 2] = c;
        st[4 * i + 3] = 1.0 / c;
    }
}

bool dense_inverse(int nx, int nz, const std::vector<double>& A9, std::vector<float>& inv)
{
    std::vector<double> inv64;
    if (!dense_inverse64(nx, nz, A9, inv64)) return false;
    inv.assign(inv64.begin(), inv64.end());
    return true;
}

bool dense_inverse64(int nx, int nz, const std::vector<double>& A9, std::vector<double>& inv)
{
    const int n = nx * nz;
    std::vector<double> M((size_t)n * 2 * n, 0.0);  // [A | I], row-major, row length 2n
    const size_t w = 2 * (size_t)n;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j) {
            const int r = i * nz + j;
            for (int di = -1; di <= 1; ++di)
                for (int dj = -1; dj <= 1; ++dj) {
                    const int ii = i + di, jj = j + dj;
                    if (ii < 0 || ii >= nx || jj < 0 || jj >= nz) continue;
                    M[r * w + (size_t)(ii * nz + jj)] = A9[(size_t)plane(di, dj) * n + r];
                }
            M[r * w + n + r] = 1.0;
        }
    for (int c = 0; c < n; ++c) {
        int piv = c;
        double best = std::abs(M[c * w + c]);
        for (int r = c + 1; r < n; ++r)
            if (std::abs(M[r * w + c]) > best) {
                best = std::abs(M[r * w + c]);
                piv = r;
            }
        if (!(best > 0.0)) return false;
        if (piv != c)
            for (size_t q = 0; q < w; ++q) std::swap(M[c * w + q], M[piv * w + q]);
        const double d = 1.0 / M[c * w + c];
        for (size_t q = 0; q < w; ++q) M[c * w + q] *= d;
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = M[r * w + c];
            if (f == 0.0) continue;
            for (size_t q = (size_t)c; q < w; ++q) M[r * w + q] -= f * M[c * w + q];
        }
    }
    inv.assign((size_t)n * n, 0.0);
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) inv[(size_t)c * n + r] = M[r * w + n + c];
    return true;
}

void choose_tile(int nx, int nz, int nblocks, int halo, long long budget_nodes, int& ti, int& tj)
{
    long long best = -1, best_reg = 0;
    ti = tj = 1;
    for (int a = 1; a <= std::min(nx, 512); ++a)
        for (int b = 1; b <= std::min(nz, 1024); ++b) {
            const long long reg = (long long)(a + 2 * halo) * (b + 2 * halo);
            if (reg > budget_nodes) break;
            const long long tiles = (long long)((nx + a - 1) / a) * ((nz + b - 1) / b);
            const long long cost = (tiles + nblocks - 1) / nblocks * reg;
            if (best < 0 || cost < best || (cost == best && reg < best_reg)) {
                best = cost;
                best_reg = reg;
                ti = a;
                tj = b;
            }
        }
}

}  // namespace mag
