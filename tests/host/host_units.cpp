// Host-side units of the GPU library checked without a GPU: the division
// magic numbers of the multigrid levels, the level hierarchy, the tile choice
// of multi-block solves and the dense inverse of a coarsest level.
// Built and run by tests/test_host_units.py; exits non-zero on a failure.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "device.hpp"
#include "multigrid_host.hpp"

using namespace mag;

static int failures = 0;
#define CHECK(c)                                                           \
    do {                                                                   \
        if (!(c)) {                                                        \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);     \
            ++failures;                                                    \
        }                                                                  \
    } while (0)

// the device's division by a DivMagic, restated on the host
static unsigned magic_div(const DivMagic& m, unsigned n)
{
    if (m.d == 1) return n;
    const unsigned t = (unsigned)(((unsigned long long)m.m * n) >> 32);
    return (t + ((n - t) >> 1)) >> (m.l - 1);
}

int main()
{
    // exact for every divisor up to the largest grid dimension and any 32-bit numerator
    std::mt19937 g(7);
    for (unsigned d = 1; d <= 5000; ++d) {
        const DivMagic m = div_magic(d);
        for (int k = 0; k < 200; ++k) {
            const unsigned n = k < 100 ? (unsigned)k * 131u : (unsigned)g();
            if (magic_div(m, n) != n / d) {
                CHECK(magic_div(m, n) == n / d);
                break;
            }
        }
    }
    // the large r-z grid (cells with dz = 2 dx: r couplings 4x the z ones):
    // halved in r only once, then in both, down to at most kDenseCoarseGridMax nodes
    std::vector<int> lnx, lnz, lm;
    multigrid_levels(1025, 2049, 4.0, kMaxLevels, lnx, lnz, lm, kDenseCoarseGridMax);
    const int ex[7][2] = {{1025, 2049}, {513, 2049}, {257, 1025}, {129, 513}, {65, 257}, {33, 129}, {17, 65}};
    CHECK(lnx.size() == 7);
    for (size_t l = 0; l < lnx.size() && l < 7; ++l) CHECK(lnx[l] == ex[l][0] && lnz[l] == ex[l][1]);
    CHECK(lm[1] == kCoarsenX && lm[2] == kCoarsenFull);
    // one-block grids stop at kDenseCoarseMax
    multigrid_levels(65, 129, 1.0, kMaxLevels, lnx, lnz, lm);
    CHECK((long long)lnx.back() * lnz.back() <= kDenseCoarseMax);
    for (size_t l = 1; l < lm.size(); ++l) CHECK(lm[l] == kCoarsenFull);
    // tiles of the fine level: one per block, region within the shared-memory budget
    int ti = 0, tj = 0;
    const long long budget = (200LL << 10) / kTileNodeBytes;
    choose_tile(1025, 2049, 152, kTileHalo, budget, ti, tj);
    CHECK((long long)(ti + 2 * kTileHalo) * (tj + 2 * kTileHalo) <= budget);
    CHECK((long long)((1025 + ti - 1) / ti) * ((2049 + tj - 1) / tj) <= 152);
    // dense inverse of a 9-point operator (a diagonally dominant Galerkin-like stencil)
    const int nx = 9, nz = 11, n = nx * nz;
    std::vector<double> A(9 * (size_t)n, 0.0);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j) {
            const int k = i * nz + j;
            for (int di = -1; di <= 1; ++di)
                for (int dj = -1; dj <= 1; ++dj)
                    A[(size_t)plane(di, dj) * n + k] = (di == 0 && dj == 0) ? 8.5 + 0.01 * i : -1.0 + 0.02 * j;
        }
    std::vector<double> inv;
    CHECK(dense_inverse64(nx, nz, A, inv));
    double err = 0.0;
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) {
            const int i = r / nz, j = r % nz;
            double acc = 0.0;
            for (int di = -1; di <= 1; ++di)
                for (int dj = -1; dj <= 1; ++dj) {
                    const int ii = i + di, jj = j + dj;
                    if (ii < 0 || ii >= nx || jj < 0 || jj >= nz) continue;
                    acc += A[(size_t)plane(di, dj) * n + r] * inv[(size_t)c * n + ii * nz + jj];
                }
            err = std::fmax(err, std::fabs(acc - (r == c ? 1.0 : 0.0)));
        }
    CHECK(err < 1e-12);
    std::printf("%s (%d failures)\n", failures ? "host units FAILED" : "host units ok", failures);
    return failures ? 1 : 0;
}
