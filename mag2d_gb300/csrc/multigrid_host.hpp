// Host set-up of the multigrid hierarchy of the Poisson solve: level sizes
// and Galerkin coarse operators (used by the simulation and by the
// allocation-free solve entry point).
#pragma once
#include <cstdint>
#include <vector>

namespace mag {

// 9-point operator planes: plane (di+1)*3 + (dj+1) holds the coefficient of node (i+di, j+dj)
inline int plane(int di, int dj) { return (di + 1) * 3 + (dj + 1); }

// Fine-level operator of the correction equation: the reference's rows
// (src/fields.cpp:149-238) on free nodes with the columns of Dirichlet nodes
// removed; Dirichlet rows are identity.  coord: 0 Cartesian, 1 cylindrical.
void fine_operator(int coord, int nx, int nz, double dx, double dz, const std::vector<int8_t>& mask,
                   std::vector<double>& A);

// How a level is coarsened to the next: both directions, or only x (r), or
// only z.  A level whose x couplings are at least kSemiCoarsenRatio times its
// z couplings (the cylindrical operator on cells with dz = 2 dx has 4) is
// halved in x only, which makes the next level's couplings alike; point
// Gauss-Seidel with full coarsening converges slowly on such levels.
constexpr int kCoarsenFull = 0, kCoarsenX = 1, kCoarsenZ = 2;
constexpr double kSemiCoarsenRatio = 2.5;

// Galerkin coarse operator Ac = P^T Af P with P bilinear in the coarsened
// directions (mode: kCoarsen*; rows of fixed fine nodes are zero).  Coarse
// rows left without a diagonal become identity.
void galerkin(int nxf, int nzf, const std::vector<double>& Af, const std::vector<char>& fixed_f, int mode, int& nxc,
              int& nzc, std::vector<double>& Ac);

// Coarsest levels up to this many nodes are solved exactly with a dense inverse
// (one block applies it); multi-block solves stop coarsening at this larger
// size and apply the inverse with every block, one warp per row.
constexpr long long kDenseCoarseMax = 200;
constexpr long long kDenseCoarseGridMax = 1280;

// Level sizes: halve while the sizes are odd and >= 5 (at most max_levels
// levels), and stop at the first level of at most coarse_max nodes.
// couple_ratio = x couplings / z couplings of the fine operator ((dz/dx)^2 for
// the cylindrical one, 1 for the reference's Cartesian one); lmode[l] says how
// level l - 1 was coarsened to level l (lmode[0] unused).
void multigrid_levels(int nx, int nz, double couple_ratio, int max_levels, std::vector<int>& lnx, std::vector<int>& lnz,
                      std::vector<int>& lmode, long long coarse_max = kDenseCoarseMax);

// Per-row coefficients (w, e, c, 1/c) of the fine 5-point stencil, FP64,
// 4 * nx values, and the common s/n coefficient k2 (src/fields.cpp:149-238);
// rows of the axis (i = 0, cylindrical) have w = 0.  Cartesian: (1, 1, -4),
// k2 = 1.
void fine_stencil_table(int coord, int nx, double dx, double dz, std::vector<double>& st, double& k2);

// Dense inverse of a level's 9-point operator (n = nx*nz nodes), FP64
// Gauss-Jordan with partial pivoting, stored in FP32 column-major
// (inv[col * n + row]).  Returns false when the operator is singular.
bool dense_inverse(int nx, int nz, const std::vector<double>& A9, std::vector<float>& inv);
// the same inverse kept in FP64
bool dense_inverse64(int nx, int nz, const std::vector<double>& A9, std::vector<double>& inv);

// Tile of a level of a multi-block solve: the interior size ti x tj that
// minimises (tiles per block, rounded up) x (region nodes), the region being
// the tile with halo rings on each side, within budget_nodes region nodes.
void choose_tile(int nx, int nz, int nblocks, int halo, long long budget_nodes, int& ti, int& tj);

}  // namespace mag
