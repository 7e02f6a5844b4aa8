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

// Galerkin coarse operator Ac = P^T Af P with bilinear P (rows of fixed fine
// nodes are zero).  Coarse rows left without a diagonal become identity.
void galerkin(int nxf, int nzf, const std::vector<double>& Af, const std::vector<char>& fixed_f, int& nxc,
              int& nzc, std::vector<double>& Ac);

// Level sizes: halve while both sizes are odd and >= 5 (at most max_levels levels).
void multigrid_levels(int nx, int nz, int max_levels, std::vector<int>& lnx, std::vector<int>& lnz);

}  // namespace mag
