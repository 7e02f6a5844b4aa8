// C-callable harness around the reference's Field3D (src/Field3D.hpp:40-163),
// test infrastructure for the 3D path.  The header is compiled unchanged; its
// private members are opened so that the harness can set the domain extent
// (xmax, ymax, zmax) that grad_component clamps against and that no
// constructor of the reference sets.  Nothing in the product links this file.
#define private public
#include "Field3D.hpp"
#undef private

extern "C" {

// Field3D::accumulate of n charges at (x, y, z) into a zeroed grid (rho_out,
// nx ny nz, z fastest); then, on the grid u_in, Field3D::interpolate and
// Field3D::grad at the same points.
int ref3d_field(int nx, int ny, int nz, double dx, double dy, double dz, int n, const double* x, const double* y,
                const double* z, const double* charge, double* rho_out, const double* u_in, double* interp_out,
                double* grad_out)
{
    Field3D f(nx, ny, nz, dx, dy, dz);
    f.xmax = (nx - 1) * dx;
    f.ymax = (ny - 1) * dy;
    f.zmax = (nz - 1) * dz;
    const long nn = (long)nx * ny * nz;
    for (long q = 0; q < nn; ++q) f.data[0][0][q] = 0.0;
    for (int p = 0; p < n; ++p) f.accumulate(charge[p], x[p], y[p], z[p]);
    for (long q = 0; q < nn; ++q) rho_out[q] = f.data[0][0][q];
    for (long q = 0; q < nn; ++q) f.data[0][0][q] = u_in[q];
    for (int p = 0; p < n; ++p) {
        interp_out[p] = f.interpolate(x[p], y[p], z[p]);
        f.grad(x[p], y[p], z[p], grad_out[3 * p], grad_out[3 * p + 1], grad_out[3 * p + 2]);
    }
    return 0;
}
}
