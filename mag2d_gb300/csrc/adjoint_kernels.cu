// Adjoint pieces of the self-consistent step that are not particle pushes:
// face adjoints to node adjoints (transpose of the face difference of
// Field2D::grad), the transpose Poisson solve's right-hand side and read-out,
// the charge deposit's adjoint, and the loss with its initial adjoint.
#include "device.hpp"
#include "kernels.hpp"

namespace mag {

namespace {

__device__ __forceinline__ bool fixed_node(int8_t m) { return m == 0 || m == 1; }

// g[i][j] += transpose of Exf[r][j] = -(u[ic][j] - u[ic-1][j]) / dx with
// ic = clamp(r, 1, nx-1) and Ezf[i][c] = -(u[i][jc] - u[i][jc-1]) / dz
__global__ void k_adj_faces(int nx, int nz, double idx, double idz, const float* __restrict__ lExf,
                            const float* __restrict__ lEzf, double* __restrict__ g)
{
    const long long n = (long long)nx * nz;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q / nz), j = (int)(q % nz);
        double acc = 0.0;
        // x faces r with ic(r) == i contribute -idx, with ic(r) == i + 1 contribute +idx
        auto fx = [&](int r) { return (double)lExf[(size_t)r * nz + j]; };
        if (i >= 1 && i <= nx - 1) acc -= fx(i) * idx;
        if (i == 1) acc -= fx(0) * idx;
        if (i == nx - 1) acc -= fx(nx) * idx;
        if (i + 1 >= 1 && i + 1 <= nx - 1) acc += fx(i + 1) * idx;
        if (i == 0) acc += fx(0) * idx;
        if (i + 1 == nx - 1) acc += fx(nx) * idx;
        auto fz = [&](int c) { return (double)lEzf[(size_t)i * (nz + 1) + c]; };
        if (j >= 1 && j <= nz - 1) acc -= fz(j) * idz;
        if (j == 1) acc -= fz(0) * idz;
        if (j == nz - 1) acc -= fz(nz) * idz;
        if (j + 1 >= 1 && j + 1 <= nz - 1) acc += fz(j + 1) * idz;
        if (j == 0) acc += fz(0) * idz;
        if (j + 1 == nz - 1) acc += fz(nz) * idz;
        g[q] += acc;
    }
}

// right-hand side of A_ff x = W^-1 g_f, given to the solver as rho with its
// own row scaling: rho = g / (w_i scale_i) on free nodes
__global__ void k_adj_rhs(int nx, int nz, const int8_t* __restrict__ mask, const double* __restrict__ g,
                          const double* __restrict__ w_scale, double* __restrict__ rho)
{
    const long long n = (long long)nx * nz;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q / nz);
        rho[q] = fixed_node(mask[q]) ? 0.0 : g[q] / w_scale[i];
    }
}

// after the solve: y = W x on free nodes; d loss / d rho = scale_i y_i (free)
__global__ void k_adj_post(int nx, int nz, const int8_t* __restrict__ mask, const double* __restrict__ x,
                           const double* __restrict__ w, const double* __restrict__ scale, double* __restrict__ y,
                           double* __restrict__ lrho)
{
    const long long n = (long long)nx * nz;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q / nz);
        const bool f = !fixed_node(mask[q]);
        y[q] = f ? w[i] * x[q] : 0.0;
        lrho[q] = f ? scale[i] * w[i] * x[q] : 0.0;
    }
}

// d loss / d u_d of every Dirichlet node d = g_d - sum over free neighbours f
// of A[f][d] y_f, projected on the voltage parameters: grad[p] += basis[p][d] * that
__global__ void k_adj_dirichlet(int nx, int nz, const int8_t* __restrict__ mask, const double* __restrict__ g,
                                const double* __restrict__ y, const double* __restrict__ st64, double k2,
                                const double* __restrict__ basis, int nparam, double* __restrict__ grad)
{
    extern __shared__ double sacc[];
    for (int p = threadIdx.x; p < nparam; p += blockDim.x) sacc[p] = 0.0;
    __syncthreads();
    const long long n = (long long)nx * nz;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        if (!fixed_node(mask[q])) continue;
        const int i = (int)(q / nz), j = (int)(q % nz);
        double v = g[q];
        // the free neighbour f's row holds the coefficient of d: west of f is d when d = f - nz, etc.
        if (i + 1 < nx && !fixed_node(mask[q + nz])) v -= st64[4 * (i + 1)] * y[q + nz];      // f east of d: A[f][d] = w(f)
        if (i - 1 >= 0 && !fixed_node(mask[q - nz])) v -= st64[4 * (i - 1) + 1] * y[q - nz];  // f west of d: e(f)
        if (j + 1 < nz && !fixed_node(mask[q + 1])) v -= k2 * y[q + 1];
        if (j - 1 >= 0 && !fixed_node(mask[q - 1])) v -= k2 * y[q - 1];
        if (v == 0.0) continue;
        for (int p = 0; p < nparam; ++p) {
            const double b = basis[(size_t)p * n + q];
            if (b != 0.0) atomicAdd(&sacc[p], b * v);
        }
    }
    __syncthreads();
    for (int p = threadIdx.x; p < nparam; p += blockDim.x)
        if (sacc[p] != 0.0) atomicAdd(&grad[p], sacc[p]);
}

// lr, lz += charge * d(sum_nodes lrho w_node(x)) / dx for every live particle
__global__ void k_adj_deposit(const uint32_t* __restrict__ x, const uint32_t* __restrict__ z, int64_t n, int nx,
                              int nz, const double* __restrict__ lrho, double charge, float* lr, float* lz)
{
    const double inv = 1.0 / (double)(1u << kFracBits);
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t xf = x[k];
        if (xf == kDead) continue;
        const uint32_t zf = z[k];
        const int ic = min((int)(xf >> kFracBits), nx - 2);
        const int jc = min((int)(zf >> kFracBits), nz - 2);
        const double U = (double)(xf - ((uint32_t)ic << kFracBits)) * inv;
        const double V = (double)(zf - ((uint32_t)jc << kFracBits)) * inv;
        const size_t b = (size_t)ic * nz + jc;
        const double l00 = lrho[b], l10 = lrho[b + nz], l01 = lrho[b + 1], l11 = lrho[b + nz + 1];
        const double dU = -(1 - V) * l00 + (1 - V) * l10 - V * l01 + V * l11;
        const double dV = -(1 - U) * l00 - U * l10 + (1 - U) * l01 + U * l11;
        lr[k] += (float)(charge * dU);
        lz[k] += (float)(charge * dV);
    }
}

// loss pieces: sum over live particles of m vz^2 / 2 (eV) and the live count
__global__ void k_adj_loss(const uint32_t* __restrict__ x, const float* __restrict__ vz, int64_t n, double half_m_eV,
                           double* __restrict__ out_e, unsigned long long* __restrict__ out_n)
{
    double e = 0.0;
    unsigned long long c = 0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        if (x[k] == kDead) continue;
        e += half_m_eV * (double)vz[k] * (double)vz[k];
        ++c;
    }
    for (int o = 16; o > 0; o >>= 1) {
        e += __shfl_xor_sync(0xffffffffu, e, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (e != 0.0) atomicAdd(out_e, e);
        if (c) atomicAdd(out_n, c);
    }
}

// initial adjoint of the loss w_e * mean(m vz^2 / 2) / e: lvz = w_e m vz / (e N_live)
__global__ void k_adj_seed(const uint32_t* __restrict__ x, const float* __restrict__ vz, int64_t n, double coef,
                           float* lr, float* lz, float* lvx, float* lvy, float* lvz)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        lr[k] = lz[k] = lvx[k] = lvy[k] = 0.f;
        lvz[k] = x[k] == kDead ? 0.f : (float)(coef * (double)vz[k]);
    }
}

unsigned grid_for(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152 * 8); }

}  // namespace

int launch_adj_faces(int nx, int nz, double dx, double dz, const float* lExf, const float* lEzf, double* g,
                     cudaStream_t s)
{
    k_adj_faces<<<grid_for((long long)nx * nz), 256, 0, s>>>(nx, nz, 1.0 / dx, 1.0 / dz, lExf, lEzf, g);
    return 1;
}

int launch_adj_rhs(int nx, int nz, const int8_t* mask, const double* g, const double* w_scale, double* rho,
                   cudaStream_t s)
{
    k_adj_rhs<<<grid_for((long long)nx * nz), 256, 0, s>>>(nx, nz, mask, g, w_scale, rho);
    return 1;
}

int launch_adj_post(int nx, int nz, const int8_t* mask, const double* x, const double* w, const double* scale,
                    double* y, double* lrho, cudaStream_t s)
{
    k_adj_post<<<grid_for((long long)nx * nz), 256, 0, s>>>(nx, nz, mask, x, w, scale, y, lrho);
    return 1;
}

int launch_adj_dirichlet(int nx, int nz, const int8_t* mask, const double* g, const double* y, const double* st64,
                         double k2, const double* basis, int nparam, double* grad, cudaStream_t s)
{
    if (nparam <= 0) return 0;
    k_adj_dirichlet<<<grid_for((long long)nx * nz), 256, (size_t)nparam * sizeof(double), s>>>(
        nx, nz, mask, g, y, st64, k2, basis, nparam, grad);
    return 1;
}

int launch_adj_deposit(const uint32_t* x, const uint32_t* z, int64_t n, int nx, int nz, const double* lrho,
                       double charge, float* lr, float* lz, cudaStream_t s)
{
    if (n == 0) return 0;
    k_adj_deposit<<<grid_for(n), 256, 0, s>>>(x, z, n, nx, nz, lrho, charge, lr, lz);
    return 1;
}

int launch_adj_loss(const uint32_t* x, const float* vz, int64_t n, double half_m_eV, double* out_e,
                    unsigned long long* out_n, cudaStream_t s)
{
    if (n == 0) return 0;
    k_adj_loss<<<grid_for(n), 256, 0, s>>>(x, vz, n, half_m_eV, out_e, out_n);
    return 1;
}

int launch_adj_seed(const uint32_t* x, const float* vz, int64_t n, double coef, float* lr, float* lz, float* lvx,
                    float* lvy, float* lvz, cudaStream_t s)
{
    if (n == 0) return 0;
    k_adj_seed<<<grid_for(n), 256, 0, s>>>(x, vz, n, coef, lr, lz, lvx, lvy, lvz);
    return 1;
}

}  // namespace mag
