// Poisson solve without any device allocation: the same persistent multigrid
// kernel as Fields::boundary_solve on the simulation path (poisson.cu), with
// all of its working memory carved out of one file-scope device array.
//
// Who needs it: code that must not call cudaMalloc — a host application that
// runs under a fixed, pre-reserved device-memory budget or a caching
// allocator it does not own, or that calls the solver from a context where a
// device allocation would synchronise the whole device (allocation implies an
// implicit device-wide synchronisation in the CUDA runtime).  Such a caller
// owns rho and u in device memory and passes them in; everything else lives
// in the static array below, which every GPU that loads the library keeps for
// the life of the process.
//
// Limits and rules of use (also stated in include/mag2d_gpu.h):
//   * at most kNoAllocMaxNodes grid nodes (257 x 257), and the scratch layout
//     of the grid must fit kNoAllocScratchBytes; larger grids are rejected;
//   * the first call on a device looks up the device address of the array
//     (cudaGetSymbolAddress) with that device current and keeps it for the
//     process.  The kept address does not survive cudaDeviceReset of that
//     device;
//   * with info == NULL the call returns once the work is queued and reports
//     nothing about the solve (convergence or a barrier timeout stays in the
//     array and the next call clears it); voltage_host is copied
//     asynchronously, so page-locked voltage_host memory must stay valid until
//     the stream has reached the solve;
//   * all calls share the one array and it keeps the contents of the last call;
//     calls that overlap on the GPU (different streams, or different host
//     threads on the same device) race on it.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "device.hpp"
#include "kernels.hpp"
#include "mag2d_gpu.h"
#include "multigrid_host.hpp"

namespace mag {
void set_last_error(const std::string& msg);  // api.cpp
}

namespace {

constexpr long long kNoAllocMaxNodes = 257LL * 257LL;
constexpr size_t kNoAllocScratchBytes = 4u << 20;  // 4 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Errors go to the same per-thread message as the rest of the C ABI.
struct ErrorSink {
    std::string msg;
    void clear() { msg.clear(); }
    ErrorSink& operator=(const std::string& m)
    {
        msg = m;
        mag::set_last_error(m);
        return *this;
    }
    ErrorSink& operator=(const char* m) { return *this = std::string(m); }
};
thread_local ErrorSink g_noalloc_err;

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Device address of the scratch array on the current device (looked up once).
int scratch_address(unsigned char** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        g_noalloc_err = "mag_poisson_solve_noalloc: no current CUDA device";
        return MAG_ECUDA;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            g_noalloc_err = std::string("mag_poisson_solve_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return MAG_ECUDA;
        }
        g_noalloc_ptr[dev] = p;
    }
    *out = (unsigned char*)g_noalloc_ptr[dev];
    return MAG_OK;
}

}  // namespace

extern "C" int mag_poisson_solve_noalloc(int coord, int nx, int nz, double dx, double dz, double macroparticle_factor,
                                         double dV, const int8_t* mask_host, const double* voltage_host,
                                         const double* rho_dev, double* u_dev, double tol, int max_iter,
                                         void* stream, mag_solve_info* info)
{
    using namespace mag;
    g_noalloc_err.clear();
    if ((coord != 0 && coord != 1) || nx < 3 || nz < 3 || !mask_host || !voltage_host || !rho_dev || !u_dev ||
        !(dx > 0) || !(dz > 0)) {
        g_noalloc_err = "mag_poisson_solve_noalloc: invalid arguments";
        return MAG_EINVAL;
    }
    if ((long long)nx * nz > kNoAllocMaxNodes) {
        g_noalloc_err = "mag_poisson_solve_noalloc: grid of " + std::to_string((long long)nx * nz) +
                        " nodes exceeds the allocation-free limit of " + std::to_string(kNoAllocMaxNodes) +
                        " nodes (257 x 257)";
        return MAG_EINVAL;
    }
    const size_t nn = (size_t)nx * nz;
    std::vector<int8_t> mask(mask_host, mask_host + nn);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j) {
            const int8_t m = mask[(size_t)i * nz + j];
            if (m == 0 || m == 1) continue;
            const bool axis_ok = coord == 1 && i == 0;
            if ((i == 0 && !axis_ok) || i == nx - 1 || j == 0 || j == nz - 1) {
                g_noalloc_err = "mag_poisson_solve_noalloc: free node on the domain edge";
                return MAG_EINVAL;
            }
        }
    // multigrid hierarchy (host, FP64) and the scratch layout
    // full coarsening only, so that the scratch layout of every accepted grid fits the static array
    std::vector<int> lnx, lnz, lmode;
    multigrid_levels(nx, nz, 1.0, kMaxLevels, lnx, lnz, lmode);
    const int nlev = (int)lnx.size();
    std::vector<std::vector<float>> coef(nlev), idiag(nlev);
    std::vector<float> cinv;
    {
        std::vector<double> A, Ac;
        fine_operator(coord, nx, nz, dx, dz, mask, A);
        std::vector<char> fixed_f(nn);
        for (size_t k = 0; k < nn; ++k) fixed_f[k] = mask[k] == 0 || mask[k] == 1;
        for (int l = 1; l < nlev; ++l) {
            int cx, cz;
            galerkin(lnx[l - 1], lnz[l - 1], A, fixed_f, kCoarsenFull, cx, cz, Ac);
            const size_t n = (size_t)cx * cz;
            coef[l].assign(Ac.begin(), Ac.end());
            idiag[l].resize(n);
            for (size_t k = 0; k < n; ++k) idiag[l][k] = (float)(1.0 / Ac[4 * n + k]);
            A.swap(Ac);
            fixed_f.assign(n, 0);
        }
        if (nlev > 1 && (long long)lnx.back() * lnz.back() <= kDenseCoarseMax)
            if (!dense_inverse(lnx.back(), lnz.back(), A, cinv)) cinv.clear();
    }
    std::vector<double> st64;
    double k2 = 1.0;
    fine_stencil_table(coord, nx, dx, dz, st64, k2);
    std::vector<float> st32(st64.begin(), st64.end());
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align256(off + bytes);
        return o;
    };
    const size_t o_mask = take(nn), o_volt = take(nn * 8), o_b = take(nn * 8), o_red = take(8 * 8),
                 o_status = take(sizeof(SolveStatus)), o_bar = take(sizeof(GridBarrier)), o_err = take(sizeof(int));
    std::vector<size_t> o_e(nlev), o_r(nlev), o_t(nlev), o_c(nlev), o_d(nlev);
    for (int l = 0; l < nlev; ++l) {
        const size_t n = (size_t)lnx[l] * lnz[l];
        o_e[l] = take(n * 4);
        o_r[l] = take(n * 4);
        o_t[l] = take(n * 4);
        if (l > 0) {
            o_c[l] = take(9 * n * 4);
            o_d[l] = take(n * 4);
        }
    }
    const size_t o_st64 = take(st64.size() * 8), o_st32 = take(st32.size() * 4);
    size_t o_cinv = 0;
    if (!cinv.empty()) {  // the dense coarsest solve, when it still fits
        if (align256(off + cinv.size() * 4) <= kNoAllocScratchBytes) o_cinv = take(cinv.size() * 4);
        else cinv.clear();
    }
    if (off > kNoAllocScratchBytes) {
        g_noalloc_err = "mag_poisson_solve_noalloc: scratch layout of " + std::to_string(off) +
                        " bytes exceeds the static array of " + std::to_string(kNoAllocScratchBytes) + " bytes";
        return MAG_EINVAL;
    }
    unsigned char* base = nullptr;
    int rc = scratch_address(&base);
    if (rc != MAG_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    auto ck = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess && rc == MAG_OK) {
            g_noalloc_err = std::string("mag_poisson_solve_noalloc: ") + what + ": " + cudaGetErrorString(e);
            rc = MAG_ECUDA;
        }
    };
    ck(cudaMemcpyAsync(base + o_mask, mask.data(), nn, cudaMemcpyHostToDevice, s), "mask copy");
    ck(cudaMemcpyAsync(base + o_volt, voltage_host, nn * 8, cudaMemcpyHostToDevice, s), "voltage copy");
    for (int l = 1; l < nlev; ++l) {
        ck(cudaMemcpyAsync(base + o_c[l], coef[l].data(), coef[l].size() * 4, cudaMemcpyHostToDevice, s), "coef copy");
        ck(cudaMemcpyAsync(base + o_d[l], idiag[l].data(), idiag[l].size() * 4, cudaMemcpyHostToDevice, s),
           "diag copy");
    }
    ck(cudaMemcpyAsync(base + o_st64, st64.data(), st64.size() * 8, cudaMemcpyHostToDevice, s), "stencil copy");
    ck(cudaMemcpyAsync(base + o_st32, st32.data(), st32.size() * 4, cudaMemcpyHostToDevice, s), "stencil copy");
    if (!cinv.empty())
        ck(cudaMemcpyAsync(base + o_cinv, cinv.data(), cinv.size() * 4, cudaMemcpyHostToDevice, s), "inverse copy");
    // state left by the previous call that must start at zero
    ck(cudaMemsetAsync(base + o_red, 0, 8 * 8, s), "clear");
    ck(cudaMemsetAsync(base + o_status, 0, sizeof(SolveStatus), s), "clear");
    ck(cudaMemsetAsync(base + o_bar, 0, sizeof(GridBarrier), s), "clear");
    ck(cudaMemsetAsync(base + o_err, 0, sizeof(int), s), "clear");
    if (rc != MAG_OK) return rc;

    SolveArgs a{};
    a.coord = coord;
    a.nx = nx;
    a.nz = nz;
    a.dx = dx;
    a.dz = dz;
    a.idx = 1.0 / dx;
    a.idz = 1.0 / dz;
    a.mask = (const int8_t*)(base + o_mask);
    a.voltage = (const double*)(base + o_volt);
    a.u = u_dev;
    a.b = (double*)(base + o_b);
    a.rf_solve = 0;
    a.rho_src = 2;
    a.rho64 = rho_dev;
    a.clear_rho = 0;
    a.mpf = macroparticle_factor;
    a.dV = dV;
    a.st64 = (const double*)(base + o_st64);
    a.st32 = (const float*)(base + o_st32);
    a.k2 = k2;
    a.coarse_inv = cinv.empty() ? nullptr : (const float*)(base + o_cinv);
    a.nlev = nlev;
    for (int l = 0; l < nlev; ++l) {
        a.lev[l].nx = lnx[l];
        a.lev[l].nz = lnz[l];
        a.lev[l].dz = div_magic((unsigned)lnz[l]);
        a.lev[l].dhz = div_magic((unsigned)((lnz[l] + 1) / 2));
        a.lev[l].e = (float*)(base + o_e[l]);
        a.lev[l].r = (float*)(base + o_r[l]);
        a.lev[l].t = (float*)(base + o_t[l]);
        a.lev[l].coef = l > 0 ? (const float*)(base + o_c[l]) : nullptr;
        a.lev[l].inv_diag = l > 0 ? (const float*)(base + o_d[l]) : nullptr;
    }
    a.nu1 = 2;
    a.nu2 = 2;
    a.ncoarse = nlev == 1 ? 20 : 40;
    a.omega = nlev == 1 ? (float)(2.0 / (1.0 + std::sin(3.14159265358979323846 / std::max(nx, nz)))) : 1.f;
    a.tol = tol > 0 ? tol : 1e-12;
    const int mi = max_iter > 0 ? max_iter : 200;
    a.max_outer = nlev == 1 ? 20 * mi : mi;
    a.Exf = nullptr;
    a.Ezf = nullptr;
    a.red = (double*)(base + o_red);
    a.bar = (GridBarrier*)(base + o_bar);
    a.status = (SolveStatus*)(base + o_status);
    a.err = (int*)(base + o_err);
    launch_solve(a, 1, s);
    ck(cudaGetLastError(), "launch");
    if (rc != MAG_OK || !info) return rc;
    ck(cudaStreamSynchronize(s), "synchronize");
    SolveStatus st{};
    int err = 0;
    ck(cudaMemcpy(&st, base + o_status, sizeof st, cudaMemcpyDeviceToHost), "status copy");
    ck(cudaMemcpy(&err, base + o_err, sizeof err, cudaMemcpyDeviceToHost), "status copy");
    if (rc != MAG_OK) return rc;
    info->iterations = st.iterations;
    info->residual = st.residual;
    info->status = err != 0 ? err : (st.converged ? MAG_OK : MAG_ENOTCONV);
    info->levels = nlev;
    if (err == MAG_ETIMEOUT) {
        g_noalloc_err = "mag_poisson_solve_noalloc: a grid barrier of the solve kernel gave up waiting (timeout)";
        return err;
    }
    if (err != 0) {
        g_noalloc_err = "mag_poisson_solve_noalloc: the solve did not reach its tolerance";
        return err;
    }
    return MAG_OK;
}
