// Poisson solve of Fields::boundary_solve / boundary_solve_rf
// (src/fields.cpp:278-348) on the reference's own 5-point operator
// (assembly src/fields.cpp:136-259, solved as the row stencil through
// UMFPACK_At at :311).
//
// One persistent kernel runs the whole solve: it builds the FP64 right-hand
// side exactly as the reference scales rho, then iterates
//     r = b - A u            (FP64, Jacobi-scaled max-norm as stopping test)
//     A e = r                (FP32 multigrid V-cycle: red-black Gauss-Seidel
//                             on the fine 5-point operator, 4-colour
//                             Gauss-Seidel on Galerkin 9-point coarse levels)
//     u += e                 (FP64)
// until |r/diag|_inf <= tol * |u|_inf, and finally writes the face electric
// field used by the particle kernel.  When the grid cannot be coarsened the
// inner solve is red-black SOR.  A single block (barrier = __syncthreads)
// serves grids up to a few 1e4 nodes; larger grids run the same code on many
// blocks under a cooperative launch with a bounded grid barrier.
#include <cooperative_groups.h>
#include <utility>

#include "device.hpp"
#include "kernels.hpp"
#include "multigrid_host.hpp"

namespace mag {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kEps0d = 8.854187817e-12;
constexpr long long kBarrierSpinLimit = 20000000;  // ~seconds of __nanosleep(64) polling
constexpr int kDenseCoarseMaxDev = (int)kDenseCoarseMax;
constexpr int kCoarseChunks = 6;

// The threads that share a piece of the solve: the whole grid (synchronised
// by a bounded grid barrier) or one block (synchronised by __syncthreads).
//
// The grid barrier counts arrivals on one monotonic counter (zeroed before the
// launch): barrier number e of the launch is passed when the counter reaches
// e * nblocks.  Thread 0 of each block adds its arrival with a release
// reduction (no return value, no reset) and polls with acquire loads, so no
// block waits for another block's atomic to come back.
struct Team {
    GridBarrier* bar;
    unsigned nblocks;
    unsigned tid, nthreads;
    unsigned epoch = 0;  // barriers passed so far (the same in every thread)
    double* prof = nullptr;  // phase times (thread 0 of block 0 records them), or null
    unsigned long long t_mark = 0;
    __device__ static unsigned long long now()
    {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        return t;
    }
    // add the time since the last mark to phase slot `phase` (called after a barrier)
    __device__ void mark(int phase)
    {
        if (prof == nullptr || blockIdx.x != 0 || threadIdx.x != 0) return;
        const unsigned long long t = now();
        prof[phase] += (double)(t - t_mark);
        t_mark = t;
    }
    __device__ Team(GridBarrier* b)
        : bar(b), nblocks(gridDim.x), tid(blockIdx.x * blockDim.x + threadIdx.x), nthreads(gridDim.x * blockDim.x)
    {
    }
    // this block alone
    __device__ static Team block(GridBarrier* b)
    {
        Team t(b);
        t.nblocks = 1;
        t.tid = threadIdx.x;
        t.nthreads = blockDim.x;
        return t;
    }
    // returns false when the grid barrier gave up (the kernel then returns)
    __device__ bool sync()
    {
        __syncthreads();
        if (nblocks == 1) return true;
        __shared__ int s_ok;
        ++epoch;
        if (threadIdx.x == 0) {
            const unsigned target = epoch * nblocks;
            asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&bar->count) : "memory");
            int ok = 1;
            long long spins = 0;
            for (;;) {
                unsigned c;
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(&bar->count) : "memory");
                if ((int)(c - target) >= 0) break;
                if (++spins > kBarrierSpinLimit || *((volatile unsigned*)&bar->abort)) {
                    atomicExch(&bar->abort, 1u);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
            s_ok = ok && !*((volatile unsigned*)&bar->abort);
        }
        __syncthreads();
        return s_ok;
    }
};

__device__ __forceinline__ bool is_fixed(int8_t m) { return m == 0 || m == 1; }

// Unsigned division by a divisor fixed for a whole pass, as a multiply-high
// and shifts (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994, figure 4.1): exact for every 32-bit n.
struct FastDiv {
    unsigned d, mp;
    int l;
    __device__ FastDiv() : d(1), mp(0), l(0) {}
    __device__ explicit FastDiv(unsigned dd) : d(dd)
    {
        l = dd > 1 ? 32 - __clz(dd - 1) : 0;  // ceil(log2 d)
        mp = (unsigned)(((1ull << 32) * ((1ull << l) - dd)) / dd + 1);
    }
    __device__ explicit FastDiv(const DivMagic& m) : d(m.d), mp(m.m), l(m.l) {}
    __device__ __forceinline__ unsigned div(unsigned n) const
    {
        if (d == 1) return n;
        const unsigned t1 = __umulhi(mp, n);
        return (t1 + ((n - t1) >> 1)) >> (l - 1);
    }
};

// Face fields of Field2D::grad: Exf[r][j] = -(u[ic][j] - u[ic-1][j]) / dx with
// ic = clamp(r, 1, nx-1), Ezf[i][c] = -(u[i][jc] - u[i][jc-1]) / dz with
// jc = clamp(c, 1, nz-1); idx, idz = 1/dx, 1/dz from the host
__device__ void faces_pass(const double* __restrict__ u, int nx, int nz, double idx, double idz, float* __restrict__ Exf,
                           float* __restrict__ Ezf, unsigned tid, unsigned nthreads)
{
    const FastDiv dz((unsigned)nz), dz1((unsigned)(nz + 1));
    const unsigned n1 = (unsigned)((nx + 1) * nz), n2 = (unsigned)(nx * (nz + 1));
    for (unsigned q = tid; q < n1; q += nthreads) {
        int i = (int)dz.div(q);
        const int j = (int)(q - (unsigned)i * nz);
        i = i < 1 ? 1 : (i > nx - 1 ? nx - 1 : i);
        Exf[q] = (float)(-(u[(size_t)i * nz + j] - u[(size_t)(i - 1) * nz + j]) * idx);
    }
    for (unsigned p = tid; p < n2; p += nthreads) {
        const int i = (int)dz1.div(p);
        int j = (int)(p - (unsigned)i * (nz + 1));
        j = j < 1 ? 1 : (j > nz - 1 ? nz - 1 : j);
        Ezf[p] = (float)(-(u[(size_t)i * nz + j] - u[(size_t)i * nz + j - 1]) * idz);
    }
}

// 5-point row of the fine operator (fields.cpp:149-238) of row i, from the
// per-row table built on the host
struct Stencil5 {
    double w, e, s, n, c, inv_c;
};
__device__ __forceinline__ Stencil5 fine_stencil(const SolveArgs& a, int i)
{
    const double* t = a.st64 + 4 * i;
    return {t[0], t[1], a.k2, a.k2, t[2], t[3]};
}
// the reference's scaling of rho into the right-hand side of row i (fields.cpp:283-300)
__device__ __forceinline__ double rhs_scale(const SolveArgs& a, int i)
{
    if (a.rscale) return a.rscale[i];  // the table holds the same expression (no FP64 division per node)
    if (a.coord == 1)
        return i > 0 ? -1.0 / kEps0d / (kPi * a.dx * a.dx * 2.0 * i * a.dz) * a.mpf
                     : -1.0 / kEps0d / (kPi * a.dx * a.dx * 0.25 * a.dz) * a.mpf;
    return -(a.dx * a.dx) / kEps0d / a.dV;
}

__device__ __forceinline__ double atomic_max_nonneg(double* p, double v)
{
    return __longlong_as_double(
        (long long)atomicMax((unsigned long long*)p, (unsigned long long)__double_as_longlong(v)));
}

template <class T>
__device__ T block_max(T v)
{
    __shared__ T s[32];
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) s[w] = v;
    __syncthreads();
    if (w == 0) {
        v = l < (int)(blockDim.x >> 5) ? s[l] : T(0);
        for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (l == 0) s[0] = v;
    }
    __syncthreads();
    const T r = s[0];
    __syncthreads();
    return r;
}

// ---- FP32 multigrid pieces -------------------------------------------------
//
// Every pass is a strided loop over the nodes of a level, unrolled so that a
// thread issues the loads of several nodes before it computes and stores any.
// Within one pass a node is either only read or only written (the other
// colour, or another array), so the arrays are accessed through separate
// __restrict__ read and write pointers and the compiler may batch the loads.

// red-black Gauss-Seidel (or SOR) sweeps on the fine level
__device__ void smooth_fine(const SolveArgs& a, Team& t, int sweeps, bool reverse, float omega, bool& ok)
{
    const MGLevelDev& L = a.lev[0];
    const int nx = L.nx, nz = L.nz, hz = (nz + 1) / 2;
    const float* __restrict__ ein = L.e;
    float* __restrict__ eout = L.e;
    const float* __restrict__ r = L.r;
    const int8_t* __restrict__ mask = a.mask;
    const float* __restrict__ st = a.st32;
    const float k2 = (float)a.k2;
    const unsigned n = (unsigned)(nx * hz);
    const FastDiv dh(L.dhz);
    for (int s = 0; s < sweeps && ok; ++s)
        for (int cc = 0; cc < 2 && ok; ++cc) {
            const int color = reverse ? 1 - cc : cc;
#pragma unroll 4
            for (unsigned q = t.tid; q < n; q += t.nthreads) {
                const int i = (int)dh.div(q);
                const int j = 2 * (int)(q - (unsigned)i * hz) + ((i + color) & 1);
                if (j >= nz) continue;
                const size_t k = (size_t)i * nz + j;
                if (is_fixed(mask[k])) continue;
                float acc = r[k];
                if (i > 0) acc -= st[4 * i] * ein[k - nz];
                acc -= st[4 * i + 1] * ein[k + nz];
                acc -= k2 * ein[k - 1];
                acc -= k2 * ein[k + 1];
                const float enew = acc / st[4 * i + 2];
                if (omega == 1.f) {
                    eout[k] = enew;
                } else {
                    const float e0 = ein[k];  // this node is read and written by this thread only
                    eout[k] = e0 + omega * (enew - e0);
                }
            }
            ok = t.sync();
        }
}

__device__ __forceinline__ float coarse_apply(const float* __restrict__ coef, int nx, int nz, int i, int j, size_t k,
                                              const float* __restrict__ e, bool skip_center)
{
    const size_t n = (size_t)nx * nz;
    float acc = 0.f;
#pragma unroll
    for (int di = -1; di <= 1; ++di) {
        if (i + di < 0 || i + di >= nx) continue;
#pragma unroll
        for (int dj = -1; dj <= 1; ++dj) {
            if (j + dj < 0 || j + dj >= nz) continue;
            if (skip_center && di == 0 && dj == 0) continue;
            const int p = (di + 1) * 3 + (dj + 1);
            acc += coef[p * n + k] * e[k + (ptrdiff_t)di * nz + dj];  // coef may sit in shared memory
        }
    }
    return acc;
}

// 4-colour Gauss-Seidel on a Galerkin level (9-point stencil)
__device__ void smooth_coarse(const SolveArgs& a, Team& t, int l, int sweeps, bool reverse, bool& ok)
{
    const MGLevelDev& L = a.lev[l];
    const int nx = L.nx, nz = L.nz;
    const int hx = (nx + 1) / 2, hz = (nz + 1) / 2;
    const float* __restrict__ ein = L.e;
    float* __restrict__ eout = L.e;
    const float* __restrict__ r = L.r;
    const float* __restrict__ coef = L.coef;
    const float* __restrict__ idg = L.inv_diag;
    const unsigned n = (unsigned)(hx * hz);
    const FastDiv dh(L.dhz);
    for (int s = 0; s < sweeps && ok; ++s)
        for (int cc = 0; cc < 4 && ok; ++cc) {
            const int color = reverse ? 3 - cc : cc;
            const int ci = color >> 1, cj = color & 1;
#pragma unroll 2
            for (unsigned q = t.tid; q < n; q += t.nthreads) {
                const unsigned qi = dh.div(q);
                const int i = 2 * (int)qi + ci, j = 2 * (int)(q - qi * hz) + cj;
                if (i >= nx || j >= nz) continue;
                const size_t k = (size_t)i * nz + j;
                const float off = coarse_apply(coef, nx, nz, i, j, k, ein, true);
                eout[k] = (r[k] - off) * idg[k];
            }
            ok = t.sync();
        }
}

// t = r - A e on level l (fine level: free nodes only)
__device__ void residual_level(const SolveArgs& a, Team& t, int l, float* __restrict__ out)
{
    const MGLevelDev& L = a.lev[l];
    const int nx = L.nx, nz = L.nz;
    const float* __restrict__ e = L.e;
    const float* __restrict__ r = L.r;
    const unsigned n = (unsigned)(nx * nz);
    const FastDiv dz(L.dz);
    if (l == 0) {
        const int8_t* __restrict__ mask = a.mask;
        const float* __restrict__ st = a.st32;
        const float k2 = (float)a.k2;
#pragma unroll 4
        for (unsigned q = t.tid; q < n; q += t.nthreads) {
            const int i = (int)dz.div(q);
            if (is_fixed(mask[q])) {
                out[q] = 0.f;
                continue;
            }
            float acc = r[q] - st[4 * i + 2] * e[q];
            if (i > 0) acc -= st[4 * i] * e[q - nz];
            acc -= st[4 * i + 1] * e[q + nz];
            acc -= k2 * e[q - 1];
            acc -= k2 * e[q + 1];
            out[q] = acc;
        }
    } else {
        const float* __restrict__ coef = L.coef;
#pragma unroll 2
        for (unsigned q = t.tid; q < n; q += t.nthreads) {
            const unsigned i = dz.div(q);
            out[q] = r[q] - coarse_apply(coef, nx, nz, (int)i, (int)(q - i * nz), q, e, false);
        }
    }
}

// Interpolation between level l and l + 1 (coarsening mode m): coarse node
// (I, J) sits on fine node (sx I, sz J) with sx = 2 where x is coarsened
// (1 where it is kept), likewise sz; the reach is 1 in a coarsened direction
// (weights 1, 1/2), 0 in a kept one.
__device__ __forceinline__ int coarsen_sx(int m) { return m == 2 ? 1 : 2; }
__device__ __forceinline__ int coarsen_sz(int m) { return m == 1 ? 1 : 2; }

// coarse residual of node (I, J): P^T t around fine (sx I, sz J); get(i, j)
// returns the fine residual (0 at fixed fine nodes) as float or double
template <class Get, class T = decltype(std::declval<Get>()(0, 0))>
__device__ __forceinline__ T restrict_node(int I, int J, int m, int nxf, int nzf, const Get& get)
{
    const int sx = coarsen_sx(m), sz = coarsen_sz(m);
    const int rx = sx - 1, rz = sz - 1;
    T acc = T(0);
#pragma unroll
    for (int di = -1; di <= 1; ++di) {
        if (di < -rx || di > rx) continue;
        const int i = sx * I + di;
        if (i < 0 || i >= nxf) continue;
        const T wi = di == 0 ? T(1) : T(0.5);
#pragma unroll
        for (int dj = -1; dj <= 1; ++dj) {
            if (dj < -rz || dj > rz) continue;
            const int j = sz * J + dj;
            if (j < 0 || j >= nzf) continue;
            const T wj = dj == 0 ? T(1) : T(0.5);
            acc += wi * wj * get(i, j);
        }
    }
    return acc;
}

// fine value (i, j) of P e_coarse
template <class T>
__device__ __forceinline__ T prolong_node(int i, int j, int m, const T* __restrict__ ec, int ncz)
{
    const int sx = coarsen_sx(m), sz = coarsen_sz(m);
    const int I0 = sx == 2 ? i >> 1 : i, J0 = sz == 2 ? j >> 1 : j;
    const bool oi = sx == 2 && (i & 1), oj = sz == 2 && (j & 1);
    const size_t b = (size_t)I0 * ncz + J0;
    if (!oi && !oj) return ec[b];
    if (oi && !oj) return T(0.5) * (ec[b] + ec[b + ncz]);
    if (!oi && oj) return T(0.5) * (ec[b] + ec[b + 1]);
    return T(0.25) * (ec[b] + ec[b + ncz] + ec[b + 1] + ec[b + ncz + 1]);
}

// r_{l+1} = P^T t_l (weights 1, 1/2, 1/4; fixed fine nodes carry no residual); e_{l+1} = 0
__device__ void restrict_level(const SolveArgs& a, Team& t, int l, const float* __restrict__ tl)
{
    const MGLevelDev& F = a.lev[l];
    const MGLevelDev& C = a.lev[l + 1];
    float* __restrict__ cr = C.r;
    float* __restrict__ ce = C.e;
    const unsigned n = (unsigned)(C.nx * C.nz);
    const FastDiv dz(C.dz);
    const int fnz = F.nz;
    auto get = [&](int i, int j) { return tl[(size_t)i * fnz + j]; };
#pragma unroll 2
    for (unsigned q = t.tid; q < n; q += t.nthreads) {
        const int I = (int)dz.div(q), J = (int)(q - (unsigned)I * C.nz);
        cr[q] = restrict_node(I, J, F.cmode, F.nx, F.nz, get);
        ce[q] = 0.f;
    }
}

// e_l += P e_{l+1} (bilinear; fixed fine nodes untouched)
__device__ void prolong_level(const SolveArgs& a, Team& t, int l)
{
    const MGLevelDev& F = a.lev[l];
    const MGLevelDev& C = a.lev[l + 1];
    const float* __restrict__ ec = C.e;
    float* __restrict__ fe = F.e;
    const unsigned n = (unsigned)(F.nx * F.nz);
    const FastDiv dz(F.dz);
#pragma unroll 4
    for (unsigned q = t.tid; q < n; q += t.nthreads) {
        if (l == 0 && is_fixed(a.mask[q])) continue;
        const int i = (int)dz.div(q), j = (int)(q - (unsigned)i * F.nz);
        fe[q] += prolong_node(i, j, F.cmode, ec, C.nz);
    }
}

// Coarsest level: e = A^-1 r with the dense inverse (one pass), else
// Gauss-Seidel sweeps.
__device__ void coarse_solve(const SolveArgs& a, Team& t, bool& ok)
{
    const int l = a.nlev - 1;
    const MGLevelDev& L = a.lev[l];
    if (a.coarse_inv == nullptr) {
        smooth_coarse(a, t, l, a.ncoarse, false, ok);
        return;
    }
    const unsigned n = (unsigned)(L.nx * L.nz);
    if (t.nblocks == 1 && n <= (unsigned)kDenseCoarseMaxDev) {
        // e = G r with the columns split into kCoarseChunks ranges: thread (k, row)
        // sums its range (independent, coalesced loads), then the ranges are
        // added in a fixed order, so the result does not depend on the thread count
        __shared__ float part[kCoarseChunks][kDenseCoarseMaxDev];
        constexpr int kSpan = (kDenseCoarseMaxDev + kCoarseChunks - 1) / kCoarseChunks;
        for (unsigned q = t.tid; q < kCoarseChunks * n; q += t.nthreads) {
            const unsigned k = q / n, row = q - k * n;
            const unsigned c0 = k * n / kCoarseChunks, c1 = (k + 1) * n / kCoarseChunks;
            float acc = 0.f;
#pragma unroll
            for (int c = 0; c < kSpan; ++c)  // every load of the range in flight at once
                if (c0 + c < c1) acc += a.coarse_inv[(size_t)(c0 + c) * n + row] * L.r[c0 + c];
            part[k][row] = acc;
        }
        __syncthreads();
        for (unsigned row = t.tid; row < n; row += t.nthreads) {
            float acc = part[0][row];
#pragma unroll
            for (int k = 1; k < kCoarseChunks; ++k) acc += part[k][row];
            L.e[row] = acc;
        }
        ok = t.sync();
        return;
    }
    for (unsigned row = t.tid; row < n; row += t.nthreads) {
        float acc = 0.f;
        for (unsigned c = 0; c < n; ++c) acc += a.coarse_inv[(size_t)c * n + row] * L.r[c];
        L.e[row] = acc;
    }
    ok = t.sync();
}

// Coarsest level of a multi-block solve (a.coarse_grid): e = A^-1 r with the
// row-major dense inverse, one warp per row over all blocks; each lane sums a
// fixed set of columns and the warp adds them in a fixed tree, so the result
// does not depend on the launch shape.
__device__ void coarse_solve_grid(const SolveArgs& a, Team& t, bool& ok)
{
    const MGLevelDev& L = a.lev[a.nlev - 1];
    const unsigned n = (unsigned)(L.nx * L.nz);
    const unsigned lane = threadIdx.x & 31u, nwarps = t.nthreads >> 5;
    const float* __restrict__ r = L.r;
    for (unsigned row = t.tid >> 5; row < n; row += nwarps) {
        const float* __restrict__ g = a.coarse_inv_rows + (size_t)row * n;
        float acc = 0.f;
#pragma unroll 8
        for (unsigned c = lane; c < n; c += 32) acc += __ldg(&g[c]) * r[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) L.e[row] = acc;
    }
    ok = t.sync();
}

// The part of a V-cycle from level l0 down to the coarsest level and back up
// to l0, pre- and post-smoothing on l0 included.
__device__ void vcycle_from(const SolveArgs& a, Team& t, int l0, bool& ok)
{
    const int L = a.nlev;
    for (int l = l0; l < L - 1 && ok; ++l) {
        if (l == 0) smooth_fine(a, t, a.nu1, false, 1.f, ok);
        else smooth_coarse(a, t, l, a.nu1, false, ok);
        if (!ok) return;
        residual_level(a, t, l, a.lev[l].t);
        ok = t.sync();
        if (!ok) return;
        restrict_level(a, t, l, a.lev[l].t);
        ok = t.sync();
        t.mark(kPhaseDown + l);
    }
    if (!ok) return;
    coarse_solve(a, t, ok);
    t.mark(kPhaseCoarse);
    for (int l = L - 2; l >= l0 && ok; --l) {
        prolong_level(a, t, l);
        ok = t.sync();
        if (!ok) return;
        if (l == 0) smooth_fine(a, t, a.nu2, true, 1.f, ok);
        else smooth_coarse(a, t, l, a.nu2, true, ok);
        t.mark(kPhaseUp + l);
    }
}

// One V-cycle.  On a multi-block grid the levels from a.l_single down (at most
// kSingleBlockLevel nodes each) run on block 0 alone, synchronised by
// __syncthreads, while the other blocks wait at one grid barrier: a coarse
// level has too little work to pay for the grid barriers of its sweeps.  The
// Galerkin levels above it are smoothed with one 4-colour sweep each way (a
// sweep costs four grid barriers; the outer FP64 iterations do not increase).
constexpr int kCoarseSweepsGrid = 1;
__device__ void vcycle(const SolveArgs& a, Team& t, bool& ok)
{
    const int L = a.nlev;
    if (L == 1) {
        smooth_fine(a, t, a.ncoarse, false, a.omega, ok);
        return;
    }
    if (t.nblocks == 1 || a.l_single <= 0 || a.l_single >= L) {
        vcycle_from(a, t, 0, ok);
        return;
    }
    const int ls = a.l_single;
    for (int l = 0; l < ls && ok; ++l) {
        if (l == 0) smooth_fine(a, t, a.nu1, false, 1.f, ok);
        else smooth_coarse(a, t, l, kCoarseSweepsGrid, false, ok);
        if (!ok) return;
        residual_level(a, t, l, a.lev[l].t);
        ok = t.sync();
        if (!ok) return;
        restrict_level(a, t, l, a.lev[l].t);
        ok = t.sync();
        t.mark(kPhaseDown + l);
    }
    if (!ok) return;
    if (a.coarse_grid) {
        coarse_solve_grid(a, t, ok);
    } else {
        if (blockIdx.x == 0) {
            Team tb = Team::block(a.bar);
            bool okb = true;
            vcycle_from(a, tb, ls, okb);
            __threadfence();
        }
        ok = t.sync();
    }
    t.mark(kPhaseCoarse);
    for (int l = ls - 1; l >= 0 && ok; --l) {
        prolong_level(a, t, l);
        ok = t.sync();
        if (!ok) return;
        if (l == 0) smooth_fine(a, t, a.nu2, true, 1.f, ok);
        else smooth_coarse(a, t, l, kCoarseSweepsGrid, true, ok);
        t.mark(kPhaseUp + l);
    }
}

// ---- tile phases of a multi-block solve -------------------------------------
//
// On the levels above l_single every block owns tiles of ti x tj nodes.  A
// phase stages a tile and kTileHalo rings around it in shared memory, runs
// all colour passes of the phase there and writes back only the tile: pass p
// updates the nodes at most kTileHalo - 1 - p rings out, which are exactly
// the nodes whose neighbours are still up to date in shared memory, so the
// tile's values equal those of the same colour passes over the whole level.
// Down phase of level l: pre-smoothing from e = 0, residual, restriction to
// level l + 1 (one grid barrier instead of one per colour pass, residual and
// restriction).  Up phase: prolongation of level l + 1's correction,
// post-smoothing and, on the fine level, the FP64 update u += e.
struct TileRegion {
    int i0, j0, ni, nj;  // interior: rows i0 .. i0+ni-1, columns j0 .. j0+nj-1
    int ri, rj;          // global indices of region node (0, 0)
    int rh, rw;          // region rows and columns
};

__device__ __forceinline__ TileRegion tile_region(int t, int nx, int nz, int ti, int tj)
{
    const int ntj = (nz + tj - 1) / tj;
    const int a = t / ntj, b = t - a * ntj;
    TileRegion T;
    T.i0 = a * ti;
    T.j0 = b * tj;
    T.ni = min(ti, nx - T.i0);
    T.nj = min(tj, nz - T.j0);
    T.ri = T.i0 - kTileHalo;
    T.rj = T.j0 - kTileHalo;
    T.rh = T.ni + 2 * kTileHalo;
    T.rw = T.nj + 2 * kTileHalo;
    return T;
}

// rings between region node (li, lj) and the tile interior (0 inside)
__device__ __forceinline__ int tile_ring(const TileRegion& T, int li, int lj)
{
    const int di = max(max(kTileHalo - li, li - (T.ni + kTileHalo - 1)), 0);
    const int dj = max(max(kTileHalo - lj, lj - (T.nj + kTileHalo - 1)), 0);
    return max(di, dj);
}

struct TileShared {
    float* e;    // correction
    float* r;    // right-hand side, overwritten by the residual
    float* cf;   // Galerkin levels: the 9 operator planes of the region (plane p of node q at p * n + q)
    float* dg;   // Galerkin levels: inverse diagonal
    uint8_t* f;  // 1: outside the grid, or a fixed node of the fine level
    // divisions of the tile's loops, set up once per tile (the set-up itself
    // is a 64-bit division): by the region width, by its half (colour passes)
    // and by the interior width
    FastDiv dw, dh, dj;
};

__device__ __forceinline__ TileShared tile_shared(const TileRegion& T, const MGLevelDev& L, bool staged)
{
    extern __shared__ __align__(16) unsigned char tile_smem[];
    const int n = T.rh * T.rw;
    TileShared S;
    S.e = reinterpret_cast<float*>(tile_smem);
    S.r = S.e + n;
    S.cf = S.r + n;
    S.dg = S.cf + 9 * n;
    S.f = reinterpret_cast<uint8_t*>(staged ? S.dg + n : S.cf);
    const int c = T.nj == L.tj ? 0 : 1;  // the last column of tiles may be narrower
    S.dw = FastDiv(L.tw[c]);
    S.dh = FastDiv(L.th[c]);
    S.dj = FastDiv(L.tn[c]);
    return S;
}

// stage r (and e, or zeros), the flags and, on a Galerkin level, the operator
// of the region: every load of the phase is issued here at once
__device__ void tile_load(const SolveArgs& a, int l, const TileRegion& T, const TileShared& S, bool load_e)
{
    const MGLevelDev& L = a.lev[l];
    const int n = T.rh * T.rw;
    const FastDiv& dw = S.dw;
    const size_t nn = (size_t)L.nx * L.nz;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int li = (int)dw.div((unsigned)q), lj = q - li * T.rw;
        const int gi = T.ri + li, gj = T.rj + lj;
        const bool in = gi >= 0 && gi < L.nx && gj >= 0 && gj < L.nz;
        const size_t k = in ? (size_t)gi * L.nz + gj : 0;
        S.r[q] = in ? L.r[k] : 0.f;
        S.e[q] = (in && load_e) ? L.e[k] : 0.f;
        S.f[q] = (!in || (l == 0 && is_fixed(a.mask[k]))) ? 1 : 0;
        if (l > 0 && L.staged) {
#pragma unroll
            for (int p = 0; p < 9; ++p) S.cf[p * n + q] = in ? __ldg(&L.coef[p * nn + k]) : 0.f;
            S.dg[q] = in ? __ldg(&L.inv_diag[k]) : 0.f;
        }
    }
}

// one colour pass over the region nodes at most `reach` rings out
__device__ void tile_pass(const SolveArgs& a, int l, const TileRegion& T, const TileShared& S, int color, int reach)
{
    const MGLevelDev& L = a.lev[l];
    if (l == 0) {  // red-black Gauss-Seidel on the 5-point operator (smooth_fine, omega = 1)
        const float* __restrict__ st = a.st32;
        const float k2 = (float)a.k2;
        const int hw = (T.rw + 1) / 2;
        const int n = T.rh * hw;
        const FastDiv& dh = S.dh;
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const int li = (int)dh.div((unsigned)q);
            const int lj = 2 * (q - li * hw) + ((color + T.ri + T.rj + li) & 1);
            if (lj >= T.rw || tile_ring(T, li, lj) > reach) continue;
            const int p = li * T.rw + lj;
            if (S.f[p]) continue;
            const int i = T.ri + li;
            float acc = S.r[p];
            if (i > 0) acc -= st[4 * i] * S.e[p - T.rw];
            acc -= st[4 * i + 1] * S.e[p + T.rw];
            acc -= k2 * S.e[p - 1];
            acc -= k2 * S.e[p + 1];
            S.e[p] = acc * st[4 * i + 3];
        }
    } else {  // 4-colour Gauss-Seidel on the 9-point Galerkin operator (smooth_coarse)
        const int ci = color >> 1, cj = color & 1;
        const int hh = (T.rh + 1) / 2, hw = (T.rw + 1) / 2;
        const int n = hh * hw;
        const int nr = T.rh * T.rw;
        const FastDiv& dh = S.dh;
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const int a2 = (int)dh.div((unsigned)q);
            const int li = 2 * a2 + ((ci + T.ri) & 1);
            const int lj = 2 * (q - a2 * hw) + ((cj + T.rj) & 1);
            if (li >= T.rh || lj >= T.rw || tile_ring(T, li, lj) > reach) continue;
            const int p = li * T.rw + lj;
            if (S.f[p]) continue;
            const int i = T.ri + li, j = T.rj + lj;
            // the operator row from the staged planes or from the level's own
            const float* cf = L.staged ? S.cf + p : L.coef + ((size_t)i * L.nz + j);
            const size_t cs = L.staged ? (size_t)nr : (size_t)L.nx * L.nz;
            float off = 0.f;
#pragma unroll
            for (int di = -1; di <= 1; ++di) {
                if (i + di < 0 || i + di >= L.nx) continue;
#pragma unroll
                for (int dj = -1; dj <= 1; ++dj) {
                    if (j + dj < 0 || j + dj >= L.nz) continue;
                    if (di == 0 && dj == 0) continue;
                    off += cf[((di + 1) * 3 + (dj + 1)) * cs] * S.e[p + di * T.rw + dj];
                }
            }
            const float dg = L.staged ? S.dg[p] : __ldg(&L.inv_diag[(size_t)i * L.nz + j]);
            S.e[p] = (S.r[p] - off) * dg;
        }
    }
}

// residual t = r - A e in place of r, for the region nodes at most `reach` rings out
__device__ void tile_residual(const SolveArgs& a, int l, const TileRegion& T, const TileShared& S, int reach)
{
    const MGLevelDev& L = a.lev[l];
    const int n = T.rh * T.rw;
    const FastDiv& dw = S.dw;
    const float* __restrict__ st = a.st32;
    const float k2 = (float)a.k2;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int li = (int)dw.div((unsigned)q), lj = q - li * T.rw;
        if (tile_ring(T, li, lj) > reach) continue;
        if (S.f[q]) {
            S.r[q] = 0.f;
            continue;
        }
        const int i = T.ri + li, j = T.rj + lj;
        float acc;
        if (l == 0) {
            acc = S.r[q] - st[4 * i + 2] * S.e[q];
            if (i > 0) acc -= st[4 * i] * S.e[q - T.rw];
            acc -= st[4 * i + 1] * S.e[q + T.rw];
            acc -= k2 * S.e[q - 1];
            acc -= k2 * S.e[q + 1];
        } else {
            const float* cf = L.staged ? S.cf + q : L.coef + ((size_t)i * L.nz + j);
            const size_t cs = L.staged ? (size_t)n : (size_t)L.nx * L.nz;
            float ae = 0.f;
#pragma unroll
            for (int di = -1; di <= 1; ++di) {
                if (i + di < 0 || i + di >= L.nx) continue;
#pragma unroll
                for (int dj = -1; dj <= 1; ++dj) {
                    if (j + dj < 0 || j + dj >= L.nz) continue;
                    ae += cf[((di + 1) * 3 + (dj + 1)) * cs] * S.e[q + di * T.rw + dj];
                }
            }
            acc = S.r[q] - ae;
        }
        S.r[q] = acc;
    }
}

// down phase of level l: pre-smoothing, residual, restriction to level l + 1
__device__ void tile_down(const SolveArgs& a, int l)
{
    const MGLevelDev& L = a.lev[l];
    const MGLevelDev& C = a.lev[l + 1];
    const int ntiles = ((L.nx + L.ti - 1) / L.ti) * ((L.nz + L.tj - 1) / L.tj);
    const int sweeps = l == 0 ? a.nu1 : kCoarseSweepsGrid;
    const int ncolors = l == 0 ? 2 : 4;
    for (int tt = blockIdx.x; tt < ntiles; tt += gridDim.x) {
        const TileRegion T = tile_region(tt, L.nx, L.nz, L.ti, L.tj);
        const TileShared S = tile_shared(T, L, l > 0 && L.staged);
        tile_load(a, l, T, S, false);
        __syncthreads();
        int pass = 0;
        for (int s = 0; s < sweeps; ++s)
            for (int c = 0; c < ncolors; ++c, ++pass) {
                tile_pass(a, l, T, S, c, kTileHalo - 1 - pass);
                __syncthreads();
            }
        // the tile's correction back to the level (read again by the up phase)
        for (int q = threadIdx.x; q < T.ni * T.nj; q += blockDim.x) {
            const int ii = (int)S.dj.div((unsigned)q), jj = q - ii * T.nj;
            L.e[(size_t)(T.i0 + ii) * L.nz + T.j0 + jj] = S.e[(ii + kTileHalo) * T.rw + jj + kTileHalo];
        }
        tile_residual(a, l, T, S, kTileHalo - 1 - pass);
        __syncthreads();
        // coarse nodes (I, J) whose fine node (sx I, sz J) lies in the tile (restrict_level)
        const int sx = coarsen_sx(L.cmode), sz = coarsen_sz(L.cmode);
        const int I0 = (T.i0 + sx - 1) / sx, I1 = (T.i0 + T.ni - 1) / sx;
        const int J0 = (T.j0 + sz - 1) / sz, J1 = (T.j0 + T.nj - 1) / sz;
        const int cw = J1 - J0 + 1, nc = (I1 - I0 + 1) * cw;
        auto get = [&](int i, int j) { return S.r[(i - T.ri) * T.rw + (j - T.rj)]; };
        const FastDiv dcw((unsigned)cw);
        for (int q = threadIdx.x; q < nc; q += blockDim.x) {
            const int qi = (int)dcw.div((unsigned)q);
            const int I = I0 + qi, J = J0 + (q - qi * cw);
            const size_t K = (size_t)I * C.nz + J;
            C.r[K] = restrict_node(I, J, L.cmode, L.nx, L.nz, get);
            C.e[K] = 0.f;
        }
        __syncthreads();
    }
}

// up phase of level l: prolongation of level l + 1's correction, post-smoothing,
// and on the fine level the FP64 update of u.  The phase reads the pre-smoothed
// correction of its halo from L.e, which the down phase wrote, and writes its
// post-smoothed tile to L.t, so that no block reads what another one writes
// in the same phase; level l - 1 prolongs from L.t (level l_single's
// correction, computed by block 0, stays in its e).
//
// res_slot >= 0 (fine level): the phase also writes the next residual
// r - A e of its tile interior into L.r, in FP32 from the FP32 correction, and
// adds the block's max |r / c| and max |u| into a.red[res_slot], [res_slot + 1].
// The residual that r approximates changes by exactly -A e in the iteration,
// so the difference to the FP64 residual b - A u grows only by the rounding of
// each update, about 2^-24 of that iteration's residual: a few 1e-13 of max|u|
// after the whole solve.
__device__ void tile_up(const SolveArgs& a, int l, int res_slot)
{
    const MGLevelDev& L = a.lev[l];
    const MGLevelDev& C = a.lev[l + 1];
    const float* __restrict__ ce = l + 1 < a.l_single ? C.t : C.e;
    const int ntiles = ((L.nx + L.ti - 1) / L.ti) * ((L.nz + L.tj - 1) / L.tj);
    const int sweeps = l == 0 ? a.nu2 : kCoarseSweepsGrid;
    const int ncolors = l == 0 ? 2 : 4;
    for (int tt = blockIdx.x; tt < ntiles; tt += gridDim.x) {
        const TileRegion T = tile_region(tt, L.nx, L.nz, L.ti, L.tj);
        const TileShared S = tile_shared(T, L, l > 0 && L.staged);
        tile_load(a, l, T, S, true);
        __syncthreads();
        // e += P e_coarse on every region node of the grid (prolong_level)
        const int n = T.rh * T.rw;
        const FastDiv& dw = S.dw;
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            if (S.f[q]) continue;
            const int li = (int)dw.div((unsigned)q), lj = q - li * T.rw;
            S.e[q] += prolong_node(T.ri + li, T.rj + lj, L.cmode, ce, C.nz);
        }
        __syncthreads();
        int pass = 0;
        for (int s = 0; s < sweeps; ++s)
            for (int c = ncolors - 1; c >= 0; --c, ++pass) {
                tile_pass(a, l, T, S, c, kTileHalo - 1 - pass);
                __syncthreads();
            }
        float lres = 0.f;
        unsigned lumax_hi = 0u;
        for (int q = threadIdx.x; q < T.ni * T.nj; q += blockDim.x) {
            const int ii = (int)S.dj.div((unsigned)q), jj = q - ii * T.nj;
            const int p = (ii + kTileHalo) * T.rw + jj + kTileHalo;
            const size_t k = (size_t)(T.i0 + ii) * L.nz + T.j0 + jj;
            if (l > 0) {
                L.t[k] = S.e[p];
            } else if (!S.f[p]) {
                const double un = a.u[k] + (double)S.e[p];
                a.u[k] = un;
                if (res_slot >= 0) {
                    // every neighbour of an interior node holds its final value after the last pass
                    const int i = T.i0 + ii;
                    const float* st = a.st32 + 4 * i;
                    const float k2 = (float)a.k2;
                    float acc = S.r[p] - st[2] * S.e[p] - st[1] * S.e[p + T.rw] - k2 * (S.e[p - 1] + S.e[p + 1]);
                    if (i > 0) acc -= st[0] * S.e[p - T.rw];
                    L.r[k] = acc;
                    lres = fmaxf(lres, fabsf(acc * st[3]));
                    lumax_hi = max(lumax_hi, (unsigned)__double2hiint(un) & 0x7FFFFFFFu);
                }
            } else if (res_slot >= 0) {
                lumax_hi = max(lumax_hi, (unsigned)__double2hiint(a.u[k]) & 0x7FFFFFFFu);
            }
        }
        if (res_slot >= 0) {
            const double br = block_max((double)lres), bu = block_max(__hiloint2double((int)lumax_hi, 0));
            if (threadIdx.x == 0) {
                atomic_max_nonneg(&a.red[res_slot], br);
                atomic_max_nonneg(&a.red[res_slot + 1], bu);
            }
        }
        __syncthreads();
    }
}

// Block copy of n floats from global to shared memory, 16-byte vectors where
// both sides allow (level arrays start 16-byte aligned on both sides).
__device__ __forceinline__ void stage_copy(float* dst, const float* __restrict__ src, int n)
{
    const int n4 = n >> 2;
    const float4* s4 = reinterpret_cast<const float4*>(src);
    float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll 4
    for (int k = threadIdx.x; k < n4; k += blockDim.x) d4[k] = __ldg(&s4[k]);
    for (int k = 4 * n4 + threadIdx.x; k < n; k += blockDim.x) dst[k] = src[k];
}

// Block 0's part of a multi-block V-cycle: the levels from l_single down.
// With a.coarse_staged those levels (Galerkin planes, inverse diagonal,
// correction, right-hand side, scratch) are staged in the block's dynamic
// shared memory, which the tile phases do not use meanwhile, and the V-cycle
// runs on a copy of the arguments that points there: its ~40 colour passes
// then wait on shared memory instead of L2.  Level l_single's correction is
// copied back for the up phase of the level above.
__device__ void coarse_part(const SolveArgs& a, bool& okb)
{
    Team tb = Team::block(a.bar);
    const int ls = a.l_single;
    if (!a.coarse_staged) {
        vcycle_from(a, tb, ls, okb);
        return;
    }
    extern __shared__ __align__(16) unsigned char tile_smem[];
    static_assert(sizeof(SolveArgs) % 8 == 0, "word copy");
    SolveArgs* sa = reinterpret_cast<SolveArgs*>(tile_smem);
    {
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&a);
        unsigned long long* dst = reinterpret_cast<unsigned long long*>(tile_smem);
        for (int w = threadIdx.x; w < (int)(sizeof(SolveArgs) / 8); w += blockDim.x) dst[w] = src[w];
    }
    __syncthreads();
    float* base = reinterpret_cast<float*>(tile_smem + kStagedArgsBytes);
    size_t off = 0;
    for (int l = ls; l < a.nlev; ++l) {
        const MGLevelDev& G = a.lev[l];
        const int n = G.nx * G.nz;
        const int n4 = (n + 3) & ~3;  // every array of the level starts 16-byte aligned
        float* e = base + off;
        float* r = e + n4;
        float* t = r + n4;
        float* idg = t + n4;
        float* coef = idg + n4;
        off += 4 * (size_t)n4 + (((size_t)9 * n + 3) & ~(size_t)3);
        if (threadIdx.x == 0) {
            sa->lev[l].e = e;
            sa->lev[l].r = r;
            sa->lev[l].t = t;
            sa->lev[l].inv_diag = idg;
            sa->lev[l].coef = coef;
        }
        stage_copy(coef, G.coef, 9 * n);
        stage_copy(idg, G.inv_diag, n);
        if (l == ls) stage_copy(r, G.r, n);
        for (int k = threadIdx.x; k < n; k += blockDim.x) e[k] = 0.f;
    }
    __syncthreads();
    vcycle_from(*sa, tb, ls, okb);
    __syncthreads();
    const MGLevelDev& G = a.lev[ls];
    const float* e = sa->lev[ls].e;
    for (int k = threadIdx.x; k < G.nx * G.nz; k += blockDim.x) G.e[k] = e[k];
}

// One V-cycle of a multi-block solve with tile phases on the levels above
// l_single and block 0 alone below; ends with u += e (done by the fine level's
// up phase, which also leaves the next residual in the fine r when res_slot >= 0).
__device__ void vcycle_tiled(const SolveArgs& a, Team& t, bool& ok, int res_slot)
{
    const int ls = a.l_single;
    for (int l = 0; l < ls && ok; ++l) {
        tile_down(a, l);
        ok = t.sync();
        t.mark(kPhaseDown + l);
    }
    if (!ok) return;
    if (a.coarse_grid) {
        coarse_solve_grid(a, t, ok);
    } else {
        if (blockIdx.x == 0) {
            bool okb = true;
            coarse_part(a, okb);
            __threadfence();
        }
        ok = t.sync();
    }
    t.mark(kPhaseCoarse);
    for (int l = ls - 1; l >= 0 && ok; --l) {
        tile_up(a, l, l == 0 ? res_slot : -1);
        ok = t.sync();
        t.mark(kPhaseUp + l);
    }
}

// Steps 0 and 1 of a solve, shared by the FP32 and the FP64 multigrid
__device__ void solve_prologue(const SolveArgs& a, Team& t, bool& ok)
{
    const int nx = a.nx, nz = a.nz;
    const unsigned nn = (unsigned)(nx * nz);
    // 0. start of a step's solve: the linear extrapolation of the last two
    //    solutions on the free nodes (u_prev <- u), and
    // 1. right-hand side and Dirichlet values (boundary_solve / boundary_solve_rf),
    // one pass: both are per node
    const bool extrap = a.u_prev != nullptr;
    const bool valid = extrap && *((volatile const int*)a.u_prev_valid) != 0;
    const FastDiv dnz(a.lev[0].dz);
#pragma unroll 2
    for (unsigned k = t.tid; k < nn; k += t.nthreads) {
        const int i = (int)dnz.div(k);
        const int8_t m = a.mask[k];
        if (is_fixed(m)) {
            const double v = a.rf_solve ? (m == 1 ? a.voltage[k] : 0.0) : (m == 0 ? a.voltage[k] : 0.0);
            a.u[k] = v;
            a.b[k] = v;
        } else {
            if (extrap) {
                const double u = a.u[k];
                if (valid) a.u[k] = 2.0 * u - a.u_prev[k];
                a.u_prev[k] = u;
            }
            double rho = 0.0;
            if (a.rho_src == 1) {
                for (int s = 0; s < a.nsp; ++s) rho += a.rho_weight[s] * (double)a.rho_fixed[s][k];
            } else if (a.rho_src == 2) {
                rho = a.rho64[k];
            }
            a.b[k] = a.rho_src == 3 ? ((long long)k == a.unit_node ? 1.0 : 0.0) : rho * rhs_scale(a, i);
        }
        if (a.clear_rho && a.rho_src == 1)
            for (int s = 0; s < a.nsp; ++s) ((unsigned long long*)a.rho_fixed[s])[k] = 0ull;
    }
    ok = t.sync();
    if (extrap && t.tid == 0) *a.u_prev_valid = 1;  // every block read the flag before the barrier
}

// the solve's status words (thread 0 of the team)
__device__ void solve_report(const SolveArgs& a, const Team& t, int it, double res, bool conv, bool ok)
{
    if (t.tid != 0) return;
    a.status->iterations = it;
    a.status->residual = res;
    a.status->converged = conv ? 1 : 0;
    a.status->aborted = ok ? 0 : 1;
    if (!ok) atomicCAS(a.err, 0, -5);
    else if (!conv) atomicCAS(a.err, 0, -4);
}

__device__ void solve_body(const SolveArgs& a, Team& t)
{
    const int nx = a.nx, nz = a.nz;
    const unsigned nn = (unsigned)(nx * nz);
    bool ok = true;
    t.prof = a.prof;
    const unsigned long long t_start = Team::now();
    t.t_mark = t_start;
    solve_prologue(a, t, ok);
    const FastDiv dnz(a.lev[0].dz);
    t.mark(kPhaseStart);
    // 2. FP64 residual refinement around the FP32 multigrid
    int it = 0;
    double res = 0.0, ref0 = 0.0;
    bool conv = false;
    const MGLevelDev& F = a.lev[0];
    const double* __restrict__ uin = a.u;
    const double* __restrict__ bb = a.b;
    const int8_t* __restrict__ mask = a.mask;
    const float* __restrict__ st32 = a.st32;
    // A multi-block tiled solve takes the residual of each V-cycle from the
    // cycle's fine up phase (tile_up) and computes it in FP64 only at the start
    // and to confirm convergence; the other paths compute it in FP64 every time.
    const bool tiled = a.tiled && t.nblocks > 1;
    int cycles = 0, n64 = 0;
    bool updated = false;  // this pass's residual was left by the last fine up phase
    for (; ok; ++it) {
        double lres, lumax;
        if (updated) {
            const int slot = 4 + ((cycles - 1) & 1) * 2;
            lres = *((volatile double*)&a.red[slot]);
            lumax = *((volatile double*)&a.red[slot + 1]);
            if (t.tid == 0) {  // clear the next cycle's slots (last read right after the cycle before this one)
                a.red[10 - slot] = 0.0;
                a.red[11 - slot] = 0.0;
            }
        } else {
            // residual in FP64; its Jacobi-scaled max norm and max|u| only steer
            // the stopping test and are taken in FP32
            // max|u| from the high words of the doubles (sign cleared): integer
            // compares, no FP64 conversion; 20 mantissa bits are plenty for the
            // stopping test, and the truncation only makes the test stricter
            float lres32 = 0.f;
            unsigned lumax_hi = 0u;
            const bool zero_e = !tiled;  // the tile phases start from e = 0 in shared memory
#pragma unroll 2
            for (unsigned k = t.tid; k < nn; k += t.nthreads) {
                const int i = (int)dnz.div(k);
                const double uk = uin[k];
                lumax_hi = max(lumax_hi, (unsigned)__double2hiint(uk) & 0x7FFFFFFFu);
                if (zero_e) F.e[k] = 0.f;
                if (is_fixed(mask[k])) {
                    F.r[k] = 0.f;
                    continue;
                }
                const Stencil5 st = fine_stencil(a, i);
                double acc = st.c * uk;
                if (i > 0) acc += st.w * uin[k - nz];
                acc += st.e * uin[k + nz];
                acc += st.s * uin[k - 1];
                acc += st.n * uin[k + 1];
                const float rf = (float)(bb[k] - acc);
                F.r[k] = rf;
                lres32 = fmaxf(lres32, fabsf(rf * st32[4 * i + 3]));
            }
            lres = lres32;
            lumax = __hiloint2double((int)lumax_hi, 0);
            lres = block_max(lres);
            lumax = block_max(lumax);
            if (t.nblocks > 1) {
                const int slot = (n64 & 1) * 2;
                if (threadIdx.x == 0) {
                    atomic_max_nonneg(&a.red[slot], lres);
                    atomic_max_nonneg(&a.red[slot + 1], lumax);
                }
                ok = t.sync();
                if (!ok) break;
                lres = *((volatile double*)&a.red[slot]);
                lumax = *((volatile double*)&a.red[slot + 1]);
                if (t.tid == 0) {
                    a.red[2 - slot] = 0.0;
                    a.red[3 - slot] = 0.0;
                }
            }
            ++n64;
        }
        t.mark(kPhaseResidual);
        // relative to max|u|; a cold start from u = 0 (a homogeneous solve)
        // measures against its own initial residual instead
        if (it == 0) ref0 = lres;
        const double uref = lumax > 0.0 ? lumax : ref0;
        res = uref > 0.0 ? lres / uref : lres;
        if (res <= a.tol || lres == 0.0) {
            if (!updated) {
                conv = true;
                break;
            }
            updated = false;  // confirm with the FP64 residual
            continue;
        }
        if (cycles >= a.max_outer) break;
        if (tiled) {
            // the barrier of the reduction above (or of the last up phase)
            // already ordered F.r; the fine level's up phase adds the
            // correction to u and leaves the next residual
            vcycle_tiled(a, t, ok, 4 + (cycles & 1) * 2);
            ++cycles;
            updated = true;
            continue;
        }
        ok = t.sync();
        if (!ok) break;
        vcycle(a, t, ok);
        if (!ok) break;
        for (unsigned k = t.tid; k < nn; k += t.nthreads)
            if (!is_fixed(a.mask[k])) a.u[k] += (double)F.e[k];
        ok = t.sync();
        ++cycles;
        t.mark(kPhaseUp);
    }
    // 3. face electric field E = -grad u for the particle kernel
    if (ok && a.Exf != nullptr) faces_pass(a.u, nx, nz, a.idx, a.idz, a.Exf, a.Ezf, t.tid, t.nthreads);
    t.mark(kPhaseFaces);
    if (a.prof && blockIdx.x == 0 && threadIdx.x == 0) a.prof[kPhaseTotal] += (double)(Team::now() - t_start);
    solve_report(a, t, cycles, res, conv, ok);
}

__global__ void __launch_bounds__(1024) k_solve(const __grid_constant__ SolveArgs a)
{
    Team t(a.bar);
    solve_body(a, t);
}

// Independent solves, one per block (batched instances): the block copies its
// arguments to shared memory and runs the single-block solve.
__global__ void __launch_bounds__(1024) k_solve_batch(const SolveArgs* __restrict__ args)
{
    __shared__ __align__(16) unsigned char raw[sizeof(SolveArgs)];
    static_assert(sizeof(SolveArgs) % 8 == 0, "word copy");
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(args + blockIdx.x);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(raw);
    for (int w = threadIdx.x; w < (int)(sizeof(SolveArgs) / 8); w += blockDim.x) dst[w] = src[w];
    __syncthreads();
    Team t = Team::block(nullptr);
    solve_body(*reinterpret_cast<const SolveArgs*>(raw), t);
}

// ---- FP64 multigrid (the all-FP64 solver option) ---------------------------
//
// The same V-cycle as the single-block FP32 path (red-black Gauss-Seidel on
// the fine level, 4-colour Gauss-Seidel on the Galerkin levels, bilinear
// transfers, dense coarsest inverse) with every level in FP64, iterated on the
// FP64 residual to the same stopping rule.  It is what the FP32 multigrid with
// FP64 refinement replaces, kept as a solver option so that the two can be
// timed against each other at the same tolerance.  One block per solve: grids
// up to kSingleBlockNodes nodes.

__device__ void smooth_fine64(const SolveArgs& a, const MG64Args& g, Team& t, int sweeps, bool reverse, double omega)
{
    const MG64Level& L = g.lev[0];
    const int nx = L.nx, nz = L.nz, hz = (nz + 1) / 2;
    double* __restrict__ e = L.e;
    const double* __restrict__ r = L.r;
    const double k2 = a.k2;
    const unsigned n = (unsigned)(nx * hz);
    const FastDiv dh((unsigned)hz);
    for (int s = 0; s < sweeps; ++s)
        for (int cc = 0; cc < 2; ++cc) {
            const int color = reverse ? 1 - cc : cc;
            for (unsigned q = t.tid; q < n; q += t.nthreads) {
                const int i = (int)dh.div(q);
                const int j = 2 * (int)(q - (unsigned)i * hz) + ((i + color) & 1);
                if (j >= nz) continue;
                const size_t k = (size_t)i * nz + j;
                if (is_fixed(a.mask[k])) continue;
                const double* st = a.st64 + 4 * i;
                double acc = r[k] - st[1] * e[k + nz] - k2 * (e[k - 1] + e[k + 1]);
                if (i > 0) acc -= st[0] * e[k - nz];
                const double enew = acc * st[3];
                e[k] = omega == 1.0 ? enew : e[k] + omega * (enew - e[k]);
            }
            __syncthreads();
        }
}

__device__ __forceinline__ double coarse_apply64(const double* __restrict__ coef, int nx, int nz, int i, int j, size_t k,
                                                 const double* __restrict__ e, bool skip_center)
{
    const size_t n = (size_t)nx * nz;
    double acc = 0.0;
#pragma unroll
    for (int di = -1; di <= 1; ++di) {
        if (i + di < 0 || i + di >= nx) continue;
#pragma unroll
        for (int dj = -1; dj <= 1; ++dj) {
            if (j + dj < 0 || j + dj >= nz) continue;
            if (skip_center && di == 0 && dj == 0) continue;
            acc += coef[((di + 1) * 3 + (dj + 1)) * n + k] * e[k + (ptrdiff_t)di * nz + dj];
        }
    }
    return acc;
}

__device__ void smooth_coarse64(const MG64Level& L, Team& t, int sweeps, bool reverse)
{
    const int nx = L.nx, nz = L.nz, hx = (nx + 1) / 2, hz = (nz + 1) / 2;
    const unsigned n = (unsigned)(hx * hz);
    const FastDiv dh((unsigned)hz);
    for (int s = 0; s < sweeps; ++s)
        for (int cc = 0; cc < 4; ++cc) {
            const int color = reverse ? 3 - cc : cc;
            const int ci = color >> 1, cj = color & 1;
            for (unsigned q = t.tid; q < n; q += t.nthreads) {
                const unsigned qi = dh.div(q);
                const int i = 2 * (int)qi + ci, j = 2 * (int)(q - qi * hz) + cj;
                if (i >= nx || j >= nz) continue;
                const size_t k = (size_t)i * nz + j;
                L.e[k] = (L.r[k] - coarse_apply64(L.coef, nx, nz, i, j, k, L.e, true)) * L.inv_diag[k];
            }
            __syncthreads();
        }
}

// t = r - A e on level l (fine level: free nodes only)
__device__ void residual64(const SolveArgs& a, const MG64Args& g, Team& t, int l)
{
    const MG64Level& L = g.lev[l];
    const int nx = L.nx, nz = L.nz;
    const unsigned n = (unsigned)(nx * nz);
    const FastDiv dz((unsigned)nz);
    for (unsigned q = t.tid; q < n; q += t.nthreads) {
        const int i = (int)dz.div(q);
        if (l == 0) {
            if (is_fixed(a.mask[q])) {
                L.t[q] = 0.0;
                continue;
            }
            const double* st = a.st64 + 4 * i;
            double acc = L.r[q] - st[2] * L.e[q] - st[1] * L.e[q + nz] - a.k2 * (L.e[q - 1] + L.e[q + 1]);
            if (i > 0) acc -= st[0] * L.e[q - nz];
            L.t[q] = acc;
        } else {
            L.t[q] = L.r[q] - coarse_apply64(L.coef, nx, nz, i, (int)(q - (unsigned)i * nz), q, L.e, false);
        }
    }
    __syncthreads();
}

__device__ void restrict64(const MG64Args& g, Team& t, int l)
{
    const MG64Level& F = g.lev[l];
    const MG64Level& C = g.lev[l + 1];
    const unsigned n = (unsigned)(C.nx * C.nz);
    const FastDiv dz((unsigned)C.nz);
    auto get = [&](int i, int j) { return F.t[(size_t)i * F.nz + j]; };
    for (unsigned q = t.tid; q < n; q += t.nthreads) {
        const int I = (int)dz.div(q), J = (int)(q - (unsigned)I * C.nz);
        C.r[q] = restrict_node(I, J, F.cmode, F.nx, F.nz, get);
        C.e[q] = 0.0;
    }
    __syncthreads();
}

__device__ void prolong64(const SolveArgs& a, const MG64Args& g, Team& t, int l)
{
    const MG64Level& F = g.lev[l];
    const MG64Level& C = g.lev[l + 1];
    const unsigned n = (unsigned)(F.nx * F.nz);
    const FastDiv dz((unsigned)F.nz);
    for (unsigned q = t.tid; q < n; q += t.nthreads) {
        if (l == 0 && is_fixed(a.mask[q])) continue;
        const int i = (int)dz.div(q), j = (int)(q - (unsigned)i * F.nz);
        F.e[q] += prolong_node(i, j, F.cmode, (const double*)C.e, C.nz);
    }
    __syncthreads();
}

__device__ void vcycle64(const SolveArgs& a, const MG64Args& g, Team& t)
{
    const int L = a.nlev;
    if (L == 1) {
        smooth_fine64(a, g, t, a.ncoarse, false, (double)a.omega);
        return;
    }
    for (int l = 0; l < L - 1; ++l) {
        if (l == 0) smooth_fine64(a, g, t, a.nu1, false, 1.0);
        else smooth_coarse64(g.lev[l], t, a.nu1, false);
        residual64(a, g, t, l);
        restrict64(g, t, l);
    }
    const MG64Level& Lc = g.lev[L - 1];
    if (g.coarse_inv) {
        const unsigned n = (unsigned)(Lc.nx * Lc.nz);
        for (unsigned row = t.tid; row < n; row += t.nthreads) {
            double acc = 0.0;
            for (unsigned c = 0; c < n; ++c) acc += g.coarse_inv[(size_t)c * n + row] * Lc.r[c];
            Lc.e[row] = acc;
        }
        __syncthreads();
    } else {
        smooth_coarse64(Lc, t, a.ncoarse, false);
    }
    for (int l = L - 2; l >= 0; --l) {
        prolong64(a, g, t, l);
        if (l == 0) smooth_fine64(a, g, t, a.nu2, true, 1.0);
        else smooth_coarse64(g.lev[l], t, a.nu2, true);
    }
}

__global__ void __launch_bounds__(1024) k_solve64(const __grid_constant__ SolveArgs a, const __grid_constant__ MG64Args g)
{
    Team t = Team::block(nullptr);
    bool ok = true;
    solve_prologue(a, t, ok);
    const int nz = a.nz;
    const unsigned nn = (unsigned)(a.nx * nz);
    const FastDiv dnz((unsigned)nz);
    const MG64Level& F = g.lev[0];
    int it = 0;
    double res = 0.0, ref0 = 0.0;
    bool conv = false;
    for (;; ++it) {
        // r = b - A u in FP64 and its Jacobi-scaled max norm against max|u|
        double lres = 0.0, lumax = 0.0;
        for (unsigned k = t.tid; k < nn; k += t.nthreads) {
            const int i = (int)dnz.div(k);
            const double uk = a.u[k];
            lumax = fmax(lumax, fabs(uk));
            F.e[k] = 0.0;
            if (is_fixed(a.mask[k])) {
                F.r[k] = 0.0;
                continue;
            }
            const Stencil5 st = fine_stencil(a, i);
            double acc = st.c * uk + st.e * a.u[k + nz] + st.s * a.u[k - 1] + st.n * a.u[k + 1];
            if (i > 0) acc += st.w * a.u[k - nz];
            const double rk = a.b[k] - acc;
            F.r[k] = rk;
            lres = fmax(lres, fabs(rk * st.inv_c));
        }
        lres = block_max(lres);
        lumax = block_max(lumax);
        if (it == 0) ref0 = lres;
        const double uref = lumax > 0.0 ? lumax : ref0;
        res = uref > 0.0 ? lres / uref : lres;
        if (res <= a.tol || lres == 0.0) {
            conv = true;
            break;
        }
        if (it >= a.max_outer) break;
        vcycle64(a, g, t);
        for (unsigned k = t.tid; k < nn; k += t.nthreads)
            if (!is_fixed(a.mask[k])) a.u[k] += F.e[k];
        __syncthreads();
    }
    if (a.Exf != nullptr) faces_pass(a.u, a.nx, a.nz, a.idx, a.idz, a.Exf, a.Ezf, t.tid, t.nthreads);
    solve_report(a, t, it, res, conv, ok);
}

// ---- direct solve with the precomputed inverse ----------------------------
//
// For grids small enough to keep G = A_ff^-1 in HBM (column j = the solution
// for a unit right-hand side at node j, zero Dirichlet values), a solve is
//   u_f = u_vac,f + sum over j with b'_j != 0 of G[:, j] b'_j
//   u_d = the Dirichlet values
// where b' = scale_i rho on free nodes and u_vac = G (- sum over fixed
// neighbours d of A[f][d] u_d) is the potential of the electrodes alone,
// computed once (the voltages of an instance do not change).  Without a
// stored u_vac (other Dirichlet values, e.g. the zero ones of the adjoint
// solve) b' carries the Dirichlet term itself.
//
// The nonzero entries of b' are compacted in node order into a list; the
// product is split into chunks of equal numbers of list entries whose partial
// sums are added in chunk order, so the result does not depend on scheduling
// and the work does not depend on where the charge sits.

constexpr int kGreenTile = 1024;  // nodes per block of the right-hand side and its compaction
constexpr int kGemvLoads = 8;     // independent column loads in flight per thread of the product

__device__ __forceinline__ double green_rhs_node(const SolveArgs& a, long long k, bool dirichlet)
{
    const int nx = a.nx, nz = a.nz;
    const int8_t m = a.mask[k];
    auto value = [&](long long d) {
        const int8_t md = a.mask[d];
        return a.rf_solve ? (md == 1 ? a.voltage[d] : 0.0) : (md == 0 ? a.voltage[d] : 0.0);
    };
    double b = 0.0;
    if (is_fixed(m)) {
        a.u[k] = value(k);
    } else {
        const int i = (int)(k / nz), j = (int)(k - (long long)i * nz);
        double rho = 0.0;
        if (a.rho_src == 1) {
            for (int s = 0; s < a.nsp; ++s) rho += a.rho_weight[s] * (double)a.rho_fixed[s][k];
        } else if (a.rho_src == 2) {
            rho = a.rho64[k];
        }
        b = rho * rhs_scale(a, i);
        if (dirichlet) {
            const Stencil5 st = fine_stencil(a, i);
            if (i > 0 && is_fixed(a.mask[k - nz])) b -= st.w * value(k - nz);
            if (i + 1 < nx && is_fixed(a.mask[k + nz])) b -= st.e * value(k + nz);
            if (j > 0 && is_fixed(a.mask[k - 1])) b -= st.s * value(k - 1);
            if (j + 1 < nz && is_fixed(a.mask[k + 1])) b -= st.n * value(k + 1);
        }
    }
    if (a.clear_rho && a.rho_src == 1)
        for (int s = 0; s < a.nsp; ++s) ((unsigned long long*)a.rho_fixed[s])[k] = 0ull;
    return b;
}

// b' of every node (one node per thread); block t compacts the nonzero
// entries of its tile of kGreenTile nodes, in node order, to list slots
// [t kGreenTile, t kGreenTile + tile_count[t]).
__global__ void __launch_bounds__(kGreenTile) k_green_rhs(const SolveArgs a, bool dirichlet, int* __restrict__ list_j,
                                                          double* __restrict__ list_b, int* __restrict__ tile_count,
                                                          uint8_t* __restrict__ charged)
{
    asm volatile("griddepcontrol.wait;" ::: "memory");  // the previous kernel's results (launched with PDL)
    asm volatile("griddepcontrol.launch_dependents;");
    __shared__ int wcount[kGreenTile / 32];
    const long long nn = (long long)a.nx * a.nz;
    const long long k = (long long)blockIdx.x * kGreenTile + threadIdx.x;
    const double b = k < nn ? green_rhs_node(a, k, dirichlet) : 0.0;
    if (charged && k < nn) charged[k] = b != 0.0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned m = __ballot_sync(0xffffffffu, b != 0.0);
    if (lane == 0) wcount[warp] = __popc(m);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < kGreenTile / 32; ++w) {
        const int c = wcount[w];
        before += w < warp ? c : 0;
        total += c;
    }
    if (b != 0.0) {
        const long long pos = (long long)blockIdx.x * kGreenTile + before + __popc(m & ((1u << lane) - 1u));
        list_j[pos] = (int)k;
        list_b[pos] = b;
    }
    if (threadIdx.x == 0) tile_count[blockIdx.x] = total;
}

// part[c][i] = sum over the list entries q of chunk c of G[j_q][i] b_q, in
// list order; the list is the tiles' entries one after the other (L in all),
// chunk c of nchunks holds entries [c L / nchunks, (c+1) L / nchunks).
// position q of a list stored tile by tile (tile t's entries at t kGreenTile,
// start[] the first position of every tile)
__device__ __forceinline__ long long tile_slot(const int* start, int ntiles, int q)
{
    int lo = 0, hi = ntiles - 1;  // last tile whose first entry is <= q
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= q) lo = mid;
        else hi = mid - 1;
    }
    return (long long)lo * kGreenTile + (q - start[lo]);
}

__device__ __forceinline__ void tile_starts(const int* __restrict__ count, int ntiles, int* start)
{
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int t = 0; t < ntiles; ++t) {
            start[t] = acc;
            acc += count[t];
        }
        start[ntiles] = acc;
    }
}

// rows: null for every node, else the nodes to compute (tile layout, counts
// in row_count); part is indexed by the row's position in that list
__global__ void __launch_bounds__(256) k_green_gemv(const double* __restrict__ G, const int* __restrict__ list_j,
                                                    const double* __restrict__ list_b,
                                                    const int* __restrict__ tile_count, int ntiles, long long nn,
                                                    const int* __restrict__ rows, const int* __restrict__ row_count,
                                                    double* __restrict__ part)
{
    asm volatile("griddepcontrol.wait;" ::: "memory");  // the previous kernel's results (launched with PDL)
    asm volatile("griddepcontrol.launch_dependents;");
    __shared__ double sb[256];
    __shared__ int sj[256];
    __shared__ int start[kGreenMaxTiles + 1], rstart[kGreenMaxTiles + 1];
    tile_starts(tile_count, ntiles, start);
    if (rows) tile_starts(row_count, ntiles, rstart);
    __syncthreads();
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long R = rows ? rstart[ntiles] : nn;
    if ((long long)blockIdx.x * blockDim.x >= R) return;  // uniform per block
    const bool row = r < R;
    const long long i = !row ? 0 : rows ? rows[tile_slot(rstart, ntiles, (int)r)] : r;
    const long long L = start[ntiles], nch = gridDim.y;
    const long long q0 = L * blockIdx.y / nch, q1 = L * (blockIdx.y + 1) / nch;
    const double* __restrict__ gi = G + i;
    double acc = 0.0;
    for (long long t0 = q0; t0 < q1; t0 += 256) {
        const int total = (int)min(256LL, q1 - t0);
        if (threadIdx.x < total) {
            const long long slot = tile_slot(start, ntiles, (int)(t0 + threadIdx.x));
            sj[threadIdx.x] = list_j[slot];
            sb[threadIdx.x] = list_b[slot];
        }
        __syncthreads();
        if (row) {
            int q = 0;
            for (; q + kGemvLoads <= total; q += kGemvLoads) {
                double g[kGemvLoads];
#pragma unroll
                for (int r = 0; r < kGemvLoads; ++r) g[r] = __ldcs(gi + (long long)sj[q + r] * nn);
#pragma unroll
                for (int r = 0; r < kGemvLoads; ++r) acc = fma(g[r], sb[q + r], acc);
            }
            for (; q < total; ++q) acc = fma(__ldcs(gi + (long long)sj[q] * nn), sb[q], acc);
        }
        __syncthreads();
    }
    if (row) part[(long long)blockIdx.y * nn + r] = acc;
}

// the nodes a particle kernel reads the potential of: every free node within
// two nodes (in i and j) of a node with charge, tile by tile in node order
__global__ void __launch_bounds__(kGreenTile) k_green_rows(int nx, int nz, const int8_t* __restrict__ mask,
                                                           const uint8_t* __restrict__ charged,
                                                           int* __restrict__ rows, int* __restrict__ row_count)
{
    asm volatile("griddepcontrol.wait;" ::: "memory");  // the previous kernel's results (launched with PDL)
    asm volatile("griddepcontrol.launch_dependents;");
    __shared__ int wcount[kGreenTile / 32];
    const long long nn = (long long)nx * nz;
    const long long k = (long long)blockIdx.x * kGreenTile + threadIdx.x;
    bool need = false;
    if (k < nn && !is_fixed(mask[k])) {
        const int i = (int)(k / nz), j = (int)(k - (long long)i * nz);
        for (int di = -2; di <= 2 && !need; ++di) {
            const int ii = i + di;
            if (ii < 0 || ii >= nx) continue;
            for (int dj = -2; dj <= 2; ++dj) {
                const int jj = j + dj;
                if (jj >= 0 && jj < nz && charged[(long long)ii * nz + jj]) {
                    need = true;
                    break;
                }
            }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (lane == 0) wcount[warp] = __popc(m);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < kGreenTile / 32; ++w) {
        const int c = wcount[w];
        before += w < warp ? c : 0;
        total += c;
    }
    if (need) rows[(long long)blockIdx.x * kGreenTile + before + __popc(m & ((1u << lane) - 1u))] = (int)k;
    if (threadIdx.x == 0) row_count[blockIdx.x] = total;
}

__global__ void __launch_bounds__(64) k_green_sum(const SolveArgs a, const double* __restrict__ part, int nchunks,
                                                  const double* __restrict__ u_vac, const int* __restrict__ rows,
                                                  const int* __restrict__ row_count, int ntiles)
{
    asm volatile("griddepcontrol.wait;" ::: "memory");  // the previous kernel's results (launched with PDL)
    asm volatile("griddepcontrol.launch_dependents;");
    __shared__ int rstart[kGreenMaxTiles + 1];
    const long long nn = (long long)a.nx * a.nz;
    if (rows) tile_starts(row_count, ntiles, rstart);
    __syncthreads();
    const long long R = rows ? rstart[ntiles] : nn;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < R; r += (long long)gridDim.x * blockDim.x) {
        const long long k = rows ? rows[tile_slot(rstart, ntiles, (int)r)] : r;
        if (is_fixed(a.mask[k])) continue;
        double p[kGreenMaxChunks];
#pragma unroll
        for (int c = 0; c < kGreenMaxChunks; ++c) p[c] = c < nchunks ? part[(long long)c * nn + r] : 0.0;
        double u = u_vac ? u_vac[k] : 0.0;
#pragma unroll
        for (int c = 0; c < kGreenMaxChunks; ++c)
            if (c < nchunks) u += p[c];
        a.u[k] = u;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.status->iterations = 0;
        a.status->residual = 0.0;
        a.status->converged = 1;
        a.status->aborted = 0;
    }
}

__global__ void k_faces(const double* __restrict__ u, int nx, int nz, double idx, double idz, float* Exf, float* Ezf)
{
    asm volatile("griddepcontrol.wait;" ::: "memory");  // the previous kernel's results (launched with PDL)
    asm volatile("griddepcontrol.launch_dependents;");
    faces_pass(u, nx, nz, idx, idz, Exf, Ezf, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

}  // namespace

// allow smem bytes of dynamic shared memory for k_solve (false when refused)
bool solve_allow_smem(size_t smem)
{
    static size_t allowed = 0;
    if (smem <= allowed) return true;
    if (cudaFuncSetAttribute(k_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    allowed = smem;
    return true;
}

int solve_max_blocks(int sm_count, size_t smem)
{
    int per_sm = 0, coop = 0, dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return 1;
    if (smem && !solve_allow_smem(smem)) return 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve, 1024, smem) != cudaSuccess || per_sm < 1)
        return 1;
    return per_sm * sm_count;
}

int launch_solve(const SolveArgs& a, int nblocks, cudaStream_t s, size_t smem)
{
    if (nblocks <= 1) {
        k_solve<<<1, 1024, 0, s>>>(a);
    } else {
        if (smem) solve_allow_smem(smem);
        void* args[] = {(void*)&a};
        cudaLaunchCooperativeKernel((const void*)k_solve, dim3(nblocks), dim3(1024), args, smem, s);
    }
    return 1;
}

int launch_solve64(const SolveArgs& a, const MG64Args& g, cudaStream_t s)
{
    k_solve64<<<1, 1024, 0, s>>>(a, g);
    return 1;
}

int launch_solve_batch(const SolveArgs* d_args, int n, int threads, cudaStream_t s)
{
    if (n <= 0) return 0;
    k_solve_batch<<<n, threads, 0, s>>>(d_args);
    return 1;
}

int green_chunks(long long nn, int sm_count)
{
    const long long rows = (nn + 255) / 256;
    return (int)std::max<long long>(1, std::min<long long>(kGreenMaxChunks, (8LL * sm_count + rows - 1) / rows));
}

// A launch with programmatic stream serialisation: the kernel may be scheduled
// while the previous one on the stream finishes, and waits for it
// (griddepcontrol.wait) before it reads anything that one wrote.
template <class... KArgs, class... Args>
void pdl_launch(void (*k)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, args...);
}

int launch_green_solve(const SolveArgs& a, const GreenArgs& g, cudaStream_t s)
{
    const long long nn = (long long)a.nx * a.nz;
    const int ntiles = (int)((nn + kGreenTile - 1) / kGreenTile);
    const bool partial = g.rows != nullptr;
    pdl_launch(k_green_rhs, dim3(ntiles), dim3(kGreenTile), s, a, g.u_vac == nullptr, g.list_j, g.list_b,
               g.tile_count, partial ? g.charged : (uint8_t*)nullptr);
    int n = 1;
    if (partial) {
        pdl_launch(k_green_rows, dim3(ntiles), dim3(kGreenTile), s, a.nx, a.nz, a.mask, (const uint8_t*)g.charged,
                   g.rows, g.row_count);
        ++n;
    }
    n += launch_green_product(a, g, partial, s);
    if (a.Exf) {
        const long long nf = (long long)(a.nx + 1) * a.nz + (long long)a.nx * (a.nz + 1);
        pdl_launch(k_faces, dim3((unsigned)std::min<long long>((nf + 255) / 256, 152 * 8)), dim3(256), s,
                   (const double*)a.u, a.nx, a.nz, a.idx, a.idz, a.Exf, a.Ezf);
        ++n;
    }
    return n;
}

int launch_green_product(const SolveArgs& a, const GreenArgs& g, bool partial, cudaStream_t s)
{
    const long long nn = (long long)a.nx * a.nz;
    const int ntiles = (int)((nn + kGreenTile - 1) / kGreenTile);
    const int* rows = partial ? g.rows : nullptr;
    pdl_launch(k_green_gemv, dim3((unsigned)((nn + 255) / 256), (unsigned)g.nchunks), dim3(256), s, g.G,
               (const int*)g.list_j, (const double*)g.list_b, (const int*)g.tile_count, ntiles, nn, rows,
               (const int*)g.row_count, g.part);
    const unsigned g1 = (unsigned)std::min<long long>((nn + 63) / 64, 152 * 16);
    pdl_launch(k_green_sum, dim3(g1), dim3(64), s, a, (const double*)g.part, g.nchunks, g.u_vac, rows,
               (const int*)g.row_count, ntiles);
    return 2;
}

// Fields::u_smooth (fields.cpp:28-111) with its default arguments, on the
// copy t of u: rows 1..nx-2, columns 1..nz-1 take the 3x3 weights 1, 1/2
// (edges), 1/4 (corners), added in the reference's order and divided by 4;
// every other node keeps its value.  The reference addresses neighbours on
// one contiguous row-major array, so column nz is column 0 of the next row;
// the one neighbour past the array (row nx-2, column nz-1, its +1/+1
// neighbour) is taken as 0.  Products by 1/2 and 1/4 are exact, so the
// explicit round-to-nearest adds reproduce the reference bit for bit.
__global__ void k_u_smooth(const double* __restrict__ t, double* __restrict__ u, int nx, int nz)
{
    const long long n = (long long)nx * nz;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x; f < n; f += stride) {
        const int i = (int)(f / nz);
        const int j = (int)(f - (long long)i * nz);
        if (i < 1 || i > nx - 2 || j < 1) continue;
        const double last = f + nz + 1 < n ? t[f + nz + 1] : 0.0;
        double sum = __dadd_rn(t[f], __dmul_rn(t[f - nz], 0.5));
        sum = __dadd_rn(sum, __dmul_rn(t[f + nz], 0.5));
        sum = __dadd_rn(sum, __dmul_rn(t[f - 1], 0.5));
        sum = __dadd_rn(sum, __dmul_rn(t[f + 1], 0.5));
        sum = __dadd_rn(sum, __dmul_rn(t[f - nz - 1], 0.25));
        sum = __dadd_rn(sum, __dmul_rn(t[f + nz - 1], 0.25));
        sum = __dadd_rn(sum, __dmul_rn(t[f - nz + 1], 0.25));
        sum = __dadd_rn(sum, __dmul_rn(last, 0.25));
        u[f] = __dmul_rn(sum, 0.25);
    }
}

int launch_u_smooth(const double* t, double* u, int nx, int nz, cudaStream_t s)
{
    const long long n = (long long)nx * nz;
    const int grid = (int)std::min<long long>((n + 255) / 256, 152 * 8);
    k_u_smooth<<<grid, 256, 0, s>>>(t, u, nx, nz);
    return 1;
}

int launch_faces(const double* u, int nx, int nz, double dx, double dz, float* Exf, float* Ezf, cudaStream_t s)
{
    const long long n = (long long)(nx + 1) * nz + (long long)nx * (nz + 1);
    const int grid = (int)std::min<long long>((n + 255) / 256, 152 * 8);
    k_faces<<<grid, 256, 0, s>>>(u, nx, nz, 1.0 / dx, 1.0 / dz, Exf, Ezf);
    return 1;
}

}  // namespace mag
