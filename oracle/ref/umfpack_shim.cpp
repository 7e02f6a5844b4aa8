// Banded-LU stand-in for the UMFPACK calls of the reference (oracle build only).
// See shim/suitesparse/umfpack.h for what is solved and why.
#include "suitesparse/umfpack.h"

#include <cstdlib>
#include <vector>

namespace {

struct Symbolic { int n; int bw; };

struct Numeric {
    int n, bw;                 // order and half bandwidth
    std::vector<double> band;  // row-major band: row r, column c -> band[r*(2bw+1) + (c-r+bw)]
    double& at(int r, int c) { return band[(size_t)r * (2 * bw + 1) + (c - r + bw)]; }
};

}  // namespace

extern "C" int umfpack_di_symbolic(int n_row, int n_col, const int* Ap, const int* Ai,
                                   const double*, void** Sym, const double*, double*)
{
    if (n_row != n_col) return UMFPACK_ERROR_invalid_system;
    Symbolic* s = new Symbolic;
    s->n = n_row;
    s->bw = 0;
    // Column k of the CSC arrays holds row k of S (filled row by row).
    for (int k = 0; k < n_col; ++k)
        for (int l = Ap[k]; l < Ap[k + 1]; ++l) {
            int d = std::abs(Ai[l] - k);
            if (d > s->bw) s->bw = d;
        }
    *Sym = s;
    return UMFPACK_OK;
}

extern "C" int umfpack_di_numeric(const int* Ap, const int* Ai, const double* Ax,
                                  void* Sym, void** Num, const double*, double*)
{
    const Symbolic* s = static_cast<const Symbolic*>(Sym);
    Numeric* f = new Numeric;
    f->n = s->n;
    f->bw = s->bw;
    f->band.assign((size_t)f->n * (2 * f->bw + 1), 0.0);
    for (int k = 0; k < f->n; ++k)
        for (int l = Ap[k]; l < Ap[k + 1]; ++l)
            f->at(k, Ai[l]) += Ax[l];
    // Doolittle elimination inside the band, no pivoting.
    const int n = f->n, bw = f->bw;
    for (int k = 0; k < n; ++k) {
        const double piv = f->at(k, k);
        const int rmax = k + bw < n - 1 ? k + bw : n - 1;
        for (int r = k + 1; r <= rmax; ++r) {
            double& lrk = f->at(r, k);
            if (lrk == 0.0) continue;
            lrk /= piv;
            const double m = lrk;
            for (int c = k + 1; c <= rmax; ++c) f->at(r, c) -= m * f->at(k, c);
        }
    }
    *Num = f;
    return UMFPACK_OK;
}

extern "C" int umfpack_di_solve(int sys, const int*, const int*, const double*,
                                double* X, const double* B, void* Num, const double*, double*)
{
    if (sys != UMFPACK_At) return UMFPACK_ERROR_invalid_system;
    Numeric* f = static_cast<Numeric*>(Num);
    const int n = f->n, bw = f->bw;
    std::vector<double> y(B, B + n);
    for (int r = 0; r < n; ++r) {
        const int c0 = r - bw > 0 ? r - bw : 0;
        double acc = y[r];
        for (int c = c0; c < r; ++c) acc -= f->at(r, c) * y[c];
        y[r] = acc;
    }
    for (int r = n - 1; r >= 0; --r) {
        const int c1 = r + bw < n - 1 ? r + bw : n - 1;
        double acc = y[r];
        for (int c = r + 1; c <= c1; ++c) acc -= f->at(r, c) * X[c];
        X[r] = acc / f->at(r, r);
    }
    return UMFPACK_OK;
}

extern "C" void umfpack_di_free_symbolic(void** Sym)
{
    delete static_cast<Symbolic*>(*Sym);
    *Sym = 0;
}

extern "C" void umfpack_di_free_numeric(void** Num)
{
    delete static_cast<Numeric*>(*Num);
    *Num = 0;
}
