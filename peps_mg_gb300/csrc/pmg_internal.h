// pmg_internal.h -- host-side declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "pmg_common.cuh"

namespace pmg {

constexpr int kMaxLevels = 24;

// Launch geometry of a level: grid-stride loops in every kernel let an axis be
// collapsed to one CTA column (the CGPSA step-down mapping).
struct Launch {
    bool collapse[3];   // one CTA spans the whole axis
};

// Single-CTA persistent coarse tail (levels l0..nl): the CGA mapping, and the
// coarsest-level solve of every method.
template <typename T>
struct TailDesc {
    int l0, nl;
    int maxit;
    int coarse_solver;
    int coarse_maxit;
    T omega, omw;
    double tol;
    T *p, *ap, *rr;               // coarsest-level CG / residual scratch (full arrays)
    int *iters_out;               // device: iterations of the coarsest solver
    LevelK<T> L[kMaxLevels];
    XferK<T> X[kMaxLevels];       // X[l]: transfer between l and l+1
    T *x[kMaxLevels], *b[kMaxLevels], *r[kMaxLevels];
};

// ---- FP64 (bitwise) launchers, pmg_f64.cu -------------------------------------
int f64_rbgs_sweeps(const LevelK<double> &L, const Launch &ln, double *x, const double *b, int iters,
                    double omega, cudaStream_t s);
// r = b - A x (interior); if partials != nullptr also writes per-block sums of r^2
// and returns the number of partials in *npart.
int f64_residual(const LevelK<double> &L, const Launch &ln, double *r, const double *x, const double *b,
                 double *partials, int *npart, cudaStream_t s);
int f64_mv_mul(const LevelK<double> &L, const Launch &ln, double *y, const double *x, cudaStream_t s);
int f64_dot_partials(const LevelK<double> &L, const Launch &ln, const double *x, const double *y,
                     double *partials, int *npart, cudaStream_t s);
// Sum partials[0..n) in a fixed order into *out (device).
int f64_reduce(const double *partials, int n, double *out, cudaStream_t s);
int f64_restrict(const XferK<double> &X, const Launch &ln, const double *vf, double *vc, cudaStream_t s);
int f64_prolong(const XferK<double> &X, const Launch &ln, const double *vc, double *vf, bool add,
                cudaStream_t s);
int zero_ghosts_f64(double *a, int nx, int ny, int nz, cudaStream_t s);
int f64_tail(const TailDesc<double> *dev_desc, cudaStream_t s);
// CG building blocks on device scalars (src/cg_poisson_matrix.f90:99-138)
int f64_copy_interior(const LevelK<double> &L, double *dst, const double *src, cudaStream_t s);
int f64_cg_scalar(const double *num, const double *den, double *out, cudaStream_t s);
int f64_cg_update_xr(const LevelK<double> &L, const Launch &ln, const double *alpha, double *x, double *r,
                     const double *p, const double *ap, cudaStream_t s);
int f64_cg_update_p(const LevelK<double> &L, const Launch &ln, const double *beta, double *p, const double *r,
                    cudaStream_t s);
// Convergence flag for device-looped solvers: flag = (sqrt(num/den) <= tol) (le=1) or
// < tol (le=0); also records the iteration.
int f64_check(const double *num, const double *den, double tol, int le, int iter, int *flag, int *iter_out,
              cudaStream_t s);

// Fixed launch shapes (shared with the host driver for partial-sum sizing).
void grid_for_cells(const LevelK<double> &L, const Launch &ln, dim3 *grid, dim3 *block);

// ---- errors ---------------------------------------------------------------------
void set_error(const std::string &msg);
int cuda_status(cudaError_t e, const char *what);

}  // namespace pmg
