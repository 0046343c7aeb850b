// pmg_tail64.cuh -- block-level (single-CTA) FP64 building blocks of the persistent
// coarse tail and the coarsest-level solvers.  Every floating-point operation is an
// explicit round-to-nearest intrinsic, so the results are the reference's non-FMA
// arithmetic whatever the translation unit's --fmad setting.  All threads of the block
// must call each function; phases end with __syncthreads().
#pragma once

#include "pmg_common.cuh"

namespace pmg {
namespace {

__device__ void tail_zero(double *a, long long n)
{
    for (long long q = threadIdx.x; q < n; q += blockDim.x) a[q] = 0.0;
}

__device__ void tail_rbgs(const LevelK<double> &L, double *x, const double *b, int iters, double omega, double omw)
{
    const int hx = (L.nx + 1) / 2;
    const long long nq = (long long)hx * L.ny * L.nz;
    for (int it = 0; it < iters; ++it)
        for (int colour = 0; colour < 2; ++colour) {
            for (long long q = threadIdx.x; q < nq; q += blockDim.x) {
                const int t = (int)(q % hx);
                const long long rr = q / hx;
                const int j = (int)(rr % L.ny) + 1, k = (int)(rr / L.ny) + 1;
                const int i = 2 * t + 1 + ((j + k + colour) & 1);
                if (i <= L.nx) x[lin(i, j, k, L.sy, L.sz)] = rbgs_cell_f64(L, x, b, i, j, k, omega, omw);
            }
            __syncthreads();
        }
}

// r = b - A x; returns sum(r^2) over the block (fixed order) when NORM.
// Sum of x*y over the interior in an order fixed by the level alone: 64 lanes (threads
// 0..63, blocks have at least 64 threads) each accumulate the cells q = lane (mod 64) in
// increasing q, then the lanes are combined by a fixed tree.  The result therefore does
// not depend on the block size the tail runs with.
__device__ double tail_dot(const LevelK<double> &L, const double *x, const double *y, double *sw)
{
    const long long n = (long long)L.nx * L.ny * L.nz;
    double acc = 0.0;
    if (threadIdx.x < 64) {
        for (long long q = threadIdx.x; q < n; q += 64) {
            const int i = (int)(q % L.nx) + 1;
            const long long rr = q / L.nx;
            const int j = (int)(rr % L.ny) + 1, k = (int)(rr / L.ny) + 1;
            const long long p = lin(i, j, k, L.sy, L.sz);
            acc = __dadd_rn(acc, __dmul_rn(x[p], y[p]));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc = __dadd_rn(acc, __shfl_down_sync(0xffffffffu, acc, o));
        if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = acc;
    }
    __syncthreads();
    const double s = __dadd_rn(sw[0], sw[1]);
    __syncthreads();
    return s;
}

// r = b - A x on the interior; with NORM also returns sum(r^2) (tail_dot order).
template <bool NORM>
__device__ double tail_residual(const LevelK<double> &L, double *r, const double *x, const double *b, double *sw)
{
    const long long n = (long long)L.nx * L.ny * L.nz;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) {
        const int i = (int)(q % L.nx) + 1;
        const long long rr = q / L.nx;
        const int j = (int)(rr % L.ny) + 1, k = (int)(rr / L.ny) + 1;
        const long long p = lin(i, j, k, L.sy, L.sz);
        r[p] = __dsub_rn(b[p], ax_cell_f64(L, x, i, j, k));
    }
    __syncthreads();
    if (NORM) return tail_dot(L, r, r, sw);
    return 0.0;
}

__device__ void tail_mvmul(const LevelK<double> &L, double *y, const double *x)
{
    const long long n = (long long)L.nx * L.ny * L.nz;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) {
        const int i = (int)(q % L.nx) + 1;
        const long long rr = q / L.nx;
        const int j = (int)(rr % L.ny) + 1, k = (int)(rr / L.ny) + 1;
        y[lin(i, j, k, L.sy, L.sz)] = ax_cell_f64(L, x, i, j, k);
    }
    __syncthreads();
}

__device__ void tail_restrict(const XferK<double> &X, const double *vf, double *vc)
{
    const long long n = (long long)X.ncx * X.ncy * X.ncz;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) {
        const int i = (int)(q % X.ncx) + 1;
        const long long rr = q / X.ncx;
        const int j = (int)(rr % X.ncy) + 1, k = (int)(rr / X.ncy) + 1;
        vc[lin(i, j, k, X.csy, X.csz)] = restrict_cell_f64(X, vf, i, j, k);
    }
    __syncthreads();
}

__device__ void tail_prolong_add(const XferK<double> &X, const double *vc, double *vf)
{
    const long long n = (long long)X.ncx * X.ncy * X.ncz;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) {
        const int i = (int)(q % X.ncx) + 1;
        const long long rr = q / X.ncx;
        const int j = (int)(rr % X.ncy) + 1, k = (int)(rr / X.ncy) + 1;
        prolong_cell_f64<true>(X, vc, vf, i, j, k);
    }
    __syncthreads();
}

__device__ void tail_interior_op(const LevelK<double> &L, int op, double s, double *a, double *bb, const double *c,
                                 const double *d)
{
    // op 0: a = c (copy); op 1: a += s c, bb -= s d; op 2: a = c + s a
    const long long n = (long long)L.nx * L.ny * L.nz;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) {
        const int i = (int)(q % L.nx) + 1;
        const long long rr = q / L.nx;
        const int j = (int)(rr % L.ny) + 1, k = (int)(rr / L.ny) + 1;
        const long long p = lin(i, j, k, L.sy, L.sz);
        if (op == 0) {
            a[p] = c[p];
        } else if (op == 1) {
            a[p] = __dadd_rn(a[p], __dmul_rn(s, c[p]));
            bb[p] = __dsub_rn(bb[p], __dmul_rn(s, d[p]));
        } else {
            a[p] = __dadd_rn(c[p], __dmul_rn(s, a[p]));
        }
    }
    __syncthreads();
}


// The context's host abort flag (pmg_set_abort), read by thread 0 and shared, so that the
// whole block takes the same decision; every thread of the block must call it.
__device__ __forceinline__ bool block_abort(const volatile int *abort)
{
    if (!abort) return false;
    __shared__ int s_abort;
    __syncthreads();
    if (threadIdx.x == 0) s_abort = *abort;
    __syncthreads();
    return s_abort != 0;
}

// The same for one warp (lane 0 reads, the value is broadcast).
__device__ __forceinline__ bool warp_abort(const volatile int *abort)
{
    int v = 0;
    if ((threadIdx.x & 31) == 0 && abort) v = *abort;
    return __shfl_sync(0xffffffffu, v, 0) != 0;
}

// Coarsest-level solve on one CTA (src/multigrid.f90:1819-1851): x = 0, then x = b/c0 for
// a single cell, else rbgs_solver_poisson_matrix (src/rbgs_poisson_matrix.f90:69-171,
// solver 0) or cg_solver_poisson_matrix (src/cg_poisson_matrix.f90:80-138, solver 1)
// with `maxit` iterations and `tol`.  p, ap, rr: full-size scratch arrays with zero
// ghosts.  Every 16 iterations the host abort flag (if any) is polled; when it is set the
// solve stops there.  Returns the solver's iteration counter.
__device__ int coarse_solve_f64(const LevelK<double> &L, double *x, const double *b, double *p, double *ap,
                                double *rr, int solver, int maxit, double tol, double omega, double omw, double *sw,
                                const volatile int *abort = nullptr)
{
    tail_zero(x, (long long)L.sz * (L.nz + 2));
    __syncthreads();
    int iters = 0;
    if ((long long)L.nx * L.ny * L.nz == 1) {
        if (threadIdx.x == 0) {
            const long long q = lin(1, 1, 1, L.sy, L.sz);
            x[q] = __ddiv_rn(b[q], diag_f64(L, 1, 1, 1));
        }
        __syncthreads();
    } else if (solver == 0) {
        const double r0 = tail_residual<true>(L, rr, x, b, sw);
        int it = 0;
        for (it = 0; it < maxit; ++it) {
            tail_rbgs(L, x, b, 1, omega, omw);
            const double rn = tail_residual<true>(L, rr, x, b, sw);
            if (sqrt(__ddiv_rn(rn, r0)) <= tol) break;
            if ((it & 15) == 15 && block_abort(abort)) break;
        }
        iters = it;
    } else {
        tail_residual<false>(L, rr, x, b, sw);
        tail_interior_op(L, 0, 0.0, p, nullptr, rr, nullptr);
        const double r0 = tail_dot(L, rr, rr, sw);
        // temp1 = r.r of the unchanged r (:107) equals the previous iteration's temp2 (and
        // rsd0tol at the first), so it is carried instead of summed again
        double t1 = r0;
        int it = 0;
        for (it = 0; it < maxit; ++it) {
            tail_mvmul(L, ap, p);
            const double t2a = tail_dot(L, ap, p, sw);
            const double alpha = __ddiv_rn(t1, t2a);
            tail_interior_op(L, 1, alpha, x, rr, p, ap);
            const double t2 = tail_dot(L, rr, rr, sw);
            if (sqrt(__ddiv_rn(t2, r0)) < tol) break;
            const double beta = __ddiv_rn(t2, t1);
            tail_interior_op(L, 2, beta, p, nullptr, rr, nullptr);
            t1 = t2;
            if ((it & 15) == 15 && block_abort(abort)) break;
        }
        iters = it;
    }
    return iters;
}

// Coarsest-level solve by ONE warp on a level held in shared memory (at most
// kWarpCoarseMax stored values, ghosts included), for the FP32 cycle of the mixed solver:
// the iterations of coarse_solve_f64 (RBGS or CG, the same exit tests; levels of at most
// 64 cells take a register fast path with reordered arithmetic), the sums in a 32-lane
// butterfly order (every lane obtains the same bits, so the exit decision is uniform),
// and __syncwarp instead of block barriers.  x, b, p, ap, rr are shared
// arrays of the level's layout; only the calling warp touches them.
constexpr int kWarpCoarseMax = 1000;

__device__ __forceinline__ double warp_sum_f64(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ int coarse_solve_warp_f64(const LevelK<double> &L, double *x, const double *b, double *p, double *ap,
                                     double *rr, int solver, int maxit, double tol, double omega, double omw,
                                     const volatile int *abort = nullptr)
{
    const int lane = threadIdx.x & 31;
    const int nx = L.nx, ny = L.ny, n = L.nx * L.ny * L.nz;
    const int total = (int)(L.sz * (L.nz + 2));
    for (int q = lane; q < total; q += 32) {
        x[q] = 0.0;
        p[q] = 0.0;
        ap[q] = 0.0;
        rr[q] = 0.0;
    }
    __syncwarp();
    if (n == 1) {
        if (lane == 0) {
            const long long c = lin(1, 1, 1, L.sy, L.sz);
            x[c] = __ddiv_rn(b[c], diag_f64(L, 1, 1, 1));
        }
        __syncwarp();
        return 0;
    }
    auto residual = [&](bool norm) -> double {
        double acc = 0.0;
        for (int q = lane; q < n; q += 32) {
            const int i = q % nx + 1, r2 = q / nx, j = r2 % ny + 1, k = r2 / ny + 1;
            const long long c = lin(i, j, k, L.sy, L.sz);
            const double r = __dsub_rn(b[c], ax_cell_f64(L, x, i, j, k));
            rr[c] = r;
            acc = __dadd_rn(acc, __dmul_rn(r, r));
        }
        __syncwarp();
        return norm ? warp_sum_f64(acc) : 0.0;
    };
    auto dot = [&](const double *u, const double *v) -> double {
        double acc = 0.0;
        for (int q = lane; q < n; q += 32) {
            const int i = q % nx + 1, r2 = q / nx, j = r2 % ny + 1, k = r2 / ny + 1;
            const long long c = lin(i, j, k, L.sy, L.sz);
            acc = __dadd_rn(acc, __dmul_rn(u[c], v[c]));
        }
        return warp_sum_f64(acc);
    };
    // op 0: a = c; op 1: a += s c, bb -= s d; op 2: a = c + s a
    auto interior = [&](int op, double sc, double *a, double *bb, const double *c, const double *d) {
        for (int q = lane; q < n; q += 32) {
            const int i = q % nx + 1, r2 = q / nx, j = r2 % ny + 1, k = r2 / ny + 1;
            const long long e = lin(i, j, k, L.sy, L.sz);
            if (op == 0) {
                a[e] = c[e];
            } else if (op == 1) {
                a[e] = __dadd_rn(a[e], __dmul_rn(sc, c[e]));
                bb[e] = __dsub_rn(bb[e], __dmul_rn(sc, d[e]));
            } else {
                a[e] = __dadd_rn(c[e], __dmul_rn(sc, a[e]));
            }
        }
        __syncwarp();
    };
    int it = 0;
    if (solver == 0 && n <= 64) {
        // at most two cells per lane: their offsets, coefficients, omega/c0 and b stay in
        // registers.  Each dependent FP64 operation costs on the order of a hundred
        // cycles here, so the arithmetic is arranged for short chains: the neighbour sum
        // as a tree of FMAs, the update x = (omega/c0)(b - t) + (1-omega) x, and the exit
        // test sqrt(|r|^2/|r0|^2) <= tol as |r|^2 <= tol^2 |r0|^2 (no division or square
        // root per iteration).  The same RBGS iteration as the reference's solver; the
        // FP32 cycle that calls it is not bound to the reference's bits.
        long long cidx[2];
        double cw[2][6], c0v[2], wv[2], bv[2];
        bool has[2], odd[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int q = lane + 32 * u;
            has[u] = q < n;
            const int qq = has[u] ? q : 0;
            const int i = qq % nx + 1, r2 = qq / nx, j = r2 % ny + 1, k = r2 / ny + 1;
            cidx[u] = lin(i, j, k, L.sy, L.sz);
            odd[u] = ((i + j + k) & 1) != 0;
            cw[u][0] = L.cxm[i];
            cw[u][1] = L.cxp[i];
            cw[u][2] = L.cym[j];
            cw[u][3] = L.cyp[j];
            cw[u][4] = L.czm[k];
            cw[u][5] = L.czp[k];
            c0v[u] = diag_f64(L, i, j, k);
            wv[u] = __ddiv_rn(omega, c0v[u]);
            bv[u] = b[cidx[u]];
        }
        const long long sy = L.sy, sz = L.sz;
        auto nbsum = [&](int u) {
            const long long c = cidx[u];
            const double tx = fma(cw[u][1], x[c + 1], __dmul_rn(cw[u][0], x[c - 1]));
            const double ty = fma(cw[u][3], x[c + sy], __dmul_rn(cw[u][2], x[c - sy]));
            const double tz = fma(cw[u][5], x[c + sz], __dmul_rn(cw[u][4], x[c - sz]));
            return __dadd_rn(__dadd_rn(tx, ty), tz);
        };
        auto norm = [&]() {
            double acc = 0.0;
#pragma unroll
            for (int u = 0; u < 2; ++u)
                if (has[u]) {
                    const double r = __dsub_rn(bv[u], fma(c0v[u], x[cidx[u]], nbsum(u)));
                    acc = fma(r, r, acc);
                }
            return warp_sum_f64(acc);
        };
        const double r0 = norm();
        const double thr = __dmul_rn(__dmul_rn(tol, tol), r0);
        for (it = 0; it < maxit; ++it) {
#pragma unroll
            for (int colour = 0; colour < 2; ++colour) {
                // first colour: (i + j + k) odd (src/rbgs_poisson_matrix.f90:242)
#pragma unroll
                for (int u = 0; u < 2; ++u)
                    if (has[u] && odd[u] == (colour == 0)) {
                        const double old = x[cidx[u]];
                        const double t = nbsum(u);
                        x[cidx[u]] = fma(wv[u], __dsub_rn(bv[u], t), __dmul_rn(omw, old));
                    }
                __syncwarp();
            }
            if (norm() <= thr) break;
            if ((it & 15) == 15 && warp_abort(abort)) break;
        }
    } else if (solver == 0) {
        const int hx = (nx + 1) / 2, nq = hx * ny * L.nz;
        const double r0 = residual(true);
        for (it = 0; it < maxit; ++it) {
            for (int colour = 0; colour < 2; ++colour) {
                for (int q = lane; q < nq; q += 32) {
                    const int t = q % hx, r2 = q / hx, j = r2 % ny + 1, k = r2 / ny + 1;
                    const int i = 2 * t + 1 + ((j + k + colour) & 1);
                    if (i <= nx) x[lin(i, j, k, L.sy, L.sz)] = rbgs_cell_f64(L, x, b, i, j, k, omega, omw);
                }
                __syncwarp();
            }
            const double rn = residual(true);
            if (sqrt(__ddiv_rn(rn, r0)) <= tol) break;
            if ((it & 15) == 15 && warp_abort(abort)) break;
        }
    } else {
        residual(false);
        interior(0, 0.0, p, nullptr, rr, nullptr);
        const double r0 = dot(rr, rr);
        // Fused passes: A p with the sum Ap.p, and the x/r update with the sum r.r.  Each
        // lane visits its cells in the order dot() does, so the sums are dot()'s; temp1
        // (r.r of the unchanged r) is the previous iteration's temp2.
        double t1 = r0;
        for (it = 0; it < maxit; ++it) {
            double pap = 0.0;
            for (int q = lane; q < n; q += 32) {
                const int i = q % nx + 1, r2 = q / nx, j = r2 % ny + 1, k = r2 / ny + 1;
                const long long c = lin(i, j, k, L.sy, L.sz);
                const double v = ax_cell_f64(L, p, i, j, k);
                ap[c] = v;
                pap = __dadd_rn(pap, __dmul_rn(v, p[c]));
            }
            const double alpha = __ddiv_rn(t1, warp_sum_f64(pap));
            double rr2 = 0.0;
            for (int q = lane; q < n; q += 32) {
                const int i = q % nx + 1, r2 = q / nx, j = r2 % ny + 1, k = r2 / ny + 1;
                const long long c = lin(i, j, k, L.sy, L.sz);
                x[c] = __dadd_rn(x[c], __dmul_rn(alpha, p[c]));
                const double v = __dsub_rn(rr[c], __dmul_rn(alpha, ap[c]));
                rr[c] = v;
                rr2 = __dadd_rn(rr2, __dmul_rn(v, v));
            }
            const double t2 = warp_sum_f64(rr2);
            __syncwarp();
            if (sqrt(__ddiv_rn(t2, r0)) < tol) break;
            interior(2, __ddiv_rn(t2, t1), p, nullptr, rr, nullptr);
            t1 = t2;
            if ((it & 15) == 15 && warp_abort(abort)) break;
        }
    }
    return it;
}

}  // namespace
}  // namespace pmg
