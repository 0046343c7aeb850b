// pmg_f64.cu -- FP64 kernels of the V-cycle that reproduce the reference's arithmetic
// bit for bit.  Compiled with --fmad=false; every floating-point operation is also
// spelled out with an explicit round-to-nearest intrinsic in pmg_common.cuh.
//
// All grid kernels use grid-stride loops along all three axes, so a level can be run
// with any grid shape: the full grid (CGS), or with an axis collapsed to one CTA
// column (the CGPSA per-axis step-down), without changing any cell's arithmetic.
#include <cuda_runtime.h>

#include "../../include/peps_mg.h"
#include "pmg_internal.h"
#include "pmg_tail64.cuh"

namespace pmg {

namespace {

constexpr int kBX = 32, kBY = 8;          // 256-thread CTAs for the grid kernels
constexpr int kTailThreads = 1024;        // single-CTA persistent tail
constexpr int kMaxGridZ = 65535;

__device__ __forceinline__ int tid_in_block()
{
    return threadIdx.x + blockDim.x * threadIdx.y;
}

__device__ __forceinline__ int block_lin()
{
    return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
}

// The diagonal c0 of cell p: read from the level's per-cell table (TAB; the values
// k_diag_f64 stored, diag_f64's bits) or formed from the 1-D tables.  The table takes four
// of the 28 FP64 instructions of an RBGS update off a pipe that bounds these kernels.
template <bool TAB>
__device__ __forceinline__ double diag_at(const LevelK<double> &L, const double *c0t, long long p, int i, int j,
                                          int k)
{
    return TAB ? c0t[p] : diag_f64(L, i, j, k);
}

// One colour of the red-black sweep.  colour 0 is the reference's first half-sweep:
// ista = 1 + mod(j+k, 2) (src/rbgs_poisson_matrix.f90:242); colour 1 the second
// (:260).  Thread t of a row updates i = 2t + ista.
template <bool TAB, bool OMEGA1>
__global__ void __launch_bounds__(kBX *kBY) k_rbgs_f64(LevelK<double> L, double *__restrict__ x,
                                                       const double *__restrict__ b, double omega, double omw,
                                                       int colour, const double *__restrict__ c0t)
{
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y) {
            const int ista = 1 + ((j + k + colour) & 1);
            for (int i = ista + 2 * (blockIdx.x * blockDim.x + threadIdx.x); i <= L.nx;
                 i += 2 * gridDim.x * blockDim.x) {
                const long long p = lin(i, j, k, L.sy, L.sz);
                x[p] = rbgs_cell_c0_f64<OMEGA1>(L, x, b, i, j, k, omega, omw, diag_at<TAB>(L, c0t, p, i, j, k));
            }
        }
}

// c0t = the diagonal of every interior cell (diag_f64); the ghosts are left as they are.
__global__ void __launch_bounds__(kBX *kBY) k_diag_f64(LevelK<double> L, double *__restrict__ c0t)
{
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x)
                c0t[lin(i, j, k, L.sy, L.sz)] = diag_f64(L, i, j, k);
}

// r = b - A x on the interior (src/multigrid.f90:1795-1805); optional per-block sum of r^2.
template <bool NORM, bool TAB>
__global__ void __launch_bounds__(kBX *kBY) k_residual_f64(LevelK<double> L, double *__restrict__ r,
                                                           const double *__restrict__ x,
                                                           const double *__restrict__ b, double *partials,
                                                           const double *__restrict__ c0t)
{
    double acc = 0.0;
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x) {
                const long long p = lin(i, j, k, L.sy, L.sz);
                const double v = __dsub_rn(b[p], ax_cell_c0_f64(L, x, i, j, k, diag_at<TAB>(L, c0t, p, i, j, k)));
                r[p] = v;
                if (NORM) acc = __dadd_rn(acc, __dmul_rn(v, v));
            }
    if (NORM) {
        __shared__ double sw[kBX * kBY / 32];
        const double s = block_sum(acc, sw);
        if (tid_in_block() == 0) partials[block_lin()] = s;
    }
}

template <bool TAB>
__global__ void __launch_bounds__(kBX *kBY) k_mvmul_f64(LevelK<double> L, double *__restrict__ y,
                                                        const double *__restrict__ x, const double *__restrict__ c0t)
{
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x) {
                const long long p = lin(i, j, k, L.sy, L.sz);
                y[p] = ax_cell_c0_f64(L, x, i, j, k, diag_at<TAB>(L, c0t, p, i, j, k));
            }
}

__global__ void __launch_bounds__(kBX *kBY) k_dot_f64(LevelK<double> L, const double *__restrict__ x,
                                                      const double *__restrict__ y, double *partials)
{
    double acc = 0.0;
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x) {
                const long long p = lin(i, j, k, L.sy, L.sz);
                acc = __dadd_rn(acc, __dmul_rn(x[p], y[p]));
            }
    __shared__ double sw[kBX * kBY / 32];
    const double s = block_sum(acc, sw);
    if (tid_in_block() == 0) partials[block_lin()] = s;
}

__global__ void __launch_bounds__(1024) k_reduce_f64(const double *__restrict__ partials, int n, double *out)
{
    double acc = 0.0;
    for (int q = threadIdx.x; q < n; q += blockDim.x) acc = __dadd_rn(acc, partials[q]);
    __shared__ double sw[32];
    const double s = block_sum(acc, sw);
    if (threadIdx.x == 0) *out = s;
}

__global__ void __launch_bounds__(kBX *kBY) k_restrict_f64(XferK<double> X, const double *__restrict__ vf,
                                                           double *__restrict__ vc)
{
    for (int k = blockIdx.z + 1; k <= X.ncz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= X.ncy; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= X.ncx; i += gridDim.x * blockDim.x)
                vc[lin(i, j, k, X.csy, X.csz)] = restrict_cell_f64(X, vf, i, j, k);
}

template <bool ADD>
__global__ void __launch_bounds__(kBX *kBY) k_prolong_f64(XferK<double> X, const double *__restrict__ vc,
                                                          double *__restrict__ vf)
{
    for (int k = blockIdx.z + 1; k <= X.ncz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= X.ncy; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= X.ncx; i += gridDim.x * blockDim.x)
                prolong_cell_f64<ADD>(X, vc, vf, i, j, k);
}

// Zero the six ghost faces of a (nx+2)(ny+2)(nz+2) array.
__global__ void k_zero_ghosts_f64(double *a, int nx, int ny, int nz)
{
    const int sy = nx + 2;
    const long long sz = (long long)(nx + 2) * (ny + 2);
    const long long nxy = sz, nxz = (long long)(nx + 2) * (nz + 2), nyz = (long long)(ny + 2) * (nz + 2);
    const long long total = 2 * (nxy + nxz + nyz);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        long long r = q;
        int face = 0;
        if (r < 2 * nxy) {
            face = (int)(r / nxy);
            r %= nxy;
            const int i = (int)(r % sy), j = (int)(r / sy);
            a[lin(i, j, face ? nz + 1 : 0, sy, sz)] = 0.0;
            continue;
        }
        r -= 2 * nxy;
        if (r < 2 * nxz) {
            face = (int)(r / nxz);
            r %= nxz;
            const int i = (int)(r % sy), k = (int)(r / sy);
            a[lin(i, face ? ny + 1 : 0, k, sy, sz)] = 0.0;
            continue;
        }
        r -= 2 * nxz;
        face = (int)(r / nyz);
        r %= nyz;
        const int j = (int)(r % (ny + 2)), k = (int)(r / (ny + 2));
        a[lin(face ? nx + 1 : 0, j, k, sy, sz)] = 0.0;
    }
}

// ------------------------------------------------------------------------------------
// Fused CG (cg_solver_poisson_matrix / cg_iterator_poisson_matrix,
// src/cg_poisson_matrix.f90:80-138 and :190-238).  Per iteration the reference makes
// six passes over the level (r.r, A p, Ap.p, the x/r update, r.r, the p update) plus two
// scalar divisions; here three kernels do the same arithmetic:
//   k_cg_apdot   Ap = A p and the sum Ap.p; its last CTA forms alpha = temp1 / (Ap.p)
//   k_cg_update  x += alpha p, r -= alpha Ap and the sum r.r; its last CTA forms temp2,
//                the exit test sqrt(temp2/rsd0tol) < tol and beta = temp2 / temp1
//   k_cg_p       p = r + beta p
// temp1 of an iteration is r.r of the previous one: the reference recomputes it from the
// same r (:107), which gives the same value.  Each kernel's sum is one partial per CTA
// (fixed order inside the CTA), added by the last CTA to arrive in a fixed order, so the
// result depends only on the grid, which is a function of the level.  The scalars stay
// on the device (CgState); kernels launched after the exit test was met return at once,
// so the host only reads the state every few iterations.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ bool cg_arrive_last(CgState *st, double s, double *partials)
{
    __shared__ unsigned int ticket;
    if (tid_in_block() == 0) {
        partials[block_lin()] = s;
        __threadfence();
        ticket = atomicAdd(&st->arrive, 1u);
    }
    __syncthreads();
    return ticket == gridDim.x * gridDim.y * gridDim.z - 1;
}

// Sum of the CTAs' partials in a fixed order (called by every thread of the last CTA).
__device__ __forceinline__ double cg_sum_partials(const double *partials, double *sw)
{
    __threadfence();
    const int n = (int)(gridDim.x * gridDim.y * gridDim.z);
    double acc = 0.0;
    for (int q = tid_in_block(); q < n; q += blockDim.x * blockDim.y) acc = __dadd_rn(acc, __ldcg(partials + q));
    return block_sum(acc, sw);
}

// r = b - A x, p = r (src/cg_poisson_matrix.f90:80-91), rsd0tol = temp1 = r.r (:94, :107)
template <bool TAB>
__global__ void __launch_bounds__(kBX *kBY) k_cg_init(LevelK<double> L, double *__restrict__ r,
                                                      double *__restrict__ p, const double *__restrict__ x,
                                                      const double *__restrict__ b, double *partials, CgState *st,
                                                      const double *__restrict__ c0t)
{
    double acc = 0.0;
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x) {
                const long long q = lin(i, j, k, L.sy, L.sz);
                const double v = __dsub_rn(b[q], ax_cell_c0_f64(L, x, i, j, k, diag_at<TAB>(L, c0t, q, i, j, k)));
                r[q] = v;
                p[q] = v;
                acc = __dadd_rn(acc, __dmul_rn(v, v));
            }
    __shared__ double sw[kBX * kBY / 32];
    const double s = block_sum(acc, sw);
    if (cg_arrive_last(st, s, partials)) {
        const double t = cg_sum_partials(partials, sw);
        if (tid_in_block() == 0) {
            st->r0 = t;
            st->t1 = t;
            st->t2 = t;
            st->done = 0;
            st->iter = 0;
            st->arrive = 0;
        }
    }
}

// Ap = A p (src/poisson_matrix_operator.f90:146-159), temp2 = Ap.p (:112), alpha (:114)
template <bool TAB>
__global__ void __launch_bounds__(kBX *kBY) k_cg_apdot(LevelK<double> L, const double *__restrict__ p,
                                                       double *__restrict__ ap, double *partials, CgState *st,
                                                       const double *__restrict__ c0t)
{
    if (st->done) return;
    double acc = 0.0;
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x) {
                const long long q = lin(i, j, k, L.sy, L.sz);
                const double v = ax_cell_c0_f64(L, p, i, j, k, diag_at<TAB>(L, c0t, q, i, j, k));
                ap[q] = v;
                acc = __dadd_rn(acc, __dmul_rn(v, p[q]));
            }
    __shared__ double sw[kBX * kBY / 32];
    const double s = block_sum(acc, sw);
    if (cg_arrive_last(st, s, partials)) {
        const double t = cg_sum_partials(partials, sw);
        if (tid_in_block() == 0) {
            st->pap = t;
            st->alpha = __ddiv_rn(st->t1, t);
            st->arrive = 0;
        }
    }
}

// sol += alpha p, rsd -= alpha Ap (:117-118), temp2 = r.r (:123), exit test (:126),
// beta = temp2 / temp1 (:128)
__global__ void __launch_bounds__(kBX *kBY) k_cg_update(LevelK<double> L, double *__restrict__ x,
                                                        double *__restrict__ r, const double *__restrict__ p,
                                                        const double *__restrict__ ap, double *partials, CgState *st,
                                                        double tol, int check, int iter)
{
    if (st->done) return;
    const double alpha = st->alpha;
    double acc = 0.0;
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x) {
                const long long q = lin(i, j, k, L.sy, L.sz);
                x[q] = __dadd_rn(x[q], __dmul_rn(alpha, p[q]));
                const double v = __dsub_rn(r[q], __dmul_rn(alpha, ap[q]));
                r[q] = v;
                acc = __dadd_rn(acc, __dmul_rn(v, v));
            }
    __shared__ double sw[kBX * kBY / 32];
    const double s = block_sum(acc, sw);
    if (cg_arrive_last(st, s, partials)) {
        const double t = cg_sum_partials(partials, sw);
        if (tid_in_block() == 0) {
            st->t2 = t;
            if (check && sqrt(__ddiv_rn(t, st->r0)) < tol) {
                st->done = 1;
                st->iter = iter;
            } else {
                st->beta = __ddiv_rn(t, st->t1);
                st->t1 = t;
            }
            st->arrive = 0;
        }
    }
}

// p = rsd + beta p (:134)
__global__ void __launch_bounds__(kBX *kBY) k_cg_p(LevelK<double> L, double *__restrict__ p,
                                                   const double *__restrict__ r, const CgState *st)
{
    if (st->done) return;
    const double beta = st->beta;
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x) {
                const long long q = lin(i, j, k, L.sy, L.sz);
                p[q] = __dadd_rn(r[q], __dmul_rn(beta, p[q]));
            }
}

// ------------------------------------------------------------------------------------
// Single-CTA persistent coarse tail.  Runs, for levels l0..nl of one V-cycle, exactly
// the operation sequence of src/multigrid.f90:1936-1962 (the part of the CGA cycle that
// rank 0 executes after the gather, :2108-2135): smoothing, residual and restriction
// down to the coarsest level, the coarsest-level solve (:1819-1851), then prolongation,
// correction and smoothing back up to l0.  Phases are separated by __syncthreads();
// every cell is computed by the same per-cell functions as the grid kernels.
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kTailThreads) k_tail_f64(const TailDesc<double> *__restrict__ Dp)
{
    __shared__ double sw[kTailThreads / 32];
    const TailDesc<double> &D = *Dp;
    const double omega = D.omega, omw = D.omw;
    for (int l = D.l0; l < D.nl; ++l) {
        const LevelK<double> L = D.L[l];
        const XferK<double> X = D.X[l];
        double *x = D.x[l], *b = D.b[l], *r = D.r[l], *bc = D.b[l + 1];
        tail_zero(x, (long long)L.sz * (L.nz + 2));
        __syncthreads();
        tail_rbgs(L, x, b, D.maxit, omega, omw);
        tail_residual<false>(L, r, x, b, sw);
        tail_restrict(X, r, bc);
    }
    // coarsest level, src/multigrid.f90:1819-1851
    {
        const int iters = coarse_solve_f64(D.C64, D.cx64, D.cb64, D.cp64, D.cap64, D.crr64, D.coarse_solver,
                                           D.coarse_maxit, D.tol, D.omega64, D.omw64, sw, D.abort);
        if (threadIdx.x == 0 && D.iters_out) *D.iters_out = iters;
        __syncthreads();
    }
    for (int l = D.nl - 1; l >= D.l0; --l) {
        const LevelK<double> L = D.L[l];
        const XferK<double> X = D.X[l];
        double *x = D.x[l], *b = D.b[l], *xc = D.x[l + 1];
        tail_prolong_add(X, xc, x);
        tail_rbgs(L, x, b, D.maxit, omega, omw);
    }
}

// ------------------------------------------------------------------------------------
// Device-side hierarchy set-up (multigrid_subdomain_create_*, src/multigrid.f90:167-495,
// and matrix_heptadiagonal_create, src/matrix.f90:39-94): one CTA per axis builds the
// meshes of every coarse level from the finer one (unless the meshes are given), then the
// per-axis coefficient tables of every level and the transfer weights between levels, in
// the host layout described by HierDesc.  Same expressions, same rounding as the host code
// (this translation unit is compiled without FMA contraction).
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_hierarchy(const HierDesc *__restrict__ Hp, double *__restrict__ meshes,
                                                   double *__restrict__ tables)
{
    const HierDesc &H = *Hp;
    const int d = blockIdx.x;
    const int nl = H.nl;
    // coarse meshes
    if (!H.meshes_given)
        for (int l = 1; l <= nl; ++l) {
            const int n = H.n[l][d], nf = H.n[l - 1][d];
            double *dm = meshes + H.mesh_off[l][d], *dg = dm + (n + 2), *xg = dg + (n + 2);
            const double *dmf = meshes + H.mesh_off[l - 1][d], *dgf = dmf + (nf + 2), *xgf = dgf + (nf + 2);
            if (l <= H.lvc[d]) {
                for (int i = threadIdx.x + 1; i <= n; i += blockDim.x) dm[i] = dmf[2 * i - 1] + dmf[2 * i];
                if (threadIdx.x == 0) {
                    dm[0] = dmf[0];
                    dm[n + 1] = dmf[2 * n + 1];
                }
                __syncthreads();
                for (int i = threadIdx.x + 1; i <= n + 1; i += blockDim.x) dg[i] = 0.5 * (dm[i] + dm[i - 1]);
                __syncthreads();
                if (threadIdx.x == 0) {
                    const bool from_origin = H.method == PMG_CGS || (H.method == PMG_CGA && l <= H.agg_level);
                    xg[0] = from_origin ? H.ox[d] - 0.5 * dm[0] : (xgf[0] + 0.5 * dmf[0]) - 0.5 * dm[0];
                    dg[0] = 0.0;
                    for (int i = 1; i <= n + 1; ++i) xg[i] = xg[i - 1] + dg[i];
                }
            } else {
                for (int i = threadIdx.x; i <= n + 1; i += blockDim.x) {
                    dm[i] = dmf[i];
                    dg[i] = dgf[i];
                    xg[i] = xgf[i];
                }
            }
            __syncthreads();
        }
    // coefficient tables (src/matrix.f90:75-82) and transfer weights
    for (int l = 0; l <= nl; ++l) {
        const int n = H.n[l][d];
        const double *dm = meshes + H.mesh_off[l][d], *dg = dm + (n + 2);
        double *cm = tables + H.cm[l][d], *cp = tables + H.cp[l][d];
        double *sx = d == 0 ? tables + H.sx[l] : nullptr;
        for (int i = threadIdx.x + 1; i <= n; i += blockDim.x) {
            const double a = __ddiv_rn(1.0, __dmul_rn(dm[i], dg[i]));
            const double b = __ddiv_rn(1.0, __dmul_rn(dm[i], dg[i + 1]));
            cm[i] = a;
            cp[i] = b;
            if (sx) sx[i] = __dadd_rn(a, b);
        }
        if (l == nl) break;
        const int nc = H.n[l + 1][d];
        const double *dmc = meshes + H.mesh_off[l + 1][d];
        double *w = tables + H.w[l][d], *pp = tables + H.pp[l][d], *pn = tables + H.pn[l][d];
        if (l >= H.lvc[d]) {   // the axis is no longer coarsened: stride 1 (src/multigrid.f90:1415-1458)
            for (int i = threadIdx.x; i <= n + 1; i += blockDim.x) {
                w[i] = dm[i];
                pp[i] = dmc[i];
                pn[i] = dmc[i];
            }
        } else {
            for (int i = threadIdx.x + 1; i <= n; i += blockDim.x) w[i] = __dsub_rn(dmc[(i - 1) / 2 + 1], dm[i]);
            for (int i = threadIdx.x + 1; i <= nc; i += blockDim.x) {   // src/multigrid.f90:1604-1610
                const int f = 2 * i;
                pp[f - 1] = __dadd_rn(__dmul_rn(1.0, dm[f - 2]), __dmul_rn(0.5, dm[f - 1]));
                pp[f] = __dmul_rn(0.5, dm[f - 1]);
                pn[f - 1] = __dmul_rn(0.5, dm[f]);
                pn[f] = __dadd_rn(__dmul_rn(1.0, dm[f + 1]), __dmul_rn(0.5, dm[f]));
            }
        }
    }
}

dim3 grid3(int nx_threads, int ny, int nz, const Launch &ln)
{
    dim3 g;
    g.x = ln.collapse[0] ? 1u : (unsigned)((nx_threads + kBX - 1) / kBX);
    g.y = ln.collapse[1] ? 1u : (unsigned)((ny + kBY - 1) / kBY);
    g.z = ln.collapse[2] ? 1u : (unsigned)(nz < kMaxGridZ ? nz : kMaxGridZ);
    if (g.x == 0) g.x = 1;
    if (g.y == 0) g.y = 1;
    if (g.z == 0) g.z = 1;
    return g;
}

}  // namespace

void grid_for_cells(const LevelK<double> &L, const Launch &ln, dim3 *grid, dim3 *block)
{
    *grid = grid3(L.nx, L.ny, L.nz, ln);
    *block = dim3(kBX, kBY, 1);
}

static void launch_rbgs_colour(const LevelK<double> &L, dim3 g, double *x, const double *b, double omega,
                               double omw, int colour, const double *c0t, cudaStream_t s)
{
    const dim3 bl(kBX, kBY, 1);
    // omega == 1 exactly: 1 * v is v for every double, so the OMEGA1 kernel's bits are the same
    if (c0t && omega == 1.0)
        k_rbgs_f64<true, true><<<g, bl, 0, s>>>(L, x, b, omega, omw, colour, c0t);
    else if (c0t)
        k_rbgs_f64<true, false><<<g, bl, 0, s>>>(L, x, b, omega, omw, colour, c0t);
    else if (omega == 1.0)
        k_rbgs_f64<false, true><<<g, bl, 0, s>>>(L, x, b, omega, omw, colour, nullptr);
    else
        k_rbgs_f64<false, false><<<g, bl, 0, s>>>(L, x, b, omega, omw, colour, nullptr);
}

int f64_rbgs_sweeps(const LevelK<double> &L, const Launch &ln, double *x, const double *b, int iters,
                    double omega, cudaStream_t s, const double *c0t)
{
    const double omw = 1.0 - omega;   // (1.0d0-omega), src/rbgs_poisson_matrix.f90:250
    const dim3 g = grid3((L.nx + 1) / 2, L.ny, L.nz, ln);
    for (int it = 0; it < iters; ++it)
        for (int c = 0; c < 2; ++c) launch_rbgs_colour(L, g, x, b, omega, omw, c, c0t, s);
    count_launches(2LL * iters);
    return cuda_status(cudaGetLastError(), "rbgs sweep");
}

int f64_rbgs_colour(const LevelK<double> &L, const Launch &ln, double *x, const double *b, double omega, int colour,
                    cudaStream_t s, const double *c0t)
{
    const dim3 g = grid3((L.nx + 1) / 2, L.ny, L.nz, ln);
    launch_rbgs_colour(L, g, x, b, omega, 1.0 - omega, colour & 1, c0t, s);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "rbgs half-sweep");
}

int f64_diag_table(const LevelK<double> &L, double *c0t, cudaStream_t s)
{
    const dim3 g = grid3(L.nx, L.ny, L.nz, Launch{{false, false, false}}), bl(kBX, kBY, 1);
    k_diag_f64<<<g, bl, 0, s>>>(L, c0t);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "diagonal table");
}

int f64_residual(const LevelK<double> &L, const Launch &ln, double *r, const double *x, const double *b,
                 double *partials, int *npart, cudaStream_t s, const double *c0t)
{
    const dim3 g = grid3(L.nx, L.ny, L.nz, ln), bl(kBX, kBY, 1);
    if (partials) {
        if (c0t)
            k_residual_f64<true, true><<<g, bl, 0, s>>>(L, r, x, b, partials, c0t);
        else
            k_residual_f64<true, false><<<g, bl, 0, s>>>(L, r, x, b, partials, nullptr);
        *npart = (int)(g.x * g.y * g.z);
    } else if (c0t) {
        k_residual_f64<false, true><<<g, bl, 0, s>>>(L, r, x, b, nullptr, c0t);
    } else {
        k_residual_f64<false, false><<<g, bl, 0, s>>>(L, r, x, b, nullptr, nullptr);
    }
    count_launches(1);
    return cuda_status(cudaGetLastError(), "residual");
}

int f64_mv_mul(const LevelK<double> &L, const Launch &ln, double *y, const double *x, cudaStream_t s,
               const double *c0t)
{
    const dim3 g = grid3(L.nx, L.ny, L.nz, ln), bl(kBX, kBY, 1);
    if (c0t)
        k_mvmul_f64<true><<<g, bl, 0, s>>>(L, y, x, c0t);
    else
        k_mvmul_f64<false><<<g, bl, 0, s>>>(L, y, x, nullptr);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "mv_mul");
}

int f64_dot_partials(const LevelK<double> &L, const Launch &ln, const double *x, const double *y,
                     double *partials, int *npart, cudaStream_t s)
{
    const dim3 g = grid3(L.nx, L.ny, L.nz, ln), bl(kBX, kBY, 1);
    k_dot_f64<<<g, bl, 0, s>>>(L, x, y, partials);
    *npart = (int)(g.x * g.y * g.z);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "dot");
}

int f64_reduce(const double *partials, int n, double *out, cudaStream_t s)
{
    k_reduce_f64<<<1, 1024, 0, s>>>(partials, n, out);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "reduce");
}

int f64_restrict(const XferK<double> &X, const Launch &ln, const double *vf, double *vc, cudaStream_t s)
{
    const dim3 g = grid3(X.ncx, X.ncy, X.ncz, ln), bl(kBX, kBY, 1);
    k_restrict_f64<<<g, bl, 0, s>>>(X, vf, vc);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "restriction");
}

int f64_prolong(const XferK<double> &X, const Launch &ln, const double *vc, double *vf, bool add,
                cudaStream_t s)
{
    const dim3 g = grid3(X.ncx, X.ncy, X.ncz, ln), bl(kBX, kBY, 1);
    if (add)
        k_prolong_f64<true><<<g, bl, 0, s>>>(X, vc, vf);
    else
        k_prolong_f64<false><<<g, bl, 0, s>>>(X, vc, vf);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "prolongation");
}

int zero_ghosts_f64(double *a, int nx, int ny, int nz, cudaStream_t s)
{
    const long long total = 2LL * ((long long)(nx + 2) * (ny + 2) + (long long)(nx + 2) * (nz + 2) +
                                   (long long)(ny + 2) * (nz + 2));
    long long blocks = (total + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_zero_ghosts_f64<<<(unsigned)blocks, 256, 0, s>>>(a, nx, ny, nz);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "zero ghosts");
}

int hierarchy_setup(const HierDesc *dev_desc, double *meshes, double *tables, cudaStream_t s)
{
    k_hierarchy<<<3, 256, 0, s>>>(dev_desc, meshes, tables);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "hierarchy set-up");
}

int f64_tail(const TailDesc<double> *dev_desc, int threads, cudaStream_t s)
{
    k_tail_f64<<<1, threads, 0, s>>>(dev_desc);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "coarse tail");
}


// Grid of the fused CG kernels: the level's CTA tiles in x and y, and enough z planes per
// CTA that the grid is about four waves of 256-thread CTAs (at most 4864 CTAs, so the
// last CTA's sum over the partials stays short); collapsed axes keep one CTA column.
static dim3 cg_grid(const LevelK<double> &L, const Launch &ln)
{
    dim3 g = grid3(L.nx, L.ny, L.nz, ln);
    const unsigned plane = g.x * g.y;
    const unsigned target = 4864;
    unsigned gz = plane >= target ? 1u : (target + plane - 1) / plane;
    if (gz > g.z) gz = g.z;
    g.z = gz;
    return g;
}

int f64_cg_partials(const LevelK<double> &L, const Launch &ln)
{
    const dim3 g = cg_grid(L, ln);
    return (int)(g.x * g.y * g.z);
}

int f64_cg_init(const LevelK<double> &L, const Launch &ln, double *r, double *p, const double *x, const double *b,
                double *partials, CgState *st, cudaStream_t s, const double *c0t)
{
    if (c0t)
        k_cg_init<true><<<cg_grid(L, ln), dim3(kBX, kBY, 1), 0, s>>>(L, r, p, x, b, partials, st, c0t);
    else
        k_cg_init<false><<<cg_grid(L, ln), dim3(kBX, kBY, 1), 0, s>>>(L, r, p, x, b, partials, st, nullptr);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "cg init");
}

int f64_cg_iteration(const LevelK<double> &L, const Launch &ln, double *x, double *r, double *p, double *ap,
                     double *partials, CgState *st, double tol, bool check, int iter, cudaStream_t s,
                     const double *c0t)
{
    const dim3 g = cg_grid(L, ln), bl(kBX, kBY, 1);
    if (c0t)
        k_cg_apdot<true><<<g, bl, 0, s>>>(L, p, ap, partials, st, c0t);
    else
        k_cg_apdot<false><<<g, bl, 0, s>>>(L, p, ap, partials, st, nullptr);
    k_cg_update<<<g, bl, 0, s>>>(L, x, r, p, ap, partials, st, tol, check ? 1 : 0, iter);
    k_cg_p<<<g, bl, 0, s>>>(L, p, r, st);
    count_launches(3);
    return cuda_status(cudaGetLastError(), "cg iteration");
}

}  // namespace pmg
