/*
 * pmg_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C CPU restatement of the PEPS_MG multigrid V-cycle hot path, used as the
 * parity oracle for the CUDA implementation in peps_mg_gb300/csrc.  Only tests/,
 * __graft_entry__.smoke() and bench.py (cpu_baseline leg and --impl reference arm)
 * may load it, and only as the checker or as the timed CPU baseline; the product
 * never links or calls it.
 *
 * Parity status: PARITY UNPINNED by the reference itself.  The reference is
 * Fortran 90 + MPI (mpiifort, MKL link flags), ships no tests or golden vectors, and
 * no Fortran compiler exists where this project is built, so it could not be run.
 * The restatement is cross-checked instead against (a) an independent vectorised
 * numpy restatement (tests/golden/numpy_restatement.py, fixtures written by
 * tests/golden/make_golden.py) that must agree bit for bit, and (b) hand-derived
 * known answers of the reference formulas (tests/test_oracle_golden.py).
 *
 * Every function follows the loops and the floating-point operation order of the
 * reference expression it cites (files relative to the reference project root).
 * Build with -ffp-contract=off: the reference is compiled with -fp-model=precise for
 * an SSE2 target, i.e. without fused multiply-add.
 *
 * Arrays are Fortran-ordered (i fastest) with one ghost layer: (0:nx+1,0:ny+1,0:nz+1).
 * The coefficient array is coeff(0:6, nx, ny, nz) exactly as src/matrix.f90:62.
 *
 * With -fopenmp the k-loops run in parallel (this is the timed CPU baseline); the
 * reference's shared `ista`/`temp` race (src/rbgs_poisson_matrix.f90:120-134) is
 * fixed by declaring them inside the loop body.  Reductions are then order-dependent,
 * exactly as the reference's OpenMP reductions are; parity tests run one thread.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_EINVAL 1
#define ORC_ENOMEM 2

#define IDX(i, j, k, nx, ny) ((size_t)(i) + ((size_t)(nx) + 2) * ((size_t)(j) + ((size_t)(ny) + 2) * (size_t)(k)))
#define CO(c, i, j, k, nx, ny) ((size_t)(c) + 7 * ((size_t)((i) - 1) + (size_t)(nx) * ((size_t)((j) - 1) + (size_t)(ny) * (size_t)((k) - 1))))

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

static int imax3(const int *v)
{
    int m = v[0];
    if (v[1] > m) m = v[1];
    if (v[2] > m) m = v[2];
    return m;
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------------ */
/* Geometry: one axis of geometry_domain_create (src/geometry.f90:179-209).          */
/* ------------------------------------------------------------------------------ */

/* Fortran real**integer evaluated by repeated squaring (the usual lowering). */
static double ipow(double a, int n)
{
    double r = 1.0;
    double b = a;
    int e = n;
    if (e < 0) return 1.0 / ipow(a, -n);
    while (e > 0) {
        if (e & 1) r = r * b;
        e >>= 1;
        if (e) b = b * b;
    }
    return r;
}

void orc_mesh_axis(int n, double o, double l, double a, double *dxm, double *dxg, double *xg)
{
    int i;
    if (a == 1.0) {
        /* uniform grid, src/geometry.f90:180-189 */
        dxm[0] = 0.0;
        dxg[0] = 0.0;
        xg[0] = o;
        for (i = 1; i <= n; ++i) {
            dxm[i] = l / (double)n;
            dxg[i] = 0.5 * (dxm[i] + dxm[i - 1]);
            xg[i] = xg[i - 1] + dxg[i];
        }
        dxm[n + 1] = 0.0;
        dxg[n + 1] = 0.5 * (dxm[n + 1] + dxm[n]);
        xg[n + 1] = xg[n] + dxg[n + 1];
    } else {
        /* symmetric geometric stretch, src/geometry.f90:190-209 */
        dxm[0] = 0.0;
        dxm[1] = 0.5 * l * (a - 1.0) / (ipow(a, n / 2) - 1.0);
        for (i = 2; i <= n / 2; ++i) {
            dxm[i] = dxm[i - 1] * a;
            dxm[n - i + 1] = dxm[i];
        }
        dxm[n] = dxm[1];
        dxm[n + 1] = 0.0;
        dxg[0] = 0.0;
        xg[0] = o;
        for (i = 1; i <= n; ++i) {
            dxg[i] = 0.5 * (dxm[i] + dxm[i - 1]);
            xg[i] = xg[i - 1] + dxg[i];
        }
        dxg[n + 1] = 0.5 * (dxm[n + 1] + dxm[n]);
        xg[n + 1] = xg[n] + dxg[n + 1];
    }
}

/* dxg/xg from given cell widths dxm(0:n+1) with the ghost widths already set, in the
 * form used for every coarse level (src/multigrid.f90:480-487). */
static void grid_from_widths(int n, double x0, const double *dxm, double *dxg, double *xg)
{
    int i;
    dxg[0] = 0.0;
    xg[0] = x0;
    for (i = 1; i <= n; ++i) {
        dxg[i] = 0.5 * (dxm[i] + dxm[i - 1]);
        xg[i] = xg[i - 1] + dxg[i];
    }
    dxg[n + 1] = 0.5 * (dxm[n + 1] + dxm[n]);
    xg[n + 1] = xg[n] + dxg[n + 1];
}

/* ------------------------------------------------------------------------------ */
/* Level-size rules at one MPI rank.                                                */
/*   CGS   src/multigrid.f90:183-299                                                 */
/*   CGA   src/multigrid.f90:527-742                                                 */
/*   CGPSA src/multigrid.f90:1024-1201 (aggregation levels forced to 0 at one rank,  */
/*         src/multigrid.f90:1032-1036)                                              */
/* sizes[3*l + d] for l = 1..n_levels (index 0 = finest); coarsest[d] = last level   */
/* at which axis d was halved (0 if never).  Returns ORC_EINVAL on the reference's   */
/* error conditions.                                                                */
/* ------------------------------------------------------------------------------ */
int orc_level_sizes(int nx, int ny, int nz, int n_levels, int method, int cga_level,
                    int *sizes, int *coarsest)
{
    int n[3] = {nx, ny, nz};
    int lvc[3] = {0, 0, 0};
    int l, d;
    if (n_levels <= 1) return ORC_EINVAL;                 /* src/multigrid.f90:101-107 */
    if (nx < 1 || ny < 1 || nz < 1) return ORC_EINVAL;
    sizes[0] = nx; sizes[1] = ny; sizes[2] = nz;
    for (l = 1; l <= n_levels; ++l)
        for (d = 0; d < 3; ++d) sizes[3 * l + d] = 0;

    if (method == 0) {
        if (cga_level != 0) return ORC_EINVAL;           /* src/multigrid.f90:190-195 */
        for (l = 1; l <= n_levels; ++l) {
            for (d = 0; d < 3; ++d) {
                if (n[d] % 2 == 0) { n[d] /= 2; lvc[d] = l; }
                /* odd: kept, allowed because one rank is always aggregated */
                sizes[3 * l + d] = n[d];
            }
        }
        if (n_levels > imax3(lvc)) return ORC_EINVAL;   /* src/multigrid.f90:302-309 */
    } else if (method == 1) {
        if (cga_level == 0) return ORC_EINVAL;           /* src/multigrid.f90:530-534 */
        for (l = 1; l <= n_levels; ++l) {
            for (d = 0; d < 3; ++d) {
                if (l < cga_level) {
                    if (n[d] % 2 == 1) return ORC_EINVAL; /* src/multigrid.f90:545-553 */
                    sizes[3 * l + d] = n[d] / 2;
                } else if (l == cga_level) {
                    if (n[d] % 2 == 1) return ORC_EINVAL; /* src/multigrid.f90:593-601 */
                    sizes[3 * l + d] = n[d] / 2;          /* x nprocs = 1 */
                    lvc[d] = l;
                } else {
                    if (n[d] % 2 == 1) sizes[3 * l + d] = n[d];
                    else { sizes[3 * l + d] = n[d] / 2; lvc[d] = l; }
                }
            }
            for (d = 0; d < 3; ++d) n[d] = sizes[3 * l + d];
            if (((long long)n[0] * n[1] * n[2]) % 2 == 1) break;   /* src/multigrid.f90:700-703 */
        }
        if (n_levels > imax3(lvc)) return ORC_EINVAL;   /* src/multigrid.f90:732-740 */
    } else if (method == 2) {
        for (l = 1; l <= n_levels; ++l) {
            for (d = 0; d < 3; ++d) {
                if (n[d] % 2 == 1) sizes[3 * l + d] = n[d];
                else { sizes[3 * l + d] = n[d] / 2; lvc[d] = l; }
            }
            for (d = 0; d < 3; ++d) n[d] = sizes[3 * l + d];
            if (((long long)n[0] * n[1] * n[2]) % 2 == 1) break;   /* src/multigrid.f90:1160-1163 */
        }
        if (n_levels != imax3(lvc)) return ORC_EINVAL;  /* src/multigrid.f90:1193-1201 */
    } else {
        return ORC_EINVAL;                                /* src/multigrid.f90:124-128 */
    }
    for (d = 0; d < 3; ++d) coarsest[d] = lvc[d];
    return ORC_OK;
}

/* ------------------------------------------------------------------------------ */
/* Mesh of a coarse level along one axis.                                            */
/*   CGS   multigrid_subdomain_CGS_make_grid, src/multigrid.f90:419-495              */
/*   CGA/CGPSA multigrid_subdomain_aggregation_make_grid, src/multigrid.f90:859-990  */
/* The three differ only in xg(0) beyond the aggregation level; dxm/dxg (which alone */
/* define the operator) are identical at one rank.                                  */
/* ------------------------------------------------------------------------------ */
void orc_coarsen_axis(int method, int agg_level, int n, const double *dxm_f, const double *dxg_f,
                      const double *xg_f, double ox, int lv, int lv_coarsest,
                      double *dxm, double *dxg, double *xg)
{
    int i;
    memset(dxm, 0, sizeof(double) * (size_t)(n + 2));
    memset(dxg, 0, sizeof(double) * (size_t)(n + 2));
    memset(xg, 0, sizeof(double) * (size_t)(n + 2));
    if (lv <= lv_coarsest) {
        double x0;
        for (i = 1; i <= n; ++i) dxm[i] = dxm_f[2 * i - 1] + dxm_f[2 * i];   /* :452-454 */
        dxm[0] = dxm_f[0];                                                  /* :462 */
        dxm[n + 1] = dxm_f[2 * n + 1];                                      /* :470 */
        if (method == 0 || (method == 1 && lv <= agg_level))
            x0 = ox - 0.5 * dxm[0];                                         /* :481, :926 */
        else
            x0 = (xg_f[0] + 0.5 * dxm_f[0]) - 0.5 * dxm[0];                  /* :945 */
        grid_from_widths(n, x0, dxm, dxg, xg);
    } else {
        for (i = 0; i <= n + 1; ++i) {                                      /* :489-491 */
            dxm[i] = dxm_f[i];
            dxg[i] = dxg_f[i];
            xg[i] = xg_f[i];
        }
    }
}

/* ------------------------------------------------------------------------------ */
/* matrix_heptadiagonal_create, src/matrix.f90:39-94                                */
/* ------------------------------------------------------------------------------ */
void orc_matrix_create(int nx, int ny, int nz, const double *dxm, const double *dxg,
                       const double *dym, const double *dyg, const double *dzm, const double *dzg,
                       double *coeff)
{
    int i, j, k;
    for (k = 1; k <= nz; ++k) {
        double dzmp2i = 1.0 / (dzm[k] * dzg[k]);
        double dzmn2i = 1.0 / (dzm[k] * dzg[k + 1]);
        for (j = 1; j <= ny; ++j) {
            double dymp2i = 1.0 / (dym[j] * dyg[j]);
            double dymn2i = 1.0 / (dym[j] * dyg[j + 1]);
            for (i = 1; i <= nx; ++i) {
                double dxmp2i = 1.0 / (dxm[i] * dxg[i]);
                double dxmn2i = 1.0 / (dxm[i] * dxg[i + 1]);
                double *c = coeff + CO(0, i, j, k, nx, ny);
                c[0] = -(dxmp2i + dxmn2i + dymp2i + dymn2i + dzmp2i + dzmn2i);
                c[1] = 1.0 * dxmp2i;
                c[2] = 1.0 * dxmn2i;
                c[3] = 1.0 * dymp2i;
                c[4] = 1.0 * dymn2i;
                c[5] = 1.0 * dzmp2i;
                c[6] = 1.0 * dzmn2i;
            }
        }
    }
}

/* ------------------------------------------------------------------------------ */
/* mv_mul_poisson_matrix, src/poisson_matrix_operator.f90:110-161                   */
/* ------------------------------------------------------------------------------ */
void orc_mv_mul(int nx, int ny, int nz, const double *coeff, const double *x, double *y)
{
    long long kk;
    size_t total = ((size_t)nx + 2) * ((size_t)ny + 2) * ((size_t)nz + 2);
    memset(y, 0, sizeof(double) * total);                     /* :136-143 */
#pragma omp parallel for schedule(static)
    for (kk = 1; kk <= nz; ++kk) {
        int k = (int)kk, i, j;
        for (j = 1; j <= ny; ++j)
            for (i = 1; i <= nx; ++i) {
                const double *c = coeff + CO(0, i, j, k, nx, ny);
                y[IDX(i, j, k, nx, ny)] = c[0] * x[IDX(i, j, k, nx, ny)]
                                        + c[1] * x[IDX(i - 1, j, k, nx, ny)]
                                        + c[2] * x[IDX(i + 1, j, k, nx, ny)]
                                        + c[3] * x[IDX(i, j - 1, k, nx, ny)]
                                        + c[4] * x[IDX(i, j + 1, k, nx, ny)]
                                        + c[5] * x[IDX(i, j, k - 1, nx, ny)]
                                        + c[6] * x[IDX(i, j, k + 1, nx, ny)];
            }
    }
}

/* ------------------------------------------------------------------------------ */
/* vv_dot_3d_matrix, src/poisson_matrix_operator.f90:40-99 (one rank: no allreduce)  */
/* ------------------------------------------------------------------------------ */
double orc_vv_dot(int nx, int ny, int nz, const double *x, const double *y)
{
    double result_local = 0.0;
    long long kk;
#pragma omp parallel for schedule(static) reduction(+ : result_local)
    for (kk = 1; kk <= nz; ++kk) {
        int k = (int)kk, i, j;
        for (j = 1; j <= ny; ++j)
            for (i = 1; i <= nx; ++i)
                result_local = result_local + x[IDX(i, j, k, nx, ny)] * y[IDX(i, j, k, nx, ny)];
    }
    return result_local;
}

/* ------------------------------------------------------------------------------ */
/* multigrid_residual, src/multigrid.f90:1782-1807: r = b - A x, ghosts of r = 0    */
/* ------------------------------------------------------------------------------ */
void orc_residual(int nx, int ny, int nz, const double *coeff, const double *x, const double *b,
                  double *r)
{
    long long kk;
    orc_mv_mul(nx, ny, nz, coeff, x, r);
#pragma omp parallel for schedule(static)
    for (kk = 1; kk <= nz; ++kk) {
        int k = (int)kk, i, j;
        for (j = 1; j <= ny; ++j)
            for (i = 1; i <= nx; ++i)
                r[IDX(i, j, k, nx, ny)] = b[IDX(i, j, k, nx, ny)] - r[IDX(i, j, k, nx, ny)];
    }
}

/* One colour of the red-black sweep: src/rbgs_poisson_matrix.f90:239-253 (first,
 * colour 0) and :257-271 (second, colour 1).  First colour starts at
 * ista = 1 + mod(j+k+offset, 2). */
static void rbgs_colour(int nx, int ny, int nz, const double *coeff, double *sol, const double *rhs,
                        double omega, int colour, int offset)
{
    long long kk;
#pragma omp parallel for schedule(static)
    for (kk = 1; kk <= nz; ++kk) {
        int k = (int)kk, i, j;
        for (j = 1; j <= ny; ++j) {
            int ista = 1 + (j + k + colour + offset) % 2;
            for (i = ista; i <= nx; i += 2) {
                const double *c = coeff + CO(0, i, j, k, nx, ny);
                double temp = c[1] * sol[IDX(i - 1, j, k, nx, ny)]
                            + c[2] * sol[IDX(i + 1, j, k, nx, ny)]
                            + c[3] * sol[IDX(i, j - 1, k, nx, ny)]
                            + c[4] * sol[IDX(i, j + 1, k, nx, ny)]
                            + c[5] * sol[IDX(i, j, k - 1, nx, ny)]
                            + c[6] * sol[IDX(i, j, k + 1, nx, ny)];
                size_t p = IDX(i, j, k, nx, ny);
                sol[p] = omega * (rhs[p] - temp) / c[0] + (1.0 - omega) * sol[p];
            }
        }
    }
}

/* rbgs_iterator_poisson_matrix, src/rbgs_poisson_matrix.f90:191-279 (offset = 0 at
 * one rank, :230-232) */
void orc_rbgs_iterator(int nx, int ny, int nz, const double *coeff, double *sol, const double *rhs,
                       int maxiteration, double omega)
{
    int iter;
    for (iter = 0; iter < maxiteration; ++iter) {
        rbgs_colour(nx, ny, nz, coeff, sol, rhs, omega, 0, 0);
        rbgs_colour(nx, ny, nz, coeff, sol, rhs, omega, 1, 0);
    }
}

/* rbgs_solver_poisson_matrix, src/rbgs_poisson_matrix.f90:47-179.  Returns the
 * iteration counter as the reference leaves it (the exit iteration, or maxiteration
 * when the loop ran out).  rsd is caller-provided scratch of the full array size. */
int orc_rbgs_solver(int nx, int ny, int nz, const double *coeff, double *sol, const double *rhs,
                    int maxiteration, double tolerance, double omega, double *rsd,
                    double *out_norm2, double *out_norm02)
{
    int iter;
    double rsd0tol, rsd_norm;
    orc_residual(nx, ny, nz, coeff, sol, rhs, rsd);             /* :73-81 */
    rsd0tol = orc_vv_dot(nx, ny, nz, rsd, rsd);
    rsd_norm = rsd0tol;
    for (iter = 0; iter < maxiteration; ++iter) {
        rbgs_colour(nx, ny, nz, coeff, sol, rhs, omega, 0, 0);
        rbgs_colour(nx, ny, nz, coeff, sol, rhs, omega, 1, 0);
        orc_residual(nx, ny, nz, coeff, sol, rhs, rsd);          /* :154-164 */
        rsd_norm = orc_vv_dot(nx, ny, nz, rsd, rsd);
        if (sqrt(rsd_norm / rsd0tol) <= tolerance) break;       /* :167 */
    }
    if (out_norm2) *out_norm2 = rsd_norm;
    if (out_norm02) *out_norm02 = rsd0tol;
    return iter;
}

/* CG update loops of src/cg_poisson_matrix.f90:113-121 and :130-137 */
static void cg_update_xr(int nx, int ny, int nz, double alpha, double *sol, double *rsd,
                         const double *p, const double *ap)
{
    long long kk;
#pragma omp parallel for schedule(static)
    for (kk = 1; kk <= nz; ++kk) {
        int k = (int)kk, i, j;
        for (j = 1; j <= ny; ++j)
            for (i = 1; i <= nx; ++i) {
                size_t q = IDX(i, j, k, nx, ny);
                sol[q] = sol[q] + alpha * p[q];
                rsd[q] = rsd[q] - alpha * ap[q];
            }
    }
}

static void cg_update_p(int nx, int ny, int nz, double beta, double *p, const double *rsd)
{
    long long kk;
#pragma omp parallel for schedule(static)
    for (kk = 1; kk <= nz; ++kk) {
        int k = (int)kk, i, j;
        for (j = 1; j <= ny; ++j)
            for (i = 1; i <= nx; ++i) {
                size_t q = IDX(i, j, k, nx, ny);
                p[q] = rsd[q] + beta * p[q];
            }
    }
}

/* cg_solver_poisson_matrix (check_tol = 1, src/cg_poisson_matrix.f90:47-146) and
 * cg_iterator_poisson_matrix (check_tol = 0, :157-241).  work holds 4 full arrays
 * (p, Ax, Ap, rsd), zeroed here as at :75-78. */
int orc_cg(int nx, int ny, int nz, const double *coeff, double *sol, const double *rhs,
           int maxiteration, double tolerance, int check_tol, double *work,
           double *out_norm2, double *out_norm02)
{
    size_t total = ((size_t)nx + 2) * ((size_t)ny + 2) * ((size_t)nz + 2);
    double *p = work, *ax = work + total, *ap = work + 2 * total, *rsd = work + 3 * total;
    double alpha, beta, temp1 = 0.0, temp2 = 0.0, rsd0tol = 0.0;
    int iter, i, j, k;
    memset(work, 0, sizeof(double) * 4 * total);
    orc_mv_mul(nx, ny, nz, coeff, sol, ax);                                  /* :81 */
    for (k = 1; k <= nz; ++k)
        for (j = 1; j <= ny; ++j)
            for (i = 1; i <= nx; ++i) {
                size_t q = IDX(i, j, k, nx, ny);
                rsd[q] = rhs[q] - ax[q];
                p[q] = rsd[q];
            }
    if (check_tol) rsd0tol = orc_vv_dot(nx, ny, nz, rsd, rsd);               /* :94 */
    for (iter = 0; iter < maxiteration; ++iter) {
        temp1 = orc_vv_dot(nx, ny, nz, rsd, rsd);                            /* :106 */
        orc_mv_mul(nx, ny, nz, coeff, p, ap);                                /* :108 */
        temp2 = orc_vv_dot(nx, ny, nz, ap, p);                               /* :109 */
        alpha = temp1 / temp2;
        cg_update_xr(nx, ny, nz, alpha, sol, rsd, p, ap);
        temp2 = orc_vv_dot(nx, ny, nz, rsd, rsd);                            /* :123 */
        if (check_tol && sqrt(temp2 / rsd0tol) < tolerance) break;           /* :126 */
        beta = temp2 / temp1;
        cg_update_p(nx, ny, nz, beta, p, rsd);
    }
    if (out_norm2) *out_norm2 = temp2;
    if (out_norm02) *out_norm02 = rsd0tol;
    return iter;
}

/* ------------------------------------------------------------------------------ */
/* multigrid_restriction, src/multigrid.f90:1345-1504                               */
/* level = index of the fine level; coarsest[] = last halving level per axis.       */
/* ------------------------------------------------------------------------------ */
void orc_restriction(int nxc, int nyc, int nzc, const double *dxm_c, const double *dym_c, const double *dzm_c,
                     int nxf, int nyf, int nzf, const double *dxm_f, const double *dym_f, const double *dzm_f,
                     int level, const int *coarsest, const double *val_f, double *val_c)
{
    double *dxf = (double *)calloc((size_t)nxf + 2, sizeof(double));
    double *dyf = (double *)calloc((size_t)nyf + 2, sizeof(double));
    double *dzf = (double *)calloc((size_t)nzf + 2, sizeof(double));
    int is, io, js, jo, ks, ko, i;
    long long kk;
    memset(val_c, 0, sizeof(double) * ((size_t)nxc + 2) * ((size_t)nyc + 2) * ((size_t)nzc + 2));   /* :1366 */
    if (level >= coarsest[0]) {                                             /* :1415-1425 */
        for (i = 0; i <= nxf + 1; ++i) dxf[i] = dxm_f[i];
        is = 1; io = 0;
    } else {
        for (i = 1; i <= nxf; ++i) dxf[i] = dxm_c[(i - 1) / 2 + 1] - dxm_f[i];
        is = 2; io = 1;
    }
    if (level >= coarsest[1]) {
        for (i = 0; i <= nyf + 1; ++i) dyf[i] = dym_f[i];
        js = 1; jo = 0;
    } else {
        for (i = 1; i <= nyf; ++i) dyf[i] = dym_c[(i - 1) / 2 + 1] - dym_f[i];
        js = 2; jo = 1;
    }
    if (level >= coarsest[2]) {
        for (i = 0; i <= nzf + 1; ++i) dzf[i] = dzm_f[i];
        ks = 1; ko = 0;
    } else {
        for (i = 1; i <= nzf; ++i) dzf[i] = dzm_c[(i - 1) / 2 + 1] - dzm_f[i];
        ks = 2; ko = 1;
    }
#pragma omp parallel for schedule(static)
    for (kk = 1; kk <= nzc; ++kk) {                                         /* :1461-1494 */
        int k = (int)kk, j, ii;
        int kp = k * ks, kz = kp - ko;
        for (j = 1; j <= nyc; ++j) {
            int jp = j * js, jz = jp - jo;
            for (ii = 1; ii <= nxc; ++ii) {
                int ip = ii * is, iz = ip - io;
                double v111 = dxf[iz] * dyf[jz] * dzf[kz];
                double v211 = dxf[ip] * dyf[jz] * dzf[kz];
                double v121 = dxf[iz] * dyf[jp] * dzf[kz];
                double v221 = dxf[ip] * dyf[jp] * dzf[kz];
                double v112 = dxf[iz] * dyf[jz] * dzf[kp];
                double v212 = dxf[ip] * dyf[jz] * dzf[kp];
                double v122 = dxf[iz] * dyf[jp] * dzf[kp];
                double v222 = dxf[ip] * dyf[jp] * dzf[kp];
                double vol_c = 0.0;
                vol_c = vol_c + v111; vol_c = vol_c + v211; vol_c = vol_c + v121; vol_c = vol_c + v221;
                vol_c = vol_c + v112; vol_c = vol_c + v212; vol_c = vol_c + v122; vol_c = vol_c + v222;
                val_c[IDX(ii, j, k, nxc, nyc)] =
                    (v111 * val_f[IDX(ip, jp, kp, nxf, nyf)]
                   + v211 * val_f[IDX(iz, jp, kp, nxf, nyf)]
                   + v121 * val_f[IDX(ip, jz, kp, nxf, nyf)]
                   + v221 * val_f[IDX(iz, jz, kp, nxf, nyf)]
                   + v112 * val_f[IDX(ip, jp, kz, nxf, nyf)]
                   + v212 * val_f[IDX(iz, jp, kz, nxf, nyf)]
                   + v122 * val_f[IDX(ip, jz, kz, nxf, nyf)]
                   + v222 * val_f[IDX(iz, jz, kz, nxf, nyf)]) / vol_c;
            }
        }
    }
    free(dxf); free(dyf); free(dzf);
}

/* Prolongation weights along one axis, src/multigrid.f90:1594-1649. */
static void prolong_weights(int nc, int nf, const double *dm_c, const double *dm_f, int stride1,
                            double *dp, double *dn)
{
    int i;
    memset(dp, 0, sizeof(double) * (size_t)(nf + 2));
    memset(dn, 0, sizeof(double) * (size_t)(nf + 2));
    if (stride1) {
        for (i = 0; i <= nc + 1; ++i) { dp[i] = dm_c[i]; dn[i] = dm_c[i]; }
    } else {
        for (i = 1; i <= nc; ++i) {
            int ipf = 2 * i;
            dp[ipf - 1] = 1.0 * dm_f[ipf - 2] + 0.5 * dm_f[ipf - 1];
            dp[ipf] = 0.5 * dm_f[ipf - 1];
            dn[ipf - 1] = 0.5 * dm_f[ipf];
            dn[ipf] = 1.0 * dm_f[ipf + 1] + 0.5 * dm_f[ipf];
        }
    }
}

/* ------------------------------------------------------------------------------ */
/* multigrid_prolongation_linear_on_nonuniform_grid, src/multigrid.f90:1516-1771    */
/* Writes the eight children of every coarse cell into val_f; nothing else of val_f */
/* is touched (val_f is intent(out) but only these elements are assigned).          */
/* ------------------------------------------------------------------------------ */
void orc_prolongation(int nxc, int nyc, int nzc, const double *dxm_c, const double *dym_c, const double *dzm_c,
                      int nxf, int nyf, int nzf, const double *dxm_f, const double *dym_f, const double *dzm_f,
                      int level, const int *coarsest, const double *val_c, double *val_f)
{
    int sx = level >= coarsest[0], sy = level >= coarsest[1], sz = level >= coarsest[2];
    int is = sx ? 1 : 2, io = sx ? 0 : 1;
    int js = sy ? 1 : 2, jo = sy ? 0 : 1;
    int ks = sz ? 1 : 2, ko = sz ? 0 : 1;
    double *dxp = (double *)malloc(sizeof(double) * ((size_t)nxf + 2));
    double *dxn = (double *)malloc(sizeof(double) * ((size_t)nxf + 2));
    double *dyp = (double *)malloc(sizeof(double) * ((size_t)nyf + 2));
    double *dyn = (double *)malloc(sizeof(double) * ((size_t)nyf + 2));
    double *dzp = (double *)malloc(sizeof(double) * ((size_t)nzf + 2));
    double *dzn = (double *)malloc(sizeof(double) * ((size_t)nzf + 2));
    long long kk;
    prolong_weights(nxc, nxf, dxm_c, dxm_f, sx, dxp, dxn);
    prolong_weights(nyc, nyf, dym_c, dym_f, sy, dyp, dyn);
    prolong_weights(nzc, nzf, dzm_c, dzm_f, sz, dzp, dzn);
#define VC(a, b, c) val_c[IDX(a, b, c, nxc, nyc)]
#pragma omp parallel for schedule(static)
    for (kk = 1; kk <= nzc; ++kk) {                                         /* :1652-1758 */
        int k = (int)kk, j, i;
        int kp = k * ks, kz = kp - ko, km = k - ko, kq = k + ko;
        for (j = 1; j <= nyc; ++j) {
            int jp = j * js, jz = jp - jo, jm = j - jo, jq = j + jo;
            for (i = 1; i <= nxc; ++i) {
                int ip = i * is, iz = ip - io, im = i - io, iq = i + io;
                val_f[IDX(iz, jz, kz, nxf, nyf)] =
                    (dxp[iz] * dyp[jz] * dzp[kz] * VC(i, j, k)
                   + dxp[ip] * dyp[jz] * dzp[kz] * VC(im, j, k)
                   + dxp[iz] * dyp[jp] * dzp[kz] * VC(i, jm, k)
                   + dxp[iz] * dyp[jz] * dzp[kp] * VC(i, j, km)
                   + dxp[ip] * dyp[jp] * dzp[kz] * VC(im, jm, k)
                   + dxp[ip] * dyp[jz] * dzp[kp] * VC(im, j, km)
                   + dxp[iz] * dyp[jp] * dzp[kp] * VC(i, jm, km)
                   + dxp[ip] * dyp[jp] * dzp[kp] * VC(im, jm, km))
                    / ((dxp[iz] + dxp[ip]) * (dyp[jz] + dyp[jp]) * (dzp[kz] + dzp[kp]));
                val_f[IDX(ip, jz, kz, nxf, nyf)] =
                    (dxn[ip] * dyp[jz] * dzp[kz] * VC(i, j, k)
                   + dxn[iz] * dyp[jz] * dzp[kz] * VC(iq, j, k)
                   + dxn[ip] * dyp[jp] * dzp[kz] * VC(i, jm, k)
                   + dxn[ip] * dyp[jz] * dzp[kp] * VC(i, j, km)
                   + dxn[iz] * dyp[jp] * dzp[kz] * VC(iq, jm, k)
                   + dxn[iz] * dyp[jz] * dzp[kp] * VC(iq, j, km)
                   + dxn[ip] * dyp[jp] * dzp[kp] * VC(i, jm, km)
                   + dxn[iz] * dyp[jp] * dzp[kp] * VC(iq, jm, km))
                    / ((dxn[iz] + dxn[ip]) * (dyp[jz] + dyp[jp]) * (dzp[kz] + dzp[kp]));
                val_f[IDX(iz, jp, kz, nxf, nyf)] =
                    (dxp[iz] * dyn[jp] * dzp[kz] * VC(i, j, k)
                   + dxp[ip] * dyn[jp] * dzp[kz] * VC(im, j, k)
                   + dxp[iz] * dyn[jz] * dzp[kz] * VC(i, jq, k)
                   + dxp[iz] * dyn[jp] * dzp[kp] * VC(i, j, km)
                   + dxp[ip] * dyn[jz] * dzp[kz] * VC(im, jq, k)
                   + dxp[ip] * dyn[jp] * dzp[kp] * VC(im, j, km)
                   + dxp[iz] * dyn[jz] * dzp[kp] * VC(i, jq, km)
                   + dxp[ip] * dyn[jz] * dzp[kp] * VC(im, jq, km))
                    / ((dxp[iz] + dxp[ip]) * (dyn[jz] + dyn[jp]) * (dzp[kz] + dzp[kp]));
                val_f[IDX(ip, jp, kz, nxf, nyf)] =
                    (dxn[ip] * dyn[jp] * dzp[kz] * VC(i, j, k)
                   + dxn[iz] * dyn[jp] * dzp[kz] * VC(iq, j, k)
                   + dxn[ip] * dyn[jz] * dzp[kz] * VC(i, jq, k)
                   + dxn[ip] * dyn[jp] * dzp[kp] * VC(i, j, km)
                   + dxn[iz] * dyn[jz] * dzp[kz] * VC(iq, jq, k)
                   + dxn[iz] * dyn[jp] * dzp[kp] * VC(iq, j, km)
                   + dxn[ip] * dyn[jz] * dzp[kp] * VC(i, jq, km)
                   + dxn[iz] * dyn[jz] * dzp[kp] * VC(iq, jq, km))
                    / ((dxn[iz] + dxn[ip]) * (dyn[jz] + dyn[jp]) * (dzp[kz] + dzp[kp]));
                val_f[IDX(iz, jz, kp, nxf, nyf)] =
                    (dxp[iz] * dyp[jz] * dzn[kp] * VC(i, j, k)
                   + dxp[ip] * dyp[jz] * dzn[kp] * VC(im, j, k)
                   + dxp[iz] * dyp[jp] * dzn[kp] * VC(i, jm, k)
                   + dxp[iz] * dyp[jz] * dzn[kz] * VC(i, j, kq)
                   + dxp[ip] * dyp[jp] * dzn[kp] * VC(im, jm, k)
                   + dxp[ip] * dyp[jz] * dzn[kz] * VC(im, j, kq)
                   + dxp[iz] * dyp[jp] * dzn[kz] * VC(i, jm, kq)
                   + dxp[ip] * dyp[jp] * dzn[kz] * VC(im, jm, kq))
                    / ((dxp[iz] + dxp[ip]) * (dyp[jz] + dyp[jp]) * (dzn[kz] + dzn[kp]));
                val_f[IDX(ip, jz, kp, nxf, nyf)] =
                    (dxn[ip] * dyp[jz] * dzn[kp] * VC(i, j, k)
                   + dxn[iz] * dyp[jz] * dzn[kp] * VC(iq, j, k)
                   + dxn[ip] * dyp[jp] * dzn[kp] * VC(i, jm, k)
                   + dxn[ip] * dyp[jz] * dzn[kz] * VC(i, j, kq)
                   + dxn[iz] * dyp[jp] * dzn[kp] * VC(iq, jm, k)
                   + dxn[iz] * dyp[jz] * dzn[kz] * VC(iq, j, kq)
                   + dxn[ip] * dyp[jp] * dzn[kz] * VC(i, jm, kq)
                   + dxn[iz] * dyp[jp] * dzn[kz] * VC(iq, jm, kq))
                    / ((dxn[iz] + dxn[ip]) * (dyp[jz] + dyp[jp]) * (dzn[kz] + dzn[kp]));
                val_f[IDX(iz, jp, kp, nxf, nyf)] =
                    (dxp[iz] * dyn[jp] * dzn[kp] * VC(i, j, k)
                   + dxp[ip] * dyn[jp] * dzn[kp] * VC(im, j, k)
                   + dxp[iz] * dyn[jz] * dzn[kp] * VC(i, jq, k)
                   + dxp[iz] * dyn[jp] * dzn[kz] * VC(i, j, kq)
                   + dxp[ip] * dyn[jz] * dzn[kp] * VC(im, jq, k)
                   + dxp[ip] * dyn[jp] * dzn[kz] * VC(im, j, kq)
                   + dxp[iz] * dyn[jz] * dzn[kz] * VC(i, jq, kq)
                   + dxp[ip] * dyn[jz] * dzn[kz] * VC(im, jq, kq))
                    / ((dxp[iz] + dxp[ip]) * (dyn[jz] + dyn[jp]) * (dzn[kz] + dzn[kp]));
                val_f[IDX(ip, jp, kp, nxf, nyf)] =
                    (dxn[ip] * dyn[jp] * dzn[kp] * VC(i, j, k)
                   + dxn[iz] * dyn[jp] * dzn[kp] * VC(iq, j, k)
                   + dxn[ip] * dyn[jz] * dzn[kp] * VC(i, jq, k)
                   + dxn[ip] * dyn[jp] * dzn[kz] * VC(i, j, kq)
                   + dxn[iz] * dyn[jz] * dzn[kp] * VC(iq, jq, k)
                   + dxn[iz] * dyn[jp] * dzn[kz] * VC(iq, j, kq)
                   + dxn[ip] * dyn[jz] * dzn[kz] * VC(i, jq, kq)
                   + dxn[iz] * dyn[jz] * dzn[kz] * VC(iq, jq, kq))
                    / ((dxn[iz] + dxn[ip]) * (dyn[jz] + dyn[jp]) * (dzn[kz] + dzn[kp]));
            }
        }
    }
#undef VC
    free(dxp); free(dxn); free(dyp); free(dyn); free(dzp); free(dzn);
}

/* ------------------------------------------------------------------------------ */
/* Multigrid state (module globals of src/multigrid.f90:40-55 made explicit).       */
/* ------------------------------------------------------------------------------ */
typedef struct {
    int nx, ny, nz;
    double *dm[3], *dg[3], *xg[3];   /* per axis, length n+2 */
    double *coeff;                   /* (0:6, nx, ny, nz) */
    double *x, *b, *r;               /* (0:n+1)^3 */
} orc_level;

typedef struct {
    int n_levels, n_vcycles, method, cga_level, coarse_solver;
    int coarsest[3];
    orc_level *lv;                   /* lv[0] = finest (caller's subdomain), 1..n_levels */
    double *work;                    /* coarse-solver scratch */
} orc_mg;

static size_t lv_total(const orc_level *L)
{
    return ((size_t)L->nx + 2) * ((size_t)L->ny + 2) * ((size_t)L->nz + 2);
}

void orc_mg_destroy(orc_mg *mg)
{
    int l, d;
    if (!mg) return;
    if (mg->lv) {
        for (l = 0; l <= mg->n_levels; ++l) {
            orc_level *L = &mg->lv[l];
            for (d = 0; d < 3; ++d) { free(L->dm[d]); free(L->dg[d]); free(L->xg[d]); }
            free(L->coeff); free(L->x); free(L->b); free(L->r);
        }
        free(mg->lv);
    }
    free(mg->work);
    free(mg);
}

/* multigrid_create, src/multigrid.f90:75-159, for one rank.  The finest mesh arrays
 * (length n+2 each, Fortran index 0..n+1) are those of the caller's subdomain; the
 * finest coefficient matrix is built here as main_peps.f90:162 does.
 * coarse_solver: 0 = RBGS solver (the reference's choice), 1 = CG solver. */
orc_mg *orc_mg_create(int nx, int ny, int nz,
                      const double *dxm, const double *dxg, const double *xg,
                      const double *dym, const double *dyg, const double *yg,
                      const double *dzm, const double *dzg, const double *zg,
                      int n_levels, int n_vcycles, int method, int cga_level,
                      int coarse_solver, int *err)
{
    orc_mg *mg;
    int *sizes, l, d, rc;
    size_t maxtot = 0;
    const double *fm[3] = {dxm, dym, dzm}, *fg[3] = {dxg, dyg, dzg}, *fx[3] = {xg, yg, zg};
    double o[3];
    *err = ORC_EINVAL;
    if (n_levels <= 1) return NULL;
    sizes = (int *)calloc((size_t)(n_levels + 1) * 3, sizeof(int));
    mg = (orc_mg *)calloc(1, sizeof(orc_mg));
    rc = orc_level_sizes(nx, ny, nz, n_levels, method, cga_level, sizes, mg->coarsest);
    if (rc != ORC_OK) { free(sizes); free(mg); return NULL; }
    mg->n_levels = n_levels; mg->n_vcycles = n_vcycles; mg->method = method;
    mg->cga_level = cga_level; mg->coarse_solver = coarse_solver;
    mg->lv = (orc_level *)calloc((size_t)n_levels + 1, sizeof(orc_level));
    for (l = 0; l <= n_levels; ++l) {
        orc_level *L = &mg->lv[l];
        int n[3];
        L->nx = sizes[3 * l]; L->ny = sizes[3 * l + 1]; L->nz = sizes[3 * l + 2];
        n[0] = L->nx; n[1] = L->ny; n[2] = L->nz;
        for (d = 0; d < 3; ++d) {
            L->dm[d] = (double *)calloc((size_t)n[d] + 2, sizeof(double));
            L->dg[d] = (double *)calloc((size_t)n[d] + 2, sizeof(double));
            L->xg[d] = (double *)calloc((size_t)n[d] + 2, sizeof(double));
            if (l == 0) {
                memcpy(L->dm[d], fm[d], sizeof(double) * ((size_t)n[d] + 2));
                memcpy(L->dg[d], fg[d], sizeof(double) * ((size_t)n[d] + 2));
                memcpy(L->xg[d], fx[d], sizeof(double) * ((size_t)n[d] + 2));
                o[d] = fx[d][1] - 0.5 * fm[d][1];      /* sdm%ox, src/geometry.f90:378-380 */
            } else {
                const orc_level *F = &mg->lv[l - 1];
                orc_coarsen_axis(method, cga_level, n[d], F->dm[d], F->dg[d], F->xg[d], o[d], l,
                                 mg->coarsest[d], L->dm[d], L->dg[d], L->xg[d]);
            }
        }
        L->coeff = (double *)calloc((size_t)7 * n[0] * n[1] * n[2], sizeof(double));
        orc_matrix_create(L->nx, L->ny, L->nz, L->dm[0], L->dg[0], L->dm[1], L->dg[1], L->dm[2], L->dg[2],
                          L->coeff);
        if (l > 0) {                                   /* src/multigrid.f90:1293-1314 */
            L->x = (double *)calloc(lv_total(L), sizeof(double));
            L->b = (double *)calloc(lv_total(L), sizeof(double));
            L->r = (double *)calloc(lv_total(L), sizeof(double));
            if (lv_total(L) > maxtot) maxtot = lv_total(L);
        }
    }
    mg->work = (double *)calloc(4 * maxtot, sizeof(double));
    free(sizes);
    *err = ORC_OK;
    return mg;
}

void orc_mg_level_dims(const orc_mg *mg, int l, int *dims)
{
    dims[0] = mg->lv[l].nx; dims[1] = mg->lv[l].ny; dims[2] = mg->lv[l].nz;
}

void orc_mg_coarsest(const orc_mg *mg, int *c)
{
    c[0] = mg->coarsest[0]; c[1] = mg->coarsest[1]; c[2] = mg->coarsest[2];
}

/* Copy out a level's mesh (axis d): dm, dg, xg each of length n+2. */
void orc_mg_level_mesh(const orc_mg *mg, int l, int d, double *dm, double *dg, double *xg)
{
    int n = d == 0 ? mg->lv[l].nx : d == 1 ? mg->lv[l].ny : mg->lv[l].nz;
    memcpy(dm, mg->lv[l].dm[d], sizeof(double) * ((size_t)n + 2));
    memcpy(dg, mg->lv[l].dg[d], sizeof(double) * ((size_t)n + 2));
    memcpy(xg, mg->lv[l].xg[d], sizeof(double) * ((size_t)n + 2));
}

const double *orc_mg_level_coeff(const orc_mg *mg, int l) { return mg->lv[l].coeff; }
double *orc_mg_level_x(orc_mg *mg, int l) { return mg->lv[l].x; }
double *orc_mg_level_b(orc_mg *mg, int l) { return mg->lv[l].b; }
double *orc_mg_level_r(orc_mg *mg, int l) { return mg->lv[l].r; }

static void restrict_lv(orc_mg *mg, int l, const double *val_f, double *val_c)
{
    const orc_level *F = &mg->lv[l], *C = &mg->lv[l + 1];
    orc_restriction(C->nx, C->ny, C->nz, C->dm[0], C->dm[1], C->dm[2],
                    F->nx, F->ny, F->nz, F->dm[0], F->dm[1], F->dm[2], l, mg->coarsest, val_f, val_c);
}

static void prolong_lv(orc_mg *mg, int l, const double *val_c, double *val_f)
{
    const orc_level *F = &mg->lv[l], *C = &mg->lv[l + 1];
    orc_prolongation(C->nx, C->ny, C->nz, C->dm[0], C->dm[1], C->dm[2],
                     F->nx, F->ny, F->nz, F->dm[0], F->dm[1], F->dm[2], l, mg->coarsest, val_c, val_f);
}

/* whole-array x = x + r (src/multigrid.f90:1958, 1966) */
static void add_inplace(size_t total, double *x, const double *r)
{
    size_t q;
    for (q = 0; q < total; ++q) x[q] = x[q] + r[q];
}

/* multigrid_solve_coarset_level, src/multigrid.f90:1819-1851; returns the solver's
 * iteration count (0 for the one-cell direct solve). */
static int solve_coarsest(orc_mg *mg, double tolerance, double omega)
{
    orc_level *L = &mg->lv[mg->n_levels];
    memset(L->x, 0, sizeof(double) * lv_total(L));
    if (L->nx * L->ny * L->nz == 1) {
        L->x[IDX(1, 1, 1, 1, 1)] = L->b[IDX(1, 1, 1, 1, 1)] / L->coeff[0];
        return 0;
    }
    if (mg->coarse_solver == 1)
        return orc_cg(L->nx, L->ny, L->nz, L->coeff, L->x, L->b, 1000, tolerance, 1, mg->work, NULL, NULL);
    return orc_rbgs_solver(L->nx, L->ny, L->nz, L->coeff, L->x, L->b, 1000, tolerance, omega, mg->work,
                           NULL, NULL);
}

/* multigrid_solve_vcycle (src/multigrid.f90:1864-1894) for one rank, where CGS
 * (:1907-1976), CGA (:1990-2173) and CGPSA (:2187-2718) execute the same sequence of
 * operations.  sol/rsd/rhs are (0:nx+1)^3 arrays of the finest level.
 * hist receives 3 doubles per completed cycle: sqrt(rsd_val), sqrt(res0tol),
 * sqrt(rsd_val/res0tol) as printed at :1972.  coarse_iters receives one count per
 * cycle.  Returns the number of cycles run. */
int orc_mg_solve(orc_mg *mg, double *sol, double *rsd, const double *rhs, int maxiteration,
                 double tolerance, double omega, double *hist, int *coarse_iters)
{
    orc_level *S = &mg->lv[0];
    int nl = mg->n_levels, l, cyc, ncyc = 0;
    double res0tol, rsd_val;
    orc_residual(S->nx, S->ny, S->nz, S->coeff, sol, rhs, rsd);             /* :1924 */
    res0tol = orc_vv_dot(S->nx, S->ny, S->nz, rsd, rsd);                    /* :1925 */
    for (cyc = 1; cyc <= mg->n_vcycles; ++cyc) {
        double ratio;
        int ci;
        orc_rbgs_iterator(S->nx, S->ny, S->nz, S->coeff, sol, rhs, maxiteration, omega);   /* :1931 */
        orc_residual(S->nx, S->ny, S->nz, S->coeff, sol, rhs, rsd);
        restrict_lv(mg, 0, rsd, mg->lv[1].b);
        for (l = 1; l <= nl - 1; ++l) {                                    /* :1936-1941 */
            orc_level *L = &mg->lv[l];
            memset(L->x, 0, sizeof(double) * lv_total(L));
            orc_rbgs_iterator(L->nx, L->ny, L->nz, L->coeff, L->x, L->b, maxiteration, omega);
            orc_residual(L->nx, L->ny, L->nz, L->coeff, L->x, L->b, L->r);
            restrict_lv(mg, l, L->r, mg->lv[l + 1].b);
        }
        ci = solve_coarsest(mg, tolerance, omega);                           /* :1944-1949 */
        if (coarse_iters) coarse_iters[cyc - 1] = ci;
        for (l = nl - 1; l >= 1; --l) {                                    /* :1957-1962 */
            orc_level *L = &mg->lv[l];
            prolong_lv(mg, l, mg->lv[l + 1].x, L->r);
            add_inplace(lv_total(L), L->x, L->r);
            orc_rbgs_iterator(L->nx, L->ny, L->nz, L->coeff, L->x, L->b, maxiteration, omega);
        }
        prolong_lv(mg, 0, mg->lv[1].x, rsd);                                /* :1965 */
        add_inplace(lv_total(S), sol, rsd);                                  /* :1966 */
        orc_rbgs_iterator(S->nx, S->ny, S->nz, S->coeff, sol, rhs, maxiteration, omega);
        orc_residual(S->nx, S->ny, S->nz, S->coeff, sol, rhs, rsd);         /* :1970 */
        rsd_val = orc_vv_dot(S->nx, S->ny, S->nz, rsd, rsd);
        ratio = sqrt(rsd_val / res0tol);
        if (hist) {
            hist[3 * (cyc - 1) + 0] = sqrt(rsd_val);
            hist[3 * (cyc - 1) + 1] = sqrt(res0tol);
            hist[3 * (cyc - 1) + 2] = ratio;
        }
        ncyc = cyc;
        if (ratio < tolerance) break;                                       /* :1973 */
    }
    return ncyc;
}

/* ------------------------------------------------------------------------------ */
/* Several ranks: the CGS V-cycle of src/multigrid.f90:1907-1976 on a px x py x pz  */
/* Cartesian decomposition (src/mpi_topology.f90:53-99, src/geometry.f90), every     */
/* rank simulated in this process.  Each rank holds its subdomain's hierarchy; the   */
/* ghost layers facing a neighbour are filled by the halo exchange of               */
/* geometry_halocell_update_selectively (src/geometry.f90:621-660: x, then y, then  */
/* z, full planes) at the points where the reference calls it: before each RBGS     */
/* colour (src/rbgs_poisson_matrix.f90:237,255 and :116,134), before every          */
/* mv_mul (src/poisson_matrix_operator.f90:131-133, so in every residual), and after */
/* the post-smoothing of each coarse level (src/multigrid.f90:1961).  Dot products   */
/* are local sums added over the ranks in rank order (the MPI_Allreduce of          */
/* src/poisson_matrix_operator.f90:68-97).  The RBGS colour of a rank starts at the  */
/* parity offset of src/rbgs_poisson_matrix.f90:230-232.                             */
/*                                                                                  */
/* Level sizes follow the multi-rank CGS rule (src/multigrid.f90:221-299): an axis   */
/* split over several ranks must halve at every level (an odd local size stops the  */
/* reference).  A rank's coarse meshes are the global coarse meshes restricted to    */
/* its cells, ghost widths from the neighbours (src/multigrid.f90:452-477), so they  */
/* are built here by slicing the one-rank hierarchy of the global mesh.              */
/* Ranks are numbered x fastest.  The finest post-smoothing uses the finest level's  */
/* partition flags: the reference reads mg_sdm(0) there, one element before that     */
/* array (src/multigrid.f90:1967), which with bounds checks off is not defined.      */
/* ------------------------------------------------------------------------------ */
typedef struct {
    int p[3], nr;
    int n_levels, n_vcycles, coarse_solver;
    orc_mg *glob;          /* one-rank hierarchy of the global mesh (meshes only) */
    orc_mg **rk;           /* per rank */
    int (*c)[3];           /* rank coordinates */
    double **sol, **rsd, **rhs;
} orc_dd;

static int dd_rank(const orc_dd *dd, int cx, int cy, int cz) { return cx + dd->p[0] * (cy + dd->p[1] * cz); }

void orc_dd_destroy(orc_dd *dd)
{
    int r;
    if (!dd) return;
    for (r = 0; r < dd->nr; ++r) {
        if (dd->rk) orc_mg_destroy(dd->rk[r]);
        if (dd->sol) free(dd->sol[r]);
        if (dd->rsd) free(dd->rsd[r]);
        if (dd->rhs) free(dd->rhs[r]);
    }
    free(dd->rk); free(dd->sol); free(dd->rsd); free(dd->rhs); free(dd->c);
    orc_mg_destroy(dd->glob);
    free(dd);
}

/* Level sizes of one rank under the multi-rank CGS rule; returns ORC_EINVAL where the
 * reference stops (a split axis with an odd local size, or more levels than any axis
 * allows, :302-309).  nloc: the rank's finest sizes. */
static int dd_level_sizes(const int nloc[3], const int p[3], int n_levels, int *sizes, int coarsest[3])
{
    int n[3] = {nloc[0], nloc[1], nloc[2]}, l, d;
    coarsest[0] = coarsest[1] = coarsest[2] = 0;
    for (d = 0; d < 3; ++d) sizes[d] = n[d];
    for (l = 1; l <= n_levels; ++l)
        for (d = 0; d < 3; ++d) {
            if (n[d] % 2 == 0) { n[d] /= 2; coarsest[d] = l; }
            else if (p[d] > 1) return ORC_EINVAL;
            sizes[3 * l + d] = n[d];
        }
    if (n_levels > imax3(coarsest)) return ORC_EINVAL;
    return ORC_OK;
}

/* The rank's hierarchy: its level sizes, meshes sliced from the global hierarchy and its
 * coefficient matrices (built from those meshes as src/matrix.f90:39-94 does). */
static orc_mg *dd_rank_mg(const orc_dd *dd, const int *sizes, const int coarsest[3], const int c[3])
{
    orc_mg *mg = (orc_mg *)calloc(1, sizeof(orc_mg));
    size_t maxtot = 0;
    int l, d;
    mg->n_levels = dd->n_levels; mg->n_vcycles = dd->n_vcycles; mg->method = 0;
    mg->coarse_solver = dd->coarse_solver;
    for (d = 0; d < 3; ++d) mg->coarsest[d] = coarsest[d];
    mg->lv = (orc_level *)calloc((size_t)dd->n_levels + 1, sizeof(orc_level));
    for (l = 0; l <= dd->n_levels; ++l) {
        orc_level *L = &mg->lv[l];
        const orc_level *G = &dd->glob->lv[l];
        int n[3];
        L->nx = sizes[3 * l]; L->ny = sizes[3 * l + 1]; L->nz = sizes[3 * l + 2];
        n[0] = L->nx; n[1] = L->ny; n[2] = L->nz;
        for (d = 0; d < 3; ++d) {
            const int off = c[d] * n[d];       /* global index of the rank's ghost cell 0 */
            L->dm[d] = (double *)malloc(sizeof(double) * ((size_t)n[d] + 2));
            L->dg[d] = (double *)malloc(sizeof(double) * ((size_t)n[d] + 2));
            L->xg[d] = (double *)malloc(sizeof(double) * ((size_t)n[d] + 2));
            memcpy(L->dm[d], G->dm[d] + off, sizeof(double) * ((size_t)n[d] + 2));
            memcpy(L->dg[d], G->dg[d] + off, sizeof(double) * ((size_t)n[d] + 2));
            memcpy(L->xg[d], G->xg[d] + off, sizeof(double) * ((size_t)n[d] + 2));
        }
        L->coeff = (double *)calloc((size_t)7 * n[0] * n[1] * n[2], sizeof(double));
        orc_matrix_create(L->nx, L->ny, L->nz, L->dm[0], L->dg[0], L->dm[1], L->dg[1], L->dm[2], L->dg[2],
                          L->coeff);
        if (l > 0) {
            L->x = (double *)calloc(lv_total(L), sizeof(double));
            L->b = (double *)calloc(lv_total(L), sizeof(double));
            L->r = (double *)calloc(lv_total(L), sizeof(double));
        }
        if (lv_total(L) > maxtot) maxtot = lv_total(L);
    }
    mg->work = (double *)calloc(4 * maxtot, sizeof(double));
    return mg;
}

/* multigrid_create on every rank of a px x py x pz decomposition of the global mesh
 * (global sizes divisible by the rank counts).  *err: ORC_EINVAL where the reference
 * stops. */
orc_dd *orc_dd_create(int nx, int ny, int nz,
                      const double *dxm, const double *dxg, const double *xg,
                      const double *dym, const double *dyg, const double *yg,
                      const double *dzm, const double *dzg, const double *zg,
                      int px, int py, int pz, int n_levels, int n_vcycles, int coarse_solver, int *err)
{
    orc_dd *dd;
    int *sizes, coarsest[3], nloc[3], r, cx, cy, cz, gerr = 0;
    *err = ORC_EINVAL;
    if (px < 1 || py < 1 || pz < 1 || nx % px || ny % py || nz % pz) return NULL;
    nloc[0] = nx / px; nloc[1] = ny / py; nloc[2] = nz / pz;
    dd = (orc_dd *)calloc(1, sizeof(orc_dd));
    dd->p[0] = px; dd->p[1] = py; dd->p[2] = pz;
    dd->nr = px * py * pz;
    dd->n_levels = n_levels; dd->n_vcycles = n_vcycles; dd->coarse_solver = coarse_solver;
    sizes = (int *)calloc((size_t)(n_levels + 1) * 3, sizeof(int));
    if (n_levels <= 1 || dd_level_sizes(nloc, dd->p, n_levels, sizes, coarsest) != ORC_OK) {
        free(sizes); free(dd); return NULL;
    }
    dd->glob = orc_mg_create(nx, ny, nz, dxm, dxg, xg, dym, dyg, yg, dzm, dzg, zg, n_levels, n_vcycles, 0, 0,
                             coarse_solver, &gerr);
    if (!dd->glob) { free(sizes); free(dd); return NULL; }
    dd->rk = (orc_mg **)calloc((size_t)dd->nr, sizeof(orc_mg *));
    dd->c = (int (*)[3])calloc((size_t)dd->nr, sizeof(int[3]));
    dd->sol = (double **)calloc((size_t)dd->nr, sizeof(double *));
    dd->rsd = (double **)calloc((size_t)dd->nr, sizeof(double *));
    dd->rhs = (double **)calloc((size_t)dd->nr, sizeof(double *));
    for (cz = 0; cz < pz; ++cz)
        for (cy = 0; cy < py; ++cy)
            for (cx = 0; cx < px; ++cx) {
                r = dd_rank(dd, cx, cy, cz);
                dd->c[r][0] = cx; dd->c[r][1] = cy; dd->c[r][2] = cz;
                dd->rk[r] = dd_rank_mg(dd, sizes, coarsest, dd->c[r]);
                dd->sol[r] = (double *)calloc(lv_total(&dd->rk[r]->lv[0]), sizeof(double));
                dd->rsd[r] = (double *)calloc(lv_total(&dd->rk[r]->lv[0]), sizeof(double));
                dd->rhs[r] = (double *)calloc(lv_total(&dd->rk[r]->lv[0]), sizeof(double));
            }
    free(sizes);
    *err = ORC_OK;
    return dd;
}

/* level arrays of every rank: which = 0 x, 1 b, 2 r (levels >= 1) */
static double *dd_arr(orc_dd *dd, int r, int l, int which)
{
    orc_level *L = &dd->rk[r]->lv[l];
    return which == 0 ? L->x : which == 1 ? L->b : L->r;
}

/* plane `idx` along axis d of a (0:n+1)^3 array, every index of the other two axes */
static void dd_copy_plane(int d, const int n[3], double *dst, int dst_idx, const double *src, int src_idx)
{
    int a, b;
    if (d == 0) {
        for (b = 0; b <= n[2] + 1; ++b)
            for (a = 0; a <= n[1] + 1; ++a) dst[IDX(dst_idx, a, b, n[0], n[1])] = src[IDX(src_idx, a, b, n[0], n[1])];
    } else if (d == 1) {
        for (b = 0; b <= n[2] + 1; ++b)
            for (a = 0; a <= n[0] + 1; ++a) dst[IDX(a, dst_idx, b, n[0], n[1])] = src[IDX(a, src_idx, b, n[0], n[1])];
    } else {
        for (b = 0; b <= n[1] + 1; ++b)
            for (a = 0; a <= n[0] + 1; ++a) dst[IDX(a, b, dst_idx, n[0], n[1])] = src[IDX(a, b, src_idx, n[0], n[1])];
    }
}

/* geometry_halocell_update_selectively (src/geometry.f90:621-660) of one array of level l
 * on every rank: along each split axis in turn (x, y, z), a rank's last interior plane
 * becomes its east neighbour's ghost plane 0 and the neighbour's first interior plane
 * its ghost plane n+1.  arr[r] is rank r's array. */
static void dd_halo(orc_dd *dd, int l, double **arr)
{
    const orc_level *L0 = &dd->rk[0]->lv[l];
    const int n[3] = {L0->nx, L0->ny, L0->nz};
    int d, r;
    for (d = 0; d < 3; ++d) {
        if (dd->p[d] == 1) continue;
        for (r = 0; r < dd->nr; ++r) {
            int ce[3] = {dd->c[r][0], dd->c[r][1], dd->c[r][2]}, e;
            if (ce[d] + 1 >= dd->p[d]) continue;
            ce[d] += 1;
            e = dd_rank(dd, ce[0], ce[1], ce[2]);
            dd_copy_plane(d, n, arr[e], 0, arr[r], n[d]);
            dd_copy_plane(d, n, arr[r], n[d] + 1, arr[e], 1);
        }
    }
}

/* the RBGS start offset of rank r on level l (src/rbgs_poisson_matrix.f90:230-232) */
static int dd_offset(const orc_dd *dd, int r, int l)
{
    const orc_level *L = &dd->rk[r]->lv[l];
    const int n[3] = {L->nx, L->ny, L->nz};
    int s = 0, d;
    for (d = 0; d < 3; ++d) s += (n[d] % 2) * ((dd->c[r][d] * (dd->p[d] > 1 ? 1 : 0)) % 2);
    return s % 2;
}

/* vv_dot_3d_matrix with its all-reduce: the local sums added in rank order */
static double dd_dot(orc_dd *dd, int l, double **x, double **y)
{
    double s = 0.0;
    int r;
    for (r = 0; r < dd->nr; ++r) {
        const orc_level *L = &dd->rk[r]->lv[l];
        s += orc_vv_dot(L->nx, L->ny, L->nz, x[r], y[r]);
    }
    return s;
}

static void dd_rbgs_iterator(orc_dd *dd, int l, double **x, double **b, int maxiteration, double omega)
{
    int it, c, r;
    for (it = 0; it < maxiteration; ++it)
        for (c = 0; c < 2; ++c) {
            dd_halo(dd, l, x);
            for (r = 0; r < dd->nr; ++r) {
                const orc_level *L = &dd->rk[r]->lv[l];
                rbgs_colour(L->nx, L->ny, L->nz, L->coeff, x[r], b[r], omega, c, dd_offset(dd, r, l));
            }
        }
}

/* multigrid_residual (mv_mul updates the halo of x first) */
static void dd_residual(orc_dd *dd, int l, double **rr, double **x, double **b)
{
    int r;
    dd_halo(dd, l, x);
    for (r = 0; r < dd->nr; ++r) {
        const orc_level *L = &dd->rk[r]->lv[l];
        orc_residual(L->nx, L->ny, L->nz, L->coeff, x[r], b[r], rr[r]);
    }
}

/* rbgs_solver_poisson_matrix on every rank (src/rbgs_poisson_matrix.f90:47-179) */
static int dd_rbgs_solver(orc_dd *dd, int l, double **x, double **b, double **rr, int maxiteration,
                          double tolerance, double omega)
{
    double r0, rn;
    int it;
    dd_residual(dd, l, rr, x, b);
    r0 = dd_dot(dd, l, rr, rr);
    for (it = 0; it < maxiteration; ++it) {
        dd_rbgs_iterator(dd, l, x, b, 1, omega);
        dd_residual(dd, l, rr, x, b);
        rn = dd_dot(dd, l, rr, rr);
        if (sqrt(rn / r0) <= tolerance) break;
    }
    return it;
}

/* cg_solver_poisson_matrix on every rank (src/cg_poisson_matrix.f90:47-146); p, ap, rs are
 * per-rank scratch of the level's size */
static int dd_cg_solver(orc_dd *dd, int l, double **x, double **b, double **p, double **ap, double **rs,
                        int maxiteration, double tolerance)
{
    double r0, t1, t2, alpha, beta;
    int it, r;
    dd_residual(dd, l, rs, x, b);
    for (r = 0; r < dd->nr; ++r) {
        const orc_level *L = &dd->rk[r]->lv[l];
        int i, j, k;
        for (k = 1; k <= L->nz; ++k)
            for (j = 1; j <= L->ny; ++j)
                for (i = 1; i <= L->nx; ++i) p[r][IDX(i, j, k, L->nx, L->ny)] = rs[r][IDX(i, j, k, L->nx, L->ny)];
    }
    r0 = dd_dot(dd, l, rs, rs);
    t2 = 0.0;
    for (it = 0; it < maxiteration; ++it) {
        t1 = dd_dot(dd, l, rs, rs);
        dd_halo(dd, l, p);                                     /* mv_mul's halo update */
        for (r = 0; r < dd->nr; ++r) {
            const orc_level *L = &dd->rk[r]->lv[l];
            orc_mv_mul(L->nx, L->ny, L->nz, L->coeff, p[r], ap[r]);
        }
        t2 = dd_dot(dd, l, ap, p);
        alpha = t1 / t2;
        for (r = 0; r < dd->nr; ++r) {
            const orc_level *L = &dd->rk[r]->lv[l];
            cg_update_xr(L->nx, L->ny, L->nz, alpha, x[r], rs[r], p[r], ap[r]);
        }
        t2 = dd_dot(dd, l, rs, rs);
        if (sqrt(t2 / r0) < tolerance) break;
        beta = t2 / t1;
        for (r = 0; r < dd->nr; ++r) {
            const orc_level *L = &dd->rk[r]->lv[l];
            cg_update_p(L->nx, L->ny, L->nz, beta, p[r], rs[r]);
        }
    }
    return it;
}

/* Scatter of a global (0:N+1)^3 array to the ranks' (0:n+1)^3 arrays (ghost layers from the
 * neighbours' cells or the global ghost layers), and gather of the interiors back. */
static void dd_scatter(const orc_dd *dd, const double *g, double **loc)
{
    const orc_level *L = &dd->rk[0]->lv[0];
    const int n[3] = {L->nx, L->ny, L->nz}, gn[3] = {dd->glob->lv[0].nx, dd->glob->lv[0].ny, dd->glob->lv[0].nz};
    int r, i, j, k;
    for (r = 0; r < dd->nr; ++r) {
        const int o[3] = {dd->c[r][0] * n[0], dd->c[r][1] * n[1], dd->c[r][2] * n[2]};
        for (k = 0; k <= n[2] + 1; ++k)
            for (j = 0; j <= n[1] + 1; ++j)
                for (i = 0; i <= n[0] + 1; ++i)
                    loc[r][IDX(i, j, k, n[0], n[1])] = g[IDX(o[0] + i, o[1] + j, o[2] + k, gn[0], gn[1])];
    }
}

static void dd_gather(const orc_dd *dd, double **loc, double *g)
{
    const orc_level *L = &dd->rk[0]->lv[0];
    const int n[3] = {L->nx, L->ny, L->nz}, gn[3] = {dd->glob->lv[0].nx, dd->glob->lv[0].ny, dd->glob->lv[0].nz};
    int r, i, j, k;
    for (r = 0; r < dd->nr; ++r) {
        const int o[3] = {dd->c[r][0] * n[0], dd->c[r][1] * n[1], dd->c[r][2] * n[2]};
        for (k = 1; k <= n[2]; ++k)
            for (j = 1; j <= n[1]; ++j)
                for (i = 1; i <= n[0]; ++i)
                    g[IDX(o[0] + i, o[1] + j, o[2] + k, gn[0], gn[1])] = loc[r][IDX(i, j, k, n[0], n[1])];
    }
}

/* multigrid_CGS_vcycle_solver (src/multigrid.f90:1907-1976) on every rank.  gsol / grsd /
 * grhs are the global (0:N+1)^3 arrays: they are scattered to the ranks (ghost layers from
 * the neighbours) and the interiors gathered back (grsd's ghost layers are zero, as the
 * residual leaves them).  hist and coarse_iters as orc_mg_solve.  Returns the cycles run. */
int orc_dd_solve(orc_dd *dd, double *gsol, double *grsd, const double *grhs, int maxiteration,
                 double tolerance, double omega, double *hist, int *coarse_iters)
{
    const int nl = dd->n_levels, nr = dd->nr;
    double ***X = (double ***)calloc((size_t)nl + 1, sizeof(double **));
    double ***B = (double ***)calloc((size_t)nl + 1, sizeof(double **));
    double ***R = (double ***)calloc((size_t)nl + 1, sizeof(double **));
    double **P = (double **)calloc((size_t)nr, sizeof(double *));
    double **AP = (double **)calloc((size_t)nr, sizeof(double *));
    double **RS = (double **)calloc((size_t)nr, sizeof(double *));
    double res0tol, rsd_val;
    int l, r, cyc, ncyc = 0;
    for (l = 1; l <= nl; ++l) {
        X[l] = (double **)calloc((size_t)nr, sizeof(double *));
        B[l] = (double **)calloc((size_t)nr, sizeof(double *));
        R[l] = (double **)calloc((size_t)nr, sizeof(double *));
        for (r = 0; r < nr; ++r) {
            X[l][r] = dd_arr(dd, r, l, 0);
            B[l][r] = dd_arr(dd, r, l, 1);
            R[l][r] = dd_arr(dd, r, l, 2);
        }
    }
    for (r = 0; r < nr; ++r) {
        const size_t t = lv_total(&dd->rk[r]->lv[nl]);
        memset(dd->rk[r]->work, 0, sizeof(double) * 3 * t);
        P[r] = dd->rk[r]->work;
        AP[r] = dd->rk[r]->work + t;
        RS[r] = dd->rk[r]->work + 2 * t;
        memset(dd->rsd[r], 0, sizeof(double) * lv_total(&dd->rk[r]->lv[0]));
    }
    dd_scatter(dd, gsol, dd->sol);
    dd_scatter(dd, grhs, dd->rhs);
    dd_residual(dd, 0, dd->rsd, dd->sol, dd->rhs);                          /* :1924 */
    res0tol = dd_dot(dd, 0, dd->rsd, dd->rsd);
    for (cyc = 1; cyc <= dd->n_vcycles; ++cyc) {
        double ratio;
        int ci;
        dd_rbgs_iterator(dd, 0, dd->sol, dd->rhs, maxiteration, omega);      /* :1931-1933 */
        dd_residual(dd, 0, dd->rsd, dd->sol, dd->rhs);
        for (r = 0; r < nr; ++r) restrict_lv(dd->rk[r], 0, dd->rsd[r], B[1][r]);
        for (l = 1; l <= nl - 1; ++l) {                                      /* :1936-1941 */
            for (r = 0; r < nr; ++r) memset(X[l][r], 0, sizeof(double) * lv_total(&dd->rk[r]->lv[l]));
            dd_rbgs_iterator(dd, l, X[l], B[l], maxiteration, omega);
            dd_residual(dd, l, R[l], X[l], B[l]);
            for (r = 0; r < nr; ++r) restrict_lv(dd->rk[r], l, R[l][r], B[l + 1][r]);
        }
        for (r = 0; r < nr; ++r) memset(X[nl][r], 0, sizeof(double) * lv_total(&dd->rk[r]->lv[nl]));
        if (dd->coarse_solver == 1)                                          /* :1944-1949 */
            ci = dd_cg_solver(dd, nl, X[nl], B[nl], P, AP, RS, 1000, tolerance);
        else
            ci = dd_rbgs_solver(dd, nl, X[nl], B[nl], R[nl], 1000, tolerance, omega);
        if (coarse_iters) coarse_iters[cyc - 1] = ci;
        dd_residual(dd, nl, R[nl], X[nl], B[nl]);                            /* :1951, halo of x */
        for (l = nl - 1; l >= 1; --l) {                                      /* :1957-1962 */
            for (r = 0; r < nr; ++r) {
                prolong_lv(dd->rk[r], l, X[l + 1][r], R[l][r]);
                add_inplace(lv_total(&dd->rk[r]->lv[l]), X[l][r], R[l][r]);
            }
            dd_rbgs_iterator(dd, l, X[l], B[l], maxiteration, omega);
            dd_halo(dd, l, X[l]);
        }
        for (r = 0; r < nr; ++r) {                                           /* :1965-1967 */
            prolong_lv(dd->rk[r], 0, X[1][r], dd->rsd[r]);
            add_inplace(lv_total(&dd->rk[r]->lv[0]), dd->sol[r], dd->rsd[r]);
        }
        dd_rbgs_iterator(dd, 0, dd->sol, dd->rhs, maxiteration, omega);
        dd_residual(dd, 0, dd->rsd, dd->sol, dd->rhs);                      /* :1970-1971 */
        rsd_val = dd_dot(dd, 0, dd->rsd, dd->rsd);
        ratio = sqrt(rsd_val / res0tol);
        if (hist) {
            hist[3 * (cyc - 1) + 0] = sqrt(rsd_val);
            hist[3 * (cyc - 1) + 1] = sqrt(res0tol);
            hist[3 * (cyc - 1) + 2] = ratio;
        }
        ncyc = cyc;
        if (ratio < tolerance) break;                                       /* :1973 */
    }
    dd_gather(dd, dd->sol, gsol);
    memset(grsd, 0, sizeof(double) * lv_total(&dd->glob->lv[0]));
    dd_gather(dd, dd->rsd, grsd);
    for (l = 1; l <= nl; ++l) { free(X[l]); free(B[l]); free(R[l]); }
    free(X); free(B); free(R); free(P); free(AP); free(RS);
    return ncyc;
}

/* the rank (cx, cy, cz)'s colour offset on level l and its level sizes (test hooks) */
int orc_dd_offset(const orc_dd *dd, int cx, int cy, int cz, int l) { return dd_offset(dd, dd_rank(dd, cx, cy, cz), l); }
void orc_dd_level_dims(const orc_dd *dd, int l, int *dims) { orc_mg_level_dims(dd->rk[0], l, dims); }

/* One RBGS colour with a rank's start offset (src/rbgs_poisson_matrix.f90:239-271), for
 * drivers that run one rank per process. */
void orc_rbgs_colour(int nx, int ny, int nz, const double *coeff, double *sol, const double *rhs, double omega,
                     int colour, int offset)
{
    rbgs_colour(nx, ny, nz, coeff, sol, rhs, omega, colour, offset);
}
