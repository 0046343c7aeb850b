/*
 * peps_mg.h -- C-ABI of the GB300 (sm_103a) multigrid V-cycle solver.
 *
 * Drop-in for the solve path of PEPS_MG (Fortran module `multigrid`).  Every entry
 * point is `extern "C"`, takes plain pointers and sizes, returns an int status and
 * never aborts the process.  Grid arrays are Fortran-ordered (i fastest) with one
 * ghost layer, (0:nx+1, 0:ny+1, 0:nz+1), 8-byte doubles; a Fortran caller passes
 * c_loc(x(0,0,0)).  Physical-boundary ghost cells hold the Dirichlet values, exactly
 * as in the reference, and are never overwritten.
 *
 * Interface citations are relative to the reference project root.
 */
#ifndef PEPS_MG_H
#define PEPS_MG_H

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference prints and stops (MPI_Finalize; stop / MPI_Abort);
 * this library returns one of these instead. */
#define PMG_OK 0
#define PMG_EINVAL 1      /* argument or configuration the reference rejects          */
#define PMG_ENOMEM 2      /* device or host allocation failed                         */
#define PMG_EDIVERGED 3   /* residual norm became NaN or Inf                          */
#define PMG_ETIMEOUT 4    /* a bounded device wait gave up, or the abort flag was set */
#define PMG_ECUDA 5       /* CUDA runtime error (see pmg_last_error)                  */

/* aggregation_method (&control aggregation_method, src/multigrid.f90:113-124) */
#define PMG_CGS 0
#define PMG_CGA 1
#define PMG_CGPSA 2

/* coarsest-level solver: the reference calls rbgs_solver_poisson_matrix
 * (src/multigrid.f90:1837-1849); CG selects cg_solver_poisson_matrix
 * (src/cg_poisson_matrix.f90:47) with the same 1000-iteration cap and tolerance. */
#define PMG_COARSE_RBGS 0
#define PMG_COARSE_CG 1

/* precision of the V-cycle */
#define PMG_FP64 0        /* plain FP64, bitwise the reference's arithmetic             */
#define PMG_MIXED 1       /* FP32 V-cycles inside FP64 defect correction                */
#define PMG_FP64_FAST 2   /* FP64 V-cycles with FMA, a stored omega/c0 per cell and
                           * per-axis normalised transfer weights: the same level sequence
                           * and exit test as PMG_FP64, not its bits (rounding differs)  */

typedef struct pmg_ctx pmg_ctx;

/* Solver configuration: the caller's subdomain mesh plus &control of PARA_INPUT.inp
 * (src/main_peps.f90:44-60).  Mesh arrays are host memory, nx+2 (ny+2, nz+2) values
 * each, indexed 0..n+1 as the subdomain type of src/geometry.f90:59-118. */
typedef struct {
    int nx, ny, nz;
    const double *dxm, *dxg, *xg;
    const double *dym, *dyg, *yg;
    const double *dzm, *dzg, *zg;
    int number_of_levels;      /* coarse levels below the finest (the finest is level 0) */
    int number_of_vcycles;     /* V-cycle cap                                            */
    int aggregation_method;    /* PMG_CGS / PMG_CGA / PMG_CGPSA                          */
    int cga_level;             /* CGA_level                                              */
    int cgpsa_level[3];        /* CGPSA_level(3)                                         */
    int coarse_solver;         /* PMG_COARSE_RBGS or PMG_COARSE_CG                       */
    int precision;             /* PMG_FP64, PMG_MIXED or PMG_FP64_FAST                   */
    int mixed_inner_cycles;    /* PMG_MIXED: FP32 V-cycles per FP64 correction (0 = 2)   */
} pmg_config_t;

/* Per-solve report (replaces the reference's rank-0 prints, src/multigrid.f90:1972). */
typedef struct {
    int cycles;                /* V-cycles run                                           */
    int converged;             /* 1 if sqrt(rsd/res0) < tolerance was reached            */
    double res0;               /* sqrt(res0tol)                                          */
    double final_ratio;        /* sqrt(rsd_val/res0tol) after the last cycle             */
    double *history;           /* optional, 3*number_of_vcycles doubles:                 */
                               /*   sqrt(rsd_val), sqrt(res0tol), sqrt(rsd_val/res0tol)  */
    int *coarse_iterations;    /* optional, number_of_vcycles ints                       */
    float elapsed_ms;          /* device time of the whole call (CUDA events)            */
    int inner_cycles;          /* PMG_MIXED: FP32 V-cycles run in total (else = cycles)  */
} pmg_report_t;

/* multigrid_create(sdm, nlevel, ncycle, aggr_method, single_aggr_level,
 * adaptive_aggr_level) -- src/multigrid.f90:75.  Builds the level hierarchy (level
 * sizes, meshes, coefficient tables) and allocates the device state.  `stream` is a
 * cudaStream_t (NULL = legacy default stream); all device work of the context is
 * issued on it.  The finest-level operator is the reference's a_poisson built by
 * matrix_heptadiagonal_create (src/matrix.f90:39) from the same mesh. */
int pmg_create(pmg_ctx **ctx, const pmg_config_t *cfg, void *stream);

/* multigrid_solve_vcycle(sol, rsd, a_poisson, rhs, sdm, maxiteration, tolerance,
 * omega_sor) -- src/multigrid.f90:1864.  sol (in/out), rsd (out: final residual,
 * ghosts zero) and rhs (in) are (nx+2)(ny+2)(nz+2) doubles, either all device memory
 * or all host memory (host buffers are staged through the device; pageable ones are
 * page-locked for the duration of the call unless PEPS_MG_NO_HOST_REGISTER=1, and
 * released before it returns).  report may be NULL. */
int pmg_solve_vcycle(pmg_ctx *ctx, double *sol, double *rsd, const double *rhs, int maxiteration,
                     double tolerance, double omega_sor, pmg_report_t *report);

/* multigrid_destroy -- src/multigrid.f90:1320 */
int pmg_destroy(pmg_ctx *ctx);

/* Level sizes of the hierarchy without creating a context (host only, no GPU needed):
 * the one-rank rules of multigrid_subdomain_create_CGS / _CGA / _CGPSA
 * (src/multigrid.f90:167-402, 503-838, 998-1288).  sizes receives 3*(n_levels+1) ints
 * (level 0 = nx,ny,nz), lv_coarsest the last level at which each axis was halved.
 * Returns PMG_EINVAL where the reference stops with an error. */
int pmg_level_sizes(int nx, int ny, int nz, int n_levels, int aggregation_method, int cga_level, int *sizes,
                    int lv_coarsest[3]);

/* Hierarchy queries: level 0 is the caller's subdomain, 1..number_of_levels the
 * coarse levels (mg_sdm(l) of src/multigrid.f90:54). */
int pmg_level_dims(const pmg_ctx *ctx, int level, int dims[3]);
int pmg_level_mesh(const pmg_ctx *ctx, int level, int axis, double *dm, double *dg, double *xg);
int pmg_coarsest_levels(const pmg_ctx *ctx, int lv_coarsest[3]);

/* ---- Lower API: operate on device arrays of one level's shape ------------------ */
/* Calls are asynchronous on the context stream unless they return a scalar.        */

/* mv_mul_poisson_matrix(y, a_poisson, x, dm, is_serial) -- src/poisson_matrix_operator.f90:110 */
int pmg_mv_mul(pmg_ctx *ctx, int level, double *y, const double *x);
/* vv_dot_3d_matrix(result, x, y, nx, ny, nz, is_serial) -- src/poisson_matrix_operator.f90:40 */
int pmg_vv_dot(pmg_ctx *ctx, int level, const double *x, const double *y, double *result);
/* multigrid_residual(rsd, a_poisson, x, rhs, dm, is_aggregated) -- src/multigrid.f90:1782 */
int pmg_residual(pmg_ctx *ctx, int level, double *r, const double *x, const double *b);
/* rbgs_iterator_poisson_matrix(sol, a_poisson, rhs, dm, maxiteration, omega, ...) --
 * src/rbgs_poisson_matrix.f90:191 */
int pmg_rbgs_iterator(pmg_ctx *ctx, int level, double *x, const double *b, int maxiteration, double omega);
/* rbgs_solver_poisson_matrix(sol, a_poisson, rhs, dm, maxiteration, tolerance, omega,
 * ...) -- src/rbgs_poisson_matrix.f90:47.  iterations/ratio may be NULL. */
int pmg_rbgs_solver(pmg_ctx *ctx, int level, double *x, const double *b, int maxiteration, double tolerance,
                    double omega, int *iterations, double *ratio);
/* cg_iterator_poisson_matrix -- src/cg_poisson_matrix.f90:157 */
int pmg_cg_iterator(pmg_ctx *ctx, int level, double *x, const double *b, int maxiteration);
/* cg_solver_poisson_matrix -- src/cg_poisson_matrix.f90:47 */
int pmg_cg_solver(pmg_ctx *ctx, int level, double *x, const double *b, int maxiteration, double tolerance,
                  int *iterations, double *ratio);
/* multigrid_restriction(val_c, val_f, dm_c, dm_f, level) -- src/multigrid.f90:1345.
 * level is the fine level; val_c is zeroed (ghosts included) then filled. */
int pmg_restriction(pmg_ctx *ctx, int level, double *val_c, const double *val_f);
/* multigrid_prolongation_linear_on_nonuniform_grid(val_f, val_c, dm_f, dm_c, level) --
 * src/multigrid.f90:1516.  Writes only the interior children of val_f. */
int pmg_prolongation(pmg_ctx *ctx, int level, double *val_f, const double *val_c);
/* Fused prolongation + correction x_f = x_f + P x_c, the pair of statements at
 * src/multigrid.f90:1957-1958 (interior; the reference's ghost add is of zeros). */
int pmg_prolong_add(pmg_ctx *ctx, int level, double *x_f, const double *x_c);

/* ---- Adjoint (no counterpart in the reference) ------------------------------------- */
/* Gradients of a loss L(u) of the last solution u of this context with respect to the
 * right-hand side and the six Dirichlet face values, given dLdu = dL/du (device array of
 * the finest level; ghost entries ignored):
 *   dLdb    = A^{-T} dLdu on the interior, 0 on the ghosts       (device array)
 *   dLdg[f] = -sum over the cells next to face f of c_f * dLdb   (host, 6 doubles, order
 *             x-, x+, y-, y+, z-, z+; each face's ghost layer is one scalar value)
 * A^T = V A V^{-1} with V = diag(dxm dym dzm), so the transposed system is solved by this
 * context's own V-cycle (FP64 or mixed) with zero ghost values; only the finest-level
 * right-hand side and solution of that solve are held.  report may be NULL. */
int pmg_adjoint(pmg_ctx *ctx, const double *dLdu, double *dLdb, double dLdg[6], int maxiteration, double tolerance,
                double omega_sor, pmg_report_t *report);

/* ---- Batched solver (no counterpart in the reference) ------------------------------ */
/* Many independent problems of uneven sizes, each with its own hierarchy (the CGS level
 * rules with as many levels as its sizes allow), solved together in mixed precision:
 * every V-cycle operation at a depth is one persistent launch over all problems, one
 * outer correction is captured in a CUDA graph, smoother tiles are autotuned per depth.
 * dims: 3 ints per problem.  meshes: NULL (uniform meshes of cubic cells, width
 * 1/max(nx,ny,nz), so the longest axis spans [0,1]) or 6 host pointers per problem (dxm,
 * dxg, dym, dyg, dzm, dzg, each n+2 values; NULL entries mean that uniform axis).  sol and rhs are packed device arrays: problem p occupies elements
 * offsets[p] .. offsets[p+1]-1 in the usual (0:n+1)^3 Fortran layout
 * (pmg_batch_layout). */
typedef struct pmg_batch pmg_batch;
int pmg_batch_create(pmg_batch **batch, int n_problems, const int *dims, const double *const *meshes,
                     int mixed_inner_cycles, void *stream);
int pmg_batch_layout(const pmg_batch *batch, long long *offsets, int *levels);
/* Solves until every problem reaches sqrt(|r|^2/|r0|^2) < tolerance or max_cycles outer
 * corrections ran; cycles/ratio (per problem, may be NULL) receive the corrections used
 * and the final ratio; elapsed_ms (may be NULL) the device time.  Synchronous. */
int pmg_batch_solve(pmg_batch *batch, double *sol, const double *rhs, int maxiteration, double tolerance,
                    double omega_sor, int max_cycles, int *cycles, double *ratio, float *elapsed_ms);
int pmg_batch_destroy(pmg_batch *batch);

/* ---- Domain decomposition: the reference's multi-rank execution --------------------- */
/* The CGS V-cycle on a procs[0] x procs[1] x procs[2] Cartesian decomposition of one grid,
 * as the reference runs it on that many MPI ranks (src/mpi_topology.f90:53-99): each
 * subdomain has its own hierarchy, built from the global hierarchy's meshes restricted to
 * its cells (coarse ghost widths from the neighbours, src/multigrid.f90:452-477); ghost
 * layers are exchanged where the reference calls geometry_halocell_update_selectively
 * (src/geometry.f90:621-660: before each RBGS colour, before every residual, after each
 * coarse level's post-smoothing), by device-side packing, a cudaMemcpyAsync to the
 * neighbour's buffer and unpacking; dot products are summed over the subdomains in rank order
 * (src/poisson_matrix_operator.f90:68-97); each subdomain's RBGS colours start at the
 * rank-parity offset of src/rbgs_poisson_matrix.f90:230-232.  Every subdomain lives on this
 * process's current GPU.  The solution equals the one-grid solution bit for bit.
 * cfg: the global problem (plain FP64, CGS, RBGS coarsest solver); the global sizes must be
 * divisible by procs, and an axis split over several ranks must halve at every level (the
 * reference stops otherwise, src/multigrid.f90:226-246): PMG_EINVAL. */
typedef struct pmg_dd pmg_dd;
int pmg_dd_create(pmg_dd **dd, const pmg_config_t *cfg, const int procs[3], void *stream);
/* multigrid_solve_vcycle (src/multigrid.f90:1864) on every subdomain; sol, rsd, rhs are
 * the global (0:nx+1,0:ny+1,0:nz+1) device arrays (scattered to the subdomains, ghost layers
 * included, and gathered back).  Synchronous. */
int pmg_dd_solve(pmg_dd *dd, double *sol, double *rsd, const double *rhs, int maxiteration, double tolerance,
                 double omega_sor, pmg_report_t *report);
int pmg_dd_destroy(pmg_dd *dd);
/* The subdomain of the rank at coords (host only, no GPU needed): its sizes on `level`, its
 * mesh there (mesh: 9 host pointers dxm, dxg, xg, dym, dyg, yg, dzm, dzg, zg of n+2 values,
 * any may be NULL) and its RBGS colour offset there. */
int pmg_dd_partition(const pmg_config_t *cfg, const int procs[3], const int coords[3], int level, int dims[3],
                     double *const mesh[9], int *offset);

/* ---- Dot product without device allocation (no counterpart in the reference) ------ */
/* For host codes that must not have a library call cudaMalloc: one whose device memory
 * is handed to its own allocator at start-up, or one calling from inside its iteration
 * loop, where cudaMalloc/cudaFree would synchronise the whole device.  Such a caller keeps
 * its own CG loop around vv_dot_3d_matrix (src/poisson_matrix_operator.f90:40) and has no
 * pmg_ctx (creating one allocates the level hierarchy).
 *   *result = sum over the interior cells of x(i,j,k) * y(i,j,k)
 * x, y: device arrays in the (0:nx+1, 0:ny+1, 0:nz+1) layout; stream: a cudaStream_t
 * (NULL = the default stream).  The value equals pmg_vv_dot's on the same arrays to
 * within FP64 rounding (bit for bit when nz * ceil(nx/32) * ceil(ny/8) <= 16384).
 * Nothing is allocated: the partial sums live in a static 128 KiB device array that every
 * GPU loading this library holds until the process exits.  Limit: ceil(nx/32) *
 * ceil(ny/8) <= 16384 (e.g. planes up to 2048 x 2048); larger planes return PMG_EINVAL
 * with a message in pmg_last_error.  Every call looks up the array's address on the
 * current device (a host query that allocates nothing), so it stays valid after the
 * device's context was re-created (cudaDeviceReset); the first call on each device also
 * clears the array with a cudaMemsetAsync: make that first call before any stream
 * capture.  All calls on one device share the array, so
 * calls that overlap in time (from several host threads, or on several streams at once)
 * race: serialise them.  Synchronous: returns after *result is written. */
int pmg_vv_dot_static(const double *x, const double *y, int nx, int ny, int nz, void *stream, double *result);

/* ---- Telemetry (no counterpart in the reference; it only prints MPI_Wtime) ------ */
/* Kernel classes of pmg_profile_read: the finest level's launches by kernel, and the grid
 * levels below it as one class per precision (the single-CTA tails are classes of their
 * own).  Algorithmic bytes count every array a launch reads or writes once. */
#define PMG_PROF_SMOOTH32 0       /* FP32 RBGS half-sweep                    */
#define PMG_PROF_OUTER_RESIDUAL 1 /* FP64 outer residual of PMG_MIXED        */
#define PMG_PROF_RESRESTRICT32 2  /* FP32 residual fused with restriction    */
#define PMG_PROF_PROLONG32 3      /* FP32 prolongation + correction          */
#define PMG_PROF_ADD_CORRECTION 4 /* FP64 x += e                             */
#define PMG_PROF_TAIL32 5         /* FP32 single-CTA coarse tail             */
#define PMG_PROF_SMOOTH64 6       /* FP64 RBGS half-sweep                    */
#define PMG_PROF_RESIDUAL64 7     /* FP64 residual                           */
#define PMG_PROF_RESTRICT64 8     /* FP64 restriction                        */
#define PMG_PROF_PROLONG64 9      /* FP64 prolongation + correction          */
#define PMG_PROF_TAIL64 10        /* FP64 single-CTA coarse tail             */
#define PMG_PROF_UPDATE_RESIDUAL 11 /* PMG_MIXED residual update r -= A e    */
#define PMG_PROF_COARSE32 12      /* FP32 grid levels below the finest: their smoothing and transfers, together */
#define PMG_PROF_COARSE64 13      /* FP64 grid levels below the finest: smoothing, residuals, transfers       */
/* Enable (1) or disable (0) CUDA-event timing of the classes above; resets the
 * accumulated figures.  While it is on, the FP32 V-cycles are launched kernel by kernel
 * instead of as CUDA graphs. */
int pmg_profile(pmg_ctx *ctx, int enable);
/* Accumulated device time, launch count and algorithmic bytes per launch (averaged over
 * the launches) of a class. */
int pmg_profile_read(pmg_ctx *ctx, int kernel_class, double *total_ms, long long *launches, double *bytes);
/* Kernels launched by this library so far (all contexts of the process). */
int pmg_launch_count(long long *count);

/* Self-test of the integer-pipe conversions used by the mixed-precision outer kernels
 * (no counterpart in the reference): out32[q] = (float)in64[q] rounded to nearest even,
 * out64[q] = (double)in32[q]; device pointers, synchronous. */
int pmg_selftest_convert(const double *in64, float *out32, const float *in32, double *out64, int n);

/* Self-test of the fused FP32 smoother of a mixed-precision context (no counterpart in the
 * reference): e_out = one red-black iteration (src/rbgs_poisson_matrix.f90:235-273) of
 * e_in for right-hand side b on `level`, computed in FP32 by the fused kernel.
 * impl: 0 = TMA-fed kernel, 1 = register-window kernel, 2 = one-launch cell-pair kernel
 * (variant and kchunk unused); variant 0/1/2/3 = tiles 60 x 14 / 60 x 6 / 60 x 10 /
 * 60 x 22 (3: TMA-fed kernel only); kchunk: planes per work item (0 = automatic); zero_in: treat e_in as
 * zero.  Host arrays of the level's (0:nx+1,0:ny+1,0:nz+1) Fortran layout (ghosts of
 * e_in and b must be zero); e_out receives every cell.  PMG_EINVAL when the level has no
 * fused smoother or impl 0 is unavailable for it.  Synchronous; overwrites the context's
 * FP32 work arrays of that level. */
int pmg_selftest_smooth32(pmg_ctx *ctx, int level, int impl, int variant, int kchunk, int zero_in, double omega,
                          const double *e_in, const double *b, double *e_out);

/* Self-test of the timeout path of the TMA-fed FP32 smoother (no counterpart in the
 * reference): one launch on `level` of a mixed-precision context in a mode that issues no
 * copies and limits each bounded wait to a few microseconds, so the waits run out with no
 * copy in flight.  Returns PMG_ETIMEOUT (the status a solve returns when a wait gives up)
 * if the kernel raised its error flag, PMG_EINVAL when the level has no TMA-fed smoother.
 * Clears the level's FP32 work arrays afterwards; the context stays usable.  Synchronous. */
int pmg_selftest_wait_timeout(pmg_ctx *ctx, int level);

/* ---- Abort and fault injection (no counterpart in the reference) ------------------ */
/* Sets (flag != 0) or clears the context's abort flag.  The flag lives in mapped
 * page-locked host memory, so it may be set from another host thread while a solve runs:
 * the solve loops (V-cycles, outer corrections, the lower API's RBGS and CG solvers) test
 * it before each cycle and the coarse solvers of the single-CTA tail kernels poll it on
 * the device every 16 iterations; a solve that sees it returns PMG_ETIMEOUT with the
 * solution of the last completed cycle.  The flag stays set until cleared. */
int pmg_set_abort(pmg_ctx *ctx, int flag);
/* Host-side fault injection for tests: n >= 0 makes the n-th next device allocation of the
 * library (0 = the next one; every context, batch and lower-API scratch allocation counts)
 * fail as cudaMalloc fails on an exhausted device, so the call that made it returns
 * PMG_ENOMEM and releases what it had allocated; the injection is then disarmed.  n < 0
 * disarms it.  Process-wide. */
int pmg_inject_alloc_failure(long long n);

/* Wait for all work issued on the context stream. */
int pmg_sync(pmg_ctx *ctx);
/* Text of the last CUDA error seen by this thread ("" if none). */
const char *pmg_last_error(void);
const char *pmg_status_string(int status);

#ifdef __cplusplus
}
#endif
#endif /* PEPS_MG_H */
