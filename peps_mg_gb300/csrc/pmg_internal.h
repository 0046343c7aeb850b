// pmg_internal.h -- host-side declarations shared by the library's translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <exception>
#include <new>
#include <string>
#include <vector>

#include "../../include/peps_mg.h"
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
    // The coarsest-level solve always runs in FP64 on the FP64 copy of that level.
    LevelK<double> C64;
    double *cx64, *cb64, *cp64, *cap64, *crr64;
    double omega64, omw64;
    // FP32 tail only: floats of dynamic shared memory holding x and b of every tail level
    // (0 = the tail works on the global arrays)
    int sm_floats;
    // host abort flag of the context (pmg_set_abort; mapped host memory), or nullptr
    const volatile int *abort;
};

// Layout of a hierarchy built on the device (pmg_f64.cu): level sizes and, per level and
// axis, the offsets (in doubles) of the mesh (dm, dg, xg, n+2 values each, consecutive) in
// the mesh blob and of the coefficient tables / transfer weights in the table blob.
struct HierDesc {
    int nl;
    int method, agg_level;
    int meshes_given;           // 1: every level's mesh is in the blob already
    int lvc[3];
    double ox[3];
    int n[kMaxLevels][3];
    long long mesh_off[kMaxLevels][3];
    long long cm[kMaxLevels][3], cp[kMaxLevels][3], sx[kMaxLevels];
    long long w[kMaxLevels][3], pp[kMaxLevels][3], pn[kMaxLevels][3];
};

// ---- FP64 (bitwise) launchers, pmg_f64.cu -------------------------------------
// Builds the coarse meshes (unless given) and every level's tables on the device.
int hierarchy_setup(const HierDesc *dev_desc, double *meshes, double *tables, cudaStream_t s);
// c0t (optional, every FP64 grid launcher below): the level's per-cell diagonal table
// (f64_diag_table), read instead of summing the 1-D tables per cell; the same bits.
int f64_rbgs_sweeps(const LevelK<double> &L, const Launch &ln, double *x, const double *b, int iters,
                    double omega, cudaStream_t s, const double *c0t = nullptr);
// One half-sweep: the cells with (i + j + k + colour) odd, i.e. ista = 1 + mod(j+k+colour, 2)
// (src/rbgs_poisson_matrix.f90:242, :260; colour carries a rank's parity offset).
int f64_rbgs_colour(const LevelK<double> &L, const Launch &ln, double *x, const double *b, double omega, int colour,
                    cudaStream_t s, const double *c0t = nullptr);
// c0t = diag_f64 of every interior cell of level L (an array of the level's layout).
int f64_diag_table(const LevelK<double> &L, double *c0t, cudaStream_t s);
// r = b - A x (interior); if partials != nullptr also writes per-block sums of r^2
// and returns the number of partials in *npart.
int f64_residual(const LevelK<double> &L, const Launch &ln, double *r, const double *x, const double *b,
                 double *partials, int *npart, cudaStream_t s, const double *c0t = nullptr);
int f64_mv_mul(const LevelK<double> &L, const Launch &ln, double *y, const double *x, cudaStream_t s,
               const double *c0t = nullptr);
int f64_dot_partials(const LevelK<double> &L, const Launch &ln, const double *x, const double *y,
                     double *partials, int *npart, cudaStream_t s);
// Sum partials[0..n) in a fixed order into *out (device).
int f64_reduce(const double *partials, int n, double *out, cudaStream_t s);
int f64_restrict(const XferK<double> &X, const Launch &ln, const double *vf, double *vc, cudaStream_t s);
int f64_prolong(const XferK<double> &X, const Launch &ln, const double *vc, double *vf, bool add,
                cudaStream_t s);
int zero_ghosts_f64(double *a, int nx, int ny, int nz, cudaStream_t s);
int f64_tail(const TailDesc<double> *dev_desc, int threads, cudaStream_t s);
// Device state of a fused CG solve (src/cg_poisson_matrix.f90:80-138): the reference's
// scalars, the exit flag, and the arrival counter of the kernels' last-CTA reductions
// (zero between launches).
struct CgState {
    double r0;              // rsd0tol
    double t1;              // temp1 = r.r at the start of the iteration
    double pap;             // temp2 = Ap.p
    double alpha;           // temp1 / (Ap.p)
    double t2;              // temp2 = r.r after the update
    double beta;            // temp2 / temp1
    int done;               // exit test met (solver only)
    int iter;               // iteration at which it was met
    unsigned int arrive;    // CTAs that have added their partial sum
    int pad;
};
// Number of partial sums of the fused CG kernels on a level (the partials buffer must hold them).
int f64_cg_partials(const LevelK<double> &L, const Launch &ln);
// r = b - A x, p = r, st->r0 = st->t1 = r.r, st->done = 0.
int f64_cg_init(const LevelK<double> &L, const Launch &ln, double *r, double *p, const double *x, const double *b,
                double *partials, CgState *st, cudaStream_t s, const double *c0t = nullptr);
// One CG iteration (three fused kernels); with check, the exit test sqrt(t2/r0) < tol sets
// st->done and st->iter = iter, after which further iterations do nothing.
int f64_cg_iteration(const LevelK<double> &L, const Launch &ln, double *x, double *r, double *p, double *ap,
                     double *partials, CgState *st, double tol, bool check, int iter, cudaStream_t s,
                     const double *c0t = nullptr);

// ---- FP64 performance mode, pmg_f64fast.cu -----------------------------------------
// Tables of one grid level: per-axis diagonal sums (x: LevelK::sx) and omega / c0 per cell.
struct FastLevelK {
    double *dy, *dz;
    double *wdiag;
};
// Normalised per-axis transfer weights of the fine indices between level l and l + 1:
// restriction weight of a child's value, prolongation weights of the own and the
// neighbouring coarse cell.
struct FastXferK {
    double *rx, *ry, *rz;
    double *pax, *pbx, *pay, *pby, *paz, *pbz;
};
// Fills fl->dy, fl->dz and (X != nullptr) the transfer weights *fx from the plain tables.
int fast_tables(const LevelK<double> &L, const XferK<double> *X, int nfx, int nfy, int nfz, FastLevelK *fl,
                FastXferK *fx, cudaStream_t s);
int fast_wdiag(const LevelK<double> &L, double omega, double *wdiag, cudaStream_t s);
int fast_rbgs_sweeps(const LevelK<double> &L, const FastLevelK &F, const Launch &ln, double *x, const double *b,
                     int iters, double omega, cudaStream_t s);
int fast_residual(const LevelK<double> &L, const FastLevelK &F, const Launch &ln, double *r, const double *x,
                  const double *b, double *partials, int *npart, cudaStream_t s);
int fast_restrict(const XferK<double> &X, const FastXferK &W, const Launch &ln, const double *vf, double *vc,
                  cudaStream_t s);
// x_f += P x_c
int fast_prolong(const XferK<double> &X, const FastXferK &W, const Launch &ln, const double *vc, double *vf,
                 cudaStream_t s);

// ---- FP32 fused smoother, pmg_smooth32.cu ----------------------------------------
// One out-of-place red-black iteration e_out = RB(e_in) of a whole level (zero_in: e_in
// is zero and is not read).  Needs the padded FP32 layout checked by rb32_fused_layout_ok.
bool rb32_fused_layout_ok(const LevelK<float> &L, const void *e, const void *b);
// Tensor maps of one padded FP32 level for the TMA-fed variant of the smoother: the two
// e buffers and b, one map per tile variant (the copy box depends on the tile height).
struct Rb32Tma {
    bool ok = false;
    CUtensorMap e[2][4];
    CUtensorMap b[4];
};
// base[3]: allocation starts of e[0], e[1], b (cell (0,0,0) at base + 5 + sy + sz);
// rows, planes: allocated rows per plane and planes.  Leaves t->ok false (and returns
// PMG_OK) when the tensor-map encoder is unavailable or rejects the layout.
int rb32_tma_setup(Rb32Tma *t, const LevelK<float> &L, float *const base[3], long long rows, long long planes);
// variant: 0 = 60 x 14 tiles (512 threads), 1 = 60 x 6 (256), 2 = 60 x 10 (384), 3 = 60 x 22
// (TMA-fed kernel only, 384 threads; the register-window kernel runs variant 0 for it);
// kchunk: planes per work item (0 = automatic).  With tma (tma->ok), the TMA-fed kernel
// runs; ein must then be buffer in_buf of the maps, and err receives 1 if one of its
// bounded pipeline waits gave up.  stall (self-test of that path, TMA-fed kernel only):
// the kernel issues no copies and its waits give up after a few microseconds.
int rb32_fused(const LevelK<float> &L, const Launch &ln, const float *ein, float *eout, const float *b, float omega,
               float omw, bool zero_in, cudaStream_t s, int variant = 0, int kchunk = 0,
               const Rb32Tma *tma = nullptr, int in_buf = 0, int *err = nullptr, bool stall = false);
// Picks the fastest kernel, tile variant and k-chunk for a level (process-wide cache).
// With tensor maps (tma) the TMA-fed and the register-window kernels compete; when the
// register-window one wins, *variant carries kTuneWindow on top of the tile variant and the
// caller must run that level without its maps.
constexpr int kTuneWindow = 8;
// variant of rb32_fused (and tune_smoother's answer) for the one-launch cell-pair kernel
// (no tiles, no marching: levels that live in L2, where the marching kernels' serial plane
// pipeline is the longer path)
constexpr int kCellVariant = 4;
// allow_cell: the one-launch cell-pair kernel is a candidate too (on levels of at most 2^22
// cells), answered as kCellVariant.
int tune_smoother(const LevelK<float> &L, const Launch &ln, float *e0, float *e1, const float *b, cudaStream_t s,
                  int *variant, int *kchunk, const Rb32Tma *tma = nullptr, int *err = nullptr,
                  bool allow_cell = true);
// Integer-pipe precision conversions used by the outer kernels (self-test hook).
int convert_selftest(const double *in64, float *out32, const float *in32, double *out64, int n, cudaStream_t s);

// Coarse tails of a batch: one CTA per problem (pmg_mixed.cu).
int batch_tail32(const TailDesc<float> *const *descs, int n, const int *done, int threads, cudaStream_t s);

// ---- batched solver, pmg_batch.cu ---------------------------------------------------
struct Batch;
int batch_create(Batch **out, int n, const int *dims, const double *const *meshes, int inner, cudaStream_t user);
int batch_solve(Batch &B, double *sol, const double *rhs, int maxit, double tol, double omega, int max_cycles,
                int *cycles, double *ratio, float *elapsed_ms);
void batch_destroy(Batch *B);
void batch_layout(const Batch &B, long long *offsets, int *levels);
int batch_size(const Batch &B);

// Fixed launch shapes (shared with the host driver for partial-sum sizing).
void grid_for_cells(const LevelK<double> &L, const Launch &ln, dim3 *grid, dim3 *block);

// ---- telemetry --------------------------------------------------------------------
// Kernel classes timed by the optional profiler: the finest level's kernels one class each,
// the grid levels below it as one class per precision.
enum ProfClass {
    PC_SMOOTH32 = 0,     // FP32 RBGS half-sweep                     8 B/cell algorithmic
    PC_OUTER_RES = 1,    // FP64 outer residual (+FP32 copy, norm)  28 B/cell
    PC_RESRESTRICT32 = 2,// FP32 residual fused with restriction   8.5 B/cell
    PC_PROLONG32 = 3,    // FP32 prolongation + correction         8.5 B/cell
    PC_ADDCORR = 4,      // FP64 x += e                             20 B/cell
    PC_TAIL32 = 5,       // FP32 single-CTA coarse tail
    PC_SMOOTH64 = 6,     // FP64 RBGS half-sweep                    16 B/cell
    PC_RES64 = 7,        // FP64 residual (+norm)                   24 B/cell
    PC_RESTRICT64 = 8,   // FP64 restriction                         9 B/cell
    PC_PROLONG64 = 9,    // FP64 prolongation + correction          17 B/cell
    PC_TAIL64 = 10,      // FP64 single-CTA coarse tail
    PC_UPDATE_RES = 11,  // x += e, r -= A e, FP32 copy, norm       40 B/cell
    PC_COARSE32 = 12,    // FP32 grid levels below the finest (smoothing and transfers)
    PC_COARSE64 = 13,    // FP64 grid levels below the finest (smoothing, residual, transfers)
    PC_COUNT = 14
};
// Number of kernels this library has launched (all contexts).
void count_launches(long long n);
long long launches_total();

// ---- device allocation ------------------------------------------------------------
// Every device allocation of the library goes through dev_malloc: cudaMalloc, unless the
// host-side fault injector (pmg_inject_alloc_failure) has armed a failure, in which case
// the chosen call allocates nothing and fails with cudaErrorMemoryAllocation, as cudaMalloc
// does when the device memory is exhausted.
cudaError_t dev_malloc_bytes(void **p, size_t bytes);
template <typename T>
inline cudaError_t dev_malloc(T **p, size_t bytes)
{
    return dev_malloc_bytes(reinterpret_cast<void **>(p), bytes);
}
// Releases what dev_malloc returned: cudaFree, except for memory of a device arena (which
// frees its chunks when it is destroyed).  nullptr is accepted.
cudaError_t dev_free(void *p);

// A device arena: a bump allocator over large device chunks (256 MiB, or the request when
// larger; 256-byte aligned pieces).  While an ArenaScope is alive on a thread, every
// dev_malloc of that thread takes its memory from the scope's arena, so building many
// small hierarchies (a batch's problems) costs a few cudaMalloc calls instead of thousands.
struct DevArena;
DevArena *arena_create();
void arena_destroy(DevArena *a);
struct ArenaScope {
    explicit ArenaScope(DevArena *a);
    ~ArenaScope();
    ArenaScope(const ArenaScope &) = delete;
    ArenaScope &operator=(const ArenaScope &) = delete;
    DevArena *prev;
};

// ---- tracing ----------------------------------------------------------------------
// An NVTX range over a scope: the solve, its cycles and their phases appear by name in
// Nsight Systems and in `ncu --nvtx` filters.  Without a tool attached a range costs a few
// nanoseconds on the host.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// ---- errors ---------------------------------------------------------------------
void set_error(const std::string &msg);
int cuda_status(cudaError_t e, const char *what);

// Runs f() (returning a status) so that no C++ exception leaves the C interface: a host
// allocation that throws becomes PMG_ENOMEM, anything else PMG_ECUDA with its message.
template <class F>
int guarded(F &&f)
{
    try {
        return f();
    } catch (const std::bad_alloc &) {
        set_error("host allocation failed");
        return PMG_ENOMEM;
    } catch (const std::exception &e) {
        set_error(std::string("internal error: ") + e.what());
        return PMG_ECUDA;
    } catch (...) {
        set_error("internal error");
        return PMG_ECUDA;
    }
}

}  // namespace pmg
