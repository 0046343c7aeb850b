// pmg_batch.cu -- many independent Poisson problems of uneven sizes solved together.
//
// Every problem has its own hierarchy (the CGS level rules with as many levels as its
// sizes allow, uniform or given meshes) and is solved in mixed precision: FP32 V-cycles
// inside FP64 defect correction, exactly the per-problem algorithm of pmg_mixed.cu.  The
// batch runs depth by depth: each operation of the V-cycle at depth d is ONE persistent
// launch over a work list of (problem, tile) items gathered from every problem that has
// that depth; the coarsest-level solves are one launch with one CTA per problem.  One
// outer correction -- the FP32 V-cycles, the FP64 correction, the FP64 residual, the
// per-problem norms and convergence test -- is captured once in a CUDA graph and then
// replayed.  Converged problems skip their work items, so their results stay those of
// the correction at which they converged; a problem predicted to end with a correction
// skips that correction's last V-cycle when its inner residual already meets the tolerance.
//
// The smoother (register-window or TMA-fed kernel, tiles of 60 columns by 6, 10, 14 or 22
// rows, k-chunk) is chosen per depth by timing the batch's own work lists (autotuning at the
// first solve).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "pmg_cell32.cuh"
#include "pmg_ctx.h"
#include "pmg_mixed.h"
#include "pmg_smooth32.cuh"
#include "pmg_smooth32_tma.cuh"

#define PMG_TRY_B(expr)                \
    do {                               \
        int _rc = (expr);              \
        if (_rc != PMG_OK) return _rc; \
    } while (0)

namespace pmg {

namespace {

constexpr int NTB = 256;
constexpr int kVariants = 7;   // smoother variants: register-window TY 14/6/10, TMA-fed TY 14/6/10/22

// per (depth, problem) descriptor
struct BLevel {
    LevelK<float> L;
    XferK<float> X;        // transfer to depth + 1 (valid when depth < nl)
    float *e[2];
    float *b;
    int nl;                // coarsest depth of the problem
    int kchunk;
};

// per problem, finest level
struct BOuter {
    LevelK<double> L;
    const double *dyy, *dzz;
    double *sol, *rsd;
    const double *rhs;
    int sy32;
    long long sz32;
    float *r32;
    float *e0;             // the depth-0 correction buffer the V-cycle leaves its result in
    SplitCoef sc;          // coefficients as FP32 pairs (residual update)
};

struct Item {
    // problem and: smoother -- tile (bx, by), first plane k0; transfers -- column block bx,
    // chunk of by coarse planes from k0
    int p, bx, by, k0;
};

// ---- smoother ----------------------------------------------------------------------------
template <int TY, bool ZERO_IN, bool OMEGA1>
__global__ void __launch_bounds__(rb_threads<TY>()) k_batch_rb32(const BLevel *__restrict__ lv,
                                                                 const Item *__restrict__ items, int nitems, int which,
                                                                 float omega, float omw, const int *__restrict__ done)
{
    __shared__ __align__(16) RbSmem<TY> S;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const Item w = items[it];
        if (done[w.p]) continue;
        const BLevel &D = lv[w.p];
        const LevelK<float> L = D.L;
        const int k1 = min(L.nz, w.k0 + D.kchunk - 1);
        rb32_item<TY, ZERO_IN, OMEGA1>(S, L, D.e[which], D.e[1 - which], D.b, omega, omw, w.bx, w.by, w.k0, k1);
    }
}

// ---- TMA-fed smoother over a (problem, tile) list ------------------------------------------
// Item source of the TMA-fed smoother for one depth: the CTA's items of unconverged
// problems in list order, each item's planes from its problem's k-chunk and the tensor
// maps of its problem (buffer `which` of e as input, tile variant vi).
struct BatchTmaArgs {
    const BLevel *lv;
    const Rb32Tma *maps;
    const Item *items;
    const int *done;
    int nitems, which, vi;
};

// Reads its fields through a pointer to the kernel parameter (the constant bank), so the
// persistent CTA holds no registers for them across its items.
struct BatchTmaSrc {
    const BatchTmaArgs *A;
    __device__ __forceinline__ int skip(int it) const
    {
        while (it < A->nitems && A->done[A->items[it].p]) it += gridDim.x;
        return it;
    }
    __device__ __forceinline__ int first() const { return skip(blockIdx.x); }
    __device__ __forceinline__ int next(int it) const { return skip(it + gridDim.x); }
    __device__ __forceinline__ bool valid(int it) const { return it < A->nitems; }
    __device__ __forceinline__ void geom(int it, int &bx, int &by, int &k0, int &k1) const
    {
        const Item w = A->items[it];
        bx = w.bx;
        by = w.by;
        k0 = w.k0;
        k1 = min(A->lv[w.p].L.nz, w.k0 + A->lv[w.p].kchunk - 1);
    }
    __device__ __forceinline__ const CUtensorMap *map_e(int it) const
    {
        return &A->maps[A->items[it].p].e[A->which][A->vi];
    }
    __device__ __forceinline__ const CUtensorMap *map_b(int it) const { return &A->maps[A->items[it].p].b[A->vi]; }
    static constexpr bool kStall = false;
    __device__ __forceinline__ bool stall() const { return false; }
};

template <int TY, bool ZERO_IN, bool OMEGA1>
__global__ void __launch_bounds__(RbtShape<TY>::THREADS, rbt_min_ctas<TY>())
    k_batch_rb32_tma(const __grid_constant__ BatchTmaArgs A, float omega, float omw, int *err)
{
    const BatchTmaSrc src{&A};
    rbt_cta<TY, ZERO_IN, OMEGA1>(
        src,
        [&](int it, const LevelK<float> *&L, float *&eo) {
            const BLevel &D = A.lv[A.items[it].p];
            L = &D.L;
            eo = D.e[1 - A.which];
        },
        omega, omw, err);
}

// ---- residual + restriction into depth d+1, prolongation + correction back ----------------
// An item is (problem, block bx of NTB consecutive columns, chunk of `by` coarse planes
// from k0): a column is one thread's marching column (a coarse column of the residual-
// restriction, a fine x-pair column of the prolongation) or, where an axis is no longer
// halved, one coarse cell per plane.  One chunk length per depth (set from the depth's
// total work, like the single-grid kernels' chunks) gives items of equal size, which keep
// the CTAs of a launch equally busy whatever the problems' sizes.

// NORM (the inner residual check of a correction predicted to end a problem's solve):
// also one partial per item of the fine residual's squared norm (FP32 per-thread sums
// scaled by a power of two near 1 / (1e-10 rms r0), so residuals near the tolerance stay
// in FP32's range), from the marching path only (a problem whose depth-0 transfer does not
// halve every axis is never checked).
template <bool NORM>
__global__ void __launch_bounds__(NTB, 3) k_batch_resrestrict(const BLevel *__restrict__ lvd,
                                                           const BLevel *__restrict__ lvc, const Item *__restrict__ items,
                                                           int nitems, int which, const int *__restrict__ skip,
                                                           double *__restrict__ partials,
                                                           const double *__restrict__ res0,
                                                           const int *__restrict__ mode)
{
    __shared__ double sw[NORM ? NTB / 32 : 1];
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const Item w = items[it];
        // (the check only concerns problems predicted to end with this correction)
        if (skip[w.p] || (NORM && !mode[w.p])) continue;        // uniform over the block
        const BLevel &D = lvd[w.p];
        const XferK<float> X = D.X;
        const LevelK<float> L = D.L;
        const float *e = D.e[which];
        float *bc = lvc[w.p].b;
        const int m0 = w.k0, m1 = min(X.ncz, w.k0 + w.by - 1);
        const int q = w.bx * NTB + threadIdx.x;
        float ss = 0.f, nscale = 1.f;
        if (NORM) {
            const double rms = sqrt(res0[w.p] / ((double)L.nx * L.ny * L.nz)) * 1e-10;
            const int ex = rms > 0.0 && rms < 1e300 ? max(-100, min(100, ilogb(rms))) : 0;
            nscale = ldexpf(1.0f, -ex);
        }
        if (q < X.ncx * X.ncy) {
            const int i = q % X.ncx + 1, j = q / X.ncx + 1;
            if (X.stx == 2 && X.sty == 2 && X.stz == 2) {
                resrestrict_column_march32<NORM>(L, X, i, j, m0, m1, e, D.b, bc, nscale, &ss);
            } else {
                for (int k = m0; k <= m1; ++k)
                    bc[lin(i, j, k, X.csy, X.csz)] = resrestrict_cell32(L, X, e, D.b, i, j, k);
            }
        }
        if (NORM) {
            const double t = block_sum((double)ss, sw);
            if (threadIdx.x == 0) partials[it] = t / ((double)nscale * (double)nscale);
        }
    }
}

__global__ void __launch_bounds__(NTB, 3) k_batch_prolong(const BLevel *__restrict__ lvd, const BLevel *__restrict__ lvc,
                                                       const Item *__restrict__ items, int nitems, int which,
                                                       int which_c, int d, const int *__restrict__ done)
{
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const Item w = items[it];
        if (done[w.p]) continue;
        const BLevel &D = lvd[w.p];
        const XferK<float> X = D.X;
        // the coarsest depth of a problem is solved in place in buffer 0
        const float *ec = (d + 1 == D.nl) ? lvc[w.p].e[0] : lvc[w.p].e[which_c];
        float *e = D.e[which];
        const int m0 = w.k0, m1 = min(X.ncz, w.k0 + w.by - 1);
        const int q = w.bx * NTB + threadIdx.x;
        if (X.stx == 2 && X.stz == 2) {
            // one thread per fine x-pair column of the item's planes
            if (q >= X.ncx * D.L.ny) continue;
            prolong_column_march32(X, q / X.ncx + 1, q % X.ncx + 1, m0, m1, ec, e);
        } else {
            if (q >= X.ncx * X.ncy) continue;
            const int i = q % X.ncx + 1, j = q / X.ncx + 1;
            for (int k = m0; k <= m1; ++k) prolong_add_cell32(X, ec, e, i, j, k);
        }
    }
}

// ---- outer FP64 kernels: one item per fine plane ------------------------------------------
// nonzero[p] |= 1 unless problem p's initial guess (its whole packed range, ghosts
// included) is +0 everywhere; grid (blocks per problem, problems).
__global__ void __launch_bounds__(NTB) k_batch_nonzero(const double *__restrict__ sol,
                                                       const long long *__restrict__ offset, int *__restrict__ nonzero)
{
    const int p = blockIdx.y;
    const unsigned long long *u = reinterpret_cast<const unsigned long long *>(sol);
    unsigned long long bits = 0ull;
    const long long end = offset[p + 1], stride = (long long)gridDim.x * NTB;
    long long q = offset[p] + blockIdx.x * (long long)NTB + threadIdx.x;
    for (; q + 3 * stride < end; q += 4 * stride) {
        unsigned long long v[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) v[t] = __ldg(u + q + t * stride);
        bits |= v[0] | v[1] | v[2] | v[3];
    }
    for (; q < end; q += stride) bits |= __ldg(u + q);
    if (__syncthreads_or(bits != 0ull) && threadIdx.x == 0) atomicOr(nonzero + p, 1);
}

// An outer item is a set of fine rows of one problem: rows j0 .. j1 of planes k0 .. k1
// (whole planes of small problems, row blocks of large ones), about kOuterCells cells, so
// the per-item set-up (descriptor loads) is spread over enough cells and the items of a
// launch are of about equal size.  Warp w takes the item's rows w, w + 8, ... (in plane-
// major order); lane l the cells i = 1 + l + 32 u of a row.  Each warp leaves its partial
// norm in partials[item * kOuterWarps + w] (no block barrier); the norm kernels sum a
// problem's partials in that order.
constexpr int kOuterWarps = NTB / 32;
constexpr int kOuterCells = 8192;

struct OItem {
    int p, j0, j1, k0, k1;
};

__device__ __forceinline__ double warp_sum_outer(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// check (NULL: every problem): the problems whose residual is recomputed.  nonzero
// (non-NULL for the first residual of a solve): where a problem's initial guess is zero,
// every product of the FMA chain is a signed zero and the chain returns b + 0.
__global__ void __launch_bounds__(NTB, 4) k_batch_outer_residual(const BOuter *__restrict__ po,
                                                                 const OItem *__restrict__ items, int nitems,
                                                                 double *__restrict__ partials,
                                                                 const int *__restrict__ done,
                                                                 const int *__restrict__ check,
                                                                 const int *__restrict__ nonzero)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const OItem w = items[it];
        if (done[w.p] || (check && !check[w.p])) continue;       // uniform over the block
        const BOuter &O = po[w.p];
        const LevelK<double> L = O.L;
        const double *__restrict__ x = O.sol;
        const double *__restrict__ b = O.rhs;
        double *__restrict__ r = O.rsd;
        float *__restrict__ r32 = O.r32;
        const bool zero_x = nonzero && !nonzero[w.p];
        const int nrow = w.j1 - w.j0 + 1, rows = nrow * (w.k1 - w.k0 + 1);
        double acc = 0.0;
        for (int t = wid; t < rows; t += kOuterWarps) {
            const int j = w.j0 + t % nrow, k = w.k0 + t / nrow;
            const long long row = lin(0, j, k, L.sy, L.sz), row32 = lin(0, j, k, O.sy32, O.sz32);
            if (zero_x) {
                for (int i = 1 + lane; i <= L.nx; i += 32) {
                    const double v = plus_zero(b[row + i]);
                    r[row + i] = v;
                    r32[row32 + i] = f64_to_f32_rn(v);
                    acc = fma(v, v, acc);
                }
                continue;
            }
            const double dyz = O.dyy[j] + O.dzz[k];
            for (int i = 1 + lane; i <= L.nx; i += 32) {
                const double v = outer_residual_cell(L, dyz, x, b, i, j, k, row + i);
                r[row + i] = v;
                r32[row32 + i] = f64_to_f32_rn(v);
                acc = fma(v, v, acc);
            }
        }
        acc = warp_sum_outer(acc);
        if (lane == 0) partials[(long long)it * kOuterWarps + wid] = acc;
    }
}

// After the V-cycles of a correction, per outer item: x += e, and for problems in update
// mode (mode 0) also r -= A e with A e in compensated FP32 arithmetic (comp_term), the
// FP32 copy of r and the warps' partial norms (FP32 sums of the squares scaled by a power
// of two set by the problem's initial residual; they only decide whether the residual is
// recomputed).  Problems in mode 1 get the FP64 residual recomputed after this.
__global__ void __launch_bounds__(NTB, 4) k_batch_correct(const BOuter *__restrict__ po,
                                                          const OItem *__restrict__ items, int nitems,
                                                          double *__restrict__ partials,
                                                          const int *__restrict__ done, const int *__restrict__ mode,
                                                          const double *__restrict__ res0)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const OItem w = items[it];
        if (done[w.p]) continue;
        const BOuter &O = po[w.p];
        const LevelK<double> L = O.L;
        double *__restrict__ x = O.sol;
        const float *__restrict__ e = O.e0;
        const int sy32 = O.sy32;
        const long long sz32 = O.sz32;
        const int nrow = w.j1 - w.j0 + 1, rows = nrow * (w.k1 - w.k0 + 1);
        if (mode[w.p]) {
            for (int t = wid; t < rows; t += kOuterWarps) {
                const int j = w.j0 + t % nrow, k = w.k0 + t / nrow;
                const long long row = lin(0, j, k, L.sy, L.sz), row32 = lin(0, j, k, sy32, sz32);
                for (int i = 1 + lane; i <= L.nx; i += 32) x[row + i] = x[row + i] + f32_to_f64(e[row32 + i]);
            }
            continue;
        }
        double *__restrict__ r = O.rsd;
        float *__restrict__ r32 = O.r32;
        const double rms0 = sqrt(res0[w.p] / ((double)L.nx * L.ny * L.nz));
        const int ex = rms0 > 0.0 && rms0 < 1e300 ? max(-100, min(100, ilogb(rms0))) : 0;
        const float nscale = ldexpf(1.0f, -ex);
        const SplitCoef C = O.sc;
        float acc32 = 0.f;
        for (int t = wid; t < rows; t += kOuterWarps) {
            const int j = w.j0 + t % nrow, k = w.k0 + t / nrow;
            const long long row = lin(0, j, k, L.sy, L.sz), row32 = lin(0, j, k, sy32, sz32);
            const float2 cym = C.cym[j], cyp = C.cyp[j], czm = C.czm[k], czp = C.czp[k];
            for (int i = 1 + lane; i <= L.nx; i += 32) {
                const long long c = row32 + i;
                const float ec = e[c];
                float S = 0.f, Sl = 0.f;
                comp_term(C.cxm[i], e[c - 1], ec, S, Sl);
                comp_term(C.cxp[i], e[c + 1], ec, S, Sl);
                comp_term(cym, e[c - sy32], ec, S, Sl);
                comp_term(cyp, e[c + sy32], ec, S, Sl);
                comp_term(czm, e[c - sz32], ec, S, Sl);
                comp_term(czp, e[c + sz32], ec, S, Sl);
                x[row + i] = x[row + i] + f32_to_f64(ec);
                const double v = __dsub_rn(__dsub_rn(r[row + i], f32_to_f64_fast(S)), f32_to_f64_fast(Sl));
                r[row + i] = v;
                const float v32 = f64_to_f32_rn(v);
                r32[c] = v32;
                const float wv = v32 * nscale;
                acc32 = fmaf(wv, wv, acc32);
            }
        }
        const double s = warp_sum_outer((double)acc32 / ((double)nscale * (double)nscale));
        if (lane == 0) partials[(long long)it * kOuterWarps + wid] = s;
    }
}

// After k_batch_correct: the updated residual's ratio of every problem in update mode;
// check[p] = 1 where the FP64 residual is recomputed next: mode 1, an updated ratio below
// the tolerance (or not finite), or the last allowed correction.
__global__ void __launch_bounds__(NTB) k_batch_norms_update(const double *__restrict__ partials,
                                                            const int *__restrict__ first_item,
                                                            const double *__restrict__ res0,
                                                            const int *__restrict__ done, const int *__restrict__ mode,
                                                            const int *__restrict__ cycles, int *__restrict__ check,
                                                            double *__restrict__ cheap, double tol, int max_cycles)
{
    __shared__ double sw[NTB / 32];
    const int p = blockIdx.x;
    if (done[p]) return;
    if (mode[p]) {
        if (threadIdx.x == 0) check[p] = 1;
        return;
    }
    double acc = 0.0;
    for (int q = first_item[p] + threadIdx.x; q < first_item[p + 1]; q += NTB) acc += partials[q];
    const double s = block_sum(acc, sw);
    if (threadIdx.x == 0) {
        const double r = sqrt(s / res0[p]);
        cheap[p] = r;
        check[p] = (r < tol || !(r == r) || cycles[p] + 1 >= max_cycles) ? 1 : 0;
    }
}

// per problem: norm = sum of its items' partials in item order; first = 1 stores res0,
// else the ratio test of src/multigrid.f90:1973 updates done/cycles/ratio.
// Only a recomputed FP64 residual (check[p]) ends a problem; after an update alone the
// ratio is the updated one.  The contraction of the last correction predicts the next:
// where it would pass the tolerance by a factor of 10, the next correction recomputes
// the FP64 residual directly (mode 1) instead of updating it first.
__global__ void __launch_bounds__(NTB) k_batch_norms(const double *__restrict__ partials,
                                                     const int *__restrict__ first_item, double *__restrict__ res0,
                                                     double *__restrict__ ratio, int *__restrict__ done,
                                                     int *__restrict__ cycles, int *__restrict__ ndone, double tol,
                                                     int first, const int *__restrict__ check,
                                                     const double *__restrict__ cheap, int *__restrict__ mode,
                                                     double *__restrict__ prev, double *__restrict__ contraction)
{
    __shared__ double sw[NTB / 32];
    const int p = blockIdx.x;
    if (!first && done[p]) return;
    double acc = 0.0;
    if (first || check[p])
        for (int q = first_item[p] + threadIdx.x; q < first_item[p + 1]; q += NTB) acc += partials[q];
    const double s = block_sum(acc, sw);
    if (threadIdx.x == 0) {
        if (first) {
            res0[p] = s;
            ratio[p] = 1.0;
            cycles[p] = 0;
            done[p] = 0;
            mode[p] = 0;
            prev[p] = 1.0;
            contraction[p] = 1.0;
        } else {
            const double r = check[p] ? sqrt(s / res0[p]) : cheap[p];
            ratio[p] = r;
            cycles[p] += 1;
            if (check[p] && (r < tol || !(r == r))) {
                done[p] = 1;
                atomicAdd(ndone, 1);
            }
            const double c = r / prev[p];
            contraction[p] = c;
            prev[p] = r;
            mode[p] = r * c < 0.1 * tol ? 1 : 0;
        }
    }
}


}  // namespace

// skip[p] = done[p]: the problems the V-cycles of a correction leave out, at its start.
__global__ void k_batch_skip_init(const int *__restrict__ done, int *__restrict__ skip, int n)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) skip[p] = done[p];
}

// After all but the last V-cycle of a correction: a problem predicted to end its solve
// with this correction (mode 1) whose fine inner residual |b - A e|^2 (its items' partials,
// summed in item order) is below thresh (0.95 tol)^2 |r0|^2 runs no more cycles -- the
// residual the correction leaves equals it to about 1e-14 of |r0|, and the FP64 recompute
// of the outer step confirms convergence.  The reference stops after the first cycle that
// meets the tolerance (src/multigrid.f90:1973).
__global__ void __launch_bounds__(NTB) k_batch_inner_stop(const double *__restrict__ partials,
                                                          const int *__restrict__ first,
                                                          const double *__restrict__ res0,
                                                          const int *__restrict__ mode,
                                                          const int *__restrict__ can, int *__restrict__ skip,
                                                          double thresh)
{
    __shared__ double sw[NTB / 32];
    const int p = blockIdx.x;
    if (skip[p] || !mode[p] || !can[p]) return;
    double acc = 0.0;
    for (int q = first[p] + threadIdx.x; q < first[p + 1]; q += NTB) acc += partials[q];
    const double s = block_sum(acc, sw);
    if (threadIdx.x == 0 && s < thresh * res0[p]) skip[p] = 1;
}

// ---------------------------------------------------------------------------------------
// Batch object
// ---------------------------------------------------------------------------------------
struct Batch {
    cudaStream_t stream = nullptr;
    int n = 0, dmax = 0;
    std::vector<std::unique_ptr<Ctx>> probs;
    std::vector<long long> offset;          // element offsets of each problem in the packed arrays
    long long total = 0;
    // descriptors
    BLevel *d_lv = nullptr;                 // [(dmax+1) * n]
    BOuter *d_outer = nullptr;
    std::vector<BOuter> h_outer;
    // work lists
    struct List {
        Item *d = nullptr;
        int n = 0;
    };
    std::vector<List> smooth;               // [depth]: (problem, tile, k-chunk) items of the chosen variant
    std::vector<List> xfer_rr, xfer_pr;     // [depth]: items of the residual-restriction into depth+1 and
                                            // of the prolongation back (problems with nl > depth)
    struct OList {
        OItem *d = nullptr;
        int n = 0;
    } outer;                                // row sets of the finest level
    std::vector<int> first_item;            // per problem range of the outer partials (kOuterWarps per item)
    int *d_first = nullptr;
    double *d_partials = nullptr, *d_res0 = nullptr, *d_ratio = nullptr;
    int *d_done = nullptr, *d_cycles = nullptr, *d_ndone = nullptr;
    // the V-cycles' problem mask (done, or stopped early within a correction) and the
    // inner residual check: per-item partials of the depth-0 residual-restriction, each
    // problem's first item there, whether the check applies to it (marching depth-0 transfer)
    int *d_skip = nullptr;
    double *d_rr_part = nullptr;
    int *d_rr_first = nullptr, *d_can_check = nullptr;
    bool any_check = false;
    // residual update state per problem: mode (1: recompute directly), check (recompute
    // after this correction's update), updated ratio, previous ratio, last contraction
    int *d_mode = nullptr, *d_check = nullptr;
    int *d_nonzero = nullptr;               // per problem: the initial guess has a non-zero value
    long long *d_offset = nullptr;          // device copy of offset
    const double *cur_sol = nullptr;        // the packed solution of the running solve
    double *d_cheap = nullptr, *d_prev = nullptr, *d_contr = nullptr;
    int graph_maxcyc = -1;
    double *rsd = nullptr;                  // packed FP64 residual
    const TailDesc<float> **d_tails = nullptr;
    int tail_threads = 64;
    std::vector<BLevel> h_lv;               // host copy of d_lv
    std::vector<int> variant, kchunk;       // chosen smoother variant (kVariantTY) and k-chunk per depth
    int slots[kVariants] = {};
    Rb32Tma *d_maps = nullptr;              // [(dmax+1) * n] tensor maps of every depth and problem
    std::vector<bool> tma_ok;               // per depth: every problem with that depth has maps
    int *d_err = nullptr;                   // set by a TMA-fed launch whose bounded wait gave up
    cudaGraphExec_t graph = nullptr;
    int graph_maxit = -1;
    double graph_omega = 0.0, graph_tol = 0.0;
    int inner = 2;
    // every device allocation of the batch and of its problems' hierarchies comes from this
    // arena (a few large cudaMalloc calls instead of thousands); released last
    DevArena *arena = nullptr;
    ~Batch();
};

Batch::~Batch()
{
    if (graph) cudaGraphExecDestroy(graph);
    dev_free(d_lv);
    dev_free(d_outer);
    for (auto &l : smooth) dev_free(l.d);
    for (auto &l : xfer_rr) dev_free(l.d);
    for (auto &l : xfer_pr) dev_free(l.d);
    dev_free(outer.d);
    dev_free(d_first);
    dev_free(d_partials);
    dev_free(d_res0);
    dev_free(d_ratio);
    dev_free(d_done);
    dev_free(d_skip);
    dev_free(d_rr_part);
    dev_free(d_rr_first);
    dev_free(d_can_check);
    dev_free(d_cycles);
    dev_free(d_mode);
    dev_free(d_nonzero);
    dev_free(d_offset);
    dev_free(d_check);
    dev_free(d_cheap);
    dev_free(d_prev);
    dev_free(d_contr);
    dev_free(d_ndone);
    dev_free(rsd);
    dev_free(d_tails);
    dev_free(d_maps);
    dev_free(d_err);
    if (stream) cudaStreamSynchronize(stream);
    probs.clear();
    arena_destroy(arena);
}

}  // namespace pmg

// ---------------------------------------------------------------------------------------
// Creation, scheduling, graph and solve
// ---------------------------------------------------------------------------------------
namespace pmg {

namespace {

int v2(int n)
{
    int c = 0;
    while (n > 0 && n % 2 == 0) {
        n /= 2;
        ++c;
    }
    return c;
}

template <typename T>
int upload(const std::vector<T> &h, T **d)
{
    if (h.empty()) return PMG_OK;
    int rc = cuda_status(dev_malloc(d, h.size() * sizeof(T)), "batch allocation");
    if (rc != PMG_OK) return rc;
    return cuda_status(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice), "batch upload");
}

constexpr int kVariantTY[kVariants] = {14, 6, 10, 14, 6, 10, 22};   // tile height of each smoother variant

template <int TY>
int setup_variant(int *slots)
{
    int per = 0, dev = 0, sms = 0;
    int rc = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_rb32<TY, false, false>,
                                                                       rb_threads<TY>(), 0),
                         "batch smoother occupancy");
    if (rc != PMG_OK) return rc;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    *slots = std::max(1, per) * std::max(1, sms);
    return PMG_OK;
}

template <int TY, bool Z, bool O>
int tma_batch_attr()
{
    int rc = cuda_status(cudaFuncSetAttribute(k_batch_rb32_tma<TY, Z, O>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              RbtShape<TY>::SMEM),
                         "batch TMA smoother shared memory");
    if (rc != PMG_OK) return rc;
    return cuda_status(cudaFuncSetAttribute(k_batch_rb32_tma<TY, Z, O>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                            100),
                       "batch TMA smoother carveout");
}

template <int TY>
int setup_tma_variant(int *slots)
{
    PMG_TRY_B((tma_batch_attr<TY, false, false>()));
    PMG_TRY_B((tma_batch_attr<TY, false, true>()));
    PMG_TRY_B((tma_batch_attr<TY, true, false>()));
    PMG_TRY_B((tma_batch_attr<TY, true, true>()));
    int per = 0, dev = 0, sms = 0;
    PMG_TRY_B(cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_rb32_tma<TY, false, false>,
                                                                        RbtShape<TY>::THREADS, RbtShape<TY>::SMEM),
                          "batch TMA smoother occupancy"));
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    *slots = std::max(1, per) * std::max(1, sms);
    return PMG_OK;
}

template <int TY>
void launch_batch_tma(const Batch &B, int d, const Batch::List &Ls, int slots, int vi, int which, float om, float omw,
                      bool zs)
{
    const int grid = std::max(1, std::min(Ls.n, slots));
    const BLevel *lv = B.d_lv + (size_t)d * B.n;
    const Rb32Tma *mp = B.d_maps + (size_t)d * B.n;
    const bool one = om == 1.f;
    constexpr int nt = RbtShape<TY>::THREADS, sm = RbtShape<TY>::SMEM;
    const BatchTmaArgs A{lv, mp, Ls.d, B.d_skip, Ls.n, which, vi};
    if (zs && one)
        k_batch_rb32_tma<TY, true, true><<<grid, nt, sm, B.stream>>>(A, om, omw, B.d_err);
    else if (zs)
        k_batch_rb32_tma<TY, true, false><<<grid, nt, sm, B.stream>>>(A, om, omw, B.d_err);
    else if (one)
        k_batch_rb32_tma<TY, false, true><<<grid, nt, sm, B.stream>>>(A, om, omw, B.d_err);
    else
        k_batch_rb32_tma<TY, false, false><<<grid, nt, sm, B.stream>>>(A, om, omw, B.d_err);
}

template <int TY>
void launch_batch_rb(const Batch &B, int d, const Batch::List &Ls, int slots, int which, float om, float omw, bool zs)
{
    const int grid = std::max(1, std::min(Ls.n, slots));
    const BLevel *lv = B.d_lv + (size_t)d * B.n;
    const bool one = om == 1.f;
    const int nt = rb_threads<TY>();
    if (zs && one)
        k_batch_rb32<TY, true, true><<<grid, nt, 0, B.stream>>>(lv, Ls.d, Ls.n, which, om, omw, B.d_skip);
    else if (zs)
        k_batch_rb32<TY, true, false><<<grid, nt, 0, B.stream>>>(lv, Ls.d, Ls.n, which, om, omw, B.d_skip);
    else if (one)
        k_batch_rb32<TY, false, true><<<grid, nt, 0, B.stream>>>(lv, Ls.d, Ls.n, which, om, omw, B.d_skip);
    else
        k_batch_rb32<TY, false, false><<<grid, nt, 0, B.stream>>>(lv, Ls.d, Ls.n, which, om, omw, B.d_skip);
}

// Smoother over the work list Ls of depth d with variant v: 0, 1, 2 the register-window
// kernel with 60 x 14 / 6 / 10 tiles; 3, 4, 5, 6 the TMA-fed kernel with 60 x 14 / 6 / 10
// / 22 tiles (tensor-map variant v - 3).
void launch_rb(const Batch &B, int v, int d, const Batch::List &Ls, int which, float om, float omw, bool zs)
{
    if (!Ls.n) return;
    switch (v) {
    case 0: launch_batch_rb<14>(B, d, Ls, B.slots[0], which, om, omw, zs); break;
    case 1: launch_batch_rb<6>(B, d, Ls, B.slots[1], which, om, omw, zs); break;
    case 2: launch_batch_rb<10>(B, d, Ls, B.slots[2], which, om, omw, zs); break;
    case 3: launch_batch_tma<14>(B, d, Ls, B.slots[3], 0, which, om, omw, zs); break;
    case 4: launch_batch_tma<6>(B, d, Ls, B.slots[4], 1, which, om, omw, zs); break;
    case 5: launch_batch_tma<10>(B, d, Ls, B.slots[5], 2, which, om, omw, zs); break;
    default: launch_batch_tma<22>(B, d, Ls, B.slots[6], 3, which, om, omw, zs); break;
    }
    count_launches(1);
}

// The (problem, tile, k-chunk) items of depth d for tile height ty and k-chunk kc (each
// problem's chunk is min(nz, kc)), every problem with a level below depth d.
std::vector<Item> smooth_items(const Batch &B, int d, int ty, int kc)
{
    std::vector<Item> it;
    for (int p = 0; p < B.n; ++p) {
        if (B.probs[p]->nl <= d) continue;
        const BLevel &x = B.h_lv[(size_t)d * B.n + p];
        const int kch = std::min(x.L.nz, kc);
        const int ntx = (x.L.nx + RB_TX - 1) / RB_TX, nty = (x.L.ny + ty - 1) / ty;
        for (int k0 = 1; k0 <= x.L.nz; k0 += kch)
            for (int by = 0; by < nty; ++by)
                for (int bx = 0; bx < ntx; ++bx) it.push_back({p, bx, by, k0});
    }
    return it;
}

// Sets the k-chunk of depth d's descriptors (host and device copies) to min(nz, kc).
int set_kchunk(Batch &B, int d, int kc)
{
    for (int p = 0; p < B.n; ++p) {
        BLevel &x = B.h_lv[(size_t)d * B.n + p];
        x.kchunk = std::min(x.L.nz, kc);
    }
    return cuda_status(cudaMemcpy(B.d_lv + (size_t)d * B.n, B.h_lv.data() + (size_t)d * B.n, B.n * sizeof(BLevel),
                                  cudaMemcpyHostToDevice),
                       "batch descriptors");
}

int grid_for(int items) { return std::max(1, std::min(items, 8 * 152)); }

}  // namespace

int batch_create(Batch **out, int n, const int *dims, const double *const *meshes, int inner, cudaStream_t user)
{
    (void)user;
    *out = nullptr;
    if (n <= 0 || !dims) {
        set_error("batch needs at least one problem and its sizes");
        return PMG_EINVAL;
    }
    std::unique_ptr<Batch> B(new (std::nothrow) Batch());
    if (!B) return PMG_ENOMEM;
    B->arena = arena_create();
    if (!B->arena) return PMG_ENOMEM;
    ArenaScope scope(B->arena);
    B->n = n;
    B->inner = inner > 0 ? inner : 2;
    PMG_TRY_B(cuda_status(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking), "batch stream"));
    B->offset.assign((size_t)n + 1, 0);
    for (int p = 0; p < n; ++p) {
        const int nx = dims[3 * p], ny = dims[3 * p + 1], nz = dims[3 * p + 2];
        if (nx < 1 || ny < 1 || nz < 1) {
            set_error("batch problem sizes must be positive");
            return PMG_EINVAL;
        }
        const int nl = std::max(v2(nx), std::max(v2(ny), v2(nz)));
        if (nl < 2) {
            set_error("every batch problem needs at least two coarsening levels (an axis divisible by 4)");
            return PMG_EINVAL;
        }
        std::vector<double> ax[3][3];
        const double *mp[9];
        const int nn[3] = {nx, ny, nz};
        const double h = 1.0 / (double)std::max(nx, std::max(ny, nz));   // cubic cells
        for (int d = 0; d < 3; ++d) {
            if (meshes && meshes[6 * p + 2 * d] && meshes[6 * p + 2 * d + 1]) {
                mp[3 * d] = meshes[6 * p + 2 * d];
                mp[3 * d + 1] = meshes[6 * p + 2 * d + 1];
                mp[3 * d + 2] = nullptr;
            } else {
                // uniform mesh of cubic cells of width 1/max(nx,ny,nz), so the longest axis
                // spans [0,1] (src/geometry.f90:180-189)
                auto &dm = ax[d][0], &dg = ax[d][1], &xg = ax[d][2];
                const int m = nn[d];
                dm.assign((size_t)m + 2, 0.0);
                dg.assign((size_t)m + 2, 0.0);
                xg.assign((size_t)m + 2, 0.0);
                for (int i = 1; i <= m; ++i) {
                    dm[i] = h;
                    dg[i] = 0.5 * (dm[i] + dm[i - 1]);
                    xg[i] = xg[i - 1] + dg[i];
                }
                dg[m + 1] = 0.5 * (dm[m + 1] + dm[m]);
                xg[m + 1] = xg[m] + dg[m + 1];
                mp[3 * d] = dm.data();
                mp[3 * d + 1] = dg.data();
                mp[3 * d + 2] = xg.data();
            }
        }
        pmg_config_t cfg;
        std::memset(&cfg, 0, sizeof(cfg));
        cfg.nx = nx; cfg.ny = ny; cfg.nz = nz;
        cfg.dxm = mp[0]; cfg.dxg = mp[1]; cfg.xg = mp[2];
        cfg.dym = mp[3]; cfg.dyg = mp[4]; cfg.yg = mp[5];
        cfg.dzm = mp[6]; cfg.dzg = mp[7]; cfg.zg = mp[8];
        cfg.number_of_levels = nl;
        cfg.number_of_vcycles = 1;
        cfg.aggregation_method = PMG_CGS;
        cfg.coarse_solver = PMG_COARSE_RBGS;
        cfg.precision = PMG_MIXED;
        cfg.mixed_inner_cycles = B->inner;
        std::unique_ptr<Ctx> c(new (std::nothrow) Ctx());
        if (!c) return PMG_ENOMEM;
        c->autotune = false;
        c->deep_tail = false;   // the batch runs every depth above the coarsest on its grid launches
        c->light = true;
        PMG_TRY_B(c->build(&cfg, B->stream));
        PMG_TRY_B(c->setup_mixed());
        B->dmax = std::max(B->dmax, c->nl);
        B->offset[p + 1] = B->offset[p] + (long long)c->lv[0].total;
        B->tail_threads = std::max(B->tail_threads, c->tail32_threads);
        B->probs.push_back(std::move(c));
    }
    B->total = B->offset[n];
    const int D = B->dmax;
    // descriptors
    std::vector<BLevel> lv((size_t)(D + 1) * n);
    std::memset(lv.data(), 0, lv.size() * sizeof(BLevel));
    for (int p = 0; p < n; ++p) {
        Ctx &c = *B->probs[p];
        MixedState *m = c.mixed;
        for (int d = 0; d <= c.nl; ++d) {
            BLevel &x = lv[(size_t)d * n + p];
            x.L = m->K[d];
            if (d < c.nl) x.X = m->X[d];
            x.e[0] = m->e[0][d];
            x.e[1] = m->e[1][d];
            x.b = m->b[d];
            if (!rb32_fused_layout_ok(x.L, x.e[0], x.b) || !rb32_fused_layout_ok(x.L, x.e[1], x.b)) {
                set_error("batch problem too large for the fused smoother layout");
                return PMG_EINVAL;
            }
            x.nl = c.nl;
            x.kchunk = std::min(x.L.nz, 32);
        }
    }
    PMG_TRY_B(upload(lv, &B->d_lv));
    // tensor maps of the TMA-fed smoother (encoded by each problem's setup)
    {
        std::vector<Rb32Tma> maps((size_t)(D + 1) * n);
        B->tma_ok.assign((size_t)D + 1, true);
        for (int p = 0; p < n; ++p) {
            MixedState *m = B->probs[p]->mixed;
            for (int d = 0; d <= B->probs[p]->nl; ++d) {
                maps[(size_t)d * n + p] = m->tma[d];
                if (d < B->probs[p]->nl && !m->tma[d].ok) B->tma_ok[d] = false;
            }
        }
        PMG_TRY_B(upload(maps, &B->d_maps));
        PMG_TRY_B(cuda_status(dev_malloc(&B->d_err, sizeof(int)), "batch allocation"));
        PMG_TRY_B(cuda_status(cudaMemset(B->d_err, 0, sizeof(int)), "batch init"));
    }
    // work lists: the smoother's are built by the autotuner at the first solve; the
    // transfers' chunk length per depth gives about four waves of full SMs of threads (as the
    // single-grid marching kernels' chunks)
    B->h_lv = lv;
    B->smooth.resize((size_t)D);
    B->xfer_rr.resize((size_t)D);
    B->xfer_pr.resize((size_t)D);
    int sms = 0;
    {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            sms = 148;
    }
    const double want_threads = 4.0 * sms * 2048.0;
    for (int d = 0; d < D; ++d) {
        std::vector<Item> rr, pr;
        double work_rr = 0.0, work_pr = 0.0;      // columns x coarse planes
        for (int p = 0; p < n; ++p) {
            if (B->probs[p]->nl <= d) continue;
            const XferK<float> &X = lv[(size_t)d * n + p].X;
            const double nfy = lv[(size_t)d * n + p].L.ny;
            work_rr += (double)X.ncx * X.ncy * X.ncz;
            work_pr += (X.stx == 2 && X.stz == 2 ? X.ncx * nfy : (double)X.ncx * X.ncy) * X.ncz;
        }
        // (the residual-restriction marches three fine planes per coarse plane and measured
        // fastest with chunks of at most 8 coarse planes)
        const int kc_rr = (int)std::max(1.0, std::min(8.0, std::ceil(work_rr / want_threads)));
        const int kc_pr = (int)std::max(1.0, std::min(64.0, std::ceil(work_pr / want_threads)));
        std::vector<int> rr_first((size_t)n + 1, 0), can((size_t)n, 0);
        for (int p = 0; p < n; ++p) {
            rr_first[p] = (int)rr.size();
            if (B->probs[p]->nl <= d) continue;
            const XferK<float> &X = lv[(size_t)d * n + p].X;
            const int nfy = lv[(size_t)d * n + p].L.ny;
            const int crr = X.ncx * X.ncy;
            const int cpr = (X.stx == 2 && X.stz == 2) ? X.ncx * nfy : X.ncx * X.ncy;
            for (int k = 1; k <= X.ncz; k += kc_rr)
                for (int c = 0; c * NTB < crr; ++c) rr.push_back({p, c, kc_rr, k});
            for (int k = 1; k <= X.ncz; k += kc_pr)
                for (int c = 0; c * NTB < cpr; ++c) pr.push_back({p, c, kc_pr, k});
            can[p] = X.stx == 2 && X.sty == 2 && X.stz == 2;
        }
        rr_first[n] = (int)rr.size();
        B->xfer_rr[d].n = (int)rr.size();
        B->xfer_pr[d].n = (int)pr.size();
        PMG_TRY_B(upload(rr, &B->xfer_rr[d].d));
        PMG_TRY_B(upload(pr, &B->xfer_pr[d].d));
        if (d == 0) {
            // the inner residual check runs on the depth-0 residual-restriction's items
            for (int p = 0; p < n; ++p) B->any_check = B->any_check || can[p];
            PMG_TRY_B(upload(rr_first, &B->d_rr_first));
            PMG_TRY_B(upload(can, &B->d_can_check));
            if (!rr.empty())
                PMG_TRY_B(cuda_status(dev_malloc(&B->d_rr_part, rr.size() * sizeof(double)), "batch allocation"));
        }
    }
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_skip, n * sizeof(int)), "batch allocation"));
    PMG_TRY_B(cuda_status(cudaMemset(B->d_skip, 0, n * sizeof(int)), "batch init"));
    {
        // outer items: whole planes (up to kOuterCells cells together) or row blocks of a
        // plane (multiples of kOuterWarps rows), in plane order per problem
        std::vector<OItem> it;
        B->first_item.assign((size_t)n + 1, 0);
        for (int p = 0; p < n; ++p) {
            B->first_item[p] = (int)it.size() * kOuterWarps;
            const int *nn = B->probs[p]->lv[0].n;
            const long long plane = (long long)nn[0] * nn[1];
            if (plane >= kOuterCells) {
                int rows = (kOuterCells + nn[0] - 1) / nn[0];
                rows = (rows + kOuterWarps - 1) / kOuterWarps * kOuterWarps;
                for (int k = 1; k <= nn[2]; ++k)
                    for (int j0 = 1; j0 <= nn[1]; j0 += rows) it.push_back({p, j0, std::min(nn[1], j0 + rows - 1), k, k});
            } else {
                const int planes = (int)(kOuterCells / plane);
                for (int k0 = 1; k0 <= nn[2]; k0 += planes) it.push_back({p, 1, nn[1], k0, std::min(nn[2], k0 + planes - 1)});
            }
        }
        B->first_item[n] = (int)it.size() * kOuterWarps;
        B->outer.n = (int)it.size();
        PMG_TRY_B(upload(it, &B->outer.d));
        PMG_TRY_B(upload(B->first_item, &B->d_first));
    }
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_partials, (size_t)B->outer.n * kOuterWarps * sizeof(double)),
                          "batch allocation"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_res0, n * sizeof(double)), "batch allocation"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_ratio, n * sizeof(double)), "batch allocation"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_done, n * sizeof(int)), "batch allocation"));
    PMG_TRY_B(cuda_status(cudaMemset(B->d_done, 0, n * sizeof(int)), "batch init"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_cycles, n * sizeof(int)), "batch allocation"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_mode, n * sizeof(int)), "batch allocation"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_nonzero, n * sizeof(int)), "batch allocation"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_offset, (n + 1) * sizeof(long long)), "batch allocation"));
    PMG_TRY_B(cuda_status(cudaMemcpy(B->d_offset, B->offset.data(), (n + 1) * sizeof(long long),
                                     cudaMemcpyHostToDevice), "batch upload"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_check, n * sizeof(int)), "batch allocation"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_cheap, n * sizeof(double)), "batch allocation"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_prev, n * sizeof(double)), "batch allocation"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_contr, n * sizeof(double)), "batch allocation"));
    PMG_TRY_B(cuda_status(cudaMemset(B->d_check, 0, n * sizeof(int)), "batch init"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->d_ndone, sizeof(int)), "batch allocation"));
    PMG_TRY_B(cuda_status(dev_malloc(&B->rsd, (size_t)B->total * sizeof(double)), "batch allocation"));
    PMG_TRY_B(cuda_status(cudaMemset(B->rsd, 0, (size_t)B->total * sizeof(double)), "batch init"));
    {
        std::vector<const TailDesc<float> *> t((size_t)n);
        for (int p = 0; p < n; ++p) t[p] = B->probs[p]->mixed->d_tail;
        PMG_TRY_B(upload(t, &B->d_tails));
    }
    PMG_TRY_B(setup_variant<14>(&B->slots[0]));
    PMG_TRY_B(setup_variant<6>(&B->slots[1]));
    PMG_TRY_B(setup_variant<10>(&B->slots[2]));
    PMG_TRY_B(setup_tma_variant<14>(&B->slots[3]));
    PMG_TRY_B(setup_tma_variant<6>(&B->slots[4]));
    PMG_TRY_B(setup_tma_variant<10>(&B->slots[5]));
    PMG_TRY_B(setup_tma_variant<22>(&B->slots[6]));
    B->variant.assign((size_t)D, -1);
    B->kchunk.assign((size_t)D, 0);
    B->h_outer.resize((size_t)n);
    *out = B.release();
    return PMG_OK;
}

// Times every smoother variant with k-chunks of 8 .. 128 planes on each depth's work list
// (the register-window kernel stages at most RB_ZC - 3 planes of z coefficients per item)
// and keeps the fastest (variant, k-chunk) with its list.
static int batch_autotune(Batch &B)
{
    cudaEvent_t a, z;
    PMG_TRY_B(cuda_status(cudaEventCreate(&a), "batch tuner"));
    PMG_TRY_B(cuda_status(cudaEventCreate(&z), "batch tuner"));
    const int kcs[] = {8, 16, 32, 64, 128};
    const char *log_env = std::getenv("PEPS_MG_TUNE_LOG");   // print every candidate's time
    const bool log = log_env && log_env[0] == '1';
    int rc = PMG_OK;
    for (int d = 0; d < B.dmax && rc == PMG_OK; ++d) {
        int nzmax = 0;
        long long cells = 0;
        for (int p = 0; p < B.n; ++p)
            if (B.probs[p]->nl > d) {
                const LevelK<float> &L = B.h_lv[(size_t)d * B.n + p].L;
                nzmax = std::max(nzmax, L.nz);
                cells += (long long)L.nx * L.ny * L.nz;
            }
        float best = 1e30f;
        int bv = 0, bk = 32;
        // the register-window kernel only wins on small depths (at most 2^22 cells); the
        // time is unimodal in the k-chunk, so each variant's walk goes up from 16 planes
        // while it stays within 10% of the variant's best (and down to 8 from a minimum at 16)
        for (int v = 0; v < kVariants && rc == PMG_OK; ++v) {
            if (v >= 3 && !B.tma_ok[d]) continue;
            if (v < 3 && B.tma_ok[d] && cells > (1LL << 22)) continue;
            float v_best = 1e30f;
            int v_best_kc = 0;
            auto time_kc = [&](int kc, float *ms) -> bool {
                const std::vector<Item> it = smooth_items(B, d, kVariantTY[v], kc);
                if (it.empty()) return false;
                Batch::List L;
                L.n = (int)it.size();
                rc = upload(it, &L.d);
                if (rc == PMG_OK) rc = set_kchunk(B, d, kc);
                if (rc == PMG_OK) {
                    launch_rb(B, v, d, L, 0, 1.f, 0.f, false);
                    cudaEventRecord(a, B.stream);
                    for (int r = 0; r < 3; ++r) launch_rb(B, v, d, L, 0, 1.f, 0.f, false);
                    cudaEventRecord(z, B.stream);
                    rc = cuda_status(cudaEventSynchronize(z), "batch tuner");
                }
                dev_free(L.d);
                if (rc != PMG_OK) return false;
                cudaEventElapsedTime(ms, a, z);
                if (log)
                    std::fprintf(stderr, "[peps_mg batch tune] depth %d %s TY=%d kchunk=%d items=%d: %.1f us\n", d,
                                 v >= 3 ? "tma" : "window", kVariantTY[v], kc, L.n, *ms * 1e3f / 3.f);
                if (*ms < v_best) {
                    v_best = *ms;
                    v_best_kc = kc;
                }
                if (*ms < best) {
                    best = *ms;
                    bv = v;
                    bk = kc;
                }
                return true;
            };
            for (const int kc : kcs) {
                if (kc < 16 && nzmax > 8) continue;
                if (v < 3 && kc > RB_ZC - 3) break;
                float ms = 0.f;
                if (!time_kc(kc, &ms) || ms > 1.1f * v_best) break;
                if (kc >= nzmax) break;        // larger chunks give the same list
            }
            if (rc == PMG_OK && v_best_kc == 16) {
                float ms = 0.f;
                time_kc(8, &ms);
            }
        }
        if (rc != PMG_OK) break;
        B.variant[d] = bv;
        B.kchunk[d] = bk;
        const std::vector<Item> it = smooth_items(B, d, kVariantTY[bv], bk);
        dev_free(B.smooth[d].d);
        B.smooth[d].d = nullptr;
        B.smooth[d].n = (int)it.size();
        rc = upload(it, &B.smooth[d].d);
        if (rc == PMG_OK) rc = set_kchunk(B, d, bk);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(z);
    if (rc != PMG_OK) {
        B.variant.assign(B.variant.size(), -1);
        return rc;
    }
    return cuda_status(cudaGetLastError(), "batch autotuning");
}

// One FP32 V-cycle on every unconverged problem.
static void batch_vcycle(Batch &B, int maxit, float om, float omw, bool zero_start)
{
    const int D = B.dmax, n = B.n;
    std::vector<int> par((size_t)D + 1, 0);
    auto smooth = [&](int d, bool zs) {
        for (int it = 0; it < maxit; ++it) {
            launch_rb(B, B.variant[d], d, B.smooth[d], par[d], om, omw, zs && it == 0);
            par[d] ^= 1;
        }
    };
    for (int d = 0; d < D; ++d) {
        smooth(d, d > 0 || zero_start);
        const Batch::List &X = B.xfer_rr[d];
        if (X.n) {
            k_batch_resrestrict<false><<<grid_for(X.n), NTB, 0, B.stream>>>(
                B.d_lv + (size_t)d * n, B.d_lv + (size_t)(d + 1) * n, X.d, X.n, par[d], B.d_skip, nullptr, nullptr,
                nullptr);
            count_launches(1);
        }
    }
    batch_tail32(B.d_tails, n, B.d_skip, B.tail_threads, B.stream);
    for (int d = D - 1; d >= 0; --d) {
        const Batch::List &X = B.xfer_pr[d];
        if (X.n) {
            k_batch_prolong<<<grid_for(X.n), NTB, 0, B.stream>>>(B.d_lv + (size_t)d * n, B.d_lv + (size_t)(d + 1) * n,
                                                                 X.d, X.n, par[d], par[d + 1], d, B.d_skip);
            count_launches(1);
        }
        smooth(d, false);
    }
}

// The outer step of a correction (first: the initial residual only).  After the
// V-cycles: x += e with the residual updated (or, in mode 1, left for the recompute), the
// updated ratios, the FP64 residual b - A x recomputed for the problems that may end here,
// and the ratios, convergence flags and next modes.
static void batch_outer(Batch &B, bool first, double tol, int max_cycles)
{
    const int n = B.n;
    if (first) {
        cudaMemsetAsync(B.d_nonzero, 0, n * sizeof(int), B.stream);
        k_batch_nonzero<<<dim3(64, (unsigned)n), NTB, 0, B.stream>>>(B.cur_sol, B.d_offset, B.d_nonzero);
        k_batch_outer_residual<<<grid_for(B.outer.n), NTB, 0, B.stream>>>(B.d_outer, B.outer.d, B.outer.n,
                                                                          B.d_partials, B.d_done, nullptr,
                                                                          B.d_nonzero);
        k_batch_norms<<<n, NTB, 0, B.stream>>>(B.d_partials, B.d_first, B.d_res0, B.d_ratio, B.d_done, B.d_cycles,
                                               B.d_ndone, tol, 1, B.d_check, B.d_cheap, B.d_mode, B.d_prev,
                                               B.d_contr);
        count_launches(3);
        return;
    }
    k_batch_correct<<<grid_for(B.outer.n), NTB, 0, B.stream>>>(B.d_outer, B.outer.d, B.outer.n, B.d_partials,
                                                               B.d_done, B.d_mode, B.d_res0);
    k_batch_norms_update<<<n, NTB, 0, B.stream>>>(B.d_partials, B.d_first, B.d_res0, B.d_done, B.d_mode, B.d_cycles,
                                                  B.d_check, B.d_cheap, tol, max_cycles);
    k_batch_outer_residual<<<grid_for(B.outer.n), NTB, 0, B.stream>>>(B.d_outer, B.outer.d, B.outer.n, B.d_partials,
                                                                      B.d_done, B.d_check, nullptr);
    k_batch_norms<<<n, NTB, 0, B.stream>>>(B.d_partials, B.d_first, B.d_res0, B.d_ratio, B.d_done, B.d_cycles,
                                           B.d_ndone, tol, 0, B.d_check, B.d_cheap, B.d_mode, B.d_prev, B.d_contr);
    count_launches(4);
}

int batch_solve(Batch &B, double *sol, const double *rhs, int maxit, double tol, double omega, int max_cycles,
                int *cycles, double *ratio, float *elapsed_ms)
{
    NvtxRange nvtx_range("pmg_batch_solve");
    const int n = B.n;
    if (!sol || !rhs || maxit < 0 || max_cycles < 0) {
        set_error("invalid batch solve arguments");
        return PMG_EINVAL;
    }
    cudaEvent_t e0, e1;
    PMG_TRY_B(cuda_status(cudaEventCreate(&e0), "batch event"));
    PMG_TRY_B(cuda_status(cudaEventCreate(&e1), "batch event"));
    // the caller's work on the legacy stream (its inputs) comes first
    PMG_TRY_B(cuda_status(cudaEventRecord(e0, 0), "batch event"));
    PMG_TRY_B(cuda_status(cudaStreamWaitEvent(B.stream, e0, 0), "batch event"));
    PMG_TRY_B(cuda_status(cudaEventRecord(e0, B.stream), "batch event"));
    // per-problem outer descriptors (the caller's packed arrays)
    bool changed = false;
    for (int p = 0; p < n; ++p) {
        Ctx &c = *B.probs[p];
        BOuter o;
        std::memset(&o, 0, sizeof(o));
        o.L = c.K[0];
        o.dyy = c.mixed->dyy[0];
        o.dzz = c.mixed->dzz[0];
        o.sy32 = c.mixed->K[0].sy;
        o.sz32 = c.mixed->K[0].sz;
        o.r32 = c.mixed->b[0];
        o.e0 = c.mixed->e[0][0];
        o.sol = sol + B.offset[p];
        o.rhs = rhs + B.offset[p];
        o.rsd = B.rsd + B.offset[p];
        o.sc = c.mixed->sc;
        if (std::memcmp(&o, &B.h_outer[p], sizeof(BOuter)) != 0) changed = true;
        B.h_outer[p] = o;
        PMG_TRY_B(c.upload_tail32(maxit, omega, tol));
    }
    if (!B.d_outer) PMG_TRY_B(cuda_status(dev_malloc(&B.d_outer, n * sizeof(BOuter)), "batch allocation"));
    PMG_TRY_B(cuda_status(cudaMemcpyAsync(B.d_outer, B.h_outer.data(), n * sizeof(BOuter), cudaMemcpyHostToDevice,
                                          B.stream), "batch upload"));
    if (B.variant[0] < 0) PMG_TRY_B(batch_autotune(B));
    PMG_TRY_B(cuda_status(cudaMemsetAsync(B.d_ndone, 0, sizeof(int), B.stream), "batch init"));
    PMG_TRY_B(cuda_status(cudaMemsetAsync(B.d_done, 0, n * sizeof(int), B.stream), "batch init"));
    B.cur_sol = sol;
    batch_outer(B, true, tol, max_cycles);
    const float om = (float)omega, omw = (float)(1.0 - omega);
    if (!B.graph || B.graph_maxit != maxit || B.graph_omega != omega || B.graph_tol != tol ||
        B.graph_maxcyc != max_cycles || changed) {
        if (B.graph) cudaGraphExecDestroy(B.graph);
        B.graph = nullptr;
        cudaGraph_t g;
        PMG_TRY_B(cuda_status(cudaStreamBeginCapture(B.stream, cudaStreamCaptureModeThreadLocal), "graph capture"));
        k_batch_skip_init<<<(n + 255) / 256, 256, 0, B.stream>>>(B.d_done, B.d_skip, n);
        count_launches(1);
        for (int q = 0; q < B.inner; ++q) {
            batch_vcycle(B, maxit, om, omw, q == 0);
            if (q == B.inner - 2 && B.any_check && B.xfer_rr.size() > 0 && B.xfer_rr[0].n > 0) {
                // the inner residual after all but the last cycle (depth-0 e is in buffer 0
                // after a whole V-cycle); problems predicted to end here may stop
                const Batch::List &X = B.xfer_rr[0];
                k_batch_resrestrict<true><<<grid_for(X.n), NTB, 0, B.stream>>>(
                    B.d_lv, B.d_lv + (size_t)n, X.d, X.n, 0, B.d_skip, B.d_rr_part, B.d_res0, B.d_mode);
                k_batch_inner_stop<<<n, NTB, 0, B.stream>>>(B.d_rr_part, B.d_rr_first, B.d_res0, B.d_mode,
                                                            B.d_can_check, B.d_skip, 0.95 * 0.95 * tol * tol);
                count_launches(2);
            }
        }
        batch_outer(B, false, tol, max_cycles);
        PMG_TRY_B(cuda_status(cudaStreamEndCapture(B.stream, &g), "graph capture"));
        const cudaError_t ie = cudaGraphInstantiate(&B.graph, g, 0);
        cudaGraphDestroy(g);
        PMG_TRY_B(cuda_status(ie, "graph instantiate"));
        B.graph_maxit = maxit;
        B.graph_maxcyc = max_cycles;
        B.graph_omega = omega;
        B.graph_tol = tol;
    }
    int ndone = 0;
    for (int c = 0; c < max_cycles && ndone < n; ++c) {
        PMG_TRY_B(cuda_status(cudaGraphLaunch(B.graph, B.stream), "graph launch"));
        PMG_TRY_B(cuda_status(cudaMemcpyAsync(&ndone, B.d_ndone, sizeof(int), cudaMemcpyDeviceToHost, B.stream),
                              "batch progress"));
        PMG_TRY_B(cuda_status(cudaStreamSynchronize(B.stream), "batch sync"));
    }
    PMG_TRY_B(cuda_status(cudaEventRecord(e1, B.stream), "batch event"));
    PMG_TRY_B(cuda_status(cudaEventSynchronize(e1), "batch event"));
    if (elapsed_ms) cudaEventElapsedTime(elapsed_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (cycles) PMG_TRY_B(cuda_status(cudaMemcpy(cycles, B.d_cycles, n * sizeof(int), cudaMemcpyDeviceToHost), "copy"));
    if (ratio) PMG_TRY_B(cuda_status(cudaMemcpy(ratio, B.d_ratio, n * sizeof(double), cudaMemcpyDeviceToHost), "copy"));
    int err = 0;
    PMG_TRY_B(cuda_status(cudaMemcpy(&err, B.d_err, sizeof(int), cudaMemcpyDeviceToHost), "batch error flag"));
    if (err) {
        cudaMemset(B.d_err, 0, sizeof(int));
        set_error("batched smoother: a wait for a TMA copy timed out");
        return PMG_ETIMEOUT;
    }
    return PMG_OK;
}

void batch_destroy(Batch *B)
{
    if (!B) return;
    cudaStreamSynchronize(B->stream);
    cudaStream_t s = B->stream;
    delete B;
    if (s) cudaStreamDestroy(s);
}

void batch_layout(const Batch &B, long long *offsets, int *levels)
{
    for (int p = 0; p <= B.n; ++p)
        if (offsets) offsets[p] = B.offset[p];
    for (int p = 0; p < B.n; ++p)
        if (levels) levels[p] = B.probs[p]->nl;
}

int batch_size(const Batch &B) { return B.n; }

}  // namespace pmg
