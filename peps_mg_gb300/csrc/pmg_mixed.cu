// pmg_mixed.cu -- mixed precision: FP32 V-cycles inside FP64 defect correction.
//
//   r   = b - A x                  (FP64, with the FP64 norm used for convergence)
//   A e = r                        (FP32 V-cycles, e starting at 0, homogeneous ghosts)
//   x   = x + e                    (FP64)
//
// repeated until sqrt(|r|^2 / |r0|^2) < tolerance, the reference's convergence test
// (src/multigrid.f90:1970-1973), always decided on a residual recomputed in FP64.  Between
// corrections that cannot end the solve the residual is updated as r -= A e instead (A e
// in compensated FP32 arithmetic, k_update_residual_march), and x gets those corrections,
// in order, where it is next needed (the stash).
//
// The FP32 V-cycle follows the operation sequence of the reference cycle
// (src/multigrid.f90:1931-1967) with the same smoother, transfer operators and
// coarsest-level solver, but in FP32 arithmetic with FMA contraction and approximate
// reciprocals; the coarsest-level solver's dot products and convergence test stay in FP64.
// The finest FP32 residual is fused with the restriction.  The V-cycles of a correction
// are replayed as CUDA graphs (run_vcycles); a correction predicted to end the solve stops
// its cycles once one inner residual check shows the tolerance met, as the reference stops
// after the first cycle that meets it.
//
// This translation unit is compiled with --fmad=true.
#include <cuda_runtime.h>

#include <cstdlib>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pmg_cell32.cuh"
#include "pmg_ctx.h"
#include "pmg_mixed.h"
#include "pmg_smooth32.cuh"
#include "pmg_smooth32_tma.cuh"

namespace pmg {

namespace {

constexpr int kBX = 32, kBY = 8;
constexpr int kTail32Threads = 512;
constexpr long long kTail32SmemBytes = 128 * 1024;   // dynamic shared memory of an on-chip tail
constexpr int kMaxGridZ = 65535;

__device__ __forceinline__ int tid2() { return threadIdx.x + blockDim.x * threadIdx.y; }
__device__ __forceinline__ int blin() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }

// ---------------------------------------------------------------------------------
// FP32 grid kernels
// ---------------------------------------------------------------------------------
// colour half-sweep; ZERO = the first half-sweep from e = 0, writing every interior
// cell (colour-0 cells get omega b / c0, colour-1 cells 0), so e needs no reset pass.
template <bool ZERO>
__global__ void __launch_bounds__(kBX *kBY) k_rbgs32(LevelK<float> L, float *__restrict__ x,
                                                     const float *__restrict__ b, float omega, float omw, int colour)
{
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y) {
            if (ZERO) {
                for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x) {
                    const long long p = lin(i, j, k, L.sy, L.sz);
                    const bool mine = ((i + j + k + colour) & 1) == 1;
                    x[p] = mine ? __fdividef(omega * b[p], diag32(L, i, j, k)) : 0.f;
                }
            } else {
                const int ista = 1 + ((j + k + colour) & 1);
                for (int i = ista + 2 * (blockIdx.x * blockDim.x + threadIdx.x); i <= L.nx;
                     i += 2 * gridDim.x * blockDim.x)
                    x[lin(i, j, k, L.sy, L.sz)] = rbgs32(L, x, b, i, j, k, omega, omw);
            }
        }
}

__global__ void __launch_bounds__(kBX *kBY, 4) k_resrestrict32(LevelK<float> F, XferK<float> X,
                                                            const float *__restrict__ e, const float *__restrict__ b,
                                                            float *__restrict__ bc)
{
    for (int k = blockIdx.z + 1; k <= X.ncz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= X.ncy; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= X.ncx; i += gridDim.x * blockDim.x)
                bc[lin(i, j, k, X.csy, X.csz)] = resrestrict_cell32(F, X, e, b, i, j, k);
}

// Squared norm of the finest level's inner residual b - A e (FP32 cells, FP64 sum; one
// partial per CTA): the estimate of the outer residual after a correction that ends a
// correction's V-cycles early (Ctx::run_vcycles).
template <int UV>
__global__ void __launch_bounds__(kBX *kBY) k_inner_norm(LevelK<float> L, const float *__restrict__ e,
                                                        const float *__restrict__ b, double *partials)
{
    double acc = 0.0;
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int i0 = blockIdx.x * (blockDim.x * UV) + threadIdx.x + 1; i0 <= L.nx;
                 i0 += gridDim.x * blockDim.x * UV) {
                // UV cells of the row, 32 apart, computed together (their loads in flight at once)
                float v[UV];
#pragma unroll
                for (int u = 0; u < UV; ++u) {
                    const int i = i0 + u * kBX;
                    v[u] = i <= L.nx ? resid32(L, e, b, i, j, k) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < UV; ++u) acc = fma((double)v[u], (double)v[u], acc);
            }
    __shared__ double sw[kBX * kBY / 32];
    const double s = block_sum(acc, sw);
    if (tid2() == 0) partials[blin()] = s;
}

// e_f += P e_c with one thread per fine x-pair (the two x-children of a coarse cell share
// its coarse values), or per fine cell along an x-axis that is no longer coarsened.
__global__ void __launch_bounds__(kBX *kBY) k_prolong_add32(XferK<float> X, int nfy, int nfz,
                                                            const float *__restrict__ vc, float *__restrict__ vf)
{
    for (int kf = blockIdx.z + 1; kf <= nfz; kf += gridDim.z) {
        int kc, kn;
        float az, bz;
        side_weights(X.stz, kf, X.pzp, X.pzn, &kc, &kn, &az, &bz);
        for (int jf = blockIdx.y * blockDim.y + threadIdx.y + 1; jf <= nfy; jf += gridDim.y * blockDim.y) {
            int jc, jn;
            float ay, by;
            side_weights(X.sty, jf, X.pyp, X.pyn, &jc, &jn, &ay, &by);
            const float *r00 = vc + lin(0, jc, kc, X.csy, X.csz), *rn0 = vc + lin(0, jn, kc, X.csy, X.csz);
            const float *r0n = vc + lin(0, jc, kn, X.csy, X.csz), *rnn = vc + lin(0, jn, kn, X.csy, X.csz);
            for (int ic = blockIdx.x * blockDim.x + threadIdx.x + 1; ic <= X.ncx; ic += gridDim.x * blockDim.x) {
                const float c000 = __ldg(r00 + ic), c0n0 = __ldg(rn0 + ic), c00n = __ldg(r0n + ic),
                            c0nn = __ldg(rnn + ic);
                if (X.stx == 2) {
                    const int iz = 2 * ic - 1, ip = 2 * ic;
                    const float lo = prolong_child32(X.pxp[iz], X.pxp[ip], ay, by, az, bz, c000, __ldg(r00 + ic - 1),
                                                     c0n0, c00n, __ldg(rn0 + ic - 1), __ldg(r0n + ic - 1), c0nn,
                                                     __ldg(rnn + ic - 1));
                    const float hi = prolong_child32(X.pxn[ip], X.pxn[iz], ay, by, az, bz, c000, __ldg(r00 + ic + 1),
                                                     c0n0, c00n, __ldg(rn0 + ic + 1), __ldg(r0n + ic + 1), c0nn,
                                                     __ldg(rnn + ic + 1));
                    float *q = vf + lin(iz, jf, kf, X.fsy, X.fsz);
                    q[0] += lo;
                    q[1] += hi;
                } else {
                    const float wx = X.pxn[ic];
                    vf[lin(ic, jf, kf, X.fsy, X.fsz)] +=
                        prolong_child32(wx, wx, ay, by, az, bz, c000, c000, c0n0, c00n, c0n0, c00n, c0nn, c0nn);
                }
            }
        }
    }
}

// e_f += P e_c where x and z are halved: one thread per fine x-pair (coarse x index ic)
// and fine row jf, marching up a chunk of coarse planes (prolong_column_march32).
__global__ void __launch_bounds__(kBX *kBY) k_prolong_march32(XferK<float> X, int nfy, int kchunk, int nchunks,
                                                              const float *__restrict__ vc, float *__restrict__ vf)
{
    for (int ch = blockIdx.z; ch < nchunks; ch += gridDim.z) {
        const int m0 = 1 + ch * kchunk, m1 = min(X.ncz, m0 + kchunk - 1);
        for (int jf = blockIdx.y * blockDim.y + threadIdx.y + 1; jf <= nfy; jf += gridDim.y * blockDim.y)
            for (int ic = blockIdx.x * blockDim.x + threadIdx.x + 1; ic <= X.ncx; ic += gridDim.x * blockDim.x)
                prolong_column_march32(X, jf, ic, m0, m1, vc, vf);
    }
}

// Fused residual + restriction where every axis is halved: one thread per coarse column
// (ic, jc), marching up a chunk of coarse planes (resrestrict_column_march32).  Capped at
// 80 registers (three CTAs per SM): the extra resident warps hide more load latency than
// its few spilled bytes cost (measured 9% faster).
// NORM: also the squared norm of the fine residual (one FP64 partial per CTA, the FP32
// per-thread sums scaled by nscale^2): the inner residual check of Ctx::run_vcycles.
template <bool NORM>
__global__ void __launch_bounds__(kBX *kBY, 3) k_resrestrict_march32(LevelK<float> F, XferK<float> X, int kchunk,
                                                                  int nchunks, const float *__restrict__ e,
                                                                  const float *__restrict__ b,
                                                                  float *__restrict__ bc, float nscale,
                                                                  double *partials)
{
    float ss = 0.f;
    for (int ch = blockIdx.z; ch < nchunks; ch += gridDim.z) {
        const int m0 = 1 + ch * kchunk, m1 = min(X.ncz, m0 + kchunk - 1);
        for (int jc = blockIdx.y * blockDim.y + threadIdx.y + 1; jc <= X.ncy; jc += gridDim.y * blockDim.y)
            for (int ic = blockIdx.x * blockDim.x + threadIdx.x + 1; ic <= X.ncx; ic += gridDim.x * blockDim.x)
                resrestrict_column_march32<NORM>(F, X, ic, jc, m0, m1, e, b, bc, nscale, &ss);
    }
    if (NORM) {
        __shared__ double sw[kBX * kBY / 32];
        const double s = block_sum((double)ss, sw);
        if (tid2() == 0) partials[blin()] = s / ((double)nscale * (double)nscale);
    }
}

// ---------------------------------------------------------------------------------
// FP64 outer kernels
// ---------------------------------------------------------------------------------
// r = b - A x in FP64 (FMA form: r = b + d x - sum c x_nb with d = -c0, the diagonal
// from the per-axis sums dxx = cxm+cxp, dyy, dzz), stored both as the FP64 residual and
// as the FP32 right-hand side of the inner system, with the per-block sum of r^2.
// Each thread handles four cells of a row, 32 apart.
constexpr int kOuterVec = 4;
// *flag |= 1 unless every value of x (ghosts included) is +0 (all bits clear).
__global__ void __launch_bounds__(256) k_nonzero_f64(const double *__restrict__ x, long long n, int *flag)
{
    const unsigned long long *u = reinterpret_cast<const unsigned long long *>(x);
    unsigned long long bits = 0ull;
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; q + 7 * stride < n; q += 8 * stride) {
        unsigned long long v[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) v[t] = __ldg(u + q + t * stride);
#pragma unroll
        for (int t = 0; t < 8; ++t) bits |= v[t];
    }
    for (; q < n; q += stride) bits |= __ldg(u + q);
    if (__syncthreads_or(bits != 0ull) && threadIdx.x == 0) atomicOr(flag, 1);
}


// The part of v that its round-to-nearest FP32 value v32 (f64_to_f32_rn) leaves out, v -
// v32, times 2^nexp, rounded to FP32, from the encodings on the integer pipe: the 29
// mantissa bits the rounding dropped, as a signed count of units 2^(e-52) (negative when
// the rounding went up).  Zero outside the normal FP32 range and where the scaled unit is
// not a normal FP32 number (values far below the ones that make up a norm).
__device__ __forceinline__ float f64_low_part_scaled(double v, int nexp)
{
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;
    const int k = e - 52 + nexp;
    if (e < -126 || e > 127 || k < -126 || k > 127) return 0.f;
    const unsigned long long m = bits & 0xFFFFFFFFFFFFFull;
    const unsigned hi = (unsigned)(m >> 29);
    const int rem = (int)(m & 0x1FFFFFFFull);
    const bool up = rem > 0x10000000 || (rem == 0x10000000 && (hi & 1u));
    const float d = (float)(up ? rem - 0x20000000 : rem) * __int_as_float((k + 127) << 23);
    return (bits >> 63) ? -d : d;
}

// (S, Sl) += (w + wl)^2 to about 2^-46 relative: w^2 exactly as a product and its FMA
// rounding error, 2 w wl on top (wl^2 is below 2^-46 w^2), two-sum into S.
__device__ __forceinline__ void norm_add_ff(float w, float wl, float &S, float &Sl)
{
    const float p = __fmul_rn(w, w);
    float pe = __fmaf_rn(w, w, -p);
    pe = __fmaf_rn(__fmul_rn(2.f, w), wl, pe);
    float sum, err;
    two_sum32(S, p, sum, err);
    S = sum;
    Sl = __fadd_rn(Sl, __fadd_rn(err, pe));
}

// ZS (the first residual of a solve): *nonzero, set by k_nonzero_f64, tells whether the
// initial guess has a non-zero value; where it has none, every product of the FMA chain
// is a signed zero and the chain returns b + 0, so the kernel streams b alone.
// CN: the squared norm is summed on the FP32 and integer pipes instead of by one FP64 FMA
// per cell (the FP64 pipe bounds this kernel): each r = r32 + rl (r32 the FP32 copy, rl
// the low part), scaled by nscale = 2^nexp, squared and summed in an FP32 pair per thread,
// to about 1e-11 relative.  The FP64 residual itself is unchanged.
template <bool ZS, bool CN>
__global__ void __launch_bounds__(kBX *kBY) k_outer_residual(LevelK<double> L, const double *__restrict__ dyy,
                                                             const double *__restrict__ dzz,
                                                             const double *__restrict__ x,
                                                             const double *__restrict__ b, double *__restrict__ r,
                                                             float *__restrict__ r32, int sy32, long long sz32,
                                                             double *partials, const int *__restrict__ nonzero,
                                                             float nscale, int nexp)
{
    double acc = 0.0;
    float accS = 0.f, accL = 0.f;
    const bool zero_x = ZS && *nonzero == 0;
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z) {
        const double dz = dzz[k];
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y) {
            const double dyz = dyy[j] + dz;
            for (int i0 = blockIdx.x * (blockDim.x * kOuterVec) + threadIdx.x + 1; i0 <= L.nx;
                 i0 += gridDim.x * blockDim.x * kOuterVec) {
                if (zero_x) {
                    double bv[kOuterVec];
#pragma unroll
                    for (int u = 0; u < kOuterVec; ++u) {
                        const int i = i0 + u * kBX;
                        bv[u] = i <= L.nx ? b[lin(i, j, k, L.sy, L.sz)] : 0.0;
                    }
#pragma unroll
                    for (int u = 0; u < kOuterVec; ++u) {
                        const int i = i0 + u * kBX;
                        if (i > L.nx) break;
                        const double v = plus_zero(bv[u]);
                        r[lin(i, j, k, L.sy, L.sz)] = v;
                        r32[lin(i, j, k, sy32, sz32)] = f64_to_f32_rn(v);
                        acc = fma(v, v, acc);
                    }
                } else {
#pragma unroll
                    for (int u = 0; u < kOuterVec; ++u) {
                        const int i = i0 + u * kBX;
                        if (i > L.nx) break;
                        const long long p = lin(i, j, k, L.sy, L.sz);
                        const double v = outer_residual_cell(L, dyz, x, b, i, j, k, p);
                        r[p] = v;
                        const float v32 = f64_to_f32_rn(v);
                        r32[lin(i, j, k, sy32, sz32)] = v32;
                        if (CN)
                            norm_add_ff(v32 * nscale, f64_low_part_scaled(v, nexp), accS, accL);
                        else
                            acc = fma(v, v, acc);
                    }
                }
            }
        }
    }
    if (CN) acc = ((double)accS + (double)accL) / ((double)nscale * (double)nscale);
    __shared__ double sw[kBX * kBY / 32];
    const double s = block_sum(acc, sw);
    if (tid2() == 0) partials[blin()] = s;
}

// x = ((x + s0) + s1) + e: the NS stashed corrections s0, s1 (earlier corrections whose
// residual update left x alone), then e unless WITH_E is false, added one at a time in
// the order they were made, so x gets the same bits as when each correction was added at
// once.  Each thread handles kOuterVec cells of a row, 32 apart, with their loads issued
// together, on the grid of the outer kernels.
template <int NS, bool WITH_E>
__global__ void __launch_bounds__(kBX *kBY) k_add_correction(LevelK<double> L, double *__restrict__ x,
                                                             const float *__restrict__ e,
                                                             const float *__restrict__ s0,
                                                             const float *__restrict__ s1, int sy32, long long sz32)
{
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int i0 = blockIdx.x * (blockDim.x * kOuterVec) + threadIdx.x + 1; i0 <= L.nx;
                 i0 += gridDim.x * blockDim.x * kOuterVec) {
                double xv[kOuterVec];
                float ev[kOuterVec], a0[kOuterVec], a1[kOuterVec];
#pragma unroll
                for (int u = 0; u < kOuterVec; ++u) {
                    const int i = i0 + u * kBX;
                    if (i <= L.nx) {
                        const long long q = lin(i, j, k, sy32, sz32);
                        xv[u] = x[lin(i, j, k, L.sy, L.sz)];
                        if (NS > 0) a0[u] = s0[q];
                        if (NS > 1) a1[u] = s1[q];
                        if (WITH_E) ev[u] = e[q];
                    }
                }
#pragma unroll
                for (int u = 0; u < kOuterVec; ++u) {
                    const int i = i0 + u * kBX;
                    if (i <= L.nx) {
                        double v = xv[u];
                        if (NS > 0) v = v + f32_to_f64(a0[u]);
                        if (NS > 1) v = v + f32_to_f64(a1[u]);
                        if (WITH_E) v = v + f32_to_f64(ev[u]);
                        x[lin(i, j, k, L.sy, L.sz)] = v;
                    }
                }
            }
}

// After a correction: x += e and r -= A e (the residual of the corrected x without the
// FP64 stencil; A e in compensated FP32 arithmetic, see comp_term), the FP32 copy of r
// and its norm.  e's ghost cells are zero (the correction has homogeneous boundary
// values), so the difference form covers the boundary cells too.  The norm only decides
// whether the FP64 residual is recomputed (which then decides convergence), so each
// thread sums (nscale r32)^2 in FP32 -- nscale a power of two that brings the initial
// residual's RMS to about 1, keeping the squares in FP32's range for residual ratios
// down to about 1e-19 -- and the block sums the threads' sums in FP64.
template <int UV>
__global__ void __launch_bounds__(kBX *kBY) k_update_residual(LevelK<double> L, SplitCoef C, double *__restrict__ x,
                                                              const float *__restrict__ e, double *__restrict__ r,
                                                              float *__restrict__ r32, int sy32, long long sz32,
                                                              float nscale, double *partials)
{
    float acc32 = 0.f;
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z) {
        const float2 czm = C.czm[k], czp = C.czp[k];
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y) {
            const float2 cym = C.cym[j], cyp = C.cyp[j];
            for (int i0 = blockIdx.x * (blockDim.x * UV) + threadIdx.x + 1; i0 <= L.nx;
                 i0 += gridDim.x * blockDim.x * UV) {
                // every load of the thread's cells first (the kernel is bound by load latency
                // when each cell's loads wait for the previous cell's arithmetic)
                float ev[UV][7];
                double xv[UV], rv[UV];
                float2 cm[UV], cp[UV];
#pragma unroll
                for (int u = 0; u < UV; ++u) {
                    const int i = i0 + u * kBX;
                    if (i <= L.nx) {
                        const long long p = lin(i, j, k, L.sy, L.sz), q = lin(i, j, k, sy32, sz32);
                        ev[u][0] = e[q];
                        ev[u][1] = e[q - 1];
                        ev[u][2] = e[q + 1];
                        ev[u][3] = e[q - sy32];
                        ev[u][4] = e[q + sy32];
                        ev[u][5] = e[q - sz32];
                        ev[u][6] = e[q + sz32];
                        xv[u] = x[p];
                        rv[u] = r[p];
                        cm[u] = C.cxm[i];
                        cp[u] = C.cxp[i];
                    }
                }
#pragma unroll
                for (int u = 0; u < UV; ++u) {
                    const int i = i0 + u * kBX;
                    if (i > L.nx) break;
                    const long long p = lin(i, j, k, L.sy, L.sz), q = lin(i, j, k, sy32, sz32);
                    const float ec = ev[u][0];
                    float S = 0.f, Sl = 0.f;
                    comp_term(cm[u], ev[u][1], ec, S, Sl);
                    comp_term(cp[u], ev[u][2], ec, S, Sl);
                    comp_term(cym, ev[u][3], ec, S, Sl);
                    comp_term(cyp, ev[u][4], ec, S, Sl);
                    comp_term(czm, ev[u][5], ec, S, Sl);
                    comp_term(czp, ev[u][6], ec, S, Sl);
                    x[p] = xv[u] + f32_to_f64(ec);
                    // S and Sl: subnormal parts (below 2^-126) are far below the 2^-48
                    // relative accuracy of A e
                    const double v = __dsub_rn(__dsub_rn(rv[u], f32_to_f64_fast(S)), f32_to_f64_fast(Sl));
                    r[p] = v;
                    const float v32 = f64_to_f32_rn(v);
                    r32[q] = v32;
                    const float w = v32 * nscale;
                    acc32 = fmaf(w, w, acc32);
                }
            }
        }
    }
    __shared__ double sw[kBX * kBY / 32];
    const double inv = 1.0 / ((double)nscale * (double)nscale);
    const double s = block_sum((double)acc32 * inv, sw);
    if (tid2() == 0) partials[blin()] = s;
}

// The same update with one thread per column (i, j) marching up a chunk of planes: e of the
// planes below, at and above the current one stays in registers (the z-neighbours), and
// the next plane's loads (its e neighbours, x and r) are in flight while a plane is
// computed.  Per cell the same operations in the same order as k_update_residual, so r
// and r32 are the same bits; only the norm's summation order differs.  What happens to x:
//  * XM_ADD: x += e;
//  * XM_STASH: x is not touched, e is copied to the stash array s_out (a later
//    k_add_correction or XM_FOLD adds it);
//  * XM_FOLD: x = ((x + s0) + s1) + e, the two stashed corrections and this one.
enum { XM_ADD = 0, XM_STASH = 1, XM_FOLD = 2 };
template <int XM>
__global__ void __launch_bounds__(kBX *kBY, 4) k_update_residual_march(LevelK<double> L, SplitCoef C,
                                                                     double *__restrict__ x,
                                                                     const float *__restrict__ e,
                                                                     double *__restrict__ r, float *__restrict__ r32,
                                                                     int sy32, long long sz32, float nscale,
                                                                     int kchunk, int nchunks, double *partials,
                                                                     float *__restrict__ s_out,
                                                                     const float *__restrict__ s0,
                                                                     const float *__restrict__ s1)
{
    constexpr bool kX = XM != XM_STASH;   // x is read and written
    float acc32 = 0.f;
    for (int ch = blockIdx.z; ch < nchunks; ch += gridDim.z) {
        const int k0 = 1 + ch * kchunk, k1 = min(L.nz, k0 + kchunk - 1);
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y) {
            const float2 cym = C.cym[j], cyp = C.cyp[j];
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x) {
                const float2 cm = C.cxm[i], cp = C.cxp[i];
                const long long c32 = lin(i, j, 0, sy32, sz32);   // the column at plane 0
                const float *ec = e + c32;
                float *rc32 = r32 + c32;
                double *xc = x + lin(i, j, 0, L.sy, L.sz);
                double *rc = r + lin(i, j, 0, L.sy, L.sz);
                // plane k: e below (em), at (e0), above (ep); its x/y neighbours, x and r
                float em = ec[sz32 * (k0 - 1)], e0 = ec[sz32 * k0], ep = ec[sz32 * (k0 + 1)];
                float xl = ec[sz32 * k0 - 1], xr = ec[sz32 * k0 + 1];
                float yd = ec[sz32 * k0 - sy32], yu = ec[sz32 * k0 + sy32];
                double xv = kX ? xc[L.sz * k0] : 0.0, rv = rc[L.sz * k0];
                float a0 = XM == XM_FOLD ? s0[c32 + sz32 * k0] : 0.f;
                float a1 = XM == XM_FOLD ? s1[c32 + sz32 * k0] : 0.f;
                for (int k = k0; k <= k1; ++k) {
                    // plane k+1's loads (its upper neighbour is plane k+2 <= nz+1)
                    float ep2 = 0.f, nxl = 0.f, nxr = 0.f, nyd = 0.f, nyu = 0.f, na0 = 0.f, na1 = 0.f;
                    double nxv = 0.0, nrv = 0.0;
                    if (k < k1) {
                        const long long o = sz32 * (k + 1);
                        ep2 = ec[o + sz32];
                        nxl = ec[o - 1];
                        nxr = ec[o + 1];
                        nyd = ec[o - sy32];
                        nyu = ec[o + sy32];
                        if (kX) nxv = xc[L.sz * (k + 1)];
                        nrv = rc[L.sz * (k + 1)];
                        if (XM == XM_FOLD) {
                            na0 = s0[c32 + o];
                            na1 = s1[c32 + o];
                        }
                    }
                    const float2 czm = C.czm[k], czp = C.czp[k];
                    float S = 0.f, Sl = 0.f;
                    comp_term(cm, xl, e0, S, Sl);
                    comp_term(cp, xr, e0, S, Sl);
                    comp_term(cym, yd, e0, S, Sl);
                    comp_term(cyp, yu, e0, S, Sl);
                    comp_term(czm, em, e0, S, Sl);
                    comp_term(czp, ep, e0, S, Sl);
                    if (XM == XM_ADD) xc[L.sz * k] = xv + f32_to_f64(e0);
                    if (XM == XM_FOLD) xc[L.sz * k] = ((xv + f32_to_f64(a0)) + f32_to_f64(a1)) + f32_to_f64(e0);
                    if (XM == XM_STASH) s_out[c32 + sz32 * k] = e0;
                    const double v = __dsub_rn(__dsub_rn(rv, f32_to_f64_fast(S)), f32_to_f64_fast(Sl));
                    rc[L.sz * k] = v;
                    const float v32 = f64_to_f32_rn(v);
                    rc32[sz32 * k] = v32;
                    const float w = v32 * nscale;
                    acc32 = fmaf(w, w, acc32);
                    a0 = na0;
                    a1 = na1;
                    em = e0;
                    e0 = ep;
                    ep = ep2;
                    xl = nxl;
                    xr = nxr;
                    yd = nyd;
                    yu = nyu;
                    xv = nxv;
                    rv = nrv;
                }
            }
        }
    }
    __shared__ double sw[kBX * kBY / 32];
    const double inv = 1.0 / ((double)nscale * (double)nscale);
    const double s = block_sum((double)acc32 * inv, sw);
    if (tid2() == 0) partials[blin()] = s;
}

// Test hook: convert n values with the integer-pipe conversions.
__global__ void k_convert_test(const double *in64, float *out32, const float *in32, double *out64, int n)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        out32[q] = f64_to_f32_rn(in64[q]);
        out64[q] = f32_to_f64(in32[q]);
    }
}

// ---------------------------------------------------------------------------------
// FP32 single-CTA coarse tail (same sequence as the FP64 tail in pmg_f64.cu); the
// coarsest solver's dot products and its convergence test are FP64.
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(kTail32Threads) k_tail32(const TailDesc<float> *__restrict__ Dp)
{
    __shared__ double sw[kTail32Threads / 32];
    extern __shared__ float tail_sm[];
    if (Dp->sm_floats > 0)
        tail32_body_smem(*Dp, sw, tail_sm);
    else
        tail32_body(*Dp, sw);
}

// One CTA per problem: the coarse tails of a batch (problems marked done are skipped).
__global__ void __launch_bounds__(kTail32Threads) k_batch_tail32(const TailDesc<float> *const *__restrict__ descs,
                                                                 const int *__restrict__ done)
{
    __shared__ double sw[kTail32Threads / 32];
    if (done[blockIdx.x]) return;
    tail32_body(*descs[blockIdx.x], sw);
}

dim3 grid3m(int nxt, int ny, int nz, const Launch &ln)
{
    dim3 g;
    g.x = ln.collapse[0] ? 1u : (unsigned)std::max(1, (nxt + kBX - 1) / kBX);
    g.y = ln.collapse[1] ? 1u : (unsigned)std::max(1, (ny + kBY - 1) / kBY);
    g.z = ln.collapse[2] ? 1u : (unsigned)std::max(1, std::min(nz, kMaxGridZ));
    return g;
}

// Chunks of coarse planes for the marching transfer kernels: about `waves` resident
// threads' worth of (column, chunk) work per SM thread slot.
void march_chunks(long long columns, int ncz, const Launch &ln, int *kchunk, int *nchunks, int waves = 4)
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                      cudaSuccess)
            sms = 148;
    }
    long long want = ((long long)waves * sms * 2048 + columns - 1) / std::max(1LL, columns);
    if (ln.collapse[2]) want = 1;
    want = std::max(1LL, std::min<long long>(want, ncz));
    *kchunk = (int)((ncz + want - 1) / want);
    *nchunks = (ncz + *kchunk - 1) / *kchunk;
}

// Grid of the finest-level FP64 outer kernels (k_outer_residual, k_update_residual): the
// z extent is cut to about eight waves of three resident CTAs per SM, so every thread
// walks many planes before the block's FP64 norm reduction (one reduction per four cells
// cost more than one FP64 operation per cell on a pipe that bounds these kernels).
dim3 grid_outer(const LevelK<double> &L, const Launch &ln)
{
    dim3 g = grid3m((L.nx + kOuterVec - 1) / kOuterVec, L.ny, L.nz, ln);
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                      cudaSuccess)
            sms = 148;
    }
    const long long gxy = (long long)g.x * g.y, want = 8LL * 3 * sms;
    g.z = (unsigned)std::max(1LL, std::min<long long>(g.z, (want + gxy - 1) / gxy));
    return g;
}

}  // namespace

#define PMG_TRY_M(expr)                \
    do {                               \
        int _rc = (expr);              \
        if (_rc != PMG_OK) return _rc; \
    } while (0)

static int mstatus(cudaError_t e, const char *what) { return cuda_status(e, what); }

// FP32 arrays of the mixed V-cycle.  Besides the (0:nx+1,0:ny+1,0:nz+1) cells every array
// carries zero padding that the fused smoother reads without bounds checks: columns
// -3 .. pitch-4 (pitch >= 60*ceil(nx/60)+8 and >= 64*ceil(nx/64)+8, even), rows -1 ..
// ny+1+RB_PAD_ROWS, planes -1 .. nz+1+RB_PAD_PLANES.  The data pointer (cell (0,0,0)) sits
// an odd number of floats past the 256-byte aligned allocation, so the pair of cells
// (i, i+1) with i odd is 8-byte aligned.  Padding is never written.
// Padded FP32 level array: pitch a multiple of 4 floats with room for every smoother
// tile's 64 columns, one row and one plane of padding in front, zero rows and planes
// behind; cell (0,0,0) at base + RBT_DATA_OFF + pitch + plane (an odd float offset, so
// the smoother's cell pairs (odd i, i+1) are 8-byte aligned and its TMA boxes, which
// start at cell i0 - 2 = 60 bx - 1, begin on a 16-byte boundary).
static int alloc_f32(MixedState *m, int nx, int ny, int nz, int *pitch, long long *plane, float **data,
                     float **base, long long *rows_out, long long *planes_out)
{
    int p = std::max(64 * ((nx + 63) / 64) + 8, RB_TX * ((nx + RB_TX - 1) / RB_TX) + 8);
    p = (p + 3) & ~3;
    const long long rows = (long long)ny + 2 + 1 + RB_PAD_ROWS;
    const long long planes = (long long)nz + 2 + 1 + RB_PAD_PLANES;
    const long long pl = (long long)p * rows;
    const size_t n = (size_t)pl * (size_t)planes + 8;
    float *a = nullptr;
    PMG_TRY_M(mstatus(dev_malloc(&a, n * sizeof(float)), "mixed level allocation"));
    PMG_TRY_M(mstatus(cudaMemset(a, 0, n * sizeof(float)), "mixed level init"));
    m->alloc.push_back(a);
    *pitch = p;
    *plane = pl;
    *data = a + RBT_DATA_OFF + p + pl;
    *base = a;
    *rows_out = rows;
    *planes_out = planes;
    return PMG_OK;
}

// The FP32 state is built on the first mixed solve.  A failure part way (an allocation, a
// copy, the autotuner) releases what was built, so the next solve starts the set-up
// again instead of finding a half-built state.
int Ctx::setup_mixed()
{
    if (mixed) return PMG_OK;
    const int rc = build_mixed();
    if (rc != PMG_OK) destroy_mixed();
    return rc;
}

int Ctx::build_mixed()
{
    if (tail_l0 > nl) {
        set_error("mixed precision needs a coarsest level small enough for the single-CTA coarse solver");
        return PMG_EINVAL;
    }
    // The FP32 cycle hands every level of at most kTail32Cells cells (and the levels the
    // aggregation method already assigns to the tail) to the single-CTA tail kernel: such
    // levels are latency bound on the grid kernels (a few microseconds of work behind
    // each launch and each plane step), and one 1024-thread CTA runs them back to back.
    tail32_l0 = tail_l0;
    if (deep_tail)
        while (tail32_l0 > 1 && (long long)lv[tail32_l0 - 1].n[0] * lv[tail32_l0 - 1].n[1] * lv[tail32_l0 - 1].n[2] <=
                                    kTail32Cells)
            --tail32_l0;
    {
        long long cells = 1;
        for (int l = tail32_l0; l <= nl; ++l) cells = std::max(cells, (long long)lv[l].n[0] * lv[l].n[1] * lv[l].n[2]);
        tail32_threads = (int)std::min<long long>(kTail32Threads, std::max<long long>(64, ((cells / 2 + 31) / 32) * 32));
    }
    MixedState *m = new (std::nothrow) MixedState();
    if (!m) return PMG_ENOMEM;
    mixed = m;
    m->inner = mixed_inner > 0 ? mixed_inner : 2;
    m->tables_host.resize(tables_host.size());
    for (size_t q = 0; q < tables_host.size(); ++q) m->tables_host[q] = (float)tables_host[q];
    PMG_TRY_M(mstatus(dev_malloc(&m->tables, m->tables_host.size() * sizeof(float)), "mixed tables"));
    PMG_TRY_M(mstatus(cudaMemcpy(m->tables, m->tables_host.data(), m->tables_host.size() * sizeof(float),
                                 cudaMemcpyHostToDevice),
                      "mixed tables"));
    // FP64 per-axis diagonal sums of the finest level (outer residual)
    {
        const Level &S = lv[0];
        std::vector<double> h((size_t)S.n[1] + 2 + (size_t)S.n[2] + 2, 0.0);
        for (int j = 1; j <= S.n[1]; ++j) h[j] = 1.0 / (S.dm[1][j] * S.dg[1][j]) + 1.0 / (S.dm[1][j] * S.dg[1][j + 1]);
        for (int k = 1; k <= S.n[2]; ++k)
            h[S.n[1] + 2 + k] = 1.0 / (S.dm[2][k] * S.dg[2][k]) + 1.0 / (S.dm[2][k] * S.dg[2][k + 1]);
        PMG_TRY_M(mstatus(dev_malloc(&m->diag64, h.size() * sizeof(double)), "mixed tables"));
        PMG_TRY_M(mstatus(cudaMemcpy(m->diag64, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice),
                          "mixed tables"));
        m->dyy.push_back(m->diag64);
        m->dzz.push_back(m->diag64 + S.n[1] + 2);
    }
    // finest-level coefficients as FP32 (hi, lo) pairs for the residual update
    {
        const LevelK<double> &k0 = K[0];
        const double *src[6] = {k0.cxm, k0.cxp, k0.cym, k0.cyp, k0.czm, k0.czp};
        const int len[6] = {k0.nx + 2, k0.nx + 2, k0.ny + 2, k0.ny + 2, k0.nz + 2, k0.nz + 2};
        std::vector<float2> h;
        size_t off[6];
        for (int a = 0; a < 6; ++a) {
            off[a] = h.size();
            const double *t = tables_host.data() + (src[a] - d_tables);
            for (int q = 0; q < len[a]; ++q) {
                const float hi = (float)t[q];
                h.push_back(make_float2(hi, (float)(t[q] - (double)hi)));
            }
        }
        PMG_TRY_M(mstatus(dev_malloc(&m->split, h.size() * sizeof(float2)), "mixed tables"));
        PMG_TRY_M(mstatus(cudaMemcpy(m->split, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice),
                          "mixed tables"));
        m->sc = SplitCoef{m->split + off[0], m->split + off[1], m->split + off[2],
                          m->split + off[3], m->split + off[4], m->split + off[5]};
    }
    // PEPS_MG_GRAPHS=0: the FP32 V-cycles are launched kernel by kernel, not as graphs
    {
        const char *ge = std::getenv("PEPS_MG_GRAPHS");
        m->use_graphs = !(ge && std::strcmp(ge, "0") == 0);
    }
    // PEPS_MG_OUTER=recompute: the residual after every correction is b - A x in FP64
    {
        const char *oe = std::getenv("PEPS_MG_OUTER");
        m->update_residual = !(oe && std::strcmp(oe, "recompute") == 0);
    }
    // PEPS_MG_STASH=off: every residual update adds its correction to x at once (no stash
    // arrays: two finest-level FP32 arrays less; x moves 16 more bytes per cell per update)
    const char *se = std::getenv("PEPS_MG_STASH");
    const bool use_stash = m->update_residual && !(se && std::strcmp(se, "off") == 0);
    auto F = [&](const double *p) { return (const float *)(m->tables + (p - d_tables)); };
    m->K.resize((size_t)nl + 1);
    m->X.resize((size_t)nl);
    m->e[0].assign((size_t)nl + 1, nullptr);
    m->e[1].assign((size_t)nl + 1, nullptr);
    m->b.assign((size_t)nl + 1, nullptr);
    m->cur.assign((size_t)nl + 1, 0);
    m->fused.assign((size_t)nl + 1, false);
    m->window.assign((size_t)nl + 1, false);
    m->variant.assign((size_t)nl + 1, 0);
    m->kchunk.assign((size_t)nl + 1, 0);
    m->tma.assign((size_t)nl + 1, Rb32Tma());
    m->rows.assign((size_t)nl + 1, 0);
    m->planes.assign((size_t)nl + 1, 0);
    // PEPS_MG_SMOOTHER=window selects the register-window smoother everywhere, =cell the
    // one-launch cell-pair kernel everywhere (otherwise the autotuner picks per level)
    const char *sm_env = std::getenv("PEPS_MG_SMOOTHER");
    const bool use_tma = !(sm_env && std::strcmp(sm_env, "window") == 0);
    const bool force_cell = sm_env && std::strcmp(sm_env, "cell") == 0;
    // PEPS_MG_TRANSFER=cell selects the one-thread-per-cell transfer kernels everywhere
    const char *tr_env = std::getenv("PEPS_MG_TRANSFER");
    m->march = !(tr_env && std::strcmp(tr_env, "cell") == 0);
    for (int l = 0; l <= nl; ++l) {
        const LevelK<double> &k = K[l];
        LevelK<float> &f = m->K[l];
        int pitch = 0;
        long long plane = 0;
        float *base[3];
        long long rows = 0, planes = 0;
        PMG_TRY_M(alloc_f32(m, k.nx, k.ny, k.nz, &pitch, &plane, &m->e[0][l], &base[0], &rows, &planes));
        PMG_TRY_M(alloc_f32(m, k.nx, k.ny, k.nz, &pitch, &plane, &m->e[1][l], &base[1], &rows, &planes));
        PMG_TRY_M(alloc_f32(m, k.nx, k.ny, k.nz, &pitch, &plane, &m->b[l], &base[2], &rows, &planes));
        f.nx = k.nx; f.ny = k.ny; f.nz = k.nz; f.sy = pitch; f.sz = plane;
        f.cxm = F(k.cxm); f.cxp = F(k.cxp); f.sx = F(k.sx);
        f.cym = F(k.cym); f.cyp = F(k.cyp); f.czm = F(k.czm); f.czp = F(k.czp);
        m->fused[l] = l < tail32_l0 && rb32_fused_layout_ok(f, m->e[0][l], m->b[l]) &&
                      rb32_fused_layout_ok(f, m->e[1][l], m->b[l]);
        m->rows[l] = rows;
        m->planes[l] = planes;
        if (m->fused[l] && use_tma) PMG_TRY_M(rb32_tma_setup(&m->tma[l], f, base, rows, planes));
    }
    for (int l = 0; l < nl; ++l) {
        const XferK<double> &x = X[l];
        XferK<float> &y = m->X[l];
        y.ncx = x.ncx; y.ncy = x.ncy; y.ncz = x.ncz;
        y.csy = m->K[l + 1].sy; y.csz = m->K[l + 1].sz;
        y.fsy = m->K[l].sy; y.fsz = m->K[l].sz;
        y.stx = x.stx; y.sty = x.sty; y.stz = x.stz;
        y.wx = F(x.wx); y.wy = F(x.wy); y.wz = F(x.wz);
        y.pxp = F(x.pxp); y.pxn = F(x.pxn); y.pyp = F(x.pyp); y.pyn = F(x.pyn);
        y.pzp = F(x.pzp); y.pzn = F(x.pzn);
    }
    // the stash of the residual update: two more finest-level FP32 arrays
    if (use_stash)
        for (float *&st : m->stash) {
            int pitch = 0;
            long long plane = 0, rows = 0, planes = 0;
            float *base = nullptr;
            PMG_TRY_M(alloc_f32(m, K[0].nx, K[0].ny, K[0].nz, &pitch, &plane, &st, &base, &rows, &planes));
        }
    PMG_TRY_M(mstatus(dev_malloc(&m->d_tail, sizeof(TailDesc<float>)), "mixed tail descriptor"));
    PMG_TRY_M(mstatus(dev_malloc(&m->d_err, sizeof(int)), "mixed error flag"));
    PMG_TRY_M(mstatus(cudaMemset(m->d_err, 0, sizeof(int)), "mixed error flag"));
    for (int l = 0; l < tail32_l0; ++l)
        if (m->fused[l] && force_cell) {
            m->variant[l] = kCellVariant;
        } else if (m->fused[l] && autotune) {
            PMG_TRY_M(tune_smoother(m->K[l], launch[l], m->e[0][l], m->e[1][l], m->b[l], stream, &m->variant[l],
                                    &m->kchunk[l], &m->tma[l], m->d_err, use_tma));
            if (m->variant[l] & kTuneWindow) {
                m->variant[l] &= ~kTuneWindow;
                m->window[l] = true;   // the register-window kernel is faster on this level
            }
        }
    PMG_TRY_M(check_pipeline());
    return PMG_OK;
}

int Ctx::upload_tail32(int maxit, double omega, double tol)
{
    MixedState *m = mixed;
    TailDesc<float> &D = m->tail_host;
    std::memset(&D, 0, sizeof(D));
    D.l0 = tail32_l0;
    D.nl = nl;
    D.maxit = maxit;
    D.coarse_solver = coarse_solver;
    D.coarse_maxit = 1000;
    D.omega = (float)omega;
    D.omw = (float)(1.0 - omega);
    D.tol = tol;
    D.iters_out = d_iscal + 2;
    for (int l = 0; l <= nl; ++l) {
        D.L[l] = m->K[l];
        if (l < nl) D.X[l] = m->X[l];
        D.x[l] = m->e[0][l];   // the tail works in place on buffer 0
        D.b[l] = m->b[l];
        D.r[l] = nullptr;
    }
    fill_coarse64(D.C64, D.cx64, D.cb64, D.cp64, D.cap64, D.crr64, D.omega64, D.omw64, omega);
    D.abort = abort_dev;
    // x and b of the tail levels in shared memory when they fit (not for batch members,
    // whose tails share one launch)
    D.sm_floats = 0;
    if (deep_tail) {
        long long fl = 0;
        for (int l = tail32_l0; l <= nl; ++l) {
            const long long tot = (long long)(lv[l].n[0] + 2) * (lv[l].n[1] + 2) * (lv[l].n[2] + 2);
            fl += 2 * ((tot + 3) & ~3LL);
        }
        if (fl * (long long)sizeof(float) <= kTail32SmemBytes) D.sm_floats = (int)fl;
    }
    tail32_smem = D.sm_floats * (int)sizeof(float);
    if (tail32_smem > 0)
        PMG_TRY_M(mstatus(cudaFuncSetAttribute(k_tail32, cudaFuncAttributeMaxDynamicSharedMemorySize, tail32_smem),
                          "tail shared memory"));
    return mstatus(cudaMemcpyAsync(m->d_tail, &D, sizeof(D), cudaMemcpyHostToDevice, stream), "tail upload");
}

// One FP32 V-cycle on A e = b[0] (e = e[0]); zero_start: e[0] enters as 0.
int Ctx::vcycle32(int maxit, double omega, bool zero_start)
{
    NvtxRange cycle_range("fp32 V-cycle");
    MixedState *m = mixed;
    const float om = (float)omega, omw = (float)(1.0 - omega);
    const dim3 bl(kBX, kBY, 1);
    const double N = (double)m->K[0].nx * m->K[0].ny * m->K[0].nz;
    long long nlaunch = 0;
    auto sweeps = [&](int l, bool zs) -> int {
        const LevelK<float> &L = m->K[l];
        const int pi = l == 0 ? prof.begin(stream) : -1;
        if (m->fused[l]) {
            for (int it = 0; it < maxit; ++it) {
                PMG_TRY_M(rb32_fused(L, launch[l], m->E(l), m->Eother(l), m->b[l], om, omw, zs && it == 0, stream,
                                     m->variant[l], m->kchunk[l], m->window[l] ? nullptr : &m->tma[l], m->cur[l],
                                     m->d_err));
                m->cur[l] = 1 - m->cur[l];
            }
            // 12 B per cell (e_in, b read, e_out written); 8 B for an iteration from e = 0
            prof.end(pi, PC_SMOOTH32, maxit, (12.0 * maxit - (zs ? 4.0 : 0.0)) / std::max(1, maxit) * N, stream);
        } else {
            const dim3 gc = grid3m((L.nx + 1) / 2, L.ny, L.nz, launch[l]), gf = grid3m(L.nx, L.ny, L.nz, launch[l]);
            for (int it = 0; it < maxit; ++it)
                for (int c = 0; c < 2; ++c) {
                    if (zs && it == 0 && c == 0)
                        k_rbgs32<true><<<gf, bl, 0, stream>>>(L, m->E(l), m->b[l], om, omw, c);
                    else
                        k_rbgs32<false><<<gc, bl, 0, stream>>>(L, m->E(l), m->b[l], om, omw, c);
                    ++nlaunch;
                }
            prof.end(pi, PC_SMOOTH32, 2 * maxit, 8.0 * N, stream);
        }
        if (zs && maxit == 0) cudaMemsetAsync(m->E(l), 0, (size_t)(L.sz * (L.nz + 2)) * sizeof(float), stream);
        return PMG_OK;
    };
    PMG_TRY_M(sweeps(0, zero_start));
    {
        const XferK<float> &X0 = m->X[0];
        const int pi = prof.begin(stream);
        PMG_TRY_M(resrestrict32(0));
        prof.end(pi, PC_RESRESTRICT32, 1, 8.5 * N, stream);
        ++nlaunch;
    }
    // the grid levels below the finest: one profiler record for the way down and one for
    // the way up (smoothing 8 + 12 B per cell from e = 0, 12 B per later iteration;
    // residual-restriction and prolongation 8.5 B per fine cell each)
    auto coarse_bytes = [&](bool down) {
        double b = 0.0;
        for (int l = 1; l < tail32_l0; ++l) {
            const double n = (double)m->K[l].nx * m->K[l].ny * m->K[l].nz;
            b += down ? (12.0 * maxit - 4.0 + 8.5) * n : (12.0 * maxit + 8.5) * n;
        }
        return b;
    };
    const int coarse_launches = std::max(0, tail32_l0 - 1) * (maxit + 1);
    int pc = tail32_l0 > 1 ? prof.begin(stream) : -1;
    for (int l = 1; l < tail32_l0; ++l) {
        PMG_TRY_M(sweeps(l, true));
        PMG_TRY_M(resrestrict32(l));
        ++nlaunch;
    }
    if (coarse_launches > 0) prof.end(pc, PC_COARSE32, coarse_launches, coarse_bytes(true) / coarse_launches, stream);
    {
        const int pi = prof.begin(stream);
        k_tail32<<<1, tail32_threads, tail32_smem, stream>>>(m->d_tail);
        prof.end(pi, PC_TAIL32, 1, 0.0, stream);
        ++nlaunch;
    }
    pc = tail32_l0 > 1 ? prof.begin(stream) : -1;
    for (int l = tail32_l0 - 1; l >= 0; --l) {
        if (l == 0 && coarse_launches > 0)
            prof.end(pc, PC_COARSE32, coarse_launches, coarse_bytes(false) / coarse_launches, stream);
        const XferK<float> &Xl = m->X[l];
        const int pi = l == 0 ? prof.begin(stream) : -1;
        {
            const LevelK<float> &Lf = m->K[l];
            if (m->march && Xl.stx == 2 && Xl.stz == 2) {
                int kchunk = 1, nchunks = 1;
                march_chunks((long long)Xl.ncx * Lf.ny, Xl.ncz, launch[l], &kchunk, &nchunks);
                dim3 g = grid3m(Xl.ncx, Lf.ny, 1, launch[l]);
                g.z = (unsigned)std::min(nchunks, kMaxGridZ);
                k_prolong_march32<<<g, bl, 0, stream>>>(Xl, Lf.ny, kchunk, nchunks, m->E(l + 1), m->E(l));
            } else {
                k_prolong_add32<<<grid3m(Xl.ncx, Lf.ny, Lf.nz, launch[l]), bl, 0, stream>>>(Xl, Lf.ny, Lf.nz,
                                                                                          m->E(l + 1), m->E(l));
            }
        }
        prof.end(pi, PC_PROLONG32, 1, 8.5 * N, stream);
        ++nlaunch;
        PMG_TRY_M(sweeps(l, false));
    }
    count_launches(nlaunch);
    return cuda_status(cudaGetLastError(), "fp32 v-cycle");
}

// b_{l+1} = R (b_l - A_l e_l): the marching kernel where every axis is halved, else one
// thread per coarse cell.
int Ctx::resrestrict32(int l)
{
    MixedState *m = mixed;
    const XferK<float> &X = m->X[l];
    const dim3 bl(kBX, kBY, 1);
    if (m->march && X.stx == 2 && X.sty == 2 && X.stz == 2) {
        int kchunk = 1, nchunks = 1;
        march_chunks((long long)X.ncx * X.ncy, X.ncz, launch[l + 1], &kchunk, &nchunks);
        dim3 g = grid3m(X.ncx, X.ncy, 1, launch[l + 1]);
        g.z = (unsigned)std::min(nchunks, kMaxGridZ);
        k_resrestrict_march32<false><<<g, bl, 0, stream>>>(m->K[l], X, kchunk, nchunks, m->E(l), m->b[l], m->b[l + 1],
                                                           1.f, nullptr);
    } else {
        k_resrestrict32<<<grid3m(X.ncx, X.ncy, X.ncz, launch[l + 1]), bl, 0, stream>>>(m->K[l], X, m->E(l), m->b[l],
                                                                                       m->b[l + 1]);
    }
    return PMG_OK;
}

int Ctx::outer_residual(double *sol, double *rsd, const double *rhs, int slot, double res0)
{
    NvtxRange nvtx_range("FP64 outer residual");
    const LevelK<double> &L = K[0];
    const dim3 g = grid_outer(L, launch[0]), bl(kBX, kBY, 1);
    int *nonzero = d_iscal + 3;
    if (slot == 0) {
        // the first residual of a solve: is the initial guess exactly zero?
        // (skipped when a staged solve's host scan already found it zero)
        PMG_TRY_M(mstatus(cudaMemsetAsync(nonzero, 0, sizeof(int), stream), "zero test"));
        const long long n = (long long)lv[0].total;
        if (!x0_known_zero) {
            k_nonzero_f64<<<(unsigned)std::max<long long>(1, std::min<long long>((n + 1023) / 1024, 4096)), 256, 0,
                            stream>>>(sol, n, nonzero);
            count_launches(1);
        }
    }
    // a recomputed residual (the initial one known) sums its norm with the FP32 pair, scaled
    // like the residual update's norm
    const int ex = norm_exponent(res0);
    const bool cn = slot != 0 && res0 > 0.0 && std::isfinite(res0);
    const float nscale = std::ldexp(1.0f, -ex);
    const int pi = prof.begin(stream);
    if (slot == 0)
        k_outer_residual<true, false><<<g, bl, 0, stream>>>(L, mixed->dyy[0], mixed->dzz[0], sol, rhs, rsd,
                                                            mixed->b[0], mixed->K[0].sy, mixed->K[0].sz, d_partials,
                                                            nonzero, 1.f, 0);
    else if (cn)
        k_outer_residual<false, true><<<g, bl, 0, stream>>>(L, mixed->dyy[0], mixed->dzz[0], sol, rhs, rsd,
                                                            mixed->b[0], mixed->K[0].sy, mixed->K[0].sz, d_partials,
                                                            nonzero, nscale, -ex);
    else
        k_outer_residual<false, false><<<g, bl, 0, stream>>>(L, mixed->dyy[0], mixed->dzz[0], sol, rhs, rsd,
                                                             mixed->b[0], mixed->K[0].sy, mixed->K[0].sz, d_partials,
                                                             nonzero, 1.f, 0);
    prof.end(pi, PC_OUTER_RES, 1, 28.0 * (double)L.nx * L.ny * L.nz, stream);
    count_launches(1);
    PMG_TRY_M(cuda_status(cudaGetLastError(), "outer residual"));
    return f64_reduce(d_partials, (int)(g.x * g.y * g.z), d_scal + slot, stream);
}

// The inner FP32 V-cycles of one correction.  A V-cycle toggles every level's buffer an
// even number of times, so a captured cycle stays valid for every later replay; the two
// graphs (the first cycle of a correction, from e = 0, and the later ones) are captured at
// the first solve and again when maxit or omega change.  Back-to-back launches of the small
// levels' kernels cost about 4 us each on the device, about 1 us inside a graph.  With the
// event profiler on, the kernels are launched one by one.
// The inner residual's squared norm at the finest level into *out (synchronises).
int Ctx::inner_norm(double *out, double res0)
{
    MixedState *m = mixed;
    const dim3 bl(kBX, kBY, 1);
    int np = 0;
    const XferK<float> &X = m->X[0];
    if (nl >= 1 && tail32_l0 > 0 && m->march && X.stx == 2 && X.sty == 2 && X.stz == 2) {
        // the marching residual-restriction of the finest level with the norm added (its
        // restriction into level 1 is overwritten by the next cycle, if there is one)
        int kchunk = 1, nchunks = 1;
        march_chunks((long long)X.ncx * X.ncy, X.ncz, launch[1], &kchunk, &nchunks);
        dim3 g = grid3m(X.ncx, X.ncy, 1, launch[1]);
        g.z = (unsigned)std::min(nchunks, kMaxGridZ);
        np = (int)(g.x * g.y * g.z);
        if ((size_t)np > npart_cap) np = 0;
        if (np) {
            // nscale: a power of two near 1 / (1e-10 rms r0), so the squares of residuals near
            // the tolerance stay well inside FP32's range
            const double rms = std::sqrt(res0 / ((double)K[0].nx * K[0].ny * K[0].nz)) * 1e-10;
            const int ex = rms > 0.0 && std::isfinite(rms) ? std::max(-100, std::min(100, (int)std::floor(std::log2(rms)))) : 0;
            k_resrestrict_march32<true><<<g, bl, 0, stream>>>(m->K[0], X, kchunk, nchunks, m->E(0), m->b[0],
                                                              m->b[1], std::ldexp(1.f, -ex), d_partials);
        }
    }
    if (!np) {
        const dim3 g = grid_outer(K[0], launch[0]);
        k_inner_norm<1><<<g, bl, 0, stream>>>(m->K[0], m->E(0), m->b[0], d_partials);
        np = (int)(g.x * g.y * g.z);
    }
    count_launches(1);
    PMG_TRY_M(cuda_status(cudaGetLastError(), "inner residual norm"));
    PMG_TRY_M(f64_reduce(d_partials, np, d_scal + 2, stream));
    double h[3];
    PMG_TRY_M(fetch_scalars(h, 3));
    *out = h[2];
    return PMG_OK;
}

// The FP32 V-cycles of one correction: m->inner cycles, or (check_after > 0) fewer when,
// after check_after of them, the inner residual's squared norm is below thresh2 (the
// outer residual the correction leaves is that residual to about 1e-14 of the initial
// one, so the FP64 recompute that follows confirms the stop).  *ran = cycles run.
int Ctx::run_vcycles(int maxit, double omega, int check_after, double thresh2, int *ran, double res0)
{
    NvtxRange nvtx_range("FP32 V-cycles of a correction");
    MixedState *m = mixed;
    if (ran) *ran = m->inner;
    auto stop_here = [&](int done, bool *stop) -> int {
        *stop = false;
        if (check_after <= 0 || done != check_after || done >= m->inner) return PMG_OK;
        double v = 0.0;
        PMG_TRY_M(inner_norm(&v, res0));
        if (std::isfinite(v) && v < thresh2) {
            *stop = true;
            if (ran) *ran = done;
        }
        return PMG_OK;
    };
    if (prof.on || !m->use_graphs) {
        for (int q = 0; q < m->inner; ++q) {
            PMG_TRY_M(vcycle32(maxit, omega, q == 0));
            bool stop = false;
            PMG_TRY_M(stop_here(q + 1, &stop));
            if (stop) break;
        }
        return PMG_OK;
    }
    if (!m->vgraph[0] || m->vgraph_maxit != maxit || m->vgraph_omega != omega) {
        if (!m->cap_stream)
            PMG_TRY_M(mstatus(cudaStreamCreateWithFlags(&m->cap_stream, cudaStreamNonBlocking), "capture stream"));
        for (int f = 0; f < 2; ++f) {
            if (m->vgraph[f]) {
                cudaGraphExecDestroy(m->vgraph[f]);
                m->vgraph[f] = nullptr;
            }
            // capture on the private stream (the context's stream may be the legacy one,
            // which cannot be captured); nothing runs while capturing
            const long long c0 = launches_total();
            cudaStream_t own = stream;
            stream = m->cap_stream;
            cudaError_t ce = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
            int rc = ce == cudaSuccess ? vcycle32(maxit, omega, f == 0) : PMG_OK;
            cudaGraph_t g = nullptr;
            if (ce == cudaSuccess) ce = cudaStreamEndCapture(stream, &g);
            stream = own;
            const long long captured = launches_total() - c0;
            count_launches(-captured);   // recorded, not launched
            if (rc == PMG_OK) rc = mstatus(ce, "V-cycle graph capture");
            if (rc == PMG_OK) rc = mstatus(cudaGraphInstantiate(&m->vgraph[f], g, 0), "V-cycle graph instantiate");
            if (g) cudaGraphDestroy(g);
            if (rc != PMG_OK) {
                cudaGetLastError();
                m->vgraph[f] = nullptr;
                return rc;
            }
            m->vgraph_launches[f] = captured;
        }
        m->vgraph_maxit = maxit;
        m->vgraph_omega = omega;
    }
    for (int q = 0; q < m->inner; ++q) {
        const int f = q == 0 ? 0 : 1;
        PMG_TRY_M(mstatus(cudaGraphLaunch(m->vgraph[f], stream), "V-cycle graph launch"));
        count_launches(m->vgraph_launches[f]);
        bool stop = false;
        PMG_TRY_M(stop_here(q + 1, &stop));
        if (stop) break;
    }
    return PMG_OK;
}

// r -= A e with its norm into d_scal[slot] (after a correction); e goes to a free stash
// array (x untouched), or, with both taken, x gets the two stashed corrections and e here;
// res0 = the initial residual's squared norm (sets the norm's FP32 scale).
int Ctx::update_residual(double *sol, double *rsd, int slot, double res0)
{
    NvtxRange nvtx_range("correction and residual update");
    const LevelK<double> &L = K[0];
    constexpr int UV = 2;   // cells per thread (64 registers: more resident warps)
    dim3 g = grid_outer(L, launch[0]);
    if (!launch[0].collapse[0]) g.x = (unsigned)std::max(1, (L.nx + UV * kBX - 1) / (UV * kBX));
    const dim3 bl(kBX, kBY, 1);
    const int ex = norm_exponent(res0);
    const float nscale = std::ldexp(1.0f, -ex);
    // eight waves of chunks: shorter columns at four CTAs per SM measured 6% faster
    int kchunk = 1, nchunks = 1;
    march_chunks((long long)L.nx * L.ny, L.nz, launch[0], &kchunk, &nchunks, 8);
    dim3 gm = grid3m(L.nx, L.ny, 1, launch[0]);
    gm.z = (unsigned)std::min(nchunks, kMaxGridZ);
    const bool march = (size_t)gm.x * gm.y * gm.z <= npart_cap;
    MixedState *m = mixed;
    const int sy32 = m->K[0].sy;
    const long long sz32 = m->K[0].sz;
    // x: the correction goes to a free stash array (x untouched), or, with both taken, all
    // three are added to x here; the plane-grid kernel adds to x directly (after the stash)
    if (!march) PMG_TRY_M(flush_stash(sol));
    const int xm = !march ? XM_ADD : !m->stash[0] ? XM_ADD : m->nstash < 2 ? XM_STASH : XM_FOLD;
    const double bytes = xm == XM_STASH ? 28.0 : xm == XM_FOLD ? 48.0 : 40.0;
    const int pi = prof.begin(stream);
    if (!march)
        k_update_residual<UV><<<g, bl, 0, stream>>>(L, m->sc, sol, m->E(0), rsd, m->b[0], sy32, sz32, nscale,
                                                d_partials);
    else if (xm == XM_STASH)
        k_update_residual_march<XM_STASH><<<gm, bl, 0, stream>>>(L, m->sc, sol, m->E(0), rsd, m->b[0], sy32, sz32,
                                                                 nscale, kchunk, nchunks, d_partials,
                                                                 m->stash[m->nstash], nullptr, nullptr);
    else if (xm == XM_FOLD)
        k_update_residual_march<XM_FOLD><<<gm, bl, 0, stream>>>(L, m->sc, sol, m->E(0), rsd, m->b[0], sy32, sz32,
                                                                nscale, kchunk, nchunks, d_partials, nullptr,
                                                                m->stash[0], m->stash[1]);
    else
        k_update_residual_march<XM_ADD><<<gm, bl, 0, stream>>>(L, m->sc, sol, m->E(0), rsd, m->b[0], sy32, sz32,
                                                               nscale, kchunk, nchunks, d_partials, nullptr,
                                                               nullptr, nullptr);
    if (xm == XM_STASH) ++m->nstash;
    if (xm == XM_FOLD) m->nstash = 0;
    prof.end(pi, PC_UPDATE_RES, 1, bytes * (double)L.nx * L.ny * L.nz, stream);
    count_launches(1);
    PMG_TRY_M(cuda_status(cudaGetLastError(), "residual update"));
    const dim3 gu = march ? gm : g;
    return f64_reduce(d_partials, (int)(gu.x * gu.y * gu.z), d_scal + slot, stream);
}

// The power of two 2^ex nearest below the finest level's RMS initial residual
// sqrt(res0 / N): the scaled FP32 norms sum r 2^-ex (0 when res0 is not a positive number).
int Ctx::norm_exponent(double res0) const
{
    const LevelK<double> &L = K[0];
    const double rms0 = std::sqrt(res0 / ((double)L.nx * L.ny * L.nz));
    return rms0 > 0.0 && std::isfinite(rms0) ? std::max(-100, std::min(100, (int)std::floor(std::log2(rms0)))) : 0;
}

// x += e (with the stashed corrections before it) followed by the FP64 residual b - A x
// (slot 1).
int Ctx::correct_and_recompute(double *sol, double *rsd, const double *rhs, double res0)
{
    NvtxRange nvtx_range("correction and FP64 residual");
    PMG_TRY_M(before_x_change());
    PMG_TRY_M(add_corrections(sol, true));
    PMG_TRY_M(early_copy_sol(sol));
    return outer_residual(sol, rsd, rhs, 1, res0);
}

// x = ((x + s0) + s1) + e with the stashed corrections (none, one or two) and, with
// with_e, the current one; the stash is empty afterwards.
int Ctx::add_corrections(double *sol, bool with_e)
{
    MixedState *m = mixed;
    const int ns = m->nstash;
    if (ns == 0 && !with_e) return PMG_OK;
    const LevelK<double> &L = K[0];
    const dim3 g = grid_outer(L, launch[0]), bl(kBX, kBY, 1);
    const float *e = m->E(0), *s0 = m->stash[0], *s1 = m->stash[1];
    const int sy32 = m->K[0].sy;
    const long long sz32 = m->K[0].sz;
    const int pi = prof.begin(stream);
    if (with_e) {
        if (ns == 0) k_add_correction<0, true><<<g, bl, 0, stream>>>(L, sol, e, s0, s1, sy32, sz32);
        else if (ns == 1) k_add_correction<1, true><<<g, bl, 0, stream>>>(L, sol, e, s0, s1, sy32, sz32);
        else k_add_correction<2, true><<<g, bl, 0, stream>>>(L, sol, e, s0, s1, sy32, sz32);
    } else {
        if (ns == 1) k_add_correction<1, false><<<g, bl, 0, stream>>>(L, sol, e, s0, s1, sy32, sz32);
        else k_add_correction<2, false><<<g, bl, 0, stream>>>(L, sol, e, s0, s1, sy32, sz32);
    }
    prof.end(pi, PC_ADDCORR, 1, (16.0 + 4.0 * (ns + (with_e ? 1 : 0))) * (double)L.nx * L.ny * L.nz, stream);
    count_launches(1);
    m->nstash = 0;
    return cuda_status(cudaGetLastError(), "correction");
}

// Adds the stashed corrections to x (the point where x has to hold every correction: the
// FP64 residual b - A x, or the end of the solve).
int Ctx::flush_stash(double *sol)
{
    if (!mixed || mixed->nstash == 0) return PMG_OK;
    PMG_TRY_M(before_x_change());
    return add_corrections(sol, false);
}

// Defect correction.  After a correction the residual is normally updated (r -= A e in
// one pass, no FP64 stencil, e stashed for x); the FP64 residual b - A x is recomputed where the
// solve may end: when the updated residual passes the test (the recomputed one decides,
// and it is the residual returned), when the previous contraction predicts that this
// correction passes it by a margin of 10, and after the last allowed correction.
int Ctx::solve_mixed(double *sol, double *rsd, const double *rhs, int maxit, double tol, double omega,
                     pmg_report_t *rep)
{
    PMG_TRY_M(setup_mixed());
    MixedState *m = mixed;
    m->nstash = 0;
    const Level &S = lv[0];
    // the residual's ghost cells are zero (src/multigrid.f90:1795); the outer residual
    // writes every interior cell
    PMG_TRY_M(zero_ghosts_f64(rsd, S.n[0], S.n[1], S.n[2], stream));
    PMG_TRY_M(outer_residual(sol, rsd, rhs, 0));
    double h[2];
    PMG_TRY_M(fetch_scalars(h, 1));
    const double res0tol = h[0];
    if (res0tol == 0.0) {
        // an exactly zero initial residual: sol is returned unchanged with rsd = b - A x
        // and no cycles (the FP64 path does the same; see Ctx::solve_f64)
        if (rep) {
            rep->cycles = 0;
            rep->converged = 1;
            rep->res0 = 0.0;
            rep->final_ratio = 0.0;
            rep->inner_cycles = 0;
        }
        return check_pipeline();
    }
    PMG_TRY_M(upload_tail32(maxit, omega, tol));
    int cycles = 0, converged = 0, inner_total = 0;
    double ratio = 0.0, prev_ratio = 1.0, contraction = 1.0;
    for (int cyc = 1; cyc <= n_vcycles; ++cyc) {
        if (aborted()) {
            if (rep) {
                rep->cycles = cycles;
                rep->converged = 0;
                rep->res0 = std::sqrt(res0tol);
                rep->final_ratio = ratio;
                rep->inner_cycles = inner_total;
            }
            PMG_TRY_M(flush_stash(sol));
            return abort_status();
        }
        const bool recompute = !m->update_residual || cyc == n_vcycles || prev_ratio * contraction < 0.1 * tol;
        // A correction predicted to end the solve stops its V-cycles once the residual it
        // leaves is below 0.95 tol: the cycles it needs at the last correction's rate per
        // cycle, checked by one inner residual norm (the reference stops as soon as a cycle
        // meets the tolerance, src/multigrid.f90:1973).
        int check_after = 0;
        double thresh2 = 0.0;
        if (recompute && cyc > 1 && m->inner > 1 && contraction > 0.0 && contraction < 1.0 && prev_ratio > 0.0) {
            const double per_cycle = std::pow(contraction, 1.0 / m->inner);
            const double need = std::log(0.95 * tol / prev_ratio) / std::log(per_cycle);
            if (std::isfinite(need) && need < m->inner - 0.5) {
                check_after = std::max(1, (int)std::ceil(need));
                thresh2 = 0.95 * 0.95 * tol * tol * res0tol;
            }
        }
        int ran = m->inner;
        PMG_TRY_M(run_vcycles(maxit, omega, check_after, thresh2, &ran, res0tol));
        inner_total += ran;
        if (recompute) {
            PMG_TRY_M(correct_and_recompute(sol, rsd, rhs, res0tol));
            PMG_TRY_M(fetch_scalars(h, 2));
        } else {
            PMG_TRY_M(before_x_change());
            PMG_TRY_M(update_residual(sol, rsd, 1, res0tol));
            PMG_TRY_M(fetch_scalars(h, 2));
            if (std::isfinite(h[1]) && std::sqrt(h[1] / res0tol) < tol) {
                PMG_TRY_M(flush_stash(sol));
                PMG_TRY_M(early_copy_sol(sol));
                PMG_TRY_M(outer_residual(sol, rsd, rhs, 1, res0tol));
                PMG_TRY_M(fetch_scalars(h, 2));
            }
        }
        const double rsd_val = h[1];
        ratio = std::sqrt(rsd_val / res0tol);
        contraction = ratio / prev_ratio;
        prev_ratio = ratio;
        cycles = cyc;
        if (rep && rep->history) {
            rep->history[3 * (cyc - 1) + 0] = std::sqrt(rsd_val);
            rep->history[3 * (cyc - 1) + 1] = std::sqrt(res0tol);
            rep->history[3 * (cyc - 1) + 2] = ratio;
        }
        if (rep && rep->coarse_iterations) {
            int ci = 0;
            cudaMemcpy(&ci, d_iscal + 2, sizeof(int), cudaMemcpyDeviceToHost);
            rep->coarse_iterations[cyc - 1] = ci;
        }
        if (!std::isfinite(rsd_val)) {
            if (rep) {
                rep->cycles = cycles;
                rep->converged = 0;
                rep->res0 = std::sqrt(res0tol);
                rep->final_ratio = ratio;
                rep->inner_cycles = inner_total;
            }
            PMG_TRY_M(flush_stash(sol));
            set_error("residual norm is not finite");
            return PMG_EDIVERGED;
        }
        if (ratio < tol) {
            converged = 1;
            break;
        }
    }
    // every way out of the loop above has emptied the stash already (the FP64 residual that
    // ends a solve needs x whole); this keeps it so should that change
    PMG_TRY_M(flush_stash(sol));
    if (rep) {
        rep->cycles = cycles;
        rep->converged = converged;
        rep->res0 = std::sqrt(res0tol);
        rep->final_ratio = ratio;
        rep->inner_cycles = inner_total;
    }
    return check_pipeline();
}

int Ctx::selftest_smooth32(int level, int impl, int variant, int kchunk, bool zero_in, double omega,
                           const double *e_in, const double *b, double *e_out)
{
    PMG_TRY_M(setup_mixed());
    MixedState *m = mixed;
    if (!m->fused[level] || (impl == 0 && !m->tma[level].ok)) {
        set_error("the level has no fused smoother of that kind");
        return PMG_EINVAL;
    }
    const LevelK<float> &L = m->K[level];
    const size_t total = (size_t)L.sz * (size_t)m->planes[level] + 8;
    const long long front = RBT_DATA_OFF + L.sy + L.sz;
    const int nx = L.nx, ny = L.ny, nz = L.nz;
    std::vector<float> he(total, 0.f), hb(total, 0.f);
    for (int k = 0; k <= nz + 1; ++k)
        for (int j = 0; j <= ny + 1; ++j)
            for (int i = 0; i <= nx + 1; ++i) {
                const size_t src = (size_t)i + (size_t)(nx + 2) * ((size_t)j + (size_t)(ny + 2) * k);
                const size_t dst = (size_t)(front + i + (long long)L.sy * j + L.sz * k);
                he[dst] = (float)e_in[src];
                hb[dst] = (float)b[src];
            }
    float *be = m->e[0][level] - front, *bo = m->e[1][level] - front, *bb = m->b[level] - front;
    PMG_TRY_M(mstatus(cudaMemcpy(be, he.data(), total * sizeof(float), cudaMemcpyHostToDevice), "self-test upload"));
    PMG_TRY_M(mstatus(cudaMemcpy(bb, hb.data(), total * sizeof(float), cudaMemcpyHostToDevice), "self-test upload"));
    PMG_TRY_M(mstatus(cudaMemset(bo, 0, total * sizeof(float)), "self-test init"));
    const float om = (float)omega, omw = (float)(1.0 - omega);
    PMG_TRY_M(rb32_fused(L, launch[level], m->e[0][level], m->e[1][level], m->b[level], om, omw, zero_in, stream,
                         impl == 2 ? kCellVariant : variant, kchunk, impl == 0 ? &m->tma[level] : nullptr, 0,
                         m->d_err));
    PMG_TRY_M(check_pipeline());
    PMG_TRY_M(mstatus(cudaMemcpy(he.data(), bo, total * sizeof(float), cudaMemcpyDeviceToHost), "self-test read"));
    for (int k = 0; k <= nz + 1; ++k)
        for (int j = 0; j <= ny + 1; ++j)
            for (int i = 0; i <= nx + 1; ++i)
                e_out[(size_t)i + (size_t)(nx + 2) * ((size_t)j + (size_t)(ny + 2) * k)] =
                    (double)he[(size_t)(front + i + (long long)L.sy * j + L.sz * k)];
    m->cur[level] = 0;
    return PMG_OK;
}

// Self-test of the timeout path of the TMA-fed smoother: one launch on `level` in its stall
// mode (no copies issued, waits limited to a few microseconds), so every CTA's first wait
// runs out with nothing in flight; the error flag then turns into PMG_ETIMEOUT exactly as
// in a solve.  The level's FP32 work arrays are cleared afterwards (the stalled launch
// wrote values computed from unfilled stages into the interior of one of them), so the
// context stays usable.
int Ctx::selftest_wait_timeout(int level)
{
    PMG_TRY_M(setup_mixed());
    MixedState *m = mixed;
    if (level < 0 || level > nl || !m->fused[level] || !m->tma[level].ok) {
        set_error("the level has no TMA-fed smoother");
        return PMG_EINVAL;
    }
    const LevelK<float> &L = m->K[level];
    const int rc = rb32_fused(L, launch[level], m->e[0][level], m->e[1][level], m->b[level], 1.f, 0.f, false, stream,
                              0, 0, &m->tma[level], 0, m->d_err, true);
    const int timeout = rc == PMG_OK ? check_pipeline() : rc;
    const std::string msg = timeout == PMG_ETIMEOUT ? std::string("fused smoother: a wait for a TMA copy timed out")
                                                    : std::string();
    const size_t total = (size_t)L.sz * (size_t)m->planes[level] + 8;
    const long long front = RBT_DATA_OFF + L.sy + L.sz;
    for (int q = 0; q < 2; ++q)
        PMG_TRY_M(mstatus(cudaMemsetAsync(m->e[q][level] - front, 0, total * sizeof(float), stream), "self-test reset"));
    PMG_TRY_M(mstatus(cudaStreamSynchronize(stream), "self-test reset"));
    m->cur[level] = 0;
    if (!msg.empty()) set_error(msg);
    return timeout;
}

// The TMA-fed smoother sets the error flag when one of its bounded waits for a copied
// plane gave up (its results are then incomplete).
int Ctx::check_pipeline()
{
    int e = 0;
    PMG_TRY_M(mstatus(cudaMemcpyAsync(&e, mixed->d_err, sizeof(int), cudaMemcpyDeviceToHost, stream), "error flag"));
    PMG_TRY_M(mstatus(cudaStreamSynchronize(stream), "error flag"));
    if (e) {
        cudaMemsetAsync(mixed->d_err, 0, sizeof(int), stream);
        set_error("fused smoother: a wait for a TMA copy timed out");
        return PMG_ETIMEOUT;
    }
    return PMG_OK;
}

int convert_selftest(const double *in64, float *out32, const float *in32, double *out64, int n, cudaStream_t s)
{
    k_convert_test<<<std::max(1, std::min((n + 255) / 256, 4096)), 256, 0, s>>>(in64, out32, in32, out64, n);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "conversion self-test");
}

int batch_tail32(const TailDesc<float> *const *descs, int n, const int *done, int threads, cudaStream_t s)
{
    k_batch_tail32<<<n, threads, 0, s>>>(descs, done);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "batch coarse tails");
}

void Ctx::destroy_mixed()
{
    delete mixed;
    mixed = nullptr;
}

}  // namespace pmg
