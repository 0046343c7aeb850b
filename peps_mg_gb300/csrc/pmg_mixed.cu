// pmg_mixed.cu -- mixed precision: FP32 V-cycles inside FP64 defect correction.
//
//   r   = b - A x                  (FP64, with the FP64 norm used for convergence)
//   A e = r                        (FP32 V-cycles, e starting at 0, homogeneous ghosts)
//   x   = x + e                    (FP64)
//
// repeated until sqrt(|r|^2 / |r0|^2) < tolerance, the reference's convergence test
// (src/multigrid.f90:1970-1973).  The FP32 V-cycle follows the operation sequence of
// the reference cycle (src/multigrid.f90:1931-1967) with the same smoother, transfer
// operators and coarsest-level solver, but in FP32 arithmetic with FMA contraction and
// approximate reciprocals; the coarsest-level solver's dot products and convergence
// test stay in FP64.  The finest FP32 residual is fused with the restriction.
//
// This translation unit is compiled with --fmad=true.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pmg_ctx.h"
#include "pmg_tail64.cuh"
#include "pmg_smooth32.cuh"

namespace pmg {

namespace {

constexpr int kBX = 32, kBY = 8;
constexpr int kTail32Threads = 1024;
constexpr int kMaxGridZ = 65535;

__device__ __forceinline__ int tid2() { return threadIdx.x + blockDim.x * threadIdx.y; }
__device__ __forceinline__ int blin() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }

// ---------------------------------------------------------------------------------
// FP32 per-cell arithmetic
// ---------------------------------------------------------------------------------
__device__ __forceinline__ float diag32(const LevelK<float> &L, int i, int j, int k)
{
    return -((L.sx[i] + (L.cym[j] + L.cyp[j])) + (L.czm[k] + L.czp[k]));
}

__device__ __forceinline__ float nbsum32(const LevelK<float> &L, const float *x, long long p, int i, int j, int k)
{
    float t = L.cxm[i] * x[p - 1];
    t = fmaf(L.cxp[i], x[p + 1], t);
    t = fmaf(L.cym[j], x[p - L.sy], t);
    t = fmaf(L.cyp[j], x[p + L.sy], t);
    t = fmaf(L.czm[k], x[p - L.sz], t);
    t = fmaf(L.czp[k], x[p + L.sz], t);
    return t;
}

__device__ __forceinline__ float rbgs32(const LevelK<float> &L, const float *x, const float *b, int i, int j, int k,
                                        float omega, float omw)
{
    const long long p = lin(i, j, k, L.sy, L.sz);
    const float t = nbsum32(L, x, p, i, j, k);
    const float c0 = diag32(L, i, j, k);
    return fmaf(omw, x[p], __fdividef(omega * (b[p] - t), c0));
}

__device__ __forceinline__ float resid32(const LevelK<float> &L, const float *x, const float *b, int i, int j, int k)
{
    const long long p = lin(i, j, k, L.sy, L.sz);
    return b[p] - fmaf(diag32(L, i, j, k), x[p], nbsum32(L, x, p, i, j, k));
}

// Fused residual + restriction: b_c(i,j,k) = R (b_f - A_f e_f) without storing the
// fine residual (src/multigrid.f90:1932-1933 and :1939-1940); the eight children in the
// reference's term order (src/multigrid.f90:1474-1491), accumulated one at a time.
__device__ __forceinline__ float resrestrict_cell32(const LevelK<float> &F, const XferK<float> &X, const float *e,
                                                    const float *b, int i, int j, int k)
{
    const int ip = i * X.stx, iz = ip - (X.stx - 1);
    const int jp = j * X.sty, jz = jp - (X.sty - 1);
    const int kp = k * X.stz, kz = kp - (X.stz - 1);
    const float xz = X.wx[iz], xp = X.wx[ip], yz = X.wy[jz], yp = X.wy[jp], zz = X.wz[kz], zp = X.wz[kp];
    float vol = 0.f, s = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int fi = (c & 1) ? iz : ip, fj = (c & 2) ? jz : jp, fk = (c & 4) ? kz : kp;
        const float wv = ((c & 1) ? xp : xz) * ((c & 2) ? yp : yz) * ((c & 4) ? zp : zz);
        vol += wv;
        s = fmaf(wv, resid32(F, e, b, fi, fj, fk), s);
    }
    return __fdividef(s, vol);
}

__device__ __forceinline__ float prolong_child32(float ax, float bx, float ay, float by, float az, float bz,
                                                 float v000, float v100, float v010, float v001, float v110,
                                                 float v101, float v011, float v111)
{
    const float axy = ax * ay, bxy = bx * ay, axby = ax * by, bxby = bx * by;
    float t = axy * az * v000;
    t = fmaf(bxy * az, v100, t);
    t = fmaf(axby * az, v010, t);
    t = fmaf(axy * bz, v001, t);
    t = fmaf(bxby * az, v110, t);
    t = fmaf(bxy * bz, v101, t);
    t = fmaf(axby * bz, v011, t);
    t = fmaf(bxby * bz, v111, t);
    return __fdividef(t, (ax + bx) * (ay + by) * (az + bz));
}

// e_f += P e_c for the children of one coarse cell (src/multigrid.f90:1652-1758 and
// the correction x = x + r of :1958).
__device__ __forceinline__ void prolong_add_cell32(const XferK<float> &X, const float *vc, float *vf, int i, int j,
                                                   int k)
{
    const int ox = X.stx - 1, oy = X.sty - 1, oz = X.stz - 1;
    const int ip = i * X.stx, iz = ip - ox;
    const int jp = j * X.sty, jz = jp - oy;
    const int kp = k * X.stz, kz = kp - oz;
    const int csy = X.csy;
    const long long csz = X.csz;
    auto V = [&](int a, int b, int c) { return vc[lin(a, b, c, csy, csz)]; };
#pragma unroll
    for (int sk = 0; sk < 2; ++sk) {
        if (sk == 0 && oz == 0) continue;
        const float az = sk ? X.pzn[kp] : X.pzp[kz];
        const float bz = sk ? X.pzn[kz] : X.pzp[kp];
        const int kn = sk ? k + oz : k - oz;
        const int kf = sk ? kp : kz;
#pragma unroll
        for (int sj = 0; sj < 2; ++sj) {
            if (sj == 0 && oy == 0) continue;
            const float ay = sj ? X.pyn[jp] : X.pyp[jz];
            const float by = sj ? X.pyn[jz] : X.pyp[jp];
            const int jn = sj ? j + oy : j - oy;
            const int jf = sj ? jp : jz;
#pragma unroll
            for (int si = 0; si < 2; ++si) {
                if (si == 0 && ox == 0) continue;
                const float ax = si ? X.pxn[ip] : X.pxp[iz];
                const float bx = si ? X.pxn[iz] : X.pxp[ip];
                const int in = si ? i + ox : i - ox;
                const int ifn = si ? ip : iz;
                const float v = prolong_child32(ax, bx, ay, by, az, bz, V(i, j, k), V(in, j, k), V(i, jn, k),
                                                V(i, j, kn), V(in, jn, k), V(in, j, kn), V(i, jn, kn),
                                                V(in, jn, kn));
                const long long q = lin(ifn, jf, kf, X.fsy, X.fsz);
                vf[q] += v;
            }
        }
    }
}

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

// Coarse index, neighbour and the two 1-D weights of fine index f along one axis
// (stride 2: odd f is the low child (z_f), even f the high child (p_f); stride 1: the
// high child, src/multigrid.f90:1594-1649).
__device__ __forceinline__ void side_weights(int st, int f, const float *pp, const float *pn, int *c, int *nb,
                                             float *wa, float *wb)
{
    if (st == 2) {
        const int cc = (f + 1) >> 1;
        *c = cc;
        if (f & 1) {
            *nb = cc - 1;
            *wa = pp[f];
            *wb = pp[f + 1];
        } else {
            *nb = cc + 1;
            *wa = pn[f];
            *wb = pn[f - 1];
        }
    } else {
        *c = f;
        *nb = f;
        *wa = pn[f];
        *wb = pn[f];
    }
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

// ---------------------------------------------------------------------------------
// FP64 outer kernels
// ---------------------------------------------------------------------------------
// Round-to-nearest-even double -> float, from the IEEE-754 encodings, on the integer
// pipe (the FP64 pipe is the bottleneck of the outer kernels).  Results that are not
// normal floats (zero, subnormal, overflow, NaN) use the hardware conversion.
__device__ __forceinline__ float f64_to_f32_rn(double v)
{
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;
    if (e < -126 || e > 127) return __double2float_rn(v);
    const unsigned long long m = bits & 0xFFFFFFFFFFFFFull;
    const unsigned hi = (unsigned)(m >> 29);
    const unsigned long long rem = m & 0x1FFFFFFFull;
    unsigned f = ((unsigned)(e + 127) << 23) | hi;
    if (rem > 0x10000000ull || (rem == 0x10000000ull && (hi & 1u))) f += 1u;   // carry may reach the exponent
    f |= (unsigned)(bits >> 32) & 0x80000000u;
    return __uint_as_float(f);
}

// Exact float -> double from the encodings (integer pipe); subnormal, Inf and NaN
// inputs use the hardware conversion.
__device__ __forceinline__ double f32_to_f64(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    if (e == 0u) {
        if ((u & 0x7fffffu) == 0u) return __longlong_as_double((long long)sign);
        return (double)f;
    }
    if (e == 255u) return (double)f;
    const unsigned long long bits = sign | ((unsigned long long)(e + 896u) << 52) |
                                    ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)bits);
}

// r = b - A x in FP64 (FMA form: r = b + d x - sum c x_nb with d = -c0, the diagonal
// from the per-axis sums dxx = cxm+cxp, dyy, dzz), stored both as the FP64 residual and
// as the FP32 right-hand side of the inner system, with the per-block sum of r^2.
// Each thread handles four cells of a row, 32 apart.
constexpr int kOuterVec = 4;
__global__ void __launch_bounds__(kBX *kBY) k_outer_residual(LevelK<double> L, const double *__restrict__ dyy,
                                                             const double *__restrict__ dzz,
                                                             const double *__restrict__ x,
                                                             const double *__restrict__ b, double *__restrict__ r,
                                                             float *__restrict__ r32, int sy32, long long sz32,
                                                             double *partials)
{
    double acc = 0.0;
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z) {
        const double dz = dzz[k];
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y) {
            const double dyz = dyy[j] + dz;
            for (int i0 = blockIdx.x * (blockDim.x * kOuterVec) + threadIdx.x + 1; i0 <= L.nx;
                 i0 += gridDim.x * blockDim.x * kOuterVec) {
#pragma unroll
                for (int u = 0; u < kOuterVec; ++u) {
                    const int i = i0 + u * kBX;
                    if (i > L.nx) break;
                    const long long p = lin(i, j, k, L.sy, L.sz);
                    const double d = L.sx[i] + dyz;
                    double v = fma(d, x[p], b[p]);
                    v = fma(-L.cxm[i], x[p - 1], v);
                    v = fma(-L.cxp[i], x[p + 1], v);
                    v = fma(-L.cym[j], x[p - L.sy], v);
                    v = fma(-L.cyp[j], x[p + L.sy], v);
                    v = fma(-L.czm[k], x[p - L.sz], v);
                    v = fma(-L.czp[k], x[p + L.sz], v);
                    r[p] = v;
                    r32[lin(i, j, k, sy32, sz32)] = f64_to_f32_rn(v);
                    acc = fma(v, v, acc);
                }
            }
        }
    }
    __shared__ double sw[kBX * kBY / 32];
    const double s = block_sum(acc, sw);
    if (tid2() == 0) partials[blin()] = s;
}

// x = x + e (the FP64 correction)
__global__ void __launch_bounds__(kBX *kBY) k_add_correction(LevelK<double> L, double *__restrict__ x,
                                                             const float *__restrict__ e, int sy32, long long sz32)
{
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x) {
                const long long p = lin(i, j, k, L.sy, L.sz);
                x[p] = x[p] + f32_to_f64(e[lin(i, j, k, sy32, sz32)]);
            }
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
template <typename F>
__device__ __forceinline__ void for_cells(int nx, int ny, int nz, F f)
{
    const long long n = (long long)nx * ny * nz;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) {
        const int i = (int)(q % nx) + 1;
        const long long rr = q / nx;
        f(i, (int)(rr % ny) + 1, (int)(rr / ny) + 1);
    }
}

__device__ void t32_sweeps(const LevelK<float> &L, float *x, const float *b, int iters, float omega, float omw,
                           bool zero_start)
{
    const int hx = (L.nx + 1) / 2;
    const long long nq = (long long)hx * L.ny * L.nz;
    for (int it = 0; it < iters; ++it)
        for (int colour = 0; colour < 2; ++colour) {
            if (zero_start && it == 0 && colour == 0) {
                for_cells(L.nx, L.ny, L.nz, [&](int i, int j, int k) {
                    const long long p = lin(i, j, k, L.sy, L.sz);
                    x[p] = ((i + j + k) & 1) ? __fdividef(omega * b[p], diag32(L, i, j, k)) : 0.f;
                });
            } else {
                for (long long q = threadIdx.x; q < nq; q += blockDim.x) {
                    const int t = (int)(q % hx);
                    const long long rr = q / hx;
                    const int j = (int)(rr % L.ny) + 1, k = (int)(rr / L.ny) + 1;
                    const int i = 2 * t + 1 + ((j + k + colour) & 1);
                    if (i <= L.nx) x[lin(i, j, k, L.sy, L.sz)] = rbgs32(L, x, b, i, j, k, omega, omw);
                }
            }
            __syncthreads();
        }
}

__global__ void __launch_bounds__(kTail32Threads) k_tail32(const TailDesc<float> *__restrict__ Dp)
{
    __shared__ double sw[kTail32Threads / 32];
    const TailDesc<float> &D = *Dp;
    const float omega = D.omega, omw = D.omw;
    for (int l = D.l0; l < D.nl; ++l) {
        const LevelK<float> L = D.L[l];
        const XferK<float> X = D.X[l];
        float *x = D.x[l], *bc = D.b[l + 1];
        const float *b = D.b[l];
        t32_sweeps(L, x, b, D.maxit, omega, omw, true);
        for_cells(X.ncx, X.ncy, X.ncz, [&](int i, int j, int k) {
            bc[lin(i, j, k, X.csy, X.csz)] = resrestrict_cell32(L, X, x, b, i, j, k);
        });
        __syncthreads();
    }
    // coarsest level: solved in FP64 (b converted up, x converted down), so its
    // convergence test against the FP64 tolerance is attainable
    {
        const LevelK<float> L = D.L[D.nl];
        const LevelK<double> &C = D.C64;
        float *x = D.x[D.nl];
        const float *b = D.b[D.nl];
        for_cells(L.nx, L.ny, L.nz, [&](int i, int j, int k) {
            D.cb64[lin(i, j, k, C.sy, C.sz)] = (double)b[lin(i, j, k, L.sy, L.sz)];
        });
        __syncthreads();
        const int iters = coarse_solve_f64(C, D.cx64, D.cb64, D.cp64, D.cap64, D.crr64, D.coarse_solver,
                                           D.coarse_maxit, D.tol, D.omega64, D.omw64, sw);
        for_cells(L.nx, L.ny, L.nz, [&](int i, int j, int k) {
            x[lin(i, j, k, L.sy, L.sz)] = (float)D.cx64[lin(i, j, k, C.sy, C.sz)];
        });
        if (threadIdx.x == 0 && D.iters_out) *D.iters_out = iters;
        __syncthreads();
    }
    for (int l = D.nl - 1; l >= D.l0; --l) {
        const LevelK<float> L = D.L[l];
        const XferK<float> X = D.X[l];
        float *x = D.x[l], *xc = D.x[l + 1];
        const float *b = D.b[l];
        for_cells(X.ncx, X.ncy, X.ncz, [&](int i, int j, int k) { prolong_add_cell32(X, xc, x, i, j, k); });
        __syncthreads();
        t32_sweeps(L, x, b, D.maxit, omega, omw, false);
    }
}

dim3 grid3m(int nxt, int ny, int nz, const Launch &ln)
{
    dim3 g;
    g.x = ln.collapse[0] ? 1u : (unsigned)std::max(1, (nxt + kBX - 1) / kBX);
    g.y = ln.collapse[1] ? 1u : (unsigned)std::max(1, (ny + kBY - 1) / kBY);
    g.z = ln.collapse[2] ? 1u : (unsigned)std::max(1, std::min(nz, kMaxGridZ));
    return g;
}

}  // namespace

struct MixedState {
    std::vector<float> tables_host;
    float *tables = nullptr;
    double *diag64 = nullptr;        // per level: dyy (ny+2) and dzz (nz+2) for the outer residual
    std::vector<const double *> dyy, dzz;
    std::vector<LevelK<float>> K;
    std::vector<XferK<float>> X;
    std::vector<float *> alloc;      // raw allocations
    std::vector<float *> e[2], b;    // e[buf][l] (two buffers for out-of-place sweeps), b[l]
    std::vector<int> cur;            // current buffer of e at each level
    std::vector<bool> fused;         // level uses the fused out-of-place smoother
    std::vector<int> variant, kchunk;  // autotuned tile variant and k-chunk of the fused smoother
    TailDesc<float> tail_host;
    TailDesc<float> *d_tail = nullptr;
    int inner = 2;
    ~MixedState()
    {
        cudaFree(tables);
        cudaFree(diag64);
        for (auto p : alloc) cudaFree(p);
        cudaFree(d_tail);
    }
    float *E(int l) const { return e[cur[l]][l]; }
    float *Eother(int l) const { return e[1 - cur[l]][l]; }
};

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
static int alloc_f32(MixedState *m, int nx, int ny, int nz, int *pitch, long long *plane, float **data)
{
    int p = std::max(64 * ((nx + 63) / 64) + 8, RB_TX * ((nx + RB_TX - 1) / RB_TX) + 8);
    p += p & 1;
    const long long rows = (long long)ny + 2 + 1 + RB_PAD_ROWS;
    const long long pl = (long long)p * rows;
    const size_t n = (size_t)pl * (size_t)(nz + 2 + 1 + RB_PAD_PLANES) + 8;
    float *a = nullptr;
    PMG_TRY_M(mstatus(cudaMalloc(&a, n * sizeof(float)), "mixed level allocation"));
    PMG_TRY_M(mstatus(cudaMemset(a, 0, n * sizeof(float)), "mixed level init"));
    m->alloc.push_back(a);
    *pitch = p;
    *plane = pl;
    *data = a + 3 + p + pl;     // skip 3 columns, one row and one plane of padding
    return PMG_OK;
}

int Ctx::setup_mixed()
{
    if (mixed) return PMG_OK;
    if (tail_l0 > nl) {
        set_error("mixed precision needs a coarsest level small enough for the single-CTA coarse solver");
        return PMG_EINVAL;
    }
    MixedState *m = new (std::nothrow) MixedState();
    if (!m) return PMG_ENOMEM;
    mixed = m;
    m->inner = mixed_inner > 0 ? mixed_inner : 2;
    m->tables_host.resize(tables_host.size());
    for (size_t q = 0; q < tables_host.size(); ++q) m->tables_host[q] = (float)tables_host[q];
    PMG_TRY_M(mstatus(cudaMalloc(&m->tables, m->tables_host.size() * sizeof(float)), "mixed tables"));
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
        PMG_TRY_M(mstatus(cudaMalloc(&m->diag64, h.size() * sizeof(double)), "mixed tables"));
        PMG_TRY_M(mstatus(cudaMemcpy(m->diag64, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice),
                          "mixed tables"));
        m->dyy.push_back(m->diag64);
        m->dzz.push_back(m->diag64 + S.n[1] + 2);
    }
    auto F = [&](const double *p) { return (const float *)(m->tables + (p - d_tables)); };
    m->K.resize((size_t)nl + 1);
    m->X.resize((size_t)nl);
    m->e[0].assign((size_t)nl + 1, nullptr);
    m->e[1].assign((size_t)nl + 1, nullptr);
    m->b.assign((size_t)nl + 1, nullptr);
    m->cur.assign((size_t)nl + 1, 0);
    m->fused.assign((size_t)nl + 1, false);
    m->variant.assign((size_t)nl + 1, 0);
    m->kchunk.assign((size_t)nl + 1, 0);
    for (int l = 0; l <= nl; ++l) {
        const LevelK<double> &k = K[l];
        LevelK<float> &f = m->K[l];
        int pitch = 0;
        long long plane = 0;
        PMG_TRY_M(alloc_f32(m, k.nx, k.ny, k.nz, &pitch, &plane, &m->e[0][l]));
        PMG_TRY_M(alloc_f32(m, k.nx, k.ny, k.nz, &pitch, &plane, &m->e[1][l]));
        PMG_TRY_M(alloc_f32(m, k.nx, k.ny, k.nz, &pitch, &plane, &m->b[l]));
        f.nx = k.nx; f.ny = k.ny; f.nz = k.nz; f.sy = pitch; f.sz = plane;
        f.cxm = F(k.cxm); f.cxp = F(k.cxp); f.sx = F(k.sx);
        f.cym = F(k.cym); f.cyp = F(k.cyp); f.czm = F(k.czm); f.czp = F(k.czp);
        m->fused[l] = l < tail_l0 && rb32_fused_layout_ok(f, m->e[0][l], m->b[l]) &&
                      rb32_fused_layout_ok(f, m->e[1][l], m->b[l]);
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
    PMG_TRY_M(mstatus(cudaMalloc(&m->d_tail, sizeof(TailDesc<float>)), "mixed tail descriptor"));
    for (int l = 0; l < tail_l0; ++l)
        if (m->fused[l]) PMG_TRY_M(tune_smoother(m->K[l], launch[l], m->e[0][l], m->e[1][l], m->b[l], stream,
                                                 &m->variant[l], &m->kchunk[l]));
    return PMG_OK;
}

int Ctx::upload_tail32(int maxit, double omega, double tol)
{
    MixedState *m = mixed;
    TailDesc<float> &D = m->tail_host;
    std::memset(&D, 0, sizeof(D));
    D.l0 = tail_l0;
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
    return mstatus(cudaMemcpyAsync(m->d_tail, &D, sizeof(D), cudaMemcpyHostToDevice, stream), "tail upload");
}

// One FP32 V-cycle on A e = b[0] (e = e[0]); zero_start: e[0] enters as 0.
int Ctx::vcycle32(int maxit, double omega, bool zero_start)
{
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
                                     m->variant[l], m->kchunk[l]));
                m->cur[l] = 1 - m->cur[l];
            }
            prof.end(pi, PC_SMOOTH32, maxit, 12.0 * N, stream);
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
        k_resrestrict32<<<grid3m(X0.ncx, X0.ncy, X0.ncz, launch[1]), bl, 0, stream>>>(m->K[0], X0, m->E(0), m->b[0],
                                                                                     m->b[1]);
        prof.end(pi, PC_RESRESTRICT32, 1, 8.5 * N, stream);
        ++nlaunch;
    }
    for (int l = 1; l < tail_l0; ++l) {
        PMG_TRY_M(sweeps(l, true));
        const XferK<float> &Xl = m->X[l];
        k_resrestrict32<<<grid3m(Xl.ncx, Xl.ncy, Xl.ncz, launch[l + 1]), bl, 0, stream>>>(m->K[l], Xl, m->E(l),
                                                                                         m->b[l], m->b[l + 1]);
        ++nlaunch;
    }
    {
        const int pi = prof.begin(stream);
        k_tail32<<<1, tail_threads, 0, stream>>>(m->d_tail);
        prof.end(pi, PC_TAIL32, 1, 0.0, stream);
        ++nlaunch;
    }
    for (int l = tail_l0 - 1; l >= 0; --l) {
        const XferK<float> &Xl = m->X[l];
        const int pi = l == 0 ? prof.begin(stream) : -1;
        {
            const LevelK<float> &Lf = m->K[l];
            k_prolong_add32<<<grid3m(Xl.ncx, Lf.ny, Lf.nz, launch[l]), bl, 0, stream>>>(Xl, Lf.ny, Lf.nz,
                                                                                      m->E(l + 1), m->E(l));
        }
        prof.end(pi, PC_PROLONG32, 1, 8.5 * N, stream);
        ++nlaunch;
        PMG_TRY_M(sweeps(l, false));
    }
    count_launches(nlaunch);
    return cuda_status(cudaGetLastError(), "fp32 v-cycle");
}

int Ctx::outer_residual(double *sol, double *rsd, const double *rhs, int slot)
{
    const LevelK<double> &L = K[0];
    const dim3 g = grid3m((L.nx + kOuterVec - 1) / kOuterVec, L.ny, L.nz, launch[0]), bl(kBX, kBY, 1);
    const int pi = prof.begin(stream);
    k_outer_residual<<<g, bl, 0, stream>>>(L, mixed->dyy[0], mixed->dzz[0], sol, rhs, rsd, mixed->b[0],
                                           mixed->K[0].sy, mixed->K[0].sz, d_partials);
    prof.end(pi, PC_OUTER_RES, 1, 28.0 * (double)L.nx * L.ny * L.nz, stream);
    count_launches(1);
    PMG_TRY_M(cuda_status(cudaGetLastError(), "outer residual"));
    return f64_reduce(d_partials, (int)(g.x * g.y * g.z), d_scal + slot, stream);
}

int Ctx::solve_mixed(double *sol, double *rsd, const double *rhs, int maxit, double tol, double omega,
                     pmg_report_t *rep)
{
    PMG_TRY_M(setup_mixed());
    MixedState *m = mixed;
    const Level &S = lv[0];
    PMG_TRY_M(mstatus(cudaMemsetAsync(rsd, 0, S.total * sizeof(double), stream), "rsd init"));
    PMG_TRY_M(outer_residual(sol, rsd, rhs, 0));
    double h[2];
    PMG_TRY_M(fetch_scalars(h, 1));
    const double res0tol = h[0];
    PMG_TRY_M(upload_tail32(maxit, omega, tol));
    int cycles = 0, converged = 0, inner_total = 0;
    double ratio = 0.0;
    const LevelK<double> &L = K[0];
    const dim3 g = grid3m(L.nx, L.ny, L.nz, launch[0]), bl(kBX, kBY, 1);
    for (int cyc = 1; cyc <= n_vcycles; ++cyc) {
        for (int q = 0; q < m->inner; ++q) PMG_TRY_M(vcycle32(maxit, omega, q == 0));
        inner_total += m->inner;
        const int pi = prof.begin(stream);
        k_add_correction<<<g, bl, 0, stream>>>(L, sol, m->E(0), m->K[0].sy, m->K[0].sz);
        prof.end(pi, PC_ADDCORR, 1, 20.0 * (double)L.nx * L.ny * L.nz, stream);
        count_launches(1);
        PMG_TRY_M(outer_residual(sol, rsd, rhs, 1));
        PMG_TRY_M(fetch_scalars(h, 2));
        const double rsd_val = h[1];
        ratio = std::sqrt(rsd_val / res0tol);
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
            set_error("residual norm is not finite");
            return PMG_EDIVERGED;
        }
        if (ratio < tol) {
            converged = 1;
            break;
        }
    }
    if (rep) {
        rep->cycles = cycles;
        rep->converged = converged;
        rep->res0 = std::sqrt(res0tol);
        rep->final_ratio = ratio;
        rep->inner_cycles = inner_total;
    }
    return PMG_OK;
}

int convert_selftest(const double *in64, float *out32, const float *in32, double *out64, int n, cudaStream_t s)
{
    k_convert_test<<<std::max(1, std::min((n + 255) / 256, 4096)), 256, 0, s>>>(in64, out32, in32, out64, n);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "conversion self-test");
}

void Ctx::destroy_mixed()
{
    delete mixed;
    mixed = nullptr;
}

}  // namespace pmg
