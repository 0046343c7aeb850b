// pmg_cell32.cuh -- per-cell arithmetic of the mixed-precision V-cycle (FP32 smoother,
// residual, transfer operators, the FP64 outer residual and the integer-pipe precision
// conversions) and the body of the FP32 single-CTA coarse tail; shared by the single-
// problem solver (pmg_mixed.cu) and the batched solver (pmg_batch.cu).  Translation
// units including it are compiled with --fmad=true.
#pragma once

#include "pmg_internal.h"
#include "pmg_tail64.cuh"

namespace pmg {
namespace {

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

// e_f += P e_c on the fine x-pair (2 ic - 1, 2 ic) of fine row jf for the coarse planes
// m0 .. m1 of a transfer that halves x and z: the coarse values of planes kc-1, kc, kc+1
// (x-indices ic-1 .. ic+1, rows jc and jn) stay in registers, so each fine pair is read
// and written once with 8-byte accesses and each coarse plane is loaded once; the
// arithmetic per child is that of prolong_add_cell32.
__device__ __forceinline__ void prolong_column_march32(const XferK<float> &X, int jf, int ic, int m0, int m1,
                                                       const float *__restrict__ vc, float *__restrict__ vf)
{
    int jc, jn;
    float ay, by;
    side_weights(X.sty, jf, X.pyp, X.pyn, &jc, &jn, &ay, &by);
    const int iz = 2 * ic - 1, ip = 2 * ic;
    const float lo_a = X.pxp[iz], lo_b = X.pxp[ip], hi_a = X.pxn[ip], hi_b = X.pxn[iz];
    const float *rc = vc + lin(ic, jc, 0, X.csy, X.csz), *rn = vc + lin(ic, jn, 0, X.csy, X.csz);
    // [row jc: x-1, x, x+1, row jn: x-1, x, x+1] of coarse planes m-1 (A), m (B)
    float A[6], B[6], C[6];
    auto load = [&](float (&V)[6], int kc) {
        const long long o = X.csz * kc;
        V[0] = __ldg(rc + o - 1);
        V[1] = __ldg(rc + o);
        V[2] = __ldg(rc + o + 1);
        V[3] = __ldg(rn + o - 1);
        V[4] = __ldg(rn + o);
        V[5] = __ldg(rn + o + 1);
    };
    load(A, m0 - 1);
    load(B, m0);
    float *pf = vf + lin(iz, jf, 0, X.fsy, X.fsz);
    auto fine = [&](int kf) { return reinterpret_cast<float2 *>(pf + X.fsz * kf); };
    // the fine pairs of the next two coarse planes are loaded while this one is computed
    // (each pair is read, updated and written by this thread only)
    float2 F[2] = {*fine(2 * m0 - 1), *fine(2 * m0)};
    float2 N[2] = {F[0], F[1]};
    if (m0 < m1) {
        N[0] = *fine(2 * m0 + 1);
        N[1] = *fine(2 * m0 + 2);
    }
    for (int m = m0; m <= m1; ++m) {
        load(C, m + 1);
        float2 NN[2] = {N[0], N[1]};
        if (m + 1 < m1) {
            NN[0] = *fine(2 * m + 3);
            NN[1] = *fine(2 * m + 4);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            // h = 0: fine plane 2m-1 (neighbour plane m-1); h = 1: 2m (m+1)
            const int kf = 2 * m - 1 + h;
            const float az = h ? X.pzn[kf] : X.pzp[kf];
            const float bz = h ? X.pzn[kf - 1] : X.pzp[kf + 1];
            const float *Z = h ? C : A;
            const float lo = prolong_child32(lo_a, lo_b, ay, by, az, bz, B[1], B[0], B[4], Z[1], B[3],
                                             Z[0], Z[4], Z[3]);
            const float hi = prolong_child32(hi_a, hi_b, ay, by, az, bz, B[1], B[2], B[4], Z[1], B[5],
                                             Z[2], Z[4], Z[5]);
            F[h].x += lo;
            F[h].y += hi;
            *fine(kf) = F[h];
        }
        F[0] = N[0];
        F[1] = N[1];
        N[0] = NN[0];
        N[1] = NN[1];
#pragma unroll
        for (int u = 0; u < 6; ++u) {
            A[u] = B[u];
            B[u] = C[u];
        }
    }
}

// Fused residual + restriction on coarse column (ic, jc), coarse planes m0 .. m1, of a
// transfer that halves every axis: each fine plane's 2 x 2 block of e (own pairs, 8-byte
// loads) is held for planes k-1 .. k+1 in registers; x- and y-neighbours and b are loaded
// per plane.  Residuals and the restriction sum are those of resrestrict_cell32 (same
// operations, same order).
// NORM: also adds the squares of the fine residuals, times nscale^2 (a power of two that
// keeps them in FP32's range), to *ss.
template <bool NORM = false>
__device__ __forceinline__ void resrestrict_column_march32(const LevelK<float> &F, const XferK<float> &X, int ic,
                                                           int jc, int m0, int m1, const float *__restrict__ e,
                                                           const float *__restrict__ b, float *__restrict__ bc,
                                                           float nscale = 1.f, float *ss = nullptr)
{
    const int jz = 2 * jc - 1, jp = 2 * jc;
    const int iz = 2 * ic - 1, ip = 2 * ic;
    const float xz = X.wx[iz], xp = X.wx[ip], yz = X.wy[jz], yp = X.wy[jp];
    const float cxm0 = F.cxm[iz], cxp0 = F.cxp[iz], sx0 = F.sx[iz];
    const float cxm1 = F.cxm[ip], cxp1 = F.cxp[ip], sx1 = F.sx[ip];
    const float cym0 = F.cym[jz], cyp0 = F.cyp[jz], dy0 = cym0 + cyp0;
    const float cym1 = F.cym[jp], cyp1 = F.cyp[jp], dy1 = cym1 + cyp1;
    const float *e0 = e + lin(iz, jz, 0, F.sy, F.sz);   // row jz; row jp at + sy
    const float *b0 = b + lin(iz, jz, 0, F.sy, F.sz);
    const long long sz = F.sz;
    const int sy = F.sy;
    auto own = [&](float2 (&V)[2], int k) {
        V[0] = __ldg(reinterpret_cast<const float2 *>(e0 + sz * k));
        V[1] = __ldg(reinterpret_cast<const float2 *>(e0 + sz * k + sy));
    };
    // the x- and y-neighbours and b of the 2 x 2 block on fine plane k
    struct Nb {
        float xl0, xr0, xl1, xr1;
        float2 yd, yu, b0v, b1v;
    };
    auto neighbours = [&](int k, Nb &N) {
        const float *pe = e0 + sz * k;
        N.xl0 = __ldg(pe - 1);
        N.xr0 = __ldg(pe + 2);
        N.xl1 = __ldg(pe + sy - 1);
        N.xr1 = __ldg(pe + sy + 2);
        N.yd = __ldg(reinterpret_cast<const float2 *>(pe - sy));
        N.yu = __ldg(reinterpret_cast<const float2 *>(pe + 2 * sy));
        N.b0v = __ldg(reinterpret_cast<const float2 *>(b0 + sz * k));
        N.b1v = __ldg(reinterpret_cast<const float2 *>(b0 + sz * k + sy));
    };
    // residuals of fine plane k into r[0..3] = (iz,jz), (ip,jz), (iz,jp), (ip,jp)
    auto resid_plane = [&](const float2 (&Em)[2], const float2 (&E0)[2], const float2 (&Ep)[2], int k, const Nb &N,
                           float (&r)[4]) {
        const float czm = F.czm[k], czp = F.czp[k], dz = czm + czp;
        const float xl0 = N.xl0, xr0 = N.xr0, xl1 = N.xl1, xr1 = N.xr1;
        const float2 yd = N.yd, yu = N.yu, b0v = N.b0v, b1v = N.b1v;
        auto cell = [&](float cxm, float cxp, float sx, float cym, float cyp, float dy, float xm, float xp_,
                        float ym, float yp_, float zm, float zp_, float x0, float bb) {
            float t = cxm * xm;
            t = fmaf(cxp, xp_, t);
            t = fmaf(cym, ym, t);
            t = fmaf(cyp, yp_, t);
            t = fmaf(czm, zm, t);
            t = fmaf(czp, zp_, t);
            const float d = -((sx + dy) + dz);
            return bb - fmaf(d, x0, t);
        };
        r[0] = cell(cxm0, cxp0, sx0, cym0, cyp0, dy0, xl0, E0[0].y, yd.x, E0[1].x, Em[0].x, Ep[0].x,
                    E0[0].x, b0v.x);
        r[1] = cell(cxm1, cxp1, sx1, cym0, cyp0, dy0, E0[0].x, xr0, yd.y, E0[1].y, Em[0].y, Ep[0].y,
                    E0[0].y, b0v.y);
        r[2] = cell(cxm0, cxp0, sx0, cym1, cyp1, dy1, xl1, E0[1].y, E0[0].x, yu.x, Em[1].x, Ep[1].x,
                    E0[1].x, b1v.x);
        r[3] = cell(cxm1, cxp1, sx1, cym1, cyp1, dy1, E0[1].x, xr1, E0[0].y, yu.y, Em[1].y, Ep[1].y,
                    E0[1].y, b1v.y);
    };
    // software pipeline: the loads of coarse plane m + 1 are in flight while plane m is
    // computed
    float2 Wm[2], W0[2], Wp[2], Wq[2];
    Nb Nz, Np;
    own(Wm, 2 * m0 - 2);
    own(W0, 2 * m0 - 1);
    own(Wp, 2 * m0);
    own(Wq, 2 * m0 + 1);
    neighbours(2 * m0 - 1, Nz);
    neighbours(2 * m0, Np);
    for (int m = m0; m <= m1; ++m) {
        const int kz = 2 * m - 1, kp = 2 * m;
        float2 Wr[2] = {Wp[0], Wp[1]}, Ws[2] = {Wq[0], Wq[1]};
        Nb Mz = Nz, Mp = Np;
        if (m < m1) {
            own(Wr, kp + 2);
            own(Ws, kp + 3);
            neighbours(kz + 2, Mz);
            neighbours(kp + 2, Mp);
        }
        float rz[4], rp[4];
        resid_plane(Wm, W0, Wp, kz, Nz, rz);
        resid_plane(W0, Wp, Wq, kp, Np, rp);
        if (NORM) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float a = rz[q] * nscale, c = rp[q] * nscale;
                *ss = fmaf(a, a, *ss);
                *ss = fmaf(c, c, *ss);
            }
        }
        const float zz = X.wz[kz], zp = X.wz[kp];
        // children in the order of resrestrict_cell32: c = 0..7 with bit 0 ->
        // x (iz), bit 1 -> y (jz), bit 2 -> z (kz); unset bits take the p child
        float vol = 0.f, s = 0.f;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const float wv = ((c & 1) ? xp : xz) * ((c & 2) ? yp : yz) * ((c & 4) ? zp : zz);
            const int q = ((c & 1) ? 0 : 1) + ((c & 2) ? 0 : 2);
            vol += wv;
            s = fmaf(wv, (c & 4) ? rz[q] : rp[q], s);
        }
        bc[lin(ic, jc, m, X.csy, X.csz)] = __fdividef(s, vol);
        Wm[0] = Wp[0];
        Wm[1] = Wp[1];
        W0[0] = Wq[0];
        W0[1] = Wq[1];
        Wp[0] = Wr[0];
        Wp[1] = Wr[1];
        Wq[0] = Ws[0];
        Wq[1] = Ws[1];
        Nz = Mz;
        Np = Mp;
    }
}

// Round-to-nearest-even double -> float from the IEEE-754 encodings, entirely on the
// integer pipe (the FP64 pipe is the bottleneck of the outer kernels): normal results by
// truncating the mantissa to 23 bits and rounding the 29 dropped bits to nearest even (a
// carry may reach the exponent, up to infinity); results below the normal range by
// shifting the full 53-bit mantissa into the float's subnormal unit 2^-149 with the same
// rounding; overflow to infinity; NaN stays NaN (quiet, top payload bits kept).
__device__ __forceinline__ float f64_to_f32_rn(double v)
{
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const unsigned sign = (unsigned)(bits >> 32) & 0x80000000u;
    const int ef = (int)((bits >> 52) & 0x7ff);
    const int e = ef - 1023;
    const unsigned long long m = bits & 0xFFFFFFFFFFFFFull;
    if (e >= -126 && e <= 127) {
        const unsigned hi = (unsigned)(m >> 29);
        const unsigned long long rem = m & 0x1FFFFFFFull;
        unsigned f = ((unsigned)(e + 127) << 23) | hi;
        if (rem > 0x10000000ull || (rem == 0x10000000ull && (hi & 1u))) f += 1u;
        return __uint_as_float(f | sign);
    }
    if (ef == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? (0x400000u | (unsigned)(m >> 29)) : 0u));
    if (e > 127) return __uint_as_float(sign | 0x7f800000u);
    // below the normal range: value = (2^52 + m) 2^(e-52) = q 2^-149 with q = (2^52 + m) 2^(e+97)
    const int shift = -e - 97;                       // >= 30 here
    if (ef == 0 || shift > 53) return __uint_as_float(sign);   // below half the smallest subnormal
    const unsigned long long mf = m | (1ull << 52);
    unsigned q = (unsigned)(mf >> shift);
    const unsigned long long rem = mf & ((1ull << shift) - 1ull), half = 1ull << (shift - 1);
    if (rem > half || (rem == half && (q & 1u))) q += 1u;     // may become the smallest normal
    return __uint_as_float(sign | q);
}

// Exact float -> double from the encodings, on the integer pipe: subnormal floats are
// normalised (leading-zero count), Inf and NaN keep their payload.
__device__ __forceinline__ double f32_to_f64(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned mant = u & 0x7fffffu;
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    unsigned long long bits;
    if (e == 0u) {
        if (mant == 0u) return __longlong_as_double((long long)sign);
        // value = mant 2^-149; shift the leading one to bit 23
        const int s = __clz(mant) - 8;
        bits = sign | ((unsigned long long)(1023 - 126 - s) << 52) |
               ((unsigned long long)((mant << s) & 0x7fffffu) << 29);
    } else if (e == 255u) {
        bits = sign | (0x7ffull << 52) | ((unsigned long long)mant << 29);
    } else {
        bits = sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)mant << 29);
    }
    return __longlong_as_double((long long)bits);
}

// b + 0 on the integer pipe for every b that is not a NaN (-0 becomes +0, every other
// value is unchanged); a NaN stays a (quiet) NaN.
__device__ __forceinline__ double plus_zero(double b)
{
    unsigned long long u = (unsigned long long)__double_as_longlong(b);
    if (u == 0x8000000000000000ull) u = 0ull;
    if ((u & 0x7ff0000000000000ull) == 0x7ff0000000000000ull && (u & 0x000fffffffffffffull))
        u |= 0x0008000000000000ull;
    return __longlong_as_double((long long)u);
}

// float -> double on the integer pipe with one select: exact for normal values, zeros,
// infinities and NaNs; subnormal floats (below 2^-126) become zero.  For sums whose
// subnormal parts are far below the accuracy asked of them (the residual update).
__device__ __forceinline__ double f32_to_f64_fast(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned mag = u & 0x7fffffffu, e = mag >> 23;
    // normal: the exponent rebased by 1023 - 127 = 896; Inf/NaN: exponent field 0x7ff
    const unsigned long long body =
        e == 0u ? 0ull : (e == 255u ? ((0x7ffull << 52) | ((unsigned long long)(mag & 0x7fffffu) << 29))
                                    : (((unsigned long long)mag + (896ull << 23)) << 29));
    return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) | body));
}

// r(i,j,k) = b - A x in FP64, FMA form r = b + d x - sum c x_nb with d = -c0 = sx(i) + dyz
// (the per-axis diagonal sums), as the outer residual of the mixed solver.
__device__ __forceinline__ double outer_residual_cell_b(const LevelK<double> &L, double dyz, const double *x,
                                                        double bp, int i, int j, int k, long long p)
{
    const double d = L.sx[i] + dyz;
    double v = fma(d, x[p], bp);
    v = fma(-L.cxm[i], x[p - 1], v);
    v = fma(-L.cxp[i], x[p + 1], v);
    v = fma(-L.cym[j], x[p - L.sy], v);
    v = fma(-L.cyp[j], x[p + L.sy], v);
    v = fma(-L.czm[k], x[p - L.sz], v);
    v = fma(-L.czp[k], x[p + L.sz], v);
    return v;
}

// ---------------------------------------------------------------------------------------
// Compensated FP32 arithmetic for the residual update r_new = r - A e of the mixed solver
// (e is the FP32 correction, r the FP64 residual).  A e is formed in the difference form
// sum over the six neighbours of c_n (e_n - e_c) (c0 = -(c1 + ... + c6) per the reference's
// matrix, src/matrix.f90:67-92), so no term carries the large diagonal product:
//  * e_n - e_c exactly as an unevaluated FP32 pair by Knuth's two-sum;
//  * c_n = hi + lo (the FP64 coefficient split into two FP32 values, 48 bits);
//  * c_hi * d exactly as a pair by the FMA two-product; the small cross terms by FMAs;
//  * the six products summed with two-sum into (S, Sl).
// Every rounding error is of order 2^-48 of a term, so A e carries a relative error of
// about 2^-48 times sum |c_n (e_n - e_c)| / |A e| -- far below the FP64 rounding noise of a
// recomputed b - A x, with 4 instead of 10 FP64 operations per cell.  All operations use
// the _rn intrinsics, which the compiler never contracts.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void two_sum32(float a, float b, float &s, float &err)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (S, Sl) += c * (en - ec), c = (hi, lo)
__device__ __forceinline__ void comp_term(float2 c, float en, float ec, float &S, float &Sl)
{
    float d, dl;
    two_sum32(en, -ec, d, dl);
    const float p = __fmul_rn(c.x, d);
    float pe = __fmaf_rn(c.x, d, -p);
    pe = __fmaf_rn(c.x, dl, pe);
    pe = __fmaf_rn(c.y, d, pe);
    float s, t;
    two_sum32(S, p, s, t);
    S = s;
    Sl = __fadd_rn(Sl, __fadd_rn(t, pe));
}

__device__ __forceinline__ double outer_residual_cell(const LevelK<double> &L, double dyz, const double *x,
                                                      const double *b, int i, int j, int k, long long p)
{
    return outer_residual_cell_b(L, dyz, x, b[p], i, j, k, p);
}

template <typename F>
__device__ __forceinline__ void for_cells(int nx, int ny, int nz, F f)
{
    // tail levels hold at most 2^18 cells, so 32-bit index arithmetic suffices
    const int n = nx * ny * nz;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int rr = q / nx;
        f(q - rr * nx + 1, rr % ny + 1, rr / ny + 1);
    }
}

__device__ void t32_sweeps(const LevelK<float> &L, float *x, const float *b, int iters, float omega, float omw,
                           bool zero_start)
{
    const int hx = (L.nx + 1) / 2;
    const int nq = hx * L.ny * L.nz;
    for (int it = 0; it < iters; ++it)
        for (int colour = 0; colour < 2; ++colour) {
            if (zero_start && it == 0 && colour == 0) {
                for_cells(L.nx, L.ny, L.nz, [&](int i, int j, int k) {
                    const long long p = lin(i, j, k, L.sy, L.sz);
                    x[p] = ((i + j + k) & 1) ? __fdividef(omega * b[p], diag32(L, i, j, k)) : 0.f;
                });
            } else {
                for (int q = threadIdx.x; q < nq; q += blockDim.x) {
                    const int rr = q / hx;
                    const int t = q - rr * hx;
                    const int j = rr % L.ny + 1, k = rr / L.ny + 1;
                    const int i = 2 * t + 1 + ((j + k + colour) & 1);
                    if (i <= L.nx) x[lin(i, j, k, L.sy, L.sz)] = rbgs32(L, x, b, i, j, k, omega, omw);
                }
            }
            __syncthreads();
        }
}

// The single-CTA FP32 coarse tail for one problem on the level descriptors Ls / Xs and
// arrays xs / bs (the global arrays of D, or shared-memory copies).
__device__ void tail32_run(const TailDesc<float> &D, const LevelK<float> *Ls, const XferK<float> *Xs,
                           float *const *xs, float *const *bs, double *sw)
{
    const float omega = D.omega, omw = D.omw;
    for (int l = D.l0; l < D.nl; ++l) {
        const LevelK<float> L = Ls[l];
        const XferK<float> X = Xs[l];
        float *x = xs[l], *bc = bs[l + 1];
        const float *b = bs[l];
        t32_sweeps(L, x, b, D.maxit, omega, omw, true);
        for_cells(X.ncx, X.ncy, X.ncz, [&](int i, int j, int k) {
            bc[lin(i, j, k, X.csy, X.csz)] = resrestrict_cell32(L, X, x, b, i, j, k);
        });
        __syncthreads();
    }
    // coarsest level: solved in FP64 (b converted up, x converted down), so its
    // convergence test against the FP64 tolerance is attainable
    {
        const LevelK<float> L = Ls[D.nl];
        const LevelK<double> &C = D.C64;
        float *x = xs[D.nl];
        const float *b = bs[D.nl];
        if (C.sz * (C.nz + 2) <= kWarpCoarseMax) {
            // small coarsest level: shared memory, one warp, no block barriers per iteration
            __shared__ double cs[5][kWarpCoarseMax];
            const int total = (int)(C.sz * (C.nz + 2));
            for (int q = threadIdx.x; q < total; q += blockDim.x) cs[1][q] = 0.0;
            __syncthreads();
            for_cells(L.nx, L.ny, L.nz, [&](int i, int j, int k) {
                cs[1][lin(i, j, k, C.sy, C.sz)] = (double)b[lin(i, j, k, L.sy, L.sz)];
            });
            __syncthreads();
            int iters = 0;
            if (threadIdx.x < 32)
                iters = coarse_solve_warp_f64(C, cs[0], cs[1], cs[2], cs[3], cs[4], D.coarse_solver, D.coarse_maxit,
                                              D.tol, D.omega64, D.omw64, D.abort);
            if (threadIdx.x == 0 && D.iters_out) *D.iters_out = iters;
            __syncthreads();
            for_cells(L.nx, L.ny, L.nz, [&](int i, int j, int k) {
                x[lin(i, j, k, L.sy, L.sz)] = (float)cs[0][lin(i, j, k, C.sy, C.sz)];
            });
        } else {
            for_cells(L.nx, L.ny, L.nz, [&](int i, int j, int k) {
                D.cb64[lin(i, j, k, C.sy, C.sz)] = (double)b[lin(i, j, k, L.sy, L.sz)];
            });
            __syncthreads();
            const int iters = coarse_solve_f64(C, D.cx64, D.cb64, D.cp64, D.cap64, D.crr64, D.coarse_solver,
                                               D.coarse_maxit, D.tol, D.omega64, D.omw64, sw, D.abort);
            for_cells(L.nx, L.ny, L.nz, [&](int i, int j, int k) {
                x[lin(i, j, k, L.sy, L.sz)] = (float)D.cx64[lin(i, j, k, C.sy, C.sz)];
            });
            if (threadIdx.x == 0 && D.iters_out) *D.iters_out = iters;
        }
        __syncthreads();
    }
    for (int l = D.nl - 1; l >= D.l0; --l) {
        const LevelK<float> L = Ls[l];
        const XferK<float> X = Xs[l];
        float *x = xs[l], *xc = xs[l + 1];
        const float *b = bs[l];
        for_cells(X.ncx, X.ncy, X.ncz, [&](int i, int j, int k) { prolong_add_cell32(X, xc, x, i, j, k); });
        __syncthreads();
        t32_sweeps(L, x, b, D.maxit, omega, omw, false);
    }
}

__device__ void tail32_body(const TailDesc<float> &D, double *sw) { tail32_run(D, D.L, D.X, D.x, D.b, sw); }

// The tail with x and b of every tail level copied into shared memory `sm` (D.sm_floats
// floats, each array in the level's unpadded (nx+2)(ny+2)(nz+2) layout): b of the first
// tail level comes in from global memory and x of that level goes back, every other
// access stays on chip.
__device__ void tail32_body_smem(const TailDesc<float> &D, double *sw, float *sm)
{
    __shared__ LevelK<float> sL[kMaxLevels];
    __shared__ XferK<float> sX[kMaxLevels];
    __shared__ float *sxp[kMaxLevels], *sbp[kMaxLevels];
    if (threadIdx.x == 0) {
        int off = 0;
        for (int l = D.l0; l <= D.nl; ++l) {
            LevelK<float> L = D.L[l];
            L.sy = L.nx + 2;
            L.sz = (long long)L.sy * (L.ny + 2);
            const int tot = (int)(L.sz * (L.nz + 2));
            sL[l] = L;
            sxp[l] = sm + off;
            off += (tot + 3) & ~3;
            sbp[l] = sm + off;
            off += (tot + 3) & ~3;
        }
        for (int l = D.l0; l < D.nl; ++l) {
            XferK<float> X = D.X[l];
            X.fsy = sL[l].sy;
            X.fsz = sL[l].sz;
            X.csy = sL[l + 1].sy;
            X.csz = sL[l + 1].sz;
            sX[l] = X;
        }
    }
    for (int q = threadIdx.x; q < D.sm_floats; q += blockDim.x) sm[q] = 0.f;
    __syncthreads();
    const LevelK<float> &G = D.L[D.l0];
    const LevelK<float> &S = sL[D.l0];
    {
        const float *gb = D.b[D.l0];
        float *sb = sbp[D.l0];
        for_cells(G.nx, G.ny, G.nz,
                  [&](int i, int j, int k) { sb[lin(i, j, k, S.sy, S.sz)] = gb[lin(i, j, k, G.sy, G.sz)]; });
    }
    __syncthreads();
    tail32_run(D, sL, sX, sxp, sbp, sw);
    {
        float *gx = D.x[D.l0];
        const float *sx = sxp[D.l0];
        for_cells(G.nx, G.ny, G.nz,
                  [&](int i, int j, int k) { gx[lin(i, j, k, G.sy, G.sz)] = sx[lin(i, j, k, S.sy, S.sz)]; });
    }
    __syncthreads();
}

}  // namespace
}  // namespace pmg
