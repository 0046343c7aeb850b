// pmg_f64fast.cu -- the FP64 performance mode (PMG_FP64_FAST): the plain FP64 V-cycle with
// fewer FP64 instructions per cell, not bound to the reference's bits.
//
// The bitwise kernels (pmg_f64.cu) are FP64-pipe bound on this part (83-86% of the FP64
// pipe, 2-11% of HBM): an RBGS update costs 28 FP64 instructions there, an IEEE division
// among them.  This mode changes only the arithmetic of the grid levels, in three ways:
//   * FMA chains: b - sum c_n x_n as six DFMA, b - A x as seven;
//   * the diagonal enters as a stored per-cell factor omega / c0 (an FP64 array per grid
//     level, rebuilt when omega changes), so an update needs no division: 7 FP64
//     instructions for omega = 1, 8 otherwise;
//   * restriction and prolongation use per-axis weights normalised once at set-up: the
//     reference's volume weights are products of per-axis widths and their sums products
//     of per-axis sums (src/multigrid.f90:1474-1491, :1676-1754), so sum(V r)/sum(V) and
//     sum(w V)/prod(sum w) factor into three nested 2-term interpolations (14 FP64
//     instructions per coarse cell for the restriction, about 12 per fine cell for the
//     prolongation instead of 46 and 40).
// The coarse tail (single CTA) is the bitwise one.  The level sequence, the exit test
// and the reductions' order are those of the plain path, so the solve converges in the
// same number of cycles to the same solution within rounding (the tests bound the
// difference to the oracle's solution).
//
// Compiled with --fmad=true.
#include <cuda_runtime.h>

#include <algorithm>

#include "pmg_internal.h"

namespace pmg {

namespace {

constexpr int kBX = 32, kBY = 8;
constexpr int kMaxGridZ = 65535;

__device__ __forceinline__ int tid_in_block() { return threadIdx.x + blockDim.x * threadIdx.y; }
__device__ __forceinline__ int block_lin() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }

// omega / c0 for every interior cell, c0 summed in the reference's order (src/matrix.f90:82)
__global__ void __launch_bounds__(kBX *kBY) k_fast_wdiag(LevelK<double> L, double omega, double *__restrict__ w)
{
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x)
                w[lin(i, j, k, L.sy, L.sz)] = omega / diag_f64(L, i, j, k);
}

// One colour of the red-black sweep (colour 0: (i+j+k) odd first, as the bitwise kernel).
template <bool OMEGA1>
__global__ void __launch_bounds__(kBX *kBY) k_rbgs_fast(LevelK<double> L, const double *__restrict__ wd,
                                                        double *__restrict__ x, const double *__restrict__ b,
                                                        double omw, int colour)
{
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y) {
            const int ista = 1 + ((j + k + colour) & 1);
            const double cym = L.cym[j], cyp = L.cyp[j], czm = L.czm[k], czp = L.czp[k];
            for (int i = ista + 2 * (blockIdx.x * blockDim.x + threadIdx.x); i <= L.nx;
                 i += 2 * gridDim.x * blockDim.x) {
                const long long p = lin(i, j, k, L.sy, L.sz);
                double acc = fma(-L.cxm[i], x[p - 1], b[p]);
                acc = fma(-L.cxp[i], x[p + 1], acc);
                acc = fma(-cym, x[p - L.sy], acc);
                acc = fma(-cyp, x[p + L.sy], acc);
                acc = fma(-czm, x[p - L.sz], acc);
                acc = fma(-czp, x[p + L.sz], acc);
                x[p] = OMEGA1 ? wd[p] * acc : fma(wd[p], acc, omw * x[p]);
            }
        }
}

// r = b - A x with -c0 = sx(i) + dy(j) + dz(k); with NORM the per-block sums of r^2.
template <bool NORM>
__global__ void __launch_bounds__(kBX *kBY) k_residual_fast(LevelK<double> L, const double *__restrict__ dy,
                                                            const double *__restrict__ dz, double *__restrict__ r,
                                                            const double *__restrict__ x,
                                                            const double *__restrict__ b, double *partials)
{
    double acc2 = 0.0;
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y) {
            const double dyz = dy[j] + dz[k];
            const double cym = L.cym[j], cyp = L.cyp[j], czm = L.czm[k], czp = L.czp[k];
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= L.nx; i += gridDim.x * blockDim.x) {
                const long long p = lin(i, j, k, L.sy, L.sz);
                double acc = fma(L.sx[i] + dyz, x[p], b[p]);
                acc = fma(-L.cxm[i], x[p - 1], acc);
                acc = fma(-L.cxp[i], x[p + 1], acc);
                acc = fma(-cym, x[p - L.sy], acc);
                acc = fma(-cyp, x[p + L.sy], acc);
                acc = fma(-czm, x[p - L.sz], acc);
                acc = fma(-czp, x[p + L.sz], acc);
                r[p] = acc;
                if (NORM) acc2 = fma(acc, acc, acc2);
            }
        }
    if (NORM) {
        __shared__ double sw[kBX * kBY / 32];
        const double s = block_sum(acc2, sw);
        if (tid_in_block() == 0) partials[block_lin()] = s;
    }
}

// b_c = sum over the (up to) eight children of rw_x rw_y rw_z r_f, the per-axis weights
// normalised by their pair sums (a stride-1 axis has the pair (i, i) with weights 1/2).
__global__ void __launch_bounds__(kBX *kBY) k_restrict_fast(XferK<double> X, FastXferK W,
                                                            const double *__restrict__ vf, double *__restrict__ vc)
{
    for (int k = blockIdx.z + 1; k <= X.ncz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= X.ncy; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= X.ncx; i += gridDim.x * blockDim.x) {
                const int ip = i * X.stx, iz = ip - (X.stx - 1);
                const int jp = j * X.sty, jz = jp - (X.sty - 1);
                const int kp = k * X.stz, kz = kp - (X.stz - 1);
                const double ax = W.rx[iz], bx = W.rx[ip];
                double s[2][2];
#pragma unroll
                for (int c = 0; c < 2; ++c)
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        const long long p = lin(iz, q ? jp : jz, c ? kp : kz, X.fsy, X.fsz);
                        s[c][q] = fma(ax, vf[p], bx * vf[p + (ip - iz)]);
                    }
                const double t0 = fma(W.ry[jz], s[0][0], W.ry[jp] * s[0][1]);
                const double t1 = fma(W.ry[jz], s[1][0], W.ry[jp] * s[1][1]);
                vc[lin(i, j, k, X.csy, X.csz)] = fma(W.rz[kz], t0, W.rz[kp] * t1);
            }
}

// The eight children of a coarse cell, x_f += P x_c (ADD) or x_f = P x_c: per child a
// z-interpolation of y-interpolations of x-interpolations of the coarse values, with the
// weights of the reference's trilinear formula normalised per axis (pa own side, pb the
// neighbour's).  The x-interpolations of the 3 x 3 coarse lines around the cell are
// shared by the children.  Coarse ghost values (zero for a correction) enter as in the
// reference; along a stride-1 axis the neighbour is the cell itself.
template <bool ADD>
__global__ void __launch_bounds__(kBX *kBY) k_prolong_fast(XferK<double> X, FastXferK W,
                                                           const double *__restrict__ vc, double *__restrict__ vf)
{
    for (int k = blockIdx.z + 1; k <= X.ncz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= X.ncy; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= X.ncx; i += gridDim.x * blockDim.x) {
                const int ox = X.stx - 1, oy = X.sty - 1, oz = X.stz - 1;
                const int ip = i * X.stx, iz = ip - ox;
                const int jp = j * X.sty, jz = jp - oy;
                const int kp = k * X.stz, kz = kp - oz;
                // xi[s][b][c]: x-side s (0 low child iz, 1 high child ip) on coarse line
                // (j + (b-1) oy, k + (c-1) oz)
                double xi[2][3][3];
                const double alo = W.pax[iz], blo = W.pbx[iz], ahi = W.pax[ip], bhi = W.pbx[ip];
#pragma unroll
                for (int c = 0; c < 3; ++c)
#pragma unroll
                    for (int bb = 0; bb < 3; ++bb) {
                        const long long p = lin(i, j + (bb - 1) * oy, k + (c - 1) * oz, X.csy, X.csz);
                        const double v0 = vc[p];
                        xi[0][bb][c] = fma(alo, v0, blo * vc[p - ox]);
                        xi[1][bb][c] = fma(ahi, v0, bhi * vc[p + ox]);
                    }
#pragma unroll
                for (int sk = 0; sk < 2; ++sk) {
                    if (sk == 0 && oz == 0) continue;
                    const int kf = sk ? kp : kz, cz = sk ? 2 : 0;
                    const double az = W.paz[kf], bz = W.pbz[kf];
#pragma unroll
                    for (int sj = 0; sj < 2; ++sj) {
                        if (sj == 0 && oy == 0) continue;
                        const int jf = sj ? jp : jz, by = sj ? 2 : 0;
                        const double ay = W.pay[jf], byw = W.pby[jf];
#pragma unroll
                        for (int si = 0; si < 2; ++si) {
                            if (si == 0 && ox == 0) continue;
                            const int ifn = si ? ip : iz;
                            const double yo = fma(ay, xi[si][1][1], byw * xi[si][by][1]);
                            const double yn = fma(ay, xi[si][1][cz], byw * xi[si][by][cz]);
                            const double v = fma(az, yo, bz * yn);
                            const long long q = lin(ifn, jf, kf, X.fsy, X.fsz);
                            if (ADD)
                                vf[q] = vf[q] + v;
                            else
                                vf[q] = v;
                        }
                    }
                }
            }
}

// Per-axis tables of a level and of its transfer to the next (device side, from the
// plain path's tables): dy, dz = per-axis diagonal sums; restriction weights rw(f) =
// w(f) / (w(low) + w(high)) of f's pair; prolongation weights of fine index f (own side a,
// neighbour side b of the reference's dxp/dxn choice, src/multigrid.f90:1604-1610)
// normalised as a/(a+b), b/(a+b).  One thread per entry.
__global__ void k_fast_tables(LevelK<double> L, double *dy, double *dz, int has_x, XferK<double> X, int nfx, int nfy,
                              int nfz, double *rx, double *ry, double *rz, double *pax, double *pbx, double *pay,
                              double *pby, double *paz, double *pbz)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t <= L.ny + 1) dy[t] = (t >= 1 && t <= L.ny) ? L.cym[t] + L.cyp[t] : 0.0;
    if (t <= L.nz + 1) dz[t] = (t >= 1 && t <= L.nz) ? L.czm[t] + L.czp[t] : 0.0;
    if (!has_x) return;
    auto axis = [&](int f, int nf, int st, const double *w, const double *pp, const double *pn, double *rw,
                    double *pa, double *pb) {
        if (f > nf + 1) return;
        if (f < 1 || f > nf) {
            rw[f] = 0.0;
            pa[f] = 0.0;
            pb[f] = 0.0;
            return;
        }
        const int o = st - 1;
        const bool high = st == 1 || (f % 2 == 0);
        const int fp = high ? f : f + 1, fz = fp - o;   // the pair (fz, fp) of f's coarse cell
        // the reference weighs a child's value with the table entry of its sibling
        // (dxf = dxm_c - dxm_f, src/multigrid.f90:1422-1425; on a stride-1 axis the pair is
        // (f, f) and both terms are the same value)
        rw[f] = w[high ? fz : fp] / (w[fz] + w[fp]);
        const double a = high ? pn[fp] : pp[fz], b = high ? pn[fz] : pp[fp];
        pa[f] = a / (a + b);
        pb[f] = b / (a + b);
    };
    axis(t, nfx, X.stx, X.wx, X.pxp, X.pxn, rx, pax, pbx);
    axis(t, nfy, X.sty, X.wy, X.pyp, X.pyn, ry, pay, pby);
    axis(t, nfz, X.stz, X.wz, X.pzp, X.pzn, rz, paz, pbz);
}

dim3 grid3f(int nx_threads, int ny, int nz, const Launch &ln)
{
    dim3 g;
    g.x = ln.collapse[0] ? 1u : (unsigned)std::max(1, (nx_threads + kBX - 1) / kBX);
    g.y = ln.collapse[1] ? 1u : (unsigned)std::max(1, (ny + kBY - 1) / kBY);
    g.z = ln.collapse[2] ? 1u : (unsigned)std::max(1, std::min(nz, kMaxGridZ));
    return g;
}

}  // namespace

int fast_tables(const LevelK<double> &L, const XferK<double> *X, int nfx, int nfy, int nfz, FastLevelK *fl,
                FastXferK *fx, cudaStream_t s)
{
    const int n = std::max(std::max(L.ny, L.nz), std::max(nfx, std::max(nfy, nfz))) + 2;
    XferK<double> xx{};
    if (X) xx = *X;
    FastXferK w = fx ? *fx : FastXferK{};
    k_fast_tables<<<(n + 255) / 256, 256, 0, s>>>(L, fl->dy, fl->dz, X ? 1 : 0, xx, nfx, nfy, nfz, w.rx, w.ry, w.rz,
                                                 w.pax, w.pbx, w.pay, w.pby, w.paz, w.pbz);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "fast tables");
}

int fast_wdiag(const LevelK<double> &L, double omega, double *wdiag, cudaStream_t s)
{
    const Launch ln{{false, false, false}};
    k_fast_wdiag<<<grid3f(L.nx, L.ny, L.nz, ln), dim3(kBX, kBY, 1), 0, s>>>(L, omega, wdiag);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "fast diagonal");
}

int fast_rbgs_sweeps(const LevelK<double> &L, const FastLevelK &F, const Launch &ln, double *x, const double *b,
                     int iters, double omega, cudaStream_t s)
{
    const double omw = 1.0 - omega;
    const dim3 g = grid3f((L.nx + 1) / 2, L.ny, L.nz, ln), bl(kBX, kBY, 1);
    for (int it = 0; it < iters; ++it)
        for (int c = 0; c < 2; ++c) {
            if (omega == 1.0)
                k_rbgs_fast<true><<<g, bl, 0, s>>>(L, F.wdiag, x, b, omw, c);
            else
                k_rbgs_fast<false><<<g, bl, 0, s>>>(L, F.wdiag, x, b, omw, c);
        }
    count_launches(2LL * iters);
    return cuda_status(cudaGetLastError(), "fast rbgs sweep");
}

int fast_residual(const LevelK<double> &L, const FastLevelK &F, const Launch &ln, double *r, const double *x,
                  const double *b, double *partials, int *npart, cudaStream_t s)
{
    const dim3 g = grid3f(L.nx, L.ny, L.nz, ln), bl(kBX, kBY, 1);
    if (partials) {
        k_residual_fast<true><<<g, bl, 0, s>>>(L, F.dy, F.dz, r, x, b, partials);
        *npart = (int)(g.x * g.y * g.z);
    } else {
        k_residual_fast<false><<<g, bl, 0, s>>>(L, F.dy, F.dz, r, x, b, nullptr);
    }
    count_launches(1);
    return cuda_status(cudaGetLastError(), "fast residual");
}

int fast_restrict(const XferK<double> &X, const FastXferK &W, const Launch &ln, const double *vf, double *vc,
                  cudaStream_t s)
{
    k_restrict_fast<<<grid3f(X.ncx, X.ncy, X.ncz, ln), dim3(kBX, kBY, 1), 0, s>>>(X, W, vf, vc);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "fast restriction");
}

int fast_prolong(const XferK<double> &X, const FastXferK &W, const Launch &ln, const double *vc, double *vf,
                 cudaStream_t s)
{
    k_prolong_fast<true><<<grid3f(X.ncx, X.ncy, X.ncz, ln), dim3(kBX, kBY, 1), 0, s>>>(X, W, vc, vf);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "fast prolongation");
}

}  // namespace pmg
