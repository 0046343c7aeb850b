// pmg_common.cuh -- shared device-side descriptors and the per-cell FP64 arithmetic of
// the multigrid hot path.
//
// Every per-cell function here reproduces the floating-point operation order of the
// reference Fortran expression it cites (paths relative to the reference project
// root), and the translation units that include this header for FP64 are compiled
// with --fmad=false, so the FP64 results are bit-identical to the reference's
// non-FMA arithmetic.  Each function is used both by the grid-wide kernels and by
// the single-CTA persistent coarse-tail kernel, which is what makes the CGS, CGA and
// CGPSA execution mappings produce identical bits.
#pragma once

#include <cstdint>

namespace pmg {

// One level of the hierarchy as the kernels see it.  Arrays are (0:nx+1,0:ny+1,0:nz+1)
// with element (i,j,k) at i + sy*j + sz*k.  Coefficient tables are per axis, indexed by
// the cell index 1..n: cm = 1/(dm*dg) (coefficient to the lower neighbour), cp =
// 1/(dm*dg(+1)) (upper neighbour), sx = cxm + cxp (first partial sum of the diagonal).
// Built on the host exactly as src/matrix.f90:67-77.
template <typename T>
struct LevelK {
    int nx, ny, nz;
    int sy;
    long long sz;
    const T *cxm, *cxp, *sx, *cym, *cyp, *czm, *czp;
};

// Transfer between fine level l and coarse level l+1 (restriction and prolongation).
// st{x,y,z} = 2 (halving) or 1 (axis no longer coarsened, src/multigrid.f90:1415-1458).
// w* = restriction weights dxf (src/multigrid.f90:1415-1458) on the fine index,
// p*/n* = prolongation weights dxp/dxn (src/multigrid.f90:1594-1649) on the fine index.
template <typename T>
struct XferK {
    int ncx, ncy, ncz;
    int csy;
    long long csz;
    int fsy;
    long long fsz;
    int stx, sty, stz;
    const T *wx, *wy, *wz;
    const T *pxp, *pxn, *pyp, *pyn, *pzp, *pzn;
};

__host__ __device__ inline long long lin(int i, int j, int k, int sy, long long sz)
{
    return (long long)i + (long long)sy * j + sz * k;
}

// Diagonal coefficient: -(dxmp2i + dxmn2i + dymp2i + dymn2i + dzmp2i + dzmn2i),
// summed left to right (src/matrix.f90:82).
__device__ __forceinline__ double diag_f64(const LevelK<double> &L, int i, int j, int k)
{
    double s = L.sx[i];
    s = __dadd_rn(s, L.cym[j]);
    s = __dadd_rn(s, L.cyp[j]);
    s = __dadd_rn(s, L.czm[k]);
    s = __dadd_rn(s, L.czp[k]);
    return -s;
}

// RBGS update of one cell (src/rbgs_poisson_matrix.f90:244-250):
//   temp = c1 x(i-1) + c2 x(i+1) + c3 x(j-1) + c4 x(j+1) + c5 x(k-1) + c6 x(k+1)
//   x    = omega (rhs - temp) / c0 + (1 - omega) x
// with c0 given (diag_f64's value, computed or read from a per-cell table).  OMEGA1: omega
// is exactly 1, and 1 * v equals v for every double, so that product is not formed.
template <bool OMEGA1>
__device__ __forceinline__ double rbgs_cell_c0_f64(const LevelK<double> &L, const double *x, const double *b, int i,
                                                   int j, int k, double omega, double omw, double c0)
{
    const long long p = lin(i, j, k, L.sy, L.sz);
    double t = __dmul_rn(L.cxm[i], x[p - 1]);
    t = __dadd_rn(t, __dmul_rn(L.cxp[i], x[p + 1]));
    t = __dadd_rn(t, __dmul_rn(L.cym[j], x[p - L.sy]));
    t = __dadd_rn(t, __dmul_rn(L.cyp[j], x[p + L.sy]));
    t = __dadd_rn(t, __dmul_rn(L.czm[k], x[p - L.sz]));
    t = __dadd_rn(t, __dmul_rn(L.czp[k], x[p + L.sz]));
    const double d = __dsub_rn(b[p], t);
    const double q = __ddiv_rn(OMEGA1 ? d : __dmul_rn(omega, d), c0);
    return __dadd_rn(q, __dmul_rn(omw, x[p]));
}

__device__ __forceinline__ double rbgs_cell_f64(const LevelK<double> &L, const double *x, const double *b, int i,
                                                int j, int k, double omega, double omw)
{
    return rbgs_cell_c0_f64<false>(L, x, b, i, j, k, omega, omw, diag_f64(L, i, j, k));
}

// (A x)(i,j,k) = c0 x + c1 x(i-1) + c2 x(i+1) + c3 x(j-1) + c4 x(j+1) + c5 x(k-1) + c6 x(k+1)
// (src/poisson_matrix_operator.f90:150-156), with c0 given
__device__ __forceinline__ double ax_cell_c0_f64(const LevelK<double> &L, const double *x, int i, int j, int k,
                                                 double c0)
{
    const long long p = lin(i, j, k, L.sy, L.sz);
    double t = __dmul_rn(c0, x[p]);
    t = __dadd_rn(t, __dmul_rn(L.cxm[i], x[p - 1]));
    t = __dadd_rn(t, __dmul_rn(L.cxp[i], x[p + 1]));
    t = __dadd_rn(t, __dmul_rn(L.cym[j], x[p - L.sy]));
    t = __dadd_rn(t, __dmul_rn(L.cyp[j], x[p + L.sy]));
    t = __dadd_rn(t, __dmul_rn(L.czm[k], x[p - L.sz]));
    t = __dadd_rn(t, __dmul_rn(L.czp[k], x[p + L.sz]));
    return t;
}

__device__ __forceinline__ double ax_cell_f64(const LevelK<double> &L, const double *x, int i, int j, int k)
{
    const long long p = lin(i, j, k, L.sy, L.sz);
    double t = __dmul_rn(diag_f64(L, i, j, k), x[p]);
    t = __dadd_rn(t, __dmul_rn(L.cxm[i], x[p - 1]));
    t = __dadd_rn(t, __dmul_rn(L.cxp[i], x[p + 1]));
    t = __dadd_rn(t, __dmul_rn(L.cym[j], x[p - L.sy]));
    t = __dadd_rn(t, __dmul_rn(L.cyp[j], x[p + L.sy]));
    t = __dadd_rn(t, __dmul_rn(L.czm[k], x[p - L.sz]));
    t = __dadd_rn(t, __dmul_rn(L.czp[k], x[p + L.sz]));
    return t;
}

// Restriction of one coarse cell (src/multigrid.f90:1474-1491): volume-weighted mean
// of the (up to) eight children; vol_c = sum(vol_f) in array-element order.
__device__ __forceinline__ double restrict_cell_f64(const XferK<double> &X, const double *vf, int i, int j, int k)
{
    const int ip = i * X.stx, iz = ip - (X.stx - 1);
    const int jp = j * X.sty, jz = jp - (X.sty - 1);
    const int kp = k * X.stz, kz = kp - (X.stz - 1);
    const double xz = X.wx[iz], xp = X.wx[ip], yz = X.wy[jz], yp = X.wy[jp], zz = X.wz[kz], zp = X.wz[kp];
    const double v111 = __dmul_rn(__dmul_rn(xz, yz), zz);
    const double v211 = __dmul_rn(__dmul_rn(xp, yz), zz);
    const double v121 = __dmul_rn(__dmul_rn(xz, yp), zz);
    const double v221 = __dmul_rn(__dmul_rn(xp, yp), zz);
    const double v112 = __dmul_rn(__dmul_rn(xz, yz), zp);
    const double v212 = __dmul_rn(__dmul_rn(xp, yz), zp);
    const double v122 = __dmul_rn(__dmul_rn(xz, yp), zp);
    const double v222 = __dmul_rn(__dmul_rn(xp, yp), zp);
    double vol = __dadd_rn(v111, v211);
    vol = __dadd_rn(vol, v121);
    vol = __dadd_rn(vol, v221);
    vol = __dadd_rn(vol, v112);
    vol = __dadd_rn(vol, v212);
    vol = __dadd_rn(vol, v122);
    vol = __dadd_rn(vol, v222);
    const int sy = X.fsy;
    const long long sz = X.fsz;
    double s = __dmul_rn(v111, vf[lin(ip, jp, kp, sy, sz)]);
    s = __dadd_rn(s, __dmul_rn(v211, vf[lin(iz, jp, kp, sy, sz)]));
    s = __dadd_rn(s, __dmul_rn(v121, vf[lin(ip, jz, kp, sy, sz)]));
    s = __dadd_rn(s, __dmul_rn(v221, vf[lin(iz, jz, kp, sy, sz)]));
    s = __dadd_rn(s, __dmul_rn(v112, vf[lin(ip, jp, kz, sy, sz)]));
    s = __dadd_rn(s, __dmul_rn(v212, vf[lin(iz, jp, kz, sy, sz)]));
    s = __dadd_rn(s, __dmul_rn(v122, vf[lin(ip, jz, kz, sy, sz)]));
    s = __dadd_rn(s, __dmul_rn(v222, vf[lin(iz, jz, kz, sy, sz)]));
    return __ddiv_rn(s, vol);
}

// One child of a coarse cell in the prolongation (src/multigrid.f90:1676-1754).  The
// eight terms are, in the reference's order: centre, x-neighbour, y-neighbour,
// z-neighbour, xy, xz, yz, xyz; each weight is the product (wx*wy)*wz of the own-side
// (a*) or the neighbour-side (b*) 1-D weights, then times the coarse value.
// The denominator is ((ax+bx)*(ay+by))*(az+bz).
__device__ __forceinline__ double prolong_child_f64(double ax, double bx, double ay, double by, double az,
                                                    double bz, double v000, double v100, double v010,
                                                    double v001, double v110, double v101, double v011,
                                                    double v111)
{
    double t = __dmul_rn(__dmul_rn(__dmul_rn(ax, ay), az), v000);
    t = __dadd_rn(t, __dmul_rn(__dmul_rn(__dmul_rn(bx, ay), az), v100));
    t = __dadd_rn(t, __dmul_rn(__dmul_rn(__dmul_rn(ax, by), az), v010));
    t = __dadd_rn(t, __dmul_rn(__dmul_rn(__dmul_rn(ax, ay), bz), v001));
    t = __dadd_rn(t, __dmul_rn(__dmul_rn(__dmul_rn(bx, by), az), v110));
    t = __dadd_rn(t, __dmul_rn(__dmul_rn(__dmul_rn(bx, ay), bz), v101));
    t = __dadd_rn(t, __dmul_rn(__dmul_rn(__dmul_rn(ax, by), bz), v011));
    t = __dadd_rn(t, __dmul_rn(__dmul_rn(__dmul_rn(bx, by), bz), v111));
    const double den = __dmul_rn(__dmul_rn(__dadd_rn(ax, bx), __dadd_rn(ay, by)), __dadd_rn(az, bz));
    return __ddiv_rn(t, den);
}

// Prolongation of one coarse cell into its children.  ADD = false writes the children
// (the reference's val_f, src/multigrid.f90:1676-1754); ADD = true adds them to the
// fine array, which is the reference's val_f write followed by x = x + r
// (src/multigrid.f90:1957-1958).  Along an axis with stride 1 the two children
// coincide; the reference writes that element twice with identical values (the
// weights dxp and dxn are both dm_c there), so only the later write is formed.
template <bool ADD>
__device__ __forceinline__ void prolong_cell_f64(const XferK<double> &X, const double *vc, double *vf, int i, int j,
                                                 int k)
{
    const int ox = X.stx - 1, oy = X.sty - 1, oz = X.stz - 1;
    const int ip = i * X.stx, iz = ip - ox;
    const int jp = j * X.sty, jz = jp - oy;
    const int kp = k * X.stz, kz = kp - oz;
    const int csy = X.csy;
    const long long csz = X.csz;
    auto V = [&](int a, int b, int c) { return vc[lin(a, b, c, csy, csz)]; };
    // child sides: s = 0 (low: weights p(z_f), p(p_f), neighbour i-1) or 1 (high:
    // weights n(p_f), n(z_f), neighbour i+1)
#pragma unroll
    for (int sk = 0; sk < 2; ++sk) {
        if (sk == 0 && oz == 0) continue;
        const double az = sk ? X.pzn[kp] : X.pzp[kz];
        const double bz = sk ? X.pzn[kz] : X.pzp[kp];
        const int kn = sk ? k + oz : k - oz;
        const int kf = sk ? kp : kz;
#pragma unroll
        for (int sj = 0; sj < 2; ++sj) {
            if (sj == 0 && oy == 0) continue;
            const double ay = sj ? X.pyn[jp] : X.pyp[jz];
            const double by = sj ? X.pyn[jz] : X.pyp[jp];
            const int jn = sj ? j + oy : j - oy;
            const int jf = sj ? jp : jz;
#pragma unroll
            for (int si = 0; si < 2; ++si) {
                if (si == 0 && ox == 0) continue;
                const double ax = si ? X.pxn[ip] : X.pxp[iz];
                const double bx = si ? X.pxn[iz] : X.pxp[ip];
                const int in = si ? i + ox : i - ox;
                const int ifn = si ? ip : iz;
                const double v = prolong_child_f64(ax, bx, ay, by, az, bz, V(i, j, k), V(in, j, k), V(i, jn, k),
                                                   V(i, j, kn), V(in, jn, k), V(in, j, kn), V(i, jn, kn),
                                                   V(in, jn, kn));
                const long long q = lin(ifn, jf, kf, X.fsy, X.fsz);
                if (ADD)
                    vf[q] = __dadd_rn(vf[q], v);
                else
                    vf[q] = v;
            }
        }
    }
}

// Deterministic block-wide sum (fixed shuffle tree, then warps in order).  All
// threads of the block must call it; returns the sum in every thread.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T *smem_warp)
{
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = tid & 31, warp = tid >> 5;
    const int nwarp = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = v + __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) smem_warp[warp] = v;
    __syncthreads();
    T s = T(0);
    if (tid == 0) {
        for (int w = 0; w < nwarp; ++w) s = s + smem_warp[w];
        smem_warp[0] = s;
    }
    __syncthreads();
    s = smem_warp[0];
    __syncthreads();
    return s;
}

}  // namespace pmg
