// pmg_smooth32.cuh -- device code of the fused FP32 red-black iteration (one item).
//
// One item = one RBGS iteration of src/rbgs_poisson_matrix.f90:235-273 (first colour,
// then second colour) on a tile of (TX = 60) x TY interior cells over a chunk of planes
// k0..k1, out of place (e_out = RB(e_in); every value read from e_in is an old value, so
// tiles need no ordering among themselves).
//
// Mapping: warp w owns row j = j0 - 1 + w (TY tile rows plus one ring row on each side);
// lane l owns the cell pair (i0 - 2 + 2l, i0 - 1 + 2l), so lanes 1..30 cover the tile's
// 60 columns and lanes 0 and 31 the ring columns.  Each thread keeps its pair for planes
// t-2 .. t+3 in registers (the z-neighbours), takes its x-neighbours from the adjacent
// lanes by shuffles, and its y-neighbours from a 4-slot ring of shared planes in which
// every warp deposits its row.  Step t updates the first colour on plane t (tile + ring)
// and, after one barrier, the second colour on plane t-1 (tile), whose final pair is
// stored with one 8-byte store.  Global loads run three planes ahead in registers.
// DRAM traffic per iteration: e_in read once, b read once, e_out written once (12 B per
// cell; 8 B when e_in = 0, which is not read).
//
// The plane loop is unrolled by the six-plane register window (fixed register roles),
// and the colour of the pair's first-colour cell is a template parameter of each
// unrolled step, so the per-cell work is a handful of FMAs, two shuffles, two shared
// loads and one reciprocal.
#pragma once

#include "pmg_common.cuh"

namespace pmg {

constexpr int RB_TX = 60;        // tile columns
constexpr int RB_SW = 64;        // shared row width (one pair per lane)
constexpr int RB_NS = 4;         // shared plane slots
constexpr int RB_TYMAX = 14;     // tallest tile
constexpr int RB_PAD_ROWS = RB_TYMAX + 2;   // zero rows above ny+1 read by the last tile row
constexpr int RB_PAD_PLANES = 3;            // zero planes above nz+1 read ahead by the last chunk
constexpr int RB_ZC = 128;       // z coefficients staged per item (planes k0-1 .. k0+RB_ZC-2)

template <int TY>
constexpr int rb_threads() { return (TY + 2) * 32; }

template <int TY>
struct RbSmem {
    float s[RB_NS][TY + 4][RB_SW];   // rows j0-2 .. j0+TY+1
    float2 zc[RB_ZC];                // (czm, czp) of planes k0-1 ..
};

namespace rbdetail {

// pair load (8-byte aligned; padding makes every pair the kernel reads addressable)
__device__ __forceinline__ float2 ld2(const float *q) { return __ldg(reinterpret_cast<const float2 *>(q)); }

template <int Q>
__device__ __forceinline__ float cq(const float2 &v) { return Q ? v.y : v.x; }
template <int Q>
__device__ __forceinline__ void sq(float2 &v, float x)
{
    if (Q)
        v.y = x;
    else
        v.x = x;
}

}  // namespace rbdetail

template <int TY, bool ZERO_IN, bool OMEGA1>
struct RbItem {
    // per-thread constants of the item
    const float2 *zc;                // staged (czm, czp), index t - (k0 - 1)
    int nz, k0, k1, lane, r, ro, sz32;
    bool has_outer, store_lane;
    bool need0, need1;               // the lane updates the first-colour cell when it is cell 0 / 1
    bool st_full;                    // the final pair is stored whole (else only its first cell)
    const float *pe, *po, *pb;       // e_in row, outer row, b row at plane 0
    float *pw;                       // e_out row at plane 0
    float omega, omw;
    float dxy[2], cxm[2], cxp[2], cym, cyp;   // dxy = x-part + y-part of -c0
    float2 E[6], B[6];               // planes t-2 .. t+3 at window positions (P .. P+5) % 6
    float2 O[3];                     // outer row, planes t+1 .. t+3 at positions (P .. P+2) % 3

    __device__ __forceinline__ float2 LE(int k) const
    {
        if (ZERO_IN) return make_float2(0.f, 0.f);
        return rbdetail::ld2(pe + sz32 * k);
    }
    __device__ __forceinline__ float2 LO(int k) const
    {
        if (ZERO_IN || !has_outer) return make_float2(0.f, 0.f);
        return rbdetail::ld2(po + sz32 * k);
    }
    __device__ __forceinline__ float2 LB(int k) const { return rbdetail::ld2(pb + sz32 * k); }

    __device__ __forceinline__ float upd(float old, float bb, float s, float c0) const
    {
        if (OMEGA1) return __fdividef(bb - s, c0);
        return fmaf(omw, old, __fdividef(omega * (bb - s), c0));
    }

    // One step: first colour on plane t, second colour on plane t-1.  P = window position
    // of plane t-2; Q = index within the pair of the first-colour cell on plane t (and of
    // the second-colour cell on plane t-1).
    template <int P, int Q>
    __device__ __forceinline__ void step(RbSmem<TY> &S, int t)
    {
        using namespace rbdetail;
        constexpr int im2 = P % 6, im1 = (P + 1) % 6, i00 = (P + 2) % 6, ip1 = (P + 3) % 6, ip3 = (P + 5) % 6;
        constexpr int o1 = P % 3, o3 = (P + 2) % 3;
        E[ip3] = LE(t + 3);
        O[o3] = LO(t + 3);
        B[ip3] = LB(t + 3);
        {
            float(*St)[RB_SW] = S.s[t & 3];
            const float up = __shfl_up_sync(0xffffffffu, E[i00].y, 1);
            const float dn = __shfl_down_sync(0xffffffffu, E[i00].x, 1);
            if ((Q ? need1 : need0) && t >= 1 && t <= nz) {
                // only second-colour words of the neighbouring rows are read here
                const float yl = St[r - 1][2 * lane + Q];
                const float yr = St[r + 1][2 * lane + Q];
                const float2 cz = zc[t - k0 + 1];
                const float czm = cz.x, czp = cz.y;
                const float left = Q ? E[i00].x : up;
                const float right = Q ? dn : E[i00].y;
                float s = cxm[Q] * left;
                s = fmaf(cxp[Q], right, s);
                s = fmaf(cym, yl, s);
                s = fmaf(cyp, yr, s);
                s = fmaf(czm, cq<Q>(E[im1]), s);
                s = fmaf(czp, cq<Q>(E[ip1]), s);
                const float c0 = -(dxy[Q] + (czm + czp));
                const float v = upd(cq<Q>(E[i00]), cq<Q>(B[i00]), s, c0);
                sq<Q>(E[i00], v);
                St[r][2 * lane + Q] = v;
            }
            float(*Sn)[RB_SW] = S.s[(t + 1) & 3];
            *reinterpret_cast<float2 *>(&Sn[r][2 * lane]) = E[ip1];
            if (has_outer) *reinterpret_cast<float2 *>(&Sn[ro][2 * lane]) = O[o1];
        }
        __syncthreads();
        {
            const int s1 = t - 1;
            const float up = __shfl_up_sync(0xffffffffu, E[im1].y, 1);
            const float dn = __shfl_down_sync(0xffffffffu, E[im1].x, 1);
            if (store_lane && s1 >= k0 && s1 <= k1) {
                if (Q == 0 || st_full) {
                    float(*Ss)[RB_SW] = S.s[s1 & 3];
                    const float yl = Ss[r - 1][2 * lane + Q];
                    const float yr = Ss[r + 1][2 * lane + Q];
                    const float2 cz = zc[s1 - k0 + 1];
                    const float czm = cz.x, czp = cz.y;
                    const float left = Q ? E[im1].x : up;
                    const float right = Q ? dn : E[im1].y;
                    float s = cxm[Q] * left;
                    s = fmaf(cxp[Q], right, s);
                    s = fmaf(cym, yl, s);
                    s = fmaf(cyp, yr, s);
                    s = fmaf(czm, cq<Q>(E[im2]), s);
                    s = fmaf(czp, cq<Q>(E[i00]), s);
                    const float c0 = -(dxy[Q] + (czm + czp));
                    const float v = upd(cq<Q>(E[im1]), cq<Q>(B[im1]), s, c0);
                    sq<Q>(E[im1], v);
                }
                float *g = pw + sz32 * s1;
                if (st_full)
                    *reinterpret_cast<float2 *>(g) = E[im1];
                else
                    g[0] = E[im1].x;
            }
        }
    }

    template <int Q0>
    __device__ __forceinline__ void run(RbSmem<TY> &S)
    {
        int t = k0 - 1;
        for (; t + 5 <= k1 + 1; t += 6) {
            step<0, Q0>(S, t);
            step<1, 1 - Q0>(S, t + 1);
            step<2, Q0>(S, t + 2);
            step<3, 1 - Q0>(S, t + 3);
            step<4, Q0>(S, t + 4);
            step<5, 1 - Q0>(S, t + 5);
        }
        if (t <= k1 + 1) step<0, Q0>(S, t++);
        if (t <= k1 + 1) step<1, 1 - Q0>(S, t++);
        if (t <= k1 + 1) step<2, Q0>(S, t++);
        if (t <= k1 + 1) step<3, 1 - Q0>(S, t++);
        if (t <= k1 + 1) step<4, Q0>(S, t++);
    }
};

template <int TY, bool ZERO_IN, bool OMEGA1>
__device__ __forceinline__ void rb32_item(RbSmem<TY> &S, const LevelK<float> &L, const float *__restrict__ ein,
                                          float *__restrict__ eout, const float *__restrict__ b, float omega,
                                          float omw, int bx, int by, int k0, int k1)
{
    RbItem<TY, ZERO_IN, OMEGA1> I;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i0 = 1 + RB_TX * bx, j0 = 1 + TY * by;
    const int nx = L.nx, ny = L.ny;
    const int a = i0 - 2 + 2 * lane;
    const int j = j0 - 1 + w;
    for (int q = threadIdx.x; q < k1 - k0 + 3; q += blockDim.x) {
        const int k = k0 - 1 + q;
        S.zc[q] = (k >= 1 && k <= L.nz) ? make_float2(L.czm[k], L.czp[k]) : make_float2(0.f, 0.f);
    }
    I.zc = S.zc;
    I.nz = L.nz;
    I.k0 = k0;
    I.k1 = k1;
    I.lane = lane;
    I.r = w + 1;
    I.sz32 = (int)L.sz;
    I.omega = omega;
    I.omw = omw;
    const bool row_in = j >= 1 && j <= ny;
    const int jo = w == 0 ? j0 - 2 : j0 + TY + 1;
    I.ro = w == 0 ? 0 : TY + 3;
    I.has_outer = (w == 0 || w == TY + 1);
    // a lane updates the first-colour cell of its pair when it is interior and in the tile
    // or the ring cell beside it (lane 0: its second cell, lane 31: its first cell)
    const bool in0 = a >= 1 && a <= nx, in1 = a + 1 >= 1 && a + 1 <= nx;
    const bool mid = lane >= 1 && lane <= 30;
    I.need0 = row_in && in0 && (mid || lane == 31);
    I.need1 = row_in && in1 && (mid || lane == 0);
    I.store_lane = (w >= 1 && w <= TY) && row_in && mid && a <= nx;
    I.st_full = a + 1 <= nx;
    const long long rowoff = (long long)a + (long long)L.sy * j;
    I.pe = ein + rowoff;
    I.pb = b + rowoff;
    I.pw = eout + rowoff;
    I.po = ein + (long long)a + (long long)L.sy * jo;
    I.cym = row_in ? L.cym[j] : 0.f;
    I.cyp = row_in ? L.cyp[j] : 0.f;
    const float dy = I.cym + I.cyp;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int i = a + q;
        const bool in = i >= 1 && i <= nx;
        I.dxy[q] = (in ? L.sx[i] : 0.f) + dy;
        I.cxm[q] = in ? L.cxm[i] : 0.f;
        I.cxp[q] = in ? L.cxp[i] : 0.f;
    }

    // window at the first step t = k0 - 1: positions 0..5 = planes k0-3 .. k0+2
    I.E[0] = make_float2(0.f, 0.f);
    I.E[1] = I.LE(k0 - 2);
    I.E[2] = I.LE(k0 - 1);
    I.E[3] = I.LE(k0);
    I.E[4] = I.LE(k0 + 1);
    I.O[0] = I.LO(k0);
    I.O[1] = I.LO(k0 + 1);
    I.B[1] = make_float2(0.f, 0.f);
    I.B[2] = I.LB(k0 - 1);
    I.B[3] = I.LB(k0);
    I.B[4] = I.LB(k0 + 1);
    {
        const float2 o0 = I.LO(k0 - 1);
        *reinterpret_cast<float2 *>(&S.s[(k0 - 1) & 3][I.r][2 * lane]) = I.E[2];
        if (I.has_outer) *reinterpret_cast<float2 *>(&S.s[(k0 - 1) & 3][I.ro][2 * lane]) = o0;
    }
    __syncthreads();
    // the pair's first cell a is odd, so it carries the first colour on plane k when j + k
    // is even ((i + j + k) odd, src/rbgs_poisson_matrix.f90:242)
    if (((j + k0 - 1) & 1) == 0)
        I.template run<0>(S);
    else
        I.template run<1>(S);
    __syncthreads();
}

}  // namespace pmg
