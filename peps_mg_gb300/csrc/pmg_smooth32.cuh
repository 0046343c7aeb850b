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
#pragma once

#include "pmg_common.cuh"

namespace pmg {

constexpr int RB_TX = 60;        // tile columns
constexpr int RB_SW = 64;        // shared row width (one pair per lane)
constexpr int RB_NS = 4;         // shared plane slots

template <int TY>
constexpr int rb_threads() { return (TY + 2) * 32; }

template <int TY>
struct RbSmem {
    float s[RB_NS][TY + 4][RB_SW];   // rows j0-2 .. j0+TY+1
};

namespace rbdetail {

// pair (a, a+1) of plane k, row j, columns valid in [0, nx+1], rows in [0, ny+1], planes in
// [0, nz+1]; elsewhere 0
__device__ __forceinline__ float2 load_pair(const float *__restrict__ p, int a, int j, int k, int nx, int ny, int nz,
                                            int sy, long long sz)
{
    float2 v = make_float2(0.f, 0.f);
    if (j < 0 || j > ny + 1 || k < 0 || k > nz + 1) return v;
    const float *q = p + (long long)a + (long long)sy * j + sz * k;
    if (a >= 0 && a + 1 <= nx + 1) {
        v = __ldg(reinterpret_cast<const float2 *>(q));
    } else {
        if (a >= 0 && a <= nx + 1) v.x = __ldg(q);
        if (a + 1 >= 0 && a + 1 <= nx + 1) v.y = __ldg(q + 1);
    }
    return v;
}

__device__ __forceinline__ float comp(const float2 &v, int q) { return q ? v.y : v.x; }
__device__ __forceinline__ void setc(float2 &v, int q, float x)
{
    if (q)
        v.y = x;
    else
        v.x = x;
}

}  // namespace rbdetail

template <int TY, bool ZERO_IN>
__device__ void rb32_item(RbSmem<TY> &S, const LevelK<float> &L, const float *__restrict__ ein,
                          float *__restrict__ eout, const float *__restrict__ b, float omega, float omw, int bx,
                          int by, int k0, int k1)
{
    using namespace rbdetail;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i0 = 1 + RB_TX * bx, j0 = 1 + TY * by;
    const int nx = L.nx, ny = L.ny, nz = L.nz;
    const int sy = L.sy;
    const long long sz = L.sz;
    const int a = i0 - 2 + 2 * lane;           // first cell of the lane's pair
    const int j = j0 - 1 + w;                  // the warp's row
    const int r = w + 1;                       // its shared row
    const bool row_in = j >= 1 && j <= ny;
    const bool tile_row = w >= 1 && w <= TY;
    // the outer rows j0-2 and j0+TY+1 are deposited by the first and the last warp
    const bool has_outer = (w == 0) || (w == TY + 1);
    const int jo = w == 0 ? j0 - 2 : j0 + TY + 1;
    const int ro = w == 0 ? 0 : TY + 3;

    // per-lane x-coefficients (both cells of the pair) and per-warp y-coefficients
    float dxc[2], cxm[2], cxp[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int i = a + q;
        const bool in = i >= 1 && i <= nx;
        dxc[q] = in ? L.sx[i] : 0.f;
        cxm[q] = in ? L.cxm[i] : 0.f;
        cxp[q] = in ? L.cxp[i] : 0.f;
    }
    const float cym = row_in ? L.cym[j] : 0.f, cyp = row_in ? L.cyp[j] : 0.f;
    const float dy = cym + cyp;

    auto LE = [&](int k) -> float2 {
        if (ZERO_IN) return make_float2(0.f, 0.f);
        return load_pair(ein, a, j, k, nx, ny, nz, sy, sz);
    };
    auto LO = [&](int k) -> float2 {
        if (ZERO_IN || !has_outer) return make_float2(0.f, 0.f);
        return load_pair(ein, a, jo, k, nx, ny, nz, sy, sz);
    };
    auto LB = [&](int k) -> float2 {
        if (k < 1 || k > nz || !row_in) return make_float2(0.f, 0.f);
        return load_pair(b, a, j, k, nx, ny, nz, sy, sz);
    };

    // register window at the start of step t: E[0..5] = planes t-2 .. t+3
    float2 Em2 = make_float2(0.f, 0.f);
    float2 Em1 = LE(k0 - 2), E0 = LE(k0 - 1), Ep1 = LE(k0), Ep2 = LE(k0 + 1), Ep3;
    float2 Op1 = LO(k0), Op2 = LO(k0 + 1), Op3;
    float2 Bm1 = make_float2(0.f, 0.f), B0 = LB(k0 - 1), Bp1 = LB(k0), Bp2 = LB(k0 + 1), Bp3;
    // plane k0-1 in the shared ring
    {
        const float2 o0 = LO(k0 - 1);
        *reinterpret_cast<float2 *>(&S.s[(k0 - 1) & 3][r][2 * lane]) = E0;
        if (has_outer) *reinterpret_cast<float2 *>(&S.s[(k0 - 1) & 3][ro][2 * lane]) = o0;
    }
    __syncthreads();

    for (int t = k0 - 1; t <= k1 + 1; ++t) {
        Ep3 = LE(t + 3);
        Op3 = LO(t + 3);
        Bp3 = LB(t + 3);
        float(*St)[RB_SW] = S.s[t & 3];

        // ---- A: first colour on plane t (tile and ring) --------------------------------
        {
            const int q = (j + t) & 1;                       // first-colour cell of the pair
            const float up = __shfl_up_sync(0xffffffffu, E0.y, 1);
            const float dn = __shfl_down_sync(0xffffffffu, E0.x, 1);
            const int i = a + q;
            const bool need = (lane >= 1 && lane <= 30) || (lane == 0 && q == 1) || (lane == 31 && q == 0);
            if (need && row_in && i >= 1 && i <= nx && t >= 1 && t <= nz) {
                // only the second-colour words of the neighbouring rows are read (the
                // first-colour words of those rows are being written in this phase)
                const float yl = St[r - 1][2 * lane + q];
                const float yr = St[r + 1][2 * lane + q];
                const float left = q ? E0.x : up;
                const float right = q ? dn : E0.y;
                const float czm = L.czm[t], czp = L.czp[t];
                float s = cxm[q] * left;
                s = fmaf(cxp[q], right, s);
                s = fmaf(cym, yl, s);
                s = fmaf(cyp, yr, s);
                s = fmaf(czm, comp(Em1, q), s);
                s = fmaf(czp, comp(Ep1, q), s);
                const float c0 = -((dxc[q] + dy) + (czm + czp));
                const float v = fmaf(omw, comp(E0, q), __fdividef(omega * (comp(B0, q) - s), c0));
                setc(E0, q, v);
                St[r][2 * lane + q] = v;
            }
            // the next plane's old values for the y-neighbours of step t+1
            float(*Sn)[RB_SW] = S.s[(t + 1) & 3];
            *reinterpret_cast<float2 *>(&Sn[r][2 * lane]) = Ep1;
            if (has_outer) *reinterpret_cast<float2 *>(&Sn[ro][2 * lane]) = Op1;
        }
        __syncthreads();

        // ---- C: second colour on plane t-1 (tile), store the final pair -----------------
        const int s1 = t - 1;
        {
            const int qb = 1 - ((j + s1) & 1);               // second-colour cell of the pair
            const float up = __shfl_up_sync(0xffffffffu, Em1.y, 1);
            const float dn = __shfl_down_sync(0xffffffffu, Em1.x, 1);
            if (s1 >= k0 && s1 <= k1 && tile_row && row_in && lane >= 1 && lane <= 30 && a <= nx) {
                const int i = a + qb;
                if (i <= nx) {
                    float(*Ss)[RB_SW] = S.s[s1 & 3];
                    const float2 yl = *reinterpret_cast<const float2 *>(&Ss[r - 1][2 * lane]);
                    const float2 yr = *reinterpret_cast<const float2 *>(&Ss[r + 1][2 * lane]);
                    const float left = qb ? Em1.x : up;
                    const float right = qb ? dn : Em1.y;
                    const float czm = L.czm[s1], czp = L.czp[s1];
                    float s = cxm[qb] * left;
                    s = fmaf(cxp[qb], right, s);
                    s = fmaf(cym, comp(yl, qb), s);
                    s = fmaf(cyp, comp(yr, qb), s);
                    s = fmaf(czm, comp(Em2, qb), s);
                    s = fmaf(czp, comp(E0, qb), s);
                    const float c0 = -((dxc[qb] + dy) + (czm + czp));
                    const float v = fmaf(omw, comp(Em1, qb), __fdividef(omega * (comp(Bm1, qb) - s), c0));
                    setc(Em1, qb, v);
                }
                float *g = eout + (long long)a + (long long)sy * j + sz * s1;
                if (a + 1 <= nx)
                    *reinterpret_cast<float2 *>(g) = Em1;
                else
                    g[0] = Em1.x;
            }
        }
        // rotate the register window
        Em2 = Em1;
        Em1 = E0;
        E0 = Ep1;
        Ep1 = Ep2;
        Ep2 = Ep3;
        Op1 = Op2;
        Op2 = Op3;
        Bm1 = B0;
        B0 = Bp1;
        Bp1 = Bp2;
        Bp2 = Bp3;
    }
    __syncthreads();
}

}  // namespace pmg
