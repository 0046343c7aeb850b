// pmg_smooth32_tma.cuh -- device code of the TMA-fed fused FP32 red-black iteration.
//
// Same arithmetic and thread mapping as pmg_smooth32.cuh (one RBGS iteration of
// src/rbgs_poisson_matrix.f90:235-273, out of place, on (TX = 60) x TY tiles over chunks
// of planes; warp w owns row j0 - 1 + w, lane l the cell pair (i0 - 2 + 2l, i0 - 1 + 2l)),
// but the planes reach shared memory through the tensor-memory accelerator instead of
// per-thread loads:
//
//  * A ring of NS stages; stage s holds one plane of e_in (rows j0-2 .. j0+TY+1, 64
//    columns from i0-2) and of b (rows j0-1 .. j0+TY).  One thread issues both copies of
//    a plane with cp.async.bulk.tensor and an mbarrier counts their bytes; every thread
//    waits on the mbarrier (bounded by a clock limit) before it reads the plane.
//  * The planes of all the work items of a CTA form one stream of slots, so the copies of
//    the next item's first planes are in flight while the current item finishes.
//  * Step t: first colour on plane t, written back into its stage (the y-neighbours of
//    the second colour), barrier, then the stage of plane t-2 is refilled NS slots ahead
//    and the second colour on plane t-1 is computed and stored to e_out.
//  * Each thread keeps its pair of planes t-2 .. t+1 and b of planes t-1, t in registers
//    (z-neighbours), takes x-neighbours by shuffles and y-neighbours from the stage.
//
// DRAM traffic per iteration: e_in and b read once, e_out written once (12 B per cell,
// 8 B when e_in = 0: then no e_in copies are issued at all).
#pragma once

#include <cuda.h>

#include "pmg_common.cuh"

namespace pmg {

constexpr int RBT_TX = 60;       // tile columns (same as the register-window kernel)
constexpr int RBT_W = 64;        // stage row width in floats
constexpr int RBT_NS = 8;        // stages
constexpr int RBT_DATA_OFF = 5;  // floats from the start of a padded row to cell i = 0

template <int TY>
struct RbtShape {
    static constexpr int EROWS = TY + 4, BROWS = TY + 2;
    static constexpr int EBYTES = EROWS * RBT_W * 4, BBYTES = BROWS * RBT_W * 4;
    static constexpr int STAGE = EBYTES + BBYTES;
    static constexpr int SMEM = RBT_NS * STAGE + RBT_NS * 8 + 128;   // stages, mbarriers, alignment slack
    static constexpr int THREADS = (TY + 2) * 32;
};

namespace rbtdetail {

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the given phase parity; gives up after about one second of clock cycles.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > (1LL << 31)) return false;
    return true;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, unsigned long long *bar, int x, int y,
                                            int z)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

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

}  // namespace rbtdetail

// Work item geometry: item it -> tile (bx, by) and planes k0..k1.
struct RbtItems {
    int ntx, nty, kchunk, nz, nitems;
    __device__ __forceinline__ void decode(int it, int &bx, int &by, int &k0, int &k1) const
    {
        const int per = ntx * nty;
        const int bz = it / per, rem = it - bz * per;
        by = rem / ntx;
        bx = rem - by * ntx;
        k0 = 1 + kchunk * bz;
        k1 = min(nz, k0 + kchunk - 1);
    }
};

// The producer: one thread issuing the planes of the CTA's items, slot after slot.
template <int TY, bool ZERO_IN>
struct RbtProducer {
    int it, q, k0, k1, bx, by;   // item being issued and its next plane q
    int slot;                    // next slot to issue
    __device__ __forceinline__ void start(const RbtItems &W)
    {
        it = blockIdx.x;
        slot = 0;
        if (it < W.nitems) {
            W.decode(it, bx, by, k0, k1);
            q = k0 - 2;
        }
    }
    // issue every slot up to and including `limit`
    __device__ __forceinline__ void issue_upto(int limit, const RbtItems &W, unsigned char *smem,
                                               unsigned long long *bars, const CUtensorMap *me,
                                               const CUtensorMap *mb)
    {
        using S = RbtShape<TY>;
        while (slot <= limit && it < W.nitems) {
            const int s = slot % RBT_NS;
            unsigned char *st = smem + s * S::STAGE;
            const bool with_b = q >= k0 - 1 && q <= k1 + 1;
            const unsigned bytes = (ZERO_IN ? 0u : (unsigned)S::EBYTES) + (with_b ? (unsigned)S::BBYTES : 0u);
            const int x = RBT_DATA_OFF + RBT_TX * bx - 1;      // column of cell i0 - 2
            if (bytes) {
                rbtdetail::mbar_expect_tx(&bars[s], bytes);
                if (!ZERO_IN) rbtdetail::tma_load_3d(st, me, &bars[s], x, TY * by, q + 1);
                if (with_b) rbtdetail::tma_load_3d(st + S::EBYTES, mb, &bars[s], x, TY * by + 1, q + 1);
            } else {
                rbtdetail::mbar_arrive(&bars[s]);
            }
            ++slot;
            if (++q > k1 + 2) {
                it += gridDim.x;
                if (it < W.nitems) {
                    W.decode(it, bx, by, k0, k1);
                    q = k0 - 2;
                }
            }
        }
    }
};

template <int TY, bool ZERO_IN, bool OMEGA1>
struct RbtItem {
    using S = RbtShape<TY>;
    static_assert((RBT_NS & (RBT_NS - 1)) == 0, "stage count must be a power of two");
    unsigned char *smem;
    unsigned long long *bars;
    const float *czm_t, *czp_t;
    int nz, k0, k1, lane, w, r, cbase;
    bool need0, need1, store_lane, st_full;
    float *pw;
    long long sz;
    float omega, omw;
    float dxy[2], cxm[2], cxp[2], cym, cyp;   // dxy = x-part + y-part of -c0
    float2 E[4], B[2];
    float czm_n, czp_n;     // z coefficients of the next plane (prefetched)
    bool fail;

    __device__ __forceinline__ float *stage_e(int slot) const
    {
        return reinterpret_cast<float *>(smem + (unsigned)(slot & (RBT_NS - 1)) * (unsigned)S::STAGE);
    }
    __device__ __forceinline__ void wait(int slot)
    {
        if (!rbtdetail::mbar_wait_bounded(&bars[slot & (RBT_NS - 1)], (unsigned)(slot / RBT_NS) & 1u)) fail = true;
    }
    __device__ __forceinline__ float2 own_e(const float *st) const
    {
        if (ZERO_IN) return make_float2(0.f, 0.f);
        return *reinterpret_cast<const float2 *>(st + r * RBT_W + 2 * lane);
    }
    __device__ __forceinline__ float2 own_b(const float *st) const
    {
        return *reinterpret_cast<const float2 *>(st + S::EBYTES / 4 + w * RBT_W + 2 * lane);
    }
    __device__ __forceinline__ float upd(float old, float bb, float s, float c0) const
    {
        if (OMEGA1) return __fdividef(bb - s, c0);
        return fmaf(omw, old, __fdividef(omega * (bb - s), c0));
    }
    // z coefficients of plane k; CHECKED clamps k to the table (entries 0 and nz+1 are 0)
    template <bool CHECKED>
    __device__ __forceinline__ void load_cz(int k)
    {
        if (CHECKED) k = min(k, nz + 1);
        czm_n = __ldg(czm_t + k);
        czp_n = __ldg(czp_t + k);
    }

    // Step t: first colour on plane t, second colour on plane t-1.  P = window position of
    // plane t-2; Q = index within the pair of the first-colour cell on plane t.  CHECKED
    // steps test at run time whether plane t is a grid plane (first colour) and whether
    // plane t-1 belongs to the item (second colour); the steps in between, k0 < t <= k1,
    // need neither test.  Returns false when a wait gave up (uniform across the CTA).
    template <int P, int Q, bool CHECKED>
    __device__ __forceinline__ bool step(int t, float (&cz)[6], RbtProducer<TY, ZERO_IN> &prod, const RbtItems &W,
                                         const CUtensorMap *me, const CUtensorMap *mb)
    {
        using namespace rbtdetail;
        constexpr int im2 = P % 4, im1 = (P + 1) % 4, i00 = (P + 2) % 4, ip1 = (P + 3) % 4;
        constexpr int bm1 = P % 2, b00 = (P + 1) % 2;
        const int cs = cbase + (t - k0 + 2);      // slot of plane t
        float *St = stage_e(cs);
        wait(cs + 1);
        E[ip1] = own_e(stage_e(cs + 1));
        B[b00] = own_b(St);
        // z coefficients (czm, czp, czm + czp) of plane t-1 in cz[0..2] and of plane t in
        // cz[3..5]; plane t+1 is prefetched
        cz[0] = cz[3];
        cz[1] = cz[4];
        cz[2] = cz[5];
        cz[3] = czm_n;
        cz[4] = czp_n;
        cz[5] = czm_n + czp_n;
        load_cz<CHECKED>(t + 1);
        {
            const float up = __shfl_up_sync(0xffffffffu, E[i00].y, 1);
            const float dn = __shfl_down_sync(0xffffffffu, E[i00].x, 1);
            if ((Q ? need1 : need0) && (!CHECKED || (t >= 1 && t <= nz))) {
                const float yl = ZERO_IN ? 0.f : St[(r - 1) * RBT_W + 2 * lane + Q];
                const float yr = ZERO_IN ? 0.f : St[(r + 1) * RBT_W + 2 * lane + Q];
                const float left = Q ? E[i00].x : up;
                const float right = Q ? dn : E[i00].y;
                float s = cxm[Q] * left;
                s = fmaf(cxp[Q], right, s);
                s = fmaf(cym, yl, s);
                s = fmaf(cyp, yr, s);
                s = fmaf(cz[3], cq<Q>(E[im1]), s);
                s = fmaf(cz[4], cq<Q>(E[ip1]), s);
                const float c0 = -(dxy[Q] + cz[5]);
                const float v = upd(cq<Q>(E[i00]), cq<Q>(B[b00]), s, c0);
                sq<Q>(E[i00], v);
            }
            // the whole pair: with e_in = 0 the stage holds no copied plane, and cells that
            // are not updated (ghosts, cells beyond the grid) must read as zero there
            *reinterpret_cast<float2 *>(St + r * RBT_W + 2 * lane) = E[i00];
        }
        fence_proxy_async();
        if (__syncthreads_or(fail)) return false;
        if (threadIdx.x == 0) prod.issue_upto(cs - 2 + RBT_NS, W, smem, bars, me, mb);
        {
            const int s1 = t - 1;
            const float up = __shfl_up_sync(0xffffffffu, E[im1].y, 1);
            const float dn = __shfl_down_sync(0xffffffffu, E[im1].x, 1);
            if (store_lane && (!CHECKED || (s1 >= k0 && s1 <= k1))) {
                if (Q == 0 || st_full) {
                    const float *Ss = stage_e(cs - 1);
                    const float yl = Ss[(r - 1) * RBT_W + 2 * lane + Q];
                    const float yr = Ss[(r + 1) * RBT_W + 2 * lane + Q];
                    const float left = Q ? E[im1].x : up;
                    const float right = Q ? dn : E[im1].y;
                    float s = cxm[Q] * left;
                    s = fmaf(cxp[Q], right, s);
                    s = fmaf(cym, yl, s);
                    s = fmaf(cyp, yr, s);
                    s = fmaf(cz[0], cq<Q>(E[im2]), s);
                    s = fmaf(cz[1], cq<Q>(E[i00]), s);
                    const float c0 = -(dxy[Q] + cz[2]);
                    const float v = upd(cq<Q>(E[im1]), cq<Q>(B[bm1]), s, c0);
                    sq<Q>(E[im1], v);
                }
                float *g = pw + sz * s1;
                if (st_full)
                    *reinterpret_cast<float2 *>(g) = E[im1];
                else
                    g[0] = E[im1].x;
            }
        }
        return true;
    }

    // Steps t = k0-1 .. k1+1: two checked steps, unchecked steps k0+1 .. k1 unrolled by
    // the four-plane register window, then the remaining steps checked.
    template <int Q0>
    __device__ __forceinline__ bool run(RbtProducer<TY, ZERO_IN> &prod, const RbtItems &W, const CUtensorMap *me,
                                        const CUtensorMap *mb)
    {
        float cz[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        load_cz<true>(k0 - 1);
        int t = k0 - 1;
        if (!step<0, Q0, true>(t, cz, prod, W, me, mb)) return false;
        if (!step<1, 1 - Q0, true>(t + 1, cz, prod, W, me, mb)) return false;
        t += 2;
        for (; t + 3 <= k1; t += 4) {
            if (!step<2, Q0, false>(t, cz, prod, W, me, mb)) return false;
            if (!step<3, 1 - Q0, false>(t + 1, cz, prod, W, me, mb)) return false;
            if (!step<0, Q0, false>(t + 2, cz, prod, W, me, mb)) return false;
            if (!step<1, 1 - Q0, false>(t + 3, cz, prod, W, me, mb)) return false;
        }
        if (t <= k1 + 1 && !step<2, Q0, true>(t++, cz, prod, W, me, mb)) return false;
        if (t <= k1 + 1 && !step<3, 1 - Q0, true>(t++, cz, prod, W, me, mb)) return false;
        if (t <= k1 + 1 && !step<0, Q0, true>(t++, cz, prod, W, me, mb)) return false;
        if (t <= k1 + 1 && !step<1, 1 - Q0, true>(t++, cz, prod, W, me, mb)) return false;
        return true;
    }
};

// One work item.  cbase = slot of plane k0 - 2.  Returns false when a wait gave up.
template <int TY, bool ZERO_IN, bool OMEGA1>
__device__ __forceinline__ bool rbt_item(unsigned char *smem, unsigned long long *bars, const LevelK<float> &L,
                                         float *__restrict__ eout, float omega, float omw, int bx, int by, int k0,
                                         int k1, int cbase, RbtProducer<TY, ZERO_IN> &prod, const RbtItems &W,
                                         const CUtensorMap *me, const CUtensorMap *mb)
{
    RbtItem<TY, ZERO_IN, OMEGA1> I;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i0 = 1 + RBT_TX * bx, j0 = 1 + TY * by;
    const int nx = L.nx, ny = L.ny;
    const int a = i0 - 2 + 2 * lane;
    const int j = j0 - 1 + w;
    I.smem = smem;
    I.bars = bars;
    I.czm_t = L.czm;
    I.czp_t = L.czp;
    I.nz = L.nz;
    I.k0 = k0;
    I.k1 = k1;
    I.lane = lane;
    I.w = w;
    I.r = w + 1;
    I.cbase = cbase;
    I.sz = L.sz;
    I.omega = omega;
    I.omw = omw;
    I.fail = false;
    const bool row_in = j >= 1 && j <= ny;
    const bool in0 = a >= 1 && a <= nx, in1 = a + 1 >= 1 && a + 1 <= nx;
    const bool mid = lane >= 1 && lane <= 30;
    I.need0 = row_in && in0 && (mid || lane == 31);
    I.need1 = row_in && in1 && (mid || lane == 0);
    I.store_lane = (w >= 1 && w <= TY) && row_in && mid && a <= nx;
    I.st_full = a + 1 <= nx;
    I.pw = eout + (long long)a + (long long)L.sy * j;
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
    // window at the first step t = k0 - 1: positions 0..3 = planes k0-3 .. k0; position 0
    // (plane k0-3) is never read, position 3 is loaded by the step itself
    I.E[0] = make_float2(0.f, 0.f);
    I.wait(cbase);
    I.E[1] = I.own_e(I.stage_e(cbase));
    I.wait(cbase + 1);
    I.E[2] = I.own_e(I.stage_e(cbase + 1));
    I.B[0] = make_float2(0.f, 0.f);
    // the pair's first cell a is odd, so it carries the first colour on plane k when j + k
    // is even ((i + j + k) odd, src/rbgs_poisson_matrix.f90:242)
    if (((j + k0 - 1) & 1) == 0) return I.template run<0>(prod, W, me, mb);
    return I.template run<1>(prod, W, me, mb);
}

}  // namespace pmg
