// pmg_smooth32_tma.cuh -- device code of the TMA-fed fused FP32 red-black iteration.
//
// Same arithmetic as pmg_smooth32.cuh (one RBGS iteration of
// src/rbgs_poisson_matrix.f90:235-273, out of place, on (TX = 60) x TY tiles over chunks
// of planes; lane l owns the cell pair (i0 - 2 + 2l, i0 - 1 + 2l)), but warp w owns TWO
// rows, j0 - 1 + 2w and j0 + 2w (so the y-neighbour between them stays in registers and
// the per-plane overhead is shared by two rows), and the planes reach shared memory
// through the tensor-memory accelerator instead of per-thread loads:
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
//  * Each thread keeps its two pairs of planes t-2 .. t+1 and b of planes t-1, t in
//    registers (z-neighbours), takes x-neighbours by shuffles and the outer y-neighbours
//    from the stage.
//  * A wait that runs out (about a second) sets a shared abort flag, after which every
//    wait of the CTA returns at once; the CTA stops at the end of the item, thread 0
//    waits (bounded, about a second each) for the copies it issued to land, and the host
//    reads the error flag.  A self-test mode ("stall": the item source says so) issues
//    no copies at all and gives each wait a limit of a few microseconds, so the waits
//    run out with nothing in flight and that path can be tested on the GPU.
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
    // stages, mbarriers, abort flag and producer state, alignment slack
    static constexpr int SMEM = RBT_NS * STAGE + RBT_NS * 8 + 64 + 128;
    static constexpr int WARPS = (TY + 2) / 2;                               // two rows per warp
    static constexpr int THREADS = WARPS * 32;
    static_assert(TY % 2 == 0, "tile height must be even");
};

template <int TY>
__host__ __device__ constexpr int S_EB() { return RbtShape<TY>::EBYTES; }

// CTAs per SM the TMA-fed kernels' register budget is sized for
template <int TY>
constexpr int rbt_min_ctas() { return TY <= 6 ? 5 : TY <= 14 ? 3 : 2; }

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

// Wait limits in clock cycles: about a second in production, a few microseconds in the
// stall self-test (no copies are in flight there).
constexpr long long kWaitCycles = 1LL << 31;
constexpr long long kStallWaitCycles = 1LL << 13;

// Slow path of a wait: spins until the phase completes, LIMIT clock cycles pass (then it
// raises the CTA's abort flag) or another thread has raised the flag.  Returns false on
// failure.  The limit is a template constant: a limit read at run time costs the
// production kernels' sweep loop registers (spills) around this call.
template <long long LIMIT>
static __device__ __noinline__ bool mbar_wait_slow(unsigned long long *bar, unsigned parity, volatile int *abort_flag)
{
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > LIMIT) {
            *abort_flag = 1;
            return false;
        }
    }
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

// Work item geometry of one level: item it -> tile (bx, by) and planes k0..k1.
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

// A source of work items for the TMA-fed smoother: the CTA's items in order (first /
// next / valid), each item's tile and planes (geom) and the tensor maps of its e_in and b
// (map_e / map_b).  RbtGridSrc serves one level; the batched solver has its own source
// over (problem, tile) lists.  STALL (a separate instantiation, so the production kernels
// carry no trace of it): the self-test source, which issues no copies and gives every wait
// a limit of a few microseconds.
template <bool STALL>
struct RbtGridSrc {
    const RbtItems *W;            // the kernel parameter (read from the constant bank)
    const CUtensorMap *me, *mb;
    __device__ __forceinline__ int first() const { return blockIdx.x; }
    __device__ __forceinline__ int next(int it) const { return it + gridDim.x; }
    __device__ __forceinline__ bool valid(int it) const { return it < W->nitems; }
    __device__ __forceinline__ void geom(int it, int &bx, int &by, int &k0, int &k1) const
    {
        W->decode(it, bx, by, k0, k1);
    }
    __device__ __forceinline__ const CUtensorMap *map_e(int) const { return me; }
    __device__ __forceinline__ const CUtensorMap *map_b(int) const { return mb; }
    static constexpr bool kStall = STALL;
    __device__ __forceinline__ constexpr bool stall() const { return STALL; }
};

// The producer: one thread issuing the planes of the CTA's items, slot after slot.  Its
// state lives in shared memory (only thread 0 touches it), so it costs the other
// threads no registers.
template <int TY, bool ZERO_IN, class Src>
struct RbtProducer {
    int it, q, k0, k1, bx, by;   // item being issued and its next plane q
    int slot;                    // next slot to issue
    const CUtensorMap *me, *mb;  // tensor maps of the item being issued
    __device__ __forceinline__ void load_item(const Src &src)
    {
        if (src.valid(it)) {
            src.geom(it, bx, by, k0, k1);
            q = k0 - 2;
            me = src.map_e(it);
            mb = src.map_b(it);
        }
    }
    __device__ __forceinline__ void start(const Src &src)
    {
        it = src.first();
        slot = 0;
        load_item(src);
    }
    // issue every slot up to and including `limit`
    __device__ __forceinline__ void issue_upto(int limit, const Src &src, unsigned char *smem, unsigned long long *bars)
    {
        using S = RbtShape<TY>;
        if (src.stall()) return;   // self-test: nothing is issued, every wait runs out
        while (slot <= limit && src.valid(it)) {
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
                it = src.next(it);
                load_item(src);
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
    volatile int *abort_flag;
    const float *czm_t, *czp_t;
    int nz, k0, k1, cbase;
    int oe, ob;                        // byte offsets in a stage of row a's own e pair and b pair
    bool nA[2], nB[2];                 // rows a / b: cell 0 / 1 of the pair takes a first-colour update
    bool stA, stB, st_full;            // rows a / b are stored; the pair is stored whole
    float *pwA;                        // e_out at row a, plane 0 (row b at + sy)
    int sy;
    long long sz;
    float omega, omw;
    float cxm[2], cxp[2];
    float dA[2], dB[2];                // x-part + y-part of -c0, rows a and b
    float cymA, cypA, cymB, cypB;
    float2 EA[4], EB[4], BA[2], BB[2];
    float czm_n, czp_n;                // z coefficients of the next plane (prefetched)
    bool fail;

    __device__ __forceinline__ unsigned stage_off(int slot) const
    {
        return (unsigned)(slot & (RBT_NS - 1)) * (unsigned)S::STAGE;
    }
    template <bool STALL>
    __device__ __forceinline__ void wait(int slot)
    {
        unsigned long long *bar = &bars[slot & (RBT_NS - 1)];
        const unsigned par = (unsigned)(slot / RBT_NS) & 1u;
        constexpr long long lim = STALL ? rbtdetail::kStallWaitCycles : rbtdetail::kWaitCycles;
        if (!rbtdetail::mbar_try_wait(bar, par) && !rbtdetail::mbar_wait_slow<lim>(bar, par, abort_flag)) fail = true;
    }
    __device__ __forceinline__ float2 lds2(unsigned off) const
    {
        return *reinterpret_cast<const float2 *>(smem + off);
    }
    __device__ __forceinline__ float lds(unsigned off) const { return *reinterpret_cast<const float *>(smem + off); }
    __device__ __forceinline__ void sts2(unsigned off, float2 v) const
    {
        *reinterpret_cast<float2 *>(smem + off) = v;
    }
    // first- or second-colour update of one cell: s = off-diagonal sum, d = -c0
    __device__ __forceinline__ float upd(float old, float bb, float s, float d) const
    {
        if (OMEGA1) return __fdividef(s - bb, d);
        return fmaf(omw, old, __fdividef(omega * (s - bb), d));
    }
    template <bool CHECKED>
    __device__ __forceinline__ void load_cz(int k)
    {
        if (CHECKED) k = min(k, nz + 1);   // table entries 0 and nz+1 are 0
        czm_n = __ldg(czm_t + k);
        czp_n = __ldg(czp_t + k);
    }

    // Step t: first colour on plane t, second colour on plane t-1, for both rows.  P =
    // window position of plane t-2; Q = index within the pair of row a's first-colour
    // cell on plane t (row b's is 1 - Q; on plane t-1 the second-colour cells are at the
    // same indices).  CHECKED steps test at run time whether plane t is a grid plane
    // and whether plane t-1 belongs to the item; the steps k0 < t <= k1 need neither.
    template <int P, int Q, bool CHECKED, class Src>
    __device__ __forceinline__ void step(int t, float (&cz)[6], RbtProducer<TY, ZERO_IN, Src> *prod, const Src &src)
    {
        using namespace rbtdetail;
        constexpr int im2 = P % 4, im1 = (P + 1) % 4, i00 = (P + 2) % 4, ip1 = (P + 3) % 4;
        constexpr int bm1 = P % 2, b00 = (P + 1) % 2;
        constexpr int QB = 1 - Q;
        const int cs = cbase + (t - k0 + 2);      // slot of plane t
        const unsigned s0 = stage_off(cs), sp = stage_off(cs + 1), sm = stage_off(cs - 1);
        wait<Src::kStall>(cs + 1);
        if (!ZERO_IN) {
            EA[ip1] = lds2(sp + oe);
            EB[ip1] = lds2(sp + oe + RBT_W * 4);
        }
        BA[b00] = lds2(s0 + ob);
        BB[b00] = lds2(s0 + ob + RBT_W * 4);
        // z coefficients (czm, czp, czm + czp) of plane t-1 in cz[0..2], of plane t in
        // cz[3..5]; plane t+1 is prefetched
        cz[0] = cz[3];
        cz[1] = cz[4];
        cz[2] = cz[5];
        cz[3] = czm_n;
        cz[4] = czp_n;
        cz[5] = czm_n + czp_n;
        load_cz<CHECKED>(t + 1);
        const bool plane_in = !CHECKED || (t >= 1 && t <= nz);
        if (ZERO_IN) {
            // every neighbour of a first-colour cell still holds the zero input
            const float vA = nA[Q] && plane_in ? upd(0.f, cq<Q>(BA[b00]), 0.f, dA[Q] + cz[5]) : 0.f;
            const float vB = nB[QB] && plane_in ? upd(0.f, cq<QB>(BB[b00]), 0.f, dB[QB] + cz[5]) : 0.f;
            EA[i00] = Q ? make_float2(0.f, vA) : make_float2(vA, 0.f);
            EB[i00] = QB ? make_float2(0.f, vB) : make_float2(vB, 0.f);
            sts2(s0 + oe, EA[i00]);
            sts2(s0 + oe + RBT_W * 4, EB[i00]);
        } else {
            const float upA = __shfl_up_sync(0xffffffffu, EA[i00].y, 1);
            const float dnA = __shfl_down_sync(0xffffffffu, EA[i00].x, 1);
            const float upB = __shfl_up_sync(0xffffffffu, EB[i00].y, 1);
            const float dnB = __shfl_down_sync(0xffffffffu, EB[i00].x, 1);
            // row a, cell Q: y-neighbours = the stage row below and row b (old values)
            const float yA = ZERO_IN ? 0.f : lds(s0 + oe - RBT_W * 4 + 4 * Q);
            const float yB = ZERO_IN ? 0.f : lds(s0 + oe + 2 * RBT_W * 4 + 4 * QB);
            float vA = 0.f, vB = 0.f;
            if (nA[Q] && plane_in) {
                float s = cxm[Q] * (Q ? EA[i00].x : upA);
                s = fmaf(cxp[Q], Q ? dnA : EA[i00].y, s);
                s = fmaf(cymA, yA, s);
                s = fmaf(cypA, cq<Q>(EB[i00]), s);
                s = fmaf(cz[3], cq<Q>(EA[im1]), s);
                s = fmaf(cz[4], cq<Q>(EA[ip1]), s);
                vA = upd(cq<Q>(EA[i00]), cq<Q>(BA[b00]), s, dA[Q] + cz[5]);
            }
            if (nB[QB] && plane_in) {
                float s = cxm[QB] * (QB ? EB[i00].x : upB);
                s = fmaf(cxp[QB], QB ? dnB : EB[i00].y, s);
                s = fmaf(cymB, cq<QB>(EA[i00]), s);
                s = fmaf(cypB, yB, s);
                s = fmaf(cz[3], cq<QB>(EB[im1]), s);
                s = fmaf(cz[4], cq<QB>(EB[ip1]), s);
                vB = upd(cq<QB>(EB[i00]), cq<QB>(BB[b00]), s, dB[QB] + cz[5]);
            }
            if (nA[Q] && plane_in) sq<Q>(EA[i00], vA);
            if (nB[QB] && plane_in) sq<QB>(EB[i00], vB);
            // whole pairs: with e_in = 0 the stage holds no copied plane, and cells that are
            // not updated (ghosts, cells beyond the grid) must read as zero there
            sts2(s0 + oe, EA[i00]);
            sts2(s0 + oe + RBT_W * 4, EB[i00]);
        }
        fence_proxy_async();
        __syncthreads();
        if (threadIdx.x == 0) prod->issue_upto(cs - 2 + RBT_NS, src, smem, bars);
        if (!CHECKED || (t - 1 >= k0 && t - 1 <= k1)) {
            const float upA = __shfl_up_sync(0xffffffffu, EA[im1].y, 1);
            const float dnA = __shfl_down_sync(0xffffffffu, EA[im1].x, 1);
            const float upB = __shfl_up_sync(0xffffffffu, EB[im1].y, 1);
            const float dnB = __shfl_down_sync(0xffffffffu, EB[im1].x, 1);
            // row a, cell Q: y-neighbours = the stage row below (first colour, plane t-1)
            // and row b's updated first-colour cell; row b, cell 1-Q: row a and the row above
            const float yA = lds(sm + oe - RBT_W * 4 + 4 * Q);
            const float yB = lds(sm + oe + 2 * RBT_W * 4 + 4 * QB);
            float *gA = pwA + sz * (t - 1);
            if (stA && (Q == 0 || st_full)) {
                float s = cxm[Q] * (Q ? EA[im1].x : upA);
                s = fmaf(cxp[Q], Q ? dnA : EA[im1].y, s);
                s = fmaf(cymA, yA, s);
                s = fmaf(cypA, cq<Q>(EB[im1]), s);
                s = fmaf(cz[0], cq<Q>(EA[im2]), s);
                s = fmaf(cz[1], cq<Q>(EA[i00]), s);
                const float v = upd(cq<Q>(EA[im1]), cq<Q>(BA[bm1]), s, dA[Q] + cz[2]);
                sq<Q>(EA[im1], v);
            }
            if (stB && (QB == 0 || st_full)) {
                float s = cxm[QB] * (QB ? EB[im1].x : upB);
                s = fmaf(cxp[QB], QB ? dnB : EB[im1].y, s);
                s = fmaf(cymB, cq<QB>(EA[im1]), s);
                s = fmaf(cypB, yB, s);
                s = fmaf(cz[0], cq<QB>(EB[im2]), s);
                s = fmaf(cz[1], cq<QB>(EB[i00]), s);
                const float v = upd(cq<QB>(EB[im1]), cq<QB>(BB[bm1]), s, dB[QB] + cz[2]);
                sq<QB>(EB[im1], v);
            }
            if (stA) {
                if (st_full)
                    *reinterpret_cast<float2 *>(gA) = EA[im1];
                else
                    gA[0] = EA[im1].x;
            }
            if (stB) {
                if (st_full)
                    *reinterpret_cast<float2 *>(gA + sy) = EB[im1];
                else
                    gA[sy] = EB[im1].x;
            }
        }
    }

    // Steps t = k0-1 .. k1+1: two checked steps, unchecked steps k0+1 .. k1 unrolled by
    // the four-plane register window, then the remaining steps checked.
    template <int Q0, class Src>
    __device__ __forceinline__ void run(RbtProducer<TY, ZERO_IN, Src> *prod, const Src &src)
    {
        float cz[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        load_cz<true>(k0 - 1);
        int t = k0 - 1;
        step<0, Q0, true>(t, cz, prod, src);
        step<1, 1 - Q0, true>(t + 1, cz, prod, src);
        t += 2;
        for (; t + 3 <= k1; t += 4) {
            step<2, Q0, false>(t, cz, prod, src);
            step<3, 1 - Q0, false>(t + 1, cz, prod, src);
            step<0, Q0, false>(t + 2, cz, prod, src);
            step<1, 1 - Q0, false>(t + 3, cz, prod, src);
        }
        if (t <= k1 + 1) step<2, Q0, true>(t++, cz, prod, src);
        if (t <= k1 + 1) step<3, 1 - Q0, true>(t++, cz, prod, src);
        if (t <= k1 + 1) step<0, Q0, true>(t++, cz, prod, src);
        if (t <= k1 + 1) step<1, 1 - Q0, true>(t++, cz, prod, src);
    }
};

// One work item.  cbase = slot of plane k0 - 2.  Returns false (uniformly across the
// CTA) when a wait gave up.
template <int TY, bool ZERO_IN, bool OMEGA1, class Src>
__device__ __forceinline__ bool rbt_item(unsigned char *smem, unsigned long long *bars, volatile int *abort_flag,
                                         const LevelK<float> &L, float *__restrict__ eout, float omega, float omw,
                                         int bx, int by, int k0, int k1, int cbase, RbtProducer<TY, ZERO_IN, Src> *prod,
                                         const Src &src)
{
    RbtItem<TY, ZERO_IN, OMEGA1> I;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i0 = 1 + RBT_TX * bx, j0 = 1 + TY * by;
    const int nx = L.nx, ny = L.ny;
    const int a = i0 - 2 + 2 * lane;
    const int ja = j0 - 1 + 2 * w, jb = ja + 1;
    I.smem = smem;
    I.bars = bars;
    I.abort_flag = abort_flag;
    I.czm_t = L.czm;
    I.czp_t = L.czp;
    I.nz = L.nz;
    I.k0 = k0;
    I.k1 = k1;
    I.cbase = cbase;
    I.oe = ((2 * w + 1) * RBT_W + 2 * lane) * 4;
    I.ob = S_EB<TY>() + ((2 * w) * RBT_W + 2 * lane) * 4;
    I.sy = L.sy;
    I.sz = L.sz;
    I.omega = omega;
    I.omw = omw;
    I.fail = false;
    const bool inA = ja >= 1 && ja <= ny, inB = jb >= 1 && jb <= ny;
    const bool in0 = a >= 1 && a <= nx, in1 = a + 1 >= 1 && a + 1 <= nx;
    const bool mid = lane >= 1 && lane <= 30;
    // a lane updates the first-colour cell of its pair when it is interior and in the tile
    // or the ring cell beside it (lane 0: its second cell, lane 31: its first cell)
    const bool c0ok = in0 && (mid || lane == 31), c1ok = in1 && (mid || lane == 0);
    I.nA[0] = inA && c0ok;
    I.nA[1] = inA && c1ok;
    I.nB[0] = inB && c0ok;
    I.nB[1] = inB && c1ok;
    const bool col_store = mid && a <= nx;
    I.stA = col_store && inA && w >= 1;                          // row a of warp 0 is the ring row
    I.stB = col_store && inB && w <= RbtShape<TY>::WARPS - 2;               // row b of the last warp is the ring row
    I.st_full = a + 1 <= nx;
    I.pwA = eout + (long long)a + (long long)L.sy * ja;
    I.cymA = inA ? L.cym[ja] : 0.f;
    I.cypA = inA ? L.cyp[ja] : 0.f;
    I.cymB = inB ? L.cym[jb] : 0.f;
    I.cypB = inB ? L.cyp[jb] : 0.f;
    const float dyA = I.cymA + I.cypA, dyB = I.cymB + I.cypB;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int i = a + q;
        const bool in = i >= 1 && i <= nx;
        const float sx = in ? L.sx[i] : 0.f;
        I.dA[q] = sx + dyA;
        I.dB[q] = sx + dyB;
        I.cxm[q] = in ? L.cxm[i] : 0.f;
        I.cxp[q] = in ? L.cxp[i] : 0.f;
    }
    // window at the first step t = k0 - 1: positions 0..3 = planes k0-3 .. k0; position 0
    // (plane k0-3) is never read, position 3 is loaded by the step itself
    I.EA[0] = I.EB[0] = make_float2(0.f, 0.f);
    I.template wait<Src::kStall>(cbase);
    I.template wait<Src::kStall>(cbase + 1);
    if (ZERO_IN) {
        I.EA[1] = I.EB[1] = I.EA[2] = I.EB[2] = make_float2(0.f, 0.f);
    } else {
        const unsigned s1 = I.stage_off(cbase), s2 = I.stage_off(cbase + 1);
        I.EA[1] = I.lds2(s1 + I.oe);
        I.EB[1] = I.lds2(s1 + I.oe + RBT_W * 4);
        I.EA[2] = I.lds2(s2 + I.oe);
        I.EB[2] = I.lds2(s2 + I.oe + RBT_W * 4);
    }
    I.BA[0] = I.BB[0] = make_float2(0.f, 0.f);
    // the pair's first cell a is odd, so on row a it carries the first colour on plane k
    // when ja + k is even ((i + j + k) odd, src/rbgs_poisson_matrix.f90:242)
    if (((ja + k0 - 1) & 1) == 0)
        I.template run<0>(prod, src);
    else
        I.template run<1>(prod, src);
    return !__syncthreads_or(I.fail);
}

// One CTA of a TMA-fed launch over the items of `src`: shared-memory ring and mbarriers,
// the producer's first fills, then every item in order; per(it, L, eout) gives an item's
// level descriptor (a pointer) and output array.  When a wait gave up, thread 0 sets *err, lets the
// copies in flight land (bounded) and the CTA returns.
template <int TY, bool ZERO_IN, bool OMEGA1, class Src, class Per>
__device__ __forceinline__ void rbt_cta(const Src &src, Per per, float omega, float omw, int *err)
{
    using S = RbtShape<TY>;
    extern __shared__ unsigned char rbt_smem_raw[];
    // 128-byte aligned stages (TMA destinations), then the mbarriers, the abort flag and
    // the producer state
    unsigned char *smem = rbt_smem_raw + ((128u - (rbtdetail::smem_addr(rbt_smem_raw) & 127u)) & 127u);
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(smem + RBT_NS * S::STAGE);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(bars + RBT_NS);
    using Prod = RbtProducer<TY, ZERO_IN, Src>;
    static_assert(sizeof(Prod) <= 48, "producer state exceeds its shared-memory slot");
    Prod *prod = reinterpret_cast<Prod *>(bars + RBT_NS + 2);
    if (threadIdx.x == 0) {
        for (int q = 0; q < RBT_NS; ++q) rbtdetail::mbar_init(&bars[q], 1);
        *abort_flag = 0;
        rbtdetail::fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        prod->start(src);
        prod->issue_upto(RBT_NS - 1, src, smem, bars);
    }
    int cbase = 0;
    for (int it = src.first(); src.valid(it); it = src.next(it)) {
        int bx, by, k0, k1;
        src.geom(it, bx, by, k0, k1);
        const LevelK<float> *L;
        float *eout;
        per(it, L, eout);
        if (!rbt_item<TY, ZERO_IN, OMEGA1>(smem, bars, abort_flag, *L, eout, omega, omw, bx, by, k0, k1, cbase, prod,
                                            src)) {
            if (threadIdx.x == 0) {
                atomicOr(err, 1);
                for (int q = max(0, prod->slot - RBT_NS); q < prod->slot; ++q)
                    rbtdetail::mbar_wait_bounded(&bars[q % RBT_NS], (unsigned)(q / RBT_NS) & 1u);
            }
            return;
        }
        cbase += k1 - k0 + 5;
    }
}

}  // namespace pmg
