// pmg_smooth32.cu -- fused red-black iteration of the FP32 smoother.
//
// One launch performs one full RBGS iteration of src/rbgs_poisson_matrix.f90:235-273
// (first colour, then second colour) on a whole level, out of place:
//
//     e_out = RB(e_in)        (e_in = 0 for the first iteration from a zero start)
//
// so that every global value read is an old value and CTAs need no ordering.  Work is
// split into items = (TX x TY tile of (i, j)) x (chunk of k planes); a persistent grid
// of resident CTAs walks the items chunk-major.  For an item the CTA marches along k
// keeping a ring of planes in shared memory, filled two planes ahead by 4-byte cp.async
// copies: the first colour is updated on plane t over the tile plus a one-cell ring,
// then the second colour on plane t-1 over the tile, which then holds final values of
// both colours and is stored with coalesced 8-byte stores.  DRAM traffic per iteration
// is one read of e_in, one of b and one write of e_out: 12 B per cell (8 B from a zero
// start).
//
// Shared rows are split by column parity (even columns, then odd columns), so the
// stride-2 accesses of a colour are unit-stride and free of bank conflicts.
//
// FP32 layout (internal arrays of the mixed-precision V-cycle): element (i,j,k) at
// base[i + sy*j + sz*k]; columns -3 .. TX*ceil(nx/TX)+4 of every row are valid memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <map>
#include <mutex>

#include "../../include/peps_mg.h"
#include "pmg_internal.h"

namespace pmg {

namespace {

constexpr int TX = 64;                 // tile width (interior cells)
constexpr int RW = TX + 8;             // shared row: columns i0-4 .. i0+TX+3
constexpr int RH = RW / 2;             // one parity half of a row
constexpr int NE = 6;                  // e planes t-2 .. t+3
constexpr int NB = 4;                  // b planes t-1 .. t+2
constexpr int NT = 256;
constexpr int PR = TX / 2 + 2;         // pairs per ring row (columns i0-2 .. i0+TX+1)

template <int TY>
struct Smem {
    static constexpr int ER = TY + 4;  // e rows j0-2 .. j0+TY+1
    static constexpr int BR = TY + 2;  // b rows j0-1 .. j0+TY
    float e[NE][2][ER][RH];
    float b[NB][2][BR][RH];
    float dx[2][RH], cxm[2][RH], cxp[2][RH];
    float dy[ER], cym[ER], cyp[ER];
};

__device__ __forceinline__ void cp4(float *smem, const float *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_wait(int n)
{
    if (n <= 0)
        asm volatile("cp.async.wait_group 0;\n" ::);
    else if (n == 1)
        asm volatile("cp.async.wait_group 1;\n" ::);
    else
        asm volatile("cp.async.wait_group 2;\n" ::);
}

#define PMG_TRY_S(expr)                \
    do {                               \
        int _rc = (expr);              \
        if (_rc != PMG_OK) return _rc; \
    } while (0)

// value at shared column c (0..RW-1) of a split row
#define SC(arr, c) (arr)[(c)&1][(c) >> 1]

template <int TY, bool ZERO_IN>
__device__ void rb32_item(Smem<TY> &S, const LevelK<float> &L, const float *__restrict__ ein,
                          float *__restrict__ eout, const float *__restrict__ b, float omega, float omw, int bx,
                          int by, int k0, int k1)
{
    constexpr int ER = Smem<TY>::ER, BR = Smem<TY>::BR;
    const int tid = threadIdx.x;
    const int i0 = 1 + TX * bx, j0 = 1 + TY * by;
    const int nx = L.nx, ny = L.ny, nz = L.nz;
    const int sy = L.sy;
    const long long sz = L.sz;

    for (int c = tid; c < RW; c += NT) {
        const int i = i0 - 4 + c;
        const bool in = i >= 1 && i <= nx;
        SC(S.dx, c) = in ? L.sx[i] : 0.f;
        SC(S.cxm, c) = in ? L.cxm[i] : 0.f;
        SC(S.cxp, c) = in ? L.cxp[i] : 0.f;
    }
    for (int r = tid; r < ER; r += NT) {
        const int j = j0 - 2 + r;
        const bool in = j >= 1 && j <= ny;
        S.cym[r] = in ? L.cym[j] : 0.f;
        S.cyp[r] = in ? L.cyp[j] : 0.f;
        S.dy[r] = in ? L.cym[j] + L.cyp[j] : 0.f;
    }

    auto load_e = [&](int k) {
        if (ZERO_IN || k < 0 || k > nz + 1) return;
        const int slot = (k + NE) % NE;
        for (int q = tid; q < ER * RW; q += NT) {
            const int r = q / RW, c = q % RW;
            const int j = j0 - 2 + r;
            if (j < 0 || j > ny + 1) continue;
            cp4(&S.e[slot][c & 1][r][c >> 1], ein + (long long)(i0 - 4 + c) + (long long)sy * j + sz * k);
        }
    };
    auto load_b = [&](int k) {
        if (k < 1 || k > nz) return;
        const int slot = k % NB;
        for (int q = tid; q < BR * RW; q += NT) {
            const int r = q / RW, c = q % RW;
            const int j = j0 - 1 + r;
            if (j > ny + 1) continue;
            cp4(&S.b[slot][c & 1][r][c >> 1], b + (long long)(i0 - 4 + c) + (long long)sy * j + sz * k);
        }
    };

    load_e(k0 - 2);
    load_e(k0 - 1);
    load_e(k0);
    load_e(k0 + 1);
    load_b(k0 - 1);
    load_b(k0);
    cp_commit();

    for (int t = k0 - 1; t <= k1 + 1; ++t) {
        load_e(t + 3);
        load_b(t + 2);
        cp_commit();
        cp_wait(t == k0 - 1 ? 1 : 2);
        __syncthreads();

        // ---- first colour on plane t over the tile plus a one-cell ring -------------
        {
            auto &E = S.e[(t + NE) % NE];
            if (ZERO_IN && (t < 1 || t > nz)) {
                // a ghost plane of a zero start reads as zero
                for (int q = tid; q < PR * (TY + 2); q += NT) {
                    const int rr = q / PR, p = q % PR;
                    const int c = 2 + 2 * p;
                    E[0][rr + 1][c >> 1] = 0.f;
                    E[1][rr + 1][c >> 1] = 0.f;
                }
            } else if (t >= 1 && t <= nz) {
                const auto &Em = S.e[(t - 1 + NE) % NE];
                const auto &Ep = S.e[(t + 1) % NE];
                const auto &B = S.b[t % NB];
                const float czm = L.czm[t], czp = L.czp[t], dz = czm + czp;
                // rows of the ring: a warp takes 32 consecutive pairs of one row; the two
                // edge pairs of every row are spread over the remaining passes
                constexpr int MAIN = (TY + 2) * 32;
                constexpr int ITEMS = MAIN + (TY + 2) * 2;
                for (int q = tid; q < ITEMS; q += NT) {
                    int rr, p;
                    if (q < MAIN) {
                        rr = q >> 5;
                        p = 1 + (q & 31);
                    } else {
                        rr = (q - MAIN) >> 1;
                        p = ((q - MAIN) & 1) ? PR - 1 : 0;
                    }
                    const int re = rr + 1;
                    const int j = j0 - 1 + rr;
                    const int par = (j + t) & 1;                 // first-colour cell is ipair + par
                    const int ir = i0 - 2 + 2 * p + par;
                    const int c = 2 + 2 * p + par;               // shared column of ir
                    const int h = c & 1, x = c >> 1, o = h ^ 1;  // o: the other parity
                    const bool interior = ir >= 1 && ir <= nx && j >= 1 && j <= ny;
                    float v = 0.f;
                    if (interior) {
                        const float bb = B[h][rr][x];
                        const float c0 = -((S.dx[h][x] + S.dy[re]) + dz);
                        if (ZERO_IN) {
                            v = __fdividef(omega * bb, c0);
                        } else {
                            // columns c-1 and c+1 have the other parity: indices (c-1)>>1 and (c+1)>>1
                            float s = S.cxm[h][x] * E[o][re][(c - 1) >> 1];
                            s = fmaf(S.cxp[h][x], E[o][re][(c + 1) >> 1], s);
                            s = fmaf(S.cym[re], E[h][re - 1][x], s);
                            s = fmaf(S.cyp[re], E[h][re + 1][x], s);
                            s = fmaf(czm, Em[h][re][x], s);
                            s = fmaf(czp, Ep[h][re][x], s);
                            v = fmaf(omw, E[h][re][x], __fdividef(omega * (bb - s), c0));
                        }
                    }
                    if (ZERO_IN) {
                        E[h][re][x] = v;
                        // the second-colour cell of the pair reads as zero
                        const int cb = par ? c - 1 : c + 1;
                        E[cb & 1][re][cb >> 1] = 0.f;
                    } else if (interior) {
                        E[h][re][x] = v;
                    }
                }
            }
        }
        __syncthreads();

        // ---- second colour on plane s = t-1 over the tile; store both colours --------
        const int s = t - 1;
        if (s >= k0 && s <= k1) {
            auto &E = S.e[s % NE];
            const auto &Em = S.e[(s - 1 + NE) % NE];
            const auto &Ep = S.e[(s + 1) % NE];
            const auto &B = S.b[s % NB];
            const float czm = L.czm[s], czp = L.czp[s], dz = czm + czp;
            for (int q = tid; q < (TX / 2) * TY; q += NT) {
                const int rr = q >> 5, p = q & 31;           // one warp per tile row
                const int re = rr + 2, rb = rr + 1;
                const int j = j0 + rr;
                const int ipair = i0 + 2 * p;
                if (j > ny || ipair > nx) continue;
                const int odd = (j + s) & 1;                 // first-colour cell is ipair + odd
                const int cb = 4 + 2 * p + 1 - odd;          // shared column of the second-colour cell
                const int cr = 4 + 2 * p + odd;
                const int hb = cb & 1, xb = cb >> 1, ob = hb ^ 1;
                float vb = 0.f;
                if (ipair + 1 - odd <= nx) {
                    const float bb = B[hb][rb][xb];
                    const float c0 = -((S.dx[hb][xb] + S.dy[re]) + dz);
                    float sum = S.cxm[hb][xb] * E[ob][re][(cb - 1) >> 1];
                    sum = fmaf(S.cxp[hb][xb], E[ob][re][(cb + 1) >> 1], sum);
                    sum = fmaf(S.cym[re], E[hb][re - 1][xb], sum);
                    sum = fmaf(S.cyp[re], E[hb][re + 1][xb], sum);
                    sum = fmaf(czm, Em[hb][re][xb], sum);
                    sum = fmaf(czp, Ep[hb][re][xb], sum);
                    const float old = ZERO_IN ? 0.f : E[hb][re][xb];
                    vb = fmaf(omw, old, __fdividef(omega * (bb - sum), c0));
                }
                const float vr = E[cr & 1][re][cr >> 1];
                float *g = eout + (long long)ipair + (long long)sy * j + sz * s;
                if (ipair + 1 <= nx) {
                    float2 w;
                    w.x = odd ? vb : vr;
                    w.y = odd ? vr : vb;
                    *reinterpret_cast<float2 *>(g) = w;
                } else {
                    g[0] = odd ? vb : vr;
                }
            }
        }
        __syncthreads();
    }
    cp_wait(0);
    __syncthreads();
}

template <int TY, bool ZERO_IN>
__global__ void __launch_bounds__(NT) k_rb32_fused(LevelK<float> L, const float *__restrict__ ein,
                                                   float *__restrict__ eout, const float *__restrict__ b,
                                                   float omega, float omw, int kchunk, int ntx, int nty, int nitems)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem<TY> &S = *reinterpret_cast<Smem<TY> *>(smem_raw);
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int bz = it / (ntx * nty), rem = it % (ntx * nty);
        const int by = rem / ntx, bx = rem % ntx;
        const int k0 = 1 + kchunk * bz;
        const int k1 = min(L.nz, k0 + kchunk - 1);
        rb32_item<TY, ZERO_IN>(S, L, ein, eout, b, omega, omw, bx, by, k0, k1);
    }
}

struct Variant {
    int ty;
    int blocks_per_sm = 0;
    int sms = 0;
};

template <int TY>
int occupancy(int *blocks, int *sms)
{
    static std::once_flag once;
    static int b = 0, m = 0;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        const int bytes = (int)sizeof(Smem<TY>);
        err = cudaFuncSetAttribute(k_rb32_fused<TY, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k_rb32_fused<TY, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (err == cudaSuccess)
            err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_rb32_fused<TY, false>, NT, bytes);
        int dev = 0;
        if (err == cudaSuccess) err = cudaGetDevice(&dev);
        if (err == cudaSuccess) err = cudaDeviceGetAttribute(&m, cudaDevAttrMultiProcessorCount, dev);
    });
    *blocks = std::max(1, b);
    *sms = std::max(1, m);
    return cuda_status(err, "fused smoother setup");
}

template <int TY>
int launch_ty(const LevelK<float> &L, const Launch &ln, const float *ein, float *eout, const float *b, float omega,
              float omw, bool zero_in, int kchunk_hint, cudaStream_t s)
{
    int per_sm = 0, sms = 0;
    PMG_TRY_S(occupancy<TY>(&per_sm, &sms));
    const int ntx = (L.nx + TX - 1) / TX, nty = (L.ny + TY - 1) / TY;
    const int slots = per_sm * sms;
    int kchunk = kchunk_hint;
    if (kchunk <= 0) {
        // about four items per resident CTA, chunks of at least 16 planes
        const int want = std::max(1, (4 * slots + ntx * nty - 1) / (ntx * nty));
        kchunk = std::max(16, (L.nz + want - 1) / want);
    }
    if (ln.collapse[2]) kchunk = L.nz;
    kchunk = std::min(kchunk, L.nz);
    const int chunks = (L.nz + kchunk - 1) / kchunk;
    const int nitems = ntx * nty * chunks;
    const int grid = std::max(1, std::min(nitems, slots));
    const size_t bytes = sizeof(Smem<TY>);
    if (zero_in)
        k_rb32_fused<TY, true><<<grid, NT, bytes, s>>>(L, ein, eout, b, omega, omw, kchunk, ntx, nty, nitems);
    else
        k_rb32_fused<TY, false><<<grid, NT, bytes, s>>>(L, ein, eout, b, omega, omw, kchunk, ntx, nty, nitems);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "fused fp32 smoother");
}

}  // namespace

// ---- autotuner -------------------------------------------------------------------
// Times every (tile variant, k-chunk) candidate on the level's own buffers and keeps the
// fastest; results are cached per level shape for the process.
int tune_smoother(const LevelK<float> &L, const Launch &ln, float *e0, float *e1, const float *b, cudaStream_t s,
                  int *variant, int *kchunk)
{
    static std::mutex mu;
    static std::map<std::array<int, 4>, std::pair<int, int>> cache;
    const std::array<int, 4> key = {L.nx, L.ny, L.nz, ln.collapse[2] ? 1 : 0};
    *variant = 0;
    *kchunk = 0;
    if ((long long)L.nx * L.ny * L.nz < (1LL << 15)) return PMG_OK;
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = cache.find(key);
        if (it != cache.end()) {
            *variant = it->second.first;
            *kchunk = it->second.second;
            return PMG_OK;
        }
    }
    cudaEvent_t a = nullptr, z = nullptr;
    PMG_TRY_S(cuda_status(cudaEventCreate(&a), "tuner event"));
    PMG_TRY_S(cuda_status(cudaEventCreate(&z), "tuner event"));
    float best = 1e30f;
    int bv = 0, bk = 0;
    const int chunks[4] = {0, 8, 32, 128};
    for (int v = 0; v < 3; ++v)
        for (int c : chunks) {
            int rc = rb32_fused(L, ln, e0, e1, b, 1.f, 0.f, false, s, v, c);
            if (rc != PMG_OK) continue;
            cudaEventRecord(a, s);
            for (int r = 0; r < 3; ++r) rb32_fused(L, ln, e0, e1, b, 1.f, 0.f, false, s, v, c);
            cudaEventRecord(z, s);
            if (cudaEventSynchronize(z) != cudaSuccess) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, z);
            if (ms < best) {
                best = ms;
                bv = v;
                bk = c;
            }
        }
    cudaEventDestroy(a);
    cudaEventDestroy(z);
    PMG_TRY_S(cuda_status(cudaGetLastError(), "smoother autotuning"));
    *variant = bv;
    *kchunk = bk;
    std::lock_guard<std::mutex> g(mu);
    cache[key] = {bv, bk};
    return PMG_OK;
}

bool rb32_fused_layout_ok(const LevelK<float> &L, const void *e, const void *b)
{
    const int ntx = (L.nx + TX - 1) / TX;
    (void)e;
    (void)b;
    return L.sy % 2 == 0 && L.sz % 2 == 0 && L.sy >= TX * ntx + 8;
}

int rb32_fused(const LevelK<float> &L, const Launch &ln, const float *ein, float *eout, const float *b, float omega,
               float omw, bool zero_in, cudaStream_t s, int variant, int kchunk)
{
    switch (variant) {
    case 1: return launch_ty<8>(L, ln, ein, eout, b, omega, omw, zero_in, kchunk, s);
    case 2: return launch_ty<12>(L, ln, ein, eout, b, omega, omw, zero_in, kchunk, s);
    default: return launch_ty<16>(L, ln, ein, eout, b, omega, omw, zero_in, kchunk, s);
    }
}

}  // namespace pmg
