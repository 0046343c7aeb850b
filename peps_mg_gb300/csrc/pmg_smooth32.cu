// pmg_smooth32.cu -- launchers and autotuner of the fused FP32 red-black iteration
// (device code in pmg_smooth32.cuh).
//
// A launch performs one RBGS iteration of a whole level, out of place.  Work items are
// (60 x TY tile) x (chunk of k planes); a persistent grid of resident CTAs walks them
// chunk-major.  TY is 6, 10 or 14 (CTAs of 256, 384 or 512 threads); the autotuner
// times every (TY, k-chunk) candidate on the level's own buffers and keeps the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <map>
#include <mutex>

#include "../../include/peps_mg.h"
#include "pmg_internal.h"
#include "pmg_smooth32.cuh"

namespace pmg {

namespace {

#define PMG_TRY_S(expr)                \
    do {                               \
        int _rc = (expr);              \
        if (_rc != PMG_OK) return _rc; \
    } while (0)

// blocks per SM the register budget is sized for
template <int TY>
constexpr int rb_min_blocks() { return TY <= 6 ? 3 : TY <= 10 ? 2 : 1; }

template <int TY, bool ZERO_IN, bool OMEGA1>
__global__ void __launch_bounds__(rb_threads<TY>(), rb_min_blocks<TY>()) k_rb32_fused(LevelK<float> L, const float *__restrict__ ein,
                                                                 float *__restrict__ eout, const float *__restrict__ b,
                                                                 float omega, float omw, int kchunk, int ntx, int nty,
                                                                 int nitems)
{
    __shared__ __align__(16) RbSmem<TY> S;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int bz = it / (ntx * nty), rem = it % (ntx * nty);
        const int by = rem / ntx, bx = rem % ntx;
        const int k0 = 1 + kchunk * bz;
        const int k1 = min(L.nz, k0 + kchunk - 1);
        rb32_item<TY, ZERO_IN, OMEGA1>(S, L, ein, eout, b, omega, omw, bx, by, k0, k1);
    }
}

template <int TY>
int slots_for(int *slots)
{
    static std::once_flag once;
    static int per = 0, sms = 0;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rb32_fused<TY, false, false>, rb_threads<TY>(),
                                                            0);
        int dev = 0;
        if (err == cudaSuccess) err = cudaGetDevice(&dev);
        if (err == cudaSuccess) err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    });
    *slots = std::max(1, per) * std::max(1, sms);
    return cuda_status(err, "fused smoother occupancy");
}

template <int TY>
int launch_ty(const LevelK<float> &L, const Launch &ln, const float *ein, float *eout, const float *b, float omega,
              float omw, bool zero_in, int kchunk_hint, cudaStream_t s)
{
    int slots = 0;
    PMG_TRY_S(slots_for<TY>(&slots));
    const int ntx = (L.nx + RB_TX - 1) / RB_TX, nty = (L.ny + TY - 1) / TY;
    int kchunk = kchunk_hint;
    if (kchunk <= 0) {
        // about four items per resident CTA, chunks of at least 16 planes
        const int want = std::max(1, (4 * slots + ntx * nty - 1) / (ntx * nty));
        kchunk = std::max(16, (L.nz + want - 1) / want);
    }
    if (ln.collapse[2]) kchunk = L.nz;
    kchunk = std::max(1, std::min(std::min(kchunk, L.nz), RB_ZC - 3));
    const int chunks = (L.nz + kchunk - 1) / kchunk;
    const int nitems = ntx * nty * chunks;
    const int grid = std::max(1, std::min(nitems, slots));
    const bool one = omega == 1.f;
    if (zero_in && one)
        k_rb32_fused<TY, true, true><<<grid, rb_threads<TY>(), 0, s>>>(L, ein, eout, b, omega, omw, kchunk, ntx, nty,
                                                                       nitems);
    else if (zero_in)
        k_rb32_fused<TY, true, false><<<grid, rb_threads<TY>(), 0, s>>>(L, ein, eout, b, omega, omw, kchunk, ntx,
                                                                        nty, nitems);
    else if (one)
        k_rb32_fused<TY, false, true><<<grid, rb_threads<TY>(), 0, s>>>(L, ein, eout, b, omega, omw, kchunk, ntx,
                                                                        nty, nitems);
    else
        k_rb32_fused<TY, false, false><<<grid, rb_threads<TY>(), 0, s>>>(L, ein, eout, b, omega, omw, kchunk, ntx,
                                                                         nty, nitems);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "fused fp32 smoother");
}

}  // namespace

int rb32_fused(const LevelK<float> &L, const Launch &ln, const float *ein, float *eout, const float *b, float omega,
               float omw, bool zero_in, cudaStream_t s, int variant, int kchunk)
{
    switch (variant) {
    case 1: return launch_ty<6>(L, ln, ein, eout, b, omega, omw, zero_in, kchunk, s);
    case 2: return launch_ty<10>(L, ln, ein, eout, b, omega, omw, zero_in, kchunk, s);
    default: return launch_ty<14>(L, ln, ein, eout, b, omega, omw, zero_in, kchunk, s);
    }
}

bool rb32_fused_layout_ok(const LevelK<float> &L, const void *e, const void *b)
{
    // 8-byte pair loads and stores at odd cell indices: data pointers at an odd float
    // offset from an 8-byte boundary, even pitches, room for the tiles' columns and
    // 32-bit plane offsets
    const auto ae = reinterpret_cast<uintptr_t>(e), ab = reinterpret_cast<uintptr_t>(b);
    const int ntx = (L.nx + RB_TX - 1) / RB_TX;
    return L.sy % 2 == 0 && L.sz % 2 == 0 && (ae + 4) % 8 == 0 && (ab + 4) % 8 == 0 &&
           L.sy >= RB_TX * ntx + 8 && L.sz * (long long)(L.nz + 6) < (1LL << 31);
}

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
    const int chunks[4] = {0, 16, 32, 64};
    for (int v = 0; v < 3; ++v)
        for (int c : chunks) {
            if (rb32_fused(L, ln, e0, e1, b, 1.f, 0.f, false, s, v, c) != PMG_OK) continue;
            cudaEventRecord(a, s);
            for (int q = 0; q < 3; ++q) rb32_fused(L, ln, e0, e1, b, 1.f, 0.f, false, s, v, c);
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

}  // namespace pmg
