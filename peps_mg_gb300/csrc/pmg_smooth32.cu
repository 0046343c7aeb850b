// pmg_smooth32.cu -- launchers and autotuner of the fused FP32 red-black iteration
// (device code in pmg_smooth32_tma.cuh and pmg_smooth32.cuh).
//
// A launch performs one RBGS iteration of a whole level, out of place.  Work items are
// (60 x TY tile) x (chunk of k planes); a persistent grid of resident CTAs walks them
// chunk-major.  TY is 6, 10 or 14 (register-window CTAs of 256, 384 or 512 threads; the
// TMA-fed kernel also has TY = 22, two rows per warp: 128 to 384 threads); the autotuner
// times every (TY, k-chunk) candidate on the level's own buffers and keeps the fastest.
// Two kernels share that mapping: the TMA-fed one (planes copied into a ring of shared
// stages by the tensor-memory accelerator) wherever the level's tensor maps could be
// encoded, and the register-window one (per-thread loads three planes ahead) otherwise.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/peps_mg.h"
#include "pmg_internal.h"
#include "pmg_smooth32.cuh"
#include "pmg_smooth32_tma.cuh"

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

// One red-black iteration (src/rbgs_poisson_matrix.f90:235-273), out of place, one thread
// per cell pair (i odd, i + 1) and no marching.  The pair's first-colour cell (i + j + k
// odd) is updated from e_in; its second-colour cell from its six neighbours' first-colour
// updates, one of them the pair's own and five recomputed here from e_in.  Each update
// has the operations, in order, of the marching kernels' (s = cxm e_w, then FMAs of the
// east, south, north, lower and upper terms; d = (sx + (cym + cyp)) + (czm + czp); e =
// (s - b) / d, or (1 - omega) e + omega (s - b) / d), so the result has their bits.  Cells
// outside the grid are not updated and read as e_in (their zero ghosts); ZERO_IN reads e_in
// as zero everywhere.  The redundant updates cost FP32 work and L1/L2 reads, not DRAM
// traffic, on the levels it is chosen for (those that live in L2).
template <bool ZERO_IN, bool OMEGA1>
struct RbCell {
    const LevelK<float> &L;
    const float *ein, *b;
    float omega, omw;
    __device__ __forceinline__ float ld(long long p) const { return ZERO_IN ? 0.f : ein[p]; }
    __device__ __forceinline__ float upd(float old, float bb, float s, float d) const
    {
        if (OMEGA1) return __fdividef(s - bb, d);
        return fmaf(omw, old, __fdividef(omega * (s - bb), d));
    }
    __device__ __forceinline__ float diag(int i, int j, int k) const
    {
        return (L.sx[i] + (L.cym[j] + L.cyp[j])) + (L.czm[k] + L.czp[k]);
    }
    // update of cell (i, j, k) from neighbour values w, e (x), s, n (y), l, u (z)
    __device__ __forceinline__ float update(int i, int j, int k, long long p, float w, float e, float so, float no,
                                            float lo, float up) const
    {
        float s = L.cxm[i] * w;
        s = fmaf(L.cxp[i], e, s);
        s = fmaf(L.cym[j], so, s);
        s = fmaf(L.cyp[j], no, s);
        s = fmaf(L.czm[k], lo, s);
        s = fmaf(L.czp[k], up, s);
        return upd(ld(p), b[p], s, diag(i, j, k));
    }
    // first-colour value of cell (i, j, k) after the first half of the iteration
    __device__ __forceinline__ float first(int i, int j, int k) const
    {
        const long long p = lin(i, j, k, L.sy, L.sz);
        if (i < 1 || i > L.nx || j < 1 || j > L.ny || k < 1 || k > L.nz) return ld(p);
        if (ZERO_IN) return upd(0.f, b[p], 0.f, diag(i, j, k));
        return update(i, j, k, p, ein[p - 1], ein[p + 1], ein[p - L.sy], ein[p + L.sy], ein[p - L.sz],
                      ein[p + L.sz]);
    }
};

template <bool ZERO_IN, bool OMEGA1>
__global__ void __launch_bounds__(256) k_rb32_cell(LevelK<float> L, const float *__restrict__ ein,
                                                   float *__restrict__ eout, const float *__restrict__ b, float omega,
                                                   float omw)
{
    const RbCell<ZERO_IN, OMEGA1> C{L, ein, b, omega, omw};
    const int npx = (L.nx + 1) / 2;
    for (int k = blockIdx.z + 1; k <= L.nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= L.ny; j += gridDim.y * blockDim.y)
            for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npx; t += gridDim.x * blockDim.x) {
                const int i = 2 * t + 1;
                // (i + j + k) odd: cell i takes the first colour, else cell i + 1
                const int f = ((j + k) & 1) ? i + 1 : i, sc = ((j + k) & 1) ? i : i + 1;
                const float vf = C.first(f, j, k);
                if (f <= L.nx) eout[lin(f, j, k, L.sy, L.sz)] = vf;
                if (sc <= L.nx) {
                    const long long p = lin(sc, j, k, L.sy, L.sz);
                    const float w = sc - 1 == f ? vf : C.first(sc - 1, j, k);
                    const float e = sc + 1 == f ? vf : C.first(sc + 1, j, k);
                    eout[p] = C.update(sc, j, k, p, w, e, C.first(sc, j - 1, k), C.first(sc, j + 1, k),
                                       C.first(sc, j, k - 1), C.first(sc, j, k + 1));
                }
            }
}

int launch_cell(const LevelK<float> &L, const Launch &ln, const float *ein, float *eout, const float *b, float omega,
                float omw, bool zero_in, cudaStream_t s)
{
    const dim3 bl(32, 8, 1);
    dim3 g;
    g.x = ln.collapse[0] ? 1u : (unsigned)std::max(1, ((L.nx + 1) / 2 + 31) / 32);
    g.y = ln.collapse[1] ? 1u : (unsigned)std::max(1, (L.ny + 7) / 8);
    g.z = ln.collapse[2] ? 1u : (unsigned)std::max(1, std::min(L.nz, 65535));
    const bool one = omega == 1.f;
    if (zero_in && one) k_rb32_cell<true, true><<<g, bl, 0, s>>>(L, ein, eout, b, omega, omw);
    else if (zero_in) k_rb32_cell<true, false><<<g, bl, 0, s>>>(L, ein, eout, b, omega, omw);
    else if (one) k_rb32_cell<false, true><<<g, bl, 0, s>>>(L, ein, eout, b, omega, omw);
    else k_rb32_cell<false, false><<<g, bl, 0, s>>>(L, ein, eout, b, omega, omw);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "fp32 cell smoother");
}

// blocks per SM the TMA-fed kernel's register budget is sized for
template <int TY>
constexpr int rbt_min_blocks() { return rbt_min_ctas<TY>(); }

template <int TY, bool ZERO_IN, bool OMEGA1, bool STALL = false>
__global__ void __launch_bounds__(RbtShape<TY>::THREADS, rbt_min_blocks<TY>())
    k_rb32_tma(const __grid_constant__ CUtensorMap me, const __grid_constant__ CUtensorMap mb, LevelK<float> L,
               float *__restrict__ eout, float omega, float omw, RbtItems W, int *err)
{
    const RbtGridSrc<STALL> src{&W, &me, &mb};
    rbt_cta<TY, ZERO_IN, OMEGA1>(
        src,
        [&](int, const LevelK<float> *&Li, float *&eo) {
            Li = &L;
            eo = eout;
        },
        omega, omw, err);
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

template <int TY, bool Z, bool O, bool STALL = false>
int tma_attr()
{
    static std::once_flag once;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        err = cudaFuncSetAttribute(k_rb32_tma<TY, Z, O, STALL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   RbtShape<TY>::SMEM);
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k_rb32_tma<TY, Z, O, STALL>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       100);
    });
    return cuda_status(err, "TMA smoother shared memory attribute");
}

template <int TY>
int tma_attr_all()
{
    PMG_TRY_S((tma_attr<TY, false, false>()));
    PMG_TRY_S((tma_attr<TY, false, true>()));
    PMG_TRY_S((tma_attr<TY, true, false>()));
    return tma_attr<TY, true, true>();
}

template <int TY>
int tma_slots(int *slots)
{
    static std::once_flag once;
    static int per = 0, sms = 0;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        err = cudaFuncSetAttribute(k_rb32_tma<TY, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   RbtShape<TY>::SMEM);
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k_rb32_tma<TY, false, false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       100);
        if (err == cudaSuccess)
            err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rb32_tma<TY, false, false>,
                                                                RbtShape<TY>::THREADS, RbtShape<TY>::SMEM);
        int dev = 0;
        if (err == cudaSuccess) err = cudaGetDevice(&dev);
        if (err == cudaSuccess) err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    });
    *slots = std::max(1, per) * std::max(1, sms);
    return cuda_status(err, "TMA smoother occupancy");
}

template <int TY>
int launch_tma(const LevelK<float> &L, const Launch &ln, const Rb32Tma &t, int vi, int in_buf, float *eout,
               float omega, float omw, bool zero_in, int kchunk_hint, int *err, cudaStream_t s, bool stall)
{
    int slots = 0;
    PMG_TRY_S(tma_slots<TY>(&slots));
    RbtItems W;
    W.ntx = (L.nx + RBT_TX - 1) / RBT_TX;
    W.nty = (L.ny + TY - 1) / TY;
    W.nz = L.nz;
    int kchunk = kchunk_hint;
    if (kchunk <= 0) {
        const int want = std::max(1, (4 * slots + W.ntx * W.nty - 1) / (W.ntx * W.nty));
        kchunk = std::max(16, (L.nz + want - 1) / want);
    }
    if (ln.collapse[2]) kchunk = L.nz;
    W.kchunk = std::max(1, std::min(kchunk, L.nz));
    W.nitems = W.ntx * W.nty * ((L.nz + W.kchunk - 1) / W.kchunk);
    const int grid = std::max(1, std::min(W.nitems, slots));
    const bool one = omega == 1.f;
    const CUtensorMap &me = t.e[in_buf][vi], &mb = t.b[vi];
    constexpr int T = RbtShape<TY>::THREADS, SM = RbtShape<TY>::SMEM;
    if (stall) {
        // the self-test instantiation: e_in read (no zero start), omega = 1
        if (zero_in || !one) {
            set_error("the stall self-test runs the omega = 1 iteration from a given e");
            return PMG_EINVAL;
        }
        PMG_TRY_S((tma_attr<TY, false, true, true>()));
        k_rb32_tma<TY, false, true, true><<<grid, T, SM, s>>>(me, mb, L, eout, omega, omw, W, err);
    } else if (zero_in && one) {
        PMG_TRY_S((tma_attr<TY, true, true>()));
        k_rb32_tma<TY, true, true><<<grid, T, SM, s>>>(me, mb, L, eout, omega, omw, W, err);
    } else if (zero_in) {
        PMG_TRY_S((tma_attr<TY, true, false>()));
        k_rb32_tma<TY, true, false><<<grid, T, SM, s>>>(me, mb, L, eout, omega, omw, W, err);
    } else if (one) {
        PMG_TRY_S((tma_attr<TY, false, true>()));
        k_rb32_tma<TY, false, true><<<grid, T, SM, s>>>(me, mb, L, eout, omega, omw, W, err);
    } else {
        PMG_TRY_S((tma_attr<TY, false, false>()));
        k_rb32_tma<TY, false, false><<<grid, T, SM, s>>>(me, mb, L, eout, omega, omw, W, err);
    }
    count_launches(1);
    return cuda_status(cudaGetLastError(), "TMA fp32 smoother");
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        cudaGetLastError();
    });
    return fn;
}

// 3-D map of a padded FP32 array: x = column (pitch sy), y = row, z = plane; box of 64
// columns x `box_rows` rows x 1 plane; out-of-range elements read as zero.
bool encode_map(CUtensorMap *m, float *base, const LevelK<float> &L, long long rows, long long planes, int box_rows)
{
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)L.sy, (cuuint64_t)rows, (cuuint64_t)planes};
    const cuuint64_t strides[2] = {(cuuint64_t)L.sy * 4u, (cuuint64_t)L.sz * 4u};
    const cuuint32_t box[3] = {(cuuint32_t)RBT_W, (cuuint32_t)box_rows, 1u};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

int rb32_tma_setup(Rb32Tma *t, const LevelK<float> &L, float *const base[3], long long rows, long long planes)
{
    t->ok = false;
    // TMA: 16-byte aligned bases and strides; the first copied column, 5 + 60 bx - 1, is a
    // multiple of 4 floats for every tile
    static_assert((RBT_DATA_OFF - 1) % 4 == 0 && RBT_TX % 4 == 0, "TMA column alignment");
    if (L.sy % 4 != 0 || L.sz % 4 != 0) return PMG_OK;
    for (int q = 0; q < 3; ++q)
        if (reinterpret_cast<uintptr_t>(base[q]) % 16 != 0) return PMG_OK;
    if (L.sy < RBT_TX * ((L.nx + RBT_TX - 1) / RBT_TX) + 8) return PMG_OK;
    const int tys[4] = {14, 6, 10, 22};
    for (int v = 0; v < 4; ++v) {
        for (int q = 0; q < 2; ++q)
            if (!encode_map(&t->e[q][v], base[q], L, rows, planes, tys[v] + 4)) return PMG_OK;
        if (!encode_map(&t->b[v], base[2], L, rows, planes, tys[v] + 2)) return PMG_OK;
    }
    // every kernel instance's shared-memory attributes now, so that no launch (one being
    // captured into a graph included) sets them first
    PMG_TRY_S(tma_attr_all<14>());
    PMG_TRY_S(tma_attr_all<6>());
    PMG_TRY_S(tma_attr_all<10>());
    PMG_TRY_S(tma_attr_all<22>());
    t->ok = true;
    return PMG_OK;
}

int rb32_fused(const LevelK<float> &L, const Launch &ln, const float *ein, float *eout, const float *b, float omega,
               float omw, bool zero_in, cudaStream_t s, int variant, int kchunk, const Rb32Tma *tma, int in_buf,
               int *err, bool stall)
{
    if (variant == kCellVariant) {
        if (stall) {
            set_error("the stall self-test needs the TMA-fed smoother");
            return PMG_EINVAL;
        }
        return launch_cell(L, ln, ein, eout, b, omega, omw, zero_in, s);
    }
    if (tma && tma->ok && err) {
        switch (variant) {
        case 1: return launch_tma<6>(L, ln, *tma, 1, in_buf, eout, omega, omw, zero_in, kchunk, err, s, stall);
        case 2: return launch_tma<10>(L, ln, *tma, 2, in_buf, eout, omega, omw, zero_in, kchunk, err, s, stall);
        case 3: return launch_tma<22>(L, ln, *tma, 3, in_buf, eout, omega, omw, zero_in, kchunk, err, s, stall);
        default: return launch_tma<14>(L, ln, *tma, 0, in_buf, eout, omega, omw, zero_in, kchunk, err, s, stall);
        }
    }
    if (stall) {
        set_error("the stall self-test needs the TMA-fed smoother");
        return PMG_EINVAL;
    }
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
                  int *variant, int *kchunk, const Rb32Tma *tma, int *err, bool allow_cell)
{
    static std::mutex mu;
    static std::map<std::array<int, 6>, std::pair<int, int>> cache;
    const bool use_tma = tma && tma->ok && err;
    const std::array<int, 6> key = {L.nx, L.ny, L.nz, ln.collapse[2] ? 1 : 0, use_tma ? 1 : 0, allow_cell ? 1 : 0};
    *variant = 0;
    *kchunk = 0;

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
    const char *log_env = std::getenv("PEPS_MG_TUNE_LOG");   // print every candidate's time
    const bool log = log_env && log_env[0] == '1';
    // the register-window kernel stages at most RB_ZC - 3 planes of z coefficients
    const int chunks_window[] = {0, 16, 32, 64}, chunks_tma[] = {4, 8, 16, 32, 64, 128};
    const int tys[4] = {14, 6, 10, 22};
    bool best_window = !use_tma;
    // The register-window kernel (no copy pipeline to fill) only wins on small levels: it is
    // timed where the TMA-fed one cannot run or the level has at most 2^22 cells.
    const bool try_window = !use_tma || (long long)L.nx * L.ny * L.nz <= (1LL << 22);
    bool best_cell = false;
    auto time_one = [&](bool tk, int v, int c, float *ms) -> bool {
        const Rb32Tma *tm = tk ? tma : nullptr;
        if (rb32_fused(L, ln, e0, e1, b, 1.f, 0.f, false, s, v, c, tm, 0, err) != PMG_OK) return false;
        cudaEventRecord(a, s);
        for (int q = 0; q < 3; ++q) rb32_fused(L, ln, e0, e1, b, 1.f, 0.f, false, s, v, c, tm, 0, err);
        cudaEventRecord(z, s);
        if (cudaEventSynchronize(z) != cudaSuccess) return false;
        cudaEventElapsedTime(ms, a, z);
        const bool cell = v == kCellVariant;
        if (log)
            std::fprintf(stderr, "[peps_mg tune] %dx%dx%d %s TY=%d kchunk=%d: %.1f us\n", L.nx, L.ny, L.nz,
                         cell ? "cell" : tk ? "tma" : "window", cell ? 0 : tys[v], c, *ms * 1e3f / 3.f);
        if (*ms < best) {
            best = *ms;
            bv = v;
            bk = c;
            best_window = !tk && !cell;
            best_cell = cell;
        }
        return true;
    };
    // the one-launch cell-pair kernel, on the levels where the register-window one is tried
    if (try_window && allow_cell) {
        float ms = 0.f;
        time_one(false, kCellVariant, 0, &ms);
    }
    for (int kind = use_tma ? 0 : 1; kind < 2; ++kind) {
        const bool tk = kind == 0;
        if (!tk && !try_window) break;
        for (int v = 0; v < (tk ? 4 : 3); ++v) {
            if (!tk) {
                for (const int c : chunks_window) {
                    float ms = 0.f;
                    if (!time_one(false, v, c, &ms)) break;
                }
                continue;
            }
            // The k-chunks that spread the tiles' items evenly over the resident CTA slots
            // (one to three rounds) are all timed: they are the fast ones where the level
            // has few items.  The powers of two are walked from 16 planes up while they stay
            // within 10% of this tile's best, and down only from a minimum at 16.
            std::vector<int> pow2;
            for (const int c : chunks_tma) pow2.push_back(std::min(c, L.nz));
            std::sort(pow2.begin(), pow2.end());
            pow2.erase(std::unique(pow2.begin(), pow2.end()), pow2.end());
            std::vector<int> balanced;
            int slots = 0;
            const int r = v == 1 ? tma_slots<6>(&slots) : v == 2 ? tma_slots<10>(&slots)
                                                               : v == 3 ? tma_slots<22>(&slots) : tma_slots<14>(&slots);
            const int tiles = ((L.nx + RBT_TX - 1) / RBT_TX) * ((L.ny + tys[v] - 1) / tys[v]);
            if (r == PMG_OK && slots > 0)
                for (int rounds = 1; rounds <= 3; ++rounds) {
                    const int nch = std::max(1, (rounds * slots) / std::max(1, tiles));
                    const int c = std::min((L.nz + nch - 1) / nch, L.nz);
                    if (c >= 4 && std::find(pow2.begin(), pow2.end(), c) == pow2.end() &&
                        std::find(balanced.begin(), balanced.end(), c) == balanced.end())
                        balanced.push_back(c);
                }
            for (const int c : balanced) {
                float ms = 0.f;
                time_one(true, v, c, &ms);
            }
            const size_t start = std::lower_bound(pow2.begin(), pow2.end(), std::min(16, L.nz)) - pow2.begin();
            float walk_best = 1e30f;
            size_t walk_best_at = start;
            for (size_t q = start; q < pow2.size(); ++q) {
                float ms = 0.f;
                if (!time_one(true, v, pow2[q], &ms)) break;
                if (ms < walk_best) {
                    walk_best = ms;
                    walk_best_at = q;
                } else if (ms > 1.1f * walk_best) {
                    break;
                }
            }
            if (walk_best_at == start)
                for (size_t q = start; q-- > 0;) {
                    float ms = 0.f;
                    if (!time_one(true, v, pow2[q], &ms) || ms > 1.1f * walk_best) break;
                    walk_best = std::min(walk_best, ms);
                }
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(z);
    PMG_TRY_S(cuda_status(cudaGetLastError(), "smoother autotuning"));
    // a level with tensor maps whose fastest kernel is the register-window one is flagged
    // (kTuneWindow): its caller runs the window kernel there
    const int code = best_cell ? kCellVariant : bv + (use_tma && best_window ? kTuneWindow : 0);
    *variant = code;
    *kchunk = bk;
    if (log)
        std::fprintf(stderr, "[peps_mg tune] %dx%dx%d chosen %s TY=%d kchunk=%d (%.1f us)\n", L.nx, L.ny, L.nz,
                     best_cell ? "cell" : best_window ? "window" : "tma", best_cell ? 0 : tys[bv], bk,
                     best * 1e3f / 3.f);
    std::lock_guard<std::mutex> g(mu);
    cache[key] = {code, bk};
    return PMG_OK;
}

}  // namespace pmg
