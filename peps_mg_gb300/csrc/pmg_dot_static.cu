// pmg_dot_static.cu -- interior dot product of two fields with no device allocation.
//
// Some host codes cannot let a library call cudaMalloc: a Fortran solver that hands its
// device memory to its own allocator at start-up (so a later cudaMalloc can fail), or
// one calling from inside its iteration loop, where the device-wide synchronisation of
// cudaMalloc/cudaFree would stall its other streams.  Such a caller keeps its own CG
// loop (the reference's vv_dot_3d_matrix) and has no pmg_ctx, because creating one
// allocates the whole level hierarchy.  pmg_vv_dot_static serves it: the per-CTA
// partial sums live in a fixed file-scope __device__ array that every GPU loading this
// library holds until the process exits, and nothing is allocated per call.
//
// The sum is the same as pmg_vv_dot's: FP64 products and sums rounded to nearest, one
// partial per 32x8 CTA over a grid-stride loop, the partials added in a fixed order by
// one CTA.  The grid's z extent is capped so that the partials fit the static array;
// when it is not capped (nz <= kStaticPartials / (CTAs per plane)) the order of
// operations, and so the result, is bit for bit that of pmg_vv_dot.
//
// Compiled with --fmad=false like the rest of the FP64 code.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/peps_mg.h"
#include "pmg_internal.h"

namespace pmg {

namespace {

#define PMG_TRY_D(expr)                \
    do {                               \
        int _rc = (expr);              \
        if (_rc != PMG_OK) return _rc; \
    } while (0)

constexpr int kBX = 32, kBY = 8;
constexpr int kStaticPartials = 16384;   // 128 KiB of partial sums per GPU
constexpr int kMaxDevices = 64;

// [0, kStaticPartials): one partial sum per CTA; [kStaticPartials]: the result; the rest
// pads the array to a multiple of 256 bytes.  Every slot that a call reads is written
// earlier in the same call, so no slot has to start at zero between calls; the whole
// array is cleared once at set-up, so a slot never holds anything but a sum of this
// entry point.
__device__ __align__(256) double g_dot_scratch[kStaticPartials + 32];

__global__ void __launch_bounds__(kBX *kBY) k_dot_static(int nx, int ny, int nz, long long sy, long long sz,
                                                         const double *__restrict__ x,
                                                         const double *__restrict__ y, double *partials)
{
    double acc = 0.0;
    for (int k = blockIdx.z + 1; k <= nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= ny; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= nx; i += gridDim.x * blockDim.x) {
                const long long p = i + sy * j + sz * k;
                acc = __dadd_rn(acc, __dmul_rn(x[p], y[p]));
            }
    __shared__ double sw[kBX * kBY / 32];
    const double s = block_sum(acc, sw);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0)
        partials[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s;
}

__global__ void __launch_bounds__(1024) k_reduce_static(const double *__restrict__ partials, int n, double *out)
{
    double acc = 0.0;
    for (int q = threadIdx.x; q < n; q += blockDim.x) acc = __dadd_rn(acc, partials[q]);
    __shared__ double sw[32];
    const double s = block_sum(acc, sw);
    if (threadIdx.x == 0) *out = s;
}

std::mutex g_setup_mu;
double *g_scratch_ptr[kMaxDevices] = {};

// With the device current: the address of this device's copy of the scratch array.  The
// address is looked up on every call (a host-side query that allocates nothing), so a
// context that the caller destroyed and re-created, e.g. by cudaDeviceReset, is served
// with the array of the new context and never with a stale address.  The array is
// cleared (in the order of stream s) whenever its address differs from the one this
// device's previous call saw, which includes the first call on each device; no result
// depends on that clearing, since every slot a call reads is written earlier in the call.
int scratch_for_current_device(cudaStream_t s, double **out)
{
    int dev = 0;
    PMG_TRY_D(cuda_status(cudaGetDevice(&dev), "pmg_vv_dot_static: current device"));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("pmg_vv_dot_static: device ordinal " + std::to_string(dev) + " is beyond the " +
                  std::to_string(kMaxDevices) + " devices this entry point serves");
        return PMG_EINVAL;
    }
    double *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_dot_scratch);
    if (e != cudaSuccess || !ptr)
        return cuda_status(e != cudaSuccess ? e : cudaErrorInvalidSymbol,
                           "pmg_vv_dot_static: address of the static scratch");
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (g_scratch_ptr[dev] != ptr) {
        PMG_TRY_D(cuda_status(cudaMemsetAsync(ptr, 0, sizeof(g_dot_scratch), s),
                              "pmg_vv_dot_static: clearing the static scratch"));
        g_scratch_ptr[dev] = ptr;
    }
    *out = ptr;
    return PMG_OK;
}

}  // namespace

}  // namespace pmg

extern "C" int pmg_vv_dot_static(const double *x, const double *y, int nx, int ny, int nz, void *stream,
                                 double *result)
{
    using namespace pmg;
    if (!x || !y || !result) {
        set_error("pmg_vv_dot_static: x, y and result must not be NULL");
        return PMG_EINVAL;
    }
    if (nx < 1 || ny < 1 || nz < 1) {
        set_error("pmg_vv_dot_static: nx, ny, nz must be positive");
        return PMG_EINVAL;
    }
    const long long gx = (nx + kBX - 1) / kBX, gy = (ny + kBY - 1) / kBY;
    if (gx * gy > kStaticPartials) {
        set_error("pmg_vv_dot_static: an x-y plane of " + std::to_string(nx) + " x " + std::to_string(ny) +
                  " cells needs " + std::to_string(gx * gy) + " partial sums but the static scratch holds " +
                  std::to_string(kStaticPartials) + " (ceil(nx/32) * ceil(ny/8) must not exceed " +
                  std::to_string(kStaticPartials) + ")");
        return PMG_EINVAL;
    }
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    double *scratch = nullptr;
    PMG_TRY_D(scratch_for_current_device(s, &scratch));
    const long long gz = std::min<long long>(std::min<long long>(nz, 65535), kStaticPartials / (gx * gy));
    const long long sy = nx + 2, sz = sy * (ny + 2);
    k_dot_static<<<dim3((unsigned)gx, (unsigned)gy, (unsigned)gz), dim3(kBX, kBY, 1), 0, s>>>(nx, ny, nz, sy, sz, x,
                                                                                             y, scratch);
    k_reduce_static<<<1, 1024, 0, s>>>(scratch, (int)(gx * gy * gz), scratch + kStaticPartials);
    count_launches(2);
    PMG_TRY_D(cuda_status(cudaGetLastError(), "pmg_vv_dot_static: launch"));
    PMG_TRY_D(cuda_status(cudaMemcpyAsync(result, scratch + kStaticPartials, sizeof(double), cudaMemcpyDeviceToHost, s),
                          "pmg_vv_dot_static: result read"));
    return cuda_status(cudaStreamSynchronize(s), "pmg_vv_dot_static: stream sync");
}
