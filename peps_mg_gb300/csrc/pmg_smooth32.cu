// pmg_smooth32.cu -- fused red-black iteration of the FP32 smoother.
//
// One launch performs one full RBGS iteration of src/rbgs_poisson_matrix.f90:235-273
// (first colour, then second colour) on a whole level, out of place:
//
//     e_out = RB(e_in)        (e_in = 0 for the first iteration from a zero start)
//
// so that every global value read is an old value and CTAs need no ordering.  Each CTA
// owns a TX x TY tile of (i, j) and marches along k through a chunk of planes, keeping
// a ring of planes in shared memory (filled by cp.async 16-byte copies one plane ahead):
// the first colour is updated on plane t over the tile plus a one-cell ring, then the
// second colour on plane t-1 over the tile, which then holds final values of both
// colours and is stored with coalesced 8-byte stores.  DRAM traffic per iteration is
// one read of e_in, one of b and one write of e_out: 12 B per cell (8 B with e_in = 0).
//
// FP32 layout (internal arrays of the mixed-precision V-cycle): element (i,j,k) at
// base[i + sy*j + sz*k] with sy a multiple of 4 and at least TX*ceil(nx/TX) + 8, and
// base + 1 aligned to 16 bytes; columns -3..sy-4 of every row are valid memory.
#include <cuda_runtime.h>

#include <algorithm>

#include "pmg_internal.h"

namespace pmg {

namespace {

constexpr int TX = 64, TY = 16;        // tile of interior cells per CTA
constexpr int RW = TX + 8;             // shared row: columns i0-4 .. i0+TX+3 (16-byte aligned copies)
constexpr int ER = TY + 4;             // e rows j0-2 .. j0+TY+1
constexpr int BR = TY + 2;             // b rows j0-1 .. j0+TY
constexpr int NE = 5;                  // e planes t-2 .. t+2
constexpr int NB = 3;                  // b planes t-1 .. t+1
constexpr int NT = 256;
constexpr int PR = TX / 2 + 2;         // pairs per row in the ring (columns i0-2 .. i0+TX+1)

struct Smem {
    float e[NE][ER][RW];
    float b[NB][BR][RW];
    float dx[RW], cxm[RW], cxp[RW];
    float dy[ER], cym[ER], cyp[ER];
};

__device__ __forceinline__ void cp16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;\n" ::); }
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.wait_group 0;\n" ::); }

template <bool ZERO_IN>
__global__ void __launch_bounds__(NT) k_rb32_fused(LevelK<float> L, const float *__restrict__ ein,
                                                   float *__restrict__ eout, const float *__restrict__ b,
                                                   float omega, float omw, int kchunk)
{
    __shared__ __align__(16) Smem S;
    const int tid = threadIdx.x;
    const int i0 = 1 + TX * blockIdx.x, j0 = 1 + TY * blockIdx.y;
    const int k0 = 1 + kchunk * blockIdx.z;
    const int k1 = min(L.nz, k0 + kchunk - 1);
    const int nx = L.nx, ny = L.ny, nz = L.nz;
    const int sy = L.sy;
    const long long sz = L.sz;

    // 1-D coefficient tables of the tile
    for (int c = tid; c < RW; c += NT) {
        const int i = i0 - 4 + c;
        const bool in = i >= 1 && i <= nx;
        S.dx[c] = in ? L.sx[i] : 0.f;
        S.cxm[c] = in ? L.cxm[i] : 0.f;
        S.cxp[c] = in ? L.cxp[i] : 0.f;
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
        float(*dst)[RW] = S.e[(k + NE) % NE];
        for (int q = tid; q < ER * (RW / 4); q += NT) {
            const int r = q / (RW / 4), c4 = q % (RW / 4);
            const int j = j0 - 2 + r;
            if (j < 0 || j > ny + 1) continue;
            cp16(&dst[r][4 * c4], ein + (long long)(i0 - 4 + 4 * c4) + (long long)sy * j + sz * k);
        }
    };
    auto load_b = [&](int k) {
        if (k < 1 || k > nz) return;
        float(*dst)[RW] = S.b[k % NB];
        for (int q = tid; q < BR * (RW / 4); q += NT) {
            const int r = q / (RW / 4), c4 = q % (RW / 4);
            const int j = j0 - 1 + r;
            if (j > ny + 1) continue;
            cp16(&dst[r][4 * c4], b + (long long)(i0 - 4 + 4 * c4) + (long long)sy * j + sz * k);
        }
    };

    load_e(k0 - 2);
    load_e(k0 - 1);
    load_e(k0);
    load_b(k0 - 1);
    cp_commit();

    for (int t = k0 - 1; t <= k1 + 1; ++t) {
        load_e(t + 2);
        load_b(t + 1);
        cp_commit();
        cp_wait1();
        __syncthreads();

        // ---- first colour on plane t over the tile plus a one-cell ring -------------
        if (ZERO_IN && (t < 1 || t > nz)) {
            // a ghost plane of a zero start reads as zero
            float(*E)[RW] = S.e[t % NE];
            for (int q = tid; q < PR * (TY + 2); q += NT) {
                const int rr = q / PR, p = q % PR;
                const int c = 2 + 2 * p;
                E[rr + 1][c] = 0.f;
                E[rr + 1][c + 1] = 0.f;
            }
        } else if (t >= 1 && t <= nz) {
            float(*E)[RW] = S.e[t % NE];
            const float(*Em)[RW] = S.e[(t - 1 + NE) % NE];
            const float(*Ep)[RW] = S.e[(t + 1) % NE];
            const float(*B)[RW] = S.b[t % NB];
            const float czm = L.czm[t], czp = L.czp[t], dz = czm + czp;
            for (int q = tid; q < PR * (TY + 2); q += NT) {
                const int rr = q / PR, p = q % PR;          // ring row 0..TY+1, pair 0..PR-1
                const int re = rr + 1;                       // e row
                const int j = j0 - 1 + rr;
                const int ipair = i0 - 2 + 2 * p;            // odd cell index of the pair
                const int ir = ipair + ((j + t) & 1);        // first-colour cell: i+j+t odd
                const int c = ir - (i0 - 4);
                float v = 0.f;
                const bool interior = ir >= 1 && ir <= nx && j >= 1 && j <= ny;
                if (interior) {
                    const float bb = B[rr][c];
                    const float c0 = -((S.dx[c] + S.dy[re]) + dz);
                    if (ZERO_IN) {
                        v = __fdividef(omega * bb, c0);
                    } else {
                        float s = S.cxm[c] * E[re][c - 1];
                        s = fmaf(S.cxp[c], E[re][c + 1], s);
                        s = fmaf(S.cym[re], E[re - 1][c], s);
                        s = fmaf(S.cyp[re], E[re + 1][c], s);
                        s = fmaf(czm, Em[re][c], s);
                        s = fmaf(czp, Ep[re][c], s);
                        v = fmaf(omw, E[re][c], __fdividef(omega * (bb - s), c0));
                    }
                }
                if (ZERO_IN) {
                    // plane t holds only first-colour values: zero the second-colour cell
                    E[re][c] = v;
                    E[re][c + (((j + t) & 1) ? -1 : 1)] = 0.f;
                } else if (interior) {
                    E[re][c] = v;
                }
            }
        }
        __syncthreads();

        // ---- second colour on plane s = t-1 over the tile; store both colours --------
        const int s = t - 1;
        if (s >= k0 && s <= k1) {
            float(*E)[RW] = S.e[s % NE];
            const float(*Em)[RW] = S.e[(s - 1 + NE) % NE];
            const float(*Ep)[RW] = S.e[(s + 1) % NE];
            const float(*B)[RW] = S.b[s % NB];
            const float czm = L.czm[s], czp = L.czp[s], dz = czm + czp;
            for (int q = tid; q < (TX / 2) * TY; q += NT) {
                const int rr = q / (TX / 2), p = q % (TX / 2);
                const int re = rr + 2, rb = rr + 1;
                const int j = j0 + rr;
                const int ipair = i0 + 2 * p;
                if (j > ny || ipair > nx) continue;
                const int odd = (j + s) & 1;                 // first-colour cell is ipair + odd
                const int ib = ipair + 1 - odd;              // second-colour cell
                const int cb = ib - (i0 - 4);
                const int cr = ipair + odd - (i0 - 4);
                float vb = 0.f;
                if (ib <= nx) {
                    const float bb = B[rb][cb];
                    const float c0 = -((S.dx[cb] + S.dy[re]) + dz);
                    float sum = S.cxm[cb] * E[re][cb - 1];
                    sum = fmaf(S.cxp[cb], E[re][cb + 1], sum);
                    sum = fmaf(S.cym[re], E[re - 1][cb], sum);
                    sum = fmaf(S.cyp[re], E[re + 1][cb], sum);
                    sum = fmaf(czm, Em[re][cb], sum);
                    sum = fmaf(czp, Ep[re][cb], sum);
                    const float old = ZERO_IN ? 0.f : E[re][cb];
                    vb = fmaf(omw, old, __fdividef(omega * (bb - sum), c0));
                }
                const float vr = E[re][cr];
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
    cp_wait0();
}

}  // namespace

bool rb32_fused_layout_ok(const LevelK<float> &L, const void *e, const void *b)
{
    const int ntx = (L.nx + TX - 1) / TX;
    if (L.sy % 4 != 0 || L.sy < TX * ntx + 8 || L.sz % 4 != 0) return false;
    const auto a1 = reinterpret_cast<uintptr_t>(static_cast<const float *>(e) + 1);
    const auto a2 = reinterpret_cast<uintptr_t>(static_cast<const float *>(b) + 1);
    return a1 % 16 == 0 && a2 % 16 == 0;
}

int rb32_fused(const LevelK<float> &L, const Launch &ln, const float *ein, float *eout, const float *b, float omega,
               float omw, bool zero_in, cudaStream_t s)
{
    const int ntx = (L.nx + TX - 1) / TX, nty = (L.ny + TY - 1) / TY;
    // enough CTAs to fill the GPU: split k into chunks (each chunk recomputes one plane
    // of the first colour below its start)
    int chunks = std::max(1, std::min((L.nz + 15) / 16, (4 * 152 + ntx * nty - 1) / (ntx * nty)));
    if (ln.collapse[2]) chunks = 1;
    const int kchunk = (L.nz + chunks - 1) / chunks;
    chunks = (L.nz + kchunk - 1) / kchunk;
    const dim3 g(ntx, nty, chunks);
    if (zero_in)
        k_rb32_fused<true><<<g, NT, 0, s>>>(L, ein, eout, b, omega, omw, kchunk);
    else
        k_rb32_fused<false><<<g, NT, 0, s>>>(L, ein, eout, b, omega, omw, kchunk);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "fused fp32 smoother");
}

}  // namespace pmg
