// pmg_adjoint.cu -- adjoint of the V-cycle solve: gradients of a loss L(u) with respect
// to the right-hand side and the six Dirichlet face values.
//
// The forward solve computes the interior u of  A u = b  where the ghost cells hold the
// Dirichlet values g, i.e.  A_int u = b - A_bnd g.  For a loss with gradient w = dL/du:
//
//   lambda   = A_int^{-T} w
//   dL/db    = lambda                                    (interior cells)
//   dL/dg_f  = - sum over the cells next to face f of  c_f(cell) lambda(cell)
//
// where c_f is the coefficient that couples the cell to its ghost across face f (each
// face's ghost layer is one scalar g_f).  The operator is symmetric only on uniform
// meshes, but V A is symmetric for V = diag(dxm dym dzm) (the coefficient to the lower
// neighbour, 1/(dm(i) dg(i)), times V(i) equals the coefficient to the upper neighbour of
// cell i-1 times V(i-1); src/matrix.f90:75-76), so  A^T = V A V^{-1}  and
//
//   A^T lambda = w   <=>   A (V^{-1} lambda) = V^{-1} w,
//
// which is solved by the forward V-cycle itself (any precision mode) with zero ghost
// values.  Only the finest-level right-hand side and solution are held; no V-cycle state
// of the forward solve is kept.
//
// Compiled with --fmad=false like the rest of the FP64 code.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pmg_ctx.h"

namespace pmg {

namespace {

#define PMG_TRY_A(expr)                \
    do {                               \
        int _rc = (expr);              \
        if (_rc != PMG_OK) return _rc; \
    } while (0)

constexpr int kBX = 32, kBY = 8;

// out = w / vol on the interior, 0 on the ghosts (mode 0); out = vol * w on the interior
// (mode 1).  vol = dxm(i) dym(j) dzm(k).
__global__ void __launch_bounds__(kBX *kBY) k_volume_scale(int nx, int ny, int nz, int sy, long long sz,
                                                           const double *__restrict__ dxm,
                                                           const double *__restrict__ dym,
                                                           const double *__restrict__ dzm,
                                                           const double *__restrict__ in, double *__restrict__ out,
                                                           int mode)
{
    for (int k = blockIdx.z + 1; k <= nz; k += gridDim.z)
        for (int j = blockIdx.y * blockDim.y + threadIdx.y + 1; j <= ny; j += gridDim.y * blockDim.y)
            for (int i = blockIdx.x * blockDim.x + threadIdx.x + 1; i <= nx; i += gridDim.x * blockDim.x) {
                const long long p = lin(i, j, k, sy, sz);
                const double vol = __dmul_rn(__dmul_rn(dxm[i], dym[j]), dzm[k]);
                out[p] = mode == 0 ? __ddiv_rn(in[p], vol) : __dmul_rn(vol, in[p]);
            }
}

// dL/dg for the six faces: block f sums -c_f * lambda over face f (x-, x+, y-, y+, z-, z+)
// in a fixed order.
__global__ void __launch_bounds__(1024) k_face_gradients(LevelK<double> L, const double *__restrict__ lam,
                                                         double *__restrict__ out)
{
    __shared__ double sw[32];
    const int f = blockIdx.x;
    const int axis = f >> 1, hi = f & 1;
    const int n1 = axis == 0 ? L.ny : L.nx;
    const int n2 = axis == 2 ? L.ny : L.nz;
    double acc = 0.0;
    for (long long q = threadIdx.x; q < (long long)n1 * n2; q += blockDim.x) {
        const int a = (int)(q % n1) + 1, c = (int)(q / n1) + 1;
        int i, j, k;
        double coef;
        if (axis == 0) {
            i = hi ? L.nx : 1; j = a; k = c;
            coef = hi ? L.cxp[i] : L.cxm[i];
        } else if (axis == 1) {
            i = a; j = hi ? L.ny : 1; k = c;
            coef = hi ? L.cyp[j] : L.cym[j];
        } else {
            i = a; j = c; k = hi ? L.nz : 1;
            coef = hi ? L.czp[k] : L.czm[k];
        }
        acc = __dadd_rn(acc, __dmul_rn(coef, lam[lin(i, j, k, L.sy, L.sz)]));
    }
    const double s = block_sum(acc, sw);
    if (threadIdx.x == 0) out[f] = -s;
}

}  // namespace

int Ctx::adjoint(const double *dLdu, double *dLdb, double *dLdg, int maxit, double tol, double omega,
                 pmg_report_t *rep)
{
    NvtxRange nvtx_range("pmg_adjoint");
    const Level &S = lv[0];
    const size_t bytes = S.total * sizeof(double);
    if (!adj_rhs) {
        // all buffers or none: a failure part way releases what it had allocated, so a
        // later call starts again instead of finding a partial set
        double *a[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
        const size_t sz[5] = {bytes, bytes, bytes, (S.n[0] + S.n[1] + S.n[2] + 6) * sizeof(double),
                              6 * sizeof(double)};
        int st = PMG_OK;
        for (int q = 0; q < 5 && st == PMG_OK; ++q) st = cuda_status(dev_malloc(&a[q], sz[q]), "adjoint allocation");
        if (st == PMG_OK) {
            std::vector<double> h;
            for (int d = 0; d < 3; ++d) h.insert(h.end(), S.dm[d].begin(), S.dm[d].end());
            st = cuda_status(cudaMemcpy(a[3], h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice),
                             "adjoint tables");
        }
        if (st != PMG_OK) {
            for (auto p : a) dev_free(p);
            return st;
        }
        adj_rhs = a[0];
        adj_sol = a[1];
        adj_rsd = a[2];
        adj_vol = a[3];
        adj_faces = a[4];
    }
    const double *dxm = adj_vol, *dym = adj_vol + S.n[0] + 2, *dzm = dym + S.n[1] + 2;
    const dim3 g((S.n[0] + kBX - 1) / kBX, (S.n[1] + kBY - 1) / kBY, std::min(S.n[2], 65535)), bl(kBX, kBY, 1);
    PMG_TRY_A(cuda_status(cudaMemsetAsync(adj_rhs, 0, bytes, stream), "adjoint init"));
    PMG_TRY_A(cuda_status(cudaMemsetAsync(adj_sol, 0, bytes, stream), "adjoint init"));
    k_volume_scale<<<g, bl, 0, stream>>>(S.n[0], S.n[1], S.n[2], S.sy, S.sz, dxm, dym, dzm, dLdu, adj_rhs, 0);
    count_launches(1);
    PMG_TRY_A(cuda_status(cudaGetLastError(), "adjoint rhs"));
    const int rc = precision == PMG_MIXED ? solve_mixed(adj_sol, adj_rsd, adj_rhs, maxit, tol, omega, rep)
                                          : solve_f64(adj_sol, adj_rsd, adj_rhs, maxit, tol, omega, rep);
    if (rc != PMG_OK) return rc;
    PMG_TRY_A(cuda_status(cudaMemsetAsync(dLdb, 0, bytes, stream), "adjoint output"));
    k_volume_scale<<<g, bl, 0, stream>>>(S.n[0], S.n[1], S.n[2], S.sy, S.sz, dxm, dym, dzm, adj_sol, dLdb, 1);
    k_face_gradients<<<6, 1024, 0, stream>>>(K[0], dLdb, adj_faces);
    count_launches(2);
    PMG_TRY_A(cuda_status(cudaGetLastError(), "adjoint gradients"));
    if (dLdg) {
        PMG_TRY_A(cuda_status(cudaMemcpyAsync(dLdg, adj_faces, 6 * sizeof(double), cudaMemcpyDeviceToHost, stream),
                              "adjoint face gradients"));
    }
    return cuda_status(cudaStreamSynchronize(stream), "adjoint sync");
}

}  // namespace pmg
