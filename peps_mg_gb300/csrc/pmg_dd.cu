// pmg_dd.cu -- the CGS V-cycle on a px x py x pz Cartesian decomposition of one grid
// (the reference's MPI execution: src/mpi_topology.f90:53-99, src/geometry.f90:579-660,
// src/multigrid.f90:1907-1976), with every subdomain on this process's GPU.
//
// Each subdomain is a context of its own (its levels, coefficient tables and work arrays),
// built from the global hierarchy's meshes restricted to its cells: the coarse ghost widths
// are then the neighbours' coarse widths, as the reference exchanges them
// (src/multigrid.f90:452-477).  The driver runs the reference's operation sequence on all
// subdomains in turn and exchanges ghost layers where the reference calls
// geometry_halocell_update_selectively: before each RBGS colour
// (src/rbgs_poisson_matrix.f90:237,255 and :116,134), before every mv_mul, hence every
// residual (src/poisson_matrix_operator.f90:131-133), and after the post-smoothing of each
// coarse level (src/multigrid.f90:1961).  An exchange goes axis by axis (x, y, z) with full
// planes, so edge and corner ghosts are current too: a kernel packs a subdomain's boundary
// plane into a contiguous buffer, a cudaMemcpyAsync moves it to the neighbour's receive
// buffer (a peer copy when the neighbour lives on another GPU), and a kernel unpacks it into
// the ghost plane.  Dot products are per-subdomain sums added on the host in rank order (the
// MPI_Allreduce of src/poisson_matrix_operator.f90:68-97); the RBGS colours of a subdomain
// start at the rank-parity offset of src/rbgs_poisson_matrix.f90:230-232.
//
// Because the red-black colours follow the global cell parity and every ghost read is
// current, each cell's arithmetic is the one-grid arithmetic: the solution equals the
// single-context (and the oracle's one-rank) solution bit for bit; only the norms' sums are
// split differently.  The finest post-smoothing uses the finest level's partition flags (the
// reference reads mg_sdm(0) there, one element before that array, src/multigrid.f90:1967).
// Scope: the plain FP64 path with the RBGS coarsest solver and the CGS rules
// (a split axis must halve at every level, src/multigrid.f90:221-299).
//
// Compiled with --fmad=false: the grid kernels it launches are the bitwise FP64 ones.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/peps_mg.h"
#include "pmg_ctx.h"

namespace pmg {

#define PMG_TRY_D(expr)                \
    do {                               \
        int _rc = (expr);              \
        if (_rc != PMG_OK) return _rc; \
    } while (0)

namespace {

constexpr int kT = 256;

// plane `idx` along axis d of a (0:n0+1, 0:n1+1, 0:n2+1) array, every index of the other
// two axes, as a contiguous buffer: pack (to_buf) or unpack
__global__ void k_plane(int d, int n0, int n1, int n2, double *arr, int idx, double *buf, int to_buf)
{
    const long long sy = n0 + 2, sz = (long long)(n0 + 2) * (n1 + 2);
    const int a_n = d == 0 ? n1 + 2 : n0 + 2, b_n = d == 2 ? n1 + 2 : n2 + 2;
    const long long total = (long long)a_n * b_n;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(q % a_n), b = (int)(q / a_n);
        long long p;
        if (d == 0)
            p = idx + sy * a + sz * b;
        else if (d == 1)
            p = a + sy * idx + sz * b;
        else
            p = a + sy * b + sz * idx;
        if (to_buf)
            buf[q] = arr[p];
        else
            arr[p] = buf[q];
    }
}

// a subdomain's (0:n+1)^3 array from the global (0:N+1)^3 array at offset o, ghost layers
// included (scatter)
__global__ void k_scatter(const double *__restrict__ g, int gn0, int gn1, double *__restrict__ loc, int n0, int n1,
                          int n2, int o0, int o1, int o2)
{
    const long long gsy = gn0 + 2, gsz = (long long)(gn0 + 2) * (gn1 + 2);
    const long long sy = n0 + 2, sz = (long long)(n0 + 2) * (n1 + 2);
    const long long total = sz * (n2 + 2);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q % sy), j = (int)((q / sy) % (n1 + 2)), k = (int)(q / sz);
        loc[q] = g[(o0 + i) + gsy * (o1 + j) + gsz * (o2 + k)];
    }
}

// the subdomain's interior back into the global array (gather)
__global__ void k_gather(const double *__restrict__ loc, int n0, int n1, int n2, double *__restrict__ g, int gn0,
                         int gn1, int o0, int o1, int o2)
{
    const long long gsy = gn0 + 2, gsz = (long long)(gn0 + 2) * (gn1 + 2);
    const long long sy = n0 + 2, sz = (long long)(n0 + 2) * (n1 + 2);
    const long long total = (long long)n0 * n1 * n2;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q % n0) + 1, j = (int)((q / n0) % n1) + 1, k = (int)(q / ((long long)n0 * n1)) + 1;
        g[(o0 + i) + gsy * (o1 + j) + gsz * (o2 + k)] = loc[i + sy * j + sz * k];
    }
}

unsigned blocks_for(long long n)
{
    long long b = (n + kT - 1) / kT;
    if (b < 1) b = 1;
    if (b > 4096) b = 4096;
    return (unsigned)b;
}

}  // namespace

struct Dd {
    int p[3] = {1, 1, 1};
    int nr = 1, nl = 0, n_vcycles = 0;
    int gn[3] = {0, 0, 0};
    cudaStream_t stream = nullptr;
    std::vector<std::unique_ptr<Ctx>> rk;
    std::vector<std::array<int, 3>> c;
    std::vector<std::vector<Level>> levels;
    std::vector<double *> sol, rsd, rhs;        // each subdomain's finest arrays
    std::vector<double *> halo;                 // per subdomain: send lo, send hi, recv lo, recv hi
    size_t plane_cap = 0;
    std::vector<int> offset;                    // [r * (nl + 1) + l]
    ~Dd()
    {
        if (stream) cudaStreamSynchronize(stream);
        for (auto v : sol) dev_free(v);
        for (auto v : rsd) dev_free(v);
        for (auto v : rhs) dev_free(v);
        for (auto v : halo) dev_free(v);
    }
    int rank(int cx, int cy, int cz) const { return cx + p[0] * (cy + p[1] * cz); }
};

// The global hierarchy, the multi-rank level-size check and the subdomain of rank
// coordinates `co`: its level sizes and meshes (the global meshes restricted to its cells
// and ghost cells) and its colour offsets.  Host only.
static int dd_subdomain(const pmg_config_t *g, const int p[3], const std::vector<Level> &G, const int co[3],
                        std::vector<Level> &out, std::vector<int> &offs)
{
    const int nl = g->number_of_levels;
    int n[3] = {g->nx / p[0], g->ny / p[1], g->nz / p[2]};
    out.assign((size_t)nl + 1, Level());
    offs.assign((size_t)nl + 1, 0);
    for (int l = 0; l <= nl; ++l) {
        if (l > 0)
            for (int d = 0; d < 3; ++d) {
                if (n[d] % 2 == 0) {
                    n[d] /= 2;
                } else if (p[d] > 1) {
                    set_error("an axis split over several ranks must halve at every level (odd local size " +
                              std::to_string(n[d]) + " at level " + std::to_string(l) + ")");
                    return PMG_EINVAL;
                }
            }
        Level &L = out[l];
        int s = 0;
        for (int d = 0; d < 3; ++d) {
            L.n[d] = n[d];
            if (G[l].n[d] != p[d] * n[d]) {
                set_error("the global hierarchy does not split evenly over the ranks at level " + std::to_string(l));
                return PMG_EINVAL;
            }
            const size_t o = (size_t)co[d] * n[d];
            L.dm[d].assign(G[l].dm[d].begin() + o, G[l].dm[d].begin() + o + n[d] + 2);
            L.dg[d].assign(G[l].dg[d].begin() + o, G[l].dg[d].begin() + o + n[d] + 2);
            L.xg[d].assign(G[l].xg[d].begin() + o, G[l].xg[d].begin() + o + n[d] + 2);
            s += (n[d] % 2) * ((co[d] * (p[d] > 1 ? 1 : 0)) % 2);   // src/rbgs_poisson_matrix.f90:230-232
        }
        offs[l] = s % 2;
    }
    return PMG_OK;
}

static int dd_check(const pmg_config_t *g, const int p[3])
{
    if (!g || !p) {
        set_error("cfg and procs are required");
        return PMG_EINVAL;
    }
    for (int d = 0; d < 3; ++d)
        if (p[d] < 1) {
            set_error("rank counts must be positive");
            return PMG_EINVAL;
        }
    if (g->nx % p[0] || g->ny % p[1] || g->nz % p[2]) {
        set_error("the global sizes must be divisible by the rank counts");
        return PMG_EINVAL;
    }
    if (g->aggregation_method != PMG_CGS || g->precision != PMG_FP64 || g->coarse_solver != PMG_COARSE_RBGS) {
        set_error("the decomposed solve runs the CGS method, plain FP64, with the RBGS coarsest solver");
        return PMG_EINVAL;
    }
    return PMG_OK;
}

int dd_create(Dd **out, const pmg_config_t *g, const int procs[3], cudaStream_t stream)
{
    *out = nullptr;
    PMG_TRY_D(dd_check(g, procs));
    std::vector<Level> G;
    int lvc[3];
    PMG_TRY_D(host_level_meshes(g, G, lvc));
    std::unique_ptr<Dd> D(new (std::nothrow) Dd());
    if (!D) return PMG_ENOMEM;
    for (int d = 0; d < 3; ++d) D->p[d] = procs[d];
    D->nr = procs[0] * procs[1] * procs[2];
    D->nl = g->number_of_levels;
    D->n_vcycles = g->number_of_vcycles;
    D->gn[0] = g->nx;
    D->gn[1] = g->ny;
    D->gn[2] = g->nz;
    D->stream = stream;
    D->levels.resize((size_t)D->nr);
    D->offset.assign((size_t)D->nr * (D->nl + 1), 0);
    for (int cz = 0; cz < procs[2]; ++cz)          // rank numbering: x fastest
        for (int cy = 0; cy < procs[1]; ++cy)
            for (int cx = 0; cx < procs[0]; ++cx) D->c.push_back({cx, cy, cz});
    for (int r = 0; r < D->nr; ++r) {
        std::vector<int> offs;
        PMG_TRY_D(dd_subdomain(g, procs, G, D->c[r].data(), D->levels[r], offs));
        for (int l = 0; l <= D->nl; ++l) D->offset[(size_t)r * (D->nl + 1) + l] = offs[l];
        const std::vector<Level> &Lv = D->levels[r];
        pmg_config_t cfg = *g;
        cfg.nx = Lv[0].n[0];
        cfg.ny = Lv[0].n[1];
        cfg.nz = Lv[0].n[2];
        cfg.dxm = Lv[0].dm[0].data(); cfg.dxg = Lv[0].dg[0].data(); cfg.xg = Lv[0].xg[0].data();
        cfg.dym = Lv[0].dm[1].data(); cfg.dyg = Lv[0].dg[1].data(); cfg.yg = Lv[0].xg[1].data();
        cfg.dzm = Lv[0].dm[2].data(); cfg.dzg = Lv[0].dg[2].data(); cfg.zg = Lv[0].xg[2].data();
        std::unique_ptr<Ctx> c(new (std::nothrow) Ctx());
        if (!c) return PMG_ENOMEM;
        c->preset_levels = &D->levels[r];
        PMG_TRY_D(c->build(&cfg, stream));
        c->preset_levels = nullptr;
        D->rk.push_back(std::move(c));
    }
    // each subdomain's finest arrays and plane buffers (the largest plane of any level)
    const Level &L0 = D->levels[0][0];
    size_t cap = 0;
    for (int d = 0; d < 3; ++d) {
        const size_t a = d == 0 ? L0.n[1] + 2 : L0.n[0] + 2, b = d == 2 ? L0.n[1] + 2 : L0.n[2] + 2;
        cap = std::max(cap, a * b);
    }
    D->plane_cap = cap;
    const size_t tot = D->rk[0]->lv[0].total;
    for (int r = 0; r < D->nr; ++r) {
        double *a[3] = {nullptr, nullptr, nullptr}, *h = nullptr;
        for (int q = 0; q < 3; ++q) {
            PMG_TRY_D(cuda_status(dev_malloc(&a[q], tot * sizeof(double)), "subdomain arrays"));
            (q == 0 ? D->sol : q == 1 ? D->rsd : D->rhs).push_back(a[q]);
        }
        PMG_TRY_D(cuda_status(dev_malloc(&h, 4 * cap * sizeof(double)), "halo buffers"));
        D->halo.push_back(h);
        PMG_TRY_D(cuda_status(cudaMemsetAsync(D->rsd[r], 0, tot * sizeof(double), stream), "subdomain init"));
    }
    *out = D.release();
    return PMG_OK;
}

void dd_destroy(Dd *D) { delete D; }

namespace {

// which: 0 = x (sol at level 0), 1 = b (rhs), 2 = r (rsd)
double *dd_array(Dd &D, int r, int l, int which)
{
    if (l == 0) return which == 0 ? D.sol[r] : which == 1 ? D.rhs[r] : D.rsd[r];
    Level &L = D.rk[r]->lv[l];
    return which == 0 ? L.x : which == 1 ? L.b : L.r;
}

// geometry_halocell_update_selectively of one array of level l on every subdomain
int dd_halo(Dd &D, int l, int which)
{
    const Level &L = D.rk[0]->lv[l];
    const int n[3] = {L.n[0], L.n[1], L.n[2]};
    for (int d = 0; d < 3; ++d) {
        if (D.p[d] == 1) continue;
        const long long plane = (long long)(d == 0 ? n[1] + 2 : n[0] + 2) * (d == 2 ? n[1] + 2 : n[2] + 2);
        for (int r = 0; r < D.nr; ++r) {
            std::array<int, 3> ce = D.c[r];
            if (ce[d] + 1 >= D.p[d]) continue;
            ce[d] += 1;
            const int e = D.rank(ce[0], ce[1], ce[2]);
            double *xr = dd_array(D, r, l, which), *xe = dd_array(D, e, l, which);
            double *send_hi_r = D.halo[r] + D.plane_cap, *recv_hi_r = D.halo[r] + 3 * D.plane_cap;
            double *send_lo_e = D.halo[e], *recv_lo_e = D.halo[e] + 2 * D.plane_cap;
            const unsigned g = blocks_for(plane);
            k_plane<<<g, kT, 0, D.stream>>>(d, n[0], n[1], n[2], xr, n[d], send_hi_r, 1);
            k_plane<<<g, kT, 0, D.stream>>>(d, n[0], n[1], n[2], xe, 1, send_lo_e, 1);
            PMG_TRY_D(cuda_status(cudaMemcpyAsync(recv_lo_e, send_hi_r, plane * sizeof(double),
                                                  cudaMemcpyDeviceToDevice, D.stream),
                                  "halo copy"));
            PMG_TRY_D(cuda_status(cudaMemcpyAsync(recv_hi_r, send_lo_e, plane * sizeof(double),
                                                  cudaMemcpyDeviceToDevice, D.stream),
                                  "halo copy"));
            k_plane<<<g, kT, 0, D.stream>>>(d, n[0], n[1], n[2], xe, 0, recv_lo_e, 0);
            k_plane<<<g, kT, 0, D.stream>>>(d, n[0], n[1], n[2], xr, n[d] + 1, recv_hi_r, 0);
            count_launches(4);
        }
    }
    return cuda_status(cudaGetLastError(), "halo exchange");
}

// rbgs_iterator_poisson_matrix on every subdomain: a halo exchange before each colour
int dd_rbgs(Dd &D, int l, int maxit, double omega)
{
    for (int it = 0; it < maxit; ++it)
        for (int c = 0; c < 2; ++c) {
            PMG_TRY_D(dd_halo(D, l, 0));
            for (int r = 0; r < D.nr; ++r) {
                Ctx &C = *D.rk[r];
                PMG_TRY_D(f64_rbgs_colour(C.K[l], C.launch[l], dd_array(D, r, l, 0), dd_array(D, r, l, 1), omega,
                                          D.offset[(size_t)r * (D.nl + 1) + l] + c, D.stream, C.diag(l)));
            }
        }
    return PMG_OK;
}

// multigrid_residual on every subdomain (halo of x first); with norm, the sum of r^2 over
// the subdomains in rank order
int dd_residual(Dd &D, int l, double *norm)
{
    PMG_TRY_D(dd_halo(D, l, 0));
    for (int r = 0; r < D.nr; ++r) {
        Ctx &C = *D.rk[r];
        if (norm)
            PMG_TRY_D(C.residual_norm(l, dd_array(D, r, l, 2), dd_array(D, r, l, 0), dd_array(D, r, l, 1), 0));
        else
            PMG_TRY_D(f64_residual(C.K[l], C.launch[l], dd_array(D, r, l, 2), dd_array(D, r, l, 0),
                                   dd_array(D, r, l, 1), nullptr, nullptr, D.stream, C.diag(l)));
    }
    if (norm) {
        double s = 0.0;
        for (int r = 0; r < D.nr; ++r) {
            double h = 0.0;
            PMG_TRY_D(D.rk[r]->fetch_scalars(&h, 1));
            s += h;
        }
        *norm = s;
    }
    return PMG_OK;
}

}  // namespace

int dd_solve(Dd &D, double *gsol, double *grsd, const double *grhs, int maxit, double tol, double omega,
             pmg_report_t *rep)
{
    NvtxRange range("pmg_dd_solve");
    const int nl = D.nl, nr = D.nr;
    const Level &L0 = D.rk[0]->lv[0];
    const long long gtot = (long long)(D.gn[0] + 2) * (D.gn[1] + 2) * (D.gn[2] + 2);
    for (int r = 0; r < nr; ++r) {
        const auto &co = D.c[r];
        for (int q = 0; q < 2; ++q)
            k_scatter<<<blocks_for((long long)L0.total), kT, 0, D.stream>>>(
                q == 0 ? gsol : grhs, D.gn[0], D.gn[1], q == 0 ? D.sol[r] : D.rhs[r], L0.n[0], L0.n[1], L0.n[2],
                co[0] * L0.n[0], co[1] * L0.n[1], co[2] * L0.n[2]);
        count_launches(2);
    }
    double res0tol = 0.0, rsd_val = 0.0, ratio = 0.0;
    PMG_TRY_D(dd_residual(D, 0, &res0tol));                                   // :1924-1925
    int cycles = 0, converged = 0;
    for (int cyc = 1; cyc <= D.n_vcycles; ++cyc) {
        if (D.rk[0]->aborted()) return D.rk[0]->abort_status();
        PMG_TRY_D(dd_rbgs(D, 0, maxit, omega));                                // :1931-1933
        PMG_TRY_D(dd_residual(D, 0, nullptr));
        for (int r = 0; r < nr; ++r)
            PMG_TRY_D(f64_restrict(D.rk[r]->X[0], D.rk[r]->launch[1], D.rsd[r], dd_array(D, r, 1, 1), D.stream));
        for (int l = 1; l <= nl - 1; ++l) {                                   // :1936-1941
            for (int r = 0; r < nr; ++r)
                PMG_TRY_D(cuda_status(cudaMemsetAsync(dd_array(D, r, l, 0), 0, D.rk[r]->lv[l].total * sizeof(double),
                                                      D.stream),
                                      "level reset"));
            PMG_TRY_D(dd_rbgs(D, l, maxit, omega));
            PMG_TRY_D(dd_residual(D, l, nullptr));
            for (int r = 0; r < nr; ++r)
                PMG_TRY_D(f64_restrict(D.rk[r]->X[l], D.rk[r]->launch[l + 1], dd_array(D, r, l, 2),
                                       dd_array(D, r, l + 1, 1), D.stream));
        }
        // coarsest level: rbgs_solver_poisson_matrix on every subdomain (:1944-1949,
        // src/rbgs_poisson_matrix.f90:47-179), then its residual, which also updates the
        // ghost layers of x that the first prolongation reads (:1951)
        for (int r = 0; r < nr; ++r)
            PMG_TRY_D(cuda_status(cudaMemsetAsync(dd_array(D, r, nl, 0), 0, D.rk[r]->lv[nl].total * sizeof(double),
                                                  D.stream),
                                  "coarsest reset"));
        double r0 = 0.0, rn = 0.0;
        PMG_TRY_D(dd_residual(D, nl, &r0));
        int it = 0;
        for (it = 0; it < 1000; ++it) {
            PMG_TRY_D(dd_rbgs(D, nl, 1, omega));
            PMG_TRY_D(dd_residual(D, nl, &rn));
            if (std::sqrt(rn / r0) <= tol) break;
        }
        PMG_TRY_D(dd_residual(D, nl, nullptr));
        if (rep && rep->coarse_iterations) rep->coarse_iterations[cyc - 1] = it;
        for (int l = nl - 1; l >= 1; --l) {                                   // :1957-1962
            for (int r = 0; r < nr; ++r)
                PMG_TRY_D(f64_prolong(D.rk[r]->X[l], D.rk[r]->launch[l + 1], dd_array(D, r, l + 1, 0),
                                      dd_array(D, r, l, 0), true, D.stream));
            PMG_TRY_D(dd_rbgs(D, l, maxit, omega));
            PMG_TRY_D(dd_halo(D, l, 0));
        }
        for (int r = 0; r < nr; ++r)                                          // :1965-1967
            PMG_TRY_D(f64_prolong(D.rk[r]->X[0], D.rk[r]->launch[1], dd_array(D, r, 1, 0), D.sol[r], true,
                                  D.stream));
        PMG_TRY_D(dd_rbgs(D, 0, maxit, omega));
        PMG_TRY_D(dd_residual(D, 0, &rsd_val));                               // :1970-1971
        ratio = std::sqrt(rsd_val / res0tol);
        cycles = cyc;
        if (rep && rep->history) {
            rep->history[3 * (cyc - 1) + 0] = std::sqrt(rsd_val);
            rep->history[3 * (cyc - 1) + 1] = std::sqrt(res0tol);
            rep->history[3 * (cyc - 1) + 2] = ratio;
        }
        if (!std::isfinite(rsd_val)) {
            set_error("residual norm is not finite");
            return PMG_EDIVERGED;
        }
        if (ratio < tol) {                                                    // :1973
            converged = 1;
            break;
        }
    }
    PMG_TRY_D(cuda_status(cudaMemsetAsync(grsd, 0, (size_t)gtot * sizeof(double), D.stream), "rsd init"));
    for (int r = 0; r < nr; ++r) {
        const auto &co = D.c[r];
        for (int q = 0; q < 2; ++q)
            k_gather<<<blocks_for((long long)L0.n[0] * L0.n[1] * L0.n[2]), kT, 0, D.stream>>>(
                q == 0 ? D.sol[r] : D.rsd[r], L0.n[0], L0.n[1], L0.n[2], q == 0 ? gsol : grsd, D.gn[0], D.gn[1],
                co[0] * L0.n[0], co[1] * L0.n[1], co[2] * L0.n[2]);
        count_launches(2);
    }
    PMG_TRY_D(cuda_status(cudaStreamSynchronize(D.stream), "decomposed solve"));
    if (rep) {
        rep->cycles = cycles;
        rep->converged = converged;
        rep->res0 = std::sqrt(res0tol);
        rep->final_ratio = ratio;
        rep->inner_cycles = cycles;
    }
    return PMG_OK;
}

// Host-only description of one rank's subdomain (no GPU needed).
int dd_partition(const pmg_config_t *g, const int procs[3], const int coords[3], int level, int dims[3],
                 double *const mesh[9], int *offset)
{
    PMG_TRY_D(dd_check(g, procs));
    if (!coords || level < 0 || level > g->number_of_levels) {
        set_error("invalid rank coordinates or level");
        return PMG_EINVAL;
    }
    for (int d = 0; d < 3; ++d)
        if (coords[d] < 0 || coords[d] >= procs[d]) {
            set_error("rank coordinates out of range");
            return PMG_EINVAL;
        }
    std::vector<Level> G, out;
    std::vector<int> offs;
    int lvc[3];
    PMG_TRY_D(host_level_meshes(g, G, lvc));
    PMG_TRY_D(dd_subdomain(g, procs, G, coords, out, offs));
    const Level &L = out[level];
    if (dims)
        for (int d = 0; d < 3; ++d) dims[d] = L.n[d];
    if (mesh)
        for (int d = 0; d < 3; ++d) {
            if (mesh[3 * d]) std::memcpy(mesh[3 * d], L.dm[d].data(), L.dm[d].size() * sizeof(double));
            if (mesh[3 * d + 1]) std::memcpy(mesh[3 * d + 1], L.dg[d].data(), L.dg[d].size() * sizeof(double));
            if (mesh[3 * d + 2]) std::memcpy(mesh[3 * d + 2], L.xg[d].data(), L.xg[d].size() * sizeof(double));
        }
    if (offset) *offset = offs[level];
    return PMG_OK;
}

}  // namespace pmg

struct pmg_dd {
    pmg::Dd *impl;
};

extern "C" {

int pmg_dd_create(pmg_dd **dd, const pmg_config_t *cfg, const int procs[3], void *stream)
{
    if (!dd) {
        pmg::set_error("dd is required");
        return PMG_EINVAL;
    }
    *dd = nullptr;
    pmg::Dd *d = nullptr;
    const int rc = pmg::guarded([&] { return pmg::dd_create(&d, cfg, procs, static_cast<cudaStream_t>(stream)); });
    if (rc != PMG_OK) return rc;
    pmg_dd *h = new (std::nothrow) pmg_dd{d};
    if (!h) {
        pmg::dd_destroy(d);
        return PMG_ENOMEM;
    }
    *dd = h;
    return PMG_OK;
}

int pmg_dd_solve(pmg_dd *dd, double *sol, double *rsd, const double *rhs, int maxiteration, double tolerance,
                 double omega_sor, pmg_report_t *report)
{
    if (!dd || !sol || !rsd || !rhs || maxiteration < 0) {
        pmg::set_error("invalid decomposed solve arguments");
        return PMG_EINVAL;
    }
    return pmg::guarded([&] { return pmg::dd_solve(*dd->impl, sol, rsd, rhs, maxiteration, tolerance, omega_sor, report); });
}

int pmg_dd_destroy(pmg_dd *dd)
{
    if (!dd) return PMG_OK;
    pmg::dd_destroy(dd->impl);
    delete dd;
    return PMG_OK;
}

int pmg_dd_partition(const pmg_config_t *cfg, const int procs[3], const int coords[3], int level, int dims[3],
                     double *const mesh[9], int *offset)
{
    return pmg::dd_partition(cfg, procs, coords, level, dims, mesh, offset);
}

}  // extern "C"
