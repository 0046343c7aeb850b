// pmg_api.cu -- host side of the library: the level hierarchy, the per-level
// coefficient and transfer tables, the device state, the FP64 V-cycle driver and the
// C-ABI entry points declared in include/peps_mg.h.
//
// Host arithmetic that feeds the kernels (mesh coarsening, coefficient tables,
// transfer weights) is compiled with -ffp-contract=off and follows the reference
// expressions cited beside it, so the tables hold exactly the values the reference
// computes inline.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/peps_mg.h"
#include "pmg_ctx.h"

namespace pmg {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int cuda_status(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return PMG_OK;
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? PMG_ENOMEM : PMG_ECUDA;
}

// Host-side fault injection of device allocations: -1 = off; n >= 0 = the n-th next
// dev_malloc call (0 = the next one) fails once.
static std::atomic<long long> g_alloc_fail_countdown{-1};

struct DevArena {
    std::vector<std::pair<char *, size_t>> chunks;
    char *cur = nullptr;
    size_t left = 0;
};
static std::mutex g_arena_mu;
static std::vector<DevArena *> g_arenas;           // live arenas (dev_free's ownership test)
static thread_local DevArena *t_arena = nullptr;   // the arena of the thread's ArenaScope

DevArena *arena_create()
{
    DevArena *a = new (std::nothrow) DevArena();
    if (!a) return nullptr;
    std::lock_guard<std::mutex> g(g_arena_mu);
    g_arenas.push_back(a);
    return a;
}

void arena_destroy(DevArena *a)
{
    if (!a) return;
    {
        std::lock_guard<std::mutex> g(g_arena_mu);
        g_arenas.erase(std::remove(g_arenas.begin(), g_arenas.end(), a), g_arenas.end());
    }
    for (auto &c : a->chunks) cudaFree(c.first);
    delete a;
}

ArenaScope::ArenaScope(DevArena *a) : prev(t_arena) { t_arena = a; }
ArenaScope::~ArenaScope() { t_arena = prev; }

cudaError_t dev_malloc_bytes(void **p, size_t bytes)
{
    long long c = g_alloc_fail_countdown.load();
    while (c >= 0) {
        if (g_alloc_fail_countdown.compare_exchange_weak(c, c - 1)) {
            if (c == 0) {
                *p = nullptr;
                return cudaErrorMemoryAllocation;
            }
            break;
        }
    }
    DevArena *a = t_arena;
    if (!a) return cudaMalloc(p, bytes);
    const size_t need = (bytes + 255) & ~(size_t)255;
    if (need > a->left) {
        const size_t chunk = std::max(need, (size_t)256 << 20);
        void *m = nullptr;
        const cudaError_t e = cudaMalloc(&m, chunk);
        if (e != cudaSuccess) {
            *p = nullptr;
            return e;
        }
        std::lock_guard<std::mutex> g(g_arena_mu);
        a->chunks.push_back({static_cast<char *>(m), chunk});
        a->cur = static_cast<char *>(m);
        a->left = chunk;
    }
    *p = a->cur;
    a->cur += need;
    a->left -= need;
    return cudaSuccess;
}

cudaError_t dev_free(void *p)
{
    if (!p) return cudaSuccess;
    {
        std::lock_guard<std::mutex> g(g_arena_mu);
        const char *q = static_cast<const char *>(p);
        for (const DevArena *a : g_arenas)
            for (const auto &c : a->chunks)
                if (q >= c.first && q < c.first + c.second) return cudaSuccess;
    }
    return cudaFree(p);
}

static std::atomic<long long> g_launches{0};
void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches_total() { return g_launches.load(); }

Profiler::~Profiler()
{
    for (auto e : pool) cudaEventDestroy(e);
    for (auto &r : pending) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
}

void Profiler::reset()
{
    for (int c = 0; c < PC_COUNT; ++c) {
        total_ms[c] = 0.0;
        count[c] = 0;
        bytes[c] = 0.0;
    }
}

cudaEvent_t Profiler::get()
{
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

int Profiler::begin(cudaStream_t s)
{
    if (!on) return -1;
    Rec r{0, 0, 0.0, get(), get()};
    cudaEventRecord(r.a, s);
    pending.push_back(r);
    return (int)pending.size() - 1;
}

void Profiler::end(int idx, int cls, int launches, double bytes_per_launch, cudaStream_t s)
{
    if (idx < 0 || !on) return;
    Rec &r = pending[idx];
    r.cls = cls;
    r.launches = launches;
    r.bytes = bytes_per_launch;
    cudaEventRecord(r.b, s);
}

void Profiler::flush()
{
    for (auto &r : pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            total_ms[r.cls] += ms;
            count[r.cls] += r.launches;
            bytes[r.cls] += r.bytes * r.launches;
        } else {
            cudaGetLastError();
        }
        pool.push_back(r.a);
        pool.push_back(r.b);
    }
    pending.clear();
}

#define PMG_TRY(expr)                      \
    do {                                   \
        int _rc = (expr);                  \
        if (_rc != PMG_OK) return _rc;     \
    } while (0)

#define PMG_CUDA(expr, what) PMG_TRY(cuda_status((expr), (what)))

// ---------------------------------------------------------------------------------
// Level-size rules at one rank (CGS src/multigrid.f90:221-309, CGA :541-740, CGPSA
// :1029-1201 with its aggregation levels forced to 0 at one rank, :1032-1036).
// ---------------------------------------------------------------------------------
int level_sizes(const int n0[3], int n_levels, int method, int cga_level, std::vector<std::array<int, 3>> &sizes,
                int lvc[3])
{
    if (n_levels <= 1 || n_levels >= kMaxLevels) {
        set_error("number_of_levels must be larger than 1 (and below the library limit)");
        return PMG_EINVAL;
    }
    int n[3] = {n0[0], n0[1], n0[2]};
    lvc[0] = lvc[1] = lvc[2] = 0;
    sizes.assign((size_t)n_levels + 1, {0, 0, 0});
    sizes[0] = {n[0], n[1], n[2]};
    if (method == PMG_CGS) {
        if (cga_level != 0) {
            set_error("Aggregation level should be 0 for CGS method");
            return PMG_EINVAL;
        }
        for (int l = 1; l <= n_levels; ++l)
            for (int d = 0; d < 3; ++d) {
                if (n[d] % 2 == 0) {
                    n[d] /= 2;
                    lvc[d] = l;
                }
                sizes[l][d] = n[d];
            }
        if (n_levels > std::max(lvc[0], std::max(lvc[1], lvc[2]))) {
            set_error("Number of levels is greater than the coarsest level in global domain");
            return PMG_EINVAL;
        }
    } else if (method == PMG_CGA) {
        if (cga_level == 0) {
            set_error("Aggregation level should be larger than 0");
            return PMG_EINVAL;
        }
        for (int l = 1; l <= n_levels; ++l) {
            for (int d = 0; d < 3; ++d) {
                if (l <= cga_level) {
                    if (n[d] % 2 == 1) {
                        set_error("grid coarsening impossible at or before the aggregation level (odd size)");
                        return PMG_EINVAL;
                    }
                    sizes[l][d] = n[d] / 2;
                    if (l == cga_level) lvc[d] = l;
                } else if (n[d] % 2 == 1) {
                    sizes[l][d] = n[d];
                } else {
                    sizes[l][d] = n[d] / 2;
                    lvc[d] = l;
                }
            }
            for (int d = 0; d < 3; ++d) n[d] = sizes[l][d];
            if (((long long)n[0] * n[1] * n[2]) % 2 == 1) break;
        }
        if (n_levels > std::max(lvc[0], std::max(lvc[1], lvc[2]))) {
            set_error("Number of levels is greater than the coarsest level in global domain");
            return PMG_EINVAL;
        }
    } else if (method == PMG_CGPSA) {
        for (int l = 1; l <= n_levels; ++l) {
            for (int d = 0; d < 3; ++d) {
                if (n[d] % 2 == 1) {
                    sizes[l][d] = n[d];
                } else {
                    sizes[l][d] = n[d] / 2;
                    lvc[d] = l;
                }
            }
            for (int d = 0; d < 3; ++d) n[d] = sizes[l][d];
            if (((long long)n[0] * n[1] * n[2]) % 2 == 1) break;
        }
        if (n_levels != std::max(lvc[0], std::max(lvc[1], lvc[2]))) {
            set_error("Number of levels should be equal to the coarsest level in global domain");
            return PMG_EINVAL;
        }
    } else {
        set_error("Aggregation method should be 0, 1, or 2");
        return PMG_EINVAL;
    }
    return PMG_OK;
}

// Mesh of a coarse level along one axis (src/multigrid.f90:450-491 and :872-987).
static void coarsen_axis(int method, int agg_level, int n, const std::vector<double> &dm_f,
                         const std::vector<double> &dg_f, const std::vector<double> &xg_f, double ox, int lv,
                         int lv_coarsest, std::vector<double> &dm, std::vector<double> &dg, std::vector<double> &xg)
{
    dm.assign((size_t)n + 2, 0.0);
    dg.assign((size_t)n + 2, 0.0);
    xg.assign((size_t)n + 2, 0.0);
    if (lv <= lv_coarsest) {
        for (int i = 1; i <= n; ++i) dm[i] = dm_f[2 * i - 1] + dm_f[2 * i];
        dm[0] = dm_f[0];
        dm[n + 1] = dm_f[2 * n + 1];
        double x0;
        if (method == PMG_CGS || (method == PMG_CGA && lv <= agg_level))
            x0 = ox - 0.5 * dm[0];
        else
            x0 = (xg_f[0] + 0.5 * dm_f[0]) - 0.5 * dm[0];
        xg[0] = x0;
        for (int i = 1; i <= n; ++i) {
            dg[i] = 0.5 * (dm[i] + dm[i - 1]);
            xg[i] = xg[i - 1] + dg[i];
        }
        dg[n + 1] = 0.5 * (dm[n + 1] + dm[n]);
        xg[n + 1] = xg[n] + dg[n + 1];
    } else {
        dm = dm_f;
        dg = dg_f;
        xg = xg_f;
    }
}

// ---------------------------------------------------------------------------------
// Device tables
// ---------------------------------------------------------------------------------
static void axis_coeff_tables(const std::vector<double> &dm, const std::vector<double> &dg, int n,
                              std::vector<double> &cm, std::vector<double> &cp, std::vector<double> &s)
{
    cm.assign((size_t)n + 2, 0.0);
    cp.assign((size_t)n + 2, 0.0);
    s.assign((size_t)n + 2, 0.0);
    for (int i = 1; i <= n; ++i) {
        cm[i] = 1.0 / (dm[i] * dg[i]);        // dxmp2i, src/matrix.f90:75
        cp[i] = 1.0 / (dm[i] * dg[i + 1]);    // dxmn2i, src/matrix.f90:76
        s[i] = cm[i] + cp[i];                 // first partial sum of c0, src/matrix.f90:82
    }
}

// Restriction weight dxf on the fine index (src/multigrid.f90:1415-1425).
static void restrict_weights(const std::vector<double> &dm_c, const std::vector<double> &dm_f, int nf, bool stride1,
                             std::vector<double> &w)
{
    w.assign((size_t)nf + 2, 0.0);
    if (stride1) {
        w = dm_f;
    } else {
        for (int i = 1; i <= nf; ++i) w[i] = dm_c[(i - 1) / 2 + 1] - dm_f[i];
    }
}

// Prolongation weights dxp/dxn on the fine index (src/multigrid.f90:1594-1612).
static void prolong_weights(const std::vector<double> &dm_c, const std::vector<double> &dm_f, int nc, int nf,
                            bool stride1, std::vector<double> &dp, std::vector<double> &dn)
{
    dp.assign((size_t)nf + 2, 0.0);
    dn.assign((size_t)nf + 2, 0.0);
    if (stride1) {
        dp = dm_c;
        dn = dm_c;
        dp.resize((size_t)nf + 2, 0.0);
        dn.resize((size_t)nf + 2, 0.0);
    } else {
        for (int i = 1; i <= nc; ++i) {
            const int f = 2 * i;
            dp[f - 1] = 1.0 * dm_f[f - 2] + 0.5 * dm_f[f - 1];
            dp[f] = 0.5 * dm_f[f - 1];
            dn[f - 1] = 0.5 * dm_f[f];
            dn[f] = 1.0 * dm_f[f + 1] + 0.5 * dm_f[f];
        }
    }
}

// ---------------------------------------------------------------------------------
// Context life cycle
// ---------------------------------------------------------------------------------
static int validate_mesh(const pmg_config_t *c)
{
    if (!c->dxm || !c->dxg || !c->dym || !c->dyg || !c->dzm || !c->dzg) {
        set_error("mesh arrays dxm/dxg/dym/dyg/dzm/dzg are required");
        return PMG_EINVAL;
    }
    if (c->nx < 1 || c->ny < 1 || c->nz < 1) {
        set_error("nx, ny, nz must be positive");
        return PMG_EINVAL;
    }
    if ((long long)(c->nx + 2) * (c->ny + 2) >= (1LL << 31)) {
        set_error("plane of the grid is too large");
        return PMG_EINVAL;
    }
    return PMG_OK;
}

// The level hierarchy's sizes and meshes at one rank (multigrid_subdomain_create_CGS /
// _CGA / _CGPSA, src/multigrid.f90:167-495, 503-990, 998-1288): level 0 is the caller's
// mesh, every coarser one from coarsen_axis.  Host only.
int host_level_meshes(const pmg_config_t *c, std::vector<Level> &lv, int lvc[3])
{
    const int nl = c->number_of_levels, method = c->aggregation_method, cga_level = c->cga_level;
    const int n0[3] = {c->nx, c->ny, c->nz};
    std::vector<std::array<int, 3>> sizes;
    PMG_TRY(level_sizes(n0, nl, method, cga_level, sizes, lvc));
    lv.assign((size_t)nl + 1, Level());
    const double *fm[3] = {c->dxm, c->dym, c->dzm}, *fg[3] = {c->dxg, c->dyg, c->dzg}, *fx[3] = {c->xg, c->yg, c->zg};
    double o[3];
    for (int l = 0; l <= nl; ++l) {
        Level &L = lv[l];
        for (int d = 0; d < 3; ++d) L.n[d] = sizes[l][d];
        L.sy = L.n[0] + 2;
        L.sz = (long long)(L.n[0] + 2) * (L.n[1] + 2);
        L.total = (size_t)L.sz * (size_t)(L.n[2] + 2);
        for (int d = 0; d < 3; ++d) {
            const int n = L.n[d];
            if (l == 0) {
                L.dm[d].assign(fm[d], fm[d] + n + 2);
                L.dg[d].assign(fg[d], fg[d] + n + 2);
                if (fx[d])
                    L.xg[d].assign(fx[d], fx[d] + n + 2);
                else {
                    // cell centres from the widths when the caller gives none
                    L.xg[d].assign((size_t)n + 2, 0.0);
                    for (int i = 1; i <= n + 1; ++i) L.xg[d][i] = L.xg[d][i - 1] + L.dg[d][i];
                }
                o[d] = L.xg[d][1] - 0.5 * L.dm[d][1];   // sdm%ox, src/geometry.f90:378-380
            } else {
                const Level &F = lv[l - 1];
                coarsen_axis(method, cga_level, n, F.dm[d], F.dg[d], F.xg[d], o[d], l, lvc[d], L.dm[d], L.dg[d],
                             L.xg[d]);
            }
        }
    }
    return PMG_OK;
}

// PEPS_MG_HOST_SETUP=1: coarse meshes and tables computed on the host as well (the same
// expressions), for checking the device set-up against it
bool host_setup()
{
    const char *e = std::getenv("PEPS_MG_HOST_SETUP");
    return e && std::strcmp(e, "1") == 0;
}

// The coarse meshes (unless lv holds every level's mesh already) and the per-axis
// coefficient tables and transfer weights of every level, built on the device by one
// launch (hierarchy_setup) into d_tables; the meshes and tables are copied back for the
// host-side uses (level queries, the FP32 tables of the mixed path).  The layout: per level
// and axis cm, cp (and sx for x), then per transfer and axis w, pp, pn, each table padded to
// an even length (16-byte alignment).
int Ctx::setup_tables()
{
    const bool meshes_given = preset_levels || host_setup();
    HierDesc H;
    std::memset(&H, 0, sizeof(H));
    H.nl = nl;
    H.method = method;
    H.agg_level = cga_level;
    H.meshes_given = meshes_given ? 1 : 0;
    long long mo = 0, to = 0;
    auto tab = [&](int n) {
        const long long o = to;
        to += n + 2 + ((n + 2) & 1);
        return o;
    };
    for (int d = 0; d < 3; ++d) {
        H.lvc[d] = lvc[d];
        H.ox[d] = lv[0].xg[d][1] - 0.5 * lv[0].dm[d][1];   // sdm%ox, src/geometry.f90:378-380
    }
    for (int l = 0; l <= nl; ++l) {
        for (int d = 0; d < 3; ++d) {
            H.n[l][d] = lv[l].n[d];
            H.mesh_off[l][d] = mo;
            mo += 3LL * (lv[l].n[d] + 2);
        }
        for (int d = 0; d < 3; ++d) {
            H.cm[l][d] = tab(lv[l].n[d]);
            H.cp[l][d] = tab(lv[l].n[d]);
            if (d == 0) H.sx[l] = tab(lv[l].n[d]);
        }
        if (l < nl)
            for (int d = 0; d < 3; ++d) {
                H.w[l][d] = tab(lv[l].n[d]);
                H.pp[l][d] = tab(lv[l].n[d]);
                H.pn[l][d] = tab(lv[l].n[d]);
            }
    }
    std::vector<double> hm((size_t)mo, 0.0);
    for (int l = 0; l <= (meshes_given ? nl : 0); ++l)
        for (int d = 0; d < 3; ++d) {
            double *p = hm.data() + H.mesh_off[l][d];
            const size_t m = (size_t)lv[l].n[d] + 2;
            std::memcpy(p, lv[l].dm[d].data(), m * sizeof(double));
            std::memcpy(p + m, lv[l].dg[d].data(), m * sizeof(double));
            std::memcpy(p + 2 * m, lv[l].xg[d].data(), m * sizeof(double));
        }
    double *d_meshes = nullptr;
    HierDesc *d_hier = nullptr;
    PMG_CUDA(dev_malloc(&d_tables, (size_t)to * sizeof(double)), "table allocation");
    int rc = cuda_status(dev_malloc(&d_meshes, (size_t)mo * sizeof(double)), "set-up allocation");
    if (rc == PMG_OK) rc = cuda_status(dev_malloc(&d_hier, sizeof(HierDesc)), "set-up allocation");
    if (rc == PMG_OK)
        rc = cuda_status(cudaMemcpyAsync(d_meshes, hm.data(), hm.size() * sizeof(double), cudaMemcpyHostToDevice,
                                         stream),
                         "mesh upload");
    if (rc == PMG_OK)
        rc = cuda_status(cudaMemcpyAsync(d_hier, &H, sizeof(H), cudaMemcpyHostToDevice, stream), "set-up upload");
    if (rc == PMG_OK)
        rc = cuda_status(cudaMemsetAsync(d_tables, 0, (size_t)to * sizeof(double), stream), "table init");
    if (rc == PMG_OK) rc = hierarchy_setup(d_hier, d_meshes, d_tables, stream);
    tables_host.assign((size_t)to, 0.0);
    if (rc == PMG_OK)
        rc = cuda_status(cudaMemcpyAsync(hm.data(), d_meshes, hm.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                         stream),
                         "mesh download");
    if (rc == PMG_OK)
        rc = cuda_status(cudaMemcpyAsync(tables_host.data(), d_tables, (size_t)to * sizeof(double),
                                         cudaMemcpyDeviceToHost, stream),
                         "table download");
    if (rc == PMG_OK) rc = cuda_status(cudaStreamSynchronize(stream), "hierarchy set-up");
    dev_free(d_meshes);
    dev_free(d_hier);
    if (rc != PMG_OK) return rc;
    if (!meshes_given)
        for (int l = 1; l <= nl; ++l)
            for (int d = 0; d < 3; ++d) {
                const double *p = hm.data() + H.mesh_off[l][d];
                const size_t m = (size_t)lv[l].n[d] + 2;
                lv[l].dm[d].assign(p, p + m);
                lv[l].dg[d].assign(p + m, p + 2 * m);
                lv[l].xg[d].assign(p + 2 * m, p + 3 * m);
            }

    K.resize((size_t)nl + 1);
    X.resize((size_t)nl);
    for (int l = 0; l <= nl; ++l) {
        const Level &L = lv[l];
        LevelK<double> &k = K[l];
        k.nx = L.n[0]; k.ny = L.n[1]; k.nz = L.n[2];
        k.sy = L.sy; k.sz = L.sz;
        k.cxm = d_tables + H.cm[l][0]; k.cxp = d_tables + H.cp[l][0]; k.sx = d_tables + H.sx[l];
        k.cym = d_tables + H.cm[l][1]; k.cyp = d_tables + H.cp[l][1];
        k.czm = d_tables + H.cm[l][2]; k.czp = d_tables + H.cp[l][2];
        if (l < nl) {
            const Level &C = lv[l + 1];
            XferK<double> &x = X[l];
            x.ncx = C.n[0]; x.ncy = C.n[1]; x.ncz = C.n[2];
            x.csy = C.sy; x.csz = C.sz;
            x.fsy = L.sy; x.fsz = L.sz;
            x.stx = l >= lvc[0] ? 1 : 2;
            x.sty = l >= lvc[1] ? 1 : 2;
            x.stz = l >= lvc[2] ? 1 : 2;
            x.wx = d_tables + H.w[l][0]; x.wy = d_tables + H.w[l][1]; x.wz = d_tables + H.w[l][2];
            x.pxp = d_tables + H.pp[l][0]; x.pxn = d_tables + H.pn[l][0];
            x.pyp = d_tables + H.pp[l][1]; x.pyn = d_tables + H.pn[l][1];
            x.pzp = d_tables + H.pp[l][2]; x.pzn = d_tables + H.pn[l][2];
        }
    }
    if (host_setup()) {
        // the host computation of the same tables, for checking the device set-up
        std::vector<double> hb((size_t)to, 0.0);
        for (int l = 0; l <= nl; ++l) {
            for (int d = 0; d < 3; ++d) {
                std::vector<double> cm, cp, sxv;
                axis_coeff_tables(lv[l].dm[d], lv[l].dg[d], lv[l].n[d], cm, cp, sxv);
                std::copy(cm.begin(), cm.end(), hb.begin() + H.cm[l][d]);
                std::copy(cp.begin(), cp.end(), hb.begin() + H.cp[l][d]);
                if (d == 0) std::copy(sxv.begin(), sxv.end(), hb.begin() + H.sx[l]);
            }
            if (l < nl)
                for (int d = 0; d < 3; ++d) {
                    const bool s1 = l >= lvc[d];
                    std::vector<double> w, dp, dn;
                    restrict_weights(lv[l + 1].dm[d], lv[l].dm[d], lv[l].n[d], s1, w);
                    prolong_weights(lv[l + 1].dm[d], lv[l].dm[d], lv[l + 1].n[d], lv[l].n[d], s1, dp, dn);
                    std::copy(w.begin(), w.end(), hb.begin() + H.w[l][d]);
                    std::copy(dp.begin(), dp.end(), hb.begin() + H.pp[l][d]);
                    std::copy(dn.begin(), dn.end(), hb.begin() + H.pn[l][d]);
                }
        }
        if (std::memcmp(hb.data(), tables_host.data(), hb.size() * sizeof(double)) != 0) {
            set_error("device-built tables differ from the host-built ones");
            return PMG_ECUDA;
        }
    }
    return PMG_OK;
}

int Ctx::build(const pmg_config_t *c, cudaStream_t s)
{
    PMG_TRY(validate_mesh(c));
    if (c->number_of_vcycles < 0) {
        set_error("number_of_vcycles must be non-negative");
        return PMG_EINVAL;
    }
    if (c->coarse_solver != PMG_COARSE_RBGS && c->coarse_solver != PMG_COARSE_CG) {
        set_error("coarse_solver must be PMG_COARSE_RBGS or PMG_COARSE_CG");
        return PMG_EINVAL;
    }
    if (c->precision != PMG_FP64 && c->precision != PMG_MIXED && c->precision != PMG_FP64_FAST) {
        set_error("precision must be PMG_FP64, PMG_MIXED or PMG_FP64_FAST");
        return PMG_EINVAL;
    }
    stream = s;
    nl = c->number_of_levels;
    n_vcycles = c->number_of_vcycles;
    method = c->aggregation_method;
    cga_level = c->cga_level;
    for (int d = 0; d < 3; ++d) cgpsa_level[d] = c->cgpsa_level[d];
    coarse_solver = c->coarse_solver;
    precision = c->precision;
    mixed_inner = c->mixed_inner_cycles;
    if (mixed_inner < 0) {
        set_error("mixed_inner_cycles must be non-negative");
        return PMG_EINVAL;
    }
    if (preset_levels) {
        // the levels of a subdomain of a decomposed solve: sizes and meshes given (the
        // global hierarchy's meshes restricted to the subdomain, ghost widths from the
        // neighbours); an axis was coarsened up to the last level that halved it
        if ((int)preset_levels->size() != nl + 1) {
            set_error("preset levels do not match number_of_levels");
            return PMG_EINVAL;
        }
        lv = *preset_levels;
        lvc[0] = lvc[1] = lvc[2] = 0;
        for (int l = 1; l <= nl; ++l)
            for (int d = 0; d < 3; ++d)
                if (2 * lv[l].n[d] == lv[l - 1].n[d]) lvc[d] = l;
        for (auto &L : lv) {
            L.sy = L.n[0] + 2;
            L.sz = (long long)(L.n[0] + 2) * (L.n[1] + 2);
            L.total = (size_t)L.sz * (size_t)(L.n[2] + 2);
            L.x = L.b = L.r = nullptr;
        }
    } else if (host_setup()) {
        PMG_TRY(host_level_meshes(c, lv, lvc));
    } else {
        // level sizes here, the coarse meshes on the device (setup_tables)
        const int n0[3] = {c->nx, c->ny, c->nz};
        std::vector<std::array<int, 3>> sizes;
        PMG_TRY(level_sizes(n0, nl, method, cga_level, sizes, lvc));
        lv.assign((size_t)nl + 1, Level());
        const double *fm[3] = {c->dxm, c->dym, c->dzm}, *fg[3] = {c->dxg, c->dyg, c->dzg};
        const double *fx[3] = {c->xg, c->yg, c->zg};
        for (int l = 0; l <= nl; ++l) {
            Level &L = lv[l];
            for (int d = 0; d < 3; ++d) L.n[d] = sizes[l][d];
            L.sy = L.n[0] + 2;
            L.sz = (long long)(L.n[0] + 2) * (L.n[1] + 2);
            L.total = (size_t)L.sz * (size_t)(L.n[2] + 2);
        }
        for (int d = 0; d < 3; ++d) {
            const int n = lv[0].n[d];
            lv[0].dm[d].assign(fm[d], fm[d] + n + 2);
            lv[0].dg[d].assign(fg[d], fg[d] + n + 2);
            if (fx[d]) {
                lv[0].xg[d].assign(fx[d], fx[d] + n + 2);
            } else {
                lv[0].xg[d].assign((size_t)n + 2, 0.0);
                for (int i = 1; i <= n + 1; ++i) lv[0].xg[d][i] = lv[0].xg[d][i - 1] + lv[0].dg[d][i];
            }
        }
    }
    // finest widths are checked before any device work; coarse ones after the set-up
    for (int d = 0; d < 3; ++d)
        for (int i = 1; i <= lv[0].n[d]; ++i)
            if (!(lv[0].dm[d][i] > 0.0) || !(lv[0].dg[d][i] > 0.0) || !(lv[0].dg[d][i + 1] > 0.0)) {
                set_error("mesh widths and spacings of interior cells must be positive");
                return PMG_EINVAL;
            }
    PMG_TRY(setup_tables());
    for (int l = 1; l <= nl; ++l)
        for (int d = 0; d < 3; ++d)
            for (int i = 1; i <= lv[l].n[d]; ++i)
                if (!(lv[l].dm[d][i] > 0.0) || !(lv[l].dg[d][i] > 0.0) || !(lv[l].dg[d][i + 1] > 0.0)) {
                    set_error("mesh widths and spacings of interior cells must be positive");
                    return PMG_EINVAL;
                }

    // ---- execution mapping --------------------------------------------------------
    // CGS: every level on the full grid; the coarsest solve in the single-CTA kernel.
    // CGA: from CGA_level on, the whole coarse tail runs in one CTA (the reference
    //      gathers everything onto rank 0 there, src/multigrid.f90:2095-2135).
    // CGPSA: an axis is collapsed to one CTA column from its CGPSA_level on (the
    //      reference aggregates that axis there); once all three are collapsed the
    //      rest of the tail runs in the single-CTA kernel.
    launch.assign((size_t)nl + 1, Launch{{false, false, false}});
    tail_l0 = nl;
    if (method == PMG_CGA) {
        tail_l0 = std::min(std::max(cga_level, 1), nl);
    } else if (method == PMG_CGPSA) {
        bool every_axis = true;
        int last = 0;
        for (int d = 0; d < 3; ++d) {
            if (cgpsa_level[d] > 0) {
                for (int l = cgpsa_level[d]; l <= nl; ++l) launch[l].collapse[d] = true;
                last = std::max(last, cgpsa_level[d]);
            } else {
                every_axis = false;
            }
        }
        if (every_axis) tail_l0 = std::min(last, nl);
    }
    // A level too large for one CTA is kept on the grid kernels.
    while (tail_l0 <= nl && lv[tail_l0].total > kTailMaxCells) ++tail_l0;
    // Tail block size: about two cells per thread at the largest tail level (barriers of
    // a 1024-thread CTA dominate the coarsest solve of a few cells).
    {
        long long cells = 1;
        for (int l = tail_l0; l <= nl; ++l) cells = std::max(cells, (long long)lv[l].n[0] * lv[l].n[1] * lv[l].n[2]);
        tail_threads = (int)std::min<long long>(1024, std::max<long long>(64, ((cells / 2 + 31) / 32) * 32));
    }

    // ---- device arrays -------------------------------------------------------------
    size_t max_part = 1;
    for (int l = 1; l <= nl; ++l) {
        Level &L = lv[l];
        PMG_CUDA(dev_malloc(&L.x, L.total * sizeof(double)), "level allocation");
        PMG_CUDA(dev_malloc(&L.b, L.total * sizeof(double)), "level allocation");
        PMG_CUDA(dev_malloc(&L.r, L.total * sizeof(double)), "level allocation");
        PMG_CUDA(cudaMemset(L.x, 0, L.total * sizeof(double)), "level init");
        PMG_CUDA(cudaMemset(L.b, 0, L.total * sizeof(double)), "level init");
        PMG_CUDA(cudaMemset(L.r, 0, L.total * sizeof(double)), "level init");
    }
    for (int l = 0; l <= nl; ++l) {
        dim3 g, b;
        grid_for_cells(K[l], launch[l], &g, &b);
        max_part = std::max(max_part, (size_t)g.x * g.y * g.z);
    }
    npart_cap = max_part;
    PMG_CUDA(dev_malloc(&d_partials, npart_cap * sizeof(double)), "scratch allocation");
    PMG_CUDA(dev_malloc(&d_scal, 16 * sizeof(double)), "scratch allocation");
    PMG_CUDA(dev_malloc(&d_iscal, 16 * sizeof(int)), "scratch allocation");
    PMG_CUDA(dev_malloc(&d_cg, sizeof(CgState)), "scratch allocation");
    PMG_CUDA(cudaMemset(d_cg, 0, sizeof(CgState)), "scratch init");
    if (!light) {
        void *h = nullptr, *d = nullptr;
        PMG_CUDA(cudaHostAlloc(&h, sizeof(int), cudaHostAllocMapped), "abort flag allocation");
        abort_host = static_cast<int *>(h);
        *abort_host = 0;
        PMG_CUDA(cudaHostGetDevicePointer(&d, h, 0), "abort flag mapping");
        abort_dev = static_cast<const int *>(d);
    }
    PMG_CUDA(cudaMemset(d_iscal, 0, 16 * sizeof(int)), "scratch init");
    {
        const Level &C = lv[nl];
        for (double **p : {&d_cp, &d_cap, &d_crr}) {
            PMG_CUDA(dev_malloc(p, C.total * sizeof(double)), "coarse scratch");
            PMG_CUDA(cudaMemset(*p, 0, C.total * sizeof(double)), "coarse scratch");
        }
    }
    PMG_CUDA(dev_malloc(&d_tail, sizeof(TailDesc<double>)), "tail descriptor");
    if (!light) {
        PMG_CUDA(cudaEventCreate(&ev0), "event");
        PMG_CUDA(cudaEventCreate(&ev1), "event");
        PMG_CUDA(cudaEventCreateWithFlags(&ev_x, cudaEventDisableTiming), "event");
        PMG_CUDA(cudaEventCreateWithFlags(&ev_copied, cudaEventDisableTiming), "event");
        PMG_CUDA(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking), "copy stream");
    }
    if (precision == PMG_FP64_FAST) PMG_TRY(setup_fast64());
    if (precision == PMG_FP64) {
        // per-cell diagonal tables of the plain FP64 path (the grid kernels read c0 instead
        // of summing five 1-D table entries per cell; the values are diag_f64's bits)
        c0t.assign((size_t)nl + 1, nullptr);
        for (int l = 0; l <= nl; ++l) {
            PMG_CUDA(dev_malloc(&c0t[l], lv[l].total * sizeof(double)), "diagonal table");
            PMG_CUDA(cudaMemsetAsync(c0t[l], 0, lv[l].total * sizeof(double), stream), "diagonal table");
            PMG_TRY(f64_diag_table(K[l], c0t[l], stream));
        }
        // complete before any other stream (a decomposed solve's) reads the tables
        PMG_CUDA(cudaStreamSynchronize(stream), "diagonal table");
    }
    return PMG_OK;
}

// Tables of the FP64 performance mode for the grid levels 0 .. min(tail_l0, nl) - 1 (the
// levels the V-cycle runs on the grid kernels): one blob of per-axis tables, derived on
// the device from the plain path's tables, and one omega/c0 array per level.
int Ctx::setup_fast64()
{
    fast64 = true;
    const int grid_end = std::min(tail_l0, nl);
    fastK.assign((size_t)std::max(grid_end, 1), FastLevelK{});
    fastX.assign((size_t)std::max(grid_end, 1), FastXferK{});
    size_t total = 0;
    std::vector<size_t> lvl_off((size_t)grid_end + 1, 0);
    for (int l = 0; l < grid_end; ++l) {
        lvl_off[l] = total;
        const Level &L = lv[l];
        total += (size_t)(L.n[1] + 2) + (size_t)(L.n[2] + 2) + 3 * (size_t)(L.n[0] + 2 + L.n[1] + 2 + L.n[2] + 2);
    }
    PMG_CUDA(dev_malloc(&d_fast, std::max<size_t>(total, 1) * sizeof(double)), "fast tables");
    for (int l = 0; l < grid_end; ++l) {
        const Level &L = lv[l];
        double *p = d_fast + lvl_off[l];
        FastLevelK &F = fastK[l];
        FastXferK &W = fastX[l];
        F.dy = p;
        p += L.n[1] + 2;
        F.dz = p;
        p += L.n[2] + 2;
        double **ax[3][3] = {{&W.rx, &W.pax, &W.pbx}, {&W.ry, &W.pay, &W.pby}, {&W.rz, &W.paz, &W.pbz}};
        for (int d = 0; d < 3; ++d)
            for (int t = 0; t < 3; ++t) {
                *ax[d][t] = p;
                p += L.n[d] + 2;
            }
        double *w = nullptr;
        PMG_CUDA(dev_malloc(&w, L.total * sizeof(double)), "fast diagonal");
        fast_wdiag_alloc.push_back(w);
        F.wdiag = w;
        PMG_TRY(fast_tables(K[l], &X[l], L.n[0], L.n[1], L.n[2], &F, &W, stream));
    }
    PMG_CUDA(cudaStreamSynchronize(stream), "fast tables");
    fast_omega_set = false;
    return PMG_OK;
}

// omega / c0 of the fast mode's grid levels for this solve's omega.
int Ctx::fast_prepare(double omega)
{
    if (fast_omega_set && fast_omega == omega) return PMG_OK;
    const int grid_end = std::min(tail_l0, nl);
    for (int l = 0; l < grid_end; ++l) PMG_TRY(fast_wdiag(K[l], omega, fastK[l].wdiag, stream));
    fast_omega = omega;
    fast_omega_set = true;
    return PMG_OK;
}

Ctx::~Ctx()
{
    for (auto &L : lv) {
        dev_free(L.x);
        dev_free(L.b);
        dev_free(L.r);
    }
    dev_free(d_tables);
    for (auto p : c0t) dev_free(p);
    dev_free(d_partials);
    dev_free(d_scal);
    dev_free(d_iscal);
    dev_free(d_cg);
    if (abort_host) cudaFreeHost(abort_host);
    dev_free(d_fast);
    for (auto p : fast_wdiag_alloc) dev_free(p);
    dev_free(d_cp);
    dev_free(d_cap);
    dev_free(d_crr);
    dev_free(d_tail);
    dev_free(stage_sol);
    dev_free(stage_rsd);
    dev_free(stage_rhs);
    for (auto &v : scratch_levels) dev_free(v);
    dev_free(adj_rhs);
    dev_free(adj_sol);
    dev_free(adj_rsd);
    dev_free(adj_vol);
    dev_free(adj_faces);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (ev_x) cudaEventDestroy(ev_x);
    if (ev_copied) cudaEventDestroy(ev_copied);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    destroy_mixed();
}

// Sum of x*y (or of r^2 from residual partials) into d_scal[slot].
int Ctx::dot(int l, const double *x, const double *y, int slot)
{
    int np = 0;
    PMG_TRY(f64_dot_partials(K[l], launch[l], x, y, d_partials, &np, stream));
    return f64_reduce(d_partials, np, d_scal + slot, stream);
}

int Ctx::residual_norm(int l, double *r, const double *x, const double *b, int slot)
{
    int np = 0;
    PMG_TRY(f64_residual(K[l], launch[l], r, x, b, d_partials, &np, stream, diag(l)));
    return f64_reduce(d_partials, np, d_scal + slot, stream);
}

// The finest-level residual and its norm of an FP64 solve: bitwise, or in the FP64
// performance mode its FMA form.
int Ctx::solve_residual_norm(double *r, const double *x, const double *b, int slot)
{
    if (!fast64) return residual_norm(0, r, x, b, slot);
    int np = 0;
    PMG_TRY(fast_residual(K[0], fastK[0], launch[0], r, x, b, d_partials, &np, stream));
    return f64_reduce(d_partials, np, d_scal + slot, stream);
}

int Ctx::fetch_scalars(double *h, int n)
{
    PMG_CUDA(cudaMemcpyAsync(h, d_scal, sizeof(double) * n, cudaMemcpyDeviceToHost, stream), "scalar read");
    PMG_CUDA(cudaStreamSynchronize(stream), "stream sync");
    return PMG_OK;
}

// Upload the tail descriptor for levels l0..nl.
int Ctx::upload_tail(int l0, int maxit, double omega, double tol)
{
    TailDesc<double> &D = tail_host;
    std::memset(&D, 0, sizeof(D));
    D.l0 = l0;
    D.nl = nl;
    D.maxit = maxit;
    D.coarse_solver = coarse_solver;
    D.coarse_maxit = 1000;   // src/multigrid.f90:1948
    D.omega = omega;
    D.omw = 1.0 - omega;
    D.tol = tol;
    D.p = d_cp;
    D.ap = d_cap;
    D.rr = d_crr;
    D.iters_out = d_iscal + 1;
    for (int l = 0; l <= nl; ++l) {
        D.L[l] = K[l];
        if (l < nl) D.X[l] = X[l];
        D.x[l] = lv[l].x;
        D.b[l] = lv[l].b;
        D.r[l] = lv[l].r;
    }
    fill_coarse64(D.C64, D.cx64, D.cb64, D.cp64, D.cap64, D.crr64, D.omega64, D.omw64, omega);
    D.abort = abort_dev;
    PMG_CUDA(cudaMemcpyAsync(d_tail, &D, sizeof(D), cudaMemcpyHostToDevice, stream), "tail descriptor upload");
    return PMG_OK;
}

void Ctx::fill_coarse64(LevelK<double> &C, double *&x, double *&b, double *&p, double *&ap, double *&rr, double &om,
                        double &omw, double omega) const
{
    C = K[nl];
    x = lv[nl].x;
    b = lv[nl].b;
    p = d_cp;
    ap = d_cap;
    rr = d_crr;
    om = omega;
    omw = 1.0 - omega;
}

// Coarsest-level solve with the grid kernels (a coarsest level too large for one CTA).
int Ctx::coarse_solve_grid(double tol, double omega, int *iters)
{
    Level &C = lv[nl];
    PMG_CUDA(cudaMemsetAsync(C.x, 0, C.total * sizeof(double), stream), "coarse init");
    if (coarse_solver == PMG_COARSE_CG) return cg_dev(nl, C.x, C.b, 1000, tol, true, iters, nullptr);
    return rbgs_solver_dev(nl, C.x, C.b, 1000, tol, omega, iters, nullptr);
}

// One V-cycle from the finest level (src/multigrid.f90:1931-1967), FP64.
int Ctx::vcycle_f64(double *sol, double *rsd, const double *rhs, int maxit, double omega, double tol,
                    int *coarse_iters)
{
    NvtxRange cycle_range(fast64 ? "fp64-fast V-cycle" : "fp64 V-cycle");
    const double N = (double)K[0].nx * K[0].ny * K[0].nz;
    const int grid_end = std::min(tail_l0, nl);
    // the grid levels' operations: bitwise kernels, or those of the FP64 performance mode
    // (which stores omega/c0: 4 more bytes per updated cell and half-sweep)
    const bool fast = fast64;
    auto sweeps = [&](int l, double *x, const double *b) {
        return fast ? fast_rbgs_sweeps(K[l], fastK[l], launch[l], x, b, maxit, omega, stream)
                    : f64_rbgs_sweeps(K[l], launch[l], x, b, maxit, omega, stream, diag(l));
    };
    auto resid = [&](int l, double *r, const double *x, const double *b) {
        return fast ? fast_residual(K[l], fastK[l], launch[l], r, x, b, nullptr, nullptr, stream)
                    : f64_residual(K[l], launch[l], r, x, b, nullptr, nullptr, stream, diag(l));
    };
    auto restr = [&](int l, const double *vf, double *vc) {
        return fast ? fast_restrict(X[l], fastX[l], launch[l + 1], vf, vc, stream)
                    : f64_restrict(X[l], launch[l + 1], vf, vc, stream);
    };
    auto prolong = [&](int l, const double *vc, double *vf) {
        return fast ? fast_prolong(X[l], fastX[l], launch[l + 1], vc, vf, stream)
                    : f64_prolong(X[l], launch[l + 1], vc, vf, true, stream);
    };
    // algorithmic bytes per cell: a half-sweep reads x and half of b and writes half of x
    // (16 B), plus half a diagonal value (4 B) where one is stored per cell (the performance
    // mode's omega/c0, the plain path's c0); the residual 24 B, plus 8 B of the stored c0
    const bool tab = !fast && diag(0);
    const double sweep_bytes = (fast || tab) ? 20.0 : 16.0, resid_bytes = tab ? 32.0 : 24.0;
    int pi = prof.begin(stream);
    {
        NvtxRange r("pre-smoothing");
        PMG_TRY(sweeps(0, sol, rhs));
    }
    prof.end(pi, PC_SMOOTH64, 2 * maxit, sweep_bytes * N, stream);
    NvtxRange down_range("residual, restriction, coarse levels, tail, prolongation");
    pi = prof.begin(stream);
    PMG_TRY(resid(0, rsd, sol, rhs));
    prof.end(pi, PC_RES64, 1, resid_bytes * N, stream);
    pi = prof.begin(stream);
    PMG_TRY(restr(0, rsd, lv[1].b));
    prof.end(pi, PC_RESTRICT64, 1, 9.0 * N, stream);
    // grid levels below the finest, one profiler record each way: per cell of level l,
    // sweep_bytes per half-sweep, resid_bytes residual, 9 B restriction (down); 17 B
    // prolongation + add, sweep_bytes per half-sweep (up)
    auto coarse_bytes = [&](bool down) {
        double b = 0.0;
        for (int l = 1; l < grid_end; ++l) {
            const double n = (double)K[l].nx * K[l].ny * K[l].nz;
            b += down ? (2.0 * sweep_bytes * maxit + resid_bytes + 9.0) * n : (17.0 + 2.0 * sweep_bytes * maxit) * n;
        }
        return b;
    };
    const int coarse_launches = std::max(0, grid_end - 1) * (2 * maxit + 2);
    int pc = grid_end > 1 ? prof.begin(stream) : -1;
    for (int l = 1; l < grid_end; ++l) {
        Level &L = lv[l];
        PMG_CUDA(cudaMemsetAsync(L.x, 0, L.total * sizeof(double), stream), "level reset");
        PMG_TRY(sweeps(l, L.x, L.b));
        PMG_TRY(resid(l, L.r, L.x, L.b));
        PMG_TRY(restr(l, L.r, lv[l + 1].b));
    }
    if (coarse_launches > 0) prof.end(pc, PC_COARSE64, coarse_launches, coarse_bytes(true) / coarse_launches, stream);
    if (tail_l0 <= nl) {
        pi = prof.begin(stream);
        PMG_TRY(f64_tail(d_tail, tail_threads, stream));
        prof.end(pi, PC_TAIL64, 1, 0.0, stream);
        if (coarse_iters) {
            int h = 0;
            PMG_CUDA(cudaMemcpyAsync(&h, d_iscal + 1, sizeof(int), cudaMemcpyDeviceToHost, stream), "iters");
            PMG_CUDA(cudaStreamSynchronize(stream), "sync");
            *coarse_iters = h;
        }
    } else {
        PMG_TRY(coarse_solve_grid(tol, omega, coarse_iters));
    }
    pc = grid_end > 1 ? prof.begin(stream) : -1;
    for (int l = grid_end - 1; l >= 1; --l) {
        Level &L = lv[l];
        PMG_TRY(prolong(l, lv[l + 1].x, L.x));
        PMG_TRY(sweeps(l, L.x, L.b));
    }
    const int up_launches = std::max(0, grid_end - 1) * (2 * maxit + 1);
    if (up_launches > 0) prof.end(pc, PC_COARSE64, up_launches, coarse_bytes(false) / up_launches, stream);
    pi = prof.begin(stream);
    PMG_TRY(prolong(0, lv[1].x, sol));
    prof.end(pi, PC_PROLONG64, 1, 17.0 * N, stream);
    pi = prof.begin(stream);
    {
        NvtxRange r("post-smoothing");
        PMG_TRY(sweeps(0, sol, rhs));
    }
    prof.end(pi, PC_SMOOTH64, 2 * maxit, sweep_bytes * N, stream);
    return PMG_OK;
}

// Status of a solve that stopped because the abort flag was set.
int Ctx::abort_status()
{
    set_error("stopped by the abort flag (pmg_set_abort)");
    return PMG_ETIMEOUT;
}

int Ctx::solve_f64(double *sol, double *rsd, const double *rhs, int maxit, double tol, double omega,
                   pmg_report_t *rep)
{
    const Level &S = lv[0];
    // rsd(:,:,:) = 0 then r = b - A x (src/multigrid.f90:1794-1805, :1924-1925)
    PMG_CUDA(cudaMemsetAsync(rsd, 0, S.total * sizeof(double), stream), "rsd init");
    if (fast64) PMG_TRY(fast_prepare(omega));
    PMG_TRY(solve_residual_norm(rsd, sol, rhs, 0));
    double h[2];
    PMG_TRY(fetch_scalars(h, 1));
    const double res0tol = h[0];
    if (res0tol == 0.0) {
        // An exactly zero initial residual (e.g. rhs = 0 and sol = 0): sol already solves
        // the system, so the solve returns at once with sol unchanged, rsd = b - A x, no
        // cycles and ratio 0.  The reference divides by the zero norm instead
        // (src/multigrid.f90:1973) and runs all its cycles on NaN ratios; for rhs = 0,
        // sol = 0 those leave sol = 0 as well.
        if (rep) {
            rep->cycles = 0;
            rep->converged = 1;
            rep->res0 = 0.0;
            rep->final_ratio = 0.0;
            rep->inner_cycles = 0;
        }
        return PMG_OK;
    }
    if (tail_l0 <= nl) PMG_TRY(upload_tail(tail_l0, maxit, omega, tol));
    int cycles = 0, converged = 0;
    double ratio = 0.0;
    for (int cyc = 1; cyc <= n_vcycles; ++cyc) {
        if (aborted()) {
            if (rep) {
                rep->cycles = cycles;
                rep->converged = 0;
                rep->res0 = std::sqrt(res0tol);
                rep->final_ratio = ratio;
                rep->inner_cycles = cycles;
            }
            return abort_status();
        }
        int ci = 0;
        PMG_TRY(vcycle_f64(sol, rsd, rhs, maxit, omega, tol, rep && rep->coarse_iterations ? &ci : nullptr));
        int pr = prof.begin(stream);
        PMG_TRY(solve_residual_norm(rsd, sol, rhs, 1));  // :1970-1971
        prof.end(pr, PC_RES64, 1, (!fast64 && diag(0) ? 32.0 : 24.0) * (double)K[0].nx * K[0].ny * K[0].nz, stream);
        PMG_TRY(fetch_scalars(h, 2));
        const double rsd_val = h[1];
        ratio = std::sqrt(rsd_val / res0tol);
        cycles = cyc;
        if (rep) {
            if (rep->history) {
                rep->history[3 * (cyc - 1) + 0] = std::sqrt(rsd_val);
                rep->history[3 * (cyc - 1) + 1] = std::sqrt(res0tol);
                rep->history[3 * (cyc - 1) + 2] = ratio;
            }
            if (rep->coarse_iterations) rep->coarse_iterations[cyc - 1] = ci;
        }
        if (!std::isfinite(rsd_val)) {
            if (rep) {
                rep->cycles = cycles;
                rep->converged = 0;
                rep->res0 = std::sqrt(res0tol);
                rep->final_ratio = ratio;
            }
            set_error("residual norm is not finite");
            return PMG_EDIVERGED;
        }
        if (ratio < tol) {                                 // :1973
            converged = 1;
            break;
        }
    }
    if (rep) {
        rep->cycles = cycles;
        rep->converged = converged;
        rep->res0 = std::sqrt(res0tol);
        rep->final_ratio = ratio;
        rep->inner_cycles = cycles;
    }
    return PMG_OK;
}

// ---------------------------------------------------------------------------------
// Device-looped solvers for the lower API (any level size)
// ---------------------------------------------------------------------------------
int Ctx::level_scratch(int l, double **bufs, int count)
{
    // count full-size arrays of level l, zero-initialised (ghosts stay zero)
    const size_t need = lv[l].total * (size_t)count;
    if (scratch_cap < need) {
        for (auto &v : scratch_levels) dev_free(v);
        scratch_levels.clear();
        double *p = nullptr;
        PMG_CUDA(dev_malloc(&p, need * sizeof(double)), "scratch allocation");
        scratch_levels.push_back(p);
        scratch_cap = need;
    }
    PMG_CUDA(cudaMemsetAsync(scratch_levels[0], 0, need * sizeof(double), stream), "scratch init");
    for (int q = 0; q < count; ++q) bufs[q] = scratch_levels[0] + (size_t)q * lv[l].total;
    return PMG_OK;
}

// rbgs_solver_poisson_matrix (src/rbgs_poisson_matrix.f90:47-179)
int Ctx::rbgs_solver_dev(int l, double *x, const double *b, int maxit, double tol, double omega, int *iters,
                         double *ratio_out)
{
    double *rs;
    PMG_TRY(level_scratch(l, &rs, 1));
    PMG_TRY(residual_norm(l, rs, x, b, 2));
    double h[4];
    PMG_TRY(fetch_scalars(h, 3));
    const double r0 = h[2];
    double rn = r0;
    int it = 0;
    for (it = 0; it < maxit; ++it) {
        if (aborted()) return abort_status();
        PMG_TRY(f64_rbgs_sweeps(K[l], launch[l], x, b, 1, omega, stream, diag(l)));
        PMG_TRY(residual_norm(l, rs, x, b, 3));
        PMG_TRY(fetch_scalars(h, 4));
        rn = h[3];
        if (std::sqrt(rn / r0) <= tol) break;
    }
    if (iters) *iters = it;
    if (ratio_out) *ratio_out = std::sqrt(rn / r0);
    return PMG_OK;
}

// cg_solver_poisson_matrix / cg_iterator_poisson_matrix (src/cg_poisson_matrix.f90) with
// the fused kernels of pmg_f64.cu: the scalars stay on the device, and the solver reads
// the exit flag once every kCgCheckEvery iterations (iterations queued after the exit
// return at once).
int Ctx::cg_dev(int l, double *x, const double *b, int maxit, double tol, bool check, int *iters,
                double *ratio_out)
{
    constexpr int kCgCheckEvery = 8;
    double *bufs[3];
    PMG_TRY(level_scratch(l, bufs, 3));
    double *p = bufs[0], *ap = bufs[1], *rs = bufs[2];
    if ((size_t)f64_cg_partials(K[l], launch[l]) > npart_cap) {
        set_error("cg: partial-sum buffer too small for the level");
        return PMG_EINVAL;
    }
    PMG_TRY(f64_cg_init(K[l], launch[l], rs, p, x, b, d_partials, d_cg, stream, diag(l)));
    CgState h{};
    for (int it0 = 0; it0 < maxit; it0 += kCgCheckEvery) {
        if (aborted()) return abort_status();
        const int it1 = std::min(maxit, it0 + kCgCheckEvery);
        for (int it = it0; it < it1; ++it)
            PMG_TRY(f64_cg_iteration(K[l], launch[l], x, rs, p, ap, d_partials, d_cg, tol, check, it, stream,
                                     diag(l)));
        if (check && it1 < maxit) {
            PMG_CUDA(cudaMemcpyAsync(&h, d_cg, sizeof(h), cudaMemcpyDeviceToHost, stream), "cg state read");
            PMG_CUDA(cudaStreamSynchronize(stream), "stream sync");
            if (h.done) break;
        }
    }
    PMG_CUDA(cudaMemcpyAsync(&h, d_cg, sizeof(h), cudaMemcpyDeviceToHost, stream), "cg state read");
    PMG_CUDA(cudaStreamSynchronize(stream), "stream sync");
    if (iters) *iters = h.done ? h.iter : maxit;
    if (ratio_out) *ratio_out = check ? std::sqrt(h.t2 / h.r0) : std::sqrt(h.t2);
    return PMG_OK;
}

// Stage host buffers through the device when the caller passes host memory.
static bool is_device_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Page-locked (registered or cudaHostAlloc'ed) host memory: copies to it are asynchronous.
static bool is_pinned_host_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Pageable host buffers of one solve, page-locked for the duration of the call
// (cudaHostRegister): their copies then run as DMA at the host link's rate and the
// solution's early copy-back applies, where pageable copies measured 35-200 GB/s depending
// on the pages' state.  All or none: a buffer that cannot be registered (for instance one
// that shares pages with another) leaves every buffer pageable.  The destructor waits for
// both streams before it unregisters.
struct HostRegistration {
    std::vector<void *> regs;
    cudaStream_t s1 = nullptr, s2 = nullptr;
    HostRegistration(void *const *bufs, int n, size_t bytes, cudaStream_t a, cudaStream_t b) : s1(a), s2(b)
    {
        const char *env = std::getenv("PEPS_MG_NO_HOST_REGISTER");
        if (env && env[0] == '1') return;
        for (int q = 0; q < n; ++q) {
            cudaPointerAttributes at;
            if (cudaPointerGetAttributes(&at, bufs[q]) == cudaSuccess && at.type == cudaMemoryTypeHost) continue;
            cudaGetLastError();
            if (cudaHostRegister(bufs[q], bytes, cudaHostRegisterDefault) != cudaSuccess) {
                cudaGetLastError();
                release();
                return;
            }
            regs.push_back(bufs[q]);
        }
    }
    void release()
    {
        if (regs.empty()) return;
        if (s2) cudaStreamSynchronize(s2);
        if (s1) cudaStreamSynchronize(s1);
        for (void *p : regs) cudaHostUnregister(p);
        cudaGetLastError();
        regs.clear();
    }
    ~HostRegistration() { release(); }
};

// True when every 64-bit word of the host array is zero (+0.0 everywhere, ghosts
// included: the test of the device-side zero test, k_nonzero_f64).  Scanned by up to 8
// host threads, at most half the cores (a scan thread that has to wait for a core holds
// up the whole solve), each stopping at the first non-zero word it sees or once another
// thread has found one; a solve from a zero initial guess then sends no initial guess over
// the host link at all (the staging buffer is cleared on the device instead), and the scan
// runs while the right-hand side is being copied.
static bool host_all_zero(const double *a, size_t n)
{
    const unsigned long long *u = reinterpret_cast<const unsigned long long *>(a);
    std::atomic<bool> found{false};
    auto scan = [&](size_t b, size_t e) {
        size_t q = b;
        while (q < e && !found.load(std::memory_order_relaxed)) {
            const size_t stop = std::min(e, q + 4096);
            unsigned long long bits = 0;
            for (; q < stop; ++q) bits |= u[q];
            if (bits) found.store(true, std::memory_order_relaxed);
        }
    };
    const size_t per_thread = (size_t)1 << 23;   // 64 MB
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = (unsigned)std::min<size_t>(std::min(8u, std::max(1u, hw / 2)), std::max<size_t>(1, n / per_thread));
    if (nt <= 1) {
        scan(0, n);
        return !found.load();
    }
    std::vector<std::thread> th;
    const size_t chunk = (n + nt - 1) / nt;
    unsigned started = 1;
    try {
        for (; started < nt; ++started)
            th.emplace_back(scan, std::min(n, started * chunk), std::min(n, (started + 1) * chunk));
    } catch (...) {
        // no thread to be had: the remaining chunks are scanned here (no exception may
        // leave the C interface)
    }
    scan(0, std::min(n, chunk));
    for (unsigned t = started; t < nt; ++t) scan(std::min(n, t * chunk), std::min(n, (t + 1) * chunk));
    for (auto &x : th) x.join();
    return !found.load();
}

int Ctx::early_copy_sol(const double *sol)
{
    if (!early_sol_host) return PMG_OK;
    PMG_CUDA(cudaEventRecord(ev_x, stream), "event");
    PMG_CUDA(cudaStreamWaitEvent(copy_stream, ev_x, 0), "event");
    PMG_CUDA(cudaMemcpyAsync(early_sol_host, sol, lv[0].total * sizeof(double), cudaMemcpyDeviceToHost, copy_stream),
             "D2H");
    PMG_CUDA(cudaEventRecord(ev_copied, copy_stream), "event");
    early_pending = early_valid = true;
    return PMG_OK;
}

int Ctx::before_x_change()
{
    if (early_pending) PMG_CUDA(cudaStreamWaitEvent(stream, ev_copied, 0), "event");
    early_pending = early_valid = false;
    return PMG_OK;
}

int Ctx::solve(double *sol, double *rsd, const double *rhs, int maxit, double tol, double omega, pmg_report_t *rep)
{
    NvtxRange solve_range("pmg_solve_vcycle");
    if (!sol || !rsd || !rhs) {
        set_error("sol, rsd and rhs are required");
        return PMG_EINVAL;
    }
    if (maxit < 0) {
        set_error("maxiteration must be non-negative");
        return PMG_EINVAL;
    }
    const bool dev = is_device_ptr(sol);
    if (dev != is_device_ptr(rhs) || dev != is_device_ptr(rsd)) {
        set_error("sol, rsd and rhs must all be device memory or all host memory");
        return PMG_EINVAL;
    }
    const size_t bytes = lv[0].total * sizeof(double);
    void *const host_bufs[3] = {sol, rsd, const_cast<double *>(rhs)};
    HostRegistration host_reg(host_bufs, dev ? 0 : 3, bytes, stream, copy_stream);
    PMG_CUDA(cudaEventRecord(ev0, stream), "event");
    double *s = sol, *r = rsd;
    const double *b = rhs;
    if (!dev) {
        if (!stage_sol) {
            // all three or none: a failed allocation leaves no partial set behind
            double *a[3] = {nullptr, nullptr, nullptr};
            for (int q = 0; q < 3; ++q) {
                const int st = cuda_status(dev_malloc(&a[q], bytes), "staging allocation");
                if (st != PMG_OK) {
                    for (int u = 0; u < q; ++u) dev_free(a[u]);
                    return st;
                }
            }
            stage_sol = a[0];
            stage_rsd = a[1];
            stage_rhs = a[2];
        }
        // the right-hand side first; the initial guess only if it is not all zero (tested
        // on the host while the right-hand side is on its way)
        PMG_CUDA(cudaMemcpyAsync(stage_rhs, rhs, bytes, cudaMemcpyHostToDevice, stream), "H2D");
        x0_known_zero = host_all_zero(sol, lv[0].total);
        if (x0_known_zero)
            PMG_CUDA(cudaMemsetAsync(stage_sol, 0, bytes, stream), "staging init");
        else
            PMG_CUDA(cudaMemcpyAsync(stage_sol, sol, bytes, cudaMemcpyHostToDevice, stream), "H2D");
        s = stage_sol;
        r = stage_rsd;
        b = stage_rhs;
        if (is_pinned_host_ptr(sol)) early_sol_host = sol;
    }
    early_valid = early_pending = false;
    int rc = precision == PMG_MIXED ? solve_mixed(s, r, b, maxit, tol, omega, rep)
                                    : solve_f64(s, r, b, maxit, tol, omega, rep);
    x0_known_zero = false;
    early_sol_host = nullptr;
    if (rc != PMG_OK && rc != PMG_EDIVERGED) {
        if (early_pending) cudaStreamWaitEvent(stream, ev_copied, 0);
        cudaStreamSynchronize(stream);
        early_valid = early_pending = false;
        return rc;
    }
    if (!dev) {
        if (early_valid) {
            // the residual follows the solution's copy on the copy stream (one transfer
            // at a time over the link)
            PMG_CUDA(cudaEventRecord(ev_x, stream), "event");
            PMG_CUDA(cudaStreamWaitEvent(copy_stream, ev_x, 0), "event");
            PMG_CUDA(cudaMemcpyAsync(rsd, stage_rsd, bytes, cudaMemcpyDeviceToHost, copy_stream), "D2H");
            PMG_CUDA(cudaEventRecord(ev_copied, copy_stream), "event");
            PMG_CUDA(cudaStreamWaitEvent(stream, ev_copied, 0), "event");
        } else {
            PMG_CUDA(cudaMemcpyAsync(sol, stage_sol, bytes, cudaMemcpyDeviceToHost, stream), "D2H");
            PMG_CUDA(cudaMemcpyAsync(rsd, stage_rsd, bytes, cudaMemcpyDeviceToHost, stream), "D2H");
        }
    } else if (early_pending) {
        PMG_CUDA(cudaStreamWaitEvent(stream, ev_copied, 0), "event");
    }
    early_valid = early_pending = false;
    PMG_CUDA(cudaEventRecord(ev1, stream), "event");
    PMG_CUDA(cudaEventSynchronize(ev1), "event sync");
    prof.flush();
    if (rep) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev0, ev1);
        rep->elapsed_ms = ms;
    }
    return rc;
}

}  // namespace pmg

// =====================================================================================
// C-ABI
// =====================================================================================
using pmg::Ctx;
using pmg::cuda_status;

struct pmg_ctx {
    Ctx impl;
};

static int check_ctx_level(const pmg_ctx *c, int level)
{
    if (!c) {
        pmg::set_error("null context");
        return PMG_EINVAL;
    }
    if (level < 0 || level > c->impl.nl) {
        pmg::set_error("level out of range");
        return PMG_EINVAL;
    }
    return PMG_OK;
}

extern "C" {

int pmg_create(pmg_ctx **ctx, const pmg_config_t *cfg, void *stream)
{
    if (!ctx || !cfg) {
        pmg::set_error("ctx and cfg are required");
        return PMG_EINVAL;
    }
    *ctx = nullptr;
    pmg::NvtxRange r("pmg_create");
    pmg_ctx *c = new (std::nothrow) pmg_ctx();
    if (!c) return PMG_ENOMEM;
    const int rc = pmg::guarded([&] { return c->impl.build(cfg, (cudaStream_t)stream); });
    if (rc != PMG_OK) {
        delete c;
        return rc;
    }
    *ctx = c;
    return PMG_OK;
}

int pmg_destroy(pmg_ctx *ctx)
{
    if (!ctx) return PMG_OK;
    cudaStreamSynchronize(ctx->impl.stream);
    delete ctx;
    return PMG_OK;
}

int pmg_solve_vcycle(pmg_ctx *ctx, double *sol, double *rsd, const double *rhs, int maxiteration, double tolerance,
                     double omega_sor, pmg_report_t *report)
{
    if (!ctx) {
        pmg::set_error("null context");
        return PMG_EINVAL;
    }
    return pmg::guarded([&] { return ctx->impl.solve(sol, rsd, rhs, maxiteration, tolerance, omega_sor, report); });
}

int pmg_level_sizes(int nx, int ny, int nz, int n_levels, int aggregation_method, int cga_level, int *sizes,
                    int lv_coarsest[3])
{
    if (!sizes || !lv_coarsest) {
        pmg::set_error("sizes and lv_coarsest are required");
        return PMG_EINVAL;
    }
    if (nx < 1 || ny < 1 || nz < 1) {
        pmg::set_error("nx, ny, nz must be positive");
        return PMG_EINVAL;
    }
    const int n0[3] = {nx, ny, nz};
    std::vector<std::array<int, 3>> sz;
    PMG_TRY(pmg::level_sizes(n0, n_levels, aggregation_method, cga_level, sz, lv_coarsest));
    for (size_t l = 0; l < sz.size(); ++l)
        for (int d = 0; d < 3; ++d) sizes[3 * l + d] = sz[l][d];
    return PMG_OK;
}

int pmg_level_dims(const pmg_ctx *ctx, int level, int dims[3])
{
    PMG_TRY(check_ctx_level(ctx, level));
    for (int d = 0; d < 3; ++d) dims[d] = ctx->impl.lv[level].n[d];
    return PMG_OK;
}

int pmg_level_mesh(const pmg_ctx *ctx, int level, int axis, double *dm, double *dg, double *xg)
{
    PMG_TRY(check_ctx_level(ctx, level));
    if (axis < 0 || axis > 2) {
        pmg::set_error("axis out of range");
        return PMG_EINVAL;
    }
    const auto &L = ctx->impl.lv[level];
    const size_t n = L.dm[axis].size();
    if (dm) std::memcpy(dm, L.dm[axis].data(), n * sizeof(double));
    if (dg) std::memcpy(dg, L.dg[axis].data(), n * sizeof(double));
    if (xg) std::memcpy(xg, L.xg[axis].data(), n * sizeof(double));
    return PMG_OK;
}

int pmg_coarsest_levels(const pmg_ctx *ctx, int lv_coarsest[3])
{
    PMG_TRY(check_ctx_level(ctx, 0));
    for (int d = 0; d < 3; ++d) lv_coarsest[d] = ctx->impl.lvc[d];
    return PMG_OK;
}

int pmg_mv_mul(pmg_ctx *ctx, int level, double *y, const double *x)
{
    PMG_TRY(check_ctx_level(ctx, level));
    Ctx &c = ctx->impl;
    const auto &L = c.lv[level];
    // y = 0 everywhere, then the interior (src/poisson_matrix_operator.f90:136-159)
    PMG_TRY(pmg::zero_ghosts_f64(y, L.n[0], L.n[1], L.n[2], c.stream));
    return pmg::f64_mv_mul(c.K[level], c.launch[level], y, x, c.stream, c.diag(level));
}

int pmg_vv_dot(pmg_ctx *ctx, int level, const double *x, const double *y, double *result)
{
    PMG_TRY(check_ctx_level(ctx, level));
    Ctx &c = ctx->impl;
    PMG_TRY(c.dot(level, x, y, 10));
    double h[11];
    PMG_TRY(c.fetch_scalars(h, 11));
    if (result) *result = h[10];
    return PMG_OK;
}

int pmg_residual(pmg_ctx *ctx, int level, double *r, const double *x, const double *b)
{
    PMG_TRY(check_ctx_level(ctx, level));
    Ctx &c = ctx->impl;
    const auto &L = c.lv[level];
    PMG_TRY(pmg::zero_ghosts_f64(r, L.n[0], L.n[1], L.n[2], c.stream));
    return pmg::f64_residual(c.K[level], c.launch[level], r, x, b, nullptr, nullptr, c.stream, c.diag(level));
}

int pmg_rbgs_iterator(pmg_ctx *ctx, int level, double *x, const double *b, int maxiteration, double omega)
{
    PMG_TRY(check_ctx_level(ctx, level));
    Ctx &c = ctx->impl;
    return pmg::f64_rbgs_sweeps(c.K[level], c.launch[level], x, b, maxiteration, omega, c.stream, c.diag(level));
}

int pmg_rbgs_solver(pmg_ctx *ctx, int level, double *x, const double *b, int maxiteration, double tolerance,
                    double omega, int *iterations, double *ratio)
{
    PMG_TRY(check_ctx_level(ctx, level));
    return ctx->impl.rbgs_solver_dev(level, x, b, maxiteration, tolerance, omega, iterations, ratio);
}

int pmg_cg_iterator(pmg_ctx *ctx, int level, double *x, const double *b, int maxiteration)
{
    PMG_TRY(check_ctx_level(ctx, level));
    return ctx->impl.cg_dev(level, x, b, maxiteration, 0.0, false, nullptr, nullptr);
}

int pmg_cg_solver(pmg_ctx *ctx, int level, double *x, const double *b, int maxiteration, double tolerance,
                  int *iterations, double *ratio)
{
    PMG_TRY(check_ctx_level(ctx, level));
    return ctx->impl.cg_dev(level, x, b, maxiteration, tolerance, true, iterations, ratio);
}

int pmg_restriction(pmg_ctx *ctx, int level, double *val_c, const double *val_f)
{
    PMG_TRY(check_ctx_level(ctx, level));
    Ctx &c = ctx->impl;
    if (level >= c.nl) {
        pmg::set_error("restriction needs a level below the coarsest");
        return PMG_EINVAL;
    }
    const auto &C = c.lv[level + 1];
    PMG_CUDA(cudaMemsetAsync(val_c, 0, C.total * sizeof(double), c.stream), "restriction init");
    return pmg::f64_restrict(c.X[level], c.launch[level + 1], val_f, val_c, c.stream);
}

int pmg_prolongation(pmg_ctx *ctx, int level, double *val_f, const double *val_c)
{
    PMG_TRY(check_ctx_level(ctx, level));
    Ctx &c = ctx->impl;
    if (level >= c.nl) {
        pmg::set_error("prolongation needs a level below the coarsest");
        return PMG_EINVAL;
    }
    return pmg::f64_prolong(c.X[level], c.launch[level + 1], val_c, val_f, false, c.stream);
}

int pmg_prolong_add(pmg_ctx *ctx, int level, double *x_f, const double *x_c)
{
    PMG_TRY(check_ctx_level(ctx, level));
    Ctx &c = ctx->impl;
    if (level >= c.nl) {
        pmg::set_error("prolongation needs a level below the coarsest");
        return PMG_EINVAL;
    }
    return pmg::f64_prolong(c.X[level], c.launch[level + 1], x_c, x_f, true, c.stream);
}

int pmg_adjoint(pmg_ctx *ctx, const double *dLdu, double *dLdb, double dLdg[6], int maxiteration, double tolerance,
                double omega_sor, pmg_report_t *report)
{
    PMG_TRY(check_ctx_level(ctx, 0));
    if (!dLdu || !dLdb || maxiteration < 0) {
        pmg::set_error("dLdu and dLdb are required");
        return PMG_EINVAL;
    }
    cudaPointerAttributes a1, a2;
    if (cudaPointerGetAttributes(&a1, dLdu) != cudaSuccess || cudaPointerGetAttributes(&a2, dLdb) != cudaSuccess ||
        a1.type != cudaMemoryTypeDevice || a2.type != cudaMemoryTypeDevice) {
        cudaGetLastError();
        pmg::set_error("pmg_adjoint takes device arrays");
        return PMG_EINVAL;
    }
    return pmg::guarded([&] { return ctx->impl.adjoint(dLdu, dLdb, dLdg, maxiteration, tolerance, omega_sor, report); });
}

struct pmg_batch {
    pmg::Batch *impl;
};

int pmg_batch_create(pmg_batch **batch, int n_problems, const int *dims, const double *const *meshes,
                     int mixed_inner_cycles, void *stream)
{
    if (!batch) {
        pmg::set_error("batch is required");
        return PMG_EINVAL;
    }
    *batch = nullptr;
    pmg::Batch *b = nullptr;
    const int rc = pmg::guarded(
        [&] { return pmg::batch_create(&b, n_problems, dims, meshes, mixed_inner_cycles, (cudaStream_t)stream); });
    if (rc != PMG_OK) return rc;
    pmg_batch *h = new (std::nothrow) pmg_batch{b};
    if (!h) {
        pmg::batch_destroy(b);
        return PMG_ENOMEM;
    }
    *batch = h;
    return PMG_OK;
}

int pmg_batch_layout(const pmg_batch *batch, long long *offsets, int *levels)
{
    if (!batch) return PMG_EINVAL;
    pmg::batch_layout(*batch->impl, offsets, levels);
    return PMG_OK;
}

int pmg_batch_solve(pmg_batch *batch, double *sol, const double *rhs, int maxiteration, double tolerance,
                    double omega_sor, int max_cycles, int *cycles, double *ratio, float *elapsed_ms)
{
    if (!batch) return PMG_EINVAL;
    return pmg::guarded([&] {
        return pmg::batch_solve(*batch->impl, sol, rhs, maxiteration, tolerance, omega_sor, max_cycles, cycles, ratio,
                                elapsed_ms);
    });
}

int pmg_batch_destroy(pmg_batch *batch)
{
    if (!batch) return PMG_OK;
    pmg::batch_destroy(batch->impl);
    delete batch;
    return PMG_OK;
}

int pmg_profile(pmg_ctx *ctx, int enable)
{
    PMG_TRY(check_ctx_level(ctx, 0));
    Ctx &c = ctx->impl;
    cudaStreamSynchronize(c.stream);
    c.prof.flush();
    c.prof.reset();
    c.prof.on = enable != 0;
    return PMG_OK;
}

int pmg_profile_read(pmg_ctx *ctx, int kernel_class, double *total_ms, long long *launches, double *bytes)
{
    PMG_TRY(check_ctx_level(ctx, 0));
    if (kernel_class < 0 || kernel_class >= pmg::PC_COUNT) {
        pmg::set_error("kernel class out of range");
        return PMG_EINVAL;
    }
    Ctx &c = ctx->impl;
    cudaStreamSynchronize(c.stream);
    c.prof.flush();
    if (total_ms) *total_ms = c.prof.total_ms[kernel_class];
    if (launches) *launches = c.prof.count[kernel_class];
    if (bytes) *bytes = c.prof.count[kernel_class] ? c.prof.bytes[kernel_class] / (double)c.prof.count[kernel_class] : 0.0;
    return PMG_OK;
}

int pmg_launch_count(long long *count)
{
    if (!count) return PMG_EINVAL;
    *count = pmg::launches_total();
    return PMG_OK;
}

int pmg_inject_alloc_failure(long long n)
{
    pmg::g_alloc_fail_countdown.store(n < 0 ? -1 : n);
    return PMG_OK;
}

int pmg_set_abort(pmg_ctx *ctx, int flag)
{
    if (!ctx) {
        pmg::set_error("pmg_set_abort: ctx is NULL");
        return PMG_EINVAL;
    }
    __atomic_store_n(ctx->impl.abort_host, flag ? 1 : 0, __ATOMIC_RELEASE);
    return PMG_OK;
}

int pmg_selftest_convert(const double *in64, float *out32, const float *in32, double *out64, int n)
{
    if (n < 0 || (n > 0 && (!in64 || !out32 || !in32 || !out64))) {
        pmg::set_error("invalid conversion self-test arguments");
        return PMG_EINVAL;
    }
    if (n == 0) return PMG_OK;
    PMG_TRY(pmg::convert_selftest(in64, out32, in32, out64, n, nullptr));
    return pmg::cuda_status(cudaDeviceSynchronize(), "conversion self-test");
}

int pmg_selftest_smooth32(pmg_ctx *ctx, int level, int impl, int variant, int kchunk, int zero_in, double omega,
                          const double *e_in, const double *b, double *e_out)
{
    PMG_TRY(check_ctx_level(ctx, level));
    if (!e_in || !b || !e_out || impl < 0 || impl > 2 || variant < 0 || variant > (impl == 0 ? 3 : 2) ||
        kchunk < 0) {
        pmg::set_error("invalid smoother self-test arguments");
        return PMG_EINVAL;
    }
    return ctx->impl.selftest_smooth32(level, impl, variant, kchunk, zero_in != 0, omega, e_in, b, e_out);
}

int pmg_selftest_wait_timeout(pmg_ctx *ctx, int level)
{
    PMG_TRY(check_ctx_level(ctx, level));
    return ctx->impl.selftest_wait_timeout(level);
}

int pmg_sync(pmg_ctx *ctx)
{
    if (!ctx) return PMG_EINVAL;
    return pmg::cuda_status(cudaStreamSynchronize(ctx->impl.stream), "sync");
}

const char *pmg_last_error(void) { return pmg::g_last_error.c_str(); }

const char *pmg_status_string(int status)
{
    switch (status) {
    case PMG_OK: return "ok";
    case PMG_EINVAL: return "invalid argument";
    case PMG_ENOMEM: return "out of memory";
    case PMG_EDIVERGED: return "diverged";
    case PMG_ETIMEOUT: return "timeout";
    case PMG_ECUDA: return "cuda error";
    default: return "unknown";
    }
}

}  // extern "C"
