// pmg_ctx.h -- the solver context behind the opaque pmg_ctx handle.
#pragma once

#include <array>
#include <vector>

#include "../../include/peps_mg.h"
#include "pmg_internal.h"

namespace pmg {

// Levels above this many cells (ghosts included) stay on the grid kernels instead of
// the single-CTA tail.
constexpr size_t kTailMaxCells = 1u << 18;
// FP32 levels of at most this many cells run inside the single-CTA tail of the mixed cycle.
constexpr long long kTail32Cells = 1LL << 12;

struct Level {
    int n[3] = {0, 0, 0};
    int sy = 0;
    long long sz = 0;
    size_t total = 0;
    std::vector<double> dm[3], dg[3], xg[3];
    double *x = nullptr, *b = nullptr, *r = nullptr;   // device, levels >= 1
};

struct MixedState;   // FP32 V-cycle state (pmg_mixed.cu)

// Event-pair timing of finest-level launches, accumulated per kernel class.
struct Profiler {
    bool on = false;
    struct Rec {
        int cls;
        int launches;
        double bytes;
        cudaEvent_t a, b;
    };
    std::vector<cudaEvent_t> pool;
    std::vector<Rec> pending;
    double total_ms[PC_COUNT] = {};
    long long count[PC_COUNT] = {};
    double bytes[PC_COUNT] = {};     // algorithmic bytes summed over launches
    ~Profiler();
    void reset();
    cudaEvent_t get();
    // begin/end around `launches` launches of class cls moving `bytes` per launch
    int begin(cudaStream_t s);
    void end(int idx, int cls, int launches, double bytes_per_launch, cudaStream_t s);
    void flush();   // call after the stream is synchronised
};

int level_sizes(const int n0[3], int n_levels, int method, int cga_level, std::vector<std::array<int, 3>> &sizes,
                int lvc[3]);
int host_level_meshes(const pmg_config_t *c, std::vector<Level> &lv, int lvc[3]);

struct Ctx {
    cudaStream_t stream = nullptr;
    int nl = 0, n_vcycles = 0, method = 0, cga_level = 0, cgpsa_level[3] = {0, 0, 0};
    int coarse_solver = 0, precision = 0, mixed_inner = 0;
    int lvc[3] = {0, 0, 0};
    std::vector<Level> lv;
    std::vector<double> tables_host;
    double *d_tables = nullptr;
    std::vector<LevelK<double>> K;
    std::vector<XferK<double>> X;
    std::vector<Launch> launch;
    int tail_l0 = 0;
    int tail_threads = 1024;   // block size of the single-CTA tail kernels
    int tail32_l0 = 0;         // first level of the mixed cycle's single-CTA tail
    int tail32_threads = 1024;
    int tail32_smem = 0;       // dynamic shared memory bytes of the mixed cycle's tail
    bool deep_tail = true;     // mixed cycle: move small levels into the tail (batch members keep tail_l0)
    TailDesc<double> tail_host;
    TailDesc<double> *d_tail = nullptr;
    double *d_partials = nullptr;
    size_t npart_cap = 0;
    double *d_scal = nullptr;
    int *d_iscal = nullptr;
    double *d_cp = nullptr, *d_cap = nullptr, *d_crr = nullptr;
    CgState *d_cg = nullptr;   // scalars of the fused CG solver (lower API, large coarsest levels)
    std::vector<double *> c0t; // plain FP64 contexts: per-cell diagonal of every level (f64_diag_table)
    bool x0_known_zero = false; // the staged initial guess of the running solve is all zero (host scan)
    const double *diag(int l) const { return (size_t)l < c0t.size() ? c0t[l] : nullptr; }
    // Abort flag (pmg_set_abort) in mapped page-locked host memory: the host loops read it
    // between cycles, the coarse solvers of the single-CTA tails poll it on the device.
    int *abort_host = nullptr;
    const int *abort_dev = nullptr;
    bool aborted() const { return abort_host && __atomic_load_n(abort_host, __ATOMIC_ACQUIRE) != 0; }
    int abort_status();
    double *stage_sol = nullptr, *stage_rsd = nullptr, *stage_rhs = nullptr;
    std::vector<double *> scratch_levels;
    size_t scratch_cap = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // Early copy-back of a staged solve: the mixed solver starts the device-to-host copy of
    // the solution when it recomputes the residual that may end the solve, so the copy
    // overlaps that residual; a later change of x first waits for the copy and voids it.
    double *early_sol_host = nullptr;   // the caller's pinned host sol during a staged solve
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_x = nullptr, ev_copied = nullptr;
    bool early_valid = false, early_pending = false;
    int early_copy_sol(const double *sol);
    int before_x_change();
    // FP64 performance mode (PMG_FP64_FAST): per grid level the diagonal sums and omega/c0,
    // per transfer the normalised weights (pmg_f64fast.cu); tables in one device blob
    bool fast64 = false;
    std::vector<FastLevelK> fastK;
    std::vector<FastXferK> fastX;
    double *d_fast = nullptr;
    std::vector<double *> fast_wdiag_alloc;
    double fast_omega = 0.0;
    bool fast_omega_set = false;
    int setup_fast64();
    int fast_prepare(double omega);
    MixedState *mixed = nullptr;
    Profiler prof;
    bool autotune = true;       // tune the fused smoother per level in setup_mixed
    // adjoint scratch (finest level)
    double *adj_rhs = nullptr, *adj_sol = nullptr, *adj_rsd = nullptr, *adj_vol = nullptr, *adj_faces = nullptr;

    // a member of a batch: no events, copy stream or abort flag of its own (set before build)
    bool light = false;
    // subdomain of a decomposed solve: the level sizes and meshes to use (set before build)
    const std::vector<Level> *preset_levels = nullptr;
    int build(const pmg_config_t *c, cudaStream_t s);
    int setup_tables();
    ~Ctx();

    int dot(int l, const double *x, const double *y, int slot);
    int residual_norm(int l, double *r, const double *x, const double *b, int slot);
    int solve_residual_norm(double *r, const double *x, const double *b, int slot);
    int fetch_scalars(double *h, int n);
    int upload_tail(int l0, int maxit, double omega, double tol);
    void fill_coarse64(LevelK<double> &C, double *&x, double *&b, double *&p, double *&ap, double *&rr, double &om,
                       double &omw, double omega) const;
    int coarse_solve_grid(double tol, double omega, int *iters);
    int vcycle_f64(double *sol, double *rsd, const double *rhs, int maxit, double omega, double tol,
                   int *coarse_iters);
    int solve_f64(double *sol, double *rsd, const double *rhs, int maxit, double tol, double omega,
                  pmg_report_t *rep);
    int solve_mixed(double *sol, double *rsd, const double *rhs, int maxit, double tol, double omega,
                    pmg_report_t *rep);
    int setup_mixed();
    int build_mixed();
    int upload_tail32(int maxit, double omega, double tol);
    int vcycle32(int maxit, double omega, bool zero_start);
    int outer_residual(double *sol, double *rsd, const double *rhs, int slot, double res0 = 0.0);
    int norm_exponent(double res0) const;
    int update_residual(double *sol, double *rsd, int slot, double res0);
    int run_vcycles(int maxit, double omega, int check_after = 0, double thresh2 = 0.0, int *ran = nullptr,
                    double res0 = 0.0);
    int inner_norm(double *out, double res0);
    int correct_and_recompute(double *sol, double *rsd, const double *rhs, double res0);
    int add_corrections(double *sol, bool with_e);
    int flush_stash(double *sol);
    int check_pipeline();
    int resrestrict32(int l);
    int selftest_smooth32(int level, int impl, int variant, int kchunk, bool zero_in, double omega,
                          const double *e_in, const double *b, double *e_out);
    int selftest_wait_timeout(int level);
    void destroy_mixed();
    int solve(double *sol, double *rsd, const double *rhs, int maxit, double tol, double omega, pmg_report_t *rep);
    int level_scratch(int l, double **bufs, int count);
    int rbgs_solver_dev(int l, double *x, const double *b, int maxit, double tol, double omega, int *iters,
                        double *ratio_out);
    int cg_dev(int l, double *x, const double *b, int maxit, double tol, bool check, int *iters, double *ratio_out);
    int adjoint(const double *dLdu, double *dLdb, double *dLdg, int maxit, double tol, double omega, pmg_report_t *rep);
};

}  // namespace pmg
