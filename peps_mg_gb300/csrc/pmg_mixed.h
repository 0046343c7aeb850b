// pmg_mixed.h -- state of the mixed-precision V-cycle of one problem (FP32 hierarchy).
#pragma once

#include <vector>

#include "pmg_internal.h"

namespace pmg {

// Finest-level coefficients split into FP32 pairs (hi = c rounded to FP32, lo = c - hi
// rounded to FP32), per axis and side, for the compensated residual update.
struct SplitCoef {
    const float2 *cxm, *cxp, *cym, *cyp, *czm, *czp;
};

struct MixedState {
    std::vector<float> tables_host;
    float *tables = nullptr;
    double *diag64 = nullptr;        // per level: dyy (ny+2) and dzz (nz+2) for the outer residual
    float2 *split = nullptr;         // storage of sc
    SplitCoef sc{};
    bool update_residual = true;     // residual after a correction by r -= A e (else b - A x)
    std::vector<const double *> dyy, dzz;
    std::vector<LevelK<float>> K;
    std::vector<XferK<float>> X;
    std::vector<float *> alloc;      // raw allocations
    std::vector<float *> e[2], b;    // e[buf][l] (two buffers for out-of-place sweeps), b[l]
    // Finest-level corrections not yet added to x (the residual update leaves x alone for
    // up to two corrections; x = ((x + stash[0]) + stash[1]) + e when it is needed)
    float *stash[2] = {nullptr, nullptr};
    int nstash = 0;
    std::vector<int> cur;            // current buffer of e at each level
    std::vector<bool> fused;         // level uses the fused out-of-place smoother
    std::vector<bool> window;        // the autotuner chose the register-window kernel over the TMA-fed one
    std::vector<int> variant, kchunk;  // autotuned tile variant and k-chunk of the fused smoother
    std::vector<Rb32Tma> tma;        // tensor maps of the TMA-fed smoother, per level
    std::vector<long long> rows, planes;   // allocated rows per plane and planes, per level
    int *d_err = nullptr;
    bool march = true;               // marching transfer kernels where every axis involved is halved            // set by the TMA-fed smoother when a bounded wait gave up
    TailDesc<float> tail_host;
    TailDesc<float> *d_tail = nullptr;
    int inner = 2;
    // The FP32 V-cycle as CUDA graphs (first cycle of a correction, from e = 0, and the
    // later ones), captured on cap_stream and launched on the context's stream.
    bool use_graphs = true;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t vgraph[2] = {nullptr, nullptr};
    long long vgraph_launches[2] = {0, 0};
    int vgraph_maxit = -1;
    double vgraph_omega = 0.0;
    ~MixedState()
    {
        dev_free(tables);
        dev_free(diag64);
        dev_free(split);
        for (auto p : alloc) dev_free(p);
        dev_free(d_tail);
        dev_free(d_err);
        for (auto &g : vgraph)
            if (g) cudaGraphExecDestroy(g);
        if (cap_stream) cudaStreamDestroy(cap_stream);
    }
    float *E(int l) const { return e[cur[l]][l]; }
    float *Eother(int l) const { return e[1 - cur[l]][l]; }
};


}  // namespace pmg
