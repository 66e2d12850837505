// Internal state of an LbmHandle and the launchers the C ABI calls.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/lbm_gb300.h"

#include <nvtx3/nvToolsExt.h>

// NVTX range over one C ABI call (header-only NVTX; a no-op unless a profiler
// such as Nsight attaches), so a timeline shows where the host calls start and
// end: "lbm_step", "lbm_run_to_convergence", "lbm_set_geometry", ...
struct LbmNvtxRange {
    explicit LbmNvtxRange(const char* name) { nvtxRangePushA(name); }
    ~LbmNvtxRange() { nvtxRangePop(); }
    LbmNvtxRange(const LbmNvtxRange&) = delete;
    LbmNvtxRange& operator=(const LbmNvtxRange&) = delete;
};

// Per-launch constants of the single-phase step (template on compute type R).
template <typename R>
struct SpConsts {
    int32_t nx, ny, nz;
    int32_t n_fluid;
    int64_t np;        // element stride between populations (padded n_fluid)
    int32_t bc[6];
    int32_t bc_form;
    int32_t any_bc;
    int32_t any_pressure;
    int32_t guo;
    R rho_bc[6];
    R rho_bc_dev[6];   // rho_bc - 1, rounded once from FP64
    R vel_bc[6][3];
    R sv, so;          // S_dig values s_v, s_other (SP:128-131)
    R fext[3];
    R fhalf[3];        // fext / 2 (SP:388)
    // Deviation-form kernels: moments of the Guo term in closed form, M (w o g)
    // with g = gc (e - u).F + gd (e.u)(e.F); the (gc, gd) of the convention
    R gc, gd;
    // 16-bit codecs: reference density of the stored deviations (x-linear
    // between two fixed-pressure x faces, else 0) and the launch's step index
    // (the stochastic-rounding seed)
    R ref_a, ref_b;
    uint32_t seed;
};

// int32 entries of -1 allocated after the dense map's last cell (bulk-copy rounding).
#define LBM_MAP_PAD 16

struct LbmHandle {
    LbmParams p{};
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    int64_t ncell = 0;
    int32_t n_fluid = 0;
    int64_t np = 0;
    bool have_geometry = false, initialized = false, macros_valid = false, have_psi = false;
    int64_t steps_done = 0;
    int32_t block = 256;
    size_t elem = 4;          // bytes per stored population
    bool f64 = false;         // compute in FP64
    bool force = false;

    std::vector<int8_t> solid;             // dense host copy (made on demand: geom_host_index)
    std::vector<int32_t> cell_of_node;     // n_fluid (made on demand)
    bool host_index_valid = false;
    bool l2_persist = false;               // the map is this stream's persisting L2 window
    std::vector<float> psi0;               // dense initial psi (two phase)

    int32_t* d_map = nullptr;              // dense: node index or -1 (solid); LBM_MAP_PAD extra -1 entries
    int2* d_tinfo = nullptr;               // staged step: per 256-node tile, first staged row and plane/rows
    int32_t ntile = 0;
    bool tiled = false;                    // single-phase steps use a staged kernel
    int tiled_mode = 0;                    // 1: persistent staged kernel, 2: one tile per CTA
    unsigned long long* d_spt_ctr = nullptr;  // its tile claim counter (inside the d_tinfo allocation)
    unsigned long long spt_base = 0;       // counter value at the next launch's first claim
    uint32_t* d_coord = nullptr;           // packed (i,j,k) per node
    void* d_f[2] = {nullptr, nullptr};     // populations, 19 x np elements in AoSoA-32 chunks
    int cur = 0;
    void* d_vprev = nullptr;               // [3][np] previous-step v (pressure faces)
    void* d_rho = nullptr;                 // [np]
    void* d_v = nullptr;                   // [3][np]
    // two phase
    void* d_psi = nullptr;                 // [np] psi at fluid nodes
    void* d_rr[2] = {nullptr, nullptr};    // rho_r, double-buffered [np]
    void* d_rb[2] = {nullptr, nullptr};    // rho_b
    void* d_cs = nullptr;                  // recolouring amounts of the 9 pairs [9][np]
    int ccur = 0;
    // grey scale (partial bounce-back)
    bool grey = false;
    void* d_ns = nullptr;                  // [np] grey value per node (compute type)
    void* d_gstale = nullptr;              // [2][ny*nz][19] post-face F of fixed-velocity x faces
    // reductions
    double* d_red = nullptr;               // per-block partials
    int red_blocks = 0;
    double* d_red_out = nullptr;
    int64_t device_bytes = 0;
    std::string err;
};

int lbm_set_err(LbmHandle* h, int code, const std::string& msg);
int lbm_cuda_check(LbmHandle* h, cudaError_t e, const char* what);

// index construction and dense output (lbm_geom.cu)
int geom_build(LbmHandle* h, const int8_t* solid, int64_t si, int64_t sj, int64_t sk);
int geom_host_index(LbmHandle* h);
template <typename O>
int geom_dense_out(LbmHandle* h, const void* dsrc, int comps, O* out, O fill);

// single phase (lbm_sp.cu)
int sp_launch_init(LbmHandle* h, const void* rho_nodes, const void* v_nodes);
int sp_launch_steps(LbmHandle* h, int32_t n, bool macros_last);
int sp_launch_debug_stream(LbmHandle* h, const float* d_in, float* d_out);
int sp_tiles_setup(LbmHandle* h);
template <typename R>
SpConsts<R> sp_make_consts(const LbmHandle* h);

// grey scale (lbm_grey.cu)
int grey_launch_steps(LbmHandle* h, int32_t n, bool macros_last);
// Result of the -DLBM_DEBUG index checks since the last call (LBM_OK in other builds).
int sp_debug_take(LbmHandle* h);

// two phase (lbm_tp.cu)
int tp_launch_init(LbmHandle* h);
int tp_launch_steps(LbmHandle* h, int32_t n, bool macros_last);

// reductions (lbm_reduce.cu)
int red_launch(LbmHandle* h, LbmStats* out, float* max_v_f32);

// TMA-fed 3x3x3 convolution (nn_tma.cu).
bool nn_tma_usable(int cin, int cout);
int nn_conv3d_tma(const void* in, const void* w, const float* bias, const void* mask, void* out, void* pre, int n, int d,
                  int h, int wd, int cin, int cout, int mode, cudaStream_t s);
int nn_tma_take_error(int* flag);
bool nn_halo_usable(int cin, int cout);
int nn_conv3d_halo(const void* in, const void* w, const float* bias, const void* mask, void* out, void* pre, int n, int d,
                   int h, int wd, int cin, int cout, int mode, cudaStream_t s);
bool nn_wgrad_tma_usable(int cin, int cout);
int64_t nn_wgrad_tma_chunks(int n, int d, int h, int w);
bool nn_wgrad_ws_usable(int cin, int cout);
int64_t nn_wgrad_ws_chunks(int n, int d, int h, int w);
int nn_wgrad_ws(const void* in, const void* g, float* part, float* dbpart, int n, int d, int h, int wd, int cin, int cout,
                cudaStream_t s);
int nn_wgrad_tma(const void* in, const void* g, float* part, float* dbpart, int n, int d, int h, int wd, int cin,
                 int cout, cudaStream_t s);
