/* lbm_gb300.h -- C ABI of the GB300-native D3Q19 MRT lattice Boltzmann hot path.
 *
 * The library (taichi_lbm3d_gb300/liblbm_gb300.so) implements one time step of
 * taichi_LBM3D's solvers as fused sm_103a CUDA kernels over a compacted list of
 * fluid nodes.  It replaces the Taichi kernels that the reference's Python
 * solver classes launch; each entry point names the reference interface it
 * stands in for (paths inside the taichi_LBM3D tree):
 *
 *   SP = Single_phase/LBM_3D_SinglePhase_Solver.py
 *   TP = 2phase/lbm_solver_3d_2phase_sparse.py
 *
 * Conventions
 *   - Every call returns 0 on success or a negative LBM_E* code; the message of
 *     the last failure is available from lbm_last_error().
 *   - Host arrays are caller-owned, dense over the lattice, cell order x fastest:
 *     cell = i + nx*(j + ny*k)  (the order of the reference's geometry files,
 *     SP:173-177).  Vector fields are interleaved: v[cell*3 + c].
 *   - A handle owns its device memory and one CUDA stream; use a handle from one
 *     host thread at a time.  Calls are synchronous unless named *_async.
 *   - There is no CPU fallback: lbm_create fails with LBM_ENODEV when no CUDA
 *     device of compute capability 10.3 (GB300) is present.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_ABI_VERSION 1

enum {
    LBM_OK = 0,
    LBM_EINVAL = -1,   /* bad argument / parameter */
    LBM_ENODEV = -2,   /* no usable sm_103 device */
    LBM_ENOMEM = -3,   /* device or host allocation failed */
    LBM_ECUDA = -4,    /* CUDA runtime error */
    LBM_ESTATE = -5,   /* call out of order (e.g. step before geometry) */
    LBM_EDIVERGED = -6 /* NaN/Inf detected by a reduction */
};

/* Boundary codes per face (SP:22-28): 0 periodic, 1 fixed pressure, 2 fixed velocity.
 * Face order everywhere: x-left, x-right, y-left, y-right, z-left, z-right. */
enum { LBM_BC_PERIODIC = 0, LBM_BC_PRESSURE = 1, LBM_BC_VELOCITY = 2 };

/* Population storage of the fused kernels.  F32 and F64 compute on f itself,
 * as the reference does (F32 reproduces its FP32 rounding bit for bit).  The
 * *_DEV modes compute in FP32 on f - w and rho - 1 (deviation form); F16_DEV and
 * BF16_DEV store each node's populations relative to its own density,
 * g = f - w*rho_node, with rho_node - 1 kept per node in FP32. */
enum {
    LBM_STORE_F32 = 0,       /* FP32 f, reference arithmetic */
    LBM_STORE_F16_DEV = 1,   /* FP16 of g * 2^16, deviation-form FP32 collide */
    LBM_STORE_BF16_DEV = 2,  /* BF16 of g, deviation-form FP32 collide */
    LBM_STORE_F64 = 3,       /* FP64 f and arithmetic (accuracy reference) */
    LBM_STORE_F32_DEV = 4    /* FP32 of f - w, deviation-form FP32 collide */
};

/* Solver parameters: the attributes the reference's class sets before
 * init_simulation() (SP:11-28, :118-149) and the two-phase script's module
 * globals (TP:17-40).  Doubles are Python floats; the kernels round them to
 * the compute type exactly as Taichi folds Python constants. */
typedef struct LbmParams {
    int32_t nx, ny, nz;
    int32_t bc[6];
    double rho_bc[6];
    double vel_bc[6][3];
    double niu;
    double force[3];
    int32_t visc_convention; /* 0: tau = niu/3+0.5 (SP:127); 1: tau = 3*niu+0.5 (scripts, TP:104) */
    int32_t guo_convention;  /* 0: class Guo term /3, /9 (SP:236); 1: script form (TP:246); 2: standard 3, 9 */
    int32_t bc_form;         /* velocity faces: 0 feq(s,1,u) (SP:288); 1 in-place form (TP:506) */
    int32_t storage;         /* LBM_STORE_* */
    int32_t two_phase;       /* 0 single phase (SP), 1 colour-gradient two phase (TP) */
    double niu_l, niu_g, psi_solid, cap_a;  /* TP:22-25 */
    int32_t psi_bc[6];       /* TP:35-40: 0 periodic, 1 constant psi */
    double psi_val[6];
    int32_t device;          /* CUDA device ordinal */
    int32_t block_size;      /* threads per CTA of the step kernel, 0 = default (128 single-phase, 256 two-phase) */
} LbmParams;

typedef struct LbmInfo {
    int64_t n_cells;
    int64_t n_fluid;
    int64_t steps_done;
    int64_t device_bytes;    /* bytes of device memory held by the handle */
    int32_t storage;
    int32_t two_phase;
    int32_t sm_count;
    int32_t abi_version;
} LbmInfo;

/* FP64 reductions over the fluid nodes of the last completed step. */
typedef struct LbmStats {
    double mass;             /* sum of rho */
    double mom[3];           /* sum of v (not rho*v), per component */
    double max_v;            /* max |v| over fluid nodes (solid cells have v = 0) */
    int64_t n_nonfinite;     /* rho or v not finite */
    int64_t n_fluid;
} LbmStats;

typedef struct LbmHandle LbmHandle;

int lbm_abi_version(void);

/* Stands in for LB3D_Solver_Single_Phase.__init__ (SP:11-114) plus the field
 * allocation that Taichi does; two-phase: the module-level allocations (TP:53-96). */
int lbm_create(const LbmParams* params, LbmHandle** out);
int lbm_destroy(LbmHandle* h);

/* Geometry: solid[cell] > 0 is solid (init_geo, SP:173-177; solid.from_numpy in
 * example_poiseuille_flow.py:24).  Builds the compacted fluid index and the
 * neighbour map on the device.  The lattice size is the one in LbmParams. */
int lbm_set_geometry(LbmHandle* h, const int8_t* solid);

/* The same with the mask addressed as solid[i*si + j*sj + k*sk] (element
 * strides >= 0), e.g. a C-ordered (nx, ny, nz) numpy array without a
 * transposing copy.  The index is built on the device. */
int lbm_set_geometry_strided(LbmHandle* h, const int8_t* solid, int64_t si, int64_t sj, int64_t sk);

/* Two-phase initial phase field psi[cell] (TP:195-203, psi.from_numpy). */
int lbm_set_psi(LbmHandle* h, const float* psi);

/* Grey-scale lattice: partial bounce-back fraction ns[cell] of every cell
 * (ns.from_numpy, Grey_Scale/lbm_solver_3d_Macro_Sukop.py:320-324; the caller
 * passes the solid mask ns.astype(int) != 0 to lbm_set_geometry first).  The
 * step then runs the script's streaming0/streaming1 rule (:234-252) in place
 * of halfway bounce-back.  Fixed faces on x only (LBM_EINVAL otherwise, as
 * the script's Boundary_condition treats x only, :263-293); call lbm_init
 * afterwards.  A new lbm_set_geometry clears it. */
int lbm_set_grey(LbmHandle* h, const double* ns);

/* Initial state: rho = 1, v = 0, f = feq (init, SP:160-170 / TP:174-187) when
 * rho and v are NULL; otherwise f = feq(rho, v) from the given dense fields
 * (the warm start).  Resets the step counter. */
int lbm_init(LbmHandle* h, const float* rho, const float* v);

/* Advance n time steps (SP:477-481 step(); TP:626-632).  lbm_step waits for the
 * GPU; lbm_step_async only enqueues on the handle's stream. */
int lbm_step(LbmHandle* h, int32_t n);
int lbm_step_async(LbmHandle* h, int32_t n);
int lbm_synchronize(LbmHandle* h);

/* The handle's CUDA stream (cudaStream_t), for event timing by the caller. */
int lbm_get_stream(LbmHandle* h, void** stream);

/* rho / v after the last step, dense (SP:470-473 to_numpy); solid cells hold
 * rho = 1, v = 0 (SP:390-392).  Either pointer may be NULL. */
int lbm_get_macros(LbmHandle* h, float* rho, float* v);

/* Same as lbm_get_macros in FP64 (exact for LBM_STORE_F64 handles; FP32 values
 * widened otherwise): the accuracy-reference readback. */
int lbm_get_macros_f64(LbmHandle* h, double* rho, double* v);

/* Two-phase fields after the last step: psi, rho_r, rho_b (dense; NULL to skip). */
int lbm_get_phase(LbmHandle* h, float* psi, float* rho_r, float* rho_b);
/* psi alone (the two-phase script's psi.to_numpy()): lbm_get_phase(h, psi, NULL, NULL). */
int lbm_get_psi(LbmHandle* h, float* psi);

/* get_max_v / cal_max_v (SP:394-402): max |v| over all cells. */
int lbm_get_max_v(LbmHandle* h, float* out);

/* FP64 reductions (mass, momentum, max |v|, non-finite count). */
int lbm_reductions(LbmHandle* h, LbmStats* out);

int lbm_get_info(LbmHandle* h, LbmInfo* out);

/* Permeability driver (no counterpart in the reference, whose examples loop on
 * step() and print get_max_v): run until the FP64 Darcy velocity along `axis`
 * (sum of v over fluid nodes / all cells, proportional to the permeability)
 * changes by at most tol (relative) between checks `check_every` steps apart,
 * or until max_steps.  Outputs the last Darcy velocity, the steps taken and
 * whether the criterion was met.  Returns LBM_EDIVERGED on NaN/Inf. */
int lbm_run_to_convergence(LbmHandle* h, double tol, int32_t check_every, int64_t max_steps, int32_t axis,
                           double* darcy_v, int64_t* steps, int32_t* converged);

/* Compacted fluid index: cell id of each fluid node, in node order (n_fluid). */
int lbm_get_fluid_index(LbmHandle* h, int32_t* cell_of_node);

/* Pull sources of the neighbour table, [18][n_fluid] for directions 1..18:
 * the node pulled from (x - e_s, periodic wrap of SP:247-257), or -1 - node
 * when that cell is solid (halfway bounce-back from the node's own LR slot). */
int lbm_get_neighbors(LbmHandle* h, int32_t* src);

/* Populations in node order, [19][n_fluid] as FP64 (checkpoint / tests). */
int lbm_get_populations(LbmHandle* h, double* f);
int lbm_set_populations(LbmHandle* h, const double* f);

/* One pull-stream of given populations with identity collision and no
 * boundary condition (streaming1, SP:259-269): in/out [19][n_fluid] FP32. */
int lbm_debug_stream(LbmHandle* h, const float* f_in, float* f_out);

/* ------------------------------------------------------------------ batches
 * Many independent porous subvolumes (no counterpart in the reference, which
 * runs one lattice per process): all faces periodic, shared parameters, one
 * persistent kernel per time step over all active subvolumes, check_every
 * steps captured in one CUDA graph.  dims: [n_sub][3]; solids: the n_sub
 * x-fastest masks back to back. */
typedef struct LbmBatch LbmBatch;
int lbm_batch_create(const LbmParams* params, int32_t n_sub, const int32_t* dims, const int8_t* solids,
                     LbmBatch** out);
int lbm_batch_destroy(LbmBatch* b);
/* Work-tile length in nodes per subvolume and CTA size of the persistent kernel
 * (chosen by the autotuner in taichi_lbm3d_gb300/autotune.py). */
int lbm_batch_configure(LbmBatch* b, const int32_t* tile_len, int32_t block);
/* Rest state f = feq(1, 0) in every subvolume, all subvolumes active. */
int lbm_batch_init(LbmBatch* b);
/* nsteps steps of the active subvolumes, in graph launches of `chunk` steps
 * (use_graph = 1) or plain launches (0). */
int lbm_batch_step(LbmBatch* b, int32_t nsteps, int32_t chunk, int32_t use_graph);
/* Run until each subvolume's FP64 Darcy velocity along x changes by <= tol
 * between checks; converged subvolumes drop out of the work list.  Per
 * subvolume outputs: Darcy velocity, steps taken, converged flag. */
int lbm_batch_run_to_convergence(LbmBatch* b, double tol, int32_t check_every, int64_t max_steps, int32_t use_graph,
                                 double* darcy, int64_t* steps, int32_t* converged);
/* rho and v (dense, x fastest, solid cells 1 and 0) of subvolume `sub` from its
 * current populations: e.g. the converged field of a training sample. */
int lbm_batch_get_macros(LbmBatch* b, int32_t sub, float* rho, float* v);
int lbm_batch_get_stream(LbmBatch* b, void** stream);
int lbm_batch_info(LbmBatch* b, int64_t* n_nodes, int64_t* n_fluid, int32_t* grid, int32_t* n_tiles);

/* Copy the message of the last error on this handle (or the last global error
 * when h is NULL) into buf. */
int lbm_last_error(LbmHandle* h, char* buf, size_t n);

/* Replaces the np.loadtxt inside init_geo (SP:173-177; the two-phase and grey
 * scripts' geometry/psi/ns files): the whitespace-separated numbers of an ASCII
 * file, parsed on the host in parallel, needs no GPU.  *count = how many the
 * file holds; with out non-NULL the file must hold exactly n (else LBM_EINVAL)
 * and they are written to out as double, rounded as np.loadtxt rounds them.  A
 * token that is not a number (comments included) is LBM_EINVAL with its byte
 * offset in the message (lbm_last_error(NULL, ...)). */
int lbm_read_ascii(const char* path, double* out, int64_t n, int64_t* count);

/* No counterpart in the reference.  The FP64 reduction of lbm_reductions for
 * callers that cannot allocate device memory: a host framework whose own pool
 * allocator already owns the GPU's memory, or a time-critical loop that must not
 * risk the device-wide synchronisation of cudaMalloc / cudaFree.  The caller
 * passes device arrays in node order (rho[n], v[3][v_stride], FP32), a stream
 * (NULL = default stream) and a host LbmStats; the call allocates nothing.  Its
 * scratch is a static device array of LBM_NOALLOC_SCRATCH_BYTES that every GPU
 * loading the library holds until exit.  n above LBM_NOALLOC_MAX_NODES is
 * rejected with LBM_EINVAL.  The call is synchronous: it waits for `stream` and
 * returns the sums in *out.  Its first call on a device looks up the scratch's
 * device address (make that first call before any stream capture begins); the
 * lookup is repeated when the device's context has been re-created since (for
 * example after cudaDeviceReset).  Calls share the scratch: calls that overlap
 * on the GPU race and must be serialised by the caller. */
#define LBM_NOALLOC_MAX_NODES 67108864
#define LBM_NOALLOC_SCRATCH_BYTES 196656
int lbm_reduce_macros_noalloc(const float* rho, const float* v, int64_t n, int64_t v_stride, void* stream,
                              LbmStats* out);

#ifdef __cplusplus
}
#endif
#endif /* LBM_GB300_H */
