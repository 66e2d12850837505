// C ABI of liblbm_gb300.so (declared in include/lbm_gb300.h): handle
// lifecycle, geometry / compacted index, initial state, stepping, readback.
// The Python solver classes call these through ctypes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "lbm_common.cuh"
#include "lbm_internal.h"

namespace {
std::mutex g_err_mu;

// L2 residency of the neighbour map.  The 18 map lookups of every node sit on
// the step's critical path (coordinates -> map -> populations) and the map
// (4 B per cell) is otherwise evicted by the populations streaming through L2
// every step.  Each handle marks its map as a persisting access-policy window
// on its stream; the process-wide set-aside (a limit of this process's CUDA
// context, released when the process exits) is the largest map in use, capped
// at the device maximum, and is returned to 0 when the last handle on the
// device that used it is destroyed.  Best effort: failures only skip it.
std::mutex g_l2_mu;
int g_l2_users[64];
size_t g_l2_size[64];

void l2_persist_map(LbmHandle* h) {
    if (h->device < 0 || h->device >= 64 || !h->d_map) return;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, h->device) != cudaSuccess || prop.persistingL2CacheMaxSize <= 0 ||
        prop.accessPolicyMaxWindowSize <= 0) {
        cudaGetLastError();
        return;
    }
    const size_t map_bytes = sizeof(int32_t) * (size_t)h->ncell;
    const size_t want = std::min<size_t>(map_bytes, (size_t)prop.persistingL2CacheMaxSize);
    {
        std::lock_guard<std::mutex> lk(g_l2_mu);
        if (want > g_l2_size[h->device]) {
            if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) != cudaSuccess) {
                cudaGetLastError();
                return;
            }
            g_l2_size[h->device] = want;
        }
        ++g_l2_users[h->device];
    }
    // A window no larger than the set-aside, all of it persisting: for maps larger
    // than the set-aside only their first part persists (a window wider than the
    // set-aside with a fractional hit ratio made the persisting lines thrash).
    cudaStreamAttrValue attr = {};
    attr.accessPolicyWindow.base_ptr = (void*)h->d_map;
    attr.accessPolicyWindow.num_bytes = std::min<size_t>(want, (size_t)prop.accessPolicyMaxWindowSize);
    attr.accessPolicyWindow.hitRatio = 1.0f;
    attr.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    attr.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    if (cudaStreamSetAttribute(h->stream, cudaStreamAttributeAccessPolicyWindow, &attr) != cudaSuccess) cudaGetLastError();
    h->l2_persist = true;
}

void l2_release(LbmHandle* h) {
    if (!h->l2_persist) return;
    h->l2_persist = false;
    cudaStreamAttrValue attr = {};
    attr.accessPolicyWindow.num_bytes = 0;   // clear the window
    if (h->stream && cudaStreamSetAttribute(h->stream, cudaStreamAttributeAccessPolicyWindow, &attr) != cudaSuccess)
        cudaGetLastError();
    std::lock_guard<std::mutex> lk(g_l2_mu);
    if (--g_l2_users[h->device] == 0) {
        if (cudaCtxResetPersistingL2Cache() != cudaSuccess) cudaGetLastError();
        if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0) != cudaSuccess) cudaGetLastError();
        g_l2_size[h->device] = 0;
    }
}
std::string g_err;

int set_global_err(int code, const std::string& m) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_err = m;
    return code;
}

template <typename T>
int dev_alloc(LbmHandle* h, T** p, size_t bytes, const char* what) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc((void**)p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return lbm_set_err(h, LBM_ENOMEM, std::string("cudaMalloc failed for ") + what + ": " + cudaGetErrorString(e));
    }
    h->device_bytes += (int64_t)bytes;
    return LBM_OK;
}

template <typename T>
void dev_free(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

void free_lattice(LbmHandle* h) {
    dev_free(h->d_map);
    dev_free(h->d_coord);
    dev_free(h->d_tinfo);
    h->d_spt_ctr = nullptr;
    h->spt_base = 0;
    h->ntile = 0;
    h->tiled = false;
    dev_free(h->d_f[0]);
    dev_free(h->d_f[1]);
    dev_free(h->d_vprev);
    dev_free(h->d_rho);
    dev_free(h->d_v);
    dev_free(h->d_psi);
    dev_free(h->d_rr[0]);
    dev_free(h->d_rr[1]);
    dev_free(h->d_rb[0]);
    dev_free(h->d_rb[1]);
    dev_free(h->d_cs);
    dev_free(h->d_ns);
    dev_free(h->d_gstale);
    h->grey = false;
    dev_free(h->d_red);
    dev_free(h->d_red_out);
    h->device_bytes = 0;
}

size_t store_elem(int storage) {
    switch (storage) {
    case LBM_STORE_F32: return 4;
    case LBM_STORE_F16_DEV: return 2;
    case LBM_STORE_BF16_DEV: return 2;
    case LBM_STORE_F64: return 8;
    case LBM_STORE_F32_DEV: return 4;
    }
    return 0;
}

int validate(const LbmParams* p, std::string* why) {
    char b[256];
    if (p->nx < 1 || p->ny < 1 || p->nz < 1) { *why = "lattice size must be positive"; return LBM_EINVAL; }
    if (p->nx > 2047 || p->ny > 2047 || p->nz > 1023) {
        *why = "lattice too large: nx, ny <= 2047 and nz <= 1023 (packed node coordinates)";
        return LBM_EINVAL;
    }
    if ((int64_t)p->nx * p->ny * p->nz >= (int64_t)1 << 31) { *why = "lattice has >= 2^31 cells"; return LBM_EINVAL; }
    const int n[3] = {p->nx, p->ny, p->nz};
    for (int f = 0; f < 6; ++f) {
        if (p->bc[f] < 0 || p->bc[f] > 2) {
            snprintf(b, sizeof b, "bc[%d]=%d: must be 0 (periodic), 1 (pressure) or 2 (velocity)", f, p->bc[f]);
            *why = b;
            return LBM_EINVAL;
        }
        if (p->bc[f] != 0 && n[f / 2] < 2) {
            snprintf(b, sizeof b, "face %d has a non-periodic BC but the lattice is 1 cell thick there", f);
            *why = b;
            return LBM_EINVAL;
        }
        if (p->psi_bc[f] < 0 || p->psi_bc[f] > 1) { *why = "psi_bc must be 0 or 1"; return LBM_EINVAL; }
    }
    if (!(p->niu > 0) && !p->two_phase) { *why = "niu must be > 0"; return LBM_EINVAL; }
    if (store_elem(p->storage) == 0) { *why = "unknown storage"; return LBM_EINVAL; }
    if (p->visc_convention < 0 || p->visc_convention > 1 || p->guo_convention < 0 || p->guo_convention > 2 ||
        p->bc_form < 0 || p->bc_form > 1) {
        *why = "convention flags must be 0 or 1";
        return LBM_EINVAL;
    }
    if (p->two_phase && (!(p->niu_l > 0) || !(p->niu_g > 0))) { *why = "niu_l and niu_g must be > 0"; return LBM_EINVAL; }
    if (p->block_size != 0 && (p->block_size < 32 || p->block_size > 256 || p->block_size % 32)) {
        *why = "block_size must be a multiple of 32 in [32, 256]";
        return LBM_EINVAL;
    }
    return LBM_OK;
}
}  // namespace

int lbm_set_err(LbmHandle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    set_global_err(code, msg);
    return code;
}

int lbm_cuda_check(LbmHandle* h, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return LBM_OK;
    return lbm_set_err(h, LBM_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

extern "C" {

int lbm_abi_version(void) { return LBM_ABI_VERSION; }

int lbm_create(const LbmParams* params, LbmHandle** out) {
    if (!params || !out) return set_global_err(LBM_EINVAL, "lbm_create: NULL argument");
    *out = nullptr;
    std::string why;
    int rc = validate(params, &why);
    if (rc) return set_global_err(rc, "lbm_create: " + why);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return set_global_err(LBM_ENODEV, "lbm_create: no CUDA device (this library has no CPU path)");
    if (params->device < 0 || params->device >= ndev) return set_global_err(LBM_EINVAL, "lbm_create: bad device ordinal");
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, params->device) != cudaSuccess)
        return set_global_err(LBM_ENODEV, "lbm_create: cudaGetDeviceProperties failed");
    if (!(prop.major == 10 && prop.minor == 3)) {
        char b[160];
        snprintf(b, sizeof b, "lbm_create: device %d is sm_%d%d; this library is built for sm_103a (GB300) only",
                 params->device, prop.major, prop.minor);
        return set_global_err(LBM_ENODEV, b);
    }
    LbmHandle* h = new LbmHandle();
    h->p = *params;
    h->device = params->device;
    h->sm_count = prop.multiProcessorCount;
    h->elem = store_elem(params->storage);
    h->f64 = params->storage == LBM_STORE_F64;
    h->force = params->force[0] != 0 || params->force[1] != 0 || params->force[2] != 0;
    /* 128-thread CTAs measured 1.9% faster than 256 on the single-phase step
       (same 1536 resident threads per SM); the two-phase kernels keep 256. */
    h->block = params->block_size ? params->block_size : (params->two_phase ? 256 : 128);
    h->ncell = (int64_t)params->nx * params->ny * params->nz;
    cudaSetDevice(h->device);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return set_global_err(LBM_ECUDA, "lbm_create: cudaStreamCreate failed");
    }
    *out = h;
    return LBM_OK;
}

int lbm_destroy(LbmHandle* h) {
    if (!h) return LBM_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    l2_release(h);
    free_lattice(h);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return LBM_OK;
}

// Compacted index: fluid nodes in cell order (x fastest), the order in which
// the reference's block-sparse storage is activated by init (SP:160-170);
// built on the device (lbm_geom.cu).  The mask is addressed as
// solid[i*si + j*sj + k*sk] (element strides).
int lbm_set_geometry_strided(LbmHandle* h, const int8_t* solid, int64_t si, int64_t sj, int64_t sk) {
    LbmNvtxRange nvtx("lbm_set_geometry");
    if (!h || !solid) return lbm_set_err(h, LBM_EINVAL, "lbm_set_geometry: NULL argument");
    if (si < 0 || sj < 0 || sk < 0) return lbm_set_err(h, LBM_EINVAL, "lbm_set_geometry: negative stride");
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    l2_release(h);
    free_lattice(h);
    h->have_geometry = h->initialized = h->macros_valid = false;
    int rc = geom_build(h, solid, si, sj, sk);
    if (!rc) rc = sp_tiles_setup(h);
    if (rc) { free_lattice(h); return rc; }
    const size_t rbytes = h->f64 ? 8 : 4;
    rc = rc ? rc : dev_alloc(h, &h->d_f[0], h->elem * 19 * h->np, "f_A");
    rc = rc ? rc : dev_alloc(h, &h->d_f[1], h->elem * 19 * h->np, "f_B");
    rc = rc ? rc : dev_alloc(h, &h->d_vprev, rbytes * 3 * h->np, "vprev");
    rc = rc ? rc : dev_alloc(h, &h->d_rho, rbytes * h->np, "rho");
    rc = rc ? rc : dev_alloc(h, &h->d_v, rbytes * 3 * h->np, "v");
    if (!rc && h->p.two_phase) {
        rc = rc ? rc : dev_alloc(h, &h->d_psi, rbytes * h->np, "psi");
        rc = rc ? rc : dev_alloc(h, &h->d_rr[0], rbytes * h->np, "rho_r A");
        rc = rc ? rc : dev_alloc(h, &h->d_rr[1], rbytes * h->np, "rho_r B");
        rc = rc ? rc : dev_alloc(h, &h->d_rb[0], rbytes * h->np, "rho_b A");
        rc = rc ? rc : dev_alloc(h, &h->d_rb[1], rbytes * h->np, "rho_b B");
        rc = rc ? rc : dev_alloc(h, &h->d_cs, rbytes * 9 * h->np, "recolouring amounts");
    }
    h->red_blocks = (int)std::min<int64_t>(4 * h->sm_count, (h->n_fluid + 255) / 256 + 1);
    rc = rc ? rc : dev_alloc(h, &h->d_red, sizeof(double) * 8 * h->red_blocks, "reduction partials");
    rc = rc ? rc : dev_alloc(h, &h->d_red_out, sizeof(double) * 8, "reduction result");
    if (rc) { free_lattice(h); return rc; }
    rc = lbm_cuda_check(h, cudaMemsetAsync(h->d_f[0], 0, h->elem * 19 * h->np, h->stream), "clear f");
    if (!rc) rc = lbm_cuda_check(h, cudaMemsetAsync(h->d_f[1], 0, h->elem * 19 * h->np, h->stream), "clear f");
    if (!rc) rc = lbm_cuda_check(h, cudaMemsetAsync(h->d_vprev, 0, rbytes * 3 * h->np, h->stream), "clear vprev");
    if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "lbm_set_geometry");
    if (rc) { free_lattice(h); return rc; }
    h->have_geometry = true;
    h->have_psi = false;
    l2_persist_map(h);
    return LBM_OK;
}

int lbm_set_geometry(LbmHandle* h, const int8_t* solid) {
    if (!h) return lbm_set_err(h, LBM_EINVAL, "lbm_set_geometry: NULL handle");
    return lbm_set_geometry_strided(h, solid, 1, h->p.nx, (int64_t)h->p.nx * h->p.ny);
}

// Grey-scale lattice (Grey_Scale/lbm_solver_3d_Macro_Sukop.py): ns per cell,
// stored per fluid node in the compute type (FP32 modes round it as the
// script's f32 field does, :44).  The script applies fixed faces on x only.
int lbm_set_grey(LbmHandle* h, const double* ns) {
    if (!h || !ns) return lbm_set_err(h, LBM_EINVAL, "lbm_set_grey: NULL argument");
    if (h->p.two_phase) return lbm_set_err(h, LBM_ESTATE, "lbm_set_grey: handle is two phase");
    if (!h->have_geometry) return lbm_set_err(h, LBM_ESTATE, "lbm_set_grey: call lbm_set_geometry first");
    for (int f = 2; f < 6; ++f)
        if (h->p.bc[f] != 0) return lbm_set_err(h, LBM_EINVAL, "lbm_set_grey: grey-scale lattices take fixed faces on x only");
    if ((h->p.bc[0] || h->p.bc[1]) && h->p.nx < 2) return lbm_set_err(h, LBM_EINVAL, "lbm_set_grey: x faces need nx >= 2");
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    dev_free(h->d_ns);
    dev_free(h->d_gstale);
    h->grey = false;
    h->initialized = false;
    int rc = geom_host_index(h);
    if (rc) return rc;
    const size_t rb = h->f64 ? 8 : 4;
    std::vector<unsigned char> host(rb * h->np, 0);
    for (int32_t n = 0; n < h->n_fluid; ++n) {
        const double x = ns[h->cell_of_node[n]];
        if (h->f64) ((double*)host.data())[n] = x;
        else ((float*)host.data())[n] = (float)x;
    }
    rc = dev_alloc(h, &h->d_ns, rb * h->np, "grey ns");
    if (!rc && (h->p.bc[0] == LBM_BC_VELOCITY || h->p.bc[1] == LBM_BC_VELOCITY))
        rc = dev_alloc(h, &h->d_gstale, rb * 19 * 2 * (size_t)h->p.ny * h->p.nz, "grey face slots");
    if (!rc) rc = lbm_cuda_check(h, cudaMemcpyAsync(h->d_ns, host.data(), host.size(), cudaMemcpyHostToDevice, h->stream), "copy ns");
    if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "lbm_set_grey");
    if (rc) {
        dev_free(h->d_ns);
        dev_free(h->d_gstale);
        return rc;
    }
    h->grey = true;
    return LBM_OK;
}

int lbm_set_psi(LbmHandle* h, const float* psi) {
    if (!h || !psi) return lbm_set_err(h, LBM_EINVAL, "lbm_set_psi: NULL argument");
    if (!h->p.two_phase) return lbm_set_err(h, LBM_ESTATE, "lbm_set_psi: handle is single phase");
    if (!h->have_geometry) return lbm_set_err(h, LBM_ESTATE, "lbm_set_psi: call lbm_set_geometry first");
    h->psi0.assign(psi, psi + h->ncell);
    h->have_psi = true;
    h->initialized = false;
    return LBM_OK;
}

int lbm_init(LbmHandle* h, const float* rho, const float* v) {
    LbmNvtxRange nvtx("lbm_init");
    if (!h) return lbm_set_err(h, LBM_EINVAL, "lbm_init: NULL handle");
    if (!h->have_geometry) return lbm_set_err(h, LBM_ESTATE, "lbm_init: call lbm_set_geometry first");
    if ((rho == nullptr) != (v == nullptr)) return lbm_set_err(h, LBM_EINVAL, "lbm_init: give both rho and v, or neither");
    cudaSetDevice(h->device);
    h->cur = 0;
    h->steps_done = 0;
    h->macros_valid = false;
    int rc = LBM_OK;
    if (h->p.two_phase) {
        if (!h->have_psi) return lbm_set_err(h, LBM_ESTATE, "lbm_init: two-phase handle needs lbm_set_psi first");
        if (rho) return lbm_set_err(h, LBM_EINVAL, "lbm_init: two phase starts from rest (rho, v must be NULL)");
        rc = tp_launch_init(h);
    } else {
        float* d_in = nullptr;
        if (rho) {
            // gather the dense fields into node order: rho [np], v [3][np]
            rc = geom_host_index(h);
            if (rc) return rc;
            std::vector<float> hin(4 * h->np, 0.0f);
            for (int32_t n = 0; n < h->n_fluid; ++n) {
                const int64_t c = h->cell_of_node[n];
                hin[n] = rho[c];
                for (int d = 0; d < 3; ++d) hin[(1 + d) * h->np + n] = v[c * 3 + d];
            }
            if (cudaMalloc((void**)&d_in, sizeof(float) * 4 * h->np) != cudaSuccess)
                return lbm_set_err(h, LBM_ENOMEM, "lbm_init: staging allocation failed");
            rc = lbm_cuda_check(h, cudaMemcpyAsync(d_in, hin.data(), sizeof(float) * 4 * h->np, cudaMemcpyHostToDevice, h->stream), "copy init fields");
        }
        if (!rc) rc = sp_launch_init(h, d_in, d_in ? d_in + h->np : nullptr);
        if (!rc && h->grey && h->d_gstale) {
            // fixed-velocity face slots start as init's F = feq(s, 1, 0) = w_s (0 in deviation form)
            const bool dev = h->p.storage == LBM_STORE_F32_DEV || h->p.storage == LBM_STORE_F16_DEV ||
                             h->p.storage == LBM_STORE_BF16_DEV;
            const size_t cnt = 19 * 2 * (size_t)h->p.ny * h->p.nz;
            const size_t rb = h->f64 ? 8 : 4;
            std::vector<unsigned char> st(rb * cnt);
            for (size_t q = 0; q < cnt; ++q) {
                const double w = dev ? 0.0 : lbm_w((int)(q % 19));
                if (h->f64) ((double*)st.data())[q] = w;
                else ((float*)st.data())[q] = (float)w;
            }
            rc = lbm_cuda_check(h, cudaMemcpyAsync(h->d_gstale, st.data(), st.size(), cudaMemcpyHostToDevice, h->stream), "init face slots");
            if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "init face slots");
        }
        if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "lbm_init");
        if (d_in) cudaFree(d_in);
    }
    if (!rc) h->initialized = true;
    return rc;
}

int lbm_step_async(LbmHandle* h, int32_t n) {
    LbmNvtxRange nvtx("lbm_step");
    if (!h) return lbm_set_err(h, LBM_EINVAL, "lbm_step: NULL handle");
    if (!h->initialized) return lbm_set_err(h, LBM_ESTATE, "lbm_step: call lbm_init first");
    if (n < 0) return lbm_set_err(h, LBM_EINVAL, "lbm_step: negative step count");
    if (n == 0) return LBM_OK;
    cudaSetDevice(h->device);
    int rc = h->p.two_phase ? tp_launch_steps(h, n, true) : sp_launch_steps(h, n, true);
    if (rc) return rc;
    h->steps_done += n;
    h->macros_valid = true;
    return LBM_OK;
}

int lbm_synchronize(LbmHandle* h) {
    if (!h) return lbm_set_err(h, LBM_EINVAL, "lbm_synchronize: NULL handle");
    const int rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "stream synchronize");
    return rc ? rc : sp_debug_take(h);
}

int lbm_step(LbmHandle* h, int32_t n) {
    int rc = lbm_step_async(h, n);
    if (rc) return rc;
    return lbm_synchronize(h);
}

int lbm_get_stream(LbmHandle* h, void** stream) {
    if (!h || !stream) return lbm_set_err(h, LBM_EINVAL, "lbm_get_stream: NULL argument");
    *stream = (void*)h->stream;
    return LBM_OK;
}

}  // extern "C"

namespace {
// Copy a node-ordered device array (n components of stride np, FP32 or FP64)
// into a dense host array with `comps` interleaved components; solid cells get
// `fill` (scattered on the device, lbm_geom.cu).
template <typename O>
int scatter_dense(LbmHandle* h, const void* dsrc, int comps, O* out, O fill) {
    return geom_dense_out<O>(h, dsrc, comps, out, fill);
}
}  // namespace

extern "C" {

int lbm_get_macros(LbmHandle* h, float* rho, float* v) {
    LbmNvtxRange nvtx("lbm_get_macros");
    if (!h) return lbm_set_err(h, LBM_EINVAL, "lbm_get_macros: NULL handle");
    if (!h->have_geometry) return lbm_set_err(h, LBM_ESTATE, "lbm_get_macros: no geometry");
    cudaSetDevice(h->device);
    if (!h->macros_valid) {
        // before the first step: the initial state rho = 1, v = 0 (init, SP:160-170)
        if (rho) for (int64_t c = 0; c < h->ncell; ++c) rho[c] = 1.0f;
        if (v) for (int64_t c = 0; c < 3 * h->ncell; ++c) v[c] = 0.0f;
        return LBM_OK;
    }
    int rc = LBM_OK;
    if (rho) rc = scatter_dense<float>(h, h->d_rho, 1, rho, 1.0f);
    if (!rc && v) rc = scatter_dense<float>(h, h->d_v, 3, v, 0.0f);
    return rc;
}

int lbm_get_macros_f64(LbmHandle* h, double* rho, double* v) {
    if (!h) return lbm_set_err(h, LBM_EINVAL, "lbm_get_macros_f64: NULL handle");
    if (!h->have_geometry) return lbm_set_err(h, LBM_ESTATE, "lbm_get_macros_f64: no geometry");
    cudaSetDevice(h->device);
    if (!h->macros_valid) {
        if (rho) for (int64_t c = 0; c < h->ncell; ++c) rho[c] = 1.0;
        if (v) for (int64_t c = 0; c < 3 * h->ncell; ++c) v[c] = 0.0;
        return LBM_OK;
    }
    int rc = LBM_OK;
    if (rho) rc = scatter_dense<double>(h, h->d_rho, 1, rho, 1.0);
    if (!rc && v) rc = scatter_dense<double>(h, h->d_v, 3, v, 0.0);
    return rc;
}

int lbm_get_psi(LbmHandle* h, float* psi) {
    if (!psi) return lbm_set_err(h, LBM_EINVAL, "lbm_get_psi: NULL output");
    return lbm_get_phase(h, psi, nullptr, nullptr);
}

int lbm_get_phase(LbmHandle* h, float* psi, float* rho_r, float* rho_b) {
    if (!h) return lbm_set_err(h, LBM_EINVAL, "lbm_get_phase: NULL handle");
    if (!h->p.two_phase) return lbm_set_err(h, LBM_ESTATE, "lbm_get_phase: handle is single phase");
    if (!h->initialized) return lbm_set_err(h, LBM_ESTATE, "lbm_get_phase: call lbm_init first");
    cudaSetDevice(h->device);
    int rc = LBM_OK;
    if (psi) {
        // fluid cells from the device; solid cells keep the input psi (the reference never updates them)
        std::vector<float> fl(h->ncell);
        rc = geom_host_index(h);
        if (!rc) rc = scatter_dense<float>(h, h->d_psi, 1, fl.data(), 0.0f);
        if (!rc)
            for (int64_t c = 0; c < h->ncell; ++c) psi[c] = h->solid[c] ? h->psi0[c] : fl[c];
    }
    if (!rc && rho_r) rc = scatter_dense<float>(h, h->d_rr[h->ccur], 1, rho_r, 0.0f);
    if (!rc && rho_b) rc = scatter_dense<float>(h, h->d_rb[h->ccur], 1, rho_b, 0.0f);
    return rc;
}

int lbm_reductions(LbmHandle* h, LbmStats* out) {
    LbmNvtxRange nvtx("lbm_reductions");
    if (!h || !out) return lbm_set_err(h, LBM_EINVAL, "lbm_reductions: NULL argument");
    if (!h->have_geometry) return lbm_set_err(h, LBM_ESTATE, "lbm_reductions: no geometry");
    cudaSetDevice(h->device);
    if (!h->macros_valid) {
        out->mass = (double)h->n_fluid;
        out->mom[0] = out->mom[1] = out->mom[2] = 0;
        out->max_v = 0;
        out->n_nonfinite = 0;
        out->n_fluid = h->n_fluid;
        return LBM_OK;
    }
    return red_launch(h, out, nullptr);
}

int lbm_get_max_v(LbmHandle* h, float* out) {
    if (!h || !out) return lbm_set_err(h, LBM_EINVAL, "lbm_get_max_v: NULL argument");
    if (!h->have_geometry) return lbm_set_err(h, LBM_ESTATE, "lbm_get_max_v: no geometry");
    if (!h->macros_valid) { *out = 0.0f; return LBM_OK; }
    cudaSetDevice(h->device);
    LbmStats st;
    return red_launch(h, &st, out);
}

int lbm_run_to_convergence(LbmHandle* h, double tol, int32_t check_every, int64_t max_steps, int32_t axis,
                           double* darcy_v, int64_t* steps, int32_t* converged) {
    LbmNvtxRange nvtx("lbm_run_to_convergence");
    if (!h || !darcy_v || !steps || !converged) return lbm_set_err(h, LBM_EINVAL, "lbm_run_to_convergence: NULL argument");
    if (check_every < 1 || max_steps < 1 || axis < 0 || axis > 2 || !(tol >= 0))
        return lbm_set_err(h, LBM_EINVAL, "lbm_run_to_convergence: bad tol / check_every / max_steps / axis");
    if (!h->initialized) return lbm_set_err(h, LBM_ESTATE, "lbm_run_to_convergence: call lbm_init first");
    cudaSetDevice(h->device);
    double prev = 0.0, vm = 0.0;
    bool have_prev = false;
    int64_t done = 0;
    *converged = 0;
    while (done < max_steps) {
        const int32_t n = (int32_t)std::min<int64_t>(check_every, max_steps - done);
        int rc = lbm_step_async(h, n);
        if (rc) return rc;
        done += n;
        LbmStats st;
        rc = red_launch(h, &st, nullptr);
        if (rc) return rc;
        rc = sp_debug_take(h);       // -DLBM_DEBUG builds: index checks of these steps (LBM_OK otherwise)
        if (rc) return rc;
        if (st.n_nonfinite) {
            *darcy_v = NAN;
            *steps = done;
            return lbm_set_err(h, LBM_EDIVERGED, "lbm_run_to_convergence: non-finite rho or v");
        }
        vm = st.mom[axis] / (double)h->ncell;
        if (have_prev && std::fabs(vm - prev) <= tol * std::fabs(vm)) {
            *converged = 1;
            break;
        }
        prev = vm;
        have_prev = true;
    }
    *darcy_v = vm;
    *steps = done;
    return LBM_OK;
}

int lbm_get_info(LbmHandle* h, LbmInfo* out) {
    if (!h || !out) return lbm_set_err(h, LBM_EINVAL, "lbm_get_info: NULL argument");
    out->n_cells = h->ncell;
    out->n_fluid = h->n_fluid;
    out->steps_done = h->steps_done;
    out->device_bytes = h->device_bytes;
    out->storage = h->p.storage;
    out->two_phase = h->p.two_phase;
    out->sm_count = h->sm_count;
    out->abi_version = LBM_ABI_VERSION;
    return LBM_OK;
}

int lbm_get_fluid_index(LbmHandle* h, int32_t* cell_of_node) {
    if (!h || !cell_of_node) return lbm_set_err(h, LBM_EINVAL, "lbm_get_fluid_index: NULL argument");
    if (!h->have_geometry) return lbm_set_err(h, LBM_ESTATE, "lbm_get_fluid_index: no geometry");
    cudaSetDevice(h->device);
    const int rc = geom_host_index(h);
    if (rc) return rc;
    std::memcpy(cell_of_node, h->cell_of_node.data(), sizeof(int32_t) * h->n_fluid);
    return LBM_OK;
}

int lbm_get_neighbors(LbmHandle* h, int32_t* src) {
    if (!h || !src) return lbm_set_err(h, LBM_EINVAL, "lbm_get_neighbors: NULL argument");
    if (!h->have_geometry) return lbm_set_err(h, LBM_ESTATE, "lbm_get_neighbors: no geometry");
    // Read the map back from the device: the table is what the kernels use.
    cudaSetDevice(h->device);
    int rc = geom_host_index(h);
    if (rc) return rc;
    std::vector<int32_t> map(h->ncell);
    rc = lbm_cuda_check(h, cudaMemcpy(map.data(), h->d_map, sizeof(int32_t) * h->ncell, cudaMemcpyDeviceToHost), "copy map");
    if (rc) return rc;
    const int nx = h->p.nx, ny = h->p.ny, nz = h->p.nz;
    for (int32_t n = 0; n < h->n_fluid; ++n) {
        const int64_t c = h->cell_of_node[n];
        const int i = (int)(c % nx), j = (int)((c / nx) % ny), k = (int)(c / ((int64_t)nx * ny));
        for (int s = 1; s < 19; ++s) {
            int x = i - lbm_ex(s), y = j - lbm_ey(s), z = k - lbm_ez(s);
            if (x < 0) x = nx - 1;
            if (x > nx - 1) x = 0;
            if (y < 0) y = ny - 1;
            if (y > ny - 1) y = 0;
            if (z < 0) z = nz - 1;
            if (z > nz - 1) z = 0;
            const int32_t m = map[x + (int64_t)nx * (y + (int64_t)ny * z)];
            src[(int64_t)(s - 1) * h->n_fluid + n] = m >= 0 ? m : -1 - n;
        }
    }
    return LBM_OK;
}

// Reference density of the 16-bit codecs per fluid node (the device's FP32
// rho'_ref = a + b i at the node's x), empty for the other storages.
static int host_ref_density(LbmHandle* h, std::vector<float>& rr) {
    rr.clear();
    if (h->p.storage != LBM_STORE_F16_DEV && h->p.storage != LBM_STORE_BF16_DEV) return LBM_OK;
    int rc = geom_host_index(h);
    if (rc) return rc;
    const SpConsts<float> C = sp_make_consts<float>(h);
    rr.resize(h->np, 0.0f);
    for (int32_t n = 0; n < h->n_fluid; ++n)
        rr[n] = std::fmaf(C.ref_b, (float)(h->cell_of_node[n] % h->p.nx), C.ref_a);
    return LBM_OK;
}

int lbm_get_populations(LbmHandle* h, double* f) {
    if (!h || !f) return lbm_set_err(h, LBM_EINVAL, "lbm_get_populations: NULL argument");
    if (!h->initialized || h->p.two_phase) return lbm_set_err(h, LBM_ESTATE, "lbm_get_populations: needs an initialised single-phase handle");
    std::vector<unsigned char> tmp(h->elem * 19 * h->np);
    int rc = lbm_cuda_check(h, cudaMemcpy(tmp.data(), h->d_f[h->cur], tmp.size(), cudaMemcpyDeviceToHost), "copy f");
    if (rc) return rc;
    std::vector<float> rr;
    rc = host_ref_density(h, rr);
    if (rc) return rc;
    for (int s = 0; s < 19; ++s)
        for (int32_t n = 0; n < h->n_fluid; ++n) {
            const int64_t idx = lbm_pidx(n, s);
            double val = 0;
            switch (h->p.storage) {
            case LBM_STORE_F32: val = ((const float*)tmp.data())[idx]; break;
            case LBM_STORE_F64: val = ((const double*)tmp.data())[idx]; break;
            case LBM_STORE_F32_DEV: val = lbm_w(s) + (double)((const float*)tmp.data())[idx]; break;
            case LBM_STORE_F16_DEV:
                val = lbm_w(s) * (1.0 + rr[n]) + (double)__half2float(((const __half*)tmp.data())[idx]) / 65536.0;
                break;
            case LBM_STORE_BF16_DEV:
                val = lbm_w(s) * (1.0 + rr[n]) + (double)__bfloat162float(((const __nv_bfloat16*)tmp.data())[idx]);
                break;
            }
            f[(int64_t)s * h->n_fluid + n] = val;
        }
    return LBM_OK;
}

int lbm_set_populations(LbmHandle* h, const double* f) {
    if (!h || !f) return lbm_set_err(h, LBM_EINVAL, "lbm_set_populations: NULL argument");
    if (!h->initialized || h->p.two_phase) return lbm_set_err(h, LBM_ESTATE, "lbm_set_populations: needs an initialised single-phase handle");
    std::vector<unsigned char> tmp(h->elem * 19 * h->np, 0);
    std::vector<float> rr;
    int rc = host_ref_density(h, rr);
    if (rc) return rc;
    for (int s = 0; s < 19; ++s)
        for (int32_t n = 0; n < h->n_fluid; ++n) {
            const int64_t idx = lbm_pidx(n, s);
            const double val = f[(int64_t)s * h->n_fluid + n];
            const double g = rr.empty() ? 0.0 : val - lbm_w(s) * (1.0 + (double)rr[n]);   // 16-bit codecs only
            switch (h->p.storage) {
            case LBM_STORE_F32: ((float*)tmp.data())[idx] = (float)val; break;
            case LBM_STORE_F64: ((double*)tmp.data())[idx] = val; break;
            case LBM_STORE_F32_DEV: ((float*)tmp.data())[idx] = (float)(val - lbm_w(s)); break;
            case LBM_STORE_F16_DEV: ((__half*)tmp.data())[idx] = __float2half_rn((float)(g * 65536.0)); break;
            case LBM_STORE_BF16_DEV: ((__nv_bfloat16*)tmp.data())[idx] = __float2bfloat16_rn((float)g); break;
            }
        }
    rc = lbm_cuda_check(h, cudaMemcpy(h->d_f[h->cur], tmp.data(), tmp.size(), cudaMemcpyHostToDevice), "copy f");
    h->macros_valid = false;
    return rc;
}

int lbm_debug_stream(LbmHandle* h, const float* f_in, float* f_out) {
    if (!h || !f_in || !f_out) return lbm_set_err(h, LBM_EINVAL, "lbm_debug_stream: NULL argument");
    if (!h->have_geometry) return lbm_set_err(h, LBM_ESTATE, "lbm_debug_stream: no geometry");
    cudaSetDevice(h->device);
    float *din = nullptr, *dout = nullptr;
    const size_t bytes = sizeof(float) * 19 * h->np;
    if (cudaMalloc((void**)&din, bytes) != cudaSuccess || cudaMalloc((void**)&dout, bytes) != cudaSuccess) {
        if (din) cudaFree(din);
        return lbm_set_err(h, LBM_ENOMEM, "lbm_debug_stream: allocation failed");
    }
    std::vector<float> tmp(19 * h->np, 0.0f);
    for (int s = 0; s < 19; ++s)
        for (int32_t n = 0; n < h->n_fluid; ++n) tmp[lbm_pidx(n, s)] = f_in[(int64_t)s * h->n_fluid + n];
    int rc = lbm_cuda_check(h, cudaMemcpy(din, tmp.data(), bytes, cudaMemcpyHostToDevice), "copy in");
    if (!rc) rc = sp_launch_debug_stream(h, din, dout);
    if (!rc) rc = lbm_cuda_check(h, cudaStreamSynchronize(h->stream), "debug stream");
    if (!rc) rc = lbm_cuda_check(h, cudaMemcpy(tmp.data(), dout, bytes, cudaMemcpyDeviceToHost), "copy out");
    if (!rc)
        for (int s = 0; s < 19; ++s)
            for (int32_t n = 0; n < h->n_fluid; ++n) f_out[(int64_t)s * h->n_fluid + n] = tmp[lbm_pidx(n, s)];
    cudaFree(din);
    cudaFree(dout);
    return rc;
}

int lbm_last_error(LbmHandle* h, char* buf, size_t n) {
    if (!buf || n == 0) return LBM_EINVAL;
    std::string m;
    if (h) m = h->err;
    else {
        std::lock_guard<std::mutex> lk(g_err_mu);
        m = g_err;
    }
    std::snprintf(buf, n, "%s", m.c_str());
    return LBM_OK;
}

}  // extern "C"
