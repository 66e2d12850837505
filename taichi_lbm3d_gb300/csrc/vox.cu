// STL -> voxel solid flags (include/lbm_vox.h).  VX = Single_phase/Convert_stl_to_binary.cpp
// (taichi_LBM3D tree).
//
// The reference classifies every grid point with libigl's
// signed_distance_fast_winding_number (VX:117-123): solid when the signed value
// (1 - 2|w|) * distance is <= 0, w the (Barnes-Hut approximated) winding
// number.  Here w is the exact generalized winding number
//     w(p) = sum over triangles of Omega_t(p) / (4 pi),
//     tan(Omega/2) = det[a b c] / (|a||b||c| + (a.b)|c| + (a.c)|b| + (b.c)|a|),
// a, b, c the triangle's vertices relative to p (Van Oosterom & Strackee, 1983),
// and "distance = 0" is a point-triangle distance <= surf_eps.
//
// Kernel: one thread per grid point, 128 points per CTA; triangles are staged
// through shared memory in tiles of 256 (every thread reads the same triangle:
// a broadcast), per-tile partial angles summed in FP32 and tiles in FP64.  The
// point-triangle distance (closest point by Voronoi regions, Ericson,
// Real-Time Collision Detection 5.1.5) is evaluated only for nearly coplanar
// pairs, the only ones that can be within surf_eps.  Work is points x
// triangles; this is compute-bound (atan2, three square roots per pair).
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "../../include/lbm_vox.h"
#include "lbm_internal.h"

namespace {
constexpr int VOX_THREADS = 128;
constexpr int VOX_TILE = 256;

__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return ax * bx + ay * by + az * bz;
}

// Squared distance from the origin to triangle (a, b, c) (coordinates relative to the point).
__device__ float tri_dist2(float ax, float ay, float az, float bx, float by, float bz, float cx, float cy, float cz) {
    // p = 0: ap = -a, bp = -b, cp = -c
    const float abx = bx - ax, aby = by - ay, abz = bz - az;
    const float acx = cx - ax, acy = cy - ay, acz = cz - az;
    const float d1 = -dot3(abx, aby, abz, ax, ay, az), d2 = -dot3(acx, acy, acz, ax, ay, az);
    if (d1 <= 0.f && d2 <= 0.f) return dot3(ax, ay, az, ax, ay, az);
    const float d3 = -dot3(abx, aby, abz, bx, by, bz), d4 = -dot3(acx, acy, acz, bx, by, bz);
    if (d3 >= 0.f && d4 <= d3) return dot3(bx, by, bz, bx, by, bz);
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
        const float v = d1 / (d1 - d3);
        const float qx = ax + v * abx, qy = ay + v * aby, qz = az + v * abz;
        return dot3(qx, qy, qz, qx, qy, qz);
    }
    const float d5 = -dot3(abx, aby, abz, cx, cy, cz), d6 = -dot3(acx, acy, acz, cx, cy, cz);
    if (d6 >= 0.f && d5 <= d6) return dot3(cx, cy, cz, cx, cy, cz);
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
        const float w = d2 / (d2 - d6);
        const float qx = ax + w * acx, qy = ay + w * acy, qz = az + w * acz;
        return dot3(qx, qy, qz, qx, qy, qz);
    }
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
        const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        const float qx = bx + w * (cx - bx), qy = by + w * (cy - by), qz = bz + w * (cz - bz);
        return dot3(qx, qy, qz, qx, qy, qz);
    }
    const float sum = va + vb + vc;
    if (!(sum > 0.f)) {   // degenerate triangle: nearest vertex
        return fminf(dot3(ax, ay, az, ax, ay, az), fminf(dot3(bx, by, bz, bx, by, bz), dot3(cx, cy, cz, cx, cy, cz)));
    }
    const float v = vb / sum, w = vc / sum;
    const float qx = ax + abx * v + acx * w, qy = ay + aby * v + acy * w, qz = az + abz * v + acz * w;
    return dot3(qx, qy, qz, qx, qy, qz);
}

__global__ void __launch_bounds__(VOX_THREADS) vox_winding_kernel(const float* __restrict__ tri, int64_t ntri, float x0,
                                                                 float y0, float z0, float dx, int nx, int ny,
                                                                 int64_t npts, float eps2, double* __restrict__ wout,
                                                                 int8_t* __restrict__ flag) {
    __shared__ float s_tri[VOX_TILE * 9];
    const int64_t q = (int64_t)blockIdx.x * VOX_THREADS + threadIdx.x;
    const bool live = q < npts;
    // grid point in FP32 as the reference forms it (VX:86-93)
    const int i = live ? (int)(q % nx) : 0;
    const int j = live ? (int)((q / nx) % ny) : 0;
    const int k = live ? (int)(q / ((int64_t)nx * ny)) : 0;
    const float px = x0 + dx * (float)i, py = y0 + dx * (float)j, pz = z0 + dx * (float)k;
    double total = 0.0;
    bool on_surface = false;
    for (int64_t t0 = 0; t0 < ntri; t0 += VOX_TILE) {
        const int nt = (int)min((int64_t)VOX_TILE, ntri - t0);
        __syncthreads();
        for (int e = threadIdx.x; e < nt * 9; e += VOX_THREADS) s_tri[e] = tri[t0 * 9 + e];
        __syncthreads();
        float part = 0.f;
        for (int t = 0; t < nt; ++t) {
            const float* v = s_tri + 9 * t;
            const float ax = v[0] - px, ay = v[1] - py, az = v[2] - pz;
            const float bx = v[3] - px, by = v[4] - py, bz = v[5] - pz;
            const float cx = v[6] - px, cy = v[7] - py, cz = v[8] - pz;
            const float la = sqrtf(dot3(ax, ay, az, ax, ay, az));
            const float lb = sqrtf(dot3(bx, by, bz, bx, by, bz));
            const float lc = sqrtf(dot3(cx, cy, cz, cx, cy, cz));
            const float det = ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
            const float lll = la * lb * lc;
            const float den = lll + dot3(ax, ay, az, bx, by, bz) * lc + dot3(ax, ay, az, cx, cy, cz) * lb +
                              dot3(bx, by, bz, cx, cy, cz) * la;
            part += 2.f * atan2f(det, den);
            if (fabsf(det) <= 1e-4f * lll && !on_surface)
                on_surface = tri_dist2(ax, ay, az, bx, by, bz, cx, cy, cz) <= eps2;
        }
        total += (double)part;
    }
    if (!live) return;
    const double w = total / (4.0 * 3.14159265358979323846);
    if (wout) wout[q] = w;
    flag[q] = (fabs(w) >= 0.5 || on_surface) ? 1 : 0;
}

template <typename T>
void vfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}
}  // namespace

extern "C" int lbm_voxelize(const float* tri, int64_t ntri, const float* origin, float dx, int32_t nx, int32_t ny,
                            int32_t nz, float surf_eps, int32_t device, int8_t* solid, double* winding) {
    if (!origin || !solid || (ntri > 0 && !tri)) return lbm_set_err(nullptr, LBM_EINVAL, "lbm_voxelize: NULL argument");
    if (ntri < 0 || nx < 1 || ny < 1 || nz < 1 || !(dx > 0.f))
        return lbm_set_err(nullptr, LBM_EINVAL, "lbm_voxelize: bad sizes (need ntri >= 0, nx, ny, nz >= 1, dx > 0)");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return lbm_set_err(nullptr, LBM_ENODEV, "lbm_voxelize: no such CUDA device");
    cudaSetDevice(device);
    const int64_t npts = (int64_t)nx * ny * nz;
    const float eps = surf_eps < 0.f ? 1e-5f * dx : surf_eps;
    float* d_tri = nullptr;
    double* d_w = nullptr;
    int8_t* d_flag = nullptr;
    cudaStream_t st = nullptr;
    std::string why;
    int code = LBM_ECUDA;
    auto ok = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess && why.empty()) why = std::string(what) + ": " + cudaGetErrorString(e);
        return why.empty();
    };
    auto alloc = [&](void** ptr, size_t bytes, const char* what) {
        if (!why.empty()) return false;
        if (cudaMalloc(ptr, bytes) != cudaSuccess) {
            *ptr = nullptr;
            why = std::string("out of device memory for ") + what;
            code = LBM_ENOMEM;
        }
        return why.empty();
    };
    if (ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream") &&
        alloc((void**)&d_tri, sizeof(float) * 9 * (size_t)(ntri > 0 ? ntri : 1), "triangles") &&
        alloc((void**)&d_flag, (size_t)npts, "flags") &&
        (!winding || alloc((void**)&d_w, sizeof(double) * (size_t)npts, "winding")) &&
        (ntri == 0 || ok(cudaMemcpyAsync(d_tri, tri, sizeof(float) * 9 * (size_t)ntri, cudaMemcpyHostToDevice, st), "copy triangles"))) {
        const int64_t blocks = (npts + VOX_THREADS - 1) / VOX_THREADS;
        vox_winding_kernel<<<(unsigned)blocks, VOX_THREADS, 0, st>>>(d_tri, ntri, origin[0], origin[1], origin[2], dx, nx,
                                                                    ny, npts, eps * eps, d_w, d_flag);
        if (ok(cudaGetLastError(), "vox_winding_kernel launch") &&
            ok(cudaMemcpyAsync(solid, d_flag, (size_t)npts, cudaMemcpyDeviceToHost, st), "copy flags") &&
            (!winding || ok(cudaMemcpyAsync(winding, d_w, sizeof(double) * (size_t)npts, cudaMemcpyDeviceToHost, st), "copy winding")))
            ok(cudaStreamSynchronize(st), "voxelize");
    }
    vfree(d_tri);
    vfree(d_w);
    vfree(d_flag);
    if (st) cudaStreamDestroy(st);
    if (!why.empty()) return lbm_set_err(nullptr, code, "lbm_voxelize: " + why);
    return LBM_OK;
}
