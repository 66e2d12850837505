/* STL surface mesh -> voxel solid flags on the GPU.
 *
 * Replaces Single_phase/Convert_stl_to_binary.cpp (taichi_LBM3D tree), which
 * flags grid point (i, j, k) = (x0 + dx i, y0 + dx j, z0 + dx k) (:86-93) as
 * solid when libigl's signed_distance_fast_winding_number is <= 0 (:117-123),
 * i.e. when the point's winding number has magnitude >= 1/2 or the point lies
 * on the surface.  Here the winding number is the exact generalized winding
 * number (sum of the signed solid angles of all triangles / 4 pi) that libigl's
 * fast winding number approximates, and "on the surface" is a point-triangle
 * distance <= surf_eps.
 */
#ifndef LBM_VOX_H
#define LBM_VOX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* tri: host array of ntri triangles x 3 vertices x 3 coordinates (FP32, as
 * STL stores them).  Grid points are formed in FP32 as origin[c] + dx * index.
 * solid (host, nx*ny*nz, x fastest): 1 solid / 0 fluid.  winding (host,
 * optional, may be NULL): the winding number of every grid point.
 * surf_eps < 0 selects 1e-5 * dx.  Runs on CUDA device `device` and waits for
 * the result.  Returns 0 or an LBM_E* code (message: lbm_last_error(NULL, ...)). */
int lbm_voxelize(const float* tri, int64_t ntri, const float* origin, float dx, int32_t nx, int32_t ny, int32_t nz,
                 float surf_eps, int32_t device, int8_t* solid, double* winding);

#ifdef __cplusplus
}
#endif

#endif
