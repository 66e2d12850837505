/* CPU oracle of the STL voxeliser (include/lbm_vox.h).
 *
 * TEST INFRASTRUCTURE ONLY: tests/ are its only callers.  FP64 restatement of
 * the classification rule of Single_phase/Convert_stl_to_binary.cpp:86-123
 * (taichi_LBM3D tree): grid point (x0 + dx i, ...) formed in FP32, solid when
 * the generalized winding number has magnitude >= 1/2 or the point-triangle
 * distance is <= surf_eps.  The reference evaluates it with libigl (fast
 * winding number + AABB distance; libigl and Eigen are not in the reference
 * tree and not installed here), so this oracle restates the published
 * definitions instead: the solid angle of a triangle by Van Oosterom &
 * Strackee (1983) and the point-triangle distance by closest-point Voronoi
 * regions; every pair is evaluated, no acceleration structure.
 */
#include <math.h>
#include <stdint.h>

static double d3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static double seg_dist2(const double *p, const double *a, const double *b) {
    double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, ap[3] = {p[0] - a[0], p[1] - a[1], p[2] - a[2]};
    double L = d3(ab, ab), t = L > 0 ? d3(ap, ab) / L : 0.0;
    if (t < 0) t = 0;
    if (t > 1) t = 1;
    double q[3] = {ap[0] - t * ab[0], ap[1] - t * ab[1], ap[2] - t * ab[2]};
    return d3(q, q);
}

/* Squared distance from p to triangle abc: the plane projection when it falls
 * inside the triangle, else the nearest of the three edges. */
static double tri_dist2(const double *p, const double *a, const double *b, const double *c) {
    double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double n[3] = {ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2], ab[0] * ac[1] - ab[1] * ac[0]};
    double nn = d3(n, n);
    if (nn > 0) {
        double ap[3] = {p[0] - a[0], p[1] - a[1], p[2] - a[2]};
        double h = d3(ap, n) / nn;
        double q[3] = {p[0] - h * n[0], p[1] - h * n[1], p[2] - h * n[2]};
        /* barycentric sign test of q against the three edges */
        const double *v[3] = {a, b, c};
        int inside = 1;
        for (int e = 0; e < 3; ++e) {
            const double *u = v[e], *w = v[(e + 1) % 3];
            double uw[3] = {w[0] - u[0], w[1] - u[1], w[2] - u[2]}, uq[3] = {q[0] - u[0], q[1] - u[1], q[2] - u[2]};
            double cr[3] = {uw[1] * uq[2] - uw[2] * uq[1], uw[2] * uq[0] - uw[0] * uq[2], uw[0] * uq[1] - uw[1] * uq[0]};
            if (d3(cr, n) < 0) { inside = 0; break; }
        }
        if (inside) return h * h * nn;
    }
    double s0 = seg_dist2(p, a, b), s1 = seg_dist2(p, b, c), s2 = seg_dist2(p, c, a);
    return fmin(s0, fmin(s1, s2));
}

int lbm_oracle_voxelize(const float *tri, int64_t ntri, const float *origin, float dx, int32_t nx, int32_t ny,
                        int32_t nz, float surf_eps, int8_t *solid, double *winding) {
    if (!tri && ntri > 0) return -1;
    const int64_t npts = (int64_t)nx * ny * nz;
    const double eps = surf_eps < 0 ? 1e-5 * (double)dx : (double)surf_eps;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t q = 0; q < npts; ++q) {
        int i = (int)(q % nx), j = (int)((q / nx) % ny), k = (int)(q / ((int64_t)nx * ny));
        float pxf = origin[0] + dx * (float)i, pyf = origin[1] + dx * (float)j, pzf = origin[2] + dx * (float)k;
        double p[3] = {pxf, pyf, pzf};
        double sum = 0.0, dmin2 = INFINITY;
        for (int64_t t = 0; t < ntri; ++t) {
            const float *v = tri + 9 * t;
            double A[3] = {v[0], v[1], v[2]}, B[3] = {v[3], v[4], v[5]}, C[3] = {v[6], v[7], v[8]};
            double a[3] = {A[0] - p[0], A[1] - p[1], A[2] - p[2]};
            double b[3] = {B[0] - p[0], B[1] - p[1], B[2] - p[2]};
            double c[3] = {C[0] - p[0], C[1] - p[1], C[2] - p[2]};
            double la = sqrt(d3(a, a)), lb = sqrt(d3(b, b)), lc = sqrt(d3(c, c));
            double det = a[0] * (b[1] * c[2] - b[2] * c[1]) + a[1] * (b[2] * c[0] - b[0] * c[2]) +
                         a[2] * (b[0] * c[1] - b[1] * c[0]);
            double den = la * lb * lc + d3(a, b) * lc + d3(a, c) * lb + d3(b, c) * la;
            sum += 2.0 * atan2(det, den);
            double d2 = tri_dist2(p, A, B, C);
            if (d2 < dmin2) dmin2 = d2;
        }
        double w = sum / (4.0 * 3.14159265358979323846);
        if (winding) winding[q] = w;
        solid[q] = (fabs(w) >= 0.5 || dmin2 <= eps * eps) ? 1 : 0;
    }
    return 0;
}

/* Distance from each grid point to the mesh (for the tests' ambiguity band). */
int lbm_oracle_mesh_distance(const float *tri, int64_t ntri, const float *origin, float dx, int32_t nx, int32_t ny,
                             int32_t nz, double *dist) {
    const int64_t npts = (int64_t)nx * ny * nz;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t q = 0; q < npts; ++q) {
        int i = (int)(q % nx), j = (int)((q / nx) % ny), k = (int)(q / ((int64_t)nx * ny));
        double p[3] = {origin[0] + dx * (float)i, origin[1] + dx * (float)j, origin[2] + dx * (float)k};
        double dmin2 = INFINITY;
        for (int64_t t = 0; t < ntri; ++t) {
            const float *v = tri + 9 * t;
            double A[3] = {v[0], v[1], v[2]}, B[3] = {v[3], v[4], v[5]}, C[3] = {v[6], v[7], v[8]};
            double d2 = tri_dist2(p, A, B, C);
            if (d2 < dmin2) dmin2 = d2;
        }
        dist[q] = sqrt(dmin2);
    }
    return 0;
}
