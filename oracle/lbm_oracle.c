/* CPU oracle for the D3Q19 MRT hot path of taichi_LBM3D.
 *
 * TEST INFRASTRUCTURE ONLY: tests/, the smoke check and bench.py's CPU-baseline
 * leg are its only callers.  It restates the reference's Taichi kernels in
 * plain C (OpenMP across cells), in FP32 (the parity build) and FP64 (the
 * accuracy build), keeping the reference's algorithm form: dense AoS lattice,
 * four sweeps per step, literal 19x19 moment products.
 *
 * Reference files restated (paths inside the taichi_LBM3D checkout):
 *   Single_phase/LBM_3D_SinglePhase_Solver.py   lines 9-481  (single phase, class)
 *   2phase/lbm_solver_3d_2phase_sparse.py        lines 99-606 (two phase, script)
 *   Grey_Scale/lbm_solver_3d_Macro_Sukop.py      lines 112-336 (grey scale, script)
 *
 * Parity pinning: tests/golden/make_golden.py runs those reference files
 * unmodified on small lattices (through a numpy stand-in for Taichi) and
 * stores their outputs; tests/test_oracle_golden.py checks this oracle against
 * every fixture.
 *
 * Build:  gcc -O3 -fopenmp -ffp-contract=off -fPIC -shared lbm_oracle.c -o liblbm_oracle.so -lm
 * (-ffp-contract=off: no fused multiply-add that the reference's own sums do not have).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct OracleParams {
    int32_t nx, ny, nz;
    int32_t bc[6];            /* x-left, x-right, y-left, y-right, z-left, z-right: 0 periodic, 1 pressure, 2 velocity */
    double rho_bc[6];
    double vel_bc[6][3];
    double niu;
    double force[3];
    int32_t visc_convention;  /* 0: tau = niu/3 + 0.5 (class, :127); 1: tau = 3 niu + 0.5 (scripts) */
    int32_t guo_convention;   /* 0: class /3, /9 (:236); 1: script, no factors; 2: standard 3, 9 */
    int32_t bc_form;          /* velocity faces: 0 class feq(s,1,u); 1 script in-place form */
    int32_t two_phase;
    double niu_l, niu_g, psi_solid, cap_a;
    int32_t psi_bc[6];
    double psi_val[6];
    /* Test-only emulation of the numpy-executed reference (golden fixtures):
     * bit 0: colour push applied sequentially in the reference's loop order
     *        (cells i-slowest, k-fastest; directions in order), as a serial run
     *        of colission's += would; bit 1: sv taken as the Python double wl/wg
     *        (then sother in FP64) where Compute_S_local assigns the constant. */
    int32_t ref_emulation;
    /* Grey-scale script (partial bounce-back, Grey_Scale/lbm_solver_3d_Macro_Sukop.py):
     * per-cell ns set through lbm_oracle_set(what = 8); x faces only. */
    int32_t grey;
} OracleParams;

/* e, w, LR: LBM_3D_SinglePhase_Solver.py:183-197, :85 */
static const int E[19][3] = {
    {0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
    {1, 1, 0}, {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 0, 1}, {-1, 0, -1}, {1, 0, -1},
    {-1, 0, 1}, {0, 1, 1}, {0, -1, -1}, {0, 1, -1}, {0, -1, 1}};
static const double W[19] = {1.0 / 3.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0,
                             1.0 / 18.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                             1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                             1.0 / 36.0};
static const int LR[19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};
/* M: LBM_3D_SinglePhase_Solver.py:64-82 */
static const int MMAT[19][19] = {
    {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
    {-1, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
    {1, -2, -2, -2, -2, -2, -2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
    {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0},
    {0, -2, 2, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0},
    {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1},
    {0, 0, 0, -2, 2, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1},
    {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1},
    {0, 0, 0, 0, 0, -2, 2, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1},
    {0, 2, 2, -1, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2},
    {0, -2, -2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2},
    {0, 0, 0, 1, 1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0},
    {0, 0, 0, -1, -1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, -1, 1, -1, 1, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0, -1, 1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, -1, 1, 1, -1}};

/* inv_M: the reference takes np.linalg.inv(M) in FP64 (:83).  Gauss-Jordan with
 * partial pivoting in FP64 gives the same matrix to ~1e-16; entries below 1e-12
 * are FP64 round-off of exact zeros (numpy leaves ~1e-18 there) and are set to
 * zero, which no FP32 partial sum can see. */
static void oracle_invert_M(double inv[19][19]) {
    double a[19][38];
    for (int r = 0; r < 19; ++r)
        for (int c = 0; c < 38; ++c) a[r][c] = c < 19 ? (double)MMAT[r][c] : (c - 19 == r ? 1.0 : 0.0);
    for (int col = 0; col < 19; ++col) {
        int piv = col;
        for (int r = col + 1; r < 19; ++r)
            if (fabs(a[r][col]) > fabs(a[piv][col])) piv = r;
        if (piv != col)
            for (int c = 0; c < 38; ++c) { double t = a[col][c]; a[col][c] = a[piv][c]; a[piv][c] = t; }
        double d = a[col][col];
        for (int c = 0; c < 38; ++c) a[col][c] /= d;
        for (int r = 0; r < 19; ++r) {
            if (r == col) continue;
            double fct = a[r][col];
            if (fct == 0) continue;
            for (int c = 0; c < 38; ++c) a[r][c] -= fct * a[col][c];
        }
    }
    for (int r = 0; r < 19; ++r)
        for (int c = 0; c < 19; ++c) {
            double x = a[r][c + 19];
            inv[r][c] = fabs(x) < 1e-12 ? 0.0 : x;
        }
}

#define REAL float
#define SFX f32
#include "lbm_oracle_body.h"
#undef REAL
#undef SFX

#define REAL double
#define SFX f64
#include "lbm_oracle_body.h"
#undef REAL
#undef SFX

/* ----------------------------------------------------------------- C ABI */
typedef struct OracleHandle {
    int precision;  /* 32 or 64 */
    void *impl;
} OracleHandle;

OracleHandle *lbm_oracle_create(const OracleParams *p, const int8_t *solid, const float *psi, int precision) {
    if (!p || !solid || p->nx < 1 || p->ny < 1 || p->nz < 1) return NULL;
    if (p->two_phase && !psi) return NULL;
    OracleHandle *h = (OracleHandle *)calloc(1, sizeof(*h));
    if (!h) return NULL;
    h->precision = precision == 64 ? 64 : 32;
    h->impl = h->precision == 64 ? (void *)oracle_create_f64(p, solid, psi) : (void *)oracle_create_f32(p, solid, psi);
    if (!h->impl) { free(h); return NULL; }
    return h;
}

void lbm_oracle_destroy(OracleHandle *h) {
    if (!h) return;
    if (h->precision == 64) oracle_destroy_f64((oracle_sp_f64 *)h->impl);
    else oracle_destroy_f32((oracle_sp_f32 *)h->impl);
    free(h);
}

int lbm_oracle_step(OracleHandle *h, int n) {
    if (!h) return -1;
    return h->precision == 64 ? oracle_step_f64((oracle_sp_f64 *)h->impl, n) : oracle_step_f32((oracle_sp_f32 *)h->impl, n);
}

int lbm_oracle_stream_only(OracleHandle *h) {
    if (!h) return -1;
    return h->precision == 64 ? oracle_stream_only_f64((oracle_sp_f64 *)h->impl)
                              : oracle_stream_only_f32((oracle_sp_f32 *)h->impl);
}

/* what: 0 rho, 1 v, 2 f, 3 F, 4 psi, 5 rho_r, 6 rho_b, 7 inv_M (19x19), 8 ns (grey) */
int lbm_oracle_get(OracleHandle *h, int what, double *out) {
    if (!h || !out) return -1;
    return h->precision == 64 ? oracle_get_f64((oracle_sp_f64 *)h->impl, what, out)
                              : oracle_get_f32((oracle_sp_f32 *)h->impl, what, out);
}

int lbm_oracle_set(OracleHandle *h, int what, const double *in) {
    if (!h || !in) return -1;
    return h->precision == 64 ? oracle_set_f64((oracle_sp_f64 *)h->impl, what, in)
                              : oracle_set_f32((oracle_sp_f32 *)h->impl, what, in);
}

int lbm_oracle_sizeof_params(void) { return (int)sizeof(OracleParams); }
