/* Body of the CPU oracle, included once per arithmetic type by lbm_oracle.c
 * with REAL (float|double) and SFX (token suffix) defined.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a literal restatement of the reference's
 * Taichi kernels: the same four sweeps per time step (collide, push-stream,
 * face boundary conditions, macroscopic update), AoS storage of 19 values per
 * cell over the dense lattice, the full 19x19 moment products with the FP32
 * rounding of numpy's inverse.  Every function cites the reference lines it
 * follows.  The product never links or calls it; only tests/, the smoke check
 * and bench.py's CPU-baseline leg do.
 */
#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)
#define ST(name) CAT(name, SFX)

typedef struct ST(oracle_sp_) {
    OracleParams p;
    int64_t ncell;
    int8_t *solid;
    REAL *f, *F, *rho, *v;           /* AoS: f[cell*19+s], v[cell*3+c] */
    REAL S[19];
    REAL Mf[19][19], Minv[19][19];
    REAL fext[3];
    int force_flag;
    /* two-phase */
    REAL *psi, *rho_r, *rho_b, *Gr, *Gb;  /* Gr/Gb: colour slots [cell*19+s] */
    REAL wl, wg, lg0, l1, l2, g1, g2, psi_solid, capa;
    double wl_d, wg_d;
    /* grey scale */
    REAL *ns, *f2;                   /* ns[cell], f2[cell*19+s] */
} ST(oracle_sp_);

static inline int64_t FN(cid_)(const OracleParams *p, int i, int j, int k) {
    return (int64_t)i + (int64_t)p->nx * ((int64_t)j + (int64_t)p->ny * k);
}

/* feq: LBM_3D_SinglePhase_Solver.py:152-158 (w*rho*(1+3eu+4.5eu^2-1.5u^2)) */
static inline REAL FN(feq_)(int k, REAL rho, const REAL u[3]) {
    REAL eu = (REAL)E[k][0] * u[0];
    eu = eu + (REAL)E[k][1] * u[1];
    eu = eu + (REAL)E[k][2] * u[2];
    REAL uv = u[0] * u[0];
    uv = uv + u[1] * u[1];
    uv = uv + u[2] * u[2];
    REAL w = (REAL)W[k];
    REAL t = (REAL)1.0 + (REAL)3.0 * eu;
    t = t + ((REAL)4.5 * eu) * eu;
    t = t - (REAL)1.5 * uv;
    return (w * rho) * t;
}

/* meq_vec: LBM_3D_SinglePhase_Solver.py:209-215 */
static inline void FN(meq_)(REAL rho, const REAL u[3], REAL out[19]) {
    for (int s = 0; s < 19; ++s) out[s] = 0;
    out[0] = rho; out[3] = u[0]; out[5] = u[1]; out[7] = u[2];
    REAL uu = u[0] * u[0]; uu = uu + u[1] * u[1]; uu = uu + u[2] * u[2];
    out[1] = uu;
    out[9] = (((REAL)2 * u[0]) * u[0] - u[1] * u[1]) - u[2] * u[2];
    out[11] = u[1] * u[1] - u[2] * u[2];
    out[13] = u[0] * u[1];
    out[14] = u[1] * u[2];
    out[15] = u[0] * u[2];
}

/* Sequential 19x19 product out = A @ x, accumulated left to right from the
 * first product (Taichi's unrolled matmul). */
static inline void FN(matvec_)(REAL A[19][19], const REAL *x, REAL out[19]) {
    for (int r = 0; r < 19; ++r) {
        REAL acc = A[r][0] * x[0];
        for (int c = 1; c < 19; ++c) acc = acc + A[r][c] * x[c];
        out[r] = acc;
    }
}

static void FN(setup_consts_)(ST(oracle_sp_) *o) {
    /* M: LBM_3D_SinglePhase_Solver.py:64-82; inv_M = fp32(np.linalg.inv(M)) (:83,:110) */
    double inv[19][19];
    oracle_invert_M(inv);
    for (int r = 0; r < 19; ++r)
        for (int c = 0; c < 19; ++c) {
            o->Mf[r][c] = (REAL)MMAT[r][c];
            o->Minv[r][c] = (REAL)inv[r][c];
        }
    /* init_simulation: LBM_3D_SinglePhase_Solver.py:126-131 (tau convention Q1) */
    double tau = o->p.visc_convention == 0 ? o->p.niu / 3.0 + 0.5 : 3.0 * o->p.niu + 0.5;
    double sv = 1.0 / tau;
    double so = 8.0 * (2.0 - sv) / (8.0 - sv);
    REAL svr = (REAL)sv, sor = (REAL)so;
    const int kind[19] = {0, 1, 1, 0, 2, 0, 2, 0, 2, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2};
    for (int s = 0; s < 19; ++s) o->S[s] = kind[s] == 0 ? (REAL)0 : (kind[s] == 1 ? svr : sor);
    for (int c = 0; c < 3; ++c) o->fext[c] = (REAL)o->p.force[c];
    o->force_flag = (o->p.force[0] != 0 || o->p.force[1] != 0 || o->p.force[2] != 0);
    /* two-phase relaxation constants: 2phase/lbm_solver_3d_2phase_sparse.py:102-110,
     * Python doubles that Taichi folds to f32 constants */
    double wl = 1.0 / (o->p.niu_l / (1.0 / 3.0) + 0.5);
    double wg = 1.0 / (o->p.niu_g / (1.0 / 3.0) + 0.5);
    double lg0 = 2 * wl * wg / (wl + wg);
    double l1 = 2 * (wl - lg0) * 10, l2 = -l1 / 0.2;
    double g1 = 2 * (lg0 - wg) * 10, g2 = g1 / 0.2;
    o->wl = (REAL)wl; o->wg = (REAL)wg; o->lg0 = (REAL)lg0;
    o->wl_d = wl; o->wg_d = wg;
    o->l1 = (REAL)l1; o->l2 = (REAL)l2; o->g1 = (REAL)g1; o->g2 = (REAL)g2;
    o->psi_solid = (REAL)o->p.psi_solid;
    o->capa = (REAL)o->p.cap_a;
}

ST(oracle_sp_) *FN(oracle_create_)(const OracleParams *p, const int8_t *solid, const float *psi) {
    ST(oracle_sp_) *o = (ST(oracle_sp_) *)calloc(1, sizeof(*o));
    if (!o) return NULL;
    o->p = *p;
    o->ncell = (int64_t)p->nx * p->ny * p->nz;
    int64_t n = o->ncell;
    o->solid = (int8_t *)malloc(n);
    o->f = (REAL *)malloc(sizeof(REAL) * n * 19);
    o->F = (REAL *)malloc(sizeof(REAL) * n * 19);
    o->rho = (REAL *)malloc(sizeof(REAL) * n);
    o->v = (REAL *)malloc(sizeof(REAL) * n * 3);
    if (!o->solid || !o->f || !o->F || !o->rho || !o->v) return NULL;
    for (int64_t c = 0; c < n; ++c) o->solid[c] = solid[c] > 0 ? 1 : 0;   /* init_geo: :175 */
    FN(setup_consts_)(o);
    const REAL zero[3] = {0, 0, 0};
    /* init: LBM_3D_SinglePhase_Solver.py:160-170 (dense: every cell) */
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < n; ++c) {
        o->rho[c] = 1;
        o->v[c * 3 + 0] = o->v[c * 3 + 1] = o->v[c * 3 + 2] = 0;
        for (int s = 0; s < 19; ++s) o->f[c * 19 + s] = o->F[c * 19 + s] = FN(feq_)(s, (REAL)1.0, zero);
    }
    if (p->grey) {
        /* ns = 0 until set; f2 as the script allocates it (:32) */
        o->ns = (REAL *)calloc((size_t)n, sizeof(REAL));
        o->f2 = (REAL *)calloc((size_t)n * 19, sizeof(REAL));
        if (!o->ns || !o->f2) return NULL;
    }
    if (p->two_phase) {
        o->psi = (REAL *)malloc(sizeof(REAL) * n);
        o->rho_r = (REAL *)malloc(sizeof(REAL) * n);
        o->rho_b = (REAL *)malloc(sizeof(REAL) * n);
        o->Gr = (REAL *)malloc(sizeof(REAL) * n * 19);
        o->Gb = (REAL *)malloc(sizeof(REAL) * n * 19);
        if (!o->psi || !o->rho_r || !o->rho_b || !o->Gr || !o->Gb) return NULL;
        /* init: 2phase/lbm_solver_3d_2phase_sparse.py:174-187 */
        for (int64_t c = 0; c < n; ++c) {
            o->psi[c] = (REAL)psi[c];
            o->rho_r[c] = o->rho_b[c] = 0;
            if (!o->solid[c]) {
                o->rho_r[c] = (o->psi[c] + (REAL)1.0) / (REAL)2.0;
                o->rho_b[c] = (REAL)1.0 - o->rho_r[c];
            }
        }
    }
    return o;
}

void FN(oracle_destroy_)(ST(oracle_sp_) *o) {
    if (!o) return;
    free(o->solid); free(o->f); free(o->F); free(o->rho); free(o->v);
    free(o->psi); free(o->rho_r); free(o->rho_b); free(o->Gr); free(o->Gb);
    free(o->ns); free(o->f2);
    free(o);
}

/* periodic_index: LBM_3D_SinglePhase_Solver.py:247-257 */
static inline int64_t FN(wrap_)(const OracleParams *p, int i, int j, int k) {
    if (i < 0) i = p->nx - 1;
    if (i > p->nx - 1) i = 0;
    if (j < 0) j = p->ny - 1;
    if (j > p->ny - 1) j = 0;
    if (k < 0) k = p->nz - 1;
    if (k > p->nz - 1) k = 0;
    return FN(cid_)(p, i, j, k);
}

/* periodic_index_for_psi: 2phase/lbm_solver_3d_2phase_sparse.py:390-429 */
static inline int64_t FN(wrap_psi_)(const OracleParams *p, int i, int j, int k) {
    if (i < 0) i = p->psi_bc[0] == 0 ? p->nx - 1 : 0;
    if (i > p->nx - 1) i = p->psi_bc[1] == 0 ? 0 : p->nx - 1;
    if (j < 0) j = p->psi_bc[2] == 0 ? p->ny - 1 : 0;
    if (j > p->ny - 1) j = p->psi_bc[3] == 0 ? 0 : p->ny - 1;
    if (k < 0) k = p->psi_bc[4] == 0 ? p->nz - 1 : 0;
    if (k > p->nz - 1) k = p->psi_bc[5] == 0 ? 0 : p->nz - 1;
    return FN(cid_)(p, i, j, k);
}

/* colission (single phase): LBM_3D_SinglePhase_Solver.py:222-241.
 * guo_convention 0 = class (/3, /9, :236); 1 = scripts (no factors,
 * lbm_solver_3d_sparse.py:201). */
static void FN(collide_sp_)(ST(oracle_sp_) *o) {
    const OracleParams *p = &o->p;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < o->ncell; ++c) {
        if (o->solid[c]) continue;
        REAL m[19], meq[19], out[19];
        FN(matvec_)(o->Mf, &o->F[c * 19], m);
        const REAL *u = &o->v[c * 3];
        FN(meq_)(o->rho[c], u, meq);
        for (int s = 0; s < 19; ++s) m[s] = m[s] - o->S[s] * (m[s] - meq[s]);
        if (o->force_flag) {
            const REAL *fv = o->fext;
            for (int s = 0; s < 19; ++s) {
                REAL fg = 0;
                for (int l = 0; l < 19; ++l) {
                    REAL a = ((REAL)E[l][0] - u[0]) * fv[0];
                    a = a + ((REAL)E[l][1] - u[1]) * fv[1];
                    a = a + ((REAL)E[l][2] - u[2]) * fv[2];
                    REAL eu = (REAL)E[l][0] * u[0]; eu = eu + (REAL)E[l][1] * u[1]; eu = eu + (REAL)E[l][2] * u[2];
                    REAL ef = (REAL)E[l][0] * fv[0]; ef = ef + (REAL)E[l][1] * fv[1]; ef = ef + (REAL)E[l][2] * fv[2];
                    REAL g;
                    if (p->guo_convention == 0) g = a / (REAL)3.0 + (eu * ef) / (REAL)9.0;
                    else if (p->guo_convention == 1) g = a + eu * ef;
                    else g = (REAL)3.0 * a + (REAL)9.0 * (eu * ef);  /* standard Guo (not in the reference) */
                    fg = fg + ((REAL)W[l] * g) * o->Mf[s][l];
                }
                m[s] = m[s] + ((REAL)1 - (REAL)0.5 * o->S[s]) * fg;
            }
        }
        FN(matvec_)(o->Minv, m, out);
        for (int s = 0; s < 19; ++s) o->f[c * 19 + s] = (REAL)0 + out[s];
    }
}

/* streaming1: LBM_3D_SinglePhase_Solver.py:259-269 (push + halfway bounce-back) */
static void FN(stream_)(ST(oracle_sp_) *o) {
    const OracleParams *p = &o->p;
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = 0; k < p->nz; ++k)
        for (int j = 0; j < p->ny; ++j)
            for (int i = 0; i < p->nx; ++i) {
                int64_t c = FN(cid_)(p, i, j, k);
                if (o->solid[c]) continue;
                for (int s = 0; s < 19; ++s) {
                    int64_t ip = FN(wrap_)(p, i + E[s][0], j + E[s][1], k + E[s][2]);
                    if (o->solid[ip] == 0) o->F[ip * 19 + s] = o->f[c * 19 + s];
                    else o->F[c * 19 + LR[s]] = o->f[c * 19 + s];
                }
            }
}

/* Boundary_condition: LBM_3D_SinglePhase_Solver.py:272-370 (class form: velocity
 * faces get feq(s,1,u_bc)); 2phase/lbm_solver_3d_2phase_sparse.py:491-584 (script
 * form: F[s]=feq(LR[s],1,u)-F[LR[s]]+feq(s,1,u), in place, in s order).
 * Faces in order x-left, x-right, y-left, y-right, z-left, z-right. */
static void FN(bc_face_)(ST(oracle_sp_) *o, int face) {
    const OracleParams *p = &o->p;
    int type = p->bc[face];
    if (type == 0) return;
    int axis = face / 2, hi = face & 1;
    int n[3] = {p->nx, p->ny, p->nz};
    int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
    int plane = hi ? n[axis] - 1 : 0, inward = hi ? n[axis] - 2 : 1;
    REAL ubc[3] = {(REAL)p->vel_bc[face][0], (REAL)p->vel_bc[face][1], (REAL)p->vel_bc[face][2]};
    REAL rbc = (REAL)p->rho_bc[face];
#pragma omp parallel for schedule(static) collapse(2)
    for (int b = 0; b < n[a2]; ++b)
        for (int a = 0; a < n[a1]; ++a) {
            int x[3], xi[3];
            x[axis] = plane; x[a1] = a; x[a2] = b;
            xi[axis] = inward; xi[a1] = a; xi[a2] = b;
            int64_t c = FN(cid_)(p, x[0], x[1], x[2]);
            if (o->solid[c] != 0) continue;
            REAL *Fc = &o->F[c * 19];
            if (type == 1) {
                int64_t ci = FN(cid_)(p, xi[0], xi[1], xi[2]);
                const REAL *u = o->solid[ci] > 0 ? &o->v[ci * 3] : &o->v[c * 3];
                for (int s = 0; s < 19; ++s) Fc[s] = FN(feq_)(s, rbc, u);
            } else if (p->bc_form == 0) {
                for (int s = 0; s < 19; ++s) Fc[s] = FN(feq_)(s, (REAL)1.0, ubc);
            } else {
                for (int s = 0; s < 19; ++s)
                    Fc[s] = (FN(feq_)(LR[s], (REAL)1.0, ubc) - Fc[LR[s]]) + FN(feq_)(s, (REAL)1.0, ubc);
            }
        }
}

/* Grey scale, streaming0: Grey_Scale/lbm_solver_3d_Macro_Sukop.py:234-240.
 * Partial bounce-back mixed with the opposite population of the neighbour the
 * population moves to: f2[c,s] = f[c,s] + ns[c] (f[c+e_s, LR s] - f[c,s]).
 * f at solid cells is never written after init (feq(s, 1, 0)). */
static void FN(grey_stream0_)(ST(oracle_sp_) *o) {
    const OracleParams *p = &o->p;
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = 0; k < p->nz; ++k)
        for (int j = 0; j < p->ny; ++j)
            for (int i = 0; i < p->nx; ++i) {
                int64_t c = FN(cid_)(p, i, j, k);
                if (o->solid[c]) continue;
                for (int s = 0; s < 19; ++s) {
                    int64_t ip = FN(wrap_)(p, i + E[s][0], j + E[s][1], k + E[s][2]);
                    const REAL a = o->f[c * 19 + s];
                    o->f2[c * 19 + s] = a + o->ns[c] * (o->f[ip * 19 + LR[s]] - a);
                }
            }
}

/* Grey scale, streaming1: Grey_Scale/lbm_solver_3d_Macro_Sukop.py:243-252.
 * Plain push of f2 from every fluid cell, also into solid cells; F of a fluid
 * cell whose upstream cell is solid keeps its previous value. */
static void FN(grey_stream1_)(ST(oracle_sp_) *o) {
    const OracleParams *p = &o->p;
    /* each (cell, s) slot has exactly one source cell, so the sweep is order-free */
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = 0; k < p->nz; ++k)
        for (int j = 0; j < p->ny; ++j)
            for (int i = 0; i < p->nx; ++i) {
                int64_t c = FN(cid_)(p, i, j, k);
                if (o->solid[c]) continue;
                for (int s = 0; s < 19; ++s) {
                    int64_t ip = FN(wrap_)(p, i + E[s][0], j + E[s][1], k + E[s][2]);
                    o->F[ip * 19 + s] = o->f2[c * 19 + s];
                }
            }
}

/* streaming3: LBM_3D_SinglePhase_Solver.py:372-392 */
static void FN(macros_sp_)(ST(oracle_sp_) *o) {
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < o->ncell; ++c) {
        REAL *vc = &o->v[c * 3];
        if (o->solid[c] == 0) {
            const REAL *Fc = &o->F[c * 19];
            REAL *fc = &o->f[c * 19];
            REAL sum = Fc[0];
            for (int s = 0; s < 19; ++s) fc[s] = Fc[s];
            for (int s = 1; s < 19; ++s) sum = sum + fc[s];
            REAL r = (REAL)0 + sum;
            REAL vx = 0, vy = 0, vz = 0;
            for (int s = 0; s < 19; ++s) {
                vx = vx + (REAL)E[s][0] * fc[s];
                vy = vy + (REAL)E[s][1] * fc[s];
                vz = vz + (REAL)E[s][2] * fc[s];
            }
            vx = vx / r; vy = vy / r; vz = vz / r;
            vx = vx + (o->fext[0] / (REAL)2) / r;
            vy = vy + (o->fext[1] / (REAL)2) / r;
            vz = vz + (o->fext[2] / (REAL)2) / r;
            o->rho[c] = r; vc[0] = vx; vc[1] = vy; vc[2] = vz;
        } else {
            o->rho[c] = 1; vc[0] = vc[1] = vc[2] = 0;
        }
    }
}

/* ---------------------------------------------------------------- two phase */

/* Compute_C: 2phase/lbm_solver_3d_2phase_sparse.py:259-276 */
static inline void FN(colour_grad_)(ST(oracle_sp_) *o, int i, int j, int k, int64_t c, REAL C[3]) {
    const OracleParams *p = &o->p;
    C[0] = C[1] = C[2] = 0;
    int ind_s = 0;
    for (int s = 0; s < 19; ++s) {
        int64_t ip = FN(wrap_psi_)(p, i + E[s][0], j + E[s][1], k + E[s][2]);
        REAL ps;
        if (o->solid[ip] == 0) ps = o->psi[ip];
        else { ind_s = 1; ps = o->psi_solid; }
        REAL tw = (REAL)3.0 * (REAL)W[s];
        for (int d = 0; d < 3; ++d) C[d] = C[d] + (tw * (REAL)E[s][d]) * ps;
    }
    REAL dr = o->rho_r[c] - o->rho_b[c];
    if (dr < 0) dr = -dr;
    if (dr > (REAL)0.9 && ind_s == 1) C[0] = C[1] = C[2] = 0;
}

/* Compute_S_local: 2phase/lbm_solver_3d_2phase_sparse.py:278-300 */
static inline void FN(s_local_)(ST(oracle_sp_) *o, REAL psi, REAL S[19]) {
    REAL sv;
    double svd = 0;
    int from_const = 0;
    if (psi > 0) {
        if (psi > (REAL)0.1) { sv = o->wl; svd = o->wl_d; from_const = 1; }
        else sv = (o->lg0 + o->l1 * psi) + (o->l2 * psi) * psi;
    } else {
        if (psi < (REAL)-0.1) { sv = o->wg; svd = o->wg_d; from_const = 1; }
        else sv = (o->lg0 + o->g1 * psi) + (o->g2 * psi) * psi;
    }
    REAL so = ((REAL)8.0 * ((REAL)2.0 - sv)) / ((REAL)8.0 - sv);
    if (from_const && (o->p.ref_emulation & 2)) so = (REAL)(8.0 * (2.0 - svd) / (8.0 - svd));
    const int kind[19] = {0, 1, 1, 0, 2, 0, 2, 0, 2, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2};
    for (int s = 0; s < 19; ++s) S[s] = kind[s] == 0 ? (REAL)0 : (kind[s] == 1 ? sv : so);
}

/* colission (two phase): 2phase/lbm_solver_3d_2phase_sparse.py:302-373.  The colour
 * push (:366-373) is written into per-(cell, direction) slots Gr/Gb exactly like
 * streaming1 moves populations; the macros sweep sums each cell's 19 slots in
 * direction order, which is one of the orders Taichi's atomic += can produce. */
static void FN(collide_tp_)(ST(oracle_sp_) *o) {
    const OracleParams *p = &o->p;
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = 0; k < p->nz; ++k)
        for (int j = 0; j < p->ny; ++j)
            for (int i = 0; i < p->nx; ++i) {
                int64_t c = FN(cid_)(p, i, j, k);
                if (o->solid[c]) continue;
                const REAL *u = &o->v[c * 3];
                REAL C[3];
                FN(colour_grad_)(o, i, j, k, c, C);
                REAL cc2 = C[0] * C[0]; cc2 = cc2 + C[1] * C[1]; cc2 = cc2 + C[2] * C[2];
                REAL cc = (REAL)sqrt((double)cc2);
                if (sizeof(REAL) == 4) cc = (REAL)sqrtf((float)cc2);
                REAL nrm[3] = {0, 0, 0};
                if (cc > 0) { nrm[0] = C[0] / cc; nrm[1] = C[1] / cc; nrm[2] = C[2] / cc; }
                REAL m[19], meq[19], out[19], S[19];
                FN(matvec_)(o->Mf, &o->F[c * 19], m);
                FN(meq_)(o->rho[c], u, meq);
                REAL hc = ((REAL)0.5 * o->capa) * cc;
                meq[1] = meq[1] + o->capa * cc;
                meq[9] = meq[9] + hc * ((((REAL)2 * nrm[0]) * nrm[0] - nrm[1] * nrm[1]) - nrm[2] * nrm[2]);
                meq[11] = meq[11] + hc * (nrm[1] * nrm[1] - nrm[2] * nrm[2]);
                meq[13] = meq[13] + hc * (nrm[0] * nrm[1]);
                meq[14] = meq[14] + hc * (nrm[1] * nrm[2]);
                meq[15] = meq[15] + hc * (nrm[0] * nrm[2]);
                FN(s_local_)(o, o->psi[c], S);
                const REAL *fv = o->fext;
                for (int s = 0; s < 19; ++s) {
                    m[s] = m[s] - S[s] * (m[s] - meq[s]);
                    /* GuoF: :242-248 (script form, no /3 /9) */
                    REAL fg = 0;
                    for (int l = 0; l < 19; ++l) {
                        REAL a = ((REAL)E[l][0] - u[0]) * fv[0];
                        a = a + ((REAL)E[l][1] - u[1]) * fv[1];
                        a = a + ((REAL)E[l][2] - u[2]) * fv[2];
                        REAL eu = (REAL)E[l][0] * u[0]; eu = eu + (REAL)E[l][1] * u[1]; eu = eu + (REAL)E[l][2] * u[2];
                        REAL ef = (REAL)E[l][0] * fv[0]; ef = ef + (REAL)E[l][1] * fv[1]; ef = ef + (REAL)E[l][2] * fv[2];
                        fg = fg + ((REAL)W[l] * (a + eu * ef)) * o->Mf[s][l];
                    }
                    m[s] = m[s] + ((REAL)1 - (REAL)0.5 * S[s]) * fg;
                }
                FN(matvec_)(o->Minv, m, out);
                REAL gr[19], gb[19];
                for (int s = 0; s < 19; ++s) {
                    o->f[c * 19 + s] = (REAL)0 + out[s];
                    gr[s] = FN(feq_)(s, o->rho_r[c], u);
                    gb[s] = FN(feq_)(s, o->rho_b[c], u);
                }
                if (cc > 0) {
                    for (int kk = 1; kk < 19; kk += 2) {
                        REAL ef = (REAL)E[kk][0] * C[0]; ef = ef + (REAL)E[kk][1] * C[1]; ef = ef + (REAL)E[kk][2] * C[2];
                        REAL cp = gr[kk] < gr[kk + 1] ? gr[kk] : gr[kk + 1];
                        cp = cp < gb[kk] ? cp : gb[kk];
                        cp = cp < gb[kk + 1] ? cp : gb[kk + 1];
                        cp = cp * (ef / cc);
                        gr[kk] = gr[kk] + cp;
                        gr[kk + 1] = gr[kk + 1] - cp;
                        gb[kk] = gb[kk] - cp;
                        gb[kk + 1] = gb[kk + 1] + cp;
                    }
                }
                if (p->ref_emulation & 1) {
                    /* keep this cell's 19 colour values for the serial push below */
                    for (int s = 0; s < 19; ++s) { o->Gr[c * 19 + s] = gr[s]; o->Gb[c * 19 + s] = gb[s]; }
                    continue;
                }
                for (int s = 0; s < 19; ++s) {
                    int64_t ip = FN(wrap_)(p, i + E[s][0], j + E[s][1], k + E[s][2]);
                    if (o->solid[ip] == 0) { o->Gr[ip * 19 + s] = gr[s]; o->Gb[ip * 19 + s] = gb[s]; }
                    else { o->Gr[c * 19 + LR[s]] = gr[s]; o->Gb[c * 19 + LR[s]] = gb[s]; }
                }
            }
    if (p->ref_emulation & 1) {
        /* colission :366-373 run serially: cells i-slowest, k-fastest (Taichi's
         * struct-for order over rho), += into rhor/rhob from 0 */
        int64_t n = o->ncell;
        REAL *acc_r = (REAL *)calloc(n, sizeof(REAL)), *acc_b = (REAL *)calloc(n, sizeof(REAL));
        for (int i = 0; i < p->nx; ++i)
            for (int j = 0; j < p->ny; ++j)
                for (int k = 0; k < p->nz; ++k) {
                    int64_t c = FN(cid_)(p, i, j, k);
                    if (o->solid[c]) continue;
                    for (int s = 0; s < 19; ++s) {
                        int64_t ip = FN(wrap_)(p, i + E[s][0], j + E[s][1], k + E[s][2]);
                        int64_t dst = o->solid[ip] == 0 ? ip : c;
                        acc_r[dst] = acc_r[dst] + o->Gr[c * 19 + s];
                        acc_b[dst] = acc_b[dst] + o->Gb[c * 19 + s];
                    }
                }
        /* hand the sums to the macros sweep in slot 0 (slots 1..18 zero) */
        for (int64_t c = 0; c < n; ++c) {
            for (int s = 0; s < 19; ++s) o->Gr[c * 19 + s] = o->Gb[c * 19 + s] = 0;
            o->Gr[c * 19] = acc_r[c]; o->Gb[c * 19] = acc_b[c];
        }
        free(acc_r); free(acc_b);
    }
}

/* streaming3 (two phase): 2phase/lbm_solver_3d_2phase_sparse.py:587-606 (psi quirk Q9) */
static void FN(macros_tp_)(ST(oracle_sp_) *o) {
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < o->ncell; ++c) {
        if (o->solid[c]) continue;
        const REAL *Fc = &o->F[c * 19];
        REAL *fc = &o->f[c * 19];
        REAL r = 0, vx = 0, vy = 0, vz = 0, rr = 0, rb = 0;
        for (int s = 0; s < 19; ++s) {
            fc[s] = Fc[s];
            r = r + fc[s];
            vx = vx + (REAL)E[s][0] * fc[s];
            vy = vy + (REAL)E[s][1] * fc[s];
            vz = vz + (REAL)E[s][2] * fc[s];
            rr = rr + o->Gr[c * 19 + s];
            rb = rb + o->Gb[c * 19 + s];
        }
        vx = vx / r; vy = vy / r; vz = vz / r;
        vx = vx + (o->fext[0] / (REAL)2) / r;
        vy = vy + (o->fext[1] / (REAL)2) / r;
        vz = vz + (o->fext[2] / (REAL)2) / r;
        o->rho[c] = r; o->v[c * 3] = vx; o->v[c * 3 + 1] = vy; o->v[c * 3 + 2] = vz;
        o->rho_r[c] = rr; o->rho_b[c] = rb;
        o->psi[c] = rr - rb / (rr + rb);
    }
}

/* Boundary_condition_psi: 2phase/lbm_solver_3d_2phase_sparse.py:445-487 */
static void FN(bc_psi_)(ST(oracle_sp_) *o) {
    const OracleParams *p = &o->p;
    int n[3] = {p->nx, p->ny, p->nz};
    for (int face = 0; face < 6; ++face) {
        if (p->psi_bc[face] != 1) continue;
        int axis = face / 2, hi = face & 1;
        int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
        int plane = hi ? n[axis] - 1 : 0;
        REAL pv = (REAL)p->psi_val[face];
        REAL rr = (pv + (REAL)1.0) / (REAL)2.0;
        for (int b = 0; b < n[a2]; ++b)
            for (int a = 0; a < n[a1]; ++a) {
                int x[3];
                x[axis] = plane; x[a1] = a; x[a2] = b;
                int64_t c = FN(cid_)(p, x[0], x[1], x[2]);
                if (o->solid[c]) continue;
                o->psi[c] = pv;
                o->rho_r[c] = rr;
                o->rho_b[c] = (REAL)1.0 - rr;
            }
    }
}

/* One reference time step: LBM_3D_SinglePhase_Solver.py:477-481 (single phase),
 * 2phase/lbm_solver_3d_2phase_sparse.py:626-632 (two phase). */
int FN(oracle_step_)(ST(oracle_sp_) *o, int nsteps) {
    for (int it = 0; it < nsteps; ++it) {
        if (o->p.grey) {
            /* Grey_Scale/lbm_solver_3d_Macro_Sukop.py:330-336; its
             * Boundary_condition treats the x faces only (:263-293) and
             * streaming3 (:296-312) is the single-phase macroscopic update */
            FN(collide_sp_)(o);
            FN(grey_stream0_)(o);
            FN(grey_stream1_)(o);
            FN(bc_face_)(o, 0);
            FN(bc_face_)(o, 1);
            FN(macros_sp_)(o);
        } else if (o->p.two_phase) {
            FN(collide_tp_)(o);
            FN(stream_)(o);
            for (int face = 0; face < 6; ++face) FN(bc_face_)(o, face);
            FN(macros_tp_)(o);
            FN(bc_psi_)(o);
        } else {
            FN(collide_sp_)(o);
            FN(stream_)(o);
            for (int face = 0; face < 6; ++face) FN(bc_face_)(o, face);
            FN(macros_sp_)(o);
        }
    }
    return 0;
}

/* Only the streaming sweep (collision replaced by identity, no BC): used by the
 * bit-exact permutation test. */
int FN(oracle_stream_only_)(ST(oracle_sp_) *o) {
    FN(stream_)(o);
    return 0;
}

/* Copy state out (dense, x-fastest cell order; v/f as [cell][3] / [cell][19]). */
int FN(oracle_get_)(ST(oracle_sp_) *o, int what, double *out) {
    int64_t n = o->ncell;
    switch (what) {
    case 0: for (int64_t c = 0; c < n; ++c) out[c] = (double)o->rho[c]; break;
    case 1: for (int64_t c = 0; c < n * 3; ++c) out[c] = (double)o->v[c]; break;
    case 2: for (int64_t c = 0; c < n * 19; ++c) out[c] = (double)o->f[c]; break;
    case 3: for (int64_t c = 0; c < n * 19; ++c) out[c] = (double)o->F[c]; break;
    case 4: if (!o->psi) return -1; for (int64_t c = 0; c < n; ++c) out[c] = (double)o->psi[c]; break;
    case 5: if (!o->rho_r) return -1; for (int64_t c = 0; c < n; ++c) out[c] = (double)o->rho_r[c]; break;
    case 6: if (!o->rho_b) return -1; for (int64_t c = 0; c < n; ++c) out[c] = (double)o->rho_b[c]; break;
    case 7: for (int r = 0; r < 19; ++r) for (int c = 0; c < 19; ++c) out[r * 19 + c] = (double)o->Minv[r][c]; break;
    case 8: if (!o->ns) return -1; for (int64_t c = 0; c < n; ++c) out[c] = (double)o->ns[c]; break;
    default: return -1;
    }
    return 0;
}

int FN(oracle_set_)(ST(oracle_sp_) *o, int what, const double *in) {
    int64_t n = o->ncell;
    switch (what) {
    case 2: for (int64_t c = 0; c < n * 19; ++c) o->f[c] = (REAL)in[c]; break;
    case 3: for (int64_t c = 0; c < n * 19; ++c) o->F[c] = (REAL)in[c]; break;
    case 8: if (!o->ns) return -1; for (int64_t c = 0; c < n; ++c) o->ns[c] = (REAL)in[c]; break;
    default: return -1;
    }
    return 0;
}

#undef FN
#undef ST
