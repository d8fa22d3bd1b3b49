/*
 * gbns_oracle.c — CPU restatement of the reference's explicit RHS path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA library is checked
 * against; it is imported only by tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg, never by the product path.
 *
 * It restates, in plain C and in the reference's own operation order, the
 * arithmetic of:
 *   pde-algs/flux-div/flux_div_basic.h:17-76    (cell loop, 6 face evaluations per cell)
 *   omni/infos/info_value.h:19-40               (face value = average of the two cells)
 *   omni/infos/info_gradient.h:21-86            (face gradient, 10-cell stencil)
 *   core/coord_system.h:206-302                 (normals and Jacobian)
 *   navier-stokes/convective.h:54-94, 96-192, 194-246, 335-497
 *                                                (totani_lr, cent_keep, pressure_diss_lr, fweno_t)
 *   navier-stokes/viscous.h:39-112, viscous_laws.h:62-135
 *   omni/compose.h:19-24                        (composite sum conv + (diss + visc))
 *   grid/get_transaction.h:11-97, grid/exchange_config.h:321-350
 *                                                (single-level block exchange, periodic filter)
 *   grid/boundary_fill.h:106-129                (mirror ghost fill)
 *   time-integration/advance.h:56-102, 234-280  (transform_advance_to, SSPRK3 driver)
 *   navier-stokes/fluid_state.h:151-184         (prim <-> cons)
 * Parity of the identity-coordinate, constant/power-law, cent_keep / totani /
 * fweno / pressure_diss paths is pinned against the reference itself
 * (oracle/ref_harness.cc, tests/golden/).  Features with no reference
 * implementation (WENO5, Sutherland, stretched-grid metrics) follow the
 * same structure and are "parity unpinned".
 *
 * Built with -ffp-contract=off so that every operation rounds as written.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include "gbns.h"

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* geometry                                                            */
/* ------------------------------------------------------------------ */

typedef struct
{
    int nb[3], n[3], ng, ni, nj, nk, nblk;
    size_t cells_per_block;           /* ni*nj*nk */
    int coords;
    double bounds[6];
    double cp[4];
    const double* boxes;    /* refined layouts: per block min/max per direction (6 doubles), else NULL */
} geom_t;

static int geom_init(const gbns_grid_desc* g, geom_t* G)
{
    for (int d = 0; d < 3; ++d)
    {
        if (g->nblk[d] < 1 || g->ncell[d] < 1) return -1;
        G->nb[d] = g->nblk[d];
        G->n[d] = g->ncell[d];
    }
    if (g->ng < 1) return -1;
    G->ng = g->ng;
    G->ni = G->n[0] + 2*G->ng;
    G->nj = G->n[1] + 2*G->ng;
    G->nk = G->n[2] + 2*G->ng;
    G->nblk = G->nb[0]*G->nb[1]*G->nb[2];
    G->cells_per_block = (size_t)G->ni*G->nj*G->nk;
    G->coords = g->coords;
    for (int i = 0; i < 6; ++i) G->bounds[i] = g->bounds[i];
    for (int i = 0; i < 4; ++i) G->cp[i] = g->coord_param[i];
    G->boxes = NULL;
    return 0;
}

static inline size_t cell_off(const geom_t* G, int lb, int i, int j, int k)
{
    return 5*((size_t)(i+G->ng) + (size_t)G->ni*((size_t)(j+G->ng) + (size_t)G->nj*((size_t)(k+G->ng) + (size_t)G->nk*lb)));
}

static inline void block_pos(const geom_t* G, int lb, int b[3])
{
    b[0] = lb % G->nb[0];
    b[1] = (lb / G->nb[0]) % G->nb[1];
    b[2] = lb / (G->nb[0]*G->nb[1]);
}

/* cartesian_blocks.h:49,69-70 and cartesian_grid.h:130-136 / grid_geometry.h:85-89;
 * a refined layout's block takes its own bounding box (grid_geometry.h:85-89:
 * dx = box size / cells) */
static void block_box(const geom_t* G, int lb, double bmin[3], double dx[3])
{
    if (G->boxes)
    {
        for (int d = 0; d < 3; ++d)
        {
            const double mn = G->boxes[6*lb + 2*d], mx = G->boxes[6*lb + 2*d + 1];
            bmin[d] = mn;
            dx[d] = (mx - mn) / G->n[d];
        }
        return;
    }
    int b[3];
    block_pos(G, lb, b);
    for (int d = 0; d < 3; ++d)
    {
        const double bsize = (G->bounds[2*d+1] - G->bounds[2*d]) / G->nb[d];
        const double mn = G->bounds[2*d] + b[d]*bsize;
        const double mx = mn + bsize;
        bmin[d] = mn;
        dx[d] = (mx - mn) / G->n[d];
    }
}

/* dy/deta of the y map at computational coordinate eta. */
static double y_deriv(const geom_t* G, double eta)
{
    if (G->coords == GBNS_COORDS_TANH_Y)
    {
        const double beta = G->cp[0];
        const double y0 = G->bounds[2], y1 = G->bounds[3];
        const double s = (2.0*eta - (y0 + y1)) / (y1 - y0);
        const double th = tanh(beta*s);
        return beta*(1.0 - th*th)/tanh(beta);
    }
    if (G->coords == GBNS_COORDS_INTEGRATED_TANH_Y)
    {
        /* coords::integrated_tanh_1D (core/coord_system.h:103-140) */
        const double eta1 = G->cp[0], eta0 = G->cp[1];
        const double deta = eta1 - eta0;
        const double k = G->cp[3], strch = G->cp[2];
        const double alpha0 = k/deta, alpha1 = -k/deta;
        const double beta0 = alpha0*(strch*deta - eta0);
        const double beta1 = alpha0*(eta1 + strch*deta);
#define GBNS_ITANH_F(e) (log(fabs(cosh(alpha0*(e)+beta0)))/alpha0 + log(fabs(cosh(alpha1*(e)+beta1)))/alpha1 - (e))
        const double f0 = GBNS_ITANH_F(eta0);
        const double normInv = 1.0/(GBNS_ITANH_F(eta1) - f0);
#undef GBNS_ITANH_F
        return (deta*(tanh(alpha0*eta + beta0) + tanh(alpha1*eta + beta1) - 1.0))*normInv;
    }
    return 1.0;
}

/* ------------------------------------------------------------------ */
/* scheme evaluation                                                   */
/* ------------------------------------------------------------------ */

typedef struct { double v[5]; } st5;   /* prim (p,T,u,v,w) or flux (c,e,mx,my,mz) */

typedef struct
{
    const geom_t* G;
    const gbns_scheme_desc* S;
    const double* q;      /* AoS5 prims */
    double inv_dx[3];     /* per-block, from the stored geometry (grid_geometry.h:91-99) */
    double bmin[3], dx[3];
    int lb;
} ctx_t;

static inline const double* cellp(const ctx_t* C, int i, int j, int k)
{
    return C->q + cell_off(C->G, C->lb, i, j, k);
}

/* centered_finite_diff_t<idx, order>::value (core/finite_diff.h:25-34) */
static double cfd_coeff(int idx, int order)
{
    const int h = order/2;
    double fh = 1, fhp = 1, fhm = 1;
    for (int i = 2; i <= h; ++i) fh *= i;
    for (int i = 2; i <= h+idx; ++i) fhp *= i;
    for (int i = 2; i <= h-idx; ++i) fhm *= i;
    const double d0 = fh/fhp;
    const double d1 = fh/fhm;
    const double sgn = ((1+idx) % 2 == 0) ? 1.0 : -1.0;
    return d0*d1*sgn/(double)idx;
}

/* Normal of a face (direction d) in the y-row of computational coordinate
 * eta: identity -> unit vector; diagonal y map -> n_d = prod_{k != d} m_k. */
static void face_normal(const ctx_t* C, int d, double eta, double n[3])
{
    n[0] = n[1] = n[2] = 0.0;
    if (C->G->coords == GBNS_COORDS_IDENTITY) { n[d] = 1.0; return; }
    n[d] = (d == 1) ? 1.0 : y_deriv(C->G, eta);
}

/* cent_keep_scheme_t<gas, order>::operator() (convective.h:117-184).
 * cells[m], m = 0..order-1, at face offsets -(order-1), ..., order-1. */
static st5 flux_cent_keep(const ctx_t* C, const double* cells[8], int order, const double ncell[8][3], const double nface[3])
{
    const double gam = C->S->gas.gamma, R = C->S->gas.R;
    const int hw = order/2;
    double un[8], rho[8], eng[8];
    for (int m = 0; m < order; ++m)
    {
        const double* q = cells[m];
        un[m]  = q[2]*ncell[m][0] + q[3]*ncell[m][1] + q[4]*ncell[m][2];
        rho[m] = q[0]/(R*q[1]);
        eng[m] = q[0]/(rho[m]*(gam - 1.0));
    }
    double c = 0, mx = 0, my = 0, mz = 0, g = 0, k = 0, ie = 0, pp = 0;
    for (int ii = 1; ii < hw+1; ++ii)
    {
        const double a = cfd_coeff(ii, order);
        for (int jj = 0; jj < ii; ++jj)
        {
            const int i0 = hw - 1 - jj, i1 = i0 + ii;
            const double* q0 = cells[i0];
            const double* q1 = cells[i1];
            const double c_loc = a*(0.25*(rho[i0] + rho[i1])*(un[i1] + un[i0]));
            c  += c_loc;
            mx += c_loc*(0.5*(q0[2] + q1[2]));
            my += c_loc*(0.5*(q0[3] + q1[3]));
            mz += c_loc*(0.5*(q0[4] + q1[4]));
            g  += a*(0.5*(q0[0] + q1[0]));
            k  += 0.5*c_loc*(q0[2]*q1[2] + q0[3]*q1[3] + q0[4]*q1[4]);
            ie += c_loc*(0.5*(eng[i0] + eng[i1]));
            pp += a*(0.5*(un[i0]*q1[0] + un[i1]*q0[0]));
        }
    }
    st5 F;
    F.v[0] = 2.0*c;
    F.v[1] = 2.0*(k + ie + pp);
    F.v[2] = 2.0*(mx + g*nface[0]);
    F.v[3] = 2.0*(my + g*nface[1]);
    F.v[4] = 2.0*(mz + g*nface[2]);
    return F;
}

/* totani_lr::operator() (convective.h:68-93) */
static st5 flux_totani(const ctx_t* C, const double* ql, const double* qr, const double nl[3], const double nr[3])
{
    const double gam = C->S->gas.gamma, R = C->S->gas.R;
    const double un_l = nl[0]*ql[2] + nl[1]*ql[3] + nl[2]*ql[4];
    const double un_r = nr[0]*qr[2] + nr[1]*qr[3] + nr[2]*qr[4];
    const double rho_l = ql[0]/(R*ql[1]);
    const double rho_r = qr[0]/(R*qr[1]);
    const double e_l = ql[0]/(rho_l*(gam - 1.0));
    const double e_r = qr[0]/(rho_r*(gam - 1.0));
    const double c = 0.25*(rho_l + rho_r)*(un_l + un_r);
    st5 F;
    F.v[0] = c;
    F.v[1] = 0.5*c*(e_l + e_r + ql[2]*qr[2] + ql[3]*qr[3] + ql[4]*qr[4]) + 0.5*(un_l*qr[0] + un_r*ql[0]);
    F.v[2] = 0.5*c*(ql[2] + qr[2]) + 0.5*(nl[0]*ql[0] + nr[0]*qr[0]);
    F.v[3] = 0.5*c*(ql[3] + qr[3]) + 0.5*(nl[1]*ql[0] + nr[1]*qr[0]);
    F.v[4] = 0.5*c*(ql[4] + qr[4]) + 0.5*(nl[2]*ql[0] + nr[2]*qr[0]);
    return F;
}

static void face_grad(const ctx_t* C, int d, int i, int j, int k, double grad[3][5]);

/* state_sensor::ducros_t::get_sensor (navier-stokes/state_sensor.h:21-43)
 * on the face gradient. */
static double ducros_sensor(const double grad[3][5], double epsilon)
{
    double theta_sq = grad[0][2] + grad[1][3] + grad[2][4];
    theta_sq *= theta_sq;
    const double vort0 = grad[1][4] - grad[2][3];
    const double vort1 = grad[2][2] - grad[0][4];
    const double vort2 = grad[0][3] - grad[1][2];
    const double vort_sq = vort0*vort0 + vort1*vort1 + vort2*vort2;
    return theta_sq / (theta_sq + vort_sq + epsilon);
}

/* pressure_diss_lr<gas, sensor>::operator() (convective.h:212-245) with
 * const_sensor_t (sensor_alpha) or ducros_t (epsilon = sensor_alpha). */
static st5 flux_pdiss(const ctx_t* C, int d, int ci, int cj, int ck, const double* ql, const double* qr)
{
    const double gam = C->S->gas.gamma, R = C->S->gas.R;
    const double eps_p = C->S->eps_p, eps_T = C->S->eps_T;
    double scl = C->S->sensor_alpha;
    if (C->S->sensor == GBNS_SENSOR_DUCROS)
    {
        double grad[3][5];
        face_grad(C, d, ci, cj, ck, grad);
        scl = ducros_sensor(grad, C->S->sensor_alpha);
    }
    const double delta_p = ql[0] - qr[0];
    const double delta_T = ql[1] - qr[1];
    const double pavg = 0.5*(ql[0] + qr[0]);
    const double Tavg = 0.5*(ql[1] + qr[1]);
    const double inv_RT = 1.0/(0.5*(R + R)*Tavg);
    const double p_inv_rt2 = pavg*inv_RT/Tavg;
    const double gamma = 0.5*(gam + gam);
    const double k = 0.5*(ql[2]*qr[2] + ql[3]*qr[3] + ql[4]*qr[4]);
    const double u = 0.5*(ql[2] + qr[2]);
    const double v = 0.5*(ql[3] + qr[3]);
    const double w = 0.5*(ql[4] + qr[4]);
    st5 F;
    F.v[0] = scl*eps_p*delta_p*inv_RT;
    F.v[1] = scl*eps_p*delta_p*(k*inv_RT + 1.0/gamma);
    F.v[2] = scl*eps_p*delta_p*u*inv_RT;
    F.v[3] = scl*eps_p*delta_p*v*inv_RT;
    F.v[4] = scl*eps_p*delta_p*w*inv_RT;
    F.v[0] -= scl*eps_T*delta_T*p_inv_rt2;
    F.v[1] -= scl*eps_T*delta_T*p_inv_rt2*(0.5*k);
    F.v[2] -= scl*eps_T*delta_T*p_inv_rt2*u;
    F.v[3] -= scl*eps_T*delta_T*p_inv_rt2*v;
    F.v[4] -= scl*eps_T*delta_T*p_inv_rt2*w;
    return F;
}

/* Per-point Rusanov split of fweno_t (convective.h:360-376, 442-493):
 * fluxv/dissv for the 5 equations at one stencil point. */
static void fweno_point(const ctx_t* C, const double* q, const double n[3], double fl[5], double ds[5])
{
    const double gam = C->S->gas.gamma, rgas = C->S->gas.R;
    double rho = rgas*q[1];
    double hsr = q[2]*q[2];
    hsr += q[3]*q[3];
    hsr += q[4]*q[4];
    hsr = sqrt(hsr);
    hsr += sqrt(rho*gam);
    rho = q[0]/rho;
    hsr *= rho;
    hsr *= 0.5;
    /* mass */
    double f = q[2]*n[0];
    f += q[3]*n[1];
    f += q[4]*n[2];
    f *= 0.5*rho;
    fl[0] = f;
    ds[0] = hsr;
    /* energy: flx keeps the mass value (mutv passes it by reference) */
    double engy = q[2]*q[2];
    engy += q[3]*q[3];
    engy += q[4]*q[4];
    engy *= 0.5;
    const double pdiff = rgas*q[1];
    engy += pdiff/(gam - 1.0);
    fl[1] = fl[0]*(engy + pdiff);
    ds[1] = ds[0]*engy;
    /* momentum */
    for (int dr = 0; dr < 3; ++dr)
    {
        double m = q[2]*n[0];
        m += q[3]*n[1];
        m += q[4]*n[2];
        m *= rho;
        m *= q[2+dr];
        m += q[0]*n[dr];
        m *= 0.5;
        fl[2+dr] = m;
        double dm = hsr;
        dm *= q[2+dr];
        ds[2+dr] = dm;
    }
}

/* apply_weno of fweno_t (convective.h:378-427) */
static double fweno_apply(const double fl[4], const double ds[4], int smooth)
{
    const double f0uk = fl[0]+ds[0], f0dk = fl[0]-ds[0];
    const double f1uk = fl[1]+ds[1], f1dk = fl[1]-ds[1];
    const double f2uk = fl[2]+ds[2], f2dk = fl[2]-ds[2];
    const double f3uk = fl[3]+ds[3], f3dk = fl[3]-ds[3];
    const double r0 = -0.5*(f0uk) + 1.5*(f1uk);
    const double r1 =  0.5*(f1uk) + 0.5*(f2uk);
    const double r2 =  0.5*(f1dk) + 0.5*(f2dk);
    const double r3 =  1.5*(f2dk) - 0.5*(f3dk);
    if (!smooth)
        return (1.0/3.0)*r0 + (2.0/3.0)*r1 + (2.0/3.0)*r2 + (1.0/3.0)*r3;
    const double eps = 1e-16;
    double as[4] = {(f0uk)-(f1uk), (f1uk)-(f2uk), (f1dk)-(f2dk), (f2dk)-(f3dk)};
    for (int i = 0; i < 4; ++i)
    {
        as[i] *= as[i];
        as[i] += eps;
        as[i] *= as[i];
    }
    as[0] += as[0];
    as[0] += as[1];
    as[0] = as[1]/as[0];
    as[3] += as[3];
    as[3] += as[2];
    as[3] = as[2]/as[3];
    as[1] = 1.0 - as[0];
    as[2] = 1.0 - as[3];
    return as[0]*r0 + as[1]*r1 + as[2]*r2 + as[3]*r3;
}

static st5 flux_fweno(const ctx_t* C, const double* cells[4], const double ncell[4][3])
{
    double fl[4][5], ds[4][5];
    for (int m = 0; m < 4; ++m) fweno_point(C, cells[m], ncell[m], fl[m], ds[m]);
    st5 F;
    for (int v = 0; v < 5; ++v)
    {
        const double a[4] = {fl[0][v], fl[1][v], fl[2][v], fl[3][v]};
        const double b[4] = {ds[0][v], ds[1][v], ds[2][v], ds[3][v]};
        F.v[v] = fweno_apply(a, b, C->S->weno_smooth);
    }
    return F;
}

/* 5th-order WENO-JS (Jiang & Shu 1996) on the same per-point Rusanov split
 * as fweno_t: cells[m], m = 0..5, at face offsets -5,-3,-1,1,3,5; the
 * upwind part reconstructs f+ = fl+ds from cells 0..4, the downwind part
 * f- = fl-ds from cells 5..1 (mirrored).  No reference counterpart: parity
 * unpinned. */
/* The WENO5 face flux as the FP64 kernels define it: per side (values a..e
 * upwind to downwind) q_k = 6 p_k, B_k = 4 beta_k, E_k = (B_k + 4 eps)^2,
 * a_k = g_k prod_{j!=k} E_j, N = sum a_k q_k, D = sum a_k, and both sides
 * share one division F = (N_u D_d + N_d D_u)/(6 D_u D_d) while that
 * denominator stays below 1e300 (else each side is divided separately). */
typedef struct { double N, D; } weno5_nd_t;

static weno5_nd_t weno5_nd(double a, double b, double c, double d, double e)
{
    const double q0 = fma(2.0, a, fma(-7.0, b, 11.0*c));
    const double q1 = fma(5.0, c, fma(2.0, d, -b));
    const double q2 = fma(2.0, c, fma(5.0, d, -e));
    const double t0 = fma(-2.0, b, a) + c, s0 = fma(3.0, c, fma(-4.0, b, a));
    const double t1 = fma(-2.0, c, b) + d, s1 = b - d;
    const double t2 = fma(-2.0, d, c) + e, s2 = fma(3.0, c, fma(-4.0, d, e));
    const double k = 13.0/3.0, eps4 = 4e-16;
    const double e0 = fma(k*t0, t0, s0*s0) + eps4;
    const double e1 = fma(k*t1, t1, s1*s1) + eps4;
    const double e2 = fma(k*t2, t2, s2*s2) + eps4;
    const double E0 = e0*e0, E1 = e1*e1, E2 = e2*e2;
    const double a0 = 0.1*(E1*E2), a1 = 0.6*(E0*E2), a2 = 0.3*(E0*E1);
    weno5_nd_t r;
    r.N = fma(a0, q0, fma(a1, q1, a2*q2));
    r.D = (a0 + a1) + a2;
    return r;
}

static double weno5_pair(const double up[6], const double dn[6], int smooth)
{
    const double ua = up[0], ub = up[1], uc = up[2], ud = up[3], ue = up[4];
    const double da = dn[5], db = dn[4], dc = dn[3], dd = dn[2], de = dn[1];
    if (!smooth)
    {
        const double pu = fma(0.1, fma(2.0, ua, fma(-7.0, ub, 11.0*uc)),
                              fma(0.6, fma(5.0, uc, fma(2.0, ud, -ub)), 0.3*fma(2.0, uc, fma(5.0, ud, -ue))));
        const double pd = fma(0.1, fma(2.0, da, fma(-7.0, db, 11.0*dc)),
                              fma(0.6, fma(5.0, dc, fma(2.0, dd, -db)), 0.3*fma(2.0, dc, fma(5.0, dd, -de))));
        return (pu + pd)*(1.0/6.0);
    }
    const weno5_nd_t u = weno5_nd(ua, ub, uc, ud, ue);
    const weno5_nd_t d = weno5_nd(da, db, dc, dd, de);
    const double den = 6.0*(u.D*d.D);
    if (den < 1.0e300) return fma(u.N, d.D, d.N*u.D)/den;
    return u.N/(6.0*u.D) + d.N/(6.0*d.D);
}

static st5 flux_weno5(const ctx_t* C, const double* cells[6], const double ncell[6][3])
{
    double fl[6][5], ds[6][5];
    for (int m = 0; m < 6; ++m) fweno_point(C, cells[m], ncell[m], fl[m], ds[m]);
    st5 F;
    const int sm = C->S->weno_smooth;
    for (int v = 0; v < 5; ++v)
    {
        double up[6], dn[6];
        for (int m = 0; m < 6; ++m) { up[m] = fl[m][v] + ds[m][v]; dn[m] = fl[m][v] - ds[m][v]; }
        F.v[v] = weno5_pair(up, dn, sm);
    }
    return F;
}

/* viscous law: mu, beta, alpha at the face state (viscous_laws.h:62-135) */
static void visc_law(const gbns_scheme_desc* S, double T, double* mu, double* beta, double* alpha)
{
    if (S->visc_law == GBNS_LAW_POWER)
    {
        const double m = S->mu*pow(T/S->T_ref, S->power);
        *mu = m;
        *beta = -0.66666666667*m;
        *alpha = m/S->prandtl;
        return;
    }
    if (S->visc_law == GBNS_LAW_SUTHERLAND)
    {
        /* mu_ref (T/T_ref)^1.5 (T_ref + S)/(T + S); beta = -2/3 mu as a
         * product with the rounded constant (no reference counterpart) */
        const double x = T/S->T_ref;
        const double m = S->mu*(x*sqrt(x))*((S->T_ref + S->S)/(T + S->S));
        *mu = m;
        *beta = m*(-2.0/3.0);
        *alpha = m*(S->prandtl_inv > 0.0 ? S->prandtl_inv : 1.0/S->prandtl);
        return;
    }
    *mu = S->mu;
    *beta = -2.0*S->mu/3.0;
    *alpha = S->mu*(S->prandtl_inv > 0.0 ? S->prandtl_inv : 1.0/S->prandtl);
}

/* info::gradient at the face in direction d whose right cell is (i,j,k)
 * (info_gradient.h:61-123); grad[a][v] for every primitive v. */
static void face_grad(const ctx_t* C, int d, int i, int j, int k, double grad[3][5])
{
    const int idir[3] = {d, (d+1)%3, (d+2)%3};
    int ic[3] = {i, j, k};
    ic[d] -= 1;                       /* left cell */
    for (int a = 0; a < 3; ++a) for (int v = 0; v < 5; ++v) grad[a][v] = 0.0;
    const double* inv = C->inv_dx;
#define GBNS_APPLY(iset, coeff) do { const double* qq = cellp(C, ic[0], ic[1], ic[2]); \
        for (int v = 0; v < 5; ++v) grad[iset][v] += (coeff)*qq[v]*inv[iset]; } while (0)
    GBNS_APPLY(idir[0], -1.0);
    for (int ii = 1; ii < 3; ++ii)
    {
        ic[idir[ii]] += 1;  GBNS_APPLY(idir[ii],  0.25);
        ic[idir[ii]] -= 2;  GBNS_APPLY(idir[ii], -0.25);
        ic[idir[ii]] += 1;
    }
    ic[idir[0]] += 1;
    GBNS_APPLY(idir[0], 1.0);
    for (int ii = 1; ii < 3; ++ii)
    {
        ic[idir[ii]] += 1;  GBNS_APPLY(idir[ii],  0.25);
        ic[idir[ii]] -= 2;  GBNS_APPLY(idir[ii], -0.25);
        ic[idir[ii]] += 1;
    }
#undef GBNS_APPLY
    if (C->G->coords != GBNS_COORDS_IDENTITY)
    {
        /* physical y-derivative = (1/m_y) d/deta at the face */
        const double eta = (d == 1) ? C->bmin[1] + (double)j*C->dx[1]
                                    : C->bmin[1] + ((double)j + 0.5)*C->dx[1];
        const double im = 1.0/y_deriv(C->G, eta);
        for (int v = 0; v < 5; ++v) grad[1][v] *= im;
    }
}

/* visc_lr::operator() (viscous.h:39-79) with the face value of
 * info_value.h:28-40 and the face gradient above. */
static st5 flux_visc(const ctx_t* C, int d, int i, int j, int k, const double n[3])
{
    double grad[3][5];
    face_grad(C, d, i, j, k, grad);
    const double* qL = cellp(C, i - (d==0), j - (d==1), k - (d==2));
    const double* qR = cellp(C, i, j, k);
    double qf[5];
    for (int v = 0; v < 5; ++v) { qf[v] = qL[v]; qf[v] += qR[v]; qf[v] *= 0.5; }

    double visc, visc2, dfs;
    visc_law(C->S, qf[1], &visc, &visc2, &dfs);
    /* gradient components: grad[a][2..4] = du,dv,dw ; grad[a][1] = dT */
    const double div = grad[0][2] + grad[1][3] + grad[2][4];
    double tau[3][3];
    tau[0][0] = visc*(grad[0][2] + grad[0][2]) + visc2*div;
    tau[0][1] = visc*(grad[0][3] + grad[1][2]);
    tau[0][2] = visc*(grad[0][4] + grad[2][2]);
    tau[1][2] = visc*(grad[1][4] + grad[2][3]);
    tau[1][1] = visc*(grad[1][3] + grad[1][3]) + visc2*div;
    tau[1][0] = tau[0][1];
    tau[2][0] = tau[0][2];
    tau[2][1] = tau[1][2];
    tau[2][2] = visc*(grad[2][4] + grad[2][4]) + visc2*div;
    const double gam = C->S->gas.gamma, rgas = C->S->gas.R;
    const double spec_heat = gam*rgas/(gam - 1.0);
    const double cond = spec_heat*dfs;
    double ht[3];
    ht[0] = qf[2]*tau[0][0] + qf[3]*tau[0][1] + qf[4]*tau[0][2] + cond*grad[0][1];
    ht[1] = qf[2]*tau[1][0] + qf[3]*tau[1][1] + qf[4]*tau[1][2] + cond*grad[1][1];
    ht[2] = qf[2]*tau[2][0] + qf[3]*tau[2][1] + qf[4]*tau[2][2] + cond*grad[2][1];
    st5 F;
    F.v[0] = 0.0;
    F.v[1] = -(n[0]*ht[0] + n[1]*ht[1] + n[2]*ht[2]);
    F.v[2] = -(n[0]*tau[0][0] + n[1]*tau[0][1] + n[2]*tau[0][2]);
    F.v[3] = -(n[0]*tau[1][0] + n[1]*tau[1][1] + n[2]*tau[1][2]);
    F.v[4] = -(n[0]*tau[2][0] + n[1]*tau[2][1] + n[2]*tau[2][2]);
    return F;
}

/* Stencil of `width` cells centred on the face (direction d, right cell
 * (i,j,k)) with each cell's metric normal (info_metric.h:188-197). */
static void face_window(const ctx_t* C, int d, int i, int j, int k, int width,
                        const double* cells[8], double ncell[8][3])
{
    const int dd[3] = {d == 0, d == 1, d == 2};
    const int hw = width/2;
    for (int m = 0; m < width; ++m)
    {
        const int off = m - hw;
        const int ci = i + off*dd[0], cj = j + off*dd[1], ck = k + off*dd[2];
        cells[m] = cellp(C, ci, cj, ck);
        const double eta_c = C->bmin[1] + ((double)cj + 0.5)*C->dx[1];
        face_normal(C, d, eta_c, ncell[m]);
    }
}

/* hybrid_scheme_t<cent_keep_scheme_t, fweno_t, blender, tag>::operator()
 * (navier-stokes/hybrid_scheme.h:30-46): s = blender at the face
 * (const_sensor_t alpha, or ducros_t on the face gradient); F = c0 F_centred
 * + s F_fweno with c0 = 1 - s (full_flux) or 1 (diss_flux). */
static st5 flux_hybrid(const ctx_t* C, int d, int i, int j, int k, const double nface[3])
{
    const gbns_scheme_desc* S = C->S;
    double blend = S->hybrid_param;
    if (S->hybrid_sensor == GBNS_SENSOR_DUCROS)
    {
        double grad[3][5];
        face_grad(C, d, i, j, k, grad);
        blend = ducros_sensor(grad, S->hybrid_param);
    }
    const double* cells[8];
    double ncell[8][3];
    face_window(C, d, i, j, k, S->order, cells, ncell);
    st5 f0 = flux_cent_keep(C, cells, S->order, (const double (*)[3])ncell, nface);
    face_window(C, d, i, j, k, 4, cells, ncell);
    st5 f1 = flux_fweno(C, cells, (const double (*)[3])ncell);
    const double coeff0 = (S->hybrid_flux == GBNS_HYBRID_DISS_FLUX) ? 1.0 : (1.0 - blend);
    for (int v = 0; v < 5; ++v)
    {
        f0.v[v] *= coeff0;
        f1.v[v] *= blend;
        f0.v[v] += f1.v[v];
    }
    return f0;
}

/* Face flux of the lowered composite for the face in direction d whose
 * right cell is (i,j,k): conv + (diss + visc) (compose.h:19-24). */
static st5 face_flux(const ctx_t* C, int d, int i, int j, int k)
{
    const gbns_scheme_desc* S = C->S;
    const int dd[3] = {d == 0, d == 1, d == 2};
    /* face eta (y computational coordinate) for the metric */
    const double eta_face = (d == 1) ? C->bmin[1] + (double)j*C->dx[1]
                                     : C->bmin[1] + ((double)j + 0.5)*C->dx[1];
    double nface[3];
    face_normal(C, d, eta_face, nface);

    st5 terms[3];
    int nterm = 0;
    if (S->convective == GBNS_CONV_HYBRID)
    {
        terms[nterm++] = flux_hybrid(C, d, i, j, k, nface);
    }
    else if (S->convective != GBNS_CONV_NONE)
    {
        st5 F;
        int width = 2;
        if (S->convective == GBNS_CONV_CENT_KEEP) width = S->order;
        if (S->convective == GBNS_CONV_FWENO) width = 4;
        if (S->convective == GBNS_CONV_WENO5) width = 6;
        const double* cells[8];
        double ncell[8][3];
        const int hw = width/2;
        for (int m = 0; m < width; ++m)
        {
            const int off = m - hw;   /* cell offset relative to the right cell */
            const int ci = i + off*dd[0], cj = j + off*dd[1], ck = k + off*dd[2];
            cells[m] = cellp(C, ci, cj, ck);
            /* per-cell metric along d (info_metric.h:188-197) */
            const double eta_c = C->bmin[1] + ((double)cj + 0.5)*C->dx[1];
            face_normal(C, d, eta_c, ncell[m]);
        }
        switch (S->convective)
        {
            case GBNS_CONV_CENT_KEEP: F = flux_cent_keep(C, cells, S->order, (const double (*)[3])ncell, nface); break;
            case GBNS_CONV_TOTANI:    F = flux_totani(C, cells[0], cells[1], ncell[0], ncell[1]); break;
            case GBNS_CONV_FWENO:     F = flux_fweno(C, cells, (const double (*)[3])ncell); break;
            default:                  F = flux_weno5(C, cells, (const double (*)[3])ncell); break;
        }
        terms[nterm++] = F;
    }
    if (S->dissipation == GBNS_DISS_PRESSURE)
    {
        terms[nterm++] = flux_pdiss(C, d, i, j, k, cellp(C, i - dd[0], j - dd[1], k - dd[2]), cellp(C, i, j, k));
    }
    if (S->viscous == GBNS_VISC_LR)
    {
        terms[nterm++] = flux_visc(C, d, i, j, k, nface);
    }
    st5 out;
    if (nterm == 0) { memset(&out, 0, sizeof(out)); return out; }
    if (nterm == 1) return terms[0];
    if (nterm == 2)
    {
        for (int v = 0; v < 5; ++v) out.v[v] = terms[0].v[v] + terms[1].v[v];
        return out;
    }
    for (int v = 0; v < 5; ++v) out.v[v] = terms[0].v[v] + (terms[1].v[v] + terms[2].v[v]);
    return out;
}

static int stencil_halo(const gbns_scheme_desc* S)
{
    int h = 0;
    if (S->convective == GBNS_CONV_CENT_KEEP) h = S->order/2;
    else if (S->convective == GBNS_CONV_TOTANI) h = 1;
    else if (S->convective == GBNS_CONV_FWENO) h = 2;
    else if (S->convective == GBNS_CONV_WENO5) h = 3;
    else if (S->convective == GBNS_CONV_HYBRID) h = S->order/2 > 2 ? S->order/2 : 2;
    if (S->dissipation && h < 1) h = 1;
    if (S->viscous && h < 1) h = 1;
    return h;
}

/* ------------------------------------------------------------------ */
/* public oracle entry points                                          */
/* ------------------------------------------------------------------ */

static int flux_div_geom(const geom_t* Gp, const gbns_scheme_desc* S,
                         const double* prims, double* rhs, int increment, int nthreads);

int oracle_flux_div(const gbns_grid_desc* g, const gbns_scheme_desc* S,
                    const double* prims, double* rhs, int increment, int nthreads)
{
    geom_t G;
    if (geom_init(g, &G)) return -1;
    return flux_div_geom(&G, S, prims, rhs, increment, nthreads);
}

/* flux_div on a refined layout: grid->nblk = (blocks, 1, 1), identity
 * coordinates, each block's box from `boxes` (6 doubles per block). */
int oracle_flux_div_blocks(const gbns_grid_desc* g, const gbns_scheme_desc* S, const double* boxes,
                           const double* prims, double* rhs, int increment, int nthreads)
{
    geom_t G;
    if (geom_init(g, &G)) return -1;
    if (G.coords != GBNS_COORDS_IDENTITY || G.nb[1] != 1 || G.nb[2] != 1) return -1;
    G.boxes = boxes;
    return flux_div_geom(&G, S, prims, rhs, increment, nthreads);
}

static int flux_div_geom(const geom_t* Gp, const gbns_scheme_desc* S,
                         const double* prims, double* rhs, int increment, int nthreads)
{
    const geom_t G = *Gp;
    if (stencil_halo(S) > G.ng) return -2;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int lb = 0; lb < G.nblk; ++lb)
    {
        ctx_t C;
        C.G = &G; C.S = S; C.q = prims; C.lb = lb;
        block_box(&G, lb, C.bmin, C.dx);
        for (int d = 0; d < 3; ++d) C.inv_dx[d] = 1.0/C.dx[d];
        for (int k = 0; k < G.n[2]; ++k)
        for (int j = 0; j < G.n[1]; ++j)
        for (int i = 0; i < G.n[0]; ++i)
        {
            double* r = rhs + cell_off(&G, lb, i, j, k);
            double relem[5];
            for (int v = 0; v < 5; ++v) relem[v] = increment ? r[v] : 0.0;
            /* calc_jacobian at the cell's computational coordinates */
            double jac = 1.0;
            if (G.coords != GBNS_COORDS_IDENTITY)
                jac = 1.0/(1.0*y_deriv(&G, C.bmin[1] + ((double)j + 0.5)*C.dx[1])*1.0);
            for (int d = 0; d < 3; ++d)
            {
                const double inv_dx = 1.0/C.dx[d];
                for (int pm = 0; pm < 2; ++pm)
                {
                    const st5 F = face_flux(&C, d, i + (d==0)*pm, j + (d==1)*pm, k + (d==2)*pm);
                    const double mult = jac*(1.0 - 2.0*pm)*inv_dx;
                    for (int v = 0; v < 5; ++v)
                    {
                        double acc = 0.0;
                        acc += F.v[v];
                        acc *= mult;
                        relem[v] += acc;
                    }
                }
            }
            for (int v = 0; v < 5; ++v) r[v] = relem[v];
        }
    }
    return 0;
}

/* pde_algs::boundary_flux (pde-algs/boundary_flux.h:16-105), restated from
 * its loop (the reference's version does not compile against its current grid
 * headers, so this restatement is unpinned): for each block, for dir = 0..5
 * (rdir = dir/2, mdir = dir%2), if the block lies on that domain boundary and
 * apply[dir] is set, every face between cell il and ir = il + e_rdir with
 * il[rdir] = -1 (mdir 0) or n-1 (mdir 1) and the transverse indices in
 * [-1, n) (flux_bounds.min = -1 in every direction, boundary_flux.h:37-58)
 * adds accum = 0 + F (the composite face flux) as
 * rhs(il) -= jac_l*accum/dx, rhs(ir) += jac_r*accum/dx (:76-99), with dx the
 * block's spacing along rdir and jac = 1 (identity coordinates). */
int oracle_boundary_flux(const gbns_grid_desc* g, const gbns_scheme_desc* S, const double* prims, double* rhs,
                         const int* apply)
{
    geom_t G;
    if (geom_init(g, &G)) return -1;
    if (G.coords != GBNS_COORDS_IDENTITY) return -3;
    int halo = stencil_halo(S);
    const int grad = S->viscous || (S->dissipation && S->sensor == GBNS_SENSOR_DUCROS) ||
                     (S->convective == GBNS_CONV_HYBRID && S->hybrid_sensor == GBNS_SENSOR_DUCROS);
    if (grad && halo < 2) halo = 2;
    if (halo > G.ng) return -2;
    for (int lb = 0; lb < G.nblk; ++lb)
    {
        int b[3];
        block_pos(&G, lb, b);
        ctx_t C;
        C.G = &G; C.S = S; C.q = prims; C.lb = lb;
        block_box(&G, lb, C.bmin, C.dx);
        for (int d = 0; d < 3; ++d) C.inv_dx[d] = 1.0/C.dx[d];
        for (int dir = 0; dir < 6; ++dir)
        {
            const int rdir = dir/2, mdir = dir%2;
            const int on_boundary = mdir == 0 ? b[rdir] == 0 : b[rdir] == G.nb[rdir] - 1;
            if (!(on_boundary && apply[dir])) continue;
            int lo[3] = {-1, -1, -1}, hi[3] = {G.n[0], G.n[1], G.n[2]};
            if (mdir == 0) hi[rdir] = 0;
            else lo[rdir] = G.n[rdir] - 1;
            const double dx = C.dx[rdir];
            for (int k = lo[2]; k < hi[2]; ++k)
            for (int j = lo[1]; j < hi[1]; ++j)
            for (int i = lo[0]; i < hi[0]; ++i)
            {
                const int ir[3] = {i + (rdir == 0), j + (rdir == 1), k + (rdir == 2)};
                const st5 F = face_flux(&C, rdir, ir[0], ir[1], ir[2]);
                double* rl = rhs + cell_off(&G, lb, i, j, k);
                double* rr = rhs + cell_off(&G, lb, ir[0], ir[1], ir[2]);
                const double jac_l = 1.0, jac_r = 1.0;
                for (int v = 0; v < 5; ++v)
                {
                    double accum = 0.0;
                    accum += F.v[v];
                    rl[v] -= jac_l*accum/dx;
                    rr[v] += jac_r*accum/dx;
                }
            }
        }
    }
    return 0;
}

/* pde_algs::source_term (pde-algs/source_term.h:19-51) for the lowered
 * point sources of gbns.h: rhs += S(q)/jac per interior cell, S in the
 * operation order of the reference-side lambdas (oracle/ref_harness.cc). */
int oracle_source_term(const gbns_grid_desc* g, const gbns_source_desc* src, const double* prims, double* rhs)
{
    geom_t G;
    if (geom_init(g, &G)) return -1;
    if (src->kind < GBNS_SOURCE_CONST || src->kind > GBNS_SOURCE_BODY_ACCEL) return -2;
    for (int lb = 0; lb < G.nblk; ++lb)
    {
        double bmin[3], dx[3];
        block_box(&G, lb, bmin, dx);
        for (int k = 0; k < G.n[2]; ++k)
        for (int j = 0; j < G.n[1]; ++j)
        for (int i = 0; i < G.n[0]; ++i)
        {
            const double* w = prims + cell_off(&G, lb, i, j, k);
            double* r = rhs + cell_off(&G, lb, i, j, k);
            double s[5];
            if (src->kind == GBNS_SOURCE_CONST)
            {
                for (int v = 0; v < 5; ++v) s[v] = src->c[v];
            }
            else
            {
                const double fu = src->c[2]*w[2] + src->c[3]*w[3] + src->c[4]*w[4];
                if (src->kind == GBNS_SOURCE_BODY_FORCE)
                {
                    s[0] = 0.0; s[1] = fu; s[2] = src->c[2]; s[3] = src->c[3]; s[4] = src->c[4];
                }
                else
                {
                    const double rho = w[0]/(src->gas.R*w[1]);
                    s[0] = 0.0; s[1] = rho*fu; s[2] = rho*src->c[2]; s[3] = rho*src->c[3]; s[4] = rho*src->c[4];
                }
            }
            double jac = 1.0;
            if (G.coords != GBNS_COORDS_IDENTITY)
                jac = 1.0/(1.0*y_deriv(&G, bmin[1] + ((double)j + 0.5)*dx[1])*1.0);
            for (int v = 0; v < 5; ++v) r[v] += s[v]/jac;
        }
    }
    return 0;
}

/* Ghost fill: exchange resolved to the donor's interior, then walls.
 * Value of ghost (i,j,k) of block lb: for directions crossing a wall face
 * the index is mirrored first (boundary_fill.h:113-114) and the wall
 * transform applied to the value found there; remaining out-of-range
 * directions are resolved by the periodic / inter-block exchange
 * (get_transaction.h:55-87; non-periodic domain faces are skipped,
 * exchange_config.h:336-344). */
static int resolve_exchange(const geom_t* G, const gbns_bc_desc* bc, int lb, int c[3], int* lb_out)
{
    int b[3];
    block_pos(G, lb, b);
    for (int d = 0; d < 3; ++d)
    {
        int o = 0;
        if (c[d] < 0) o = -1;
        else if (c[d] >= G->n[d]) o = 1;
        if (o == 0) continue;
        const int at_min = (b[d] == 0), at_max = (b[d] == G->nb[d]-1);
        if ((o < 0 && at_min && bc->kind[2*d] != GBNS_BC_PERIODIC) ||
            (o > 0 && at_max && bc->kind[2*d+1] != GBNS_BC_PERIODIC)) return 0;
        b[d] += o;
        if (b[d] < 0) b[d] += G->nb[d];
        if (b[d] >= G->nb[d]) b[d] -= G->nb[d];
        c[d] -= o*G->n[d];
    }
    *lb_out = b[0] + G->nb[0]*(b[1] + G->nb[1]*b[2]);
    return 1;
}

int oracle_fill_ghosts(const gbns_grid_desc* g, const gbns_bc_desc* bc, double* prims)
{
    geom_t G;
    if (geom_init(g, &G)) return -1;
    for (int d = 0; d < 3; ++d)
    {
        const int pmn = bc->kind[2*d] == GBNS_BC_PERIODIC, pmx = bc->kind[2*d+1] == GBNS_BC_PERIODIC;
        if (pmn != pmx) return -1;
    }
    const size_t total = 5*G.cells_per_block*G.nblk;
    double* src = (double*)malloc(total*sizeof(double));
    if (!src) return -1;
    memcpy(src, prims, total*sizeof(double));
    for (int lb = 0; lb < G.nblk; ++lb)
    {
        int b[3];
        block_pos(&G, lb, b);
        for (int k = -G.ng; k < G.n[2]+G.ng; ++k)
        for (int j = -G.ng; j < G.n[1]+G.ng; ++j)
        for (int i = -G.ng; i < G.n[0]+G.ng; ++i)
        {
            int c[3] = {i, j, k};
            if (i >= 0 && i < G.n[0] && j >= 0 && j < G.n[1] && k >= 0 && k < G.n[2]) continue;
            /* walls: mirror in each direction that crosses a wall face */
            int wall_dir[3] = {-1, -1, -1};
            int nwall = 0;
            for (int d = 0; d < 3; ++d)
            {
                int face = -1;
                if (c[d] < 0 && b[d] == 0) face = 2*d;
                if (c[d] >= G.n[d] && b[d] == G.nb[d]-1) face = 2*d+1;
                if (face < 0) continue;
                const int kind = bc->kind[face];
                if (kind == GBNS_BC_ISOTHERMAL_NOSLIP || kind == GBNS_BC_SLIP_ADIABATIC)
                {
                    c[d] = (face % 2 == 0) ? -1 - c[d] : 2*G.n[d] - (c[d] + 1);
                    wall_dir[nwall++] = face;
                }
            }
            int lbs;
            double val[5];
            if (!resolve_exchange(&G, bc, lb, c, &lbs)) continue;   /* untouched */
            const double* s = src + cell_off(&G, lbs, c[0], c[1], c[2]);
            for (int v = 0; v < 5; ++v) val[v] = s[v];
            /* apply the wall transforms in boundary_fill's face order
             * (xmin..zmax): a later face's fill reads the earlier one's */
            for (int w = 0; w < nwall; ++w)
            {
                const int face = wall_dir[w];
                if (bc->kind[face] == GBNS_BC_ISOTHERMAL_NOSLIP)
                {
                    val[1] = 2.0*bc->t_wall[face] - val[1];
                    val[2] = -val[2]; val[3] = -val[3]; val[4] = -val[4];
                }
                else
                {
                    val[2 + face/2] = -val[2 + face/2];
                }
            }
            double* dst = prims + cell_off(&G, lb, i, j, k);
            for (int v = 0; v < 5; ++v) dst[v] = val[v];
        }
    }
    free(src);
    return 0;
}

/* transform_advance_to (advance.h:75-101): in-place stage update. */
int oracle_rk_stage(const gbns_grid_desc* g, const gbns_gas_desc* gas, double* prims,
                    const double* const* res, const double* coeffs, int nres)
{
    geom_t G;
    if (geom_init(g, &G)) return -1;
    const double gam = gas->gamma, R = gas->R;
    for (int lb = 0; lb < G.nblk; ++lb)
    for (int k = 0; k < G.n[2]; ++k)
    for (int j = 0; j < G.n[1]; ++j)
    for (int i = 0; i < G.n[0]; ++i)
    {
        const size_t off = cell_off(&G, lb, i, j, k);
        double* q = prims + off;
        /* prim -> cons (fluid_state.h:151-165) */
        const double rho = q[0]/(R*q[1]);
        const double rhoU2 = rho*(q[2]*q[2] + q[3]*q[3] + q[4]*q[4]);
        const double rhoE = 0.5*rhoU2 + (q[0]/((gam - 1.0)));
        double c[5] = {rho, rhoE, rho*q[2], rho*q[3], rho*q[4]};
        for (int r = 0; r < nres; ++r)
        {
            const double* rr = res[r] + off;
            for (int v = 0; v < 5; ++v) c[v] += coeffs[r]*rr[v];
        }
        /* cons -> prim (fluid_state.h:167-184) */
        const double rh = c[0];
        const double invrho = 1.0/rh;
        const double u = invrho*c[2], v = invrho*c[3], w = invrho*c[4];
        const double ru2 = rh*(u*u + v*v + w*w);
        const double p = (gam - 1.0)*(c[1] - 0.5*ru2);
        const double T = p/(R*rh);
        q[0] = p; q[1] = T; q[2] = u; q[3] = v; q[4] = w;
    }
    return 0;
}

/* Cell volume weight (physical volume / computational volume) = 1/jac. */
static double cell_weight(const geom_t* G, const double bmin[3], const double dx[3], int j)
{
    if (G->coords == GBNS_COORDS_IDENTITY) return 1.0;
    return y_deriv(G, bmin[1] + ((double)j + 0.5)*dx[1]);
}

int oracle_reduce(const gbns_grid_desc* g, const gbns_gas_desc* gas, const double* prims, int kind, double* out)
{
    geom_t G;
    if (geom_init(g, &G)) return -1;
    const double gam = gas->gamma, R = gas->R;
    double acc[5] = {0, 0, 0, 0, 0};
    double wsum = 0.0;
    double mx = 0.0;
    double bad = 0.0;
    for (int lb = 0; lb < G.nblk; ++lb)
    {
        double bmin[3], dx[3];
        block_box(&G, lb, bmin, dx);
        const double vol = dx[0]*dx[1]*dx[2];
        for (int k = 0; k < G.n[2]; ++k)
        for (int j = 0; j < G.n[1]; ++j)
        for (int i = 0; i < G.n[0]; ++i)
        {
            const double* q = prims + cell_off(&G, lb, i, j, k);
            const double wgt = cell_weight(&G, bmin, dx, j)*vol;
            const double rho = q[0]/(R*q[1]);
            const double uu = q[2]*q[2] + q[3]*q[3] + q[4]*q[4];
            if (kind == GBNS_RED_MAX_WAVESPEED)
            {
                const double a = sqrt(gam*R*q[1]) + sqrt(uu);
                if (a > mx) mx = a;
            }
            else if (kind == GBNS_RED_KINETIC)
            {
                acc[0] += 0.5*rho*uu*wgt;
                wsum += wgt;
            }
            else if (kind == GBNS_RED_CONSERVED)
            {
                acc[0] += rho*wgt;
                acc[1] += (0.5*rho*uu + q[0]/(gam - 1.0))*wgt;
                acc[2] += rho*q[2]*wgt;
                acc[3] += rho*q[3]*wgt;
                acc[4] += rho*q[4]*wgt;
            }
            else
            {
                int ok = 1;
                for (int v = 0; v < 5; ++v) if (!isfinite(q[v])) ok = 0;
                if (!(q[0] > 0.0) || !(q[1] > 0.0)) ok = 0;
                if (!ok) bad += 1.0;
            }
        }
    }
    if (kind == GBNS_RED_MAX_WAVESPEED) out[0] = mx;
    else if (kind == GBNS_RED_KINETIC) out[0] = acc[0]/wsum;
    else if (kind == GBNS_RED_CONSERVED) for (int v = 0; v < 5; ++v) out[v] = acc[v];
    else out[0] = bad;
    return 0;
}

/* integrate_advance with state_transform_t (advance.h:234-280), SSPRK3. */
int oracle_ssprk3_step(const gbns_grid_desc* g, const gbns_scheme_desc* S, const gbns_bc_desc* bc,
                       double* prims, double* work, double dt, int nthreads)
{
    size_t n;
    geom_t G;
    if (geom_init(g, &G)) return -1;
    n = 5*G.cells_per_block*G.nblk;
    double* R0 = work;
    double* R1 = work + n;
    double* R2 = work + 2*n;
    /* ratio_diff_t of consecutive ssprk3_t rows (explicit.h:80-88) */
    const double c1[1] = {(1.0/1.0)*dt};
    const double c2[2] = {(-3.0/4.0)*dt, (1.0/4.0)*dt};
    const double c3[3] = {(-1.0/12.0)*dt, (-1.0/12.0)*dt, (2.0/3.0)*dt};
    const double* r01[3] = {R0, R1, R2};
    int rc = 0;
    memset(R0, 0, n*sizeof(double));
    rc |= oracle_flux_div(g, S, prims, R0, 1, nthreads);
    rc |= oracle_rk_stage(g, &S->gas, prims, r01, c1, 1);
    rc |= oracle_fill_ghosts(g, bc, prims);
    memset(R1, 0, n*sizeof(double));
    rc |= oracle_flux_div(g, S, prims, R1, 1, nthreads);
    rc |= oracle_rk_stage(g, &S->gas, prims, r01, c2, 2);
    rc |= oracle_fill_ghosts(g, bc, prims);
    memset(R2, 0, n*sizeof(double));
    rc |= oracle_flux_div(g, S, prims, R2, 1, nthreads);
    rc |= oracle_rk_stage(g, &S->gas, prims, r01, c3, 3);
    rc |= oracle_fill_ghosts(g, bc, prims);
    return rc;
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}


/* Exchange plan of a refined block layout (the reference's transactions,
 * grid/make_exchange.h:111-410 with grid/get_transaction.h:10-263): records
 * of 18 ints (gbns_patch: kind, source block, dest block, source box min,
 * dest box [min, max), i_coeff, i_incr), injections run first, then
 * interpolations, each in plan order.  An injection copies an equally sized
 * donor box; an interpolation sets each destination cell to
 * (0 + sum of 8 donors in order d = (0,0,0), (1,0,0), (0,1,0), ...) * 0.125,
 * donor index ((i << (c + 1)) >> 1) + d*incr per direction. */
int oracle_exchange_patches(int nx, int ny, int nz, int ng, int nblocks, const int* plan, int nplan, double* prims)
{
    const long long ni = nx + 2*ng, nj = ny + 2*ng, nk = nz + 2*ng;
    const long long bstride = 5*ni*nj*nk;
    (void)nblocks;
    for (int pass = 0; pass < 2; ++pass)
        for (int t = 0; t < nplan; ++t)
        {
            const int* r = plan + 18*(long long)t;
            if (r[0] != pass) continue;
            const int sb = r[1], db = r[2];
            const int* slo = r + 3;
            const int* dlo = r + 6;
            const int* dhi = r + 9;
            const int* c = r + 12;
            const int* inc = r + 15;
            for (int dk = 0; dk < dhi[2] - dlo[2]; ++dk)
            for (int dj = 0; dj < dhi[1] - dlo[1]; ++dj)
            for (int di = 0; di < dhi[0] - dlo[0]; ++di)
            {
                double* dst = prims + db*bstride + (((dlo[2] + dk + ng)*nj + (dlo[1] + dj + ng))*ni + (dlo[0] + di + ng))*5;
                if (pass == 0)
                {
                    const double* src = prims + sb*bstride + (((slo[2] + dk + ng)*nj + (slo[1] + dj + ng))*ni + (slo[0] + di + ng))*5;
                    for (int v = 0; v < 5; ++v) dst[v] = src[v];
                }
                else
                {
                    const int i0 = (di << (c[0] + 1)) >> 1, j0 = (dj << (c[1] + 1)) >> 1, k0 = (dk << (c[2] + 1)) >> 1;
                    double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
                    for (int iv = 0; iv < 8; ++iv)
                    {
                        const int d0 = iv & 1, d1 = (iv >> 1) & 1, d2 = (iv >> 2) & 1;
                        const long long ii = slo[0] + i0 + d0*inc[0], jj = slo[1] + j0 + d1*inc[1], kk = slo[2] + k0 + d2*inc[2];
                        const double* src = prims + sb*bstride + (((kk + ng)*nj + (jj + ng))*ni + (ii + ng))*5;
                        for (int v = 0; v < 5; ++v) acc[v] += src[v];
                    }
                    for (int v = 0; v < 5; ++v) dst[v] = acc[v]*0.125;
                }
            }
        }
    return 0;
}
