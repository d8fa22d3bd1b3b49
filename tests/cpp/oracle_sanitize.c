/* Runs every entry point of the CPU restatement (oracle/gbns_oracle.c) under
 * AddressSanitizer and UndefinedBehaviorSanitizer, compiled into this program
 * (tests/test_oracle_sanitize.py): every scheme family, stretched and
 * identity coordinates, periodic, wall, slip and untouched ghosts, the stage
 * update, SSPRK3, reductions, sources and boundary_flux, on small grids whose
 * sizes are not multiples of anything.  Any out-of-bounds access or undefined
 * operation aborts the run. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "gbns.h"

int oracle_flux_div(const gbns_grid_desc*, const gbns_scheme_desc*, const double*, double*, int, int);
int oracle_boundary_flux(const gbns_grid_desc*, const gbns_scheme_desc*, const double*, double*, const int*);
int oracle_source_term(const gbns_grid_desc*, const gbns_source_desc*, const double*, double*);
int oracle_fill_ghosts(const gbns_grid_desc*, const gbns_bc_desc*, double*);
int oracle_rk_stage(const gbns_grid_desc*, const gbns_gas_desc*, double*, const double* const*, const double*, int);
int oracle_reduce(const gbns_grid_desc*, const gbns_gas_desc*, const double*, int, double*);
int oracle_ssprk3_step(const gbns_grid_desc*, const gbns_scheme_desc*, const gbns_bc_desc*, double*, double*, double, int);

static unsigned long long g_rng = 88172645463325252ull;
static double urand(void)
{
    g_rng ^= g_rng << 13; g_rng ^= g_rng >> 7; g_rng ^= g_rng << 17;
    return (double)(g_rng >> 11) * (1.0/9007199254740992.0);
}

static size_t count_of(const gbns_grid_desc* g)
{
    size_t n = 5;
    for (int d = 0; d < 3; ++d) n *= (size_t)(g->ncell[d] + 2*g->ng);
    return n*(size_t)g->nblk[0]*g->nblk[1]*g->nblk[2];
}

static void fill_state(double* q, size_t n)
{
    for (size_t i = 0; i < n; i += 5)
    {
        q[i] = 86100.0*(1.0 + 0.02*(urand() - 0.5));
        q[i + 1] = 300.0*(1.0 + 0.02*(urand() - 0.5));
        q[i + 2] = 30.0*(urand() - 0.5);
        q[i + 3] = 30.0*(urand() - 0.5);
        q[i + 4] = 30.0*(urand() - 0.5);
    }
}

static gbns_scheme_desc scheme(int conv, int order, int diss, int visc, int law, int sensor)
{
    gbns_scheme_desc s;
    memset(&s, 0, sizeof(s));
    s.convective = conv; s.order = order; s.weno_smooth = 1; s.dissipation = diss; s.sensor = sensor;
    s.viscous = visc; s.visc_law = law; s.precision = GBNS_PREC_FP64;
    s.eps_p = 0.3; s.eps_T = 0.2; s.sensor_alpha = 0.7; s.mu = 2e-2; s.prandtl = 0.72;
    s.T_ref = 300.0; s.power = 0.76; s.S = 110.4;
    s.gas.gamma = 1.4; s.gas.R = 287.0;
    s.hybrid_flux = GBNS_HYBRID_FULL_FLUX; s.hybrid_sensor = GBNS_SENSOR_DUCROS; s.hybrid_param = 1e-3;
    return s;
}

#define CHECK(x) do { int rc_ = (x); if (rc_) { fprintf(stderr, "%s returned %d\n", #x, rc_); return 1; } } while (0)

int main(void)
{
    const int coords[3] = {GBNS_COORDS_IDENTITY, GBNS_COORDS_TANH_Y, GBNS_COORDS_INTEGRATED_TANH_Y};
    const gbns_scheme_desc schemes[] = {
        scheme(GBNS_CONV_CENT_KEEP, 2, 0, 1, GBNS_LAW_CONSTANT, 0),
        scheme(GBNS_CONV_CENT_KEEP, 8, 1, 1, GBNS_LAW_SUTHERLAND, 0),
        scheme(GBNS_CONV_TOTANI, 2, 1, 1, GBNS_LAW_POWER, GBNS_SENSOR_DUCROS),
        scheme(GBNS_CONV_FWENO, 2, 1, 1, GBNS_LAW_CONSTANT, GBNS_SENSOR_DUCROS),
        scheme(GBNS_CONV_WENO5, 2, 1, 1, GBNS_LAW_SUTHERLAND, 0),
        scheme(GBNS_CONV_HYBRID, 4, 1, 1, GBNS_LAW_CONSTANT, 0),
        scheme(GBNS_CONV_NONE, 2, 1, 0, GBNS_LAW_CONSTANT, 0),
    };
    const int nsch = (int)(sizeof(schemes)/sizeof(schemes[0]));
    for (int ci = 0; ci < 3; ++ci)
    for (int si = 0; si < nsch; ++si)
    {
        gbns_grid_desc g;
        memset(&g, 0, sizeof(g));
        g.nblk[0] = 2; g.nblk[1] = 3; g.nblk[2] = 1;
        g.ncell[0] = 5; g.ncell[1] = 4; g.ncell[2] = 3;
        g.ng = 4;
        g.coords = coords[ci];
        g.bounds[0] = 0.0; g.bounds[1] = 2.0; g.bounds[2] = -1.0; g.bounds[3] = 1.0; g.bounds[4] = 0.0; g.bounds[5] = 1.0;
        if (coords[ci] == GBNS_COORDS_TANH_Y) g.coord_param[0] = 2.0;
        if (coords[ci] == GBNS_COORDS_INTEGRATED_TANH_Y)
        { g.coord_param[0] = 1.0; g.coord_param[1] = -1.0; g.coord_param[2] = 0.3; g.coord_param[3] = 2.5; }
        const size_t n = count_of(&g);
        double* q = malloc(n*sizeof(double));
        double* r = malloc(n*sizeof(double));
        double* w = malloc(3*n*sizeof(double));
        fill_state(q, n);
        memset(r, 0, n*sizeof(double));
        gbns_bc_desc bc;
        memset(&bc, 0, sizeof(bc));
        const int kinds[4] = {GBNS_BC_PERIODIC, GBNS_BC_ISOTHERMAL_NOSLIP, GBNS_BC_SLIP_ADIABATIC, GBNS_BC_NONE};
        const int kb = si % 4;
        for (int f = 0; f < 6; ++f) { bc.kind[f] = (f < 2 || f >= 4) ? GBNS_BC_PERIODIC : kinds[kb]; bc.t_wall[f] = 290.0; }
        if (kinds[kb] == GBNS_BC_PERIODIC) { bc.kind[2] = bc.kind[3] = GBNS_BC_PERIODIC; }
        CHECK(oracle_fill_ghosts(&g, &bc, q));
        CHECK(oracle_flux_div(&g, &schemes[si], q, r, 0, 1));
        CHECK(oracle_flux_div(&g, &schemes[si], q, r, 1, 1));
        const double* res[1] = {r};
        const double cf[1] = {1e-9};
        gbns_gas_desc gas = {1.4, 287.0};
        CHECK(oracle_rk_stage(&g, &gas, q, res, cf, 1));
        double out[5];
        for (int k = 0; k < 4; ++k) CHECK(oracle_reduce(&g, &gas, q, k, out));
        gbns_source_desc src;
        memset(&src, 0, sizeof(src));
        src.kind = GBNS_SOURCE_BODY_ACCEL; src.c[2] = 1.0; src.gas = gas;
        CHECK(oracle_source_term(&g, &src, q, r));
        if (coords[ci] == GBNS_COORDS_IDENTITY)
        {
            const int apply[6] = {1, 1, 1, 1, 1, 1};
            CHECK(oracle_boundary_flux(&g, &schemes[si], q, r, apply));
        }
        CHECK(oracle_ssprk3_step(&g, &schemes[si], &bc, q, w, 1e-9, 1));
        for (size_t i = 0; i < n; ++i)
            if (!isfinite(q[i])) { fprintf(stderr, "non-finite state (coords %d, scheme %d)\n", ci, si); return 1; }
        free(q); free(r); free(w);
    }
    printf("sanitized oracle runs ok\n");
    return 0;
}
