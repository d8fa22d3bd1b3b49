// Host-only check of include/spade_gb300.h against the reference's headers:
// the gb300 trait must select the drop-in flux_div overload, which lowers the
// composed functor and the grid_array into the C-ABI descriptors.  The GPU
// call is replaced by a hook (GBNS_DROPIN_HOOK) that prints the descriptors.
#include <cstdio>
#include "gbns.h"

static int g_calls = 0;
static int record(const gbns_grid_desc* g, const gbns_scheme_desc* s, const double* q, double* r, int incr)
{
    ++g_calls;
    std::printf("grid %d %d %d %d %d %d %d %.17g %.17g %.17g %.17g %.17g %.17g\n",
                g->nblk[0], g->nblk[1], g->nblk[2], g->ncell[0], g->ncell[1], g->ncell[2], g->ng,
                g->bounds[0], g->bounds[1], g->bounds[2], g->bounds[3], g->bounds[4], g->bounds[5]);
    std::printf("scheme %d %d %d %d %d %d %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g incr %d ptrs %d sensor %d hyb %d %d %.17g\n",
                s->convective, s->order, s->weno_smooth, s->dissipation, s->viscous, s->visc_law, s->precision,
                s->eps_p, s->eps_T, s->sensor_alpha, s->mu, s->prandtl_inv, s->gas.gamma, s->gas.R, s->T_ref,
                incr, int(q != nullptr && r != nullptr), s->sensor, s->hybrid_flux, s->hybrid_sensor, s->hybrid_param);
    std::printf("coords %d %.17g %.17g %.17g %.17g law %d S %.17g Tref %.17g pr %.17g\n", g->coords, g->coord_param[0],
                g->coord_param[1], g->coord_param[2], g->coord_param[3], s->visc_law, s->S, s->T_ref, s->prandtl);
    return 0;
}
#define GBNS_DROPIN_HOOK record

static int g_src_calls = 0;
static int record_source(const gbns_grid_desc* g, const gbns_source_desc* d, const double* q, double* r)
{
    ++g_src_calls;
    std::printf("source %d %.17g %.17g %.17g %.17g %.17g R %.17g ptrs %d\n", d->kind, d->c[0], d->c[1], d->c[2], d->c[3],
                d->c[4], d->gas.R, int(q != nullptr && r != nullptr));
    return 0;
}
#define GBNS_DROPIN_SOURCE_HOOK record_source

static int g_bf_calls = 0;
static int record_bflux(const gbns_grid_desc* g, const gbns_scheme_desc* s, const double* q, double* r, const int* apply)
{
    ++g_bf_calls;
    std::printf("bflux %d %d %d %d %d %d conv %d order %d visc %d ng %d ptrs %d\n", apply[0], apply[1], apply[2], apply[3],
                apply[4], apply[5], s->convective, s->order, s->viscous, g->ng, int(q != nullptr && r != nullptr));
    return 0;
}
#define GBNS_DROPIN_BFLUX_HOOK record_bflux

static int g_bc_calls = 0;
static int record_bc(const gbns_grid_desc* g, const gbns_bc_desc* bc, const gbns_scheme_desc* s, double* q, double dt)
{
    ++g_bc_calls;
    std::printf("bc %d %d %d %d %d %d tw %.17g %.17g step %d conv %d dt %.17g ng %d ptr %d\n", bc->kind[0], bc->kind[1],
                bc->kind[2], bc->kind[3], bc->kind[4], bc->kind[5], bc->t_wall[2], bc->t_wall[3], int(s != nullptr),
                s ? s->convective : -1, dt, g->ng, int(q != nullptr));
    return 0;
}
#define GBNS_DROPIN_BC_HOOK record_bc

#include "spade.h"
#include "spade_gb300.h"

int main(int argc, char** argv)
{
    using real_t = double;
    spade::parallel::compute_env_t env(&argc, &argv, {0});
    env.exec([&](spade::parallel::pool_t& group)
    {
        spade::ctrs::array<int, 3> num_blocks(2, 3, 1);
        spade::ctrs::array<int, 3> cells(8, 6, 4);
        spade::bound_box_t<real_t, 3> bounds;
        bounds.min(0) = 0.0; bounds.max(0) = 2.0;
        bounds.min(1) = -1.0; bounds.max(1) = 1.0;
        bounds.min(2) = 0.0; bounds.max(2) = 0.5;
        spade::coords::identity<real_t> coords;
        spade::grid::cartesian_blocks_t blocks(num_blocks, bounds);
        spade::grid::cartesian_grid_t grid(cells, blocks, coords, group);
        spade::ctrs::array<int, 3> nexch(3, 3, 3);
        spade::grid::grid_array q  (grid, spade::fluid_state::prim_t<real_t>(0.0), nexch, spade::device::cpu);
        spade::grid::grid_array rhs(grid, spade::fluid_state::flux_t<real_t>(0.0), nexch, spade::device::cpu);
        spade::fluid_state::ideal_gas_t<real_t> air(1.4, 287.0);
        spade::viscous_laws::constant_viscosity_t<real_t> law(1.5e-5, 0.72);
        spade::viscous::visc_lr visc(law, air);
        spade::state_sensor::const_sensor_t<real_t> sens(0.25);
        spade::convective::pressure_diss_lr diss(air, sens, 0.1, 0.2);
        // 1: the C1 composite, default (increment) mode
        spade::pde_algs::flux_div(q, rhs, spade::omni::compose(spade::convective::cent_keep<2>(air), visc),
                                  spade::algs::make_traits(spade::pde_algs::gb300));
        // 2: the channel composite, overwrite mode, FP32 flux
        spade::pde_algs::flux_div(q, rhs, spade::omni::compose(spade::convective::fweno_t<decltype(air)>(air), diss, visc),
                                  spade::algs::make_traits(spade::pde_algs::gb300, spade::pde_algs::overwrite, spade::gb300::fp32_flux));
        // 3: a single functor
        spade::pde_algs::flux_div(q, rhs, spade::convective::totani_lr(air),
                                  spade::algs::make_traits(spade::pde_algs::gb300, spade::pde_algs::overwrite));
        // 4: pressure dissipation scaled by the Ducros sensor
        spade::state_sensor::ducros_t<real_t> ducros(0.5);
        spade::convective::pressure_diss_lr ddiss(air, ducros, 0.1, 0.2);
        spade::pde_algs::flux_div(q, rhs, spade::omni::compose(spade::convective::fweno_t<decltype(air)>(air), ddiss, visc),
                                  spade::algs::make_traits(spade::pde_algs::gb300));
        // 5: hybrid centred/WENO flux blended by the Ducros sensor, diss_flux tag
        spade::convective::hybrid_scheme_t hyb(spade::convective::cent_keep<4>(air), spade::convective::fweno_t<decltype(air)>(air),
                                               spade::state_sensor::ducros_t<real_t>(0.125), spade::convective::diss_flux);
        spade::pde_algs::flux_div(q, rhs, spade::omni::compose(hyb, visc), spade::algs::make_traits(spade::pde_algs::gb300));
        // 6, 7: lowered point sources through the source_term overload
        spade::pde_algs::source_term(q, rhs, spade::gb300::body_force_t{2.5, 0.0, -1.0});
        spade::pde_algs::source_term(q, rhs, spade::gb300::body_accel_t{air, 0.0, -9.81, 0.0});
        // 8: boundary_flux on the y walls with the gb300 traits appended
        spade::bound_box_t<bool, 3> walls = false;
        walls.min(1) = true;
        walls.max(1) = true;
        spade::pde_algs::boundary_flux(q, rhs, walls, spade::omni::compose(spade::convective::cent_keep<4>(air), visc),
                                       spade::algs::make_traits(spade::pde_algs::gb300));
        // 9, 10: the channel at scale's scheme, compose(weno5_t, pressure_diss_lr,
        // visc_lr(sutherland_t)), on tanh-stretched and integrated-tanh y grids
        spade::gb300::sutherland_t<real_t> suth(1.8e-5, 300.0, 110.4, 0.72);
        spade::viscous::visc_lr svisc(suth, air);
        const auto channel_flux = spade::omni::compose(spade::gb300::weno5_t<decltype(air)>(air), diss, svisc);
        spade::coords::diagonal_coords scoords(spade::coords::identity_1D<real_t>(), spade::gb300::tanh_stretch_1D<real_t>(2.0),
                                               spade::coords::identity_1D<real_t>());
        spade::grid::cartesian_grid_t sgrid(cells, blocks, scoords, group);
        spade::grid::grid_array sq  (sgrid, spade::fluid_state::prim_t<real_t>(0.0), nexch, spade::device::cpu);
        spade::grid::grid_array srhs(sgrid, spade::fluid_state::flux_t<real_t>(0.0), nexch, spade::device::cpu);
        spade::pde_algs::flux_div(sq, srhs, channel_flux, spade::algs::make_traits(spade::pde_algs::gb300, spade::pde_algs::overwrite));
        spade::coords::diagonal_coords icoords(spade::coords::identity_1D<real_t>(),
                                               spade::coords::integrated_tanh_1D<real_t>(-1.0, 1.0, 0.3, 2.5),
                                               spade::coords::identity_1D<real_t>());
        spade::grid::cartesian_grid_t igrid(cells, blocks, icoords, group);
        spade::grid::grid_array iq  (igrid, spade::fluid_state::prim_t<real_t>(0.0), nexch, spade::device::cpu);
        spade::grid::grid_array irhs(igrid, spade::fluid_state::flux_t<real_t>(0.0), nexch, spade::device::cpu);
        spade::pde_algs::flux_div(iq, irhs, channel_flux, spade::algs::make_traits(spade::pde_algs::gb300));
        // 11, 12: the channel's ghost fill (periodic x and z, isothermal walls
        // in y) and its fused SSPRK3 integrator on the stretched grid
        const spade::ctrs::array<bool, 3> periodic(true, false, true);
        spade::bound_box_t<bool, 3> ywalls = false;
        ywalls.min(1) = true;
        ywalls.max(1) = true;
        const spade::gb300::isothermal_wall_t<real_t> wall{300.0};
        spade::gb300::fill_ghosts(sq, periodic, ywalls, wall);
        spade::gb300::ssprk3_integrator_t step(sq, channel_flux, periodic, ywalls, wall, 2.5e-4);
        step.advance();
        step.advance();
        std::printf("integrator t %.17g\n", step.time());
        // 13: a slip wall on z-min only
        spade::bound_box_t<bool, 3> zwall = false;
        zwall.min(2) = true;
        spade::gb300::fill_ghosts(q, spade::ctrs::array<bool, 3>(true, true, false), zwall, spade::gb300::slip_wall_t<real_t>{});
        // the same wall kernel through the reference's own CPU boundary_fill:
        // a ghost below y-min takes T = 2 T_wall - T and negated velocities
        spade::fluid_state::prim_t<real_t> inside;
        inside.p() = 1.0e5; inside.T() = 310.0; inside.u() = 2.0; inside.v() = -1.0; inside.w() = 0.5;
        spade::grid::cartesian_blocks_t wblocks(spade::ctrs::array<int, 3>(1, 1, 1), bounds);
        spade::grid::cartesian_grid_t wgrid(spade::ctrs::array<int, 3>(4, 4, 4), wblocks, coords, group);
        // (the reference's fill_array tiles the padded range in fours: 4 + 2*2 cells)
        spade::grid::grid_array wq(wgrid, spade::fluid_state::prim_t<real_t>(0.0), spade::ctrs::array<int, 3>(2, 2, 2),
                                   spade::device::cpu);
        using point_t = spade::coords::point_t<real_t>;
        spade::algs::fill_array(wq, [=](const point_t&) { return inside; });
        spade::algs::boundary_fill(wq, spade::boundary::ymin, wall);
        const auto img = wq.image();
        spade::grid::cell_idx_t gi(0, -1, 0, 0);
        const auto ghost = img.get_elem(gi);
        std::printf("cpu_wall %.17g %.17g %.17g %.17g %.17g\n", ghost.p(), ghost.T(), ghost.u(), ghost.v(), ghost.w());
    });
    std::printf("calls %d sources %d bflux %d bc %d\n", g_calls, g_src_calls, g_bf_calls, g_bc_calls);
    return (g_calls == 7 && g_src_calls == 2 && g_bf_calls == 1 && g_bc_calls == 4) ? 0 : 1;
}
