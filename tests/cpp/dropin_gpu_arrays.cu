// Compile-only check (nvcc, the reference's CUDA build options) of
// include/spade_gb300.h without the test hooks on device::gpu grid_arrays:
// the gb300 flux_div overload, the ghost fill and the fused SSPRK3 integrator
// instantiate against the C ABI (gbns_flux_div, gbns_fill_ghosts,
// gbns_ssprk3_step), and on a refined (amr_blocks_t) grid the exchange plan,
// flux_div and the refined-grid integrator (gbns_exchange_plan_*,
// gbns_flux_div_blocks, gbns_ssprk3_step_blocks).
#include "spade.h"
#include "spade_gb300.h"

void run_on_gpu_arrays(spade::parallel::pool_t& group)
{
    using real_t = double;
    spade::ctrs::array<int, 3> num_blocks(2, 2, 2);
    spade::ctrs::array<int, 3> cells(16, 16, 16);
    spade::bound_box_t<real_t, 3> bounds;
    for (int d = 0; d < 3; ++d) { bounds.min(d) = 0.0; bounds.max(d) = 1.0; }
    spade::coords::identity<real_t> coords;
    spade::grid::cartesian_blocks_t blocks(num_blocks, bounds);
    spade::grid::cartesian_grid_t grid(cells, blocks, coords, group);
    spade::ctrs::array<int, 3> nexch(2, 2, 2);
    spade::grid::grid_array q  (grid, spade::fluid_state::prim_t<real_t>(0.0), nexch, spade::device::gpu);
    spade::grid::grid_array rhs(grid, spade::fluid_state::flux_t<real_t>(0.0), nexch, spade::device::gpu);
    spade::fluid_state::ideal_gas_t<real_t> air(1.4, 287.0);
    spade::viscous_laws::constant_viscosity_t<real_t> law(1.5e-5, 0.72);
    spade::viscous::visc_lr visc(law, air);
    const auto flux = spade::omni::compose(spade::convective::cent_keep<2>(air), visc);
    spade::pde_algs::flux_div(q, rhs, flux, spade::algs::make_traits(spade::pde_algs::gb300));
    const spade::ctrs::array<bool, 3> periodic(true, false, true);
    spade::bound_box_t<bool, 3> walls = false;
    walls.min(1) = true;
    walls.max(1) = true;
    const spade::gb300::isothermal_wall_t<real_t> wall{300.0};
    spade::gb300::fill_ghosts(q, periodic, walls, wall);
    spade::gb300::ssprk3_integrator_t step(q, flux, periodic, walls, wall, 1.0e-4);
    step.advance();

    // a refined grid: block 0 split in place, its exchange as boundary condition
    spade::ctrs::array<bool, 3> all_periodic(true, true, true);
    spade::amr::amr_blocks_t ablocks(num_blocks, bounds);
    spade::grid::cartesian_grid_t agrid(cells, ablocks, coords, group);
    agrid.refine_blocks(std::vector<std::size_t>{0}, all_periodic);
    spade::grid::grid_array aq  (agrid, spade::fluid_state::prim_t<real_t>(0.0), nexch, spade::device::gpu);
    spade::grid::grid_array arhs(agrid, spade::fluid_state::flux_t<real_t>(0.0), nexch, spade::device::gpu);
    auto handle = spade::grid::make_exchange(aq, all_periodic);
    const spade::gb300::exchange_plan_t plan(handle, aq);
    plan.exchange(aq);
    spade::pde_algs::flux_div(aq, arhs, flux, spade::algs::make_traits(spade::pde_algs::gb300));
    spade::gb300::ssprk3_refined_integrator_t astep(aq, flux, plan, 1.0e-4);
    astep.advance();
    spade::gb300::ssprk3_refined_integrator_t wstep(aq, flux, plan, periodic, walls, wall, 1.0e-4);
    wstep.advance();
}
