// Compile-only check of include/spade_gb300.h without the test hooks: the
// gb300 flux_div overload on device::cpu arrays takes the host path
// (gbns_flux_div_host), so SPADE's CPU grid_arrays reach the GPU kernels.
#include "spade.h"
#include "spade_gb300.h"

void run_on_cpu_arrays(spade::parallel::pool_t& group)
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
    spade::grid::grid_array q  (grid, spade::fluid_state::prim_t<real_t>(0.0), nexch, spade::device::cpu);
    spade::grid::grid_array rhs(grid, spade::fluid_state::flux_t<real_t>(0.0), nexch, spade::device::cpu);
    spade::fluid_state::ideal_gas_t<real_t> air(1.4, 287.0);
    spade::viscous_laws::constant_viscosity_t<real_t> law(1.5e-5, 0.72);
    spade::viscous::visc_lr visc(law, air);
    spade::pde_algs::flux_div(q, rhs, spade::omni::compose(spade::convective::cent_keep<2>(air), visc),
                              spade::algs::make_traits(spade::pde_algs::gb300));
}
