// Host-only check of spade::gb300::lower_exchange (include/spade_gb300.h):
// an amr_blocks_t grid refined in place (cartesian_grid_t::refine_blocks),
// the reference's own exchange handle (grid::make_exchange), and the
// gbns_patch records the drop-in lowers it into, printed one per line for
// comparison with the reference harness's dump of the same handle.
#include <cstdio>
#include "gbns.h"
static int no_hook(const gbns_grid_desc*, const gbns_scheme_desc*, const double*, double*, int) { return 0; }
#define GBNS_DROPIN_HOOK no_hook
#include "spade.h"
#include "spade_gb300.h"

int main(int argc, char** argv)
{
    using real_t = double;
    using prim_t = spade::fluid_state::prim_t<real_t>;
    spade::parallel::compute_env_t env(&argc, &argv, {0});
    env.exec([&](spade::parallel::pool_t& group)
    {
        spade::bound_box_t<real_t, 3> bounds;
        for (int d = 0; d < 3; ++d) { bounds.min(d) = 0.0; bounds.max(d) = 1.0; }
        spade::coords::identity<real_t> coords;
        spade::ctrs::array<int, 3> nb(2, 2, 2), cells(4, 4, 4);
        spade::amr::amr_blocks_t blocks(nb, bounds);
        spade::grid::cartesian_grid_t grid(cells, blocks, coords, group);
        spade::ctrs::array<bool, 3> per = {true, false, true};
        std::vector<std::size_t> first = {0};
        grid.refine_blocks(first, per);
        grid.refine_blocks(first, per);
        spade::ctrs::array<int, 3> nexch(3, 3, 3);
        spade::grid::grid_array q(grid, prim_t(0.0), nexch, spade::device::cpu);
        auto handle = spade::grid::make_exchange(q, per);
        const auto plan = spade::gb300::lower_exchange(handle);
        spade::gb300::exchange_plan_t gpu_plan(handle, q);   // constructs without a GPU under the hook
        std::printf("blocks %d patches %zu\n", int(grid.get_num_global_blocks()), plan.size());
        for (const auto& p : plan)
            std::printf("%d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d\n", p.kind, p.src_block, p.dst_block,
                        p.src_lo[0], p.src_lo[1], p.src_lo[2], p.dst_lo[0], p.dst_lo[1], p.dst_lo[2],
                        p.dst_hi[0], p.dst_hi[1], p.dst_hi[2], p.i_coeff[0], p.i_coeff[1], p.i_coeff[2],
                        p.i_incr[0], p.i_incr[1], p.i_incr[2]);
    });
    return 0;
}
