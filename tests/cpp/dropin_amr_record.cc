// The C++ drop-in (include/spade_gb300.h) on a refined (AMR) grid at a SPADE
// call site, device::cpu grid_arrays, no test hook: spade::pde_algs::flux_div
// with the gb300 traits lowers the grid to per-block boxes and hands the call
// to gbns_flux_div_blocks_host.  Linked with tests/cpp/gbns_record_stub.c in
// place of libgbns.so, the call is recorded for replay through the real
// library on a GPU; the reference's own CPU flux_div on the same arrays is
// written to argv[1] (one array of doubles per case, in order).
//
// Grid: 2x2x2 amr_blocks_t blocks of 4^3 cells on [0,1]^3, 2 ghost layers,
// periodic, block 0 refined in place (cartesian_grid_t::refine_blocks): 15
// blocks on two levels; a seeded state, ghosts from the reference's exchange.
//   1. compose(cent_keep<2>, visc_lr(constant)), overwrite
//   2. compose(fweno_t, pressure_diss_lr(const_sensor), visc_lr(constant)), increment from 0.25
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <vector>
#include "spade.h"
#include "spade_gb300.h"

namespace
{
    // deterministic state: p ~ 1e5, T ~ 300, |u| ~ 30 (splitmix64 noise)
    double noise(uint64_t k)
    {
        k += 0x9E3779B97F4A7C15ull;
        k = (k ^ (k >> 30))*0xBF58476D1CE4E5B9ull;
        k = (k ^ (k >> 27))*0x94D049BB133111EBull;
        k ^= k >> 31;
        return double(k >> 11)*(1.0/9007199254740992.0) - 0.5;
    }

    template <typename arr_t>
    void write(const char* path, const arr_t& a)
    {
        FILE* f = std::fopen(path, "ab");
        std::fwrite(a.data.data(), 8, a.data.size(), f);
        std::fclose(f);
    }
}

int main(int argc, char** argv)
{
    if (argc != 2) { std::fprintf(stderr, "usage: %s reference_results_file\n", argv[0]); return 2; }
    using real_t = double;
    using prim_t = spade::fluid_state::prim_t<real_t>;
    using flux_t = spade::fluid_state::flux_t<real_t>;
    int eargc = 0;
    char** eargv = nullptr;
    spade::parallel::compute_env_t env(&eargc, &eargv, {0});
    env.exec([&](spade::parallel::pool_t& group)
    {
        spade::ctrs::array<int, 3> num_blocks(2, 2, 2), cells(4, 4, 4), nexch(2, 2, 2);
        spade::bound_box_t<real_t, 3> bounds;
        for (int d = 0; d < 3; ++d) { bounds.min(d) = 0.0; bounds.max(d) = 1.0; }
        spade::ctrs::array<bool, 3> periodic(true, true, true);
        spade::coords::identity<real_t> coords;
        spade::amr::amr_blocks_t blocks(num_blocks, bounds);
        spade::grid::cartesian_grid_t grid(cells, blocks, coords, group);
        grid.refine_blocks(std::vector<std::size_t>{0}, periodic);

        spade::grid::grid_array q  (grid, prim_t(0.0), nexch, spade::device::cpu);
        spade::grid::grid_array rhs(grid, flux_t(0.0), nexch, spade::device::cpu);
        spade::grid::grid_array ref(grid, flux_t(0.0), nexch, spade::device::cpu);
        for (std::size_t i = 0; i < q.data.size(); i += 5)
        {
            q.data[i + 0] = 1.0e5*(1.0 + 0.02*noise(i));
            q.data[i + 1] = 300.0*(1.0 + 0.02*noise(i + 1));
            q.data[i + 2] = 30.0*noise(i + 2);
            q.data[i + 3] = 30.0*noise(i + 3);
            q.data[i + 4] = 30.0*noise(i + 4);
        }
        auto handle = spade::grid::make_exchange(q, periodic);
        handle.exchange(q, group);

        spade::fluid_state::ideal_gas_t<real_t> air(1.4, 287.0);
        spade::viscous_laws::constant_viscosity_t<real_t> law(2.0e-3, 0.72);
        spade::viscous::visc_lr visc(law, air);
        spade::state_sensor::const_sensor_t<real_t> sens(1.0);
        spade::convective::pressure_diss_lr diss(air, sens, 3.0, 3.0);

        // 1. overwrite mode
        const auto f1 = spade::omni::compose(spade::convective::cent_keep<2>(air), visc);
        spade::pde_algs::flux_div(q, ref, f1, spade::algs::make_traits(spade::pde_algs::basic, spade::pde_algs::overwrite));
        spade::pde_algs::flux_div(q, rhs, f1, spade::algs::make_traits(spade::pde_algs::gb300, spade::pde_algs::overwrite));
        write(argv[1], ref);

        // 2. increment mode from rhs = 0.25 everywhere
        const auto f2 = spade::omni::compose(spade::convective::fweno_t<decltype(air)>(air), diss, visc);
        for (auto& x : rhs.data) x = 0.25;
        for (auto& x : ref.data) x = 0.25;
        spade::pde_algs::flux_div(q, ref, f2);
        spade::pde_algs::flux_div(q, rhs, f2, spade::algs::make_traits(spade::pde_algs::gb300));
        write(argv[1], ref);
    });
    return 0;
}
