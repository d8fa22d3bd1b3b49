// The C++ drop-in (include/spade_gb300.h) run for real at a SPADE call site,
// on device::cpu grid_arrays, with no test hook: spade::pde_algs::flux_div
// with the gb300 traits lowers the call and hands it to gbns_flux_div_host.
// Linked here with tests/cpp/gbns_record_stub.c in place of libgbns.so, the
// call is recorded (descriptors and host arrays as the header produced them)
// for replay through the real library on a GPU.  For the schemes the
// reference can run, the reference's own CPU flux_div on the same arrays is
// written next to it (argv[1]: one file of doubles per such case, in order).
//
// Cases (2x1x1 blocks of 8x4x4 cells, 3 ghost layers, one seeded state):
//   1. compose(cent_keep<2>, visc_lr(constant)), identity, increment mode
//   2. compose(fweno_t, pressure_diss_lr(const_sensor), visc_lr(constant)), overwrite
//   3. compose(gb300::weno5_t, pressure_diss_lr, visc_lr(gb300::sutherland_t)) on
//      diagonal_coords(identity_1D, gb300::tanh_stretch_1D(2), identity_1D), overwrite
//      (no reference counterpart: compared with the oracle after replay)
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
    void fill_state(arr_t& q)
    {
        for (std::size_t i = 0; i < q.data.size(); i += 5)
        {
            q.data[i + 0] = 1.0e5*(1.0 + 0.02*noise(i));
            q.data[i + 1] = 300.0*(1.0 + 0.02*noise(i + 1));
            q.data[i + 2] = 30.0*noise(i + 2);
            q.data[i + 3] = 30.0*noise(i + 3);
            q.data[i + 4] = 30.0*noise(i + 4);
        }
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
        spade::ctrs::array<int, 3> num_blocks(2, 1, 1), cells(8, 4, 4), nexch(3, 3, 3);
        spade::bound_box_t<real_t, 3> bounds;
        bounds.min(0) = 0.0; bounds.max(0) = 2.0;
        bounds.min(1) = -1.0; bounds.max(1) = 1.0;
        bounds.min(2) = 0.0; bounds.max(2) = 1.0;
        spade::grid::cartesian_blocks_t blocks(num_blocks, bounds);
        for (std::size_t lb = 0; lb < blocks.block_is_domain_boundary.size(); ++lb)
            for (int d = 0; d < 3; ++d)
            {
                blocks.block_is_domain_boundary[lb].min(d) = (d != 0 || lb == 0);
                blocks.block_is_domain_boundary[lb].max(d) = (d != 0 || lb == 1);
            }
        spade::fluid_state::ideal_gas_t<real_t> air(1.4, 287.0);
        spade::viscous_laws::constant_viscosity_t<real_t> law(2.0e-3, 0.72);
        spade::viscous::visc_lr visc(law, air);
        spade::state_sensor::const_sensor_t<real_t> sens(1.0);
        spade::convective::pressure_diss_lr diss(air, sens, 3.0, 3.0);

        spade::coords::identity<real_t> coords;
        spade::grid::cartesian_grid_t grid(cells, blocks, coords, group);
        spade::grid::grid_array q  (grid, prim_t(0.0), nexch, spade::device::cpu);
        spade::grid::grid_array rhs(grid, flux_t(0.0), nexch, spade::device::cpu);
        spade::grid::grid_array ref(grid, flux_t(0.0), nexch, spade::device::cpu);
        fill_state(q);

        // 1. increment mode from rhs = 0.5 everywhere
        const auto f1 = spade::omni::compose(spade::convective::cent_keep<2>(air), visc);
        for (auto& x : rhs.data) x = 0.5;
        for (auto& x : ref.data) x = 0.5;
        spade::pde_algs::flux_div(q, ref, f1);
        spade::pde_algs::flux_div(q, rhs, f1, spade::algs::make_traits(spade::pde_algs::gb300));
        write(argv[1], ref);

        // 2. overwrite mode
        const auto f2 = spade::omni::compose(spade::convective::fweno_t<decltype(air)>(air), diss, visc);
        for (auto& x : rhs.data) x = 0.0;
        for (auto& x : ref.data) x = 0.0;
        spade::pde_algs::flux_div(q, ref, f2, spade::algs::make_traits(spade::pde_algs::basic, spade::pde_algs::overwrite));
        spade::pde_algs::flux_div(q, rhs, f2, spade::algs::make_traits(spade::pde_algs::gb300, spade::pde_algs::overwrite));
        write(argv[1], ref);

        // 3. the benchmarked channel scheme on a tanh-stretched grid
        spade::coords::diagonal_coords scoords(spade::coords::identity_1D<real_t>(), spade::gb300::tanh_stretch_1D<real_t>(2.0),
                                               spade::coords::identity_1D<real_t>());
        spade::grid::cartesian_grid_t sgrid(cells, blocks, scoords, group);
        spade::grid::grid_array sq  (sgrid, prim_t(0.0), nexch, spade::device::cpu);
        spade::grid::grid_array srhs(sgrid, flux_t(0.0), nexch, spade::device::cpu);
        fill_state(sq);
        spade::gb300::sutherland_t<real_t> suth(2.0e-3, 300.0, 110.4, 0.72);
        const auto f3 = spade::omni::compose(spade::gb300::weno5_t<decltype(air)>(air), diss, spade::viscous::visc_lr(suth, air));
        spade::pde_algs::flux_div(sq, srhs, f3, spade::algs::make_traits(spade::pde_algs::gb300, spade::pde_algs::overwrite));
    });
    return 0;
}
