// Test-infrastructure harness around the REFERENCE's own CPU path.
//
// This file is compiled (by oracle/Makefile) against the reference's headers
// where they lie, plus the single-rank MPI stand-in in oracle/mpi_stub, into
// oracle/_ref/libspade_ref.so.  It only drives the reference's public API:
//   - spade::pde_algs::flux_div               (pde-algs/flux-div/flux_div.h:16-56)
//   - spade::grid::make_exchange / exchange   (grid/make_exchange.h:98-421)
//   - spade::algs::boundary_fill              (grid/boundary_fill.h:31-133)
//   - spade::time_integration::integrator_t   (time-integration/integrator.h:18-59)
//     with ssprk3_t (time-integration/explicit.h:80-88) and
//     fluid_state::state_transform_t (navier-stokes/state_transformation.h:38-66)
// and copies plain AoS5 arrays (ghosts included) in and out, so the tests can
// compare the CPU restatement and the CUDA path with the reference itself on
// identical seeded inputs.  Nothing here is part of the shipped library.
#include <cstring>
#include <vector>
#include <cmath>
#include <stdexcept>

#include "spade.h"

namespace
{
    template <typename grid_t> struct utils_grid_point { using type = typename grid_t::coord_point_type; };
    using real_t = double;
    using prim_t = spade::fluid_state::prim_t<real_t>;
    using flux_t = spade::fluid_state::flux_t<real_t>;
    using cons_t = spade::fluid_state::cons_t<real_t>;
    using gas_t  = spade::fluid_state::ideal_gas_t<real_t>;

    struct problem_t
    {
        int nb[3], nc[3], ng;
        double bounds[6];
        double gamma, rgas, mu, prandtl;
        double eps_p, eps_T, sensor;
        double hybrid_param;   // hybrid_scheme_t blender: const_sensor_t alpha or ducros_t epsilon
        int periodic[3];
        int wall_y;
        double t_wall;
    };

    // Scheme identifiers shared with oracle/oracle.py.
    enum scheme_id
    {
        S_CK2_VISC    = 0,  // compose(cent_keep<2>, visc_lr(constant))
        S_TOTANI_VISC = 1,  // compose(totani_lr, visc_lr(constant))
        S_CK4_VISC    = 2,  // compose(cent_keep<4>, visc_lr(constant))
        S_CK2         = 3,  // cent_keep<2>
        S_VISC        = 4,  // visc_lr(constant)
        S_FWENO_DISS_VISC = 5, // compose(fweno_t, pressure_diss_lr(const_sensor), visc_lr(constant))
        S_FWENO       = 6,  // fweno_t
        S_DISS        = 7,  // pressure_diss_lr(const_sensor)
        S_TOTANI      = 8,  // totani_lr
        S_CK6         = 9,  // cent_keep<6>
        S_CK8         = 10, // cent_keep<8>
        S_FWENO_NOSMOOTH = 11, // fweno_t<gas, disable_smooth>
        S_CK2_DISS_VISC  = 12, // compose(cent_keep<2>, pressure_diss_lr(const_sensor), visc_lr(constant))
        S_DUCROS_DISS    = 13, // pressure_diss_lr(ducros_t)
        S_FWENO_DUCROS_VISC = 14, // compose(fweno_t, pressure_diss_lr(ducros_t), visc_lr(constant))
        S_HYB_CK2_FULL      = 15, // hybrid_scheme_t(cent_keep<2>, fweno_t, ducros_t, full_flux)
        S_HYB_CK4_DISS_VISC = 16, // compose(hybrid_scheme_t(cent_keep<4>, fweno_t, ducros_t, diss_flux), visc_lr(constant))
        S_HYB_CK2_CONST_DISS_VISC = 17 // compose(hybrid_scheme_t(cent_keep<2>, fweno_t, const_sensor_t, full_flux),
                                       //         pressure_diss_lr(ducros_t), visc_lr(constant))
    };

    template <typename func_t>
    void with_flux(const problem_t& pb, int scheme, const func_t& func)
    {
        gas_t air(pb.gamma, pb.rgas);
        spade::viscous_laws::constant_viscosity_t<real_t> law(pb.mu, pb.prandtl);
        spade::viscous::visc_lr visc(law, air);
        spade::state_sensor::const_sensor_t<real_t> sens(pb.sensor);
        spade::convective::pressure_diss_lr diss(air, sens, pb.eps_p, pb.eps_T);
        spade::state_sensor::ducros_t<real_t> ducros(pb.sensor);
        spade::state_sensor::const_sensor_t<real_t> hsens(pb.hybrid_param);
        spade::state_sensor::ducros_t<real_t> hducros(pb.hybrid_param);
        spade::convective::pressure_diss_lr ddiss(air, ducros, pb.eps_p, pb.eps_T);
        switch (scheme)
        {
            case S_CK2_VISC:    func(spade::omni::compose(spade::convective::cent_keep<2>(air), visc)); break;
            case S_TOTANI_VISC: func(spade::omni::compose(spade::convective::totani_lr(air), visc)); break;
            case S_CK4_VISC:    func(spade::omni::compose(spade::convective::cent_keep<4>(air), visc)); break;
            case S_CK2:         func(spade::convective::cent_keep<2>(air)); break;
            case S_VISC:        func(visc); break;
            case S_FWENO_DISS_VISC:
                func(spade::omni::compose(spade::convective::fweno_t<gas_t>(air), diss, visc)); break;
            case S_FWENO:       func(spade::convective::fweno_t<gas_t>(air)); break;
            case S_DISS:        func(diss); break;
            case S_TOTANI:      func(spade::convective::totani_lr(air)); break;
            case S_CK6:         func(spade::convective::cent_keep<6>(air)); break;
            case S_CK8:         func(spade::convective::cent_keep<8>(air)); break;
            case S_FWENO_NOSMOOTH:
                func(spade::convective::fweno_t<gas_t, spade::convective::disable_smooth>(air)); break;
            case S_CK2_DISS_VISC:
                func(spade::omni::compose(spade::convective::cent_keep<2>(air), diss, visc)); break;
            case S_DUCROS_DISS: func(ddiss); break;
            case S_FWENO_DUCROS_VISC:
                func(spade::omni::compose(spade::convective::fweno_t<gas_t>(air), ddiss, visc)); break;
            case S_HYB_CK2_FULL:
                func(spade::convective::hybrid_scheme_t(spade::convective::cent_keep<2>(air), spade::convective::fweno_t<gas_t>(air),
                                                        hducros, spade::convective::full_flux)); break;
            case S_HYB_CK4_DISS_VISC:
                func(spade::omni::compose(spade::convective::hybrid_scheme_t(spade::convective::cent_keep<4>(air),
                                                                             spade::convective::fweno_t<gas_t>(air),
                                                                             hducros, spade::convective::diss_flux), visc)); break;
            case S_HYB_CK2_CONST_DISS_VISC:
                func(spade::omni::compose(spade::convective::hybrid_scheme_t(spade::convective::cent_keep<2>(air),
                                                                             spade::convective::fweno_t<gas_t>(air),
                                                                             hsens, spade::convective::full_flux), ddiss, visc)); break;
            default: throw std::runtime_error("unknown scheme id");
        }
    }

    // Runs `body(grid, group)` on a single-rank compute environment with an
    // identity-coordinate grid built from the problem description.
    template <typename body_t>
    void with_grid(const problem_t& pb, const body_t& body)
    {
        int argc = 0;
        char** argv = nullptr;
        spade::parallel::compute_env_t env(&argc, &argv, {0});
        env.exec([&](spade::parallel::pool_t& group)
        {
            spade::ctrs::array<int, 3> num_blocks(pb.nb[0], pb.nb[1], pb.nb[2]);
            spade::ctrs::array<int, 3> cells(pb.nc[0], pb.nc[1], pb.nc[2]);
            spade::bound_box_t<real_t, 3> bounds;
            for (int d = 0; d < 3; ++d)
            {
                bounds.min(d) = pb.bounds[2*d];
                bounds.max(d) = pb.bounds[2*d+1];
            }
            spade::coords::identity<real_t> coords;
            spade::grid::cartesian_blocks_t blocks(num_blocks, bounds);
            // cartesian_blocks_t (grid/cartesian_blocks.h:51-64) resizes
            // block_is_domain_boundary with bound_box_t's empty default
            // constructor (core/bounding_box.h:22, ctrs.h:173) and only ever
            // sets the true flags, so non-boundary flags are indeterminate.
            // Give every flag its defined value before the grid reads them.
            for (std::size_t lb = 0; lb < blocks.block_is_domain_boundary.size(); ++lb)
            {
                const int b[3] = {int(lb % pb.nb[0]), int((lb / pb.nb[0]) % pb.nb[1]), int(lb / (pb.nb[0]*pb.nb[1]))};
                for (int d = 0; d < 3; ++d)
                {
                    blocks.block_is_domain_boundary[lb].min(d) = (b[d] == 0);
                    blocks.block_is_domain_boundary[lb].max(d) = (b[d] == pb.nb[d]-1);
                }
            }
            spade::grid::cartesian_grid_t grid(cells, blocks, coords, group);
            body(grid, group);
        });
    }

    template <typename arr_t>
    void copy_in(arr_t& arr, const double* src)
    {
        std::memcpy(&arr.data[0], src, arr.data.size()*sizeof(double));
    }

    template <typename arr_t>
    void copy_out(const arr_t& arr, double* dst)
    {
        std::memcpy(dst, &arr.data[0], arr.data.size()*sizeof(double));
    }

    // Isothermal no-slip wall: p_g = p, T_g = 2 T_w - T, u_g = -u.
    struct isothermal_wall_t
    {
        real_t t_wall;
        prim_t operator()(const prim_t& q_dom, const int) const
        {
            prim_t out;
            out.p() = q_dom.p();
            out.T() = real_t(2.0)*t_wall - q_dom.T();
            out.u() = -q_dom.u();
            out.v() = -q_dom.v();
            out.w() = -q_dom.w();
            return out;
        }
    };

    template <typename arr_t, typename exch_t, typename group_t>
    void apply_bc(const problem_t& pb, arr_t& q, exch_t& handle, group_t& group)
    {
        handle.exchange(q, group);
        if (pb.wall_y)
        {
            isothermal_wall_t wall{pb.t_wall};
            spade::algs::boundary_fill(q, spade::boundary::ymin, wall);
            spade::algs::boundary_fill(q, spade::boundary::ymax, wall);
        }
    }

    template <typename arr_t>
    double kinetic_energy(const problem_t& pb, const arr_t& q)
    {
        // Volume-averaged 0.5*rho*|u|^2 over interior cells, rho = p/(R T).
        const int ng = pb.ng;
        const int ni = pb.nc[0]+2*ng, nj = pb.nc[1]+2*ng, nk = pb.nc[2]+2*ng;
        const int nblk = pb.nb[0]*pb.nb[1]*pb.nb[2];
        double sum = 0.0;
        std::size_t count = 0;
        for (int lb = 0; lb < nblk; ++lb)
        for (int k = 0; k < pb.nc[2]; ++k)
        for (int j = 0; j < pb.nc[1]; ++j)
        for (int i = 0; i < pb.nc[0]; ++i)
        {
            const std::size_t off = 5*(std::size_t(i+ng) + std::size_t(ni)*(std::size_t(j+ng) + std::size_t(nj)*(std::size_t(k+ng) + std::size_t(nk)*lb)));
            const double* c = &q.data[off];
            const double rho = c[0]/(pb.rgas*c[1]);
            sum += 0.5*rho*(c[2]*c[2] + c[3]*c[3] + c[4]*c[4]);
            ++count;
        }
        return sum/double(count);
    }
    // Runs `body(grid, group, periodic)` on a single-rank compute environment
    // with the refined identity-coordinate grid of spade_ref_amr_exchange's
    // `ints`: an amr_blocks_t grid built unrefined, then refined in place pass
    // by pass (grid/cartesian_grid.h:331-367).
    template <typename body_t>
    void with_amr_grid(const problem_t& pb, const int* ints, const body_t& body)
    {
        int argc = 0;
        char** argv = nullptr;
        spade::parallel::compute_env_t env(&argc, &argv, {0});
        env.exec([&](spade::parallel::pool_t& group)
        {
            spade::ctrs::array<bool, 3> per(ints[7] != 0, ints[8] != 0, ints[9] != 0);
            spade::bound_box_t<real_t, 3> bbx;
            for (int d = 0; d < 3; ++d) { bbx.min(d) = pb.bounds[2*d]; bbx.max(d) = pb.bounds[2*d + 1]; }
            spade::coords::identity<real_t> coords;
            spade::ctrs::array<int, 3> num_blocks(pb.nb[0], pb.nb[1], pb.nb[2]), cells(pb.nc[0], pb.nc[1], pb.nc[2]);
            spade::amr::amr_blocks_t blocks(num_blocks, bbx);
            spade::grid::cartesian_grid_t grid(cells, blocks, coords, group);
            const int npass = ints[10];
            int pos = 11;
            for (int pss = 0; pss < npass; ++pss)
            {
                const int cnt = ints[pos++];
                std::vector<std::size_t> list;
                for (int i = 0; i < cnt; ++i) list.push_back(std::size_t(ints[pos++]));
                grid.refine_blocks(list, per);
            }
            body(grid, group, per);
        });
    }
}


extern "C"
{
    // Fills `pb` from flat arrays (see oracle/oracle.py:_problem).
    static problem_t make_problem(const int* ints, const double* reals)
    {
        problem_t pb;
        for (int d = 0; d < 3; ++d) { pb.nb[d] = ints[d]; pb.nc[d] = ints[3+d]; pb.periodic[d] = ints[7+d]; }
        pb.ng = ints[6];
        pb.wall_y = ints[10];
        for (int i = 0; i < 6; ++i) pb.bounds[i] = reals[i];
        pb.gamma = reals[6]; pb.rgas = reals[7]; pb.mu = reals[8]; pb.prandtl = reals[9];
        pb.eps_p = reals[10]; pb.eps_T = reals[11]; pb.sensor = reals[12]; pb.t_wall = reals[13];
        pb.hybrid_param = reals[14];
        return pb;
    }

    // The same from the refined-layout ints of spade_ref_amr_exchange (no
    // wall flag: index 10 there is the pass count).
    static problem_t make_problem_amr(const int* ints, const double* reals)
    {
        int flat[11];
        for (int i = 0; i < 10; ++i) flat[i] = ints[i];
        flat[10] = 0;
        return make_problem(flat, reals);
    }

    // One flux_div call.  `prims` is the full AoS5 array including ghosts,
    // used as given; `rhs` is the full AoS5 array including ghosts.  With
    // overwrite != 0 the reference's `overwrite` trait zeroes rhs first,
    // otherwise rhs is incremented (the reference default).
    int spade_ref_flux_div(int scheme, const int* ints, const double* reals, int overwrite,
                           const double* prims, double* rhs)
    {
        try
        {
            const problem_t pb = make_problem(ints, reals);
            with_grid(pb, [&](auto& grid, auto& group)
            {
                spade::ctrs::array<int, 3> nexch(pb.ng, pb.ng, pb.ng);
                spade::grid::grid_array q (grid, prim_t(0.0), nexch, spade::device::cpu);
                spade::grid::grid_array r (grid, flux_t(0.0), nexch, spade::device::cpu);
                copy_in(q, prims);
                copy_in(r, rhs);
                with_flux(pb, scheme, [&](const auto& flx)
                {
                    if (overwrite)
                        spade::pde_algs::flux_div(q, r, flx, spade::algs::make_traits(spade::pde_algs::basic, spade::pde_algs::overwrite));
                    else
                        spade::pde_algs::flux_div(q, r, flx);
                });
                copy_out(r, rhs);
            });
        }
        catch (const std::exception& e) { std::fprintf(stderr, "spade_ref_flux_div: %s\n", e.what()); return -1; }
        return 0;
    }

    // One source_term call (pde-algs/source_term.h:19-51) with a point
    // source written as a lambda of the cell's primitive state:
    //   kind 0: the constant flux_t c
    //   kind 1: body force per unit volume f = c[2..4]: (0, f.u, f)
    //   kind 2: acceleration g = c[2..4]: rho (0, g.u, g), rho = p/(R T)
    // rhs (AoS5 with ghosts) is incremented in place.
    int spade_ref_source_term(int kind, const int* ints, const double* reals, const double* c,
                              const double* prims, double* rhs)
    {
        try
        {
            const problem_t pb = make_problem(ints, reals);
            const double c0 = c[0], c1 = c[1], fx = c[2], fy = c[3], fz = c[4];
            const double rgas = pb.rgas;
            with_grid(pb, [&](auto& grid, auto& group)
            {
                spade::ctrs::array<int, 3> nexch(pb.ng, pb.ng, pb.ng);
                spade::grid::grid_array q (grid, prim_t(0.0), nexch, spade::device::cpu);
                spade::grid::grid_array r (grid, flux_t(0.0), nexch, spade::device::cpu);
                copy_in(q, prims);
                copy_in(r, rhs);
                if (kind == 0)
                {
                    spade::pde_algs::source_term(q, r, [=](const prim_t&)
                    {
                        flux_t s;
                        s[0] = c0; s[1] = c1; s[2] = fx; s[3] = fy; s[4] = fz;
                        return s;
                    });
                }
                else if (kind == 1)
                {
                    spade::pde_algs::source_term(q, r, [=](const prim_t& w)
                    {
                        flux_t s;
                        s[0] = 0.0;
                        s[1] = fx*w.u() + fy*w.v() + fz*w.w();
                        s[2] = fx; s[3] = fy; s[4] = fz;
                        return s;
                    });
                }
                else
                {
                    spade::pde_algs::source_term(q, r, [=](const prim_t& w)
                    {
                        const double rho = w.p()/(rgas*w.T());
                        flux_t s;
                        s[0] = 0.0;
                        s[1] = rho*(fx*w.u() + fy*w.v() + fz*w.w());
                        s[2] = rho*fx; s[3] = rho*fy; s[4] = rho*fz;
                        return s;
                    });
                }
                copy_out(r, rhs);
            });
        }
        catch (const std::exception& e) { std::fprintf(stderr, "spade_ref_source_term: %s\n", e.what()); return -1; }
        return 0;
    }

    // Ghost fill through the reference's block exchange (periodic flags per
    // direction) followed, when wall_y != 0, by boundary_fill on y-min and
    // y-max with the isothermal no-slip wall.
    int spade_ref_fill_ghosts(const int* ints, const double* reals, double* prims)
    {
        try
        {
            const problem_t pb = make_problem(ints, reals);
            with_grid(pb, [&](auto& grid, auto& group)
            {
                spade::ctrs::array<int, 3> nexch(pb.ng, pb.ng, pb.ng);
                spade::grid::grid_array q (grid, prim_t(0.0), nexch, spade::device::cpu);
                copy_in(q, prims);
                spade::ctrs::array<bool, 3> periodic(pb.periodic[0] != 0, pb.periodic[1] != 0, pb.periodic[2] != 0);
                auto handle = spade::grid::make_exchange(q, periodic);
                apply_bc(pb, q, handle, group);
                copy_out(q, prims);
            });
        }
        catch (const std::exception& e) { std::fprintf(stderr, "spade_ref_fill_ghosts: %s\n", e.what()); return -1; }
        return 0;
    }

    // nsteps of SSPRK3 through integrator_t with the conservative-variable
    // state transform, the same calc_rhs/bc structure as the reference's
    // drivers (rhs = 0; flux_div(q, rhs, scheme); bc = exchange [+ walls]).
    // `prims` holds the initial state on entry (ghosts are refreshed here
    // first) and the final state on exit.  ke_hist[n] is the volume-averaged
    // kinetic energy after step n (ke_hist[0] = initial).
    int spade_ref_ssprk3(int scheme, const int* ints, const double* reals, double dt, int nsteps,
                         double* prims, double* ke_hist)
    {
        try
        {
            const problem_t pb = make_problem(ints, reals);
            with_grid(pb, [&](auto& grid, auto& group)
            {
                spade::ctrs::array<int, 3> nexch(pb.ng, pb.ng, pb.ng);
                spade::grid::grid_array q  (grid, prim_t(0.0), nexch, spade::device::cpu);
                spade::grid::grid_array rhs(grid, flux_t(0.0), nexch, spade::device::cpu);
                copy_in(q, prims);
                spade::ctrs::array<bool, 3> periodic(pb.periodic[0] != 0, pb.periodic[1] != 0, pb.periodic[2] != 0);
                auto handle = spade::grid::make_exchange(q, periodic);
                apply_bc(pb, q, handle, group);
                gas_t air(pb.gamma, pb.rgas);
                with_flux(pb, scheme, [&](const auto& flx)
                {
                    auto bc = [&](auto& sol, const auto&) { apply_bc(pb, sol, handle, group); };
                    auto calc_rhs = [&](auto& rhs_in, const auto& sol, const auto&)
                    {
                        rhs_in = real_t(0.0);
                        spade::pde_algs::flux_div(sol, rhs_in, flx);
                    };
                    cons_t transform_state;
                    spade::fluid_state::state_transform_t trans(transform_state, air);
                    spade::time_integration::time_axis_t axis(real_t(0.0), dt);
                    spade::time_integration::ssprk3_t alg;
                    spade::time_integration::integrator_data_t data(q, rhs, alg);
                    spade::time_integration::integrator_t time_int(axis, alg, data, calc_rhs, bc, trans);
                    ke_hist[0] = kinetic_energy(pb, time_int.solution());
                    for (int n = 0; n < nsteps; ++n)
                    {
                        time_int.advance();
                        ke_hist[n+1] = kinetic_energy(pb, time_int.solution());
                    }
                    copy_out(time_int.solution(), prims);
                });
            });
        }
        catch (const std::exception& e) { std::fprintf(stderr, "spade_ref_ssprk3: %s\n", e.what()); return -1; }
        return 0;
    }

    // AMR coarse/fine exchange through the reference's current API: an
    // amr_blocks_t grid built unrefined, refined in place pass by pass with
    // cartesian_grid_t::refine_blocks (grid/cartesian_grid.h:331-367; the
    // factor-2 constraint refines neighbours as needed), then make_exchange
    // and one exchange (grid/make_exchange.h:98-421).
    //   ints: nb[3], nc[3], ng, periodic[3], npass, then per pass its block
    //         count and the global block indices refined in it
    //   bounds: 6 doubles
    // The interior is filled with p = 3 + x, T = 1 + y^2, u = z, v = x*y,
    // w = 2 at cell centres (exact in binary floating point for power-of-two
    // geometry), ghosts start at 0.  Outputs: the array before and after the
    // exchange (cap doubles each), per block its box (6 doubles) and level,
    // and the exchange plan the reference built: one record of 18 ints per
    // transaction, injections first, each list in the reference's order:
    //   kind (0 injection, 1 interpolation), source block, dest block,
    //   source box min (3), dest box min (3), dest box max (3),
    //   i_coeff (3), i_incr (3).
    int spade_ref_amr_exchange(const int* ints, const double* bounds, long long cap, double* before, double* after,
                               int* nblk_out, double* boxes, int* levels, int box_cap,
                               int* plan, int plan_cap, int* nplan_out, int* ninject_out)
    {
        try
        {
            const int nb[3] = {ints[0], ints[1], ints[2]};
            const int nc[3] = {ints[3], ints[4], ints[5]};
            const int ng = ints[6];
            spade::ctrs::array<bool, 3> per(ints[7] != 0, ints[8] != 0, ints[9] != 0);
            int argc = 0;
            char** argv = nullptr;
            spade::parallel::compute_env_t env(&argc, &argv, {0});
            int rc = 0;
            env.exec([&](spade::parallel::pool_t& group)
            {
                spade::bound_box_t<real_t, 3> bbx;
                for (int d = 0; d < 3; ++d) { bbx.min(d) = bounds[2*d]; bbx.max(d) = bounds[2*d + 1]; }
                spade::coords::identity<real_t> coords;
                spade::ctrs::array<int, 3> num_blocks(nb[0], nb[1], nb[2]), cells(nc[0], nc[1], nc[2]);
                spade::amr::amr_blocks_t blocks(num_blocks, bbx);
                spade::grid::cartesian_grid_t grid(cells, blocks, coords, group);
                const int npass = ints[10];
                int pos = 11;
                for (int pss = 0; pss < npass; ++pss)
                {
                    const int cnt = ints[pos++];
                    std::vector<std::size_t> list;
                    for (int i = 0; i < cnt; ++i) list.push_back(std::size_t(ints[pos++]));
                    grid.refine_blocks(list, per);
                }
                spade::ctrs::array<int, 3> nexch(ng, ng, ng);
                spade::grid::grid_array q(grid, prim_t(0.0), nexch, spade::device::cpu);
                auto handle = spade::grid::make_exchange(q, per);
                using point_t = typename utils_grid_point<decltype(grid)>::type;
                spade::algs::fill_array(q, [](const point_t& x)
                {
                    prim_t o;
                    o.p() = 3.0 + x[0];
                    o.T() = 1.0 + x[1]*x[1];
                    o.u() = x[2];
                    o.v() = x[0]*x[1];
                    o.w() = 2.0;
                    return o;
                }, spade::grid::exclude_exchanges);
                const int nblk = int(grid.get_num_global_blocks());
                *nblk_out = nblk;
                if ((long long)q.data.size() > cap || nblk > box_cap) { rc = -2; return; }
                copy_out(q, before);
                handle.exchange(q, group);
                copy_out(q, after);
                for (int lb = 0; lb < nblk; ++lb)
                {
                    const auto b = grid.get_bounding_box(spade::utils::tag[spade::partition::global](std::size_t(lb)));
                    for (int d = 0; d < 3; ++d) { boxes[6*lb + 2*d] = b.min(d); boxes[6*lb + 2*d + 1] = b.max(d); }
                    levels[lb] = grid.get_blocks().get_amr_node(lb).level[0];
                }
                using namespace spade::sym::literals;
                const auto& inj = handle.config.send_data[0_c];
                const auto& itp = handle.config.send_data[1_c];
                *ninject_out = int(inj.size());
                *nplan_out = int(inj.size() + itp.size());
                if (*nplan_out > plan_cap) { rc = -3; return; }
                int* r = plan;
                for (std::size_t i = 0; i < inj.size(); ++i, r += 18)
                {
                    const auto& t = inj[i];
                    const int rec[18] = {0, t.source.min(3), t.dest.min(3),
                                         t.source.min(0), t.source.min(1), t.source.min(2),
                                         t.dest.min(0), t.dest.min(1), t.dest.min(2),
                                         t.dest.max(0), t.dest.max(1), t.dest.max(2), 0, 0, 0, 0, 0, 0};
                    std::memcpy(r, rec, sizeof(rec));
                }
                for (std::size_t i = 0; i < itp.size(); ++i, r += 18)
                {
                    const auto& t = itp[i];
                    const auto& pt = t.patches;
                    const int rec[18] = {1, pt.source.min(3), pt.dest.min(3),
                                         pt.source.min(0), pt.source.min(1), pt.source.min(2),
                                         pt.dest.min(0), pt.dest.min(1), pt.dest.min(2),
                                         pt.dest.max(0), pt.dest.max(1), pt.dest.max(2),
                                         t.i_coeff[0], t.i_coeff[1], t.i_coeff[2], t.i_incr[0], t.i_incr[1], t.i_incr[2]};
                    std::memcpy(r, rec, sizeof(rec));
                }
            });
            return rc;
        }
        catch (const std::exception& e) { std::fprintf(stderr, "spade_ref_amr_exchange: %s\n", e.what()); return -1; }
    }

    // flux_div on a refined layout: the grid of spade_ref_amr_exchange (same
    // `ints` and bounds = reals[0..5]), the given state copied in (ghosts
    // included, as the exchange left them) and one flux_div of `scheme` in
    // overwrite mode (pde-algs/flux-div/flux_div_basic.h:17-76; each block
    // takes 1/dx from its own bounding box, grid/grid_geometry.h:85-89).
    //   reals: the problem layout of make_problem (bounds, gas, viscosity,
    //          dissipation and sensor constants)
    // `prims` and `rhs` hold cap doubles; nblk_out receives the block count.
    int spade_ref_amr_flux_div(int scheme, const int* ints, const double* reals, long long cap,
                               const double* prims, double* rhs, int* nblk_out)
    {
        try
        {
            const problem_t pb = make_problem_amr(ints, reals);
            int rc = 0;
            with_amr_grid(pb, ints, [&](auto& grid, auto&, auto&)
            {
                spade::ctrs::array<int, 3> nexch(pb.ng, pb.ng, pb.ng);
                spade::grid::grid_array q(grid, prim_t(0.0), nexch, spade::device::cpu);
                spade::grid::grid_array r(grid, flux_t(0.0), nexch, spade::device::cpu);
                *nblk_out = int(grid.get_num_global_blocks());
                if ((long long)q.data.size() > cap) { rc = -2; return; }
                copy_in(q, prims);
                with_flux(pb, scheme, [&](const auto& flx)
                {
                    spade::pde_algs::flux_div(q, r, flx, spade::algs::make_traits(spade::pde_algs::basic, spade::pde_algs::overwrite));
                });
                copy_out(r, rhs);
            });
            return rc;
        }
        catch (const std::exception& e) { std::fprintf(stderr, "spade_ref_amr_flux_div: %s\n", e.what()); return -1; }
    }

    // nsteps of SSPRK3 on a refined layout (the grid of spade_ref_amr_flux_div)
    // through integrator_t with the conservative-variable state transform; the
    // boundary condition is the layout's exchange (make_exchange with the
    // periodic flags; ghost cells it does not write keep their values), then
    // with wall_y the y walls' boundary_fill as in spade_ref_amr_fill.
    // `prims` (cap doubles) holds the initial state on entry and the final
    // state on exit; the exchange runs once before the first step.
    // The boundary condition of a refined layout: the exchange, then (wall_y)
    // the reference's boundary_fill of the y faces with the isothermal wall
    // kernel at reals[13] (grid/boundary_fill.h:31-133), as apply_bc pairs them.
    // `prims` (cap doubles) is filled in place.
    int spade_ref_amr_fill(const int* ints, const double* reals, int wall_y, long long cap, double* prims)
    {
        try
        {
            const problem_t pb = make_problem_amr(ints, reals);
            int rc = 0;
            with_amr_grid(pb, ints, [&](auto& grid, auto& group, auto& per)
            {
                spade::ctrs::array<int, 3> nexch(pb.ng, pb.ng, pb.ng);
                spade::grid::grid_array q(grid, prim_t(0.0), nexch, spade::device::cpu);
                if ((long long)q.data.size() > cap) { rc = -2; return; }
                copy_in(q, prims);
                auto handle = spade::grid::make_exchange(q, per);
                handle.exchange(q, group);
                if (wall_y)
                {
                    isothermal_wall_t wall{pb.t_wall};
                    spade::algs::boundary_fill(q, spade::boundary::ymin, wall);
                    spade::algs::boundary_fill(q, spade::boundary::ymax, wall);
                }
                copy_out(q, prims);
            });
            return rc;
        }
        catch (const std::exception& e) { std::fprintf(stderr, "spade_ref_amr_fill: %s\n", e.what()); return -1; }
    }

    int spade_ref_amr_ssprk3(int scheme, const int* ints, const double* reals, double dt, int nsteps, long long cap,
                             double* prims, int wall_y)
    {
        try
        {
            const problem_t pb = make_problem_amr(ints, reals);
            int rc = 0;
            with_amr_grid(pb, ints, [&](auto& grid, auto& group, auto& per)
            {
                spade::ctrs::array<int, 3> nexch(pb.ng, pb.ng, pb.ng);
                spade::grid::grid_array q  (grid, prim_t(0.0), nexch, spade::device::cpu);
                spade::grid::grid_array rhs(grid, flux_t(0.0), nexch, spade::device::cpu);
                if ((long long)q.data.size() > cap) { rc = -2; return; }
                copy_in(q, prims);
                auto handle = spade::grid::make_exchange(q, per);
                isothermal_wall_t wall{pb.t_wall};
                auto fill = [&](auto& sol)
                {
                    handle.exchange(sol, group);
                    if (wall_y)
                    {
                        spade::algs::boundary_fill(sol, spade::boundary::ymin, wall);
                        spade::algs::boundary_fill(sol, spade::boundary::ymax, wall);
                    }
                };
                fill(q);
                gas_t air(pb.gamma, pb.rgas);
                with_flux(pb, scheme, [&](const auto& flx)
                {
                    auto bc = [&](auto& sol, const auto&) { fill(sol); };
                    auto calc_rhs = [&](auto& rhs_in, const auto& sol, const auto&)
                    {
                        rhs_in = real_t(0.0);
                        spade::pde_algs::flux_div(sol, rhs_in, flx);
                    };
                    cons_t transform_state;
                    spade::fluid_state::state_transform_t trans(transform_state, air);
                    spade::time_integration::time_axis_t axis(real_t(0.0), dt);
                    spade::time_integration::ssprk3_t alg;
                    spade::time_integration::integrator_data_t data(q, rhs, alg);
                    spade::time_integration::integrator_t time_int(axis, alg, data, calc_rhs, bc, trans);
                    for (int n = 0; n < nsteps; ++n) time_int.advance();
                    copy_out(time_int.solution(), prims);
                });
            });
            return rc;
        }
        catch (const std::exception& e) { std::fprintf(stderr, "spade_ref_amr_ssprk3: %s\n", e.what()); return -1; }
    }
}
