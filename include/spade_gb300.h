/*
 * spade_gb300.h — drop-in GB300 path for spade::pde_algs::flux_div.
 *
 * Include after "spade.h".  Passing the `gb300` algorithm trait selects the
 * GB300 kernels through overload resolution; nothing else in the caller
 * changes:
 *
 *     #include "spade.h"
 *     #include "spade_gb300.h"
 *     ...
 *     spade::pde_algs::flux_div(prims, rhs, spade::omni::compose(tscheme, vscheme),
 *                               spade::algs::make_traits(spade::pde_algs::gb300));
 *
 * The overload below replaces flux_div (pde-algs/flux-div/flux_div.h:16-56):
 * it carries the reference's constraints plus "the traits select gb300", so
 * it is the more constrained candidate.  It lowers the composed functor type
 * at compile time into a gbns_scheme_desc (static_assert on anything the
 * kernels do not implement: there is no CPU fallback), the grid_array into a
 * gbns_grid_desc, calls gbns_flux_div on the arrays' device storage
 * (device::gpu) or gbns_flux_div_host on their host storage (device::cpu,
 * staged through the GPU), and then synchronises and throws
 * except::sp_exception on failure, like the reference's dispatch
 * (dispatch/execute.h:84-96).
 *
 * Lowered functors: convective::cent_keep_scheme_t<gas, 2|4|6|8>,
 * convective::totani_lr, convective::fweno_t<gas, smooth>,
 * spade::gb300::weno5_t<gas> (5th-order WENO, no reference counterpart),
 * convective::pressure_diss_lr<gas, state_sensor::const_sensor_t | ducros_t>,
 * convective::hybrid_scheme_t<cent_keep_scheme_t<gas, 2|4>, fweno_t, const_sensor_t | ducros_t, full_flux | diss_flux>,
 * viscous::visc_lr<viscous_laws::constant_viscosity_t | power_law_t | spade::gb300::sutherland_t, gas>,
 * and omni::compose of one of each (convective, dissipation, viscous).
 * Coordinates: coords::identity, and coords::diagonal_coords(identity_1D, y, identity_1D)
 * with y = spade::gb300::tanh_stretch_1D (beta) or coords::integrated_tanh_1D.
 *
 * Exchange on refined (AMR) block layouts: spade::gb300::exchange_plan_t built
 * from the reference's own exchange handle (grid::make_exchange) runs its
 * injections and coarse/fine interpolations on the GPU (gbns_exchange_plan_*);
 * spade::gb300::lower_exchange gives the plan as gbns_patch records.
 *
 * source_term: spade::gb300::const_source_t / body_force_t / body_accel_t
 * passed to spade::pde_algs::source_term run on the GPU (gbns_source_term).
 *
 * boundary_flux: the reference's call with the gb300 traits appended,
 *     spade::pde_algs::boundary_flux(prims, rhs, apply_to_boundary, flux_func,
 *                                    spade::algs::make_traits(spade::pde_algs::gb300));
 * runs gbns_boundary_flux (the overload below is more specialised than the
 * reference's variadic template, pde-algs/boundary_flux.h:10-20).
 *
 * Ghost fill and time integration: spade::gb300::fill_ghosts(q, periodic,
 * walls, wall) stands for the exchange + boundary_fill pair the reference's
 * drivers call (one launch, gbns_fill_ghosts), with the wall kernel
 * spade::gb300::isothermal_wall_t or slip_wall_t (also usable as the
 * reference's own boundary_fill kernel); spade::gb300::ssprk3_integrator_t
 * is integrator_t with ssprk3_t, flux_div of the lowered functor and that
 * ghost fill, fused (advance() is gbns_ssprk3_step).
 *
 * Define GBNS_DROPIN_HOOK before including to route the lowered call to a
 * user function `int GBNS_DROPIN_HOOK(const gbns_grid_desc*, const
 * gbns_scheme_desc*, const double*, double*, int)` instead of the library
 * (used by the host-only tests of the lowering); GBNS_DROPIN_SOURCE_HOOK,
 * `int (const gbns_grid_desc*, const gbns_source_desc*, const double*, double*)`,
 * does the same for source_term, and GBNS_DROPIN_BFLUX_HOOK, `int (const
 * gbns_grid_desc*, const gbns_scheme_desc*, const double*, double*, const int*)`,
 * for boundary_flux, and GBNS_DROPIN_BC_HOOK, `int (const gbns_grid_desc*,
 * const gbns_bc_desc*, const gbns_scheme_desc*, double*, double dt)`, for the
 * ghost fill (scheme NULL) and the SSPRK3 integrator's step.
 */
#pragma once

#include <cmath>
#include <string>
#include <type_traits>
#include <vector>
#include <cuda_runtime_api.h>

#include "gbns.h"

namespace spade::pde_algs
{
    // flux_div algorithm tag (pde-algs/flux-div/tags.h:5-33)
    static struct tgb300_t : public fdiv_alg_base_t {} gb300;
}

namespace spade::gb300
{
    // ------------------------------------------------------------------
    // Functors and coordinate maps of the GB300 path with no counterpart in
    // the reference; they compose with the reference's own types
    // (omni::compose, coords::diagonal_coords) and lower like them.
    // ------------------------------------------------------------------

    // 5th-order WENO-JS with the Rusanov flux splitting of fweno_t
    // (navier-stokes/convective.h:335-497 is the 3rd-order model): six cells
    // per face, linear weights 0.1/0.6/0.3, epsilon 1e-16.  Evaluated by the
    // GB300 kernels only (flux_div with the gb300 traits); calling it on the
    // CPU throws.
    template <typename gas_t>
    struct weno5_t
    {
        using float_t     = typename gas_t::value_type;
        using output_type = fluid_state::flux_t<float_t>;
        using m_info_type = omni::info_list_t<omni::info::value, omni::info::metric>;
        using g_info_type = typename gas_t::info_type;
        using info_type   = omni::info_union<m_info_type, g_info_type>;
        using omni_type   = omni::stencil_t<
                grid::face_centered,
                omni::elem_t<omni::offset_t<-5, 0, 0>, info_type>,
                omni::elem_t<omni::offset_t<-3, 0, 0>, info_type>,
                omni::elem_t<omni::offset_t<-1, 0, 0>, info_type>,
                omni::elem_t<omni::offset_t< 1, 0, 0>, info_type>,
                omni::elem_t<omni::offset_t< 3, 0, 0>, info_type>,
                omni::elem_t<omni::offset_t< 5, 0, 0>, info_type>
            >;
        const gas_t gas;
        weno5_t(const gas_t& gas_in) : gas{gas_in} {}
        output_type operator()(const auto&) const
        {
            throw except::sp_exception("gb300::weno5_t is evaluated by the GB300 kernels: use flux_div with the gb300 traits");
        }
    };

    // Sutherland's law mu = mu_ref (T/T_ref)^(3/2) (T_ref + S)/(T + S) at the
    // face state, beta = -2/3 mu, conductivity mu/Pr (the constant law's
    // conventions, navier-stokes/viscous_laws.h:62-100).  State-dependent, in
    // the form of power_law_t (viscous_laws.h:102-135).
    template <typename dtype>
    struct sutherland_t
    : public viscous_laws::visc_law_interface_t<sutherland_t<dtype>, omni::info_list_t<omni::info::value>>
    {
        using value_type = dtype;
        using base_t = viscous_laws::visc_law_interface_t<sutherland_t<dtype>, omni::info_list_t<omni::info::value>>;
        using base_t::get_visc;
        using base_t::get_beta;
        using base_t::get_diffuse;
        using base_t::info_type;
        dtype mu_ref, T_ref, S, prandtl;
        sutherland_t(const dtype& mu_ref_in, const dtype& T_ref_in, const dtype& S_in, const dtype& prandtl_in)
        : mu_ref{mu_ref_in}, T_ref{T_ref_in}, S{S_in}, prandtl{prandtl_in} {}
        template <fluid_state::is_state_type state_t> dtype get_visc(const state_t& q) const
        {
            const dtype x = q.T()/T_ref;
            return (mu_ref*(x*std::sqrt(x)))*((T_ref + S)/(q.T() + S));
        }
        template <fluid_state::is_state_type state_t> dtype get_beta(const state_t& q) const
        {
            return this->get_visc(q)*dtype(-2.0/3.0);
        }
        template <fluid_state::is_state_type state_t> dtype get_diffuse(const state_t& q) const
        {
            return this->get_visc(q)/prandtl;
        }
    };

    // Wall-normal tanh stretching y = tanh(beta eta)/tanh(beta) for eta in the
    // grid's y bounds, usable as the y map of coords::diagonal_coords
    // (core/coord_system.h:65-90; the reference parametrises its own tanh map,
    // integrated_tanh_1D, by y0, y1, inflation and rate instead).
    template <typename dtype>
    struct tanh_stretch_1D
    {
        typedef dtype coord_type;
        dtype beta = dtype(1.0);
        tanh_stretch_1D() {}
        tanh_stretch_1D(const dtype& beta_in) : beta{beta_in} {}
        dtype map(const dtype& eta) const { return std::tanh(beta*eta)/std::tanh(beta); }
        dtype coord_deriv(const dtype& eta) const
        {
            const dtype th = std::tanh(beta*eta);
            return beta*(dtype(1.0) - th*th)/std::tanh(beta);
        }
    };

    // flux arithmetic precision trait
    struct flux_precision_base_t
    {
        constexpr static auto trait_label() { using namespace sym::literals; return "flux_precision"_sym; }
    };
    static struct tfp64_t      : public flux_precision_base_t { static constexpr int value = GBNS_PREC_FP64; }      fp64;
    static struct tfp64_fma_t  : public flux_precision_base_t { static constexpr int value = GBNS_PREC_FP64_FMA; }  fp64_fma;
    static struct tfp32_flux_t : public flux_precision_base_t { static constexpr int value = GBNS_PREC_FP32_FLUX; } fp32_flux;

    namespace detail
    {
        template <typename T> struct always_false : std::false_type {};

        template <typename gas_t>
        inline void set_gas(gbns_scheme_desc& s, const gas_t& gas, bool& have_gas)
        {
            static_assert(std::is_same_v<gas_t, fluid_state::ideal_gas_t<double>>, "the GB300 path lowers ideal_gas_t<double>");
            if (have_gas && (s.gas.gamma != gas.gamma || s.gas.R != gas.R))
                throw except::sp_exception("gb300 flux_div: all functors of a composite must share one gas");
            s.gas.gamma = gas.gamma;
            s.gas.R = gas.R;
            have_gas = true;
        }

        // slot: 0 convective, 1 dissipation, 2 viscous
        template <typename T> struct lower
        {
            static_assert(always_false<T>::value, "gb300 flux_div: this flux functor has no GB300 kernel");
        };

        template <typename gas_t, const int order>
        struct lower<convective::cent_keep_scheme_t<gas_t, order>>
        {
            static constexpr int slot = 0;
            static void apply(gbns_scheme_desc& s, const convective::cent_keep_scheme_t<gas_t, order>& f, bool& g)
            {
                static_assert(order == 2 || order == 4 || order == 6 || order == 8, "cent_keep order 2, 4, 6 or 8");
                s.convective = GBNS_CONV_CENT_KEEP;
                s.order = order;
                set_gas(s, f.gas, g);
            }
        };

        template <typename gas_t>
        struct lower<weno5_t<gas_t>>
        {
            static constexpr int slot = 0;
            static void apply(gbns_scheme_desc& s, const weno5_t<gas_t>& f, bool& g)
            {
                s.convective = GBNS_CONV_WENO5;
                set_gas(s, f.gas, g);
            }
        };

        template <typename gas_t>
        struct lower<convective::totani_lr<gas_t>>
        {
            static constexpr int slot = 0;
            static void apply(gbns_scheme_desc& s, const convective::totani_lr<gas_t>& f, bool& g)
            {
                s.convective = GBNS_CONV_TOTANI;
                set_gas(s, f.gas, g);
            }
        };

        template <typename gas_t, const convective::weno_smooth_indicator sm>
        struct lower<convective::fweno_t<gas_t, sm>>
        {
            static constexpr int slot = 0;
            static void apply(gbns_scheme_desc& s, const convective::fweno_t<gas_t, sm>& f, bool& g)
            {
                s.convective = GBNS_CONV_FWENO;
                s.weno_smooth = (sm == convective::enable_smooth) ? 1 : 0;
                set_gas(s, f.gas, g);
            }
        };

        // blender of hybrid_scheme_t: kind and parameter
        template <typename T> struct blender
        {
            static_assert(always_false<T>::value, "gb300 flux_div: hybrid blender must be const_sensor_t or ducros_t");
        };
        template <typename ft> struct blender<state_sensor::const_sensor_t<ft>>
        {
            static constexpr int kind = GBNS_SENSOR_CONST;
            static double param(const state_sensor::const_sensor_t<ft>& b) { return b.alpha; }
        };
        template <typename ft> struct blender<state_sensor::ducros_t<ft>>
        {
            static constexpr int kind = GBNS_SENSOR_DUCROS;
            static double param(const state_sensor::ducros_t<ft>& b) { return b.epsilon; }
        };

        // hybrid_scheme_t<cent_keep<2|4>, fweno_t, blender, tag> (navier-stokes/hybrid_scheme.h:14-47)
        template <typename gas_t, const int order, const convective::weno_smooth_indicator sm, typename blend_t, typename tag_t>
        struct lower<convective::hybrid_scheme_t<convective::cent_keep_scheme_t<gas_t, order>, convective::fweno_t<gas_t, sm>,
                                                 blend_t, tag_t>>
        {
            static constexpr int slot = 0;
            template <typename hyb_t>
            static void apply(gbns_scheme_desc& s, const hyb_t& f, bool& g)
            {
                static_assert(order == 2 || order == 4, "hybrid_scheme_t is lowered with cent_keep order 2 or 4");
                s.convective = GBNS_CONV_HYBRID;
                s.order = order;
                s.weno_smooth = (sm == convective::enable_smooth) ? 1 : 0;
                s.hybrid_flux = tag_t::value ? GBNS_HYBRID_FULL_FLUX : GBNS_HYBRID_DISS_FLUX;
                s.hybrid_sensor = blender<blend_t>::kind;
                s.hybrid_param = blender<blend_t>::param(f.blender);
                set_gas(s, f.scheme0.gas, g);
                set_gas(s, f.scheme1.gas, g);
            }
        };

        template <typename gas_t, typename ft>
        struct lower<convective::pressure_diss_lr<gas_t, state_sensor::const_sensor_t<ft>>>
        {
            static constexpr int slot = 1;
            static void apply(gbns_scheme_desc& s, const convective::pressure_diss_lr<gas_t, state_sensor::const_sensor_t<ft>>& f, bool& g)
            {
                s.dissipation = GBNS_DISS_PRESSURE;
                s.sensor = GBNS_SENSOR_CONST;
                s.sensor_alpha = f.scale.alpha;
                s.eps_p = f.eps_p;
                s.eps_T = f.eps_T;
                set_gas(s, f.gas, g);
            }
        };

        template <typename gas_t, typename ft>
        struct lower<convective::pressure_diss_lr<gas_t, state_sensor::ducros_t<ft>>>
        {
            static constexpr int slot = 1;
            static void apply(gbns_scheme_desc& s, const convective::pressure_diss_lr<gas_t, state_sensor::ducros_t<ft>>& f, bool& g)
            {
                s.dissipation = GBNS_DISS_PRESSURE;
                s.sensor = GBNS_SENSOR_DUCROS;
                s.sensor_alpha = f.scale.epsilon;   // ducros_t epsilon
                s.eps_p = f.eps_p;
                s.eps_T = f.eps_T;
                set_gas(s, f.gas, g);
            }
        };

        template <typename dt, typename gas_t>
        struct lower<viscous::visc_lr<viscous_laws::constant_viscosity_t<dt>, gas_t>>
        {
            static constexpr int slot = 2;
            static void apply(gbns_scheme_desc& s, const viscous::visc_lr<viscous_laws::constant_viscosity_t<dt>, gas_t>& f, bool& g)
            {
                s.viscous = GBNS_VISC_LR;
                s.visc_law = GBNS_LAW_CONSTANT;
                s.mu = f.vlaw.visc;
                s.prandtl = 1.0/f.vlaw.prandtl_inv;
                s.prandtl_inv = f.vlaw.prandtl_inv;   // the law stores 1/Pr (viscous_laws.h:190-192)
                set_gas(s, f.gas, g);
            }
        };

        template <typename dt, typename gas_t>
        struct lower<viscous::visc_lr<viscous_laws::power_law_t<dt>, gas_t>>
        {
            static constexpr int slot = 2;
            static void apply(gbns_scheme_desc& s, const viscous::visc_lr<viscous_laws::power_law_t<dt>, gas_t>& f, bool& g)
            {
                s.viscous = GBNS_VISC_LR;
                s.visc_law = GBNS_LAW_POWER;
                s.mu = f.vlaw.mu_ref;
                s.T_ref = f.vlaw.T_ref;
                s.power = f.vlaw.power;
                s.prandtl = f.vlaw.prandtl;
                set_gas(s, f.gas, g);
            }
        };

        template <typename dt, typename gas_t>
        struct lower<viscous::visc_lr<sutherland_t<dt>, gas_t>>
        {
            static constexpr int slot = 2;
            static void apply(gbns_scheme_desc& s, const viscous::visc_lr<sutherland_t<dt>, gas_t>& f, bool& g)
            {
                s.viscous = GBNS_VISC_LR;
                s.visc_law = GBNS_LAW_SUTHERLAND;
                s.mu = f.vlaw.mu_ref;
                s.T_ref = f.vlaw.T_ref;
                s.S = f.vlaw.S;
                s.power = 1.5;
                s.prandtl = f.vlaw.prandtl;
                set_gas(s, f.gas, g);
            }
        };

        // coordinate systems: identity, or diagonal_coords with identity x
        // and z and a tanh-stretched y (gbns_grid_desc coords, coord_param)
        template <typename T> struct lower_coords
        {
            static_assert(always_false<T>::value,
                          "the GB300 drop-in lowers coords::identity and diagonal_coords(identity_1D, "
                          "tanh_stretch_1D | integrated_tanh_1D, identity_1D)");
        };
        template <> struct lower_coords<coords::identity<double>>
        {
            static void apply(gbns_grid_desc& g, const coords::identity<double>&) { g.coords = GBNS_COORDS_IDENTITY; }
        };
        template <> struct lower_coords<coords::diagonal_coords<coords::identity_1D<double>, tanh_stretch_1D<double>,
                                                                coords::identity_1D<double>>>
        {
            template <typename c_t>
            static void apply(gbns_grid_desc& g, const c_t& c)
            {
                g.coords = GBNS_COORDS_TANH_Y;
                g.coord_param[0] = c.ycoord.beta;
            }
        };
        template <> struct lower_coords<coords::diagonal_coords<coords::identity_1D<double>, coords::integrated_tanh_1D<double>,
                                                                coords::identity_1D<double>>>
        {
            // integrated_tanh_1D keeps (eta1 = y0, eta0 = y1, deta, alpha0 =
            // rate/deta, beta0 = alpha0 (inflation deta - eta0), ...)
            // (core/coord_system.h:107-125); its constructor arguments are
            // recovered from them (rate and inflation to rounding)
            template <typename c_t>
            static void apply(gbns_grid_desc& g, const c_t& c)
            {
                const auto& y = c.ycoord;
                g.coords = GBNS_COORDS_INTEGRATED_TANH_Y;
                g.coord_param[0] = y.eta1;
                g.coord_param[1] = y.eta0;
                g.coord_param[2] = (y.beta0/y.alpha0 + y.eta0)/y.deta;
                g.coord_param[3] = y.alpha0*y.deta;
            }
        };

        template <typename k0_t, typename... ks_t>
        struct lower<omni::composite_kernel_t<k0_t, ks_t...>>
        {
            static constexpr int slot = -1;
            static void apply(gbns_scheme_desc& s, const omni::composite_kernel_t<k0_t, ks_t...>& f, bool& g, int* used)
            {
                static_assert(lower<k0_t>::slot >= 0, "nested composites are not lowered");
                if (used[lower<k0_t>::slot]) throw except::sp_exception("gb300 flux_div: two functors of the same kind in one composite");
                used[lower<k0_t>::slot] = 1;
                lower<k0_t>::apply(s, f.kern, g);
                if constexpr (sizeof...(ks_t) > 0)
                {
                    // compose(a, b, c) sums a + (b + c) (omni/compose.h:19-24); the
                    // kernels sum conv + (diss + visc): a three-term composite must
                    // come in that order, a two-term sum commutes exactly.
                    static_assert(sizeof...(ks_t) < 2 || lower<k0_t>::slot == 0,
                                  "three-term composites must be compose(convective, dissipation, viscous)");
                    lower<omni::composite_kernel_t<ks_t...>>::apply(s, f.next, g, used);
                }
            }
        };

        template <typename kern_t>
        struct lower<omni::composite_kernel_t<kern_t>>
        {
            static constexpr int slot = -1;
            static void apply(gbns_scheme_desc& s, const omni::composite_kernel_t<kern_t>& f, bool& g, int* used)
            {
                if (used[lower<kern_t>::slot]) throw except::sp_exception("gb300 flux_div: two functors of the same kind in one composite");
                used[lower<kern_t>::slot] = 1;
                lower<kern_t>::apply(s, f.kern, g);
            }
        };

        template <typename traits_t>
        using fdiv_tag_of = typename utils::remove_all<decltype(algs::get_trait(std::declval<const traits_t&>(),
                                                                                 std::declval<decltype(pde_algs::fdiv_alg_base_t::trait_label())>()))>::type;
    }

    // omni functor -> gbns_scheme_desc
    template <typename flux_func_t>
    gbns_scheme_desc lower_scheme(const flux_func_t& f, int precision = GBNS_PREC_FP64)
    {
        gbns_scheme_desc s{};
        s.order = 2;
        s.weno_smooth = 1;
        s.prandtl = 1.0;
        s.T_ref = 1.0;
        s.precision = precision;
        bool have_gas = false;
        int used[3] = {0, 0, 0};
        if constexpr (detail::lower<flux_func_t>::slot < 0) detail::lower<flux_func_t>::apply(s, f, have_gas, used);
        else detail::lower<flux_func_t>::apply(s, f, have_gas);
        return s;
    }

    // grid_array -> gbns_grid_desc (grid/grid_array.h:175-260, cartesian_grid.h:48-384)
    template <typename arr_t>
    gbns_grid_desc lower_grid(const arr_t& arr)
    {
        const auto& grid = arr.get_grid();
        using coord_t = typename utils::remove_all<decltype(grid.get_coord_sys())>::type;
        static_assert(std::is_same_v<typename arr_t::value_type, double>, "the GB300 path works on double arrays");
        gbns_grid_desc g{};
        const auto& blocks = grid.get_blocks();
        const auto bnd = grid.get_bounds();
        for (int d = 0; d < 3; ++d)
        {
            g.nblk[d] = blocks.num_blocks[d];
            g.ncell[d] = grid.get_num_cells(d);
            g.bounds[2*d] = bnd.min(d);
            g.bounds[2*d + 1] = bnd.max(d);
        }
        if (grid.get_num_local_blocks() != grid.get_num_global_blocks())
            throw except::sp_exception("gb300 flux_div: the grid must hold every block on this device");
        const int ng = arr.get_num_exchange(0);
        if (arr.get_num_exchange(1) != ng || arr.get_num_exchange(2) != ng)
            throw except::sp_exception("gb300 flux_div: equal ghost depth in every direction required");
        g.ng = ng;
        detail::lower_coords<coord_t>::apply(g, grid.get_coord_sys());
        return g;
    }

    namespace detail
    {
        template <typename blocks_t> struct is_refined_blocks : std::false_type {};
        template <typename val_t, typename desig_t>
        struct is_refined_blocks<amr::amr_blocks_t<val_t, desig_t>> : std::true_type {};
    }

    // A grid_array on a refined (AMR) grid -> gbns_grid_desc with
    // nblk = (blocks, 1, 1) in global block order and each block's bounding
    // box (6 doubles: min, max per direction) for gbns_flux_div_blocks; the
    // reference's flux_div takes 1/dx from that box (flux_div_basic.h:55,
    // grid/grid_geometry.h:85-89).
    template <typename arr_t>
    gbns_grid_desc lower_refined_grid(const arr_t& arr, std::vector<double>& boxes)
    {
        const auto& grid = arr.get_grid();
        using coord_t = typename utils::remove_all<decltype(grid.get_coord_sys())>::type;
        static_assert(std::is_same_v<typename arr_t::value_type, double>, "the GB300 path works on double arrays");
        if (grid.get_num_local_blocks() != grid.get_num_global_blocks())
            throw except::sp_exception("gb300 flux_div: the grid must hold every block on this device");
        const std::size_t nblk = grid.get_num_global_blocks();
        gbns_grid_desc g{};
        const auto bnd = grid.get_bounds();
        g.nblk[0] = int(nblk);
        g.nblk[1] = g.nblk[2] = 1;
        for (int d = 0; d < 3; ++d)
        {
            g.ncell[d] = grid.get_num_cells(d);
            g.bounds[2*d] = bnd.min(d);
            g.bounds[2*d + 1] = bnd.max(d);
        }
        const int ng = arr.get_num_exchange(0);
        if (arr.get_num_exchange(1) != ng || arr.get_num_exchange(2) != ng)
            throw except::sp_exception("gb300 flux_div: equal ghost depth in every direction required");
        g.ng = ng;
        detail::lower_coords<coord_t>::apply(g, grid.get_coord_sys());
        boxes.assign(6*nblk, 0.0);
        for (std::size_t lb = 0; lb < nblk; ++lb)
        {
            const auto b = grid.get_bounding_box(utils::tag[partition::global](lb));
            for (int d = 0; d < 3; ++d)
            {
                boxes[6*lb + 2*d] = b.min(d);
                boxes[6*lb + 2*d + 1] = b.max(d);
            }
        }
        return g;
    }

    template <typename traits_t>
    concept selects_gb300 = requires { typename detail::fdiv_tag_of<traits_t>; } &&
                            std::same_as<detail::fdiv_tag_of<traits_t>, pde_algs::tgb300_t>;

    template <typename traits_t>
    constexpr int precision_of()
    {
        using namespace sym::literals;
        using tr_t = typename utils::remove_all<decltype(algs::get_trait(std::declval<const traits_t&>(), "flux_precision"_sym, fp64))>::type;
        return tr_t::value;
    }
}

namespace spade::pde_algs
{
    template <
        grid::multiblock_array sol_arr_t,
        grid::multiblock_array rhs_arr_t,
        typename flux_func_t,
        typename alg_traits_t>
    requires
        grid::has_centering_type<sol_arr_t, grid::cell_centered> && gb300::selects_gb300<alg_traits_t>
    static void flux_div(
        const sol_arr_t& prims,
        rhs_arr_t& rhs,
        const flux_func_t& flux_func,
        const alg_traits_t& traits)
    {
        using namespace sym::literals;
        const auto& incr = algs::get_trait(traits, "pde_increment"_sym, increment);
        using incr_mode_t = typename utils::remove_all<decltype(incr)>::type;
        const gbns_scheme_desc s = gb300::lower_scheme(flux_func, gb300::precision_of<alg_traits_t>());
        const double* q = prims.image().base;
        double* r = rhs.image().base;
        using blocks_t = typename utils::remove_all<decltype(prims.get_grid().get_blocks())>::type;
        if constexpr (gb300::detail::is_refined_blocks<blocks_t>::value)
        {
            // refined layout: every block's own spacing (gbns_flux_div_blocks)
            std::vector<double> boxes;
            const gbns_grid_desc g = gb300::lower_refined_grid(prims, boxes);
            int rc = GBNS_OK;
#ifdef GBNS_DROPIN_HOOK
            rc = GBNS_ERR_UNSUPPORTED;
#else
            constexpr bool on_gpu = device::is_gpu<typename sol_arr_t::device_type>;
            static_assert(on_gpu == device::is_gpu<typename rhs_arr_t::device_type>,
                          "the gb300 flux_div takes prims and rhs on the same device kind");
            if constexpr (on_gpu)
            {
                rc = gbns_flux_div_blocks(&g, &s, boxes.data(), q, r, incr_mode_t::increment_mode ? 1 : 0, nullptr);
                if (rc == GBNS_OK && cudaDeviceSynchronize() != cudaSuccess) rc = GBNS_ERR_CUDA;
            }
            else
                rc = gbns_flux_div_blocks_host(&g, &s, boxes.data(), q, r, incr_mode_t::increment_mode ? 1 : 0, nullptr);
#endif
            if (rc != GBNS_OK)
            {
                char msg[512] = "refined layouts are not routed to the drop-in hook";
#ifndef GBNS_DROPIN_HOOK
                gbns_last_error(msg, sizeof(msg));
#endif
                throw except::sp_exception(std::string("gb300 flux_div failed: ") + msg);
            }
            return;
        }
        const gbns_grid_desc g = gb300::lower_grid(prims);
#ifdef GBNS_DROPIN_HOOK
        const int rc = GBNS_DROPIN_HOOK(&g, &s, q, r, incr_mode_t::increment_mode ? 1 : 0);
#else
        constexpr bool on_gpu = device::is_gpu<typename sol_arr_t::device_type>;
        static_assert(on_gpu == device::is_gpu<typename rhs_arr_t::device_type>,
                      "the gb300 flux_div takes prims and rhs on the same device kind");
        int rc = GBNS_OK;
        if constexpr (on_gpu)
        {
            rc = gbns_flux_div(&g, &s, q, r, incr_mode_t::increment_mode ? 1 : 0, nullptr);
            if (rc == GBNS_OK && cudaDeviceSynchronize() != cudaSuccess) rc = GBNS_ERR_CUDA;
        }
        else
        {
            // device::cpu arrays: staged through the GPU (synchronous)
            rc = gbns_flux_div_host(&g, &s, q, r, incr_mode_t::increment_mode ? 1 : 0, nullptr);
        }
#endif
        if (rc != GBNS_OK)
        {
            char msg[512] = "drop-in hook failed";
#ifndef GBNS_DROPIN_HOOK
            gbns_last_error(msg, sizeof(msg));
#endif
            throw except::sp_exception(std::string("gb300 flux_div failed: ") + msg);
        }
    }
}

namespace spade::gb300
{
    // The exchange plan of a reference exchange handle
    // (grid::make_exchange(q, periodic), grid/make_exchange.h:98-421): its
    // same-level injections and coarse/fine interpolations, in the
    // reference's order, as gbns_patch records for gbns_exchange_plan_create.
    // Single-rank grids (every block on this device).
    template <typename handle_t>
    std::vector<gbns_patch> lower_exchange(const handle_t& h)
    {
        using namespace sym::literals;
        const auto& inj = h.config.send_data[0_c];
        const auto& itp = h.config.send_data[1_c];
        std::vector<gbns_patch> out;
        out.reserve(inj.size() + itp.size());
        for (std::size_t i = 0; i < inj.size(); ++i)
        {
            const auto& t = inj[i];
            gbns_patch p{};
            p.kind = GBNS_PATCH_INJECT;
            p.src_block = t.source.min(3);
            p.dst_block = t.dest.min(3);
            for (int d = 0; d < 3; ++d)
            {
                p.src_lo[d] = t.source.min(d);
                p.dst_lo[d] = t.dest.min(d);
                p.dst_hi[d] = t.dest.max(d);
            }
            out.push_back(p);
        }
        for (std::size_t i = 0; i < itp.size(); ++i)
        {
            const auto& t = itp[i];
            gbns_patch p{};
            p.kind = GBNS_PATCH_INTERP;
            p.src_block = t.patches.source.min(3);
            p.dst_block = t.patches.dest.min(3);
            for (int d = 0; d < 3; ++d)
            {
                p.src_lo[d] = t.patches.source.min(d);
                p.dst_lo[d] = t.patches.dest.min(d);
                p.dst_hi[d] = t.patches.dest.max(d);
                p.i_coeff[d] = t.i_coeff[d];
                p.i_incr[d] = t.i_incr[d];
            }
            out.push_back(p);
        }
        return out;
    }

    // A reference exchange handle run on the GPU: build it once from the
    // handle and the array (blocks, cells, ghosts), then exchange(q) on
    // device::gpu grid_arrays replaces handle.exchange(q, group).
    struct exchange_plan_t
    {
        gbns_exchange_plan* plan = nullptr;
        template <typename handle_t, typename arr_t>
        exchange_plan_t(const handle_t& h, const arr_t& q)
        {
            const auto& grid = q.get_grid();
            if (grid.get_num_local_blocks() != grid.get_num_global_blocks())
                throw except::sp_exception("gb300 exchange: the grid must hold every block on this device");
            const auto patches = lower_exchange(h);
#ifndef GBNS_DROPIN_HOOK
            const int rc = gbns_exchange_plan_create(&plan, grid.get_num_cells(0), grid.get_num_cells(1), grid.get_num_cells(2),
                                                     q.get_num_exchange(0), int(grid.get_num_global_blocks()),
                                                     patches.data(), int(patches.size()), nullptr);
            if (rc != GBNS_OK)
            {
                char msg[512];
                gbns_last_error(msg, sizeof(msg));
                throw except::sp_exception(std::string("gb300 exchange plan: ") + msg);
            }
#endif
        }
        exchange_plan_t(const exchange_plan_t&) = delete;
        exchange_plan_t& operator=(const exchange_plan_t&) = delete;
        ~exchange_plan_t()
        {
#ifndef GBNS_DROPIN_HOOK
            gbns_exchange_plan_destroy(plan);
#endif
        }
        template <typename arr_t>
        void exchange(arr_t& q) const
        {
#ifndef GBNS_DROPIN_HOOK
            static_assert(device::is_gpu<typename arr_t::device_type>, "the gb300 exchange runs on device::gpu arrays");
            int rc = gbns_exchange_plan_run(plan, q.image().base, nullptr);
            if (rc == GBNS_OK && cudaDeviceSynchronize() != cudaSuccess) rc = GBNS_ERR_CUDA;
            if (rc != GBNS_OK)
            {
                char msg[512];
                gbns_last_error(msg, sizeof(msg));
                throw except::sp_exception(std::string("gb300 exchange failed: ") + msg);
            }
#endif
        }
    };

    // Point sources with a GB300 kernel (gbns_source_desc).  Passing one of
    // these instead of a lambda to spade::pde_algs::source_term selects the
    // overload below (a non-template parameter beats the reference's
    // template, pde-algs/source_term.h:19-51).
    struct const_source_t
    {
        fluid_state::flux_t<double> value;   // (rho, rhoE, rhou, rhov, rhow)
    };
    struct body_force_t                      // force per unit volume
    {
        double fx, fy, fz;
    };
    struct body_accel_t                      // force per unit mass; rho = p/(R T)
    {
        fluid_state::ideal_gas_t<double> gas;
        double gx, gy, gz;
    };

    inline gbns_source_desc lower_source(const const_source_t& f)
    {
        gbns_source_desc d{};
        d.kind = GBNS_SOURCE_CONST;
        for (int v = 0; v < 5; ++v) d.c[v] = f.value[v];
        return d;
    }
    inline gbns_source_desc lower_source(const body_force_t& f)
    {
        gbns_source_desc d{};
        d.kind = GBNS_SOURCE_BODY_FORCE;
        d.c[2] = f.fx; d.c[3] = f.fy; d.c[4] = f.fz;
        return d;
    }
    inline gbns_source_desc lower_source(const body_accel_t& f)
    {
        gbns_source_desc d{};
        d.kind = GBNS_SOURCE_BODY_ACCEL;
        d.c[2] = f.gx; d.c[3] = f.gy; d.c[4] = f.gz;
        d.gas.gamma = f.gas.gamma;
        d.gas.R = f.gas.R;
        return d;
    }

    template <typename src_t>
    concept lowered_source = std::same_as<src_t, const_source_t> || std::same_as<src_t, body_force_t> ||
                             std::same_as<src_t, body_accel_t>;
}

namespace spade::pde_algs
{
    // rhs += S(q)/jac on the interior: pde_algs::source_term
    // (pde-algs/source_term.h:19-51) on the GPU for the lowered sources.
    template <grid::multiblock_array sol_arr_t, grid::multiblock_array rhs_arr_t, gb300::lowered_source src_t>
    requires grid::has_centering_type<sol_arr_t, grid::cell_centered>
    static void source_term(const sol_arr_t& q, rhs_arr_t& rhs, const src_t& source)
    {
        const gbns_grid_desc g = gb300::lower_grid(q);
        const gbns_source_desc d = gb300::lower_source(source);
        const double* qp = q.image().base;
        double* r = rhs.image().base;
#ifdef GBNS_DROPIN_SOURCE_HOOK
        const int rc = GBNS_DROPIN_SOURCE_HOOK(&g, &d, qp, r);
#else
        static_assert(device::is_gpu<typename sol_arr_t::device_type> && device::is_gpu<typename rhs_arr_t::device_type>,
                      "the gb300 source_term runs on device::gpu arrays");
        int rc = gbns_source_term(&g, &d, qp, r, nullptr);
        if (rc == GBNS_OK && cudaDeviceSynchronize() != cudaSuccess) rc = GBNS_ERR_CUDA;
#endif
        if (rc != GBNS_OK)
        {
            char msg[512] = "drop-in hook failed";
#ifndef GBNS_DROPIN_SOURCE_HOOK
            gbns_last_error(msg, sizeof(msg));
#endif
            throw except::sp_exception(std::string("gb300 source_term failed: ") + msg);
        }
    }
}

namespace spade::pde_algs
{
    // pde_algs::boundary_flux (pde-algs/boundary_flux.h:16-105) on the GPU:
    // the faces of the selected domain boundaries add their flux to the two
    // cells they separate.  Selected by the gb300 traits after the flux
    // functor; the flags go to gbns_boundary_flux in the order min(0), max(0),
    // min(1), max(1), min(2), max(2).
    template <
        grid::multiblock_array sol_arr_t,
        grid::multiblock_array rhs_arr_t,
        typename flux_func_t,
        typename alg_traits_t>
    requires
        grid::has_centering_type<sol_arr_t, grid::cell_centered> && gb300::selects_gb300<alg_traits_t>
    static void boundary_flux(
        const sol_arr_t& prims,
        rhs_arr_t& rhs,
        const bound_box_t<bool, sol_arr_t::grid_type::dim()>& apply_to_boundary,
        const flux_func_t& flux_func,
        const alg_traits_t&)
    {
        const gbns_grid_desc g = gb300::lower_grid(prims);
        const gbns_scheme_desc s = gb300::lower_scheme(flux_func, GBNS_PREC_FP64);
        int apply[6] = {0, 0, 0, 0, 0, 0};
        for (int d = 0; d < int(sol_arr_t::grid_type::dim()); ++d)
        {
            apply[2*d] = apply_to_boundary.min(d) ? 1 : 0;
            apply[2*d + 1] = apply_to_boundary.max(d) ? 1 : 0;
        }
        const double* q = prims.image().base;
        double* r = rhs.image().base;
#ifdef GBNS_DROPIN_BFLUX_HOOK
        const int rc = GBNS_DROPIN_BFLUX_HOOK(&g, &s, q, r, apply);
#else
        static_assert(device::is_gpu<typename sol_arr_t::device_type> && device::is_gpu<typename rhs_arr_t::device_type>,
                      "the gb300 boundary_flux runs on device::gpu arrays");
        int rc = gbns_boundary_flux(&g, &s, q, r, apply, nullptr);
        if (rc == GBNS_OK && cudaDeviceSynchronize() != cudaSuccess) rc = GBNS_ERR_CUDA;
#endif
        if (rc != GBNS_OK)
        {
            char msg[512] = "drop-in hook failed";
#ifndef GBNS_DROPIN_BFLUX_HOOK
            gbns_last_error(msg, sizeof(msg));
#endif
            throw except::sp_exception(std::string("gb300 boundary_flux failed: ") + msg);
        }
    }
}

namespace spade::gb300
{
    // Wall kernels for the domain-boundary ghost fill.  Each is also the
    // reference's boundary_fill kernel form (ghost = kern(domain value, dir),
    // grid/boundary_fill.h:31-133), so the same object serves a CPU
    // spade::algs::boundary_fill and the gb300 fill below:
    //   isothermal_wall_t: no-slip, T_ghost = 2 T_wall - T, u, v, w negated;
    //   slip_wall_t:       adiabatic slip, the wall-normal velocity negated.
    template <typename dtype>
    struct isothermal_wall_t
    {
        using value_type = dtype;
        dtype t_wall;
        template <typename state_t> state_t operator()(const state_t& q, const int) const
        {
            state_t g = q;
            g.T() = dtype(2.0)*t_wall - q.T();
            g.u() = -q.u();
            g.v() = -q.v();
            g.w() = -q.w();
            return g;
        }
    };
    template <typename dtype>
    struct slip_wall_t
    {
        using value_type = dtype;
        template <typename state_t> state_t operator()(const state_t& q, const int dir) const
        {
            state_t g = q;
            g.u(dir) = -q.u(dir);
            return g;
        }
    };

    template <typename T> struct is_wall_kernel : std::false_type {};
    template <typename dtype> struct is_wall_kernel<isothermal_wall_t<dtype>> : std::true_type {};
    template <typename dtype> struct is_wall_kernel<slip_wall_t<dtype>> : std::true_type {};
    template <typename T> concept lowered_wall = is_wall_kernel<T>::value;

    // The boundary descriptor of one ghost fill: per face min(0), max(0), ...,
    // max(2): a wall where `walls` selects it, periodic where `periodic`
    // does (the flags the reference passes to make_exchange), else left alone.
    template <typename wall_t>
    requires lowered_wall<wall_t>
    gbns_bc_desc lower_bc(const ctrs::array<bool, 3>& periodic, const bound_box_t<bool, 3>& walls, const wall_t& wall)
    {
        gbns_bc_desc bc{};
        for (int d = 0; d < 3; ++d)
            for (int pm = 0; pm < 2; ++pm)
            {
                const int f = 2*d + pm;
                const bool is_wall = pm == 0 ? walls.min(d) : walls.max(d);
                if (is_wall && periodic[d])
                    throw except::sp_exception("gb300 ghost fill: a face cannot be both periodic and a wall");
                if (is_wall)
                {
                    if constexpr (std::same_as<wall_t, slip_wall_t<typename wall_t::value_type>>) bc.kind[f] = GBNS_BC_SLIP_ADIABATIC;
                    else
                    {
                        bc.kind[f] = GBNS_BC_ISOTHERMAL_NOSLIP;
                        bc.t_wall[f] = double(wall.t_wall);
                    }
                }
                else bc.kind[f] = periodic[d] ? GBNS_BC_PERIODIC : GBNS_BC_NONE;
            }
        return bc;
    }

    namespace detail
    {
        inline void check_call(int rc, const char* what)
        {
            if (rc == GBNS_OK) return;
            char msg[512] = "drop-in hook failed";
#ifndef GBNS_DROPIN_BC_HOOK
            gbns_last_error(msg, sizeof(msg));
#endif
            throw except::sp_exception(std::string(what) + msg);
        }
    }

    // Every ghost layer of a device::gpu grid_array in one launch: the
    // reference's `make_exchange(q, periodic)` handle's exchange followed by
    // `algs::boundary_fill(q, walls, wall)` (grid/make_exchange.h:98-421,
    // grid/boundary_fill.h:31-133), the pair its drivers call after each
    // stage; each ghost resolved to an interior donor, bit-identical to that
    // pair (gbns_fill_ghosts).
    template <grid::multiblock_array arr_t, typename wall_t>
    requires lowered_wall<wall_t> && grid::has_centering_type<arr_t, grid::cell_centered>
    void fill_ghosts(arr_t& q, const ctrs::array<bool, 3>& periodic, const bound_box_t<bool, 3>& walls, const wall_t& wall)
    {
        const gbns_grid_desc g = lower_grid(q);
        const gbns_bc_desc bc = lower_bc(periodic, walls, wall);
        double* p = q.image().base;
#ifdef GBNS_DROPIN_BC_HOOK
        const int rc = GBNS_DROPIN_BC_HOOK(&g, &bc, nullptr, p, 0.0);
#else
        static_assert(device::is_gpu<typename arr_t::device_type>, "the gb300 ghost fill runs on device::gpu arrays");
        int rc = gbns_fill_ghosts(&g, &bc, p, nullptr);
        if (rc == GBNS_OK && cudaDeviceSynchronize() != cudaSuccess) rc = GBNS_ERR_CUDA;
#endif
        detail::check_call(rc, "gb300 fill_ghosts failed: ");
    }

    // The reference's time integration of these flows, fused:
    // integrator_t with ssprk3_t and state_transform_t
    // (time-integration/integrator.h:18-59, advance.h:234-280, explicit.h:80-88)
    // whose rhs_calc is flux_div of `flux` and whose boundary_cond is the
    // exchange + boundary_fill pair above.  advance() is gbns_ssprk3_step:
    // three launches of flux_div with the stage update fused in, three ghost
    // fills, bit-identical to the reference in FP64.  The stepper owns the
    // scratch (two residuals and the intermediate state, 3 arrays of q's size).
    template <grid::multiblock_array arr_t, typename flux_func_t, typename wall_t>
    requires lowered_wall<wall_t> && grid::has_centering_type<arr_t, grid::cell_centered>
    struct ssprk3_integrator_t
    {
        arr_t& q;
        gbns_grid_desc grid;
        gbns_scheme_desc scheme;
        gbns_bc_desc bc;
        double dt;
        double t;
        double* work = nullptr;

        ssprk3_integrator_t(arr_t& q_in, const flux_func_t& flux, const ctrs::array<bool, 3>& periodic,
                            const bound_box_t<bool, 3>& walls, const wall_t& wall, double dt_in, double t0 = 0.0,
                            int precision = GBNS_PREC_FP64)
            : q{q_in}, grid{lower_grid(q_in)}, scheme{lower_scheme(flux, precision)},
              bc{lower_bc(periodic, walls, wall)}, dt{dt_in}, t{t0}
        {
#ifndef GBNS_DROPIN_BC_HOOK
            static_assert(device::is_gpu<typename arr_t::device_type>, "the gb300 integrator runs on device::gpu arrays");
            size_t n = 0;
            if (gbns_array_size(&grid, &n) != GBNS_OK || cudaMalloc(&work, 3*n*sizeof(double)) != cudaSuccess)
                throw except::sp_exception("gb300 integrator: cannot allocate its scratch arrays");
#endif
        }
        ssprk3_integrator_t(const ssprk3_integrator_t&) = delete;
        ssprk3_integrator_t& operator=(const ssprk3_integrator_t&) = delete;
        ~ssprk3_integrator_t()
        {
#ifndef GBNS_DROPIN_BC_HOOK
            if (work) cudaFree(work);
#endif
        }

        void advance()
        {
            double* p = q.image().base;
#ifdef GBNS_DROPIN_BC_HOOK
            const int rc = GBNS_DROPIN_BC_HOOK(&grid, &bc, &scheme, p, dt);
#else
            int rc = gbns_ssprk3_step(&grid, &scheme, &bc, p, work, dt, nullptr);
            if (rc == GBNS_OK && cudaDeviceSynchronize() != cudaSuccess) rc = GBNS_ERR_CUDA;
#endif
            detail::check_call(rc, "gb300 ssprk3 step failed: ");
            t += dt;
        }

        arr_t& solution() { return q; }
        double time() const { return t; }
    };

    // integrator_t with ssprk3_t on a refined (amr_blocks_t) grid, its exchange
    // as the boundary condition (the reference's drivers: integrator_t whose bc
    // runs handle.exchange, time-integration/advance.h:234-280): one
    // gbns_ssprk3_step_blocks per advance() with the grid's own block boxes and
    // the plan lowered from the reference's exchange handle
    // (exchange_plan_t).  device::gpu arrays; q must hold exchanged ghosts
    // (plan.exchange(q)) before the first step, as the reference's driver
    // refreshes them.
    template <typename arr_t, typename flux_func_t>
    struct ssprk3_refined_integrator_t
    {
        arr_t& q;
        const exchange_plan_t& plan;
        std::vector<double> boxes;
        gbns_grid_desc grid;
        gbns_scheme_desc scheme;
        gbns_bc_desc bc{};
        bool walls_on = false;
        double dt;
        double t;
        double* work = nullptr;

        ssprk3_refined_integrator_t(arr_t& q_in, const flux_func_t& flux, const exchange_plan_t& plan_in, double dt_in,
                                    double t0 = 0.0, int precision = GBNS_PREC_FP64)
            : q{q_in}, plan{plan_in}, grid{lower_refined_grid(q_in, boxes)}, scheme{lower_scheme(flux, precision)},
              dt{dt_in}, t{t0}
        {
            allocate();
        }

        // with walls: after each exchange the wall faces are filled as the
        // reference's boundary_fill(q, faces, wall) does (gbns_wall_fill_blocks)
        template <typename wall_t>
        ssprk3_refined_integrator_t(arr_t& q_in, const flux_func_t& flux, const exchange_plan_t& plan_in,
                                    const ctrs::array<bool, 3>& periodic, const bound_box_t<bool, 3>& walls,
                                    const wall_t& wall, double dt_in, double t0 = 0.0, int precision = GBNS_PREC_FP64)
            : q{q_in}, plan{plan_in}, grid{lower_refined_grid(q_in, boxes)}, scheme{lower_scheme(flux, precision)},
              bc{lower_bc(periodic, walls, wall)}, walls_on{true}, dt{dt_in}, t{t0}
        {
            allocate();
        }

        void allocate()
        {
#ifndef GBNS_DROPIN_HOOK
            static_assert(device::is_gpu<typename arr_t::device_type>, "the gb300 integrator runs on device::gpu arrays");
            const size_t n = size_t(5)*size_t(grid.nblk[0])*size_t(grid.ncell[0] + 2*grid.ng)*
                             size_t(grid.ncell[1] + 2*grid.ng)*size_t(grid.ncell[2] + 2*grid.ng);
            if (cudaMalloc(&work, 3*n*sizeof(double)) != cudaSuccess)
                throw except::sp_exception("gb300 integrator: cannot allocate its scratch arrays");
#endif
        }
        ssprk3_refined_integrator_t(const ssprk3_refined_integrator_t&) = delete;
        ssprk3_refined_integrator_t& operator=(const ssprk3_refined_integrator_t&) = delete;
        ~ssprk3_refined_integrator_t()
        {
#ifndef GBNS_DROPIN_HOOK
            if (work) cudaFree(work);
#endif
        }

        void advance()
        {
#ifndef GBNS_DROPIN_HOOK
            int rc = gbns_ssprk3_step_blocks(&grid, &scheme, boxes.data(), plan.plan, walls_on ? &bc : nullptr,
                                             q.image().base, work, dt, nullptr);
            if (rc == GBNS_OK && cudaDeviceSynchronize() != cudaSuccess) rc = GBNS_ERR_CUDA;
            detail::check_call(rc, "gb300 ssprk3 step failed: ");
#endif
            t += dt;
        }

        arr_t& solution() { return q; }
        double time() const { return t; }
    };
}
