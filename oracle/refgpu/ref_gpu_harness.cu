// Test infrastructure: drives the REFERENCE's own GPU flux_div
// (pde-algs/flux-div/flux_div.h:16-56 with the basic, bfoct and longf
// algorithms) on device::gpu grid_arrays, through its public API only.
//
// Compiled twice from the reference's headers (oracle/refgpu/Makefile):
//   * host side, linked with oracle/refgpu/record_cudart.cc in place of the
//     CUDA runtime: running it here, without a GPU, writes the launch script
//     (allocations, geometry uploads, the kernel launches and their argument
//     bytes) of one flux_div per algorithm;
//   * device side only, into a cubin holding the same kernels.
// oracle/refgpu/replay.cc replays the script with that cubin on a GPU, so the
// reference's kernels run unchanged on the caller's arrays.
//
// usage: ref_gpu_harness <scheme> nbx nby nbz ncx ncy ncz ng
//                        x0 x1 y0 y1 z0 z1 gamma R mu Pr eps_p eps_T sensor <alg>[,<alg>...]
//   scheme: ck2_visc       compose(cent_keep<2>, visc_lr(constant_viscosity_t))
//           fweno_diss_visc compose(fweno_t, pressure_diss_lr(const_sensor_t), visc_lr(constant))
//   alg:    basic | bfoct | longf
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "spade.h"

extern "C" void refrec_mark(const void* dptr, const char* role);
extern "C" void refrec_phase(const char* name);

namespace
{
    using real_t = double;
    using prim_t = spade::fluid_state::prim_t<real_t>;
    using flux_t = spade::fluid_state::flux_t<real_t>;
    using gas_t  = spade::fluid_state::ideal_gas_t<real_t>;

    struct problem_t
    {
        int nb[3], nc[3], ng;
        double bounds[6];
        double gamma, rgas, mu, prandtl, eps_p, eps_T, sensor;
    };

    template <typename arr_t, typename rhs_t, typename flx_t>
    void run_alg(const std::string& alg, const arr_t& q, rhs_t& r, const flx_t& flx)
    {
        refrec_phase(alg.c_str());
        if (alg == "basic")      spade::pde_algs::flux_div(q, r, flx, spade::algs::make_traits(spade::pde_algs::basic));
        else if (alg == "bfoct") spade::pde_algs::flux_div(q, r, flx, spade::algs::make_traits(spade::pde_algs::bfoct));
        else if (alg == "longf") spade::pde_algs::flux_div(q, r, flx, spade::algs::make_traits(spade::pde_algs::longf));
        else throw std::runtime_error("unknown flux_div algorithm " + alg);
    }
}

int main(int argc, char** argv)
{
    if (argc != 23)
    {
        std::fprintf(stderr, "usage: %s scheme nbx nby nbz ncx ncy ncz ng x0 x1 y0 y1 z0 z1 gamma R mu Pr eps_p eps_T sensor algs\n", argv[0]);
        return 2;
    }
    const std::string scheme = argv[1];
    problem_t pb;
    for (int d = 0; d < 3; ++d) { pb.nb[d] = std::atoi(argv[2 + d]); pb.nc[d] = std::atoi(argv[5 + d]); }
    pb.ng = std::atoi(argv[8]);
    for (int i = 0; i < 6; ++i) pb.bounds[i] = std::atof(argv[9 + i]);
    pb.gamma = std::atof(argv[15]); pb.rgas = std::atof(argv[16]); pb.mu = std::atof(argv[17]);
    pb.prandtl = std::atof(argv[18]); pb.eps_p = std::atof(argv[19]); pb.eps_T = std::atof(argv[20]);
    pb.sensor = std::atof(argv[21]);
    std::vector<std::string> algs;
    {
        std::string s = argv[22];
        size_t pos = 0;
        while (pos <= s.size())
        {
            const size_t c = s.find(',', pos);
            algs.push_back(s.substr(pos, c == std::string::npos ? std::string::npos : c - pos));
            if (c == std::string::npos) break;
            pos = c + 1;
        }
    }
    try
    {
        int eargc = 0;
        char** eargv = nullptr;
        spade::parallel::compute_env_t env(&eargc, &eargv, {0});
        env.exec([&](spade::parallel::pool_t& group)
        {
            spade::ctrs::array<int, 3> num_blocks(pb.nb[0], pb.nb[1], pb.nb[2]);
            spade::ctrs::array<int, 3> cells(pb.nc[0], pb.nc[1], pb.nc[2]);
            spade::bound_box_t<real_t, 3> bounds;
            for (int d = 0; d < 3; ++d)
            {
                bounds.min(d) = pb.bounds[2*d];
                bounds.max(d) = pb.bounds[2*d + 1];
            }
            spade::coords::identity<real_t> coords;
            spade::grid::cartesian_blocks_t blocks(num_blocks, bounds);
            // cartesian_blocks_t leaves the non-boundary domain-boundary flags
            // indeterminate (grid/cartesian_blocks.h:51-64); give every flag
            // its defined value before the grid copies them to the device.
            for (std::size_t lb = 0; lb < blocks.block_is_domain_boundary.size(); ++lb)
            {
                const int b[3] = {int(lb % pb.nb[0]), int((lb / pb.nb[0]) % pb.nb[1]), int(lb / (pb.nb[0]*pb.nb[1]))};
                for (int d = 0; d < 3; ++d)
                {
                    blocks.block_is_domain_boundary[lb].min(d) = (b[d] == 0);
                    blocks.block_is_domain_boundary[lb].max(d) = (b[d] == pb.nb[d] - 1);
                }
            }
            spade::grid::cartesian_grid_t grid(cells, blocks, coords, group);
            spade::ctrs::array<int, 3> nexch(pb.ng, pb.ng, pb.ng);
            spade::grid::grid_array q(grid, prim_t(0.0), nexch, spade::device::gpu);
            spade::grid::grid_array r(grid, flux_t(0.0), nexch, spade::device::gpu);
            refrec_mark(q.data.raw, "prims");
            refrec_mark(r.data.raw, "rhs");
            gas_t air(pb.gamma, pb.rgas);
            spade::viscous_laws::constant_viscosity_t<real_t> law(pb.mu, pb.prandtl);
            spade::viscous::visc_lr visc(law, air);
            if (scheme == "ck2_visc")
            {
                const auto flx = spade::omni::compose(spade::convective::cent_keep<2>(air), visc);
                for (const auto& a : algs) run_alg(a, q, r, flx);
            }
            else if (scheme == "fweno_diss_visc")
            {
                spade::state_sensor::const_sensor_t<real_t> sens(pb.sensor);
                spade::convective::pressure_diss_lr diss(air, sens, pb.eps_p, pb.eps_T);
                const auto flx = spade::omni::compose(spade::convective::fweno_t<gas_t>(air), diss, visc);
                for (const auto& a : algs) run_alg(a, q, r, flx);
            }
            else throw std::runtime_error("unknown scheme " + scheme);
        });
    }
    catch (const std::exception& e)
    {
        std::fprintf(stderr, "ref_gpu_harness: %s\n", e.what());
        return 1;
    }
    return 0;
}
