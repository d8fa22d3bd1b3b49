// pde_algs::boundary_flux for the faces normal to y (see boundary_flux.cuh);
// FP64 without FMA contraction (built with -fmad=false).
#include "boundary_flux.cuh"

namespace gbns
{
    namespace { status_registrar tu_status_registrar; }

    int boundary_flux_launch_d1(const GeomK& G, const SchemeK& S, const BndArgs& A, int conv, int order, cudaStream_t st)
    {
        constexpr int D = 1, TAG = 66;
        switch (conv)
        {
        case GBNS_CONV_NONE: return run_boundary_flux<BndCfg<GBNS_CONV_NONE, 2, D, TAG>, D>(G, S, A, st);
        case GBNS_CONV_CENT_KEEP:
            if (order == 2) return run_boundary_flux<BndCfg<GBNS_CONV_CENT_KEEP, 2, D, TAG>, D>(G, S, A, st);
            if (order == 4) return run_boundary_flux<BndCfg<GBNS_CONV_CENT_KEEP, 4, D, TAG>, D>(G, S, A, st);
            if (order == 6) return run_boundary_flux<BndCfg<GBNS_CONV_CENT_KEEP, 6, D, TAG>, D>(G, S, A, st);
            if (order == 8) return run_boundary_flux<BndCfg<GBNS_CONV_CENT_KEEP, 8, D, TAG>, D>(G, S, A, st);
            break;
        case GBNS_CONV_TOTANI: return run_boundary_flux<BndCfg<GBNS_CONV_TOTANI, 2, D, TAG>, D>(G, S, A, st);
        case GBNS_CONV_FWENO: return run_boundary_flux<BndCfg<GBNS_CONV_FWENO, 2, D, TAG>, D>(G, S, A, st);
        case GBNS_CONV_WENO5: return run_boundary_flux<BndCfg<GBNS_CONV_WENO5, 2, D, TAG>, D>(G, S, A, st);
        case GBNS_CONV_HYBRID:
            if (order == 2) return run_boundary_flux<BndCfg<GBNS_CONV_HYBRID, 2, D, TAG>, D>(G, S, A, st);
            if (order == 4) return run_boundary_flux<BndCfg<GBNS_CONV_HYBRID, 4, D, TAG>, D>(G, S, A, st);
            break;
        default: break;
        }
        return set_error(GBNS_ERR_UNSUPPORTED, "boundary_flux scheme not instantiated");
    }
}
