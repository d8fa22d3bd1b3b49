// Routes a lowered scheme to the translation unit holding its kernels.
#include <cstdlib>
#include "gbns_internal.cuh"
#include "flux_launch.cuh"

namespace gbns
{
    bool tma_disabled()
    {
        const char* e = std::getenv("GBNS_NO_TMA");
        return e && e[0] == '1';
    }

    int flux_variant_count(const gbns_scheme_desc* s)
    {
        if (!s) return 0;
        // FP32-flux adds one variant (the TMA-staged FP64 box); FP64 adds
        // 576-thread 8x8x8 tiles (and a 768-thread one for WENO5) in its place.
        const bool fp32 = s->precision == GBNS_PREC_FP32_FLUX;
        switch (s->convective)
        {
            case GBNS_CONV_CENT_KEEP: return (s->order == 2 ? 5 : (s->order == 4 ? 2 : 1 + (fp32 ? 1 : 0)));
            case GBNS_CONV_TOTANI:    return 3;
            case GBNS_CONV_FWENO:     return 5;
            case GBNS_CONV_WENO5:     return fp32 ? 5 : 6;
            case GBNS_CONV_HYBRID:    return 3;
            default:                  return fp32 ? 2 : 1;
        }
    }

    int launch_flux_div(const gbns_grid_desc* g, const GeomK& G, const YTabK* Y, const SchemeK& S,
                        const gbns_scheme_desc* desc, const double* prims, double* rhs,
                        int increment, cudaStream_t stream, int variant, const RkFuse* fuse,
                        int blk0, int blk1, const double* blk_inv_dx)
    {
        if (variant < 0 || variant >= flux_variant_count(desc))
            return set_error(GBNS_ERR_INVALID, "flux_div tile variant out of range");
        if (blk1 < 0) blk1 = G.nblk;
        if (blk0 < 0 || blk1 > G.nblk || blk0 > blk1) return set_error(GBNS_ERR_INVALID, "block range out of the grid");
        FluxCall c{g, &G, Y, &S, prims, rhs, increment, stream, variant, fuse, blk0, blk1, blk_inv_dx};
        const bool stretch = g->coords != GBNS_COORDS_IDENTITY;
        const bool upwind = desc->convective == GBNS_CONV_FWENO || desc->convective == GBNS_CONV_WENO5;
        const int conv = desc->convective, order = desc->order;
        if (conv == GBNS_CONV_HYBRID)
        {
            if (desc->precision == GBNS_PREC_FP64)
                return stretch ? flux_f64x_stretch_c(c, conv, order) : flux_f64x_identity_c(c, conv, order);
            if (desc->precision == GBNS_PREC_FP64_FMA)
                return stretch ? flux_f64_stretch_c(c, conv, order) : flux_f64_identity_c(c, conv, order);
            return stretch ? flux_f32_stretch_c(c, conv, order) : flux_f32_identity_c(c, conv, order);
        }
        if (desc->precision == GBNS_PREC_FP64)
        {
            if (!stretch) return upwind ? flux_f64x_identity_b(c, conv, order) : flux_f64x_identity_a(c, conv, order);
            return upwind ? flux_f64x_stretch_b(c, conv, order) : flux_f64x_stretch_a(c, conv, order);
        }
        if (desc->precision == GBNS_PREC_FP64_FMA)
        {
            if (!stretch) return upwind ? flux_f64_identity_b(c, conv, order) : flux_f64_identity_a(c, conv, order);
            return upwind ? flux_f64_stretch_b(c, conv, order) : flux_f64_stretch_a(c, conv, order);
        }
        if (!stretch) return upwind ? flux_f32_identity_b(c, conv, order) : flux_f32_identity_a(c, conv, order);
        return upwind ? flux_f32_stretch_b(c, conv, order) : flux_f32_stretch_a(c, conv, order);
    }
}
