// Launch plumbing for the flux-divergence kernel family.
#pragma once

#include "gbns_internal.cuh"

namespace gbns
{
    // Fused RK stage riding on a flux_div launch (see FluxArgs).
    struct RkFuse
    {
        int nres;
        int write_rhs;
        const double* res[2];
        double coeff[3];
        double* q_out;
    };

    struct FluxCall
    {
        const gbns_grid_desc* g;
        const GeomK* G;
        const YTabK* Y;
        const SchemeK* S;
        const double* prims;
        double* rhs;
        int increment;
        cudaStream_t stream;
        int variant;
        const RkFuse* fuse;
        int blk0, blk1;     // the blocks this launch covers: blk0 .. blk1 - 1
        const double* blk_inv_dx;   // refined layouts: per-block 1/dx (device), else nullptr
    };

    // f64x: FP64 without FMA contraction (-fmad=false): the kernels follow the
    // reference's operation order, so they reproduce its CPU results bit for
    // bit.  f64: FP64 with FMA contraction.  f32: FP32 flux arithmetic.
    // One translation unit per (precision, coordinates) pair instantiates
    // the kernels; each returns GBNS_ERR_UNSUPPORTED for combinations it
    // does not hold.
    // Group A: no / centred (cent_keep, totani_lr) convective terms.
    // Group B: upwind (fweno_t, WENO5) convective terms.
    int flux_f64x_identity_a(const FluxCall& c, int conv, int order);
    int flux_f64x_identity_b(const FluxCall& c, int conv, int order);
    int flux_f64x_stretch_a (const FluxCall& c, int conv, int order);
    int flux_f64x_stretch_b (const FluxCall& c, int conv, int order);
    int flux_f64_identity_a(const FluxCall& c, int conv, int order);
    int flux_f64_identity_b(const FluxCall& c, int conv, int order);
    int flux_f64_stretch_a (const FluxCall& c, int conv, int order);
    int flux_f64_stretch_b (const FluxCall& c, int conv, int order);
    int flux_f32_identity_a(const FluxCall& c, int conv, int order);
    int flux_f32_identity_b(const FluxCall& c, int conv, int order);
    int flux_f32_stretch_a (const FluxCall& c, int conv, int order);
    int flux_f32_stretch_b (const FluxCall& c, int conv, int order);
    int flux_f64x_identity_c(const FluxCall& c, int conv, int order);
    int flux_f64x_stretch_c (const FluxCall& c, int conv, int order);
    int flux_f64_identity_c(const FluxCall& c, int conv, int order);
    int flux_f64_stretch_c (const FluxCall& c, int conv, int order);
    int flux_f32_identity_c(const FluxCall& c, int conv, int order);
    int flux_f32_stretch_c (const FluxCall& c, int conv, int order);

    // Number of tile variants built for a scheme (autotuner search space).
    int flux_variant_count(const gbns_scheme_desc* s);

    // Environment override GBNS_NO_TMA=1 forces the coalesced-load staging.
    bool tma_disabled();


}
