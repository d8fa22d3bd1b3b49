// Instantiation helper for the flux-divergence translation units.  Each TU
// defines GBNS_REAL, GBNS_STRETCH, GBNS_GROUP, GBNS_TAG and GBNS_FN and includes this.
// Groups: 0 = none / cent_keep / totani, 1 = fweno / WENO5, 2 = hybrid.
#pragma once

#include <cstring>
#include "flux_kernel.cuh"
#include "flux_launch.cuh"

namespace gbns
{
    namespace { status_registrar tu_status_registrar; }

    namespace {
    template <class Cfg>
    int run_flux_cfg(const FluxCall& c)
    {
        const GeomK& G = *c.G;
        FluxArgs A;
        A.prims = c.prims;
        A.rhs = c.rhs;
        A.increment = c.increment;
        A.rk_nres = 0;
        A.write_rhs = 1;
        A.q_out = nullptr;
        A.blk_inv_dx = c.blk_inv_dx;
        A.rk_res[0] = A.rk_res[1] = nullptr;
        A.rk_coeff[0] = A.rk_coeff[1] = A.rk_coeff[2] = 0.0;
        if (c.fuse)
        {
            A.rk_nres = c.fuse->nres;
            A.write_rhs = c.fuse->write_rhs;
            A.rk_res[0] = c.fuse->res[0];
            A.rk_res[1] = c.fuse->res[1];
            for (int j = 0; j < 3; ++j) A.rk_coeff[j] = c.fuse->coeff[j];
            A.q_out = c.fuse->q_out;
        }
        A.ntile[0] = (G.n[0] + Cfg::TX - 1)/Cfg::TX;
        A.ntile[1] = (G.n[1] + Cfg::TY - 1)/Cfg::TY;
        A.ntile[2] = (G.n[2] + Cfg::TZ - 1)/Cfg::TZ;
        const long long ntiles = (long long)A.ntile[0]*A.ntile[1]*A.ntile[2];
        const int nrun = c.blk1 - c.blk0;
        if (nrun < 1) return GBNS_OK;
        if (ntiles > 2147483647ll || nrun > 65535)
            return set_error(GBNS_ERR_UNSUPPORTED, "grid too large for one flux_div launch (blocks > 65535)");
        CUtensorMap tmap;
        std::memset(&tmap, 0, sizeof(tmap));
        A.use_tma = 0;
        A.sh_off = 0;
        auto kern = flux_div_kernel<Cfg>;
        int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(Cfg::SMEM_BYTES)),
                            "flux_div smem attribute");
        if (rc) return rc;
        const bool aligned = (G.ni % 2 == 0) && ((reinterpret_cast<uintptr_t>(c.prims) & 15) == 0);
        ShadowK sh{nullptr, 0, 0};
        if constexpr (Cfg::SHADOW)
        {
            // FP32 copy of the state, staged by TMA (its layout is always aligned)
            rc = shadow_begin(c.prims, G, c.blk0, c.blk1, Cfg::H, Cfg::BXE, Cfg::BY, Cfg::BZ, c.stream, sh, &tmap);
            if (rc) return rc;
            A.use_tma = 1;
            A.sh_off = sh.off;
        }
        else if (!Cfg::DIRECT && aligned && !tma_disabled())
        {
            rc = encode_prims_tmap(&tmap, c.prims, G, Cfg::BXE, Cfg::BY, Cfg::BZ);
            if (rc) return rc;
            A.use_tma = 1;
        }
        const dim3 grid{unsigned(ntiles), unsigned(nrun)};
        YTabT<Cfg::STRETCH> Y;
        if constexpr (Cfg::STRETCH) Y = *c.Y;
        kern<<<grid, Cfg::NT, Cfg::SMEM_BYTES, c.stream>>>(tmap, G, Y, *c.S, A, c.blk0);
        rc = check_cuda(cudaGetLastError(), "flux_div launch");
        const int erc = shadow_end(sh, c.stream);
        return rc ? rc : erc;
    }
    }
}

#define GBNS_RUN(CONV, ORDER, TX, TY, TZ, NT) \
    return run_flux_cfg<FluxCfg<GBNS_REAL, CONV, ORDER, GBNS_STRETCH, TX, TY, TZ, NT, GBNS_TAG, 0>>(c)
// FP32 only: the box staged by TMA from the FP32 copy of the state
#define GBNS_RUN_SHADOW(CONV, ORDER, TX, TY, TZ, NT) \
    return run_flux_cfg<FluxCfg<GBNS_REAL, CONV, ORDER, GBNS_STRETCH, TX, TY, TZ, NT, GBNS_TAG, 2>>(c)
#if GBNS_FP32
#define GBNS_RUN_D GBNS_RUN_SHADOW
#else
#define GBNS_RUN_D GBNS_RUN
#endif

namespace gbns
{
    // Tile variants.  Variant 0 is the default; every variant computes the
    // same results (bit for bit in FP64, to single-precision rounding in
    // FP32-flux, whose FP32 arithmetic each instantiation contracts on its
    // own).  In FP32 TUs the GBNS_RUN_D variants stage their
    // box by TMA from the FP32 copy of the state and the last variant stages
    // the FP64 box through TMA and converts it.
    int GBNS_FN(const FluxCall& c, int conv, int order)
    {
        const int v = c.variant;
#if GBNS_GROUP == 0
        if (conv == GBNS_CONV_NONE)
        {
            if (GBNS_FP32 && v == 1) GBNS_RUN(GBNS_CONV_NONE, 2, 8, 8, 8, 256);
            GBNS_RUN_D(GBNS_CONV_NONE, 2, 8, 8, 8, 256);
        }
        if (conv == GBNS_CONV_CENT_KEEP)
        {
            if (order == 2)
            {
                if (v == 1) GBNS_RUN_D(GBNS_CONV_CENT_KEEP, 2, 16, 8, 4, 256);
                if (v == 2) GBNS_RUN_D(GBNS_CONV_CENT_KEEP, 2, 8, 8, 4, 128);
                if (v == 3) GBNS_RUN_D(GBNS_CONV_CENT_KEEP, 2, 16, 8, 8, 256);
#if !GBNS_FP32
                if (v == 4) GBNS_RUN(GBNS_CONV_CENT_KEEP, 2, 8, 8, 8, 576);
#endif
                if (GBNS_FP32 && v == 4) GBNS_RUN(GBNS_CONV_CENT_KEEP, 2, 8, 8, 8, 256);
                GBNS_RUN_D(GBNS_CONV_CENT_KEEP, 2, 8, 8, 8, 256);
            }
            if (order == 4)
            {
#if !GBNS_FP32
                if (v == 1) GBNS_RUN(GBNS_CONV_CENT_KEEP, 4, 8, 8, 8, 576);
#endif
                if (GBNS_FP32 && v == 1) GBNS_RUN(GBNS_CONV_CENT_KEEP, 4, 8, 8, 8, 256);
                GBNS_RUN_D(GBNS_CONV_CENT_KEEP, 4, 8, 8, 8, 256);
            }
            if (order == 6)
            {
                if (GBNS_FP32 && v == 1) GBNS_RUN(GBNS_CONV_CENT_KEEP, 6, 8, 8, 4, 256);
                GBNS_RUN_D(GBNS_CONV_CENT_KEEP, 6, 8, 8, 4, 256);
            }
            if (order == 8)
            {
                if (GBNS_FP32 && v == 1) GBNS_RUN(GBNS_CONV_CENT_KEEP, 8, 8, 8, 4, 256);
                GBNS_RUN_D(GBNS_CONV_CENT_KEEP, 8, 8, 8, 4, 256);
            }
        }
        if (conv == GBNS_CONV_TOTANI)
        {
            if (v == 1) GBNS_RUN_D(GBNS_CONV_TOTANI, 2, 16, 8, 4, 256);
#if !GBNS_FP32
            if (v == 2) GBNS_RUN(GBNS_CONV_TOTANI, 2, 8, 8, 8, 576);
#endif
            if (GBNS_FP32 && v == 2) GBNS_RUN(GBNS_CONV_TOTANI, 2, 8, 8, 8, 256);
            GBNS_RUN_D(GBNS_CONV_TOTANI, 2, 8, 8, 8, 256);
        }
#elif GBNS_GROUP == 1
        if (conv == GBNS_CONV_FWENO)
        {
            if (v == 1) GBNS_RUN_D(GBNS_CONV_FWENO, 2, 8, 8, 4, 128);
            if (v == 2) GBNS_RUN_D(GBNS_CONV_FWENO, 2, 16, 8, 4, 256);
            if (v == 3) GBNS_RUN_D(GBNS_CONV_FWENO, 2, 8, 8, 8, 512);
#if !GBNS_FP32
            if (v == 4) GBNS_RUN(GBNS_CONV_FWENO, 2, 8, 8, 8, 576);
#endif
            if (GBNS_FP32 && v == 4) GBNS_RUN(GBNS_CONV_FWENO, 2, 8, 8, 8, 256);
            GBNS_RUN_D(GBNS_CONV_FWENO, 2, 8, 8, 8, 256);
        }
        if (conv == GBNS_CONV_WENO5)
        {
            if (v == 1) GBNS_RUN_D(GBNS_CONV_WENO5, 2, 8, 8, 8, 256);
            if (v == 2) GBNS_RUN_D(GBNS_CONV_WENO5, 2, 8, 4, 4, 128);
            // 16 warps on one 8^3 tile: twice the warps per SM of variant 1
            // for latency hiding when one CTA fills shared memory (FP64)
            if (v == 3) GBNS_RUN_D(GBNS_CONV_WENO5, 2, 8, 8, 8, 512);
#if !GBNS_FP32
            // 18 warps at 96 registers and 24 at 80 (no or light spills in
            // FP64): one round covers each direction's 576 faces, so the face
            // loop has no tail run by two warps alone
            if (v == 4) GBNS_RUN(GBNS_CONV_WENO5, 2, 8, 8, 8, 576);
            if (v == 5) GBNS_RUN(GBNS_CONV_WENO5, 2, 8, 8, 8, 768);
#endif
            if (GBNS_FP32 && v == 4) GBNS_RUN(GBNS_CONV_WENO5, 2, 8, 8, 4, 256);
            GBNS_RUN_D(GBNS_CONV_WENO5, 2, 8, 8, 4, 256);
        }
#else
        if (conv == GBNS_CONV_HYBRID)
        {
            if (order == 2)
            {
                if (v == 1) GBNS_RUN_D(GBNS_CONV_HYBRID, 2, 8, 8, 8, 256);
#if !GBNS_FP32
                if (v == 2) GBNS_RUN(GBNS_CONV_HYBRID, 2, 8, 8, 8, 576);
#endif
                if (GBNS_FP32 && v == 2) GBNS_RUN(GBNS_CONV_HYBRID, 2, 8, 8, 4, 256);
                GBNS_RUN_D(GBNS_CONV_HYBRID, 2, 8, 8, 4, 256);
            }
            if (order == 4)
            {
                if (v == 1) GBNS_RUN_D(GBNS_CONV_HYBRID, 4, 8, 8, 8, 256);
#if !GBNS_FP32
                if (v == 2) GBNS_RUN(GBNS_CONV_HYBRID, 4, 8, 8, 8, 576);
#endif
                if (GBNS_FP32 && v == 2) GBNS_RUN(GBNS_CONV_HYBRID, 4, 8, 8, 4, 256);
                GBNS_RUN_D(GBNS_CONV_HYBRID, 4, 8, 8, 4, 256);
            }
        }
#endif
        return set_error(GBNS_ERR_UNSUPPORTED, "flux scheme not instantiated");
    }
}
