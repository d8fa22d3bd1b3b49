// Flux-divergence kernels of the batched form (one CTA per tile item).  Each TU defines
// GBNS_REAL, GBNS_TAG, GBNS_FP32, GBNS_BATCH_GROUP and GBNS_BATCH_FN and
// includes this; a TU instantiates the tile variants of its group of kernel
// classes (0: cent_keep<2>, totani_lr, fweno_t; 1: WENO5; 2: hybrid).
#pragma once

#include <cstddef>
#include "flux_kernel.cuh"
#include "batch_internal.cuh"

namespace gbns
{
    namespace
    {
        status_registrar tu_status_registrar;

        // The per-item arguments live in shared memory: a CTA copies its
        // item's geometry and scheme constants there and the tile code reads
        // them like the single-grid kernel's parameters (unpacking the scheme
        // constants itself, as the single-grid kernel does).
        struct ItemArgs
        {
            GeomK G;
            SchemeK S;
            FluxArgs A;
            const YTabK* ytab;
            const CUtensorMap* tmap;
            int lb, tile;
        };

        // One CTA per item of the class's range of the tile list (no
        // persistent loop: a loop around the tile lets the compiler keep
        // values live across items, which spilled the 256-thread FP64 tiles).
        // The arrays are read through the instance descriptors (no TMA: the
        // halo is staged with coalesced loads, or straight into FP32 for
        // FP32-flux).
        template <class Cfg>
        __global__ void __launch_bounds__(Cfg::NT, Cfg::MINB)
        flux_batch_kernel(const TileItem* __restrict__ items, const int* __restrict__ offsets,
                          const int* __restrict__ counts, const InstK* __restrict__ insts,
                          const YTabK* __restrict__ ytabs, const long long* __restrict__ left,
                          const CUtensorMap* __restrict__ tmaps, const int cls, const int stage)
        {
            extern __shared__ __align__(128) unsigned char smem_raw[];
            __shared__ __align__(16) ItemArgs arg;
            if (int(blockIdx.x) >= counts[cls]) return;
            const TileItem w = items[offsets[cls] + int(blockIdx.x)];
            // an instance that has done its steps idles until it is retired
            if (left[w.inst] == 0) return;
            const InstK& I = insts[w.inst];
            {
                // geometry and scheme constants: word copies by the whole CTA.
                // Of the per-block spacing tables only the item's block's
                // entries are copied (the tile reads no other).
                constexpr int GHEAD = int(offsetof(GeomK, inv_dx))/4;
                const int* sg = reinterpret_cast<const int*>(&I.G);
                int* dg = reinterpret_cast<int*>(&arg.G);
                for (int i = threadIdx.x; i < GHEAD; i += Cfg::NT) dg[i] = sg[i];
                const int* ss = reinterpret_cast<const int*>(&I.S);
                int* ds = reinterpret_cast<int*>(&arg.S);
                for (int i = threadIdx.x; i < int(sizeof(SchemeK)/4); i += Cfg::NT) ds[i] = ss[i];
                if (threadIdx.x < 3)
                {
                    const int d = threadIdx.x;
                    const int nb0 = I.G.nb[0], nb1 = I.G.nb[1];
                    const int bd = d == 0 ? w.lb % nb0 : (d == 1 ? (w.lb / nb0) % nb1 : w.lb / (nb0*nb1));
                    arg.G.inv_dx[d][bd] = I.G.inv_dx[d][bd];
                    arg.G.inv_dx_f[d][bd] = I.G.inv_dx_f[d][bd];
                }
            }
            if (threadIdx.x == 0)
            {
                // The SSPRK3 stage fused into the flux launch, as gbns_ssprk3_step
                // issues it, with R[2] as the second state buffer:
                //   stage 0: q    -> R0, q1 into R[2]
                //   stage 1: R[2] -> R1, q2 into q
                //   stage 2: q    -> (no store), q3 into R[2]  (copied back by the ghost pass)
                // coefficients: ratio_diff of consecutive ssprk3_t rows times dt
                // (advance.h:80-95).
                const double dt = I.dt;
                FluxArgs& A = arg.A;
                A.increment = 0;
                A.ntile[0] = (I.G.n[0] + Cfg::TX - 1)/Cfg::TX;
                A.ntile[1] = (I.G.n[1] + Cfg::TY - 1)/Cfg::TY;
                A.ntile[2] = (I.G.n[2] + Cfg::TZ - 1)/Cfg::TZ;
                // FP64 tiles stage their box by TMA from the instance's tensor
                // map of the array this stage reads (tmaps[2 inst]: q,
                // tmaps[2 inst + 1]: R[2]); items the host marked (w.pad) only
                A.use_tma = (!Cfg::DIRECT && tmaps != nullptr && w.pad) ? 1 : 0;
                A.sh_off = 0;
                A.blk_inv_dx = nullptr;
                arg.tmap = A.use_tma ? tmaps + 2*w.inst + (stage == 1 ? 1 : 0) : nullptr;
                A.rk_nres = stage + 1;
                A.rk_res[0] = I.R[0];
                A.rk_res[1] = I.R[1];
                A.rk_coeff[0] = A.rk_coeff[1] = A.rk_coeff[2] = 0.0;
                if (stage == 0)
                {
                    A.prims = I.q; A.rhs = I.R[0]; A.write_rhs = 1; A.q_out = I.R[2];
                    A.rk_coeff[0] = (1.0/1.0)*dt;
                }
                else if (stage == 1)
                {
                    A.prims = I.R[2]; A.rhs = I.R[1]; A.write_rhs = 1; A.q_out = I.q;
                    A.rk_coeff[0] = (-3.0/4.0)*dt; A.rk_coeff[1] = (1.0/4.0)*dt;
                }
                else
                {
                    A.prims = I.q; A.rhs = nullptr; A.write_rhs = 0; A.q_out = I.R[2];
                    A.rk_coeff[0] = (-1.0/12.0)*dt; A.rk_coeff[1] = (-1.0/12.0)*dt; A.rk_coeff[2] = (2.0/3.0)*dt;
                }
                arg.ytab = I.ytab >= 0 ? ytabs + I.ytab : nullptr;
                arg.lb = w.lb;
                arg.tile = w.tile;
            }
            __syncthreads();
            // the map was written to global memory by a host copy: acquire it
            // for the tensor proxy before the thread that issues the copy uses it
            if (threadIdx.x == 0 && arg.tmap) tensormap_acquire(arg.tmap);
            if constexpr (Cfg::STRETCH) flux_tile<Cfg>(smem_raw, arg.tmap, arg.G, *arg.ytab, arg.S, arg.A, arg.lb, arg.tile);
            else flux_tile<Cfg>(smem_raw, arg.tmap, arg.G, YTabNone{}, arg.S, arg.A, arg.lb, arg.tile);
        }

        // The launch of one class and stage (an action of batch_dispatch).
        struct LaunchAction
        {
            const TileItem* items; const int* offsets; const int* counts; const InstK* insts;
            const YTabK* ytabs; const long long* left; const CUtensorMap* tmaps;
            int cls, stage, nitems; cudaStream_t st;
            template <class Cfg> int run() const
            {
                if (nitems <= 0) return GBNS_OK;
                auto kern = flux_batch_kernel<Cfg>;
                int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         int(Cfg::SMEM_BYTES)), "flux_batch smem attribute");
                if (rc) return rc;
                kern<<<unsigned(nitems), Cfg::NT, Cfg::SMEM_BYTES, st>>>(items, offsets, counts, insts, ytabs, left,
                                                                         tmaps, cls, stage);
                return check_cuda(cudaGetLastError(), "flux_batch launch");
            }
        };
        // The TMA box of a variant's FP64 staging (cells along x, y, z), for
        // the tensor maps the host encodes; 0 when the variant stages no FP64
        // box by TMA.
        struct BoxAction
        {
            int* box;
            template <class Cfg> int run() const
            {
                const bool tma = !Cfg::DIRECT && !Cfg::SHADOW && Cfg::FP64;
                box[0] = tma ? Cfg::BXE : 0;
                box[1] = tma ? Cfg::BY : 0;
                box[2] = tma ? Cfg::BZ : 0;
                return GBNS_OK;
            }
        };
    }

#define GBNS_BRUN(CONV, ORDER, STRETCH, TX, TY, TZ, NT) \
    return act.template run<FluxCfg<GBNS_REAL, CONV, ORDER, STRETCH, TX, TY, TZ, NT, GBNS_TAG, GBNS_FP32>>()

    namespace
    {
    // The tile variants of each class (their shapes are listed by
    // batch_class_tile in batch.cu, in the same order); a new batch starts
    // on variant 0 in FP32-flux and on variant 2 (576 threads) in FP64.
    // Runs the action with the variant's tile configuration.
    template <class Act>
    int batch_dispatch(int cls, int v, const Act& act)
    {
#if GBNS_BATCH_GROUP == 0
        switch (cls)
        {
            case BCLASS_CK2_ID:
                if (v == 1) GBNS_BRUN(GBNS_CONV_CENT_KEEP, 2, false, 8, 8, 4, 128);
                if (v == 2) GBNS_BRUN(GBNS_CONV_CENT_KEEP, 2, false, 8, 8, 8, (GBNS_FP32 ? 512 : 576));
                GBNS_BRUN(GBNS_CONV_CENT_KEEP, 2, false, 8, 8, 8, 256);
            case BCLASS_TOTANI_ID:
                if (v == 1) GBNS_BRUN(GBNS_CONV_TOTANI, 2, false, 8, 8, 4, 128);
                if (v == 2) GBNS_BRUN(GBNS_CONV_TOTANI, 2, false, 8, 8, 8, (GBNS_FP32 ? 512 : 576));
                GBNS_BRUN(GBNS_CONV_TOTANI, 2, false, 8, 8, 8, 256);
            case BCLASS_FWENO_ID:
                if (v == 1) GBNS_BRUN(GBNS_CONV_FWENO, 2, false, 8, 8, 4, 128);
                if (v == 2) GBNS_BRUN(GBNS_CONV_FWENO, 2, false, 8, 8, 8, (GBNS_FP32 ? 512 : 576));
                GBNS_BRUN(GBNS_CONV_FWENO, 2, false, 8, 8, 8, 256);
        }
#elif GBNS_BATCH_GROUP == 1
        switch (cls)
        {
#if GBNS_FP32
            case BCLASS_WENO5_ST:
                if (v == 1) GBNS_BRUN(GBNS_CONV_WENO5, 2, true, 8, 8, 8, 256);
                if (v == 2) GBNS_BRUN(GBNS_CONV_WENO5, 2, true, 8, 8, 8, 512);
                GBNS_BRUN(GBNS_CONV_WENO5, 2, true, 8, 8, 4, 256);
            case BCLASS_WENO5_ID:
                if (v == 1) GBNS_BRUN(GBNS_CONV_WENO5, 2, false, 8, 8, 8, 256);
                if (v == 2) GBNS_BRUN(GBNS_CONV_WENO5, 2, false, 8, 8, 8, 512);
                GBNS_BRUN(GBNS_CONV_WENO5, 2, false, 8, 8, 4, 256);
#else
            case BCLASS_WENO5_ST:
                if (v == 1) GBNS_BRUN(GBNS_CONV_WENO5, 2, true, 8, 8, 4, 256);
                if (v == 2) GBNS_BRUN(GBNS_CONV_WENO5, 2, true, 8, 8, 8, 576);
                GBNS_BRUN(GBNS_CONV_WENO5, 2, true, 8, 8, 8, 256);
            case BCLASS_WENO5_ID:
                if (v == 1) GBNS_BRUN(GBNS_CONV_WENO5, 2, false, 8, 8, 4, 256);
                if (v == 2) GBNS_BRUN(GBNS_CONV_WENO5, 2, false, 8, 8, 8, 576);
                GBNS_BRUN(GBNS_CONV_WENO5, 2, false, 8, 8, 8, 256);
#endif
        }
#else
        switch (cls)
        {
            case BCLASS_HYB2_ID:
                if (v == 1) GBNS_BRUN(GBNS_CONV_HYBRID, 2, false, 8, 8, 8, 256);
#if !GBNS_FP32
                if (v == 2) GBNS_BRUN(GBNS_CONV_HYBRID, 2, false, 8, 8, 8, 576);
#endif
                GBNS_BRUN(GBNS_CONV_HYBRID, 2, false, 8, 8, 4, 256);
        }
#endif
        return set_error(GBNS_ERR_UNSUPPORTED, "no batched kernel for this class");
    }
    }
#undef GBNS_BRUN

    int GBNS_BATCH_FN(int cls, int v, const TileItem* items, const int* offsets, const int* counts,
                      const InstK* insts, const YTabK* ytabs, const long long* left, const CUtensorMap* tmaps,
                      int stage, int nitems, cudaStream_t st)
    {
        return batch_dispatch(cls, v, LaunchAction{items, offsets, counts, insts, ytabs, left, tmaps, cls, stage, nitems, st});
    }

    int GBNS_BATCH_BOX_FN(int cls, int v, int box[3])
    {
        return batch_dispatch(cls, v, BoxAction{box});
    }
}
