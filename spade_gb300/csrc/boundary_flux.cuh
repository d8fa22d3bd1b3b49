// pde_algs::boundary_flux (pde-algs/boundary_flux.h:16-105): the flux of the
// faces on selected domain boundaries, added to the two cells each face
// separates (the interior cell and the ghost cell beyond it):
//     rhs(il) -= jac_l*F/dx;   rhs(ir) += jac_r*F/dx
// with F the face flux flux_div evaluates (the same face_flux code), dx the
// block's spacing along the face normal and jac = 1 (identity coordinates).
// As in the reference's loop, the faces of a boundary plane span transverse
// cell indices -1 .. n-1, so the ghost row below each transverse direction is
// included, and the six boundaries are applied in order xmin, xmax, ymin,
// ymax, zmin, zmax (one launch each: cells on a plane edge are touched by two
// boundaries).
//
// One CTA evaluates an 8x8 patch of faces of one boundary plane of one block
// from a box one cell thick along the normal (plus the stencil halo), staged
// with plain loads that bounds-check every cell (the patch starts in the
// ghost row; cells outside the padded block read as zero and feed no face
// that is written).  FP64 without FMA contraction, like the drop-in.
#pragma once
#include "flux_kernel.cuh"

namespace gbns
{
    template <int D> struct BndDirs
    {
        static constexpr int A = D == 0 ? 1 : 0;   // first transverse direction
        static constexpr int B = D == 2 ? 1 : 2;   // second transverse direction
    };

    // Tile of one cell along D and 8x8 across: faces 0 and 1 along D are the
    // min- and max-side faces of that cell.
    template <int CONV, int ORDER, int D, int TAG>
    using BndCfg = FluxCfg<double, CONV, ORDER, false, D == 0 ? 1 : 8, D == 1 ? 1 : 8, D == 2 ? 1 : 8, 64, TAG, 0>;

    template <class Cfg, int D>
    __global__ void __launch_bounds__(Cfg::NT)
    boundary_flux_kernel(const __grid_constant__ GeomK G, const __grid_constant__ SchemeK SK, const __grid_constant__ BndArgs A)
    {
        static_assert(Cfg::FP64 && !Cfg::STRETCH && Cfg::NCELL == Cfg::NT, "one face per thread, identity coordinates");
        extern __shared__ __align__(128) unsigned char smem_raw[];
        constexpr int TX = Cfg::TX, TY = Cfg::TY, H = Cfg::H;
        constexpr int TA = BndDirs<D>::A, TB = BndDirs<D>::B;
        double* stage = reinterpret_cast<double*>(smem_raw + 128);
        double* der = reinterpret_cast<double*>(smem_raw + 128 + Cfg::STAGE_BYTES);
        const int tid = threadIdx.x;

        // block on this boundary and the patch's transverse position
        const int t1 = blockIdx.x % A.ntile1, t2 = blockIdx.x / A.ntile1;
        int b[3];
        b[D] = A.side ? G.nb[D] - 1 : 0;
        b[TA] = blockIdx.y % G.nb[TA];
        b[TB] = blockIdx.y / G.nb[TA];
        const int lb = b[0] + G.nb[0]*(b[1] + G.nb[1]*b[2]);
        int o[3];                                   // tile origin, interior cell coordinates
        o[D] = A.side ? G.n[D] - 1 : 0;
        o[TA] = 8*t1 - 1;
        o[TB] = 8*t2 - 1;

        // ---- stage the box (same geometry and x-shift convention as flux_tile)
        const int px = o[0] - H + G.ng;
        const int xs = px & ~1;
        const int shift = px - xs;
        const int ys = o[1] - H + G.ng, zs = o[2] - H + G.ng;
        const double* base = A.prims + (long long)lb*G.bstride;
        for (int e = tid; e < Cfg::BOXN; e += Cfg::NT)
        {
            const int bx = e % Cfg::BXE, by = (e / Cfg::BXE) % Cfg::BY, bz = e / (Cfg::BXE*Cfg::BY);
            const int X = xs + bx, Y_ = ys + by, Z = zs + bz;
            if (X >= 0 && X < G.ni && Y_ >= 0 && Y_ < G.nj && Z >= 0 && Z < G.nk)
            {
                const double* src = base + ((long long)(Z*G.nj + Y_)*G.ni + X)*5;
                #pragma unroll
                for (int v = 0; v < 5; ++v) stage[e*5 + v] = src[v];
            }
            else
            {
                #pragma unroll
                for (int v = 0; v < 5; ++v) stage[e*5 + v] = 0.0;
            }
        }
        __syncthreads();

        BoxView<Cfg> V;
        V.stage = stage;
        V.soa = nullptr;
        V.split = der;
        V.ymet = nullptr;
        double* dder = der;
        if constexpr (Cfg::SPLIT) dder = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(der) + Cfg::SPLIT_BYTES);
        V.der = dder;
        SchemeR<double> S;
        S.load(SK);

        if constexpr (Cfg::NDERB > 0)
        {
            constexpr int HC = Cfg::HC, TZ = Cfg::TZ;
            for (int c = tid; c < Cfg::BOXN; c += Cfg::NT)
            {
                const int bx = c % Cfg::BXE, by = (c / Cfg::BXE) % Cfg::BY, bz = c / (Cfg::BXE*Cfg::BY);
                const int rx = bx - shift - H, ry = by - H, rz = bz - H;
                const bool inx = rx >= 0 && rx < TX, iny = ry >= 0 && ry < TY, inz = rz >= 0 && rz < TZ;
                const bool need = (iny && inz && rx >= -HC && rx < TX + HC) ||
                                  (inx && inz && ry >= -HC && ry < TY + HC) ||
                                  (inx && iny && rz >= -HC && rz < TZ + HC);
                if (need) derive_cell<Cfg>(V, dder, S, c);
            }
            __syncthreads();
        }

        double inv[3];
        #pragma unroll
        for (int d = 0; d < 3; ++d) inv[d] = G.inv_dx[d][b[d]];

        // this thread's tile cell and face
        const int cx = tid % TX, cy = (tid / TX) % TY, cz = tid / (TX*TY);
        if constexpr (Cfg::SPLIT)
        {
            double dc[Cfg::CPT][3];
            const int c = (cz + H)*Cfg::SZ + (cy + H)*Cfg::SY + (cx + H + shift);
            fweno_derive<double>(S, V.q(0, c), V.q(1, c), V.q(2, c), V.q(3, c), V.q(4, c), dc[0][0], dc[0][1], dc[0][2]);
            split_fill<Cfg, D>(V, S, der, YTabNone{}, b[1], o[1], G.n[1], shift, dc);
            __syncthreads();
        }
        int fc[3] = {cx, cy, cz};
        fc[D] = A.side;                             // face 0: min side of the cell, face 1: max side
        int il[3] = {o[0] + cx, o[1] + cy, o[2] + cz};
        il[D] = A.side ? G.n[D] - 1 : -1;
        if (il[TA] >= G.n[TA] || il[TB] >= G.n[TB]) return;
        double F[5];
        const int rc = (fc[2] + H)*Cfg::SZ + (fc[1] + H)*Cfg::SY + (fc[0] + H + shift);
        face_flux<Cfg, D>(V, S, rc, SplitIdx<Cfg, D>::right(fc[0], fc[1], fc[2]), 1.0, inv, 1.0, F);

        // rhs(il) -= jac_l*accum/dx; rhs(ir) += jac_r*accum/dx with accum = 0 + F
        // (boundary_flux.h:76-99)
        int ir[3] = {il[0], il[1], il[2]};
        ir[D] += 1;
        double* rl = A.rhs + (long long)lb*G.bstride +
                     ((long long)((il[2] + G.ng)*G.nj + (il[1] + G.ng))*G.ni + (il[0] + G.ng))*5;
        double* rr = A.rhs + (long long)lb*G.bstride +
                     ((long long)((ir[2] + G.ng)*G.nj + (ir[1] + G.ng))*G.ni + (ir[0] + G.ng))*5;
        const double dx = A.dx[b[D]];
        const double jac = 1.0;
        #pragma unroll
        for (int v = 0; v < 5; ++v)
        {
            double acc = 0.0;
            acc += F[v];
            rl[v] = rl[v] - (jac*acc)/dx;
            rr[v] = rr[v] + (jac*acc)/dx;
        }
    }

    template <class Cfg, int D>
    int run_boundary_flux(const GeomK& G, const SchemeK& S, const BndArgs& A, cudaStream_t st)
    {
        auto kern = boundary_flux_kernel<Cfg, D>;
        int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(Cfg::SMEM_BYTES)),
                            "boundary_flux smem attribute");
        if (rc) return rc;
        const dim3 grid(unsigned(A.ntile1*A.ntile2), unsigned(G.nb[BndDirs<D>::A]*G.nb[BndDirs<D>::B]));
        kern<<<grid, Cfg::NT, Cfg::SMEM_BYTES, st>>>(G, S, A);
        return check_cuda(cudaGetLastError(), "boundary_flux launch");
    }
}
