// Point source terms: rhs += S(q)/jac on every interior cell
// (pde_algs::source_term, pde-algs/source_term.h:19-51).
//
// One thread per interior cell, grid-stride over all blocks; the cell's 5
// primitives and 5 residual doubles are contiguous (AoS5), so a warp reads
// and writes 32 consecutive 40-byte cells.  HBM traffic per cell: 40 B of
// prims read, 40 B of rhs read and 40 B written.  Compiled without FMA
// contraction so the arithmetic rounds like the reference's CPU loop.
#include <cstring>
#include "gbns_internal.cuh"

namespace gbns
{
    namespace
    {
        struct SourceK
        {
            int kind;
            int stretch;
            double c[5];
            double R;
            double im_cell[MAX_YTAB];   // Jacobian per y row (stretched-y grids)
        };

        __global__ void __launch_bounds__(256)
        source_term_kernel(const double* __restrict__ q, double* __restrict__ rhs,
                           const __grid_constant__ GeomK G, const __grid_constant__ SourceK K)
        {
            const long long ncell = (long long)G.n[0]*G.n[1]*G.n[2];
            const long long total = ncell*G.nblk;
            for (long long idx = blockIdx.x*(long long)blockDim.x + threadIdx.x; idx < total;
                 idx += (long long)gridDim.x*blockDim.x)
            {
                const int lb = int(idx / ncell);
                const long long rem = idx - lb*ncell;
                const int k_ = int(rem / ((long long)G.n[0]*G.n[1]));
                const int j_ = int((rem / G.n[0]) % G.n[1]);
                const int i_ = int(rem % G.n[0]);
                const long long off = (long long)lb*G.bstride +
                    ((long long)((k_ + G.ng)*G.nj + (j_ + G.ng))*G.ni + (i_ + G.ng))*5;
                const double* w = q + off;
                double s[5];
                if (K.kind == GBNS_SOURCE_CONST)
                {
                    for (int v = 0; v < 5; ++v) s[v] = K.c[v];
                }
                else
                {
                    const double u = w[2], v = w[3], ww = w[4];
                    double fu = K.c[2]*u;
                    fu += K.c[3]*v;
                    fu += K.c[4]*ww;
                    if (K.kind == GBNS_SOURCE_BODY_FORCE)
                    {
                        s[0] = 0.0; s[1] = fu; s[2] = K.c[2]; s[3] = K.c[3]; s[4] = K.c[4];
                    }
                    else
                    {
                        const double rho = w[0]/(K.R*w[1]);
                        s[0] = 0.0; s[1] = rho*fu; s[2] = rho*K.c[2]; s[3] = rho*K.c[3]; s[4] = rho*K.c[4];
                    }
                }
                // calc_jacobian at the cell (identity: 1)
                double jac = 1.0;
                if (K.stretch)
                {
                    const int by = (lb / G.nb[0]) % G.nb[1];
                    jac = K.im_cell[by*G.n[1] + j_];
                }
                double* r = rhs + off;
                #pragma unroll
                for (int v = 0; v < 5; ++v) r[v] = r[v] + s[v]/jac;
            }
        }
    }
}

extern "C"
{
    int gbns_source_term(const gbns_grid_desc* grid, const gbns_source_desc* source,
                         const double* prims, double* rhs, void* stream)
    {
        using namespace gbns;
        GeomK G;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        if (!source) return set_error(GBNS_ERR_INVALID, "source descriptor is NULL");
        if (source->kind < GBNS_SOURCE_CONST || source->kind > GBNS_SOURCE_BODY_ACCEL)
            return set_error(GBNS_ERR_INVALID, "unknown source term kind");
        if (source->kind == GBNS_SOURCE_BODY_ACCEL && !(source->gas.R > 0.0))
            return set_error(GBNS_ERR_INVALID, "body acceleration needs the gas constant R > 0");
        if (!prims || !rhs) return set_error(GBNS_ERR_INVALID, "NULL pointer");
        SourceK K;
        std::memset(&K, 0, sizeof(K));
        K.kind = source->kind;
        for (int v = 0; v < 5; ++v) K.c[v] = source->c[v];
        K.R = source->gas.R;
        K.stretch = grid->coords != GBNS_COORDS_IDENTITY;
        if (K.stretch)
        {
            YTabK Y;
            rc = make_ytab(grid, G, Y);
            if (rc) return rc;
            std::memcpy(K.im_cell, Y.im_cell, sizeof(K.im_cell));
        }
        const long long total = (long long)G.n[0]*G.n[1]*G.n[2]*G.nblk;
        if (total == 0) return GBNS_OK;
        long long want = (total + 255)/256;
        const long long cap = (long long)sm_count()*16;
        if (want > cap) want = cap;
        source_term_kernel<<<unsigned(want), 256, 0, static_cast<cudaStream_t>(stream)>>>(prims, rhs, G, K);
        return check_cuda(cudaGetLastError(), "source_term launch");
    }
}
