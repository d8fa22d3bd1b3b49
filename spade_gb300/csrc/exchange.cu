// Exchange plans: the ghost fill of block layouts with refinement levels.
//
// The plan is the reference's own list of transactions (its make_exchange on
// an AMR grid, grid/make_exchange.h:98-421): injections (same-level copies of
// an equally sized donor box) and interpolations (each destination cell the
// mean of 8 donor cells, coarse-to-fine by repeating one coarse donor,
// fine-to-coarse by averaging 2x2x2 fine cells).  The reference packs every
// transaction through host-side loops and one launch per transaction type and
// rank; here the plan is uploaded once and each exchange is two launches: a
// grid-stride loop over the cells of all injections, then over the cells of
// all interpolations (the reference's order).  A thread finds its
// transaction by binary search over the prefix sums of the transactions'
// cell counts.  Every destination is a ghost cell written once and every
// donor an interior cell (checked when the plan is created), so the threads
// of a launch are independent.  HBM-bound gather: 80 bytes per injected cell,
// 40 x 9 per interpolated one.  The arithmetic follows the reference's:
// +0.0, eight additions in donor order, then x 0.125 (compiled without FMA
// contraction).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>
#include "gbns_internal.cuh"

namespace gbns
{
    namespace
    {
        struct PatchK
        {
            int src_block, dst_block;
            int src_lo[3], dst_lo[3], ext[3];
            int i_coeff[3], i_incr[3];
            int pad;
        };

        struct PlanGeom
        {
            int ni, nj, nk, ng;
            long long bstride;      // doubles per block
        };

        __device__ __forceinline__ long long cell_off(const PlanGeom& G, int lb, int i, int j, int k)
        {
            return (long long)lb*G.bstride + ((long long)((k + G.ng)*G.nj + (j + G.ng))*G.ni + (i + G.ng))*5;
        }

        template <bool INTERP>
        __global__ void __launch_bounds__(256)
        exchange_plan_kernel(double* __restrict__ q, const PatchK* __restrict__ patches,
                             const long long* __restrict__ first, const int npatch, const PlanGeom G)
        {
            const long long total = first[npatch];
            for (long long t = blockIdx.x*(long long)blockDim.x + threadIdx.x; t < total;
                 t += (long long)gridDim.x*blockDim.x)
            {
                // the transaction holding cell t: first[p] <= t < first[p+1]
                int lo = 0, hi = npatch - 1;
                while (lo < hi)
                {
                    const int mid = (lo + hi + 1) >> 1;
                    if (first[mid] <= t) lo = mid;
                    else hi = mid - 1;
                }
                const PatchK& P = patches[lo];
                const long long c = t - first[lo];
                const int di = int(c % P.ext[0]);
                const int dj = int((c / P.ext[0]) % P.ext[1]);
                const int dk = int(c / ((long long)P.ext[0]*P.ext[1]));
                double* dst = q + cell_off(G, P.dst_block, P.dst_lo[0] + di, P.dst_lo[1] + dj, P.dst_lo[2] + dk);
                if constexpr (!INTERP)
                {
                    const double* src = q + cell_off(G, P.src_block, P.src_lo[0] + di, P.src_lo[1] + dj, P.src_lo[2] + dk);
                    #pragma unroll
                    for (int v = 0; v < 5; ++v) dst[v] = src[v];
                }
                else
                {
                    const int i0 = (di << (P.i_coeff[0] + 1)) >> 1;
                    const int j0 = (dj << (P.i_coeff[1] + 1)) >> 1;
                    const int k0 = (dk << (P.i_coeff[2] + 1)) >> 1;
                    double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
                    #pragma unroll
                    for (int iv = 0; iv < 8; ++iv)
                    {
                        const int d0 = iv & 1, d1 = (iv >> 1) & 1, d2 = (iv >> 2) & 1;
                        const double* src = q + cell_off(G, P.src_block, P.src_lo[0] + i0 + d0*P.i_incr[0],
                                                         P.src_lo[1] + j0 + d1*P.i_incr[1],
                                                         P.src_lo[2] + k0 + d2*P.i_incr[2]);
                        #pragma unroll
                        for (int v = 0; v < 5; ++v) acc[v] += src[v];
                    }
                    #pragma unroll
                    for (int v = 0; v < 5; ++v) dst[v] = acc[v]*0.125;
                }
            }
        }
    }
}

using namespace gbns;

struct gbns_exchange_plan
{
    PlanGeom G;
    int nx, ny, nz, nblocks;
    int n_inj = 0, n_int = 0;
    PatchK* d_patches = nullptr;        // injections, then interpolations
    long long* d_first = nullptr;       // prefix sums: injections (n_inj+1), then interpolations (n_int+1)
    long long cells_inj = 0, cells_int = 0;
};

namespace
{
    // donor index along one direction for destination offset d (the
    // interpolation's two donors: base and base + i_incr)
    int donor_base(int d, int coeff) { return (d << (coeff + 1)) >> 1; }

    int validate_patch(const gbns_exchange_plan& P, const gbns_patch& p, std::vector<bool>& written,
                       std::string& why)
    {
        const int n[3] = {P.nx, P.ny, P.nz};
        const int ng = P.G.ng;
        if (p.kind != GBNS_PATCH_INJECT && p.kind != GBNS_PATCH_INTERP) { why = "unknown patch kind"; return 1; }
        if (p.src_block < 0 || p.src_block >= P.nblocks || p.dst_block < 0 || p.dst_block >= P.nblocks)
        { why = "block index out of range"; return 1; }
        for (int d = 0; d < 3; ++d)
        {
            if (p.dst_lo[d] < -ng || p.dst_hi[d] > n[d] + ng || p.dst_hi[d] <= p.dst_lo[d])
            { why = "destination box outside the padded block or empty"; return 1; }
            const int ext = p.dst_hi[d] - p.dst_lo[d];
            int lo, hi;
            if (p.kind == GBNS_PATCH_INJECT) { lo = p.src_lo[d]; hi = p.src_lo[d] + ext - 1; }
            else
            {
                if (p.i_coeff[d] < -1 || p.i_coeff[d] > 1 || p.i_incr[d] < 0 || p.i_incr[d] > 1)
                { why = "interpolation coefficients must be -1, 0, 1 and increments 0, 1"; return 1; }
                lo = p.src_lo[d] + donor_base(0, p.i_coeff[d]);
                hi = p.src_lo[d] + donor_base(ext - 1, p.i_coeff[d]) + p.i_incr[d];
            }
            if (lo < 0 || hi >= n[d]) { why = "donor box not inside the donor block's interior"; return 1; }
        }
        // every destination cell: a ghost cell, written by no other patch
        const long long ni = P.G.ni, nj = P.G.nj, nk = P.G.nk;
        for (int k = p.dst_lo[2]; k < p.dst_hi[2]; ++k)
            for (int j = p.dst_lo[1]; j < p.dst_hi[1]; ++j)
                for (int i = p.dst_lo[0]; i < p.dst_hi[0]; ++i)
                {
                    if (i >= 0 && i < n[0] && j >= 0 && j < n[1] && k >= 0 && k < n[2])
                    { why = "destination box covers interior cells"; return 1; }
                    const long long c = (long long)p.dst_block*ni*nj*nk + ((k + ng)*nj + (j + ng))*ni + (i + ng);
                    if (written[c]) { why = "two patches write the same ghost cell"; return 1; }
                    written[c] = true;
                }
        return 0;
    }
}

extern "C"
{
    int gbns_exchange_plan_create(gbns_exchange_plan** out, int nx, int ny, int nz, int ng, int nblocks,
                                  const gbns_patch* patches, int npatch, void* stream)
    {
        if (!out || (npatch > 0 && !patches)) return set_error(GBNS_ERR_INVALID, "NULL argument");
        if (nx < 1 || ny < 1 || nz < 1 || ng < 1 || ng > 8 || nblocks < 1 || npatch < 0)
            return set_error(GBNS_ERR_INVALID, "exchange plan: bad block shape, ghost depth or counts");
        auto* P = new gbns_exchange_plan();
        P->nx = nx; P->ny = ny; P->nz = nz; P->nblocks = nblocks;
        P->G.ng = ng;
        P->G.ni = nx + 2*ng; P->G.nj = ny + 2*ng; P->G.nk = nz + 2*ng;
        P->G.bstride = 5ll*P->G.ni*P->G.nj*P->G.nk;
        std::vector<bool> written(size_t(nblocks)*P->G.ni*P->G.nj*P->G.nk, false);
        std::vector<PatchK> inj, itp;
        for (int i = 0; i < npatch; ++i)
        {
            std::string why;
            if (validate_patch(*P, patches[i], written, why))
            {
                delete P;
                return set_error(GBNS_ERR_INVALID, "exchange plan, patch " + std::to_string(i) + ": " + why);
            }
            const gbns_patch& p = patches[i];
            PatchK k;
            std::memset(&k, 0, sizeof(k));
            k.src_block = p.src_block;
            k.dst_block = p.dst_block;
            for (int d = 0; d < 3; ++d)
            {
                k.src_lo[d] = p.src_lo[d];
                k.dst_lo[d] = p.dst_lo[d];
                k.ext[d] = p.dst_hi[d] - p.dst_lo[d];
                k.i_coeff[d] = p.kind == GBNS_PATCH_INTERP ? p.i_coeff[d] : 0;
                k.i_incr[d] = p.kind == GBNS_PATCH_INTERP ? p.i_incr[d] : 0;
            }
            (p.kind == GBNS_PATCH_INJECT ? inj : itp).push_back(k);
        }
        P->n_inj = int(inj.size());
        P->n_int = int(itp.size());
        std::vector<long long> first;
        long long acc = 0;
        for (const auto& k : inj) { first.push_back(acc); acc += (long long)k.ext[0]*k.ext[1]*k.ext[2]; }
        first.push_back(acc);
        P->cells_inj = acc;
        acc = 0;
        for (const auto& k : itp) { first.push_back(acc); acc += (long long)k.ext[0]*k.ext[1]*k.ext[2]; }
        first.push_back(acc);
        P->cells_int = acc;
        std::vector<PatchK> all(inj);
        all.insert(all.end(), itp.begin(), itp.end());
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        int rc = check_cuda(cudaMalloc(&P->d_patches, sizeof(PatchK)*(all.size() ? all.size() : 1)), "exchange plan");
        if (!rc) rc = check_cuda(cudaMalloc(&P->d_first, sizeof(long long)*first.size()), "exchange plan offsets");
        if (!rc && !all.empty())
            rc = check_cuda(cudaMemcpyAsync(P->d_patches, all.data(), sizeof(PatchK)*all.size(), cudaMemcpyHostToDevice, st),
                            "exchange plan upload");
        if (!rc) rc = check_cuda(cudaMemcpyAsync(P->d_first, first.data(), sizeof(long long)*first.size(),
                                                 cudaMemcpyHostToDevice, st), "exchange plan upload");
        if (!rc) rc = check_cuda(cudaStreamSynchronize(st), "exchange plan upload");
        if (rc)
        {
            cudaFree(P->d_patches);
            cudaFree(P->d_first);
            delete P;
            return rc;
        }
        *out = P;
        return GBNS_OK;
    }

    int gbns_exchange_plan_run(gbns_exchange_plan* P, double* prims, void* stream)
    {
        if (!P || !prims) return set_error(GBNS_ERR_INVALID, "NULL argument");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const long long cap = (long long)sm_count()*8;
        if (P->cells_inj > 0)
        {
            long long nb = (P->cells_inj + 255)/256;
            if (nb > cap) nb = cap;
            exchange_plan_kernel<false><<<unsigned(nb), 256, 0, st>>>(prims, P->d_patches, P->d_first, P->n_inj, P->G);
            int rc = check_cuda(cudaGetLastError(), "exchange plan launch (injections)");
            if (rc) return rc;
        }
        if (P->cells_int > 0)
        {
            long long nb = (P->cells_int + 255)/256;
            if (nb > cap) nb = cap;
            exchange_plan_kernel<true><<<unsigned(nb), 256, 0, st>>>(prims, P->d_patches + P->n_inj,
                                                                    P->d_first + P->n_inj + 1, P->n_int, P->G);
            int rc = check_cuda(cudaGetLastError(), "exchange plan launch (interpolations)");
            if (rc) return rc;
        }
        return GBNS_OK;
    }

    int gbns_exchange_plan_destroy(gbns_exchange_plan* P)
    {
        if (!P) return GBNS_OK;
        cudaFree(P->d_patches);
        cudaFree(P->d_first);
        delete P;
        return GBNS_OK;
    }
}
