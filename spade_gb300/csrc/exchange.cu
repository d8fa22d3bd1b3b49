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
// cell counts.  Every destination is a ghost cell written once (checked when
// the plan is created).  A donor may be a ghost cell that another
// transaction of the same kind writes (a coarse block's ghost layer feeding
// the interpolation into a finer neighbour): the reference executes the
// transactions one after the other, so such a donor holds the new value if
// its writer comes earlier in the plan and the old one if it comes later.
// The plan is therefore split into waves: a transaction runs in a later wave
// than every earlier writer of its donors, and in an earlier wave than every
// later writer; the transactions of one wave are independent and each wave
// is one launch.  HBM-bound gather: 80 bytes per injected cell, 40 x 9 per
// interpolated one.  The arithmetic follows the reference's:
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
    // one launch per wave: injection waves, then interpolation waves
    struct Wave
    {
        bool interp;
        int p0, np;             // its transactions in d_patches
        long long f0;           // its np+1 prefix sums in d_first
        long long cells;
    };
    std::vector<Wave> waves;
    PatchK* d_patches = nullptr;
    long long* d_first = nullptr;
};

namespace
{
    // donor index along one direction for destination offset d (the
    // interpolation's two donors: base and base + i_incr)
    int donor_base(int d, int coeff) { return (d << (coeff + 1)) >> 1; }

    // Visits the donor cells of every destination cell of patch p (padded
    // indices relative to the donor block's interior origin).
    template <class F>
    void for_each_donor(const gbns_patch& p, F&& f)
    {
        const int ext[3] = {p.dst_hi[0] - p.dst_lo[0], p.dst_hi[1] - p.dst_lo[1], p.dst_hi[2] - p.dst_lo[2]};
        for (int dk = 0; dk < ext[2]; ++dk)
            for (int dj = 0; dj < ext[1]; ++dj)
                for (int di = 0; di < ext[0]; ++di)
                {
                    if (p.kind == GBNS_PATCH_INJECT)
                    {
                        f(p.src_lo[0] + di, p.src_lo[1] + dj, p.src_lo[2] + dk);
                        continue;
                    }
                    const int b[3] = {donor_base(di, p.i_coeff[0]), donor_base(dj, p.i_coeff[1]), donor_base(dk, p.i_coeff[2])};
                    for (int iv = 0; iv < 8; ++iv)
                        f(p.src_lo[0] + b[0] + (iv & 1)*p.i_incr[0], p.src_lo[1] + b[1] + ((iv >> 1) & 1)*p.i_incr[1],
                          p.src_lo[2] + b[2] + ((iv >> 2) & 1)*p.i_incr[2]);
                }
    }

    int validate_patch(const gbns_exchange_plan& P, const gbns_patch& p, int index, std::vector<int>& writer,
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
            if (lo < -ng || hi >= n[d] + ng) { why = "donor box not inside the donor block's padded array"; return 1; }
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
                    if (writer[c] >= 0) { why = "two patches write the same ghost cell"; return 1; }
                    writer[c] = index;
                }
        return 0;
    }

    // Wave of every patch of one kind, in plan order (see the file comment):
    // wave(t) > wave(w) for an earlier writer w of one of t's donors, and
    // wave(w) > wave(t) for a later one.  Returns 1 (why set) if a patch
    // reads a cell it writes itself.
    int assign_waves(const gbns_exchange_plan& P, const gbns_patch* patches, int npatch, int kind,
                     const std::vector<int>& writer, std::vector<int>& wave, std::string& why)
    {
        const long long ni = P.G.ni, nj = P.G.nj, nk = P.G.nk;
        const int ng = P.G.ng;
        std::vector<int> pending(npatch, 0);
        std::vector<int> later;
        for (int t = 0; t < npatch; ++t)
        {
            const gbns_patch& p = patches[t];
            if (p.kind != kind) continue;
            int w0 = pending[t];
            bool self = false;
            later.clear();
            for_each_donor(p, [&](int i, int j, int k) {
                const long long c = (long long)p.src_block*ni*nj*nk + ((k + ng)*nj + (j + ng))*ni + (i + ng);
                const int w = writer[c];
                if (w < 0 || patches[w].kind != kind) return;
                if (w == t) self = true;
                else if (w < t) { if (wave[w] + 1 > w0) w0 = wave[w] + 1; }
                else later.push_back(w);
            });
            if (self) { why = "patch " + std::to_string(t) + " reads a ghost cell it writes"; return 1; }
            wave[t] = w0;
            for (int w : later)
                if (pending[w] < w0 + 1) pending[w] = w0 + 1;
        }
        return 0;
    }

    // Validates a plan and assigns every patch its wave (host only).
    int plan_waves(gbns_exchange_plan& P, int nx, int ny, int nz, int ng, int nblocks, const gbns_patch* patches,
                   int npatch, std::vector<int>& wave)
    {
        if (npatch > 0 && !patches) return set_error(GBNS_ERR_INVALID, "NULL argument");
        if (nx < 1 || ny < 1 || nz < 1 || ng < 1 || ng > 8 || nblocks < 1 || npatch < 0)
            return set_error(GBNS_ERR_INVALID, "exchange plan: bad block shape, ghost depth or counts");
        P.nx = nx; P.ny = ny; P.nz = nz; P.nblocks = nblocks;
        P.G.ng = ng;
        P.G.ni = nx + 2*ng; P.G.nj = ny + 2*ng; P.G.nk = nz + 2*ng;
        P.G.bstride = 5ll*P.G.ni*P.G.nj*P.G.nk;
        std::vector<int> writer(size_t(nblocks)*P.G.ni*P.G.nj*P.G.nk, -1);
        for (int i = 0; i < npatch; ++i)
        {
            std::string why;
            if (validate_patch(P, patches[i], i, writer, why))
                return set_error(GBNS_ERR_INVALID, "exchange plan, patch " + std::to_string(i) + ": " + why);
        }
        wave.assign(npatch, 0);
        for (int kind : {GBNS_PATCH_INJECT, GBNS_PATCH_INTERP})
        {
            std::string why;
            if (assign_waves(P, patches, npatch, kind, writer, wave, why))
                return set_error(GBNS_ERR_UNSUPPORTED, "exchange plan: " + why);
        }
        return GBNS_OK;
    }
}

extern "C"
{
    int gbns_exchange_plan_create(gbns_exchange_plan** out, int nx, int ny, int nz, int ng, int nblocks,
                                  const gbns_patch* patches, int npatch, void* stream)
    {
        if (!out || (npatch > 0 && !patches)) return set_error(GBNS_ERR_INVALID, "NULL argument");
        auto* P = new gbns_exchange_plan();
        std::vector<int> wave;
        int rc = plan_waves(*P, nx, ny, nz, ng, nblocks, patches, npatch, wave);
        if (rc) { delete P; return rc; }
        // injection waves, then interpolation waves; plan order within a wave
        std::vector<int> order(npatch);
        for (int i = 0; i < npatch; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            const int ka = patches[a].kind == GBNS_PATCH_INTERP, kb = patches[b].kind == GBNS_PATCH_INTERP;
            if (ka != kb) return ka < kb;
            return wave[a] < wave[b];
        });
        std::vector<PatchK> all;
        std::vector<long long> first;
        all.reserve(npatch);
        for (int oi = 0; oi < npatch; ++oi)
        {
            const int i = order[oi];
            const gbns_patch& p = patches[i];
            const bool interp = p.kind == GBNS_PATCH_INTERP;
            if (P->waves.empty() || P->waves.back().interp != interp || wave[order[oi - 1]] != wave[i])
            {
                if (!P->waves.empty()) first.push_back(P->waves.back().cells);
                P->waves.push_back({interp, int(all.size()), 0, (long long)first.size(), 0});
            }
            gbns_exchange_plan::Wave& W = P->waves.back();
            PatchK k;
            std::memset(&k, 0, sizeof(k));
            k.src_block = p.src_block;
            k.dst_block = p.dst_block;
            for (int d = 0; d < 3; ++d)
            {
                k.src_lo[d] = p.src_lo[d];
                k.dst_lo[d] = p.dst_lo[d];
                k.ext[d] = p.dst_hi[d] - p.dst_lo[d];
                k.i_coeff[d] = interp ? p.i_coeff[d] : 0;
                k.i_incr[d] = interp ? p.i_incr[d] : 0;
            }
            all.push_back(k);
            first.push_back(W.cells);
            W.np += 1;
            W.cells += (long long)k.ext[0]*k.ext[1]*k.ext[2];
            (interp ? P->n_int : P->n_inj) += 1;
        }
        if (!P->waves.empty()) first.push_back(P->waves.back().cells);
        if (first.empty()) first.push_back(0);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        rc = check_cuda(cudaMalloc(&P->d_patches, sizeof(PatchK)*(all.size() ? all.size() : 1)), "exchange plan");
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

    int gbns_exchange_plan_waves(int nx, int ny, int nz, int ng, int nblocks, const gbns_patch* patches, int npatch,
                                 int* waves)
    {
        if (!waves && npatch > 0) return set_error(GBNS_ERR_INVALID, "NULL argument");
        gbns_exchange_plan P;
        std::vector<int> wave;
        const int rc = plan_waves(P, nx, ny, nz, ng, nblocks, patches, npatch, wave);
        if (rc) return rc;
        for (int i = 0; i < npatch; ++i) waves[i] = wave[i];
        return GBNS_OK;
    }

    int gbns_exchange_plan_run(gbns_exchange_plan* P, double* prims, void* stream)
    {
        if (!P || !prims) return set_error(GBNS_ERR_INVALID, "NULL argument");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const long long cap = (long long)sm_count()*8;
        for (const auto& W : P->waves)
        {
            if (W.cells <= 0) continue;
            long long nb = (W.cells + 255)/256;
            if (nb > cap) nb = cap;
            if (W.interp)
                exchange_plan_kernel<true><<<unsigned(nb), 256, 0, st>>>(prims, P->d_patches + W.p0, P->d_first + W.f0,
                                                                        W.np, P->G);
            else
                exchange_plan_kernel<false><<<unsigned(nb), 256, 0, st>>>(prims, P->d_patches + W.p0, P->d_first + W.f0,
                                                                         W.np, P->G);
            int rc = check_cuda(cudaGetLastError(), W.interp ? "exchange plan launch (interpolations)"
                                                             : "exchange plan launch (injections)");
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

namespace gbns
{
    int exchange_plan_shape(const gbns_exchange_plan* P, int* nx, int* ny, int* nz, int* ng, int* nblocks)
    {
        if (!P) return set_error(GBNS_ERR_INVALID, "exchange plan is NULL");
        *nx = P->nx; *ny = P->ny; *nz = P->nz; *ng = P->G.ng; *nblocks = P->nblocks;
        return GBNS_OK;
    }
}

namespace gbns
{
    namespace
    {
        // The wall fill of one domain face on a refined layout, for the blocks
        // listed (their boxes touch that face): every ghost cell of the face's
        // slab (ng layers, the full padded extent across) takes the mirrored
        // cell of its own block (boundary_fill.h:107-124): isothermal no-slip
        // T -> 2 T_w - T and the velocity negated, slip the normal component
        // negated.  The mirrored cells are interior along the face normal, so
        // no cell read is written by the launch.
        __global__ void wall_fill_blocks_kernel(double* q, PlanGeom G, int n0, int n1, int n2,
                                                const int* __restrict__ blocks, int nlist, int face, int kind,
                                                double t_wall)
        {
            const int d = face/2, hi = face % 2;
            const int n[3] = {n0, n1, n2};
            const long long per = (long long)G.ng*(d == 0 ? (long long)G.nj*G.nk : (d == 1 ? (long long)G.ni*G.nk
                                                                                           : (long long)G.ni*G.nj));
            const long long total = per*nlist;
            for (long long t = blockIdx.x*(long long)blockDim.x + threadIdx.x; t < total;
                 t += (long long)gridDim.x*blockDim.x)
            {
                const int lb = blocks[t/per];
                long long r = t % per;
                int p[3];
                if (d == 0) { p[0] = int(r % G.ng); r /= G.ng; p[1] = int(r % G.nj); p[2] = int(r / G.nj); }
                else if (d == 1) { p[0] = int(r % G.ni); r /= G.ni; p[1] = int(r % G.ng); p[2] = int(r / G.ng); }
                else { p[0] = int(r % G.ni); r /= G.ni; p[1] = int(r % G.nj); p[2] = int(r / G.nj); }
                const int c = hi ? n[d] + p[d] : p[d] - G.ng;          // ghost cell, interior-relative
                const int img = hi ? 2*n[d] - (c + 1) : -1 - c;        // its mirror (interior along d)
                int src[3] = {p[0], p[1], p[2]}, dst[3] = {p[0], p[1], p[2]};
                src[d] = img + G.ng;
                dst[d] = c + G.ng;
                const double* s = q + (long long)lb*G.bstride + ((long long)(src[2]*G.nj + src[1])*G.ni + src[0])*5;
                double v[5];
                #pragma unroll
                for (int k = 0; k < 5; ++k) v[k] = s[k];
                if (kind == GBNS_BC_ISOTHERMAL_NOSLIP)
                {
                    v[1] = 2.0*t_wall - v[1];
                    v[2] = -v[2]; v[3] = -v[3]; v[4] = -v[4];
                }
                else v[2 + d] = -v[2 + d];
                double* o = q + (long long)lb*G.bstride + ((long long)(dst[2]*G.nj + dst[1])*G.ni + dst[0])*5;
                #pragma unroll
                for (int k = 0; k < 5; ++k) o[k] = v[k];
            }
        }
    }

    int wall_lists(const gbns_grid_desc* g, const double* boxes, const gbns_bc_desc* bc, WallLists& W)
    {
        W.idx.clear();
        for (int f = 0; f < 7; ++f) W.off[f] = 0;
        for (int f = 0; f < 6; ++f)
        {
            W.off[f] = int(W.idx.size());
            const int kind = bc->kind[f];
            if (kind != GBNS_BC_ISOTHERMAL_NOSLIP && kind != GBNS_BC_SLIP_ADIABATIC) continue;
            const int d = f/2;
            if (g->ncell[d] < g->ng)
                return set_error(GBNS_ERR_UNSUPPORTED, "wall fill needs at least ng cells per block across a wall");
            for (int lb = 0; lb < g->nblk[0]; ++lb)
            {
                const double v = boxes[6*lb + f], wall = g->bounds[f];
                if (v == wall) W.idx.push_back(lb);
            }
        }
        W.off[6] = int(W.idx.size());
        return GBNS_OK;
    }

    int launch_wall_fill(const gbns_grid_desc* g, const gbns_bc_desc* bc, const WallLists& W, const int* d_idx,
                         double* prims, cudaStream_t st)
    {
        PlanGeom G;
        G.ni = g->ncell[0] + 2*g->ng;
        G.nj = g->ncell[1] + 2*g->ng;
        G.nk = g->ncell[2] + 2*g->ng;
        G.ng = g->ng;
        G.bstride = 5ll*G.ni*G.nj*G.nk;
        for (int f = 0; f < 6; ++f)
        {
            const int nlist = W.off[f + 1] - W.off[f];
            if (nlist == 0) continue;
            const int d = f/2;
            const long long per = (long long)G.ng*(d == 0 ? (long long)G.nj*G.nk : (d == 1 ? (long long)G.ni*G.nk
                                                                                           : (long long)G.ni*G.nj));
            long long nb = (per*nlist + 255)/256;
            const long long cap = (long long)sm_count()*8;
            if (nb > cap) nb = cap;
            wall_fill_blocks_kernel<<<unsigned(nb), 256, 0, st>>>(prims, G, g->ncell[0], g->ncell[1], g->ncell[2],
                                                                   d_idx + W.off[f], nlist, f, bc->kind[f], bc->t_wall[f]);
            const int rc = check_cuda(cudaGetLastError(), "wall fill launch");
            if (rc) return rc;
        }
        return GBNS_OK;
    }
}
