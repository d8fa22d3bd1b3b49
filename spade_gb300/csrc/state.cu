// Ghost fill (block exchange + wall mirror), fused RK stage update and
// interior reductions.
#include <cstring>
#include <mutex>
#include <vector>
#include "gbns_internal.cuh"
#include "batch_internal.cuh"

namespace gbns
{
    // ------------------------------------------------------------------
    // ghost fill
    // ------------------------------------------------------------------

    // Fills ghost cell (ii, jj, kk) (padded indices) of block lb.  Every
    // ghost value is resolved to an INTERIOR donor cell (mirror across wall
    // faces first, boundary_fill.h:113-114, then the block exchange with
    // periodic wrap, get_transaction.h:55-87 / exchange_config.h:336-344),
    // so one launch fills every ghost layer without ordering hazards.
    // Interior cells are left alone.
    __device__ __forceinline__ void fill_one_ghost_from(double* dstq, const double* q,
                                                        const GeomK& G, const BcK& bc,
                                                        const int lb, const int ii, const int jj, const int kk)
    {
        int c[3] = {ii - G.ng, jj - G.ng, kk - G.ng};
        if (c[0] >= 0 && c[0] < G.n[0] && c[1] >= 0 && c[1] < G.n[1] && c[2] >= 0 && c[2] < G.n[2]) return;
        int b[3] = {lb % G.nb[0], (lb / G.nb[0]) % G.nb[1], lb / (G.nb[0]*G.nb[1])};
        int walls[3];
        int nwall = 0;
        #pragma unroll
        for (int d = 0; d < 3; ++d)
        {
            int face = -1;
            if (c[d] < 0 && b[d] == 0) face = 2*d;
            if (c[d] >= G.n[d] && b[d] == G.nb[d] - 1) face = 2*d + 1;
            if (face < 0) continue;
            const int kind = bc.kind[face];
            if (kind == GBNS_BC_ISOTHERMAL_NOSLIP || kind == GBNS_BC_SLIP_ADIABATIC)
            {
                c[d] = (face % 2 == 0) ? -1 - c[d] : 2*G.n[d] - (c[d] + 1);
                walls[nwall++] = face;
            }
        }
        #pragma unroll
        for (int d = 0; d < 3; ++d)
        {
            int o = 0;
            if (c[d] < 0) o = -1;
            else if (c[d] >= G.n[d]) o = 1;
            if (o == 0) continue;
            const bool at_min = b[d] == 0, at_max = b[d] == G.nb[d] - 1;
            if ((o < 0 && at_min && bc.kind[2*d] != GBNS_BC_PERIODIC) ||
                (o > 0 && at_max && bc.kind[2*d + 1] != GBNS_BC_PERIODIC)) return;   // left untouched (GBNS_BC_NONE)
            b[d] += o;
            if (b[d] < 0) b[d] += G.nb[d];
            if (b[d] >= G.nb[d]) b[d] -= G.nb[d];
            c[d] -= o*G.n[d];
        }
        const int lbs = b[0] + G.nb[0]*(b[1] + G.nb[1]*b[2]);
        const double* s = q + (long long)lbs*G.bstride +
            ((long long)((c[2] + G.ng)*G.nj + (c[1] + G.ng))*G.ni + (c[0] + G.ng))*5;
        double val[5];
        #pragma unroll
        for (int v = 0; v < 5; ++v) val[v] = s[v];
        for (int w = 0; w < nwall; ++w)
        {
            const int face = walls[w];
            if (bc.kind[face] == GBNS_BC_ISOTHERMAL_NOSLIP)
            {
                val[1] = 2.0*bc.t_wall[face] - val[1];
                val[2] = -val[2]; val[3] = -val[3]; val[4] = -val[4];
            }
            else
            {
                val[2 + face/2] = -val[2 + face/2];
            }
        }
        double* dst = dstq + (long long)lb*G.bstride + ((long long)(kk*G.nj + jj)*G.ni + ii)*5;
        #pragma unroll
        for (int v = 0; v < 5; ++v) dst[v] = val[v];
    }

    __device__ __forceinline__ void fill_one_ghost(double* q, const GeomK& G, const BcK& bc,
                                                   const int lb, const int ii, const int jj, const int kk)
    {
        fill_one_ghost_from(q, q, G, bc, lb, ii, jj, kk);
    }

    // Ghost cells of one block enumerated directly (no thread visits an
    // interior cell): the two z slabs of full ni*nj planes, then for interior
    // k the two y slabs of full rows, then for interior k, j the 2*ng x cells.
    // Consecutive t are consecutive cells along x, so loads and stores coalesce.
    __device__ __forceinline__ long long ghosts_per_block(const GeomK& G)
    {
        return (long long)G.ni*G.nj*G.nk - (long long)G.n[0]*G.n[1]*G.n[2];
    }

    __device__ __forceinline__ void ghost_cell(long long t, const GeomK& G, int& ii, int& jj, int& kk)
    {
        const int ng = G.ng, ni = G.ni, nj = G.nj;
        const long long plane = (long long)ni*nj;
        const long long zs = 2ll*ng*plane;
        if (t < zs)
        {
            const int k = int(t / plane);
            const int r = int(t - k*plane);
            kk = k < ng ? k : k + G.n[2];
            jj = r / ni;
            ii = r - jj*ni;
            return;
        }
        t -= zs;
        const long long yrow = 2ll*ng*ni;
        const long long ys = (long long)G.n[2]*yrow;
        if (t < ys)
        {
            const int k = int(t / yrow);
            const int r = int(t - k*yrow);
            kk = ng + k;
            const int j = r / ni;
            jj = j < ng ? j : j + G.n[1];
            ii = r - j*ni;
            return;
        }
        t -= ys;
        const int xr = 2*ng;
        const long long xplane = (long long)G.n[1]*xr;
        const int k = int(t / xplane);
        const int r = int(t - k*xplane);
        kk = ng + k;
        jj = ng + r / xr;
        const int i = r - (r / xr)*xr;
        ii = i < ng ? i : i + G.n[0];
    }

    // Interior cell c (x fastest) of one block: its padded indices.
    __device__ __forceinline__ long long interior_offset(long long c, const GeomK& G, int lb)
    {
        const int i = int(c % G.n[0]);
        const long long r = c / G.n[0];
        const int j = int(r % G.n[1]);
        const int k = int(r / G.n[1]);
        return (long long)lb*G.bstride + ((long long)((k + G.ng)*G.nj + (j + G.ng))*G.ni + (i + G.ng))*5;
    }

    // One thread per ghost cell.
    __global__ void __launch_bounds__(256)
    fill_ghosts_kernel(double* __restrict__ q, const __grid_constant__ GeomK G, const BcK bc, const int blk0,
                       const int nrun)
    {
        const long long per_block = ghosts_per_block(G);
        const long long total = per_block*nrun;
        for (long long idx = blockIdx.x*(long long)blockDim.x + threadIdx.x; idx < total;
             idx += (long long)gridDim.x*blockDim.x)
        {
            const int r = int(idx / per_block);
            int ii, jj, kk;
            ghost_cell(idx - r*per_block, G, ii, jj, kk);
            fill_one_ghost(q, G, bc, blk0 + r, ii, jj, kk);
        }
    }

    // dst = src on interior cells; dst ghosts filled from src's interior
    // donors (the ghost fill of the state that the last fused stage wrote to
    // the scratch buffer, landing in the caller's array).  Ghost cells first,
    // then the interior copy, in one grid-stride range.
    __global__ void __launch_bounds__(256)
    copy_fill_kernel(double* __restrict__ dst, const double* __restrict__ src, const __grid_constant__ GeomK G, const BcK bc,
                     const int blk0, const int nrun)
    {
        const long long gpb = ghosts_per_block(G);
        const long long ipb = (long long)G.n[0]*G.n[1]*G.n[2];
        const long long ng_total = gpb*nrun;
        const long long total = ng_total + ipb*nrun;
        for (long long idx = blockIdx.x*(long long)blockDim.x + threadIdx.x; idx < total;
             idx += (long long)gridDim.x*blockDim.x)
        {
            if (idx < ng_total)
            {
                const int r = int(idx / gpb);
                int ii, jj, kk;
                ghost_cell(idx - r*gpb, G, ii, jj, kk);
                fill_one_ghost_from(dst, src, G, bc, blk0 + r, ii, jj, kk);
            }
            else
            {
                const long long c = idx - ng_total;
                const int r = int(c / ipb);
                const long long off = interior_offset(c - r*ipb, G, blk0 + r);
                #pragma unroll
                for (int v = 0; v < 5; ++v) dst[off + v] = src[off + v];
            }
        }
    }

    int sm_count()
    {
        int dev = 0, n = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return 152;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 152;
        return n;
    }

    static unsigned grid_for(long long work, int threads, int per_sm)
    {
        const long long want = (work + threads - 1)/threads;
        const long long cap = (long long)sm_count()*per_sm;
        return unsigned(want < cap ? (want > 0 ? want : 1) : cap);
    }

    static int block_range(const GeomK& G, int& blk0, int& blk1)
    {
        if (blk1 < 0) blk1 = G.nblk;
        if (blk0 < 0 || blk1 > G.nblk || blk0 > blk1) return set_error(GBNS_ERR_INVALID, "block range out of the grid");
        return GBNS_OK;
    }

    int launch_copy_fill(const GeomK& G, const gbns_bc_desc* bc, double* dst, const double* src, cudaStream_t stream,
                         int blk0, int blk1)
    {
        int rc = block_range(G, blk0, blk1);
        if (rc || blk1 == blk0) return rc;
        BcK k;
        for (int i = 0; i < 6; ++i) { k.kind[i] = bc->kind[i]; k.t_wall[i] = bc->t_wall[i]; }
        const long long total = (long long)G.ni*G.nj*G.nk*(blk1 - blk0);   // ghosts + interior
        copy_fill_kernel<<<grid_for(total, 256, 16), 256, 0, stream>>>(dst, src, G, k, blk0, blk1 - blk0);
        return check_cuda(cudaGetLastError(), "copy_fill launch");
    }

    int launch_fill_ghosts(const GeomK& G, const gbns_bc_desc* bc, double* prims, cudaStream_t stream,
                           int blk0, int blk1)
    {
        int rc = block_range(G, blk0, blk1);
        if (rc || blk1 == blk0) return rc;
        BcK k;
        for (int i = 0; i < 6; ++i) { k.kind[i] = bc->kind[i]; k.t_wall[i] = bc->t_wall[i]; }
        const long long total = ((long long)G.ni*G.nj*G.nk - (long long)G.n[0]*G.n[1]*G.n[2])*(blk1 - blk0);
        fill_ghosts_kernel<<<grid_for(total, 256, 16), 256, 0, stream>>>(prims, G, k, blk0, blk1 - blk0);
        return check_cuda(cudaGetLastError(), "fill_ghosts launch");
    }

    // ------------------------------------------------------------------
    // fused RK stage (transform_advance_to, advance.h:75-101)
    // ------------------------------------------------------------------
    struct RkK
    {
        const double* res[4];
        double coeff[4];
        int nres;
        double gamma, R, gm1;
    };

    // transform_advance_to for one cell at offset `off` (advance.h:75-101,
    // fluid_state.h:151-184): prim -> cons, cons += coeff_j R_j, cons -> prim.
    template <int NRES>
    __device__ __forceinline__ void rk_update_cell(double* __restrict__ q, const double* const* res,
                                                   const double* coeff, const double R, const double gm1,
                                                   const long long off)
    {
        double* qq = q + off;
        const double qv[5] = {qq[0], qq[1], qq[2], qq[3], qq[4]};
        double c[5];
        prim_to_cons(qv, R, gm1, c);
        #pragma unroll
        for (int r = 0; r < NRES; ++r)
        {
            const double* rr = res[r] + off;
            #pragma unroll
            for (int s = 0; s < 5; ++s) c[s] += coeff[r]*rr[s];
        }
        double out[5];
        cons_to_prim(c, R, gm1, out);
        #pragma unroll
        for (int v = 0; v < 5; ++v) qq[v] = out[v];
    }

    template <int NRES>
    __global__ void __launch_bounds__(256)
    rk_stage_kernel(double* __restrict__ q, const __grid_constant__ GeomK G, const RkK k)
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
            rk_update_cell<NRES>(q, k.res, k.coeff, k.R, k.gm1, off);
        }
    }

    int launch_rk_stage(const GeomK& G, double gamma, double R, double* prims,
                        const double* const* res, const double* coeffs, int nres, cudaStream_t stream)
    {
        RkK k;
        std::memset(&k, 0, sizeof(k));
        for (int j = 0; j < nres; ++j) { k.res[j] = res[j]; k.coeff[j] = coeffs[j]; }
        k.nres = nres;
        k.gamma = gamma; k.R = R; k.gm1 = gamma - 1.0;
        const long long total = (long long)G.n[0]*G.n[1]*G.n[2]*G.nblk;
        const unsigned grid = grid_for(total, 256, 16);
        switch (nres)
        {
            case 0: rk_stage_kernel<0><<<grid, 256, 0, stream>>>(prims, G, k); break;
            case 1: rk_stage_kernel<1><<<grid, 256, 0, stream>>>(prims, G, k); break;
            case 2: rk_stage_kernel<2><<<grid, 256, 0, stream>>>(prims, G, k); break;
            case 3: rk_stage_kernel<3><<<grid, 256, 0, stream>>>(prims, G, k); break;
            default: rk_stage_kernel<4><<<grid, 256, 0, stream>>>(prims, G, k); break;
        }
        return check_cuda(cudaGetLastError(), "rk_stage launch");
    }

    // ------------------------------------------------------------------
    // batched forms: one CTA per (instance, block) item of a device list
    // ------------------------------------------------------------------
    int persistent_grid(int ctas_per_sm)
    {
        return sm_count()*ctas_per_sm;
    }

    __global__ void __launch_bounds__(256)
    ghost_batch_kernel(const BlockItem* __restrict__ items, const int* __restrict__ count, const InstK* __restrict__ insts,
                       const long long* __restrict__ left, const int mode)
    {
        // mode 0: ghosts of q; 1: ghosts of R[2] (the fused stage's second
        // state buffer); 2: q = R[2] on the interior with q's ghosts filled
        // from R[2]'s interior donors (after the last fused stage)
        const int n = *count;
        for (int it = blockIdx.x; it < n; it += gridDim.x)
        {
            const BlockItem w = items[it];
            if (left[w.inst] == 0) continue;      // the instance has done its steps: it idles
            const InstK& I = insts[w.inst];
            const GeomK& G = I.G;
            double* dst = mode == 1 ? I.R[2] : I.q;
            const double* src = mode == 0 ? I.q : I.R[2];
            const int gpb = int(ghosts_per_block(G));
            for (int t = threadIdx.x; t < gpb; t += blockDim.x)
            {
                int ii, jj, kk;
                ghost_cell(t, G, ii, jj, kk);
                fill_one_ghost_from(dst, src, G, I.bc, w.lb, ii, jj, kk);
            }
            if (mode == 2)
            {
                const int ipb = G.n[0]*G.n[1]*G.n[2];
                for (int c = threadIdx.x; c < ipb; c += blockDim.x)
                {
                    const long long off = interior_offset(c, G, w.lb);
                    #pragma unroll
                    for (int v = 0; v < 5; ++v) dst[off + v] = src[off + v];
                }
            }
        }
    }

    int launch_ghost_batch(const BlockItem* items, const int* count, const InstK* insts, const long long* left,
                           int mode, cudaStream_t st)
    {
        ghost_batch_kernel<<<persistent_grid(8), 256, 0, st>>>(items, count, insts, left, mode);
        return check_cuda(cudaGetLastError(), "ghost_batch launch");
    }

    // End of a batched step: every limited instance that still had steps to
    // do has done one more (unlimited ones hold -1, finished ones 0).
    __global__ void steps_tick_kernel(long long* left, const int n)
    {
        for (int i = blockIdx.x*blockDim.x + threadIdx.x; i < n; i += gridDim.x*blockDim.x)
            if (left[i] > 0) left[i] -= 1;
    }

    __global__ void steps_set_kernel(long long* left, const int slot, const long long value)
    {
        left[slot] = value;
    }

    int launch_steps_tick(long long* left, int n, cudaStream_t st)
    {
        if (n <= 0) return GBNS_OK;
        steps_tick_kernel<<<(n + 255)/256, 256, 0, st>>>(left, n);
        return check_cuda(cudaGetLastError(), "batch step counters");
    }

    int launch_steps_set(long long* left, int slot, long long value, cudaStream_t st)
    {
        steps_set_kernel<<<1, 1, 0, st>>>(left, slot, value);
        return check_cuda(cudaGetLastError(), "batch step limit");
    }

    // ------------------------------------------------------------------
    // reductions: per-CTA partials in a fixed order, then one CTA folds
    // them in a fixed order, so the result is deterministic.
    // ------------------------------------------------------------------
    struct RedK
    {
        double gamma, R;
        double dx[3][MAX_BLK_PER_DIM];
        int kind;
        int stretch;
        double ywt[MAX_YTAB];                // dy/deta per (by, j) for stretched grids
    };

    constexpr int RED_THREADS = 256;

    __device__ __forceinline__ double warp_sum(double v)
    {
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        return v;
    }
    __device__ __forceinline__ double warp_max(double v)
    {
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        return v;
    }

    __global__ void __launch_bounds__(RED_THREADS)
    reduce_partial_kernel(const double* __restrict__ q, const __grid_constant__ GeomK G,
                          const __grid_constant__ RedK K, double* __restrict__ partials)
    {
        __shared__ double sh[RED_NVAL][RED_THREADS/32];
        const long long ncell = (long long)G.n[0]*G.n[1]*G.n[2];
        const long long total = ncell*G.nblk;
        double acc[RED_NVAL] = {0, 0, 0, 0, 0, 0};
        const bool is_max = K.kind == GBNS_RED_MAX_WAVESPEED;
        for (long long idx = blockIdx.x*(long long)blockDim.x + threadIdx.x; idx < total;
             idx += (long long)gridDim.x*blockDim.x)
        {
            const int lb = int(idx / ncell);
            const long long rem = idx - lb*ncell;
            const int k_ = int(rem / ((long long)G.n[0]*G.n[1]));
            const int j_ = int((rem / G.n[0]) % G.n[1]);
            const int i_ = int(rem % G.n[0]);
            const int b0 = lb % G.nb[0], b1 = (lb / G.nb[0]) % G.nb[1], b2 = lb / (G.nb[0]*G.nb[1]);
            const double* c = q + (long long)lb*G.bstride +
                ((long long)((k_ + G.ng)*G.nj + (j_ + G.ng))*G.ni + (i_ + G.ng))*5;
            const double p = c[0], T = c[1], u = c[2], v = c[3], w = c[4];
            const double vol = K.dx[0][b0]*K.dx[1][b1]*K.dx[2][b2];
            const double wgt = (K.stretch ? K.ywt[b1*G.n[1] + j_] : 1.0)*vol;
            const double rho = p/(K.R*T);
            const double uu = u*u + v*v + w*w;
            if (is_max)
            {
                const double a = sqrt(K.gamma*K.R*T) + sqrt(uu);
                acc[0] = fmax(acc[0], a);
            }
            else if (K.kind == GBNS_RED_KINETIC)
            {
                acc[0] += 0.5*rho*uu*wgt;
                acc[5] += wgt;
            }
            else if (K.kind == GBNS_RED_CONSERVED)
            {
                acc[0] += rho*wgt;
                acc[1] += (0.5*rho*uu + p/(K.gamma - 1.0))*wgt;
                acc[2] += rho*u*wgt;
                acc[3] += rho*v*wgt;
                acc[4] += rho*w*wgt;
            }
            else
            {
                const bool ok = isfinite(p) && isfinite(T) && isfinite(u) && isfinite(v) && isfinite(w) && p > 0.0 && T > 0.0;
                if (!ok) acc[0] += 1.0;
            }
        }
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        #pragma unroll
        for (int s = 0; s < RED_NVAL; ++s)
        {
            const double r = is_max ? warp_max(acc[s]) : warp_sum(acc[s]);
            if (lane == 0) sh[s][wid] = r;
        }
        __syncthreads();
        if (threadIdx.x < RED_NVAL)
        {
            double r = 0.0;
            for (int i = 0; i < RED_THREADS/32; ++i)
                r = is_max ? fmax(r, sh[threadIdx.x][i]) : r + sh[threadIdx.x][i];
            partials[blockIdx.x*RED_NVAL + threadIdx.x] = r;
        }
    }

    __global__ void __launch_bounds__(RED_THREADS)
    reduce_final_kernel(const double* __restrict__ partials, int npart, int kind, double* __restrict__ out)
    {
        __shared__ double sh[RED_NVAL][RED_THREADS/32];
        const bool is_max = kind == GBNS_RED_MAX_WAVESPEED;
        double acc[RED_NVAL] = {0, 0, 0, 0, 0, 0};
        for (int i = threadIdx.x; i < npart; i += blockDim.x)
        {
            #pragma unroll
            for (int s = 0; s < RED_NVAL; ++s)
                acc[s] = is_max ? fmax(acc[s], partials[i*RED_NVAL + s]) : acc[s] + partials[i*RED_NVAL + s];
        }
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        #pragma unroll
        for (int s = 0; s < RED_NVAL; ++s)
        {
            const double r = is_max ? warp_max(acc[s]) : warp_sum(acc[s]);
            if (lane == 0) sh[s][wid] = r;
        }
        __syncthreads();
        if (threadIdx.x == 0)
        {
            double r[RED_NVAL];
            for (int s = 0; s < RED_NVAL; ++s)
            {
                r[s] = 0.0;
                for (int i = 0; i < RED_THREADS/32; ++i) r[s] = is_max ? fmax(r[s], sh[s][i]) : r[s] + sh[s][i];
            }
            if (kind == GBNS_RED_KINETIC) out[0] = r[0]/r[5];
            else if (kind == GBNS_RED_CONSERVED) for (int s = 0; s < 5; ++s) out[s] = r[s];
            else out[0] = r[0];
        }
    }

    // Number of partial sums a reduction over G uses (depends only on the grid).
    int reduce_npart(const GeomK& G)
    {
        const long long total = (long long)G.n[0]*G.n[1]*G.n[2]*G.nblk;
        long long np = (total + RED_THREADS*8 - 1)/(RED_THREADS*8);
        if (np > RED_MAX_PART) np = RED_MAX_PART;
        if (np < 1) np = 1;
        return int(np);
    }

    int launch_reduce(const gbns_grid_desc* g, const GeomK& G, double gamma, double R, const double* prims,
                      int kind, double* scratch, int npart, cudaStream_t stream)
    {
        static thread_local RedK K;
        std::memset(&K, 0, sizeof(K));
        K.gamma = gamma; K.R = R; K.kind = kind;
        for (int d = 0; d < 3; ++d)
            for (int b = 0; b < G.nb[d]; ++b)
            {
                const double bsize = (g->bounds[2*d+1] - g->bounds[2*d]) / g->nblk[d];
                const double mn = g->bounds[2*d] + b*bsize;
                const double mx = mn + bsize;
                K.dx[d][b] = (mx - mn) / g->ncell[d];
            }
        K.stretch = g->coords != GBNS_COORDS_IDENTITY;
        if (K.stretch)
        {
            if (G.nb[1]*G.n[1] > MAX_YTAB) return set_error(GBNS_ERR_UNSUPPORTED, "stretched reduction table too large");
            for (int by = 0; by < G.nb[1]; ++by)
                for (int j = 0; j < G.n[1]; ++j)
                {
                    const double bsize = (g->bounds[3] - g->bounds[2]) / g->nblk[1];
                    const double mn = g->bounds[2] + by*bsize;
                    const double dy = ((mn + bsize) - mn) / g->ncell[1];
                    K.ywt[by*G.n[1] + j] = y_deriv(g, mn + ((double)j + 0.5)*dy);
                }
        }
        double* partials = scratch;
        double* out_dev = scratch + size_t(npart)*RED_NVAL;
        reduce_partial_kernel<<<npart, RED_THREADS, 0, stream>>>(prims, G, K, partials);
        int rc = check_cuda(cudaGetLastError(), "reduce launch");
        if (rc) return rc;
        reduce_final_kernel<<<1, RED_THREADS, 0, stream>>>(partials, npart, kind, out_dev);
        return check_cuda(cudaGetLastError(), "reduce final launch");
    }

    // Library-owned reduction scratch, one buffer per device, grown on demand.
    static std::mutex g_scratch_mu;
    static std::vector<std::pair<double*, size_t>> g_scratch;

    static int get_scratch(size_t ndouble, double** out)
    {
        int dev = 0;
        int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
        if (rc) return rc;
        std::lock_guard<std::mutex> lk(g_scratch_mu);
        if (g_scratch.size() <= size_t(dev)) g_scratch.resize(dev + 1, {nullptr, 0});
        auto& s = g_scratch[dev];
        if (s.second < ndouble)
        {
            if (s.first) cudaFree(s.first);
            s.first = nullptr;
            s.second = 0;
            rc = check_cuda(cudaMalloc(&s.first, ndouble*sizeof(double)), "reduction scratch cudaMalloc");
            if (rc) return rc;
            s.second = ndouble;
        }
        *out = s.first;
        return GBNS_OK;
    }
}

using namespace gbns;

extern "C"
{
    int gbns_reduce(const gbns_grid_desc* grid, const gbns_gas_desc* gas,
                    const double* prims, int kind, double* out, void* stream)
    {
        GeomK G;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        if (!gas || !prims || !out) return set_error(GBNS_ERR_INVALID, "NULL argument");
        if (kind < GBNS_RED_MAX_WAVESPEED || kind > GBNS_RED_HEALTH) return set_error(GBNS_ERR_INVALID, "unknown reduction");
        const int npart = reduce_npart(G);
        double* scratch = nullptr;
        rc = get_scratch(size_t(npart)*RED_NVAL + RED_RESULT_SLOTS, &scratch);
        if (rc) return rc;
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        rc = launch_reduce(grid, G, gas->gamma, gas->R, prims, kind, scratch, npart, st);
        if (rc) return rc;
        const int nout = kind == GBNS_RED_CONSERVED ? 5 : 1;
        rc = check_cuda(cudaMemcpyAsync(out, scratch + size_t(npart)*RED_NVAL, nout*sizeof(double),
                                        cudaMemcpyDeviceToHost, st), "reduce copy-out");
        if (rc) return rc;
        return check_cuda(cudaStreamSynchronize(st), "reduce sync");
    }

    // Reduction with caller-owned device scratch of gbns_reduce_scratch_size()
    // doubles; the result (1 or 5 doubles) is left in DEVICE memory at
    // scratch + gbns_reduce_result_offset().  Asynchronous.
    int gbns_reduce_scratch_size(const gbns_grid_desc* grid, size_t* ndouble, size_t* result_offset)
    {
        GeomK G;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        const int npart = reduce_npart(G);
        if (ndouble) *ndouble = size_t(npart)*RED_NVAL + RED_RESULT_SLOTS;
        if (result_offset) *result_offset = size_t(npart)*RED_NVAL;
        return GBNS_OK;
    }

    int gbns_reduce_async(const gbns_grid_desc* grid, const gbns_gas_desc* gas, const double* prims,
                          int kind, double* scratch, size_t scratch_len, void* stream)
    {
        GeomK G;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        if (!gas || !prims || !scratch) return set_error(GBNS_ERR_INVALID, "NULL argument");
        if (kind < GBNS_RED_MAX_WAVESPEED || kind > GBNS_RED_HEALTH) return set_error(GBNS_ERR_INVALID, "unknown reduction");
        const int npart = reduce_npart(G);
        if (scratch_len < size_t(npart)*RED_NVAL + RED_RESULT_SLOTS) return set_error(GBNS_ERR_INVALID, "reduction scratch too small");
        return launch_reduce(grid, G, gas->gamma, gas->R, prims, kind, scratch, npart, static_cast<cudaStream_t>(stream));
    }
}
