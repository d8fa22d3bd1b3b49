// FP32 copy of the padded AoS5 state for the FP32-flux kernels.
//
// The FP32-flux tile kernel evaluates every face in FP32 from a staged box of
// the tile plus its halo.  Converting that box from the FP64 state inside the
// kernel costs five FP64-pipe conversions per staged cell (the box holds 4-8
// times the tile's cells) on a GPU whose FP64 pipe runs at two lanes per SM
// and clock.  Instead one HBM-bound pass converts each cell once, on the
// integer pipes, into SoA float planes laid out for TMA, and the tile kernel
// stages its box from them with one tensor copy.  The copy lives in
// stream-ordered memory from a pool the library owns (cudaMallocFromPoolAsync
// / cudaFreeAsync on the caller's stream, kept by the pool between calls), so
// concurrent streams never share one and a captured graph carries its own.
#include <cstring>
#include <mutex>
#include <vector>
#include "gbns_internal.cuh"
#include "fp64_int.cuh"

namespace gbns
{
    namespace
    {
        // one thread per float column of every row of every block: columns
        // outside the padded row (alignment slack) are written as zeros so a
        // box never reads uninitialised memory
        __global__ void __launch_bounds__(256)
        to_shadow_kernel(const double* __restrict__ prims, float* __restrict__ out, const int ni, const int nj,
                         const int nk, const int blk0, const int nrun, const int ipad, const int off)
        {
            const long long rows = (long long)nj*nk*nrun;
            const long long total = rows*ipad;
            const long long plane = (long long)ipad*nj*nk;
            const long long row0 = (long long)blk0*nj*nk;
            for (long long t = blockIdx.x*(long long)blockDim.x + threadIdx.x; t < total;
                 t += (long long)gridDim.x*blockDim.x)
            {
                const int col = int(t % ipad);
                const long long row = row0 + t / ipad;        // (lb*nk + k)*nj + j
                const long long lb = row / ((long long)nj*nk);
                const long long jk = row - lb*nj*nk;          // k*nj + j
                const int i = col - off;
                float v[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
                if (i >= 0 && i < ni)
                {
                    const double* src = prims + (row*ni + i)*5;
                    #pragma unroll
                    for (int c = 0; c < 5; ++c) v[c] = d2f_int(__ldg(src + c));
                }
                float* dst = out + lb*5*plane + jk*ipad + col;
                #pragma unroll
                for (int c = 0; c < 5; ++c) dst[c*plane] = v[c];
            }
        }

        std::mutex g_pool_mu;
        std::vector<cudaMemPool_t> g_pools;

        int shadow_pool(cudaMemPool_t* out)
        {
            int dev = 0;
            int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
            if (rc) return rc;
            std::lock_guard<std::mutex> lk(g_pool_mu);
            if (g_pools.size() <= size_t(dev)) g_pools.resize(dev + 1, nullptr);
            if (!g_pools[dev])
            {
                cudaMemPoolProps props;
                std::memset(&props, 0, sizeof(props));
                props.allocType = cudaMemAllocationTypePinned;
                props.handleTypes = cudaMemHandleTypeNone;
                props.location.type = cudaMemLocationTypeDevice;
                props.location.id = dev;
                cudaMemPool_t pool = nullptr;
                rc = check_cuda(cudaMemPoolCreate(&pool, &props), "FP32-copy memory pool");
                if (rc) return rc;
                // keep freed blocks for the next launch instead of returning them
                uint64_t keep = ~uint64_t(0);
                rc = check_cuda(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep),
                                "FP32-copy pool release threshold");
                if (rc) { cudaMemPoolDestroy(pool); return rc; }
                g_pools[dev] = pool;
            }
            *out = g_pools[dev];
            return GBNS_OK;
        }
    }

    int shadow_begin(const double* prims, const GeomK& G, int blk0, int blk1, int halo, int box_x, int box_y,
                     int box_z, cudaStream_t st, ShadowK& S, CUtensorMap* map)
    {
        S.base = nullptr;
        // box start column i0 - halo + ng + off with i0 a multiple of 4
        S.off = ((halo - G.ng) % 4 + 4) % 4;
        S.ipad = (G.ni + S.off + 3) & ~3;
        cudaMemPool_t pool = nullptr;
        int rc = shadow_pool(&pool);
        if (rc) return rc;
        const size_t bytes = size_t(S.ipad)*G.nj*G.nk*size_t(G.nblk)*5*sizeof(float);
        void* p = nullptr;
        rc = check_cuda(cudaMallocFromPoolAsync(&p, bytes, pool, st), "FP32 copy of the state (pool allocation)");
        if (rc) return rc;
        S.base = static_cast<float*>(p);
        // only the launch's blocks are converted (the copy is laid out for the whole grid)
        const long long total = (long long)S.ipad*G.nj*G.nk*(blk1 - blk0);
        long long nb = (total + 255)/256;
        const long long cap = (long long)sm_count()*16;
        if (nb > cap) nb = cap;
        to_shadow_kernel<<<unsigned(nb), 256, 0, st>>>(prims, S.base, G.ni, G.nj, G.nk, blk0, blk1 - blk0, S.ipad, S.off);
        rc = check_cuda(cudaGetLastError(), "FP32 copy launch");
        if (!rc) rc = encode_shadow_tmap(map, S, G, box_x, box_y, box_z);
        if (rc)
        {
            cudaFreeAsync(S.base, st);
            S.base = nullptr;
        }
        return rc;
    }

    int pool_alloc(void** p, size_t bytes, cudaStream_t st)
    {
        cudaMemPool_t pool = nullptr;
        const int rc = shadow_pool(&pool);
        if (rc) return rc;
        return check_cuda(cudaMallocFromPoolAsync(p, bytes, pool, st), "library pool allocation");
    }

    int shadow_end(const ShadowK& S, cudaStream_t st)
    {
        if (!S.base) return GBNS_OK;
        return check_cuda(cudaFreeAsync(S.base, st), "FP32 copy of the state (pool free)");
    }
}
