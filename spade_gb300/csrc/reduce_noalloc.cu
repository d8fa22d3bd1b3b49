// Interior reduction that allocates nothing.
//
// Some callers cannot let a library call cudaMalloc: applications that hand
// all device memory to their own pool allocator at start-up and must not see
// a second allocator take memory behind its back, and solver loops that must
// not stall, since cudaMalloc can synchronise the whole device and may fail
// late in a run when memory is nearly full.  gbns_reduce_noalloc serves them:
// the partial sums of the reduction live in a file-scope device array of
// fixed size instead of library- or caller-allocated scratch.  The arithmetic
// is gbns_reduce_async's, so results equal gbns_reduce's bit for bit.
#include <mutex>
#include <string>
#include <vector>
#include "gbns_internal.cuh"

namespace gbns
{
    // Capacity in doubles: room for the most partial records a reduction
    // uses (1024 of 6 doubles) plus the result slots, 6,152 doubles or
    // 49,216 bytes.  Every GPU that loads the library holds this array until
    // the process exits.
    constexpr size_t NOALLOC_SCRATCH_DOUBLES = size_t(RED_MAX_PART)*RED_NVAL + RED_RESULT_SLOTS;
    static_assert(NOALLOC_SCRATCH_DOUBLES == 6152, "the documented capacity of the no-alloc reduction array");

    static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

    // In host code the array's name is only a host-side stand-in, not a
    // device address.  The device address is looked up once per device, with
    // that device current, and cached.
    static std::mutex g_noalloc_mu;
    static std::vector<double*> g_noalloc_addr;

    static int noalloc_scratch(double** out)
    {
        int dev = 0;
        int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
        if (rc) return rc;
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (g_noalloc_addr.size() <= size_t(dev)) g_noalloc_addr.resize(dev + 1, nullptr);
        if (!g_noalloc_addr[dev])
        {
            void* p = nullptr;
            rc = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                            "cudaGetSymbolAddress(no-alloc reduction scratch)");
            if (rc) return rc;
            g_noalloc_addr[dev] = static_cast<double*>(p);
        }
        *out = g_noalloc_addr[dev];
        return GBNS_OK;
    }
}

using namespace gbns;

extern "C" int gbns_reduce_noalloc(const gbns_grid_desc* grid, const gbns_gas_desc* gas, const double* prims,
                                   int kind, double* out_dev, void* stream)
{
    if (!out_dev) return set_error(GBNS_ERR_INVALID, "gbns_reduce_noalloc: out_dev is NULL");
    if (kind < GBNS_RED_MAX_WAVESPEED || kind > GBNS_RED_HEALTH) return set_error(GBNS_ERR_INVALID, "unknown reduction");
    size_t need = 0, off = 0;
    int rc = gbns_reduce_scratch_size(grid, &need, &off);
    if (rc) return rc;
    if (need > NOALLOC_SCRATCH_DOUBLES)
        return set_error(GBNS_ERR_CAPACITY, "gbns_reduce_noalloc: the reduction needs " + std::to_string(need) +
                         " doubles of scratch, the fixed array holds " + std::to_string(NOALLOC_SCRATCH_DOUBLES));
    double* scratch = nullptr;
    rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    // The first pass writes every partial record the second pass reads, so
    // nothing in the shared array needs zeroing between calls.
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    rc = gbns_reduce_async(grid, gas, prims, kind, scratch, NOALLOC_SCRATCH_DOUBLES, stream);
    if (rc) return rc;
    const int nout = kind == GBNS_RED_CONSERVED ? 5 : 1;
    return check_cuda(cudaMemcpyAsync(out_dev, scratch + off, nout*sizeof(double), cudaMemcpyDeviceToDevice, st),
                      "gbns_reduce_noalloc copy-out");
}
