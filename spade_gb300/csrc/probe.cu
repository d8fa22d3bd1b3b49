// Measurement aid for the benchmark: sustained FP64 and FP32 FMA rates of
// this GPU (independent dependent-FMA chains per thread, timed with CUDA
// events).  Used to state the arithmetic roof next to the HBM roof.
#include "gbns_internal.cuh"
#include "fp64_int.cuh"

namespace gbns
{
    template <class T>
    __global__ void __launch_bounds__(256) fma_chain_kernel(T* out, int iters, T a, T b)
    {
        T x0 = T(threadIdx.x)*T(1e-3), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
        T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
        for (int i = 0; i < iters; ++i)
        {
            x0 = x0*a + b; x1 = x1*a + b; x2 = x2*a + b; x3 = x3*a + b;
            x4 = x4*a + b; x5 = x5*a + b; x6 = x6*a + b; x7 = x7*a + b;
        }
        const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
        if (s == T(-12345.678)) out[blockIdx.x] = s;   // keeps the chains live
    }

    template <class T>
    static int measure(double* flops_per_s, cudaStream_t st)
    {
        int dev = 0, sms = 0;
        int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
        if (rc) return rc;
        rc = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
        if (rc) return rc;
        const int blocks = sms*8, threads = 256;
        const int iters = sizeof(T) == 8 ? 4096 : 65536;
        T* out = nullptr;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        fma_chain_kernel<T><<<blocks, threads, 0, st>>>(out, 64, T(0.999999), T(1e-7));   // warm-up
        cudaEventRecord(e0, st);
        fma_chain_kernel<T><<<blocks, threads, 0, st>>>(out, iters, T(0.999999), T(1e-7));
        cudaEventRecord(e1, st);
        rc = check_cuda(cudaEventSynchronize(e1), "fma probe");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc) return rc;
        *flops_per_s = 2.0*8.0*double(iters)*double(blocks)*threads/(double(ms)*1e-3);
        return GBNS_OK;
    }
}

namespace gbns
{
    namespace { status_registrar tu_status_registrar; }

    // The flux kernel's failure path, exercised on purpose: one CTA arms an
    // mbarrier for 16 bytes of TMA data that no copy will deliver (a flag
    // nothing sets), waits with a bounded poll, finds the phase incomplete,
    // records DEV_TMA_TIMEOUT in the device status word and returns.  No
    // copy is in flight, so nothing is left pending when the CTA exits.
    __global__ void __launch_bounds__(32) wait_timeout_selftest_kernel(long long max_cycles)
    {
        __shared__ __align__(8) uint64_t bar;
        if (threadIdx.x == 0)
        {
            mbar_init(&bar, 1);
            mbar_expect_tx(&bar, 16u);
        }
        __syncwarp();
        const bool ok = mbar_wait(&bar, 0, max_cycles);
        if (__any_sync(0xffffffffu, !ok))
        {
            if (threadIdx.x == 0) atomicExch(&g_device_status, DEV_TMA_TIMEOUT);
        }
        __syncwarp();
        if (threadIdx.x == 0) mbar_inval(&bar);
    }
}

extern "C" int gbns_selftest_wait_timeout(int* status, void* stream)
{
    using namespace gbns;
    if (!status) return set_error(GBNS_ERR_INVALID, "NULL output");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = read_device_status(status, 1, st);          // clear any earlier flag
    if (rc) return rc;
    wait_timeout_selftest_kernel<<<1, 32, 0, st>>>(20000000ll);    // ~10 ms
    rc = check_cuda(cudaGetLastError(), "wait self-test launch");
    if (rc) return rc;
    return read_device_status(status, 1, st);            // the flag the timeout set; cleared again
}

namespace gbns
{
    __device__ __forceinline__ uint64_t mix64(uint64_t x)
    {
        x += 0x9E3779B97F4A7C15ull;
        x = (x ^ (x >> 30))*0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27))*0x94D049BB133111EBull;
        return x ^ (x >> 31);
    }

    // Operand bits for pair k: all bit patterns, exponent bands where the
    // product leaves the normal range, significands with few set bits (exact
    // products and ties), zeros, subnormals, infinities and NaNs.
    __device__ __forceinline__ uint64_t dmul_operand(uint64_t k, int which)
    {
        constexpr uint64_t SG = 0x8000000000000000ull, MM = 0x000FFFFFFFFFFFFFull;
        const uint64_t r = mix64(2*k + which), r2 = mix64(r);
        switch ((int)(mix64(k ^ 0x5bd1e995ull) % 8))
        {
        case 0: return r;
        case 1: return (r & (SG | MM)) | (uint64_t(991 + r2 % 64) << 52);
        case 2: return (r & (SG | MM)) | (uint64_t(1 + r2 % 8) << 52);
        case 3: return (r & (SG | MM)) | (uint64_t(2040 + r2 % 7) << 52);
        case 4: return (r & (SG | 0x000FFF0000000000ull)) | (uint64_t(1020 + r2 % 8) << 52);
        case 5: return (r & (SG | 0xFFull)) | (uint64_t(1000 + r2 % 60) << 52);
        case 6: return (r & (SG | MM)) | (uint64_t(r2 % 3) << 52);
        default: return (r & (SG | MM)) | (uint64_t(2046 + r2 % 2) << 52);
        }
    }

    __global__ void __launch_bounds__(256) dmul_int_check_kernel(uint64_t n, uint64_t seed,
                                                                 unsigned long long* bad)
    {
        for (uint64_t i = blockIdx.x*(uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x*blockDim.x)
        {
            const uint64_t k = i + seed;
            const double a = __longlong_as_double((long long)dmul_operand(k, 0));
            const double b = __longlong_as_double((long long)dmul_operand(k, 1));
            const double h = __dmul_rn(a, b), e = dmul_int(a, b);
            const bool same = __double_as_longlong(h) == __double_as_longlong(e) || (h != h && e != e);
            const double h1 = __dmul_rn(a, 0.5), e1 = dmul_pow2<-1>(a);
            const double h2 = __dmul_rn(a, 0.25), e2 = dmul_pow2<-2>(a);
            const bool same1 = __double_as_longlong(h1) == __double_as_longlong(e1) || (h1 != h1 && e1 != e1);
            const bool same2 = __double_as_longlong(h2) == __double_as_longlong(e2) || (h2 != h2 && e2 != e2);
            const double hq = __ddiv_rn(a, b), eq = ddiv_int(a, b);
            const bool same3 = __double_as_longlong(hq) == __double_as_longlong(eq) || (hq != hq && eq != eq);
            const double hs = __dsqrt_rn(a), es = dsqrt_int(a);
            const bool same4 = __double_as_longlong(hs) == __double_as_longlong(es) || (hs != hs && es != es);
            if (!same || !same1 || !same2 || !same3 || !same4) atomicAdd(bad, 1ull);
        }
    }
}

extern "C" int gbns_selftest_dmul_int(uint64_t npairs, uint64_t seed, uint64_t* mismatches, void* stream)
{
    using namespace gbns;
    if (!mismatches) return set_error(GBNS_ERR_INVALID, "NULL output");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned long long* d = nullptr;
    int rc = check_cuda(cudaMalloc(&d, sizeof(unsigned long long)), "self-test counter");
    if (rc) return rc;
    unsigned long long h = 0;
    rc = check_cuda(cudaMemsetAsync(d, 0, sizeof(h), st), "self-test counter reset");
    if (!rc && npairs)
    {
        dmul_int_check_kernel<<<sm_count()*8, 256, 0, st>>>(npairs, seed, d);
        rc = check_cuda(cudaGetLastError(), "dmul_int self-test launch");
    }
    if (!rc) rc = check_cuda(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st), "self-test read");
    if (!rc) rc = check_cuda(cudaStreamSynchronize(st), "dmul_int self-test");
    cudaFree(d);
    if (rc) return rc;
    *mismatches = h;
    return GBNS_OK;
}

extern "C" int gbns_measure_fma_rate(int fp64, double* flops_per_s, void* stream)
{
    if (!flops_per_s) return gbns::set_error(GBNS_ERR_INVALID, "NULL output");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return fp64 ? gbns::measure<double>(flops_per_s, st) : gbns::measure<float>(flops_per_s, st);
}
