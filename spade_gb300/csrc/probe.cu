// Measurement aid for the benchmark: sustained FP64 and FP32 FMA rates of
// this GPU (independent dependent-FMA chains per thread, timed with CUDA
// events).  Used to state the arithmetic roof next to the HBM roof.
#include "gbns_internal.cuh"

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

extern "C" int gbns_measure_fma_rate(int fp64, double* flops_per_s, void* stream)
{
    if (!flops_per_s) return gbns::set_error(GBNS_ERR_INVALID, "NULL output");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return fp64 ? gbns::measure<double>(flops_per_s, st) : gbns::measure<float>(flops_per_s, st);
}
