// Test infrastructure: a recording stand-in for the CUDA runtime, linked
// (nvcc -cudart none) into oracle/refgpu/ref_gpu_harness.cu so that the
// REFERENCE's own GPU code path can be driven on a machine without a GPU.
//
// The reference's host code runs here unchanged: every cudaMalloc gets a
// distinct fake device address, every host-to-device copy, device-to-device
// copy and kernel launch is appended to a launch script (REFREC_OUT), and the
// kernel launches are recorded with the kernel's mangled name (from the
// fat-binary registration), the launch shape and the bytes of each argument.
// oracle/refgpu/replay.cc later replays the script on a GPU with the same
// kernels compiled from the same source into a cubin, relocating the fake
// addresses to real allocations.  Only the runtime calls the reference makes
// on its flux_div path are implemented; anything else aborts loudly.
//
// Script records (little-endian, all integers 64-bit unless noted):
//   'A' id size fake              allocation
//   'F' fake                      free
//   'H' dst size bytes[size]      host-to-device copy
//   'Z' dst size                  host-to-device copy of zeros
//   'D' dst src size              device-to-device copy
//   'L' namelen name gx gy gz bx by bz shmem nargs {len bytes[len]}*
//   'M' fake rolelen role         role marker (set by the harness)
//   'P' namelen name              phase marker (set by the harness)
//   'S'                           device synchronise
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

// Compiled without the CUDA headers (plain g++), so these definitions do not
// have to repeat the headers' exact declarations; only the C symbol names and
// the by-value layouts (dim3: three unsigned ints) must agree.
typedef int cudaError_t;
typedef void* cudaStream_t;
typedef void* cudaKernel_t;
struct dim3 { unsigned x, y, z; };
struct uint3 { unsigned x, y, z; };
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };

namespace
{
    constexpr uint64_t FAKE_BASE = 0x00007e0000000000ull;
    constexpr uint64_t FAKE_ALIGN = 1ull << 21;
    constexpr size_t ARG_CAP = 4096;        // bytes captured per kernel argument

    FILE* g_out = nullptr;
    uint64_t g_next = FAKE_BASE;
    uint64_t g_nid = 0;
    // Built on first use: nvcc registers the kernels from a static
    // initialiser of the harness, which may run before this file's.
    std::map<const void*, std::string>& kernels()           // host stub -> mangled name
    {
        static std::map<const void*, std::string> m;
        return m;
    }
    dim3 g_cfg_grid, g_cfg_block;
    size_t g_cfg_shmem = 0;
    cudaError_t g_last = cudaSuccess;

    [[noreturn]] void die(const char* what)
    {
        std::fprintf(stderr, "record_cudart: %s\n", what);
        std::abort();
    }

    FILE* out()
    {
        if (!g_out)
        {
            const char* p = std::getenv("REFREC_OUT");
            if (!p) die("REFREC_OUT is not set");
            g_out = std::fopen(p, "wb");
            if (!g_out) die("cannot open REFREC_OUT");
        }
        return g_out;
    }

    void put_u64(uint64_t v) { if (std::fwrite(&v, 8, 1, out()) != 1) die("write failed"); }
    void put_tag(char c) { if (std::fwrite(&c, 1, 1, out()) != 1) die("write failed"); }
    void put_bytes(const void* p, size_t n) { if (n && std::fwrite(p, 1, n, out()) != n) die("write failed"); }
    void put_str(const std::string& s) { put_u64(s.size()); put_bytes(s.data(), s.size()); }

    bool is_fake(const void* p)
    {
        const uint64_t v = reinterpret_cast<uint64_t>(p);
        return v >= FAKE_BASE && v < g_next;
    }

    // End of the readable mapping holding p (so an argument capture never
    // reads past mapped memory).
    uint64_t mapping_end(const void* p)
    {
        const uint64_t v = reinterpret_cast<uint64_t>(p);
        FILE* f = std::fopen("/proc/self/maps", "r");
        if (!f) die("cannot read /proc/self/maps");
        char line[512];
        uint64_t end = 0;
        while (std::fgets(line, sizeof line, f))
        {
            unsigned long long lo = 0, hi = 0;
            char perm[8] = {0};
            if (std::sscanf(line, "%llx-%llx %7s", &lo, &hi, perm) == 3 && v >= lo && v < hi && perm[0] == 'r')
            {
                end = hi;
                // contiguous readable mappings extend the bound
                char nl[512];
                while (std::fgets(nl, sizeof nl, f))
                {
                    unsigned long long lo2 = 0, hi2 = 0;
                    char perm2[8] = {0};
                    if (std::sscanf(nl, "%llx-%llx %7s", &lo2, &hi2, perm2) == 3 && lo2 == end && perm2[0] == 'r') end = hi2;
                    else break;
                }
                break;
            }
        }
        std::fclose(f);
        if (!end) die("kernel argument outside mapped memory");
        return end;
    }

    void record_launch(const void* func, dim3 grid, dim3 block, void** args, size_t shmem)
    {
        auto it = kernels().find(func);
        if (it == kernels().end()) die("launch of an unregistered kernel");
        // The runtime is not told how many arguments a kernel takes.  The
        // reference launches exactly two kernel templates (dispatch/execute.h):
        // k_gpu_dispatch_impl(mapping, kernel) and k_gpu_impl(kernel).
        size_t nargs = 0;
        if (it->second.find("k_gpu_dispatch_impl") != std::string::npos) nargs = 2;
        else if (it->second.find("k_gpu_impl") != std::string::npos) nargs = 1;
        else die(("launch of an unexpected kernel " + it->second).c_str());
        put_tag('L');
        put_str(it->second);
        put_u64(grid.x); put_u64(grid.y); put_u64(grid.z);
        put_u64(block.x); put_u64(block.y); put_u64(block.z);
        put_u64(shmem);
        put_u64(nargs);
        for (size_t i = 0; i < nargs; ++i)
        {
            const uint64_t lim = mapping_end(args[i]) - reinterpret_cast<uint64_t>(args[i]);
            const size_t n = lim < ARG_CAP ? size_t(lim) : ARG_CAP;
            put_u64(n);
            put_bytes(args[i], n);
        }
        std::fflush(out());
    }
}

extern "C"
{
    // ---- harness hooks ----------------------------------------------------
    void refrec_mark(const void* dptr, const char* role)
    {
        if (!is_fake(dptr)) die("refrec_mark: not a device allocation");
        put_tag('M');
        put_u64(reinterpret_cast<uint64_t>(dptr));
        put_str(role);
        std::fflush(out());
    }

    void refrec_phase(const char* name)
    {
        put_tag('P');
        put_str(name);
        std::fflush(out());
    }

    // ---- fat binary registration (emitted by nvcc into the host object) --
    void** __cudaRegisterFatBinary(void* fatCubin)
    {
        static void* handle[1];
        handle[0] = fatCubin;
        return handle;
    }
    void __cudaRegisterFatBinaryEnd(void**) {}
    void __cudaUnregisterFatBinary(void**) {}
    void __cudaRegisterFunction(void**, const char* hostFun, char*, const char* deviceName, int,
                                uint3*, uint3*, dim3*, dim3*, int*)
    {
        kernels()[reinterpret_cast<const void*>(hostFun)] = deviceName;
    }
    void __cudaRegisterVar(void**, char*, char*, const char*, int, size_t, int, int) {}
    void __cudaRegisterManagedVar(void**, void**, char*, const char*, int, size_t, int, int) {}
    char __cudaInitModule(void**) { return 0; }

    unsigned __cudaPushCallConfiguration(dim3 gridDim, dim3 blockDim, size_t sharedMem, void*)
    {
        g_cfg_grid = gridDim;
        g_cfg_block = blockDim;
        g_cfg_shmem = sharedMem;
        return 0;
    }
    cudaError_t __cudaPopCallConfiguration(dim3* gridDim, dim3* blockDim, size_t* sharedMem, void* stream)
    {
        *gridDim = g_cfg_grid;
        *blockDim = g_cfg_block;
        *sharedMem = g_cfg_shmem;
        *static_cast<cudaStream_t*>(stream) = nullptr;
        return cudaSuccess;
    }
    cudaError_t __cudaGetKernel(cudaKernel_t* k, const void* fun)
    {
        *k = reinterpret_cast<cudaKernel_t>(const_cast<void*>(fun));
        return cudaSuccess;
    }
    cudaError_t __cudaLaunchKernel(cudaKernel_t k, dim3 g, dim3 b, void** args, size_t shmem, cudaStream_t)
    {
        record_launch(reinterpret_cast<const void*>(k), g, b, args, shmem);
        return cudaSuccess;
    }
    cudaError_t cudaLaunchKernel(const void* func, dim3 g, dim3 b, void** args, size_t shmem, cudaStream_t)
    {
        record_launch(func, g, b, args, shmem);
        return cudaSuccess;
    }

    // ---- memory ---------------------------------------------------------
    cudaError_t cudaMalloc(void** p, size_t n)
    {
        const uint64_t fake = g_next;
        g_next += ((n + FAKE_ALIGN - 1)/FAKE_ALIGN + 1)*FAKE_ALIGN;
        put_tag('A'); put_u64(g_nid); put_u64(n); put_u64(fake);
        ++g_nid;
        *p = reinterpret_cast<void*>(fake);
        return cudaSuccess;
    }
    cudaError_t cudaFree(void* p)
    {
        if (!p) return cudaSuccess;
        if (!is_fake(p)) die("cudaFree of a non-device pointer");
        put_tag('F'); put_u64(reinterpret_cast<uint64_t>(p));
        return cudaSuccess;
    }
    cudaError_t cudaHostAlloc(void** p, size_t n, unsigned int)
    {
        *p = std::malloc(n ? n : 1);
        return *p ? cudaSuccess : cudaErrorMemoryAllocation;
    }
    cudaError_t cudaMallocHost(void** p, size_t n) { return cudaHostAlloc(p, n, 0); }
    cudaError_t cudaFreeHost(void* p) { std::free(p); return cudaSuccess; }

    cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, int kind)
    {
        if (kind == cudaMemcpyHostToDevice)
        {
            if (!is_fake(dst)) die("H2D copy to a non-device pointer");
            const unsigned char* s = static_cast<const unsigned char*>(src);
            bool zero = true;
            for (size_t i = 0; i < n && zero; ++i) zero = s[i] == 0;
            if (zero) { put_tag('Z'); put_u64(reinterpret_cast<uint64_t>(dst)); put_u64(n); }
            else { put_tag('H'); put_u64(reinterpret_cast<uint64_t>(dst)); put_u64(n); put_bytes(src, n); }
            return cudaSuccess;
        }
        if (kind == cudaMemcpyDeviceToDevice)
        {
            if (!is_fake(dst) || !is_fake(src)) die("D2D copy of non-device pointers");
            put_tag('D'); put_u64(reinterpret_cast<uint64_t>(dst)); put_u64(reinterpret_cast<uint64_t>(src)); put_u64(n);
            return cudaSuccess;
        }
        if (kind == cudaMemcpyDeviceToHost)
        {
            // contents of device memory are not known while recording
            std::memset(dst, 0, n);
            return cudaSuccess;
        }
        die("unsupported cudaMemcpy kind");
    }
    cudaError_t cudaMemcpyPeer(void*, int, const void*, int, size_t) { die("cudaMemcpyPeer"); }

    // ---- device and errors ----------------------------------------------
    cudaError_t cudaDeviceSynchronize(void) { put_tag('S'); return cudaSuccess; }
    cudaError_t cudaGetLastError(void) { cudaError_t e = g_last; g_last = cudaSuccess; return e; }
    cudaError_t cudaPeekAtLastError(void) { return g_last; }
    const char* cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "recording error"; }
    const char* cudaGetErrorName(cudaError_t e) { return e == cudaSuccess ? "cudaSuccess" : "cudaErrorUnknown"; }
    cudaError_t cudaSetDevice(int) { return cudaSuccess; }
    cudaError_t cudaGetDevice(int* d) { *d = 0; return cudaSuccess; }
    cudaError_t cudaGetDeviceCount(int* n) { *n = 1; return cudaSuccess; }
    cudaError_t cudaDeviceCanAccessPeer(int* can, int, int) { *can = 0; return cudaSuccess; }
    cudaError_t cudaDeviceEnablePeerAccess(int, unsigned int) { return cudaSuccess; }
}
