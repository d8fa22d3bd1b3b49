// Test infrastructure: replays a launch script written by
// oracle/refgpu/ref_gpu_harness.cu (recorded with record_cudart.cc) on a GPU,
// running the REFERENCE's own flux_div kernels from a cubin compiled from the
// same source.  Built on the GPU host against the CUDA driver API
// (oracle/refgpu/Makefile); loaded by the tests and the benchmark through
// ctypes.  Nothing here is part of the shipped library.
//
//   void* refgpu_open(script, cubin, err, errlen)
//   int   refgpu_bind(h, role, device_ptr, bytes)   caller memory for a role
//   int   refgpu_prepare(h, stream)                 allocations + uploads
//   int   refgpu_nphases(h); const char* refgpu_phase_name(h, i)
//   int   refgpu_run(h, phase, stream)              the phase's launches
//   void  refgpu_close(h)
//
// Every fake device address in a kernel argument or an uploaded buffer is
// relocated to the real allocation it points into; an argument that still
// holds an address from the recording's fake range after relocation, a
// parameter count or size that does not match the cubin's kernel, or a role
// bound with a different size is rejected before anything is launched.
#include <cuda.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

namespace
{
    constexpr uint64_t FAKE_BASE = 0x00007e0000000000ull;
    constexpr uint64_t FAKE_END  = 0x00007f0000000000ull;

    struct alloc_t { uint64_t fake, size; CUdeviceptr real; bool owned; std::string role; };
    struct launch_t
    {
        std::string name;
        unsigned g[3], b[3];
        unsigned shmem;
        std::vector<std::vector<unsigned char>> args;
        CUfunction fn = nullptr;
        std::vector<std::vector<unsigned char>> patched;
        std::vector<void*> params;
    };
    struct op_t { char tag; uint64_t a, b, c; std::vector<unsigned char> data; int launch; };

    struct replay_t
    {
        std::vector<alloc_t> allocs;
        std::vector<op_t> setup;
        std::vector<std::string> phase_names;
        std::vector<std::vector<op_t>> phases;
        std::vector<launch_t> launches;
        std::vector<unsigned char> cubin;
        CUmodule mod = nullptr;
        bool prepared = false;
        std::string err;
    };

    struct reader_t
    {
        const std::vector<unsigned char>& d;
        size_t i = 0;
        bool ok = true;
        uint64_t u64()
        {
            if (i + 8 > d.size()) { ok = false; return 0; }
            uint64_t v;
            std::memcpy(&v, &d[i], 8);
            i += 8;
            return v;
        }
        std::vector<unsigned char> bytes(uint64_t n)
        {
            if (i + n > d.size()) { ok = false; return {}; }
            std::vector<unsigned char> v(d.begin() + i, d.begin() + i + n);
            i += n;
            return v;
        }
        std::string str() { auto b = bytes(u64()); return std::string(b.begin(), b.end()); }
    };

    bool read_file(const char* path, std::vector<unsigned char>& out)
    {
        std::ifstream f(path, std::ios::binary);
        if (!f) return false;
        out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
        return true;
    }

    alloc_t* find_alloc(replay_t& R, uint64_t v)
    {
        for (auto& a : R.allocs)
            if (v >= a.fake && v <= a.fake + a.size) return &a;
        return nullptr;
    }

    // Relocates every 8-byte-aligned fake address in buf; false if one is
    // left that points into no allocation.
    bool relocate(replay_t& R, unsigned char* buf, size_t n)
    {
        for (size_t o = 0; o + 8 <= n; o += 8)
        {
            uint64_t v;
            std::memcpy(&v, buf + o, 8);
            if (v < FAKE_BASE || v >= FAKE_END) continue;
            alloc_t* a = find_alloc(R, v);
            if (!a || !a->real) return false;
            const uint64_t r = uint64_t(a->real) + (v - a->fake);
            std::memcpy(buf + o, &r, 8);
        }
        return true;
    }

    int fail(replay_t& R, const std::string& m) { R.err = m; return -1; }

    int cu(replay_t& R, CUresult r, const char* what)
    {
        if (r == CUDA_SUCCESS) return 0;
        const char* s = nullptr;
        cuGetErrorString(r, &s);
        return fail(R, std::string(what) + ": " + (s ? s : "unknown CUDA error"));
    }

    int exec_op(replay_t& R, op_t& op, CUstream st)
    {
        switch (op.tag)
        {
            case 'H':
            {
                alloc_t* a = find_alloc(R, op.a);
                if (!a || op.a + op.b > a->fake + a->size) return fail(R, "upload outside an allocation");
                return cu(R, cuMemcpyHtoDAsync(a->real + (op.a - a->fake), op.data.data(), op.b, st), "upload");
            }
            case 'Z':
            {
                alloc_t* a = find_alloc(R, op.a);
                if (!a || op.a + op.b > a->fake + a->size) return fail(R, "zero upload outside an allocation");
                return cu(R, cuMemsetD8Async(a->real + (op.a - a->fake), 0, op.b, st), "zero upload");
            }
            case 'D':
            {
                alloc_t* d = find_alloc(R, op.a);
                alloc_t* s = find_alloc(R, op.b);
                if (!d || !s || op.a + op.c > d->fake + d->size || op.b + op.c > s->fake + s->size)
                    return fail(R, "device copy outside an allocation");
                return cu(R, cuMemcpyDtoDAsync(d->real + (op.a - d->fake), s->real + (op.b - s->fake), op.c, st), "device copy");
            }
            case 'L':
            {
                launch_t& L = R.launches[op.launch];
                return cu(R, cuLaunchKernel(L.fn, L.g[0], L.g[1], L.g[2], L.b[0], L.b[1], L.b[2], L.shmem, st,
                                            L.params.data(), nullptr), L.name.c_str());
            }
            default:
                return 0;   // synchronisation points: the caller synchronises
        }
    }
}

extern "C"
{
    void* refgpu_open(const char* script, const char* cubin, char* err, size_t errlen)
    {
        auto* R = new replay_t;
        std::vector<unsigned char> d;
        auto bad = [&](const std::string& m) -> void*
        {
            if (err && errlen) std::snprintf(err, errlen, "%s", m.c_str());
            delete R;
            return nullptr;
        };
        if (!read_file(script, d)) return bad("cannot read the launch script");
        if (!read_file(cubin, R->cubin)) return bad("cannot read the cubin");
        reader_t rd{d};
        std::vector<op_t>* cur = &R->setup;
        while (rd.ok && rd.i < d.size())
        {
            const char tag = char(d[rd.i++]);
            op_t op{tag, 0, 0, 0, {}, -1};
            switch (tag)
            {
                case 'A':
                {
                    rd.u64();
                    const uint64_t size = rd.u64(), fake = rd.u64();
                    R->allocs.push_back(alloc_t{fake, size, 0, false, ""});
                    break;
                }
                case 'F': rd.u64(); break;
                case 'H': op.a = rd.u64(); op.b = rd.u64(); op.data = rd.bytes(op.b); cur->push_back(op); break;
                case 'Z': op.a = rd.u64(); op.b = rd.u64(); cur->push_back(op); break;
                case 'D': op.a = rd.u64(); op.b = rd.u64(); op.c = rd.u64(); cur->push_back(op); break;
                case 'S': cur->push_back(op); break;
                case 'M':
                {
                    const uint64_t fake = rd.u64();
                    const std::string role = rd.str();
                    bool found = false;
                    for (auto& a : R->allocs) if (a.fake == fake) { a.role = role; found = true; }
                    if (!found) return bad("role marker for an unknown allocation");
                    break;
                }
                case 'P':
                    R->phase_names.push_back(rd.str());
                    R->phases.emplace_back();
                    cur = &R->phases.back();
                    break;
                case 'L':
                {
                    launch_t L;
                    L.name = rd.str();
                    for (int k = 0; k < 3; ++k) L.g[k] = unsigned(rd.u64());
                    for (int k = 0; k < 3; ++k) L.b[k] = unsigned(rd.u64());
                    L.shmem = unsigned(rd.u64());
                    const uint64_t na = rd.u64();
                    for (uint64_t k = 0; k < na && rd.ok; ++k) L.args.push_back(rd.bytes(rd.u64()));
                    op.launch = int(R->launches.size());
                    R->launches.push_back(std::move(L));
                    cur->push_back(op);
                    break;
                }
                default: return bad(std::string("unknown record in the launch script: ") + tag);
            }
        }
        if (!rd.ok) return bad("truncated launch script");
        return R;
    }

    const char* refgpu_error(void* h) { return h ? static_cast<replay_t*>(h)->err.c_str() : "no handle"; }

    int refgpu_bind(void* h, const char* role, unsigned long long dptr, unsigned long long bytes)
    {
        auto* R = static_cast<replay_t*>(h);
        for (auto& a : R->allocs)
            if (a.role == role)
            {
                if (a.size != bytes) return fail(*R, std::string("role ") + role + ": size differs from the recording");
                a.real = CUdeviceptr(dptr);
                a.owned = false;
                return 0;
            }
        return fail(*R, std::string("no allocation has role ") + role);
    }

    int refgpu_prepare(void* h, void* stream)
    {
        auto* R = static_cast<replay_t*>(h);
        if (R->prepared) return 0;
        CUstream st = static_cast<CUstream>(stream);
        CUcontext ctx = nullptr;
        if (cu(*R, cuCtxGetCurrent(&ctx), "cuCtxGetCurrent")) return -1;
        if (!ctx) return fail(*R, "no current CUDA context (initialise the runtime first)");
        for (auto& a : R->allocs)
        {
            if (!a.role.empty())
            {
                if (!a.real) return fail(*R, "role " + a.role + " is not bound");
                continue;
            }
            if (cu(*R, cuMemAlloc(&a.real, a.size ? a.size : 1), "cuMemAlloc")) return -1;
            a.owned = true;
        }
        if (cu(*R, cuModuleLoadData(&R->mod, R->cubin.data()), "cuModuleLoadData")) return -1;
        for (auto& L : R->launches)
        {
            if (cu(*R, cuModuleGetFunction(&L.fn, R->mod, L.name.c_str()), "cuModuleGetFunction")) return -1;
            size_t np = 0;
            for (;; ++np)
            {
                size_t off = 0, sz = 0;
                if (cuFuncGetParamInfo(L.fn, np, &off, &sz) != CUDA_SUCCESS) break;
                if (np >= L.args.size()) return fail(*R, L.name + ": more parameters than recorded");
                if (sz > L.args[np].size()) return fail(*R, L.name + ": parameter larger than its recording");
                std::vector<unsigned char> p(L.args[np].begin(), L.args[np].begin() + sz);
                if (!relocate(*R, p.data(), p.size()))
                    return fail(*R, L.name + ": argument holds a device address outside every allocation");
                L.patched.push_back(std::move(p));
            }
            if (np != L.args.size()) return fail(*R, L.name + ": parameter count differs from the recording");
            if (L.shmem > 48*1024 &&
                cu(*R, cuFuncSetAttribute(L.fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, int(L.shmem)), "smem attribute"))
                return -1;
            for (auto& p : L.patched) L.params.push_back(p.data());
        }
        for (auto& op : R->setup)
            if (op.tag == 'H' && !relocate(*R, op.data.data(), op.data.size() & ~size_t(7)))
                return fail(*R, "uploaded buffer holds a device address outside every allocation");
        for (auto& ph : R->phases)
            for (auto& op : ph)
                if (op.tag == 'H' && !relocate(*R, op.data.data(), op.data.size() & ~size_t(7)))
                    return fail(*R, "uploaded buffer holds a device address outside every allocation");
        for (auto& op : R->setup)
            if (exec_op(*R, op, st)) return -1;
        if (cu(*R, cuStreamSynchronize(st), "setup sync")) return -1;
        R->prepared = true;
        return 0;
    }

    int refgpu_nphases(void* h) { return int(static_cast<replay_t*>(h)->phases.size()); }
    const char* refgpu_phase_name(void* h, int i) { return static_cast<replay_t*>(h)->phase_names.at(i).c_str(); }
    int refgpu_phase_launches(void* h, int i)
    {
        int n = 0;
        for (auto& op : static_cast<replay_t*>(h)->phases.at(i)) n += op.tag == 'L';
        return n;
    }

    int refgpu_run(void* h, int phase, void* stream)
    {
        auto* R = static_cast<replay_t*>(h);
        if (!R->prepared) return fail(*R, "refgpu_prepare has not run");
        if (phase < 0 || phase >= int(R->phases.size())) return fail(*R, "phase out of range");
        for (auto& op : R->phases[phase])
            if (exec_op(*R, op, static_cast<CUstream>(stream))) return -1;
        return 0;
    }

    void refgpu_close(void* h)
    {
        auto* R = static_cast<replay_t*>(h);
        if (!R) return;
        for (auto& a : R->allocs) if (a.owned && a.real) cuMemFree(a.real);
        if (R->mod) cuModuleUnload(R->mod);
        delete R;
    }
}
