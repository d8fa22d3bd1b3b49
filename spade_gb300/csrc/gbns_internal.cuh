// Internal definitions shared by the libgbns.so translation units.
#pragma once

#include <cuda_runtime.h>
#include <cuda.h>
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>

#include "gbns.h"
#include "fp64_int.cuh"

namespace gbns
{
    // ------------------------------------------------------------------
    // limits of the kernel-parameter geometry
    // ------------------------------------------------------------------
    constexpr int MAX_BLK_PER_DIM = 64;     // blocks per direction
    constexpr int MAX_YTAB        = 1024;   // doubles per stretched-metric table

    // Interior reductions: values per partial record (up to 5 sums and a
    // weight sum), the most partial records a reduction uses, and the result
    // slots after them.  Scratch for one reduction is
    // npart*RED_NVAL + RED_RESULT_SLOTS doubles.
    constexpr int RED_NVAL         = 6;
    constexpr int RED_MAX_PART     = 1024;
    constexpr int RED_RESULT_SLOTS = 8;

    // ------------------------------------------------------------------
    // error reporting (per host thread)
    // ------------------------------------------------------------------
    int set_error(int code, const std::string& msg);
    int sm_count();     // SMs of the current device
    int check_cuda(cudaError_t e, const char* what);

    // Device-side status words: kernels that give up on a bounded wait or
    // find an inconsistent launch set a nonzero code in their translation
    // unit's status word and return.  Each TU registers a reader at load.
    typedef int (*status_reader_fn)(int* status, int reset, cudaStream_t stream);
    void register_status_reader(status_reader_fn fn);
    int read_device_status(int* status, int reset, cudaStream_t stream);

    // ------------------------------------------------------------------
    // geometry passed by value to kernels
    // ------------------------------------------------------------------
    struct GeomK
    {
        int nb[3];          // blocks per direction
        int n[3];           // interior cells per block
        int ng;             // ghost layers
        int ni, nj, nk;     // padded extents
        int nblk;           // total blocks
        long long bstride;  // doubles per block (5*ni*nj*nk)
        double inv_dx[3][MAX_BLK_PER_DIM];   // 1/dx per direction per block index (grid_geometry.h:91-99)
        float inv_dx_f[3][MAX_BLK_PER_DIM];  // the same rounded to float (FP32-flux faces)
    };

    // Stretched-y metric tables, per block row by:
    //   m_cell[by*ny + j]      dy/deta at interior cell centres
    //   im_cell[by*ny + j]     1/(dy/deta) at interior cell centres (= Jacobian)
    //   im_face[by*(ny+1) + j] 1/(dy/deta) at y-faces j = 0..ny
    struct YTabK
    {
        double m_cell[MAX_YTAB];
        double im_cell[MAX_YTAB];
        double im_face[MAX_YTAB];
    };
    struct YTabNone { };

    // Runtime scheme constants (host-derived with the reference's formulas).
    struct SchemeK
    {
        int diss, visc, law, smooth, sensor;
        int hyb_flux, hyb_sensor;      // hybrid_scheme_t tag and blender kind
        double hyb_param;              // blender const_sensor_t alpha or ducros_t epsilon
        double gamma, R, gm1;          // gm1 = gamma - 1.0
        double inv_gm1, inv_R;         // 1/(gamma - 1), 1/R (FP32-flux stage update)
        double spec_heat;              // gamma*R/(gamma - 1.0)        (viscous.h:67)
        double inv_gamma_avg;          // 1.0/(0.5*(gamma + gamma))    (convective.h:226,233)
        double R_avg;                  // 0.5*(R + R)                   (convective.h:224)
        double eps_p, eps_T, sens;     // pressure_diss_lr; sens = const_sensor_t alpha or ducros_t epsilon
        double mu, beta_c, alpha_c;    // constant law: mu, -2.0*mu/3.0, mu*(1.0/Pr)
        double T_ref, power, inv_pr, prandtl, tref_plus_s, S;
        double ck_a[4];                // cent_keep centred coefficients a(1..order/2)
        // the FP32-flux kernels' copies, rounded once on the host (the same
        // bits a device conversion gives) so no thread converts them
        struct
        {
            float gamma, R, gm1, spec_heat, inv_gamma_avg, R_avg, eps_p, eps_T, sens;
            float mu, beta_c, alpha_c, T_ref, power, inv_pr, prandtl, tref_plus_s, S;
            float ck_a[4];
            float hyb_param;
        } f32;
    };

    // Arguments of one boundary_flux launch (one boundary of direction D).
    struct BndArgs
    {
        const double* prims;
        double* rhs;
        int side;                      // 0: the min boundary of direction D, 1: the max boundary
        int ntile1, ntile2;            // 8-face patches per block along the two transverse directions
        double dx[MAX_BLK_PER_DIM];    // block spacing along D (grid_geometry.h:85-89)
    };
    int boundary_flux_launch_d0(const GeomK& G, const SchemeK& S, const BndArgs& A, int conv, int order, cudaStream_t st);
    int boundary_flux_launch_d1(const GeomK& G, const SchemeK& S, const BndArgs& A, int conv, int order, cudaStream_t st);
    int boundary_flux_launch_d2(const GeomK& G, const SchemeK& S, const BndArgs& A, int conv, int order, cudaStream_t st);

    // Host helpers ------------------------------------------------------
    int make_geom(const gbns_grid_desc* g, GeomK& G);
    int make_ytab(const gbns_grid_desc* g, const GeomK& G, YTabK& Y);
    int make_scheme(const gbns_scheme_desc* s, SchemeK& S);
    int scheme_halo(const gbns_scheme_desc* s);
    double y_deriv(const gbns_grid_desc* g, double eta);

    // Tensor-map creation through the driver entry point (no -lcuda link).
    int encode_prims_tmap(CUtensorMap* map, const double* base, const GeomK& G,
                          int box_cells_x, int box_y, int box_z);

    // FP32 copy of a padded AoS5 state for the FP32-flux kernels: SoA per
    // block, float q32[lb][v][k][j][col], col = i + ng + off, rows of ipad
    // floats (a multiple of 4, so every row and the x start of every tile's
    // box are 16-byte aligned for TMA).  It lives in stream-ordered memory
    // from the library's own pool for the duration of one launch.
    struct ShadowK
    {
        float* base;
        int ipad;       // floats per row
        int off;        // column of padded index 0
    };
    // Allocates the copy on `st` (cudaMallocFromPoolAsync), converts
    // `prims` into it and encodes the tensor map of a (box_x, box_y, box_z,
    // 5) box.  `halo` is the kernel's stencil half width H: off is chosen
    // so that a tile starting at interior index i0 (a multiple of 4) has
    // its box start i0 - H + ng + off on a multiple of 4.
    int shadow_begin(const double* prims, const GeomK& G, int blk0, int blk1, int halo, int box_x, int box_y,
                     int box_z, cudaStream_t st, ShadowK& S, CUtensorMap* map);
    // Returns the copy to the pool, ordered after the kernel on `st`.
    int shadow_end(const ShadowK& S, cudaStream_t st);
    int encode_shadow_tmap(CUtensorMap* map, const ShadowK& S, const GeomK& G, int box_x, int box_y, int box_z);

    // Launchers (defined in the kernel translation units) -----------------
    struct RkFuse;
    int launch_flux_div(const gbns_grid_desc* g, const GeomK& G, const YTabK* Y, const SchemeK& S,
                        const gbns_scheme_desc* desc, const double* prims, double* rhs,
                        int increment, cudaStream_t stream, int variant, const RkFuse* fuse = nullptr,
                        int blk0 = 0, int blk1 = -1, const double* blk_inv_dx = nullptr);
    // Stream-ordered device memory from the library's own pool (released
    // with cudaFreeAsync on the same stream).
    int pool_alloc(void** p, size_t bytes, cudaStream_t st);
    // The cells per block, ghost layers and block count an exchange plan was
    // created for (exchange.cu).
    int exchange_plan_shape(const gbns_exchange_plan* P, int* nx, int* ny, int* nz, int* ng, int* nblocks);
    // Wall faces of a refined layout (grid nblk = (N, 1, 1), 6 box doubles per
    // block): per face f the blocks whose box touches domain face f
    // (grid->bounds[f]), idx[off[f] .. off[f+1]); faces that are not walls
    // have none (exchange.cu).
    struct WallLists
    {
        std::vector<int> idx;
        int off[7];
    };
    int wall_lists(const gbns_grid_desc* g, const double* boxes, const gbns_bc_desc* bc, WallLists& W);
    // One launch per wall face in face order (boundary_fill's order), d_idx
    // the lists in device memory.
    int launch_wall_fill(const gbns_grid_desc* g, const gbns_bc_desc* bc, const WallLists& W, const int* d_idx,
                         double* prims, cudaStream_t st);
    // gbns_flux_div_rk over the blocks blk0 .. blk1 - 1 (host.cu)
    int flux_div_rk_range(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* prims,
                          double* rhs, int write_rhs, int nres, const double* const* earlier,
                          const double* coeffs, double* q_out, void* stream, int blk0, int blk1);
    // blk0 .. blk1 - 1: the blocks whose cells the launch writes (blk1 = -1: to the last block)
    int launch_copy_fill(const GeomK& G, const gbns_bc_desc* bc, double* dst, const double* src, cudaStream_t stream,
                         int blk0 = 0, int blk1 = -1);
    int launch_fill_ghosts(const GeomK& G, const gbns_bc_desc* bc, double* prims, cudaStream_t stream,
                           int blk0 = 0, int blk1 = -1);
    int launch_rk_stage(const GeomK& G, double gamma, double R, double* prims,
                        const double* const* res, const double* coeffs, int nres, cudaStream_t stream);
    int launch_reduce(const gbns_grid_desc* g, const GeomK& G, double gamma, double R, const double* prims,
                      int kind, double* partials, int npart, cudaStream_t stream);

    // ------------------------------------------------------------------
    // device helpers
    // ------------------------------------------------------------------
    namespace
    {
        __device__ int g_device_status = 0;   // one per translation unit

        int read_tu_status(int* status, int reset, cudaStream_t stream)
        {
            int v = 0;
            cudaError_t e = cudaMemcpyFromSymbolAsync(&v, g_device_status, sizeof(int), 0, cudaMemcpyDeviceToHost, stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
            if (e != cudaSuccess) return check_cuda(e, "read device status");
            if (v && !*status) *status = v;
            if (reset && v)
            {
                const int zero = 0;
                e = cudaMemcpyToSymbolAsync(g_device_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
                if (e != cudaSuccess) return check_cuda(e, "reset device status");
            }
            return GBNS_OK;
        }

        struct status_registrar
        {
            status_registrar() { register_status_reader(read_tu_status); }
        };
    }

    // Bounded mbarrier wait: returns false if the phase did not complete
    // within `max_cycles` SM clock cycles (then the caller flags an error and
    // returns).  Each try_wait suspends for at most ~2 us (suspend-time hint),
    // so the bound holds whatever the hardware's default suspend window is.
    __device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long max_cycles)
    {
        const uint32_t addr = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
        const long long t0 = clock64();
        for (;;)
        {
            uint32_t done;
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(done) : "r"(addr), "r"(parity), "r"(2000u) : "memory");
            if (done) return true;
            if (clock64() - t0 > max_cycles) return false;
        }
    }

    __device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
    {
        const uint32_t addr = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(addr), "r"(count) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }

    __device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
    {
        const uint32_t addr = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(addr), "r"(bytes) : "memory");
    }

    __device__ __forceinline__ void mbar_inval(uint64_t* bar)
    {
        const uint32_t addr = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" :: "r"(addr) : "memory");
    }

    // 4-D tiled TMA load global -> shared, completion on `bar`.
    __device__ __forceinline__ void tma_load_4d(void* smem_dst, const CUtensorMap* map, uint64_t* bar,
                                                int c0, int c1, int c2, int c3)
    {
        const uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(smem_dst));
        const uint32_t mb  = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
        asm volatile(
            "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
            " [%0], [%1, {%2, %3, %4, %5}], [%6];"
            :: "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(mb)
            : "memory");
    }

    // A tensor map that a host copy wrote to global memory, made visible to
    // the tensor proxy (the TMA unit) before this thread's first copy with it.
    __device__ __forceinline__ void tensormap_acquire(const CUtensorMap* map)
    {
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;"
                     :: "l"(reinterpret_cast<uint64_t>(map)) : "memory");
    }

    constexpr long long MBAR_WAIT_CYCLES = 2000000000ll;   // ~1 s at 2 GHz

    // fluid_state::convert_state prim -> cons and cons -> prim
    // (navier-stokes/fluid_state.h:151-184), in the reference's operation order.
    // a*b, a/b and x/2 in FP64: with IM on the integer pipes (dmul_int,
    // ddiv_int, dmul_pow2), the same bits as the FP64 unit's
    template <bool IM>
    __device__ __forceinline__ double pmul64(double a, double b)
    {
        if constexpr (IM) return dmul_int(a, b);
        else return a*b;
    }
    template <bool IM>
    __device__ __forceinline__ double pdiv64(double a, double b)
    {
        if constexpr (IM) return ddiv_int(a, b);
        else return a/b;
    }
    template <bool IM>
    __device__ __forceinline__ double phalf64(double x)
    {
        if constexpr (IM) return dmul_pow2<-1>(x);
        else return 0.5*x;
    }

    // (IM: products on the integer pipes; ID: quotients there)
    template <bool IM = false, bool ID = IM>
    __device__ __forceinline__ void prim_to_cons(const double q[5], const double R, const double gm1, double c[5])
    {
        const double rho = pdiv64<ID>(q[0], pmul64<IM>(R, q[1]));
        const double rhoU2 = pmul64<IM>(rho, (pmul64<IM>(q[2], q[2]) + pmul64<IM>(q[3], q[3]) + pmul64<IM>(q[4], q[4])));
        c[0] = rho;
        c[1] = phalf64<IM>(rhoU2) + pdiv64<ID>(q[0], gm1);
        c[2] = pmul64<IM>(rho, q[2]);
        c[3] = pmul64<IM>(rho, q[3]);
        c[4] = pmul64<IM>(rho, q[4]);
    }

    template <bool IM = false, bool ID = IM>
    __device__ __forceinline__ void cons_to_prim(const double c[5], const double R, const double gm1, double q[5])
    {
        const double rh = c[0];
        const double invrho = pdiv64<ID>(1.0, rh);
        const double uu = pmul64<IM>(invrho, c[2]), vv = pmul64<IM>(invrho, c[3]), ww = pmul64<IM>(invrho, c[4]);
        const double ru2 = pmul64<IM>(rh, (pmul64<IM>(uu, uu) + pmul64<IM>(vv, vv) + pmul64<IM>(ww, ww)));
        const double pp = pmul64<IM>(gm1, (c[1] - phalf64<IM>(ru2)));
        q[0] = pp;
        q[1] = pdiv64<ID>(pp, pmul64<IM>(R, rh));
        q[2] = uu;
        q[3] = vv;
        q[4] = ww;
    }

    // The same conversions with two reciprocals instead of four divisions, for
    // the FP32-flux form's stage update (FP64 state; not bit-identical to the
    // reference's rounding, which only the FP64 drop-in promises).
    // (IM: the two reciprocals on the integer pipes, ddiv_int: the same bits)
    template <bool IM = false>
    __device__ __forceinline__ void prim_to_cons_fast(const double q[5], const double R, const double inv_gm1,
                                                      double c[5])
    {
        const double rho = q[0]*(IM ? ddiv_int(1.0, R*q[1]) : 1.0/(R*q[1]));
        const double rhoU2 = rho*(q[2]*q[2] + q[3]*q[3] + q[4]*q[4]);
        c[0] = rho;
        c[1] = 0.5*rhoU2 + q[0]*inv_gm1;
        c[2] = rho*q[2];
        c[3] = rho*q[3];
        c[4] = rho*q[4];
    }

    template <bool IM = false>
    __device__ __forceinline__ void cons_to_prim_fast(const double c[5], const double inv_R, const double gm1,
                                                      double q[5])
    {
        const double rh = c[0];
        const double invrho = IM ? ddiv_int(1.0, rh) : 1.0/rh;
        const double uu = invrho*c[2], vv = invrho*c[3], ww = invrho*c[4];
        const double ru2 = rh*(uu*uu + vv*vv + ww*ww);
        const double pp = gm1*(c[1] - 0.5*ru2);
        q[0] = pp;
        q[1] = (pp*invrho)*inv_R;
        q[2] = uu;
        q[3] = vv;
        q[4] = ww;
    }

    enum device_status_code
    {
        DEV_OK = GBNS_DEV_OK,
        DEV_TMA_TIMEOUT = GBNS_DEV_TMA_TIMEOUT,
        DEV_BAD_LAUNCH = 2
    };
}
