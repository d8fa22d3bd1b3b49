// Host side of libgbns.so: descriptor validation and lowering, geometry
// tables, TMA tensor maps, error reporting and the C-ABI entry points.
#include <cstdio>
#include <cstring>
#include <cmath>
#include <string>
#include <mutex>
#include <vector>

#include "gbns_internal.cuh"
#include "flux_launch.cuh"
#include <cstring>

namespace gbns
{
    static thread_local std::string t_last_error;

    static std::mutex& readers_mu() { static std::mutex m; return m; }
    static std::vector<status_reader_fn>& readers() { static std::vector<status_reader_fn> v; return v; }

    void register_status_reader(status_reader_fn fn)
    {
        std::lock_guard<std::mutex> lk(readers_mu());
        readers().push_back(fn);
    }

    int read_device_status(int* status, int reset, cudaStream_t stream)
    {
        *status = 0;
        std::vector<status_reader_fn> fns;
        {
            std::lock_guard<std::mutex> lk(readers_mu());
            fns = readers();
        }
        for (auto fn : fns)
        {
            int rc = fn(status, reset, stream);
            if (rc) return rc;
        }
        return GBNS_OK;
    }

    int set_error(int code, const std::string& msg)
    {
        t_last_error = msg;
        return code;
    }

    int check_cuda(cudaError_t e, const char* what)
    {
        if (e == cudaSuccess) return GBNS_OK;
        return set_error(GBNS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }

    // Block geometry exactly as the reference derives it:
    // cartesian_blocks.h:49 (bsize), :69-70 (box), cartesian_grid.h:134-135
    // (dx = box.size/n, inv_dx = 1/dx).
    static void block_dx(const gbns_grid_desc* g, int d, int b, double* bmin, double* dx)
    {
        const double bsize = (g->bounds[2*d+1] - g->bounds[2*d]) / g->nblk[d];
        const double mn = g->bounds[2*d] + b*bsize;
        const double mx = mn + bsize;
        *bmin = mn;
        *dx = (mx - mn) / g->ncell[d];
    }

    double y_deriv(const gbns_grid_desc* g, double eta)
    {
        if (g->coords == GBNS_COORDS_TANH_Y)
        {
            const double beta = g->coord_param[0];
            const double y0 = g->bounds[2], y1 = g->bounds[3];
            const double s = (2.0*eta - (y0 + y1)) / (y1 - y0);
            const double th = tanh(beta*s);
            return beta*(1.0 - th*th)/tanh(beta);
        }
        if (g->coords == GBNS_COORDS_INTEGRATED_TANH_Y)
        {
            // coords::integrated_tanh_1D::coord_deriv (core/coord_system.h:103-140)
            const double eta1 = g->coord_param[0], eta0 = g->coord_param[1];
            const double deta = eta1 - eta0;
            const double k = g->coord_param[3], strch = g->coord_param[2];
            const double alpha0 = k/deta, alpha1 = -k/deta;
            const double beta0 = alpha0*(strch*deta - eta0);
            const double beta1 = alpha0*(eta1 + strch*deta);
            auto f = [&](double e) { return log(fabs(cosh(alpha0*e + beta0)))/alpha0 + log(fabs(cosh(alpha1*e + beta1)))/alpha1 - e; };
            const double f0 = f(eta0);
            const double normInv = 1.0/(f(eta1) - f0);
            return (deta*(tanh(alpha0*eta + beta0) + tanh(alpha1*eta + beta1) - 1.0))*normInv;
        }
        return 1.0;
    }

    static int validate_grid(const gbns_grid_desc* g)
    {
        if (!g) return set_error(GBNS_ERR_INVALID, "grid descriptor is NULL");
        for (int d = 0; d < 3; ++d)
        {
            if (g->nblk[d] < 1 || g->nblk[d] > MAX_BLK_PER_DIM)
                return set_error(GBNS_ERR_INVALID, "blocks per direction must be in [1, 64]");
            if (g->ncell[d] < 1) return set_error(GBNS_ERR_INVALID, "cells per block must be >= 1");
            if (!(g->bounds[2*d+1] > g->bounds[2*d])) return set_error(GBNS_ERR_INVALID, "domain bounds must satisfy min < max");
        }
        if (g->ng < 1 || g->ng > 8) return set_error(GBNS_ERR_INVALID, "ghost layers must be in [1, 8]");
        if (g->coords < GBNS_COORDS_IDENTITY || g->coords > GBNS_COORDS_INTEGRATED_TANH_Y)
            return set_error(GBNS_ERR_INVALID, "unknown coordinate system");
        const double cells = double(g->nblk[0])*g->nblk[1]*g->nblk[2]*
                             (g->ncell[0] + 2.0*g->ng)*(g->ncell[1] + 2.0*g->ng)*(g->ncell[2] + 2.0*g->ng);
        if (cells*5 > 9.0e18) return set_error(GBNS_ERR_INVALID, "grid too large");
        return GBNS_OK;
    }

    int make_geom(const gbns_grid_desc* g, GeomK& G)
    {
        int rc = validate_grid(g);
        if (rc) return rc;
        std::memset(&G, 0, sizeof(G));
        for (int d = 0; d < 3; ++d) { G.nb[d] = g->nblk[d]; G.n[d] = g->ncell[d]; }
        G.ng = g->ng;
        G.ni = G.n[0] + 2*G.ng;
        G.nj = G.n[1] + 2*G.ng;
        G.nk = G.n[2] + 2*G.ng;
        G.nblk = G.nb[0]*G.nb[1]*G.nb[2];
        G.bstride = 5ll*G.ni*G.nj*G.nk;
        for (int d = 0; d < 3; ++d)
            for (int b = 0; b < G.nb[d]; ++b)
            {
                double mn, dx;
                block_dx(g, d, b, &mn, &dx);
                G.inv_dx[d][b] = 1.0/dx;
                G.inv_dx_f[d][b] = float(G.inv_dx[d][b]);
            }
        return GBNS_OK;
    }

    int make_ytab(const gbns_grid_desc* g, const GeomK& G, YTabK& Y)
    {
        const int ny = G.n[1];
        if (G.nb[1]*(ny + 1) > MAX_YTAB)
            return set_error(GBNS_ERR_UNSUPPORTED, "stretched-y metric table exceeds 1024 entries (blocks_y*(ny+1))");
        for (int by = 0; by < G.nb[1]; ++by)
        {
            double bmin, dy;
            block_dx(g, 1, by, &bmin, &dy);
            for (int j = 0; j < ny; ++j)
            {
                const double m = y_deriv(g, bmin + ((double)j + 0.5)*dy);
                Y.m_cell[by*ny + j] = m;
                Y.im_cell[by*ny + j] = 1.0/m;
            }
            for (int j = 0; j <= ny; ++j)
                Y.im_face[by*(ny + 1) + j] = 1.0/y_deriv(g, bmin + (double)j*dy);
        }
        return GBNS_OK;
    }

    static double cfd_coeff(int idx, int order)
    {
        // centered_finite_diff_t<idx, order>::value (core/finite_diff.h:25-34)
        const int h = order/2;
        double fh = 1, fhp = 1, fhm = 1;
        for (int i = 2; i <= h; ++i) fh *= i;
        for (int i = 2; i <= h + idx; ++i) fhp *= i;
        for (int i = 2; i <= h - idx; ++i) fhm *= i;
        const double d0 = fh/fhp;
        const double d1 = fh/fhm;
        const double sgn = ((1 + idx) % 2 == 0) ? 1.0 : -1.0;
        return d0*d1*sgn/(double)idx;
    }

    int scheme_halo(const gbns_scheme_desc* s)
    {
        int h = 0;
        if (s->convective == GBNS_CONV_CENT_KEEP) h = s->order/2;
        else if (s->convective == GBNS_CONV_TOTANI) h = 1;
        else if (s->convective == GBNS_CONV_FWENO) h = 2;
        else if (s->convective == GBNS_CONV_WENO5) h = 3;
        else if (s->convective == GBNS_CONV_HYBRID) h = s->order/2 > 2 ? s->order/2 : 2;
        if ((s->dissipation || s->viscous) && h < 1) h = 1;   // ducros_t's face gradient needs 1 too
        return h;
    }

    int make_scheme(const gbns_scheme_desc* s, SchemeK& S)
    {
        if (!s) return set_error(GBNS_ERR_INVALID, "scheme descriptor is NULL");
        if (s->convective < GBNS_CONV_NONE || s->convective > GBNS_CONV_HYBRID)
            return set_error(GBNS_ERR_INVALID, "unknown convective scheme");
        if (s->convective == GBNS_CONV_CENT_KEEP && !(s->order == 2 || s->order == 4 || s->order == 6 || s->order == 8))
            return set_error(GBNS_ERR_UNSUPPORTED, "cent_keep order must be 2, 4, 6 or 8");
        if (s->convective == GBNS_CONV_HYBRID)
        {
            if (!(s->order == 2 || s->order == 4))
                return set_error(GBNS_ERR_UNSUPPORTED, "hybrid_scheme_t is lowered with cent_keep order 2 or 4");
            if (s->hybrid_flux != GBNS_HYBRID_FULL_FLUX && s->hybrid_flux != GBNS_HYBRID_DISS_FLUX)
                return set_error(GBNS_ERR_INVALID, "unknown hybrid flux tag");
            if (s->hybrid_sensor != GBNS_SENSOR_CONST && s->hybrid_sensor != GBNS_SENSOR_DUCROS)
                return set_error(GBNS_ERR_UNSUPPORTED, "unknown hybrid blender");
        }
        if (s->dissipation < 0 || s->dissipation > GBNS_DISS_PRESSURE) return set_error(GBNS_ERR_INVALID, "unknown dissipation");
        if (s->dissipation && s->sensor != GBNS_SENSOR_CONST && s->sensor != GBNS_SENSOR_DUCROS)
            return set_error(GBNS_ERR_UNSUPPORTED, "unknown shock sensor");
        if (s->viscous < 0 || s->viscous > GBNS_VISC_LR) return set_error(GBNS_ERR_INVALID, "unknown viscous scheme");
        if (s->viscous && (s->visc_law < GBNS_LAW_CONSTANT || s->visc_law > GBNS_LAW_SUTHERLAND))
            return set_error(GBNS_ERR_INVALID, "unknown viscosity law");
        if (s->precision != GBNS_PREC_FP64 && s->precision != GBNS_PREC_FP32_FLUX && s->precision != GBNS_PREC_FP64_FMA)
            return set_error(GBNS_ERR_INVALID, "unknown precision");
        if (!(s->gas.gamma > 1.0) || !(s->gas.R > 0.0)) return set_error(GBNS_ERR_INVALID, "gas requires gamma > 1 and R > 0");
        if (s->viscous && !(s->prandtl > 0.0)) return set_error(GBNS_ERR_INVALID, "viscous scheme requires prandtl > 0");
        std::memset(&S, 0, sizeof(S));
        S.diss = s->dissipation;
        S.visc = s->viscous;
        S.law = s->visc_law;
        S.smooth = s->weno_smooth;
        S.sensor = s->sensor;
        S.hyb_flux = s->hybrid_flux;
        S.hyb_sensor = s->hybrid_sensor;
        S.hyb_param = s->hybrid_param;
        const double gam = s->gas.gamma, R = s->gas.R;
        S.gamma = gam; S.R = R;
        S.gm1 = gam - 1.0;
        S.inv_gm1 = 1.0/(gam - 1.0);
        S.inv_R = 1.0/R;
        S.spec_heat = gam*R/(gam - 1.0);
        S.inv_gamma_avg = 1.0/(0.5*(gam + gam));
        S.R_avg = 0.5*(R + R);
        S.eps_p = s->eps_p; S.eps_T = s->eps_T; S.sens = s->sensor_alpha;
        S.mu = s->mu;
        S.beta_c = -2.0*s->mu/3.0;
        S.inv_pr = s->prandtl_inv > 0.0 ? s->prandtl_inv : 1.0/s->prandtl;
        S.alpha_c = s->mu*S.inv_pr;
        S.T_ref = s->T_ref; S.power = s->power; S.prandtl = s->prandtl;
        S.tref_plus_s = s->T_ref + s->S;
        S.S = s->S;
        if (s->convective == GBNS_CONV_CENT_KEEP || s->convective == GBNS_CONV_HYBRID)
            for (int ii = 1; ii <= s->order/2; ++ii) S.ck_a[ii - 1] = cfd_coeff(ii, s->order);
        S.f32.gamma = float(S.gamma); S.f32.R = float(S.R); S.f32.gm1 = float(S.gm1);
        S.f32.spec_heat = float(S.spec_heat); S.f32.inv_gamma_avg = float(S.inv_gamma_avg);
        S.f32.R_avg = float(S.R_avg); S.f32.eps_p = float(S.eps_p); S.f32.eps_T = float(S.eps_T);
        S.f32.sens = float(S.sens); S.f32.mu = float(S.mu); S.f32.beta_c = float(S.beta_c);
        S.f32.alpha_c = float(S.alpha_c); S.f32.T_ref = float(S.T_ref); S.f32.power = float(S.power);
        S.f32.inv_pr = float(S.inv_pr); S.f32.prandtl = float(S.prandtl); S.f32.tref_plus_s = float(S.tref_plus_s);
        S.f32.S = float(S.S); S.f32.hyb_param = float(S.hyb_param);
        for (int ii = 0; ii < 4; ++ii) S.f32.ck_a[ii] = float(S.ck_a[ii]);
        return GBNS_OK;
    }

    // cuTensorMapEncodeTiled fetched through the runtime's driver entry point.
    typedef CUresult (*encode_tiled_fn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                        const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                        CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

    static encode_tiled_fn get_encode_fn()
    {
        static encode_tiled_fn fn = nullptr;
        static std::once_flag once;
        std::call_once(once, []()
        {
            void* p = nullptr;
            cudaDriverEntryPointQueryResult q;
            if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
                q == cudaDriverEntryPointSuccess)
                fn = reinterpret_cast<encode_tiled_fn>(p);
        });
        return fn;
    }

    int encode_prims_tmap(CUtensorMap* map, const double* base, const GeomK& G, int box_cells_x, int box_y, int box_z)
    {
        encode_tiled_fn fn = get_encode_fn();
        if (!fn) return set_error(GBNS_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        const cuuint64_t dims[4] = {cuuint64_t(G.ni)*5, cuuint64_t(G.nj), cuuint64_t(G.nk), cuuint64_t(G.nblk)};
        const cuuint64_t strides[3] = {cuuint64_t(G.ni)*5*8, cuuint64_t(G.ni)*G.nj*5*8, cuuint64_t(G.ni)*G.nj*G.nk*5*8};
        const cuuint32_t box[4] = {cuuint32_t(box_cells_x*5), cuuint32_t(box_y), cuuint32_t(box_z), 1};
        const cuuint32_t estr[4] = {1, 1, 1, 1};
        CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, const_cast<double*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return set_error(GBNS_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string(int(r)) + ")");
        return GBNS_OK;
    }

    int encode_shadow_tmap(CUtensorMap* map, const ShadowK& S, const GeomK& G, int box_x, int box_y, int box_z)
    {
        encode_tiled_fn fn = get_encode_fn();
        if (!fn) return set_error(GBNS_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        // (col, j, k, v + 5*lb): one box brings all five variables of a tile
        // box into shared memory as SoA planes
        const cuuint64_t plane = cuuint64_t(S.ipad)*G.nj*G.nk;
        const cuuint64_t dims[4] = {cuuint64_t(S.ipad), cuuint64_t(G.nj), cuuint64_t(G.nk), cuuint64_t(5)*G.nblk};
        const cuuint64_t strides[3] = {cuuint64_t(S.ipad)*4, cuuint64_t(S.ipad)*G.nj*4, plane*4};
        const cuuint32_t box[4] = {cuuint32_t(box_x), cuuint32_t(box_y), cuuint32_t(box_z), 5};
        const cuuint32_t estr[4] = {1, 1, 1, 1};
        CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, S.base, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return set_error(GBNS_ERR_CUDA, "cuTensorMapEncodeTiled (FP32 copy) failed (" + std::to_string(int(r)) + ")");
        return GBNS_OK;
    }

    static int validate_bc(const gbns_bc_desc* bc)
    {
        if (!bc) return set_error(GBNS_ERR_INVALID, "bc descriptor is NULL");
        for (int d = 0; d < 3; ++d)
        {
            for (int s = 0; s < 2; ++s)
                if (bc->kind[2*d+s] < GBNS_BC_PERIODIC || bc->kind[2*d+s] > GBNS_BC_SLIP_ADIABATIC)
                    return set_error(GBNS_ERR_INVALID, "unknown boundary kind");
            if ((bc->kind[2*d] == GBNS_BC_PERIODIC) != (bc->kind[2*d+1] == GBNS_BC_PERIODIC))
                return set_error(GBNS_ERR_INVALID, "periodic boundaries must be paired");
        }
        return GBNS_OK;
    }
}

using namespace gbns;

namespace gbns
{
    // Graphs of one fused SSPRK3 step (gbns_ssprk3_run), keyed on the
    // descriptors, pointers, dt and device they bake in; at most 8 kept.
    struct StepKey
    {
        gbns_grid_desc grid;
        gbns_scheme_desc scheme;
        gbns_bc_desc bc;
        double* prims;
        double* work;
        double dt;
        int device;
    };
    struct StepGraph
    {
        StepKey key;
        cudaGraphExec_t exec;
    };
    static std::mutex& step_graphs_mu() { static std::mutex m; return m; }
    static std::vector<StepGraph>& step_graphs() { static std::vector<StepGraph> v; return v; }
}

extern "C"
{
    int gbns_version(void) { return GBNS_ABI_VERSION; }

    int gbns_last_error(char* buf, size_t len)
    {
        if (!buf || len == 0) return GBNS_ERR_INVALID;
        std::snprintf(buf, len, "%s", t_last_error.c_str());
        return GBNS_OK;
    }

    int gbns_array_size(const gbns_grid_desc* grid, size_t* count)
    {
        GeomK G;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        if (!count) return set_error(GBNS_ERR_INVALID, "count is NULL");
        *count = size_t(G.bstride)*G.nblk;
        return GBNS_OK;
    }

    int gbns_flux_div(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                      const double* prims, double* rhs, int increment, void* stream)
    {
        GeomK G;
        SchemeK S;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        rc = make_scheme(scheme, S);
        if (rc) return rc;
        if (!prims || !rhs) return set_error(GBNS_ERR_INVALID, "prims/rhs pointer is NULL");
        if (prims == rhs) return set_error(GBNS_ERR_INVALID, "prims and rhs must not alias");
        if (scheme_halo(scheme) > G.ng)
            return set_error(GBNS_ERR_INVALID, "scheme stencil needs " + std::to_string(scheme_halo(scheme)) +
                             " ghost layers, grid has " + std::to_string(G.ng));
        YTabK* Y = nullptr;
        static thread_local YTabK ytab;
        if (grid->coords != GBNS_COORDS_IDENTITY)
        {
            rc = make_ytab(grid, G, ytab);
            if (rc) return rc;
            Y = &ytab;
        }
        return launch_flux_div(grid, G, Y, S, scheme, prims, rhs, increment, static_cast<cudaStream_t>(stream),
                               scheme->tile_variant);
    }

    // The checks and the per-block 1/dx table of a refined layout, and the
    // table in stream-ordered device memory (the caller frees *dinv on st).
    static int blocks_setup(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* block_bounds,
                            gbns::GeomK& G, gbns::SchemeK& S, cudaStream_t st, double** dinv)
    {
        using namespace gbns;
        *dinv = nullptr;
        if (!grid) return set_error(GBNS_ERR_INVALID, "grid descriptor is NULL");
        const int nblk = grid->nblk[0];
        if (nblk < 1 || nblk > 65535 || grid->nblk[1] != 1 || grid->nblk[2] != 1)
            return set_error(GBNS_ERR_INVALID, "a refined layout's blocks are given as nblk = (1..65535, 1, 1)");
        if (grid->coords != GBNS_COORDS_IDENTITY)
            return set_error(GBNS_ERR_UNSUPPORTED, "refined layouts take identity coordinates");
        if (!block_bounds) return set_error(GBNS_ERR_INVALID, "block_bounds is NULL");
        // the descriptor checks of one block, then the whole layout
        gbns_grid_desc one = *grid;
        one.nblk[0] = 1;
        int rc = make_geom(&one, G);
        if (rc) return rc;
        G.nb[0] = nblk;
        G.nblk = nblk;
        if (double(nblk)*double(G.bstride) > 9.0e18) return set_error(GBNS_ERR_INVALID, "grid too large");
        rc = make_scheme(scheme, S);
        if (rc) return rc;
        if (scheme_halo(scheme) > G.ng)
            return set_error(GBNS_ERR_INVALID, "scheme stencil needs " + std::to_string(scheme_halo(scheme)) +
                             " ghost layers, grid has " + std::to_string(G.ng));
        // per-block 1/dx as the reference forms it: dx = box size / cells
        std::vector<double> inv(3*size_t(nblk));
        for (int lb = 0; lb < nblk; ++lb)
            for (int d = 0; d < 3; ++d)
            {
                const double mn = block_bounds[6*lb + 2*d], mx = block_bounds[6*lb + 2*d + 1];
                if (!(mx > mn) || !std::isfinite(mn) || !std::isfinite(mx))
                    return set_error(GBNS_ERR_INVALID, "block " + std::to_string(lb) + ": bounds must be finite with min < max");
                const double dx = (mx - mn)/G.n[d];
                inv[3*lb + d] = 1.0/dx;
            }
        void* p = nullptr;
        rc = pool_alloc(&p, inv.size()*sizeof(double), st);
        if (rc) return rc;
        rc = check_cuda(cudaMemcpyAsync(p, inv.data(), inv.size()*sizeof(double), cudaMemcpyHostToDevice, st),
                        "per-block spacing to the device");
        if (rc) { cudaFreeAsync(p, st); return rc; }
        *dinv = static_cast<double*>(p);
        return GBNS_OK;
    }

    int gbns_flux_div_blocks(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* block_bounds,
                             const double* prims, double* rhs, int increment, void* stream)
    {
        using namespace gbns;
        if (!prims || !rhs) return set_error(GBNS_ERR_INVALID, "prims/rhs pointer is NULL");
        if (prims == rhs) return set_error(GBNS_ERR_INVALID, "prims and rhs must not alias");
        const cudaStream_t st = static_cast<cudaStream_t>(stream);
        GeomK G;
        SchemeK S;
        double* dinv = nullptr;
        int rc = blocks_setup(grid, scheme, block_bounds, G, S, st, &dinv);
        if (rc) return rc;
        rc = launch_flux_div(grid, G, nullptr, S, scheme, prims, rhs, increment, st, scheme->tile_variant, nullptr,
                             0, G.nblk, dinv);
        const int frc = check_cuda(cudaFreeAsync(dinv, st), "per-block spacing (pool free)");
        return rc ? rc : frc;
    }

    // The wall lists of a refined layout in stream-ordered device memory
    // (*d_idx stays NULL when no block touches a wall face; the caller frees
    // it on st).
    static int upload_walls(const gbns_grid_desc* grid, const double* boxes, const gbns_bc_desc* bc,
                            gbns::WallLists& W, int** d_idx, cudaStream_t st)
    {
        using namespace gbns;
        *d_idx = nullptr;
        for (int f = 0; f < 7; ++f) W.off[f] = 0;
        W.idx.clear();
        if (!bc) return GBNS_OK;
        int rc = wall_lists(grid, boxes, bc, W);
        if (rc || W.idx.empty()) return rc;
        void* p = nullptr;
        rc = pool_alloc(&p, W.idx.size()*sizeof(int), st);
        if (rc) return rc;
        rc = check_cuda(cudaMemcpyAsync(p, W.idx.data(), W.idx.size()*sizeof(int), cudaMemcpyHostToDevice, st),
                        "wall lists to the device");
        if (rc) { cudaFreeAsync(p, st); return rc; }
        *d_idx = static_cast<int*>(p);
        return GBNS_OK;
    }

    int gbns_wall_fill_blocks(const gbns_grid_desc* grid, const double* block_bounds, const gbns_bc_desc* bc,
                              double* prims, void* stream)
    {
        using namespace gbns;
        if (!grid || !block_bounds || !bc || !prims) return set_error(GBNS_ERR_INVALID, "NULL argument");
        const int nblk = grid->nblk[0];
        if (nblk < 1 || nblk > 65535 || grid->nblk[1] != 1 || grid->nblk[2] != 1)
            return set_error(GBNS_ERR_INVALID, "a refined layout's blocks are given as nblk = (1..65535, 1, 1)");
        gbns_grid_desc one = *grid;
        one.nblk[0] = 1;
        size_t per_block = 0;
        int rc = gbns_array_size(&one, &per_block);
        if (rc) return rc;
        const cudaStream_t st = static_cast<cudaStream_t>(stream);
        WallLists W;
        int* d_idx = nullptr;
        rc = upload_walls(grid, block_bounds, bc, W, &d_idx, st);
        if (rc || !d_idx) return rc;
        rc = launch_wall_fill(grid, bc, W, d_idx, prims, st);
        const int frc = check_cuda(cudaFreeAsync(d_idx, st), "wall lists (pool free)");
        return rc ? rc : frc;
    }

    int gbns_ssprk3_step_blocks(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* block_bounds,
                                gbns_exchange_plan* plan, const gbns_bc_desc* bc, double* prims, double* work, double dt,
                                void* stream)
    {
        using namespace gbns;
        if (!prims || !work) return set_error(GBNS_ERR_INVALID, "prims/work pointer is NULL");
        int px = 0, py = 0, pz = 0, pg = 0, pn = 0;
        int rc = exchange_plan_shape(plan, &px, &py, &pz, &pg, &pn);
        if (rc) return rc;
        if (!grid) return set_error(GBNS_ERR_INVALID, "grid descriptor is NULL");
        if (px != grid->ncell[0] || py != grid->ncell[1] || pz != grid->ncell[2] || pg != grid->ng || pn != grid->nblk[0])
            return set_error(GBNS_ERR_INVALID, "the exchange plan was created for another block layout");
        const cudaStream_t st = static_cast<cudaStream_t>(stream);
        GeomK G;
        SchemeK S;
        double* dinv = nullptr;
        rc = blocks_setup(grid, scheme, block_bounds, G, S, st, &dinv);
        if (rc) return rc;
        WallLists W;
        int* d_walls = nullptr;
        rc = upload_walls(grid, block_bounds, bc, W, &d_walls, st);
        if (rc) { cudaFreeAsync(dinv, st); return rc; }
        // the boundary condition: the exchange, then the walls (apply_bc's order)
        auto fill = [&](double* a) -> int
        {
            int r = gbns_exchange_plan_run(plan, a, stream);
            if (!r && d_walls) r = launch_wall_fill(grid, bc, W, d_walls, a, st);
            return r;
        };
        const size_t n = size_t(G.bstride)*G.nblk;
        double* R0 = work;
        double* R1 = work + n;
        double* B = work + 2*n;      // the state between stages
        // ratio_diff_t of consecutive ssprk3_t rows (explicit.h:80-88, advance.h:80-95)
        const double c[3][3] = {{(1.0/1.0)*dt, 0.0, 0.0}, {(-3.0/4.0)*dt, (1.0/4.0)*dt, 0.0},
                                {(-1.0/12.0)*dt, (-1.0/12.0)*dt, (2.0/3.0)*dt}};
        auto stage = [&](int k, const double* in, double* res, double* out) -> int
        {
            RkFuse f;
            std::memset(&f, 0, sizeof(f));
            f.nres = k + 1;
            f.write_rhs = res ? 1 : 0;
            f.res[0] = R0;
            f.res[1] = R1;
            for (int j = 0; j <= k; ++j) f.coeff[j] = c[k][j];
            f.q_out = out;
            return launch_flux_div(grid, G, nullptr, S, scheme, in, res ? res : out, 0, st, scheme->tile_variant, &f,
                                   0, G.nblk, dinv);
        };
        // Each stage's output array starts as a copy of its input, so before
        // the exchange it holds the ghost values the in-place update would:
        // the plan can read ghost donors before it writes them (two levels
        // with walls), and the ghosts it never writes keep their values.
        auto copy = [&](double* dst, const double* src) -> int
        {
            return check_cuda(cudaMemcpyAsync(dst, src, n*sizeof(double), cudaMemcpyDeviceToDevice, st), "state copy");
        };
        rc = copy(B, prims);
        if (!rc) rc = stage(0, prims, R0, B);
        if (!rc) rc = fill(B);
        if (!rc) rc = copy(prims, B);
        if (!rc) rc = stage(1, B, R1, prims);
        if (!rc) rc = fill(prims);
        if (!rc) rc = copy(B, prims);
        if (!rc) rc = stage(2, prims, nullptr, B);
        if (!rc) rc = fill(B);
        if (!rc) rc = copy(prims, B);
        int frc = check_cuda(cudaFreeAsync(dinv, st), "per-block spacing (pool free)");
        if (d_walls && !frc) frc = check_cuda(cudaFreeAsync(d_walls, st), "wall lists (pool free)");
        return rc ? rc : frc;
    }

    // Runs fn(ctx, q, r) on device copies of host prims and rhs (count
    // doubles each) and copies rhs back: one pair of staging arrays per
    // device, grown on demand; the lock covers the whole call so concurrent
    // host-path calls never share them.  Synchronises `stream`.
    typedef int (*staged_fn)(void* ctx, const double* q, double* r);
    static int host_staged(size_t count, const double* host_prims, double* host_rhs, void* stream, staged_fn fn,
                           void* ctx)
    {
        using namespace gbns;
        if (!host_prims || !host_rhs) return set_error(GBNS_ERR_INVALID, "prims/rhs pointer is NULL");
        if (host_prims == host_rhs) return set_error(GBNS_ERR_INVALID, "prims and rhs must not alias");
        int dev = 0;
        int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
        if (rc) return rc;
        struct Staging { double* q = nullptr; double* r = nullptr; size_t count = 0; };
        static std::mutex mu;
        static Staging staging[64];
        if (dev < 0 || dev >= 64) return set_error(GBNS_ERR_UNSUPPORTED, "device index above 63");
        std::lock_guard<std::mutex> lk(mu);
        Staging& sg = staging[dev];
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        if (sg.count < count)
        {
            rc = check_cuda(cudaStreamSynchronize(st), "host-path sync");
            if (rc) return rc;
            if (sg.q) cudaFree(sg.q);
            if (sg.r) cudaFree(sg.r);
            sg.q = sg.r = nullptr;
            sg.count = 0;
            rc = check_cuda(cudaMalloc(&sg.q, count*sizeof(double)), "host-path staging (prims)");
            if (!rc) rc = check_cuda(cudaMalloc(&sg.r, count*sizeof(double)), "host-path staging (rhs)");
            if (rc)
            {
                // never keep half a staging pair
                if (sg.q) cudaFree(sg.q);
                if (sg.r) cudaFree(sg.r);
                sg.q = sg.r = nullptr;
                return rc;
            }
            sg.count = count;
        }
        const size_t bytes = count*sizeof(double);
        rc = check_cuda(cudaMemcpyAsync(sg.q, host_prims, bytes, cudaMemcpyHostToDevice, st), "prims to device");
        // rhs goes down in both modes: overwrite leaves its ghost layers as they were
        if (!rc) rc = check_cuda(cudaMemcpyAsync(sg.r, host_rhs, bytes, cudaMemcpyHostToDevice, st), "rhs to device");
        if (!rc) rc = fn(ctx, sg.q, sg.r);
        if (!rc) rc = check_cuda(cudaMemcpyAsync(host_rhs, sg.r, bytes, cudaMemcpyDeviceToHost, st), "rhs to host");
        if (!rc) rc = check_cuda(cudaStreamSynchronize(st), "host-path sync");
        return rc;
    }

    int gbns_flux_div_host(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                           const double* host_prims, double* host_rhs, int increment, void* stream)
    {
        size_t count = 0;
        const int rc = gbns_array_size(grid, &count);
        if (rc) return rc;
        struct Ctx { const gbns_grid_desc* g; const gbns_scheme_desc* s; int incr; void* st; } c{grid, scheme, increment, stream};
        return host_staged(count, host_prims, host_rhs, stream, [](void* p, const double* q, double* r) -> int
        {
            const Ctx& c = *static_cast<const Ctx*>(p);
            return gbns_flux_div(c.g, c.s, q, r, c.incr, c.st);
        }, &c);
    }

    int gbns_flux_div_blocks_host(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                                  const double* block_bounds, const double* host_prims, double* host_rhs,
                                  int increment, void* stream)
    {
        using namespace gbns;
        if (!grid) return set_error(GBNS_ERR_INVALID, "grid descriptor is NULL");
        const int nblk = grid->nblk[0];
        if (nblk < 1 || nblk > 65535 || grid->nblk[1] != 1 || grid->nblk[2] != 1)
            return set_error(GBNS_ERR_INVALID, "a refined layout's blocks are given as nblk = (1..65535, 1, 1)");
        gbns_grid_desc one = *grid;
        one.nblk[0] = 1;
        size_t per_block = 0;
        const int rc = gbns_array_size(&one, &per_block);
        if (rc) return rc;
        struct Ctx { const gbns_grid_desc* g; const gbns_scheme_desc* s; const double* b; int incr; void* st; }
            c{grid, scheme, block_bounds, increment, stream};
        return host_staged(per_block*size_t(nblk), host_prims, host_rhs, stream,
                           [](void* p, const double* q, double* r) -> int
        {
            const Ctx& c = *static_cast<const Ctx*>(p);
            return gbns_flux_div_blocks(c.g, c.s, c.b, q, r, c.incr, c.st);
        }, &c);
    }

    int gbns_flux_div_variant(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                              const double* prims, double* rhs, int increment, int variant, void* stream)
    {
        GeomK G;
        SchemeK S;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        rc = make_scheme(scheme, S);
        if (rc) return rc;
        if (!prims || !rhs) return set_error(GBNS_ERR_INVALID, "prims/rhs pointer is NULL");
        if (scheme_halo(scheme) > G.ng) return set_error(GBNS_ERR_INVALID, "scheme stencil needs more ghost layers");
        YTabK* Y = nullptr;
        static thread_local YTabK ytab;
        if (grid->coords != GBNS_COORDS_IDENTITY)
        {
            rc = make_ytab(grid, G, ytab);
            if (rc) return rc;
            Y = &ytab;
        }
        return launch_flux_div(grid, G, Y, S, scheme, prims, rhs, increment, static_cast<cudaStream_t>(stream), variant);
    }

    int gbns_flux_variant_count(const gbns_scheme_desc* scheme)
    {
        return flux_variant_count(scheme);
    }

    int gbns_fill_ghosts(const gbns_grid_desc* grid, const gbns_bc_desc* bc, double* prims, void* stream)
    {
        GeomK G;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        rc = validate_bc(bc);
        if (rc) return rc;
        if (!prims) return set_error(GBNS_ERR_INVALID, "prims pointer is NULL");
        return launch_fill_ghosts(G, bc, prims, static_cast<cudaStream_t>(stream));
    }

    int gbns_rk_stage(const gbns_grid_desc* grid, const gbns_gas_desc* gas, double* prims,
                      const double* const* residuals, const double* coeffs, int nres, void* stream)
    {
        GeomK G;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        if (!gas || !(gas->gamma > 1.0) || !(gas->R > 0.0)) return set_error(GBNS_ERR_INVALID, "invalid gas");
        if (nres < 0 || nres > 4) return set_error(GBNS_ERR_INVALID, "nres must be in [0, 4]");
        if (!prims || (nres > 0 && (!residuals || !coeffs))) return set_error(GBNS_ERR_INVALID, "NULL pointer");
        for (int j = 0; j < nres; ++j) if (!residuals[j]) return set_error(GBNS_ERR_INVALID, "NULL residual pointer");
        return launch_rk_stage(G, gas->gamma, gas->R, prims, residuals, coeffs, nres, static_cast<cudaStream_t>(stream));
    }

    int gbns_flux_div_rk(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* prims,
                         double* rhs, int write_rhs, int nres, const double* const* earlier,
                         const double* coeffs, double* q_out, void* stream)
    {
        return gbns::flux_div_rk_range(grid, scheme, prims, rhs, write_rhs, nres, earlier, coeffs, q_out, stream, 0, -1);
    }
}

namespace gbns
{
    // gbns_flux_div_rk over the blocks blk0 .. blk1 - 1 (blk1 = -1: to the last)
    int flux_div_rk_range(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* prims,
                          double* rhs, int write_rhs, int nres, const double* const* earlier,
                          const double* coeffs, double* q_out, void* stream, int blk0, int blk1)
    {
        GeomK G;
        SchemeK S;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        rc = make_scheme(scheme, S);
        if (rc) return rc;
        if (nres < 1 || nres > 3) return set_error(GBNS_ERR_INVALID, "nres must be 1, 2 or 3");
        if (!prims || !q_out || !coeffs || (write_rhs && !rhs) || (nres > 1 && !earlier))
            return set_error(GBNS_ERR_INVALID, "NULL pointer");
        if (q_out == prims) return set_error(GBNS_ERR_INVALID, "q_out must not alias prims (other tiles still read it)");
        if (scheme_halo(scheme) > G.ng) return set_error(GBNS_ERR_INVALID, "scheme stencil needs more ghost layers");
        RkFuse f;
        std::memset(&f, 0, sizeof(f));
        f.nres = nres;
        f.write_rhs = write_rhs ? 1 : 0;
        for (int j = 0; j + 1 < nres; ++j)
        {
            if (!earlier[j]) return set_error(GBNS_ERR_INVALID, "NULL residual pointer");
            f.res[j] = earlier[j];
        }
        for (int j = 0; j < nres; ++j) f.coeff[j] = coeffs[j];
        f.q_out = q_out;
        YTabK* Y = nullptr;
        static thread_local YTabK ytab;
        if (grid->coords != GBNS_COORDS_IDENTITY)
        {
            rc = make_ytab(grid, G, ytab);
            if (rc) return rc;
            Y = &ytab;
        }
        return launch_flux_div(grid, G, Y, S, scheme, prims, write_rhs ? rhs : q_out, 0,
                               static_cast<cudaStream_t>(stream), scheme->tile_variant, &f, blk0, blk1);
    }

    namespace
    {
        // Non-blocking copy streams the library keeps, one per device and host thread.
        struct ThreadCopyStreams
        {
            std::vector<cudaStream_t> st;
            ~ThreadCopyStreams()
            {
                for (cudaStream_t s : st)
                    if (s) cudaStreamDestroy(s);
            }
        };
        thread_local ThreadCopyStreams t_copy_streams;

        int thread_copy_stream(cudaStream_t* out)
        {
            int dev = 0;
            int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
            if (rc) return rc;
            auto& v = t_copy_streams.st;
            if (v.size() <= size_t(dev)) v.resize(dev + 1, nullptr);
            if (!v[dev])
            {
                rc = check_cuda(cudaStreamCreateWithFlags(&v[dev], cudaStreamNonBlocking), "copy stream");
                if (rc) return rc;
            }
            *out = v[dev];
            return GBNS_OK;
        }

        // Events of one gbns_ssprk3_step_host call; destroyed when the call
        // returns (their resources go once the recorded work has finished).
        struct EventSet
        {
            std::vector<cudaEvent_t> ev;
            ~EventSet()
            {
                for (cudaEvent_t e : ev)
                    if (e) cudaEventDestroy(e);
            }
            int make(int n)
            {
                ev.assign(n, nullptr);
                for (int i = 0; i < n; ++i)
                {
                    int rc = check_cuda(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming), "copy event");
                    if (rc) return rc;
                }
                return GBNS_OK;
            }
        };

        // The last group (in issue order 0, 1, ...) holding a ghost donor of a
        // block of group g: the block itself and its 26 neighbours, wrapped
        // across periodic faces and dropped across the others (the donors
        // fill_one_ghost_from can read).
        int last_donor_group(const GeomK& G, const gbns_bc_desc* bc, const std::vector<int>& start, int g)
        {
            const int ngroup = int(start.size()) - 1;
            int last = g;
            for (int lb = start[g]; lb < start[g + 1]; ++lb)
            {
                const int b[3] = {lb % G.nb[0], (lb / G.nb[0]) % G.nb[1], lb / (G.nb[0]*G.nb[1])};
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx)
                        {
                            const int d[3] = {dx, dy, dz};
                            int nb[3];
                            bool skip = false;
                            for (int a = 0; a < 3; ++a)
                            {
                                nb[a] = b[a] + d[a];
                                if (nb[a] < 0)
                                {
                                    if (bc->kind[2*a] != GBNS_BC_PERIODIC) skip = true;
                                    nb[a] += G.nb[a];
                                }
                                else if (nb[a] >= G.nb[a])
                                {
                                    if (bc->kind[2*a + 1] != GBNS_BC_PERIODIC) skip = true;
                                    nb[a] -= G.nb[a];
                                }
                            }
                            if (skip) continue;
                            const int lbs = nb[0] + G.nb[0]*(nb[1] + G.nb[1]*nb[2]);
                            int h = 0;
                            while (h + 1 < ngroup && start[h + 1] <= lbs) ++h;
                            if (h > last) last = h;
                        }
            }
            return last;
        }
    }
}

extern "C"
{

    int gbns_copy_fill_ghosts(const gbns_grid_desc* grid, const gbns_bc_desc* bc, double* dst,
                              const double* src, void* stream)
    {
        GeomK G;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        rc = validate_bc(bc);
        if (rc) return rc;
        if (!dst || !src || dst == src) return set_error(GBNS_ERR_INVALID, "dst/src must be distinct non-NULL arrays");
        return launch_copy_fill(G, bc, dst, src, static_cast<cudaStream_t>(stream));
    }

    int gbns_ssprk3_step(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                         const gbns_bc_desc* bc, double* prims, double* work, double dt, void* stream)
    {
        GeomK G;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        if (!work) return set_error(GBNS_ERR_INVALID, "work pointer is NULL");
        rc = validate_bc(bc);
        if (rc) return rc;
        const size_t n = size_t(G.bstride)*G.nblk;
        double* R0 = work;
        double* R1 = work + n;
        double* B = work + 2*n;      // the state between stages
        // ratio_diff_t of consecutive ssprk3_t rows (explicit.h:80-88, advance.h:80-95)
        const double c1[1] = {(1.0/1.0)*dt};
        const double c2[2] = {(-3.0/4.0)*dt, (1.0/4.0)*dt};
        const double c3[3] = {(-1.0/12.0)*dt, (-1.0/12.0)*dt, (2.0/3.0)*dt};
        const double* e1[2] = {R0, nullptr};
        const double* e2[2] = {R0, R1};
        // each stage: residual and stage update in one launch, then the ghost fill
        if ((rc = gbns_flux_div_rk(grid, scheme, prims, R0, 1, 1, e1, c1, B, stream))) return rc;
        if ((rc = gbns_fill_ghosts(grid, bc, B, stream))) return rc;
        if ((rc = gbns_flux_div_rk(grid, scheme, B, R1, 1, 2, e1, c2, prims, stream))) return rc;
        if ((rc = gbns_fill_ghosts(grid, bc, prims, stream))) return rc;
        if ((rc = gbns_flux_div_rk(grid, scheme, prims, nullptr, 0, 3, e2, c3, B, stream))) return rc;
        return gbns_copy_fill_ghosts(grid, bc, prims, B, stream);
    }

    int gbns_ssprk3_step_host(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                              const gbns_bc_desc* bc, double* host_prims, double* prims, double* work,
                              double dt, int ngroups, void* stream, void* copy_stream)
    {
        using namespace gbns;
        GeomK G;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        if (!scheme) return set_error(GBNS_ERR_INVALID, "scheme descriptor is NULL");
        if (!work || !prims || !host_prims) return set_error(GBNS_ERR_INVALID, "NULL pointer");
        if (host_prims == prims) return set_error(GBNS_ERR_INVALID, "host_prims and prims must be distinct arrays");
        rc = validate_bc(bc);
        if (rc) return rc;
        if (ngroups < 0) return set_error(GBNS_ERR_INVALID, "ngroups must be >= 0");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        cudaStream_t cs = static_cast<cudaStream_t>(copy_stream);
        if (!cs && (rc = thread_copy_stream(&cs))) return rc;
        if (cs == st) return set_error(GBNS_ERR_INVALID, "copy_stream must differ from stream");
        const int ng = ngroups == 0 ? (G.nblk < 8 ? G.nblk : 8) : (ngroups < G.nblk ? ngroups : G.nblk);
        std::vector<int> start(ng + 1);
        for (int g = 0; g <= ng; ++g) start[g] = int((long long)g*G.nblk/ng);
        const size_t bstride = size_t(G.bstride);
        const size_t n = bstride*G.nblk;
        double* R0 = work;
        double* R1 = work + n;
        double* B = work + 2*n;
        const double c1[1] = {(1.0/1.0)*dt};
        const double c2[2] = {(-3.0/4.0)*dt, (1.0/4.0)*dt};
        const double c3[3] = {(-1.0/12.0)*dt, (-1.0/12.0)*dt, (2.0/3.0)*dt};
        const double* e1[2] = {R0, nullptr};
        const double* e2[2] = {R0, R1};
        // events: 0 = work issued on `stream` before the call, 1..ng = group
        // copied in, ng+1..2ng = group final, 2ng+1 = every copy out issued
        EventSet E;
        if ((rc = E.make(2*ng + 2))) return rc;
        cudaEvent_t* ev = E.ev.data();
        if ((rc = check_cuda(cudaEventRecord(ev[0], st), "event record"))) return rc;
        if ((rc = check_cuda(cudaStreamWaitEvent(cs, ev[0], 0), "stream wait"))) return rc;
        for (int g = 0; g < ng; ++g)
        {
            const size_t off = bstride*start[g], cnt = bstride*(start[g + 1] - start[g]);
            if ((rc = check_cuda(cudaMemcpyAsync(prims + off, host_prims + off, cnt*sizeof(double),
                                                 cudaMemcpyHostToDevice, cs), "state copy to the device")))
                return rc;
            if ((rc = check_cuda(cudaEventRecord(ev[1 + g], cs), "event record"))) return rc;
        }
        // stage 1 group by group as the groups arrive (a block's stencil reads
        // only its own padded array, whose ghosts are valid on entry)
        for (int g = 0; g < ng; ++g)
        {
            if ((rc = check_cuda(cudaStreamWaitEvent(st, ev[1 + g], 0), "stream wait"))) return rc;
            if ((rc = flux_div_rk_range(grid, scheme, prims, R0, 1, 1, e1, c1, B, stream, start[g], start[g + 1])))
                return rc;
        }
        if ((rc = gbns_fill_ghosts(grid, bc, B, stream))) return rc;
        if ((rc = gbns_flux_div_rk(grid, scheme, B, R1, 1, 2, e1, c2, prims, stream))) return rc;
        if ((rc = gbns_fill_ghosts(grid, bc, prims, stream))) return rc;
        // stage 3 group by group; a group's ghost fill and copy out follow the
        // stage-3 launch of the last group holding one of its ghost donors
        std::vector<int> ready(ng);
        for (int g = 0; g < ng; ++g) ready[g] = last_donor_group(G, bc, start, g);
        for (int h = 0; h < ng; ++h)
        {
            if ((rc = flux_div_rk_range(grid, scheme, prims, nullptr, 0, 3, e2, c3, B, stream, start[h], start[h + 1])))
                return rc;
            for (int g = 0; g < ng; ++g)
            {
                if (ready[g] != h) continue;
                if ((rc = launch_copy_fill(G, bc, prims, B, st, start[g], start[g + 1]))) return rc;
                if ((rc = check_cuda(cudaEventRecord(ev[1 + ng + g], st), "event record"))) return rc;
                if ((rc = check_cuda(cudaStreamWaitEvent(cs, ev[1 + ng + g], 0), "stream wait"))) return rc;
                const size_t off = bstride*start[g], cnt = bstride*(start[g + 1] - start[g]);
                if ((rc = check_cuda(cudaMemcpyAsync(host_prims + off, prims + off, cnt*sizeof(double),
                                                     cudaMemcpyDeviceToHost, cs), "state copy to the host")))
                    return rc;
            }
        }
        if ((rc = check_cuda(cudaEventRecord(ev[2*ng + 1], cs), "event record"))) return rc;
        return check_cuda(cudaStreamWaitEvent(st, ev[2*ng + 1], 0), "stream wait");
    }

    int gbns_boundary_flux(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* prims,
                           double* rhs, const int* apply, void* stream)
    {
        using namespace gbns;
        GeomK G;
        SchemeK S;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        rc = make_scheme(scheme, S);
        if (rc) return rc;
        if (!prims || !rhs || !apply) return set_error(GBNS_ERR_INVALID, "NULL argument");
        if (prims == rhs) return set_error(GBNS_ERR_INVALID, "prims and rhs must not alias");
        if (grid->coords != GBNS_COORDS_IDENTITY)
            return set_error(GBNS_ERR_UNSUPPORTED, "boundary_flux supports identity coordinates (the reference "
                                                   "evaluates the Jacobian at ghost cells)");
        // faces in the transverse ghost row take face gradients one layer further out
        int halo = scheme_halo(scheme);
        const bool grad = scheme->viscous || (scheme->dissipation && scheme->sensor == GBNS_SENSOR_DUCROS) ||
                          (scheme->convective == GBNS_CONV_HYBRID && scheme->hybrid_sensor == GBNS_SENSOR_DUCROS);
        if (grad && halo < 2) halo = 2;
        if (halo > G.ng)
            return set_error(GBNS_ERR_INVALID, "boundary_flux needs " + std::to_string(halo) + " ghost layers, grid has " +
                             std::to_string(G.ng));
        const cudaStream_t st = static_cast<cudaStream_t>(stream);
        // boundaries in the reference's order: dir = 2*direction + side
        for (int dir = 0; dir < 6; ++dir)
        {
            if (!apply[dir]) continue;
            const int D = dir/2;
            const int ta = D == 0 ? 1 : 0, tb = D == 2 ? 1 : 2;
            BndArgs A;
            std::memset(&A, 0, sizeof(A));
            A.prims = prims;
            A.rhs = rhs;
            A.side = dir % 2;
            A.ntile1 = (G.n[ta] + 1 + 7)/8;
            A.ntile2 = (G.n[tb] + 1 + 7)/8;
            for (int b = 0; b < G.nb[D]; ++b)
            {
                double mn = 0.0;
                block_dx(grid, D, b, &mn, &A.dx[b]);
            }
            if (D == 0) rc = boundary_flux_launch_d0(G, S, A, scheme->convective, scheme->order, st);
            else if (D == 1) rc = boundary_flux_launch_d1(G, S, A, scheme->convective, scheme->order, st);
            else rc = boundary_flux_launch_d2(G, S, A, scheme->convective, scheme->order, st);
            if (rc) return rc;
        }
        return GBNS_OK;
    }

    int gbns_ssprk3_run(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const gbns_bc_desc* bc,
                        double* prims, double* work, double dt, int nsteps, void* stream)
    {
        using namespace gbns;
        if (nsteps < 0) return set_error(GBNS_ERR_INVALID, "nsteps must be >= 0");
        if (!grid || !scheme || !bc || !prims || !work) return set_error(GBNS_ERR_INVALID, "NULL argument");
        if (nsteps == 0) return GBNS_OK;
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        // the graph of one step is keyed on everything it bakes in
        StepKey key;
        std::memset(&key, 0, sizeof(key));
        std::memcpy(&key.grid, grid, sizeof(*grid));
        std::memcpy(&key.scheme, scheme, sizeof(*scheme));
        std::memcpy(&key.bc, bc, sizeof(*bc));
        key.prims = prims; key.work = work; key.dt = dt;
        int rc = check_cuda(cudaGetDevice(&key.device), "cudaGetDevice");
        if (rc) return rc;
        // launches the cached graph of `key` nsteps times; false if none is cached.
        // Runs under the cache lock, so no other thread can evict the graph
        // between lookup and launch.
        auto replay = [&](int& out) -> bool
        {
            std::lock_guard<std::mutex> lk(step_graphs_mu());
            for (auto& e : step_graphs())
                if (std::memcmp(&e.key, &key, sizeof(key)) == 0)
                {
                    out = GBNS_OK;
                    for (int i = 0; i < nsteps && out == GBNS_OK; ++i)
                        out = check_cuda(cudaGraphLaunch(e.exec, st), "graph launch");
                    return true;
                }
            return false;
        };
        if (replay(rc)) return rc;
        cudaGraphExec_t exec = nullptr;
        {
            // capture one step on a private stream that waits for the caller's
            // work, so the captured launches see the caller's ordering
            cudaStream_t cs = nullptr;
            cudaEvent_t ev = nullptr;
            rc = check_cuda(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "capture stream");
            if (!rc) rc = check_cuda(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "capture event");
            if (!rc) rc = check_cuda(cudaEventRecord(ev, st), "capture event record");
            if (!rc) rc = check_cuda(cudaStreamWaitEvent(cs, ev, 0), "capture stream wait");
            cudaGraph_t graph = nullptr;
            if (!rc) rc = check_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture");
            if (!rc)
            {
                const int lrc = gbns_ssprk3_step(grid, scheme, bc, prims, work, dt, cs);
                const int erc = check_cuda(cudaStreamEndCapture(cs, &graph), "end capture");
                rc = lrc ? lrc : erc;
            }
            if (!rc) rc = check_cuda(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate");
            if (graph) cudaGraphDestroy(graph);
            if (ev) cudaEventDestroy(ev);
            if (cs) cudaStreamDestroy(cs);
            if (rc) return rc;
            std::lock_guard<std::mutex> lk(step_graphs_mu());
            auto& cache = step_graphs();
            if (cache.size() >= 8)
            {
                // an evicted graph still in flight is freed by the driver when
                // it completes (cuGraphExecDestroy semantics)
                cudaGraphExecDestroy(cache.front().exec);
                cache.erase(cache.begin());
            }
            cache.push_back(StepGraph{key, exec});
            for (int i = 0; i < nsteps && rc == GBNS_OK; ++i)
                rc = check_cuda(cudaGraphLaunch(exec, st), "graph launch");
        }
        return rc;
    }

    int gbns_device_status(int* status, int reset, void* stream)
    {
        if (!status) return set_error(GBNS_ERR_INVALID, "status is NULL");
        return read_device_status(status, reset, static_cast<cudaStream_t>(stream));
    }
}
