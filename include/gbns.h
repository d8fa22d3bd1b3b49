/*
 * gbns.h — C ABI of libgbns.so, the GB300-native (sm_103a) explicit
 * right-hand side of SPADE's compressible Navier–Stokes solver.
 *
 * Every entry point takes plain pointers and sizes.  Array pointers are
 * DEVICE pointers owned by the caller, laid out exactly like SPADE's
 * grid_array with the default linear memory map (core/mem_map.h:465-497,
 * 654-676): for local block lb and cell (i,j,k) with ng ghost layers,
 *
 *     offset = v + 5*((i+ng) + ni*((j+ng) + nj*((k+ng) + nk*lb)))
 *     ni = nx+2ng, nj = ny+2ng, nk = nz+2ng,
 *
 * variables fastest ("AoS5").  Primitive arrays hold (p, T, u, v, w)
 * (navier-stokes/fluid_state.h:60-82); residual arrays hold flux_t order
 * (continuity, energy, x-, y-, z-momentum) (fluid_state.h:106-126).
 *
 * Return codes: 0 = success, negative = error; the message of the last
 * error on the calling thread is available from gbns_last_error().
 * Calls are stream-ordered on the given stream (NULL = legacy default
 * stream) and do not synchronise unless stated.  The library allocates no
 * device memory on the flux_div / ghost-fill / RK-stage paths; the batched
 * and serving entry points own their work-lists.
 */
#ifndef GBNS_H
#define GBNS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBNS_ABI_VERSION 1

/* ---- error codes ---------------------------------------------------- */
#define GBNS_OK               0
#define GBNS_ERR_INVALID    (-1)   /* bad descriptor or argument */
#define GBNS_ERR_UNSUPPORTED (-2)  /* scheme/combination not built */
#define GBNS_ERR_CUDA       (-3)   /* CUDA runtime error */
#define GBNS_ERR_NONFINITE  (-4)   /* state check found NaN/Inf or p,T <= 0 */
#define GBNS_ERR_CAPACITY   (-5)   /* batch/serving capacity or budget exceeded */
#define GBNS_ERR_TIMEOUT    (-6)   /* a bounded device wait ran out */

/* ---- grid ------------------------------------------------------------
 * Replaces the geometry the reference kernels read from
 * grid::cartesian_grid_t / grid_geometry_t (grid/cartesian_grid.h:48-384,
 * grid/grid_geometry.h:16-100) and cartesian_blocks_t
 * (grid/cartesian_blocks.h:23-117).  Blocks are numbered with x fastest:
 * lb = bx + nbx*(by + nby*bz) (cartesian_blocks.h:54-105 with
 * ctrs::collapse_index, core/ctrs.h:341-353).  Block boxes and spacings are
 * derived exactly as the reference does (block min = bounds.min +
 * b*bsize, max = min + bsize, dx = (max-min)/n, inv_dx = 1/dx).
 */
#define GBNS_COORDS_IDENTITY        0  /* coords::identity (core/coord_system.h:51-56) */
#define GBNS_COORDS_TANH_Y          1  /* y = tanh(beta*eta)/tanh(beta), eta in the y bounds; x,z identity */
#define GBNS_COORDS_INTEGRATED_TANH_Y 2 /* coords::integrated_tanh_1D in y (coord_system.h:103-140); x,z identity */

typedef struct gbns_grid_desc
{
    int32_t nblk[3];       /* blocks per direction */
    int32_t ncell[3];      /* cells per block per direction (nx, ny, nz) */
    int32_t ng;            /* ghost layers (same in every direction) */
    int32_t coords;        /* GBNS_COORDS_* */
    double  bounds[6];     /* computational domain xmin,xmax,ymin,ymax,zmin,zmax */
    double  coord_param[4];/* TANH_Y: beta; INTEGRATED_TANH_Y: y0,y1,inflation,rate */
} gbns_grid_desc;

/* ---- gas ------------------------------------------------------------- */
typedef struct gbns_gas_desc
{
    double gamma;          /* fluid_state::ideal_gas_t::gamma (navier-stokes/gas.h:35-49) */
    double R;              /* fluid_state::ideal_gas_t::R */
} gbns_gas_desc;

/* ---- flux scheme ------------------------------------------------------
 * A lowered omni::compose(convective, dissipation, viscous) functor
 * (omni/compose.h:7-45): the face flux is conv + (diss + visc) with absent
 * terms dropped, summed in that nesting like composite_kernel_t.
 */
#define GBNS_CONV_NONE        0
#define GBNS_CONV_CENT_KEEP   1   /* convective::cent_keep_scheme_t<gas,order> (navier-stokes/convective.h:96-192) */
#define GBNS_CONV_TOTANI      2   /* convective::totani_lr (convective.h:54-94) */
#define GBNS_CONV_FWENO       3   /* convective::fweno_t (convective.h:335-497), 3rd order, 4-point */
#define GBNS_CONV_WENO5       4   /* 5th-order WENO-JS on fweno_t's Rusanov split (no reference counterpart) */
#define GBNS_CONV_HYBRID      5   /* convective::hybrid_scheme_t<cent_keep_scheme_t<gas,order>, fweno_t<gas,smooth>,
                                     sensor, tag> (navier-stokes/hybrid_scheme.h:14-47): the centred flux blended
                                     with fweno_t by a face sensor (hybrid_sensor, hybrid_param); order 2 or 4 */

#define GBNS_HYBRID_FULL_FLUX 0   /* convective::full_flux: (1 - s) F_centred + s F_fweno */
#define GBNS_HYBRID_DISS_FLUX 1   /* convective::diss_flux: F_centred + s F_fweno */

#define GBNS_DISS_NONE        0
#define GBNS_DISS_PRESSURE    1   /* convective::pressure_diss_lr (convective.h:194-246) */

#define GBNS_SENSOR_CONST     0   /* state_sensor::const_sensor_t (navier-stokes/state_sensor.h:46-60) */
#define GBNS_SENSOR_DUCROS    1   /* state_sensor::ducros_t on the face gradient (state_sensor.h:21-43) */

#define GBNS_VISC_NONE        0
#define GBNS_VISC_LR          1   /* viscous::visc_lr (navier-stokes/viscous.h:13-113) */

#define GBNS_LAW_CONSTANT     0   /* viscous_laws::constant_viscosity_t (viscous_laws.h:62-100) */
#define GBNS_LAW_POWER        1   /* viscous_laws::power_law_t (viscous_laws.h:102-135) */
#define GBNS_LAW_SUTHERLAND   2   /* Sutherland's law (no reference counterpart) */

#define GBNS_PREC_FP64        0   /* FP64, every operation rounded as the reference's CPU code rounds it (no FMA contraction) */
#define GBNS_PREC_FP32_FLUX   1   /* face reconstruction + flux in FP32; divergence accumulation FP64 */
#define GBNS_PREC_FP64_FMA    2   /* FP64 with fused multiply-adds (faster; differs from the reference in the last bits) */

typedef struct gbns_scheme_desc
{
    int32_t convective;    /* GBNS_CONV_* */
    int32_t order;         /* cent_keep nominal order: 2, 4, 6, 8 */
    int32_t weno_smooth;   /* fweno_t/weno5: 1 = smoothness weights, 0 = linear weights */
    int32_t dissipation;   /* GBNS_DISS_* */
    int32_t sensor;        /* GBNS_SENSOR_* */
    int32_t viscous;       /* GBNS_VISC_* */
    int32_t visc_law;      /* GBNS_LAW_* */
    int32_t precision;     /* GBNS_PREC_* */
    int32_t tile_variant;  /* flux_div tile shape, 0 .. gbns_flux_variant_count-1 (0 = default);
                              every variant gives bit-identical results */
    int32_t hybrid_flux;   /* GBNS_CONV_HYBRID: GBNS_HYBRID_FULL_FLUX or GBNS_HYBRID_DISS_FLUX */
    double  eps_p, eps_T;  /* pressure_diss_lr coefficients */
    double  sensor_alpha;  /* const_sensor_t::alpha, or ducros_t::epsilon */
    double  mu;            /* constant: mu; power/sutherland: mu_ref */
    double  prandtl;
    double  T_ref;         /* power/sutherland reference temperature */
    double  power;         /* power-law exponent */
    double  S;             /* Sutherland constant */
    double  prandtl_inv;   /* 1/Pr as the caller's law stores it; 0 = use 1.0/prandtl
                              (constant_viscosity_t keeps only 1/Pr, viscous_laws.h:190-192) */
    gbns_gas_desc gas;
    int32_t hybrid_sensor; /* GBNS_CONV_HYBRID blender: GBNS_SENSOR_* */
    int32_t reserved;      /* must be 0 */
    double  hybrid_param;  /* blender const_sensor_t::alpha, or ducros_t::epsilon */
} gbns_scheme_desc;

/* ---- boundary conditions -------------------------------------------- */
#define GBNS_BC_PERIODIC           0  /* block exchange wraps (grid/exchange_config.h:321-350) */
#define GBNS_BC_NONE               1  /* ghosts left untouched */
#define GBNS_BC_ISOTHERMAL_NOSLIP  2  /* mirror fill: p_g=p, T_g=2Tw-T, u_g=-u (grid/boundary_fill.h:106-129) */
#define GBNS_BC_SLIP_ADIABATIC     3  /* mirror fill: p_g=p, T_g=T, u_n reflected */

typedef struct gbns_bc_desc
{
    int32_t kind[6];       /* GBNS_BC_* per face xmin,xmax,ymin,ymax,zmin,zmax; periodic must pair */
    double  t_wall[6];     /* wall temperature for isothermal faces */
} gbns_bc_desc;

/* ---- reductions ----------------------------------------------------- */
#define GBNS_RED_MAX_WAVESPEED 0  /* max over interior of sqrt(gamma R T) + |u| (CFL; development/cuda-tgv/main.cc:152-172) */
#define GBNS_RED_KINETIC       1  /* volume average of 0.5 rho |u|^2 (Jacobian-weighted) */
#define GBNS_RED_CONSERVED     2  /* 5 Jacobian-weighted sums of (rho, rhoE, rhou, rhov, rhow) */
#define GBNS_RED_HEALTH        3  /* count of interior cells with NaN/Inf or p<=0 or T<=0 */

/* ---- entry points ---------------------------------------------------- */

/* Library / ABI version; no CUDA call. */
int gbns_version(void);

/* Copies the last error message of this thread into buf (NUL-terminated). */
int gbns_last_error(char* buf, size_t len);

/* Validates a grid descriptor and returns the number of doubles in one AoS5
 * array (ghosts included) in *count.  No CUDA call.  Replaces the size the
 * reference computes in grid_array's constructor (grid/grid_array.h:244-260). */
int gbns_array_size(const gbns_grid_desc* grid, size_t* count);

/* rhs (+)= flux divergence of prims.
 * Replaces spade::pde_algs::flux_div(prims, rhs, flux_func[, traits])
 * (pde-algs/flux-div/flux_div.h:16-56) with the basic algorithm
 * (flux_div_basic.h:17-76): for every interior cell,
 *   rhs += sum_d jac*[F(i-1/2) - F(i+1/2)]*inv_dx[d].
 * increment = 1 is the reference default (pde_algs::increment,
 * pde_traits.h:13-20); increment = 0 is pde_algs::overwrite (interior of rhs
 * overwritten; its ghost layers are not touched).  prims must have valid
 * ghost layers.  Asynchronous on `stream`. */
int gbns_flux_div(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                  const double* prims, double* rhs, int increment, void* stream);

/* gbns_flux_div on a refined (AMR) block layout: grid->nblk = (blocks, 1, 1)
 * (1..65535 blocks, each of grid->ncell cells and grid->ng ghost layers, in
 * the caller's global block order), identity coordinates (grid->bounds is
 * not used), and block_bounds (host memory, 6 doubles per block: min and max
 * along x, y, z) each block's bounding box.  Every block takes
 * inv_dx[d] = 1.0/((max_d - min_d)/ncell[d]), as the reference's flux_div
 * does from its own box (flux_div_basic.h:55, grid/grid_geometry.h:85-89) on
 * grids refined with cartesian_grid_t::refine_blocks
 * (grid/cartesian_grid.h:331-367).  prims carries the ghost values the
 * coarse/fine exchange wrote (gbns_exchange_plan).  The per-block table is
 * copied to stream-ordered device memory of the library's pool on `stream`
 * (from pageable memory: not for stream capture).  Asynchronous on
 * `stream`.  Stretched coordinates: GBNS_ERR_UNSUPPORTED. */
int gbns_flux_div_blocks(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* block_bounds,
                         const double* prims, double* rhs, int increment, void* stream);
/* gbns_flux_div_blocks for prims and rhs in host memory, staged through the
 * device buffers of gbns_flux_div_host (synchronises `stream`). */
int gbns_flux_div_blocks_host(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* block_bounds,
                              const double* host_prims, double* host_rhs, int increment, void* stream);

/* gbns_flux_div for prims and rhs in host memory (a grid_array on
 * device::cpu): both arrays are staged through device buffers the library
 * keeps per device and reuses across calls, the flux divergence runs on the
 * GPU (the same kernels and bits as gbns_flux_div) and rhs, ghost layers
 * included, is copied back.  Returns when rhs holds the result (synchronises
 * `stream`); calls on the host path are serialised.  Pinned host memory
 * copies at the full host link speed.  No reference counterpart (the
 * reference runs device::cpu arrays on the CPU). */
int gbns_flux_div_host(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                       const double* host_prims, double* host_rhs, int increment, void* stream);

/* Ghost fill: periodic / inter-block exchange of interior donor cells into
 * ghost layers, then wall mirror fill on non-periodic faces.
 * Replaces arr_exchange_t::exchange (grid/make_exchange.h:111-410, single
 * level injection) followed by algs::boundary_fill (grid/boundary_fill.h:31-133).
 * Asynchronous on `stream`. */
int gbns_fill_ghosts(const gbns_grid_desc* grid, const gbns_bc_desc* bc,
                     double* prims, void* stream);

/* One fused explicit-RK stage update on the primitive state, in place:
 * per interior cell  cons = prim2cons(q);  cons += coeff[j]*R_j (j < nres);
 * q = cons2prim(cons).  coeff[j] already includes dt.
 * Replaces time_integration::detail::transform_advance_to
 * (time-integration/advance.h:56-102) with fluid_state::convert_state
 * (navier-stokes/fluid_state.h:102-135).  nres <= 4.  Asynchronous. */
int gbns_rk_stage(const gbns_grid_desc* grid, const gbns_gas_desc* gas,
                  double* prims, const double* const* residuals,
                  const double* coeffs, int nres, void* stream);

/* Reduction over interior cells (GBNS_RED_*); writes 1 double (5 for
 * GBNS_RED_CONSERVED) to the HOST buffer `out` and synchronises the stream.
 * Replaces algs::transform_reduce (algs/transform_reduce.h:53-191) for the
 * reductions the reference drivers use. */
int gbns_reduce(const gbns_grid_desc* grid, const gbns_gas_desc* gas,
                const double* prims, int kind, double* out, void* stream);

/* flux_div with an explicit tile-shape variant (0 .. gbns_flux_variant_count-1);
 * every variant computes bit-identical results.  The autotuner's search
 * space; replaces the reference's choice among flux_div_{basic,bfoct,fldbc,
 * ldbal,shfus,longf} by trait (flux_div.h:30-40). */
int gbns_flux_div_variant(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                          const double* prims, double* rhs, int increment, int variant, void* stream);

/* Number of tile variants built for a scheme (>= 1); no CUDA call. */
int gbns_flux_variant_count(const gbns_scheme_desc* scheme);

/* Scratch size (doubles) and result offset for gbns_reduce_async; no CUDA call. */
int gbns_reduce_scratch_size(const gbns_grid_desc* grid, size_t* ndouble, size_t* result_offset);

/* gbns_reduce with caller-owned device scratch; the result stays in device
 * memory at scratch + result_offset.  Asynchronous.  Replaces
 * algs::transform_reduce (algs/transform_reduce.h:53-191). */
int gbns_reduce_async(const gbns_grid_desc* grid, const gbns_gas_desc* gas, const double* prims,
                      int kind, double* scratch, size_t scratch_len, void* stream);

/* Device-side status: nonzero after a kernel gave up on a bounded wait
 * (GBNS_DEV_*).  reset != 0 clears it.  Synchronises `stream`.  Replaces the
 * reference's post-launch error check (dispatch/execute.h:86-96). */
#define GBNS_DEV_OK           0
#define GBNS_DEV_TMA_TIMEOUT  1   /* a tile's TMA halo copy did not complete within the poll limit */
int gbns_device_status(int* status, int reset, void* stream);

/* pde_algs::boundary_flux (pde-algs/boundary_flux.h:16-105): for every
 * selected domain boundary (apply[2*d + side], side 0 = min, 1 = max, applied
 * in that order) of every block on it, the flux F of each face of the boundary
 * plane (transverse cell indices -1 .. n-1, as the reference's loop) is added
 * to the two cells the face separates: rhs(il) -= F/dx, rhs(ir) += F/dx (the
 * interior cell and the ghost cell beyond it), F the face flux of
 * gbns_flux_div for `scheme`, computed in FP64 without FMA contraction for
 * every precision.  Identity coordinates only; needs the scheme's halo in
 * ghost layers (at least 2 with face gradients). */
int gbns_boundary_flux(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* prims,
                       double* rhs, const int* apply, void* stream);

/* Measured FMA throughput of this GPU (FLOP/s) with dependent FMA chains:
 * fp64 != 0 -> double, else float.  Benchmark aid (no reference counterpart). */
int gbns_measure_fma_rate(int fp64, double* flops_per_s, void* stream);

/* Exercises the bounded-wait failure path of the flux kernel without a
 * fault: a one-CTA kernel arms an mbarrier for TMA bytes that never arrive,
 * gives up after a bounded poll and sets the device status word, which this
 * call reads into *status (GBNS_DEV_TMA_TIMEOUT expected) and clears.  The
 * context stays usable.  No counterpart in the reference. */
int gbns_selftest_wait_timeout(int* status, void* stream);

/* Checks the integer-pipe FP64 multiply, power-of-two scalings (x/2, x/4),
 * division and square root the flux kernels use against the hardware
 * operations on `npairs` generated operand
 * pairs (all bit patterns, range edges, exact products and ties, zeros,
 * subnormals, infinities, NaNs); *mismatches = pairs whose bits differ (NaN
 * results compare equal).  Synchronises `stream`.  No reference counterpart. */
int gbns_selftest_dmul_int(uint64_t npairs, uint64_t seed, uint64_t* mismatches, void* stream);

/* Reduction that allocates nothing.  For callers that cannot let the
 * library call cudaMalloc: applications that hand all device memory to their
 * own pool allocator at start-up, and solver loops that must not stall on an
 * allocation (cudaMalloc can synchronise the device and can fail late in a
 * run when memory is nearly full).  Same reductions and bit-identical results
 * as gbns_reduce; the result (1 double, 5 for GBNS_RED_CONSERVED) goes to the
 * caller's DEVICE buffer out_dev, asynchronously on `stream`.  Its partial
 * sums live in a fixed file-scope device array of 6,152 doubles (about 48 KB,
 * held by every GPU that loads the library until exit).  That is the most
 * scratch any grid's reduction uses (at most 1024 partial records); a need
 * beyond it is rejected with GBNS_ERR_CAPACITY.  The first call on a device
 * looks up the array's device address with that device current: make that
 * first call before any stream capture.  All calls share the one array and
 * leave their partial sums in it: calls that overlap on the GPU (several
 * streams, or several host threads on one device) race and must be
 * serialised by the caller.  No counterpart in the reference. */
int gbns_reduce_noalloc(const gbns_grid_desc* grid, const gbns_gas_desc* gas,
                        const double* prims, int kind, double* out_dev, void* stream);

/* flux_div (overwrite mode) fused with the RK stage update that consumes
 * it: the launch computes R = L(prims) for each tile and, for the same
 * cells, q_out = prim(cons(prims) + sum_j coeffs[j] R_j) with
 * R_0..R_{nres-2} = earlier[] and R_{nres-1} = R (transform_advance_to,
 * time-integration/advance.h:75-101, fused with flux_div_basic.h:17-76).
 * R is stored to rhs only if write_rhs.  q_out must not alias prims (other
 * tiles still read their halo from prims); its ghosts are not touched.
 * Arithmetic identical to gbns_flux_div followed by gbns_rk_stage.
 * Asynchronous. */
int gbns_flux_div_rk(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* prims,
                     double* rhs, int write_rhs, int nres, const double* const* earlier,
                     const double* coeffs, double* q_out, void* stream);

/* ---- exchange plans (AMR coarse/fine ghost fill) -------------------------
 * The ghost fill of a block layout with refinement levels, executed from the
 * plan the reference's make_exchange builds (grid/make_exchange.h:98-421,
 * grid/get_transaction.h:10-263): one record per transaction, either an
 * injection (same level: the destination box is a copy of an equally sized
 * donor box) or an interpolation (levels differ: every destination cell is
 * (1/8) x the sum of 8 donor cells, visited in the order
 * d = (0,0,0), (1,0,0), (0,1,0), (1,1,0), (0,0,1), ... with donor index
 * ((i << (i_coeff + 1)) >> 1) + d*i_incr per direction: i_coeff -1 takes the
 * coarse cell i/2 eight times, 1 averages the fine cells 2i and 2i+1).
 * Cell indices are block-local with the interior at [0, n); blocks are
 * numbered as the grid enumerates them (all of equal cell count). */
#define GBNS_PATCH_INJECT  0
#define GBNS_PATCH_INTERP  1
typedef struct gbns_patch
{
    int32_t kind;          /* GBNS_PATCH_INJECT or GBNS_PATCH_INTERP */
    int32_t src_block;     /* donor block */
    int32_t dst_block;     /* receiving block */
    int32_t src_lo[3];     /* donor box origin (i, j, k) */
    int32_t dst_lo[3];     /* receiving box [dst_lo, dst_hi) */
    int32_t dst_hi[3];
    int32_t i_coeff[3];    /* interpolation: -1, 0 or 1 per direction */
    int32_t i_incr[3];     /* interpolation: 0 or 1 per direction */
} gbns_patch;

typedef struct gbns_exchange_plan gbns_exchange_plan;

/* Validates a plan for blocks of nx*ny*nz cells with ng ghost layers and
 * nblocks blocks (every destination cell a ghost cell written once, every
 * donor inside its block's padded array), uploads it once and returns a
 * handle (the reference's exchange handle, make_exchange).  The result is
 * the reference's: its transactions executed one after the other in plan
 * order, injections before interpolations.  A donor that is a ghost cell
 * written by another transaction of the same kind therefore holds the new
 * value when its writer comes earlier in the plan and the old value when it
 * comes later; the plan is split into waves (one launch each) that keep this
 * order.  A transaction that reads a cell it writes itself is rejected
 * (GBNS_ERR_UNSUPPORTED).  Synchronises `stream`. */
int gbns_exchange_plan_create(gbns_exchange_plan** plan, int nx, int ny, int nz, int ng, int nblocks,
                              const gbns_patch* patches, int npatch, void* stream);
/* One exchange on the AoS5 array `prims` (arr_exchange_t::exchange,
 * grid/make_exchange.h:111-410): one launch per wave (one injection wave and
 * one interpolation wave when no donor is a ghost cell), asynchronous on
 * `stream`. */
int gbns_exchange_plan_run(gbns_exchange_plan* plan, double* prims, void* stream);
/* The wave of each transaction that gbns_exchange_plan_create would run it in
 * (injection waves, then interpolation waves, each wave one launch), after the
 * same validation; host only, no CUDA call.  waves: npatch ints. */
int gbns_exchange_plan_waves(int nx, int ny, int nz, int ng, int nblocks, const gbns_patch* patches, int npatch,
                             int* waves);
int gbns_exchange_plan_destroy(gbns_exchange_plan* plan);

/* One SSPRK3 step on a refined (AMR) layout: integrator_t::advance with
 * ssprk3_t and the conservative-variable state transform
 * (time-integration/advance.h:234-280), with the layout's exchange as the
 * boundary condition (then, with bc, the wall fill of gbns_wall_fill_blocks;
 * bc may be NULL), as the reference's drivers pair them.  grid and
 * block_bounds as for gbns_flux_div_blocks; plan the layout's exchange
 * (created for grid->ncell, grid->ng and grid->nblk[0] blocks).  Each stage
 * is one flux launch with the stage update fused (as gbns_ssprk3_step), then
 * the exchange, on a stage array that starts as a copy of the stage's input
 * (so the exchange sees the ghost values of the reference's in-place update:
 * ghost donors read before they are written, ghosts it never writes).
 * prims must hold exchanged ghosts on entry and does on exit.  work: 3 arrays
 * of prims' size.  Asynchronous on `stream` (the per-block table is copied
 * from pageable memory: not for stream capture). */
int gbns_ssprk3_step_blocks(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* block_bounds,
                            gbns_exchange_plan* plan, const gbns_bc_desc* bc, double* prims, double* work, double dt,
                            void* stream);
/* The wall faces of a refined layout: for every face whose bc kind is a wall
 * (GBNS_BC_ISOTHERMAL_NOSLIP, GBNS_BC_SLIP_ADIABATIC), in face order, the blocks
 * whose box touches that domain face (block_bounds against grid->bounds) get
 * their ghost slab (ng layers, the full padded extent across) mirrored from
 * their own cells with the wall kernel: the reference's algs::boundary_fill
 * (grid/boundary_fill.h:31-133) after its exchange.  Other faces are left
 * alone.  Asynchronous on `stream`. */
int gbns_wall_fill_blocks(const gbns_grid_desc* grid, const double* block_bounds, const gbns_bc_desc* bc,
                          double* prims, void* stream);

/* dst = src on interior cells, dst's ghost layers filled from src's interior
 * donors (gbns_fill_ghosts of src, written into dst).  Asynchronous. */
int gbns_copy_fill_ghosts(const gbns_grid_desc* grid, const gbns_bc_desc* bc, double* dst,
                          const double* src, void* stream);

/* One full SSPRK3 step with the reference's structure
 * (integrate_advance with state_transform_t, time-integration/advance.h:234-280;
 * ssprk3_t, time-integration/explicit.h:80-88):
 *   R0 = L(q);  q1 = q + dt R0;                      fill ghosts
 *   R1 = L(q1); q2 = q1 - 3/4 dt R0 + 1/4 dt R1;     fill ghosts
 *   R2 = L(q2); q  = q2 - 1/12 dt R0 - 1/12 dt R1 + 2/3 dt R2; fill ghosts
 * (updates in conservative variables, state kept primitive; bit-identical to
 * the reference in GBNS_PREC_FP64).  Each stage is one gbns_flux_div_rk
 * launch plus a ghost fill.  `work` is a caller-owned device buffer of 3
 * AoS5 arrays (3*gbns_array_size doubles) holding R0, R1 and the
 * intermediate state.  prims must have valid ghosts on entry.  Asynchronous. */
int gbns_ssprk3_step(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                     const gbns_bc_desc* bc, double* prims, double* work,
                     double dt, void* stream);

/* nsteps gbns_ssprk3_step calls replayed from a CUDA graph of one step (six
 * launches).  The graph is captured on the first call for these arguments
 * (descriptors, prims, work, dt, device) and reused while they stay the same
 * (up to 8 are kept).  Results are bit-identical to the plain calls; for small
 * grids the launch overhead disappears.  The first call for new arguments
 * captures, which must not happen while `stream` is itself being captured.
 * No counterpart in the reference (its integrator launches every kernel). */
int gbns_ssprk3_run(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                    const gbns_bc_desc* bc, double* prims, double* work,
                    double dt, int nsteps, void* stream);

/* One gbns_ssprk3_step of a state held in host memory, with the copies
 * overlapped with the stages.  The blocks are split into `ngroups`
 * contiguous groups (0: the library's choice, min(8, blocks)).  Group g is
 * copied to the device on `copy_stream` while stage 1 runs on the groups
 * already there; after stage 3 each group's ghost fill and copy back run as
 * soon as the groups holding its ghost donors are done, while stage 3 goes
 * on with the later groups.
 *   host_prims  padded AoS5 state with valid ghosts (gbns_array_size
 *               doubles), page-locked (cudaHostAlloc / cudaHostRegister) for
 *               the copies to overlap; it receives the new state
 *   prims       device array of the same size (overwritten)
 *   work        as for gbns_ssprk3_step
 *   copy_stream a stream other than `stream`; NULL: a non-blocking stream the
 *               library keeps per device and host thread
 * Asynchronous: host_prims holds the new state once the work issued on
 * `stream` so far has finished (the call makes `stream` wait for its
 * copies).  Bit-identical to copying in, gbns_ssprk3_step, copying out: the
 * copies a reference caller makes around advance() on device-resident
 * state (time-integration/advance.h:234-280). */
int gbns_ssprk3_step_host(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                          const gbns_bc_desc* bc, double* host_prims, double* prims, double* work,
                          double dt, int ngroups, void* stream, void* copy_stream);

/* ---- source terms ----------------------------------------------------
 * Lowered forms of the point source a caller passes to
 * spade::pde_algs::source_term (pde-algs/source_term.h:19-51), written as
 * the flux_t (rho, rhoE, rhou, rhov, rhow) of the cell's primitives:
 */
#define GBNS_SOURCE_CONST       0  /* S = c[0..4] */
#define GBNS_SOURCE_BODY_FORCE  1  /* f = c[2..4] per unit volume: S = (0, f_x u + f_y v + f_z w, f_x, f_y, f_z) */
#define GBNS_SOURCE_BODY_ACCEL  2  /* g = c[2..4] per unit mass, rho = p/(R T):
                                      S = (0, rho (g_x u + g_y v + g_z w), rho g_x, rho g_y, rho g_z) */

typedef struct gbns_source_desc
{
    int32_t kind;          /* GBNS_SOURCE_* */
    int32_t reserved;      /* must be 0 */
    double  c[5];
    gbns_gas_desc gas;
} gbns_source_desc;

/* rhs += S(prims)/jac on every interior cell, jac the cell's coordinate
 * Jacobian (1 on identity coordinates).  Replaces
 * spade::pde_algs::source_term(q, rhs, source_func)
 * (pde-algs/source_term.h:19-51) for the lowered forms above.
 * Asynchronous. */
int gbns_source_term(const gbns_grid_desc* grid, const gbns_source_desc* source,
                     const double* prims, double* rhs, void* stream);

/* ---- batched form ----------------------------------------------------
 * Many independent grids ("instances") of uneven size advanced together:
 * each SSPRK3 stage is one flux launch per kernel class (one CTA per item of
 * a device work-list of tiles of every instance, with the stage update fused
 * into its epilogue) and one batched ghost fill; with use_graph the step
 * (six launches for one kernel class) is captured
 * once in a CUDA graph and replayed.  Instance state stays resident in an
 * arena of hbm_budget_bytes allocated at creation; adding an instance that
 * does not fit returns GBNS_ERR_CAPACITY.  Every instance's result is
 * bit-identical to advancing it alone (gbns_ssprk3_step).  Supported kernel
 * classes: cent_keep<2>, totani_lr, fweno_t, WENO5 and hybrid_scheme_t of
 * cent_keep<2> and fweno_t on identity grids, WENO5 on stretched-y grids; precision GBNS_PREC_FP64 or GBNS_PREC_FP32_FLUX
 * (one per batch).  All calls are ordered on the batch's stream.
 * No counterpart in the reference (its integrator advances one grid,
 * time-integration/integrator.h:52-55). */
typedef struct gbns_batch gbns_batch;

int gbns_batch_create(gbns_batch** batch, size_t hbm_budget_bytes, int precision, int use_graph, void* stream);
int gbns_batch_destroy(gbns_batch* batch);

/* Adds an instance; `prims` (device or pinned host pointer) holds its AoS5
 * initial state, copied in; ghosts are refilled.  dt is its fixed step. */
int gbns_batch_add(gbns_batch* batch, const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                   const gbns_bc_desc* bc, double dt, const double* prims, int* slot);
int gbns_batch_remove(gbns_batch* batch, int slot);

/* Advances every active instance by nsteps SSPRK3 steps (asynchronous); an
 * instance with a step limit (gbns_batch_set_steps) stops when it reaches
 * it and idles (its tiles are skipped on the device) until removed. */
int gbns_batch_step(gbns_batch* batch, int nsteps);

/* Step limit of an instance: it does at most nsteps more steps, counted on
 * the device, so a request can finish inside a chunk of steps without the
 * chunk being cut to it (nsteps < 0: no limit, the default).  Results are
 * those of exactly that many steps.  No reference counterpart. */
int gbns_batch_set_steps(gbns_batch* batch, int slot, long long nsteps);
/* Steps the instance still has to do (-1: no limit), as of the work enqueued. */
int gbns_batch_steps_left(gbns_batch* batch, int slot, long long* left);

/* Device pointer to an instance's AoS5 state (owned by the batch) and its step count. */
int gbns_batch_state(gbns_batch* batch, int slot, double** prims, long long* steps_done);

/* Arena bytes in use / budget, active instances, interior cells. */
int gbns_batch_usage(gbns_batch* batch, size_t* bytes_used, size_t* bytes_budget, int* active, long long* cells);

/* Arena bytes one instance of this grid occupies (state + 3 residuals); 0 if invalid. */
size_t gbns_batch_instance_bytes(const gbns_grid_desc* grid);

/* Tile autotuner of the batched form: for every kernel class present among
 * the active instances (the compile-time flux configuration: convective
 * scheme x coordinates, numbered 0 .. gbns_batch_class_count()-1), times
 * each of its tile variants (tile shape and threads per CTA) on the
 * instances' own arrays with CUDA events, `reps` launches of the
 * first SSPRK3 stage each (which writes only scratch arrays), and keeps the
 * fastest.  variants_out (optional, gbns_batch_class_count() ints) receives
 * the choice per class, -1 for absent classes.  Synchronises the batch.
 * Results do not depend on the variant (bit-identical).  No reference
 * counterpart (the reference picks tile shapes at compile time,
 * flux_div_*.h). */
int gbns_batch_autotune(gbns_batch* batch, int reps, int* variants_out);
int gbns_batch_set_variant(gbns_batch* batch, int kernel_class, int variant);
int gbns_batch_class_count(void);
/* Tile shape (x, y, z cells) of a class's variant at a precision. */
int gbns_batch_class_variant_info(int kernel_class, int precision, int variant, int* tile_xyz);

#ifdef __cplusplus
}
#endif

#endif /* GBNS_H */
