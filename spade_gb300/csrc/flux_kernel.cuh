// Fused flux-divergence kernel (sm_103a).
//
// One CTA owns one TX*TY*TZ tile of one grid block.  It stages the tile plus
// an H-cell halo (AoS5 doubles, straight from the grid_array layout) into
// shared memory with one 4-D TMA copy (or coalesced loads when the row pitch
// is not 16-byte aligned; FP32-flux can load the stencil cells straight into
// FP32), derives the per-cell quantities every face of the stencil shares
// (rho, e; for fweno/WENO5 in FP64 the Rusanov split f+/f- of each line cell,
// cached per direction), evaluates each face flux ONCE (the reference's
// flux_div_basic, flux_div_basic.h:47-76, evaluates every face twice) into a
// shared face buffer, and accumulates
//     rhs(cell) += jac*F(i-1/2)*inv_dx - jac*F(i+1/2)*inv_dx
// per direction in FP64 registers in the reference's order
// (flux_div_basic.h:109-129).  The epilogue writes the AoS5 residual and/or
// applies the SSPRK3 stage update to the tile's cells (gbns_flux_div_rk).
//
// Real = double: every operation in FP64 (the drop-in).
// Real = float : per-cell derivation and face fluxes in FP32, state read and
//                divergence accumulated, stage update and state in FP64.
#pragma once

#include <type_traits>
#include "gbns_internal.cuh"
#include "fp64_int.cuh"

namespace gbns
{
    template <int CONV, int ORDER>
    struct ConvTraits
    {
        static constexpr int HC =
            (CONV == GBNS_CONV_CENT_KEEP) ? ORDER/2 :
            (CONV == GBNS_CONV_TOTANI)    ? 1 :
            (CONV == GBNS_CONV_FWENO)     ? 2 :
            (CONV == GBNS_CONV_WENO5)     ? 3 :
            (CONV == GBNS_CONV_HYBRID)    ? (ORDER/2 > 2 ? ORDER/2 : 2) : 0;
        // derived per-cell values: centred schemes (rho, e), fweno/WENO5
        // (rho, Rusanov speed * rho/2, total energy); the hybrid keeps the
        // fweno three plus the centred e (rho is the same value for both).
        static constexpr int NDER =
            (CONV == GBNS_CONV_HYBRID) ? 4 :
            (CONV == GBNS_CONV_FWENO || CONV == GBNS_CONV_WENO5) ? 3 :
            (CONV == GBNS_CONV_CENT_KEEP || CONV == GBNS_CONV_TOTANI) ? 2 : 0;
    };

    template <bool S> using YTabT = typename std::conditional<S, YTabK, YTabNone>::type;

    // a*b and x*2^E of a tile configuration: the integer-pipe forms in the
    // no-contraction FP64 units, the plain operators elsewhere
    template <class Cfg>
    __device__ __forceinline__ typename Cfg::Real pmul(typename Cfg::Real a, typename Cfg::Real b)
    {
        if constexpr (Cfg::IMUL) return dmul_int(a, b);
        else return a*b;
    }
    template <class Cfg, int E>
    __device__ __forceinline__ typename Cfg::Real ppow2(typename Cfg::Real x)
    {
        static_assert(E == -1 || E == -2, "x/2 or x/4");
        using Real = typename Cfg::Real;
        if constexpr (Cfg::IMUL) return dmul_pow2<E>(x);
        else return (E == -1 ? Real(0.5) : Real(0.25))*x;
    }
    // 2*x (exact): an exponent increment on the integer pipes in the IMUL tiles
    // (in the others a DMUL by 2 measured faster than the integer sequence)
    template <class Cfg>
    __device__ __forceinline__ typename Cfg::Real ptwice(typename Cfg::Real x)
    {
        using Real = typename Cfg::Real;
        if constexpr (Cfg::IMUL) return dmul_2(x);
        else return Real(2.0)*x;
    }
    // nD*x with nD the face normal's metric factor (1 on identity grids,
    // where the plain product folds away)
    template <class Cfg>
    __device__ __forceinline__ typename Cfg::Real nmul(typename Cfg::Real nD, typename Cfg::Real x)
    {
        if constexpr (Cfg::STRETCH) return pmul<Cfg>(x, nD);
        else return x*nD;
    }

    constexpr int cmax3(int a, int b, int c) { return a > b ? (a > c ? a : c) : (b > c ? b : c); }
    constexpr size_t align128(size_t x) { return (x + 127) & ~size_t(127); }

    // TAG_ distinguishes translation units that instantiate the same
    // arithmetic with different compiler settings (FMA contraction on/off),
    // so their kernels and launchers never share a symbol.
    // STG_ (FP32 only): 0 = stage the FP64 box (TMA or coalesced loads) and
    // convert it; 1 = load the stencil cells straight into FP32 shared
    // memory (no FP64 staging buffer, more CTAs per SM); 2 = one TMA copy of
    // the box from the FP32 SoA copy of the state (shadow.cu), which lands
    // in shared memory already in the kernel's SoA layout.
    // Translation units compiled without FMA contraction (-fmad=false): the
    // FP64 drop-in's flux_f64x_* (tags 0-3), the batched FP64 kernel (64) and
    // boundary_flux (66).
    constexpr bool tag_no_fma(int tag) { return tag < 4 || tag == 64 || tag == 66; }

    template <class Real_, int CONV_, int ORDER_, bool STRETCH_, int TX_, int TY_, int TZ_, int NT_, int TAG_, int STG_ = 0>
    struct FluxCfg
    {
        using Real = Real_;
        // FP64 products on the integer pipes (dmul_int / dmul_pow2: the same
        // bits) in the throughput tiles of more than 512 threads, whose 18+
        // warps per SM hide the longer integer chains (smaller tiles, chosen
        // for small latency-bound grids, keep the FP64 unit): every WENO5
        // product (explicit FMAs, so in both FP64 modes) and every division
        // (correctly rounded in both modes), and the reference's flux products
        // where no FMA contraction could have fused them
        static constexpr bool IEMU = std::is_same<Real_, double>::value && NT_ > 512;
        // FP64 quotients and square roots on the integer pipes (ddiv_int,
        // dsqrt_int: correctly rounded, the same bits) in the FP64 tiles of
        // 256 threads and more (Taylor-Green, 2.1M cells: 2.48 -> 2.40 ms at
        // 256 threads); the 128-thread tiles the autotuner picks for small,
        // latency-bound grids keep the FP64 unit's (the 32K-cell step measured
        // 0.222 vs 0.237 ms)
        static constexpr bool IDIV = std::is_same<Real_, double>::value && NT_ >= 256;
        static constexpr bool IMUL = IEMU && tag_no_fma(TAG_);
        static constexpr int CONV = CONV_, ORDER = ORDER_;
        static constexpr bool STRETCH = STRETCH_;
        static constexpr int TX = TX_, TY = TY_, TZ = TZ_, NT = NT_;
        static constexpr bool FP64 = std::is_same<Real, double>::value;
        static constexpr bool DIRECT = !FP64 && STG_ == 1;
        static constexpr bool SHADOW = !FP64 && STG_ == 2;
        static constexpr int HC = ConvTraits<CONV, ORDER>::HC;
        static constexpr int H = HC > 1 ? HC : 1;
        static constexpr int NDER = ConvTraits<CONV, ORDER>::NDER;
        // x start is rounded down to an even padded cell (TMA 16-byte rule),
        // so the box is one cell wider and its width is kept even.
        // (FP32 copy: its rows are laid out so every tile's box starts on a
        // 16-byte boundary; the width is rounded up to whole 16-byte groups)
        static constexpr int BXE = SHADOW ? ((TX + 2*H + 3) & ~3) : (((TX + 2*H + 1) + 1) & ~1);
        static constexpr int BY = TY + 2*H, BZ = TZ + 2*H;
        static constexpr int BOXN = BXE*BY*BZ;
        static constexpr int SX = 1, SY = BXE, SZ = BXE*BY;
        static constexpr int NCELL = TX*TY*TZ;
        static constexpr int NF0 = (TX + 1)*TY*TZ, NF1 = TX*(TY + 1)*TZ, NF2 = TX*TY*(TZ + 1);
        static constexpr int NFMAX = cmax3(NF0, NF1, NF2);
        static constexpr int CPT = (NCELL + NT - 1)/NT;
        static constexpr size_t STAGE_BYTES = (DIRECT || SHADOW) ? 0 : align128(size_t(BOXN)*5*sizeof(double));
        static constexpr size_t SOA_BYTES   = FP64 ? 0 : align128(size_t(BOXN)*5*sizeof(float));
        // FP64 fweno / WENO5: the Rusanov split (f+ and f- of the 5 equations)
        // of every cell on the tile's lines along the current direction is
        // computed once per cell and direction into shared memory instead of
        // once per stencil point per face (each cell sits in 4 or 6 face
        // stencils per direction); it takes the place of the derived buffer.
        // The hybrid scheme's fweno half uses the same cache; its centred half
        // keeps (rho, e) per box cell after it (NDERB = 2).
        static constexpr bool SPLIT = FP64 && (CONV == GBNS_CONV_FWENO || CONV == GBNS_CONV_WENO5 ||
                                               CONV == GBNS_CONV_HYBRID);
        static constexpr int NL0 = (TX + 2*HC)*TY*TZ, NL1 = TX*(TY + 2*HC)*TZ, NL2 = TX*TY*(TZ + 2*HC);
        static constexpr int NLMAX = cmax3(NL0, NL1, NL2);
        // derived values per box cell kept in the der buffer
        static constexpr int NDERB = SPLIT ? (CONV == GBNS_CONV_HYBRID ? 2 : 0) : NDER;
        // slot of the centred internal energy p/(rho (gamma-1))
        static constexpr int CK_E = (CONV == GBNS_CONV_HYBRID && !SPLIT) ? 3 : 1;
        static constexpr size_t SPLIT_BYTES = SPLIT ? align128(size_t(10)*NLMAX*sizeof(double)) : 0;
        static constexpr size_t DER_BYTES   = SPLIT_BYTES +
            ((SPLIT && NDERB == 0) ? 0 : align128(size_t(NDERB > 0 ? NDERB : 1)*BOXN*sizeof(Real)));
        // FP32-flux evaluates the faces of all three directions in one
        // balanced loop (warp-aligned direction boundaries), which needs the
        // face buffer for all of them; FP64 (split cache per direction) keeps
        // one direction at a time.
        static constexpr bool MERGED = !FP64 && (NF0 % 32 == 0) && ((NF0 + NF1) % 32 == 0);
        static constexpr int NFS = MERGED ? NF0 + NF1 + NF2 : NFMAX;
        // face fluxes are kept in FP64 (converted once per face)
        static constexpr size_t FLX_BYTES   = align128(size_t(5)*NFS*sizeof(double));
        // FP32 staged: the staging buffer is dead once converted, so derived
        // values and face fluxes reuse it when they fit.
        static constexpr bool REUSE = !FP64 && !DIRECT && !SHADOW && (DER_BYTES + FLX_BYTES <= STAGE_BYTES);
        // FP32-flux on stretched grids: the tile's rows of the y-metric
        // tables (m, 1/m at cell centres, 1/m at y-faces) as floats, converted
        // once per tile instead of once per face
        static constexpr size_t YM_BYTES = (!FP64 && STRETCH) ? align128(size_t(3)*(TY + 1)*sizeof(float)) : 0;
        static constexpr size_t YM_OFF = 128 + STAGE_BYTES + SOA_BYTES + (REUSE ? 0 : DER_BYTES + FLX_BYTES);
        static constexpr size_t SMEM_BYTES = YM_OFF + YM_BYTES;
        static_assert(SMEM_BYTES <= 227*1024, "tile does not fit in shared memory");
        // CTAs per SM that shared memory allows (the register budget follows)
        static constexpr int MINB_RAW = int((227*1024) / (SMEM_BYTES + 1024));
        // (tiles of more than 512 threads run one CTA per SM: two would leave
        // fewer than 57 registers per thread)
        static constexpr int MINB = NT > 512 ? 1 : (MINB_RAW < 1 ? 1 : (MINB_RAW > 4 ? 4 : MINB_RAW));
        static_assert(5*BXE <= 256, "TMA box inner extent exceeds 256 elements");
    };

    // Shared-memory view of the staged box.
    template <class Cfg>
    struct BoxView
    {
        using Real = typename Cfg::Real;
        const double* stage;   // AoS doubles (FP64 compute)
        const float*  soa;     // SoA floats (FP32 compute)
        const Real*   der;     // derived per-cell values, SoA
        const double* split;   // SPLIT: f+/f- per equation of the current direction's line cells
        const float*  ymet;    // FP32 stretched: m_cell, im_cell, im_face rows of the tile (TY + 1 each)
        __device__ __forceinline__ Real q(int v, int c) const
        {
            if constexpr (Cfg::FP64) return stage[c*5 + v];
            else return soa[v*Cfg::BOXN + c];
        }
        __device__ __forceinline__ Real d(int k, int c) const { return der[k*Cfg::BOXN + c]; }
    };

    template <class Real>
    struct SchemeR
    {
        Real gamma, R, gm1, spec_heat, inv_gamma_avg, R_avg, eps_p, eps_T, sens;
        Real mu, beta_c, alpha_c, T_ref, power, inv_pr, prandtl, tref_plus_s, S;
        Real ck_a[4];
        int diss, visc, law, smooth, sensor, hyb_flux, hyb_sensor;
        Real hyb_param;
        __device__ __forceinline__ void load(const SchemeK& s)
        {
            diss = s.diss; visc = s.visc; law = s.law; smooth = s.smooth; sensor = s.sensor;
            hyb_flux = s.hyb_flux; hyb_sensor = s.hyb_sensor;
            if constexpr (sizeof(Real) == 4)
            {
                const auto& f = s.f32;
                gamma = f.gamma; R = f.R; gm1 = f.gm1; spec_heat = f.spec_heat; inv_gamma_avg = f.inv_gamma_avg;
                R_avg = f.R_avg; eps_p = f.eps_p; eps_T = f.eps_T; sens = f.sens; mu = f.mu; beta_c = f.beta_c;
                alpha_c = f.alpha_c; T_ref = f.T_ref; power = f.power; inv_pr = f.inv_pr; prandtl = f.prandtl;
                tref_plus_s = f.tref_plus_s; S = f.S; hyb_param = f.hyb_param;
                for (int i = 0; i < 4; ++i) ck_a[i] = f.ck_a[i];
                return;
            }
            gamma = Real(s.gamma); R = Real(s.R); gm1 = Real(s.gm1); spec_heat = Real(s.spec_heat);
            inv_gamma_avg = Real(s.inv_gamma_avg); R_avg = Real(s.R_avg);
            eps_p = Real(s.eps_p); eps_T = Real(s.eps_T); sens = Real(s.sens);
            mu = Real(s.mu); beta_c = Real(s.beta_c); alpha_c = Real(s.alpha_c);
            T_ref = Real(s.T_ref); power = Real(s.power); inv_pr = Real(s.inv_pr); prandtl = Real(s.prandtl);
            tref_plus_s = Real(s.tref_plus_s); S = Real(s.S);
            for (int i = 0; i < 4; ++i) ck_a[i] = Real(s.ck_a[i]);
            hyb_param = Real(s.hyb_param);
        }
    };

    // a/b: the correctly rounded FP64 division, and in FP32-flux arithmetic the
    // fast quotient (within 2 ulp for |b| in [2^-126, 2^126], which holds for
    // every divisor below: gas constants, temperatures, densities and the
    // Ducros sensor's denominator)
    // (IM: FP64 on the integer pipes, ddiv_int, the same bits)
    template <bool IM = false>
    __device__ __forceinline__ double pdiv(double a, double b)
    {
        if constexpr (IM) return ddiv_int(a, b);
        else return a/b;
    }
    template <bool IM = false>
    __device__ __forceinline__ float pdiv(float a, float b) { return __fdividef(a, b); }
    template <bool IM = false>
    __device__ __forceinline__ double dev_sqrt(double x)
    {
        if constexpr (IM) return dsqrt_int(x);
        else return sqrt(x);
    }
    template <bool IM = false>
    __device__ __forceinline__ float dev_sqrt(float x) { return sqrtf(x); }
    __device__ __forceinline__ double dev_pow(double x, double y) { return pow(x, y); }
    __device__ __forceinline__ float  dev_pow(float x, float y)   { return powf(x, y); }

    // ------------------------------------------------------------------
    // per-cell derived quantities (computed once per staged cell)
    // fweno_t per-point quantities (convective.h:360-376, 458-467): rho,
    // h = rho (|u| + a)/2 (the Rusanov speed times rho/2) and the total
    // specific energy e.
    // (IM: quotients and square roots on the integer pipes; IMUL: the
    // products too, dmul_int / dmul_pow2; the same bits either way)
    template <class Real, bool IM = false, bool IMUL = false>
    __device__ __forceinline__ void fweno_derive(const SchemeR<Real>& S, Real p, Real T, Real u, Real v, Real w,
                                                 Real& rho_o, Real& h_o, Real& e_o)
    {
        auto mul = [](Real a, Real b) -> Real {
            if constexpr (IMUL) return dmul_int(a, b);
            else return a*b;
        };
        auto half = [](Real x) -> Real {
            if constexpr (IMUL) return dmul_pow2<-1>(x);
            else return x*Real(0.5);
        };
        Real r = mul(S.R, T);
        Real h = mul(u, u);
        h += mul(v, v);
        h += mul(w, w);
        h = dev_sqrt<IM>(h);
        h += dev_sqrt<IM>(mul(r, S.gamma));
        const Real rho = pdiv<IM>(p, r);
        h = mul(h, rho);
        h = half(h);
        Real e = mul(u, u);
        e += mul(v, v);
        e += mul(w, w);
        e = half(e);
        e += pdiv<IM>(mul(S.R, T), S.gm1);
        rho_o = rho; h_o = h; e_o = e;
    }

    // ------------------------------------------------------------------
    template <class Cfg>
    __device__ __forceinline__ void derive_cell(const BoxView<Cfg>& V, typename Cfg::Real* der,
                                                const SchemeR<typename Cfg::Real>& S, int c)
    {
        using Real = typename Cfg::Real;
        const Real p = V.q(0, c), T = V.q(1, c), u = V.q(2, c), v = V.q(3, c), w = V.q(4, c);
        if constexpr (Cfg::CONV == GBNS_CONV_CENT_KEEP || Cfg::CONV == GBNS_CONV_TOTANI ||
                      (Cfg::CONV == GBNS_CONV_HYBRID && Cfg::SPLIT))
        {
            // convective.h:130-131 / 80-84 (the hybrid's fweno half reads the split cache)
            const Real rho = pdiv<Cfg::IDIV>(p, pmul<Cfg>(S.R, T));
            der[0*Cfg::BOXN + c] = rho;
            der[1*Cfg::BOXN + c] = pdiv<Cfg::IDIV>(p, pmul<Cfg>(rho, S.gm1));
        }
        else if constexpr (Cfg::CONV == GBNS_CONV_FWENO || Cfg::CONV == GBNS_CONV_WENO5 ||
                           Cfg::CONV == GBNS_CONV_HYBRID)
        {
            Real rho, h, e;
            fweno_derive<Real, Cfg::IDIV, Cfg::IMUL>(S, p, T, u, v, w, rho, h, e);
            der[0*Cfg::BOXN + c] = rho;
            der[1*Cfg::BOXN + c] = h;
            der[2*Cfg::BOXN + c] = e;
            // cent_keep's e (convective.h:131); its rho = p/(R*T) is the
            // same rounding as fweno's p/r above
            if constexpr (Cfg::CONV == GBNS_CONV_HYBRID) der[3*Cfg::BOXN + c] = pdiv<Cfg::IDIV>(p, pmul<Cfg>(rho, S.gm1));
        }
    }

    // ------------------------------------------------------------------
    // face fluxes.  D = face direction, rc = box index of the right cell,
    // nD = normal component along D (1 for identity coordinates).
    // ------------------------------------------------------------------
    template <class Cfg, int D> struct DirStride
    {
        static constexpr int S  = D == 0 ? Cfg::SX : (D == 1 ? Cfg::SY : Cfg::SZ);
        static constexpr int S1 = (D + 1) % 3 == 0 ? Cfg::SX : ((D + 1) % 3 == 1 ? Cfg::SY : Cfg::SZ);
        static constexpr int S2 = (D + 2) % 3 == 0 ? Cfg::SX : ((D + 2) % 3 == 1 ? Cfg::SY : Cfg::SZ);
    };

    // cent_keep_scheme_t::operator() (convective.h:117-184)
    template <class Cfg, int D>
    __device__ __forceinline__ void conv_cent_keep(const BoxView<Cfg>& V, const SchemeR<typename Cfg::Real>& S,
                                                   int rc, typename Cfg::Real nD, typename Cfg::Real* out)
    {
        using Real = typename Cfg::Real;
        constexpr int W = Cfg::ORDER, hw = Cfg::ORDER/2, SD = DirStride<Cfg, D>::S;
        Real un[W], rho[W], eng[W];
        #pragma unroll
        for (int m = 0; m < W; ++m)
        {
            const int c = rc + (m - hw)*SD;
            un[m]  = nmul<Cfg>(nD, V.q(2 + D, c));
            rho[m] = V.d(0, c);
            eng[m] = V.d(Cfg::CK_E, c);
        }
        // the reference's products in its order; pmul / ppow2 / ptwice are the
        // plain operators except in the IMUL tiles (integer pipes, same bits)
        Real cc = 0, mx = 0, my = 0, mz = 0, g = 0, k = 0, ie = 0, pp = 0;
        #pragma unroll
        for (int ii = 1; ii < hw + 1; ++ii)
        {
            const Real a = S.ck_a[ii - 1];
            #pragma unroll
            for (int jj = 0; jj < ii; ++jj)
            {
                const int i0 = hw - 1 - jj, i1 = i0 + ii;
                const int c0 = rc + (i0 - hw)*SD, c1 = rc + (i1 - hw)*SD;
                const Real u0 = V.q(2, c0), v0 = V.q(3, c0), w0 = V.q(4, c0), p0 = V.q(0, c0);
                const Real u1 = V.q(2, c1), v1 = V.q(3, c1), w1 = V.q(4, c1), p1 = V.q(0, c1);
                const Real c_loc = pmul<Cfg>(a, pmul<Cfg>(ppow2<Cfg, -2>(rho[i0] + rho[i1]), un[i1] + un[i0]));
                cc += c_loc;
                mx += pmul<Cfg>(c_loc, ppow2<Cfg, -1>(u0 + u1));
                my += pmul<Cfg>(c_loc, ppow2<Cfg, -1>(v0 + v1));
                mz += pmul<Cfg>(c_loc, ppow2<Cfg, -1>(w0 + w1));
                g  += pmul<Cfg>(a, ppow2<Cfg, -1>(p0 + p1));
                k  += pmul<Cfg>(ppow2<Cfg, -1>(c_loc), pmul<Cfg>(u0, u1) + pmul<Cfg>(v0, v1) + pmul<Cfg>(w0, w1));
                ie += pmul<Cfg>(c_loc, ppow2<Cfg, -1>(eng[i0] + eng[i1]));
                pp += pmul<Cfg>(a, ppow2<Cfg, -1>(pmul<Cfg>(un[i0], p1) + pmul<Cfg>(un[i1], p0)));
            }
        }
        out[0] = ptwice<Cfg>(cc);
        out[1] = ptwice<Cfg>(k + ie + pp);
        out[2] = ptwice<Cfg>(D == 0 ? mx + nmul<Cfg>(nD, g) : mx);
        out[3] = ptwice<Cfg>(D == 1 ? my + nmul<Cfg>(nD, g) : my);
        out[4] = ptwice<Cfg>(D == 2 ? mz + nmul<Cfg>(nD, g) : mz);
    }

    // totani_lr::operator() (convective.h:68-93)
    template <class Cfg, int D>
    __device__ __forceinline__ void conv_totani(const BoxView<Cfg>& V, const SchemeR<typename Cfg::Real>& S,
                                                int rc, typename Cfg::Real nD, typename Cfg::Real* out)
    {
        using Real = typename Cfg::Real;
        constexpr int SD = DirStride<Cfg, D>::S;
        const int cl = rc - SD, cr = rc;
        const Real pl = V.q(0, cl), ul = V.q(2, cl), vl = V.q(3, cl), wl = V.q(4, cl);
        const Real pr = V.q(0, cr), ur = V.q(2, cr), vr = V.q(3, cr), wr = V.q(4, cr);
        const Real un_l = nmul<Cfg>(nD, V.q(2 + D, cl)), un_r = nmul<Cfg>(nD, V.q(2 + D, cr));
        const Real rho_l = V.d(0, cl), rho_r = V.d(0, cr);
        const Real e_l = V.d(1, cl), e_r = V.d(1, cr);
        const Real c = pmul<Cfg>(ppow2<Cfg, -2>(rho_l + rho_r), un_l + un_r);
        const Real hc = ppow2<Cfg, -1>(c);
        out[0] = c;
        out[1] = pmul<Cfg>(hc, e_l + e_r + pmul<Cfg>(ul, ur) + pmul<Cfg>(vl, vr) + pmul<Cfg>(wl, wr)) +
                 ppow2<Cfg, -1>(pmul<Cfg>(un_l, pr) + pmul<Cfg>(un_r, pl));
        const Real pn = ppow2<Cfg, -1>(nmul<Cfg>(nD, pl) + nmul<Cfg>(nD, pr));
        out[2] = pmul<Cfg>(hc, ul + ur) + (D == 0 ? pn : Real(0));
        out[3] = pmul<Cfg>(hc, vl + vr) + (D == 1 ? pn : Real(0));
        out[4] = pmul<Cfg>(hc, wl + wr) + (D == 2 ? pn : Real(0));
    }

    // fweno_t flux/dissipation of equation `eq` at one stencil point
    // (convective.h:442-493).
    template <class Cfg, int D>
    __device__ __forceinline__ void fweno_point_v(const BoxView<Cfg>& V, const SchemeR<typename Cfg::Real>& S,
                                                  int c, typename Cfg::Real rho, typename Cfg::Real hsr,
                                                  typename Cfg::Real engy_c, int eq, typename Cfg::Real nD,
                                                  typename Cfg::Real& fl, typename Cfg::Real& ds)
    {
        using Real = typename Cfg::Real;
        const Real un = nmul<Cfg>(nD, V.q(2 + D, c));
        if (eq == 0)
        {
            fl = pmul<Cfg>(un, ppow2<Cfg, -1>(rho));
            ds = hsr;
        }
        else if (eq == 1)
        {
            const Real engy = engy_c;
            fl = pmul<Cfg>(pmul<Cfg>(un, ppow2<Cfg, -1>(rho)), engy + pmul<Cfg>(S.R, V.q(1, c)));
            ds = pmul<Cfg>(hsr, engy);
        }
        else
        {
            const int dr = eq - 2;
            const Real ud = V.q(2 + dr, c);
            Real m = pmul<Cfg>(un, rho);
            m = pmul<Cfg>(m, ud);
            if (dr == D) m += nmul<Cfg>(nD, V.q(0, c));
            m = ppow2<Cfg, -1>(m);
            fl = m;
            ds = pmul<Cfg>(hsr, ud);
        }
    }

    template <class Cfg, int D>
    __device__ __forceinline__ void fweno_point(const BoxView<Cfg>& V, const SchemeR<typename Cfg::Real>& S,
                                                int c, int eq, typename Cfg::Real nD,
                                                typename Cfg::Real& fl, typename Cfg::Real& ds)
    {
        fweno_point_v<Cfg, D>(V, S, c, V.d(0, c), V.d(1, c), V.d(2, c), eq, nD, fl, ds);
    }

    // apply_weno of fweno_t (convective.h:378-427).  FP64 with IMUL: the
    // products on the integer pipes (dmul_int; x/2 as dmul_pow2 and -x/2 as
    // its negation, exact since rounding is sign-symmetric), with IM the two
    // divisions too (ddiv_int): the same bits as the FP64 unit's.
    template <class Real, bool IMUL = false, bool IM = false>
    __device__ __forceinline__ Real fweno_apply_ud(const Real fu[4], const Real fd[4], int smooth)
    {
        auto mul = [](Real a, Real b) -> Real {
            if constexpr (IMUL) return dmul_int(a, b);
            else return a*b;
        };
        auto half = [](Real x) -> Real {
            if constexpr (IMUL) return dmul_pow2<-1>(x);
            else return Real(0.5)*x;
        };
        auto mhalf = [](Real x) -> Real {
            if constexpr (IMUL) return -dmul_pow2<-1>(x);
            else return Real(-0.5)*x;
        };
        const Real f0uk = fu[0], f0dk = fd[0];
        const Real f1uk = fu[1], f1dk = fd[1];
        const Real f2uk = fu[2], f2dk = fd[2];
        const Real f3uk = fu[3], f3dk = fd[3];
        const Real r0 = mhalf(f0uk) + mul(Real(1.5), f1uk);
        const Real r1 = half(f1uk) + half(f2uk);
        const Real r2 = half(f1dk) + half(f2dk);
        const Real r3 = mul(Real(1.5), f2dk) - half(f3dk);
        if (!smooth)
            return mul(Real(1.0/3.0), r0) + mul(Real(2.0/3.0), r1) + mul(Real(2.0/3.0), r2) + mul(Real(1.0/3.0), r3);
        const Real eps = Real(1e-16);
        if constexpr (sizeof(Real) == 4)
        {
            // FP32: (d^2 + eps)^2 overflows once |d| passes ~4e9 (energy
            // fluxes of ~1e8 with steep neighbours reach it).  Each weight
            // is a ratio of two such terms, unchanged when both differences
            // and eps are scaled by the pair's largest |d| (eps by its
            // square); the floor keeps 1/s finite when both are zero (then
            // e = 1, i.e. the unscaled eps-only weights).
            auto wpair = [&](Real d0, Real d1) -> Real
            {
                const Real sc = fmaxf(fmaxf(fabsf(d0), fabsf(d1)), Real(1e-8));
                const Real is = Real(1.0)/sc;
                const Real e = (eps*is)*is;
                Real x0 = d0*is, x1 = d1*is;
                x0 = x0*x0 + e; x0 *= x0;
                x1 = x1*x1 + e; x1 *= x1;
                return x1/(x0 + x0 + x1);
            };
            const Real w0 = wpair(f0uk - f1uk, f1uk - f2uk);
            const Real w3 = wpair(f2dk - f3dk, f1dk - f2dk);
            return w0*r0 + (Real(1.0) - w0)*r1 + (Real(1.0) - w3)*r2 + w3*r3;
        }
        Real a0 = (f0uk) - (f1uk), a1 = (f1uk) - (f2uk), a2 = (f1dk) - (f2dk), a3 = (f2dk) - (f3dk);
        a0 = mul(a0, a0); a0 += eps; a0 = mul(a0, a0);
        a1 = mul(a1, a1); a1 += eps; a1 = mul(a1, a1);
        a2 = mul(a2, a2); a2 += eps; a2 = mul(a2, a2);
        a3 = mul(a3, a3); a3 += eps; a3 = mul(a3, a3);
        a0 += a0; a0 += a1; a0 = pdiv<IM>(a1, a0);
        a3 += a3; a3 += a2; a3 = pdiv<IM>(a2, a3);
        a1 = Real(1.0) - a0;
        a2 = Real(1.0) - a3;
        return mul(a0, r0) + mul(a1, r1) + mul(a2, r2) + mul(a3, r3);
    }

    template <class Real>
    __device__ __forceinline__ Real fweno_apply(const Real fl[4], const Real ds[4], int smooth)
    {
        Real fu[4], fd[4];
        #pragma unroll
        for (int m = 0; m < 4; ++m) { fu[m] = fl[m] + ds[m]; fd[m] = fl[m] - ds[m]; }
        return fweno_apply_ud<Real>(fu, fd, smooth);
    }

    // Line stride of the split cache along D and the cache index of a face's
    // right cell (tile-local fx, fy, fz).
    template <class Cfg, int D> struct SplitIdx
    {
        static constexpr int HC = Cfg::HC;
        static constexpr int LX = Cfg::TX + (D == 0 ? 2*HC : 0);
        static constexpr int LY = Cfg::TY + (D == 1 ? 2*HC : 0);
        static constexpr int LZ = Cfg::TZ + (D == 2 ? 2*HC : 0);
        static constexpr int NL = LX*LY*LZ;
        static constexpr int LS = D == 0 ? 1 : (D == 1 ? LX : LX*LY);
        __device__ __forceinline__ static int right(int fx, int fy, int fz)
        {
            return (fx + (D == 0 ? HC : 0)) + LX*((fy + (D == 1 ? HC : 0)) + LY*(fz + (D == 2 ? HC : 0)));
        }
    };

    // Fills the split cache for direction D: f+ = fl + ds and f- = fl - ds of
    // every equation at every cell of the tile's lines along D (the stencil
    // cells of all faces of the pass), with the same operations fweno_point
    // performs per face.  The tile's own cells take rho, h and e from `dc`
    // (computed once per tile, each thread for the cells it owns); the halo
    // cells along D derive them here.
    template <class Cfg, int D>
    __device__ __forceinline__ void split_fill(const BoxView<Cfg>& V, const SchemeR<double>& S, double* P,
                                               const YTabT<Cfg::STRETCH>& Y, int by, int j0, int ny, int shift,
                                               const double (&dc)[Cfg::CPT][3])
    {
        using SI = SplitIdx<Cfg, D>;
        constexpr int H = Cfg::H, HC = Cfg::HC, TX = Cfg::TX, TY = Cfg::TY, TZ = Cfg::TZ;
        auto store = [&](int l, int c, int y, double rho, double hsr, double engy)
        {
            double nD = 1.0;
            if constexpr (Cfg::STRETCH && D != 1)
            {
                if (j0 + y < ny) nD = Y.m_cell[by*ny + j0 + y];
            }
            #pragma unroll
            for (int eq = 0; eq < 5; ++eq)
            {
                double fl, ds;
                fweno_point_v<Cfg, D>(V, S, c, rho, hsr, engy, eq, nD, fl, ds);
                P[(2*eq)*Cfg::NLMAX + l] = fl + ds;
                P[(2*eq + 1)*Cfg::NLMAX + l] = fl - ds;
            }
        };
        #pragma unroll
        for (int s = 0; s < Cfg::CPT; ++s)
        {
            const int cc = threadIdx.x + s*Cfg::NT;
            if (cc >= Cfg::NCELL) break;
            const int cx = cc % TX, cy = (cc / TX) % TY, cz = cc / (TX*TY);
            const int c = (cz + H)*Cfg::SZ + (cy + H)*Cfg::SY + (cx + H + shift);
            store(SI::right(cx, cy, cz), c, cy, dc[s][0], dc[s][1], dc[s][2]);
        }
        // halo cells of the lines: 2*HC layers along D
        constexpr int TA = D == 0 ? TY : TX;              // first transverse extent
        constexpr int NH = 2*HC*(D == 0 ? TY*TZ : (D == 1 ? TX*TZ : TX*TY));
        for (int h = threadIdx.x; h < NH; h += Cfg::NT)
        {
            const int hd = h % (2*HC), t = h / (2*HC);
            const int ld = hd < HC ? hd : hd + (D == 0 ? TX : (D == 1 ? TY : TZ));   // line coordinate along D
            const int ta = t % TA, tb = t / TA;
            const int lx = D == 0 ? ld : ta;
            const int ly = D == 1 ? ld : (D == 0 ? ta : tb);
            const int lz = D == 2 ? ld : tb;
            const int l = lx + SI::LX*(ly + SI::LY*lz);
            const int x = lx - (D == 0 ? HC : 0), y = ly - (D == 1 ? HC : 0), z = lz - (D == 2 ? HC : 0);
            const int c = (z + H)*Cfg::SZ + (y + H)*Cfg::SY + (x + H + shift);
            double rho, hsr, engy;
            fweno_derive<double, Cfg::IDIV, Cfg::IMUL>(S, V.q(0, c), V.q(1, c), V.q(2, c), V.q(3, c), V.q(4, c), rho, hsr, engy);
            store(l, c, y, rho, hsr, engy);
        }
    }

    template <class Cfg, int D>
    __device__ __forceinline__ void conv_fweno(const BoxView<Cfg>& V, const SchemeR<typename Cfg::Real>& S,
                                               int rc, int lr, typename Cfg::Real nD, typename Cfg::Real* out)
    {
        using Real = typename Cfg::Real;
        constexpr int SD = DirStride<Cfg, D>::S;
        #pragma unroll
        for (int eq = 0; eq < 5; ++eq)
        {
            if constexpr (Cfg::SPLIT)
            {
                constexpr int LS = SplitIdx<Cfg, D>::LS;
                Real fu[4], fd[4];
                #pragma unroll
                for (int m = 0; m < 4; ++m)
                {
                    fu[m] = V.split[(2*eq)*Cfg::NLMAX + lr + (m - 2)*LS];
                    fd[m] = V.split[(2*eq + 1)*Cfg::NLMAX + lr + (m - 2)*LS];
                }
                out[eq] = fweno_apply_ud<Real, Cfg::IMUL, Cfg::IDIV>(fu, fd, S.smooth);
            }
            else
            {
                Real fl[4], ds[4];
                #pragma unroll
                for (int m = 0; m < 4; ++m) fweno_point<Cfg, D>(V, S, rc + (m - 2)*SD, eq, nD, fl[m], ds[m]);
                out[eq] = fweno_apply<Real>(fl, ds, S.smooth);
            }
        }
    }

    // FP32 5th-order WENO-JS side reconstruction (Jiang & Shu 1996) for two
    // independent stencils at once, lane x and lane y of float2, cells a..e
    // upwind to downwind; no reference counterpart.  The arithmetic runs on
    // Blackwell's paired FP32 instructions (FFMA2, FMUL2, FADD2: one
    // instruction for both lanes); the maxima and the two divisions stay per
    // lane.  The FP32-flux face flux evaluates its f+ and f- sides as one pair.
    // (eps + beta)^2 overflows FP32 for beta > ~1.8e19, reached by the energy
    // equation's fluxes (~1e8) in steep regions; the normalised weights
    // g_k/D_k are unchanged when every beta and eps are divided by the largest
    // beta.  With the scaled D_k <= 1 the product form (one division) cannot
    // overflow; the floor keeps the sum positive when two stencils are
    // perfectly smooth.
    __device__ __forceinline__ float2 bc2(float v) { return make_float2(v, v); }
    __device__ __forceinline__ float2 max2(float2 a, float2 b) { return make_float2(fmaxf(a.x, b.x), fmaxf(a.y, b.y)); }

    __device__ __forceinline__ float2 weno5_side2(float2 a, float2 b, float2 c, float2 d, float2 e, int smooth)
    {
        const float c13 = 1.0f/3.0f, c16 = 1.0f/6.0f, c56 = 5.0f/6.0f, c76 = 7.0f/6.0f, c116 = 11.0f/6.0f;
        const float2 p0 = __ffma2_rn(bc2(c13), a, __ffma2_rn(bc2(-c76), b, __fmul2_rn(bc2(c116), c)));
        const float2 p1 = __ffma2_rn(bc2(-c16), b, __ffma2_rn(bc2(c56), c, __fmul2_rn(bc2(c13), d)));
        const float2 p2 = __ffma2_rn(bc2(c13), c, __ffma2_rn(bc2(c56), d, __fmul2_rn(bc2(-c16), e)));
        if (!smooth) return __ffma2_rn(bc2(0.1f), p0, __ffma2_rn(bc2(0.6f), p1, __fmul2_rn(bc2(0.3f), p2)));
        const float2 t0 = __fadd2_rn(__ffma2_rn(bc2(-2.0f), b, a), c);
        const float2 s0 = __ffma2_rn(bc2(3.0f), c, __ffma2_rn(bc2(-4.0f), b, a));
        const float2 t1 = __fadd2_rn(__ffma2_rn(bc2(-2.0f), c, b), d);
        const float2 s1 = __ffma2_rn(bc2(-1.0f), d, b);
        const float2 t2 = __fadd2_rn(__ffma2_rn(bc2(-2.0f), d, c), e);
        const float2 s2 = __ffma2_rn(bc2(3.0f), c, __ffma2_rn(bc2(-4.0f), d, e));
        const float2 k13 = bc2(13.0f/12.0f), q4 = bc2(0.25f);
        const float2 b0 = __ffma2_rn(__fmul2_rn(k13, t0), t0, __fmul2_rn(__fmul2_rn(q4, s0), s0));
        const float2 b1 = __ffma2_rn(__fmul2_rn(k13, t1), t1, __fmul2_rn(__fmul2_rn(q4, s1), s1));
        const float2 b2 = __ffma2_rn(__fmul2_rn(k13, t2), t2, __fmul2_rn(__fmul2_rn(q4, s2), s2));
        const float eps = 1e-16f;
        // the fast reciprocal and quotient (within 2 ulp) instead of the
        // correctly rounded division sequence; sc is kept below 2^126, the
        // fast reciprocal's range (no WENO5 indicator reaches it)
        const float2 sc = max2(max2(b0, b1), max2(b2, bc2(eps)));
        const float2 is = make_float2(__fdividef(1.0f, fminf(sc.x, 0x1p126f)), __fdividef(1.0f, fminf(sc.y, 0x1p126f)));
        const float2 ee = __fmul2_rn(bc2(eps), is);
        const float2 fl = bc2(1e-30f);
        const float2 u0 = __ffma2_rn(b0, is, ee), u1 = __ffma2_rn(b1, is, ee), u2 = __ffma2_rn(b2, is, ee);
        const float2 q0 = max2(__fmul2_rn(u0, u0), fl);
        const float2 q1 = max2(__fmul2_rn(u1, u1), fl);
        const float2 q2 = max2(__fmul2_rn(u2, u2), fl);
        const float2 a0 = __fmul2_rn(bc2(0.1f), __fmul2_rn(q1, q2));
        const float2 a1 = __fmul2_rn(bc2(0.6f), __fmul2_rn(q0, q2));
        const float2 a2 = __fmul2_rn(bc2(0.3f), __fmul2_rn(q0, q1));
        const float2 num = __ffma2_rn(a2, p2, __ffma2_rn(a1, p1, __fmul2_rn(a0, p0)));
        const float2 den = __fadd2_rn(__fadd2_rn(a0, a1), a2);
        return make_float2(__fdividef(num.x, den.x), __fdividef(num.y, den.y));
    }

    // FP64 WENO5-JS face flux F = F(f+ side) + F(f- side), each side a..e
    // upwind to downwind (no reference counterpart; the oracle restates it
    // operation for operation with C99 fma).  Per side, with q_k = 6 p_k the
    // candidate polynomials and B_k = 4 beta_k the smoothness indicators
    // (both scalings cancel in the normalised weights):
    //   E_k = (B_k + 4 eps)^2,  a_k = g_k prod_{j!=k} E_j,  N = sum a_k q_k,  D = sum a_k
    // and the two sides share one division:
    //   F = (N_u D_d + N_d D_u) / (6 D_u D_d)
    // (D_u D_d stays finite for flux differences below ~1e19; otherwise the
    // sides are divided separately).
    struct Weno5Side { double N, D; };

    template <bool IM>
    __device__ __forceinline__ double wmul(double a, double b)
    {
        if constexpr (IM) return dmul_int(a, b);
        else return a*b;
    }

    template <bool IM>
    __device__ __forceinline__ Weno5Side weno5_nd(double a, double b, double c, double d, double e)
    {
        // products through wmul: on the integer pipes in the throughput tiles
        // (bit-identical to a*b), the additions and FMAs on the FP64 unit
        const double q0 = fma(2.0, a, fma(-7.0, b, wmul<IM>(11.0, c)));
        const double q1 = fma(5.0, c, fma(2.0, d, -b));
        const double q2 = fma(2.0, c, fma(5.0, d, -e));
        const double t0 = fma(-2.0, b, a) + c, s0 = fma(3.0, c, fma(-4.0, b, a));
        const double t1 = fma(-2.0, c, b) + d, s1 = b - d;
        const double t2 = fma(-2.0, d, c) + e, s2 = fma(3.0, c, fma(-4.0, d, e));
        const double k = 13.0/3.0, eps4 = 4e-16;
        const double e0 = fma(wmul<IM>(k, t0), t0, wmul<IM>(s0, s0)) + eps4;
        const double e1 = fma(wmul<IM>(k, t1), t1, wmul<IM>(s1, s1)) + eps4;
        const double e2 = fma(wmul<IM>(k, t2), t2, wmul<IM>(s2, s2)) + eps4;
        const double E0 = wmul<IM>(e0, e0), E1 = wmul<IM>(e1, e1), E2 = wmul<IM>(e2, e2);
        const double a0 = wmul<IM>(0.1, wmul<IM>(E1, E2)), a1 = wmul<IM>(0.6, wmul<IM>(E0, E2));
        const double a2 = wmul<IM>(0.3, wmul<IM>(E0, E1));
        Weno5Side r;
        r.N = fma(a0, q0, fma(a1, q1, wmul<IM>(a2, q2)));
        r.D = (a0 + a1) + a2;
        return r;
    }

    template <bool IM>
    __device__ __forceinline__ double weno5_pair(double ua, double ub, double uc, double ud, double ue,
                                                 double da, double db, double dc, double dd, double de, int smooth)
    {
        if (!smooth)
        {
            const double pu = fma(0.1, fma(2.0, ua, fma(-7.0, ub, 11.0*uc)),
                                  fma(0.6, fma(5.0, uc, fma(2.0, ud, -ub)), 0.3*fma(2.0, uc, fma(5.0, ud, -ue))));
            const double pd = fma(0.1, fma(2.0, da, fma(-7.0, db, 11.0*dc)),
                                  fma(0.6, fma(5.0, dc, fma(2.0, dd, -db)), 0.3*fma(2.0, dc, fma(5.0, dd, -de))));
            return (pu + pd)*(1.0/6.0);
        }
        const Weno5Side u = weno5_nd<IM>(ua, ub, uc, ud, ue);
        const Weno5Side d = weno5_nd<IM>(da, db, dc, dd, de);
        const double den = wmul<IM>(6.0, wmul<IM>(u.D, d.D));
        // den < 1e300 as an unsigned compare of the bits (den is +0, positive,
        // +inf or a NaN here: a product of 6 and two sums of non-negative
        // weights; NaNs of either sign compare false as before), which keeps
        // the test off the FP64 unit
        if ((unsigned long long)__double_as_longlong(den) < 0x7E37E43C8800759Cull)
            return pdiv<IM>(fma(u.N, d.D, wmul<IM>(d.N, u.D)), den);
        return pdiv<IM>(u.N, 6.0*u.D) + pdiv<IM>(d.N, 6.0*d.D);
    }

    template <class Cfg, int D>
    __device__ __forceinline__ void conv_weno5(const BoxView<Cfg>& V, const SchemeR<typename Cfg::Real>& S,
                                               int rc, int lr, typename Cfg::Real nD, typename Cfg::Real* out)
    {
        using Real = typename Cfg::Real;
        constexpr int SD = DirStride<Cfg, D>::S;
        #pragma unroll
        for (int eq = 0; eq < 5; ++eq)
        {
            Real up[6], dn[6];
            #pragma unroll
            for (int m = 0; m < 6; ++m)
            {
                if constexpr (Cfg::SPLIT)
                {
                    constexpr int LS = SplitIdx<Cfg, D>::LS;
                    up[m] = V.split[(2*eq)*Cfg::NLMAX + lr + (m - 3)*LS];
                    dn[m] = V.split[(2*eq + 1)*Cfg::NLMAX + lr + (m - 3)*LS];
                }
                else
                {
                    Real fl, ds;
                    fweno_point<Cfg, D>(V, S, rc + (m - 3)*SD, eq, nD, fl, ds);
                    up[m] = fl + ds;
                    dn[m] = fl - ds;
                }
            }
            if constexpr (sizeof(Real) == 8)
                out[eq] = weno5_pair<Cfg::IEMU>(up[0], up[1], up[2], up[3], up[4], dn[5], dn[4], dn[3], dn[2], dn[1], S.smooth);
            else
            {
                const float2 f = weno5_side2(make_float2(up[0], dn[5]), make_float2(up[1], dn[4]),
                                             make_float2(up[2], dn[3]), make_float2(up[3], dn[2]),
                                             make_float2(up[4], dn[1]), S.smooth);
                out[eq] = f.x + f.y;
            }
        }
    }

    // pressure_diss_lr<gas, sensor>::operator() (convective.h:212-245); scl is
    // the sensor value at the face (const_sensor_t alpha or ducros_t).
    template <class Cfg, int D>
    __device__ __forceinline__ void diss_pressure(const BoxView<Cfg>& V, const SchemeR<typename Cfg::Real>& S,
                                                  int rc, typename Cfg::Real scl, typename Cfg::Real* out)
    {
        using Real = typename Cfg::Real;
        constexpr int SD = DirStride<Cfg, D>::S;
        const int cl = rc - SD, cr = rc;
        const Real pl = V.q(0, cl), Tl = V.q(1, cl), ul = V.q(2, cl), vl = V.q(3, cl), wl = V.q(4, cl);
        const Real pr = V.q(0, cr), Tr = V.q(1, cr), ur = V.q(2, cr), vr = V.q(3, cr), wr = V.q(4, cr);
        const Real delta_p = pl - pr;
        const Real delta_T = Tl - Tr;
        const Real pavg = ppow2<Cfg, -1>(pl + pr);
        const Real Tavg = ppow2<Cfg, -1>(Tl + Tr);
        const Real inv_RT = pdiv<Cfg::IDIV>(Real(1.0), pmul<Cfg>(S.R_avg, Tavg));
        const Real p_inv_rt2 = pdiv<Cfg::IDIV>(pmul<Cfg>(pavg, inv_RT), Tavg);
        const Real k = ppow2<Cfg, -1>(pmul<Cfg>(ul, ur) + pmul<Cfg>(vl, vr) + pmul<Cfg>(wl, wr));
        const Real u = ppow2<Cfg, -1>(ul + ur);
        const Real v = ppow2<Cfg, -1>(vl + vr);
        const Real w = ppow2<Cfg, -1>(wl + wr);
        const Real ap = pmul<Cfg>(pmul<Cfg>(scl, S.eps_p), delta_p);
        const Real aT = pmul<Cfg>(pmul<Cfg>(pmul<Cfg>(scl, S.eps_T), delta_T), p_inv_rt2);
        out[0] = pmul<Cfg>(ap, inv_RT);
        out[1] = pmul<Cfg>(ap, pmul<Cfg>(k, inv_RT) + S.inv_gamma_avg);
        out[2] = pmul<Cfg>(pmul<Cfg>(ap, u), inv_RT);
        out[3] = pmul<Cfg>(pmul<Cfg>(ap, v), inv_RT);
        out[4] = pmul<Cfg>(pmul<Cfg>(ap, w), inv_RT);
        out[0] -= aT;
        out[1] -= pmul<Cfg>(aT, ppow2<Cfg, -1>(k));
        out[2] -= pmul<Cfg>(aT, u);
        out[3] -= pmul<Cfg>(aT, v);
        out[4] -= pmul<Cfg>(aT, w);
    }

    // info::gradient at the face (info_gradient.h:61-123): grad[a][t],
    // a = direction, t = 0:T 1:u 2:v 3:w (the pressure gradient is unused).
    template <class Cfg, int D>
    __device__ __forceinline__ void face_gradient(const BoxView<Cfg>& V, int rc,
                                                  const typename Cfg::Real inv[3], typename Cfg::Real im,
                                                  typename Cfg::Real (&grad)[3][4])
    {
        using Real = typename Cfg::Real;
        constexpr int SD = DirStride<Cfg, D>::S, S1 = DirStride<Cfg, D>::S1, S2 = DirStride<Cfg, D>::S2;
        constexpr int D1 = (D + 1) % 3, D2 = (D + 2) % 3;
        const int cl = rc - SD, cr = rc;
        #pragma unroll
        for (int t = 0; t < 4; ++t)
        {
            const int v = t + 1;
            // (c*q)*inv with c = -1, 1, 0.25, -0.25: the +-1 products are exact
            // sign changes, the +-0.25 ones exact exponent shifts
            grad[D][t]  = pmul<Cfg>(-V.q(v, cl), inv[D]);
            grad[D1][t] = pmul<Cfg>(ppow2<Cfg, -2>(V.q(v, cl + S1)), inv[D1]);
            grad[D1][t] += pmul<Cfg>(-ppow2<Cfg, -2>(V.q(v, cl - S1)), inv[D1]);
            grad[D2][t] = pmul<Cfg>(ppow2<Cfg, -2>(V.q(v, cl + S2)), inv[D2]);
            grad[D2][t] += pmul<Cfg>(-ppow2<Cfg, -2>(V.q(v, cl - S2)), inv[D2]);
            grad[D][t]  += pmul<Cfg>(V.q(v, cr), inv[D]);
            grad[D1][t] += pmul<Cfg>(ppow2<Cfg, -2>(V.q(v, cr + S1)), inv[D1]);
            grad[D1][t] += pmul<Cfg>(-ppow2<Cfg, -2>(V.q(v, cr - S1)), inv[D1]);
            grad[D2][t] += pmul<Cfg>(ppow2<Cfg, -2>(V.q(v, cr + S2)), inv[D2]);
            grad[D2][t] += pmul<Cfg>(-ppow2<Cfg, -2>(V.q(v, cr - S2)), inv[D2]);
            if constexpr (Cfg::STRETCH) grad[1][t] = pmul<Cfg>(grad[1][t], im);
        }
    }

    // state_sensor::ducros_t::get_sensor (state_sensor.h:21-43)
    template <class Real, bool IM = false>
    __device__ __forceinline__ Real ducros_sensor(const Real (&g)[3][4], Real epsilon)
    {
        Real theta_sq = g[0][1] + g[1][2] + g[2][3];
        theta_sq *= theta_sq;
        const Real vort0 = g[1][3] - g[2][2];
        const Real vort1 = g[2][1] - g[0][3];
        const Real vort2 = g[0][2] - g[1][1];
        const Real vort_sq = vort0*vort0 + vort1*vort1 + vort2*vort2;
        return pdiv<IM>(theta_sq, theta_sq + vort_sq + epsilon);
    }

    // visc_lr::operator() (viscous.h:39-79) with info::value / info::gradient
    // at the face (info_value.h:28-40, info_gradient.h:61-123).
    template <class Cfg, int D>
    __device__ __forceinline__ void visc_lr(const BoxView<Cfg>& V, const SchemeR<typename Cfg::Real>& S,
                                            int rc, typename Cfg::Real nD,
                                            const typename Cfg::Real (&grad)[3][4],
                                            typename Cfg::Real* out)
    {
        using Real = typename Cfg::Real;
        constexpr int SD = DirStride<Cfg, D>::S;
        const int cl = rc - SD, cr = rc;
        Real qf[5];
        #pragma unroll
        for (int v = 0; v < 5; ++v) { qf[v] = V.q(v, cl); qf[v] += V.q(v, cr); qf[v] = ppow2<Cfg, -1>(qf[v]); }
        Real visc, visc2, dfs;
        if (S.law == GBNS_LAW_CONSTANT)
        {
            visc = S.mu; visc2 = S.beta_c; dfs = S.alpha_c;
        }
        else if (S.law == GBNS_LAW_POWER)
        {
            visc = pmul<Cfg>(S.mu, dev_pow(pdiv<Cfg::IDIV>(qf[1], S.T_ref), S.power));
            visc2 = pmul<Cfg>(Real(-0.66666666667), visc);
            dfs = pdiv<Cfg::IDIV>(visc, S.prandtl);
        }
        else
        {
            const Real x = pdiv<Cfg::IDIV>(qf[1], S.T_ref);
            visc = pmul<Cfg>(pmul<Cfg>(S.mu, pmul<Cfg>(x, dev_sqrt<Cfg::IDIV>(x))), pdiv<Cfg::IDIV>(S.tref_plus_s, qf[1] + S.S));
            visc2 = pmul<Cfg>(visc, Real(-2.0/3.0));
            dfs = pmul<Cfg>(visc, S.inv_pr);
        }
        const Real div = grad[0][1] + grad[1][2] + grad[2][3];
        const Real t00 = pmul<Cfg>(visc, grad[0][1] + grad[0][1]) + pmul<Cfg>(visc2, div);
        const Real t01 = pmul<Cfg>(visc, grad[0][2] + grad[1][1]);
        const Real t02 = pmul<Cfg>(visc, grad[0][3] + grad[2][1]);
        const Real t12 = pmul<Cfg>(visc, grad[1][3] + grad[2][2]);
        const Real t11 = pmul<Cfg>(visc, grad[1][2] + grad[1][2]) + pmul<Cfg>(visc2, div);
        const Real t22 = pmul<Cfg>(visc, grad[2][3] + grad[2][3]) + pmul<Cfg>(visc2, div);
        const Real cond = pmul<Cfg>(S.spec_heat, dfs);
        // only row D of tau and component D of the heat flux survive n = nD e_D
        Real tr0, tr1, tr2;
        if constexpr (D == 0) { tr0 = t00; tr1 = t01; tr2 = t02; }
        else if constexpr (D == 1) { tr0 = t01; tr1 = t11; tr2 = t12; }
        else { tr0 = t02; tr1 = t12; tr2 = t22; }
        const Real ht = pmul<Cfg>(qf[2], tr0) + pmul<Cfg>(qf[3], tr1) + pmul<Cfg>(qf[4], tr2) + pmul<Cfg>(cond, grad[D][0]);
        out[0] = Real(0.0);
        out[1] = -nmul<Cfg>(nD, ht);
        out[2] = -nmul<Cfg>(nD, tr0);
        out[3] = -nmul<Cfg>(nD, tr1);
        out[4] = -nmul<Cfg>(nD, tr2);
    }

    // Composite face flux conv + (diss + visc)  (omni/compose.h:19-24)
    template <class Cfg, int D>
    __device__ __forceinline__ void face_flux(const BoxView<Cfg>& V, const SchemeR<typename Cfg::Real>& S,
                                              int rc, int lr, typename Cfg::Real nD,
                                              const typename Cfg::Real inv[3], typename Cfg::Real im,
                                              typename Cfg::Real* F)
    {
        using Real = typename Cfg::Real;
        // terms in fixed registers (no pointer selection: keeps them out of
        // local memory); summed conv + (diss + visc) like compose
        Real t0[5], t1[5], t2[5];
        Real grad[3][4];
        bool have_grad = false;
        const bool hd = S.diss != 0, hv = S.visc != 0;
        const bool ducros = hd && S.sensor == GBNS_SENSOR_DUCROS;
        if constexpr (Cfg::CONV == GBNS_CONV_HYBRID)
        {
            // hybrid_scheme_t::operator() (hybrid_scheme.h:30-46): the blender
            // at the face, then (1 - s) F_centred + s F_fweno (full_flux) or
            // F_centred + s F_fweno (diss_flux).  The face gradient, when the
            // blender needs it, is kept for dissipation and viscous terms.
            Real blend = S.hyb_param;
            if (S.hyb_sensor == GBNS_SENSOR_DUCROS)
            {
                face_gradient<Cfg, D>(V, rc, inv, im, grad);
                have_grad = true;
                blend = ducros_sensor<Real, Cfg::IDIV>(grad, S.hyb_param);
            }
            conv_cent_keep<Cfg, D>(V, S, rc, nD, t0);
            conv_fweno<Cfg, D>(V, S, rc, lr, nD, t1);
            const Real c0 = S.hyb_flux == GBNS_HYBRID_DISS_FLUX ? Real(1.0) : Real(1.0) - blend;
            #pragma unroll
            for (int v = 0; v < 5; ++v)
            {
                t0[v] = pmul<Cfg>(t0[v], c0);
                t1[v] = pmul<Cfg>(t1[v], blend);
                t0[v] += t1[v];
            }
        }
        else if constexpr (Cfg::CONV == GBNS_CONV_CENT_KEEP) conv_cent_keep<Cfg, D>(V, S, rc, nD, t0);
        else if constexpr (Cfg::CONV == GBNS_CONV_TOTANI) conv_totani<Cfg, D>(V, S, rc, nD, t0);
        else if constexpr (Cfg::CONV == GBNS_CONV_FWENO) conv_fweno<Cfg, D>(V, S, rc, lr, nD, t0);
        else if constexpr (Cfg::CONV == GBNS_CONV_WENO5) conv_weno5<Cfg, D>(V, S, rc, lr, nD, t0);
        // const_sensor_t dissipation runs before the gradient is formed, so
        // the gradient is not live across it; ducros_t needs the gradient first.
        if (hd && !ducros) diss_pressure<Cfg, D>(V, S, rc, S.sens, t1);
        if ((hv || ducros) && !have_grad) face_gradient<Cfg, D>(V, rc, inv, im, grad);
        if (ducros) diss_pressure<Cfg, D>(V, S, rc, ducros_sensor<Real, Cfg::IDIV>(grad, S.sens), t1);
        if (hv) visc_lr<Cfg, D>(V, S, rc, nD, grad, t2);
        #pragma unroll
        for (int v = 0; v < 5; ++v)
        {
            if constexpr (Cfg::CONV == GBNS_CONV_NONE)
                F[v] = (hd && hv) ? t1[v] + t2[v] : (hd ? t1[v] : (hv ? t2[v] : Real(0)));
            else
                F[v] = (hd && hv) ? t0[v] + (t1[v] + t2[v]) : (hd ? t0[v] + t1[v] : (hv ? t0[v] + t2[v] : t0[v]));
        }
    }

    // ------------------------------------------------------------------
    // the kernel
    // ------------------------------------------------------------------
    struct FluxArgs
    {
        const double* prims;
        double* rhs;
        int increment;
        int ntile[3];       // tiles per block per direction
        int use_tma;
        int sh_off;         // FP32 copy: column of padded index 0 (ShadowK::off)
        // Fused RK stage (0 = none): q_out = prim(cons(q) + sum_j rk_coeff[j] R_j)
        // for the tile's cells, with R_{rk_nres-1} this launch's residual (in
        // registers) and R_0..R_{rk_nres-2} read from rk_res.
        int rk_nres;
        int write_rhs;      // with a fused stage: also store this launch's residual
        const double* rk_res[2];
        double rk_coeff[3];
        double* q_out;
        // Refined layouts: 1/dx of every block (3 per block, device memory);
        // nullptr: the uniform layout's table in GeomK
        const double* blk_inv_dx;
    };

    // One face of direction D (tile-local face index f) into the face buffer
    // at column `base + f` (row v of stride Cfg::NFS).
    template <class Cfg, int D>
    __device__ __forceinline__ void face_one(const BoxView<Cfg>& V, const SchemeR<typename Cfg::Real>& S,
                                             double* sF, int base, int f, const GeomK& G, const YTabT<Cfg::STRETCH>& Y,
                                             const int b[3], int i0, int j0, int k0, int shift,
                                             const typename Cfg::Real inv[3])
    {
        using Real = typename Cfg::Real;
        constexpr int TX = Cfg::TX, TY = Cfg::TY, H = Cfg::H;
        constexpr int EX = TX + (D == 0), EY = TY + (D == 1);
        const int ny = G.n[1];
        const int fx = f % EX;
        const int r = f / EX;
        const int fy = r % EY;
        const int fz = r / EY;
        const int gi = i0 + fx, gj = j0 + fy, gk = k0 + fz;
        const bool valid = (D == 0 ? gi <= G.n[0] : gi < G.n[0]) &&
                           (D == 1 ? gj <= G.n[1] : gj < G.n[1]) &&
                           (D == 2 ? gk <= G.n[2] : gk < G.n[2]);
        Real F[5] = {Real(0), Real(0), Real(0), Real(0), Real(0)};
        if (valid)
        {
            const int rc = (fz + H)*Cfg::SZ + (fy + H)*Cfg::SY + (fx + H + shift);
            Real nD = Real(1.0), im = Real(1.0);
            if constexpr (Cfg::STRETCH)
            {
                if constexpr (!Cfg::FP64)
                {
                    if constexpr (D == 1) im = V.ymet[2*(TY + 1) + fy];
                    else
                    {
                        nD = V.ymet[fy];
                        im = V.ymet[(TY + 1) + fy];
                    }
                }
                else if constexpr (D == 1) im = Real(Y.im_face[b[1]*(ny + 1) + gj]);
                else
                {
                    nD = Real(Y.m_cell[b[1]*ny + gj]);
                    im = Real(Y.im_cell[b[1]*ny + gj]);
                }
            }
            face_flux<Cfg, D>(V, S, rc, SplitIdx<Cfg, D>::right(fx, fy, fz), nD, inv, im, F);
        }
        // FP32 fluxes widen exactly on the integer pipes (f2d_int), which
        // keeps the FP64 pipe for the accumulation
        #pragma unroll
        for (int v = 0; v < 5; ++v)
        {
            if constexpr (Cfg::FP64) sF[v*Cfg::NFS + base + f] = F[v];
            else sF[v*Cfg::NFS + base + f] = f2d_int(F[v]);
        }
    }

    // Divergence of direction D into the cells this thread owns, in the
    // reference's order (flux_div_basic.h:109-129): relem += F(i-1/2)*(jac*1*inv_dx);
    // relem += F(i+1/2)*(jac*(-1)*inv_dx).
    template <class Cfg, int D>
    __device__ __forceinline__ void face_accumulate(const double* sF, int base, const GeomK& G,
                                                    const YTabT<Cfg::STRETCH>& Y, const int b[3], int i0, int j0,
                                                    int k0, double (&relem)[Cfg::CPT][5], const double invd[3])
    {
        constexpr int TX = Cfg::TX, TY = Cfg::TY;
        const int ny = G.n[1];
        #pragma unroll
        for (int s = 0; s < Cfg::CPT; ++s)
        {
            const int c = threadIdx.x + s*Cfg::NT;
            if (c >= Cfg::NCELL) break;
            const int cx = c % TX, cy = (c / TX) % TY, cz = c / (TX*TY);
            if (i0 + cx >= G.n[0] || j0 + cy >= G.n[1] || k0 + cz >= G.n[2]) continue;
            int fL, fR;
            if constexpr (D == 0) { fL = cx + (TX + 1)*(cy + TY*cz); fR = fL + 1; }
            else if constexpr (D == 1) { fL = cx + TX*(cy + (TY + 1)*cz); fR = fL + TX; }
            else { fL = cx + TX*(cy + TY*cz); fR = fL + TX*TY; }
            double jac = 1.0;
            if constexpr (Cfg::STRETCH) jac = Y.im_cell[b[1]*ny + j0 + cy];
            // (jac*(-1.0))*invd rounds to exactly -(jac*invd): RN is symmetric;
            // the products on the integer pipes in the IMUL tiles (same bits)
            if constexpr (Cfg::IMUL)
            {
                const double multL = dmul_int(jac, invd[D]);
                const double multR = -multL;
                #pragma unroll
                for (int v = 0; v < 5; ++v)
                {
                    relem[s][v] += dmul_int(sF[v*Cfg::NFS + base + fL], multL);
                    relem[s][v] += dmul_int(sF[v*Cfg::NFS + base + fR], multR);
                }
            }
            else
            {
                const double multL = (jac*1.0)*invd[D];
                const double multR = -multL;
                #pragma unroll
                for (int v = 0; v < 5; ++v)
                {
                    relem[s][v] += sF[v*Cfg::NFS + base + fL]*multL;
                    relem[s][v] += sF[v*Cfg::NFS + base + fR]*multR;
                }
            }
        }
    }

    // One direction: [split cache], its faces, then its share of the divergence.
    template <class Cfg, int D>
    __device__ __forceinline__ void face_pass(const BoxView<Cfg>& V, const SchemeR<typename Cfg::Real>& S,
                                              double* sF, const GeomK& G, const YTabT<Cfg::STRETCH>& Y,
                                              int lb, const int b[3], int i0, int j0, int k0, int shift,
                                              const typename Cfg::Real inv[3],
                                              double (&relem)[Cfg::CPT][5], const double invd[3],
                                              const double (&dc)[Cfg::CPT][3])
    {
        constexpr int NF = D == 0 ? Cfg::NF0 : (D == 1 ? Cfg::NF1 : Cfg::NF2);
        if constexpr (Cfg::SPLIT)
        {
            split_fill<Cfg, D>(V, S, const_cast<double*>(V.split), Y, b[1], j0, G.n[1], shift, dc);
            __syncthreads();
        }
        for (int f = threadIdx.x; f < NF; f += Cfg::NT)
            face_one<Cfg, D>(V, S, sF, 0, f, G, Y, b, i0, j0, k0, shift, inv);
        __syncthreads();
        face_accumulate<Cfg, D>(sF, 0, G, Y, b, i0, j0, k0, relem, invd);
        __syncthreads();
    }

    // All three directions' faces in one balanced loop (faces of one
    // direction are contiguous, and NF0, NF0 + NF1 are multiples of the warp
    // size for the merged shapes, so no warp mixes directions), then the
    // divergence direction by direction in the same order as face_pass.
    template <class Cfg>
    __device__ __forceinline__ void face_pass_merged(const BoxView<Cfg>& V, const SchemeR<typename Cfg::Real>& S,
                                                     double* sF, const GeomK& G, const YTabT<Cfg::STRETCH>& Y,
                                                     const int b[3], int i0, int j0, int k0, int shift,
                                                     const typename Cfg::Real inv[3],
                                                     double (&relem)[Cfg::CPT][5], const double invd[3])
    {
        constexpr int N01 = Cfg::NF0 + Cfg::NF1, NALL = N01 + Cfg::NF2;
        for (int f = threadIdx.x; f < NALL; f += Cfg::NT)
        {
            if (f < Cfg::NF0) face_one<Cfg, 0>(V, S, sF, 0, f, G, Y, b, i0, j0, k0, shift, inv);
            else if (f < N01) face_one<Cfg, 1>(V, S, sF, Cfg::NF0, f - Cfg::NF0, G, Y, b, i0, j0, k0, shift, inv);
            else face_one<Cfg, 2>(V, S, sF, N01, f - N01, G, Y, b, i0, j0, k0, shift, inv);
        }
        __syncthreads();
        face_accumulate<Cfg, 0>(sF, 0, G, Y, b, i0, j0, k0, relem, invd);
        face_accumulate<Cfg, 1>(sF, Cfg::NF0, G, Y, b, i0, j0, k0, relem, invd);
        face_accumulate<Cfg, 2>(sF, N01, G, Y, b, i0, j0, k0, relem, invd);
        __syncthreads();
    }

    // One tile of one block: the whole per-CTA algorithm.  Called by the
    // per-grid kernel (one CTA per tile) and by the persistent batch kernel
    // (CTAs loop over a work-list of tiles of many grids).
    // Ssh (persistent batch kernel): the scheme constants already unpacked
    // into shared memory, read from there at each use instead of being held
    // in registers for the whole tile (the single-grid kernel reads them from
    // its parameters, which cost no registers).
    template <class Cfg>
    __device__ __forceinline__ void flux_tile(unsigned char* smem_raw, const CUtensorMap* tmap, const GeomK& G,
                                              const YTabT<Cfg::STRETCH>& Y, const SchemeK& SK, const FluxArgs& A,
                                              const int lb, const int tile,
                                              const SchemeR<typename Cfg::Real>* Ssh = nullptr)
    {
        using Real = typename Cfg::Real;
        constexpr int TX = Cfg::TX, TY = Cfg::TY, TZ = Cfg::TZ, H = Cfg::H;
        uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
        double* stage = reinterpret_cast<double*>(smem_raw + 128);
        float* soa = reinterpret_cast<float*>(smem_raw + 128 + Cfg::STAGE_BYTES);
        unsigned char* tail = smem_raw + 128 + Cfg::STAGE_BYTES + Cfg::SOA_BYTES;
        Real* der = Cfg::REUSE ? reinterpret_cast<Real*>(stage) : reinterpret_cast<Real*>(tail);
        double* sF = Cfg::REUSE ? reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(stage) + Cfg::DER_BYTES)
                                : reinterpret_cast<double*>(tail + Cfg::DER_BYTES);

        const int tid = threadIdx.x;
        const int tx = tile % A.ntile[0];
        const int ty = (tile / A.ntile[0]) % A.ntile[1];
        const int tz = tile / (A.ntile[0]*A.ntile[1]);
        const int i0 = tx*TX, j0 = ty*TY, k0 = tz*TZ;
        const int b[3] = {lb % G.nb[0], (lb / G.nb[0]) % G.nb[1], lb / (G.nb[0]*G.nb[1])};
        const int px = i0 - H + G.ng;
        const int xs = px & ~1;
        const int shift = Cfg::SHADOW ? 0 : px - xs;
        const int ys = j0 - H + G.ng, zs = k0 - H + G.ng;

        // ---- stage the tile + halo --------------------------------------
        if constexpr (Cfg::SHADOW)
        {
            // the box's five SoA planes in one tensor copy; its x start
            // px + sh_off is a multiple of 4 floats by the copy's layout
            if (tid == 0) mbar_init(bar, 1);
            __syncthreads();
            if (tid == 0)
            {
                mbar_expect_tx(bar, uint32_t(Cfg::BOXN)*5u*4u);
                tma_load_4d(soa, tmap, bar, px + A.sh_off, ys, zs, 5*lb);
            }
            const bool ok = mbar_wait(bar, 0, MBAR_WAIT_CYCLES);
            if (__syncthreads_or(!ok))
            {
                if (tid == 0) atomicExch(&g_device_status, DEV_TMA_TIMEOUT);
                return;
            }
        }
        else if constexpr (Cfg::DIRECT)
        {
            // Only the cells some face reads: the tile, the stencil cross of
            // radius max(HC, 1), and the edge cells one step out in two
            // directions (transverse neighbours of the viscous gradient).
            constexpr int R1 = Cfg::HC > 1 ? Cfg::HC : 1;
            const double* base = A.prims + (long long)lb*G.bstride;
            for (int c = tid; c < Cfg::BOXN; c += Cfg::NT)
            {
                const int bx = c % Cfg::BXE, by = (c / Cfg::BXE) % Cfg::BY, bz = c / (Cfg::BXE*Cfg::BY);
                const int rx = bx - shift - H, ry = by - H, rz = bz - H;
                const int ox = rx < 0 ? -rx : (rx >= TX ? rx - TX + 1 : 0);
                const int oy = ry < 0 ? -ry : (ry >= TY ? ry - TY + 1 : 0);
                const int oz = rz < 0 ? -rz : (rz >= TZ ? rz - TZ + 1 : 0);
                const int nout = (ox > 0) + (oy > 0) + (oz > 0);
                const int omax = ox > oy ? (ox > oz ? ox : oz) : (oy > oz ? oy : oz);
                const bool need = nout == 0 || (nout == 1 && omax <= R1) || (nout == 2 && omax == 1);
                if (!need) continue;
                const int X = xs + bx, Y_ = ys + by, Z = zs + bz;
                if (X < G.ni && Y_ < G.nj && Z < G.nk)
                {
                    const double* src = base + ((long long)(Z*G.nj + Y_)*G.ni + X)*5;
                    #pragma unroll
                    for (int v = 0; v < 5; ++v) soa[v*Cfg::BOXN + c] = float(__ldg(src + v));
                }
                else
                {
                    #pragma unroll
                    for (int v = 0; v < 5; ++v) soa[v*Cfg::BOXN + c] = 0.0f;
                }
            }
        }
        else if (A.use_tma)
        {
            if (tid == 0) mbar_init(bar, 1);
            __syncthreads();
            if (tid == 0)
            {
                mbar_expect_tx(bar, uint32_t(Cfg::BOXN)*5u*8u);
                tma_load_4d(stage, tmap, bar, xs*5, ys, zs, lb);
            }
            const bool ok = mbar_wait(bar, 0, MBAR_WAIT_CYCLES);
            if (__syncthreads_or(!ok))
            {
                if (tid == 0) atomicExch(&g_device_status, DEV_TMA_TIMEOUT);
                return;
            }
        }
        else
        {
            const double* base = A.prims + (long long)lb*G.bstride;
            const int rowlen = Cfg::BXE*5;
            for (int e = tid; e < Cfg::BOXN*5; e += Cfg::NT)
            {
                const int row = e / rowlen, col = e - row*rowlen;
                const int yy = row % Cfg::BY, zz = row / Cfg::BY;
                const int X = xs + col/5, Y_ = ys + yy, Z = zs + zz;
                double val = 0.0;
                if (X < G.ni && Y_ < G.nj && Z < G.nk)
                    val = __ldg(base + ((long long)(Z*G.nj + Y_)*G.ni + xs)*5 + col);
                stage[e] = val;
            }
        }
        // initial residual (increment mode reads it)
        double relem[Cfg::CPT][5];
        #pragma unroll
        for (int s = 0; s < Cfg::CPT; ++s)
        {
            #pragma unroll
            for (int v = 0; v < 5; ++v) relem[s][v] = 0.0;
            const int c = tid + s*Cfg::NT;
            if (A.increment && c < Cfg::NCELL)
            {
                const int cx = c % TX, cy = (c / TX) % TY, cz = c / (TX*TY);
                if (i0 + cx < G.n[0] && j0 + cy < G.n[1] && k0 + cz < G.n[2])
                {
                    const double* r = A.rhs + (long long)lb*G.bstride +
                        ((long long)((k0 + cz + G.ng)*G.nj + (j0 + cy + G.ng))*G.ni + (i0 + cx + G.ng))*5;
                    #pragma unroll
                    for (int v = 0; v < 5; ++v) relem[s][v] = r[v];
                }
            }
        }
        float* ymet = reinterpret_cast<float*>(smem_raw + Cfg::YM_OFF);
        if constexpr (!Cfg::FP64 && Cfg::STRETCH)
        {
            const int ny = G.n[1];
            for (int j = tid; j < TY + 1; j += Cfg::NT)
            {
                const int gj = j0 + j;
                ymet[j] = gj < ny ? float(Y.m_cell[b[1]*ny + gj]) : 0.0f;
                ymet[(TY + 1) + j] = gj < ny ? float(Y.im_cell[b[1]*ny + gj]) : 0.0f;
                ymet[2*(TY + 1) + j] = gj <= ny ? float(Y.im_face[b[1]*(ny + 1) + gj]) : 0.0f;
            }
        }
        __syncthreads();

        // ---- FP32 staged: convert the box to SoA floats -------------------
        if constexpr (!Cfg::FP64 && !Cfg::DIRECT && !Cfg::SHADOW)
        {
            for (int c = tid; c < Cfg::BOXN; c += Cfg::NT)
            {
                #pragma unroll
                for (int v = 0; v < 5; ++v) soa[v*Cfg::BOXN + c] = float(stage[c*5 + v]);
            }
            __syncthreads();
        }

        BoxView<Cfg> V;
        V.stage = stage;
        V.soa = soa;
        V.split = reinterpret_cast<const double*>(der);
        V.ymet = ymet;
        if constexpr (Cfg::SPLIT)
            der = reinterpret_cast<Real*>(reinterpret_cast<unsigned char*>(der) + Cfg::SPLIT_BYTES);
        V.der = der;
        SchemeR<Real> S_own;
        if (!Ssh) S_own.load(SK);
        const SchemeR<Real>& S = Ssh ? *Ssh : S_own;

        // ---- per-cell derived values on the stencil cross -------------------
        if constexpr (Cfg::NDERB > 0)
        {
            constexpr int HC = Cfg::HC;
            for (int c = tid; c < Cfg::BOXN; c += Cfg::NT)
            {
                const int bx = c % Cfg::BXE, by = (c / Cfg::BXE) % Cfg::BY, bz = c / (Cfg::BXE*Cfg::BY);
                const int rx = bx - shift - H, ry = by - H, rz = bz - H;
                const bool inx = rx >= 0 && rx < TX, iny = ry >= 0 && ry < TY, inz = rz >= 0 && rz < TZ;
                const bool need = (iny && inz && rx >= -HC && rx < TX + HC) ||
                                  (inx && inz && ry >= -HC && ry < TY + HC) ||
                                  (inx && iny && rz >= -HC && rz < TZ + HC);
                if (need) derive_cell<Cfg>(V, der, S, c);
            }
            __syncthreads();
        }

        double invd[3];
        Real inv[3];
        #pragma unroll
        for (int d = 0; d < 3; ++d)
        {
            invd[d] = A.blk_inv_dx ? A.blk_inv_dx[3*lb + d] : G.inv_dx[d][b[d]];
            if constexpr (sizeof(Real) == 4) inv[d] = A.blk_inv_dx ? float(invd[d]) : G.inv_dx_f[d][b[d]];
            else inv[d] = invd[d];
        }

        // SPLIT: rho, h, e of the cells this thread owns, shared by the three
        // directions' split fills
        double dc[Cfg::CPT][3];
        #pragma unroll
        for (int s = 0; s < Cfg::CPT; ++s) { dc[s][0] = dc[s][1] = dc[s][2] = 0.0; }
        if constexpr (Cfg::SPLIT)
        {
            #pragma unroll
            for (int s = 0; s < Cfg::CPT; ++s)
            {
                const int cc = tid + s*Cfg::NT;
                if (cc >= Cfg::NCELL) break;
                const int cx = cc % TX, cy = (cc / TX) % TY, cz = cc / (TX*TY);
                const int c = (cz + H)*Cfg::SZ + (cy + H)*Cfg::SY + (cx + H + shift);
                fweno_derive<double, Cfg::IDIV, Cfg::IMUL>(S, V.q(0, c), V.q(1, c), V.q(2, c), V.q(3, c), V.q(4, c), dc[s][0], dc[s][1], dc[s][2]);
            }
        }

        if constexpr (Cfg::MERGED)
        {
            face_pass_merged<Cfg>(V, S, sF, G, Y, b, i0, j0, k0, shift, inv, relem, invd);
        }
        else
        {
            face_pass<Cfg, 0>(V, S, sF, G, Y, lb, b, i0, j0, k0, shift, inv, relem, invd, dc);
            face_pass<Cfg, 1>(V, S, sF, G, Y, lb, b, i0, j0, k0, shift, inv, relem, invd, dc);
            face_pass<Cfg, 2>(V, S, sF, G, Y, lb, b, i0, j0, k0, shift, inv, relem, invd, dc);
        }

        // ---- write the residual (and the fused stage update) -----------------
        #pragma unroll
        for (int s = 0; s < Cfg::CPT; ++s)
        {
            const int c = tid + s*Cfg::NT;
            if (c >= Cfg::NCELL) break;
            const int cx = c % TX, cy = (c / TX) % TY, cz = c / (TX*TY);
            if (i0 + cx >= G.n[0] || j0 + cy >= G.n[1] || k0 + cz >= G.n[2]) continue;
            const long long off = (long long)lb*G.bstride +
                ((long long)((k0 + cz + G.ng)*G.nj + (j0 + cy + G.ng))*G.ni + (i0 + cx + G.ng))*5;
            if (A.rk_nres == 0 || A.write_rhs)
            {
                double* r = A.rhs + off;
                #pragma unroll
                for (int v = 0; v < 5; ++v) r[v] = relem[s][v];
            }
            if (A.rk_nres)
            {
                // transform_advance_to for this cell (advance.h:75-101)
                double qv[5];
                if constexpr (Cfg::FP64)
                {
                    const int bc_ = (cz + H)*Cfg::SZ + (cy + H)*Cfg::SY + (cx + H + shift);
                    #pragma unroll
                    for (int v = 0; v < 5; ++v) qv[v] = stage[bc_*5 + v];
                }
                else
                {
                    #pragma unroll
                    for (int v = 0; v < 5; ++v) qv[v] = __ldg(A.prims + off + v);
                }
                double cs[5];
                if constexpr (Cfg::FP64) prim_to_cons<Cfg::IMUL, Cfg::IDIV>(qv, SK.R, SK.gm1, cs);
                else prim_to_cons_fast<true>(qv, SK.R, SK.inv_gm1, cs);
                for (int j = 0; j + 1 < A.rk_nres; ++j)
                {
                    const double* rr = A.rk_res[j] + off;
                    #pragma unroll
                    for (int v = 0; v < 5; ++v) cs[v] += pmul64<Cfg::IMUL>(A.rk_coeff[j], rr[v]);
                }
                const double cl = A.rk_coeff[A.rk_nres - 1];
                #pragma unroll
                for (int v = 0; v < 5; ++v) cs[v] += pmul64<Cfg::IMUL>(cl, relem[s][v]);
                double qn[5];
                if constexpr (Cfg::FP64) cons_to_prim<Cfg::IMUL, Cfg::IDIV>(cs, SK.R, SK.gm1, qn);
                else cons_to_prim_fast<true>(cs, SK.inv_R, SK.gm1, qn);
                double* o = A.q_out + off;
                #pragma unroll
                for (int v = 0; v < 5; ++v) o[v] = qn[v];
            }
        }
        if (!Cfg::DIRECT && A.use_tma && tid == 0) mbar_inval(bar);
    }

    template <class Cfg>
    __global__ void __launch_bounds__(Cfg::NT, Cfg::MINB)
    flux_div_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ GeomK G,
                    const __grid_constant__ YTabT<Cfg::STRETCH> Y, const __grid_constant__ SchemeK SK, const FluxArgs A,
                    const int blk0)
    {
        // blockIdx.y: the block within the launch's range blk0 .. blk0 + gridDim.y - 1
        extern __shared__ __align__(128) unsigned char smem_raw[];
        flux_tile<Cfg>(smem_raw, &tmap, G, Y, SK, A, int(blockIdx.y) + blk0, int(blockIdx.x));
    }
}
