// IEEE 754 binary64 multiplication, division and square root, and the
// FP32<->FP64 conversions, computed on the integer pipes.
//
// GB300 executes FP64 at 1/64 of its FP32 rate (two FP64 lanes per SM and
// clock) while its integer multiply-add and logic pipes are mostly idle in the
// flux kernel. dmul_int returns exactly the bits of the hardware multiply
// (round to nearest, ties to even) and leaves the FP64 pipe free, so the FP64
// kernels send part of their products here and the rest to the FP64 unit.
//
// Method: the textbook software binary multiplication (Muller et al.,
// "Handbook of Floating-Point Arithmetic", 2nd ed., 2018) — multiply the two
// 53-bit significands exactly (a 106-bit product from 64x64-bit integer
// multiplies), normalise by at most one bit, round to nearest even with a
// round bit and a sticky bit, and add the biased exponent so that a carry out
// of the significand rounding increments the exponent (overflow to infinity
// comes out of the same addition). Zero, subnormal, infinite and NaN operands,
// and products whose exponent leaves the normal range, go to the hardware
// multiply, so the function is exact for every input.
#pragma once
#include <cstdint>

namespace gbns
{
    // The hardware operations the integer routines below fall back to for
    // special operands (zeros, subnormals, infinities, NaNs, results outside
    // the normal range), as calls the compiler cannot if-convert.  Inlined,
    // the fallback became an FP64 instruction predicated off in the lanes that
    // do not need it, which every warp still issues to the FP64 unit (about a
    // fifth of that unit's issue in the integer-pipe tiles, measured); as a
    // call it sits behind a branch that warps with no special lane skip.
    static __device__ __noinline__ double dmul_hw(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __noinline__ double ddiv_hw(double a, double b) { return a/b; }
    static __device__ __noinline__ double dsqrt_hw(double x) { return __dsqrt_rn(x); }
    static __device__ __noinline__ double dscale_hw(double x, double c) { return x*c; }
    static __device__ __noinline__ float d2f_hw(double x) { return __double2float_rn(x); }

    __device__ __forceinline__ double dmul_int(double a, double b)
    {
        constexpr uint64_t M52 = 0x000FFFFFFFFFFFFFull, H53 = 0x0010000000000000ull, SGN = 0x8000000000000000ull;
        const uint64_t ua = (uint64_t)__double_as_longlong(a), ub = (uint64_t)__double_as_longlong(b);
        const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
        // biased exponent of the product when the significand product is in [1, 2)
        int e = (int)ea + (int)eb - 1023;
        if (ea - 1u >= 2046u || eb - 1u >= 2046u || (unsigned)(e - 1) >= 2045u) return dmul_hw(a, b);
        // significands with the hidden bit at bit 63: the product is in [2^126, 2^128)
        const uint64_t ma = ((ua & M52) | H53) << 11, mb = ((ub & M52) | H53) << 11;
        uint64_t hi = __umul64hi(ma, mb);
        uint64_t lo = ma*mb;
        const uint32_t top = (uint32_t)(hi >> 63);
        e += (int)top;
        if (!top)
        {
            hi = (hi << 1) | (lo >> 63);
            lo <<= 1;
        }
        // 53 result bits, then the 11 bits below them, then the sticky word
        const uint64_t m = hi >> 11;
        const uint32_t rem = (uint32_t)hi & 0x7ffu;
        const uint32_t up = (uint32_t)(rem > 0x400u) | ((uint32_t)(rem == 0x400u) & ((uint32_t)(lo != 0) | (uint32_t)(m & 1)));
        const uint64_t r = ((ua ^ ub) & SGN) | ((((uint64_t)(e - 1)) << 52) + m + up);
        return __longlong_as_double((long long)r);
    }

    // a/b correctly rounded (to nearest even), the same bits as the hardware
    // division, on the integer pipes: the quotient of the 53-bit significands
    // to 54 bits plus remainder, from an FP32 reciprocal seed (the fast
    // reciprocal of the divisor's top 24 bits, relative error ~2^-21) refined
    // twice by the exact remainder (R = N - Q*mb in 128-bit integers,
    // Q += R*Y/2^115 with Y ~ 2^115/mb: each step multiplies the error by the
    // seed's), then corrected to 0 <= R < mb; round bit and sticky (R != 0)
    // give the rounding.  The classic quotient refinement by remainders
    // (Newton-Raphson on the reciprocal, Markstein-style final correction with
    // the exact remainder), done in fixed point.  Operands outside the normal
    // range and quotients near the ends of it take the hardware division.
    __device__ __forceinline__ double ddiv_int(double a, double b)
    {
        constexpr uint64_t M52 = 0x000FFFFFFFFFFFFFull, H53 = 0x0010000000000000ull, SGN = 0x8000000000000000ull;
        const uint64_t ua = (uint64_t)__double_as_longlong(a), ub = (uint64_t)__double_as_longlong(b);
        const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
        int e = (int)ea - (int)eb + 1023;
        if (ea - 1u >= 2046u || eb - 1u >= 2046u || (unsigned)(e - 2) >= 2044u) return ddiv_hw(a, b);
        uint64_t ma = (ua & M52) | H53;
        const uint64_t mb = (ub & M52) | H53;
        if (ma < mb) { ma <<= 1; e -= 1; }
        // ma/mb in [1, 2): Q = floor(N/mb) in [2^53, 2^54) with N = ma*2^53
        const uint64_t Nhi = ma >> 11, Nlo = ma << 53;
        // the divisor's top 24 bits as a float in [2^23, 2^24) (biased exponent 150)
        const float fb = __uint_as_float((150u << 23) | ((uint32_t)(mb >> 29) & 0x7fffffu));
        const uint32_t rb = __float_as_uint(__fdividef(1.0f, fb));
        const int rexp = (int)((rb >> 23) & 0xffu) - 127;                  // -24 or -23
        const uint64_t Y = (uint64_t)((rb & 0x7fffffu) | 0x800000u) << (63 + rexp);   // ~2^115/mb < 2^63
        uint64_t Q = __umul64hi(ma << 2, Y);                               // ~ma*2^53/mb
        #pragma unroll
        for (int it = 0; it < 2; ++it)
        {
            const uint64_t Plo = Q*mb, Phi = __umul64hi(Q, mb);
            uint64_t Rlo = Nlo - Plo;
            uint64_t Rhi = Nhi - Phi - (uint64_t)(Nlo < Plo);
            const bool neg = (int64_t)Rhi < 0;
            if (neg) { Rlo = ~Rlo + 1; Rhi = ~Rhi + (uint64_t)(Rlo == 0); }
            // |R| < 2^90: its top 64 bits |R| >> 26 times Y, over 2^89
            const uint64_t d = __umul64hi((Rhi << 38) | (Rlo >> 26), Y) >> 25;
            Q = neg ? Q - d : Q + d;
        }
        const uint64_t Plo = Q*mb, Phi = __umul64hi(Q, mb);
        uint64_t Rlo = Nlo - Plo;
        uint64_t Rhi = Nhi - Phi - (uint64_t)(Nlo < Plo);
        for (int k = 0; k < 4 && (int64_t)Rhi < 0; ++k)
        {
            Q -= 1;
            const uint64_t t = Rlo + mb;
            Rhi += (uint64_t)(t < Rlo);
            Rlo = t;
        }
        for (int k = 0; k < 4 && (Rhi != 0 || Rlo >= mb); ++k)
        {
            Q += 1;
            Rhi -= (uint64_t)(Rlo < mb);
            Rlo -= mb;
        }
        const uint64_t m = Q >> 1;
        const uint32_t up = (uint32_t)(Q & 1) & ((uint32_t)(Rlo != 0) | (uint32_t)(m & 1));
        return __longlong_as_double((long long)(((ua ^ ub) & SGN) | ((((uint64_t)(e - 1)) << 52) + m + up)));
    }

    // sqrt(x) correctly rounded, the same bits as the hardware square root, on
    // the integer pipes: S = floor(sqrt(M)) to 54 bits for the significand
    // scaled to M in [2^106, 2^108) (even exponent), from an FP32 seed (the
    // fast reciprocal square root r of M's top 24 bits t, sqrt(t) ~ t*r)
    // refined twice by the exact remainder (R = M - S^2, S += R/(2S) with
    // 1/(2S) from r: Newton's iteration for the square root in fixed point),
    // then corrected to 0 <= R <= 2S; round bit and sticky (R != 0) give the
    // rounding.  Zero, negative, subnormal, infinite and NaN operands take
    // the hardware square root.
    __device__ __forceinline__ double dsqrt_int(double x)
    {
        constexpr uint64_t M52 = 0x000FFFFFFFFFFFFFull, H53 = 0x0010000000000000ull;
        const uint64_t ux = (uint64_t)__double_as_longlong(x);
        const uint32_t ex = (uint32_t)(ux >> 52);            // the sign bit makes negatives fail the range test
        if (ex - 1u >= 2046u) return dsqrt_hw(x);
        const int E = (int)ex - 1023;
        const int p = E & 1;
        const uint64_t mx = (ux & M52) | H53;
        const uint64_t Mhi = mx >> (10 - p), Mlo = mx << (54 + p);   // M = mx*2^(54+p)
        // t = M >> 84 in [2^22, 2^24) as a float (exact), r ~ t^-1/2, sqrt(t) ~ t*r
        const uint32_t t = (uint32_t)(Mhi >> 20);
        const uint32_t tm = t >> 23;                                  // 1 if t >= 2^23
        const float tf = __uint_as_float(((149u + tm) << 23) | ((t << (1 - tm)) & 0x7fffffu));
        const float r = rsqrtf(tf);
        const uint32_t sb = __float_as_uint(tf*r);
        const uint32_t rb = __float_as_uint(r);
        // S0 = sqrt(t)*2^42; Yr = r*2^74 ~ 2^116/S
        uint64_t S = (uint64_t)((sb & 0x7fffffu) | 0x800000u) << ((int)((sb >> 23) & 0xffu) - 127 + 19);
        const uint64_t Yr = (uint64_t)((rb & 0x7fffffu) | 0x800000u) << ((int)((rb >> 23) & 0xffu) - 127 + 51);
        #pragma unroll
        for (int it = 0; it < 2; ++it)
        {
            const uint64_t Plo = S*S, Phi = __umul64hi(S, S);
            uint64_t Rlo = Mlo - Plo;
            uint64_t Rhi = Mhi - Phi - (uint64_t)(Mlo < Plo);
            const bool neg = (int64_t)Rhi < 0;
            if (neg) { Rlo = ~Rlo + 1; Rhi = ~Rhi + (uint64_t)(Rlo == 0); }
            // |R| < 2^94: |R|/(2S) ~ (|R| >> 30)*Yr/2^87
            const uint64_t d = __umul64hi((Rhi << 34) | (Rlo >> 30), Yr) >> 23;
            S = neg ? S - d : S + d;
        }
        const uint64_t Plo = S*S, Phi = __umul64hi(S, S);
        uint64_t Rlo = Mlo - Plo;
        uint64_t Rhi = Mhi - Phi - (uint64_t)(Mlo < Plo);
        for (int k = 0; k < 4 && (int64_t)Rhi < 0; ++k)
        {
            const uint64_t add = 2*S - 1;                             // (S-1)^2 = S^2 - (2S - 1)
            S -= 1;
            const uint64_t t2 = Rlo + add;
            Rhi += (uint64_t)(t2 < Rlo);
            Rlo = t2;
        }
        for (int k = 0; k < 4 && (Rhi != 0 || Rlo > 2*S); ++k)
        {
            const uint64_t sub = 2*S + 1;                             // (S+1)^2 = S^2 + (2S + 1)
            S += 1;
            Rhi -= (uint64_t)(Rlo < sub);
            Rlo -= sub;
        }
        const uint64_t m = S >> 1;
        const uint32_t up = (uint32_t)(S & 1) & ((uint32_t)(Rlo != 0 || Rhi != 0) | (uint32_t)(m & 1));
        return __longlong_as_double((long long)((((uint64_t)((E - p)/2 + 1022)) << 52) + m + up));
    }

    // x * 2^E (E < 0), the same bits as the hardware multiply by the constant:
    // for a normal x whose product stays normal the scaling only lowers the
    // biased exponent field (exact); zeros, subnormals, infinities, NaNs and
    // products that would become subnormal take the hardware multiply.
    template <int E>
    __device__ __forceinline__ double dmul_pow2(double x)
    {
        static_assert(E < 0 && E > -1022, "negative power of two");
        const uint64_t u = (uint64_t)__double_as_longlong(x);
        const uint32_t ex = (uint32_t)(u >> 52) & 0x7ffu;
        if (ex - uint32_t(1 - E) >= uint32_t(2046 - (1 - E) + 1))
            return dscale_hw(x, E == -1 ? 0.5 : (E == -2 ? 0.25 : __longlong_as_double((long long)(uint64_t(1023 + E) << 52))));
        return __longlong_as_double((long long)(u - (uint64_t(-E) << 52)));
    }

    // 2*x, the same bits as the hardware multiply: for a normal x whose
    // double stays finite the exponent field goes up by one (exact); zeros,
    // subnormals, infinities, NaNs and doubles that would overflow take the
    // hardware multiply.
    __device__ __forceinline__ double dmul_2(double x)
    {
        const uint64_t u = (uint64_t)__double_as_longlong(x);
        const uint32_t ex = (uint32_t)(u >> 52) & 0x7ffu;
        if (ex - 1u >= 2045u) return dscale_hw(x, 2.0);
        return __longlong_as_double((long long)(u + (uint64_t(1) << 52)));
    }

    // float -> double on the integer pipes (exact): rebias the exponent
    // (127 -> 1023, or 255 -> 2047 for infinities and NaNs, whose payload
    // bits move along) and widen the significand.  FP32 zeros keep their
    // sign; FP32 subnormals (|x| < 2^-126) become zero of the same sign.
    __device__ __forceinline__ double f2d_int(float f)
    {
        const uint32_t u = __float_as_uint(f);
        const uint32_t a = u & 0x7fffffffu;
        const uint32_t e = a >> 23;
        uint32_t hi = (a >> 3) + (e == 255u ? (1792u << 20) : (896u << 20));
        uint32_t lo = u << 29;
        if (e == 0u) { hi = 0u; lo = 0u; }
        return __hiloint2double(int(hi | (u & 0x80000000u)), int(lo));
    }

    // double -> float rounded to nearest even on the integer pipes, the same
    // bits as the hardware conversion for every double whose float result is
    // normal (biased float exponent 1..254 before rounding; a carry out of
    // the rounding moves into the exponent, up to infinity as the hardware
    // does); zeros, results in the float subnormal range, overflows,
    // infinities and NaNs take the hardware conversion.
    __device__ __forceinline__ float d2f_int(double x)
    {
        const uint64_t u = (uint64_t)__double_as_longlong(x);
        const uint32_t hi = uint32_t(u >> 32), lo = uint32_t(u);
        const uint32_t e = (hi >> 20) & 0x7ffu;
        if (e - 897u > 253u) return d2f_hw(x);
        const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);     // 23 significand bits
        const uint32_t rem = lo & 0x1fffffffu;                       // the 29 bits below
        uint32_t f = (hi & 0x80000000u) | ((e - 896u) << 23) | m;
        f += uint32_t(rem > 0x10000000u) | (uint32_t(rem == 0x10000000u) & (m & 1u));
        return __uint_as_float(f);
    }
}
