// swe_fp64.cuh -- correctly rounded FP64 division and square root on the
// integer pipe.
//
// On GB300 the FP64 pipe retires 2 lanes per SM per cycle (measured 1.26
// TFLOP/s), so one warp-wide DFMA holds an SM partition's FP64 pipe for about
// 64 cycles, and a hardware division or square root is a chain of 7-10 of them.
// The integer pipe issues one warp instruction per cycle.  These routines
// compute IEEE round-to-nearest-even a / b and sqrt(x) from the 53-bit integer
// significands, with a single-precision estimate refined by two Newton steps
// in 128-bit fixed point and an exact remainder check, so the result equals
// the hardware instruction bit for bit.  Operands or results that are zero,
// subnormal, infinite or NaN take the hardware instruction.
//
// The methods are textbook: Newton-Raphson reciprocal and reciprocal square
// root iterations (y' = y (2 - b y), y' = y (3 - x y^2) / 2) followed by
// correction of the truncated quotient/root with the exact remainder.
#pragma once

#include <cuda_runtime.h>

namespace swe {

#if defined(__CUDACC__)

// Bit moves between a double and a 64-bit integer that the optimiser cannot
// see through.  With a plain reinterpretation, integer sign-mask operations on
// the bits (x & 0x7FF..F, x | sign, x ^ sign) are folded back into FP64 abs /
// negate instructions, which issue on the FP64 pipe (measured: an integer-key
// min of two doubles cost two FP64 instructions).
__device__ __forceinline__ long long dbits(double x) {
  long long r;
  asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
  return r;
}
__device__ __forceinline__ double dfrom(long long r) {
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(r));
  return x;
}

namespace fp64detail {

constexpr unsigned long long kM52 = (1ull << 52) - 1ull;
constexpr unsigned long long kHid = 1ull << 52;

__device__ __forceinline__ unsigned long long bits(double x) { return (unsigned long long)dbits(x); }
__device__ __forceinline__ double from_bits(unsigned long long u) { return dfrom((long long)u); }

// round a 63-bit truncated significand q (value in [2^62, 2^63)) to 53 bits;
// returns the rounded significand (may be 2^53)
__device__ __forceinline__ unsigned long long round63(unsigned long long q, bool sticky) {
  unsigned long long mant = q >> 10;
  const unsigned low = (unsigned)(q & 0x3FFull);
  const bool up = (low > 0x200u) || (low == 0x200u && (sticky || (mant & 1ull)));
  return mant + (up ? 1ull : 0ull);
}

// The hardware instructions for the rare operands, kept out of line so that
// the common path never issues them (predicated in-line copies would cost FP64
// pipe slots on every call).
static __device__ __noinline__ double ddiv_hw(double a, double b) { return __ddiv_rn(a, b); }
static __device__ __noinline__ double dsqrt_hw(double x) { return __dsqrt_rn(x); }

// 64-bit fixed-point value of a float f in (0.5, 1]: f 2^shift, from its bits
// (integer ops only: 64-bit integer <-> float conversions issue on the FP64
// pipe, measured)
__device__ __forceinline__ unsigned long long fixed_from_unit_float(float f, int shift) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long m = (unsigned long long)((u & 0x7FFFFFu) | 0x800000u);  // 2^23 (1.m)
  const int e = (int)(u >> 23) - 127;                                             // f = 1.m 2^e
  return m << (shift - 23 + e);
}

}  // namespace fp64detail

// 0.5 x and -x exactly, on the integer pipe: halving lowers the exponent by
// one; zeros, subnormals and the smallest normals (value M 2^-1074, M < 2^53)
// halve M with ties to even; infinities and NaNs are returned unchanged.
__device__ __forceinline__ double dhalf_rn(double x) {
  using namespace fp64detail;
  const unsigned long long u = bits(x);
  const unsigned e = (unsigned)(u >> 52) & 0x7FFu;
  if (e >= 2u && e != 0x7FFu) return from_bits(u - kHid);
  if (e == 0x7FFu) return x;
  const unsigned long long M = u & ((1ull << 53) - 1ull);
  const unsigned long long H = (M >> 1) + (M & (M >> 1) & 1ull);
  return from_bits((u & 0x8000000000000000ull) | H);
}
__device__ __forceinline__ double dneg(double x) {
  return fp64detail::from_bits(fp64detail::bits(x) ^ 0x8000000000000000ull);
}

// ddiv_rn and dsqrt_rn are called, not inlined: a flux evaluation has half a
// dozen of them, and inlined copies of their integer sequences made the edge
// kernel stall on instruction fetch (ncu "no instruction"); out of line the
// 1M-cell step ran 5 % faster (k_flux 0.215 vs 0.244 ms), with the same bits.
static __device__ __noinline__ double ddiv_rn(double a, double b) {
  using namespace fp64detail;
  const unsigned long long ua = bits(a), ub = bits(b);
  const unsigned ea = (unsigned)(ua >> 52) & 0x7FFu, eb = (unsigned)(ub >> 52) & 0x7FFu;
  if (ea - 1u >= 2046u || eb - 1u >= 2046u) {
    // +-0 / normal (still water: zero momentum over a depth) stays in line
    if ((ua << 1) == 0ull && eb - 1u < 2046u) return from_bits((ua ^ ub) & 0x8000000000000000ull);
    return ddiv_hw(a, b);
  }
  unsigned long long ma = (ua & kM52) | kHid;
  const unsigned long long mb = (ub & kM52) | kHid;
  const unsigned long long sign = (ua ^ ub) & 0x8000000000000000ull;
  int e = (int)ea - (int)eb;
  if (ma < mb) {
    ma <<= 1;
    --e;
  }
  int E = e + 1023;
  if (E < 1 || E > 2046) return ddiv_hw(a, b);
  if (mb == kHid) return from_bits(sign | ((unsigned long long)E << 52) | (ma & kM52));  // power of two
  // R ~ 2^116 / mb in (2^63, 2^64): float estimate from mb's leading bits
  // (1 <= fb < 2, 1 / fb in (0.5, 1]), two Newton steps
  const float fb = __uint_as_float(0x3F800000u | (unsigned)((mb >> 29) & 0x7FFFFFull));
  const float rf = __frcp_rn(fb);
  unsigned long long R = rf < 1.0f ? fixed_from_unit_float(rf, 64) : ~0ull;
  {
    const unsigned __int128 P = (unsigned __int128)mb * R;
    const __int128 D = ((__int128)1 << 116) - (__int128)P;  // |D| < 2^94
    const long long Dh = (long long)(D >> 32);
    R += (unsigned long long)(long long)(((__int128)R * Dh) >> 84);
  }
  {
    const unsigned __int128 P = (unsigned __int128)mb * R;
    const __int128 D = ((__int128)1 << 116) - (__int128)P;  // |D| < 2^71
    const long long Dh = (long long)(D >> 9);
    R += (unsigned long long)(long long)(((__int128)R * Dh) >> 107);
  }
  // Q = floor(ma 2^62 / mb) in [2^62, 2^63), corrected with the exact remainder
  unsigned long long Q = (unsigned long long)(((unsigned __int128)ma * R) >> 54);
  const __int128 N = (__int128)((unsigned __int128)ma << 62);
  __int128 rem = N - (__int128)((unsigned __int128)Q * mb);
#pragma unroll 1
  for (int k = 0; k < 8 && rem < 0; ++k) {
    --Q;
    rem += (__int128)mb;
  }
#pragma unroll 1
  for (int k = 0; k < 8 && rem >= (__int128)mb; ++k) {
    ++Q;
    rem -= (__int128)mb;
  }
  if (rem < 0 || rem >= (__int128)mb || Q < (1ull << 62) || Q >= (1ull << 63)) return ddiv_hw(a, b);
  unsigned long long mant = round63(Q, rem != 0);
  if (mant == (1ull << 53)) {
    mant = kHid;
    if (++E > 2046) return ddiv_hw(a, b);
  }
  return from_bits(sign | ((unsigned long long)E << 52) | (mant & kM52));
}

static __device__ __noinline__ double dsqrt_rn(double x) {
  using namespace fp64detail;
  const unsigned long long ux = bits(x);
  const unsigned ex = (unsigned)(ux >> 52) & 0x7FFu;
  if (ex - 1u >= 2046u || (ux >> 63)) return (ux << 1) == 0ull ? x : dsqrt_hw(x);  // sqrt(+-0) = +-0 (dry side)
  unsigned long long M = (ux & kM52) | kHid;
  int e = (int)ex - 1023;  // x = M 2^(e - 52)
  if (e & 1) {             // make e - 52 even
    M <<= 1;
    --e;
  }
  // R ~ 2^89 / sqrt(M) in (2^62, 2^63]: float estimate from M's leading bits
  // (fm = M 2^-52 in [1, 4), 1 / sqrt(fm) in (0.5, 1])
  const float fm = (M >> 53) ? __uint_as_float(0x40000000u | (unsigned)((M >> 30) & 0x7FFFFFull))
                             : __uint_as_float(0x3F800000u | (unsigned)((M >> 29) & 0x7FFFFFull));
  unsigned long long R = fixed_from_unit_float(rsqrtf(fm), 63);
  {
    const unsigned long long T = (unsigned long long)(((unsigned __int128)R * R) >> 64);  // ~ 2^114 / M
    const unsigned __int128 U = (unsigned __int128)M * T;                                   // ~ 2^114
    const __int128 D = ((__int128)1 << 114) - (__int128)U;  // |D| < 2^94
    const long long Dh = (long long)(D >> 32);
    R += (unsigned long long)(long long)(((__int128)R * Dh) >> 83);
  }
  {
    const unsigned long long T = (unsigned long long)(((unsigned __int128)R * R) >> 64);
    const unsigned __int128 U = (unsigned __int128)M * T;
    const __int128 D = ((__int128)1 << 114) - (__int128)U;  // |D| < 2^73
    const long long Dh = (long long)(D >> 11);
    R += (unsigned long long)(long long)(((__int128)R * Dh) >> 104);
  }
  // S = floor(sqrt(M 2^72)) in [2^62, 2^63), corrected with exact squares
  unsigned long long S = (unsigned long long)(((unsigned __int128)M * R) >> 53);
  const unsigned __int128 N = (unsigned __int128)M << 72;
#pragma unroll 1
  for (int k = 0; k < 8 && (unsigned __int128)S * S > N; ++k) --S;
#pragma unroll 1
  for (int k = 0; k < 8 && (unsigned __int128)(S + 1) * (S + 1) <= N; ++k) ++S;
  const unsigned __int128 S2 = (unsigned __int128)S * S;
  if (S2 > N || (unsigned __int128)(S + 1) * (S + 1) <= N || S < (1ull << 62) || S >= (1ull << 63))
    return dsqrt_hw(x);
  unsigned long long mant = round63(S, S2 != N);
  int E = 26 + (e - 52) / 2 + 1023;
  if (mant == (1ull << 53)) {
    mant = kHid;
    ++E;
  }
  return from_bits(((unsigned long long)E << 52) | (mant & kM52));
}

#endif  // __CUDACC__

}  // namespace swe
