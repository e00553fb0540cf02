// IEEE binary64 arithmetic on the integer pipes.
//
// GB300 executes FP64 at about 2 lanes per clock per SM (1/58 of its FP32
// rate), while its integer pipes run at 64 lanes per clock.  A kernel whose
// time is set by the FP64 pipe (the fused particle pass) can hand some of its
// binary64 operations to these functions: they return the correctly rounded
// (round-to-nearest-even) result, bit for bit what the hardware instruction
// returns, computed with 32- and 64-bit integer multiplies, shifts and adds.
//
// Only the common case is done in integers: finite, non-zero, normal
// operands whose result is normal.  Anything else (zeros, subnormals,
// infinities, NaN, results that overflow or underflow) takes the hardware
// instruction, so every input gives the hardware's result.
//
// The functions are __host__ __device__ so that the host build can check
// them against the host's IEEE arithmetic.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define SF_HD __host__ __device__ __forceinline__
#else
#define SF_HD inline
#endif

namespace orbit {
namespace sf {

SF_HD uint64_t bits(double v) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(v);
#else
  uint64_t u;
  std::memcpy(&u, &v, 8);
  return u;
#endif
}

SF_HD double from_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double v;
  std::memcpy(&v, &u, 8);
  return v;
#endif
}

// High 64 bits of the 128-bit product of two 64-bit unsigned integers.
SF_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

#ifdef __CUDACC__
static __host__ __device__ __noinline__
#else
inline
#endif
double hw_mul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}

// a * b, correctly rounded.  Operands with biased exponents ea, eb in
// [1, 2046] and 1 <= ea + eb - 1023 <= 2045 (a normal result even after the
// normalisation and rounding carries) are multiplied in integers:
// the 53-bit significands' 106-bit product P lies in [2^104, 2^106); its
// top 53 bits are kept, the next bit rounds, the rest is sticky.
SF_HD double mul(double a, double b) {
  const uint64_t A = bits(a), B = bits(b);
  const int ea = (int)(A >> 52) & 0x7FF, eb = (int)(B >> 52) & 0x7FF;
  const int e = ea + eb - 1023;  // exponent field of the result before normalisation
  if ((unsigned)(ea - 1) >= 2046u || (unsigned)(eb - 1) >= 2046u || (unsigned)(e - 1) >= 2045u)
    return hw_mul(a, b);
  const uint64_t frac = (1ull << 52) - 1;
  const uint64_t ma = (A & frac) | (1ull << 52), mb = (B & frac) | (1ull << 52);
  const uint64_t lo = ma * mb, hi = mulhi64(ma, mb);  // P = hi 2^64 + lo, hi < 2^42
  const int s = (int)(hi >> 41);                      // 1: P >= 2^105
  // m = P >> (52 + s): the top 53 bits; r = the next bit; sticky = the rest
  const int sh = 52 + s;
  const uint64_t m0 = (hi << (64 - sh)) | (lo >> sh);
  const uint64_t r = (lo >> (sh - 1)) & 1ull;
  const uint64_t sticky = lo & ((1ull << (sh - 1)) - 1ull);
  const uint64_t m = m0 + (r & ((sticky != 0) | (m0 & 1ull)));
  // m in [2^52, 2^53]; adding it to the exponent field (e + s - 1) places
  // the implicit bit, and m = 2^53 carries into the exponent
  const uint64_t mag = ((uint64_t)(e + s - 1) << 52) + m;
  return from_bits(mag | ((A ^ B) & 0x8000000000000000ull));
}

// The hardware paths of add and fma are kept out of line: inlined, the
// compiler predicates them into the integer code, where they still issue to
// the FP64 pipe on every call.
#ifdef __CUDACC__
static __host__ __device__ __noinline__
#else
inline
#endif
double hw_add(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}

#ifdef __CUDACC__
static __host__ __device__ __noinline__
#else
inline
#endif
double hw_fma(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return __builtin_fma(a, b, c);
#endif
}

SF_HD int clz64(uint64_t v) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)v);
#else
  return v ? __builtin_clzll(v) : 64;
#endif
}

// Packs biased exponent e (of the leading bit) and the significand held in
// the top 53 bits of the normalised (bit 63 set) word n, with `rest` != 0
// when any bit below n is set, rounding to nearest even; 0 when the result
// would not be a normal number (the caller then takes the hardware path).
SF_HD bool pack_rne(int e, uint64_t n, bool rest, uint64_t sign, double* out) {
  const uint64_t m0 = n >> 11;
  const uint64_t r = (n >> 10) & 1ull;
  const bool sticky = rest || (n & 0x3FFull) != 0;
  const uint64_t m = m0 + (r & ((uint64_t)sticky | (m0 & 1ull)));
  if ((unsigned)(e - 1) >= 2045u) return false;  // 1 <= e <= 2045 leaves room for the rounding carry
  *out = from_bits((((uint64_t)(e - 1) << 52) + m) | sign);
  return true;
}

// a + b, correctly rounded.  The larger magnitude X and the smaller Y,
// significands shifted left by 10 (guard bits), Y aligned right with the
// shifted-out bits ORed into its lowest bit; the sum or difference is
// normalised and rounded.  A cancellation that leaves zero gives +0 (round
// to nearest); other cases take the hardware instruction.
SF_HD double add(double a, double b) {
  const uint64_t A = bits(a), B = bits(b);
  const uint64_t mag_mask = 0x7FFFFFFFFFFFFFFFull;
  const bool swap = (B & mag_mask) > (A & mag_mask);
  const uint64_t X = swap ? B : A, Y = swap ? A : B;
  const int ex = (int)(X >> 52) & 0x7FF, ey = (int)(Y >> 52) & 0x7FF;
  if ((unsigned)(ex - 1) >= 2046u || (unsigned)(ey - 1) >= 2046u) return hw_add(a, b);
  const uint64_t frac = (1ull << 52) - 1;
  const uint64_t mx = ((X & frac) | (1ull << 52)) << 10;
  uint64_t my = ((Y & frac) | (1ull << 52)) << 10;
  const int d = ex - ey;
  if (d >= 64) {
    my = 1ull;  // only the sticky bit remains
  } else if (d > 0) {
    my = (my >> d) | (uint64_t)((my << (64 - d)) != 0);
  }
  const bool sub = ((A ^ B) >> 63) != 0;
  const uint64_t s = sub ? mx - my : mx + my;
  if (s == 0) return 0.0;
  const int lz = clz64(s);
  double out;
  if (!pack_rne(ex + 1 - lz, s << lz, false, X & ~mag_mask, &out)) return hw_add(a, b);
  return out;
}

// a * b + c with one rounding.  The 106-bit product P (shifted left by 20
// in a 128-bit word, leading bit at 124 or 125) and c's significand
// (shifted left by 72, leading bit at 124) are aligned to the larger
// exponent with the shifted-out bits ORed into the lowest bit, added or
// subtracted, normalised and rounded.  An exact zero and results outside
// the normal range take the hardware instruction.
SF_HD double fma(double a, double b, double c) {
  const uint64_t A = bits(a), B = bits(b), C = bits(c);
  const int ea = (int)(A >> 52) & 0x7FF, eb = (int)(B >> 52) & 0x7FF, ec = (int)(C >> 52) & 0x7FF;
  const int ep = ea + eb - 1023;
  if ((unsigned)(ea - 1) >= 2046u || (unsigned)(eb - 1) >= 2046u || (unsigned)(ec - 1) >= 2046u ||
      (unsigned)(ep - 1) >= 2045u)
    return hw_fma(a, b, c);
  const uint64_t frac = (1ull << 52) - 1;
  const uint64_t ma = (A & frac) | (1ull << 52), mb = (B & frac) | (1ull << 52), mc = (C & frac) | (1ull << 52);
  const uint64_t pl0 = ma * mb, ph0 = mulhi64(ma, mb);
  // P << 20 and c << 72 as (hi, lo); bit 0 weighs 2^EP and 2^EC
  uint64_t ph = (ph0 << 20) | (pl0 >> 44), pl = pl0 << 20;
  uint64_t ch = mc << 8, cl = 0;
  const int EP = ea + eb - 2170, EC = ec - 1147;
  int E;
  const int d = EP - EC;
  if (d >= 0) {  // c is the smaller: shift it right by d, jamming
    E = EP;
    if (d >= 128) {
      cl = 1ull;
      ch = 0;
    } else if (d >= 64) {
      const int k = d - 64;
      cl = (k == 0 ? ch : (ch >> k)) | (uint64_t)((k != 0 && (ch << (64 - k)) != 0));
      ch = 0;
    } else if (d > 0) {
      cl = (ch << (64 - d));  // c's low word is zero: nothing is shifted out
      ch >>= d;
    }
  } else {  // the product is the smaller
    E = EC;
    const int k = -d;
    if (k >= 128) {
      pl = 1ull;
      ph = 0;
    } else if (k >= 64) {
      const int j = k - 64;
      const bool lost = pl != 0 || (j != 0 && (ph << (64 - j)) != 0);
      pl = (j == 0 ? ph : (ph >> j)) | (uint64_t)lost;
      ph = 0;
    } else {
      const bool lost = (pl << (64 - k)) != 0;
      pl = (pl >> k) | (ph << (64 - k)) | (uint64_t)lost;
      ph >>= k;
    }
  }
  const bool sub = ((A ^ B ^ C) >> 63) != 0;
  uint64_t sh, sl, sign = (A ^ B) & 0x8000000000000000ull;
  if (!sub) {
    sl = pl + cl;
    sh = ph + ch + (uint64_t)(sl < pl);
  } else {
    sl = pl - cl;
    sh = ph - ch - (uint64_t)(pl < cl);
    if (sh >> 63) {  // c was the larger: negate
      sl = ~sl + 1ull;
      sh = ~sh + (uint64_t)(sl == 0);
      sign ^= 0x8000000000000000ull;
    }
  }
  if ((sh | sl) == 0) return hw_fma(a, b, c);
  // normalise: leading bit to bit 127
  const int lz = sh ? clz64(sh) : 64 + clz64(sl);
  uint64_t nh, nl;
  if (lz >= 64) {
    nh = sl << (lz - 64);
    nl = 0;
  } else if (lz > 0) {
    nh = (sh << lz) | (sl >> (64 - lz));
    nl = sl << lz;
  } else {
    nh = sh;
    nl = sl;
  }
  // value = S 2^E, leading bit at 127 - lz: biased exponent E + 127 - lz + 1023
  double out;
  if (!pack_rne(E + 1150 - lz, nh, nl != 0, sign, &out)) return hw_fma(a, b, c);
  return out;
}

#ifdef __CUDACC__
static __host__ __device__ __noinline__
#else
inline
#endif
float hw_d2f(double x) {
#ifdef __CUDA_ARCH__
  return __double2float_rn(x);
#else
  return (float)x;
#endif
}

#ifdef __CUDACC__
static __host__ __device__ __noinline__
#else
inline
#endif
double hw_f2d(float f) {
  return (double)f;
}

SF_HD uint32_t fbits(float v) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__float_as_uint(v);
#else
  uint32_t u;
  std::memcpy(&u, &v, 4);
  return u;
#endif
}

SF_HD float from_fbits(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float v;
  std::memcpy(&v, &u, 4);
  return v;
#endif
}

// (float)x rounded to nearest even: for x whose float exponent is in
// [-126, 126] the top 24 significand bits are kept, bit 28 rounds and the
// 28 bits below it are sticky; the rounding carry may step the exponent
// (to at most 127, still finite).  Zeros, subnormal results, overflow,
// infinities and NaN take the hardware conversion.
SF_HD float to_float(double x) {
  const uint64_t X = bits(x);
  const int ef = (int)((X >> 52) & 0x7FF) - 1023 + 127;  // biased float exponent
  if ((unsigned)(ef - 1) >= 253u) return hw_d2f(x);
  const uint64_t m = X & ((1ull << 52) - 1);
  uint32_t r = ((uint32_t)ef << 23) | (uint32_t)(m >> 29);
  const uint32_t rest = (uint32_t)m & ((1u << 29) - 1), half = 1u << 28;
  r += (rest > half || (rest == half && (r & 1u))) ? 1u : 0u;
  return from_fbits(r | ((uint32_t)(X >> 32) & 0x80000000u));
}

// (double)f, exact: the exponent rebased and the significand widened;
// subnormal floats, infinities and NaN take the hardware conversion.
SF_HD double from_float(float f) {
  const uint32_t F = fbits(f);
  const uint32_t e = (F >> 23) & 0xFFu;
  if (e - 1u >= 254u) {
    if ((F & 0x7FFFFFFFu) == 0u) return from_bits((uint64_t)F << 32);  // signed zero
    return hw_f2d(f);
  }
  return from_bits(((uint64_t)(F & 0x80000000u) << 32) | ((uint64_t)(e + 896u) << 52) |
                   ((uint64_t)(F & 0x7FFFFFu) << 29));
}

// x * 2^k for k = -1 or +1 (exact) as an exponent change; the hardware
// multiply where x is zero, subnormal, not finite or the result leaves the
// normal range.
SF_HD double scale2(double x, int k) {
  const uint64_t X = bits(x);
  const int e = (int)(X >> 52) & 0x7FF;
  if ((unsigned)(e + k - 1) >= 2046u || e == 0 || e == 2047) return hw_mul(x, k > 0 ? 2.0 : 0.5);
  return from_bits(X + ((uint64_t)(int64_t)k << 52));
}

}  // namespace sf

// Which pipe the maps' and the kick's multiplies use, one bit per family
// (1: integer, 0: FP64; bits as in apply_ops, bit 4 the SC kick); the
// results are the same for every value.  Measured on the FODO turn (1e6
// particles, fused pass per turn): all on the FP64 pipe 26.2 ms, all on the
// integer pipes 23.5 ms, drift and quad fringe on the integer pipes 23.1
// ms (quad1 indifferent; the kick's on the integer pipes 0.4 ms slower, the
// fringe's on the FP64 pipe 1.9 ms slower).
#ifndef ORBIT_SOFT_MUL
#define ORBIT_SOFT_MUL 0x0D
#endif

#ifdef __CUDACC__
// The binary64 multiply of the TEAPOT maps and the kick: S = 1 on the
// integer pipes (sf::mul), S = 0 on the FP64 pipe.  Both return the same
// correctly rounded product, so kernels may choose either.
template <int S>
__device__ __forceinline__ double dmul(double a, double b) {
  return S ? sf::mul(a, b) : __dmul_rn(a, b);
}
template <int S>
__device__ __forceinline__ double dhalf(double a) {
  return S ? sf::scale2(a, -1) : __dmul_rn(a, 0.5);
}
template <int S>
__device__ __forceinline__ double dtwice(double a) {
  return S ? sf::scale2(a, 1) : __dmul_rn(a, 2.0);
}
#endif

}  // namespace orbit
