// The Marsaglia polar method of gsl_ran_gaussian over a stream cut into
// chunks (taus_field.cu): a deviate takes an accepted pair of the stream with
// its zero values removed (gsl_rng_uniform_pos redraws a 0), and a pair
// belongs to the chunk that holds its first value.  Plain C++ for host and
// device, checked on the CPU against the sequential method on streams with
// zeros (tests/taus_chunk_check.cpp).
#pragma once
#include <cmath>

#include "taus_index.h"

namespace exh {

#if defined(__CUDA_ARCH__)
#define EXH_DMUL(a, b) __dmul_rn(a, b)
#define EXH_DADD(a, b) __dadd_rn(a, b)
#define EXH_DDIV(a, b) __ddiv_rn(a, b)
#define EXH_DSQRT(a) __dsqrt_rn(a)
#else
#define EXH_DMUL(a, b) ((a) * (b))
#define EXH_DADD(a, b) ((a) + (b))
#define EXH_DDIV(a, b) ((a) / (b))
#define EXH_DSQRT(a) sqrt(a)
#endif

// x = -1 + 2 v / 2^32 = (v - 2^31) / 2^31, exactly
EXH_HD double polar_coord(unsigned v) { return (double)((long long)v - 2147483648LL) * (1.0 / 2147483648.0); }

// acceptance of the pair (v1, v2): r2 = x^2 + y^2 in (0, 1].  Exact in
// 64-bit integers (2^62 r2 = a^2 + b^2) away from the unit circle; within
// 2^-50 of it the reference's double operations (no fused multiply-add)
// decide.
EXH_HD bool polar_accept(unsigned v1, unsigned v2) {
  const long long a = (long long)v1 - 2147483648LL, b = (long long)v2 - 2147483648LL;
  const unsigned long long s = (unsigned long long)(a * a) + (unsigned long long)(b * b);
  const unsigned long long one = 1ull << 62;
  if (s == 0ull) return false;
  if (s > one + 4096ull) return false;
  if (s + 4096ull < one) return true;
  const double x = polar_coord(v1), y = polar_coord(v2);
  const double r2 = EXH_DADD(EXH_DMUL(x, x), EXH_DMUL(y, y));
  return !(r2 > 1.0 || r2 == 0.0);
}

#if defined(__CUDA_ARCH__)
#define EXH_CLZ64(x) __clzll((long long)(x))
#else
#define EXH_CLZ64(x) __builtin_clzll(x)
#endif

// v, v > 0, rounded to 53 significant bits (nearest, ties to even)
EXH_HD unsigned long long round53(unsigned long long v) {
  const int n = 64 - EXH_CLZ64(v);
  if (n <= 53) return v;
  const int sh = n - 53;
  unsigned long long q = v >> sh;
  const unsigned long long rem = v & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
  if (rem > half || (rem == half && (q & 1ull))) q++;
  return q << sh;
}

// The bits of the reference's r2 = x*x + y*y in double (each product and the
// sum rounded once) for the pair (v1, v2), x = a 2^-31, y = b 2^-31: the same
// roundings on the integers a^2, b^2 (2^62 x^2, 2^62 y^2), which holds for
// a^2 + b^2 > 0 (every double involved is normal).
EXH_HD unsigned long long r2_bits(unsigned v1, unsigned v2) {
  const long long a = (long long)v1 - 2147483648LL, b = (long long)v2 - 2147483648LL;
  const unsigned long long A2 = (a == 0) ? 0ull : round53((unsigned long long)(a * a));
  const unsigned long long B2 = (b == 0) ? 0ull : round53((unsigned long long)(b * b));
  const unsigned long long R = round53(A2 + B2);                 // 2^62 r2, <= 2^63
  const int n = 64 - EXH_CLZ64(R);                               // r2 in [2^(n-63), 2^(n-62))
  const unsigned long long M = n > 53 ? R >> (n - 53) : R << (53 - n);
  return ((unsigned long long)(n - 63 + 1023) << 52) | (M & 0x000fffffffffffffull);
}

// the accepted pair's deviate y sqrt(-2 ln r2 / r2), in FP64 as
// gsl_ran_gaussian forms it; `logf64` is the natural logarithm
template <class Log>
EXH_HD double polar_deviate(unsigned v1, unsigned v2, Log logf64) {
  const double x = polar_coord(v1), y = polar_coord(v2);
  const double r2 = EXH_DADD(EXH_DMUL(x, x), EXH_DMUL(y, y));
  const double w = EXH_DDIV(EXH_DMUL(-2.0, logf64(r2)), r2);
  return EXH_DMUL(y, EXH_DSQRT(w));
}

// ---------------------------------------------------------------------------
// The deviate in float without FP64 arithmetic.  The reference rounds its
// FP64 result g_d = y sqrt(-2 ln r2 / r2) (within 2^-50 of the exact value)
// to float.  Here the same value is formed in double-float arithmetic (pairs
// of floats, error-free sums and products; relative error below 2^-42) as
// g = hi + lo, and hi is the float of g_d whenever lo lies more than 2^-36 |g|
// inside hi's rounding interval.  Otherwise (about 1 deviate in 2000) the
// caller forms g_d in FP64.  GB300 runs FP64 at a small fraction of its FP32
// rate; this keeps the FP64 units for the rare undecided deviates.
#if defined(__CUDA_ARCH__)
#define EXH_FADD(a, b) __fadd_rn(a, b)
#define EXH_FSUB(a, b) __fsub_rn(a, b)
#define EXH_FMUL(a, b) __fmul_rn(a, b)
#define EXH_FMA(a, b, c) __fmaf_rn(a, b, c)
#define EXH_FDIV(a, b) __fdiv_rn(a, b)
#define EXH_FSQRT(a) __fsqrt_rn(a)
#define EXH_F_AS_U(x) __float_as_uint(x)
#define EXH_U_AS_F(x) __uint_as_float(x)
#define EXH_D_AS_U64(x) ((unsigned long long)__double_as_longlong(x))
#else
#define EXH_FADD(a, b) ((a) + (b))
#define EXH_FSUB(a, b) ((a) - (b))
#define EXH_FMUL(a, b) ((a) * (b))
#define EXH_FMA(a, b, c) fmaf(a, b, c)
#define EXH_FDIV(a, b) ((a) / (b))
#define EXH_FSQRT(a) sqrtf(a)
#define EXH_F_AS_U(x) exh_f_as_u(x)
#define EXH_U_AS_F(x) exh_u_as_f(x)
#define EXH_D_AS_U64(x) exh_d_as_u64(x)
inline unsigned exh_f_as_u(float x) { unsigned u; __builtin_memcpy(&u, &x, 4); return u; }
inline float exh_u_as_f(unsigned u) { float x; __builtin_memcpy(&x, &u, 4); return x; }
inline unsigned long long exh_d_as_u64(double x) { unsigned long long u; __builtin_memcpy(&u, &x, 8); return u; }
#endif

struct DFloat {
  float hi, lo;
};

EXH_HD DFloat df_two_sum(float a, float b) {
  const float s = EXH_FADD(a, b);
  const float bb = EXH_FSUB(s, a);
  const float e = EXH_FADD(EXH_FSUB(a, EXH_FSUB(s, bb)), EXH_FSUB(b, bb));
  return {s, e};
}

EXH_HD DFloat df_fast_two_sum(float a, float b) {   // |a| >= |b|
  const float s = EXH_FADD(a, b);
  return {s, EXH_FSUB(b, EXH_FSUB(s, a))};
}

EXH_HD DFloat df_add(DFloat x, DFloat y) {
  const DFloat s = df_two_sum(x.hi, y.hi);
  const DFloat t = df_two_sum(x.lo, y.lo);
  DFloat r = df_fast_two_sum(s.hi, EXH_FADD(s.lo, t.hi));
  return df_fast_two_sum(r.hi, EXH_FADD(r.lo, t.lo));
}

EXH_HD DFloat df_mul(DFloat x, DFloat y) {
  const float p = EXH_FMUL(x.hi, y.hi);
  float e = EXH_FMA(x.hi, y.hi, -p);
  e = EXH_FMA(x.hi, y.lo, e);
  e = EXH_FMA(x.lo, y.hi, e);
  return df_fast_two_sum(p, e);
}

EXH_HD DFloat df_div(DFloat x, DFloat y) {
  const float q1 = EXH_FDIV(x.hi, y.hi);
  // x - q1 y, exactly in its leading part
  const float p = EXH_FMUL(q1, y.hi);
  const float pe = EXH_FMA(q1, y.hi, -p);
  float r = EXH_FSUB(x.hi, p);                         // exact: x.hi and q1 y.hi agree to a few bits
  r = EXH_FSUB(EXH_FADD(r, x.lo), EXH_FMA(q1, y.lo, pe));
  return df_fast_two_sum(q1, EXH_FDIV(r, y.hi));
}

EXH_HD DFloat df_sqrt(DFloat x) {                      // x > 0
  const float s = EXH_FSQRT(x.hi);
  const float p = EXH_FMUL(s, s);
  const float pe = EXH_FMA(s, s, -p);
  const float r = EXH_FADD(EXH_FSUB(EXH_FSUB(x.hi, p), pe), x.lo);
  return df_fast_two_sum(s, EXH_FDIV(r, EXH_FADD(s, s)));
}

// a double as a double-float (48 of its 53 bits; relative error 2^-48)
EXH_HD DFloat df_from_bits(unsigned long long B) {
  // hi: sign, exponent and the 23 leading fraction bits (truncated); lo: the
  // 29 bits below, scaled
  const int be = (int)((B >> 52) & 0x7ffull);
  const unsigned top = (unsigned)((B >> 63) << 31) | (unsigned)((be - 1023 + 127) << 23) |
                       (unsigned)((B >> 29) & 0x7fffffull);
  const float hi = EXH_U_AS_F(top);
  const unsigned rest = (unsigned)(B & 0x1fffffffull);           // < 2^29
  // rest * 2^(be - 1023 - 52): split rest exactly into two floats
  const float r_hi = (float)(rest >> 5) * 32.0f, r_lo = (float)(rest & 31u);
  const unsigned sc = (unsigned)((be - 1023 - 52 + 127) << 23);  // 2^(be - 1075), normal for r2 >= 2^-62
  const float scale = EXH_U_AS_F(sc);
  float lo = EXH_FADD(EXH_FMUL(r_hi, scale), EXH_FMUL(r_lo, scale));
  if (B >> 63) lo = -lo;
  return df_fast_two_sum(hi, lo);
}

// D 2^p as a double-float, exactly for |D| < 2^47 (2^p and the parts
// normal): the two 24-bit halves of D convert exactly from 32-bit integers
// (64-bit integer conversions would take the slow FP64 pipe)
EXH_HD DFloat df_from_int(long long D, int p) {
  const int dh = (int)(D >> 24);                                 // floor(D / 2^24), |dh| < 2^23
  const int dl = (int)(D & 0xffffffll);                          // 0 <= dl < 2^24
  const float h = EXH_FMUL((float)dh, EXH_U_AS_F((unsigned)((p + 24 + 127) << 23)));
  const float l = EXH_FMUL((float)dl, EXH_U_AS_F((unsigned)((p + 127) << 23)));
  return df_two_sum(h, l);                                       // h + l is D 2^p exactly
}

// D 2^p as a double-float for any |D| < 2^63: the 47 leading bits of D
// (relative error below 2^-46)
EXH_HD DFloat df_from_big(long long D, int p) {
  const unsigned long long ad = D < 0 ? (unsigned long long)(-D) : (unsigned long long)D;
  const int nb = ad ? 64 - EXH_CLZ64(ad) : 0;
  if (nb > 47) {
    const int sh = nb - 47;
    return df_from_int(D >> sh, p + sh);
  }
  return df_from_int(D, p);
}

// ln(1 + u), |u| <= 2^-8, relative error below 2^-44: u - u^2/2 in
// double-float, the u^3 .. u^6 terms in float
EXH_HD DFloat df_log1p_small(DFloat u) {
  const float u2 = EXH_FMUL(u.hi, u.hi);
  const float u2e = EXH_FMA(u.hi, u.hi, -u2);
  const float cross = EXH_FMUL(EXH_FADD(u.hi, u.hi), u.lo);
  const DFloat h = df_fast_two_sum(EXH_FMUL(u2, 0.5f), EXH_FMUL(EXH_FADD(u2e, cross), 0.5f));   // u^2 / 2
  // u^3 (1/3 - u/4 + u^2/5 - u^3/6)
  float t = EXH_FMA(u.hi, -1.0f / 6.0f, 0.2f);
  t = EXH_FMA(u.hi, t, -0.25f);
  t = EXH_FMA(u.hi, t, 1.0f / 3.0f);
  const float tail = EXH_FMUL(EXH_FMUL(u2, u.hi), t);
  DFloat r = df_add(u, {-h.hi, -h.lo});
  return df_add(r, {tail, 0.0f});
}

// The deviate of the accepted pair (v1, v2) as a double-float, for y != 0
// and r2 < 1.  `lnc` holds ln(c_i) for the 192 table points
// c_i = 0.75 + (i + 1/2) / 256 as double-float pairs (hi, lo), `invc` their
// reciprocals the same way.
EXH_HD DFloat polar_deviate_df(unsigned v1, unsigned v2, const float* lnc, const float* invc) {
  // the exact S = 2^62 (x^2 + y^2) stands for the reference's r2 (S rounded
  // three times, relative difference below 2^-51): with 1 - r2 >= 2^-12 and
  // S >= 2^20 (the caller's conditions) that moves ln r2 by less than 2^-39
  // of itself
  const long long a = (long long)v1 - 2147483648LL, b = (long long)v2 - 2147483648LL;
  const unsigned long long S = (unsigned long long)(a * a) + (unsigned long long)(b * b);
  const int n = 64 - EXH_CLZ64(S);                              // r2 = S 2^-62 in [2^(n-63), 2^(n-62))
  // m = S 2^-top in [1, 2) (top = n - 1); from 1.5 on, m / 2 in [0.75, 1)
  int e = n - 63, top = n - 1;
  if ((S >> (n - 2)) & 1ull) {
    top = n;
    e += 1;
  }
  DFloat L;
  if (e == 0 && S >= (1ull << 62) - (1ull << 54)) {
    // r2 within 2^-8 below 1: ln(1 + u), u = r2 - 1 = (S - 2^62) 2^-62
    L = df_log1p_small(df_from_big((long long)S - (1ll << 62), -62));
  } else {
    // table point c_i = (385 + 2 i) / 512 next to m; m - c_i from the
    // integers, u = (m - c_i) / c_i
    const int i = (int)((S - (3ull << (top - 2))) >> (top - 8));
    const long long C = (385ll + 2 * i) << (top - 9);
    const DFloat u = df_mul(df_from_big((long long)S - C, -top), {invc[2 * i], invc[2 * i + 1]});
    L = df_add(df_log1p_small(u), {lnc[2 * i], lnc[2 * i + 1]});
    if (e != 0) {
      const float ef = (float)e;
      const float ln2_hi = 0.693145751953125f, ln2_lo = 1.42860682030941723212e-06f;   // ln 2 = hi + lo
      const DFloat el = df_fast_two_sum(EXH_FMUL(ef, ln2_hi), EXH_FMUL(ef, ln2_lo));  // ef * ln2_hi exact
      L = df_add(el, L);
    }
  }
  // w = -2 ln r2 / r2, g = y sqrt(w), y = b 2^-31
  const DFloat w = df_div({EXH_FMUL(-2.0f, L.hi), EXH_FMUL(-2.0f, L.lo)}, df_from_big((long long)S, -62));
  const DFloat sq = df_sqrt(w);
  const DFloat g = df_mul(df_from_int(b, 0), sq);
  return {EXH_FMUL(g.hi, 4.656612873077392578125e-10f), EXH_FMUL(g.lo, 4.656612873077392578125e-10f)};
}

// Whether every value within 2^-36 |g| of the double-float g rounds to g.hi
// in float: hi's rounding interval reaches half an ulp above and half an ulp
// (a quarter at a power of two) below in magnitude.
EXH_HD bool df_rounds_to_hi(DFloat g) {
  const unsigned hb = EXH_F_AS_U(g.hi) & 0x7fffffffu;
  if (hb < 0x0c800000u) return false;                            // |g| < 2^-102: decide in FP64
  const float ulp = EXH_U_AS_F((hb & 0x7f800000u) - (23u << 23));
  const float half_up = EXH_FMUL(ulp, 0.5f);
  const float half_down = (hb & 0x007fffffu) ? half_up : EXH_FMUL(ulp, 0.25f);
  const float margin = EXH_FMUL(EXH_U_AS_F(hb), 1.4551915228366852e-11f);     // 2^-36 |g|
  const float alo = EXH_U_AS_F(EXH_F_AS_U(g.lo) & 0x7fffffffu);
  const bool up = ((EXH_F_AS_U(g.lo) ^ EXH_F_AS_U(g.hi)) >> 31) == 0u;       // lo adds to |hi|
  return up ? alo < EXH_FSUB(half_up, margin) : alo < EXH_FSUB(half_down, margin);
}

// The float deviate of the accepted pair, or *undecided = 1 when the
// double-float value lies too close to a float rounding boundary or r2 lies
// within 2^-12 of 1 (the caller then forms it in FP64).  y = 0 gives +0.
EXH_HD float polar_deviate_f32(unsigned v1, unsigned v2, const float* lnc, const float* invc, int* undecided) {
  *undecided = 0;
  const long long a = (long long)v1 - 2147483648LL, b = (long long)v2 - 2147483648LL;
  if (b == 0) return 0.0f;
  const unsigned long long S = (unsigned long long)(a * a) + (unsigned long long)(b * b);
  if (S > (1ull << 62) - (1ull << 50) || S < (1ull << 20)) {     // 1 - r2 < 2^-12 or r2 < 2^-42: FP64 decides
    *undecided = 1;
    return 0.0f;
  }
  const DFloat g = polar_deviate_df(v1, v2, lnc, invc);
  if (!df_rounds_to_hi(g)) *undecided = 1;
  return g.hi;
}

// next(): the stream's next raw value
template <class Next>
EXH_HD unsigned next_nonzero(Next& next) {
  unsigned v = next();
  for (int t = 0; t < 64 && v == 0u; t++) v = next();   // longer zero runs do not occur; keeps the loop finite
  return v;
}

// One chunk of n raw values (n even): its zeros and its accepted pairs for
// either parity of the filtered index at its start (parity 1: the first
// non-zero value ends the previous chunk's pair).  The pair left open at the
// end takes the next non-zero value after the chunk.
template <class Next>
EXH_HD void polar_chunk_count(Next& next, int n, unsigned* zeros, unsigned* acc0, unsigned* acc1) {
  unsigned nz = 0, z = 0, c0 = 0, c1 = 0, first0 = 0, first1 = 0;
  for (int t = 0; t < n; t++) {
    const unsigned v = next();
    if (v == 0u) { z++; continue; }
    if ((nz & 1u) == 0u) {
      if (nz > 0u) c1 += polar_accept(first1, v);
      first0 = v;
    } else {
      c0 += polar_accept(first0, v);
      first1 = v;
    }
    nz++;
  }
  if (nz > 0u) {
    const unsigned v = next_nonzero(next);
    if (nz & 1u) c0 += polar_accept(first0, v);
    else c1 += polar_accept(first1, v);
  }
  *zeros = z;
  *acc0 = c0;
  *acc1 = c1;
}

// The same chunk's accepted pairs in order, for the parity `par` it has:
// emit(first, second) for each.
template <class Next, class Emit>
EXH_HD void polar_chunk_pairs(Next& next, int n, unsigned par, Emit& emit) {
  unsigned nz = 0, first = 0;
  bool open = false;
  for (int t = 0; t < n; t++) {
    const unsigned v = next();
    if (v == 0u) continue;
    if (((nz + par) & 1u) == 0u) {
      first = v;
      open = true;
    } else if (open) {
      if (polar_accept(first, v) && !emit(first, v)) return;
      open = false;
    }
    nz++;
  }
  if (open) {
    const unsigned v = next_nonzero(next);
    if (polar_accept(first, v)) emit(first, v);
  }
}

}  // namespace exh
