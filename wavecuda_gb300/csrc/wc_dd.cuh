// Double-float ("float-float") arithmetic policy for the FP64 data path.
//
// GB300's FP64 pipe is a small fraction of its FP32 rate, so WC_F64_FAST keeps
// the data as FP64 in HBM but computes on the FP32 pipes with unevaluated
// float pairs (hi + lo).  The building blocks are the error-free transforms
// of Dekker (1971) and Knuth (TAOCP vol. 2, section 4.2.2): TwoSum,
// FastTwoSum and the FMA-based TwoProduct.  Filter taps c are split at
// compile time into (ch, cl) = (fl32(c), fl32(c - ch)).
//
// Dot products use the compensated scheme of Ogita, Rump and Oishi ("Dot2",
// SIAM J. Sci. Comput. 26(6), 2005): the high parts of the products are
// summed with TwoSum, every rounding error (product errors, cross terms
// xh*cl + xl*ch, sum errors) goes into one float, and the pair is
// renormalised once per output.  About 12 FP32 instructions per tap.  The
// DWT passes use the cheaper extraction scheme at the end of this file.
//
// Conversions never touch the FP64 pipe.  A double x = (-1)^s 2^e 1.f is
// split by bit manipulation: hi keeps the top 23 fraction bits (exact,
// truncated); the next 23 bits become lo through the implicit-bit trick
// lo = float(s, e-23, f') - float(s, e-23, 0), an exact FP32 subtraction.
// The split keeps 47 significant bits (relative error below 2^-46).  Values
// whose exponent is outside [-100, 127] take the generic path through the
// FP64 conversion instructions; magnitudes above the FP32 range are not
// representable in this precision (use WC_F64_EXACT for them).
// Back to FP64 by integer assembly as well (dd_to_double).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace wc {

struct dd {
  float hi, lo;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

// Generic conversions through the FP64 unit, kept out of line so that the
// hot paths below never issue an FP64 instruction (an inlined fallback would
// be predicated and executed for every element).
static __device__ __noinline__ dd dd_from_double_slow(double x) {
  if (x == 0.0) return {0.f, 0.f};
  const float hi = __double2float_rn(x);
  return {hi, __double2float_rn(x - (double)hi)};
}
static __device__ __noinline__ double dd_to_double_slow(float hi, float lo) {
  return (double)hi + (double)lo;
}

__device__ __forceinline__ dd dd_from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int lw = (unsigned int)b, hw = (unsigned int)(b >> 32);
  const unsigned int E = (hw >> 20) & 0x7FF;  // biased FP64 exponent
  // ef = E - 1023 + 127 must lie in [27, 254]: lo's exponent ef - 23 >= 1.
  // Zeros (common after thresholding) stay inline, as the generic path
  // converts them: (+0, +0).
  if (E - (1023u - 100u) > 227u) {
    if ((b << 1) == 0ull) return {0.f, 0.f};
    return dd_from_double_slow(x);
  }
  // Bits 29..60 of x hold the top 23 fraction bits and the low 9 exponent
  // bits; subtracting 896 from that exponent field modulo 2^9 leaves ef
  // (< 256, so bit 31 stays clear), and the sign goes into bit 31.
  const unsigned int hib = (__funnelshift_r(lw, hw, 29) - (384u << 23)) | (hw & 0x80000000u);
  // lo: the next 23 fraction bits (bits 6..28 of x) under exponent ef - 23,
  // minus the implicit bit of that exponent.
  const unsigned int baseb = (hib & 0xFF800000u) - (23u << 23);
  const unsigned int rb = (lw >> 6) & 0x7FFFFFu;
  return {__uint_as_float(hib), __fsub_rn(__uint_as_float(baseb | rb), __uint_as_float(baseb))};
}

// hi + lo as an FP64 value, assembled with integer operations: hi's 24-bit
// significand is placed at the top of a 53-bit one, lo's significand is
// shifted into place and added or subtracted, and one normalising shift
// fixes a carry or borrow.  lo's bits below the 53-bit window are
// truncated, an error below one FP64 ulp.  Any pair of finite floats.
static __device__ __noinline__ double dd_to_double_gen(unsigned int hb, unsigned int lb) {
  const unsigned int eh = (hb >> 23) & 0xFF, el = (lb >> 23) & 0xFF;
  if (eh == 0 || eh == 0xFF || el == 0xFF)
    return dd_to_double_slow(__uint_as_float(hb), __uint_as_float(lb));
  unsigned long long A = (unsigned long long)((hb & 0x7FFFFFu) | 0x800000u) << 29;
  if (el != 0) {
    const unsigned long long ml = (lb & 0x7FFFFFu) | 0x800000u;
    const int d = (int)eh - (int)el;
    unsigned long long B;
    if (d <= 29) B = ml << (29 - d);
    else B = (d - 29 < 64) ? (ml >> (d - 29)) : 0ull;
    A = ((hb ^ lb) & 0x80000000u) ? A - B : A + B;
  }
  int e = (int)eh + (1023 - 127);
  if (A >> 53) {
    A >>= 1;
    e++;
  } else if (!(A >> 52)) {
    A <<= 1;
    e--;
  }
  const unsigned long long bits = ((unsigned long long)(hb & 0x80000000u) << 32) |
                                  ((unsigned long long)e << 52) | (A & ((1ull << 52) - 1));
  return __longlong_as_double((long long)bits);
}

// The same value, branch-free for the pairs the arithmetic produces (hi
// normal, lo zero, subnormal or at least 24 binades below hi, i.e. |lo| at
// most about half an ulp of hi): double(hi) by moving its fields, then lo
// counted in units of that double's ulp (truncated, as above) and added to
// the 64-bit pattern.  Adding cannot carry out of the 29 low bits, which
// double(hi) leaves zero; subtracting from a power-of-two hi borrows into
// the binade below, whose ulp is half as large, so the count is doubled
// there.  Bit-identical to dd_to_double_gen; other pairs go to it.
__device__ __forceinline__ double dd_to_double(dd v) {
  const unsigned int hb = __float_as_uint(v.hi), lb = __float_as_uint(v.lo);
  const unsigned int eh = (hb >> 23) & 0xFF, el = (lb >> 23) & 0xFF;
  if (eh - 1u > 253u || el == 0xFFu || (el != 0u && eh < el + 24u)) return dd_to_double_gen(hb, lb);
  const unsigned int hw = (hb & 0x80000000u) | (((hb & 0x7FFFFFFFu) >> 3) + (896u << 20));
  const unsigned int lw = hb << 29;
  const unsigned int ml = el ? ((lb & 0x7FFFFFu) | 0x800000u) : 0u;
  const int sh = (int)eh - (int)el - 29;  // >= -5
  unsigned int k = (sh <= 0) ? (ml << (-sh)) : (sh < 32 ? (ml >> sh) : 0u);
  const bool neg = ((hb ^ lb) & 0x80000000u) != 0u;
  if (neg && (hb & 0x7FFFFFu) == 0u) k <<= 1;
  const unsigned long long b = ((unsigned long long)hw << 32) | lw;
  return __longlong_as_double((long long)(neg ? b - k : b + k));
}

struct dd_acc {
  float s, e;
};

struct PDD {
  using T = double;
  using V = dd;
  using Acc = dd_acc;
  static __device__ __forceinline__ V ld(T x) { return dd_from_double(x); }
  static __device__ __forceinline__ T st(V v) { return dd_to_double(v); }

  static __device__ __forceinline__ Acc acc_init(V a, double c) {
    const float ch = (float)c;
    const float cl = (float)(c - (double)ch);
    const float p = __fmul_rn(a.hi, ch);
    float e = __fmaf_rn(a.hi, ch, -p);
    e = __fmaf_rn(a.hi, cl, e);
    e = __fmaf_rn(a.lo, ch, e);
    return {p, e};
  }
  static __device__ __forceinline__ Acc acc_add(Acc A, V a, double c) {
    const float ch = (float)c;
    const float cl = (float)(c - (double)ch);
    const float p = __fmul_rn(a.hi, ch);
    float pe = __fmaf_rn(a.hi, ch, -p);
    pe = __fmaf_rn(a.hi, cl, pe);
    pe = __fmaf_rn(a.lo, ch, pe);
    float s, t;
    two_sum(A.s, p, s, t);
    return {s, __fadd_rn(A.e, __fadd_rn(pe, t))};
  }
  static __device__ __forceinline__ V acc_fin(Acc A) {
    V r;
    two_sum(A.s, A.e, r.hi, r.lo);
    return r;
  }

  static __device__ __forceinline__ V mul(V a, double c) { return acc_fin(acc_init(a, c)); }
  static __device__ __forceinline__ V add(V a, V b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    V r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
  }
  static __device__ __forceinline__ V sub(V a, V b) { return add(a, {-b.hi, -b.lo}); }
  static __device__ __forceinline__ V madd(V acc, V a, double c) { return add(acc, mul(a, c)); }
  static __device__ __forceinline__ V half(V a) { return {a.hi * 0.5f, a.lo * 0.5f}; }
};

// ---------------------------------------------------------------------------
// Two Dot2 accumulators advanced together.  The sm_100-family packed FP32
// instructions (add/sub/mul/fma .rn.f32x2) perform two IEEE FP32 operations
// in one issue slot with the rounding of the scalar ones, so two dot
// products of the same inputs with different taps -- a DWT level's scaling
// and detail outputs, or the even and odd outputs of an inverse step -- cost
// half the instructions of PDD::acc_* and give bit-identical pairs.
// Lane 0 carries the first accumulator, lane 1 the second.  The error part
// is kept negated (ne = -e), which lets every product error come from one
// FMA against the negated tap and is exact under round-to-nearest symmetry.

typedef unsigned long long f32x2;

__device__ __forceinline__ f32x2 x2_pack(float a, float b) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void x2_unpack(f32x2 v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f32x2 x2_add(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 x2_sub(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 x2_mul(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 x2_fma(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

struct dd_acc2 {
  f32x2 s, ne;  // running sum of the high products; negated error sum
};

// Tap pair (c0 for lane 0, c1 for lane 1) split as for PDD: ch = fl32(c),
// cl = fl32(c - ch).
struct tap2 {
  f32x2 ch, nch, ncl;
};
__device__ __forceinline__ tap2 make_tap2(double c0, double c1) {
  const float h0 = (float)c0, h1 = (float)c1;
  const float l0 = (float)(c0 - (double)h0), l1 = (float)(c1 - (double)h1);
  return {x2_pack(h0, h1), x2_pack(-h0, -h1), x2_pack(-l0, -l1)};
}

// p = a.hi*ch (both lanes); negated product error -(a.hi*ch - p) - a.hi*cl
// - a.lo*ch, accumulated as PDD::acc_init does (signs flipped).
__device__ __forceinline__ dd_acc2 acc2_init(dd a, const tap2& c) {
  const f32x2 ah = x2_pack(a.hi, a.hi), al = x2_pack(a.lo, a.lo);
  const f32x2 p = x2_mul(ah, c.ch);
  f32x2 ne = x2_fma(ah, c.nch, p);
  ne = x2_fma(ah, c.ncl, ne);
  ne = x2_fma(al, c.nch, ne);
  return {p, ne};
}

__device__ __forceinline__ dd_acc2 acc2_add(dd_acc2 A, dd a, const tap2& c) {
  const f32x2 ah = x2_pack(a.hi, a.hi), al = x2_pack(a.lo, a.lo);
  const f32x2 p = x2_mul(ah, c.ch);
  f32x2 npe = x2_fma(ah, c.nch, p);
  npe = x2_fma(ah, c.ncl, npe);
  npe = x2_fma(al, c.nch, npe);
  // TwoSum(A.s, p) = (s, t)
  const f32x2 s = x2_add(A.s, p);
  const f32x2 bb = x2_sub(s, A.s);
  const f32x2 t = x2_add(x2_sub(A.s, x2_sub(s, bb)), x2_sub(p, bb));
  // e' = e + (pe + t)  <=>  ne' = ne + (npe - t)
  return {s, x2_add(A.ne, x2_sub(npe, t))};
}

// Renormalised pairs: lane 0 -> r0, lane 1 -> r1 (PDD::acc_fin per lane).
__device__ __forceinline__ void acc2_fin(dd_acc2 A, dd& r0, dd& r1) {
  // TwoSum(s, e) with e = -ne: hi = s - ne; lo = (s - (hi - bb)) - (ne + bb)
  const f32x2 hi = x2_sub(A.s, A.ne);
  const f32x2 bb = x2_sub(hi, A.s);
  const f32x2 lo = x2_sub(x2_sub(A.s, x2_sub(hi, bb)), x2_add(A.ne, bb));
  float h0, h1, l0, l1;
  x2_unpack(hi, h0, h1);
  x2_unpack(lo, l0, l1);
  r0 = {h0, l0};
  r1 = {h1, l1};
}

// Two dot products with the same taps on different inputs (lane 0: input
// a0, lane 1: input a1), e.g. two adjacent outputs of a filter.  The tap is
// broadcast to both lanes.
__device__ __forceinline__ dd_acc2 acc2_init_xy(dd a0, dd a1, const tap2& c) {
  const f32x2 ah = x2_pack(a0.hi, a1.hi), al = x2_pack(a0.lo, a1.lo);
  const f32x2 p = x2_mul(ah, c.ch);
  f32x2 ne = x2_fma(ah, c.nch, p);
  ne = x2_fma(ah, c.ncl, ne);
  ne = x2_fma(al, c.nch, ne);
  return {p, ne};
}

__device__ __forceinline__ dd_acc2 acc2_add_xy(dd_acc2 A, dd a0, dd a1, const tap2& c) {
  const f32x2 ah = x2_pack(a0.hi, a1.hi), al = x2_pack(a0.lo, a1.lo);
  const f32x2 p = x2_mul(ah, c.ch);
  f32x2 npe = x2_fma(ah, c.nch, p);
  npe = x2_fma(ah, c.ncl, npe);
  npe = x2_fma(al, c.nch, npe);
  const f32x2 s = x2_add(A.s, p);
  const f32x2 bb = x2_sub(s, A.s);
  const f32x2 t = x2_add(x2_sub(A.s, x2_sub(s, bb)), x2_sub(p, bb));
  return {s, x2_add(A.ne, x2_sub(npe, t))};
}

// ---------------------------------------------------------------------------
// Two dot products by extraction (ExtractScalar of Rump, Ogita and Oishi,
// "Accurate floating-point summation, part I: faithful rounding", SIAM J.
// Sci. Comput. 31(1), 2008).  sigma is a power of two with
// sigma >= 2 * sum_k |a_k.hi * c_k| over both lanes' taps.  Then
// t = fl(sigma + a.hi*ch) (one FMA) lies in [sigma/2, 3 sigma/2], so
// q = t - sigma is exact (Sterbenz) and a multiple of 2^-24 sigma, and every
// partial sum of the q's stays below sigma in magnitude: the high parts add
// up in FP32 without rounding.  The residual a.hi*ch - q (one FMA, rounded
// once, |residual| <= 2^-24 sigma) and the cross terms a.hi*cl + a.lo*ch go
// into the error float, so the error is a few units of 2^-48 sigma: over
// random windows of an exact-rational emulation of these steps, a median of
// 1.2e-14 and a worst case of 2.6e-13 of sum |a*c| (Dot2: 1.4e-15 and
// 1.3e-14).  Seven packed instructions per tap against acc2_add's twelve.
struct dd_accx {
  f32x2 S, ne;  // exact sum of the extracted high parts; negated error sum
};

// Smallest power of two >= 2 * s (s >= 0; 0 for s == 0), in both lanes.
__device__ __forceinline__ f32x2 extract_sigma(float s) {
  const unsigned int b = __float_as_uint(__fmul_rn(s, 2.f));
  const float sg = __uint_as_float((b + 0x7FFFFFu) & 0xFF800000u);
  return x2_pack(sg, sg);
}

__device__ __forceinline__ dd_accx accx_init(f32x2 ah, f32x2 al, const tap2& c, f32x2 sig) {
  const f32x2 q = x2_sub(x2_fma(ah, c.ch, sig), sig);
  f32x2 ne = x2_fma(ah, c.nch, q);  // q - a.hi*ch
  ne = x2_fma(ah, c.ncl, ne);
  ne = x2_fma(al, c.nch, ne);
  return {q, ne};
}

__device__ __forceinline__ dd_accx accx_add(dd_accx A, f32x2 ah, f32x2 al, const tap2& c,
                                            f32x2 sig) {
  const f32x2 q = x2_sub(x2_fma(ah, c.ch, sig), sig);
  const f32x2 u = x2_fma(ah, c.nch, q);
  f32x2 ne = x2_fma(ah, c.ncl, A.ne);
  ne = x2_fma(al, c.nch, ne);
  return {x2_add(A.S, q), x2_add(ne, u)};
}

// Same input in both lanes (two filters applied to one window).
__device__ __forceinline__ dd_accx accx_init(dd a, const tap2& c, f32x2 sig) {
  return accx_init(x2_pack(a.hi, a.hi), x2_pack(a.lo, a.lo), c, sig);
}
__device__ __forceinline__ dd_accx accx_add(dd_accx A, dd a, const tap2& c, f32x2 sig) {
  return accx_add(A, x2_pack(a.hi, a.hi), x2_pack(a.lo, a.lo), c, sig);
}

__device__ __forceinline__ void accx_fin(dd_accx A, dd& r0, dd& r1) {
  acc2_fin(dd_acc2{A.S, A.ne}, r0, r1);
}

}  // namespace wc
