// Double-float ("float-float") arithmetic on the FP32 pipe.
//
// A value is an unevaluated sum h + l of two floats.  The building blocks are the
// error-free transformations TwoSum (Knuth, TAOCP vol. 2, 4.2.2), Fast2Sum
// (Dekker, Numer. Math. 18, 1971) and TwoProduct by FMA; the dot-product
// accumulation is the compensated Dot2 of Ogita, Rump & Oishi (SIAM J. Sci.
// Comput. 26, 2005).  Results carry about 44-48 significant bits, which is what
// the B/F kernels need where the reference computes in double: the refinement
// residual c - C b, the likelihood residuals (I - B) V, and the per-warp sums.
// GB300 retires FP64 at about 1/64 of the FP32 rate, so a handful of float
// instructions is far cheaper than one double instruction.
//
// The _rn intrinsics keep the compiler from contracting or reassociating the
// transformations (they are only exact in IEEE round-to-nearest).
#pragma once
#include <cuda_runtime.h>

namespace nngp_df {

struct df {
  float h, l;
};

// s + e = a + b exactly (any magnitudes).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bv = __fsub_rn(s, a);
  const float av = __fsub_rn(s, bv);
  e = __fadd_rn(__fsub_rn(a, av), __fsub_rn(b, bv));
}
// s + e = a - b exactly.
__device__ __forceinline__ void two_diff(float a, float b, float &s, float &e) {
  s = __fsub_rn(a, b);
  const float bv = __fsub_rn(s, a);
  const float av = __fsub_rn(s, bv);
  e = __fsub_rn(__fsub_rn(a, av), __fadd_rn(b, bv));
}
// s + e = a + b exactly when |a| >= |b| (or a == 0).
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
// hi + lo += x * y, the product's rounding error carried (Dot2 step).
__device__ __forceinline__ void dot2_acc(float &hi, float &lo, float x, float y) {
  const float p = __fmul_rn(x, y);
  const float pe = __fmaf_rn(x, y, -p);
  float q;
  two_sum(hi, p, hi, q);
  lo = __fadd_rn(lo, __fadd_rn(q, pe));
}
// normalised h + l (|l| <= ulp(h) / 2) from any pair
__device__ __forceinline__ df norm(float h, float l) {
  df r;
  two_sum(h, l, r.h, r.l);
  return r;
}
__device__ __forceinline__ df add(df a, df b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  df r;
  fast_two_sum(s, e, r.h, r.l);
  return r;
}
__device__ __forceinline__ df sub(df a, df b) {
  float s, e;
  two_diff(a.h, b.h, s, e);
  e = __fadd_rn(e, __fsub_rn(a.l, b.l));
  df r;
  fast_two_sum(s, e, r.h, r.l);
  return r;
}
__device__ __forceinline__ df mul(df a, df b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));
  df r;
  fast_two_sum(p, e, r.h, r.l);
  return r;
}
// 1 / a: float reciprocal plus one Newton correction carried in the low part
__device__ __forceinline__ df recip(df a) {
  const float x = __frcp_rn(a.h);
  float e = __fmaf_rn(-a.h, x, 1.0f);  // exact: 1 - a.h x
  e = __fmaf_rn(-a.l, x, e);
  df r;
  fast_two_sum(x, __fmul_rn(e, x), r.h, r.l);
  return r;
}
// double <-> df (FP64 pipe: keep out of per-neighbor loops)
__device__ __forceinline__ df from_double(double v) {
  df r;
  r.h = __double2float_rn(v);
  r.l = __double2float_rn(v - (double)r.h);
  return r;
}
__device__ __forceinline__ double to_double(df a) { return (double)a.h + (double)a.l; }

// log(a.h + a.l) for a.h > 0 (normal range), absolute error <= 3e-8: the exponent part
// e ln2 is carried exactly (ln2 split into a 14-bit head and a tail), log of the mantissa
// in [sqrt(1/2), sqrt(2)) comes from logf (|log m| < 0.35, so its 1-ulp bound is < 2.1e-8
// absolute), and the low part enters as a.l / a.h (|a.l / a.h| < 2^-23, so the omitted
// log1p terms are below 2^-47).
__device__ __forceinline__ df log(df a) {
  const int bits = __float_as_int(a.h);
  int e = ((bits >> 23) & 0xff) - 127;
  float mant = __int_as_float((bits & 0x007fffff) | 0x3f800000);  // [1, 2)
  if (mant > 1.41421356f) {
    mant = __fmul_rn(mant, 0.5f);
    e += 1;
  }
  const float ef = (float)e;
  constexpr float kLn2Hi = 0.693145751953125f;        // 0x3f317200: 14 significant bits
  constexpr float kLn2Lo = 1.4286068202862268e-06f;   // ln 2 - kLn2Hi
  const float lm = logf(mant);
  const float tail = __fadd_rn(lm, __fmaf_rn(ef, kLn2Lo, __fdividef(a.l, a.h)));
  return norm(__fmul_rn(ef, kLn2Hi), tail);
}

// ------------------------------------------------------------------ exp and sqrt
// 2^(j/32), j = 0..31, as double-float pairs (hi, lo).
static __constant__ float2 kExp2Tab[32] = {
    {1.0f, 0.0f},
    {1.0218971967697144f, -4.811559861650494e-08f},
    {1.0442737340927124f, 4.8334701574503924e-08f},
    {1.0671404600143433f, -5.9337519786595294e-08f},
    {1.0905077457427979f, -1.3077539939843064e-08f},
    {1.114386796951294f, -5.435540018083884e-08f},
    {1.1387885808944702f, 5.386222312608879e-08f},
    {1.1637248992919922f, -4.051441493402308e-08f},
    {1.1892070770263672f, 3.797635272917432e-08f},
    {1.215247392654419f, -3.267394887984665e-08f},
    {1.2418577671051025f, 4.496838101886169e-08f},
    {1.2690509557724f, 1.419333317542737e-09f},
    {1.2968395948410034f, -4.018999533172973e-08f},
    {1.3252366781234741f, -3.496373324196611e-08f},
    {1.3542555570602417f, -1.0123349269974824e-08f},
    {1.3839099407196045f, -5.875577357983275e-08f},
    {1.4142135381698608f, 2.4203234971764687e-08f},
    {1.4451807737350464f, 3.324199937537742e-08f},
    {1.4768261909484863f, -4.500898853621038e-08f},
    {1.5091644525527954f, -2.4959373234878512e-08f},
    {1.5422108173370361f, 8.070904833346049e-09f},
    {1.5759809017181396f, -5.661025426206834e-08f},
    {1.610490322113037f, 9.836217174097328e-09f},
    {1.6457555294036865f, -5.124972091152813e-08f},
    {1.6817928552627563f, -2.4755326677450284e-08f},
    {1.7186193466186523f, -4.8496175963919086e-08f},
    {1.7562521696090698f, -9.235770370707996e-09f},
    {1.7947090864181519f, -1.141504490931311e-08f},
    {1.8340080976486206f, -1.1239277952768134e-08f},
    {1.8741676807403564f, -4.663005626071026e-08f},
    {1.9152065515518188f, 9.845328108326612e-09f},
    {1.9571441411972046f, -1.7021804410433106e-08f}};
constexpr float kLn2Over32Hi = 0.021660849452018738f;
constexpr float kLn2Over32Lo = -5.952044412893542e-11f;

// scale * e^(u ln2 / 32) for u = uh + ul <= 0, relative error about 2e-13 (Tang's table-driven
// method, ACM TOMS 15(2), 1989, carried in double-float): u = 32 k + j + r', the table holds
// scale * 2^(j/32) (tab[j] hi, tab[32 + j] lo; the caller folds in its scale), e^r for
// |r| <= ln2/64 is 1 + r + r^2/2 exactly in double-float plus a float tail of degree 3-5.
// Arguments below -1846 (e^-40) are clamped there: below the resolution of every sum.
__device__ __forceinline__ df exp_u(float uh, float ul, const float *tab) {
  uh = fmaxf(uh, -1846.0f);  // e^-40 and below: clamped (a value of 4e-18 sigma^2)
  const float nf = rintf(uh);
  const int n = (int)nf;
  float ruh, rul;
  fast_two_sum(__fsub_rn(uh, nf), ul, ruh, rul);  // uh - nf is exact
  // r = ru * ln2/32 in double-float (rh, rl), |rl| about 2^-23 |rh| at most
  const float rh = __fmul_rn(ruh, kLn2Over32Hi);
  const float rl = __fmaf_rn(ruh, kLn2Over32Lo, __fmaf_rn(rul, kLn2Over32Hi, __fmaf_rn(ruh, kLn2Over32Hi, -rh)));
  const float q = __fmul_rn(rh, rh), qe = __fmaf_rn(rh, rh, -q);
  float poly = __fmaf_rn(rh, 1.0f / 120.0f, 1.0f / 24.0f);
  poly = __fmaf_rn(rh, poly, 1.0f / 6.0f);
  const float tail = __fmaf_rn(__fmul_rn(q, rh), poly, __fmaf_rn(rh, rl, __fmaf_rn(0.5f, qe, rl)));
  float s, e, s2, e2;
  fast_two_sum(1.0f, rh, s, e);
  two_sum(s, __fmul_rn(0.5f, q), s2, e2);
  const df E{s2, __fadd_rn(__fadd_rn(e, e2), tail)};  // |E.l| < 2^-22 |E.h|
  const int j = n & 31, k = n >> 5;  // k >= -58: 2^k is a normal float
  const df R = mul(E, df{tab[j], tab[32 + j]});
  const float sc = __int_as_float((k + 127) << 23);
  return df{__fmul_rn(R.h, sc), __fmul_rn(R.l, sc)};
}

// x^2 + y^2 for normalised double-float x, y (the lo * lo terms are below 2^-48 relative)
__device__ __forceinline__ df sumsq(float xh, float xl, float yh, float yl) {
  const float p1 = __fmul_rn(xh, xh);
  float e1 = __fmaf_rn(xh, xh, -p1);
  e1 = __fmaf_rn(__fadd_rn(xh, xh), xl, e1);
  const float p2 = __fmul_rn(yh, yh);
  float e2 = __fmaf_rn(yh, yh, -p2);
  e2 = __fmaf_rn(__fadd_rn(yh, yh), yl, e2);
  float s, q;
  two_sum(p1, p2, s, q);
  df r;
  fast_two_sum(s, __fadd_rn(__fadd_rn(q, e1), e2), r.h, r.l);
  return r;
}

// sqrt(a) for a >= 0: float estimate and one Newton correction carried in the low part
__device__ __forceinline__ df sqrt(df a) {
  if (!(a.h > 0.0f)) return df{0.0f, 0.0f};
  const float rs = rsqrtf(a.h);
  const float y = __fmul_rn(a.h, rs);
  const float yy = __fmul_rn(y, y), yye = __fmaf_rn(y, y, -yy);
  const float num = __fadd_rn(__fsub_rn(__fsub_rn(a.h, yy), yye), a.l);  // a.h - yy is exact
  df r;
  fast_two_sum(y, __fmul_rn(num, __fmul_rn(0.5f, rs)), r.h, r.l);
  return r;
}

// (a - b) for double-float coordinates given as (hi, lo) floats, normalised
__device__ __forceinline__ df diff(float ah, float al, float bh, float bl) {
  float s, e;
  two_diff(ah, bh, s, e);
  df r;
  fast_two_sum(s, __fadd_rn(e, __fsub_rn(al, bl)), r.h, r.l);
  return r;
}

}  // namespace nngp_df

// ------------------------------------------------------------ packed pairs (f32x2)
// Two independent double-float computations in lockstep: each 64-bit register holds one float
// of each (Blackwell's packed FP32 add/sub/mul/fma, round to nearest, issue one instruction
// for both).  The error-free transformations are the scalar ones above, applied per half.
namespace nngp_df2 {

typedef unsigned long long p2;  // (lo half, hi half) = (first computation, second)

__device__ __forceinline__ p2 pack(float a, float b) {
  p2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float first(p2 a) {
  float x, y;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(a));
  return x;
}
__device__ __forceinline__ float second(p2 a) {
  float x, y;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(a));
  return y;
}
__device__ __forceinline__ p2 add(p2 a, p2 b) {
  p2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ p2 sub(p2 a, p2 b) {
  p2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ p2 mul(p2 a, p2 b) {
  p2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ p2 fma(p2 a, p2 b, p2 c) {
  p2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__device__ __forceinline__ p2 neg(p2 a) { return a ^ 0x8000000080000000ull; }
__device__ __forceinline__ p2 splat(float a) { return pack(a, a); }

struct df2 {
  p2 h, l;
};

__device__ __forceinline__ void two_sum(p2 a, p2 b, p2 &s, p2 &e) {
  s = add(a, b);
  const p2 bv = sub(s, a);
  const p2 av = sub(s, bv);
  e = add(sub(a, av), sub(b, bv));
}
__device__ __forceinline__ void fast_two_sum(p2 a, p2 b, p2 &s, p2 &e) {
  s = add(a, b);
  e = sub(b, sub(s, a));
}
// (a.h + a.l) + (b.h + b.l), normalised (the scalar add, per half)
__device__ __forceinline__ df2 add(df2 a, df2 b) {
  p2 s, e;
  two_sum(a.h, b.h, s, e);
  e = add(e, add(a.l, b.l));
  df2 r;
  fast_two_sum(s, e, r.h, r.l);
  return r;
}
// (a.h + a.l)(b.h + b.l), normalised
__device__ __forceinline__ df2 mul(df2 a, df2 b) {
  const p2 p = mul(a.h, b.h);
  p2 e = fma(a.h, b.h, neg(p));
  e = fma(a.h, b.l, fma(a.l, b.h, e));
  df2 r;
  fast_two_sum(p, e, r.h, r.l);
  return r;
}
// x^2 + y^2 for normalised double-float x, y
__device__ __forceinline__ df2 sumsq(df2 x, df2 y) {
  const p2 p1 = mul(x.h, x.h);
  p2 e1 = fma(x.h, x.h, neg(p1));
  e1 = fma(add(x.h, x.h), x.l, e1);
  const p2 p2_ = mul(y.h, y.h);
  p2 e2 = fma(y.h, y.h, neg(p2_));
  e2 = fma(add(y.h, y.h), y.l, e2);
  p2 s, q;
  two_sum(p1, p2_, s, q);
  df2 r;
  fast_two_sum(s, add(add(q, e1), e2), r.h, r.l);
  return r;
}
// sqrt(a) for a >= 0 (0 at 0): float estimate and one Newton correction in the low part
__device__ __forceinline__ df2 sqrt(df2 a) {
  const p2 rs = pack(rsqrtf(fmaxf(first(a.h), 1e-37f)), rsqrtf(fmaxf(second(a.h), 1e-37f)));
  const p2 y = mul(a.h, rs);
  const p2 yy = mul(y, y), yye = fma(y, y, neg(yy));
  const p2 num = add(sub(sub(a.h, yy), yye), a.l);  // a.h - yy is exact
  df2 r;
  fast_two_sum(y, mul(num, mul(splat(0.5f), rs)), r.h, r.l);
  return r;
}

// Dot2 step on both halves: hi + lo += x * y (each half its own compensated sum)
__device__ __forceinline__ void dot2_acc(p2 &hi, p2 &lo, p2 x, p2 y) {
  const p2 p = mul(x, y);
  const p2 pe = fma(x, y, neg(p));
  p2 q;
  two_sum(hi, p, hi, q);
  lo = add(lo, add(q, pe));
}
// The two halves of a packed compensated sum added into one double-float (hi exact, lo
// rounded: the result carries the accuracy of either half)
__device__ __forceinline__ nngp_df::df fold(p2 hi, p2 lo) {
  float s, e;
  nngp_df::two_sum(first(hi), second(hi), s, e);
  return nngp_df::df{s, __fadd_rn(e, __fadd_rn(first(lo), second(lo)))};
}

// The scalar exp_u of nngp_df (Tang's table-driven exp in double-float) for two arguments:
// scale * e^(u ln2/32), u <= 0, the table tab[j] = scale 2^(j/32) (hi at j, lo at 32 + j).
__device__ __forceinline__ df2 exp_u(df2 u, const float *tab) {
  const float u0 = fmaxf(first(u.h), -1846.0f), u1 = fmaxf(second(u.h), -1846.0f);
  const float n0f = rintf(u0), n1f = rintf(u1);
  const int n0 = (int)n0f, n1 = (int)n1f;
  p2 ruh, rul;
  fast_two_sum(sub(pack(u0, u1), pack(n0f, n1f)), u.l, ruh, rul);
  const p2 c1h = splat(nngp_df::kLn2Over32Hi), c1l = splat(nngp_df::kLn2Over32Lo);
  const p2 rh = mul(ruh, c1h);
  const p2 rl = fma(ruh, c1l, fma(rul, c1h, fma(ruh, c1h, neg(rh))));
  const p2 q = mul(rh, rh), qe = fma(rh, rh, neg(q));
  p2 poly = fma(rh, splat(1.0f / 120.0f), splat(1.0f / 24.0f));
  poly = fma(rh, poly, splat(1.0f / 6.0f));
  const p2 tail = fma(mul(q, rh), poly, fma(rh, rl, fma(splat(0.5f), qe, rl)));
  p2 s, e, s2, e2;
  fast_two_sum(splat(1.0f), rh, s, e);
  two_sum(s, mul(splat(0.5f), q), s2, e2);
  const df2 E{s2, add(add(e, e2), tail)};
  const int j0 = n0 & 31, j1 = n1 & 31, k0 = n0 >> 5, k1 = n1 >> 5;
  const df2 T{pack(tab[j0], tab[j1]), pack(tab[32 + j0], tab[32 + j1])};
  const df2 R = mul(E, T);
  const p2 sc = pack(__int_as_float((k0 + 127) << 23), __int_as_float((k1 + 127) << 23));
  return df2{mul(R.h, sc), mul(R.l, sc)};
}

}  // namespace nngp_df2
