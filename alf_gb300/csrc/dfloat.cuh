// Double-float scalars for latency-bound serial chains.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// carrying ~2^-46 relative rounding per operation.  On GB300 a dependent FP64
// instruction costs 63-76 cycles and an FP64 division ~560 (one lane or 32),
// while a dependent FP32 FMA costs ~5 (measured with register-only FMA loops), so the
// per-visit Metropolis chain runs in this arithmetic.  Algorithms: Knuth's
// two-sum, Dekker's fast two-sum (|a| >= |b|), the FMA two-product, and one
// Newton step for the reciprocal and square root.  Products use __fmul_rn so
// that the compiler cannot contract them into a later addition.
#pragma once
#include "common.cuh"

struct dff {
  float h, l;
};
struct dfz {
  dff r, i;
};

ALF_DEV dff df_make(double x) {
  dff v;
  v.h = __double2float_rn(x);
  v.l = __double2float_rn(x - (double)v.h);
  return v;
}
ALF_DEV dff df_f(float x) { return dff{x, 0.f}; }
ALF_DEV double df_wide(dff a) { return (double)a.h + (double)a.l; }
ALF_DEV dfz dz_make(zd z) { return dfz{df_make(z.x), df_make(z.y)}; }
ALF_DEV zd dz_wide(dfz z) { return zmk(df_wide(z.r), df_wide(z.i)); }

ALF_DEV dff df_qts(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return dff{s, __fsub_rn(b, __fsub_rn(s, a))};
}
ALF_DEV dff df_ts(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return dff{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
ALF_DEV dff df_neg(dff a) { return dff{-a.h, -a.l}; }
ALF_DEV dff df_abs(dff a) { return a.h < 0.f ? df_neg(a) : a; }
ALF_DEV dff df_add(dff a, dff b) {
  dff s = df_ts(a.h, b.h);
  return df_qts(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
ALF_DEV dff df_sub(dff a, dff b) { return df_add(a, df_neg(b)); }
// error term of the product a*b beyond p = fl(a.h*b.h)
ALF_DEV float df_perr(dff a, dff b, float p) {
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  return fmaf(a.l, b.h, e);
}
ALF_DEV dff df_mul(dff a, dff b) {
  const float p = __fmul_rn(a.h, b.h);
  return df_qts(p, df_perr(a, b, p));
}
ALF_DEV dff df_mulf(dff a, float b) {
  const float p = __fmul_rn(a.h, b);
  return df_qts(p, fmaf(a.l, b, fmaf(a.h, b, -p)));
}
// a*b + c*d
ALF_DEV dff df_dot2(dff a, dff b, dff c, dff d) {
  const float p1 = __fmul_rn(a.h, b.h), p2 = __fmul_rn(c.h, d.h);
  const float e1 = df_perr(a, b, p1), e2 = df_perr(c, d, p2);
  dff s = df_ts(p1, p2);
  return df_qts(s.h, __fadd_rn(s.l, __fadd_rn(e1, e2)));
}
// z + a*b + c*d
ALF_DEV dff df_dot2acc(dff z, dff a, dff b, dff c, dff d) {
  const float p1 = __fmul_rn(a.h, b.h), p2 = __fmul_rn(c.h, d.h);
  const float e1 = df_perr(a, b, p1), e2 = df_perr(c, d, p2);
  dff s = df_ts(z.h, p1);
  dff t = df_ts(s.h, p2);
  return df_qts(t.h, __fadd_rn(__fadd_rn(t.l, s.l), __fadd_rn(z.l, __fadd_rn(e1, e2))));
}
ALF_DEV bool df_gt(dff a, dff b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }
// 1/a: correctly rounded float reciprocal, then one Newton correction in double-float
ALF_DEV dff df_rcp(dff a) {
  const float q = __frcp_rn(a.h);
  const float p = __fmul_rn(a.h, q);
  const float e = fmaf(a.h, q, -p);
  float r = __fsub_rn(__fsub_rn(1.0f, p), e);
  r = fmaf(-a.l, q, r);
  return df_qts(q, __fmul_rn(q, r));
}
// sqrt(a), a >= 0
ALF_DEV dff df_sqrt(dff a) {
  if (a.h <= 0.f) return dff{0.f, 0.f};
  const float s = __fsqrt_rn(a.h);
  const float p = __fmul_rn(s, s);
  const float e = fmaf(s, s, -p);
  const float res = __fadd_rn(__fsub_rn(__fsub_rn(a.h, p), e), a.l);
  return df_qts(s, __fdiv_rn(res, __fmul_rn(2.0f, s)));
}

ALF_DEV dfz dz_add(dfz a, dfz b) { return dfz{df_add(a.r, b.r), df_add(a.i, b.i)}; }
ALF_DEV dfz dz_sub(dfz a, dfz b) { return dfz{df_sub(a.r, b.r), df_sub(a.i, b.i)}; }
ALF_DEV dfz dz_mul(dfz a, dfz b) {
  return dfz{df_dot2(a.r, b.r, df_neg(a.i), b.i), df_dot2(a.r, b.i, a.i, b.r)};
}
// z + a*b
ALF_DEV dfz dz_mac(dfz z, dfz a, dfz b) {
  return dfz{df_dot2acc(z.r, a.r, b.r, df_neg(a.i), b.i), df_dot2acc(z.i, a.r, b.i, a.i, b.r)};
}
ALF_DEV dfz dz_scale(dfz a, dff s) { return dfz{df_mul(a.r, s), df_mul(a.i, s)}; }
ALF_DEV dff dz_abs2(dfz a) { return df_dot2(a.r, a.r, a.i, a.i); }
ALF_DEV dfz dz_conj(dfz a) { return dfz{a.r, df_neg(a.i)}; }
ALF_DEV dfz dz_rcp(dfz a) { return dz_scale(dz_conj(a), df_rcp(dz_abs2(a))); }
// a / |a| (a != 0)
ALF_DEV dfz dz_unit(dfz a) { return dz_scale(a, df_rcp(df_sqrt(dz_abs2(a)))); }
