#pragma once
#include "common.cuh"
#include "dfloat.cuh"

// Scalar arithmetic shared by the update and QR kernels.  ArD: FP64 complex (the
// plain form: ratios must agree with an FP64 reference to ~1e-10 even where
// 1 + Delta (1 - G_jj) cancels).  ArF: double-float on the FP32 pipes (the mixed
// form; dfloat.cuh).  Z is a complex value, R a real one; both types are 16 and
// 8 bytes in either arithmetic, so shared-memory layouts do not change.
struct ArD {
  typedef zd Z;
  typedef double R;
  static constexpr bool kDoubleFloat = false;
  static ALF_DEV Z mk(zd a) { return a; }
  static ALF_DEV zd wide(Z a) { return a; }
  static ALF_DEV R mkr(double a) { return a; }
  static ALF_DEV Z one() { return zmk(1.0, 0.0); }
  static ALF_DEV Z zero() { return zmk(0.0, 0.0); }
  static ALF_DEV Z mul(Z a, Z b) { return zmul(a, b); }
  static ALF_DEV Z sub(Z a, Z b) { return zsub(a, b); }
  static ALF_DEV Z add(Z a, Z b) { return zadd(a, b); }
  static ALF_DEV Z neg(Z a) { return zmk(-a.x, -a.y); }
  static ALF_DEV Z mac(Z c, Z a, Z b) { return zfma(a, b, c); }
  static ALF_DEV Z scale(Z a, R s) { return zscale(a, s); }
  static ALF_DEV R re_mul(Z a, Z b) { return a.x * b.x - a.y * b.y; }
  static ALF_DEV R re(Z a) { return a.x; }
  static ALF_DEV R absr(R a) { return fabs(a); }
  static ALF_DEV R mulr(R a, R b) { return a * b; }
  static ALF_DEV bool gt(R a, R b) { return a > b; }
  // 1/d, d > 0 real: float seed, two Newton-Raphson steps r <- r + r (1 - d r) (quadratic
  // convergence, 2^-24 -> 2^-48 -> below 2^-53); an FP64 division costs ~560 cycles here.
  static ALF_DEV double rcp_pos(double d) {
    if (!(d > 1e-30 && d < 1e30)) return 1.0 / d;
    double r = (double)__frcp_rn(__double2float_rn(d));
    r = fma(r, fma(-d, r, 1.0), r);
    return fma(r, fma(-d, r, 1.0), r);
  }
  static ALF_DEV Z rcp(Z a) {
    const double s = rcp_pos(a.x * a.x + a.y * a.y);
    return zmk(a.x * s, -a.y * s);
  }
  // FP64 range holds the unnormalised phase of a block (<= 32 ratio factors); it is
  // normalised once at block end
  static ALF_DEV Z renorm(Z a) { return a; }
  static ALF_DEV zd unit(Z a) { const double r = sqrt(a.x * a.x + a.y * a.y); return zmk(a.x / r, a.y / r); }
  static ALF_DEV Z shfl(Z a, int src) {
    return zmk(__shfl_sync(0xffffffffu, a.x, src), __shfl_sync(0xffffffffu, a.y, src));
  }
  static ALF_DEV Z shfl_xor(Z a, int o) {
    return zmk(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
  }
  static ALF_DEV Z conj(Z a) { return zmk(a.x, -a.y); }
  static ALF_DEV Z mkz(R r, R i) { return zmk(r, i); }
  static ALF_DEV R im(Z a) { return a.y; }
  static ALF_DEV R abs2(Z a) { return a.x * a.x + a.y * a.y; }
  static ALF_DEV R rzero() { return 0.0; }
  static ALF_DEV R radd(R a, R b) { return a + b; }
  static ALF_DEV R rsub(R a, R b) { return a - b; }
  static ALF_DEV R rneg(R a) { return -a; }
  static ALF_DEV R rsqrt_(R a) { return sqrt(a); }
  static ALF_DEV R rrcp(R a) {
    const double m = fabs(a);
    if (!(m > 1e-30 && m < 1e30)) return 1.0 / a;
    double r = (double)__frcp_rn(__double2float_rn(a));
    r = fma(r, fma(-a, r, 1.0), r);
    return fma(r, fma(-a, r, 1.0), r);
  }
  static ALF_DEV R rmax0(R a) { return a > 0.0 ? a : 0.0; }
  static ALF_DEV bool rzero_p(R a) { return a == 0.0; }
  static ALF_DEV bool rneg_p(R a) { return a < 0.0; }
  static ALF_DEV double rwide(R a) { return a; }
  static ALF_DEV R rcopysign(R mag, R sgn) { return copysign(mag, sgn); }
  static ALF_DEV R rshfl_xor(R a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
};
struct ArF {
  typedef dfz Z;
  typedef dff R;
  static constexpr bool kDoubleFloat = true;
  static ALF_DEV Z mk(zd a) { return dz_make(a); }
  static ALF_DEV zd wide(Z a) { return dz_wide(a); }
  static ALF_DEV R mkr(double a) { return df_make(a); }
  static ALF_DEV Z one() { return dfz{{1.f, 0.f}, {0.f, 0.f}}; }
  static ALF_DEV Z zero() { return dfz{{0.f, 0.f}, {0.f, 0.f}}; }
  static ALF_DEV Z mul(Z a, Z b) { return dz_mul(a, b); }
  static ALF_DEV Z sub(Z a, Z b) { return dz_sub(a, b); }
  static ALF_DEV Z add(Z a, Z b) { return dz_add(a, b); }
  static ALF_DEV Z neg(Z a) { return dfz{df_neg(a.r), df_neg(a.i)}; }
  static ALF_DEV Z mac(Z c, Z a, Z b) { return dz_mac(c, a, b); }
  static ALF_DEV Z scale(Z a, R s) { return dz_scale(a, s); }
  static ALF_DEV R re_mul(Z a, Z b) { return df_dot2(a.r, b.r, df_neg(a.i), b.i); }
  static ALF_DEV R re(Z a) { return a.r; }
  static ALF_DEV R absr(R a) { return df_abs(a); }
  static ALF_DEV R mulr(R a, R b) { return df_mul(a, b); }
  static ALF_DEV bool gt(R a, R b) { return df_gt(a, b); }
  static ALF_DEV Z rcp(Z a) { return dz_rcp(a); }
  static ALF_DEV Z renorm(Z a) {
    const float m2 = a.r.h * a.r.h + a.i.h * a.i.h;
    return (m2 > 0.f && m2 < 3e38f) ? dz_scale(a, df_f(rsqrtf(m2))) : a;
  }
  static ALF_DEV zd unit(Z a) { return dz_wide(dz_unit(a)); }
  static ALF_DEV Z shfl(Z a, int src) {
    Z r;
    r.r.h = __shfl_sync(0xffffffffu, a.r.h, src); r.r.l = __shfl_sync(0xffffffffu, a.r.l, src);
    r.i.h = __shfl_sync(0xffffffffu, a.i.h, src); r.i.l = __shfl_sync(0xffffffffu, a.i.l, src);
    return r;
  }
  static ALF_DEV Z shfl_xor(Z a, int o) {
    Z r;
    r.r.h = __shfl_xor_sync(0xffffffffu, a.r.h, o); r.r.l = __shfl_xor_sync(0xffffffffu, a.r.l, o);
    r.i.h = __shfl_xor_sync(0xffffffffu, a.i.h, o); r.i.l = __shfl_xor_sync(0xffffffffu, a.i.l, o);
    return r;
  }
  static ALF_DEV Z conj(Z a) { return dz_conj(a); }
  static ALF_DEV Z mkz(R r, R i) { return dfz{r, i}; }
  static ALF_DEV R im(Z a) { return a.i; }
  static ALF_DEV R abs2(Z a) { return dz_abs2(a); }
  static ALF_DEV R rzero() { return dff{0.f, 0.f}; }
  static ALF_DEV R radd(R a, R b) { return df_add(a, b); }
  static ALF_DEV R rsub(R a, R b) { return df_sub(a, b); }
  static ALF_DEV R rneg(R a) { return df_neg(a); }
  static ALF_DEV R rsqrt_(R a) { return df_sqrt(a); }
  static ALF_DEV R rrcp(R a) { return df_rcp(a); }
  static ALF_DEV R rmax0(R a) { return a.h > 0.f ? a : dff{0.f, 0.f}; }
  static ALF_DEV bool rzero_p(R a) { return a.h == 0.f && a.l == 0.f; }
  static ALF_DEV bool rneg_p(R a) { return a.h < 0.f; }
  static ALF_DEV double rwide(R a) { return df_wide(a); }
  static ALF_DEV R rcopysign(R mag, R sgn) { return ((mag.h < 0.f) != (sgn.h < 0.f)) ? df_neg(mag) : mag; }
  static ALF_DEV R rshfl_xor(R a, int o) {
    return dff{__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o)};
  }
};

