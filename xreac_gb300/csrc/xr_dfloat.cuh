// Double-float arithmetic for FP64-accurate exponentials and logarithms on the FP32 pipe.
//
// GB300 issues FP32 at 64 times its FP64 rate, and the pair and bond-order kernels spend most of
// their FP64 issue on exp and log. A double-float (Dekker, "A floating-point technique for extending
// the available precision", Numer. Math. 18, 1971) holds a value as the unevaluated sum hi + lo of
// two floats with |lo| <= ulp(hi) / 2, 48 significant bits; sums and products use the error-free
// transformations TwoSum (Knuth, TAOCP vol. 2) and the FMA product error. Every operation is an
// explicitly rounded FP32 intrinsic (__fadd_rn, __fmul_rn, __fmaf_rn), which the compiler neither
// contracts nor reassociates, so the error terms stay exact.
//
// exp: Tang's table-driven reduction (ACM TOMS 15, 144-157, 1989), x = (64 n + j) ln2 / 64 + r with
// |r| <= ln2 / 128 (Cody-Waite: ln2 / 64 split so that the products with k are exact), the table
// 2^(j/64) as double-floats (relative error below 1.5e-15), exp(r) - 1 = r + r^2 (1/2 + r/6 + r^2/24 +
// r^3/120) (truncation below 4e-17), and the power 2^n applied to the FP64 result's exponent field. log: one Newton step on
// exp(y) = a from the FP32 logarithm y0: log a = y0 + t - t^2 / 2 with t = a exp(-y0) - 1 (|t| below
// 1e-5 for |log a| < 70, so the next term is below 1e-15 relative to log a). About 48 bits either way: the device test of these
// functions bounds them against CUDA's FP64 exp and log at 2e-14 (relative for exp, absolute for log).
//
// Domain: |x| < 80 for exp, arguments in [1e-30, 1e30] for log; outside it (and for non-finite input)
// both fall back to the FP64 functions.
#pragma once
#include <cuda_runtime.h>

struct xr_df {
  float hi, lo;
};

__device__ inline xr_df xr_df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

// |a| >= |b| (or a == 0)
__device__ inline xr_df xr_df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ inline xr_df xr_df_from_double(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}

__device__ inline xr_df xr_df_add(xr_df a, xr_df b) {
  xr_df s = xr_df_two_sum(a.hi, b.hi);
  const xr_df t = xr_df_two_sum(a.lo, b.lo);
  s = xr_df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return xr_df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}

__device__ inline xr_df xr_df_add_f(xr_df a, float b) {
  const xr_df s = xr_df_two_sum(a.hi, b);
  return xr_df_fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}

__device__ inline xr_df xr_df_mul(xr_df a, xr_df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return xr_df_fast_two_sum(p, e);
}

// 2^(j/64) as (hi, lo), j = 0..63
static __device__ const float2 xr_df_exp2_64[64] = {
    {0x1.0000000000000p+0f, 0x0.0p+0f}, {0x1.02c9a40000000p+0f, -0x1.887fa00000000p-28f},
    {0x1.059b0e0000000p+0f, -0x1.9d4f520000000p-25f}, {0x1.0874520000000p+0f, -0x1.e2990e0000000p-26f},
    {0x1.0b55860000000p+0f, 0x1.9f31220000000p-25f}, {0x1.0e3ec40000000p+0f, -0x1.a585cc0000000p-25f},
    {0x1.11301e0000000p+0f, -0x1.fdb4960000000p-25f}, {0x1.1429aa0000000p+0f, 0x1.d525bc0000000p-25f},
    {0x1.172b840000000p+0f, -0x1.c157420000000p-27f}, {0x1.1a35be0000000p+0f, 0x1.6df96e0000000p-25f},
    {0x1.1d48740000000p+0f, -0x1.d2e8ca0000000p-25f}, {0x1.2063b80000000p+0f, 0x1.0c519a0000000p-25f},
    {0x1.2387a60000000p+0f, 0x1.ceac480000000p-25f}, {0x1.26b4560000000p+0f, 0x1.789f380000000p-26f},
    {0x1.29e9e00000000p+0f, -0x1.5c04240000000p-25f}, {0x1.2d285a0000000p+0f, 0x1.b900c20000000p-26f},
    {0x1.306fe00000000p+0f, 0x1.4636e20000000p-25f}, {0x1.33c08c0000000p+0f, -0x1.b37d200000000p-25f},
    {0x1.371a740000000p+0f, -0x1.18aac60000000p-25f}, {0x1.3a7db40000000p+0f, -0x1.634c020000000p-25f},
    {0x1.3dea640000000p+0f, 0x1.8246840000000p-25f}, {0x1.4160a20000000p+0f, 0x1.f72e2a0000000p-28f},
    {0x1.44e0860000000p+0f, 0x1.8624b40000000p-30f}, {0x1.486a2c0000000p+0f, -0x1.47d8660000000p-25f},
    {0x1.4bfdae0000000p+0f, -0x1.593abc0000000p-25f}, {0x1.4f9b280000000p+0f, -0x1.2c5a6c0000000p-25f},
    {0x1.5342b60000000p+0f, -0x1.2c56100000000p-25f}, {0x1.56f4740000000p+0f, -0x1.295b040000000p-25f},
    {0x1.5ab07e0000000p+0f, -0x1.5bd5ec0000000p-27f}, {0x1.5e76f20000000p+0f, -0x1.4a5bd60000000p-25f},
    {0x1.6247ec0000000p+0f, -0x1.f8b5500000000p-25f}, {0x1.6623880000000p+0f, 0x1.2a91120000000p-27f},
    {0x1.6a09e60000000p+0f, 0x1.9fcef40000000p-26f}, {0x1.6dfb240000000p+0f, -0x1.cd72e80000000p-27f},
    {0x1.71f75e0000000p+0f, 0x1.1d8bee0000000p-25f}, {0x1.75feb60000000p+0f, -0x1.37b3060000000p-25f},
    {0x1.7a11480000000p+0f, -0x1.829fd00000000p-25f}, {0x1.7e2f340000000p+0f, -0x1.2616340000000p-25f},
    {0x1.82589a0000000p+0f, -0x1.accc7c0000000p-26f}, {0x1.868d9a0000000p+0f, -0x1.2edb440000000p-26f},
    {0x1.8ace540000000p+0f, 0x1.15506e0000000p-27f}, {0x1.8f1aea0000000p+0f, -0x1.baa2320000000p-26f},
    {0x1.93737c0000000p+0f, -0x1.e647440000000p-25f}, {0x1.97d82a0000000p+0f, -0x1.0d8d840000000p-31f},
    {0x1.9c49180000000p+0f, 0x1.51f8480000000p-27f}, {0x1.a0c6680000000p+0f, -0x1.2886a60000000p-26f},
    {0x1.a5503c0000000p+0f, -0x1.b83b540000000p-25f}, {0x1.a9e6b60000000p+0f, -0x1.50c0480000000p-25f},
    {0x1.ae89fa0000000p+0f, -0x1.a94b140000000p-26f}, {0x1.b33a2c0000000p+0f, -0x1.ec3a820000000p-26f},
    {0x1.b7f7700000000p+0f, -0x1.a094380000000p-25f}, {0x1.bcc1ea0000000p+0f, -0x1.f687c60000000p-25f},
    {0x1.c199be0000000p+0f, -0x1.3d56b20000000p-27f}, {0x1.c67f120000000p+0f, 0x1.cafa2a0000000p-25f},
    {0x1.cb720e0000000p+0f, -0x1.8837cc0000000p-27f}, {0x1.d072d40000000p+0f, 0x1.40f1300000000p-25f},
    {0x1.d5818e0000000p+0f, -0x1.822dbc0000000p-27f}, {0x1.da9e600000000p+0f, 0x1.ed99420000000p-27f},
    {0x1.dfc9740000000p+0f, -0x1.908c940000000p-25f}, {0x1.e502ee0000000p+0f, 0x1.e2cffe0000000p-26f},
    {0x1.ea4afa0000000p+0f, 0x1.52486c0000000p-27f}, {0x1.efa1be0000000p+0f, 0x1.cc2b440000000p-25f},
    {0x1.f507660000000p+0f, -0x1.246eb00000000p-26f}, {0x1.fa7c180000000p+0f, 0x1.9e90d80000000p-28f}
};

// exp(r) 2^(j/64) for the reduced argument r (|r| <= ln2 / 128 + 1e-6) and k = 64 n + j: the
// double-float m in [0.99, 2.02] with exp(x) = m 2^n.
__device__ inline xr_df xr_df_exp_finish(xr_df r, int k, int* n) {
  const float d = __fmul_rn(r.hi, __fmaf_rn(r.hi, __fmaf_rn(r.hi, 1.0f / 120.0f, 1.0f / 24.0f), 1.0f / 6.0f));
  const xr_df em1 = xr_df_add(r, xr_df_mul(xr_df_mul(r, r), xr_df_two_sum(0.5f, d)));  // exp(r) - 1
  *n = k >> 6;  // floor(k / 64)
  const float2 tj = __ldg(&xr_df_exp2_64[k & 63]);
  const xr_df t{tj.x, tj.y};
  return xr_df_add(t, xr_df_mul(t, em1));
}

// exp(x) = m 2^n for a float x with |x| < 80 (exact input): the reduction in FP32, ln2 / 64 split
// into C1 + C2 + C3 + C4 with C1 and C2 of at most 11 significant bits, so that k C1 and k C2 are
// exact (|k| < 2^13) and x - k C1 is exact (Sterbenz).
__device__ inline xr_df xr_df_exp_float(float x, int* n) {
  const float C1 = 0x1.63p-7f, C2 = -0x1.bdp-19f, C3 = -0x1.05c61p-35f, C4 = -0x1.950d88p-60f;
  const float kf = rintf(__fmul_rn(x, 0x1.715476p+6f));  // round(x 64 / ln2)
  xr_df r = xr_df_two_sum(__fsub_rn(x, __fmul_rn(kf, C1)), -__fmul_rn(kf, C2));
  const float p3 = __fmul_rn(kf, C3);
  r = xr_df_add(r, {-p3, -__fmaf_rn(kf, C3, -p3)});  // k C3 as a double-float
  r = xr_df_add_f(r, -__fmul_rn(kf, C4));
  return xr_df_exp_finish(r, (int)kf, n);
}

// exp(x), FP64 in and out. The reduction is FP64 (two FMAs with ln2 / 64 = hi + lo, hi of 40
// significant bits so that k hi is exact): a double-float input would lose the bits of x beyond 48,
// 1e-13 of exp(x) at |x| = 70.
__device__ inline double xr_exp(double x) {
  const float xf = __double2float_rn(x);
  if (!(fabsf(xf) < 80.0f)) return exp(x);
  const float kf = rintf(__fmul_rn(xf, 0x1.715476p+6f));  // round(x 64 / ln2), |kf| < 2^13
  const double kd = (double)kf;
  double r = fma(-kd, 0x1.62e42fefa4000p-7, x);
  r = fma(-kd, -0x1.8432a1b0e2634p-49, r);
  int n;
  const xr_df m = xr_df_exp_finish(xr_df_from_double(r), (int)kf, &n);
  const double v = (double)m.hi + (double)m.lo;
  return __longlong_as_double(__double_as_longlong(v) + ((long long)n << 52));  // v 2^n: both normal
}

// exp(x) as a double-float for a double-float x with |x| < 80 whose own 48 bits are all it has (the
// vdW shielding chain, |x| below 5 there): the reduction in FP32 as in xr_df_exp_float, with x.lo
// added after the exact steps; 2^n applied to both floats (exact while they stay normal, n >= -100).
__device__ inline xr_df xr_df_exp_df(xr_df x) {
  if (!(fabsf(x.hi) < 80.0f)) {
    const double v = exp((double)x.hi + (double)x.lo);
    return xr_df_from_double(v);
  }
  const float C1 = 0x1.63p-7f, C2 = -0x1.bdp-19f, C3 = -0x1.05c61p-35f, C4 = -0x1.950d88p-60f;
  const float kf = rintf(__fmul_rn(x.hi, 0x1.715476p+6f));
  xr_df r = xr_df_two_sum(__fsub_rn(x.hi, __fmul_rn(kf, C1)), -__fmul_rn(kf, C2));
  r = xr_df_add_f(r, x.lo);
  const float p3 = __fmul_rn(kf, C3);
  r = xr_df_add(r, {-p3, -__fmaf_rn(kf, C3, -p3)});
  r = xr_df_add_f(r, -__fmul_rn(kf, C4));
  int n;
  xr_df m = xr_df_exp_finish(r, (int)kf, &n);
  const float s = __int_as_float((127 + n) << 23);
  m.hi = __fmul_rn(m.hi, s);
  m.lo = __fmul_rn(m.lo, s);
  return m;
}

// log(a) as a double-float for a double-float a in [1e-30, 1e30] (the Newton step of xr_log).
__device__ inline xr_df xr_df_log_df(xr_df a) {
  if (!(a.hi >= 1e-30f && a.hi <= 1e30f)) return xr_df_from_double(log((double)a.hi + (double)a.lo));
  const float y0 = logf(a.hi);
  int n;
  xr_df e = xr_df_exp_float(-y0, &n);
  const float s = __int_as_float((127 + n) << 23);
  e.hi = __fmul_rn(e.hi, s);
  e.lo = __fmul_rn(e.lo, s);
  const xr_df t = xr_df_add_f(xr_df_mul(a, e), -1.0f);
  return xr_df_add_f(xr_df_add_f(t, y0), __fmul_rn(-0.5f, __fmul_rn(t.hi, t.hi)));
}

// log(a), FP64 in and out.
__device__ inline double xr_log(double a) {
  const xr_df ad = xr_df_from_double(a);
  if (!(ad.hi >= 1e-30f && ad.hi <= 1e30f)) return log(a);
  const float y0 = logf(ad.hi);
  int n;
  xr_df e = xr_df_exp_float(-y0, &n);  // exp(-y0) = e 2^n, |n| <= 100
  const float s = __int_as_float((127 + n) << 23);  // 2^n, a normal float
  e.hi = __fmul_rn(e.hi, s);
  e.lo = __fmul_rn(e.lo, s);
  const xr_df t = xr_df_add_f(xr_df_mul(ad, e), -1.0f);  // a exp(-y0) - 1
  const xr_df l = xr_df_add_f(t, y0);
  return (double)l.hi + ((double)l.lo - 0.5 * (double)t.hi * (double)t.hi);
}
