// Correctly rounded double sin, cos and acos for the FP64 time-step path.
//
// The reference takes sin/cos/acos from the C library (Quat3D.h:117-166, called from the link and
// voxel updates).  A GPU cannot call the host C library, and CUDA's own functions are not correctly
// rounded, so this header evaluates the functions in double-double arithmetic (error below 2^-100
// relative) and rounds once; a Ziv-style test decides whether that rounding is certain.  The same
// code compiles for host and device, so both give identical bits.
//
// Methods (all public textbook material):
//   * double-double arithmetic: Dekker/Knuth error-free transformations, two_prod through fma;
//   * sin/cos: Cody-Waite reduction by pi/2 held as three doubles, then the Taylor series of sin
//     and cos in double-double, term count chosen from the reduced argument;
//   * acos: one Newton step on cos(y) = w from the platform acos (|w| <= 0.999; the residual is
//     formed as (1-|w|) - 2 sin^2(y/2) to avoid cancellation), otherwise 2*asin(sqrt((1-|w|)/2))
//     with the asin Taylor series.
//
// Each evaluation reports two flags through *flags (bitwise or):
//   VXM_AMBIGUOUS   the Ziv test could not certify the rounding (expected rate ~2^-40)
//   VXM_LIBM_BAND   the exact value lies within 1/64 ulp of a rounding midpoint; a C library whose
//                   error exceeds 0.5 ulp (glibc's sin/cos/acos do, by up to ~0.012 ulp) may round
//                   such a value the other way.  These counts bound the expected disagreements
//                   with the reference's C library.
// Constants: 1/n! and the asin series coefficients (2k)!/(4^k k!^2 (2k+1)) split into two doubles,
// and pi/2, pi split into three doubles; generated with 300-bit arithmetic.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define VXM_HD __host__ __device__ __forceinline__
#else
#define VXM_HD inline
#endif

namespace vxm {

enum { VXM_AMBIGUOUS = 1, VXM_LIBM_BAND = 2 };

struct dd {
  double hi, lo;
};

VXM_HD double fma_(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
  return ::fma(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
VXM_HD dd mk(double h, double l) { dd r; r.hi = h; r.lo = l; return r; }
VXM_HD dd neg(dd a) { return mk(-a.hi, -a.lo); }
VXM_HD dd two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  double e = (a - (s - bb)) + (b - bb);
  return mk(s, e);
}
VXM_HD dd quick_two_sum(double a, double b) {
  double s = a + b;
  double e = b - (s - a);
  return mk(s, e);
}
VXM_HD dd two_prod(double a, double b) {
  double p = a * b;
  return mk(p, fma_(a, b, -p));
}
VXM_HD dd add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  dd t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
VXM_HD dd sub(dd a, dd b) { return add(a, neg(b)); }
VXM_HD dd mul(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return quick_two_sum(p.hi, p.lo);
}
VXM_HD dd mul_d(dd a, double b) {
  dd p = two_prod(a.hi, b);
  p.lo += a.lo * b;
  return quick_two_sum(p.hi, p.lo);
}
VXM_HD dd div(dd a, dd b) {
  double q1 = a.hi / b.hi;
  dd r = sub(a, mul_d(b, q1));
  double q2 = r.hi / b.hi;
  r = sub(r, mul_d(b, q2));
  double q3 = r.hi / b.hi;
  dd q = quick_two_sum(q1, q2);
  return add(q, mk(q3, 0.0));
}

VXM_HD uint64_t bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}
VXM_HD double from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}
VXM_HD double ulp_of(double x) {  // spacing above |x| (x finite, nonzero)
  double a = std::fabs(x);
  return from_bits(bits(a) + 1) - a;
}

// Round a double-double value whose relative error is below 2^-98 to the nearest double.
VXM_HD double round_dd(dd y, int* flags) {
  double eb = std::fabs(y.hi) * 0x1p-98;
  double r1 = y.hi + (y.lo + eb);
  double r2 = y.hi + (y.lo - eb);
  if (r1 != r2) *flags |= VXM_AMBIGUOUS;
  if (y.hi != 0.0) {
    double u = ulp_of(y.hi);
    double d = std::fabs(std::fabs(y.lo) - 0.5 * u);
    if (d < 0.015625 * u) *flags |= VXM_LIBM_BAND;
  }
  return r1;
}

// 1/n! as double-double, n = 0..31 (entries 0 and 1 are exact ones), and the asin series
// coefficients c_k = (2k)!/(4^k k!^2 (2k+1)), k = 0..11.  One copy for host code, one in constant
// memory for device code.
#define VXM_F(h, l) {h, l}
struct ddc {
  double hi, lo;
};
#define VXM_INV_FACT_INIT { \
    VXM_F(1.0, 0.0), VXM_F(1.0, 0.0), VXM_F(0x1.0000000000000p-1, 0.0), \
    VXM_F(0x1.5555555555555p-3, 0x1.5555555555555p-57), VXM_F(0x1.5555555555555p-5, 0x1.5555555555555p-59), \
    VXM_F(0x1.1111111111111p-7, 0x1.1111111111111p-63), VXM_F(0x1.6c16c16c16c17p-10, -0x1.f49f49f49f49fp-65), \
    VXM_F(0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-73), VXM_F(0x1.a01a01a01a01ap-16, 0x1.a01a01a01a01ap-76), \
    VXM_F(0x1.71de3a556c734p-19, -0x1.c154f8ddc6c00p-73), VXM_F(0x1.27e4fb7789f5cp-22, 0x1.cbbc05b4fa99ap-76), \
    VXM_F(0x1.ae64567f544e4p-26, -0x1.c062e06d1f209p-80), VXM_F(0x1.1eed8eff8d898p-29, -0x1.2aec959e14c06p-83), \
    VXM_F(0x1.6124613a86d09p-33, 0x1.f28e0cc748ebep-87), VXM_F(0x1.93974a8c07c9dp-37, 0x1.05d6f8a2efd1fp-92), \
    VXM_F(0x1.ae7f3e733b81fp-41, 0x1.1d8656b0ee8cbp-97), VXM_F(0x1.ae7f3e733b81fp-45, 0x1.1d8656b0ee8cbp-101), \
    VXM_F(0x1.952c77030ad4ap-49, 0x1.ac981465ddc6cp-103), VXM_F(0x1.6827863b97d97p-53, 0x1.eec01221a8b0bp-107), \
    VXM_F(0x1.2f49b46814157p-57, 0x1.2650f61dbdcb4p-112), VXM_F(0x1.e542ba4020225p-62, 0x1.ea72b4afe3c2fp-120), \
    VXM_F(0x1.71b8ef6dcf572p-66, -0x1.d043ae40c4647p-120), VXM_F(0x1.0ce396db7f853p-70, -0x1.aebcdbd20331cp-124), \
    VXM_F(0x1.761b41316381ap-75, -0x1.3423c7d91404fp-130), VXM_F(0x1.f2cf01972f578p-80, -0x1.9ada5fcc1ab14p-135), \
    VXM_F(0x1.3f3ccdd165fa9p-84, -0x1.58ddadf344487p-139), VXM_F(0x1.88e85fc6a4e5ap-89, -0x1.71c37ebd16540p-143), \
    VXM_F(0x1.d1ab1c2dccea3p-94, 0x1.054d0c78aea14p-149), VXM_F(0x1.0a18a2635085dp-98, 0x1.b9e2e28e1aa54p-153), \
    VXM_F(0x1.259f98b4358adp-103, 0x1.eaf8c39dd9bc5p-157), VXM_F(0x1.3932c5047d60ep-108, 0x1.832b7b530a627p-162), \
    VXM_F(0x1.434d2e783f5bcp-113, 0x1.0b87b91be9affp-167)}
#define VXM_ASIN_INIT { \
    VXM_F(1.0, 0.0), \
    VXM_F(0x1.5555555555555p-3, 0x1.5555555555555p-57), VXM_F(0x1.3333333333333p-4, 0x1.999999999999ap-59), \
    VXM_F(0x1.6db6db6db6db7p-5, -0x1.2492492492492p-60), VXM_F(0x1.f1c71c71c71c7p-6, 0x1.c71c71c71c71cp-62), \
    VXM_F(0x1.6e8ba2e8ba2e9p-6, -0x1.1745d1745d174p-60), VXM_F(0x1.1c4ec4ec4ec4fp-6, -0x1.d89d89d89d89ep-61), \
    VXM_F(0x1.c99999999999ap-7, -0x1.999999999999ap-61), VXM_F(0x1.7a87878787878p-7, 0x1.e1e1e1e1e1e1ep-61), \
    VXM_F(0x1.3fde50d79435ep-7, 0x1.435e50d79435ep-61), VXM_F(0x1.12ef3cf3cf3cfp-7, 0x1.e79e79e79e79ep-62), \
    VXM_F(0x1.df3bd37a6f4dfp-8, -0x1.90b21642c8591p-62)}
static const ddc kInvFactH[32] = VXM_INV_FACT_INIT;
static const ddc kAsinH[12] = VXM_ASIN_INIT;
#if defined(__CUDACC__)
static __device__ __constant__ ddc kInvFactD[32] = VXM_INV_FACT_INIT;
static __device__ __constant__ ddc kAsinD[12] = VXM_ASIN_INIT;
#endif
VXM_HD ddc inv_fact(int i) {
#if defined(__CUDA_ARCH__)
  return kInvFactD[i];
#else
  return kInvFactH[i];
#endif
}
VXM_HD ddc asin_c(int i) {
#if defined(__CUDA_ARCH__)
  return kAsinD[i];
#else
  return kAsinH[i];
#endif
}
#undef VXM_F

static constexpr double kPio2_1 = 0x1.921fb54442d18p+0;
static constexpr double kPio2_2 = 0x1.1a62633145c07p-54;
static constexpr double kPio2_3 = -0x1.f1976b7ed8fbcp-110;
static constexpr double kPi_1 = 0x1.921fb54442d18p+1;
static constexpr double kPi_2 = 0x1.1a62633145c07p-53;

VXM_HD dd cf(const ddc& c) { return mk(c.hi, c.lo); }

// sin and cos of a double-double |r| <= ~0.8 (Taylor series, adaptive length).
VXM_HD void sincos_small(dd r, dd* s, dd* c) {
  dd u = mul(r, r);
  double ua = std::fabs(u.hi);
  // number of terms: stop once u^k/(2k)! < 2^-112
  int K = 1;
  double t = 1.0;
  for (int k = 1; k <= 15; ++k) {
    t *= ua / (double)((2 * k - 1) * (2 * k));
    K = k;
    if (t < 0x1p-112) break;
  }
  // sin(r)/r = sum_k (-1)^k u^k/(2k+1)!, cos(r) = sum_k (-1)^k u^k/(2k)!
  dd ps = cf(inv_fact(2 * K + 1));
  dd pc = cf(inv_fact(2 * K));
  if (K & 1) { ps = neg(ps); pc = neg(pc); }
  for (int k = K - 1; k >= 0; --k) {
    dd as = cf(inv_fact(2 * k + 1));
    dd ac = cf(inv_fact(2 * k));
    if (k & 1) { as = neg(as); ac = neg(ac); }
    ps = add(as, mul(u, ps));
    pc = add(ac, mul(u, pc));
  }
  *s = mul(r, ps);
  *c = pc;
}

// sin/cos of a double x with |x| <= 8, as double-double.
VXM_HD void sincos_dd(double x, dd* s, dd* c) {
  double k = std::rint(x * 0.63661977236758134);  // 2/pi
  dd r = mk(x, 0.0);
  if (k != 0.0) {
    r = sub(r, two_prod(k, kPio2_1));
    r = sub(r, two_prod(k, kPio2_2));
    r = sub(r, mk(k * kPio2_3, 0.0));
  }
  dd ss, cc;
  sincos_small(r, &ss, &cc);
  int q = ((int)k) & 3;
  switch (q) {
    case 0: *s = ss; *c = cc; break;
    case 1: *s = cc; *c = neg(ss); break;
    case 2: *s = neg(ss); *c = neg(cc); break;
    default: *s = neg(cc); *c = ss; break;
  }
}

VXM_HD double cr_sin(double x, int* flags) {
  if (x == 0.0) return x;
  dd s, c;
  sincos_dd(x, &s, &c);
  return round_dd(s, flags);
}
VXM_HD double cr_cos(double x, int* flags) {
  dd s, c;
  sincos_dd(x, &s, &c);
  return round_dd(c, flags);
}

// sqrt of a positive double as double-double (one Newton correction on the rounded root).
VXM_HD dd sqrt_dd(double t) {
  if (t == 0.0) return mk(0.0, 0.0);
  double s0 = std::sqrt(t);
  double e = fma_(-s0, s0, t);  // exact t - s0^2
  return quick_two_sum(s0, e / (2.0 * s0));
}

VXM_HD double cr_acos(double w, int* flags) {
  if (!(w >= -1.0 && w <= 1.0)) return (w - w) / (w - w);  // NaN
  if (w == 1.0) return 0.0;
  double aw = std::fabs(w);
  if (aw <= 0.999) {
    double y0 = std::acos(w);
    // f(y) = cos(y) - w, computed from half-angle terms; one Newton step y1 = y0 + f(y0)/sin(y0)
    dd sh, ch;
    sincos_dd(0.5 * y0, &sh, &ch);
    dd f;
    dd omw = mk(1.0 - aw, 0.0);  // exact (Sterbenz) for aw >= 0.5, and exact enough below
    if (aw >= 0.5) {
      if (w > 0) f = sub(omw, mul_d(mul(sh, sh), 2.0));   // (1-w) - 2 sin^2(y/2)
      else f = sub(mul_d(mul(ch, ch), 2.0), omw);         // 2 cos^2(y/2) - (1-|w|)
    } else {
      dd cy = sub(mk(1.0, 0.0), mul_d(mul(sh, sh), 2.0));  // cos(y)
      f = sub(cy, mk(w, 0.0));
    }
    dd sy = mul_d(mul(sh, ch), 2.0);
    dd y = add(mk(y0, 0.0), div(f, sy));
    return round_dd(y, flags);
  }
  // near +-1: acos(|w|) = 2 asin(s), s = sqrt((1-|w|)/2) <= 0.0224
  double t = (1.0 - aw) * 0.5;
  dd s = sqrt_dd(t);
  dd u = mul(s, s);
  dd p = cf(asin_c(11));
  for (int k = 10; k >= 0; --k) p = add(cf(asin_c(k)), mul(u, p));
  dd a = mul_d(mul(s, p), 2.0);
  if (w < 0) a = sub(mk(kPi_1, kPi_2), a);
  return round_dd(a, flags);
}

}  // namespace vxm
