/*
 * sflow_math.h -- FP64 pow, log and cos written for this library, giving
 * the same bits in CUDA device code and in C host code.
 *
 * Why: the settling velocity (constitutive_2d.f90:5326-5404) is a
 * fixed-point iteration that stops on a 1e-6 relative-change test, and the
 * hindered-settling and entrainment closures (constitutive_2d.f90:4850-4851,
 * 5046-5057) raise to non-integer powers.  CUDA's pow and a host libm's pow
 * differ in the last bit for some arguments; inside the fixed point such a
 * bit can move a cell across the 1e-6 test, and at a wet/dry front the
 * deposition then decides whether a thin cell keeps its mass.  These
 * functions use only IEEE-754 operations that every conforming platform
 * rounds the same way (+, -, *, / rounded to nearest, fused multiply-add,
 * rint), evaluated in a fixed order: in device code through the _rn
 * intrinsics, which the compiler never contracts or reorders; in C through
 * plain operators, compiled with -ffp-contract=off.  So a GPU kernel and a
 * CPU program that call them get identical results.
 *
 * Method (double-double arithmetic: a value is an unevaluated sum hi + lo
 * of two doubles; the error-free sum of Knuth and the error-free product
 * through one fused multiply-add give about 104 significant bits):
 *  log x   x = 2^k m with m in [sqrt(1/2), sqrt(2)], f = (m - 1)/(m + 1),
 *          log m = 2 atanh f = 2f (1 + f^2/3 + f^4/5 + ...); the first
 *          three terms of the series in double-double, the rest (|f| <=
 *          0.1716, 10 terms) in double; plus k ln 2 with ln 2 in
 *          double-double.  Absolute error below 2^-72.
 *  exp z   z in double-double, k = rint(z / ln 2), r = z - k ln 2 (|r| <=
 *          0.347), Taylor series of exp(r) to r^17/17!: terms up to
 *          r^6/6! in double-double, the rest in double; times 2^k.
 *          Relative error below 2^-70 before the final rounding.
 *  pow x^y exp(y log x) with y log x in double-double.  One final
 *          rounding of the double-double result, so the value is the
 *          correctly rounded x^y except when x^y lies within ~2^-70
 *          relative of a rounding boundary.
 *  cos x   x = k pi/2 + r (pi/2 in double-double, |k| < 2^20), the
 *          Taylor series of sin or cos of r (|r| <= pi/4) with the first
 *          terms in double-double.
 * The double-double constants (ln 2, 1/ln 2, pi/2, 2/pi, 1/3, 1/5, 1/7,
 * 1/n!) are the exact values split into a nearest double and the nearest
 * double of the remainder; tests/test_math.py recomputes them.
 *
 * The functions handle every input (NaN, infinities, zeros, subnormals,
 * negative bases with integer exponents) with the C99 Annex F values of
 * pow, log and cos; subnormal results may differ from the correctly rounded
 * value by one unit in the last place (the scaling by 2^k rounds a second
 * time there).
 */
#ifndef SFLOW_MATH_H
#define SFLOW_MATH_H

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define SFM_FN static __device__ __forceinline__
#define SFM_ADD(a, b) __dadd_rn((a), (b))
#define SFM_SUB(a, b) __dsub_rn((a), (b))
#define SFM_MUL(a, b) __dmul_rn((a), (b))
#define SFM_DIV(a, b) __ddiv_rn((a), (b))
#define SFM_FMA(a, b, c) __fma_rn((a), (b), (c))
#define SFM_RINT(a) rint(a)
SFM_FN int64_t sfm_bits(double x) { return (int64_t)__double_as_longlong(x); }
SFM_FN double sfm_from_bits(int64_t b) { return __longlong_as_double((long long)b); }
#else
#include <string.h>
#define SFM_FN static inline
#define SFM_ADD(a, b) ((a) + (b))
#define SFM_SUB(a, b) ((a) - (b))
#define SFM_MUL(a, b) ((a) * (b))
#define SFM_DIV(a, b) ((a) / (b))
#define SFM_FMA(a, b, c) fma((a), (b), (c))
#define SFM_RINT(a) rint(a)
SFM_FN int64_t sfm_bits(double x) { int64_t b; memcpy(&b, &x, sizeof b); return b; }
SFM_FN double sfm_from_bits(int64_t b) { double x; memcpy(&x, &b, sizeof x); return x; }
#endif

typedef struct {
  double hi, lo;
} sfm_dd;

SFM_FN sfm_dd sfm_mk(double hi, double lo) {
  sfm_dd r;
  r.hi = hi;
  r.lo = lo;
  return r;
}
/* a + b exactly (Knuth's two-sum) */
SFM_FN sfm_dd sfm_two_sum(double a, double b) {
  const double s = SFM_ADD(a, b);
  const double bb = SFM_SUB(s, a);
  const double e = SFM_ADD(SFM_SUB(a, SFM_SUB(s, bb)), SFM_SUB(b, bb));
  return sfm_mk(s, e);
}
/* a + b exactly when |a| >= |b| or a == 0 (Dekker's fast two-sum) */
SFM_FN sfm_dd sfm_fast_two_sum(double a, double b) {
  const double s = SFM_ADD(a, b);
  return sfm_mk(s, SFM_SUB(b, SFM_SUB(s, a)));
}
/* a * b exactly (no overflow or underflow) */
SFM_FN sfm_dd sfm_two_prod(double a, double b) {
  const double p = SFM_MUL(a, b);
  return sfm_mk(p, SFM_FMA(a, b, -p));
}
SFM_FN sfm_dd sfm_dd_add(sfm_dd x, sfm_dd y) {
  sfm_dd s = sfm_two_sum(x.hi, y.hi);
  const sfm_dd t = sfm_two_sum(x.lo, y.lo);
  s = sfm_fast_two_sum(s.hi, SFM_ADD(s.lo, t.hi));
  return sfm_fast_two_sum(s.hi, SFM_ADD(s.lo, t.lo));
}
SFM_FN sfm_dd sfm_dd_neg(sfm_dd x) { return sfm_mk(-x.hi, -x.lo); }
SFM_FN sfm_dd sfm_dd_mul(sfm_dd x, sfm_dd y) {
  const sfm_dd p = sfm_two_prod(x.hi, y.hi);
  const double c = SFM_ADD(SFM_MUL(x.hi, y.lo), SFM_MUL(x.lo, y.hi));
  return sfm_fast_two_sum(p.hi, SFM_ADD(p.lo, c));
}
SFM_FN sfm_dd sfm_dd_mul_d(sfm_dd x, double y) {
  const sfm_dd p = sfm_two_prod(x.hi, y);
  return sfm_fast_two_sum(p.hi, SFM_ADD(p.lo, SFM_MUL(x.lo, y)));
}
/* x / y: three quotient digits, each from the remainder of the last */
SFM_FN sfm_dd sfm_dd_div(sfm_dd x, sfm_dd y) {
  const double q1 = SFM_DIV(x.hi, y.hi);
  sfm_dd r = sfm_dd_add(x, sfm_dd_neg(sfm_dd_mul_d(y, q1)));
  const double q2 = SFM_DIV(r.hi, y.hi);
  r = sfm_dd_add(r, sfm_dd_neg(sfm_dd_mul_d(y, q2)));
  const double q3 = SFM_DIV(r.hi, y.hi);
  return sfm_dd_add(sfm_fast_two_sum(q1, q2), sfm_mk(q3, 0.0));
}

#define SFM_LN2_HI 0x1.62e42fefa39efp-1
#define SFM_LN2_LO 0x1.abc9e3b39803fp-56
#define SFM_INV_LN2 0x1.71547652b82fep+0
#define SFM_PIO2_HI 0x1.921fb54442d18p+0
#define SFM_PIO2_LO 0x1.1a62633145c07p-54
#define SFM_TWO_OVER_PI 0x1.45f306dc9c883p-1
#define SFM_SQRT2 0x1.6a09e667f3bcdp+0

/* natural logarithm of a finite x > 0 in double-double */
SFM_FN sfm_dd sfm_log_dd(double x) {
  int64_t b = sfm_bits(x);
  int k = 0;
  if ((b >> 52) == 0) {            /* subnormal: scale by 2^54 */
    x = SFM_MUL(x, 0x1p54);
    b = sfm_bits(x);
    k = -54;
  }
  k += (int)(b >> 52) - 1023;
  double m = sfm_from_bits((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);   /* [1, 2) */
  if (m > SFM_SQRT2) {
    m = SFM_MUL(m, 0.5);
    k += 1;
  }
  /* m - 1 is exact for m in [1/2, 2] (Sterbenz) */
  const sfm_dd f = sfm_dd_div(sfm_mk(SFM_SUB(m, 1.0), 0.0), sfm_two_sum(m, 1.0));
  const sfm_dd f2 = sfm_dd_mul(f, f);
  /* V = 1/9 + f^2/11 + ... + f^18/27 in double */
  const double z = f2.hi;
  double v = 0x1.2f684bda12f68p-5;
  v = SFM_ADD(SFM_MUL(v, z), 0x1.47ae147ae147bp-5);
  v = SFM_ADD(SFM_MUL(v, z), 0x1.642c8590b2164p-5);
  v = SFM_ADD(SFM_MUL(v, z), 0x1.8618618618618p-5);
  v = SFM_ADD(SFM_MUL(v, z), 0x1.af286bca1af28p-5);
  v = SFM_ADD(SFM_MUL(v, z), 0x1.e1e1e1e1e1e1ep-5);
  v = SFM_ADD(SFM_MUL(v, z), 0x1.1111111111111p-4);
  v = SFM_ADD(SFM_MUL(v, z), 0x1.3b13b13b13b14p-4);
  v = SFM_ADD(SFM_MUL(v, z), 0x1.745d1745d1746p-4);
  v = SFM_ADD(SFM_MUL(v, z), 0x1.c71c71c71c71cp-4);
  /* S = f^2 (1/3 + f^2 (1/5 + f^2 (1/7 + f^2 V))) in double-double */
  sfm_dd s = sfm_dd_add(sfm_mk(0x1.2492492492492p-3, 0x1.2492492492492p-57), sfm_dd_mul_d(f2, v));
  s = sfm_dd_add(sfm_mk(0x1.999999999999ap-3, -0x1.999999999999ap-57), sfm_dd_mul(f2, s));
  s = sfm_dd_add(sfm_mk(0x1.5555555555555p-2, 0x1.5555555555555p-56), sfm_dd_mul(f2, s));
  s = sfm_dd_mul(f2, s);
  /* log m = 2 f (1 + S) */
  sfm_dd lm = sfm_dd_mul(f, sfm_dd_add(sfm_mk(1.0, 0.0), s));
  lm = sfm_mk(SFM_MUL(lm.hi, 2.0), SFM_MUL(lm.lo, 2.0));
  const double kd = (double)k;
  const sfm_dd kl = sfm_dd_add(sfm_two_prod(kd, SFM_LN2_HI), sfm_mk(SFM_MUL(kd, SFM_LN2_LO), 0.0));
  return sfm_dd_add(kl, lm);
}

/* exp of a double-double z, rounded once to double */
SFM_FN double sfm_exp_dd(sfm_dd z) {
  if (z.hi > 709.8) return HUGE_VAL;
  if (z.hi < -745.2) return 0.0;
  const double kd = SFM_RINT(SFM_MUL(z.hi, SFM_INV_LN2));
  sfm_dd r = sfm_dd_add(z, sfm_dd_neg(sfm_two_prod(kd, SFM_LN2_HI)));
  r = sfm_dd_add(r, sfm_mk(-SFM_MUL(kd, SFM_LN2_LO), 0.0));
  const double rh = r.hi, rl = r.lo;
  /* w = 1/7! + rh/8! + ... + rh^10/17! in double */
  double w = 0x1.952c77030ad4ap-49;                 /* 1/17! */
  w = SFM_ADD(SFM_MUL(w, rh), 0x1.ae7f3e733b81fp-45);   /* 1/16! */
  w = SFM_ADD(SFM_MUL(w, rh), 0x1.ae7f3e733b81fp-41);   /* 1/15! */
  w = SFM_ADD(SFM_MUL(w, rh), 0x1.93974a8c07c9dp-37);   /* 1/14! */
  w = SFM_ADD(SFM_MUL(w, rh), 0x1.6124613a86d09p-33);   /* 1/13! */
  w = SFM_ADD(SFM_MUL(w, rh), 0x1.1eed8eff8d898p-29);   /* 1/12! */
  w = SFM_ADD(SFM_MUL(w, rh), 0x1.ae64567f544e4p-26);   /* 1/11! */
  w = SFM_ADD(SFM_MUL(w, rh), 0x1.27e4fb7789f5cp-22);   /* 1/10! */
  w = SFM_ADD(SFM_MUL(w, rh), 0x1.71de3a556c734p-19);   /* 1/9!  */
  w = SFM_ADD(SFM_MUL(w, rh), 0x1.a01a01a01a01ap-16);   /* 1/8!  */
  w = SFM_ADD(SFM_MUL(w, rh), 0x1.a01a01a01a01ap-13);   /* 1/7!  */
  /* 1/6! + rh w, then Horner down to 1 in double-double */
  sfm_dd p = sfm_dd_add(sfm_mk(0x1.6c16c16c16c17p-10, -0x1.f49f49f49f49fp-65), sfm_two_prod(rh, w));
  p = sfm_dd_add(sfm_mk(0x1.1111111111111p-7, 0x1.1111111111111p-63), sfm_dd_mul_d(p, rh));
  p = sfm_dd_add(sfm_mk(0x1.5555555555555p-5, 0x1.5555555555555p-59), sfm_dd_mul_d(p, rh));
  p = sfm_dd_add(sfm_mk(0x1.5555555555555p-3, 0x1.5555555555555p-57), sfm_dd_mul_d(p, rh));
  p = sfm_dd_add(sfm_mk(0.5, 0.0), sfm_dd_mul_d(p, rh));
  p = sfm_dd_add(sfm_mk(1.0, 0.0), sfm_dd_mul_d(p, rh));
  p = sfm_dd_add(sfm_mk(1.0, 0.0), sfm_dd_mul_d(p, rh));
  /* exp(rh + rl) = exp(rh) (1 + rl), |rl| < 2^-54 */
  p = sfm_dd_add(p, sfm_mk(SFM_MUL(p.hi, rl), 0.0));
  double s = SFM_ADD(p.hi, p.lo);
  int k = (int)kd;
  if (k > 1000) {
    s = SFM_MUL(s, 0x1p1000);
    k -= 1000;
  } else if (k < -1000) {
    s = SFM_MUL(s, 0x1p-1000);
    k += 1000;
  }
  return SFM_MUL(s, sfm_from_bits((int64_t)(k + 1023) << 52));
}

SFM_FN int sfm_isnan(double x) { return (sfm_bits(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; }
SFM_FN int sfm_isinf(double x) { return (sfm_bits(x) & 0x7fffffffffffffffLL) == 0x7ff0000000000000LL; }

/* natural logarithm */
SFM_FN double sfm_log(double x) {
  if (sfm_isnan(x)) return x;
  if (x < 0.0) return sfm_from_bits(0x7ff8000000000000LL);
  if (x == 0.0) return -HUGE_VAL;
  if (sfm_isinf(x)) return x;
  const sfm_dd l = sfm_log_dd(x);
  return SFM_ADD(l.hi, l.lo);
}

/* x^y with the C99 special values */
SFM_FN double sfm_pow(double x, double y) {
  if (y == 0.0 || x == 1.0) return 1.0;
  if (sfm_isnan(x) || sfm_isnan(y)) return SFM_ADD(x, y);
  const double ay = fabs(y);
  const int y_int = (ay >= 0x1p53) || (floor(ay) == ay);
  const int y_odd = y_int && (ay < 0x1p53) && (floor(SFM_MUL(ay, 0.5)) != SFM_MUL(ay, 0.5));
  const int neg = sfm_bits(x) < 0;         /* sign bit of x (-0 included) */
  if (sfm_isinf(y)) {
    const double ax = fabs(x);
    if (ax == 1.0) return 1.0;
    return ((ax < 1.0) == (y > 0.0)) ? 0.0 : HUGE_VAL;
  }
  if (x == 0.0 || sfm_isinf(x)) {
    /* |x| is 0 or inf: the result is 0 or inf, negative for a negative x
       and an odd integer y */
    const int big = (x == 0.0) ? (y < 0.0) : (y > 0.0);
    const double r = big ? HUGE_VAL : 0.0;
    return (neg && y_odd) ? -r : r;
  }
  if (neg && !y_int) return sfm_from_bits(0x7ff8000000000000LL);
  const sfm_dd l = sfm_log_dd(fabs(x));
  const double yl = SFM_MUL(y, l.hi);
  if (!(fabs(yl) <= 745.2)) {          /* far outside the double range */
    const double r = (yl > 0.0) ? HUGE_VAL : 0.0;
    return (neg && y_odd) ? -r : r;
  }
  sfm_dd z = sfm_two_prod(y, l.hi);
  z = sfm_fast_two_sum(z.hi, SFM_ADD(z.lo, SFM_MUL(y, l.lo)));
  const double r = sfm_exp_dd(z);
  return (neg && y_odd) ? -r : r;
}

/* cos x for |x| < 2^20 pi/2 (NaN beyond, and for NaN or infinite x) */
SFM_FN double sfm_cos(double x) {
  const double ax = fabs(x);
  if (!(ax < 1647099.0)) return sfm_from_bits(0x7ff8000000000000LL);
  const double kd = SFM_RINT(SFM_MUL(ax, SFM_TWO_OVER_PI));
  sfm_dd r = sfm_dd_add(sfm_mk(ax, 0.0), sfm_dd_neg(sfm_two_prod(kd, SFM_PIO2_HI)));
  r = sfm_dd_add(r, sfm_dd_neg(sfm_two_prod(kd, SFM_PIO2_LO)));
  const sfm_dd r2 = sfm_dd_mul(r, r);
  const double z = r2.hi;
  const int q = ((int)kd) & 3;
  double res;
  if ((q & 1) == 0) {
    /* cos r = sum (-1)^n r^2n / (2n)!: from r^8/8! on in double */
    double w = 0x1.e542ba4020225p-62;                      /*  1/20! */
    w = SFM_ADD(SFM_MUL(w, z), -0x1.6827863b97d97p-53);    /* -1/18! */
    w = SFM_ADD(SFM_MUL(w, z), 0x1.ae7f3e733b81fp-45);     /*  1/16! */
    w = SFM_ADD(SFM_MUL(w, z), -0x1.93974a8c07c9dp-37);    /* -1/14! */
    w = SFM_ADD(SFM_MUL(w, z), 0x1.1eed8eff8d898p-29);     /*  1/12! */
    w = SFM_ADD(SFM_MUL(w, z), -0x1.27e4fb7789f5cp-22);    /* -1/10! */
    w = SFM_ADD(SFM_MUL(w, z), 0x1.a01a01a01a01ap-16);     /*  1/8!  */
    sfm_dd p = sfm_dd_add(sfm_mk(-0x1.6c16c16c16c17p-10, 0x1.f49f49f49f49fp-65), sfm_dd_mul_d(r2, w));
    p = sfm_dd_add(sfm_mk(0x1.5555555555555p-5, 0x1.5555555555555p-59), sfm_dd_mul(r2, p));
    p = sfm_dd_add(sfm_mk(-0.5, 0.0), sfm_dd_mul(r2, p));
    p = sfm_dd_add(sfm_mk(1.0, 0.0), sfm_dd_mul(r2, p));
    res = SFM_ADD(p.hi, p.lo);
  } else {
    /* sin r = r sum (-1)^n r^2n / (2n+1)!: from r^6/7! on in double */
    double w = -0x1.71b8ef6dcf572p-66;                     /* -1/21! */
    w = SFM_ADD(SFM_MUL(w, z), 0x1.2f49b46814157p-57);     /*  1/19! */
    w = SFM_ADD(SFM_MUL(w, z), -0x1.952c77030ad4ap-49);    /* -1/17! */
    w = SFM_ADD(SFM_MUL(w, z), 0x1.ae7f3e733b81fp-41);     /*  1/15! */
    w = SFM_ADD(SFM_MUL(w, z), -0x1.6124613a86d09p-33);    /* -1/13! */
    w = SFM_ADD(SFM_MUL(w, z), 0x1.ae64567f544e4p-26);     /*  1/11! */
    w = SFM_ADD(SFM_MUL(w, z), -0x1.71de3a556c734p-19);    /* -1/9!  */
    w = SFM_ADD(SFM_MUL(w, z), 0x1.a01a01a01a01ap-13);     /*  1/7!  */
    sfm_dd p = sfm_dd_add(sfm_mk(0x1.1111111111111p-7, 0x1.1111111111111p-63), sfm_dd_mul_d(r2, -w));
    p = sfm_dd_add(sfm_mk(-0x1.5555555555555p-3, -0x1.5555555555555p-57), sfm_dd_mul(r2, p));
    p = sfm_dd_add(sfm_mk(1.0, 0.0), sfm_dd_mul(r2, p));
    p = sfm_dd_mul(r, p);
    res = SFM_ADD(p.hi, p.lo);
  }
  /* cos(k pi/2 + r): cos r, -sin r, -cos r, sin r for k mod 4 = 0..3 */
  return (q == 1 || q == 2) ? -res : res;
}

#endif /* SFLOW_MATH_H */
