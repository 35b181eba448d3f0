// Pair-of-FP32 ("double-float") arithmetic for the refinement residual's operator.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2:
// about 48 significant bits, computed on the FP32 pipe (this GPU issues FP32 at
// 64 times its FP64 rate).  The operations are built from error-free
// transformations:
//   TwoSum      s + e = a + b exactly                  (Knuth, TAOCP vol. 2, 4.2.2)
//   FastTwoSum  s + e = a + b exactly when |a| >= |b|  (Dekker 1971)
//   TwoProd     p + e = a * b exactly, e = fma(a, b, -p)
// combined as in the double-double arithmetic of Hida, Li and Bailey (2001), with
// the cheap ("sloppy") addition: the error of a sum is bounded relative to
// |a| + |b| (about 2^-47 of it), which is the bound a matrix-vector product's
// rounding analysis needs (it sums |A_ij x_j| anyway).
//
// On the GPU the operations use the _rn intrinsics, which the compiler never
// contracts into fused multiply-adds (a contraction would break the error-free
// steps); the host build (test emulator) compiles without contraction.
#pragma once

#include <cmath>
#include <cstring>

#include "topo_common.cuh"

namespace topo {

namespace ddop {
TOPO_HD float add(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
TOPO_HD float sub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
TOPO_HD float mul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
TOPO_HD float fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}
}  // namespace ddop

struct dd {
  float hi, lo;
  dd() = default;
  TOPO_HD constexpr dd(float h, float l) : hi(h), lo(l) {}
  TOPO_HD constexpr dd(int v) : hi(float(v)), lo(0.f) {}  // small integers are exact
  // nearest pair to a double (constants fold at compile time)
  TOPO_HD constexpr dd(double v) : hi(float(v)), lo(float(v - double(float(v)))) {}
  TOPO_HD explicit operator double() const { return double(hi) + double(lo); }
};

template <class T>
struct IsDD {
  static constexpr bool value = false;
};
template <>
struct IsDD<dd> {
  static constexpr bool value = true;
};

TOPO_HD dd two_sum(float a, float b) {
  const float s = ddop::add(a, b);
  const float bb = ddop::sub(s, a);
  const float e = ddop::add(ddop::sub(a, ddop::sub(s, bb)), ddop::sub(b, bb));
  return dd(s, e);
}
TOPO_HD dd fast_two_sum(float a, float b) {
  const float s = ddop::add(a, b);
  return dd(s, ddop::sub(b, ddop::sub(s, a)));
}

TOPO_HD dd operator-(dd a) { return dd(-a.hi, -a.lo); }
TOPO_HD dd operator+(dd a, dd b) {
  const dd s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, ddop::add(s.lo, ddop::add(a.lo, b.lo)));
}
TOPO_HD dd operator-(dd a, dd b) { return a + (-b); }
TOPO_HD dd operator*(dd a, dd b) {
  const float p = ddop::mul(a.hi, b.hi);
  float e = ddop::fma(a.hi, b.hi, -p);
  e = ddop::fma(a.hi, b.lo, e);
  e = ddop::fma(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
// a0 b0 + a1 b1 + a2 b2 with one renormalisation: the three hi products exact
// (TwoProd), their cross terms and rounding errors summed in float, the hi parts
// by two TwoSums.  31 FP32 operations instead of 43 for three products and two
// sums, the error again bounded relative to sum |a_i b_i|.  Float and double keep
// their expression unchanged.
template <class T>
TOPO_HD T dot3(T a0, T b0, T a1, T b1, T a2, T b2) {
  if constexpr (IsDD<T>::value) {
    const float p0 = ddop::mul(a0.hi, b0.hi), p1 = ddop::mul(a1.hi, b1.hi), p2 = ddop::mul(a2.hi, b2.hi);
    float e = ddop::fma(a0.hi, b0.hi, -p0);
    e = ddop::fma(a0.hi, b0.lo, e);
    e = ddop::fma(a0.lo, b0.hi, e);
    e = ddop::add(e, ddop::fma(a1.hi, b1.hi, -p1));
    e = ddop::fma(a1.hi, b1.lo, e);
    e = ddop::fma(a1.lo, b1.hi, e);
    e = ddop::add(e, ddop::fma(a2.hi, b2.hi, -p2));
    e = ddop::fma(a2.hi, b2.lo, e);
    e = ddop::fma(a2.lo, b2.hi, e);
    const dd s1 = two_sum(p0, p1);
    const dd s2 = two_sum(s1.hi, p2);
    return fast_two_sum(s2.hi, ddop::add(ddop::add(s1.lo, s2.lo), e));
  } else {
    return a0 * b0 + a1 * b1 + a2 * b2;
  }
}

// K x for a small integer constant K, written so that the float and double
// operators keep their exact arithmetic (T(K) * x) and the pair type takes the
// cheap exact forms: a power of two scales both parts, 3 is one TwoProd.
template <int K, class T>
TOPO_HD T mul_small(T x) {
  if constexpr (IsDD<T>::value) {
    if constexpr ((K & (K - 1)) == 0) {
      return T(ddop::mul(x.hi, float(K)), ddop::mul(x.lo, float(K)));
    } else {
      const float p = ddop::mul(x.hi, float(K));
      float e = ddop::fma(x.hi, float(K), -p);
      e = ddop::fma(x.lo, float(K), e);
      return fast_two_sum(p, e);
    }
  } else {
    return T(K) * x;
  }
}
// x / 2 (exact in every type)
template <class T>
TOPO_HD T half_of(T x) {
  if constexpr (IsDD<T>::value) return T(ddop::mul(x.hi, 0.5f), ddop::mul(x.lo, 0.5f));
  else return T(0.5) * x;
}

TOPO_HD dd& operator+=(dd& a, dd b) { return a = a + b; }
TOPO_HD dd& operator-=(dd& a, dd b) { return a = a - b; }
TOPO_HD dd& operator*=(dd& a, dd b) { return a = a * b; }

// The nearest pair to a double.  On the GPU the split is done on the integer
// pipe (the double's bits give hi by rounding the mantissa to 24 bits and lo
// from the 29 bits left over) for 2^-74 <= |x| < 2^100, the range of every
// value the operator meets; zero and the rest go through conversions.
TOPO_HD dd dd_from_double(double x) {
#if defined(__CUDA_ARCH__)
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned top = unsigned(b >> 32);
  const int e = int((top >> 20) & 0x7ffu);  // biased exponent
  const unsigned sign = top & 0x80000000u;
  if (e >= 949 && e < 1123) {
    const unsigned long long m = b & 0xfffffffffffffull;       // 52 fraction bits
    unsigned fb = sign | (unsigned(e - 896) << 23) | unsigned(m >> 29);  // truncated to 23
    long long r = static_cast<long long>(m & 0x1fffffffull);    // the 29 bits below
    if (r > 0x10000000ll || (r == 0x10000000ll && (fb & 1u))) {  // round to nearest even
      fb += 1u;                                                  // (a carry moves the exponent)
      r -= 0x20000000ll;
    }
    float lo = 0.f;
    if (r != 0) {
      // |r| < 2^29 in units of 2^(e - 1075); the float conversion keeps 24 bits, and the
      // scale goes into the exponent field (the result stays a normal float in this range)
      const int ri = int(r);  // |r| <= 2^28: a 32-bit conversion
      const float f = float(sign ? -ri : ri);
      lo = __uint_as_float(__float_as_uint(f) + (unsigned(e - 1075) << 23));
    }
    return dd(__uint_as_float(fb), lo);
  }
  if (e == 0) return dd(__uint_as_float(sign), 0.f);  // zero (and FP64 subnormals, below any use)
#endif
  const float h = float(x);
  return dd(h, float(x - double(h)));
}

// A double rounded to the nearest float (ties to even), on the integer pipe on the
// GPU for results in the normal float range and zero; the rest through a conversion.
TOPO_HD float float_from_double(double x) {
#if defined(__CUDA_ARCH__)
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned top = unsigned(b >> 32);
  const int e = int((top >> 20) & 0x7ffu);
  const unsigned sign = top & 0x80000000u;
  if (e >= 897 && e < 1151) {
    const unsigned long long m = b & 0xfffffffffffffull;
    unsigned fb = sign | (unsigned(e - 896) << 23) | unsigned(m >> 29);
    const unsigned r = unsigned(m & 0x1fffffffull);
    if (r > 0x10000000u || (r == 0x10000000u && (fb & 1u))) fb += 1u;  // a carry moves the exponent
    return __uint_as_float(fb);
  }
  if (e == 0) return __uint_as_float(sign);
#endif
  return float(x);
}

// Exact float -> double on the integer pipe for normal floats and zero.
TOPO_HD double dd_widen(float f) {
#if defined(__CUDA_ARCH__)
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xffu;
  const unsigned long long s = static_cast<unsigned long long>(u & 0x80000000u) << 32;
  if (ex != 0u && ex != 255u)
    return __longlong_as_double(static_cast<long long>(s | (static_cast<unsigned long long>(ex + 896u) << 52) |
                                                       (static_cast<unsigned long long>(u & 0x7fffffu) << 29)));
  if ((u << 1) == 0u) return __longlong_as_double(static_cast<long long>(s));
#endif
  return double(f);
}

// A double carried bit for bit in the two words of a dd (no arithmetic): the
// pair-of-FP32 apply keeps its operand this way and takes the difference form's
// u_k - u_A in FP64, which is exact for nearby values (Sterbenz) and otherwise
// rounded relative to the difference; splitting u first would round each value
// to 48 bits relative to |u| instead.
TOPO_HD dd dd_pack_double(double x) {
#if defined(__CUDA_ARCH__)
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  return dd(__uint_as_float(unsigned(b)), __uint_as_float(unsigned(b >> 32)));
#else
  unsigned long long b;
  std::memcpy(&b, &x, sizeof(b));
  const unsigned lo = unsigned(b), hi = unsigned(b >> 32);
  float f0, f1;
  std::memcpy(&f0, &lo, sizeof(f0));
  std::memcpy(&f1, &hi, sizeof(f1));
  return dd(f0, f1);
#endif
}
TOPO_HD double dd_unpack_double(dd v) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(static_cast<long long>(
      (static_cast<unsigned long long>(__float_as_uint(v.lo)) << 32) | __float_as_uint(v.hi)));
#else
  unsigned lo, hi;
  std::memcpy(&lo, &v.hi, sizeof(lo));
  std::memcpy(&hi, &v.lo, sizeof(hi));
  const unsigned long long b = (static_cast<unsigned long long>(hi) << 32) | lo;
  double x;
  std::memcpy(&x, &b, sizeof(x));
  return x;
#endif
}

// hi + lo rounded to a double (one FP64 addition)
TOPO_HD double dd_to_double(dd v) { return dd_widen(v.hi) + dd_widen(v.lo); }

}  // namespace topo
