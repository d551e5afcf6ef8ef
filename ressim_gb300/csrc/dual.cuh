// Forward-mode dual numbers for the per-cell property chain: a value and its
// partial derivatives with respect to K cell unknowns (pressure and the
// component moles).  Comparisons act on the value, so branches follow the
// same path as the plain double evaluation.
#pragma once
#include <cmath>

namespace rsg {

template <int K>
struct Dual {
  double v;
  double d[K];
  __host__ __device__ Dual() : v(0) {
    for (int k = 0; k < K; ++k) d[k] = 0;
  }
  __host__ __device__ Dual(double x) : v(x) {
    for (int k = 0; k < K; ++k) d[k] = 0;
  }
  __host__ __device__ static Dual var(double x, int k) {
    Dual r(x);
    r.d[k] = 1;
    return r;
  }
};

template <int K>
__host__ __device__ inline Dual<K> operator+(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r(a.v + b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator-(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r(a.v - b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator-(const Dual<K>& a) {
  Dual<K> r(-a.v);
  for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator*(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r(a.v * b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator/(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r(a.v / b.v);
  for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
  return r;
}
#define RSG_DUAL_MIXED(op)                                                                      \
  template <int K>                                                                              \
  __host__ __device__ inline Dual<K> operator op(const Dual<K>& a, double b) {                  \
    return a op Dual<K>(b);                                                                     \
  }                                                                                             \
  template <int K>                                                                              \
  __host__ __device__ inline Dual<K> operator op(double a, const Dual<K>& b) {                  \
    return Dual<K>(a) op b;                                                                     \
  }
RSG_DUAL_MIXED(+)
RSG_DUAL_MIXED(-)
RSG_DUAL_MIXED(*)
RSG_DUAL_MIXED(/)
#undef RSG_DUAL_MIXED

template <int K>
__host__ __device__ inline Dual<K>& operator+=(Dual<K>& a, const Dual<K>& b) {
  return a = a + b;
}
template <int K>
__host__ __device__ inline Dual<K>& operator-=(Dual<K>& a, const Dual<K>& b) {
  return a = a - b;
}
template <int K>
__host__ __device__ inline Dual<K>& operator*=(Dual<K>& a, const Dual<K>& b) {
  return a = a * b;
}
template <int K>
__host__ __device__ inline Dual<K>& operator/=(Dual<K>& a, const Dual<K>& b) {
  return a = a / b;
}

template <int K>
__host__ __device__ inline Dual<K>& operator+=(Dual<K>& a, double b) {
  return a = a + Dual<K>(b);
}
template <int K>
__host__ __device__ inline Dual<K>& operator-=(Dual<K>& a, double b) {
  return a = a - Dual<K>(b);
}
template <int K>
__host__ __device__ inline Dual<K>& operator*=(Dual<K>& a, double b) {
  return a = a * Dual<K>(b);
}
template <int K>
__host__ __device__ inline Dual<K>& operator/=(Dual<K>& a, double b) {
  return a = a / Dual<K>(b);
}

#define RSG_DUAL_CMP(op)                                                                                        \
  template <int K>                                                                                              \
  __host__ __device__ inline bool operator op(const Dual<K>& a, const Dual<K>& b) { return a.v op b.v; }       \
  template <int K>                                                                                              \
  __host__ __device__ inline bool operator op(const Dual<K>& a, double b) { return a.v op b; }                 \
  template <int K>                                                                                              \
  __host__ __device__ inline bool operator op(double a, const Dual<K>& b) { return a op b.v; }
RSG_DUAL_CMP(<)
RSG_DUAL_CMP(<=)
RSG_DUAL_CMP(>)
RSG_DUAL_CMP(>=)
RSG_DUAL_CMP(==)
RSG_DUAL_CMP(!=)
#undef RSG_DUAL_CMP

// value of a scalar of either kind
__host__ __device__ inline double val(double x) { return x; }
template <int K>
__host__ __device__ inline double val(const Dual<K>& x) {
  return x.v;
}

// x^y for a constant exponent: d = y x^(y-1) dx
template <int K>
__device__ inline Dual<K> dual_pow(const Dual<K>& x, double y) {
  Dual<K> r(::pow(x.v, y));
  const double s = y * ::pow(x.v, y - 1);
  for (int k = 0; k < K; ++k) r.d[k] = s * x.d[k];
  return r;
}

__device__ inline bool is_nan(double x) { return ::isnan(x); }
template <int K>
__device__ inline bool is_nan(const Dual<K>& x) {
  return ::isnan(x.v);
}

}  // namespace rsg
