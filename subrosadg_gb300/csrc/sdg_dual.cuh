// Forward-mode dual numbers for the tangent-linear and adjoint kernels of the GB300 DG path.
//
// Dual<K> carries a value and K directional derivatives.  The pointwise physics (sdg_device.cuh) is
// generic over its scalar type: with double it is the forward path, with Dual<1> it is its tangent-linear
// model (exact, no differencing), and with Dual<K> seeded on K inputs it yields K columns of the pointwise
// Jacobian, which the adjoint kernels contract with the adjoint vector (J^T lambda, column by column).
// The scalar helpers below (fmaT, rcpT, sqrtT, expT, logT, powT, fabsT, fmaxT, valueOf) are overloaded for double, where
// they are the hardware operations the forward path uses, and for Dual<K>.
#pragma once

namespace sdg {

__device__ __forceinline__ double rcp(double x);

template <int K>
struct Dual {
  double v;
  double d[K];
  __device__ __forceinline__ Dual() {}
  __device__ __forceinline__ Dual(double x) : v(x) {
#pragma unroll
    for (int k = 0; k < K; ++k) d[k] = 0.0;
  }
};

template <class T> struct ScalarTraits { static constexpr bool dual = false; };
template <int K> struct ScalarTraits<Dual<K>> { static constexpr bool dual = true; };

__device__ __forceinline__ double valueOf(double x) { return x; }
template <int K> __device__ __forceinline__ double valueOf(const Dual<K>& x) { return x.v; }

// ---- arithmetic ------------------------------------------------------------------------------------
template <int K> __device__ __forceinline__ Dual<K> operator-(const Dual<K>& a) {
  Dual<K> r; r.v = -a.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator+(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r; r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator-(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r; r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator*(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r; r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = fma(a.d[k], b.v, a.v * b.d[k]);
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator+(const Dual<K>& a, double b) {
  Dual<K> r = a; r.v = a.v + b; return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator+(double b, const Dual<K>& a) { return a + b; }
template <int K> __device__ __forceinline__ Dual<K> operator-(const Dual<K>& a, double b) {
  Dual<K> r = a; r.v = a.v - b; return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator-(double b, const Dual<K>& a) {
  Dual<K> r; r.v = b - a.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator*(const Dual<K>& a, double b) {
  Dual<K> r; r.v = a.v * b;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b;
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator*(double b, const Dual<K>& a) { return a * b; }
template <int K> __device__ __forceinline__ Dual<K> operator/(const Dual<K>& a, const Dual<K>& b) {
  const double q = a.v / b.v, ib = 1.0 / b.v;
  Dual<K> r; r.v = q;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = fma(-q, b.d[k], a.d[k]) * ib;
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator/(const Dual<K>& a, double b) {
  const double ib = 1.0 / b;
  Dual<K> r; r.v = a.v / b;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * ib;
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> operator/(double a, const Dual<K>& b) {
  const double q = a / b.v, ib = 1.0 / b.v;
  Dual<K> r; r.v = q;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = -q * b.d[k] * ib;
  return r;
}
template <int K> __device__ __forceinline__ Dual<K>& operator+=(Dual<K>& a, const Dual<K>& b) { a = a + b; return a; }
template <int K> __device__ __forceinline__ Dual<K>& operator-=(Dual<K>& a, const Dual<K>& b) { a = a - b; return a; }
template <int K> __device__ __forceinline__ Dual<K>& operator*=(Dual<K>& a, const Dual<K>& b) { a = a * b; return a; }
template <int K> __device__ __forceinline__ Dual<K>& operator*=(Dual<K>& a, double b) { a = a * b; return a; }

// comparisons act on values (the branch structure of the forward evaluation is kept)
template <int K> __device__ __forceinline__ bool operator<(const Dual<K>& a, const Dual<K>& b) { return a.v < b.v; }
template <int K> __device__ __forceinline__ bool operator>(const Dual<K>& a, const Dual<K>& b) { return a.v > b.v; }
template <int K> __device__ __forceinline__ bool operator<=(const Dual<K>& a, const Dual<K>& b) { return a.v <= b.v; }
template <int K> __device__ __forceinline__ bool operator>=(const Dual<K>& a, const Dual<K>& b) { return a.v >= b.v; }
template <int K> __device__ __forceinline__ bool operator<(const Dual<K>& a, double b) { return a.v < b; }
template <int K> __device__ __forceinline__ bool operator>(const Dual<K>& a, double b) { return a.v > b; }
template <int K> __device__ __forceinline__ bool operator<=(const Dual<K>& a, double b) { return a.v <= b; }
template <int K> __device__ __forceinline__ bool operator>=(const Dual<K>& a, double b) { return a.v >= b; }
template <int K> __device__ __forceinline__ bool operator<(double a, const Dual<K>& b) { return a < b.v; }
template <int K> __device__ __forceinline__ bool operator>(double a, const Dual<K>& b) { return a > b.v; }
template <int K> __device__ __forceinline__ bool operator<=(double a, const Dual<K>& b) { return a <= b.v; }
template <int K> __device__ __forceinline__ bool operator>=(double a, const Dual<K>& b) { return a >= b.v; }

// ---- scalar helpers (double: the forward path's operations) ------------------------------------------
__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }
template <int K> __device__ __forceinline__ Dual<K> fmaT(const Dual<K>& a, const Dual<K>& b, const Dual<K>& c) {
  Dual<K> r; r.v = fma(a.v, b.v, c.v);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = fma(a.d[k], b.v, fma(a.v, b.d[k], c.d[k]));
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> fmaT(double a, const Dual<K>& b, const Dual<K>& c) {
  Dual<K> r; r.v = fma(a, b.v, c.v);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = fma(a, b.d[k], c.d[k]);
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> fmaT(const Dual<K>& a, double b, const Dual<K>& c) {
  return fmaT(b, a, c);
}
template <int K> __device__ __forceinline__ Dual<K> fmaT(const Dual<K>& a, const Dual<K>& b, double c) {
  Dual<K> r; r.v = fma(a.v, b.v, c);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = fma(a.d[k], b.v, a.v * b.d[k]);
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> fmaT(double a, double b, const Dual<K>& c) {
  Dual<K> r = c; r.v = fma(a, b, c.v); return r;
}
template <int K> __device__ __forceinline__ Dual<K> fmaT(const Dual<K>& a, double b, double c) {
  Dual<K> r; r.v = fma(a.v, b, c);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b;
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> fmaT(double a, const Dual<K>& b, double c) { return fmaT(b, a, c); }

__device__ __forceinline__ double rcpT(double x) { return rcp(x); }
template <int K> __device__ __forceinline__ Dual<K> rcpT(const Dual<K>& x) {
  const double r = rcp(x.v), m = -r * r;
  Dual<K> o; o.v = r;
#pragma unroll
  for (int k = 0; k < K; ++k) o.d[k] = m * x.d[k];
  return o;
}
__device__ __forceinline__ double sqrtT(double x) { return sqrt(x); }
template <int K> __device__ __forceinline__ Dual<K> sqrtT(const Dual<K>& x) {
  const double s = sqrt(x.v), h = 0.5 / s;
  Dual<K> o; o.v = s;
#pragma unroll
  for (int k = 0; k < K; ++k) o.d[k] = h * x.d[k];
  return o;
}
__device__ __forceinline__ double expT(double x) { return exp(x); }
template <int K> __device__ __forceinline__ Dual<K> expT(const Dual<K>& x) {
  const double e = exp(x.v);
  Dual<K> o; o.v = e;
#pragma unroll
  for (int k = 0; k < K; ++k) o.d[k] = e * x.d[k];
  return o;
}
__device__ __forceinline__ double logT(double x) { return log(x); }
template <int K> __device__ __forceinline__ Dual<K> logT(const Dual<K>& x) {
  const double ix = 1.0 / x.v;
  Dual<K> o; o.v = log(x.v);
#pragma unroll
  for (int k = 0; k < K; ++k) o.d[k] = ix * x.d[k];
  return o;
}
__device__ __forceinline__ double powT(double x, double y) { return pow(x, y); }
template <int K> __device__ __forceinline__ Dual<K> powT(const Dual<K>& x, double y) {
  const double p = pow(x.v, y), dp = y * pow(x.v, y - 1.0);
  Dual<K> o; o.v = p;
#pragma unroll
  for (int k = 0; k < K; ++k) o.d[k] = dp * x.d[k];
  return o;
}
__device__ __forceinline__ double fabsT(double x) { return fabs(x); }
template <int K> __device__ __forceinline__ Dual<K> fabsT(const Dual<K>& x) { return x.v < 0.0 ? -x : x; }
__device__ __forceinline__ double fmaxT(double a, double b) { return fmax(a, b); }
template <int K> __device__ __forceinline__ Dual<K> fmaxT(const Dual<K>& a, const Dual<K>& b) { return a.v >= b.v ? a : b; }
template <int K> __device__ __forceinline__ Dual<K> fmaxT(double a, const Dual<K>& b) { return a >= b.v ? Dual<K>(a) : b; }
template <int K> __device__ __forceinline__ Dual<K> fmaxT(const Dual<K>& a, double b) { return a.v >= b ? a : Dual<K>(b); }

}  // namespace sdg
