// Forward-mode dual numbers (value + K directional derivatives), FP64, host
// and device.  Used by the adjoint to form the exact local Jacobian of one
// patch's converged step from the same formulas the forward step evaluates.
#pragma once
#include <cmath>

namespace qdfn {
namespace ad {

template <int K>
struct Dual {
    double v;
    double d[K];
    __host__ __device__ Dual() : v(0) {
        for (int k = 0; k < K; ++k) d[k] = 0;
    }
    __host__ __device__ Dual(double x) : v(x) {   // a constant
        for (int k = 0; k < K; ++k) d[k] = 0;
    }
    __host__ __device__ static Dual var(double x, int k) {   // seeded in direction k
        Dual r(x);
        r.d[k] = 1.0;
        return r;
    }
};

#define QDFN_DUAL_LOOP for (int k = 0; k < K; ++k)

template <int K>
__host__ __device__ inline Dual<K> operator+(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v + b.v);
    QDFN_DUAL_LOOP r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator-(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v - b.v);
    QDFN_DUAL_LOOP r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator-(const Dual<K>& a) {
    Dual<K> r(-a.v);
    QDFN_DUAL_LOOP r.d[k] = -a.d[k];
    return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator*(const Dual<K>& a, const Dual<K>& b) {
    Dual<K> r(a.v * b.v);
    QDFN_DUAL_LOOP r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator/(const Dual<K>& a, const Dual<K>& b) {
    const double q = a.v / b.v;
    Dual<K> r(q);
    QDFN_DUAL_LOOP r.d[k] = (a.d[k] - q * b.d[k]) / b.v;
    return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator+(const Dual<K>& a, double b) { return a + Dual<K>(b); }
template <int K>
__host__ __device__ inline Dual<K> operator+(double a, const Dual<K>& b) { return Dual<K>(a) + b; }
template <int K>
__host__ __device__ inline Dual<K> operator-(const Dual<K>& a, double b) { return a - Dual<K>(b); }
template <int K>
__host__ __device__ inline Dual<K> operator-(double a, const Dual<K>& b) { return Dual<K>(a) - b; }
template <int K>
__host__ __device__ inline Dual<K> operator*(const Dual<K>& a, double b) {
    Dual<K> r(a.v * b);
    QDFN_DUAL_LOOP r.d[k] = a.d[k] * b;
    return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator*(double a, const Dual<K>& b) { return b * a; }
template <int K>
__host__ __device__ inline Dual<K> operator/(const Dual<K>& a, double b) { return a / Dual<K>(b); }
template <int K>
__host__ __device__ inline Dual<K> operator/(double a, const Dual<K>& b) { return Dual<K>(a) / b; }

template <int K>
__host__ __device__ inline Dual<K> exp(const Dual<K>& a) {
    const double e = ::exp(a.v);
    Dual<K> r(e);
    QDFN_DUAL_LOOP r.d[k] = e * a.d[k];
    return r;
}
template <int K>
__host__ __device__ inline Dual<K> log(const Dual<K>& a) {
    Dual<K> r(::log(a.v));
    QDFN_DUAL_LOOP r.d[k] = a.d[k] / a.v;
    return r;
}
template <int K>
__host__ __device__ inline Dual<K> cos(const Dual<K>& a) {
    const double s = ::sin(a.v);
    Dual<K> r(::cos(a.v));
    QDFN_DUAL_LOOP r.d[k] = -s * a.d[k];
    return r;
}
template <int K>
__host__ __device__ inline Dual<K> sin(const Dual<K>& a) {
    const double c = ::cos(a.v);
    Dual<K> r(::sin(a.v));
    QDFN_DUAL_LOOP r.d[k] = c * a.d[k];
    return r;
}
#undef QDFN_DUAL_LOOP

__host__ __device__ inline double value(double x) { return x; }
template <int K>
__host__ __device__ inline double value(const Dual<K>& x) { return x.v; }

}  // namespace ad
}  // namespace qdfn
