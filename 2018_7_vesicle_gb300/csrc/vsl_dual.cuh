// vsl_dual.cuh -- forward-mode dual numbers with N tangent directions.
//
// The adjoint kernels need, per node, the exact partial derivatives of a stage's update
// with respect to the stencil values and distances it reads.  Instantiating the per-node
// stencil templates of vsl_device.cuh / vsl_fused.cuh with Dual<T, N> in place of T
// evaluates each update once together with its N partials, so every branch the forward
// code takes (WENO weights with their epsilon, Godunov max/min switches, the interface
// insertion, minimum over the six distances) is differentiated exactly as it was
// evaluated.  Comparisons look at values only: at a switch the derivative of the branch
// taken is used.
#pragma once

#include <cmath>

namespace vsl {

template <typename T, int N> struct Dual {
    T v;
    T d[N];

    __device__ __forceinline__ Dual() : v(T(0))
    {
#pragma unroll
        for (int k = 0; k < N; ++k) d[k] = T(0);
    }
    // a constant (zero tangent); implicit so that T(c) and mixed expressions work
    __device__ __forceinline__ Dual(double c) : v(T(c))
    {
#pragma unroll
        for (int k = 0; k < N; ++k) d[k] = T(0);
    }
    // the independent variable number k with value x
    __device__ __forceinline__ static Dual var(T x, int k)
    {
        Dual r(0.0);
        r.v = x;
        r.d[k] = T(1);
        return r;
    }

    friend __device__ __forceinline__ Dual operator+(const Dual &a, const Dual &b)
    {
        Dual r;
        r.v = a.v + b.v;
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k];
        return r;
    }
    friend __device__ __forceinline__ Dual operator-(const Dual &a, const Dual &b)
    {
        Dual r;
        r.v = a.v - b.v;
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k];
        return r;
    }
    friend __device__ __forceinline__ Dual operator-(const Dual &a)
    {
        Dual r;
        r.v = -a.v;
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
        return r;
    }
    friend __device__ __forceinline__ Dual operator*(const Dual &a, const Dual &b)
    {
        Dual r;
        r.v = a.v * b.v;
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
        return r;
    }
    friend __device__ __forceinline__ Dual operator/(const Dual &a, const Dual &b)
    {
        Dual r;
        r.v = a.v / b.v;
        const T inv = T(1) / b.v;
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * inv;
        return r;
    }
    // scalar on either side (integer and floating literals of the stencil code)
    friend __device__ __forceinline__ Dual operator*(T s, const Dual &b)
    {
        Dual r;
        r.v = s * b.v;
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = s * b.d[k];
        return r;
    }
    friend __device__ __forceinline__ Dual operator*(const Dual &a, T s) { return s * a; }
    friend __device__ __forceinline__ Dual operator*(int s, const Dual &b) { return T(s) * b; }

    friend __device__ __forceinline__ bool operator<(const Dual &a, const Dual &b) { return a.v < b.v; }
    friend __device__ __forceinline__ bool operator>(const Dual &a, const Dual &b) { return a.v > b.v; }
    friend __device__ __forceinline__ bool operator<=(const Dual &a, const Dual &b) { return a.v <= b.v; }
    friend __device__ __forceinline__ bool operator>=(const Dual &a, const Dual &b) { return a.v >= b.v; }

    friend __device__ __forceinline__ Dual fabs(const Dual &a) { return a.v < T(0) ? -a : a; }
    // sqrt with a zero derivative at 0 (the Godunov norm of a flat stencil)
    friend __device__ __forceinline__ Dual sqrt(const Dual &a)
    {
        Dual r;
        r.v = sqrt(a.v);
        const T s = r.v > T(0) ? T(0.5) / r.v : T(0);
#pragma unroll
        for (int k = 0; k < N; ++k) r.d[k] = s * a.d[k];
        return r;
    }
};

}  // namespace vsl
