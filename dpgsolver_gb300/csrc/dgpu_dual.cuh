// Forward-mode dual numbers with K derivative directions, for the pointwise Jacobians of the numerical fluxes in
// the adjoint (vector-Jacobian product) kernels. The flux functions of dgpu_physics.cuh are templated on their
// scalar type, the way the reference instantiates its flux code for double and double complex to obtain its
// complex-step linearisation (def_templates_type_dc.h); comparisons and selections act on the value, as the
// reference's real_T comparisons do, so the derivative is that of the branch the value takes.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace dgpu {

template <int K>
struct Dual {
	double v;
	double d[K];
	__device__ __forceinline__ Dual() {}
	__device__ __forceinline__ Dual(double x) : v(x)
	{
#pragma unroll
		for (int k = 0; k < K; ++k)
			d[k] = 0.0;
	}
};

template <int K>
__device__ __forceinline__ Dual<K> operator+(const Dual<K>& a, const Dual<K>& b)
{
	Dual<K> r;
	r.v = a.v + b.v;
#pragma unroll
	for (int k = 0; k < K; ++k)
		r.d[k] = a.d[k] + b.d[k];
	return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(const Dual<K>& a, const Dual<K>& b)
{
	Dual<K> r;
	r.v = a.v - b.v;
#pragma unroll
	for (int k = 0; k < K; ++k)
		r.d[k] = a.d[k] - b.d[k];
	return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator-(const Dual<K>& a)
{
	Dual<K> r;
	r.v = -a.v;
#pragma unroll
	for (int k = 0; k < K; ++k)
		r.d[k] = -a.d[k];
	return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(const Dual<K>& a, const Dual<K>& b)
{
	Dual<K> r;
	r.v = a.v * b.v;
#pragma unroll
	for (int k = 0; k < K; ++k)
		r.d[k] = a.d[k] * b.v + a.v * b.d[k];
	return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator/(const Dual<K>& a, const Dual<K>& b)
{
	Dual<K> r;
	const double inv = 1.0 / b.v;
	r.v = a.v * inv;
#pragma unroll
	for (int k = 0; k < K; ++k)
		r.d[k] = (a.d[k] - r.v * b.d[k]) * inv;
	return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator+(const Dual<K>& a, double b) { return a + Dual<K>(b); }
template <int K>
__device__ __forceinline__ Dual<K> operator+(double a, const Dual<K>& b) { return Dual<K>(a) + b; }
template <int K>
__device__ __forceinline__ Dual<K> operator-(const Dual<K>& a, double b) { return a - Dual<K>(b); }
template <int K>
__device__ __forceinline__ Dual<K> operator-(double a, const Dual<K>& b) { return Dual<K>(a) - b; }
template <int K>
__device__ __forceinline__ Dual<K> operator*(const Dual<K>& a, double b)
{
	Dual<K> r;
	r.v = a.v * b;
#pragma unroll
	for (int k = 0; k < K; ++k)
		r.d[k] = a.d[k] * b;
	return r;
}
template <int K>
__device__ __forceinline__ Dual<K> operator*(double a, const Dual<K>& b) { return b * a; }
template <int K>
__device__ __forceinline__ Dual<K> operator/(const Dual<K>& a, double b) { return a * (1.0 / b); }
template <int K>
__device__ __forceinline__ Dual<K> operator/(double a, const Dual<K>& b) { return Dual<K>(a) / b; }
template <int K>
__device__ __forceinline__ Dual<K>& operator+=(Dual<K>& a, const Dual<K>& b)
{
	a = a + b;
	return a;
}
template <int K>
__device__ __forceinline__ Dual<K>& operator*=(Dual<K>& a, double b)
{
	a = a * b;
	return a;
}

template <int K>
__device__ __forceinline__ bool operator<(const Dual<K>& a, const Dual<K>& b) { return a.v < b.v; }
template <int K>
__device__ __forceinline__ bool operator>(const Dual<K>& a, const Dual<K>& b) { return a.v > b.v; }
template <int K>
__device__ __forceinline__ bool operator<(const Dual<K>& a, double b) { return a.v < b; }
template <int K>
__device__ __forceinline__ bool operator>(const Dual<K>& a, double b) { return a.v > b; }

// sqrt with the derivative 1/(2 sqrt(x)); at x = 0 the derivative is taken as 0 (the one-sided subgradient of
// |V| = sqrt(V^2) at rest), where the exact derivative does not exist.
template <int K>
__device__ __forceinline__ Dual<K> sqrt(const Dual<K>& a)
{
	Dual<K> r;
	r.v = ::sqrt(a.v);
	const double s = (r.v > 0.0 ? 0.5 / r.v : 0.0);
#pragma unroll
	for (int k = 0; k < K; ++k)
		r.d[k] = a.d[k] * s;
	return r;
}

// |a| for comparisons (the reference compares abs_T values); the derivative follows the sign of the value.
template <int K>
__device__ __forceinline__ Dual<K> fabs(const Dual<K>& a) { return a.v < 0.0 ? -a : a; }

// a^b for a constant exponent (the boundary values' pow_T): derivative b a^(b-1) = b a^b / a, for a > 0.
template <int K>
__device__ __forceinline__ Dual<K> pow(const Dual<K>& a, double b)
{
	Dual<K> r;
	r.v = ::pow(a.v, b);
	const double s = b * r.v / a.v;
#pragma unroll
	for (int k = 0; k < K; ++k)
		r.d[k] = a.d[k] * s;
	return r;
}

}  // namespace dgpu
