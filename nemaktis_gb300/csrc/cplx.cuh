// Minimal complex arithmetic for device and host code, FP32 or FP64 components.
#pragma once

#include <cuda_runtime.h>

namespace nbpm {

template <typename R>
struct alignas(2 * sizeof(R)) cx {
	R x, y;
};

template <typename R>
__host__ __device__ __forceinline__ cx<R> mk(R a, R b) { cx<R> r; r.x = a; r.y = b; return r; }
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator+(cx<R> a, cx<R> b) { return mk<R>(a.x + b.x, a.y + b.y); }
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator-(cx<R> a, cx<R> b) { return mk<R>(a.x - b.x, a.y - b.y); }
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator-(cx<R> a) { return mk<R>(-a.x, -a.y); }
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator*(cx<R> a, cx<R> b) {
	return mk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator*(R s, cx<R> a) { return mk<R>(s * a.x, s * a.y); }
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator*(cx<R> a, R s) { return mk<R>(s * a.x, s * a.y); }
template <typename R>
__host__ __device__ __forceinline__ cx<R>& operator+=(cx<R>& a, cx<R> b) { a.x += b.x; a.y += b.y; return a; }
template <typename R>
__host__ __device__ __forceinline__ cx<R>& operator-=(cx<R>& a, cx<R> b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename R>
__host__ __device__ __forceinline__ cx<R> conj(cx<R> a) { return mk<R>(a.x, -a.y); }

// Fused forms: a*b + c and c - a*b as four fused multiply-adds each, with no separately rounded
// product or sum (a * b + c through the operators above compiles to a multiply, a fused
// multiply-add and an add per component, six instructions instead of four).
__host__ __device__ __forceinline__ float fmar(float a, float b, float c) { return fmaf(a, b, c); }
__host__ __device__ __forceinline__ double fmar(double a, double b, double c) { return fma(a, b, c); }
template <typename R>
__host__ __device__ __forceinline__ cx<R> cfma(cx<R> a, cx<R> b, cx<R> c) {
	return mk<R>(fmar(a.x, b.x, fmar(-a.y, b.y, c.x)), fmar(a.x, b.y, fmar(a.y, b.x, c.y)));
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> cfnma(cx<R> a, cx<R> b, cx<R> c) {
	return mk<R>(fmar(-a.x, b.x, fmar(a.y, b.y, c.x)), fmar(-a.x, b.y, fmar(-a.y, b.x, c.y)));
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> cdiv(cx<R> a, cx<R> b) {
	// Smith's algorithm (scaled by the larger component of b) to avoid overflow.
	if(fabs(b.x) >= fabs(b.y)) {
		R r = b.y / b.x, d = b.x + b.y * r;
		return mk<R>((a.x + a.y * r) / d, (a.y - a.x * r) / d);
	}
	R r = b.x / b.y, d = b.y + b.x * r;
	return mk<R>((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> crecip(cx<R> b) { return cdiv(mk<R>(1, 0), b); }

// Narrowing / widening conversions.
template <typename R, typename S>
__host__ __device__ __forceinline__ cx<R> cvt(cx<S> a) { return mk<R>((R)a.x, (R)a.y); }

// exp, sin, cos of a complex FP64 argument from the real-valued library functions.
__host__ __device__ __forceinline__ cx<double> cexp_d(cx<double> z) {
	double e = exp(z.x), s, c;
	sincos(z.y, &s, &c);
	return mk<double>(e * c, e * s);
}
__host__ __device__ __forceinline__ cx<double> csin_d(cx<double> z) {
	double s, c;
	sincos(z.x, &s, &c);
	return mk<double>(s * cosh(z.y), c * sinh(z.y));
}
__host__ __device__ __forceinline__ cx<double> ccos_d(cx<double> z) {
	double s, c;
	sincos(z.x, &s, &c);
	return mk<double>(c * cosh(z.y), -s * sinh(z.y));
}

// FP32 counterparts (library expf, sincosf, coshf, sinhf).
__host__ __device__ __forceinline__ cx<float> cexp_f(cx<float> z) {
	float e = expf(z.x), s, c;
	sincosf(z.y, &s, &c);
	return mk<float>(e * c, e * s);
}
__host__ __device__ __forceinline__ cx<float> csin_f(cx<float> z) {
	float s, c;
	sincosf(z.x, &s, &c);
	return mk<float>(s * coshf(z.y), c * sinhf(z.y));
}
__host__ __device__ __forceinline__ cx<float> ccos_f(cx<float> z) {
	float s, c;
	sincosf(z.x, &s, &c);
	return mk<float>(c * coshf(z.y), -s * sinhf(z.y));
}

}  // namespace nbpm
