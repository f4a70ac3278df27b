/******************************************************************************
common.cuh -- complex arithmetic, fast reciprocals and shared constants for
the device code.

Complex values are plain double2 / float2 (real in .x, imaginary in .y) so
that they load and store as single 16- or 8-byte vectors.  Division is
written as multiplication by one real reciprocal of |d|^2 instead of the
reference's Smith division (include/complex.cuh:218-280): a single
reciprocal per complex divide is what the GB300 FP64 pipe can afford.
******************************************************************************/
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define CCF_HD __host__ __device__ __forceinline__
#define CCF_D __device__ __forceinline__

namespace ccf
{

constexpr int MAX_ORDER = 31;          /* highest FMM expansion order (reference: include/tree_node.cuh:20) */
constexpr int MAX_NEAR = 32;           /* leaf + neighbours star bound (include/tree_node.cuh:14) */
constexpr int MAX_TAYLOR = 101;        /* include/ccf.cuh:79 */
constexpr int MAX_SMOOTH_TERMS = 64;   /* >= (MAX_TAYLOR + 3) / 2 + 1 */
constexpr double PI = 3.141592653589793238462643383279502884;

/* ---------------- FP64 complex ---------------- */
CCF_HD double2 cx(double r, double i) { return make_double2(r, i); }
CCF_HD double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
CCF_HD double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
CCF_HD double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
CCF_HD double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
CCF_HD double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
CCF_HD double cnorm2(double2 a) { return a.x * a.x + a.y * a.y; }

/* FP64 reciprocal: hardware seed (rcp.approx.ftz.f64) refined by two
   Newton-Raphson steps r <- r + r (1 - x r); each step squares the relative
   error, taking the ~2^-20 seed below one ulp.  Valid for normal x. */
CCF_D double rcp64(double x)
{
	double r;
	asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
	double e = fma(-x, r, 1.0);
	r = fma(r, e, r);
	e = fma(-x, r, 1.0);
	r = fma(r, e, r);
	return r;
}

/* 1 / d for complex d, one real reciprocal */
CCF_D double2 cinv(double2 d)
{
	double r = rcp64(d.x * d.x + d.y * d.y);
	return make_double2(d.x * r, -d.y * r);
}
/* a / b */
CCF_D double2 cdiv(double2 a, double2 b)
{
	double r = rcp64(b.x * b.x + b.y * b.y);
	return make_double2((a.x * b.x + a.y * b.y) * r, (a.y * b.x - a.x * b.y) * r);
}
CCF_D double cabs64(double2 a) { return hypot(a.x, a.y); }

/* ---------------- FP32 complex ---------------- */
CCF_HD float2 fx(float r, float i) { return make_float2(r, i); }
CCF_HD float2 fadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
CCF_HD float2 fsub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
CCF_HD float2 fmulc(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
CCF_HD float2 fscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

/* FP32 reciprocal: the special-function unit's rcp.approx (about 1 ulp) */
CCF_D float rcp32(float x)
{
	float r;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
	return r;
}
CCF_D float2 finv(float2 d)
{
	float r = rcp32(d.x * d.x + d.y * d.y);
	return make_float2(d.x * r, -d.y * r);
}
CCF_D float2 fdivc(float2 a, float2 b)
{
	float r = rcp32(b.x * b.x + b.y * b.y);
	return make_float2((a.x * b.x + a.y * b.y) * r, (a.y * b.x - a.x * b.y) * r);
}

/* split an FP64 complex into a high FP32 part and the FP32 remainder */
CCF_D float4 split_hilo(double2 z)
{
	float hx = __double2float_rn(z.x);
	float hy = __double2float_rn(z.y);
	float lx = __double2float_rn(z.x - (double)hx);
	float ly = __double2float_rn(z.y - (double)hy);
	return make_float4(hx, hy, lx, ly);
}

/* ordered-bits max of a non-negative double (bit order equals value order) */
CCF_D void atomic_max_nonneg(unsigned long long* addr, double v)
{
	atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

} /* namespace ccf */
