/******************************************************************************
dfloat.cuh -- double-float arithmetic: a value is the unevaluated sum hi + lo
of two FP32 numbers with |lo| <= ulp(hi)/2, about 48 significant bits.

GB300 issues 62 FP32 FMAs for every FP64 FMA, so the critical-curve function
of the mixed-precision solver is evaluated in double-float on the FP32 pipe
instead of in FP64.  The building blocks are the classical error-free
transformations:
  two_sum       Knuth, TAOCP vol. 2, 4.2.2 (exact sum and rounding error)
  fast_two_sum  Dekker 1971 (|a| >= |b|)
  two_prod      product and its exact error from one FMA
and the double-float add / multiply / reciprocal built on them (Dekker 1971;
the same compositions as the QD library of Hida, Li and Bailey).  Every
operation uses the _rn intrinsics so the compiler cannot contract or
reassociate them.
******************************************************************************/
#pragma once

#include "common.cuh"

namespace ccf
{

struct dfl
{
	float hi, lo;
};

struct dfc   /* complex double-float */
{
	dfl re, im;
};

CCF_D dfl two_sum(float a, float b)
{
	float s = __fadd_rn(a, b);
	float v = __fsub_rn(s, a);
	float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
	return {s, e};
}
CCF_D dfl fast_two_sum(float a, float b)
{
	float s = __fadd_rn(a, b);
	float e = __fsub_rn(b, __fsub_rn(s, a));
	return {s, e};
}
CCF_D dfl two_prod(float a, float b)
{
	float p = __fmul_rn(a, b);
	float e = __fmaf_rn(a, b, -p);
	return {p, e};
}

CCF_D dfl df_from_double(double x)
{
	float h = __double2float_rn(x);
	float l = __double2float_rn(x - (double)h);
	return {h, l};
}
CCF_D double df_to_double(dfl a) { return (double)a.hi + (double)a.lo; }
CCF_D dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }

/* accurate sum (error relative to |a + b|) */
CCF_D dfl df_add(dfl a, dfl b)
{
	dfl s = two_sum(a.hi, b.hi);
	dfl t = two_sum(a.lo, b.lo);
	s.lo = __fadd_rn(s.lo, t.hi);
	s = fast_two_sum(s.hi, s.lo);
	s.lo = __fadd_rn(s.lo, t.lo);
	return fast_two_sum(s.hi, s.lo);
}
CCF_D dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }

CCF_D dfl df_mul(dfl a, dfl b)
{
	dfl p = two_prod(a.hi, b.hi);
	p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
	p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
	return fast_two_sum(p.hi, p.lo);
}
CCF_D dfl df_mul_f(dfl a, float b)
{
	dfl p = two_prod(a.hi, b);
	p.lo = __fmaf_rn(a.lo, b, p.lo);
	return fast_two_sum(p.hi, p.lo);
}
CCF_D dfl df_sqr(dfl a)
{
	dfl p = two_prod(a.hi, a.hi);
	p.lo = __fmaf_rn(__fmul_rn(2.0f, a.hi), a.lo, p.lo);
	return fast_two_sum(p.hi, p.lo);
}
/* sum without the low-part renormalisation: error relative to |a| + |b|,
   for accumulations whose terms do not cancel to far below their size */
CCF_D dfl df_add_fast(dfl a, dfl b)
{
	dfl s = two_sum(a.hi, b.hi);
	s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
	return fast_two_sum(s.hi, s.lo);
}

/* 1/a: FP32 estimate q1, residual r = 1 - a q1, one correction q1 r.  a q1
   is formed in double-float (p); p.hi lies within 2^-22 of 1, so 1 - p.hi is
   exact and r needs FP32 accuracy only (q1 r is 2^-23 of the result) */
CCF_D dfl df_rcp(dfl a)
{
	float q1 = rcp32(a.hi);
	dfl p = df_mul_f(a, q1);
	float r = __fsub_rn(__fsub_rn(1.0f, p.hi), p.lo);
	float q2 = __fmul_rn(r, q1);
	return fast_two_sum(q1, q2);
}

/* running double-float sum: the leading parts add exactly (two_sum), the low
   parts and those roundings collect in one FP32 word; dfacc_get
   renormalises.  Error ~2^-48 of the sum of |terms| */
struct dfacc
{
	float hi, lo;
};
CCF_D void dfacc_add(dfacc& a, dfl x)
{
	const dfl s = two_sum(a.hi, x.hi);
	a.hi = s.hi;
	a.lo = __fadd_rn(a.lo, __fadd_rn(s.lo, x.lo));
}
CCF_D dfl dfacc_get(dfacc a) { return fast_two_sum(a.hi, a.lo); }
/* a += x y */
CCF_D void dfacc_fma(dfacc& a, dfl x, dfl y)
{
	const float p = __fmul_rn(x.hi, y.hi);
	const float pe = __fmaf_rn(x.hi, y.hi, -p);
	const dfl s = two_sum(a.hi, p);
	a.hi = s.hi;
	a.lo = __fadd_rn(a.lo, __fadd_rn(s.lo, __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, pe))));
}

/* x^2 + y^2, double-float, one renormalisation (no cancellation: error
   ~2^-47 of the result) */
CCF_D dfl df_sumsq(dfl x, dfl y)
{
	const float p = __fmul_rn(x.hi, x.hi);
	const float pe = __fmaf_rn(x.hi, x.hi, -p);
	const float q = __fmul_rn(y.hi, y.hi);
	const float qe = __fmaf_rn(y.hi, y.hi, -q);
	const dfl s = two_sum(p, q);
	const float lo = __fadd_rn(__fadd_rn(pe, qe), __fmaf_rn(__fmul_rn(2.0f, x.hi), x.lo, __fmaf_rn(__fmul_rn(2.0f, y.hi), y.lo, s.lo)));
	return fast_two_sum(s.hi, lo);
}

/* complex */
CCF_D dfc dfc_from(double2 z) { return {df_from_double(z.x), df_from_double(z.y)}; }
CCF_D double2 dfc_to(dfc a) { return make_double2(df_to_double(a.re), df_to_double(a.im)); }
CCF_D dfc dfc_add(dfc a, dfc b) { return {df_add_fast(a.re, b.re), df_add_fast(a.im, b.im)}; }
CCF_D dfc dfc_mul(dfc a, dfc b)
{
	return {df_add(df_mul(a.re, b.re), df_neg(df_mul(a.im, b.im))), df_add_fast(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
CCF_D dfc dfc_load(float4 v) { return {{v.x, v.z}, {v.y, v.w}}; }

/* x y + u z + c, real double-float, one renormalisation: the products of the
   leading parts and c's leading part sum exactly (two_prod, two_sum), every
   lower-order term collects in one FP32 sum.  Error ~2^-47 of
   |x y| + |u z| + |c| */
CCF_D dfl df_dot2_add(dfl x, dfl y, dfl u, dfl z, dfl c)
{
	const float p = __fmul_rn(x.hi, y.hi);
	const float pe = __fmaf_rn(x.hi, y.hi, -p);
	const float q = __fmul_rn(u.hi, z.hi);
	const float qe = __fmaf_rn(u.hi, z.hi, -q);
	const dfl s = two_sum(p, q);
	const dfl t = two_sum(s.hi, c.hi);
	const float e1 = __fmaf_rn(x.lo, y.hi, __fmaf_rn(x.hi, y.lo, pe));
	const float e2 = __fmaf_rn(u.lo, z.hi, __fmaf_rn(u.hi, z.lo, qe));
	const float lo = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(__fadd_rn(s.lo, t.lo), c.lo));
	return fast_two_sum(t.hi, lo);
}

/* x y + u z, real double-float, one renormalisation: error ~2^-47 of
   |x y| + |u z| */
CCF_D dfl df_dot2(dfl x, dfl y, dfl u, dfl z)
{
	const float p = __fmul_rn(x.hi, y.hi);
	const float pe = __fmaf_rn(x.hi, y.hi, -p);
	const float q = __fmul_rn(u.hi, z.hi);
	const float qe = __fmaf_rn(u.hi, z.hi, -q);
	const dfl s = two_sum(p, q);
	const float e1 = __fmaf_rn(x.lo, y.hi, __fmaf_rn(x.hi, y.lo, pe));
	const float e2 = __fmaf_rn(u.lo, z.hi, __fmaf_rn(u.hi, z.lo, qe));
	return fast_two_sum(s.hi, __fadd_rn(__fadd_rn(e1, e2), s.lo));
}

/* a b + c, complex double-float (one Horner step) */
CCF_D dfc dfc_fma(dfc a, dfc b, dfc c)
{
	return {df_dot2_add(a.re, b.re, df_neg(a.im), b.im, c.re), df_dot2_add(a.re, b.im, a.im, b.re, c.im)};
}
CCF_D float4 dfc_pack(dfc a) { return make_float4(a.re.hi, a.im.hi, a.re.lo, a.im.lo); }

} /* namespace ccf */
