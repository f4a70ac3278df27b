/******************************************************************************
field_df.cuh -- the critical-curve function and the epilogue quantities in
double-float arithmetic, for the mixed-precision solver.

Same formulas as field.cuh (reference: include/alpha_star.cuh,
alpha_local.cuh, alpha_smooth.cuh, ccf_functions.cuh:33-121, :419-467), on
the FP32 pipe.  Coordinates are taken relative to the leaf centre before they
are split into double-float (the leaf-relative positions of the near stars are
formed in FP64 and stored split), so a difference z - z_i keeps ~1e-14 of the
leaf size; f comes out with an absolute error of ~1e-13 for ordinary roots,
four orders of magnitude below what moves a root by 1e-9 theta_star.  The
final assembly of f and of the caustic is done in FP64 from the
double-float partial results.  Off-field points (outside the root box) go
through the same evaluators with the direct star sums (star_term_df, summed
by the whole CTA in solver.cu) in place of the leaf's near sums and local
expansion.
******************************************************************************/
#pragma once

#include "dfloat.cuh"
#include "field.cuh"

namespace ccf
{

struct SumsDF
{
	dfc s1, s2;
};

/* s1 = sum m / d, s2 = sum m / d^2 over the leaf's near stars, d = z - z_i */
template <bool NEED1>
CCF_D SumsDF leaf_sums_df(const FieldView& F, int leaf, double2 z)
{
	const double2 c = F.leaf_center[leaf];
	const dfc zr = dfc_from(make_double2(z.x - c.x, z.y - c.y));
	SumsDF a;
	a.s1 = {{0.f, 0.f}, {0.f, 0.f}};
	a.s2 = a.s1;
	const int n = F.leaf_near_count[leaf];
	const float4* P = F.leaf_near_df + (size_t)leaf * MAX_NEAR;
	const float2* M = F.leaf_mass_df + (size_t)leaf * MAX_NEAR;
	for (int i = 0; i < n; i++)
	{
		const dfc s = dfc_load(P[i]);
		const float2 mm = M[i];
		const dfl m = {mm.x, mm.y};
		const dfl dx = df_sub(zr.re, s.re);
		const dfl dy = df_sub(zr.im, s.im);
		const dfl r = df_rcp(df_add_fast(df_sqr(dx), df_sqr(dy)));
		const dfl ix = df_mul(dx, r);
		const dfl iy = df_neg(df_mul(dy, r));                     /* 1/d */
		const dfl i2x = df_add(df_sqr(ix), df_neg(df_sqr(iy)));
		dfl i2y = df_mul(ix, iy);
		i2y = {2.f * i2y.hi, 2.f * i2y.lo};                        /* 1/d^2 */
		a.s2.re = df_add_fast(a.s2.re, df_mul(m, i2x));
		a.s2.im = df_add_fast(a.s2.im, df_mul(m, i2y));
		if (NEED1)
		{
			a.s1.re = df_add_fast(a.s1.re, df_mul(m, ix));
			a.s1.im = df_add_fast(a.s1.im, df_mul(m, iy));
		}
	}
	return a;
}

/* One star's terms at an off-field point z (absolute coordinates, double-
   float): d = z - z_i from the split star position p = (x_hi, y_hi, x_lo,
   y_lo) and split mass mm; adds m/d^2 to s2, m/d to s1 (NEED1) and m/d^3 to
   s3 in double-float (S3DF) or in FP32 to s3f.  Off-field points are at least
   the gap between the star field and the root box away from every star, so
   the ~2^-48 |z| resolution of the split coordinates is a relative error of
   ~1e-14 in each term. */
template <bool NEED1, bool S3DF>
CCF_D void star_term_df(SumsDF& a, dfc& s3, float2& s3f, const dfc& z, float4 p, float2 mm)
{
	const dfc s = dfc_load(p);
	const dfl m = {mm.x, mm.y};
	const dfl dx = df_sub(z.re, s.re);
	const dfl dy = df_sub(z.im, s.im);
	const dfl r = df_rcp(df_add_fast(df_sqr(dx), df_sqr(dy)));
	const dfl ix = df_mul(dx, r);
	const dfl iy = df_neg(df_mul(dy, r));                     /* 1/d */
	const dfl i2x = df_add(df_sqr(ix), df_neg(df_sqr(iy)));
	dfl i2y = df_mul(ix, iy);
	i2y = {2.f * i2y.hi, 2.f * i2y.lo};                        /* 1/d^2 */
	a.s2.re = df_add_fast(a.s2.re, df_mul(m, i2x));
	a.s2.im = df_add_fast(a.s2.im, df_mul(m, i2y));
	if (NEED1)
	{
		a.s1.re = df_add_fast(a.s1.re, df_mul(m, ix));
		a.s1.im = df_add_fast(a.s1.im, df_mul(m, iy));
	}
	if (S3DF)
	{
		const dfl i3x = df_add(df_mul(i2x, ix), df_neg(df_mul(i2y, iy)));
		const dfl i3y = df_add(df_mul(i2x, iy), df_mul(i2y, ix));   /* 1/d^3 */
		s3.re = df_add_fast(s3.re, df_mul(m, i3x));
		s3.im = df_add_fast(s3.im, df_mul(m, i3y));
	}
	else
	{
		const float i3x = i2x.hi * ix.hi - i2y.hi * iy.hi;
		const float i3y = i2x.hi * iy.hi + i2y.hi * ix.hi;
		s3f.x = fmaf(m.hi, i3x, s3f.x);
		s3f.y = fmaf(m.hi, i3y, s3f.y);
	}
}

/* Horner of a double-float coefficient block: sum_{i >= first} L[i] dz^(i - first) */
CCF_D dfc horner_df(const float4* L, int P, int first, dfc dz)
{
	/* each coefficient is loaded one step ahead of its use, so the load's
	   latency overlaps the previous step's arithmetic */
	dfc acc = dfc_load(L[P]);
	float4 nxt = L[P - 1];
	for (int i = P - 1; i >= first; i--)
	{
		const float4 cur = nxt;
		nxt = L[i > 0 ? i - 1 : 0];
		acc = dfc_fma(acc, dz, dfc_load(cur));
	}
	return acc;
}

CCF_D dfc leaf_dz_df(const FieldView& F, int leaf, double2 z)
{
	const double2 c = F.leaf_center[leaf];
	const dfc zr = dfc_from(make_double2(z.x - c.x, z.y - c.y));
	const float2 ihf = F.leaf_ih_df[leaf];
	const dfl ih = {ihf.x, ihf.y};
	return {df_mul(zr.re, ih), df_mul(zr.im, ih)};
}

/* d alpha_smooth / d zbar for the rectangular Taylor form, double-float */
CCF_D double2 smooth_dzbar_df(const FieldView& F, double2 z)
{
	if (F.smooth_m <= 0) return make_double2(F.smooth_k1, 0);
	const dfc zb = dfc_from(make_double2(z.x, -z.y));
	const dfc r = dfc_mul(zb, dfc_load(F.inv_corner_df));
	const dfc u = dfc_mul(r, r);
	dfc acc = dfc_load(F.smooth_d1_df[F.smooth_m - 1]);
	for (int m = F.smooth_m - 2; m >= 0; m--) acc = dfc_fma(acc, u, dfc_load(F.smooth_d1_df[m]));
	acc = dfc_mul(acc, u);
	double2 d = dfc_to(acc);
	d.x += F.smooth_k1;
	return d;
}

/* alpha_smooth for the rectangular Taylor form, double-float polynomial in
   w = zbar / c with the coefficients A_n c^n (the same polynomial as
   smooth_alpha's sum A_n zbar^n, whose coefficients underflow FP32) */
CCF_D double2 smooth_alpha_df(const FieldView& F, double2 z)
{
	const double k = F.kappa_star;
	const dfc w = dfc_mul(dfc_from(make_double2(z.x, -z.y)), dfc_load(F.inv_corner_df));
	const int n = F.taylor_smooth + 1;
	dfc acc = dfc_load(F.smooth_a_df[n]);
	for (int i = n - 1; i >= 0; i--) acc = dfc_fma(acc, w, dfc_load(F.smooth_a_df[i]));
	double2 a = cmul(dfc_to(acc), make_double2(0, -k / PI));
	a.x -= k * 2 * (F.corner.x + z.x);
	return a;
}

CCF_D double2 smooth_dzbar_any(const FieldView& F, double2 z)
{
	if (F.rectangular && F.approx && smooth_df_ok(F, z)) return smooth_dzbar_df(F, z);
	return smooth_dzbar(F, z);
}
CCF_D double2 smooth_alpha_any(const FieldView& F, double2 z)
{
	if (F.rectangular && F.approx && smooth_df_ok(F, z)) return smooth_alpha_df(F, z);
	return smooth_alpha(F, z);
}

/* f(z; phi) in double-float.  Inside the root box (leaf >= 0) the star terms
   are the leaf's near sums and local expansion; a point outside it (leaf < 0)
   takes the direct sums over every star from ext (the reference's direct sum
   there, include/tree_node.cuh:535-539), so both go through the same code. */
CCF_D double2 eval_f_df(const FieldView& F, int leaf, double2 z, double cphi, double sphi, const NearSums& ext)
{
	double2 s2 = ext.s2, dl = make_double2(0, 0);
	bool folded = false;
	if (leaf >= 0)
	{
		const SumsDF S = leaf_sums_df<false>(F, leaf, z);
		const int P = F.order;
		const dfc dz = leaf_dz_df(F, leaf, z);
		folded = F.leaf_fold != nullptr && F.leaf_fold[leaf];
		const float4* L = folded ? F.leaf_loc_df_fold : F.leaf_loc_df;
		dl = dfc_to(horner_df(L + ((size_t)leaf * 2 + 1) * (P + 1), P, 2, dz));
		s2 = dfc_to(S.s2);
	}
	/* a leaf with the smooth-mass series folded into its expansion keeps only
	   the constant of d alpha_s / d zbar */
	const double2 ds = folded ? make_double2(F.smooth_k1, 0) : smooth_dzbar_any(F, z);
	const double a = 1 - F.kappa_tot - smooth_dz(F, z);
	double2 f;
	f.x = F.shear + F.theta2 * s2.x - dl.x - ds.x - a * cphi;
	f.y = F.theta2 * s2.y - dl.y + ds.y + a * sphi;
	return f;
}

/* Double-float constants of a field for the continuation tracker: shear,
   theta^2, the constant 1 - kappa_tot - d alpha_smooth / dz of the
   approximate smooth-mass forms, the constant term of d alpha_smooth / d zbar
   of the rectangular Taylor form, kappa_star / pi, and FP32 copies of 1 / corner,
   1 / corner^2 and the squared radius inside which the Taylor form is
   evaluated in double-float. */
struct TrackConst
{
	dfl shear, theta2, a, k1, kpi;
	float2 ic, ic2;
	float r2;
	float aabs;            /* |a|, rounded up */
	double w1x, w1y, wc1;  /* the lens map's linear terms with the Taylor or folded smooth-mass
	                          forms: w = (w1x x + wc1, w1y y) + the star and series terms */
};

CCF_D TrackConst track_const(const FieldView& F)
{
	TrackConst k;
	k.shear = df_from_double(F.shear);
	k.theta2 = df_from_double(F.theta2);
	k.a = df_from_double(1 - F.kappa_tot - smooth_dz(F, make_double2(0, 0)));
	k.k1 = df_from_double(F.smooth_k1);
	k.kpi = df_from_double(F.kappa_star / PI);
	k.ic = make_float2((float)F.inv_corner.x, (float)F.inv_corner.y);
	k.ic2 = make_float2((float)F.inv_corner2.x, (float)F.inv_corner2.y);
	k.r2 = (float)(SMOOTH_DF_RANGE * F.corner_abs * F.corner_abs);
	k.aabs = __fadd_ru(fabsf(k.a.hi), fabsf(k.a.lo));
	k.w1x = 1 - F.kappa_tot + F.shear + 2 * F.kappa_star;
	k.w1y = 1 - F.kappa_tot - F.shear;
	k.wc1 = 2 * F.kappa_star * F.corner.x;
	return k;
}

/* Everything one corrector iteration of the continuation tracker needs at a
   root inside the root box, from one pass over the leaf's near stars and one
   pair of Horner passes over its local expansion:

     step   f / (f' + f pole) in FP32, with f assembled in double-float (as
            eval_f_df) and rounded, f' in FP32 (as eval_df32) and pole =
            2 sum_i 1/(z - z_i) over the near stars (+ 2/z for the exact
            disc), the part of the Aberth correction the tracker keeps;
     fz, fs f in FP64 and f' step, for the 1/mu bound at the stepped root;
     wpart  the star, local and smooth-Taylor part of the lens map w
            (as eval_point_df): w = ((1 - kappa + gamma) x, (1 - kappa - gamma) y)
            + wpart, plus 2 kappa_star (corner.x + x) when wmode is 1 (the
            Taylor form was evaluated here), minus smooth_alpha(z) when wmode
            is 0; when wmode is 2, wpart is the whole of w.

   The FP32 terms are the high words of the double-float 1/d and 1/d^2 the
   pass forms for f, so the FP64 pipe only splits the coordinates.  An
   iteration that converges writes its outputs from these values (the lens map
   and f are first-order corrected to the stepped root). rel = z - leaf
   centre in FP64; cph, sph = cos, sin phi. */
struct TrackEval
{
	float2 step;      /* f / (f' + f pole) */
	float as2;        /* |step|^2 */
	float2 fz;        /* f, rounded to FP32 (the first-order output correction) */
	float af;         /* bound on |f| at the stepped root z - step: |f - f' step|,
	                     the FP32 error of f' step, the double-float rounding of
	                     the terms of f and the FP64 spacing of the root times |f'| */
	dfc wpart;
	int wmode;
};

/* a / b in FP32 with b scaled to unit size first, so that |b|^2 neither
   overflows nor flushes to zero (a non-finite result marks a failed step) */
CCF_D float2 fdiv_scaled(float2 a, float2 b)
{
	const float m = fmaxf(fabsf(b.x), fabsf(b.y));
	const float im = 1.f / m;
	const float bx = b.x * im, by = b.y * im, ax = a.x * im, ay = a.y * im;
	const float r = 1.f / (bx * bx + by * by);
	return make_float2((ax * bx + ay * by) * r, (ay * bx - ax * by) * r);
}

CCF_D TrackEval eval_track_df(const FieldView& F, const TrackConst& K, int leaf, double2 z, double2 rel, dfl cph, dfl sph,
	bool disc_exact)
{
	const dfc zr = dfc_from(rel);
	dfacc s1r = {0.f, 0.f}, s1i = s1r, s2r = s1r, s2i = s1r;
	float2 s3 = make_float2(0.f, 0.f), pole = make_float2(0.f, 0.f);
	float tabs = 0.f;   /* sum of |m / d^2| */
	const int n = F.leaf_near_count[leaf];
	const float4* Pn = F.leaf_near_df + (size_t)leaf * MAX_NEAR;
	const float2* Mn = F.leaf_mass_df + (size_t)leaf * MAX_NEAR;
	/* the next star is loaded while this one's terms are formed */
	float4 pn = Pn[0];
	float2 mn = Mn[0];
	for (int i = 0; i < n; i++)
	{
		const dfc s = dfc_load(pn);
		const float2 mm = mn;
		pn = Pn[min(i + 1, MAX_NEAR - 1)];
		mn = Mn[min(i + 1, MAX_NEAR - 1)];
		const dfl m = {mm.x, mm.y};
		const dfl dx = df_sub(zr.re, s.re);
		const dfl dy = df_sub(zr.im, s.im);
		const dfl r = df_rcp(df_sumsq(dx, dy));
		const dfl ix = df_mul(dx, r);
		const dfl iy = df_neg(df_mul(dy, r));                     /* 1/d */
		/* ix^2 - iy^2 to 2^-47 of 1/|d|^2, the size of the term */
		const dfl i2x = df_dot2(ix, ix, df_neg(iy), iy);
		dfl i2y = df_mul(ix, iy);
		i2y = {2.f * i2y.hi, 2.f * i2y.lo};                        /* 1/d^2 */
		dfacc_fma(s2r, m, i2x);
		dfacc_fma(s2i, m, i2y);
		dfacc_fma(s1r, m, ix);
		dfacc_fma(s1i, m, iy);
		pole.x += ix.hi;
		pole.y += iy.hi;
		const float i3x = i2x.hi * ix.hi - i2y.hi * iy.hi;
		const float i3y = i2x.hi * iy.hi + i2y.hi * ix.hi;        /* 1/d^3 */
		s3.x = fmaf(m.hi, i3x, s3.x);
		s3.y = fmaf(m.hi, i3y, s3.y);
		tabs = fmaf(m.hi, fmaf(ix.hi, ix.hi, iy.hi * iy.hi), tabs);
	}
	const dfc s1 = {dfacc_get(s1r), dfacc_get(s1i)}, s2 = {dfacc_get(s2r), dfacc_get(s2i)};
	const int P = F.order;
	const float2 ihf = F.leaf_ih_df[leaf];
	const dfl ih = {ihf.x, ihf.y};
	const dfc dz = {df_mul(zr.re, ih), df_mul(zr.im, ih)};
	/* a leaf with the smooth-mass series folded into its expansion skips the series */
	const bool folded = F.leaf_fold != nullptr && F.leaf_fold[leaf];
	const float4* L = (folded ? F.leaf_loc_df_fold : F.leaf_loc_df) + (size_t)leaf * 2 * (P + 1);
	const dfc al = horner_df(L, P, 1, dz);
	const dfc dl = horner_df(L + (P + 1), P, 2, dz);
	const float2 dzf = make_float2(dz.re.hi, dz.im.hi);
	const float2* L3 = (folded ? F.leaf_loc3f_fold : F.leaf_loc3f) + (size_t)leaf * (P + 1);
	float2 d2l = L3[P], l3n = L3[P - 1];
	for (int i = P - 1; i >= 3; i--)
	{
		const float2 c = l3n;
		l3n = L3[i - 1];
		d2l = fadd(fmulc(d2l, dzf), c);
	}

	/* smooth mass: d alpha / d zbar (double-float), d2 alpha / d zbar2 (FP32)
	   and the Taylor part of alpha (double-float) */
	TrackEval e;
	dfc ds, sa = {{0.f, 0.f}, {0.f, 0.f}};
	float2 d2s;
	const float zx = (float)z.x, zy = (float)z.y;
	const bool taylor = F.rectangular && F.approx && F.smooth_m > 0 && zx * zx + zy * zy < K.r2;
	e.wmode = (taylor || folded) ? 1 : 0;
	if (folded)
	{
		/* the series are in the leaf's blocks: only d alpha_s / d zbar's constant */
		ds = {K.k1, {0.f, 0.f}};
		d2s = make_float2(0.f, 0.f);
	}
	else if (taylor)
	{
		const dfc zb = dfc_from(make_double2(z.x, -z.y));
		const dfc wc = dfc_mul(zb, dfc_load(F.inv_corner_df));   /* zbar / c */
		const dfc u = dfc_mul(wc, wc);
		dfc acc = dfc_load(F.smooth_d1_df[F.smooth_m - 1]);
		for (int m = F.smooth_m - 2; m >= 0; m--) acc = dfc_fma(acc, u, dfc_load(F.smooth_d1_df[m]));
		ds = dfc_mul(acc, u);
		ds.re = df_add(ds.re, K.k1);
		const int na = F.taylor_smooth + 1;
		dfc aa = dfc_load(F.smooth_a_df[na]);
		for (int i = na - 1; i >= 0; i--) aa = dfc_fma(aa, wc, dfc_load(F.smooth_a_df[i]));
		/* (0, -k / pi) A: re = (k / pi) A.im, im = -(k / pi) A.re */
		sa.re = df_mul(K.kpi, aa.im);
		sa.im = df_neg(df_mul(K.kpi, aa.re));
		const float2 zbf = make_float2(zx, -zy);
		const float2 r = fmulc(zbf, K.ic);
		const float2 uf = fmulc(r, r);
		float2 a2 = F.smooth_d2f[F.smooth_m - 1];
		for (int m = F.smooth_m - 2; m >= 0; m--) a2 = fadd(fmulc(a2, uf), F.smooth_d2f[m]);
		d2s = fmulc(a2, fmulc(zbf, K.ic2));
	}
	else
	{
		ds = dfc_from(smooth_dzbar(F, z));
		const double2 t = smooth_d2zbar(F, z);
		d2s = make_float2((float)t.x, (float)t.y);
	}
	const dfl a = F.approx ? K.a : df_from_double(1 - F.kappa_tot - smooth_dz(F, z));

	/* f = shear + theta^2 s2 - dl - conj(ds) - a e^{-i phi} (eval_f_df) */
	dfl fr = df_add(K.shear, df_mul(K.theta2, s2.re));
	fr = df_add(fr, df_neg(dl.re));
	fr = df_add(fr, df_neg(ds.re));
	fr = df_add(fr, df_neg(df_mul(a, cph)));
	dfl fi = df_mul(K.theta2, s2.im);
	fi = df_add(fi, df_neg(dl.im));
	fi = df_add(fi, ds.im);
	fi = df_add(fi, df_mul(a, sph));
	const float2 f32 = make_float2(fr.hi + fr.lo, fi.hi + fi.lo);
	e.fz = f32;
	const float t2 = K.theta2.hi;
	const float2 df = make_float2(-2 * t2 * s3.x - d2l.x - d2s.x, -2 * t2 * s3.y - d2l.y + d2s.y);
	pole = make_float2(2.f * pole.x, 2.f * pole.y);
	if (disc_exact)
	{
		const float2 iz = finv(make_float2(zx, zy));
		pole.x += 2.f * iz.x;
		pole.y += 2.f * iz.y;
	}
	/* the step: f / (f' + f pole), FP32 */
	const float2 st = fdiv_scaled(f32, fadd(df, fmulc(f32, pole)));
	e.step = st;
	e.as2 = st.x * st.x + st.y * st.y;
	/* |f| at z - st: f - f' st (f holomorphic), the FP32 error of f' st, the
	   double-float rounding of the terms of f (2^-47 of their sizes) and half
	   the FP64 spacing of the root times |f'|.  The difference is formed in
	   FP32 from f's double-float parts: (hi - f' st) + lo errs by 2^-23 of the
	   result plus 2^-48 |f| (the 3.6e-15 |f| term); the sum is rounded up by
	   2^-20 (its FP32 roundings are a few 2^-24): a bound, not an estimate */
	const float2 fsv = fmulc(df, st);
	const float terms = t2 * tabs + hypotf(dl.re.hi, dl.im.hi) + hypotf(ds.re.hi, ds.im.hi) + fabsf(a.hi) + fabsf(K.shear.hi);
	const float res = hypotf(__fadd_rn(__fsub_rn(fr.hi, fsv.x), fr.lo), __fadd_rn(__fsub_rn(fi.hi, fsv.y), fi.lo));
	e.af = (res + 1e-6f * hypotf(fsv.x, fsv.y) + 3.6e-15f * hypotf(f32.x, f32.y) + 7.2e-15f * terms +
		1.2e-16f * hypotf(zx, zy) * hypotf(df.x, df.y)) * (1.f + 0x1p-20f);
	/* w - the linear terms: (-theta^2 s1.x - al.x - sa.x, theta^2 s1.y + al.y - sa.y) (eval_point_df) */
	dfl wr = df_neg(df_mul(K.theta2, s1.re));
	wr = df_add(wr, df_neg(al.re));
	wr = df_add(wr, df_neg(sa.re));
	dfl wi = df_mul(K.theta2, s1.im);
	wi = df_add(wi, al.im);
	wi = df_add(wi, df_neg(sa.im));
	e.wpart = {wr, wi};
	return e;
}

/* 1/mu bound and caustic of a final point, double-float; star terms as in
   eval_f_df (leaf sums and local expansion, or ext off the root box) */
CCF_D PointResult eval_point_df(const FieldView& F, int leaf, double2 z, double cphi, double sphi, const NearSums& ext)
{
	double2 s1 = ext.s1, s2 = ext.s2, al = make_double2(0, 0), dl = make_double2(0, 0);
	if (leaf >= 0)
	{
		const SumsDF S = leaf_sums_df<true>(F, leaf, z);
		const int P = F.order;
		const dfc dz = leaf_dz_df(F, leaf, z);
		const float4* L = F.leaf_loc_df + (size_t)leaf * 2 * (P + 1);
		al = dfc_to(horner_df(L, P, 1, dz));
		dl = dfc_to(horner_df(L + (P + 1), P, 2, dz));
		s1 = dfc_to(S.s1);
		s2 = dfc_to(S.s2);
	}
	const double2 ds = smooth_dzbar_any(F, z);
	const double a = 1 - F.kappa_tot - smooth_dz(F, z);
	double2 f;
	f.x = F.shear + F.theta2 * s2.x - dl.x - ds.x - a * cphi;
	f.y = F.theta2 * s2.y - dl.y + ds.y + a * sphi;
	const double af = hypot(f.x, f.y);
	PointResult out;
	out.err = fmax(fabs(af * (af + 2 * a)), fabs(af * (af - 2 * a)));
	const double2 as = smooth_alpha_any(F, z);
	out.w.x = (1 - F.kappa_tot) * z.x + F.shear * z.x - F.theta2 * s1.x - al.x - as.x;
	out.w.y = (1 - F.kappa_tot) * z.y - F.shear * z.y + F.theta2 * s1.y + al.y - as.y;
	out.mu_length = 0;
	return out;
}

} /* namespace ccf */
