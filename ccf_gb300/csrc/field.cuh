/******************************************************************************
field.cuh -- device view of one star field and the evaluators of its
deflection field.

Deflection alpha = alpha_star (direct sum over the <= 32 stars of the leaf and
its neighbours) + alpha_local (local expansion of the far field at the leaf)
+ alpha_smooth (the compensating smooth-mass sheet).  The formulas are those
of the reference (include/alpha_star.cuh, alpha_local.cuh, alpha_smooth.cuh,
ccf_functions.cuh:33-121); the evaluation is reorganised for the GPU:

  * a leaf's local coefficients are stored pre-multiplied by the integer
    factors and powers of theta^2 / h that each derivative needs, so every
    Horner step is one complex multiply-add;
  * the rectangular Taylor form of alpha_smooth is held as polynomials whose
    coefficients are computed once on the host (the reference recomputes a
    complex exponential per term on every call, alpha_smooth.cuh:201-205);
  * one pass over the near stars produces 1/d, 1/d^2 and 1/d^3 from a single
    reciprocal.
******************************************************************************/
#pragma once

#include "common.cuh"

namespace ccf
{

/* one star in a leaf's near list (leaf + neighbours), 32 bytes */
struct NearStar
{
	double x, y, m, pad;
};

struct FieldView
{
	/* lens parameters */
	double kappa_tot;
	double shear;
	double kappa_star;
	double theta;
	double theta2;
	int rectangular;
	int approx;
	int taylor_smooth;
	int order;               /* FMM expansion order P */
	int num_roots;
	double2 corner;
	double corner_abs;

	/* smooth-mass polynomials (rectangular, approx = 1), see smooth.cpp */
	int smooth_m;            /* (taylor_smooth - 1) / 2 */
	double2 inv_corner;      /* 1 / corner */
	double2 inv_corner2;     /* 1 / corner^2 */
	double smooth_k1;        /* constant term of d alpha_smooth / d zbar */
	const double2* smooth_d1;    /* [smooth_m]   d alpha_s/dzbar  = sum D1[m-1] u^m + k1,  u = (zbar/c)^2 */
	const double2* smooth_d2;    /* [smooth_m]   d2 alpha_s/dzbar2 = zbar/c^2 sum D2[m-1] u^(m-1) */
	const double2* smooth_a;     /* [taylor_smooth + 2] alpha_s = (0,-k/pi) A(zbar) - 2k (c.re + z.re) */
	const float2* smooth_d2f;    /* FP32 copy of smooth_d2 */

	/* stars in tree order */
	int num_stars;
	const double2* star_pos;
	const double* star_mass;

	/* quadtree: node arrays (children of a node are contiguous, quadrant order) */
	int num_nodes;
	const double2* node_center;
	const double* node_half;
	const int* node_child;   /* index of child 0, or -1 for a leaf */
	const int* node_leaf;    /* leaf index of a leaf node */

	/* leaves */
	int num_leaves;
	const double2* leaf_center;
	const double* leaf_inv_half;
	const int* leaf_near_count;
	const NearStar* leaf_near;   /* [leaf * MAX_NEAR + i] */
	const double2* leaf_loc;     /* [(leaf * 3 + k) * (P + 1) + i], k = 0: alpha, 1: d/dzbar, 2: d2/dzbar2 */
	const float2* leaf_loc3f;    /* FP32 copy of the k = 2 block, [leaf * (P + 1) + i] */

	/* double-float copies for the mixed-precision evaluators (field_df.cuh) */
	const float4* leaf_near_df;  /* [leaf * MAX_NEAR + i] (z_i - leaf centre), complex double-float */
	const float2* leaf_mass_df;  /* [leaf * MAX_NEAR + i] */
	const float4* leaf_loc_df;   /* [(leaf * 2 + k) * (P + 1) + i], k = 0: alpha, 1: d/dzbar */
	const float2* leaf_ih_df;    /* [leaf] 1/h */
	const float4* smooth_d1_df;  /* [smooth_m] */
	const float4* smooth_a_df;   /* [taylor_smooth + 2] A_n c^n: the alpha polynomial in zbar / c */
	float4 inv_corner_df;
	const float4* star_df;       /* [num_stars] star positions, split (x_hi, y_hi, x_lo, y_lo) */
	const float2* star_mass_df;  /* [num_stars] */
	/* the tracker's leaf blocks with the smooth-mass series folded in
	   (fold_smooth_kernel); leaf_fold[leaf] = 1 where they hold */
	const unsigned char* leaf_fold;
	const float4* leaf_loc_df_fold;   /* like leaf_loc_df */
	const float2* leaf_loc3f_fold;    /* like leaf_loc3f */
	const double2* leaf_loc_fold64;   /* like leaf_loc, in FP64 (the FP64 polish) */
};

/* leaf containing z, or -1 when z lies outside the root box (the reference
   then returns the root and sums over all stars: include/tree_node.cuh:535-539,
   include/alpha_star.cuh:26-37).  Replicates the quadrant tests of
   include/tree_node.cuh:529-561. */
CCF_D int find_leaf(const FieldView& F, double2 z)
{
	int n = 0;
	for (int depth = 0; depth < 64; depth++)
	{
		double2 c = F.node_center[n];
		double h = F.node_half[n];
		int child = F.node_child[n];
		if (child < 0) return F.node_leaf[n];
		if (fabs(z.x - c.x) > h || fabs(z.y - c.y) > h) return -1;
		int q;
		if (z.y >= c.y) q = (z.x >= c.x) ? 0 : 1;
		else q = (z.x < c.x) ? 2 : 3;
		n = child + q;
	}
	return -1;
}

/* ---------------- smooth-mass terms (include/alpha_smooth.cuh) ---------------- */

CCF_D double heaviside(double x) { return x >= 0 ? 1.0 : 0.0; }
CCF_D double boxcar(double2 z, double2 c)
{
	return (-c.x <= z.x && z.x <= c.x && -c.y <= z.y && z.y <= c.y) ? 1.0 : 0.0;
}
CCF_D double2 clog64(double2 a) { return make_double2(log(hypot(a.x, a.y)), atan2(a.y, a.x)); }

/* d alpha_smooth / dz, a real number (alpha_smooth.cuh:142-170) */
CCF_D double smooth_dz(const FieldView& F, double2 z)
{
	if (F.approx) return -F.kappa_star;
	if (F.rectangular) return -F.kappa_star * boxcar(z, F.corner);
	return -F.kappa_star * heaviside(F.corner_abs - hypot(z.x, z.y));
}

/* d alpha_smooth / d zbar (alpha_smooth.cuh:186-236) */
CCF_D double2 smooth_dzbar(const FieldView& F, double2 z)
{
	const double k = F.kappa_star;
	const double2 zb = cconj(z);
	if (F.rectangular)
	{
		if (F.approx)
		{
			if (F.smooth_m <= 0) return make_double2(F.smooth_k1, 0);
			double2 r = cmul(zb, F.inv_corner);
			double2 u = cmul(r, r);
			double2 acc = F.smooth_d1[F.smooth_m - 1];
			for (int m = F.smooth_m - 2; m >= 0; m--) acc = cadd(cmul(acc, u), F.smooth_d1[m]);
			acc = cmul(acc, u);
			acc.x += F.smooth_k1;
			return acc;
		}
		double2 c = F.corner;
		double2 l1 = clog64(csub(cconj(c), zb));
		double2 l2 = clog64(csub(c, zb));
		double2 l3 = clog64(csub(make_double2(-c.x, -c.y), zb));
		double2 l4 = clog64(csub(make_double2(-c.x, c.y), zb));
		double2 s = cadd(csub(csub(l1, l2), l3), l4);
		double2 d = cmul(s, make_double2(0, -k / PI));
		d.x -= k * boxcar(z, c);
		return d;
	}
	if (F.approx) return make_double2(0, 0);
	/* the reference applies the exterior form everywhere for the exact disc */
	double2 z2 = cmul(zb, zb);
	return cscale(cinv(z2), k * F.corner_abs * F.corner_abs);
}

/* d2 alpha_smooth / d zbar2 (alpha_smooth.cuh:252-301), FP64 */
CCF_D double2 smooth_d2zbar(const FieldView& F, double2 z)
{
	const double k = F.kappa_star;
	const double2 zb = cconj(z);
	if (F.rectangular)
	{
		if (F.approx)
		{
			if (F.smooth_m <= 0) return make_double2(0, 0);
			double2 r = cmul(zb, F.inv_corner);
			double2 u = cmul(r, r);
			double2 acc = F.smooth_d2[F.smooth_m - 1];
			for (int m = F.smooth_m - 2; m >= 0; m--) acc = cadd(cmul(acc, u), F.smooth_d2[m]);
			return cmul(acc, cmul(zb, F.inv_corner2));
		}
		double2 c = F.corner;
		double2 i1 = cinv(csub(cconj(c), zb));
		double2 i2 = cinv(csub(c, zb));
		double2 i3 = cinv(csub(make_double2(-c.x, -c.y), zb));
		double2 i4 = cinv(csub(make_double2(-c.x, c.y), zb));
		double2 s = csub(cadd(cadd(make_double2(-i1.x, -i1.y), i2), i3), i4);
		return cmul(s, make_double2(0, -k / PI));
	}
	if (F.approx) return make_double2(0, 0);
	double2 z3 = cmul(cmul(zb, zb), zb);
	return cscale(cinv(z3), -2 * k * F.corner_abs * F.corner_abs);
}

/* alpha_smooth (alpha_smooth.cuh:63-127) */
CCF_D double2 smooth_alpha(const FieldView& F, double2 z)
{
	const double k = F.kappa_star;
	const double2 zb = cconj(z);
	if (F.rectangular)
	{
		if (F.approx)
		{
			int n = F.taylor_smooth + 1;
			double2 acc = F.smooth_a[n];
			for (int i = n - 1; i >= 0; i--) acc = cadd(cmul(acc, zb), F.smooth_a[i]);
			double2 a = cmul(acc, make_double2(0, -k / PI));
			a.x -= k * 2 * (F.corner.x + z.x);
			return a;
		}
		double2 c = F.corner;
		double2 c1 = csub(c, zb);
		double2 c2 = csub(cconj(c), zb);
		double2 c3 = csub(make_double2(-c.x, -c.y), zb);
		double2 c4 = csub(make_double2(-c.x, c.y), zb);
		double2 s = csub(cadd(csub(cmul(c1, clog64(c1)), cmul(c2, clog64(c2))), cmul(c3, clog64(c3))), cmul(c4, clog64(c4)));
		double2 a = cmul(s, make_double2(0, -k / PI));
		a.x -= k * 2 * (c.x + z.x) * boxcar(z, c);
		a.x -= k * 4 * c.x * heaviside(c.y + z.y) * heaviside(c.y - z.y) * heaviside(z.x - c.x);
		return a;
	}
	if (F.approx || hypot(z.x, z.y) <= F.corner_abs) return make_double2(-k * z.x, -k * z.y);
	return cscale(cinv(zb), -k * F.corner_abs * F.corner_abs);
}

/* ---------------- star + local terms ---------------- */

/* sums over stars of m / d^k, d = z - z_i: s1 (k = 1), s2 (k = 2), s3 (k = 3) */
struct NearSums
{
	double2 s1, s2, s3;
};

template <bool NEED1, bool NEED3>
CCF_D void star_term(NearSums& a, double2 z, double sx, double sy, double m)
{
	double dx = z.x - sx, dy = z.y - sy;
	double r = rcp64(dx * dx + dy * dy);
	double ix = dx * r, iy = -dy * r;                   /* 1/d */
	double i2x = ix * ix - iy * iy, i2y = 2 * ix * iy;  /* 1/d^2 */
	a.s2.x = fma(m, i2x, a.s2.x);
	a.s2.y = fma(m, i2y, a.s2.y);
	if (NEED1)
	{
		a.s1.x = fma(m, ix, a.s1.x);
		a.s1.y = fma(m, iy, a.s1.y);
	}
	if (NEED3)
	{
		double i3x = i2x * ix - i2y * iy, i3y = i2x * iy + i2y * ix;
		a.s3.x = fma(m, i3x, a.s3.x);
		a.s3.y = fma(m, i3y, a.s3.y);
	}
}

CCF_D NearSums zero_sums()
{
	NearSums a;
	a.s1 = make_double2(0, 0);
	a.s2 = make_double2(0, 0);
	a.s3 = make_double2(0, 0);
	return a;
}

/* direct sums over the <= 32 stars of a leaf and its neighbours
   (include/alpha_star.cuh:18-115) */
template <bool NEED1, bool NEED3>
CCF_D NearSums leaf_sums(const FieldView& F, int leaf, double2 z)
{
	NearSums a = zero_sums();
	int n = F.leaf_near_count[leaf];
	const NearStar* ns = F.leaf_near + (size_t)leaf * MAX_NEAR;
	for (int i = 0; i < n; i++)
	{
		NearStar s = ns[i];
		star_term<NEED1, NEED3>(a, z, s.x, s.y, s.m);
	}
	return a;
}

/* Off-field points (outside the root box) take the direct sum over every
   star, as the reference does when the root is the nearest node
   (include/tree_node.cuh:535-539).  The warp computes those sums together:
   every lane takes every 32nd star for one off-field point at a time, so one
   such point costs the warp N/32 terms instead of N.  Must be called by all
   32 lanes; lanes with need set receive their sums in out. */
template <bool NEED1, bool NEED3>
CCF_D void offfield_sums_warp(const FieldView& F, bool need, double2 z, NearSums& out)
{
	const unsigned full = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	unsigned m = __ballot_sync(full, need);
	while (m)
	{
		int src = __ffs(m) - 1;
		m &= m - 1;
		double2 zz = make_double2(__shfl_sync(full, z.x, src), __shfl_sync(full, z.y, src));
		NearSums a = zero_sums();
		for (int i = lane; i < F.num_stars; i += 32)
		{
			double2 p = F.star_pos[i];
			star_term<NEED1, NEED3>(a, zz, p.x, p.y, F.star_mass[i]);
		}
		double v[6] = {a.s1.x, a.s1.y, a.s2.x, a.s2.y, a.s3.x, a.s3.y};
#pragma unroll
		for (int k = 0; k < 6; k++)
		{
			for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(full, v[k], o);
		}
		if (lane == src)
		{
			out.s1 = make_double2(v[0], v[1]);
			out.s2 = make_double2(v[2], v[3]);
			out.s3 = make_double2(v[4], v[5]);
		}
	}
}

/* near sums for one point per lane: its leaf's direct sum, or (off-field)
   the warp-cooperative sum over all stars.  All lanes must call it; lanes
   with active false contribute nothing and get zeros. */
template <bool NEED1, bool NEED3>
CCF_D NearSums point_sums_warp(const FieldView& F, bool active, int leaf, double2 z)
{
	NearSums a = zero_sums();
	if (active && leaf >= 0) a = leaf_sums<NEED1, NEED3>(F, leaf, z);
	offfield_sums_warp<NEED1, NEED3>(F, active && leaf < 0, z, a);
	return a;
}

/* Horner of the pre-scaled local coefficients: sum_{i >= first} L[i] dz^(i - first) */
CCF_D double2 local_horner(const double2* L, int P, int first, double2 dz)
{
	double2 acc = L[P];
	for (int i = P - 1; i >= first; i--) acc = cadd(cmul(acc, dz), L[i]);
	return acc;
}

CCF_D double2 leaf_dz(const FieldView& F, int leaf, double2 z)
{
	double2 c = F.leaf_center[leaf];
	double ih = F.leaf_inv_half[leaf];
	return make_double2((z.x - c.x) * ih, (z.y - c.y) * ih);
}

/* parametric critical-curve function f(z; phi) (ccf_functions.cuh:69-86):
   f = gamma - conj(dalpha_star/dzbar) - conj(dalpha_local/dzbar)
       - conj(dalpha_smooth/dzbar) - (1 - kappa - dalpha_smooth/dz) e^{-i phi}
   from the star sums S, and, when DF is true, its z derivative
   (ccf_functions.cuh:108-121). */
template <bool DF>
CCF_D void eval_f64(const FieldView& F, int leaf, double2 z, double cphi, double sphi, const NearSums& S, double2& f, double2& df)
{
	/* -conj(d alpha_star / d zbar) = theta^2 sum m / d^2 */
	f = make_double2(F.shear + F.theta2 * S.s2.x, F.theta2 * S.s2.y);
	double2 dl = make_double2(0, 0), d2l = make_double2(0, 0);
	if (leaf >= 0)
	{
		const int P = F.order;
		double2 dz = leaf_dz(F, leaf, z);
		const double2* L = F.leaf_loc + (size_t)leaf * 3 * (P + 1);
		dl = local_horner(L + (P + 1), P, 2, dz);
		if (DF) d2l = local_horner(L + 2 * (P + 1), P, 3, dz);
	}
	double2 ds = smooth_dzbar(F, z);
	double sz = smooth_dz(F, z);
	double a = 1 - F.kappa_tot - sz;
	f.x -= dl.x + ds.x + a * cphi;
	f.y -= dl.y - ds.y - a * sphi;
	if (DF)
	{
		double2 d2s = smooth_d2zbar(F, z);
		/* f' = -conj(d2 alpha_star) - conj(d2 alpha_local) - conj(d2 alpha_smooth)
		      = -2 theta^2 sum m / d^3 - H3 - conj(d2s) */
		df.x = -2 * F.theta2 * S.s3.x - d2l.x - d2s.x;
		df.y = -2 * F.theta2 * S.s3.y - d2l.y + d2s.y;
	}
}

/* The reduced-precision smooth-mass polynomials (the FP32 f' below, the
   double-float ones of field_df.cuh) are used only inside the circle through
   the field's corners, |z / c|^2 < SMOOTH_DF_RANGE.  There the Taylor series
   converges and its terms are below ~1, so double-float rounding is ~1e-15.
   Outside, the terms grow like |z / c|^(2m) and cancel; the FP64 forms keep
   that cancellation at the reference's own FP64 rounding, and no FP32 part
   can overflow. */
constexpr double SMOOTH_DF_RANGE = 1.0;
CCF_D bool smooth_df_ok(const FieldView& F, double2 z)
{
	return z.x * z.x + z.y * z.y < SMOOTH_DF_RANGE * F.corner_abs * F.corner_abs;
}

/* d2 alpha_smooth / d zbar2 in FP32 (the FP32 Taylor polynomial within the
   corner circle, FP64 outside) */
CCF_D float2 smooth_d2zbar_f32(const FieldView& F, double2 z)
{
	if (F.rectangular && F.approx && F.smooth_m > 0 && smooth_df_ok(F, z))
	{
		double2 zb = cconj(z);
		double2 rd = cmul(zb, F.inv_corner);
		float2 r = make_float2((float)rd.x, (float)rd.y);
		float2 u = fmulc(r, r);
		float2 acc = F.smooth_d2f[F.smooth_m - 1];
		for (int m = F.smooth_m - 2; m >= 0; m--) acc = fadd(fmulc(acc, u), F.smooth_d2f[m]);
		double2 pre = cmul(zb, F.inv_corner2);
		return fmulc(acc, make_float2((float)pre.x, (float)pre.y));
	}
	double2 t = smooth_d2zbar(F, z);
	return make_float2((float)t.x, (float)t.y);
}

/* f'(z) in FP32 for the mixed-precision solver: only the step size depends
   on it, never the converged root.  Off-field points take s3_off, the direct
   sum over every star. */
CCF_D float2 eval_df32(const FieldView& F, int leaf, double2 z, double2 s3_off)
{
	float2 s3 = make_float2(0, 0);
	float2 d2l = make_float2(0, 0);
	bool folded = false;
	if (leaf >= 0)
	{
		folded = F.leaf_fold != nullptr && F.leaf_fold[leaf];
		int n = F.leaf_near_count[leaf];
		const NearStar* ns = F.leaf_near + (size_t)leaf * MAX_NEAR;
		for (int i = 0; i < n; i++)
		{
			NearStar s = ns[i];
			float dx = (float)(z.x - s.x), dy = (float)(z.y - s.y), m = (float)s.m;
			float r = rcp32(dx * dx + dy * dy);
			float ix = dx * r, iy = -dy * r;
			float i2x = ix * ix - iy * iy, i2y = 2 * ix * iy;
			float i3x = i2x * ix - i2y * iy, i3y = i2x * iy + i2y * ix;
			s3.x = fmaf(m, i3x, s3.x);
			s3.y = fmaf(m, i3y, s3.y);
		}
		const int P = F.order;
		double2 dzd = leaf_dz(F, leaf, z);
		float2 dz = make_float2((float)dzd.x, (float)dzd.y);
		const float2* L = (folded ? F.leaf_loc3f_fold : F.leaf_loc3f) + (size_t)leaf * (P + 1);
		float2 acc = L[P];
		for (int i = P - 1; i >= 3; i--) acc = fadd(fmulc(acc, dz), L[i]);
		d2l = acc;
	}
	else
	{
		s3 = make_float2((float)s3_off.x, (float)s3_off.y);
	}
	/* a folded leaf's block holds the smooth-mass term of f' */
	const float2 d2s = folded ? make_float2(0.f, 0.f) : smooth_d2zbar_f32(F, z);
	const float t2 = (float)F.theta2;
	return make_float2(-2 * t2 * s3.x - d2l.x - d2s.x, -2 * t2 * s3.y - d2l.y + d2s.y);
}

/* f'(z) for the mixed-precision solver: the FP32 evaluation, or FP64 where
   that is not finite (far outside the field the smooth-mass Taylor terms
   leave the FP32 range, and an infinite f' would make a zero step).
   Off-field points take s3_off, the direct sum over every star. */
CCF_D double2 eval_df_mixed(const FieldView& F, int leaf, double2 z, double2 s3_off)
{
	const float2 d = eval_df32(F, leaf, z, s3_off);
	if (isfinite(d.x) && isfinite(d.y)) return make_double2(d.x, d.y);
	double2 s3 = s3_off, d2l = make_double2(0, 0);
	if (leaf >= 0)
	{
		s3 = leaf_sums<false, true>(F, leaf, z).s3;
		const int P = F.order;
		d2l = local_horner(F.leaf_loc + (size_t)leaf * 3 * (P + 1) + 2 * (P + 1), P, 3, leaf_dz(F, leaf, z));
	}
	const double2 d2s = smooth_d2zbar(F, z);
	return make_double2(-2 * F.theta2 * s3.x - d2l.x - d2s.x, -2 * F.theta2 * s3.y - d2l.y + d2s.y);
}

/* everything the epilogue needs at a final root: the 1/mu error bound
   (ccf_functions.cuh:419-467), the caustic w = (1 - kappa) z + gamma zbar
   - alpha (ccf_functions.cuh:33-45) and the magnification length scale
   (ccf_functions.cuh:144-166), from the star sums S of the point. */
struct PointResult
{
	double err;
	double2 w;
	double mu_length;
};

template <bool WANT_W, bool WANT_MU>
CCF_D PointResult eval_point(const FieldView& F, int leaf, double2 z, double cphi, double sphi, const NearSums& S)
{
	const int P = F.order;
	double2 al = make_double2(0, 0), dl = make_double2(0, 0), d2l = make_double2(0, 0);
	if (leaf >= 0)
	{
		double2 dz = leaf_dz(F, leaf, z);
		const double2* L = F.leaf_loc + (size_t)leaf * 3 * (P + 1);
		if (WANT_W) al = local_horner(L, P, 1, dz);
		dl = local_horner(L + (P + 1), P, 2, dz);
		if (WANT_MU) d2l = local_horner(L + 2 * (P + 1), P, 3, dz);
	}
	double2 ds = smooth_dzbar(F, z);
	double sz = smooth_dz(F, z);
	double a = 1 - F.kappa_tot - sz;
	/* f0 and the 1/mu bound */
	double2 f;
	f.x = F.shear + F.theta2 * S.s2.x - dl.x - ds.x - a * cphi;
	f.y = F.theta2 * S.s2.y - dl.y + ds.y + a * sphi;
	double af = hypot(f.x, f.y);
	PointResult out;
	double e1 = fabs(af * (af + 2 * a));
	double e2 = fabs(af * (af - 2 * a));
	out.err = fmax(e1, e2);
	if (WANT_W)
	{
		/* alpha_star = theta^2 conj(s1), alpha_local = conj(H1) */
		double2 as = smooth_alpha(F, z);
		out.w.x = (1 - F.kappa_tot) * z.x + F.shear * z.x - F.theta2 * S.s1.x - al.x - as.x;
		out.w.y = (1 - F.kappa_tot) * z.y - F.shear * z.y + F.theta2 * S.s1.y + al.y - as.y;
	}
	else
	{
		out.w = make_double2(0, 0);
	}
	if (WANT_MU)
	{
		/* dw/dzbar = gamma - dalpha_star/dzbar - dalpha_local/dzbar - dalpha_smooth/dzbar */
		double2 dwdzb;
		dwdzb.x = F.shear + F.theta2 * S.s2.x - dl.x - ds.x;
		dwdzb.y = -F.theta2 * S.s2.y + dl.y - ds.y;
		double2 d2s = smooth_d2zbar(F, z);
		/* d2w/dzbar2 = -(d2 alpha_star) - (d2 alpha_local) - (d2 alpha_smooth);
		   d2 alpha_star = 2 theta^2 conj(s3), d2 alpha_local = conj(H3) */
		double2 d2w;
		d2w.x = -2 * F.theta2 * S.s3.x - d2l.x - d2s.x;
		d2w.y = 2 * F.theta2 * S.s3.y + d2l.y - d2s.y;
		double2 cct = cmul(cmul(make_double2(0, -2), cconj(dwdzb)), d2w);
		double2 ct = cadd(cscale(cct, a), cmul(dwdzb, cconj(cct)));
		out.mu_length = 1 / (2 * hypot(ct.x, ct.y));
	}
	else
	{
		out.mu_length = 0;
	}
	return out;
}

} /* namespace ccf */
