/******************************************************************************
polish.cu -- FP64 polish of the output points whose 1/mu error is above the
reference's target, or whose solver left them unconverged.

The mixed-precision solvers converge every root in FP32 / double-float
arithmetic and report a rigorous upper bound on 1/mu at the reported root.
Where that bound exceeds 1e-9 (stiff roots next to a star, where |f'| times
the rounding of the root dominates), or a solver stopped at its iteration cap
(the full-sum solver's sweep cap, the tracker's stall next to a pair of close
zeros), the point takes FP64 Newton steps with the Aberth correction of the
near poles,

    z <- z - f / (f' + f 2 sum_near 1 / (z - z_i))   [+ 2 / z, exact disc],

the reference's step (include/ccf_functions.cuh:193-243) with the near stars
of the point's leaf in place of all stars and without the other roots' terms
(the other roots sit far away at this accuracy).  It stops at the reference's
rules: 1/mu below 1e-9 (the early return, ccf_functions.cuh:207-211) or a step
below 1e-9 theta_star (ccf_functions.cuh:385).  The FP64 point with the
smallest 1/mu error is kept when it beats the stored one; its 1/mu error (the
reference's formula, ccf_functions.cuh:457-463), caustic and length scale are
then written in FP64.  A flagged point may move at most POLISH_MOVE theta_star
(an unconverged one POLISH_MOVE_LISTED, the tracker's stall radius), so a
polish never carries a root to a neighbouring zero.

The solvers mark an unconverged point by storing -1 - err in its 1/mu slot;
the polish always runs after them on the same stream and replaces every mark
by a non-negative error, so no caller ever sees one.

Two launches.  polish_scan_kernel reads the 1/mu array once (8 bytes per
point), forms the largest error of the points that need nothing, and lists
the flagged ones (warp-aggregated appends); flagged points are consecutive
phi steps of the same stiff roots, so polishing them where they are found
would serialise them in a few warps.  polish_list_kernel then gives every
listed point a lane of its own with its leaf's near sums (the FP64 pipe does
32 points' work per warp instruction); a point off the root box, whose sums
run over every star, is taken by the whole warp, the lanes splitting the
stars.  A point beyond the list's capacity is polished by the scan itself,
one warp per point.
******************************************************************************/
#include "kernels.h"

namespace ccf
{

namespace
{

constexpr int POLISH_ITERS = 8;
constexpr double POLISH_FLOOR = 4;     /* |f| within this many times |f'| half-spacings of the zero: the FP64 floor
                                          (Newton's last step in FP64 may land one spacing off the nearest point) */
constexpr double POLISH_STALL = 0.5;   /* a step that does not shrink below this share of the last ends the polish:
                                          the point sits at the FP64 rounding floor of f */

struct PolishOutcome
{
	double err;    /* the 1/mu error now stored */
	bool conv;     /* a converged zero by the reference's rules */
	bool floor;    /* |f| at the kept point is within twice what the FP64 grid
	                  leaves next to the zero (|f'| times half the spacing) */
};

/* FP64 star sums at z (every lane passes the same z; every lane returns the
   totals): the leaf's near stars, or every star off the root box.  pole is
   sum 1 / (z - z_i) over the same stars. */
__device__ void warp_point_sums(const FieldView& F, int leaf, double2 z, NearSums& S, double2& pole)
{
	const unsigned full = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	NearSums a = zero_sums();
	double px = 0, py = 0;
	if (leaf >= 0)
	{
		const int n = F.leaf_near_count[leaf];
		const NearStar* ns = F.leaf_near + (size_t)leaf * MAX_NEAR;
		for (int i = lane; i < n; i += 32)
		{
			const NearStar s = ns[i];
			star_term<true, true>(a, z, s.x, s.y, s.m);
			const double2 id = cinv(make_double2(z.x - s.x, z.y - s.y));
			px += id.x;
			py += id.y;
		}
	}
	else
	{
		for (int i = lane; i < F.num_stars; i += 32)
		{
			const double2 p = F.star_pos[i];
			star_term<true, true>(a, z, p.x, p.y, F.star_mass[i]);
			const double2 id = cinv(make_double2(z.x - p.x, z.y - p.y));
			px += id.x;
			py += id.y;
		}
	}
	double v[8] = {a.s1.x, a.s1.y, a.s2.x, a.s2.y, a.s3.x, a.s3.y, px, py};
#pragma unroll
	for (int k = 0; k < 8; k++)
	{
		for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(full, v[k], o);
		/* lane 0's bits for everyone: the polish's branches must stay warp-uniform */
		v[k] = __shfl_sync(full, v[k], 0);
	}
	S.s1 = make_double2(v[0], v[1]);
	S.s2 = make_double2(v[2], v[3]);
	S.s3 = make_double2(v[4], v[5]);
	pole = make_double2(v[6], v[7]);
}

/* the same sums for one lane's own point over its leaf's near stars */
__device__ void lane_point_sums(const FieldView& F, int leaf, double2 z, NearSums& S, double2& pole)
{
	S = zero_sums();
	double px = 0, py = 0;
	const int n = F.leaf_near_count[leaf];
	const NearStar* ns = F.leaf_near + (size_t)leaf * MAX_NEAR;
	for (int i = 0; i < n; i++)
	{
		const NearStar st = ns[i];
		star_term<true, true>(S, z, st.x, st.y, st.m);
		const double2 id = cinv(make_double2(z.x - st.x, z.y - st.y));
		px += id.x;
		py += id.y;
	}
	pole = make_double2(px, py);
}

/* phase of output column k of branch b: phi0 + sgn 2 pi j / nphi with
   phi0 = pi / nb + 2 pi b / nb, as the reference forms it
   (include/ccf_functions.cuh:338, :344) */
__device__ double column_phase(const FieldOut& O, int b, int k)
{
	const double phi0 = PI / O.nb + b * 2 * PI / O.nb;
	const int j = k < O.half ? O.half - k : k - O.half;
	const double dphi = 2 * PI / O.nphi * j;
	return k < O.half ? phi0 - dphi : phi0 + dphi;
}

/* f, f' and a = 1 - kappa - d alpha_s / dz in FP64 (the quantities of
   eval_f64), with the leaf's FP64 blocks that carry the smooth-mass series
   where the fold holds (then the series themselves are skipped) */
struct PolishEval
{
	double2 f, df;
	double a;
};

__device__ PolishEval polish_eval(const FieldView& F, int leaf, double2 z, double cphi, double sphi, const NearSums& S)
{
	const bool folded = leaf >= 0 && F.leaf_loc_fold64 != nullptr && F.leaf_fold[leaf];
	PolishEval e;
	if (!folded)
	{
		eval_f64<true>(F, leaf, z, cphi, sphi, S, e.f, e.df);
		e.a = 1 - F.kappa_tot - smooth_dz(F, z);
		return e;
	}
	const int P = F.order;
	const double2 dz = leaf_dz(F, leaf, z);
	const double2* L = F.leaf_loc_fold64 + (size_t)leaf * 3 * (P + 1);
	const double2 dl = local_horner(L + (P + 1), P, 2, dz);
	const double2 d2l = local_horner(L + 2 * (P + 1), P, 3, dz);
	/* the folded blocks hold the series; d alpha_s / d zbar keeps its constant */
	e.a = 1 - F.kappa_tot - smooth_dz(F, z);
	e.f.x = F.shear + F.theta2 * S.s2.x - dl.x - F.smooth_k1 - e.a * cphi;
	e.f.y = F.theta2 * S.s2.y - dl.y + e.a * sphi;
	e.df.x = -2 * F.theta2 * S.s3.x - d2l.x;
	e.df.y = -2 * F.theta2 * S.s3.y - d2l.y;
	return e;
}

/* |f| that the FP64 grid itself leaves next to a zero: the nearest
   representable point lies within half a spacing of z in each coordinate */
__device__ double fp64_floor(double2 z, double2 df)
{
	const double ux = ldexp(1.0, ilogb(fmax(fabs(z.x), 1e-300)) - 52);
	const double uy = ldexp(1.0, ilogb(fmax(fabs(z.y), 1e-300)) - 52);
	return 0.5 * hypot(ux, uy) * hypot(df.x, df.y);
}

/* Polish the point in output slot idx.  e0: its stored 1/mu error
   (unmarked); listed: the solver left it unconverged.  WARP: the whole warp
   works on one point (every lane passes the same arguments; the lanes split
   the star sums, which off the root box run over every star).  Otherwise each
   lane polishes a point of its own with its leaf's near sums, 32 points per
   warp instruction on the FP64 pipe; a lane whose point is (or gets) off the
   root box sets *off and writes nothing, for the warp to take it. */
template <bool WARP>
__device__ __noinline__ PolishOutcome polish_point(const FieldView& F, const FieldOut& O, size_t idx, double e0,
	bool listed, bool* off)
{
	const int lane = threadIdx.x & 31;
	const bool writer = WARP ? lane == 0 : true;
	/* branch and column of the window slot idx */
	const size_t row = idx / (size_t)O.w_cols;
	const int k = O.w_k0 + (int)(idx - row * (size_t)O.w_cols);
	const int b = (O.w_b0 + (int)(row % (size_t)O.w_nb)) % O.nb;
	double sp, cp;
	sincos(column_phase(O, b, k), &sp, &cp);
	const double2 z0 = O.ccs[idx];
	const double tol = POLISH_STEP_TOL * F.theta;
	const double move = (listed ? POLISH_MOVE_LISTED : POLISH_MOVE) * F.theta;
	const bool disc_exact = !F.rectangular && !F.approx;

	double2 z = z0, zb = z0;
	double eb = __longlong_as_double(0x7ff0000000000000LL);   /* +inf */
	double last = eb;
	NearSums Sb = zero_sums();
	int lb = -1;
	bool conv = false, have = false;
	for (int it = 0; it < POLISH_ITERS && isfinite(z.x) && isfinite(z.y); it++)
	{
		const int leaf = find_leaf(F, z);
		NearSums S;
		double2 pole;
		if constexpr (WARP) warp_point_sums(F, leaf, z, S, pole);
		else
		{
			if (leaf < 0)
			{
				*off = true;
				PolishOutcome none;
				none.err = e0;
				none.conv = false;
				none.floor = false;
				return none;
			}
			lane_point_sums(F, leaf, z, S, pole);
		}
		const PolishEval v = polish_eval(F, leaf, z, cp, sp, S);
		const double af = hypot(v.f.x, v.f.y);
		const double err = fmax(fabs(af * (af + 2 * v.a)), fabs(af * (af - 2 * v.a)));
		const bool at_floor = af <= POLISH_FLOOR * fp64_floor(z, v.df);
		if (err < eb)
		{
			eb = err;
			zb = z;
			Sb = S;
			lb = leaf;
			have = true;
		}
		if (err < POLISH_ERR) conv = true;
		if (conv) break;
		double2 Sg = make_double2(2 * pole.x, 2 * pole.y);
		if (disc_exact)
		{
			const double2 iz = cinv(z);
			Sg.x += 2 * iz.x;
			Sg.y += 2 * iz.y;
		}
		const double2 step = cdiv(v.f, cadd(v.df, cmul(v.f, Sg)));
		if (!isfinite(step.x) || !isfinite(step.y)) break;
		const double2 zn = csub(z, step);
		if (hypot(zn.x - z0.x, zn.y - z0.y) > move) break;
		const double as = hypot(step.x, step.y);
		if (as < tol)
		{
			/* a converged zero by the step test; at the FP64 floor the stepped
			   point is no better, elsewhere it is evaluated once more */
			conv = true;
			if (at_floor) break;
		}
		else if (it > 0 && as > POLISH_STALL * last) break;
		last = as;
		z = zn;
	}
	PolishOutcome out;
	out.floor = false;
	if (!have)
	{
		if (writer && listed) O.errs[idx] = e0;   /* a listed point gets its mark removed */
		out.err = e0;
		out.conv = false;
		return out;
	}
	/* The verdict on the kept point uses the reference's FP64 formulas
	   unfolded (the iterations may use the folded blocks): its 1/mu error
	   (include/ccf_functions.cuh:457-463) and whether |f| sits at the FP64
	   floor. */
	double2 fb, dfb;
	eval_f64<true>(F, lb, zb, cp, sp, Sb, fb, dfb);
	const double ab = 1 - F.kappa_tot - smooth_dz(F, zb);
	const double afb = hypot(fb.x, fb.y);
	const double erb = fmax(fabs(afb * (afb + 2 * ab)), fabs(afb * (afb - 2 * ab)));
	const bool improve = isfinite(erb) && (!(e0 <= erb) || !isfinite(e0));
	if (improve && zb.x == z0.x && zb.y == z0.y)
	{
		/* the root stays: its FP64 1/mu error replaces the bound (the caustic
		   and length scale of the solver stand) */
		if (writer) O.errs[idx] = erb;
		out.err = erb;
	}
	else if (improve)
	{
		/* the root moved: every output at the kept point in FP64 */
		PointResult pr;
		if (O.caustics && O.mu) pr = eval_point<true, true>(F, lb, zb, cp, sp, Sb);
		else if (O.caustics) pr = eval_point<true, false>(F, lb, zb, cp, sp, Sb);
		else if (O.mu) pr = eval_point<false, true>(F, lb, zb, cp, sp, Sb);
		else pr = eval_point<false, false>(F, lb, zb, cp, sp, Sb);
		if (writer)
		{
			O.ccs[idx] = zb;
			O.errs[idx] = pr.err;
			if (O.caustics) O.caustics[idx] = pr.w;
			if (O.mu) O.mu[idx] = pr.mu_length;
		}
		out.err = pr.err;
	}
	else
	{
		/* keep the stored point; a listed point gets its mark removed */
		if (writer && listed) O.errs[idx] = e0;
		out.err = e0;
	}
	out.floor = afb <= POLISH_FLOOR * fp64_floor(zb, dfb);
	out.conv = conv || out.err < POLISH_ERR;
	return out;
}

/* per-warp sums of the polish statistics into the field's words */
__device__ void polish_stats(unsigned long long* st, double maxe, bool nan, unsigned long long polished,
	unsigned long long unconv, unsigned long long above, unsigned long long at_floor)
{
	const unsigned full = 0xffffffffu;
	for (int o = 16; o > 0; o >>= 1)
	{
		maxe = fmax(maxe, __shfl_xor_sync(full, maxe, o));
		polished += __shfl_xor_sync(full, polished, o);
		unconv += __shfl_xor_sync(full, unconv, o);
		above += __shfl_xor_sync(full, above, o);
		at_floor += __shfl_xor_sync(full, at_floor, o);
	}
	nan = __any_sync(full, nan);
	if ((threadIdx.x & 31) == 0)
	{
		atomicMax(&st[STAT_POLISHED_MAX_ERR], (unsigned long long)__double_as_longlong(maxe));
		if (nan) atomicOr(&st[STAT_POLISHED_NAN], 1ull);
		if (polished) atomicAdd(&st[STAT_POLISHED], polished);
		if (unconv) atomicAdd(&st[STAT_POLISHED_UNCONV], unconv);
		if (above) atomicAdd(&st[STAT_POLISHED_ABOVE], above);
		if (at_floor) atomicAdd(&st[STAT_POLISHED_FLOOR], at_floor);
	}
}

/* list entry: field index above bit 48, output slot below */
constexpr int LIST_FIELD_SHIFT = 48;

__global__ void __launch_bounds__(256) polish_scan_kernel(const PolishArgs A)
{
	__shared__ FieldView sF;
	__shared__ FieldOut sO;
	const unsigned full = 0xffffffffu;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	if (threadIdx.x == 0)
	{
		sF = A.fields[blockIdx.y];
		sO = A.outs[blockIdx.y];
	}
	__syncthreads();
	const FieldView& F = sF;
	const FieldOut& O = sO;
	const bool box = A.nbs > 0;
	const int b0 = box ? A.b0 : O.w_b0, nbs = box ? A.nbs : O.w_nb;
	const int k0 = box ? A.k0 : O.w_k0, nks = box ? A.nks : O.w_cols;
	const size_t per_root = (size_t)nbs * nks;
	const size_t npts = (size_t)F.num_roots * per_root;
	const size_t stride = (size_t)gridDim.x * blockDim.x;

	double maxe = 0;
	bool nan = false;
	unsigned long long polished = 0, unconv = 0, above = 0, at_floor = 0;
	for (size_t base = ((size_t)blockIdx.x * (blockDim.x >> 5) + warp) * 32; base < npts; base += stride)
	{
		const size_t i = base + lane;
		bool v = i < npts;
		size_t idx = 0;
		if (v)
		{
			const size_t a = i / per_root, r = i - a * per_root;
			const int bb = (int)((b0 + r / nks) % (size_t)O.nb), kk = (int)(k0 + r % nks);
			idx = out_slot(O, (int)a, bb, kk);
			v = idx != NO_OUT;
		}
		double e = v ? O.errs[idx] : 0;
		const bool flag = v && !(e >= 0 && e <= POLISH_ERR);
		const unsigned m = __ballot_sync(full, flag);
		if (!m)
		{
			if (v) maxe = fmax(maxe, e);
			continue;
		}
		/* append the flagged points to the list, one atomic per warp */
		unsigned long long pos = 0;
		if (lane == __ffs(m) - 1) pos = atomicAdd(A.list_count, (unsigned long long)__popc(m));
		pos = __shfl_sync(full, pos, __ffs(m) - 1) + __popc(m & ((1u << lane) - 1));
		const bool listed_ok = flag && pos < (unsigned long long)A.list_cap;
		if (listed_ok) A.list[pos] = ((unsigned long long)blockIdx.y << LIST_FIELD_SHIFT) | (unsigned long long)idx;
		if (v && !flag) maxe = fmax(maxe, e);
		/* beyond the list's capacity: polished here */
		unsigned rest = __ballot_sync(full, flag && !listed_ok);
		while (rest)
		{
			const int src = __ffs(rest) - 1;
			rest &= rest - 1;
			const size_t pidx = (size_t)__shfl_sync(full, (unsigned long long)idx, src);
			const double pe = __shfl_sync(full, e, src);
			const bool listed = pe < 0;
			const PolishOutcome o = polish_point<true>(F, O, pidx, listed ? -1 - pe : pe, listed, nullptr);
			if (lane == src)
			{
				polished++;
				if (listed && !o.conv) unconv++;
				if (!(o.err <= POLISH_ERR))
				{
					if (o.floor) at_floor++;
					else above++;
				}
				if (isfinite(o.err)) maxe = fmax(maxe, o.err);
				else nan = true;
			}
		}
	}
	polish_stats(O.stats, maxe, nan, polished, unconv, above, at_floor);
}

/* one lane per listed point (lanes on points off the root box hand them to
   the whole warp) */
__global__ void __launch_bounds__(256) polish_list_kernel(const PolishArgs A)
{
	const unsigned full = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	const unsigned long long n = min(*A.list_count, (unsigned long long)A.list_cap);
	const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
	/* warp-uniform trip count: the off-field points are warp-wide calls */
	for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n;
		base += stride)
	{
		const unsigned long long q = base + lane;
		const bool v = q < n;
		int fi = 0;
		size_t idx = 0;
		double e0 = 0;
		bool listed = false, off = false;
		PolishOutcome o;
		o.err = 0;
		o.conv = true;
		o.floor = false;
		if (v)
		{
			const unsigned long long ent = A.list[q];
			fi = (int)(ent >> LIST_FIELD_SHIFT);
			idx = (size_t)(ent & ((1ull << LIST_FIELD_SHIFT) - 1));
			const double pe = A.outs[fi].errs[idx];
			listed = pe < 0;
			e0 = listed ? -1 - pe : pe;
			o = polish_point<false>(A.fields[fi], A.outs[fi], idx, e0, listed, &off);
		}
		unsigned m = __ballot_sync(full, v && off);
		while (m)
		{
			const int src = __ffs(m) - 1;
			m &= m - 1;
			const int f2 = __shfl_sync(full, fi, src);
			const size_t i2 = (size_t)__shfl_sync(full, (unsigned long long)idx, src);
			const double e2 = __shfl_sync(full, e0, src);
			const bool l2 = __shfl_sync(full, (int)listed, src) != 0;
			const PolishOutcome ow = polish_point<true>(A.fields[f2], A.outs[f2], i2, e2, l2, nullptr);
			if (lane == src) o = ow;
		}
		const bool fin = isfinite(o.err);
		const bool high = v && !(o.err <= POLISH_ERR);
		const double me = v && fin ? o.err : 0;
		const unsigned long long un = v && listed && !o.conv ? 1 : 0;
		const unsigned long long ab = high && !o.floor ? 1 : 0, fl = high && o.floor ? 1 : 0;
		/* the statistics go to each point's field: warp sums when the warp's
		   points share one field */
		const int f0 = __shfl_sync(full, fi, 0);
		if (__all_sync(full, !v || fi == f0))
		{
			polish_stats(A.outs[f0].stats, me, v && !fin, v ? 1 : 0, un, ab, fl);
		}
		else if (v)
		{
			unsigned long long* st = A.outs[fi].stats;
			atomicMax(&st[STAT_POLISHED_MAX_ERR], (unsigned long long)__double_as_longlong(me));
			if (!fin) atomicOr(&st[STAT_POLISHED_NAN], 1ull);
			atomicAdd(&st[STAT_POLISHED], 1ull);
			if (un) atomicAdd(&st[STAT_POLISHED_UNCONV], un);
			if (ab) atomicAdd(&st[STAT_POLISHED_ABOVE], ab);
			if (fl) atomicAdd(&st[STAT_POLISHED_FLOOR], fl);
		}
	}
}

} /* namespace */

cudaError_t launch_polish(cudaStream_t s, const PolishArgs& a, long long max_points, int num_sms)
{
	if (a.num_fields <= 0 || max_points <= 0) return cudaSuccess;
	/* the scan: at least 8 points per thread, about 8 blocks per SM over all fields */
	long long bx = (max_points + 256LL * 8 - 1) / (256LL * 8);
	const long long cap = std::max(1LL, (8LL * num_sms + a.num_fields - 1) / a.num_fields);
	bx = std::max(1LL, std::min(bx, cap));
	polish_scan_kernel<<<dim3((unsigned)bx, (unsigned)a.num_fields), 256, 0, s>>>(a);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess || a.list_cap <= 0) return e;
	/* the list: one lane per point, 8 blocks of 256 per SM, striding */
	polish_list_kernel<<<8 * num_sms, 256, 0, s>>>(a);
	return cudaGetLastError();
}

} /* namespace ccf */
