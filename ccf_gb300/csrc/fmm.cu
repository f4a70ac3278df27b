/******************************************************************************
fmm.cu -- 2-D complex fast multipole passes on the device, FP64.

Expansions of the log potential sum m_i log(z - z_i), in units of the node
half-length, as in the reference (include/fmm.cuh): multipole coefficients
a_0 = sum m, a_k = -sum m ((z_i - c)/h)^k / k; local coefficients c_l of
sum c_l ((z - c)/h)^l.  Translations:
  P2M  fmm.cuh:21-49       M2M  fmm.cuh:109-139      L2L  fmm.cuh:204-223
  M2L  fmm.cuh:281-322     P2L  fmm.cuh:387-413
Layout: one warp per node, lane p computes coefficient p (order <= 31, so a
whole expansion is one warp).  A translation takes one complex reciprocal
per source, not the reference's division per term; powers come from a
product scan over the warp, and the M2L sum runs over pre-scaled terms (the
FP64 pipe is the bound).  The binomial table is passed in: by default it holds the
reference's int32 Pascal triangle (whose entries above n = 33 wrap), because
the reference's M2L uses those values and its roots depend on them.
******************************************************************************/
#include "kernels.h"

namespace ccf
{

CCF_D double binom_at(const double* __restrict__ B, int n, int k)
{
	if (n < k) return 0;
	return B[n * (n + 1) / 2 + k];
}

/* t^lane on every lane of the warp (t^0 = 1): a product scan, five complex
   products instead of lane-many.  All 32 lanes must call it. */
CCF_D double2 warp_powers(double2 t, int lane)
{
	double2 x = lane == 0 ? make_double2(1, 0) : t;
	for (int o = 1; o < 32; o <<= 1)
	{
		const double2 y = make_double2(__shfl_up_sync(0xffffffffu, x.x, o), __shfl_up_sync(0xffffffffu, x.y, o));
		if (lane >= o) x = cmul(y, x);
	}
	return x;
}

CCF_D double2 shfl_c(double2 v, int src)
{
	return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

/* upward pass at one level: P2M for leaves holding stars, M2M for split
   nodes.  The stars of a leaf are taken 32 at a time, one per lane, and
   handed round the warp by shuffles; the powers come from warp_powers. */
CCF_D void fmm_upward_node(const TreeDev& T, int n, int P, int p, const double2* __restrict__ pos,
	const double* __restrict__ mass, double2* __restrict__ multi, const double* __restrict__ B)
{
	const bool act = p <= P;
	double2 r = make_double2(0, 0);
	int ch = T.child[n];
	if (ch < 0)
	{
		int s = T.star_start[n], ns = T.star_count[n];
		if (ns == 0) return;   /* warp-uniform */
		double2 c = T.center[n];
		double ih = 1.0 / T.half[n];
		for (int i0 = 0; i0 < ns; i0 += 32)
		{
			const int nq = min(32, ns - i0);
			double mq = 0;
			double2 wq = make_double2(0, 0);
			if (p < nq)
			{
				const double2 q = pos[s + i0 + p];
				mq = mass[s + i0 + p];
				wq = make_double2((q.x - c.x) * ih, (q.y - c.y) * ih);
			}
			for (int i = 0; i < nq; i++)
			{
				const double m = __shfl_sync(0xffffffffu, mq, i);
				const double2 t = warp_powers(shfl_c(wq, i), p);
				if (p == 0)
				{
					r.x += m;
				}
				else
				{
					r.x -= t.x * m;
					r.y -= t.y * m;
				}
			}
		}
		if (p > 0)
		{
			r.x /= p;
			r.y /= p;
		}
	}
	else
	{
		double2 pc = T.center[n];
		for (int q = 0; q < 4; q++)
		{
			int k = ch + q;
			const double2* a = multi + (size_t)k * (P + 1);
			double2 cc = T.center[k];
			double ih = 1.0 / T.half[k];
			double2 dz = make_double2((cc.x - pc.x) * ih, (cc.y - pc.y) * ih);
			const double2 dzp = warp_powers(dz, p);
			double2 v = make_double2(0, 0);
			if (p == 0)
			{
				v = a[0];
			}
			else if (act)
			{
				/* b_p = (sum_{i=1..p} a_i C(p-1, i-1) dz^(p-i) - a_0 dz^p / p) / 2^p */
				double2 acc = cscale(a[1], binom_at(B, p - 1, 0));
				for (int i = 2; i <= p; i++) acc = cadd(cmul(acc, dz), cscale(a[i], binom_at(B, p - 1, i - 1)));
				double2 t = cscale(cmul(a[0], dzp), 1.0 / p);
				v = cscale(csub(acc, t), ldexp(1.0, -p));
			}
			r = cadd(r, v);
		}
	}
	if (act) multi[(size_t)n * (P + 1) + p] = r;
}

__global__ void fmm_upward_kernel(TreeDev T, int start, int count, int P, const double2* __restrict__ pos,
	const double* __restrict__ mass, double2* __restrict__ multi, const double* __restrict__ B)
{
	int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	if (w >= count) return;   /* warp-uniform */
	fmm_upward_node(T, start + w, P, threadIdx.x & 31, pos, mass, multi, B);
}

/* downward pass at one level >= 2: L2L from the parent, then M2L from the
   same-level interaction list, then P2L from the coarser-leaf list, summed
   in that order (include/ccf.cuh:880-893).  GB300's FP64 pipe is 1/64 of its
   FP32 one, so the translations are arranged for few FP64 operations per
   lane: the per-source constants (the M2L ratio t = -1/dz and log(-dz); the
   P2L star offsets and their logs) are formed once, one source per lane, and
   handed round by shuffles; lane p takes t^p from a product scan; and the
   M2L sum over k is a binomial-weighted sum of the pre-scaled b_k t^k (two
   FMAs a term) instead of a complex Horner recurrence. */
/* part `part` of nparts of node n's downward coefficients, one warp: the
   L2L in part 0, the M2L sources j = part, part + nparts, ..., the P2L
   sources likewise; fmm_downward_reduce sums the parts in their order */
constexpr int DOWN_PARTS = 4;
CCF_D double2 fmm_downward_part(const TreeDev& T, int n, int P, int p, int part, int nparts, const double2* __restrict__ pos,
	const double* __restrict__ mass, const double2* __restrict__ multi, const double2* __restrict__ local,
	const double* __restrict__ B)
{
	const bool act = p <= P;
	double2 cn = T.center[n];
	double2 r = make_double2(0, 0);
	/* L2L: d_p = sum_{k>=max(p,1)} c_k C(k,p) dz^(k-p) / 2^p, dz = (c - c_parent)/h_parent */
	if (act && part == 0)
	{
		int par = T.parent[n];
		const double2* cl = local + (size_t)par * (P + 1);
		double2 pcn = T.center[par];
		double ih = 1.0 / T.half[par];
		double2 dz = make_double2((cn.x - pcn.x) * ih, (cn.y - pcn.y) * ih);
		int k0 = p > 1 ? p : 1;
		double2 acc = cscale(cl[P], binom_at(B, P, p));
		for (int k = P - 1; k >= k0; k--) acc = cadd(cmul(acc, dz), cscale(cl[k], binom_at(B, k, p)));
		if (p == 0) acc = cmul(acc, dz);
		r = cscale(acc, ldexp(1.0, -p));
	}
	/* M2L: t = 1/(-dz), dz = (c_from - c_to)/h_from;
	   c_0 = sum_k b_k t^k + b_0 log(-dz) + b_0 log h_from
	   c_p = (sum_k b_k C(p+k-1, k-1) t^k - b_0/p) (-t)^p */
	const int nm = T.m2l_count[n];
	static_assert(MAX_M2L <= 32, "one interaction per lane");
	int fq = 0;
	double2 tq = make_double2(0, 0), lq = make_double2(0, 0);
	double hq = 0;
	if (p < nm)
	{
		fq = T.m2l[n * MAX_M2L + p];
		const double2 cf = T.center[fq];
		const double hf = T.half[fq];
		const double ih = 1.0 / hf;
		const double2 dz = make_double2((cf.x - cn.x) * ih, (cf.y - cn.y) * ih);
		tq = cinv(make_double2(-dz.x, -dz.y));
		lq = make_double2(log(hypot(dz.x, dz.y)), atan2(-dz.y, -dz.x));
		hq = log(hf);
	}
	for (int j = part; j < nm; j += nparts)
	{
		const int f = __shfl_sync(0xffffffffu, fq, j);
		const double2 t = shfl_c(tq, j);
		const double2 lg = shfl_c(lq, j);
		const double lh = __shfl_sync(0xffffffffu, hq, j);
		const double2* b = multi + (size_t)f * (P + 1);
		const double2 tp = warp_powers(t, p);
		const double2 bt = act && p >= 1 ? cmul(b[p], tp) : make_double2(0, 0);   /* b_p t^p on lane p */
		double2 acc = make_double2(0, 0);
		for (int k = P; k >= 1; k--)
		{
			const double2 v = shfl_c(bt, k);
			if (act) acc = cadd(acc, cscale(v, binom_at(B, p + k - 1, k - 1)));
		}
		if (!act) continue;
		double2 v;
		if (p == 0)
		{
			v = cadd(cadd(acc, cmul(b[0], lg)), cscale(b[0], lh));
		}
		else
		{
			const double2 mtp = (p & 1) ? make_double2(-tp.x, -tp.y) : tp;   /* (-t)^p */
			v = cmul(csub(acc, cscale(b[0], 1.0 / p)), mtp);
		}
		r = cadd(r, v);
	}
	/* P2L: c_0 = sum m log(-w) + m log h, c_p = -sum m / (p w^p), w = (z_i - c)/h */
	int np = T.p2l_count[n];
	double hn = T.half[n];
	double ihn = 1.0 / hn;
	double lhn = log(hn);
	const double ip = p > 0 ? 1.0 / p : 0.0;
	for (int j = part; j < np; j += nparts)
	{
		int f = T.p2l[n * MAX_P2L + j];
		int s = T.star_start[f], ns = T.star_count[f];
		double2 v = make_double2(0, 0);
		for (int i0 = 0; i0 < ns; i0 += 32)
		{
			const int nq = min(32, ns - i0);
			double mq = 0;
			double2 iq = make_double2(0, 0), gq = make_double2(0, 0);
			if (p < nq)
			{
				const double2 q = pos[s + i0 + p];
				mq = mass[s + i0 + p];
				const double2 wz = make_double2((q.x - cn.x) * ihn, (q.y - cn.y) * ihn);
				iq = cinv(wz);
				gq = make_double2(log(hypot(wz.x, wz.y)), atan2(-wz.y, -wz.x));
			}
			for (int i = 0; i < nq; i++)
			{
				const double m = __shfl_sync(0xffffffffu, mq, i);
				const double2 lg = shfl_c(gq, i);
				const double2 t = warp_powers(shfl_c(iq, i), p);
				if (p == 0)
				{
					v.x += m * lg.x + m * lhn;
					v.y += m * lg.y;
				}
				else
				{
					v.x -= m * t.x * ip;
					v.y -= m * t.y * ip;
				}
			}
		}
		r = cadd(r, v);
	}
	return r;
}

/* node n's downward pass by the DOWN_PARTS warps of the calling block (every
   thread calls it): the parts' sums meet in shared memory in a fixed order */
CCF_D void fmm_downward_node(const TreeDev& T, int n, int P, const double2* __restrict__ pos,
	const double* __restrict__ mass, const double2* __restrict__ multi, double2* __restrict__ local,
	const double* __restrict__ B)
{
	__shared__ double2 red[DOWN_PARTS][32];
	const int p = threadIdx.x & 31, part = threadIdx.x >> 5;
	red[part][p] = fmm_downward_part(T, n, P, p, part, DOWN_PARTS, pos, mass, multi, local, B);
	__syncthreads();
	if (part == 0 && p <= P)
	{
		double2 r = red[0][p];
		for (int k = 1; k < DOWN_PARTS; k++) r = cadd(r, red[k][p]);
		local[(size_t)n * (P + 1) + p] = r;
	}
	__syncthreads();
}

/* one node per block of DOWN_PARTS warps */
__global__ void __launch_bounds__(DOWN_PARTS * 32) fmm_downward_kernel(TreeDev T, int start, int count, int P,
	const double2* __restrict__ pos, const double* __restrict__ mass, const double2* __restrict__ multi,
	double2* __restrict__ local, const double* __restrict__ B)
{
	if ((int)blockIdx.x >= count) return;   /* block-uniform */
	fmm_downward_node(T, start + blockIdx.x, P, pos, mass, multi, local, B);
}

/* leaf records for the solver: centre, 1/h, packed near stars (neighbours
   first, then the leaf's own stars, as include/alpha_star.cuh:26-37 sums
   them) and the local coefficients pre-scaled for alpha, d/dzbar, d2/dzbar2:
   L1_i = theta^2 i c_i / h, L2_i = theta^2 i (i-1) c_i / h^2,
   L3_i = theta^2 i (i-1) (i-2) c_i / h^3 */
CCF_D void leaf_build_node(const TreeDev& T, int n, int lane, const int* __restrict__ leaf_index, int P, double theta2,
	const double2* __restrict__ pos, const double* __restrict__ mass, const double2* __restrict__ local,
	double2* __restrict__ leaf_center, double* __restrict__ leaf_inv_half, int* __restrict__ leaf_near_count,
	NearStar* __restrict__ leaf_near, double2* __restrict__ leaf_loc, float2* __restrict__ leaf_loc3f,
	int* __restrict__ node_leaf, int* err)
{
	if (T.child[n] >= 0) return;
	int l = leaf_index[n];
	if (lane == 0)
	{
		node_leaf[n] = l;
		leaf_center[l] = T.center[n];
		leaf_inv_half[l] = 1.0 / T.half[n];
	}
	/* near list */
	if (lane == 0)
	{
		int cnt = 0;
		NearStar* out = leaf_near + (size_t)l * MAX_NEAR;
		int k = T.nbr_count[n];
		for (int j = 0; j <= k; j++)
		{
			int src = j < k ? T.nbr[n * MAX_NBR + j] : n;
			int s = T.star_start[src], ns = T.star_count[src];
			for (int i = 0; i < ns; i++)
			{
				if (cnt < MAX_NEAR)
				{
					double2 q = pos[s + i];
					out[cnt].x = q.x;
					out[cnt].y = q.y;
					out[cnt].m = mass[s + i];
					out[cnt].pad = 0;
				}
				cnt++;
			}
		}
		if (cnt > MAX_NEAR) atomicOr(err, 2);
		leaf_near_count[l] = cnt < MAX_NEAR ? cnt : MAX_NEAR;
	}
	/* scaled local coefficients */
	for (int i = lane; i <= P; i += 32)
	{
		double2 c = local[(size_t)n * (P + 1) + i];
		double ih = 1.0 / T.half[n];
		double f1 = theta2 * i * ih;
		double f2 = theta2 * i * (i - 1) * ih * ih;
		double f3 = theta2 * i * (i - 1) * (i - 2) * ih * ih * ih;
		double2* L = leaf_loc + (size_t)l * 3 * (P + 1);
		L[i] = cscale(c, f1);
		L[(P + 1) + i] = cscale(c, f2);
		double2 c3 = cscale(c, f3);
		L[2 * (P + 1) + i] = c3;
		leaf_loc3f[(size_t)l * (P + 1) + i] = make_float2((float)c3.x, (float)c3.y);
	}
}

__global__ void leaf_build_kernel(TreeDev T, int num_nodes, const int* __restrict__ leaf_index, int P, double theta2,
	const double2* __restrict__ pos, const double* __restrict__ mass, const double2* __restrict__ local,
	double2* __restrict__ leaf_center, double* __restrict__ leaf_inv_half, int* __restrict__ leaf_near_count,
	NearStar* __restrict__ leaf_near, double2* __restrict__ leaf_loc, float2* __restrict__ leaf_loc3f,
	int* __restrict__ node_leaf, int* err)
{
	int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	if (w >= num_nodes) return;
	leaf_build_node(T, w, threadIdx.x & 31, leaf_index, P, theta2, pos, mass, local, leaf_center, leaf_inv_half,
		leaf_near_count, leaf_near, leaf_loc, leaf_loc3f, node_leaf, err);
}

void launch_fmm_upward(cudaStream_t s, const TreeDev& T, int start, int count, int P, const double2* pos, const double* mass,
	double2* multi, const double* B)
{
	long long threads = (long long)count * 32;
	fmm_upward_kernel<<<(int)((threads + 127) / 128), 128, 0, s>>>(T, start, count, P, pos, mass, multi, B);
}
void launch_fmm_downward(cudaStream_t s, const TreeDev& T, int start, int count, int P, const double2* pos, const double* mass,
	const double2* multi, double2* local, const double* B)
{
	if (count > 0) fmm_downward_kernel<<<count, DOWN_PARTS * 32, 0, s>>>(T, start, count, P, pos, mass, multi, local, B);
}
void launch_leaf_build(cudaStream_t s, const TreeDev& T, int num_nodes, const int* leaf_index, int P, double theta2,
	const double2* pos, const double* mass, const double2* local, double2* leaf_center, double* leaf_inv_half,
	int* leaf_near_count, NearStar* leaf_near, double2* leaf_loc, float2* leaf_loc3f, int* node_leaf, int* err)
{
	long long threads = (long long)num_nodes * 32;
	leaf_build_kernel<<<(int)((threads + 127) / 128), 128, 0, s>>>(T, num_nodes, leaf_index, P, theta2, pos, mass, local,
		leaf_center, leaf_inv_half, leaf_near_count, leaf_near, leaf_loc, leaf_loc3f, node_leaf, err);
}

} /* namespace ccf */

namespace ccf
{

/* double-float copies of the leaf records for the mixed-precision evaluators:
   near stars relative to the leaf centre (formed in FP64, then split),
   masses, the alpha and d/dzbar coefficient blocks, and 1/h.  One warp per
   leaf. */
CCF_D void leaf_df_leaf(int l, int i, int P, const double2* __restrict__ leaf_center,
	const double* __restrict__ leaf_inv_half, const int* __restrict__ near_count, const NearStar* __restrict__ near,
	const double2* __restrict__ loc, float4* __restrict__ near_df, float2* __restrict__ mass_df, float4* __restrict__ loc_df,
	float2* __restrict__ ih_df)
{
	const double2 c = leaf_center[l];
	auto split = [](double x) {
		float h = __double2float_rn(x);
		return make_float2(h, __double2float_rn(x - (double)h));
	};
	if (i < near_count[l])
	{
		NearStar s = near[(size_t)l * MAX_NEAR + i];
		float2 x = split(s.x - c.x), y = split(s.y - c.y);
		near_df[(size_t)l * MAX_NEAR + i] = make_float4(x.x, y.x, x.y, y.y);
		mass_df[(size_t)l * MAX_NEAR + i] = split(s.m);
	}
	if (i <= P)
	{
		for (int k = 0; k < 2; k++)
		{
			double2 v = loc[((size_t)l * 3 + k) * (P + 1) + i];
			float2 re = split(v.x), im = split(v.y);
			loc_df[((size_t)l * 2 + k) * (P + 1) + i] = make_float4(re.x, im.x, re.y, im.y);
		}
	}
	if (i == 0) ih_df[l] = split(leaf_inv_half[l]);
}

__global__ void leaf_df_kernel(int num_leaves, int P, const double2* __restrict__ leaf_center,
	const double* __restrict__ leaf_inv_half, const int* __restrict__ near_count, const NearStar* __restrict__ near,
	const double2* __restrict__ loc, float4* __restrict__ near_df, float2* __restrict__ mass_df, float4* __restrict__ loc_df,
	float2* __restrict__ ih_df)
{
	const int l = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
	if (l >= num_leaves) return;
	leaf_df_leaf(l, threadIdx.x & 31, P, leaf_center, leaf_inv_half, near_count, near, loc, near_df, mass_df, loc_df, ih_df);
}

void launch_leaf_df(cudaStream_t s, int num_leaves, int P, const double2* leaf_center, const double* leaf_inv_half,
	const int* near_count, const NearStar* near, const double2* loc, float4* near_df, float2* mass_df, float4* loc_df,
	float2* ih_df)
{
	const int warps = 4;
	leaf_df_kernel<<<(num_leaves + warps - 1) / warps, warps * 32, 0, s>>>(num_leaves, P, leaf_center, leaf_inv_half,
		near_count, near, loc, near_df, mass_df, loc_df, ih_df);
}

} /* namespace ccf */

namespace ccf
{

/* The smooth-mass Taylor series of the rectangular field, folded into the
   local expansion of every leaf where that is exact to the evaluation's
   rounding, for the continuation tracker.  The three series enter the
   evaluators conjugated, as polynomials in z: conj(d alpha_s / d zbar) - k1
   with f's local alpha'' block (ef), conj(d2 alpha_s / d zbar2) with f''s
   alpha''' block (er), and conj of the anti-analytic part of alpha_s with the
   lens map's alpha block (eq).  Shifted to the leaf centre and scaled to the
   leaf's dz = (z - centre) / h, a polynomial adds to the block's
   coefficients up to the expansion order; the leaf is folded when the terms
   beyond it sum to less than 1e-15 at |dz| = sqrt 2 (the corner of the leaf)
   and the leaf lies inside 0.95 of the corner circle, where the series
   converges.  One warp per leaf, lane i building coefficient i of the three
   blocks (the expansion order is at most 31); the FP64 blocks stay as they
   are (the direct evaluators keep using them with the series). */
constexpr int FOLD_MAXD = 256;
static_assert(MAX_ORDER < 32, "one coefficient of a leaf block per lane");

/* h^j times the j-th Taylor coefficient at z0 of sum_k e_k z^k, i.e.
   h^j sum_{k >= j} C(k, j) e_k z0^(k - j): Horner from the top degree with
   the binomial carried down the column, C(k, j) = C(k + 1, j) (k + 1 - j) / (k + 1)
   (inv[k] = 1 / k).  Zero for j outside [0, n). */
CCF_D double2 fold_coef(const double2* __restrict__ e, int n, double2 z0, double h, int j, const double* inv)
{
	if (j < 0 || j >= n) return make_double2(0, 0);
	double b = 1;   /* C(n - 1, j) */
	for (int i = 0; i < j; i++) b *= (double)(n - 1 - i) * inv[i + 1];
	double2 acc = make_double2(b * e[n - 1].x, b * e[n - 1].y);
	for (int k = n - 2; k >= j; k--)
	{
		b *= (double)(k + 1 - j) * inv[k + 1];
		const double2 ek = e[k];
		acc = cmul(acc, z0);
		acc.x += b * ek.x;
		acc.y += b * ek.y;
	}
	double hj = 1;
	for (int i = 0; i < j; i++) hj *= h;
	return make_double2(acc.x * hj, acc.y * hj);
}

/* sum over j = start, start + 32, ... < n of |coefficient j| sqrt(2)^j: one
   lane's share of the terms beyond a block's order at the leaf corner */
CCF_D double fold_tail(const double2* __restrict__ e, int n, double2 z0, double h, int start, const double* inv)
{
	double t = 0;
	for (int j = start; j < n; j += 32)
	{
		const double2 v = fold_coef(e, n, z0, h, j, inv);
		t += hypot(v.x, v.y) * ldexp((j & 1) ? 1.4142135623730951 : 1.0, j >> 1);
	}
	return t;
}

/* one leaf per CTA of three warps: warp 0 folds the alpha series (eq) into
   block 0, warp 1 the d alpha / d zbar series (ef) into block 1, warp 2 the
   d2 alpha / d zbar2 series (er) into block 2; each lane forms one shifted
   coefficient and a share of its series' tail beyond the block's order, and
   the leaf folds when all three tails are negligible */
__global__ void __launch_bounds__(96) fold_smooth_kernel(int num_leaves, int P, const double2* __restrict__ leaf_center,
	const double* __restrict__ leaf_inv_half, const double2* __restrict__ loc, const double2* __restrict__ ef, int nf,
	const double2* __restrict__ er, int nr, const double2* __restrict__ eq, int nq, double radius,
	float4* __restrict__ loc_df, float2* __restrict__ loc3f, double2* __restrict__ loc64, unsigned char* __restrict__ fold)
{
	__shared__ double inv[FOLD_MAXD + 1];
	__shared__ int s_ok[3];
	for (int k = threadIdx.x; k <= FOLD_MAXD; k += blockDim.x) inv[k] = k ? 1.0 / k : 0.0;
	__syncthreads();
	const int lane = threadIdx.x & 31, part = threadIdx.x >> 5;
	const int l = blockIdx.x;
	if (l >= num_leaves) return;   /* block-uniform */
	const double2 c = leaf_center[l];
	const double h = 1.0 / leaf_inv_half[l];
	if (hypot(c.x, c.y) + 1.4142135623730951 * h > radius || nf > FOLD_MAXD || nr > FOLD_MAXD || nq > FOLD_MAXD)
	{
		if (threadIdx.x == 0) fold[l] = 0;
		return;
	}
	/* block 0 (alpha) gains dz^0 .. dz^(P-1) of eq at its coefficients 1 .. P,
	   block 1 (the d alpha / d zbar block) dz^0 .. dz^(P-2) of ef at 2 .. P,
	   block 2 (the d2 alpha / d zbar2 block) dz^0 .. dz^(P-3) of er at 3 .. P */
	const double2* e = part == 0 ? eq : part == 1 ? ef : er;
	const int n = part == 0 ? nq : part == 1 ? nf : nr;
	const int i = lane;
	const double2 v = i >= part + 1 && i <= P ? fold_coef(e, n, c, h, i - part - 1, inv) : make_double2(0, 0);
	double t = fold_tail(e, n, c, h, P - part + lane, inv);
	for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
	const double tol = 1e-15;
	if (lane == 0) s_ok[part] = t <= tol ? 1 : 0;
	__syncthreads();
	const bool ok = s_ok[0] && s_ok[1] && s_ok[2];
	if (threadIdx.x == 0) fold[l] = ok ? 1 : 0;
	if (!ok || i > P) return;
	auto split = [](double x) {
		float hi = __double2float_rn(x);
		return make_float2(hi, __double2float_rn(x - (double)hi));
	};
	const double2 a = cadd(loc[((size_t)l * 3 + part) * (P + 1) + i], v);
	if (part < 2)
	{
		const float2 x = split(a.x), y = split(a.y);
		loc_df[((size_t)l * 2 + part) * (P + 1) + i] = make_float4(x.x, y.x, x.y, y.y);
	}
	else
	{
		loc3f[(size_t)l * (P + 1) + i] = make_float2((float)a.x, (float)a.y);
	}
	if (loc64) loc64[((size_t)l * 3 + part) * (P + 1) + i] = a;
}

void launch_fold_smooth(cudaStream_t s, int num_leaves, int P, const double2* leaf_center, const double* leaf_inv_half,
	const double2* loc, const double2* ef, int nf, const double2* er, int nr, const double2* eq, int nq, double radius,
	float4* loc_df, float2* loc3f, double2* loc64, unsigned char* fold)
{
	if (num_leaves <= 0) return;
	fold_smooth_kernel<<<num_leaves, 96, 0, s>>>(num_leaves, P, leaf_center, leaf_inv_half, loc, ef, nf, er, nr, eq, nq,
		radius, loc_df, loc3f, loc64, fold);
}

} /* namespace ccf */

namespace ccf
{

/* The FMM passes of a batch, level by level over every field at once:
   blockIdx.y is the field, the x blocks take four of its nodes of level L
   each (one warp per node, as fmm_upward_kernel / fmm_downward_kernel do
   for one field); a field without that level, or with fewer nodes there,
   leaves its extra blocks idle.  The expansions start from zero (the first
   kernel), and the leaf numbering takes one CTA per field (the last). */
__global__ void fmm_zero_batch_kernel(const BatchSeg* __restrict__ segs)
{
	const BatchSeg& S = segs[blockIdx.y];
	const size_t nc = (size_t)S.info[1] * (S.P + 1);
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nc; i += (size_t)gridDim.x * blockDim.x)
	{
		S.multi[i] = make_double2(0, 0);
		S.local[i] = make_double2(0, 0);
	}
}

__global__ void fmm_level_batch_kernel(const BatchSeg* __restrict__ segs, int L, int upward)
{
	const BatchSeg& S = segs[blockIdx.y];
	if (L > S.info[0]) return;   /* block-uniform */
	if (upward)
	{
		/* four nodes per block, one warp each */
		const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
		if (w >= S.info[3 + TREE_MAX_LEVELS + 1 + L]) return;   /* warp-uniform */
		fmm_upward_node(S.T, S.info[3 + L] + w, S.P, threadIdx.x & 31, S.pos, S.mass, S.multi, S.B);
	}
	else
	{
		/* one node per block, DOWN_PARTS warps */
		if ((int)blockIdx.x >= S.info[3 + TREE_MAX_LEVELS + 1 + L]) return;   /* block-uniform */
		fmm_downward_node(S.T, S.info[3 + L] + blockIdx.x, S.P, S.pos, S.mass, S.multi, S.local, S.B);
	}
}

__global__ void __launch_bounds__(1024) leaf_number_batch_kernel(const BatchSeg* __restrict__ segs)
{
	const BatchSeg& S = segs[blockIdx.x];
	const int nodes = S.info[1];
	for (int i = threadIdx.x; i < nodes; i += blockDim.x) S.leaf_flag[i] = S.T.child[i] < 0;
	__syncthreads();
	const int nl = block_exclusive_scan(S.leaf_flag, S.leaf_index, nodes);
	if (threadIdx.x == 0) S.info[LEAF_INFO] = nl;
}

/* The leaf records of one field per CTA, for batches: leaf_build_kernel,
   leaf_df_kernel and star_hilo_kernel for one field, and the sum of the
   near-list lengths and the error bits for the host. */
__global__ void __launch_bounds__(512) leaf_batch_kernel(const BatchSeg* __restrict__ segs)
{
	__shared__ int s_err, s_near;
	const BatchSeg& S = segs[blockIdx.x];
	const TreeDev T = S.T;
	const unsigned full = 0xffffffffu;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
	const int nodes = S.info[1], nl = S.num_leaves;
	if (tid == 0)
	{
		s_err = 0;
		s_near = 0;
	}
	__syncthreads();
	for (int w = warp; w < nodes; w += nw)
		leaf_build_node(T, w, lane, S.leaf_index, S.P, S.theta2, S.pos, S.mass, S.local, S.leaf_center, S.leaf_inv_half,
			S.leaf_near_count, S.leaf_near, S.leaf_loc, S.leaf_loc3f, S.node_leaf, &s_err);
	__syncthreads();
	int cnt = 0;
	for (int l = tid; l < nl; l += blockDim.x) cnt += S.leaf_near_count[l];
	cnt = __reduce_add_sync(full, cnt);
	if (lane == 0) atomicAdd(&s_near, cnt);
	if (S.leaf_near_df)
	{
		for (int l = warp; l < nl; l += nw)
			leaf_df_leaf(l, lane, S.P, S.leaf_center, S.leaf_inv_half, S.leaf_near_count, S.leaf_near, S.leaf_loc,
				S.leaf_near_df, S.leaf_mass_df, S.leaf_loc_df, S.leaf_ih_df);
		for (int i = tid; i < S.n; i += blockDim.x)
		{
			S.star_hilo[i] = split_hilo(S.pos[i]);
			const double m = S.mass[i];
			const float h = __double2float_rn(m);
			S.star_mass_df[i] = make_float2(h, __double2float_rn(m - (double)h));
		}
	}
	__syncthreads();
	if (tid == 0)
	{
		S.info[LEAF_INFO + 1] = s_near;
		S.info[LEAF_INFO + 2] = s_err;
	}
}

void launch_fmm_batch(cudaStream_t s, const BatchSeg* segs, int nseg, int max_levels, int max_level_nodes,
	long long max_coefficients)
{
	if (nseg <= 0) return;
	const int gz = (int)std::min<long long>((max_coefficients + 255) / 256, 64);
	fmm_zero_batch_kernel<<<dim3(std::max(gz, 1), nseg), 256, 0, s>>>(segs);
	const int gx = std::max(1, (max_level_nodes + 3) / 4);
	for (int L = max_levels; L >= 0; L--) fmm_level_batch_kernel<<<dim3(gx, nseg), 128, 0, s>>>(segs, L, 1);
	static_assert(DOWN_PARTS * 32 == 128, "the level kernel's blocks");
	for (int L = 2; L <= max_levels; L++)
		fmm_level_batch_kernel<<<dim3(std::max(1, max_level_nodes), nseg), 128, 0, s>>>(segs, L, 0);
	leaf_number_batch_kernel<<<nseg, 1024, 0, s>>>(segs);
}
void launch_leaf_batch(cudaStream_t s, const BatchSeg* segs, int nseg)
{
	if (nseg > 0) leaf_batch_kernel<<<nseg, 512, 0, s>>>(segs);
}

} /* namespace ccf */
