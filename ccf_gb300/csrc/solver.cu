/******************************************************************************
solver.cu -- the Aberth-Ehrlich root solver and the phi continuation.

For a branch centre (initial solve) or a (branch, side) continuation row,
every root z_k of the critical-curve function f(z; phi) is updated by the
Aberth step of the reference (include/ccf_functions.cuh:193-243):

    z_k <- z_k - f / (f' + f (2 sum_i 1/(z_k - z_i) - sum_{j != k} 1/(z_k - z_j)))

and the continuation advances phi step by step away from the branch centre
(include/ccf_functions.cuh:261-394, include/ccf.cuh:979-1033).

GB300 design:
  * one thread-block cluster owns one row for all of its phi steps, so a
    whole continuation is a single launch; the CTAs of the cluster split the
    row's active roots and meet at cluster barriers between sweeps;
  * sweeps are Jacobi sweeps against a snapshot of the row, so the result
    does not depend on thread timing (the reference updates roots in place
    while other threads read them, include/ccf_functions.cuh:374-389);
  * the O(R + N) correction sums stream roots and stars through shared
    memory (cp.async, double-buffered) and every source is broadcast to all
    targets of the tile; each thread carries TPT targets;
  * mixed precision: the correction sums run in FP32 on the split hi + lo
    form of the coordinates (differences keep their relative accuracy for
    nearby roots), per-chunk partial sums are accumulated in FP64; the
    critical-curve function f is evaluated in double-float (two FP32 numbers,
    ~48 significant bits, field_df.cuh) on the FP32 pipe, which GB300 runs 62
    times faster than its FP64 pipe; f' is FP32.  The converged roots are the
    zeros of f to ~1e-13: the sums and f' only set the step size;
  * a root is final once its step is below 1e-9 theta_star (the reference's
    test, ccf_functions.cuh:385); sweeps stop when no root of the row is
    active or the sweep cap is reached;
  * the residual (1/mu error bound), the caustic and the length scale of
    each point are computed in the epilogue of its phi step and written
    straight into the output layout, so no transpose pass is needed.
******************************************************************************/
#include "field_df.cuh"
#include "kernels.h"

#include <cooperative_groups.h>
#include <type_traits>

namespace cg = cooperative_groups;

namespace ccf
{

constexpr int NT = 256;          /* threads per CTA */
constexpr int MAX_CLUSTER = 16;  /* CTAs per row (above 8: the non-portable cluster sizes) */
constexpr int TPT = 2;           /* targets per thread */
constexpr int TILE = NT * TPT;   /* targets per tile */
constexpr int CHUNK = 1024;      /* sources per shared-memory stage */

CCF_D void cp_async16(void* smem, const void* gmem)
{
	unsigned s = (unsigned)__cvta_generic_to_shared(smem);
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
CCF_D void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
CCF_D void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <bool MIXED>
struct Src
{
	using T = typename std::conditional<MIXED, float4, double2>::type;
};

constexpr int OFF_CAP = 64;      /* off-field points summed by the CTA per pass */

/* Star sums of the off-field points pts[0..K), K <= OFF_CAP.  A point outside
   the root box takes the direct sum over every star, as in the reference
   (include/tree_node.cuh:535-539, include/alpha_star.cuh:26-37).  The whole
   CTA works on each point: every thread takes every NT-th star, the warps
   reduce by shuffles and the per-warp partials meet in shared memory (red,
   K * NT/32 * 6 doubles).  MIXED evaluates in double-float on the FP32 pipe
   from the split star arrays, s3 in double-float only when S3DF; otherwise
   FP64.  All threads of the CTA must call it; it ends with a barrier, after
   which out[0..K) holds the sums. */
template <bool MIXED, bool NEED1, bool S3DF>
__device__ void offfield_sums_cta(const FieldView& F, const double2* pts, int K, NearSums* out, double* red)
{
	const unsigned full = 0xffffffffu;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (int k = 0; k < K; k++)
	{
		double v[6];
		if constexpr (MIXED)
		{
			const dfc z = dfc_from(pts[k]);
			SumsDF a;
			a.s1 = {{0.f, 0.f}, {0.f, 0.f}};
			a.s2 = a.s1;
			dfc s3 = a.s1;
			float2 s3f = make_float2(0.f, 0.f);
			for (int i = threadIdx.x; i < F.num_stars; i += NT)
				star_term_df<NEED1, S3DF>(a, s3, s3f, z, F.star_df[i], F.star_mass_df[i]);
			if (!S3DF) s3 = {{s3f.x, 0.f}, {s3f.y, 0.f}};
			dfl w[6] = {a.s1.re, a.s1.im, a.s2.re, a.s2.im, s3.re, s3.im};
#pragma unroll
			for (int c = 0; c < 6; c++)
			{
				for (int o = 16; o > 0; o >>= 1)
				{
					dfl u = {__shfl_xor_sync(full, w[c].hi, o), __shfl_xor_sync(full, w[c].lo, o)};
					w[c] = df_add(w[c], u);
				}
				v[c] = df_to_double(w[c]);
			}
		}
		else
		{
			NearSums a = zero_sums();
			for (int i = threadIdx.x; i < F.num_stars; i += NT)
			{
				const double2 p = F.star_pos[i];
				star_term<NEED1, true>(a, pts[k], p.x, p.y, F.star_mass[i]);
			}
			double u[6] = {a.s1.x, a.s1.y, a.s2.x, a.s2.y, a.s3.x, a.s3.y};
#pragma unroll
			for (int c = 0; c < 6; c++)
			{
				for (int o = 16; o > 0; o >>= 1) u[c] += __shfl_xor_sync(full, u[c], o);
				v[c] = u[c];
			}
		}
		if (lane == 0)
		{
#pragma unroll
			for (int c = 0; c < 6; c++) red[(k * (NT / 32) + warp) * 6 + c] = v[c];
		}
	}
	__syncthreads();
	if (threadIdx.x < K)
	{
		const int k = threadIdx.x;
		double v[6] = {0, 0, 0, 0, 0, 0};
		for (int q = 0; q < NT / 32; q++)
		{
#pragma unroll
			for (int c = 0; c < 6; c++) v[c] += red[(k * (NT / 32) + q) * 6 + c];
		}
		out[k].s1 = make_double2(v[0], v[1]);
		out[k].s2 = make_double2(v[2], v[3]);
		out[k].s3 = make_double2(v[4], v[5]);
	}
	__syncthreads();
}

/* phase of step j of a row (include/ccf_functions.cuh:338-344) */
CCF_D double row_phi(int c, int nb, int nphi, int side, int j)
{
	double phi0 = PI / nb + c * 2 * PI / nb;
	double dphi = 2 * PI / nphi * j;
	return side == 0 ? phi0 - dphi : phi0 + dphi;
}

/* f and f' of a root */
struct FdF
{
	double2 f, df;
};

/* f(z; phi) and f'(z) for the root of every lane with valid set, given its
   leaf.  An off-field root (leaf < 0) takes its star sums from off when
   have_off is set (the CTA computed them) and otherwise from the whole warp
   -- so all 32 lanes of the warp must call it.  Not inlined: the evaluation
   needs its registers once, not in every caller's frame. */
template <bool MIXED>
__device__ __noinline__ FdF eval_fdf_warp(const FieldView& F, bool valid, double2 z, int leaf, bool have_off, NearSums off,
	double cphi, double sphi)
{
	NearSums ns = have_off ? off : zero_sums();
	if (!MIXED && valid && leaf >= 0) ns = leaf_sums<false, true>(F, leaf, z);
	offfield_sums_warp<false, true>(F, valid && leaf < 0 && !have_off, z, ns);
	FdF r;
	r.f = make_double2(0, 0);
	r.df = make_double2(0, 0);
	if (!valid) return r;
	if constexpr (MIXED)
	{
		/* f in double-float on the FP32 pipe, off-field points included;
		   f' in FP32, or FP64 where FP32 overflows */
		r.f = eval_f_df(F, leaf, z, cphi, sphi, ns);
		r.df = eval_df_mixed(F, leaf, z, ns.s3);
	}
	else
	{
		eval_f64<true>(F, leaf, z, cphi, sphi, ns, r.f, r.df);
	}
	return r;
}

/* A root is final once its step is below this many theta_star (the
   reference's test, include/ccf_functions.cuh:385). */
constexpr double STEP_TOL = 0.000000001;

/* outputs of one final root per lane: position, 1/mu bound, caustic,
   length scale; returns false when the 1/mu bound is not finite.  All 32
   lanes must call it (see aberth_update_warp for leaf, have_off and off).
   With DF and no length scales every point is evaluated in double-float (off
   the root box from the star sums); length scales use FP64. */
constexpr size_t NO_SLOT = ~(size_t)0;

template <bool DF>
__device__ __noinline__ bool point_epilogue_warp(const FieldView& F, const FieldOut& O, bool valid, double2 z, int leaf,
	bool have_off, NearSums off, size_t out, size_t out2, double cphi, double sphi, double* maxerr, bool unconv)
{
	NearSums ns = have_off ? off : zero_sums();
	const bool mu = O.mu != nullptr;
	const bool use_df = DF && !mu;
	if (!use_df && valid && leaf >= 0) ns = mu ? leaf_sums<true, true>(F, leaf, z) : leaf_sums<true, false>(F, leaf, z);
	offfield_sums_warp<true, true>(F, valid && leaf < 0 && !have_off, z, ns);
	if (!valid) return true;
	PointResult pr;
	if (use_df) pr = eval_point_df(F, leaf, z, cphi, sphi, ns);
	else if (O.caustics && mu) pr = eval_point<true, true>(F, leaf, z, cphi, sphi, ns);
	else if (O.caustics) pr = eval_point<true, false>(F, leaf, z, cphi, sphi, ns);
	else if (mu) pr = eval_point<false, true>(F, leaf, z, cphi, sphi, ns);
	else pr = eval_point<false, false>(F, leaf, z, cphi, sphi, ns);
	/* an unconverged point is marked for the FP64 polish (polish.cu) */
	const double stored = unconv ? unconverged_mark(pr.err) : pr.err;
	if (out != NO_SLOT)
	{
		O.ccs[out] = z;
		O.errs[out] = stored;
		if (O.caustics) O.caustics[out] = pr.w;
		if (mu) O.mu[out] = pr.mu_length;
	}
	if (out2 != NO_SLOT)
	{
		O.ccs[out2] = z;
		O.errs[out2] = stored;
		if (O.caustics) O.caustics[out2] = pr.w;
		if (mu) O.mu[out2] = pr.mu_length;
	}
	if (!isfinite(pr.err)) return false;
	atomicMax((unsigned long long*)maxerr, (unsigned long long)__double_as_longlong(pr.err));
	return true;
}

template <bool MIXED>
__global__ void __launch_bounds__(NT, 2) solve_kernel(const SolveArgs A, const int initial)
{
	using SrcT = typename Src<MIXED>::T;
	cg::cluster_group cluster = cg::this_cluster();
	const int csize = (int)cluster.num_blocks();
	const int crank = (int)cluster.block_rank();
	const int item = blockIdx.x / csize;
	/* the same for every CTA of the cluster, so a cluster leaves as a whole */
	if (item >= (A.num_rows_dev ? min(*A.num_rows_dev, A.num_rows) : A.num_rows)) return;

	__shared__ FieldView sF;
	__shared__ FieldOut sO;
	__shared__ RowDesc sR;
	__shared__ int s_fill;
	__shared__ int s_cnt;
	__shared__ int s_pre[MAX_CLUSTER + 1];
	__shared__ unsigned long long s_upd, s_terms, s_unconv;
	__shared__ double s_maxerr;
	__shared__ int s_nan_err, s_nan_step;   /* set by plain stores: every writer stores 1 */
	__shared__ int s_noff;
	__shared__ double2 s_offz[OFF_CAP];
	__shared__ NearSums s_offs[OFF_CAP];
	__shared__ __align__(16) SrcT sbuf[2][CHUNK];
	static_assert(OFF_CAP * (NT / 32) * 6 * sizeof(double) <= sizeof(sbuf), "off-field scratch");
	double* const red_off = reinterpret_cast<double*>(&sbuf[0][0]);

	if (threadIdx.x == 0)
	{
		sR = A.rows[item];
		sF = A.fields[sR.field];
		sO = A.outs[sR.field];
		s_upd = 0;
		s_terms = 0;
		s_unconv = 0;
		s_maxerr = 0;
		s_nan_err = 0;
		s_nan_step = 0;
	}
	__syncthreads();
	const FieldView& F = sF;
	const int R = F.num_roots;
	const int N = F.num_stars;
	const long long base = sR.base;
	const int c = sR.branch;
	const int side = sR.side;
	const int nb = sO.nb;
	const int o0 = (int)((long long)R * crank / csize);
	const int o1 = (int)((long long)R * (crank + 1) / csize);
	const int j0 = initial ? 0 : sO.step_first;
	const int j1 = initial ? 0 : sR.steps;
	const int max_it = initial ? sO.max_iters_init : sO.max_iters_step;
	double2* __restrict__ master = A.master + base;
	unsigned char* __restrict__ fin = A.fin + base;
	int* __restrict__ list = A.list + base;
	double2* fval = A.fval + 2 * base;
	unsigned long long n_eval = 0;   /* f evaluations of this thread */
	/* the row snapshot is rewritten between sweeps by the CTAs of the cluster:
	   no __restrict__ (it would allow the non-coherent read-only path), and
	   its loads go through L2 (__ldcg here, cp.async.cg for the sources) */
	const SrcT* rsrc;
	const SrcT* ssrc;
	if constexpr (MIXED)
	{
		rsrc = A.snap32 + base;
		ssrc = A.star_hilo[sR.field];
	}
	else
	{
		rsrc = A.snap64 + base;
		ssrc = F.star_pos;
	}
	const int nrc = (R + CHUNK - 1) / CHUNK;
	const int nsc = (N + CHUNK - 1) / CHUNK;
	const int nch = nrc + nsc;
	const bool disc_exact = !F.rectangular && !F.approx;
	int sweeps_max = 0;

	for (int j = j0; j <= j1; j++)
	{
		const double phi = initial ? (PI / nb + c * 2 * PI / nb) : row_phi(c, nb, sO.nphi, side, j);
		double sphi, cphi;
		sincos(phi, &sphi, &cphi);
		for (int a = o0 + threadIdx.x; a < o1; a += NT) fin[a] = 0;
		__syncthreads();

		int it = 0;
		while (true)
		{
			/* Newton check: f and f' of this CTA's active roots, at the positions
			   the sweep starts from.  Close to a simple zero the Aberth step
			   f / (f' + f S) is the Newton step f / f' to a relative f S / f'
			   (~1e-6 and below there), so a root whose Newton step is already
			   under the tolerance takes that step and is final without its
			   O(R + N) correction sums -- the sweep that only confirms a
			   converged root costs one evaluation.  The others keep f and f' for
			   their Aberth step after the sums. */
			if (it < max_it)
			{
				for (int a0 = o0; a0 < o1; a0 += NT)
				{
					/* uniform trip count: the CTA-wide and warp-wide calls below */
					const int a = a0 + threadIdx.x;
					const bool v = a < o1 && !fin[a];
					const double2 z = v ? master[a] : make_double2(0, 0);
					const int leaf = v ? find_leaf(F, z) : 0;
					int slot = -1;
					if (threadIdx.x == 0) s_noff = 0;
					__syncthreads();
					if (v && leaf < 0)
					{
						const int q = atomicAdd(&s_noff, 1);
						if (q < OFF_CAP)
						{
							s_offz[q] = z;
							slot = q;
						}
					}
					__syncthreads();
					const int K = min(s_noff, OFF_CAP);
					offfield_sums_cta<MIXED, false, true>(F, s_offz, K, s_offs, red_off);
					const NearSums off = slot >= 0 ? s_offs[slot] : zero_sums();
					const FdF e = eval_fdf_warp<MIXED>(F, v, z, leaf, slot >= 0, off, cphi, sphi);
					if (v)
					{
						n_eval++;
						const double2 step = cdiv(e.f, e.df);
						if (isfinite(step.x) && isfinite(step.y) && hypot(step.x, step.y) < STEP_TOL * F.theta)
						{
							master[a] = csub(z, step);
							fin[a] = 1;
						}
						else
						{
							fval[2 * a] = e.f;
							fval[2 * a + 1] = e.df;
						}
					}
				}
			}

			/* compact this CTA's active roots into its segment of the row list */
			if (threadIdx.x == 0) s_fill = 0;
			__syncthreads();
			for (int a0 = o0; a0 < o1; a0 += NT)
			{
				int a = a0 + threadIdx.x;
				bool act = a < o1 && !fin[a];
				unsigned m = __ballot_sync(0xffffffffu, act);
				int lane = threadIdx.x & 31;
				int wbase = 0;
				if (lane == 0 && m) wbase = atomicAdd(&s_fill, __popc(m));
				wbase = __shfl_sync(0xffffffffu, wbase, 0);
				if (act) list[o0 + wbase + __popc(m & ((1u << lane) - 1u))] = a;
			}
			__syncthreads();
			if (threadIdx.x == 0) s_cnt = s_fill;
			cluster.sync();
			if (threadIdx.x == 0)
			{
				int acc = 0;
				for (int r = 0; r < csize; r++)
				{
					s_pre[r] = acc;
					acc += *cluster.map_shared_rank(&s_cnt, r);
				}
				s_pre[csize] = acc;
			}
			__syncthreads();
			const int total = s_pre[csize];
			if (total == 0 || it >= max_it) break;

			/* Source split S: when the sweep has fewer full tiles than the
			   cluster has CTAs, a tile shrinks to TILE / S targets and the S warps
			   of each 64-target group split every source chunk between them; the
			   partial sums meet in shared memory.  Tail sweeps with a handful of
			   active roots then cost 1/S of a full tile on every CTA instead of a
			   full tile on one CTA. */
			/* S is chosen for the shortest sweep: a CTA takes ceil(tiles / cluster)
			   tiles, each costing a fixed ~1/8 (staging, barriers, the step) plus
			   7/8 of a full tile's sums divided by S; ties keep the smaller S */
			int S = 1;
			{
				int best = 1 << 30;
				for (int s2 = 1; s2 <= NT / 32; s2 *= 2)
				{
					const int nt = (total + TILE / s2 - 1) / (TILE / s2);
					const int cost = ((nt + csize - 1) / csize) * (NT / 32 + 7 * (NT / 32) / s2);
					if (cost < best)
					{
						best = cost;
						S = s2;
					}
				}
			}
			const int TT = TILE / S;
			const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
			const int part = warp % S;
			const int group = warp / S;
			const int ntiles = (total + TT - 1) / TT;
			for (int tile = crank; tile < ntiles; tile += csize)
			{
				int tid_a[TPT];
				bool valid[TPT];
				SrcT zs[TPT];
				double2 totR[TPT], totS[TPT];
#pragma unroll
				for (int t = 0; t < TPT; t++)
				{
					int g = tile * TT + group * 64 + t * 32 + lane;
					valid[t] = g < total;
					int a = 0;
					if (valid[t])
					{
						int r = 0;
						while (r + 1 < csize && g >= s_pre[r + 1]) r++;
						int seg0 = (int)((long long)R * r / csize);
						a = list[seg0 + (g - s_pre[r])];
					}
					tid_a[t] = a;
					if constexpr (MIXED) zs[t] = valid[t] ? __ldcg(rsrc + a) : make_float4(0, 0, 0, 0);
					else zs[t] = valid[t] ? __ldcg(rsrc + a) : make_double2(0, 0);
					totR[t] = make_double2(0, 0);
					totS[t] = make_double2(0, 0);
				}

				/* stream sources: chunk ch < nrc are roots, the rest stars */
				auto issue = [&](int ch, int buf) {
					const SrcT* src;
					int n;
					if (ch < nrc)
					{
						src = rsrc + (size_t)ch * CHUNK;
						n = min(CHUNK, R - ch * CHUNK);
					}
					else
					{
						src = ssrc + (size_t)(ch - nrc) * CHUNK;
						n = min(CHUNK, N - (ch - nrc) * CHUNK);
					}
					for (int e = threadIdx.x; e < n; e += NT) cp_async16(&sbuf[buf][e], src + e);
					cp_async_commit();
				};
				issue(0, 0);
				for (int ch = 0; ch < nch; ch++)
				{
					if (ch + 1 < nch) issue(ch + 1, (ch + 1) & 1);
					else cp_async_commit();
					cp_async_wait<1>();
					__syncthreads();
					const int n = ch < nrc ? min(CHUNK, R - ch * CHUNK) : min(CHUNK, N - (ch - nrc) * CHUNK);
					const int j0 = (n * part) / S, j1 = (n * (part + 1)) / S;
					const SrcT* sb = sbuf[ch & 1];
					if constexpr (MIXED)
					{
						float ax[TPT], ay[TPT];
#pragma unroll
						for (int t = 0; t < TPT; t++) { ax[t] = 0.f; ay[t] = 0.f; }
#pragma unroll 4
						for (int jj = j0; jj < j1; jj++)
						{
							float4 s = sb[jj];
#pragma unroll
							for (int t = 0; t < TPT; t++)
							{
								float dx = (zs[t].x - s.x) + (zs[t].z - s.z);
								float dy = (zs[t].y - s.y) + (zs[t].w - s.w);
								float d2 = fmaf(dx, dx, fmaf(dy, dy, 1e-30f));
								float r = rcp32(d2);
								ax[t] = fmaf(dx, r, ax[t]);
								ay[t] = fmaf(dy, r, ay[t]);
							}
						}
#pragma unroll
						for (int t = 0; t < TPT; t++)
						{
							double2& tot = ch < nrc ? totR[t] : totS[t];
							tot.x += (double)ax[t];
							tot.y -= (double)ay[t];
						}
					}
					else
					{
						double ax[TPT], ay[TPT];
#pragma unroll
						for (int t = 0; t < TPT; t++) { ax[t] = 0; ay[t] = 0; }
#pragma unroll 2
						for (int jj = j0; jj < j1; jj++)
						{
							double2 s = sb[jj];
#pragma unroll
							for (int t = 0; t < TPT; t++)
							{
								double dx = zs[t].x - s.x;
								double dy = zs[t].y - s.y;
								double d2 = fma(dx, dx, fma(dy, dy, 1e-300));
								double r = rcp64(d2);
								ax[t] = fma(dx, r, ax[t]);
								ay[t] = fma(dy, r, ay[t]);
							}
						}
#pragma unroll
						for (int t = 0; t < TPT; t++)
						{
							double2& tot = ch < nrc ? totR[t] : totS[t];
							tot.x += ax[t];
							tot.y -= ay[t];
						}
					}
					__syncthreads();
				}
				if (S > 1)
				{
					/* combine the S partial sums of each target (the staging
					   buffer is free: the last chunk ended with a barrier) */
					double2* red = reinterpret_cast<double2*>(&sbuf[0][0]);
#pragma unroll
					for (int t = 0; t < TPT; t++)
					{
						int slot = (part * (NT / 32 / S) + group) * 64 + t * 32 + lane;
						red[2 * slot] = totR[t];
						red[2 * slot + 1] = totS[t];
					}
					__syncthreads();
					if (part == 0)
					{
						for (int q = 1; q < S; q++)
						{
#pragma unroll
							for (int t = 0; t < TPT; t++)
							{
								int slot = (q * (NT / 32 / S) + group) * 64 + t * 32 + lane;
								totR[t] = cadd(totR[t], red[2 * slot]);
								totS[t] = cadd(totS[t], red[2 * slot + 1]);
							}
						}
					}
					__syncthreads();
				}

				/* the Aberth step of each target from the f and f' of the Newton
				   check (the sweep's starting positions, as the sums) */
				if (part == 0)
				{
#pragma unroll
					for (int t = 0; t < TPT; t++)
					{
						if (!valid[t]) continue;
						const int a = tid_a[t];
						const double2 z = __ldcg(master + a);
						const double2 f = __ldcg(fval + 2 * a), df = __ldcg(fval + 2 * a + 1);
						double2 Sg = make_double2(2 * totS[t].x - totR[t].x, 2 * totS[t].y - totR[t].y);
						if (disc_exact)
						{
							const double2 iz = cinv(z);
							Sg.x += 2 * iz.x;
							Sg.y += 2 * iz.y;
						}
						const double2 znew = csub(z, cdiv(f, cadd(df, cmul(f, Sg))));
						if (isfinite(znew.x) && isfinite(znew.y))
						{
							master[a] = znew;
							if (hypot(znew.x - z.x, znew.y - z.y) < STEP_TOL * F.theta) fin[a] = 1;
						}
						else
						{
							fin[a] = 2;   /* frozen: counted as unconverged */
							s_nan_step = 1;
						}
					}
				}
			}
			if (threadIdx.x == 0)
			{
				int mine = 0;
				for (int tile = crank; tile < ntiles; tile += csize) mine += min(TT, total - tile * TT);
				s_terms += (unsigned long long)mine * (unsigned long long)(R - 1 + N);
			}
			cluster.sync();
			/* refresh the snapshot of the roots this CTA owns (any CTA of the
			   cluster may have moved them; the row list is not read here because
			   a faster CTA may already be rewriting its segment) */
			for (int a = o0 + threadIdx.x; a < o1; a += NT)
			{
				double2 z = master[a];
				if constexpr (MIXED) A.snap32[base + a] = split_hilo(z);
				else A.snap64[base + a] = z;
			}
			it++;
		}
		sweeps_max = max(sweeps_max, it);

		/* epilogue: outputs of this phi step for the roots this CTA owns */
		int ob[2] = {c, c}, ok[2] = {sO.half, 0};
		const int nslot = initial ? 1 : row_slots(nb, sO.half, sO.seg, c, side, j, ob, ok);
		for (int a0 = o0; a0 < o1; a0 += NT)
		{
			/* uniform trip count: the epilogue is a warp-wide call */
			const int a = a0 + threadIdx.x;
			const bool v = a < o1;
			double2 z = v ? master[a] : make_double2(0, 0);
			const int leaf = v ? find_leaf(F, z) : 0;
			int slot = -1;
			if (threadIdx.x == 0) s_noff = 0;
			__syncthreads();
			if (v && leaf < 0)
			{
				const int q = atomicAdd(&s_noff, 1);
				if (q < OFF_CAP)
				{
					s_offz[q] = z;
					slot = q;
				}
			}
			__syncthreads();
			const int K = min(s_noff, OFF_CAP);
			if (sO.mu) offfield_sums_cta<MIXED, true, true>(F, s_offz, K, s_offs, red_off);
			else offfield_sums_cta<MIXED, true, false>(F, s_offz, K, s_offs, red_off);
			const size_t out = out_slot(sO, v ? a : 0, ob[0], ok[0]);
			const size_t out2 = nslot > 1 ? out_slot(sO, v ? a : 0, ob[1], ok[1]) : NO_SLOT;
			const NearSums off = slot >= 0 ? s_offs[slot] : zero_sums();
			const bool unconv = v && fin[a] != 1;
			if (!point_epilogue_warp<MIXED>(F, sO, v, z, leaf, slot >= 0, off, out, out2, cphi, sphi, &s_maxerr, unconv))
				s_nan_err = 1;
			if (!v) continue;
			if (unconv) atomicAdd(&s_unconv, 1ull);
			if (initial)
			{
				long long cb = sR.cont_base;
				sO.cont_master[cb + a] = z;
				sO.cont_master[cb + R + a] = z;
				if constexpr (MIXED)
				{
					float4 h = split_hilo(z);
					sO.cont_snap32[cb + a] = h;
					sO.cont_snap32[cb + R + a] = h;
				}
				else
				{
					sO.cont_snap64[cb + a] = z;
					sO.cont_snap64[cb + R + a] = z;
				}
			}
		}
		cluster.sync();
	}

	if (n_eval) atomicAdd(&s_upd, n_eval);
	__syncthreads();
	if (threadIdx.x == 0)
	{
		unsigned long long* st = sO.stats;
		atomicMax(&st[0], (unsigned long long)__double_as_longlong(s_maxerr));
		const unsigned long long flags = (s_nan_err ? 1ull : 0ull) | (s_nan_step ? 2ull : 0ull);
		if (flags) atomicOr(&st[1], flags);
		atomicAdd(&st[2], s_upd);
		atomicAdd(&st[3], s_terms);
		if (initial)
		{
			atomicAdd(&st[7], s_upd);
			atomicAdd(&st[8], s_terms);
		}
		atomicAdd(&st[4], s_unconv);
		atomicMax(&st[initial ? 5 : 6], (unsigned long long)sweeps_max);
	}
}

/* ---------------- per-root tracking of the continuation ----------------

The Aberth correction of a root is the sum over the poles of f (the stars,
double poles, and the origin for exact discs) minus the sum over the other
roots.  Across the continuation each root starts a phi step next to the zero
it tracks, so the far terms of both sums only rescale a step that is already
a Newton step to ~1e-6; only the nearby poles change where a step from a
nearby start lands.  The tracker therefore keeps the pole terms of the leaf's
near stars (at most 32, the stars the evaluation of f visits anyway) and
drops the O(R + N) sums: each root walks its own row with no barrier and no
dependence on the other roots.

  * predictor: the polynomial through the last TRACK_HIST accepted positions
    (track_predict; the secant after sub-steps);
  * corrector: z <- z - f / (f' + f S_near) until the step is below
    1e-9 theta_star (the reference's test, include/ccf_functions.cuh:385);
    a step that does not shrink by TRACK_CONTRACT, a non-finite step or
    TRACK_ITERS iterations without convergence halve the phi sub-step and
    restart from the last accepted position;
  * check: every final root of a column is entered into that column's hash
    table of 2^-20 theta_star cells (track_check_kernel, after the launch), so
    two roots that converged to one zero are seen (the global repulsion of
    the full Aberth step is what keeps the reference's roots apart).  A row
    with such a pair, a root lost after the sub-step and evaluation limits,
    or a non-finite 1/mu bound is tracked again from its branch-centre roots
    with sub-steps of 1/TRACK_FINE_SUB of a step, and a row failing that too
    is run by the full-sum continuation (solve_kernel), so every row written
    is either a verified tracked row or the reference's scheme.  Rows whose
    results are kept report their statistics through collect_rerun_kernel;
    re-run rows through the full-sum kernel. */

constexpr int TNT = 128;                 /* threads per CTA of the tracker */
constexpr int TSUB = TRACK_TSUB;         /* one phi step in sub-step units */
constexpr int TRACK_ITERS = 6;           /* corrector iterations before the sub-step is halved */
constexpr double TRACK_CONTRACT = 0.5;   /* each corrector step after the first must halve */
constexpr double TRACK_CONTRACT_FINEST = 0.9;   /* ... or shrink by this at the finest sub-step */
constexpr double TRACK_STUCK = 1e-2;            /* theta_star: a root whose corrector stalls at the finest
                                                   sub-step with steps below this is kept, as unconverged
                                                   (the full Aberth step leaves such roots unconverged
                                                   too: pairs of nearly coincident zeros); larger steps
                                                   are a lost root and send the row to the re-run */
constexpr double TRACK_FS_REFINE = 1e-9;        /* bound on |f| above which a converged root takes one more step */
constexpr int TABLE_PROBES = 1024;       /* linear-probe bound of the column tables (load <= 1/2: the
                                            longest cluster of a table of 1e5 slots is ~60) */
constexpr double CELL_PER_THETA = 1048576.0;   /* 2^20 cells per theta_star */

/* 2 sum_i 1/(z - z_i) over the near stars of the leaf; zero off the root box.
   FP32 on the leaf-relative split positions in mixed precision (it only
   scales the step), FP64 otherwise. */
template <bool MIXED>
CCF_D double2 near_pole_sum(const FieldView& F, int leaf, double2 z)
{
	if (leaf < 0) return make_double2(0, 0);
	const int n = F.leaf_near_count[leaf];
	const double2 c = F.leaf_center[leaf];
	const double rx = z.x - c.x, ry = z.y - c.y;
	if constexpr (MIXED)
	{
		const float hx = (float)rx, hy = (float)ry;
		const float lx = (float)(rx - (double)hx), ly = (float)(ry - (double)hy);
		const float4* P = F.leaf_near_df + (size_t)leaf * MAX_NEAR;
		float ax = 0.f, ay = 0.f;
		for (int i = 0; i < n; i++)
		{
			const float4 s = P[i];
			const float dx = (hx - s.x) + (lx - s.z);
			const float dy = (hy - s.y) + (ly - s.w);
			const float r = rcp32(fmaf(dx, dx, fmaf(dy, dy, 1e-30f)));
			ax = fmaf(dx, r, ax);
			ay = fmaf(dy, r, ay);
		}
		return make_double2(2.0 * ax, -2.0 * ay);
	}
	else
	{
		const NearStar* P = F.leaf_near + (size_t)leaf * MAX_NEAR;
		double ax = 0, ay = 0;
		for (int i = 0; i < n; i++)
		{
			const NearStar s = P[i];
			const double dx = z.x - s.x, dy = z.y - s.y;
			const double r = rcp64(fma(dx, dx, fma(dy, dy, 1e-300)));
			ax = fma(dx, r, ax);
			ay = fma(dy, r, ay);
		}
		return make_double2(2 * ax, -2 * ay);
	}
}

/* 64-bit key of the cell of z (never 0, the empty slot); the mixing is the
   splitmix64 finaliser */
CCF_D unsigned long long cell_key(double2 z, double inv_cell)
{
	const long long qx = __double2ll_rn(z.x * inv_cell), qy = __double2ll_rn(z.y * inv_cell);
	unsigned long long h = (unsigned long long)qx * 0x9E3779B97F4A7C15ull ^ ((unsigned long long)qy + 0x632BE59BD9B4E019ull);
	h ^= h >> 30;
	h *= 0xBF58476D1CE4E5B9ull;
	h ^= h >> 27;
	h *= 0x94D049BB133111EBull;
	h ^= h >> 31;
	return h | 1ull;
}

/* enter key into an open-addressing table of `slots` entries; returns
   TRACK_DUPLICATE when the key is already there */
CCF_D unsigned long long table_insert(unsigned long long* tab, unsigned long long slots, unsigned long long key)
{
	unsigned long long s = (key >> 1) % slots;
	for (int p = 0; p < TABLE_PROBES; p++)
	{
		const unsigned long long old = atomicCAS(tab + s, 0ull, key);
		if (old == 0ull) return 0;
		if (old == key) return TRACK_DUPLICATE;
		s = s + 1 == slots ? 0 : s + 1;
	}
	return TRACK_TABLE_FULL;
}

/* Predictor of the continuation: the polynomial through the last accepted
   positions of the root (newest first, hz[k * TNT], k < hn <= TRACK_HIST),
   extrapolated to sub-step position t.  When the history is a run of whole
   phi steps and t is the next one, the extrapolation of order hn has the
   binomial weights (5, -10, 10, -5, 1 for five points): along the smooth
   paths of the critical curves its error is below 1e-9 theta_star for most
   roots, so they converge at the first evaluation.  After sub-steps (uneven
   history) it falls back to the secant through the two newest points. */
constexpr int TRACK_HIST = 5;
__constant__ double c_extrap_w[TRACK_HIST][TRACK_HIST] = {
	{1, 0, 0, 0, 0}, {2, -1, 0, 0, 0}, {3, -3, 1, 0, 0}, {4, -6, 4, -1, 0}, {5, -10, 10, -5, 1}};

CCF_D double2 track_predict(const double2* hz, const int* ht, int hn, int t)
{
	bool uniform = t - ht[0] == TSUB;
	for (int k = 0; k + 1 < hn; k++) uniform = uniform && ht[k * TNT] - ht[(k + 1) * TNT] == TSUB;
	const double2 z1 = hz[0];
	if (uniform && hn > 1)
	{
		double x = 0, y = 0;
		for (int k = 0; k < hn; k++)
		{
			const double2 q = hz[k * TNT];
			const double wk = c_extrap_w[hn - 1][k];
			x = fma(wk, q.x, x);
			y = fma(wk, q.y, y);
		}
		return make_double2(x, y);
	}
	if (hn < 2) return z1;
	const double2 z0 = hz[TNT];
	const double w = (double)(t - ht[0]) / (double)(ht[0] - ht[TNT]);
	return make_double2(z1.x + w * (z1.x - z0.x), z1.y + w * (z1.y - z0.y));
}

/* phase at sub-step position t of a row; integer steps use row_phi */
CCF_D double track_phi(int c, int nb, int nphi, int side, int t)
{
	if (t % TSUB == 0) return row_phi(c, nb, nphi, side, t / TSUB);
	const double phi0 = PI / nb + c * 2 * PI / nb;
	const double d = 2 * PI / nphi * ((double)t / TSUB);
	return side == 0 ? phi0 - d : phi0 + d;
}

/* Direct star sums of the off-field points of a warp (lanes with need set) in
   double-float on the FP32 pipe: for one such point at a time every lane
   takes every 32nd star of the split star arrays, and the partial sums meet
   by shuffles.  s1 when NEED1; s3 (FP32 accuracy, for f') when NEED3.  All
   32 lanes must call it. */
template <bool NEED1, bool NEED3>
CCF_D void offfield_sums_warp_df(const FieldView& F, bool need, double2 z, NearSums& out)
{
	const unsigned full = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	unsigned m = __ballot_sync(full, need);
	while (m)
	{
		const int src = __ffs(m) - 1;
		m &= m - 1;
		const dfc zd = dfc_from(make_double2(__shfl_sync(full, z.x, src), __shfl_sync(full, z.y, src)));
		SumsDF a;
		a.s1 = {{0.f, 0.f}, {0.f, 0.f}};
		a.s2 = a.s1;
		dfc s3 = a.s1;
		float2 s3f = make_float2(0.f, 0.f);
		for (int i = lane; i < F.num_stars; i += 32)
			star_term_df<NEED1, false>(a, s3, s3f, zd, F.star_df[i], F.star_mass_df[i]);
		dfl w[4] = {a.s1.re, a.s1.im, a.s2.re, a.s2.im};
#pragma unroll
		for (int c = NEED1 ? 0 : 2; c < 4; c++)
		{
			for (int o = 16; o > 0; o >>= 1)
			{
				const dfl u = {__shfl_xor_sync(full, w[c].hi, o), __shfl_xor_sync(full, w[c].lo, o)};
				w[c] = df_add(w[c], u);
			}
		}
		if (NEED3)
		{
			for (int o = 16; o > 0; o >>= 1)
			{
				s3f.x += __shfl_xor_sync(full, s3f.x, o);
				s3f.y += __shfl_xor_sync(full, s3f.y, o);
			}
		}
		if (lane == src)
		{
			out.s1 = NEED1 ? make_double2(df_to_double(w[0]), df_to_double(w[1])) : make_double2(0, 0);
			out.s2 = make_double2(df_to_double(w[2]), df_to_double(w[3]));
			out.s3 = NEED3 ? make_double2(s3f.x, s3f.y) : make_double2(0, 0);
		}
	}
}

/* The FP64 smooth-mass series of the rectangular Taylor form at a point
   outside the corner circle -- d alpha / d zbar and d2 alpha / d zbar2 in
   u = (zbar / c)^2, alpha in zbar (smooth_dzbar, smooth_d2zbar,
   smooth_alpha) -- evaluated by the 32 lanes together for one point: lane l
   forms the terms l, l + 32, ... of each series from its powers u^l and
   zbar^l (binary powering), and the partial sums meet by shuffles.  One
   point's three series cost ~140 FP64 warp instructions in chains of ~20,
   where one lane's Horner passes take ~460 in chains of ~115.  All 32 lanes
   call it with the same z. */
struct SmoothSeries
{
	double2 ds, d2s, alpha;
};

__device__ __noinline__ SmoothSeries smooth_series_warp(const FieldView& F, double2 z)
{
	const unsigned full = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	const double2 zb = cconj(z);
	const double2 r = cmul(zb, F.inv_corner);
	const double2 u = cmul(r, r);
	double2 ul = make_double2(1, 0), zl = make_double2(1, 0), up = u, zp = zb;
	for (int b = 0; b < 5; b++)
	{
		if ((lane >> b) & 1)
		{
			ul = cmul(ul, up);
			zl = cmul(zl, zp);
		}
		up = cmul(up, up);
		zp = cmul(zp, zp);
	}
	double2 p1 = make_double2(0, 0), p2 = p1, pa = p1;
	for (int m = lane; m < F.smooth_m; m += 32)
	{
		p1 = cadd(p1, cmul(F.smooth_d1[m], ul));
		p2 = cadd(p2, cmul(F.smooth_d2[m], ul));
		ul = cmul(ul, up);
	}
	const int n = F.taylor_smooth + 1;
	for (int i = lane; i <= n; i += 32)
	{
		pa = cadd(pa, cmul(F.smooth_a[i], zl));
		zl = cmul(zl, zp);
	}
	for (int o = 16; o > 0; o >>= 1)
	{
		p1.x += __shfl_xor_sync(full, p1.x, o);
		p1.y += __shfl_xor_sync(full, p1.y, o);
		p2.x += __shfl_xor_sync(full, p2.x, o);
		p2.y += __shfl_xor_sync(full, p2.y, o);
		pa.x += __shfl_xor_sync(full, pa.x, o);
		pa.y += __shfl_xor_sync(full, pa.y, o);
	}
	SmoothSeries out;
	out.ds = cmul(p1, u);
	out.ds.x += F.smooth_k1;
	out.d2s = cmul(p2, cmul(zb, F.inv_corner2));
	out.alpha = cmul(pa, make_double2(0, -F.kappa_star / PI));
	out.alpha.x -= F.kappa_star * 2 * (F.corner.x + z.x);
	return out;
}

/* The iteration quantities of the tracker (TrackEval) for the warp's lanes
   with off set, which lie outside the root box: direct double-float sums over
   every star, then f, f', the step and the whole lens map (wmode 2) in FP64
   (far from the field the smooth-mass Taylor terms leave the FP32 range).
   Kept out of line, as the rare path of the iteration.  All 32 lanes must
   call it. */
__device__ __noinline__ TrackEval track_offfield(const FieldView& F, bool off, double2 z, double cphi, double sphi,
	bool disc_exact, float wtol2)
{
	const unsigned full = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	NearSums ns = zero_sums();
	offfield_sums_warp_df<true, true>(F, off, z, ns);
	/* the Taylor form's series outside the corner circle, warp-wide per point */
	const bool series = F.rectangular && F.approx && F.smooth_m > 0 && !smooth_df_ok(F, z);
	SmoothSeries sm;
	sm.ds = sm.d2s = sm.alpha = make_double2(0, 0);
	unsigned pend = __ballot_sync(full, off && series);
	while (pend)
	{
		const int src = __ffs(pend) - 1;
		pend &= pend - 1;
		const SmoothSeries t = smooth_series_warp(F, make_double2(__shfl_sync(full, z.x, src), __shfl_sync(full, z.y, src)));
		if (lane == src) sm = t;
	}
	TrackEval r;
	r.step = make_float2(0.f, 0.f);
	r.as2 = 0;
	r.fz = make_float2(0.f, 0.f);
	r.af = 0;
	r.wpart = {{0.f, 0.f}, {0.f, 0.f}};
	r.wmode = 2;
	if (!off) return r;
	/* f as eval_f_df and w as eval_point_df off the root box, with the
	   smooth-mass d alpha / d zbar series evaluated once */
	const double2 ds = series ? sm.ds : smooth_dzbar_any(F, z);
	const double a = 1 - F.kappa_tot - smooth_dz(F, z);
	const double2 f = make_double2(F.shear + F.theta2 * ns.s2.x - ds.x - a * cphi, F.theta2 * ns.s2.y + ds.y + a * sphi);
	const double2 df = series ? make_double2(-2 * F.theta2 * ns.s3.x - sm.d2s.x, -2 * F.theta2 * ns.s3.y + sm.d2s.y)
	                          : eval_df_mixed(F, -1, z, ns.s3);
	double2 S = make_double2(0, 0);
	if (disc_exact)
	{
		const double2 iz = cinv(z);
		S = make_double2(2 * iz.x, 2 * iz.y);
	}
	const double2 st = cdiv(f, cadd(df, cmul(f, S)));
	r.step = make_float2((float)st.x, (float)st.y);
	const double as2 = st.x * st.x + st.y * st.y;
	r.as2 = as2 < 3e38 ? (float)as2 : INFINITY;   /* a step beyond the FP32 range fails */
	r.fz = make_float2((float)f.x, (float)f.y);
	const double2 fs = cmul(df, make_double2(r.step.x, r.step.y));
	r.af = __double2float_ru(hypot(f.x - fs.x, f.y - fs.y) +
		7.2e-15 * (F.theta2 * hypot(ns.s2.x, ns.s2.y) + hypot(ds.x, ds.y) + 1 + F.shear) +
		1.2e-16 * hypot(z.x, z.y) * hypot(df.x, df.y));
	/* the lens map only where the point can be final: a step below the
	   tolerance, or a stalled root kept as it is */
	if (r.as2 < wtol2)
	{
		const double2 as = series ? sm.alpha : smooth_alpha_any(F, z);
		const double2 w = make_double2((1 - F.kappa_tot) * z.x + F.shear * z.x - F.theta2 * ns.s1.x - as.x,
			(1 - F.kappa_tot) * z.y - F.shear * z.y + F.theta2 * ns.s1.y - as.y);
		r.wpart = dfc_from(w);
	}
	return r;
}

/* Is z inside the box of `leaf`?  rel = z - leaf centre. */
CCF_D bool in_leaf_box(const FieldView& F, int leaf, double2 z, double2& rel)
{
	const double2 c = F.leaf_center[leaf];
	rel = make_double2(z.x - c.x, z.y - c.y);
	const double ih = F.leaf_inv_half[leaf];
	return fabs(rel.x) * ih <= 1.0 && fabs(rel.y) * ih <= 1.0;
}

CCF_D unsigned long long warp_sum_u64(unsigned long long v)
{
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

/* the row of a work item: the last row whose first item is <= item */
CCF_D int item_row(const TrackArgs& T, int item)
{
	int lo = 0, hi = T.num_rows - 1;
	while (lo < hi)
	{
		const int mid = (lo + hi + 1) >> 1;
		if (T.item_start[mid] <= item) lo = mid;
		else hi = mid - 1;
	}
	return lo;
}

/* Roots that start outside the root box evaluate f by direct sums over
   every star, which the warp computes together, one such point at a time.  In
   a warp of 32 tracked roots a few of them would multiply the cost of every
   iteration of the other 31 and make their item the longest of the launch,
   so each of these roots is tracked alone by a warp of its own (its lane 0;
   the other lanes only help with the sums) and is left out of its item.
   This kernel lists them (in no particular order: a root's results do not
   depend on when or where it runs). */
__global__ void track_mark_kernel(const TrackArgs T)
{
	const int item = blockIdx.x * blockDim.x + threadIdx.x;
	if (item >= T.num_items) return;
	const int row = item_row(T, item);
	const RowDesc rd = T.rows[row];
	const FieldView* F = T.fields + rd.field;
	const int R = F->num_roots;
	const double2 c = F->node_center[0];
	const double h = F->node_half[0];
	const int a0 = (item - T.item_start[row]) * 32;
	for (int a = a0; a < min(a0 + 32, R); a++)
	{
		const double2 z = T.master[rd.base + a];
		const bool off = fabs(z.x - c.x) > h || fabs(z.y - c.y) > h;
		T.is_solo[rd.base + a] = off ? 1 : 0;
		if (off) T.solo[atomicAdd(T.num_solo, 1)] = make_int2(row, a);
	}
}

/* cos, sin of sub-step position t of row (c, side): the field's phase table
   for whole steps, else computed */
CCF_D void track_phase(const FieldOut& O, int c, int side, int t, double& cp, double& sp, dfl& cpd, dfl& spd)
{
	if (t % TSUB == 0)
	{
		const PhaseEntry e = O.phase[row_global_step(O.nb, O.half, c, side, t / TSUB)];
		cp = e.cs.x;
		sp = e.cs.y;
		cpd = {e.cs_df.x, e.cs_df.z};
		spd = {e.cs_df.y, e.cs_df.w};
		return;
	}
	sincos(track_phi(c, O.nb, O.nphi, side, t), &sp, &cp);
	cpd = df_from_double(cp);
	spd = df_from_double(sp);
}

/* Phase of every whole step of a field's phi grid: global step P is the
   phase row_phi gives for the branch centre nearest to it, so that with every
   centre solved the tracker sees the same phases as the full-sum solver. */
__global__ void phase_table_kernel(int nb, int nphi, PhaseEntry* out)
{
	const int P = blockIdx.x * blockDim.x + threadIdx.x;
	if (P >= nphi) return;
	const int period = nphi / nb, half = period / 2;
	int c = (P + half) / period;
	int u = P - c * period;            /* in [-half, half) */
	c %= nb;
	double sp, cp;
	sincos(row_phi(c, nb, nphi, u < 0 ? 0 : 1, u < 0 ? -u : u), &sp, &cp);
	const dfl cd = df_from_double(cp), sd = df_from_double(sp);
	PhaseEntry e;
	e.cs = make_double2(cp, sp);
	e.cs_df = make_float4(cd.hi, sd.hi, cd.lo, sd.lo);
	out[P] = e;
}

cudaError_t launch_phase_table(cudaStream_t s, int nb, int nphi, PhaseEntry* out)
{
	if (nphi <= 0) return cudaSuccess;
	phase_table_kernel<<<(nphi + 127) / 128, 128, 0, s>>>(nb, nphi, out);
	return cudaGetLastError();
}

/* A work item is 32 consecutive roots of one row, one warp; the rows of an
   item come from the prefix item_start[row].  Every warp takes items from a
   global counter until none are left, so a slow item delays only its own
   warp and no CTA waits at a barrier for its slowest warp.

   Each lane walks its own root through the phi steps of the row: one
   evaluation per iteration of the warp's loop, whatever step and sub-step
   the lane is at, so a lane that converges in one evaluation does not wait
   for a neighbour that needs three.  In mixed precision an evaluation
   carries everything the outputs need (TrackEval): a lane that converges
   writes its root, 1/mu bound and caustic at once, first-order corrected to
   the stepped root (the step is below 1e-9 theta_star; the lens map has
   dw/dz = a, dw/dzbar = conj(f + a e^{-i phi}), and f is holomorphic, so
   the remainders are O(step^2)).  The FP64 solver and the length scales use
   the direct evaluation of the outputs (a warp-wide call).  Every lane of the
   warp stays in the loop to the end: the evaluation off the root box and
   the direct epilogue are warp-wide calls. */
template <bool MIXED>
__global__ void __launch_bounds__(TNT, 3) track_kernel(const TrackArgs T)
{
	__shared__ FieldView sF[TNT / 32];
	__shared__ FieldOut sO[TNT / 32];
	__shared__ RowDesc sR[TNT / 32];
	__shared__ TrackConst sK[TNT / 32];
	__shared__ double s_maxerr[TNT / 32];
	__shared__ double2 s_hz[TRACK_HIST * TNT];   /* accepted positions of each lane's root, newest first */
	__shared__ int s_ht[TRACK_HIST * TNT];
	const unsigned full = 0xffffffffu;
	const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
	double2* const hz = s_hz + threadIdx.x;
	int* const ht = s_ht + threadIdx.x;

	while (true)
	{
		/* the solo roots first, then the items in order */
		int item = 0, solo_root = -1, row = 0;
		if (lane == 0)
		{
			const int q = T.items_per_row > 0 ? 0 : atomicAdd(&T.counter[0], 1);
			if (T.items_per_row == 0 && q < *T.num_solo)
			{
				const int2 sr = T.solo[q];
				row = sr.x;
				solo_root = sr.y;
			}
			else
			{
				item = atomicAdd(&T.counter[1], 1);
			}
		}
		item = __shfl_sync(full, item, 0);
		solo_root = __shfl_sync(full, solo_root, 0);
		if (T.items_per_row > 0)
		{
			if (item >= *T.num_rows_dev * T.items_per_row) break;
			row = item / T.items_per_row;
		}
		else if (solo_root < 0)
		{
			if (item >= T.num_items) break;
			/* the queue's order of the items (track_item_order_kernel) */
			if (T.item_order) item = T.item_order[item];
			row = item_row(T, item);
		}
		row = __shfl_sync(full, row, 0);
		__syncwarp();
		if (lane == 0)
		{
			sR[w] = T.rows[row];
			sF[w] = T.fields[sR[w].field];
			sO[w] = T.outs[sR[w].field];
			sK[w] = track_const(sF[w]);
			s_maxerr[w] = 0;
		}
		__syncwarp();
		const FieldView& F = sF[w];
		const FieldOut& O = sO[w];
		const RowDesc& RD = sR[w];
		const TrackConst& K = sK[w];
		const int R = F.num_roots;
		const int chunk = T.items_per_row > 0 ? item - row * T.items_per_row : item - T.item_start[row];
		const int a = solo_root >= 0 ? solo_root : chunk * 32 + lane;
		const bool valid = solo_root >= 0 ? lane == 0 : (a < R && (T.items_per_row > 0 || !T.is_solo[RD.base + a]));
		const int max_sub = T.max_sub;
		const int c = RD.branch, side = RD.side, nb = O.nb, nphi = O.nphi;
		const int j0 = O.step_first, j1 = RD.steps;
		const int cap = O.max_iters_step;
		const double tol = STEP_TOL * F.theta;
		/* the corrector's decisions compare squared step sizes, in FP32 when
		   the step itself is FP32 */
		typedef typename std::conditional<MIXED, float, double>::type real;
		const real tol2 = (real)(tol * tol);
		const real stuck2 = (real)(TRACK_STUCK * TRACK_STUCK * F.theta * F.theta);
		const bool disc_exact = !F.rectangular && !F.approx;
		const double inv_cell = CELL_PER_THETA / F.theta;
		const unsigned long long slots = 2ull * (unsigned long long)R;
		const bool direct_out = !MIXED || O.mu != nullptr;
		unsigned long long lane_maxerr = 0;   /* bits of the lane's largest 1/mu bound (non-negative) */

		double2 z1 = valid ? T.master[RD.base + a] : make_double2(0, 0);
		int t1 = (j0 - 1) * TSUB;
		hz[0] = z1;
		ht[0] = t1;
		int hn = 1;
		int leaf = -1;
		unsigned flags = 0;
		unsigned long long nev = 0, nhalf = 0;
		int maxev = 0;

		int j = j0;
		bool act = valid;
		int tt = min(t1 + max_sub, j * TSUB);
		double2 z = z1;
		double cp = 0, sp = 0;
		dfl cpd = {0.f, 0.f}, spd = {0.f, 0.f};
		track_phase(O, c, side, tt, cp, sp, cpd, spd);
		int it = 0, evs = 0;
		real prev2 = 0;
		bool lost = !valid;
		bool refine = false;
		unsigned unconv = 0;
		/* corrector iterations per (sub-)step target: the sweep cap of the
		   step, at most TRACK_ITERS (4 TRACK_ITERS at the finest sub-step) */
		const int iters = min(TRACK_ITERS, cap), iters_finest = min(4 * TRACK_ITERS, cap);

		while (__any_sync(full, act))
		{
			/* the leaf of z: the cached one while z stays in its box */
			double2 rel = make_double2(0, 0);
			if (act && !(leaf >= 0 && in_leaf_box(F, leaf, z, rel)))
			{
				leaf = find_leaf(F, z);
				if (leaf >= 0) in_leaf_box(F, leaf, z, rel);
			}
			const bool off = act && leaf < 0;
			double2 step = make_double2(0, 0);
			real as2 = 0;
			TrackEval e;
			e.step = make_float2(0.f, 0.f);
			e.as2 = 0;
			e.fz = make_float2(0.f, 0.f);
			e.af = 0;
			e.wpart = {{0.f, 0.f}, {0.f, 0.f}};
			e.wmode = 2;
			if constexpr (MIXED)
			{
				if (act && leaf >= 0) e = eval_track_df(F, K, leaf, z, rel, cpd, spd, disc_exact);
				if (__any_sync(full, off))
				{
					const TrackEval o = track_offfield(F, off, z, cp, sp, disc_exact, (float)stuck2);
					if (off) e = o;
				}
				step = make_double2((double)e.step.x, (double)e.step.y);
				as2 = e.as2;
			}
			else
			{
				const FdF g = eval_fdf_warp<false>(F, act, z, leaf, false, zero_sums(), cp, sp);
				if (act)
				{
					double2 S = near_pole_sum<false>(F, leaf, z);
					if (disc_exact)
					{
						const double2 iz = cinv(z);
						S.x += 2 * iz.x;
						S.y += 2 * iz.y;
					}
					step = cdiv(g.f, cadd(g.df, cmul(g.f, S)));
					as2 = step.x * step.x + step.y * step.y;
				}
			}

			/* the lane's decision; an output step that converged is written
			   here (mixed precision) or by the direct epilogue below */
			bool emit = false, stuck = false;
			double2 zf = make_double2(0, 0);
			size_t out = 0, out2 = NO_SLOT;
			double ecp = 0, esp = 0;
			if (act)
			{
				nev++;
				evs++;
				/* at the finest sub-step the corrector may take linear steps (a
				   pair of close zeros) as long as they keep shrinking */
				const bool finest = tt - t1 <= 1;
				const real contract = (real)(finest ? TRACK_CONTRACT_FINEST : TRACK_CONTRACT);
				bool conv = false, fail = !isfinite(as2);
				if (!fail && it > 0 && as2 >= tol2 && as2 > contract * contract * prev2) fail = true;
				if (!fail)
				{
					it++;
					prev2 = as2;
					if (as2 < tol2)
					{
						conv = true;
						/* a stiff root (large f' s, near a star): one more step from
						   the stepped root, so that the 1/mu bound comes from an
						   f evaluated there rather than from the first-order term */
						if (!refine && !direct_out && tt == j * TSUB && e.af > TRACK_FS_REFINE)
						{
							conv = false;
							refine = true;
						}
					}
					else if (it >= (finest ? iters_finest : iters)) fail = true;
				}
				if (!fail) z = csub(z, step);
				if (fail && finest && isfinite(as2) && as2 < stuck2)
				{
					/* the corrector stalls next to a zero (nearly coincident zeros,
					   or neighbouring leaf expansions meeting with a small jump in
					   f), as the full Aberth step does there: keep the position as
					   this target's root and count it unconverged, as the reference
					   counts a root that reaches its sweep cap */
					fail = false;
					conv = true;
					if (tt == j * TSUB)
					{
						unconv++;
						stuck = true;
					}
				}
				int tn = tt;
				if (conv)
				{
					const int dist = tt - t1;
					for (int k = min(hn, TRACK_HIST - 1); k > 0; k--)
					{
						hz[k * TNT] = hz[(k - 1) * TNT];
						ht[k * TNT] = ht[(k - 1) * TNT];
					}
					hn = min(hn + 1, TRACK_HIST);
					z1 = z;
					t1 = tt;
					hz[0] = z1;
					ht[0] = t1;
					refine = false;
					if (tt == j * TSUB)
					{
						emit = true;
						zf = z;
						ecp = cp;
						esp = sp;
						int ob[2], ok[2];
						const int nslot = row_slots(nb, O.half, O.seg, c, side, j, ob, ok);
						out = out_slot(O, a, ob[0], ok[0]);
						if (nslot > 1) out2 = out_slot(O, a, ob[1], ok[1]);
						if constexpr (MIXED)
						{
							if (!direct_out)
							{
								/* the lens map at the evaluated point ze, corrected to zf = ze - s:
								   w(zf) = w(ze) - a s - (conj(f) + a e^{i phi}) conj(s).  With
								   |s| below 1e-9 theta_star the correction and the linear terms'
								   share a s are FP32; the rest sums in FP64 at zf */
								const float sx = e.step.x, sy = e.step.y;
								double av = 0;
								float avf = K.a.hi;
								if (!F.approx)
								{
									av = 1 - F.kappa_tot - smooth_dz(F, make_double2(zf.x + step.x, zf.y + step.y));
									avf = (float)av;
								}
								double wx, wy;
								float lx = 0.f, ly = 0.f;   /* the linear terms' coefficients of s */
								if (e.wmode == 2)
								{
									wx = df_to_double(e.wpart.re);
									wy = df_to_double(e.wpart.im);
								}
								else if (e.wmode == 1)
								{
									wx = fma(K.w1x, zf.x, (double)e.wpart.re.hi) + ((double)e.wpart.re.lo + K.wc1);
									wy = fma(K.w1y, zf.y, (double)e.wpart.im.hi) + (double)e.wpart.im.lo;
									lx = (float)K.w1x;
									ly = (float)K.w1y;
								}
								else
								{
									const double2 ze = make_double2(zf.x + step.x, zf.y + step.y);
									const double2 wp = dfc_to(e.wpart);
									const double2 sa = smooth_alpha(F, ze);
									wx = (1 - F.kappa_tot + F.shear) * ze.x + wp.x - sa.x;
									wy = (1 - F.kappa_tot - F.shear) * ze.y + wp.y - sa.y;
								}
								const float gx = e.fz.x + avf * cpd.hi, gy = -e.fz.y + avf * spd.hi;
								const float cx = lx * sx - (avf * sx + gx * sx + gy * sy);
								const float cy = ly * sy - (avf * sy - gx * sy + gy * sx);
								const double2 wv = make_double2(wx + (double)cx, wy + (double)cy);
								/* max(|af (af + 2 a)|, |af (af - 2 a)|) = af (af + 2 |a|), rounded up */
								const float aabs = F.approx ? K.aabs : __double2float_ru(fabs(av));
								const float af = e.af;
								const double err = (double)__fmul_ru(af, __fadd_ru(af, __fmul_ru(2.f, aabs)));
								/* a stalled root is marked for the FP64 polish (polish.cu) */
								const double stored = stuck ? unconverged_mark(err) : err;
								if (out != NO_SLOT)
								{
									O.ccs[out] = zf;
									O.errs[out] = stored;
									if (O.caustics) O.caustics[out] = wv;
								}
								if (out2 != NO_SLOT)
								{
									O.ccs[out2] = zf;
									O.errs[out2] = stored;
									if (O.caustics) O.caustics[out2] = wv;
								}
								if (isfinite(err)) lane_maxerr = max(lane_maxerr, (unsigned long long)__double_as_longlong(err));
								else flags |= (unsigned)TRACK_NONFINITE;
							}
						}
						/* the column check: by track_check_kernel after the launch, from
						   the stored root, unless the outputs lie in host memory or the
						   window does not hold this column */
						if (O.check_inline || out == NO_OUT)
							flags |= (unsigned)table_insert(T.table + RD.cont_base + (size_t)(j - j0) * slots, slots,
								cell_key(zf, inv_cell));
						maxev = max(maxev, evs);
						evs = 0;
						j++;
						if (j > j1) act = false;
						tn = min(t1 + max_sub, j * TSUB);
					}
					else
					{
						tn = min(t1 + min(2 * dist, max_sub), j * TSUB);
					}
				}
				else if (fail)
				{
					refine = false;
					if (tt - t1 > 1)
					{
						tn = t1 + (tt - t1) / 2;
						nhalf++;
					}
					else
					{
						lost = true;
						act = false;
					}
				}
				if (act && evs >= cap * TSUB)
				{
					/* a bound on the evaluations of one phi step (sub-steps
					   included), so that the loop ends whatever the field */
					lost = true;
					act = false;
				}
				if (act && (conv || fail))
				{
					/* next target: predict, restart the corrector */
					tt = tn;
					z = track_predict(hz, ht, hn, tt);
					it = 0;
					prev2 = 0;
					track_phase(O, c, side, tt, cp, sp, cpd, spd);
				}
			}

			/* direct outputs (FP64 solver, length scales): warp-wide */
			const bool emit_direct = direct_out && emit;
			if (__any_sync(full, emit_direct))
			{
				int leafo = 0;
				if (emit_direct)
				{
					double2 r2;
					leafo = (leaf >= 0 && in_leaf_box(F, leaf, zf, r2)) ? leaf : find_leaf(F, zf);
				}
				if (!point_epilogue_warp<MIXED>(F, O, emit_direct, zf, leafo, false, zero_sums(), out, out2, ecp, esp, &s_maxerr[w],
						stuck))
					flags |= (unsigned)TRACK_NONFINITE;
			}
		}
		if (valid && lost) flags |= (unsigned)TRACK_LOST;
		for (int o = 16; o > 0; o >>= 1) lane_maxerr = max(lane_maxerr, __shfl_xor_sync(full, lane_maxerr, o));
		unconv = __reduce_add_sync(full, unconv);
		flags = __reduce_or_sync(full, flags);
		maxev = (int)__reduce_max_sync(full, (unsigned)maxev);
		nev = warp_sum_u64(nev);
		nhalf = warp_sum_u64(nhalf);
		__syncwarp();
		if (lane == 0)
		{
			unsigned long long* rs = T.row_stats + TRACK_ROW_STATS * (size_t)row;
			atomicMax(&rs[0], max(lane_maxerr, (unsigned long long)__double_as_longlong(s_maxerr[w])));
			if (flags) atomicOr(&rs[1], (unsigned long long)flags);
			atomicMax(&rs[2], (unsigned long long)maxev);
			if (unconv) atomicAdd(&rs[3], (unsigned long long)unconv);
			atomicAdd(&O.stats[2], nev);
			if (nhalf) atomicAdd(&O.stats[10], nhalf);
		}
	}
}

/* Rows the tracker flagged go to the re-run list; the others report their
   largest 1/mu bound, evaluations per step and unconverged points.  After
   the first tracking the list is for the re-tracking (counted in
   stats[12]); after the re-tracking, for the full-sum solver (stats[9],
   their flags in stats[11]). */
__global__ void collect_rerun_kernel(const TrackArgs T, RowDesc* rerun, int* count)
{
	const int r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= (T.num_rows_dev ? *T.num_rows_dev : T.num_rows)) return;
	const RowDesc row = T.rows[r];
	const unsigned long long* rs = T.row_stats + TRACK_ROW_STATS * (size_t)r;
	unsigned long long* st = T.outs[row.field].stats;
	if (rs[1])
	{
		const int q = atomicAdd(count, 1);
		rerun[q] = row;
		if (T.items_per_row > 0)
		{
			atomicAdd(&st[9], 1ull);
			atomicOr(&st[11], rs[1]);
		}
		else
		{
			atomicAdd(&st[12], 1ull);
		}
	}
	else
	{
		atomicMax(&st[0], rs[0]);
		atomicMax(&st[6], rs[2]);
		if (rs[3]) atomicAdd(&st[4], rs[3]);
	}
}

/* The queue order of the tracker's work items: by the smallest |f'| of
   their roots at the branch centre, smallest first, in TRACK_ORDER_CLASSES
   classes of |f'| theta_star (below 0.03, 0.1, 0.3, 1, 3, and the rest).
   Roots with a small |f'| move fast along the curve (dz/dphi = i a e^{-i phi}
   / f'), where the predictor misses the 1e-9 theta_star tolerance and the
   corrector takes a second evaluation at most steps; their items run
   longer.  A launch of persistent warps ends one item after its queue
   empties (on the bench field the SMs idled 20 % of the launch), so the long
   items go first and the launch ends on short ones.  The items keep their
   roots; only the order changes, and with it nothing in the results.
   Class: one warp per item, a lane per root (solo roots do not run in their
   item); order: one CTA, a stable counting sort by block scans. */
constexpr int TRACK_ORDER_CLASSES = 6;

__global__ void track_item_flag_kernel(const TrackArgs T, int* cls)
{
	const int item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int lane = threadIdx.x & 31;
	if (item >= T.num_items) return;   /* warp-uniform */
	const int row = item_row(T, item);
	const RowDesc rd = T.rows[row];
	const FieldView& F = T.fields[rd.field];
	const int a = (item - T.item_start[row]) * 32 + lane;
	int c = TRACK_ORDER_CLASSES - 1;
	if (a < F.num_roots && !T.is_solo[rd.base + a])
	{
		const double2 z = T.master[rd.base + a];
		const int leaf = find_leaf(F, z);
		if (leaf >= 0)
		{
			const float2 d = eval_df32(F, leaf, z, make_double2(0, 0));
			const float x = hypotf(d.x, d.y) * (float)F.theta;
			c = x < 0.03f ? 0 : x < 0.1f ? 1 : x < 0.3f ? 2 : x < 1.f ? 3 : x < 3.f ? 4 : 5;
		}
	}
	c = (int)__reduce_min_sync(0xffffffffu, (unsigned)c);
	if (lane == 0) cls[item] = c;
}

__global__ void __launch_bounds__(1024) track_item_order_kernel(int n, const int* cls, int* flag, int* rank, int* order)
{
	int base = 0;
	for (int c = 0; c < TRACK_ORDER_CLASSES; c++)
	{
		for (int i = threadIdx.x; i < n; i += blockDim.x) flag[i] = cls[i] == c;
		__syncthreads();
		const int cnt = block_exclusive_scan(flag, rank, n);
		for (int i = threadIdx.x; i < n; i += blockDim.x)
			if (flag[i]) order[base + rank[i]] = i;
		__syncthreads();
		base += cnt;
	}
}

cudaError_t launch_track_item_order(cudaStream_t s, const TrackArgs& a, int* work, int* order)
{
	if (a.num_items == 0) return cudaSuccess;
	track_item_flag_kernel<<<(a.num_items + 3) / 4, 128, 0, s>>>(a, work);
	track_item_order_kernel<<<1, 1024, 0, s>>>(a.num_items, work, work + a.num_items, work + 2 * (size_t)a.num_items, order);
	return cudaGetLastError();
}

cudaError_t launch_track_mark(cudaStream_t s, const TrackArgs& a)
{
	if (a.num_items == 0) return cudaSuccess;
	track_mark_kernel<<<(a.num_items + 127) / 128, 128, 0, s>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_track(cudaStream_t s, const TrackArgs& a, bool mixed)
{
	if (a.num_items == 0) return cudaSuccess;
	/* persistent warps: as many CTAs as are resident at once */
	static int per_sm[2] = {0, 0};
	int& n = per_sm[mixed ? 1 : 0];
	if (n == 0)
	{
		if (mixed) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, track_kernel<true>, TNT, 0);
		else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, track_kernel<false>, TNT, 0);
		if (n < 1) n = 1;
	}
	int dev = 0, sms = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const int blocks = std::max(1, std::min(sms * n, (a.num_items + TNT / 32 - 1) / (TNT / 32)));
	if (mixed) track_kernel<true><<<blocks, TNT, 0, s>>>(a);
	else track_kernel<false><<<blocks, TNT, 0, s>>>(a);
	return cudaGetLastError();
}

/* zeroes the column tables of the rows to re-track (a device-side list) */
__global__ void clear_tables_kernel(const TrackArgs T)
{
	const int nrows = *T.num_rows_dev;
	for (int q = blockIdx.y; q < nrows; q += gridDim.y)
	{
		const RowDesc row = T.rows[q];
		const unsigned long long n = 2ull * T.fields[row.field].num_roots * row.steps;
		unsigned long long* tab = T.table + row.cont_base;
		for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
			i += (unsigned long long)gridDim.x * blockDim.x)
			tab[i] = 0ull;
	}
}

/* The column check of a tracking launch, after it: every (row, phi step)
   column's stored roots go into that column's table of 2^-20 theta_star
   cells, and a cell taken twice (two roots of the row converged to one zero)
   flags the row, as the tracker's own insert would.  One thread per stored
   point, the steps of a root in consecutive threads (consecutive columns of
   the output layout); blockIdx.y is the row, and the blocks of a row are
   scheduled together, so the tables in use at a time stay in L2.  Points
   whose column the output window does not hold, and fields with outputs in
   host memory, were checked by the tracker itself.  A lost root leaves stale
   values in its later columns, which can only flag its own row, already
   flagged as lost. */
__global__ void track_check_kernel(const TrackArgs T)
{
	const int nrows = T.num_rows_dev ? *T.num_rows_dev : T.num_rows;
	for (int q = blockIdx.y; q < nrows; q += gridDim.y)
	{
		const RowDesc RD = T.rows[q];
		const FieldOut& O = T.outs[RD.field];
		if (O.check_inline) continue;
		const int R = T.fields[RD.field].num_roots;
		const double inv_cell = CELL_PER_THETA / T.fields[RD.field].theta;
		const int j0 = O.step_first, nsteps = RD.steps - j0 + 1;
		if (nsteps <= 0) continue;
		const int nb = O.nb, half = O.half, seg = O.seg;
		const unsigned long long slots = 2ull * (unsigned long long)R;
		const long long n = (long long)R * nsteps;
		unsigned flags = 0;
		for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		{
			const int a = (int)(i / nsteps), j = j0 + (int)(i - (long long)a * nsteps);
			int ob[2], ok[2];
			row_slots(nb, half, seg, RD.branch, RD.side, j, ob, ok);
			const size_t out = out_slot(O, a, ob[0], ok[0]);
			if (out == NO_OUT) continue;
			flags |= (unsigned)table_insert(T.table + RD.cont_base + (size_t)(j - j0) * slots, slots,
				cell_key(O.ccs[out], inv_cell));
		}
		if (flags) atomicOr(&T.row_stats[TRACK_ROW_STATS * (size_t)q + 1], (unsigned long long)flags);
	}
}

cudaError_t launch_track_check(cudaStream_t s, const TrackArgs& a, long long max_row_points)
{
	if (a.num_rows == 0 || max_row_points <= 0) return cudaSuccess;
	/* about four points per thread; a row's blocks go out together */
	const long long gx = std::min<long long>((max_row_points + 1023) / 1024, 1LL << 20);
	track_check_kernel<<<dim3((unsigned)gx, (unsigned)std::min(a.num_rows, 65535)), 256, 0, s>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_clear_tables(cudaStream_t s, const TrackArgs& a)
{
	clear_tables_kernel<<<dim3(152, 16), 256, 0, s>>>(a);
	return cudaGetLastError();
}

cudaError_t launch_collect_rerun(cudaStream_t s, const TrackArgs& a, RowDesc* rerun, int* count)
{
	if (a.num_rows == 0) return cudaSuccess;
	collect_rerun_kernel<<<(a.num_rows + 127) / 128, 128, 0, s>>>(a, rerun, count);
	return cudaGetLastError();
}

int solver_blocks_per_sm(bool mixed)
{
	int n = 0;
	if (mixed) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, solve_kernel<true>, NT, 0);
	else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, solve_kernel<false>, NT, 0);
	return n < 1 ? 1 : n;
}

cudaError_t launch_solve(cudaStream_t s, const SolveArgs& a, bool mixed, bool initial)
{
	if (a.num_rows == 0) return cudaSuccess;
	if (a.cluster < 1 || a.cluster > MAX_CLUSTER) return cudaErrorInvalidValue;
	if (a.cluster > 8)
	{
		static bool allowed[2] = {false, false};
		if (!allowed[mixed ? 1 : 0])
		{
			cudaError_t e = mixed ? cudaFuncSetAttribute(solve_kernel<true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)
			                      : cudaFuncSetAttribute(solve_kernel<false>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
			if (e != cudaSuccess) return e;
			allowed[mixed ? 1 : 0] = true;
		}
	}
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(a.num_rows * a.cluster, 1, 1);
	cfg.blockDim = dim3(NT, 1, 1);
	cfg.dynamicSmemBytes = 0;
	cfg.stream = s;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = a.cluster;
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	if (mixed) return cudaLaunchKernelEx(&cfg, solve_kernel<true>, a, initial ? 1 : 0);
	return cudaLaunchKernelEx(&cfg, solve_kernel<false>, a, initial ? 1 : 0);
}

/* pointwise evaluation of f, f', the lens map, the 1/mu bound and the
   length scale at given points (used by the checks against the oracle) */
__global__ void eval_points_kernel(const FieldView* __restrict__ Fp, int npts, const double2* __restrict__ z,
	const double* __restrict__ phi, double2* f, double2* df, double2* w, double* err, double* mu)
{
	/* every lane of a warp stays to the end: off-field sums are warp-wide */
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	const bool v = i < npts;
	const FieldView F = *Fp;
	double2 zz = v ? z[i] : make_double2(0, 0);
	double sp, cp;
	sincos(v ? phi[i] : 0.0, &sp, &cp);
	int leaf = v ? find_leaf(F, zz) : 0;
	NearSums ns = zero_sums();
	if (v && leaf >= 0) ns = leaf_sums<true, true>(F, leaf, zz);
	offfield_sums_warp<true, true>(F, v && leaf < 0, zz, ns);
	if (!v) return;
	double2 fv, dv;
	eval_f64<true>(F, leaf, zz, cp, sp, ns, fv, dv);
	if (f) f[i] = fv;
	if (df) df[i] = dv;
	PointResult pr = eval_point<true, true>(F, leaf, zz, cp, sp, ns);
	if (w) w[i] = pr.w;
	if (err) err[i] = pr.err;
	if (mu) mu[i] = pr.mu_length;
}

cudaError_t launch_eval_points(cudaStream_t s, const FieldView* F_dev, int npts, const double2* z, const double* phi,
	double2* f, double2* df, double2* w, double* err, double* mu)
{
	if (npts <= 0) return cudaSuccess;
	eval_points_kernel<<<(npts + 127) / 128, 128, 0, s>>>(F_dev, npts, z, phi, f, df, w, err, mu);
	return cudaGetLastError();
}

} /* namespace ccf */
