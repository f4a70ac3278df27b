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

namespace cg = cooperative_groups;

namespace ccf
{

constexpr int NT = 256;          /* threads per CTA */
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
		/* f in double-float on the FP32 pipe, off-field points included */
		r.f = eval_f_df(F, leaf, z, cphi, sphi, ns);
		const float2 d32 = eval_df32(F, leaf, z, ns.s3);
		r.df = make_double2(d32.x, d32.y);
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
template <bool DF>
__device__ __noinline__ bool point_epilogue_warp(const FieldView& F, const FieldOut& O, bool valid, double2 z, int leaf,
	bool have_off, NearSums off, size_t out, double cphi, double sphi, double* maxerr)
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
	O.ccs[out] = z;
	O.errs[out] = pr.err;
	if (O.caustics) O.caustics[out] = pr.w;
	if (mu) O.mu[out] = pr.mu_length;
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
	if (item >= A.num_rows) return;

	__shared__ FieldView sF;
	__shared__ FieldOut sO;
	__shared__ RowDesc sR;
	__shared__ int s_fill;
	__shared__ int s_cnt;
	__shared__ int s_pre[9];
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
	const int j1 = initial ? 0 : sO.step_last;
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
			int S = 1;
			while (S < NT / 32 && (total + TILE / S - 1) / (TILE / S) < csize) S *= 2;
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
							fin[a] = 1;
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
		const int k = initial ? sO.half : (side == 0 ? sO.half - j : sO.half + j);
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
			size_t out = ((size_t)(v ? a : 0) * nb + c) * sO.cols + k;
			const NearSums off = slot >= 0 ? s_offs[slot] : zero_sums();
			if (!point_epilogue_warp<MIXED>(F, sO, v, z, leaf, slot >= 0, off, out, cphi, sphi, &s_maxerr)) s_nan_err = 1;
			if (!v) continue;
			if (!fin[a]) atomicAdd(&s_unconv, 1ull);
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
