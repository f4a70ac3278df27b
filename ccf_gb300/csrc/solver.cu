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
    critical-curve function f is always FP64, so the converged roots are
    those of the FP64 function: the sums and f' only set the step size;
  * a root is final once its step is below 1e-9 theta_star (the reference's
    test, ccf_functions.cuh:385); sweeps stop when no root of the row is
    active or the sweep cap is reached;
  * the residual (1/mu error bound), the caustic and the length scale of
    each point are computed in the epilogue of its phi step and written
    straight into the output layout, so no transpose pass is needed.
******************************************************************************/
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

/* phase of step j of a row (include/ccf_functions.cuh:338-344) */
CCF_D double row_phi(int c, int nb, int nphi, int side, int j)
{
	double phi0 = PI / nb + c * 2 * PI / nb;
	double dphi = 2 * PI / nphi * j;
	return side == 0 ? phi0 - dphi : phi0 + dphi;
}

/* One Aberth step for the target of every lane with valid set, given its
   correction sum S; returns 0, 1 when the root became final, 2 when the step
   was not finite (the root is then frozen).  All 32 lanes of the warp must
   call it: off-field targets take their star sums from the whole warp.  Not
   inlined: the FP64 evaluation needs its registers once, not once per
   unrolled target. */
template <bool MIXED>
__device__ __noinline__ int aberth_update_warp(const FieldView& F, double2* __restrict__ master, unsigned char* __restrict__ fin,
	bool valid, int a, double2 S, bool disc_exact, double cphi, double sphi)
{
	double2 z = valid ? master[a] : make_double2(0, 0);
	int leaf = valid ? find_leaf(F, z) : 0;
	NearSums ns = zero_sums();
	if (valid && leaf >= 0) ns = leaf_sums<false, !MIXED>(F, leaf, z);
	offfield_sums_warp<false, true>(F, valid && leaf < 0, z, ns);
	if (!valid) return 0;
	if (disc_exact)
	{
		double2 iz = cinv(z);
		S.x += 2 * iz.x;
		S.y += 2 * iz.y;
	}
	double2 f, df;
	if constexpr (MIXED)
	{
		eval_f64<false>(F, leaf, z, cphi, sphi, ns, f, df);
		float2 d32 = eval_df32(F, leaf, z, ns.s3);
		df = make_double2(d32.x, d32.y);
	}
	else
	{
		eval_f64<true>(F, leaf, z, cphi, sphi, ns, f, df);
	}
	double2 den = cadd(df, cmul(f, S));
	double2 znew = csub(z, cdiv(f, den));
	if (isfinite(znew.x) && isfinite(znew.y))
	{
		double norm = hypot(znew.x - z.x, znew.y - z.y) / F.theta;
		master[a] = znew;
		if (norm < 0.000000001)
		{
			fin[a] = 1;
			return 1;
		}
		return 0;
	}
	fin[a] = 1;
	return 2;
}

/* outputs of one final root per lane: position, 1/mu bound, caustic,
   length scale.  All 32 lanes must call it (see aberth_update_warp). */
__device__ __noinline__ void point_epilogue_warp(const FieldView& F, const FieldOut& O, bool valid, double2 z, size_t out,
	double cphi, double sphi, double* maxerr, int* nan)
{
	int leaf = valid ? find_leaf(F, z) : 0;
	NearSums ns = zero_sums();
	const bool mu = O.mu != nullptr;
	if (valid && leaf >= 0) ns = mu ? leaf_sums<true, true>(F, leaf, z) : leaf_sums<true, false>(F, leaf, z);
	offfield_sums_warp<true, true>(F, valid && leaf < 0, z, ns);
	if (!valid) return;
	PointResult pr;
	if (O.caustics && mu) pr = eval_point<true, true>(F, leaf, z, cphi, sphi, ns);
	else if (O.caustics) pr = eval_point<true, false>(F, leaf, z, cphi, sphi, ns);
	else if (mu) pr = eval_point<false, true>(F, leaf, z, cphi, sphi, ns);
	else pr = eval_point<false, false>(F, leaf, z, cphi, sphi, ns);
	O.ccs[out] = z;
	O.errs[out] = pr.err;
	if (O.caustics) O.caustics[out] = pr.w;
	if (mu) O.mu[out] = pr.mu_length;
	if (isfinite(pr.err)) atomicMax((unsigned long long*)maxerr, (unsigned long long)__double_as_longlong(pr.err));
	else atomicOr(nan, 1);
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
	__shared__ int s_nan;
	__shared__ __align__(16) SrcT sbuf[2][CHUNK];

	if (threadIdx.x == 0)
	{
		sR = A.rows[item];
		sF = A.fields[sR.field];
		sO = A.outs[sR.field];
		s_upd = 0;
		s_terms = 0;
		s_unconv = 0;
		s_maxerr = 0;
		s_nan = 0;
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
	const SrcT* __restrict__ rsrc;
	const SrcT* __restrict__ ssrc;
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

			const int ntiles = (total + TILE - 1) / TILE;
			for (int tile = crank; tile < ntiles; tile += csize)
			{
				int tid_a[TPT];
				bool valid[TPT];
				SrcT zs[TPT];
				double2 totR[TPT], totS[TPT];
#pragma unroll
				for (int t = 0; t < TPT; t++)
				{
					int g = tile * TILE + t * NT + threadIdx.x;
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
					if constexpr (MIXED) zs[t] = valid[t] ? rsrc[a] : make_float4(0, 0, 0, 0);
					else zs[t] = valid[t] ? rsrc[a] : make_double2(0, 0);
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
					const SrcT* sb = sbuf[ch & 1];
					if constexpr (MIXED)
					{
						float ax[TPT], ay[TPT];
#pragma unroll
						for (int t = 0; t < TPT; t++) { ax[t] = 0.f; ay[t] = 0.f; }
#pragma unroll 4
						for (int jj = 0; jj < n; jj++)
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
						for (int jj = 0; jj < n; jj++)
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

				/* the Aberth update of each target (warp-uniform calls) */
#pragma unroll
				for (int t = 0; t < TPT; t++)
				{
					double2 S = make_double2(2 * totS[t].x - totR[t].x, 2 * totS[t].y - totR[t].y);
					if (aberth_update_warp<MIXED>(F, master, fin, valid[t], tid_a[t], S, disc_exact, cphi, sphi) == 2)
						atomicOr(&s_nan, 2);
				}
			}
			if (threadIdx.x == 0)
			{
				int mine = 0;
				for (int tile = crank; tile < ntiles; tile += csize) mine += min(TILE, total - tile * TILE);
				s_upd += mine;
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
			size_t out = ((size_t)(v ? a : 0) * nb + c) * sO.cols + k;
			point_epilogue_warp(F, sO, v, z, out, cphi, sphi, &s_maxerr, &s_nan);
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

	__syncthreads();
	if (threadIdx.x == 0)
	{
		unsigned long long* st = sO.stats;
		atomicMax(&st[0], (unsigned long long)__double_as_longlong(s_maxerr));
		if (s_nan) atomicOr(&st[1], (unsigned long long)s_nan);
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
