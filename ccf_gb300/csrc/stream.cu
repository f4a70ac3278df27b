/******************************************************************************
stream.cu -- one field solved with its outputs streamed to page-locked host
memory (ccf_params.host_outputs = 2): Engine::solve_chunked.

The outputs of a field take 40 bytes per point (16.6 GB for 20000 stars and
10240 phi steps on 128 branches).  Here they never sit on the device whole:

  * the initial Aberth solve (all solved branch centres in one launch) writes
    its centre columns into a small centre buffer (one column per branch),
    which is polished and copied out at once;
  * the continuation runs one group of solved centres at a time (the rows of
    a centre cover seg branches, half way to the next solved centre on each
    side), into one of two device chunk buffers holding the group's window
    of branches -- tracked, re-tracked, re-run and FP64-polished exactly as
    in Engine::solve, the same kernels on the group's rows;
  * a finished chunk is copied into the page-locked host arrays by 2-D copies
    (one per run of written columns, the root rows strided) on a copy stream,
    while the next group computes into the other buffer.

The results are the bits of Engine::solve's: the same rows run the same
kernels; only the rows' launch grouping differs, and a row's results do not
depend on what else its launch holds.  Device-resident outputs: the centre
buffer and the two chunk buffers (4.4 GB on the field above, each chunk 2.2
GB).  A group is as many centres (a power of two dividing their number) as
keep a chunk within CHUNK_BYTES (2 GiB; CCF_GB300_CHUNK_BYTES sets another
target, at least one centre per group).
******************************************************************************/
#include "engine.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <numeric>

namespace ccf
{

namespace
{

constexpr size_t CHUNK_BYTES = (size_t)2 << 30;

/* the chunk size target: CHUNK_BYTES, or CCF_GB300_CHUNK_BYTES (bytes) */
size_t chunk_bytes()
{
	const char* e = std::getenv("CCF_GB300_CHUNK_BYTES");
	const long long v = e ? std::atoll(e) : 0;
	return v > 0 ? (size_t)v : CHUNK_BYTES;
}

#define CCF_TRY_S(expr, what)                                   \
	do                                                          \
	{                                                           \
		cudaError_t e_ = (expr);                                \
		if (e_ != cudaSuccess) return cuda_fail_s(e_, what);    \
	} while (0)

/* a run of written slots of a chunk window: window slots [j0, j0 + n) of a
   root's row of the window, host branch b, column k of its first slot */
struct CopyRun
{
	long long j0, n;
	int b, k;
};

/* maximal runs of the mask (w_nb branches x cols, in window order); a run
   ends where the host's branch index wraps to 0 (not contiguous there) */
std::vector<CopyRun> window_runs(const std::vector<unsigned char>& mask, int w_b0, int w_nb, int cols, int nb)
{
	std::vector<CopyRun> runs;
	const long long total = (long long)w_nb * cols;
	long long j = 0;
	while (j < total)
	{
		if (!mask[j])
		{
			j++;
			continue;
		}
		const long long j0 = j;
		j++;
		while (j < total && mask[j] && !(j % cols == 0 && (w_b0 + (int)(j / cols)) % nb == 0)) j++;
		runs.push_back({j0, j - j0, (w_b0 + (int)(j0 / cols)) % nb, (int)(j0 % cols)});
	}
	return runs;
}

} /* namespace */

ccf_status Engine::solve_chunked(Field& f, int verbose)
{
	auto cuda_fail_s = [&](cudaError_t e, const char* what) { return cuda_fail(e, what); };
	cudaStream_t s = stream;
	ChunkState& C = chunk;
	const ccf_params& p = f.params;
	const bool mixed = p.precision == CCF_PRECISION_MIXED;
	const bool track = p.continuation == CCF_CONTINUATION_TRACK;
	const int R = f.d.num_roots, N = f.d.num_stars, nb = p.num_branches;
	const int cols = p.num_phi / nb + 1, half = p.num_phi / (2 * nb);
	const int seg = solved_seg(f, track), K = nb / seg;
	SolverPools& P = pools;

	if (!C.copy)
	{
		CCF_TRY_S(cudaStreamCreateWithFlags(&C.copy, cudaStreamNonBlocking), "cudaStreamCreate");
		for (cudaEvent_t* e : {&C.ready, &C.copied[0], &C.copied[1], &C.done})
			CCF_TRY_S(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "event");
	}

	/* rows: the initial solve's K centres, two continuation rows each */
	const long long ninit = (long long)K * R, ncont = 2LL * K * R;
	CCF_TRY_S(P.master_init.ensure(ninit), "cudaMalloc(roots)");
	CCF_TRY_S(P.master_cont.ensure(ncont), "cudaMalloc(roots)");
	CCF_TRY_S(P.fin_init.ensure(ninit), "cudaMalloc(roots)");
	CCF_TRY_S(P.fin_cont.ensure(ncont), "cudaMalloc(roots)");
	CCF_TRY_S(P.list_init.ensure(ninit), "cudaMalloc(roots)");
	CCF_TRY_S(P.list_cont.ensure(ncont), "cudaMalloc(roots)");
	CCF_TRY_S(P.fval_init.ensure(2 * ninit), "cudaMalloc(roots)");
	CCF_TRY_S(P.fval_cont.ensure(2 * ncont), "cudaMalloc(roots)");
	if (mixed)
	{
		CCF_TRY_S(P.snap32_init.ensure(ninit), "cudaMalloc(roots)");
		CCF_TRY_S(P.snap32_cont.ensure(ncont), "cudaMalloc(roots)");
	}
	else
	{
		CCF_TRY_S(P.snap64_init.ensure(ninit), "cudaMalloc(roots)");
		CCF_TRY_S(P.snap64_cont.ensure(ncont), "cudaMalloc(roots)");
	}
	std::vector<RowDesc> ri(K), rc(2 * K);
	for (int q = 0; q < K; q++)
	{
		RowDesc& r = ri[q];
		r.field = 0;
		r.branch = q * seg;
		r.side = -1;
		r.steps = 0;
		r.base = (long long)q * R;
		r.cont_base = (long long)(2 * q) * R;
		for (int b = 0; b < 2; b++)
		{
			RowDesc u = r;
			u.side = b;
			u.steps = seg == 1 ? half : (b == 1 ? seg * half : seg * half - 1);
			u.base = (long long)(2 * q + b) * R;
			u.cont_base = 0;   /* the column-table offset, set per group below */
			rc[2 * q + b] = u;
		}
	}

	/* groups of G centres; each group's window of branches and the columns its
	   rows write (row_slots over every step) */
	const size_t point_bytes = 16 + 8 + (p.write_caustics ? 16 : 0) + (p.write_mu_length_scales ? 8 : 0);
	int G = 1;
	const size_t budget = chunk_bytes();
	while (G < K && K % (2 * G) == 0 && (size_t)R * (2 * G * seg + 1) * cols * point_bytes <= budget) G *= 2;
	const int ngroups = K / G;
	struct Group
	{
		int w_b0 = 0, w_nb = 0;
		std::vector<CopyRun> runs;
		long long table_slots = 0;
	};
	std::vector<Group> groups(ngroups);
	int max_wnb = 0;
	long long max_slots = 0;
	for (int g = 0; g < ngroups; g++)
	{
		std::vector<unsigned char> full((size_t)nb * cols, 0);
		long long slots = 0;
		for (int q = g * G; q < (g + 1) * G; q++)
			for (int b = 0; b < 2; b++)
			{
				RowDesc& u = rc[2 * q + b];
				if (track) u.cont_base = slots;
				slots += 2LL * R * u.steps;
				for (int j = 1; j <= u.steps; j++)
				{
					int ob[2], ok[2];
					const int n = row_slots(nb, half, seg, u.branch, u.side, j, ob, ok);
					for (int t = 0; t < n; t++) full[(size_t)ob[t] * cols + ok[t]] = 1;
				}
			}
		/* the covered branches form one circular range: start after an uncovered one */
		std::vector<unsigned char> cov(nb, 0);
		int ncov = 0;
		for (int b = 0; b < nb; b++)
			for (int k = 0; k < cols; k++)
				if (full[(size_t)b * cols + k]) cov[b] = 1;
		for (int b = 0; b < nb; b++) ncov += cov[b];
		int b0 = 0;
		if (ncov < nb)
			for (int b = 0; b < nb; b++)
				if (cov[b] && !cov[(b - 1 + nb) % nb])
				{
					b0 = b;
					break;
				}
		Group& gr = groups[g];
		gr.w_b0 = b0;
		gr.w_nb = ncov;
		std::vector<unsigned char> wmask((size_t)ncov * cols, 0);
		for (int i = 0; i < ncov; i++)
		{
			const int b = (b0 + i) % nb;
			if (!cov[b])
			{
				error = "Error. A branch group's columns are not one range of branches.";
				return CCF_ERR_NUMERIC;
			}
			std::memcpy(&wmask[(size_t)i * cols], &full[(size_t)b * cols], cols);
		}
		gr.runs = window_runs(wmask, b0, ncov, cols, nb);
		gr.table_slots = slots;
		max_wnb = std::max(max_wnb, ncov);
		max_slots = std::max(max_slots, slots);
	}

	/* device buffers: centre columns (one per branch), two chunk windows */
	const size_t ctr_pts = (size_t)R * nb;
	const size_t win_pts = (size_t)R * max_wnb * cols;
	CCF_TRY_S(C.ctr_ccs.ensure(ctr_pts), "cudaMalloc(centre outputs)");
	CCF_TRY_S(C.ctr_errs.ensure(ctr_pts), "cudaMalloc(centre outputs)");
	if (p.write_caustics) CCF_TRY_S(C.ctr_caus.ensure(ctr_pts), "cudaMalloc(centre outputs)");
	if (p.write_mu_length_scales) CCF_TRY_S(C.ctr_mu.ensure(ctr_pts), "cudaMalloc(centre outputs)");
	for (int k = 0; k < std::min(2, ngroups); k++)
	{
		CCF_TRY_S(C.ccs[k].ensure(win_pts), "cudaMalloc(chunk outputs)");
		CCF_TRY_S(C.errs[k].ensure(win_pts), "cudaMalloc(chunk outputs)");
		if (p.write_caustics) CCF_TRY_S(C.caus[k].ensure(win_pts), "cudaMalloc(chunk outputs)");
		if (p.write_mu_length_scales) CCF_TRY_S(C.mu[k].ensure(win_pts), "cudaMalloc(chunk outputs)");
	}

	/* FieldOut records: [0] the initial solve's centre columns, [1 + g] group g */
	std::vector<FieldOut> outs(1 + ngroups);
	FieldOut base;
	std::memset(&base, 0, sizeof(base));
	base.nb = nb;
	base.nphi = p.num_phi;
	base.cols = cols;
	base.half = half;
	base.step_first = 1;
	base.step_last = half;
	base.max_iters_init = p.max_iters_init;
	base.max_iters_step = p.max_iters_step;
	base.seg = seg;
	if (track)
	{
		CCF_TRY_S(f.phase.ensure(p.num_phi), "cudaMalloc(phase)");
		CCF_TRY_S(launch_phase_table(s, nb, p.num_phi, f.phase.ptr), "phase_table_kernel");
		base.phase = f.phase.ptr;
	}
	base.cont_master = P.master_cont.ptr;
	base.cont_snap32 = mixed ? P.snap32_cont.ptr : nullptr;
	base.cont_snap64 = mixed ? nullptr : P.snap64_cont.ptr;
	base.stats = f.stats.ptr;
	outs[0] = base;
	outs[0].ccs = C.ctr_ccs.ptr;
	outs[0].errs = C.ctr_errs.ptr;
	outs[0].caustics = p.write_caustics ? C.ctr_caus.ptr : nullptr;
	outs[0].mu = p.write_mu_length_scales ? C.ctr_mu.ptr : nullptr;
	outs[0].w_b0 = 0;
	outs[0].w_nb = nb;
	outs[0].w_k0 = half;
	outs[0].w_cols = 1;
	for (int g = 0; g < ngroups; g++)
	{
		const int k = g & 1;
		FieldOut& o = outs[1 + g];
		o = base;
		o.ccs = C.ccs[k].ptr;
		o.errs = C.errs[k].ptr;
		o.caustics = p.write_caustics ? C.caus[k].ptr : nullptr;
		o.mu = p.write_mu_length_scales ? C.mu[k].ptr : nullptr;
		o.w_b0 = groups[g].w_b0;
		o.w_nb = groups[g].w_nb;
		o.w_k0 = 0;
		o.w_cols = cols;
	}
	const float4* hilo = mixed ? f.star_hilo.ptr : nullptr;
	CCF_TRY_S(P.views.ensure(1), "cudaMalloc(views)");
	CCF_TRY_S(C.outs.ensure(outs.size()), "cudaMalloc(outs)");
	CCF_TRY_S(P.hilo_ptrs.ensure(1), "cudaMalloc(views)");
	CCF_TRY_S(P.rows_init.ensure(ri.size()), "cudaMalloc(rows)");
	CCF_TRY_S(P.rows_cont.ensure(rc.size()), "cudaMalloc(rows)");
	CCF_TRY_S(P.error.ensure(1), "cudaMalloc(error)");
	CCF_TRY_S(cudaMemcpyAsync(P.views.ptr, &f.view, sizeof(FieldView), cudaMemcpyHostToDevice, s), "upload");
	CCF_TRY_S(cudaMemcpyAsync(C.outs.ptr, outs.data(), outs.size() * sizeof(FieldOut), cudaMemcpyHostToDevice, s), "upload");
	CCF_TRY_S(cudaMemcpyAsync(P.hilo_ptrs.ptr, &hilo, sizeof(hilo), cudaMemcpyHostToDevice, s), "upload");
	CCF_TRY_S(cudaMemcpyAsync(P.rows_init.ptr, ri.data(), ri.size() * sizeof(RowDesc), cudaMemcpyHostToDevice, s), "upload");
	CCF_TRY_S(cudaMemcpyAsync(P.rows_cont.ptr, rc.data(), rc.size() * sizeof(RowDesc), cudaMemcpyHostToDevice, s), "upload");
	CCF_TRY_S(cudaMemsetAsync(P.error.ptr, 0, sizeof(int), s), "memset");
	/* the tracker's per-group arrays, sized for the largest group */
	const int grows = 2 * G;
	std::vector<int> item_start_host((size_t)rc.size());
	int max_items = 0;
	for (int g = 0; g < ngroups; g++)
	{
		int items = 0;
		for (int r = 0; r < grows; r++)
		{
			item_start_host[(size_t)g * grows + r] = items;
			items += (R + 31) / 32;
		}
		max_items = std::max(max_items, items);
	}
	if (track)
	{
		CCF_TRY_S(P.track_table.ensure(max_slots), "cudaMalloc(tables)");
		CCF_TRY_S(P.row_stats.ensure(TRACK_ROW_STATS * grows), "cudaMalloc(rows)");
		CCF_TRY_S(P.row_stats2.ensure(TRACK_ROW_STATS * grows), "cudaMalloc(rows)");
		CCF_TRY_S(P.rows_rerun.ensure(grows), "cudaMalloc(rows)");
		CCF_TRY_S(P.rows_rerun2.ensure(grows), "cudaMalloc(rows)");
		CCF_TRY_S(P.rerun_count.ensure(6), "cudaMalloc(rows)");
		CCF_TRY_S(P.item_start.ensure(rc.size()), "cudaMalloc(rows)");
		CCF_TRY_S(P.solo.ensure((size_t)ncont + 1), "cudaMalloc(rows)");
		CCF_TRY_S(P.is_solo.ensure((size_t)ncont), "cudaMalloc(rows)");
		CCF_TRY_S(cudaMemcpyAsync(P.item_start.ptr, item_start_host.data(), rc.size() * sizeof(int), cudaMemcpyHostToDevice,
			s), "upload");
	}
	/* the polish list: room for 1 in 128 points of a chunk */
	const long long cap = std::min(1LL << 24, std::max(1LL << 16, (long long)(win_pts / 128)));
	CCF_TRY_S(P.polish_list.ensure((size_t)cap + 1), "cudaMalloc(polish)");

	launch_seed_roots(s, N, R, K, f.star_pos.ptr, f.star_mass.ptr, f.view.corner_abs, f.view.theta,
		1 - f.view.kappa_tot + f.view.kappa_star, f.view.shear, nb, seg, P.master_init.ptr,
		mixed ? P.snap32_init.ptr : nullptr, mixed ? nullptr : P.snap64_init.ptr);

	auto polish = [&](const FieldOut* outs_dev, long long npts) -> cudaError_t {
		cudaError_t e = cudaMemsetAsync(P.polish_list.ptr, 0, sizeof(unsigned long long), s);
		if (e != cudaSuccess) return e;
		PolishArgs PA;
		PA.fields = P.views.ptr;
		PA.outs = outs_dev;
		PA.num_fields = 1;
		PA.b0 = PA.nbs = PA.k0 = PA.nks = 0;
		PA.list_count = P.polish_list.ptr;
		PA.list = P.polish_list.ptr + 1;
		PA.list_cap = cap;
		return launch_polish(s, PA, npts, num_sms);
	};
	/* host arrays: the mapped page-locked buffers of the field */
	struct Arr
	{
		const void* ctr;
		const void* win[2];
		char* host;
		size_t esize;
	};
	std::vector<Arr> arrays;
	arrays.push_back({C.ctr_ccs.ptr, {C.ccs[0].ptr, C.ccs[1].ptr}, (char*)f.h_ccs.ptr, sizeof(double2)});
	arrays.push_back({C.ctr_errs.ptr, {C.errs[0].ptr, C.errs[1].ptr}, (char*)f.h_errs.ptr, sizeof(double)});
	if (p.write_caustics) arrays.push_back({C.ctr_caus.ptr, {C.caus[0].ptr, C.caus[1].ptr}, (char*)f.h_caustics.ptr, sizeof(double2)});
	if (p.write_mu_length_scales) arrays.push_back({C.ctr_mu.ptr, {C.mu[0].ptr, C.mu[1].ptr}, (char*)f.h_mu.ptr, sizeof(double)});

	/* ---------------- the initial solve: every solved centre, one launch ---------------- */
	/* slots no launch writes must read as converged: the polish scans the whole window */
	CCF_TRY_S(cudaMemsetAsync(C.ctr_errs.ptr, 0, ctr_pts * sizeof(double), s), "memset");
	CCF_TRY_S(cudaEventRecord(f.ev[3], s), "event");
	if (verbose >= 1) std::cout << "Finding initial roots...\n";
	SolveArgs A;
	std::memset(&A, 0, sizeof(A));
	A.fields = P.views.ptr;
	A.outs = C.outs.ptr;   /* record 0: the centre columns */
	A.star_hilo = P.hilo_ptrs.ptr;
	A.error = P.error.ptr;
	A.rows = P.rows_init.ptr;
	A.num_rows = K;
	{
		const int slots = num_sms * slots_per_sm;
		int cl = 1;
		while (cl < 16 && (long long)K * cl * 2 <= slots && R / (cl * 2) >= 256) cl *= 2;
		A.cluster = p.init_cluster > 0 ? p.init_cluster : cl;
		f.info.init_cluster = A.cluster;
	}
	A.master = P.master_init.ptr;
	A.snap32 = mixed ? P.snap32_init.ptr : nullptr;
	A.snap64 = mixed ? nullptr : P.snap64_init.ptr;
	A.fin = P.fin_init.ptr;
	A.list = P.list_init.ptr;
	A.fval = P.fval_init.ptr;
	CCF_TRY_S(launch_solve(s, A, mixed, true), "find_initial_roots");
	CCF_TRY_S(cudaEventRecord(f.ev[4], s), "event");
	CCF_TRY_S(polish(C.outs.ptr, (long long)R * nb), "polish");
	/* the solved centres' columns go out at once */
	CCF_TRY_S(cudaEventRecord(C.ready, s), "event");
	CCF_TRY_S(cudaStreamWaitEvent(C.copy, C.ready, 0), "event");
	for (const Arr& a : arrays)
		for (int q = 0; q < K; q++)
		{
			const int c = q * seg;
			CCF_TRY_S(cudaMemcpy2DAsync(a.host + ((size_t)c * cols + half) * a.esize, (size_t)nb * cols * a.esize,
				(const char*)a.ctr + (size_t)c * a.esize, (size_t)nb * a.esize, a.esize, R, cudaMemcpyDeviceToHost, C.copy),
				"copy centre outputs");
		}

	/* ---------------- the continuation, one group of centres at a time ---------------- */
	if (verbose >= 1) std::cout << "Finding critical curve positions...\n";
	A.master = P.master_cont.ptr;
	A.snap32 = mixed ? P.snap32_cont.ptr : nullptr;
	A.snap64 = mixed ? nullptr : P.snap64_cont.ptr;
	A.fin = P.fin_cont.ptr;
	A.list = P.list_cont.ptr;
	A.fval = P.fval_cont.ptr;
	int reordered_groups = 0;
	for (int g = 0; g < ngroups; g++)
	{
		const int k = g & 1;
		const Group& gr = groups[g];
		const FieldOut* og = C.outs.ptr + 1 + g;
		const RowDesc* rows_g = P.rows_cont.ptr + (size_t)g * grows;
		/* the buffer's previous chunk must be out first */
		if (g >= 2) CCF_TRY_S(cudaStreamWaitEvent(s, C.copied[k], 0), "event");
		CCF_TRY_S(cudaMemsetAsync(C.errs[k].ptr, 0, (size_t)R * gr.w_nb * cols * sizeof(double), s), "memset");
		A.outs = og;
		if (track)
		{
			TrackArgs T;
			T.fields = P.views.ptr;
			T.outs = og;
			T.rows = rows_g;
			T.num_rows = grows;
			T.master = P.master_cont.ptr;
			T.table = P.track_table.ptr;
			T.row_stats = P.row_stats.ptr;
			T.item_start = P.item_start.ptr + (size_t)g * grows;
			T.counter = P.rerun_count.ptr + 1;
			T.num_rows_dev = nullptr;
			T.items_per_row = 0;
			T.max_sub = TRACK_TSUB;
			T.num_items = grows * ((R + 31) / 32);
			T.solo = P.solo.ptr;
			T.num_solo = reinterpret_cast<int*>(P.solo.ptr + ncont);
			T.is_solo = P.is_solo.ptr;
			CCF_TRY_S(cudaMemsetAsync(T.num_solo, 0, sizeof(int), s), "memset");
			CCF_TRY_S(cudaMemsetAsync(P.track_table.ptr, 0, gr.table_slots * sizeof(unsigned long long), s), "memset");
			CCF_TRY_S(cudaMemsetAsync(P.row_stats.ptr, 0, TRACK_ROW_STATS * grows * sizeof(unsigned long long), s), "memset");
			CCF_TRY_S(cudaMemsetAsync(P.rerun_count.ptr, 0, 6 * sizeof(int), s), "memset");
			CCF_TRY_S(cudaMemsetAsync(P.row_stats2.ptr, 0, TRACK_ROW_STATS * grows * sizeof(unsigned long long), s), "memset");
			CCF_TRY_S(P.item_order.ensure((size_t)T.num_items + 1), "cudaMalloc(items)");
			CCF_TRY_S(P.item_work.ensure(3 * (size_t)T.num_items + 3), "cudaMalloc(items)");
			/* long items first where the launch is a few waves of items, and its
			   last wave's length is a sizeable share of it (track_item_order_kernel) */
			const bool reorder = (long long)T.num_items < 32LL * num_sms * TRACK_WARPS_PER_SM;
			if (reorder) reordered_groups++;
			T.item_order = reorder ? P.item_order.ptr : nullptr;
			CCF_TRY_S(launch_track_mark(s, T), "track_mark");
			if (reorder) CCF_TRY_S(launch_track_item_order(s, T, P.item_work.ptr, P.item_order.ptr), "track_item_order");
			CCF_TRY_S(launch_track(s, T, mixed), "track_ccs");
			CCF_TRY_S(launch_track_check(s, T, (long long)R * seg * half), "track_check");
			CCF_TRY_S(launch_collect_rerun(s, T, P.rows_rerun.ptr, P.rerun_count.ptr), "collect_rerun");
			TrackArgs T2 = T;
			T2.item_order = nullptr;
			T2.rows = P.rows_rerun.ptr;
			T2.num_rows_dev = P.rerun_count.ptr;
			T2.items_per_row = (R + 31) / 32;
			T2.num_items = grows * T2.items_per_row;
			T2.max_sub = TRACK_TSUB / TRACK_FINE_SUB;
			T2.row_stats = P.row_stats2.ptr;
			T2.counter = P.rerun_count.ptr + 4;
			CCF_TRY_S(launch_clear_tables(s, T2), "clear_tables");
			CCF_TRY_S(launch_track(s, T2, mixed), "track_ccs_fine");
			CCF_TRY_S(launch_track_check(s, T2, (long long)R * seg * half), "track_check");
			CCF_TRY_S(launch_collect_rerun(s, T2, P.rows_rerun2.ptr, P.rerun_count.ptr + 3), "collect_rerun");
			A.rows = P.rows_rerun2.ptr;
			A.num_rows = grows;
			A.num_rows_dev = P.rerun_count.ptr + 3;
		}
		else
		{
			A.rows = rows_g;
			A.num_rows = grows;
			A.num_rows_dev = nullptr;
		}
		{
			const int slots = num_sms * slots_per_sm;
			int cl = 1;
			while (cl < 16 && (long long)grows * cl * 2 <= slots && R / (cl * 2) >= 256) cl *= 2;
			A.cluster = cl;
		}
		CCF_TRY_S(launch_solve(s, A, mixed, false), "find_ccs");
		CCF_TRY_S(polish(og, (long long)R * gr.w_nb * cols), "polish");
		/* the chunk goes out while the next group computes */
		CCF_TRY_S(cudaEventRecord(C.ready, s), "event");
		CCF_TRY_S(cudaStreamWaitEvent(C.copy, C.ready, 0), "event");
		const size_t spitch_pts = (size_t)gr.w_nb * cols, dpitch_pts = (size_t)nb * cols;
		for (const Arr& a : arrays)
			for (const CopyRun& run : gr.runs)
				CCF_TRY_S(cudaMemcpy2DAsync(a.host + ((size_t)run.b * cols + run.k) * a.esize, dpitch_pts * a.esize,
					(const char*)a.win[k] + (size_t)run.j0 * a.esize, spitch_pts * a.esize, (size_t)run.n * a.esize, R,
					cudaMemcpyDeviceToHost, C.copy), "copy chunk outputs");
		CCF_TRY_S(cudaEventRecord(C.copied[k], C.copy), "event");
	}
	/* the run ends when the last chunk is out */
	CCF_TRY_S(cudaEventRecord(C.done, C.copy), "event");
	CCF_TRY_S(cudaStreamWaitEvent(s, C.done, 0), "event");
	CCF_TRY_S(cudaEventRecord(f.ev[6], s), "event");
	CCF_TRY_S(cudaEventRecord(f.ev[5], s), "event");
	CCF_TRY_S(cudaStreamSynchronize(s), "solver");
	/* seeds, (phase table), initial solve, its polish (2); per group the
	   tracker's 8 launches (marking, tracking, column check, collection,
	   table clearing, re-tracking, column check, collection) and the full-sum
	   launch, or the full-sum launch alone, then the polish (2); and the item
	   order's 2 where a group reorders its items */
	return finish_stats(f, seg, track, verbose, (track ? 5 : 4) + (track ? 11 : 3) * ngroups + 2 * reordered_groups);
}

} /* namespace ccf */
