/******************************************************************************
engine.cu -- host orchestration of the device pipeline.

Per field (CCF<T>::run, include/ccf.cuh:1265-1280):
  stars      generate (or upload) the star field, star statistics, corner
             update (include/ccf.cuh:602-730)
  tree       level-by-level split with one small device->host read per level
             (include/ccf.cuh:732-838)
  fmm        expansion order, binomial table, upward and downward passes,
             leaf records (include/ccf.cuh:840-901)
Per batch of fields:
  solve      one initial-solve launch over every branch centre of every
             field, one continuation launch over every (branch, side) row;
             residual, caustics and length scales come out of the solver
             epilogues (include/ccf.cuh:906-1121)
The engine never resets the device and reuses its buffers across runs.
******************************************************************************/
#include "engine.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <mutex>
#include <numeric>
#include <thread>

namespace ccf
{

Field::~Field()
{
	if (events)
	{
		/* the buffers go back to the device-memory cache: wait for the last
		   run's work on them first */
		cudaEventSynchronize(ev[5]);
		for (auto& e : ev) cudaEventDestroy(e);
	}
}

namespace
{
std::mutex g_dmem_mutex;
std::map<int, std::multimap<size_t, void*>> g_dmem;   /* device -> (bytes, block) */
}

cudaError_t dmem_alloc(void** p, size_t bytes, size_t* got)
{
	int dev = 0;
	cudaGetDevice(&dev);
	{
		std::lock_guard<std::mutex> g(g_dmem_mutex);
		auto& pool = g_dmem[dev];
		auto it = pool.lower_bound(bytes);
		/* a kept block of at most twice the size (and 1 MiB) */
		if (it != pool.end() && it->first <= 2 * bytes + (1u << 20))
		{
			*p = it->second;
			*got = it->first;
			pool.erase(it);
			return cudaSuccess;
		}
	}
	cudaError_t e = cudaMalloc(p, bytes);
	if (e == cudaErrorMemoryAllocation)
	{
		cudaGetLastError();
		std::lock_guard<std::mutex> g(g_dmem_mutex);
		for (auto& kv : g_dmem[dev]) cudaFree(kv.second);
		g_dmem[dev].clear();
		e = cudaMalloc(p, bytes);
	}
	if (e == cudaSuccess) *got = bytes;
	return e;
}

void dmem_release(void* p, size_t bytes)
{
	int dev = 0;
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) == cudaSuccess) dev = a.device;
	else cudaGetLastError();
	std::lock_guard<std::mutex> g(g_dmem_mutex);
	g_dmem[dev].emplace(bytes, p);
}

TreeDev Field::tree_dev() const
{
	TreeDev T;
	T.center = n_center.ptr;
	T.half = n_half.ptr;
	T.level = n_level.ptr;
	T.parent = n_parent.ptr;
	T.child = n_child.ptr;
	T.star_start = n_sstart.ptr;
	T.star_count = n_scount.ptr;
	T.nbr = n_nbr.ptr;
	T.nbr_count = n_nbrc.ptr;
	T.m2l = n_m2l.ptr;
	T.m2l_count = n_m2lc.ptr;
	T.p2l = n_p2l.ptr;
	T.p2l_count = n_p2lc.ptr;
	T.flag = n_flag.ptr;
	T.rank = n_rank.ptr;
	return T;
}

Engine::Engine() {}

Engine::~Engine()
{
	for (cudaEvent_t e : setup_events) cudaEventDestroy(e);
	if (chunk.copy)
	{
		cudaStreamSynchronize(chunk.copy);
		cudaStreamDestroy(chunk.copy);
		for (cudaEvent_t e : {chunk.ready, chunk.copied[0], chunk.copied[1], chunk.done}) cudaEventDestroy(e);
	}
	if (stream)
	{
		cudaStreamSynchronize(stream);   /* its pool buffers go back to the cache after this */
		cudaStreamDestroy(stream);
	}
}

ccf_status Engine::cuda_fail(cudaError_t e, const char* what)
{
	error = std::string("CUDA error check for ") + what + " failed: " + cudaGetErrorString(e);
	cudaGetLastError();
	return e == cudaErrorMemoryAllocation ? CCF_ERR_OUT_OF_MEMORY : CCF_ERR_CUDA;
}

bool Engine::ensure_device(int dev)
{
	if (initialized && dev == device) return true;
	int n = 0;
	cudaError_t e = cudaGetDeviceCount(&n);
	if (e != cudaSuccess || n < 1)
	{
		cudaGetLastError();
		error = "Error. No CUDA capable devices detected.";
		return false;
	}
	if (dev < 0 || dev >= n)
	{
		error = "Error. Invalid CUDA device " + std::to_string(dev);
		return false;
	}
	if (cudaSetDevice(dev) != cudaSuccess)
	{
		error = "Error. cudaSetDevice failed";
		return false;
	}
	if (stream)
	{
		cudaStreamDestroy(stream);
		stream = nullptr;
	}
	if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess)
	{
		error = "Error. cudaStreamCreate failed";
		return false;
	}
	cudaDeviceProp prop;
	cudaGetDeviceProperties(&prop, dev);
	num_sms = prop.multiProcessorCount;
	slots_per_sm = std::min(solver_blocks_per_sm(true), solver_blocks_per_sm(false));
	device = dev;
	initialized = true;
	return true;
}

static void ensure_events(Field& f)
{
	if (f.events) return;
	for (auto& e : f.ev) cudaEventCreate(&e);
	f.events = true;
}

static float ev_ms(cudaEvent_t a, cudaEvent_t b)
{
	float ms = 0;
	cudaEventElapsedTime(&ms, a, b);
	return ms;
}

/* parameters, derived values and the star buffers of a field; stars given
   by the caller or read from a file are uploaded (generation order) */
ccf_status Engine::setup_begin(Field& f, int verbose)
{
	ccf_params& p = f.params;
	std::string msg;
	std::unique_ptr<StarField> file_stars;
	const StarField* sf = f.user_stars.get();
	if (!sf && p.starfile[0])
	{
		file_stars.reset(new StarField());
		if (!read_star_file(p.starfile, *file_stars, msg))
		{
			error = msg + "\nError. Unable to read star field parameters from file " + std::string(p.starfile);
			return CCF_ERR_IO;
		}
		sf = file_stars.get();
	}
	if (!derive_params(p, sf, f.d, msg))
	{
		error = msg;
		return CCF_ERR_INVALID_ARGUMENT;
	}
	Derived& d = f.d;
	if (!d.star_input)
	{
		/* include/ccf.cuh:619-622 */
		while (d.random_seed == 0)
		{
			d.random_seed = static_cast<int>(std::chrono::system_clock::now().time_since_epoch().count());
		}
		p.random_seed = d.random_seed;
	}
	if (verbose >= 2 && sf && d.kappa_star > p.kappa_tot) std::cerr << "Warning. kappa_star > kappa_tot\n";
	const int N = d.num_stars;
	cudaStream_t s = stream;
	ensure_events(f);
	CCF_TRY(cudaEventRecord(f.ev[0], s), "event");

	CCF_TRY(f.star_gen.ensure(N), "cudaMalloc(stars)");
	CCF_TRY(f.star_pos.ensure(N), "cudaMalloc(stars)");
	CCF_TRY(f.star_tmp_pos.ensure(N), "cudaMalloc(stars)");
	CCF_TRY(f.star_mass.ensure(N), "cudaMalloc(stars)");
	CCF_TRY(f.star_tmp_mass.ensure(N), "cudaMalloc(stars)");
	CCF_TRY(f.stats5.ensure(8), "cudaMalloc(stats)");
	if (verbose >= 1 && !d.star_input) std::cout << "Generating star field...\n";
	if (d.star_input)
	{
		std::vector<double2> pos(N);
		std::vector<double> mass(N);
		for (int i = 0; i < N; i++)
		{
			pos[i] = make_double2(sf->xym[3 * i], sf->xym[3 * i + 1]);
			mass[i] = sf->xym[3 * i + 2];
		}
		CCF_TRY(cudaMemcpyAsync(f.star_gen.ptr, pos.data(), N * sizeof(double2), cudaMemcpyHostToDevice, s), "upload stars");
		CCF_TRY(cudaMemcpyAsync(f.star_mass.ptr, mass.data(), N * sizeof(double), cudaMemcpyHostToDevice, s), "upload stars");
		CCF_TRY(cudaStreamSynchronize(s), "upload stars");
	}
	return CCF_OK;
}

/* the field's info from its star statistics (include/star.cuh:124-161 and
   include/ccf.cuh:676-700), and the corner from the actual mean mass */
void Engine::setup_stats(Field& f, const double* st)
{
	ccf_params& p = f.params;
	Derived& d = f.d;
	const int N = d.num_stars;
	ccf_info& info = f.info;
	std::memset(&info, 0, sizeof(info));
	info.m_lower_actual = st[3];
	info.m_upper_actual = st[4];
	info.mean_mass_actual = st[0] / N;
	info.mean_mass2_actual = st[1] / N;
	info.mean_mass2_ln_mass_actual = st[2] / N;
	if (d.rectangular) info.kappa_star_actual = st[0] * M_PI * d.theta * d.theta / (4 * d.corner_x1 * d.corner_x2);
	else
	{
		double a = std::hypot(d.corner_x1, d.corner_x2);
		info.kappa_star_actual = st[0] * d.theta * d.theta / (a * a);
	}
	update_corner(p, d, info.mean_mass_actual);
}

ccf_status Engine::prepare_field(Field& f, int verbose)
{
	ccf_status rc = setup_begin(f, verbose);
	if (rc != CCF_OK) return rc;
	ccf_params& p = f.params;
	Derived& d = f.d;
	const int N = d.num_stars;
	cudaStream_t s = stream;
	if (!d.star_input)
	{
		MassTable mt = make_mass_table(d.mass_kind, d.m_lower, d.m_upper, p.m_solar);
		launch_generate_stars(s, N, d.random_seed, d.rectangular, make_double2(d.corner_x1, d.corner_x2),
			std::hypot(d.corner_x1, d.corner_x2), mt, f.star_gen.ptr, f.star_mass.ptr);
		CCF_TRY(cudaGetLastError(), "generate_stars_kernel");
	}
	CCF_TRY(cudaMemcpyAsync(f.star_pos.ptr, f.star_gen.ptr, N * sizeof(double2), cudaMemcpyDeviceToDevice, s), "copy stars");
	launch_star_stats(s, N, f.star_mass.ptr, f.stats5.ptr);
	double st[5];
	CCF_TRY(cudaMemcpyAsync(st, f.stats5.ptr, 5 * sizeof(double), cudaMemcpyDeviceToHost, s), "star stats");
	CCF_TRY(cudaStreamSynchronize(s), "star stats");
	setup_stats(f, st);
	CCF_TRY(cudaEventRecord(f.ev[1], s), "event");
	if (verbose >= 1) std::cout << "Done generating star field.\n";

	if (verbose >= 1) std::cout << "Creating children and sorting stars...\n";
	rc = build_tree(f);
	if (rc != CCF_OK) return rc;
	rc = build_fmm(f);
	if (rc != CCF_OK) return rc;
	CCF_TRY(cudaEventRecord(f.ev[2], s), "event");
	if (verbose >= 1) std::cout << "Done calculating multipole and local coefficients.\n";
	return setup_outputs(f);
}

/* output buffers (device, or page-locked host memory with host_outputs),
   the solver statistics and the rest of the field's info */
ccf_status Engine::setup_outputs(Field& f)
{
	ccf_params& p = f.params;
	Derived& d = f.d;
	ccf_info& info = f.info;
	const int N = d.num_stars;
	cudaStream_t s = stream;
	/* outputs */
	const int R = d.num_roots, nb = p.num_branches, cols = p.num_phi / nb + 1;
	const size_t npts = (size_t)R * nb * cols;
	if (p.host_outputs)
	{
		/* the outputs live in page-locked host memory (written there by the
		   kernels, or by the chunk copies of solve_chunked): the device buffers
		   go back to the cache */
		f.ccs.release();
		f.errs.release();
		f.caustics.release();
		f.mu.release();
		CCF_TRY(f.h_ccs.ensure(npts * sizeof(double2)), "cudaHostAlloc(ccs)");
		CCF_TRY(f.h_errs.ensure(npts * sizeof(double)), "cudaHostAlloc(errs)");
		if (p.write_caustics) CCF_TRY(f.h_caustics.ensure(npts * sizeof(double2)), "cudaHostAlloc(caustics)");
		if (p.write_mu_length_scales) CCF_TRY(f.h_mu.ensure(npts * sizeof(double)), "cudaHostAlloc(mu_length_scales)");
		f.out_ccs = (double2*)f.h_ccs.dev;
		f.out_errs = (double*)f.h_errs.dev;
		f.out_caustics = p.write_caustics ? (double2*)f.h_caustics.dev : nullptr;
		f.out_mu = p.write_mu_length_scales ? (double*)f.h_mu.dev : nullptr;
	}
	else
	{
		f.h_ccs.release();
		f.h_errs.release();
		f.h_caustics.release();
		f.h_mu.release();
		CCF_TRY(f.ccs.ensure(npts), "cudaMalloc(ccs)");
		CCF_TRY(f.errs.ensure(npts), "cudaMalloc(errs)");
		if (p.write_caustics) CCF_TRY(f.caustics.ensure(npts), "cudaMalloc(caustics)");
		if (p.write_mu_length_scales) CCF_TRY(f.mu.ensure(npts), "cudaMalloc(mu_length_scales)");
		f.out_ccs = f.ccs.ptr;
		f.out_errs = f.errs.ptr;
		f.out_caustics = p.write_caustics ? f.caustics.ptr : nullptr;
		f.out_mu = p.write_mu_length_scales ? f.mu.ptr : nullptr;
	}
	CCF_TRY(f.stats.ensure(STATS_WORDS), "cudaMalloc(stats)");
	CCF_TRY(cudaMemsetAsync(f.stats.ptr, 0, STATS_WORDS * sizeof(unsigned long long), s), "memset");

	/* info */
	info.num_stars = N;
	info.num_roots = R;
	info.taylor_smooth = d.taylor_smooth;
	info.rectangular = d.rectangular;
	info.random_seed = d.star_input ? 0 : d.random_seed;
	info.kappa_star = d.kappa_star;
	info.theta_star = d.theta;
	info.corner_x1 = d.corner_x1;
	info.corner_x2 = d.corner_x2;
	info.mu_ave = d.mu_ave;
	info.alpha_error = d.alpha_error;
	info.mean_mass = d.mean_mass;
	info.mean_mass2 = d.mean_mass2;
	info.mean_mass2_ln_mass = d.mean_mass2_ln_mass;
	info.m_lower = d.m_lower;
	info.m_upper = d.m_upper;
	info.num_points = (long long)R * (p.num_phi + nb);
	info.tree_levels = (int)f.level_start.size() - 1;
	info.num_nodes = f.num_nodes;
	info.num_leaves = f.num_leaves;
	info.expansion_order = f.view.order;
	/* kernels launched so far: star field (generate, statistics, FP32 split),
	   tree (root, one flag pass per level, scan/children/partition/neighbours
	   per split level), FMM (upward per level, downward from level 2, leaf
	   flags, scan, leaf records) */
	const int lv = info.tree_levels;
	const int tree_launches = f.tree_one_cta ? 1 : 1 + (lv + 1) + 4 * lv;
	info.kernel_launches = (d.star_input ? 0 : 1) + 1 + (p.precision == CCF_PRECISION_MIXED ? 2 : 0) + tree_launches
		+ (lv + 1) + std::max(0, lv - 1) + 3;
	return CCF_OK;
}

/* node arrays for cap nodes, the first keep of them kept */
cudaError_t Engine::tree_capacity(Field& f, int cap, int keep)
{
	cudaStream_t s = stream;
	{
		cudaError_t e;
		if ((e = f.n_center.grow(cap, keep, s)) != cudaSuccess) return e;
		if ((e = f.n_half.grow(cap, keep, s)) != cudaSuccess) return e;
		if ((e = f.n_level.grow(cap, keep, s)) != cudaSuccess) return e;
		if ((e = f.n_parent.grow(cap, keep, s)) != cudaSuccess) return e;
		if ((e = f.n_child.grow(cap, keep, s)) != cudaSuccess) return e;
		if ((e = f.n_sstart.grow(cap, keep, s)) != cudaSuccess) return e;
		if ((e = f.n_scount.grow(cap, keep, s)) != cudaSuccess) return e;
		if ((e = f.n_nbr.grow((size_t)cap * MAX_NBR, (size_t)keep * MAX_NBR, s)) != cudaSuccess) return e;
		if ((e = f.n_nbrc.grow(cap, keep, s)) != cudaSuccess) return e;
		if ((e = f.n_m2l.grow((size_t)cap * MAX_M2L, (size_t)keep * MAX_M2L, s)) != cudaSuccess) return e;
		if ((e = f.n_m2lc.grow(cap, keep, s)) != cudaSuccess) return e;
		if ((e = f.n_p2l.grow((size_t)cap * MAX_P2L, (size_t)keep * MAX_P2L, s)) != cudaSuccess) return e;
		if ((e = f.n_p2lc.grow(cap, keep, s)) != cudaSuccess) return e;
		if ((e = f.n_flag.grow(cap, keep, s)) != cudaSuccess) return e;
		if ((e = f.n_rank.grow(cap, keep, s)) != cudaSuccess) return e;
		f.node_cap = cap;
		return cudaSuccess;
	}
}

ccf_status Engine::build_tree(Field& f, bool one_cta)
{
	cudaStream_t s = stream;
	const int N = f.d.num_stars;
	const double rhl = root_half_length(f.d);
	f.info.root_half_length = rhl;
	auto alloc_nodes = [&](int cap, int keep) -> cudaError_t { return tree_capacity(f, cap, keep); };
	int cap = std::max(1024, 2 * N + 64);
	if (f.node_cap < cap) CCF_TRY(alloc_nodes(cap, 0), "cudaMalloc(tree)");
	f.tree_one_cta = false;
	/* CCF_GB300_TREE_LEVELS=1 keeps the per-level build (the tests compare the two) */
	static const bool per_level = [] {
		const char* e = std::getenv("CCF_GB300_TREE_LEVELS");
		return e && std::atoi(e) == 1;
	}();
	if (one_cta && !per_level && N <= BATCH_SETUP_MAX_STARS)
	{
		/* the whole tree in one CTA (tree_batch_kernel): the same tree as the
		   per-level launches below, without their host round trip per level;
		   a tree that outgrows the node capacity is built by those */
		BatchSeg g;
		std::memset(&g, 0, sizeof(g));
		g.n = N;
		g.pos = f.star_pos.ptr;
		g.mass = f.star_mass.ptr;
		g.tpos = f.star_tmp_pos.ptr;
		g.tmass = f.star_tmp_mass.ptr;
		g.T = f.tree_dev();
		g.node_cap = f.node_cap;
		g.limit = leaf_limit(f.params);
		g.root_half = rhl;
		CCF_TRY(batch_segs.ensure(1), "cudaMalloc(tree)");
		CCF_TRY(batch_info.ensure(BATCH_INFO_INTS), "cudaMalloc(tree)");
		g.info = batch_info.ptr;
		CCF_TRY(cudaMemcpyAsync(batch_segs.ptr, &g, sizeof(g), cudaMemcpyHostToDevice, s), "upload(tree)");
		launch_tree_batch(s, batch_segs.ptr, 1);
		CCF_TRY(cudaGetLastError(), "tree_batch_kernel");
		std::vector<int> fi(BATCH_INFO_INTS);
		CCF_TRY(cudaMemcpyAsync(fi.data(), batch_info.ptr, fi.size() * sizeof(int), cudaMemcpyDeviceToHost, s), "tree");
		CCF_TRY(cudaStreamSynchronize(s), "tree");
		if (fi[2] & 1) { error = "Error. Tree neighbour list overflow."; return CCF_ERR_NUMERIC; }
		if (!(fi[2] & 2))
		{
			const int levels = fi[0];
			f.level_start.assign(fi.begin() + 3, fi.begin() + 3 + levels + 1);
			f.level_count.assign(fi.begin() + 3 + TREE_MAX_LEVELS + 1, fi.begin() + 3 + TREE_MAX_LEVELS + 1 + levels + 1);
			f.num_nodes = fi[1];
			f.info.leaf_max_stars = g.limit;
			f.tree_one_cta = true;
			/* the per-level path's error word, read by build_fmm */
			CCF_TRY(f.level_out.ensure(4), "cudaMalloc(tree)");
			CCF_TRY(cudaMemsetAsync(f.level_out.ptr, 0, 4 * sizeof(int), s), "memset");
			return CCF_OK;
		}
	}
	CCF_TRY(f.level_out.ensure(4), "cudaMalloc(tree)");
	f.level_start.assign(1, 0);
	f.level_count.assign(1, 1);
	launch_tree_root(s, f.tree_dev(), rhl, N);
	CCF_TRY(cudaMemsetAsync(f.level_out.ptr, 0, 4 * sizeof(int), s), "memset");
	/* a node splits while its stars and its neighbours' exceed the leaf limit */
	const int limit = leaf_limit(f.params);
	int L = 0;
	while (true)
	{
		int start = f.level_start[L], count = f.level_count[L];
		CCF_TRY(cudaMemsetAsync(f.level_out.ptr, 0, 2 * sizeof(int), s), "memset");
		launch_tree_flag(s, f.tree_dev(), start, count, limit, f.level_out.ptr);
		int hv[3];
		CCF_TRY(cudaMemcpyAsync(hv, f.level_out.ptr, 3 * sizeof(int), cudaMemcpyDeviceToHost, s), "tree level");
		CCF_TRY(cudaStreamSynchronize(s), "get_node_star_info");
		if (hv[2]) { error = "Error. Tree neighbour list overflow."; return CCF_ERR_NUMERIC; }
		if (hv[0] <= limit) break;
		int nflag = hv[1];
		int child_start = start + count;
		int need = child_start + 4 * nflag;
		if (need > f.node_cap) CCF_TRY(alloc_nodes(std::max(need, 2 * f.node_cap), child_start), "cudaMalloc(tree)");
		TreeDev T = f.tree_dev();
		launch_scan(s, T.flag + start, T.rank + start, count);
		launch_tree_children(s, T, start, count, child_start);
		launch_tree_partition(s, T, start, count, f.star_pos.ptr, f.star_mass.ptr, f.star_tmp_pos.ptr, f.star_tmp_mass.ptr);
		launch_tree_neighbors(s, T, child_start, 4 * nflag, f.level_out.ptr + 2);
		CCF_TRY(cudaGetLastError(), "tree kernels");
		f.level_start.push_back(child_start);
		f.level_count.push_back(4 * nflag);
		L++;
		if (L > 40) { error = "Error. Tree deeper than 40 levels."; return CCF_ERR_NUMERIC; }
	}
	f.num_nodes = f.level_start[L] + f.level_count[L];
	f.info.leaf_max_stars = limit;
	return CCF_OK;
}

/* the expansion order (include/ccf.cuh:840-852), or the explicit one */
ccf_status Engine::fmm_order(Field& f, int levels, int& P)
{
	const Derived& d = f.d;
	P = (int)std::ceil(2 * std::log2(d.theta) + levels - std::log2(f.info.root_half_length) - std::log2(d.alpha_error));
	if (f.params.expansion_order > 0) P = f.params.expansion_order;   /* validated in [3, MAX_ORDER] */
	if (P < 3) { error = "Error. Expansion order needs to be >= 3"; return CCF_ERR_INVALID_ARGUMENT; }
	if (P > MAX_ORDER) { error = "Error. Maximum allowed expansion order is " + std::to_string(MAX_ORDER); return CCF_ERR_INVALID_ARGUMENT; }
	return CCF_OK;
}

ccf_status Engine::build_fmm(Field& f)
{
	cudaStream_t s = stream;
	ccf_params& p = f.params;
	Derived& d = f.d;
	const int levels = (int)f.level_start.size() - 1;
	int P = 0;
	ccf_status rc = fmm_order(f, levels, P);
	if (rc != CCF_OK) return rc;
	std::vector<double> B = binomial_table(2 * P, !p.exact_binomials);
	CCF_TRY(f.binom.ensure(B.size()), "cudaMalloc(binomials)");
	CCF_TRY(cudaMemcpyAsync(f.binom.ptr, B.data(), B.size() * sizeof(double), cudaMemcpyHostToDevice, s), "binomials");
	const size_t nc = (size_t)f.num_nodes * (P + 1);
	CCF_TRY(f.multi.ensure(nc), "cudaMalloc(multipole)");
	CCF_TRY(f.local.ensure(nc), "cudaMalloc(local)");
	CCF_TRY(cudaMemsetAsync(f.multi.ptr, 0, nc * sizeof(double2), s), "memset");
	CCF_TRY(cudaMemsetAsync(f.local.ptr, 0, nc * sizeof(double2), s), "memset");
	TreeDev T = f.tree_dev();
	for (int L = levels; L >= 0; L--)
	{
		launch_fmm_upward(s, T, f.level_start[L], f.level_count[L], P, f.star_pos.ptr, f.star_mass.ptr, f.multi.ptr, f.binom.ptr);
	}
	for (int L = 2; L <= levels; L++)
	{
		launch_fmm_downward(s, T, f.level_start[L], f.level_count[L], P, f.star_pos.ptr, f.star_mass.ptr, f.multi.ptr,
			f.local.ptr, f.binom.ptr);
	}
	CCF_TRY(cudaGetLastError(), "fmm kernels");

	/* leaves */
	CCF_TRY(f.leaf_flag.ensure(f.num_nodes), "cudaMalloc(leaves)");
	CCF_TRY(f.leaf_index.ensure(f.num_nodes), "cudaMalloc(leaves)");
	CCF_TRY(f.node_leaf.ensure(f.num_nodes), "cudaMalloc(leaves)");
	launch_leaf_flag(s, T, f.num_nodes, f.leaf_flag.ptr);
	launch_scan(s, f.leaf_flag.ptr, f.leaf_index.ptr, f.num_nodes);
	int tail[2];
	CCF_TRY(cudaMemcpyAsync(&tail[0], f.leaf_index.ptr + f.num_nodes - 1, sizeof(int), cudaMemcpyDeviceToHost, s), "leaves");
	CCF_TRY(cudaMemcpyAsync(&tail[1], f.leaf_flag.ptr + f.num_nodes - 1, sizeof(int), cudaMemcpyDeviceToHost, s), "leaves");
	CCF_TRY(cudaStreamSynchronize(s), "leaves");
	const int nl = tail[0] + tail[1];
	f.num_leaves = nl;
	CCF_TRY(f.leaf_center.ensure(nl), "cudaMalloc(leaves)");
	CCF_TRY(f.leaf_inv_half.ensure(nl), "cudaMalloc(leaves)");
	CCF_TRY(f.leaf_near_count.ensure(nl), "cudaMalloc(leaves)");
	CCF_TRY(f.leaf_near.ensure((size_t)nl * MAX_NEAR), "cudaMalloc(leaves)");
	CCF_TRY(f.leaf_loc.ensure((size_t)nl * 3 * (P + 1)), "cudaMalloc(leaves)");
	CCF_TRY(f.leaf_loc3f.ensure((size_t)nl * (P + 1)), "cudaMalloc(leaves)");
	CCF_TRY(cudaMemsetAsync(f.level_out.ptr + 2, 0, sizeof(int), s), "memset");
	launch_leaf_build(s, T, f.num_nodes, f.leaf_index.ptr, P, d.theta * d.theta, f.star_pos.ptr, f.star_mass.ptr, f.local.ptr,
		f.leaf_center.ptr, f.leaf_inv_half.ptr, f.leaf_near_count.ptr, f.leaf_near.ptr, f.leaf_loc.ptr, f.leaf_loc3f.ptr,
		f.node_leaf.ptr, f.level_out.ptr + 2);
	CCF_TRY(cudaGetLastError(), "leaf_build_kernel");
	if (p.precision == CCF_PRECISION_MIXED)
	{
		CCF_TRY(f.leaf_near_df.ensure((size_t)nl * MAX_NEAR), "cudaMalloc(leaves)");
		CCF_TRY(f.leaf_mass_df.ensure((size_t)nl * MAX_NEAR), "cudaMalloc(leaves)");
		CCF_TRY(f.leaf_loc_df.ensure((size_t)nl * 2 * (P + 1)), "cudaMalloc(leaves)");
		CCF_TRY(f.leaf_ih_df.ensure(nl), "cudaMalloc(leaves)");
		launch_leaf_df(s, nl, P, f.leaf_center.ptr, f.leaf_inv_half.ptr, f.leaf_near_count.ptr, f.leaf_near.ptr,
			f.leaf_loc.ptr, f.leaf_near_df.ptr, f.leaf_mass_df.ptr, f.leaf_loc_df.ptr, f.leaf_ih_df.ptr);
		CCF_TRY(cudaGetLastError(), "leaf_df_kernel");
		/* split stars: poles of the Aberth sums and the off-field direct sums */
		CCF_TRY(f.star_hilo.ensure(d.num_stars), "cudaMalloc(star hilo)");
		CCF_TRY(f.star_mass_df.ensure(d.num_stars), "cudaMalloc(star hilo)");
		launch_star_hilo(s, d.num_stars, f.star_pos.ptr, f.star_hilo.ptr, f.star_mass.ptr, f.star_mass_df.ptr);
		CCF_TRY(cudaGetLastError(), "star_hilo_kernel");
	}

	/* mean near-list length over the leaves (reported; the tracker's work per
	   evaluation grows with it) */
	double near_sum = 0;
	{
		std::vector<int> cnt(nl);
		CCF_TRY(cudaMemcpyAsync(cnt.data(), f.leaf_near_count.ptr, nl * sizeof(int), cudaMemcpyDeviceToHost, s), "near counts");
		CCF_TRY(cudaStreamSynchronize(s), "near counts");
		for (int v : cnt) near_sum += v;
	}
	int lerr = 0;
	CCF_TRY(cudaMemcpyAsync(&lerr, f.level_out.ptr + 2, sizeof(int), cudaMemcpyDeviceToHost, s), "leaves");
	CCF_TRY(cudaStreamSynchronize(s), "leaves");
	return finish_view(f, P, near_sum, lerr);
}

/* the smooth-mass polynomials, the fold of their series into the leaf
   expansions (rectangular Taylor form, mixed precision) and the field's
   device view, after the leaf records */
ccf_status Engine::finish_view(Field& f, int P, double near_sum, int lerr, UploadPack* up)
{
	cudaStream_t s = stream;
	/* host-to-device copies of small arrays: collected in up when given
	   (written by one copy and one scatter launch for a whole batch) */
	auto put = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
		if (up)
		{
			up->add(dst, src, bytes);
			return cudaSuccess;
		}
		return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
	};
	ccf_params& p = f.params;
	Derived& d = f.d;
	const int nl = f.num_leaves;
	f.info.near_mean = nl > 0 ? near_sum / nl : 0;
	if (lerr) { error = "Error. A leaf has more than 32 near stars."; return CCF_ERR_NUMERIC; }

	/* smooth-mass polynomials */
	float4 inv_corner_df = make_float4(0, 0, 0, 0);
	bool fold_ok = false;
	std::vector<unsigned char> fold_host;   /* the folded-leaf flags, for ccf_info.leaves_folded */
	SmoothPoly sp = smooth_polynomials(d.kappa_star, d.corner_x1, d.corner_x2, d.taylor_smooth);
	{
		std::vector<double2> d1(std::max(1, sp.m)), d2(std::max(1, sp.m)), a(sp.a.size());
		std::vector<float2> d2f(std::max(1, sp.m));
		for (int i = 0; i < sp.m; i++)
		{
			d1[i] = make_double2(sp.d1[i].real(), sp.d1[i].imag());
			d2[i] = make_double2(sp.d2[i].real(), sp.d2[i].imag());
			d2f[i] = make_float2((float)sp.d2[i].real(), (float)sp.d2[i].imag());
		}
		for (size_t i = 0; i < a.size(); i++) a[i] = make_double2(sp.a[i].real(), sp.a[i].imag());
		/* double-float copies (hi = nearest float, lo = float of the remainder) */
		auto split4 = [](std::complex<double> v) {
			float rh = (float)v.real(), ih = (float)v.imag();
			return make_float4(rh, ih, (float)(v.real() - (double)rh), (float)(v.imag() - (double)ih));
		};
		std::vector<float4> d1df(std::max(1, sp.m)), adf(sp.a.size());
		for (int i = 0; i < sp.m; i++) d1df[i] = split4(sp.d1[i]);
		/* alpha polynomial in w = zbar / c: B_n = A_n c^n.  |A_n| falls like
		   |c|^(1-n) and leaves the FP32 range for large fields, B_n stays O(|c|) */
		{
			std::complex<long double> cn(1.0L, 0.0L);
			const std::complex<long double> cl((long double)d.corner_x1, (long double)d.corner_x2);
			for (size_t i = 0; i < sp.a.size(); i++)
			{
				const std::complex<long double> b = std::complex<long double>(sp.a[i].real(), sp.a[i].imag()) * cn;
				adf[i] = split4(std::complex<double>((double)b.real(), (double)b.imag()));
				cn *= cl;
			}
		}
		inv_corner_df = split4(sp.inv_corner);
		CCF_TRY(f.sm_d1_df.ensure(d1df.size()), "cudaMalloc(smooth)");
		CCF_TRY(f.sm_a_df.ensure(adf.size()), "cudaMalloc(smooth)");
		CCF_TRY(put(f.sm_d1_df.ptr, d1df.data(), d1df.size() * sizeof(float4)), "smooth");
		CCF_TRY(put(f.sm_a_df.ptr, adf.data(), adf.size() * sizeof(float4)), "smooth");
		CCF_TRY(f.sm_d1.ensure(d1.size()), "cudaMalloc(smooth)");
		CCF_TRY(f.sm_d2.ensure(d2.size()), "cudaMalloc(smooth)");
		CCF_TRY(f.sm_d2f.ensure(d2f.size()), "cudaMalloc(smooth)");
		CCF_TRY(f.sm_a.ensure(a.size()), "cudaMalloc(smooth)");
		CCF_TRY(put(f.sm_d1.ptr, d1.data(), d1.size() * sizeof(double2)), "smooth");
		CCF_TRY(put(f.sm_d2.ptr, d2.data(), d2.size() * sizeof(double2)), "smooth");
		CCF_TRY(put(f.sm_d2f.ptr, d2f.data(), d2f.size() * sizeof(float2)), "smooth");
		CCF_TRY(put(f.sm_a.ptr, a.data(), a.size() * sizeof(double2)), "smooth");
		/* the tracker's leaf blocks with the Taylor series folded in (rectangular
		   Taylor smooth mass, mixed precision): the series conjugated into
		   polynomials in z, built in long double */
		fold_ok = p.precision == CCF_PRECISION_MIXED && d.rectangular && p.approx && sp.m > 0;
		if (fold_ok)
		{
			typedef std::complex<long double> cl;
			const cl icb = std::conj(cl((long double)sp.inv_corner.real(), (long double)sp.inv_corner.imag()));
			const int M = sp.m, na = (int)sp.a.size();
			std::vector<double2> coef(2 * M + 1 + 2 * M + na, make_double2(0, 0));
			double2* ef = coef.data();
			double2* er = ef + 2 * M + 1;
			double2* eq = er + 2 * M;
			cl pw(1.0L, 0.0L);
			for (int m = 1; m <= M; m++)
			{
				pw *= icb * icb;   /* conj(1 / c)^(2m) */
				const cl v1 = std::conj(cl(sp.d1[m - 1].real(), sp.d1[m - 1].imag())) * pw;
				const cl v2 = std::conj(cl(sp.d2[m - 1].real(), sp.d2[m - 1].imag())) * pw;
				ef[2 * m] = make_double2((double)v1.real(), (double)v1.imag());
				er[2 * m - 1] = make_double2((double)v2.real(), (double)v2.imag());
			}
			const long double kpi = (long double)d.kappa_star / 3.14159265358979323846264338327950288L;
			for (int n = 0; n < na; n++)
			{
				const cl v = cl(0.0L, kpi) * std::conj(cl(sp.a[n].real(), sp.a[n].imag()));
				eq[n] = make_double2((double)v.real(), (double)v.imag());
			}
			CCF_TRY(f.fold_coef.ensure(coef.size()), "cudaMalloc(fold)");
			CCF_TRY(cudaMemcpyAsync(f.fold_coef.ptr, coef.data(), coef.size() * sizeof(double2), cudaMemcpyHostToDevice, s),
				"fold");
			CCF_TRY(f.leaf_fold.ensure(nl), "cudaMalloc(fold)");
			CCF_TRY(f.leaf_loc_df_fold.ensure((size_t)nl * 2 * (P + 1)), "cudaMalloc(fold)");
			CCF_TRY(f.leaf_loc3f_fold.ensure((size_t)nl * (P + 1)), "cudaMalloc(fold)");
			CCF_TRY(f.leaf_loc_fold64.ensure((size_t)nl * 3 * (P + 1)), "cudaMalloc(fold)");
			launch_fold_smooth(s, nl, P, f.leaf_center.ptr, f.leaf_inv_half.ptr, f.leaf_loc.ptr, f.fold_coef.ptr, 2 * M + 1,
				f.fold_coef.ptr + 2 * M + 1, 2 * M, f.fold_coef.ptr + 4 * M + 1, na, 0.95 * std::hypot(d.corner_x1, d.corner_x2),
				f.leaf_loc_df_fold.ptr, f.leaf_loc3f_fold.ptr, f.leaf_loc_fold64.ptr, f.leaf_fold.ptr);
			CCF_TRY(cudaGetLastError(), "fold_smooth_kernel");
			fold_host.resize(nl);
			CCF_TRY(cudaMemcpyAsync(fold_host.data(), f.leaf_fold.ptr, nl, cudaMemcpyDeviceToHost, s), "fold");
		}
		if (fold_ok) CCF_TRY(cudaStreamSynchronize(s), "smooth");
		for (unsigned char v : fold_host) f.info.leaves_folded += v ? 1 : 0;
	}

	FieldView& V = f.view;
	std::memset(&V, 0, sizeof(V));
	V.kappa_tot = p.kappa_tot;
	V.shear = p.shear;
	V.kappa_star = d.kappa_star;
	V.theta = d.theta;
	V.theta2 = d.theta * d.theta;
	V.rectangular = d.rectangular;
	V.approx = p.approx;
	V.taylor_smooth = d.taylor_smooth;
	V.order = P;
	V.num_roots = d.num_roots;
	V.corner = make_double2(d.corner_x1, d.corner_x2);
	V.corner_abs = std::hypot(d.corner_x1, d.corner_x2);
	V.smooth_m = sp.m;
	V.inv_corner = make_double2(sp.inv_corner.real(), sp.inv_corner.imag());
	V.inv_corner2 = make_double2(sp.inv_corner2.real(), sp.inv_corner2.imag());
	V.smooth_k1 = sp.k1;
	V.smooth_d1 = f.sm_d1.ptr;
	V.smooth_d2 = f.sm_d2.ptr;
	V.smooth_a = f.sm_a.ptr;
	V.smooth_d2f = f.sm_d2f.ptr;
	V.num_stars = d.num_stars;
	V.star_pos = f.star_pos.ptr;
	V.star_mass = f.star_mass.ptr;
	V.num_nodes = f.num_nodes;
	V.node_center = f.n_center.ptr;
	V.node_half = f.n_half.ptr;
	V.node_child = f.n_child.ptr;
	V.node_leaf = f.node_leaf.ptr;
	V.num_leaves = nl;
	V.leaf_center = f.leaf_center.ptr;
	V.leaf_inv_half = f.leaf_inv_half.ptr;
	V.leaf_near_count = f.leaf_near_count.ptr;
	V.leaf_near = f.leaf_near.ptr;
	V.leaf_loc = f.leaf_loc.ptr;
	V.leaf_loc3f = f.leaf_loc3f.ptr;
	V.leaf_near_df = f.leaf_near_df.ptr;
	V.leaf_mass_df = f.leaf_mass_df.ptr;
	V.leaf_loc_df = f.leaf_loc_df.ptr;
	V.leaf_ih_df = f.leaf_ih_df.ptr;
	V.smooth_d1_df = f.sm_d1_df.ptr;
	V.smooth_a_df = f.sm_a_df.ptr;
	V.inv_corner_df = inv_corner_df;
	V.star_df = f.star_hilo.ptr;
	V.star_mass_df = f.star_mass_df.ptr;
	V.leaf_fold = fold_ok ? f.leaf_fold.ptr : nullptr;
	V.leaf_loc_df_fold = fold_ok ? f.leaf_loc_df_fold.ptr : nullptr;
	V.leaf_loc3f_fold = fold_ok ? f.leaf_loc3f_fold.ptr : nullptr;
	V.leaf_loc_fold64 = fold_ok ? f.leaf_loc_fold64.ptr : nullptr;
	CCF_TRY(f.view_dev.ensure(1), "cudaMalloc(view)");
	CCF_TRY(put(f.view_dev.ptr, &V, sizeof(V)), "view");
	return CCF_OK;
}

static size_t nb_total(const std::vector<Field*>& fields)
{
	size_t n = 0;
	for (const Field* f : fields) n += (size_t)f->params.num_branches;
	return n;
}

/* largest number of branches per solved centre the engine picks by itself */
constexpr int MAX_SEG = 16;

int Engine::solved_seg(const Field& f, bool track) const
{
	const long long lanes_wanted = 2LL * num_sms * 16 * 32;
	const int R = f.d.num_roots, nb = f.params.num_branches;
	if (!track) return 1;
	if (f.params.solved_centres > 0) return nb / f.params.solved_centres;
	for (int g = std::min(nb, MAX_SEG); g > 1; g--)
		if (nb % g == 0 && 2LL * (nb / g) * R >= lanes_wanted) return g;
	return 1;
}

ccf_status Engine::solve(std::vector<Field*>& fields, int verbose)
{
	cudaStream_t s = stream;
	const int nf = (int)fields.size();
	const bool mixed = fields[0]->params.precision == CCF_PRECISION_MIXED;
	const bool track = fields[0]->params.continuation == CCF_CONTINUATION_TRACK;
	for (Field* f : fields)
	{
		if ((f->params.precision == CCF_PRECISION_MIXED) != mixed)
		{
			error = "Error. All fields of a batch must use the same precision.";
			return CCF_ERR_INVALID_ARGUMENT;
		}
		if ((f->params.continuation == CCF_CONTINUATION_TRACK) != track)
		{
			error = "Error. All fields of a batch must use the same continuation.";
			return CCF_ERR_INVALID_ARGUMENT;
		}
	}
	/* Solved centres: with the full-sum continuation every branch centre, as
	   the reference.  With the tracker, every seg-th centre, seg the largest
	   divisor of num_branches up to 16 that still gives the continuation about
	   two resident waves of tracked roots (2 rows of R roots per centre): the
	   initial solve costs O(R (R + N)) per sweep and centre, the tracker only
	   its evaluations, and rows from a centre then cover seg branches.  The cap
	   bounds the chain of a root that starts off the root box, which one warp
	   tracks alone with direct star sums (on the 20000-star field 8 of 128
	   centres take 0.62 s per field, 2 centres 3.2 s, all 128 1.50 s). */
	std::vector<int> seg(nf);
	for (int i = 0; i < nf; i++) seg[i] = solved_seg(*fields[i], track);
	/* row offsets */
	std::vector<long long> init_off(nf), cont_off(nf);
	long long ninit = 0, ncont = 0;
	int rows_init = 0, rows_cont = 0, minR = 1 << 30, maxR = 0;
	for (int i = 0; i < nf; i++)
	{
		const int R = fields[i]->d.num_roots, nb = fields[i]->params.num_branches;
		const int K = nb / seg[i];
		init_off[i] = ninit;
		cont_off[i] = ncont;
		ninit += (long long)K * R;
		ncont += (long long)2 * K * R;
		rows_init += K;
		rows_cont += 2 * K;
		minR = std::min(minR, R);
		maxR = std::max(maxR, R);
	}
	SolverPools& P = pools;
	CCF_TRY(P.master_init.ensure(ninit), "cudaMalloc(roots)");
	CCF_TRY(P.master_cont.ensure(ncont), "cudaMalloc(roots)");
	CCF_TRY(P.fin_init.ensure(ninit), "cudaMalloc(roots)");
	CCF_TRY(P.fin_cont.ensure(ncont), "cudaMalloc(roots)");
	CCF_TRY(P.list_init.ensure(ninit), "cudaMalloc(roots)");
	CCF_TRY(P.list_cont.ensure(ncont), "cudaMalloc(roots)");
	CCF_TRY(P.fval_init.ensure(2 * ninit), "cudaMalloc(roots)");
	CCF_TRY(P.fval_cont.ensure(2 * ncont), "cudaMalloc(roots)");
	if (mixed)
	{
		CCF_TRY(P.snap32_init.ensure(ninit), "cudaMalloc(roots)");
		CCF_TRY(P.snap32_cont.ensure(ncont), "cudaMalloc(roots)");
	}
	else
	{
		CCF_TRY(P.snap64_init.ensure(ninit), "cudaMalloc(roots)");
		CCF_TRY(P.snap64_cont.ensure(ncont), "cudaMalloc(roots)");
	}
	std::vector<FieldView> views(nf);
	std::vector<FieldOut> outs(nf);
	std::vector<const float4*> hilo(nf);
	std::vector<RowDesc> ri, rc;
	std::vector<double> cost_i, cost_c;
	long long table_slots = 0;   /* tracker: 2 R slots per phi step of every continuation row */
	std::vector<int> item_start_host(2 * nb_total(fields));
	std::vector<SeedSeg> seeds;
	long long max_seeds = 0;
	/* fields with the same branches and phi steps share one phase table */
	std::vector<std::pair<std::pair<int, int>, const PhaseEntry*>> phase_tables;
	for (int i = 0; i < nf; i++)
	{
		Field& f = *fields[i];
		const int R = f.d.num_roots, N = f.d.num_stars, nb = f.params.num_branches;
		views[i] = f.view;
		FieldOut& o = outs[i];
		std::memset(&o, 0, sizeof(o));
		o.ccs = f.out_ccs;
		o.caustics = f.out_caustics;
		o.errs = f.out_errs;
		o.mu = f.out_mu;
		o.nb = nb;
		o.nphi = f.params.num_phi;
		o.cols = f.params.num_phi / nb + 1;
		o.half = f.params.num_phi / (2 * nb);
		o.step_first = 1;
		o.step_last = o.half;
		full_window(o);
		o.check_inline = f.params.host_outputs == 1 ? 1 : 0;
		o.max_iters_init = f.params.max_iters_init;
		o.max_iters_step = f.params.max_iters_step;
		o.seg = seg[i];
		if (track)
		{
			const std::pair<int, int> key(nb, f.params.num_phi);
			const PhaseEntry* shared = nullptr;
			for (const auto& t : phase_tables)
				if (t.first == key) shared = t.second;
			if (!shared)
			{
				CCF_TRY(f.phase.ensure(f.params.num_phi), "cudaMalloc(phase)");
				CCF_TRY(launch_phase_table(s, nb, f.params.num_phi, f.phase.ptr), "phase_table_kernel");
				shared = f.phase.ptr;
				phase_tables.push_back({key, shared});
			}
			o.phase = shared;
		}
		o.cont_master = P.master_cont.ptr;
		o.cont_snap32 = mixed ? P.snap32_cont.ptr : nullptr;
		o.cont_snap64 = mixed ? nullptr : P.snap64_cont.ptr;
		o.stats = f.stats.ptr;
		hilo[i] = mixed ? f.star_hilo.ptr : nullptr;
		double cost = (double)R * (double)(R + N);
		const int g = seg[i], K = nb / g;
		for (int q = 0; q < K; q++)
		{
			RowDesc r;
			r.field = i;
			r.branch = q * g;
			r.side = -1;
			r.steps = 0;
			r.base = init_off[i] + (long long)q * R;
			r.cont_base = cont_off[i] + (long long)(2 * q) * R;
			ri.push_back(r);
			cost_i.push_back(cost);
			for (int b = 0; b < 2; b++)
			{
				RowDesc u = r;
				u.side = b;
				/* side 1 reaches half way to the next solved centre; side 0 stops
				   one step short of it unless every centre is solved (row_slots) */
				u.steps = g == 1 ? o.half : (b == 1 ? g * o.half : g * o.half - 1);
				u.base = cont_off[i] + (long long)(2 * q + b) * R;
				u.cont_base = table_slots;
				table_slots += 2LL * R * u.steps;
				rc.push_back(u);
				cost_c.push_back(cost * u.steps);
			}
		}
		/* seeds of the solved centres of this field, from the stars in tree
		   order: consecutive roots (the lanes of a tracker warp) then start
		   next to neighbouring stars, in the same or adjacent leaves, so their
		   near-star loops and smooth-mass paths agree (the order of the roots
		   within a column carries no meaning; a row stays one root's path) */
		SeedSeg sd;
		sd.nstars = N;
		sd.nroots = R;
		sd.nrows = K;
		sd.nb = nb;
		sd.seg = g;
		sd.pos = f.star_pos.ptr;
		sd.mass = f.star_mass.ptr;
		sd.corner_abs = f.view.corner_abs;
		sd.theta = f.view.theta;
		sd.a_lin = 1 - f.view.kappa_tot + f.view.kappa_star;
		sd.gamma = f.view.shear;
		sd.master = P.master_init.ptr + init_off[i];
		sd.snap32 = mixed ? P.snap32_init.ptr + init_off[i] : nullptr;
		sd.snap64 = mixed ? nullptr : P.snap64_init.ptr + init_off[i];
		seeds.push_back(sd);
		max_seeds = std::max(max_seeds, (long long)R * K);
	}
	/* every field's seeds in one launch */
	CCF_TRY(P.seeds.ensure(seeds.size()), "cudaMalloc(seeds)");
	CCF_TRY(cudaMemcpyAsync(P.seeds.ptr, seeds.data(), seeds.size() * sizeof(SeedSeg), cudaMemcpyHostToDevice, s), "upload");
	for (size_t i0 = 0; i0 < seeds.size(); i0 += 65535)   /* blockIdx.y is the field */
		launch_seed_roots_batch(s, P.seeds.ptr + i0, (int)std::min<size_t>(65535, seeds.size() - i0), max_seeds);
	CCF_TRY(cudaGetLastError(), "seed_roots_batch_kernel");
	/* largest rows first */
	auto order = [](std::vector<RowDesc>& rows, std::vector<double>& cost) {
		std::vector<int> idx(rows.size());
		std::iota(idx.begin(), idx.end(), 0);
		std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return cost[a] > cost[b]; });
		std::vector<RowDesc> out(rows.size());
		for (size_t i = 0; i < idx.size(); i++) out[i] = rows[idx[i]];
		rows.swap(out);
	};
	order(ri, cost_i);
	order(rc, cost_c);
	CCF_TRY(P.views.ensure(nf), "cudaMalloc(views)");
	CCF_TRY(P.outs.ensure(nf), "cudaMalloc(outs)");
	CCF_TRY(P.hilo_ptrs.ensure(nf), "cudaMalloc(views)");
	CCF_TRY(P.rows_init.ensure(ri.size()), "cudaMalloc(rows)");
	CCF_TRY(P.rows_cont.ensure(rc.size()), "cudaMalloc(rows)");
	CCF_TRY(P.error.ensure(1), "cudaMalloc(error)");
	CCF_TRY(cudaMemcpyAsync(P.views.ptr, views.data(), nf * sizeof(FieldView), cudaMemcpyHostToDevice, s), "upload");
	CCF_TRY(cudaMemcpyAsync(P.outs.ptr, outs.data(), nf * sizeof(FieldOut), cudaMemcpyHostToDevice, s), "upload");
	CCF_TRY(cudaMemcpyAsync(P.hilo_ptrs.ptr, hilo.data(), nf * sizeof(const float4*), cudaMemcpyHostToDevice, s), "upload");
	CCF_TRY(cudaMemcpyAsync(P.rows_init.ptr, ri.data(), ri.size() * sizeof(RowDesc), cudaMemcpyHostToDevice, s), "upload");
	CCF_TRY(cudaMemcpyAsync(P.rows_cont.ptr, rc.data(), rc.size() * sizeof(RowDesc), cudaMemcpyHostToDevice, s), "upload");
	CCF_TRY(cudaMemsetAsync(P.error.ptr, 0, sizeof(int), s), "memset");
	if (track)
	{
		CCF_TRY(P.track_table.ensure(table_slots), "cudaMalloc(tables)");
		CCF_TRY(P.row_stats.ensure(TRACK_ROW_STATS * rc.size()), "cudaMalloc(rows)");
		CCF_TRY(P.rows_rerun.ensure(rc.size()), "cudaMalloc(rows)");
		CCF_TRY(P.rerun_count.ensure(6), "cudaMalloc(rows)");
		CCF_TRY(P.rows_rerun2.ensure(rc.size()), "cudaMalloc(rows)");
		CCF_TRY(P.row_stats2.ensure(TRACK_ROW_STATS * rc.size()), "cudaMalloc(rows)");
		CCF_TRY(P.item_start.ensure(rc.size()), "cudaMalloc(rows)");
	}

	/* CTAs per row: fill the resident slots without a second wave */
	const int slots = num_sms * slots_per_sm;
	auto pick_cluster = [&](int rows) {
		int cl = 1;
		while (cl < 16 && (long long)rows * cl * 2 <= slots && minR / (cl * 2) >= 256) cl *= 2;
		return cl;
	};
	/* the initial solve's CTAs per row: as given, else as many as fill the GPU once */
	const int init_cluster = fields[0]->params.init_cluster;
	SolveArgs A;
	std::memset(&A, 0, sizeof(A));
	A.fields = P.views.ptr;
	A.outs = P.outs.ptr;
	A.star_hilo = P.hilo_ptrs.ptr;
	A.error = P.error.ptr;

	for (Field* f : fields) CCF_TRY(cudaEventRecord(f->ev[3], s), "event");
	if (verbose >= 1) std::cout << "Finding initial roots...\n";
	A.rows = P.rows_init.ptr;
	A.num_rows = (int)ri.size();
	A.cluster = init_cluster > 0 ? init_cluster : pick_cluster(A.num_rows);
	for (Field* f : fields) f->info.init_cluster = A.cluster;
	A.master = P.master_init.ptr;
	A.snap32 = mixed ? P.snap32_init.ptr : nullptr;
	A.snap64 = mixed ? nullptr : P.snap64_init.ptr;
	A.fin = P.fin_init.ptr;
	A.list = P.list_init.ptr;
	A.fval = P.fval_init.ptr;
	CCF_TRY(launch_solve(s, A, mixed, true), "find_initial_roots");
	for (Field* f : fields) CCF_TRY(cudaEventRecord(f->ev[4], s), "event");
	if (verbose >= 1) std::cout << "Finding critical curve positions...\n";
	A.rows = P.rows_cont.ptr;
	A.num_rows = (int)rc.size();
	A.cluster = pick_cluster(A.num_rows);
	A.master = P.master_cont.ptr;
	A.snap32 = mixed ? P.snap32_cont.ptr : nullptr;
	A.snap64 = mixed ? nullptr : P.snap64_cont.ptr;
	A.fin = P.fin_cont.ptr;
	A.list = P.list_cont.ptr;
	A.fval = P.fval_cont.ptr;
	bool reorder = false;
	if (track)
	{
		/* every root on its own path; rows that fail the column check run
		   again from their branch-centre roots with the full Aberth step */
		TrackArgs T;
		T.fields = P.views.ptr;
		T.outs = P.outs.ptr;
		T.rows = P.rows_cont.ptr;
		T.num_rows = (int)rc.size();
		T.master = P.master_cont.ptr;
		T.table = P.track_table.ptr;
		T.row_stats = P.row_stats.ptr;
		T.item_start = P.item_start.ptr;
		T.counter = P.rerun_count.ptr + 1;
		T.num_rows_dev = nullptr;
		T.items_per_row = 0;
		T.max_sub = TRACK_TSUB;
		T.num_items = 0;
		long long max_row_points = 0;   /* the column check's points of the longest row */
		for (size_t r = 0; r < rc.size(); r++)
		{
			item_start_host[r] = T.num_items;
			T.num_items += (fields[rc[r].field]->d.num_roots + 31) / 32;
			max_row_points = std::max(max_row_points, (long long)fields[rc[r].field]->d.num_roots * rc[r].steps);
		}
		CCF_TRY(cudaMemcpyAsync(P.item_start.ptr, item_start_host.data(), rc.size() * sizeof(int), cudaMemcpyHostToDevice, s),
			"upload");
		CCF_TRY(P.solo.ensure((size_t)ncont + 1), "cudaMalloc(rows)");
		CCF_TRY(P.is_solo.ensure((size_t)ncont), "cudaMalloc(rows)");
		T.solo = P.solo.ptr;
		T.num_solo = reinterpret_cast<int*>(P.solo.ptr + ncont);
		T.is_solo = P.is_solo.ptr;
		CCF_TRY(cudaMemsetAsync(T.num_solo, 0, sizeof(int), s), "memset");
		CCF_TRY(cudaMemsetAsync(P.track_table.ptr, 0, table_slots * sizeof(unsigned long long), s), "memset");
		CCF_TRY(cudaMemsetAsync(P.row_stats.ptr, 0, TRACK_ROW_STATS * rc.size() * sizeof(unsigned long long), s), "memset");
		CCF_TRY(cudaMemsetAsync(P.rerun_count.ptr, 0, 6 * sizeof(int), s), "memset");
		CCF_TRY(cudaMemsetAsync(P.row_stats2.ptr, 0, TRACK_ROW_STATS * rc.size() * sizeof(unsigned long long), s), "memset");
		CCF_TRY(P.item_order.ensure((size_t)T.num_items + 1), "cudaMalloc(items)");
		CCF_TRY(P.item_work.ensure(3 * (size_t)T.num_items + 3), "cudaMalloc(items)");
		/* long items first where the launch is a few waves of items, and its
		   last wave's length is a sizeable share of it (track_item_order_kernel) */
		reorder = (long long)T.num_items < 32LL * num_sms * TRACK_WARPS_PER_SM;
		T.item_order = reorder ? P.item_order.ptr : nullptr;
		CCF_TRY(launch_track_mark(s, T), "track_mark");
		if (reorder) CCF_TRY(launch_track_item_order(s, T, P.item_work.ptr, P.item_order.ptr), "track_item_order");
		CCF_TRY(launch_track(s, T, mixed), "track_ccs");
		CCF_TRY(launch_track_check(s, T, max_row_points), "track_check");
		CCF_TRY(launch_collect_rerun(s, T, P.rows_rerun.ptr, P.rerun_count.ptr), "collect_rerun");
		/* rows that failed: tracked again from their centre with sub-steps of at
		   most 1/TRACK_FINE_SUB of a phi step (the predictor's error falls as
		   the fifth power of the step), then the rows failing still go to the
		   full-sum solver; all on device-side row counts */
		TrackArgs T2 = T;
		T2.item_order = nullptr;
		T2.rows = P.rows_rerun.ptr;
		T2.num_rows_dev = P.rerun_count.ptr;
		T2.items_per_row = (maxR + 31) / 32;
		T2.num_items = (int)rc.size() * T2.items_per_row;
		T2.max_sub = TRACK_TSUB / TRACK_FINE_SUB;
		T2.row_stats = P.row_stats2.ptr;
		T2.counter = P.rerun_count.ptr + 4;
		CCF_TRY(launch_clear_tables(s, T2), "clear_tables");
		CCF_TRY(launch_track(s, T2, mixed), "track_ccs_fine");
		CCF_TRY(launch_track_check(s, T2, max_row_points), "track_check");
		CCF_TRY(launch_collect_rerun(s, T2, P.rows_rerun2.ptr, P.rerun_count.ptr + 3), "collect_rerun");
		A.rows = P.rows_rerun2.ptr;
		A.num_rows_dev = P.rerun_count.ptr + 3;
	}
	CCF_TRY(launch_solve(s, A, mixed, false), "find_ccs");
	/* FP64 polish of the points above the 1/mu target or left unconverged;
	   it also forms the largest 1/mu error and the non-finite flag */
	{
		long long max_points = 0, total_points = 0;
		for (Field* f : fields)
		{
			const long long n = (long long)f->d.num_roots * f->params.num_branches *
				(f->params.num_phi / f->params.num_branches + 1);
			max_points = std::max(max_points, n);
			total_points += n;
		}
		/* room for 1 in 128 points to be listed (points beyond it are polished
		   by the scan in place) */
		const long long cap = std::min(1LL << 24, std::max(1LL << 16, total_points / 128));
		CCF_TRY(P.polish_list.ensure((size_t)cap + 1), "cudaMalloc(polish)");
		CCF_TRY(cudaMemsetAsync(P.polish_list.ptr, 0, sizeof(unsigned long long), s), "memset");
		PolishArgs PA;
		PA.fields = P.views.ptr;
		PA.outs = P.outs.ptr;
		PA.num_fields = nf;
		PA.b0 = PA.nbs = PA.k0 = PA.nks = 0;
		PA.list_count = P.polish_list.ptr;
		PA.list = P.polish_list.ptr + 1;
		PA.list_cap = cap;
		for (Field* f : fields) CCF_TRY(cudaEventRecord(f->ev[6], s), "event");
		CCF_TRY(launch_polish(s, PA, max_points, num_sms), "polish");
	}
	for (Field* f : fields) CCF_TRY(cudaEventRecord(f->ev[5], s), "event");
	CCF_TRY(cudaStreamSynchronize(s), "solver");

	ccf_status status = CCF_OK;
	/* root seeds, initial solve, continuation (tracker: phase table, item
	   marking, item order (2), tracking, column check, row collection, table clearing,
	   re-tracking, column check, row collection and the full-sum launch for
	   the rows to re-run), FP64 polish; the launches are shared by the
	   batch's fields and counted with the first */
	for (int fi = 0; fi < nf; fi++)
	{
		ccf_status rc = finish_stats(*fields[fi], seg[fi], track, verbose, fi > 0 ? 0 : track ? (reorder ? 16 : 14) : 5);
		if (rc != CCF_OK) status = rc;
	}
	return status;
}

/* statistics and timings of a field's run into its info; the field is ran
   unless a 1/mu error is not finite */
ccf_status Engine::finish_stats(Field& f, int seg, bool track, int verbose, int launches)
{
	(void)track;
	unsigned long long st[STATS_WORDS];
	CCF_TRY(cudaMemcpy(st, f.stats.ptr, STATS_WORDS * sizeof(unsigned long long), cudaMemcpyDeviceToHost), "stats");
	ccf_info& info = f.info;
	double me;
	std::memcpy(&me, &st[STAT_POLISHED_MAX_ERR], sizeof(double));
	info.max_error = me;
	std::memcpy(&me, &st[0], sizeof(double));
	info.max_error_unpolished = me;
	info.has_nan = st[STAT_POLISHED_NAN] ? 1 : 0;
	info.root_updates = (long long)st[2];
	info.sum_terms = (long long)st[3];
	info.unconverged = (long long)st[STAT_POLISHED_UNCONV];
	info.unconverged_unpolished = (long long)st[4];
	info.points_polished = (long long)st[STAT_POLISHED];
	info.points_above_target = (long long)st[STAT_POLISHED_ABOVE];
	info.points_at_fp64_floor = (long long)st[STAT_POLISHED_FLOOR];
	info.max_sweeps_init = (int)st[5];
	info.max_sweeps_step = (int)st[6];
	info.root_updates_init = (long long)st[7];
	info.sum_terms_init = (long long)st[8];
	info.rows_rerun = (long long)st[9];
	info.step_halvings = (long long)st[10];
	info.rerun_flags = (long long)st[11];
	info.rows_retracked = (int)st[12];
	info.t_stars = ev_ms(f.ev[0], f.ev[1]) * 1e-3;
	info.t_tree = ev_ms(f.ev[1], f.ev[2]) * 1e-3;
	info.t_init_roots = ev_ms(f.ev[3], f.ev[4]) * 1e-3;
	info.t_ccs = ev_ms(f.ev[4], f.ev[6]) * 1e-3;
	info.t_caustics = ev_ms(f.ev[6], f.ev[5]) * 1e-3;
	info.t_total = ev_ms(f.ev[0], f.ev[5]) * 1e-3;
	info.kernel_launches += launches;
	info.centres_solved = f.params.num_branches / seg;
	ccf_status status = CCF_OK;
	if (info.has_nan)
	{
		f.error = "Error. Errors in 1/mu contain values which are not positive real numbers.";
		error = f.error;
		status = CCF_ERR_NUMERIC;
	}
	else
	{
		f.ran = true;
	}
	if (verbose >= 1)
	{
		std::cout << "Done finding critical curve positions. Elapsed time: " << info.t_init_roots + info.t_ccs << " seconds.\n";
		std::cout << "Maximum error in 1/mu: " << info.max_error << "\n";
	}
	return status;
}

/* Star field, tree, FMM and leaf records of every field of a run.  One
   field's setup is a chain of small launches with a few host round trips
   (the star statistics, every tree level), so a batch sets its fields up on
   SETUP_THREADS host threads (12: on the 16-core Grace host 8 give 342 ms
   per 256-field pass, 12 335, 16 333), each with a CUDA stream of its own: one
   field's round trips overlap the others' device work.  The solver's stream
   waits for every setup stream, and the setup streams for the solver's
   previous work on the same fields. */
constexpr int SETUP_THREADS = 12;
constexpr int SETUP_PARALLEL_MIN = 4;

/* setup threads: SETUP_THREADS, or the CCF_GB300_SETUP_THREADS environment
   variable (1 .. 64) */
static int setup_threads()
{
	static const int n = [] {
		const char* e = std::getenv("CCF_GB300_SETUP_THREADS");
		const int v = e ? std::atoi(e) : 0;
		return v >= 1 && v <= 64 ? v : SETUP_THREADS;
	}();
	return n;
}

bool batch_setup_fits(const Field& f);   /* batch.cu */

ccf_status Engine::prepare_fields(std::vector<Field*>& fields, int verbose)
{
	/* a batch of small fields is set up by the batched launches (batch.cu);
	   the others one by one, on setup threads when there are many */
	if (fields.size() >= 2)
	{
		std::vector<Field*> small, rest;
		for (Field* f : fields) (batch_setup_fits(*f) ? small : rest).push_back(f);
		if (small.size() >= 2)
		{
			/* the batched launches index fields by blockIdx.y: at most 65535 a launch */
			for (size_t i0 = 0; i0 < small.size(); i0 += 65535)
			{
				std::vector<Field*> part(small.begin() + i0, small.begin() + std::min(small.size(), i0 + 65535));
				ccf_status rc = part.size() >= 2 ? prepare_batch(part, verbose) : prepare_fields_each(part, verbose);
				if (rc != CCF_OK) return rc;
			}
			if (rest.empty()) return CCF_OK;
			return prepare_fields_each(rest, verbose);
		}
	}
	return prepare_fields_each(fields, verbose);
}

ccf_status Engine::prepare_fields_each(std::vector<Field*>& fields, int verbose)
{
	const int nf = (int)fields.size();
	const int T = nf >= SETUP_PARALLEL_MIN ? std::min(setup_threads(), nf) : 1;
	if (T == 1)
	{
		for (Field* f : fields)
		{
			ccf_status rc = prepare_field(*f, verbose);
			if (rc != CCF_OK)
			{
				f->error = error;
				return rc;
			}
		}
		return CCF_OK;
	}
	while ((int)setup_workers.size() < T)
	{
		auto w = std::make_unique<Engine>();
		if (!w->ensure_device(device))
		{
			error = w->error;
			return CCF_ERR_CUDA;
		}
		cudaEvent_t e;
		CCF_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
		setup_events.push_back(e);
		setup_workers.push_back(std::move(w));
	}
	/* the setup streams start after the solver's previous work */
	cudaEvent_t start = setup_events[0];
	CCF_TRY(cudaEventRecord(start, stream), "event");
	for (int t = 0; t < T; t++) CCF_TRY(cudaStreamWaitEvent(setup_workers[t]->stream, start, 0), "event");
	std::atomic<int> next{0};
	std::vector<ccf_status> st(nf, CCF_OK);
	std::vector<std::thread> threads;
	for (int t = 0; t < T; t++)
	{
		threads.emplace_back([&, t] {
			Engine& w = *setup_workers[t];
			cudaSetDevice(device);
			for (int i; (i = next++) < nf;)
			{
				st[i] = w.prepare_field(*fields[i], verbose);
				if (st[i] != CCF_OK) fields[i]->error = w.error;
			}
		});
	}
	for (auto& th : threads) th.join();
	/* the solver's stream waits for every setup stream */
	for (int t = 0; t < T; t++)
	{
		CCF_TRY(cudaEventRecord(setup_events[t], setup_workers[t]->stream), "event");
		CCF_TRY(cudaStreamWaitEvent(stream, setup_events[t], 0), "event");
	}
	for (int i = 0; i < nf; i++)
		if (st[i] != CCF_OK)
		{
			error = fields[i]->error;
			return st[i];
		}
	return CCF_OK;
}

ccf_status Engine::run(std::vector<Field*>& fields, int verbose)
{
	error.clear();
	if (fields.empty()) return CCF_OK;
	if (!ensure_device(fields[0]->params.device)) return CCF_ERR_NO_DEVICE;
	for (Field* f : fields)
	{
		f->ran = false;
		f->error.clear();
	}
	if (ccf_status rc = prepare_fields(fields, verbose); rc != CCF_OK) return rc;
	ccf_status rc = fields.size() == 1 && fields[0]->params.host_outputs == 2 ? solve_chunked(*fields[0], verbose)
	                                                                            : solve(fields, verbose);
	if (rc != CCF_OK)
	{
		for (Field* f : fields)
			if (f->error.empty()) f->error = error;
	}
	return rc;
}

/* device array -> page-locked host memory mapped into the device's address
   space, by the SMs: 16-byte loads and stores, every SM (on GB300 the stores
   cross NVLink-C2C as full lines, faster than the copy engines' DMA) */
__global__ void copy_to_host_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst, size_t n16)
{
	const size_t stride = (size_t)gridDim.x * blockDim.x;
	for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) dst[i] = __ldcs(src + i);
}

/* copy bytes from device memory to host memory dst: by the copy kernel when
   dst is page-locked, mapped and 16-byte aligned, else by cudaMemcpy */
cudaError_t Engine::copy_out(void* dst, const void* src, size_t bytes)
{
	cudaPointerAttributes a;
	const bool kernel = bytes >= (1u << 20) && ((uintptr_t)dst & 15) == 0 && ((uintptr_t)src & 15) == 0 && bytes % 16 == 0 &&
		cudaPointerGetAttributes(&a, dst) == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer != nullptr;
	cudaGetLastError();
	if (!kernel) return cudaMemcpy(dst, src, bytes, cudaMemcpyDefault);
	const int blocks = 4 * num_sms;
	copy_to_host_kernel<<<blocks, 256, 0, stream>>>((const uint4*)src, (uint4*)a.devicePointer, bytes / 16);
	cudaError_t e = cudaGetLastError();
	if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
	return e;
}

ccf_status Engine::copy_results(Field& f, double* ccs, double* caustics, double* errs, double* mu, double* stars)
{
	if (!f.ran) { error = "Error. No results: run() has not completed."; return CCF_ERR_NOT_RUN; }
	const size_t npts = (size_t)f.d.num_roots * f.params.num_branches * (f.params.num_phi / f.params.num_branches + 1);
	/* the outputs sit in device memory, or (host_outputs) page-locked host
	   memory, which a plain copy reads */
	auto copy = [&](void* dst, const void* src, size_t bytes) {
		return f.params.host_outputs ? cudaMemcpy(dst, src, bytes, cudaMemcpyDefault) : copy_out(dst, src, bytes);
	};
	if (caustics && !f.params.write_caustics)
	{
		error = "Error. Caustics were not requested (write_caustics = 0).";
		return CCF_ERR_INVALID_ARGUMENT;
	}
	if (mu && !f.params.write_mu_length_scales)
	{
		error = "Error. Length scales were not requested (write_mu_length_scales = 0).";
		return CCF_ERR_INVALID_ARGUMENT;
	}
	if (ccs) CCF_TRY(copy(ccs, f.out_ccs, npts * sizeof(double2)), "copy ccs");
	if (errs) CCF_TRY(copy(errs, f.out_errs, npts * sizeof(double)), "copy errs");
	if (caustics) CCF_TRY(copy(caustics, f.out_caustics, npts * sizeof(double2)), "copy caustics");
	if (mu) CCF_TRY(copy(mu, f.out_mu, npts * sizeof(double)), "copy mu");
	if (stars)
	{
		const int N = f.d.num_stars;
		std::vector<double2> pos(N);
		std::vector<double> mass(N);
		CCF_TRY(cudaMemcpy(pos.data(), f.star_pos.ptr, N * sizeof(double2), cudaMemcpyDeviceToHost), "copy stars");
		CCF_TRY(cudaMemcpy(mass.data(), f.star_mass.ptr, N * sizeof(double), cudaMemcpyDeviceToHost), "copy stars");
		for (int i = 0; i < N; i++)
		{
			stars[3 * i] = pos[i].x;
			stars[3 * i + 1] = pos[i].y;
			stars[3 * i + 2] = mass[i];
		}
	}
	return CCF_OK;
}

ccf_status Engine::save(Field& f, int verbose)
{
	if (!f.ran) { error = "Error. No results: run() has not completed."; return CCF_ERR_NOT_RUN; }
	const ccf_params& p = f.params;
	const std::string prefix = p.outfile_prefix;
	const bool single = p.output_float != 0;
	const int R = f.d.num_roots, nb = p.num_branches, cols = p.num_phi / nb + 1;
	const size_t npts = (size_t)R * nb * cols;
	if (verbose >= 2) std::cout << "Writing parameter info...\n";
	std::string fn = prefix + "ccf_parameter_info.txt";
	if (!write_parameter_info(fn, p, f.info, f.d.star_input))
	{
		error = "Error. Failed to open file " + fn;
		return CCF_ERR_IO;
	}
	if (verbose >= 1) std::cout << "Done writing parameter info to file " << fn << "\n";
	if (p.write_stars)
	{
		StarField sf;
		sf.n = f.d.num_stars;
		sf.rectangular = f.d.rectangular;
		sf.corner_x1 = f.d.corner_x1;
		sf.corner_x2 = f.d.corner_x2;
		sf.theta = f.d.theta;
		sf.xym.resize((size_t)3 * sf.n);
		ccf_status rc = copy_results(f, nullptr, nullptr, nullptr, nullptr, sf.xym.data());
		if (rc != CCF_OK) return rc;
		fn = prefix + "ccf_stars.bin";
		if (!write_star_file(fn, sf, single))
		{
			error = "Error. Unable to write star info to file " + fn;
			return CCF_ERR_IO;
		}
		if (verbose >= 1) std::cout << "Done writing star info to file " << fn << "\n";
	}
	std::vector<double> buf;
	if (p.write_critical_curves)
	{
		buf.resize(2 * npts);
		ccf_status rc = copy_results(f, buf.data(), nullptr, nullptr, nullptr, nullptr);
		if (rc != CCF_OK) return rc;
		fn = prefix + "ccf_ccs.bin";
		if (!write_array_complex(fn, buf.data(), R * nb, cols, single))
		{
			error = "Error. Unable to write ccs info to file " + fn;
			return CCF_ERR_IO;
		}
		if (verbose >= 1) std::cout << "Done writing critical curve positions to file " << fn << "\n";
	}
	if (p.write_caustics)
	{
		buf.resize(2 * npts);
		ccf_status rc = copy_results(f, nullptr, buf.data(), nullptr, nullptr, nullptr);
		if (rc != CCF_OK) return rc;
		fn = prefix + "ccf_caustics.bin";
		if (!write_array_complex(fn, buf.data(), R * nb, cols, single))
		{
			error = "Error. Unable to write caustic info to file " + fn;
			return CCF_ERR_IO;
		}
		if (verbose >= 1) std::cout << "Done writing caustic positions to file " << fn << "\n";
	}
	if (p.write_mu_length_scales)
	{
		buf.resize(npts);
		ccf_status rc = copy_results(f, nullptr, nullptr, nullptr, buf.data(), nullptr);
		if (rc != CCF_OK) return rc;
		fn = prefix + "ccf_mu_length_scales.bin";
		if (!write_array_real(fn, buf.data(), R * nb, cols, single))
		{
			error = "Error. Unable to write magnification length scales info to file " + fn;
			return CCF_ERR_IO;
		}
		if (verbose >= 1) std::cout << "Done writing magnification length scales to file " << fn << "\n";
	}
	return CCF_OK;
}

} /* namespace ccf */
