/******************************************************************************
autotune.cpp -- the autotuner of the solver settings, and its cache.

ccf_autotune times candidate settings on the handle's own field (whole
runs, CUDA-event spans, best of two after a warm-up run) by coordinate
descent from the library's defaults:

  * init_cluster: CTAs per branch-centre row of the initial Aberth solve
    (1, 2, 4, 8, 16);
  * solved_centres: branch centres solved by the initial Aberth solve, the
    others reached by tracking (the default's count, half and twice it);
  * with fmm = 1 also leaf_max_stars (24, 16, 12) and expansion_order (the
    default's order -1, -2, -3).

A candidate is kept only if it is faster and its run is as good as the
default's: no non-finite 1/mu error, no more unconverged points and no more
points above the 1/mu target; an FMM candidate must also keep the far-field
error (ccf_fmm_error) within alpha_error = 1e-7 theta_star or within the
default's own error, whichever is larger.  FMM candidates change the far
field within that target and so move the roots by up to ~1e-7 theta_star
from the reference's FMM (the reference's own expansion order and leaf rule
are the default); the other settings change only the order of floating-point
sums.

The result is cached per field shape -- GPU (SM count), precision,
continuation, geometry, smooth-mass form, num_branches, and buckets of
num_stars and of the phi steps per branch (quarter and half octaves) -- in
memory and in a text file ($CCF_GB300_AUTOTUNE_CACHE, else
$XDG_CACHE_HOME/ccf_gb300/autotune.txt, else ~/.cache/ccf_gb300/autotune.txt;
a file that cannot be written leaves the memory cache).  ccf_run with
ccf_params.autotune set applies the cached settings of the field's shape,
tuning on a miss.
******************************************************************************/
#include "../../include/ccf_gb300.h"
#include "engine.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <limits>
#include <map>
#include <mutex>
#include <sstream>
#include <string>

ccf::Field* ccf_internal_field(ccf_handle* h);
ccf::Engine* ccf_internal_engine(ccf_handle* h);
void ccf_internal_set_error(ccf_handle* h, const std::string& msg);

namespace
{

struct Tuned
{
	int init_cluster = 0, solved_centres = 0, leaf_max_stars = 0, expansion_order = 0;
	double seconds = 0;
};

std::mutex g_mu;
std::map<std::string, Tuned> g_cache;
bool g_loaded = false;

std::string cache_path()
{
	if (const char* e = std::getenv("CCF_GB300_AUTOTUNE_CACHE"); e && *e) return e;
	if (const char* x = std::getenv("XDG_CACHE_HOME"); x && *x) return std::string(x) + "/ccf_gb300/autotune.txt";
	if (const char* h = std::getenv("HOME"); h && *h) return std::string(h) + "/.cache/ccf_gb300/autotune.txt";
	return "";
}

/* file lines: key words ... | init_cluster solved_centres leaf order seconds */
void load_cache()
{
	if (g_loaded) return;
	g_loaded = true;
	const std::string path = cache_path();
	if (path.empty()) return;
	std::ifstream in(path);
	std::string line;
	while (std::getline(in, line))
	{
		const size_t bar = line.find('|');
		if (bar == std::string::npos) continue;
		std::istringstream vs(line.substr(bar + 1));
		Tuned t;
		if (vs >> t.init_cluster >> t.solved_centres >> t.leaf_max_stars >> t.expansion_order >> t.seconds)
		{
			std::string key = line.substr(0, bar);
			while (!key.empty() && key.back() == ' ') key.pop_back();
			g_cache[key] = t;
		}
	}
}

void store_cache(const std::string& key, const Tuned& t)
{
	g_cache[key] = t;
	const std::string path = cache_path();
	if (path.empty()) return;
	std::error_code ec;
	std::filesystem::create_directories(std::filesystem::path(path).parent_path(), ec);
	std::ofstream out(path, std::ios::app);
	if (!out) return;
	out << key << " | " << t.init_cluster << ' ' << t.solved_centres << ' ' << t.leaf_max_stars << ' '
	    << t.expansion_order << ' ' << t.seconds << '\n';
}

int sm_count(int device)
{
	int n = 0;
	if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
	return n;
}

std::string shape_key(const ccf_params& p, int num_stars, int fmm)
{
	const int nb = p.num_branches, half = p.num_phi / (2 * std::max(1, nb));
	char buf[256];
	std::snprintf(buf, sizeof(buf), "v1 sms=%d prec=%d cont=%d rect=%d approx=%d nb=%d halfbin=%ld nbin=%ld fmm=%d",
		sm_count(p.device), p.precision, p.continuation, p.rectangular, p.approx, nb,
		std::lround(2 * std::log2((double)std::max(1, half))), std::lround(4 * std::log2((double)std::max(1, num_stars))),
		fmm);
	return buf;
}

/* run the handle's field with p: a warm-up run, then the best of two;
   false when a run fails */
bool trial(ccf_handle* h, const ccf_params& p, double& seconds, ccf_info& info)
{
	ccf_set_params(h, &p);
	if (ccf_run(h, -1) != CCF_OK) return false;
	seconds = std::numeric_limits<double>::infinity();
	for (int k = 0; k < 2; k++)
	{
		if (ccf_run(h, -1) != CCF_OK) return false;
		ccf_get_info(h, &info);
		seconds = std::min(seconds, info.t_total);
	}
	return true;
}

} /* namespace */

extern "C" ccf_status ccf_autotune(ccf_handle* h, int fmm, int verbose, ccf_params* best, double* best_seconds)
{
	if (!h || (fmm != 0 && fmm != 1)) return CCF_ERR_INVALID_ARGUMENT;
	ccf_params user;
	ccf_get_params(h, &user);
	ccf_params base = user;
	base.autotune = 0;
	base.init_cluster = 0;
	base.solved_centres = 0;
	base.leaf_max_stars = 0;
	base.expansion_order = 0;

	double t_base;
	ccf_info ib;
	if (!trial(h, base, t_base, ib))
	{
		ccf_set_params(h, &user);
		return CCF_ERR_CUDA;
	}
	double e_base = 0;
	if (fmm) ccf_fmm_error(h, &e_base);
	const double e_limit = std::max(ib.alpha_error, e_base);
	const int P_base = ib.expansion_order;

	ccf_params cur = base;
	double t_cur = t_base;
	auto accept = [&](const ccf_params& p, bool fmm_candidate) {
		double t;
		ccf_info info;
		if (!trial(h, p, t, info)) return;
		if (info.has_nan || info.unconverged > ib.unconverged || info.points_above_target > ib.points_above_target) return;
		if (fmm_candidate)
		{
			double e = 0;
			if (ccf_fmm_error(h, &e) != CCF_OK || !(e <= e_limit)) return;
		}
		if (verbose >= 1)
			std::printf("autotune: init_cluster %d solved_centres %d leaf %d order %d: %.3f ms\n", p.init_cluster,
				p.solved_centres, p.leaf_max_stars, p.expansion_order, 1e3 * t);
		if (t < 0.99 * t_cur)
		{
			cur = p;
			t_cur = t;
		}
	};
	for (int cl : {1, 2, 4, 8, 16})
	{
		ccf_params p = cur;
		p.init_cluster = cl;
		accept(p, false);
	}
	if (base.continuation == CCF_CONTINUATION_TRACK)
	{
		const int nb = base.num_branches, K = ib.centres_solved;
		for (int k : {K / 2, 2 * K})
		{
			if (k < 1 || k > nb || nb % k != 0 || nb / k > 16 || k == K) continue;
			ccf_params p = cur;
			p.solved_centres = k;
			accept(p, false);
		}
	}
	if (fmm)
	{
		for (int leaf : {24, 16, 12})
		{
			ccf_params p = cur;
			p.leaf_max_stars = leaf;
			accept(p, true);
		}
		for (int d : {1, 2, 3})
		{
			if (P_base - d < 3) break;
			ccf_params p = cur;
			p.expansion_order = P_base - d;
			accept(p, true);
		}
	}
	ccf_params out = user;
	out.init_cluster = cur.init_cluster;
	out.solved_centres = cur.solved_centres;
	out.leaf_max_stars = cur.leaf_max_stars;
	out.expansion_order = cur.expansion_order;
	{
		std::lock_guard<std::mutex> lock(g_mu);
		load_cache();
		Tuned t;
		t.init_cluster = cur.init_cluster;
		t.solved_centres = cur.solved_centres;
		t.leaf_max_stars = cur.leaf_max_stars;
		t.expansion_order = cur.expansion_order;
		t.seconds = t_cur;
		store_cache(shape_key(user, ib.num_stars, fmm), t);
	}
	/* the handle keeps the caller's parameters (its results are the last trial's) */
	ccf_set_params(h, &user);
	if (best) *best = out;
	if (best_seconds) *best_seconds = t_cur;
	return CCF_OK;
}

/* ccf_run with ccf_params.autotune: the cached settings of the field's
   shape, tuned on a miss; returns false when tuning failed */
bool ccf_internal_autotune_apply(ccf_handle* h)
{
	ccf::Field& f = *ccf_internal_field(h);
	const ccf_params p = f.params;
	const int fmm = p.autotune == 2 ? 1 : 0;
	int n = p.num_stars;
	if (f.user_stars) n = f.user_stars->n;
	const std::string key = shape_key(p, n, fmm);
	Tuned t;
	bool hit;
	{
		std::lock_guard<std::mutex> lock(g_mu);
		load_cache();
		auto it = g_cache.find(key);
		hit = it != g_cache.end();
		if (hit) t = it->second;
	}
	if (!hit)
	{
		ccf_params best;
		if (ccf_autotune(h, fmm, 0, &best, nullptr) != CCF_OK) return false;
		t.init_cluster = best.init_cluster;
		t.solved_centres = best.solved_centres;
		t.leaf_max_stars = best.leaf_max_stars;
		t.expansion_order = best.expansion_order;
	}
	ccf_params q = p;
	q.init_cluster = t.init_cluster;
	q.solved_centres = (t.solved_centres > 0 && p.num_branches % t.solved_centres == 0) ? t.solved_centres : 0;
	if (fmm)
	{
		q.leaf_max_stars = t.leaf_max_stars;
		q.expansion_order = t.expansion_order;
	}
	ccf_set_params(h, &q);
	return true;
}
