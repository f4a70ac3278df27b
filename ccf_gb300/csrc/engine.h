/******************************************************************************
engine.h -- host orchestration of one star field on the device (the role of
CCF<T>::run / save, include/ccf.cuh:1265-1287) and of batches of fields.
******************************************************************************/
#pragma once

#include "kernels.h"
#include "params.h"

#include <cuda_runtime.h>
#include <cstring>

#include <memory>
#include <string>
#include <vector>

namespace ccf
{

/* Device memory for DBuf: blocks that a released buffer gave back are kept
   per device and handed to later buffers of a fitting size instead of going
   through cudaFree, which synchronises the whole device -- with several
   requests running on their own streams (the server), every release would
   otherwise wait for the other requests' kernels.  A buffer is given back
   only once the work using it has finished (its field's last run event, its
   engine's stream).  When cudaMalloc fails, the kept blocks are freed and the
   allocation is retried. */
cudaError_t dmem_alloc(void** p, size_t bytes, size_t* got);
void dmem_release(void* p, size_t bytes);

/* grow-only device buffer: repeated runs of one configuration allocate once */
template <typename T>
struct DBuf
{
	T* ptr = nullptr;
	size_t cap = 0;
	size_t n = 0;
	DBuf() = default;
	DBuf(const DBuf&) = delete;
	DBuf& operator=(const DBuf&) = delete;
	~DBuf() { release(); }
	void release()
	{
		if (ptr) dmem_release(ptr, cap * sizeof(T));
		ptr = nullptr;
		cap = 0;
		n = 0;
	}
	cudaError_t ensure(size_t count)
	{
		n = count;
		if (count <= cap && ptr) return cudaSuccess;
		if (ptr) cudaFree(ptr);   /* growing in a run: the stream may still use it */
		ptr = nullptr;
		cap = 0;
		size_t bytes = std::max<size_t>(count, 1) * sizeof(T), got = 0;
		cudaError_t e = dmem_alloc((void**)&ptr, bytes, &got);
		if (e == cudaSuccess) cap = got / sizeof(T);
		else ptr = nullptr;
		n = count;
		return e;
	}
	/* grow keeping the first `keep` elements */
	cudaError_t grow(size_t count, size_t keep, cudaStream_t s)
	{
		if (count <= cap && ptr) { n = count; return cudaSuccess; }
		T* np = nullptr;
		size_t got = 0;
		cudaError_t e = dmem_alloc((void**)&np, count * sizeof(T), &got);
		if (e != cudaSuccess) return e;
		if (ptr && keep) cudaMemcpyAsync(np, ptr, keep * sizeof(T), cudaMemcpyDeviceToDevice, s);
		cudaStreamSynchronize(s);
		if (ptr) cudaFree(ptr);
		ptr = np;
		cap = got / sizeof(T);
		n = count;
		return cudaSuccess;
	}
	size_t bytes() const { return cap * sizeof(T); }
};

/* grow-only page-locked host buffer mapped into the device's address space:
   kernels write it through dev (the outputs with ccf_params.host_outputs) */
struct HostBuf
{
	void* ptr = nullptr;
	void* dev = nullptr;
	size_t cap = 0;
	HostBuf() = default;
	HostBuf(const HostBuf&) = delete;
	HostBuf& operator=(const HostBuf&) = delete;
	~HostBuf() { release(); }
	void release()
	{
		if (ptr) cudaFreeHost(ptr);
		ptr = dev = nullptr;
		cap = 0;
	}
	cudaError_t ensure(size_t bytes)
	{
		if (ptr && bytes <= cap) return cudaSuccess;
		release();
		cudaError_t e = cudaHostAlloc(&ptr, std::max<size_t>(bytes, 1), cudaHostAllocMapped | cudaHostAllocPortable);
		if (e != cudaSuccess)
		{
			ptr = nullptr;
			return e;
		}
		e = cudaHostGetDevicePointer(&dev, ptr, 0);
		if (e != cudaSuccess)
		{
			release();
			return e;
		}
		cap = bytes;
		return cudaSuccess;
	}
};

/* one field: parameters, derived values, device-resident star field, tree,
   FMM, leaf records and outputs */
struct Field
{
	ccf_params params;
	ccf_info info;
	Derived d;
	std::unique_ptr<StarField> user_stars;   /* set by ccf_set_stars */
	bool ran = false;
	std::string error;

	/* stars: generation order (seeds) and tree order */
	DBuf<double2> star_gen;
	DBuf<double2> star_pos, star_tmp_pos;
	DBuf<double> star_mass, star_tmp_mass;
	DBuf<float4> star_hilo;
	DBuf<float2> star_mass_df;
	DBuf<double> stats5;

	/* tree */
	DBuf<double2> n_center;
	DBuf<double> n_half;
	DBuf<int> n_level, n_parent, n_child, n_sstart, n_scount, n_nbr, n_nbrc, n_m2l, n_m2lc, n_p2l, n_p2lc, n_flag, n_rank;
	DBuf<int> level_out;   /* [max, nflag, err] */
	int node_cap = 0;
	int num_nodes = 0;
	bool tree_one_cta = false;   /* the last tree was built by tree_batch_kernel */
	std::vector<int> level_start, level_count;

	/* FMM and leaves */
	DBuf<double> binom;
	DBuf<double2> multi, local;
	DBuf<int> leaf_flag, leaf_index, node_leaf;
	DBuf<double2> leaf_center;
	DBuf<double> leaf_inv_half;
	DBuf<int> leaf_near_count;
	DBuf<NearStar> leaf_near;
	DBuf<double2> leaf_loc;
	DBuf<float2> leaf_loc3f;
	DBuf<float4> leaf_near_df, leaf_loc_df, leaf_loc_df_fold;
	DBuf<float2> leaf_mass_df, leaf_ih_df, leaf_loc3f_fold;
	DBuf<double2> leaf_loc_fold64;
	DBuf<unsigned char> leaf_fold;
	DBuf<double2> fold_coef;   /* the conjugated smooth-mass series in z, for the fold */
	int num_leaves = 0;

	/* smooth-mass polynomials */
	DBuf<double2> sm_d1, sm_d2, sm_a;
	DBuf<float2> sm_d2f;
	DBuf<float4> sm_d1_df, sm_a_df;

	/* device view */
	FieldView view;
	DBuf<FieldView> view_dev;

	/* phase of every whole phi step (tracker) */
	DBuf<PhaseEntry> phase;

	/* outputs, file layout: device buffers, or page-locked host buffers with
	   host_outputs; out_* point at the ones in use (device addresses) */
	DBuf<double2> ccs, caustics;
	DBuf<double> errs, mu;
	HostBuf h_ccs, h_caustics, h_errs, h_mu;
	double2* out_ccs = nullptr;
	double2* out_caustics = nullptr;
	double* out_errs = nullptr;
	double* out_mu = nullptr;
	DBuf<unsigned long long> stats;   /* solver statistics, 16 words (kernels.h, FieldOut::stats) */

	/* timing */
	cudaEvent_t ev[8] = {};
	bool events = false;

	~Field();
	TreeDev tree_dev() const;
};

/* solver row pools shared by the fields of a batch */
struct SolverPools
{
	DBuf<double2> master_init, master_cont, snap64_init, snap64_cont;
	DBuf<float4> snap32_init, snap32_cont;
	DBuf<unsigned char> fin_init, fin_cont;
	DBuf<int> list_init, list_cont;
	DBuf<double2> fval_init, fval_cont;   /* f, f' per root */
	DBuf<RowDesc> rows_init, rows_cont, rows_rerun, rows_rerun2;
	DBuf<unsigned long long> track_table;   /* column tables of the tracker */
	DBuf<unsigned long long> row_stats, row_stats2;   /* TRACK_ROW_STATS per row: tracking, re-tracking */
	DBuf<int> rerun_count;                  /* [0] rows to re-track, [1] [2] tracker work counters,
	                                           [3] rows to re-run, [4] [5] re-tracking work counters */
	DBuf<int> item_start;                   /* first tracker work item of each continuation row */
	DBuf<int2> solo;                        /* tracker roots run alone, and their count after them */
	DBuf<unsigned char> is_solo;            /* per continuation root */
	DBuf<unsigned long long> polish_list;   /* [0] count, then the points the FP64 polish works on */
	DBuf<FieldView> views;
	DBuf<FieldOut> outs;
	DBuf<const float4*> hilo_ptrs;
	DBuf<int> error;
	DBuf<SeedSeg> seeds;
	DBuf<int> item_order, item_work;   /* tracker: the queue order of the items, and its scratch */
};

/* small host-to-device copies collected for one copy of the packed bytes and
   one scatter launch (batch.cu flush_uploads): the sources are copied into
   the pack at once, so they need not outlive add() */
struct UploadPack
{
	struct Item
	{
		void* dst;
		size_t off, bytes;
	};
	std::vector<char> bytes;
	std::vector<Item> items;
	void add(void* dst, const void* src, size_t n)
	{
		const size_t off = (bytes.size() + 15) & ~(size_t)15;
		bytes.resize(off + n);
		std::memcpy(bytes.data() + off, src, n);
		items.push_back({dst, off, n});
	}
};

/* inside an Engine member returning ccf_status: a CUDA error becomes the
   engine's error message and CCF_ERR_CUDA */
#define CCF_TRY(expr, what)                              \
	do                                                   \
	{                                                    \
		cudaError_t _e = (expr);                         \
		if (_e != cudaSuccess) return cuda_fail(_e, what); \
	} while (0)

/* stars per field up to which a field's tree (and, in a batch, its whole
   setup) is built by one CTA (batch.cu) */
constexpr int BATCH_SETUP_MAX_STARS = 8192;

/* the root's half length (include/ccf.cuh:746) and the leaf limit: the
   reference's 32 unless leaf_max_stars lowers it */
inline double root_half_length(const Derived& d)
{
	const double rhl = d.rectangular ? std::max(d.corner_x1, d.corner_x2) : std::hypot(d.corner_x1, d.corner_x2);
	return rhl * 1.1;
}
inline int leaf_limit(const ccf_params& p)
{
	return p.leaf_max_stars > 0 ? std::min(p.leaf_max_stars, MAX_NEAR) : MAX_NEAR;
}

class Engine
{
public:
	Engine();
	~Engine();

	/* run a batch of fields (size 1 for ccf_run) */
	ccf_status run(std::vector<Field*>& fields, int verbose);
	ccf_status save(Field& f, int verbose);
	ccf_status copy_results(Field& f, double* ccs, double* caustics, double* errs, double* mu, double* stars);
	cudaError_t copy_out(void* dst, const void* src, size_t bytes);

	cudaStream_t stream = nullptr;
	int device = 0;
	int num_sms = 0;
	std::string error;

private:
	ccf_status prepare_fields(std::vector<Field*>& fields, int verbose);
	ccf_status prepare_fields_each(std::vector<Field*>& fields, int verbose);
	ccf_status prepare_field(Field& f, int verbose);
	ccf_status build_tree(Field& f, bool one_cta = true);
	ccf_status build_fmm(Field& f);
	cudaError_t tree_capacity(Field& f, int cap, int keep);
	ccf_status fmm_order(Field& f, int levels, int& P);
	ccf_status setup_begin(Field& f, int verbose);
	void setup_stats(Field& f, const double* st);
	ccf_status finish_view(Field& f, int P, double near_sum, int lerr, UploadPack* up = nullptr);
	ccf_status flush_uploads(UploadPack& up);
	ccf_status setup_outputs(Field& f);
	ccf_status prepare_batch(std::vector<Field*>& fields, int verbose);
	ccf_status solve(std::vector<Field*>& fields, int verbose);
	ccf_status solve_chunked(Field& f, int verbose);   /* stream.cu */
	int solved_seg(const Field& f, bool track) const;
	ccf_status finish_stats(Field& f, int seg, bool track, int verbose, int launches);
	ccf_status cuda_fail(cudaError_t e, const char* what);

public:
	bool ensure_device(int dev);

private:

	SolverPools pools;
	/* solve_chunked: the centre columns of the initial solve, two chunk
	   buffers of output windows, their FieldOut records, a copy stream and
	   its events */
	struct ChunkState
	{
		DBuf<double2> ctr_ccs, ctr_caus;
		DBuf<double> ctr_errs, ctr_mu;
		DBuf<double2> ccs[2], caus[2];
		DBuf<double> errs[2], mu[2];
		DBuf<FieldOut> outs;
		cudaStream_t copy = nullptr;
		cudaEvent_t ready = nullptr, copied[2] = {nullptr, nullptr}, done = nullptr;
	} chunk;
	/* batched setup: the fields' descriptors and their info words */
	DBuf<BatchSeg> batch_segs;
	DBuf<int> batch_info;
	DBuf<double> batch_stats;
	DBuf<double> batch_binom[2];   /* binomial tables: exact, the reference's int32 one */
	DBuf<char> upload_dev;         /* packed small uploads and their item list */
	HostBuf upload_host;
	/* batch setup: engines (their streams) of the setup threads, and events */
	std::vector<std::unique_ptr<Engine>> setup_workers;
	std::vector<cudaEvent_t> setup_events;
	bool initialized = false;
	int slots_per_sm = 1;
};

} /* namespace ccf */
