/******************************************************************************
batch.cu -- the setup of a batch of fields in a few launches.

The per-field setup (engine.cu prepare_field) runs a chain of small launches
per field: star generation, statistics, every tree level's flag, scan,
children, partition and neighbour passes, every level's FMM pass, the leaf
records -- ~50 launches and a dozen host round trips per field.  For a batch
of small fields the same work runs here with one CTA per field and a
handful of launches for the whole batch (stars_batch_kernel,
tree_batch_kernel, leaf_batch_kernel), each a loop over the per-field work
with block barriers where the per-field path has launch boundaries; the FMM
passes run level by level over every field at once (fmm_level_batch_kernel:
one warp per node, the fields side by side), as one CTA per field leaves
the FP64 translations of a level without the GPU's parallelism.  The kernels call the same node functions as the per-level
launches, so every field's tree, expansions and leaf records are bit for bit
those of the per-field path (tests/test_batch_gpu.py compares a batch with
its fields run one by one).  Host round trips: one after each launch, for
the whole batch.

A field the one-CTA build cannot take (more stars than BATCH_SETUP_MAX_STARS,
a tree deeper than its node capacity) runs the per-field path.
******************************************************************************/
#include "engine.h"

#include <cstring>
#include <iostream>

namespace ccf
{

/* the small arrays of a batch's fields from one packed copy: block i copies
   item i (8-byte words; every item is a whole number of them) */
struct UploadItem
{
	unsigned long long dst, off, bytes;
};
__global__ void scatter_uploads_kernel(const char* __restrict__ base, const UploadItem* __restrict__ items)
{
	const UploadItem it = items[blockIdx.x];
	const unsigned long long* src = reinterpret_cast<const unsigned long long*>(base + it.off);
	unsigned long long* dst = reinterpret_cast<unsigned long long*>(it.dst);
	for (unsigned long long i = threadIdx.x; i < it.bytes / 8; i += blockDim.x) dst[i] = src[i];
}

ccf_status Engine::flush_uploads(UploadPack& up)
{
	if (up.items.empty()) return CCF_OK;
	const size_t head = (up.bytes.size() + 15) & ~(size_t)15;
	const size_t total = head + up.items.size() * sizeof(UploadItem);
	CCF_TRY(upload_host.ensure(total), "cudaHostAlloc(uploads)");
	CCF_TRY(upload_dev.ensure(total), "cudaMalloc(uploads)");
	char* h = static_cast<char*>(upload_host.ptr);
	std::memcpy(h, up.bytes.data(), up.bytes.size());
	UploadItem* items = reinterpret_cast<UploadItem*>(h + head);
	for (size_t i = 0; i < up.items.size(); i++)
	{
		if (up.items[i].bytes % 8 != 0 || reinterpret_cast<uintptr_t>(up.items[i].dst) % 8 != 0)
		{
			error = "Error. Internal: an upload is not a whole number of 8-byte words.";
			return CCF_ERR_INVALID_ARGUMENT;
		}
		items[i] = {reinterpret_cast<unsigned long long>(up.items[i].dst), up.items[i].off, up.items[i].bytes};
	}
	CCF_TRY(cudaMemcpyAsync(upload_dev.ptr, h, total, cudaMemcpyHostToDevice, stream), "uploads");
	scatter_uploads_kernel<<<(unsigned)up.items.size(), 128, 0, stream>>>(upload_dev.ptr,
		reinterpret_cast<const UploadItem*>(upload_dev.ptr + head));
	CCF_TRY(cudaGetLastError(), "scatter_uploads_kernel");
	up.bytes.clear();
	up.items.clear();
	return CCF_OK;
}

/* a field with generated stars, or stars the caller set, of at most
   BATCH_SETUP_MAX_STARS (a star file is read only by the per-field path) */
bool batch_setup_fits(const Field& f)
{
	if (f.user_stars) return (long long)f.user_stars->xym.size() / 3 <= BATCH_SETUP_MAX_STARS;
	return !f.params.starfile[0] && f.params.num_stars <= BATCH_SETUP_MAX_STARS;
}

ccf_status Engine::prepare_batch(std::vector<Field*>& fields, int verbose)
{
	cudaStream_t s = stream;
	const int nf = (int)fields.size();
	auto fail = [&](Field& f, ccf_status rc) {
		f.error = error;
		return rc;
	};
	for (Field* f : fields)
	{
		ccf_status rc = setup_begin(*f, verbose);
		if (rc != CCF_OK) return fail(*f, rc);
	}
	CCF_TRY(batch_segs.ensure(nf), "cudaMalloc(batch)");
	CCF_TRY(batch_info.ensure((size_t)nf * BATCH_INFO_INTS), "cudaMalloc(batch)");
	CCF_TRY(batch_stats.ensure((size_t)nf * 8), "cudaMalloc(batch)");
	std::vector<BatchSeg> seg(nf);
	std::memset(seg.data(), 0, nf * sizeof(BatchSeg));
	std::vector<int> info((size_t)nf * BATCH_INFO_INTS);
	auto upload = [&]() {
		return cudaMemcpyAsync(batch_segs.ptr, seg.data(), nf * sizeof(BatchSeg), cudaMemcpyHostToDevice, s);
	};
	auto read_info = [&]() {
		cudaError_t e = cudaMemcpyAsync(info.data(), batch_info.ptr, info.size() * sizeof(int), cudaMemcpyDeviceToHost, s);
		return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
	};

	/* stars: generation (or the uploaded stars), the copy the tree reorders,
	   statistics; then every field's corner from its actual mean mass */
	for (int i = 0; i < nf; i++)
	{
		Field& f = *fields[i];
		const Derived& d = f.d;
		BatchSeg& g = seg[i];
		g.n = d.num_stars;
		g.gen = d.star_input ? 0 : 1;
		g.seed = d.random_seed;
		g.rectangular = d.rectangular;
		g.corner = make_double2(d.corner_x1, d.corner_x2);
		g.corner_abs = std::hypot(d.corner_x1, d.corner_x2);
		g.mt = make_mass_table(d.mass_kind, d.m_lower, d.m_upper, f.params.m_solar);
		g.star_gen = f.star_gen.ptr;
		g.pos = f.star_pos.ptr;
		g.mass = f.star_mass.ptr;
		g.tpos = f.star_tmp_pos.ptr;
		g.tmass = f.star_tmp_mass.ptr;
		g.stats5 = batch_stats.ptr + 8 * (size_t)i;
		g.info = batch_info.ptr + (size_t)i * BATCH_INFO_INTS;
	}
	CCF_TRY(upload(), "upload(batch)");
	launch_stars_batch(s, batch_segs.ptr, nf);
	CCF_TRY(cudaGetLastError(), "stars_batch_kernel");
	{
		std::vector<double> st((size_t)nf * 8);
		CCF_TRY(cudaMemcpyAsync(st.data(), batch_stats.ptr, st.size() * sizeof(double), cudaMemcpyDeviceToHost, s), "star stats");
		CCF_TRY(cudaStreamSynchronize(s), "star stats");
		for (int i = 0; i < nf; i++) setup_stats(*fields[i], st.data() + 8 * (size_t)i);
	}
	for (Field* f : fields) CCF_TRY(cudaEventRecord(f->ev[1], s), "event");

	/* trees */
	for (int i = 0; i < nf; i++)
	{
		Field& f = *fields[i];
		const int cap = std::max(1024, 2 * f.d.num_stars + 64);
		if (f.node_cap < cap) CCF_TRY(tree_capacity(f, cap, 0), "cudaMalloc(tree)");
		f.info.root_half_length = root_half_length(f.d);
		BatchSeg& g = seg[i];
		g.T = f.tree_dev();
		g.node_cap = f.node_cap;
		g.limit = leaf_limit(f.params);
		g.root_half = f.info.root_half_length;
	}
	CCF_TRY(upload(), "upload(batch)");
	launch_tree_batch(s, batch_segs.ptr, nf);
	CCF_TRY(cudaGetLastError(), "tree_batch_kernel");
	CCF_TRY(read_info(), "tree_batch_kernel");
	std::vector<char> alone(nf, 0);   /* fields whose tree outgrew the one-CTA build */
	for (int i = 0; i < nf; i++)
	{
		Field& f = *fields[i];
		const int* fi = info.data() + (size_t)i * BATCH_INFO_INTS;
		if (fi[2] & 1)
		{
			error = "Error. Tree neighbour list overflow.";
			return fail(f, CCF_ERR_NUMERIC);
		}
		if (fi[2] & 2)
		{
			alone[i] = 1;
			continue;
		}
		const int levels = fi[0];
		f.level_start.assign(fi + 3, fi + 3 + levels + 1);
		f.level_count.assign(fi + 3 + TREE_MAX_LEVELS + 1, fi + 3 + TREE_MAX_LEVELS + 1 + levels + 1);
		f.num_nodes = fi[1];
		f.info.leaf_max_stars = seg[i].limit;
	}

	/* FMM passes and leaf numbering; the binomial tables (the entries do not
	   depend on the table's size) once per kind for the largest order */
	std::vector<int> order(nf, 0);
	int maxP[2] = {0, 0};
	for (int i = 0; i < nf; i++)
	{
		if (alone[i]) continue;
		Field& f = *fields[i];
		const int levels = (int)f.level_start.size() - 1;
		ccf_status rc = fmm_order(f, levels, order[i]);
		if (rc != CCF_OK) return fail(f, rc);
		int& m = maxP[f.params.exact_binomials ? 0 : 1];
		m = std::max(m, order[i]);
	}
	for (int k = 0; k < 2; k++)
		if (maxP[k] > 0)
		{
			std::vector<double> B = binomial_table(2 * maxP[k], k == 1);
			CCF_TRY(batch_binom[k].ensure(B.size()), "cudaMalloc(binomials)");
			CCF_TRY(cudaMemcpyAsync(batch_binom[k].ptr, B.data(), B.size() * sizeof(double), cudaMemcpyHostToDevice, s),
				"binomials");
		}
	for (int i = 0; i < nf; i++)
	{
		if (alone[i]) continue;
		Field& f = *fields[i];
		const int P = order[i];
		const size_t nc = (size_t)f.num_nodes * (P + 1);
		CCF_TRY(f.multi.ensure(nc), "cudaMalloc(multipole)");
		CCF_TRY(f.local.ensure(nc), "cudaMalloc(local)");
		CCF_TRY(f.leaf_flag.ensure(f.num_nodes), "cudaMalloc(leaves)");
		CCF_TRY(f.leaf_index.ensure(f.num_nodes), "cudaMalloc(leaves)");
		CCF_TRY(f.node_leaf.ensure(f.num_nodes), "cudaMalloc(leaves)");
		BatchSeg& g = seg[i];
		g.T = f.tree_dev();
		g.P = P;
		g.B = batch_binom[f.params.exact_binomials ? 0 : 1].ptr;
		g.multi = f.multi.ptr;
		g.local = f.local.ptr;
		g.leaf_flag = f.leaf_flag.ptr;
		g.leaf_index = f.leaf_index.ptr;
	}
	/* the fields that run alone are left out of the batch launches */
	std::vector<BatchSeg> packed;
	std::vector<int> slot(nf, -1);
	for (int i = 0; i < nf; i++)
		if (!alone[i])
		{
			slot[i] = (int)packed.size();
			packed.push_back(seg[i]);
		}
	const int nb = (int)packed.size();
	auto upload_packed = [&]() {
		for (int i = 0; i < nf; i++)
			if (slot[i] >= 0) packed[slot[i]] = seg[i];
		return cudaMemcpyAsync(batch_segs.ptr, packed.data(), nb * sizeof(BatchSeg), cudaMemcpyHostToDevice, s);
	};
	/* this batch's launches: stars, tree, the FMM's zeroing, levels and leaf
	   numbering, leaf records, the uploads' scatter */
	int launches = 2;
	if (nb > 0)
	{
		int max_levels = 0, max_level_nodes = 0;
		long long max_coef = 0;
		for (int i = 0; i < nf; i++)
		{
			if (alone[i]) continue;
			const Field& f = *fields[i];
			max_levels = std::max(max_levels, (int)f.level_start.size() - 1);
			for (int c : f.level_count) max_level_nodes = std::max(max_level_nodes, c);
			max_coef = std::max(max_coef, (long long)f.num_nodes * (order[i] + 1));
		}
		CCF_TRY(upload_packed(), "upload(batch)");
		launch_fmm_batch(s, batch_segs.ptr, nb, max_levels, max_level_nodes, max_coef);
		launches += 2 + (max_levels + 1) + std::max(0, max_levels - 1) + 1 + 1;
		CCF_TRY(cudaGetLastError(), "fmm_batch_kernel");
		CCF_TRY(read_info(), "fmm_batch_kernel");
	}

	/* leaf records */
	for (int i = 0; i < nf; i++)
	{
		if (alone[i]) continue;
		Field& f = *fields[i];
		const int* fi = info.data() + (size_t)i * BATCH_INFO_INTS;
		const int nl = fi[LEAF_INFO];
		const int P = order[i];
		f.num_leaves = nl;
		CCF_TRY(f.leaf_center.ensure(nl), "cudaMalloc(leaves)");
		CCF_TRY(f.leaf_inv_half.ensure(nl), "cudaMalloc(leaves)");
		CCF_TRY(f.leaf_near_count.ensure(nl), "cudaMalloc(leaves)");
		CCF_TRY(f.leaf_near.ensure((size_t)nl * MAX_NEAR), "cudaMalloc(leaves)");
		CCF_TRY(f.leaf_loc.ensure((size_t)nl * 3 * (P + 1)), "cudaMalloc(leaves)");
		CCF_TRY(f.leaf_loc3f.ensure((size_t)nl * (P + 1)), "cudaMalloc(leaves)");
		BatchSeg& g = seg[i];
		g.theta2 = f.d.theta * f.d.theta;
		g.num_leaves = nl;
		g.leaf_center = f.leaf_center.ptr;
		g.leaf_inv_half = f.leaf_inv_half.ptr;
		g.leaf_near_count = f.leaf_near_count.ptr;
		g.leaf_near = f.leaf_near.ptr;
		g.leaf_loc = f.leaf_loc.ptr;
		g.leaf_loc3f = f.leaf_loc3f.ptr;
		g.node_leaf = f.node_leaf.ptr;
		if (f.params.precision == CCF_PRECISION_MIXED)
		{
			CCF_TRY(f.leaf_near_df.ensure((size_t)nl * MAX_NEAR), "cudaMalloc(leaves)");
			CCF_TRY(f.leaf_mass_df.ensure((size_t)nl * MAX_NEAR), "cudaMalloc(leaves)");
			CCF_TRY(f.leaf_loc_df.ensure((size_t)nl * 2 * (P + 1)), "cudaMalloc(leaves)");
			CCF_TRY(f.leaf_ih_df.ensure(nl), "cudaMalloc(leaves)");
			CCF_TRY(f.star_hilo.ensure(f.d.num_stars), "cudaMalloc(star hilo)");
			CCF_TRY(f.star_mass_df.ensure(f.d.num_stars), "cudaMalloc(star hilo)");
			g.leaf_near_df = f.leaf_near_df.ptr;
			g.leaf_mass_df = f.leaf_mass_df.ptr;
			g.leaf_loc_df = f.leaf_loc_df.ptr;
			g.leaf_ih_df = f.leaf_ih_df.ptr;
			g.star_hilo = f.star_hilo.ptr;
			g.star_mass_df = f.star_mass_df.ptr;
		}
	}
	if (nb > 0)
	{
		CCF_TRY(upload_packed(), "upload(batch)");
		launch_leaf_batch(s, batch_segs.ptr, nb);
		CCF_TRY(cudaGetLastError(), "leaf_batch_kernel");
		CCF_TRY(read_info(), "leaf_batch_kernel");
	}

	/* smooth-mass polynomials, folds, device views, outputs; the fields that
	   run alone take the per-field path from their tree on */
	UploadPack up;
	for (int i = 0; i < nf; i++)
	{
		Field& f = *fields[i];
		ccf_status rc;
		if (alone[i])
		{
			rc = build_tree(f, false);
			if (rc == CCF_OK) rc = build_fmm(f);
		}
		else
		{
			const int* fi = info.data() + (size_t)i * BATCH_INFO_INTS;
			rc = finish_view(f, order[i], (double)fi[LEAF_INFO + 1], fi[LEAF_INFO + 2], &up);
		}
		if (rc != CCF_OK) return fail(f, rc);
		CCF_TRY(cudaEventRecord(f.ev[2], s), "event");
		rc = setup_outputs(f);
		if (rc != CCF_OK) return fail(f, rc);
		/* the batch's launches are counted once, with its first field; a
		   field's fold is its own launch */
		if (!alone[i]) f.info.kernel_launches = (i == 0 ? launches : 0) + (f.info.leaves_folded > 0 ? 1 : 0);
	}
	ccf_status rc = flush_uploads(up);
	if (rc != CCF_OK) return rc;
	if (verbose >= 1) std::cout << "Done setting up " << nf << " fields.\n";
	return CCF_OK;
}

} /* namespace ccf */
