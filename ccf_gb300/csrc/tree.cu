/******************************************************************************
tree.cu -- level-by-level quadtree build on the device.

Same tree as the reference (include/ccf.cuh:781-829, include/tree_node.cuh):
a node is split when its own stars plus its neighbours' exceed 32 (the
reference's rule; ccf_params.leaf_max_stars may lower the limit); children
are the four quadrants in the order (+,+), (-,+), (-,-), (+,-); neighbour,
same-level interaction (M2L) and coarser-leaf interaction (P2L) lists follow
the reference's distance rules.  Unlike the reference, the build is
deterministic: children are placed by an exclusive scan of the split flags
(not atomicSub), and each node's stars are split by a stable warp-ballot
partition (not shared-memory atomics), so repeated runs give identical
star order and identical floating-point sums.
******************************************************************************/
#include "kernels.h"

namespace ccf
{

/* split flag of node n: its stars and its neighbours' exceed the limit
   (tree_node.cuh:321-345); returns that neighbourhood count */
CCF_D int tree_flag_node(const TreeDev& T, int n, int limit, int& flag)
{
	int ns = T.star_count[n];
	const int k = T.nbr_count[n];
	for (int j = 0; j < k; j++) ns += T.star_count[T.nbr[n * MAX_NBR + j]];
	flag = ns > limit;
	T.flag[n] = flag;
	return ns;
}

/* per-level split flags, and the level's max neighbourhood count and number
   of split nodes */
__global__ void tree_flag_kernel(TreeDev T, int start, int count, int limit, int* out)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	int ns = 0, flag = 0;
	if (i < count) ns = tree_flag_node(T, start + i, limit, flag);
	/* warp-aggregated, order-independent integer atomics */
	unsigned full = 0xffffffffu;
	int mx = ns, cnt = flag;
	for (int o = 16; o > 0; o >>= 1)
	{
		mx = max(mx, __shfl_xor_sync(full, mx, o));
		cnt += __shfl_xor_sync(full, cnt, o);
	}
	if ((threadIdx.x & 31) == 0)
	{
		atomicMax(&out[0], mx);
		atomicAdd(&out[1], cnt);
	}
}

__global__ void __launch_bounds__(1024) scan_kernel(const int* __restrict__ in, int* __restrict__ out, int n)
{
	block_exclusive_scan(in, out, n);
}

CCF_D void tree_root_node(const TreeDev& T, double half, int nstars)
{
	T.center[0] = make_double2(0, 0);
	T.half[0] = half;
	T.level[0] = 0;
	T.parent[0] = -1;
	T.child[0] = -1;
	T.star_start[0] = 0;
	T.star_count[0] = nstars;
	T.nbr_count[0] = 0;
	T.m2l_count[0] = 0;
	T.p2l_count[0] = 0;
}

__global__ void tree_root_kernel(TreeDev T, double half, int nstars)
{
	tree_root_node(T, half, nstars);
}

/* children of split node n (tree_node.cuh:151-177, 355-381) */
CCF_D void tree_children_node(const TreeDev& T, int n, int child_start)
{
	if (!T.flag[n]) return;
	int base = child_start + 4 * T.rank[n];
	T.child[n] = base;
	double h = T.half[n] / 2;
	double2 c = T.center[n];
	const double ox[4] = {1, -1, -1, 1}, oy[4] = {1, 1, -1, -1};
	for (int q = 0; q < 4; q++)
	{
		int k = base + q;
		T.center[k] = make_double2(c.x + h * ox[q], c.y + h * oy[q]);
		T.half[k] = h;
		T.level[k] = T.level[n] + 1;
		T.parent[k] = n;
		T.child[k] = -1;
		T.star_start[k] = T.star_start[n];
		T.star_count[k] = 0;
		T.nbr_count[k] = 0;
		T.m2l_count[k] = 0;
		T.p2l_count[k] = 0;
	}
}

__global__ void tree_children_kernel(TreeDev T, int start, int count, int child_start)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < count) tree_children_node(T, start + i, child_start);
}

/* stable split of split node n's stars into its four quadrants by one warp
   (all 32 lanes call it; replaces the atomic two-pass sort of
   tree_node.cuh:392-501) */
CCF_D void tree_partition_node(const TreeDev& T, int n, int lane, double2* __restrict__ pos, double* __restrict__ mass,
	double2* __restrict__ tpos, double* __restrict__ tmass)
{
	if (!T.flag[n]) return;
	int s = T.star_start[n], ns = T.star_count[n];
	if (ns == 0) return;
	double2 c = T.center[n];
	const unsigned full = 0xffffffffu;
	int cnt[4] = {0, 0, 0, 0};
	for (int b = 0; b < ns; b += 32)
	{
		int i = b + lane;
		int q = 4;
		if (i < ns)
		{
			double2 p = pos[s + i];
			q = (p.y >= c.y) ? ((p.x >= c.x) ? 0 : 1) : ((p.x < c.x) ? 2 : 3);
		}
		for (int k = 0; k < 4; k++) cnt[k] += __popc(__ballot_sync(full, q == k));
	}
	int off[4] = {0, cnt[0], cnt[0] + cnt[1], cnt[0] + cnt[1] + cnt[2]};
	int run[4] = {off[0], off[1], off[2], off[3]};
	unsigned lt = (1u << lane) - 1u;
	for (int b = 0; b < ns; b += 32)
	{
		int i = b + lane;
		int q = 4;
		double2 p = make_double2(0, 0);
		double m = 0;
		if (i < ns)
		{
			p = pos[s + i];
			m = mass[s + i];
			q = (p.y >= c.y) ? ((p.x >= c.x) ? 0 : 1) : ((p.x < c.x) ? 2 : 3);
		}
		for (int k = 0; k < 4; k++)
		{
			unsigned msk = __ballot_sync(full, q == k);
			if (q == k)
			{
				int dst = s + run[k] + __popc(msk & lt);
				tpos[dst] = p;
				tmass[dst] = m;
			}
			run[k] += __popc(msk);
		}
	}
	__syncwarp();
	for (int i = lane; i < ns; i += 32)
	{
		pos[s + i] = tpos[s + i];
		mass[s + i] = tmass[s + i];
	}
	if (lane < 4)
	{
		int k = T.child[n] + lane;
		T.star_start[k] = s + off[lane];
		T.star_count[k] = cnt[lane];
	}
}

__global__ void tree_partition_kernel(TreeDev T, int start, int count, double2* __restrict__ pos, double* __restrict__ mass,
	double2* __restrict__ tpos, double* __restrict__ tmass)
{
	int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	if (w >= count) return;   /* warp-uniform */
	tree_partition_node(T, start + w, threadIdx.x & 31, pos, mass, tpos, tmass);
}

/* neighbour and interaction lists of node n of a new level
   (tree_node.cuh:183-267); returns true when a list overflowed */
CCF_D bool tree_neighbors_node(const TreeDev& T, int n)
{
	if (T.level[n] == 0) return false;
	int p = T.parent[n];
	double h = T.half[n];
	double2 c = T.center[n];
	int nn = 0, nm = 0, np = 0;
	bool overflow = false;
	int pc = T.child[p];
	for (int q = 0; q < 4; q++)
	{
		int x = pc + q;
		if (T.star_count[x] == 0 || x == n) continue;
		if (nn < MAX_NBR) T.nbr[n * MAX_NBR + nn++] = x;
		else overflow = true;
	}
	int pn = T.nbr_count[p];
	for (int j = 0; j < pn; j++)
	{
		int nb = T.nbr[p * MAX_NBR + j];
		if (T.star_count[nb] == 0) continue;
		int nbc = T.child[nb];
		if (nbc < 0)
		{
			double2 d = T.center[nb];
			if (fabs(d.x - c.x) < 3.5 * h && fabs(d.y - c.y) < 3.5 * h)
			{
				if (nn < MAX_NBR) T.nbr[n * MAX_NBR + nn++] = nb;
				else overflow = true;
			}
			else
			{
				if (np < MAX_P2L) T.p2l[n * MAX_P2L + np++] = nb;
				else overflow = true;
			}
		}
		else
		{
			for (int q = 0; q < 4; q++)
			{
				int x = nbc + q;
				if (T.star_count[x] == 0) continue;
				double2 d = T.center[x];
				if (fabs(d.x - c.x) < 3 * h && fabs(d.y - c.y) < 3 * h)
				{
					if (nn < MAX_NBR) T.nbr[n * MAX_NBR + nn++] = x;
					else overflow = true;
				}
				else
				{
					if (nm < MAX_M2L) T.m2l[n * MAX_M2L + nm++] = x;
					else overflow = true;
				}
			}
		}
	}
	T.nbr_count[n] = nn;
	T.m2l_count[n] = nm;
	T.p2l_count[n] = np;
	return overflow;
}

__global__ void tree_neighbors_kernel(TreeDev T, int start, int count, int* err)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < count && tree_neighbors_node(T, start + i)) atomicOr(err, 1);
}

/* leaf flags for the leaf numbering scan */
__global__ void leaf_flag_kernel(TreeDev T, int num_nodes, int* flag)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < num_nodes) flag[i] = T.child[i] < 0;
}

/* The whole tree of one field per CTA, for batches of small fields: the
   node functions of the per-level launches, level after level, with block
   barriers in place of the host round trips; the same tree, bit for bit.
   The level list and the error bits go to seg.info for the host. */
__global__ void __launch_bounds__(1024) tree_batch_kernel(const BatchSeg* __restrict__ segs)
{
	__shared__ int s_mx, s_cnt, s_err, s_start, s_count, s_levels;
	const BatchSeg& S = segs[blockIdx.x];
	const TreeDev T = S.T;
	const unsigned full = 0xffffffffu;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
	int* const lstart = S.info + 3;
	int* const lcount = S.info + 3 + TREE_MAX_LEVELS + 1;
	if (tid == 0)
	{
		tree_root_node(T, S.root_half, S.n);
		s_err = 0;
		s_start = 0;
		s_count = 1;
		s_levels = 0;
		lstart[0] = 0;
		lcount[0] = 1;
	}
	__syncthreads();
	for (int L = 0;; L++)
	{
		const int start = s_start, count = s_count;
		if (tid == 0)
		{
			s_mx = 0;
			s_cnt = 0;
		}
		__syncthreads();
		int mx = 0, cnt = 0;
		for (int i = tid; i < count; i += blockDim.x)
		{
			int fl;
			mx = max(mx, tree_flag_node(T, start + i, S.limit, fl));
			cnt += fl;
		}
		mx = (int)__reduce_max_sync(full, (unsigned)mx);
		cnt = __reduce_add_sync(full, cnt);
		if (lane == 0)
		{
			atomicMax(&s_mx, mx);
			atomicAdd(&s_cnt, cnt);
		}
		__syncthreads();
		const int nflag = s_cnt;
		if (s_mx <= S.limit) break;
		const int child_start = start + count;
		if (child_start + 4 * nflag > S.node_cap || L + 1 > TREE_MAX_LEVELS)
		{
			if (tid == 0) s_err |= 2;
			break;
		}
		block_exclusive_scan(T.flag + start, T.rank + start, count);
		for (int i = tid; i < count; i += blockDim.x) tree_children_node(T, start + i, child_start);
		__syncthreads();
		for (int w = warp; w < count; w += nw) tree_partition_node(T, start + w, lane, S.pos, S.mass, S.tpos, S.tmass);
		__syncthreads();
		bool ov = false;
		for (int i = tid; i < 4 * nflag; i += blockDim.x) ov |= tree_neighbors_node(T, child_start + i);
		if (ov) atomicOr(&s_err, 1);
		__syncthreads();
		if (tid == 0)
		{
			s_start = child_start;
			s_count = 4 * nflag;
			s_levels = L + 1;
			lstart[L + 1] = child_start;
			lcount[L + 1] = 4 * nflag;
		}
		__syncthreads();
	}
	__syncthreads();
	if (tid == 0)
	{
		S.info[0] = s_levels;
		S.info[1] = s_start + s_count;
		S.info[2] = s_err;
	}
}

void launch_tree_batch(cudaStream_t s, const BatchSeg* segs, int nseg)
{
	if (nseg > 0) tree_batch_kernel<<<nseg, 1024, 0, s>>>(segs);
}

void launch_tree_root(cudaStream_t s, const TreeDev& T, double half, int nstars)
{
	tree_root_kernel<<<1, 1, 0, s>>>(T, half, nstars);
}
void launch_tree_flag(cudaStream_t s, const TreeDev& T, int start, int count, int limit, int* out)
{
	tree_flag_kernel<<<(count + 255) / 256, 256, 0, s>>>(T, start, count, limit, out);
}
void launch_scan(cudaStream_t s, const int* in, int* out, int n)
{
	scan_kernel<<<1, 1024, 0, s>>>(in, out, n);
}
void launch_tree_children(cudaStream_t s, const TreeDev& T, int start, int count, int child_start)
{
	tree_children_kernel<<<(count + 255) / 256, 256, 0, s>>>(T, start, count, child_start);
}
void launch_tree_partition(cudaStream_t s, const TreeDev& T, int start, int count, double2* pos, double* mass,
	double2* tpos, double* tmass)
{
	long long threads = (long long)count * 32;
	tree_partition_kernel<<<(int)((threads + 255) / 256), 256, 0, s>>>(T, start, count, pos, mass, tpos, tmass);
}
void launch_tree_neighbors(cudaStream_t s, const TreeDev& T, int start, int count, int* err)
{
	tree_neighbors_kernel<<<(count + 255) / 256, 256, 0, s>>>(T, start, count, err);
}
void launch_leaf_flag(cudaStream_t s, const TreeDev& T, int num_nodes, int* flag)
{
	leaf_flag_kernel<<<(num_nodes + 255) / 256, 256, 0, s>>>(T, num_nodes, flag);
}

} /* namespace ccf */
