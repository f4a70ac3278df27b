/******************************************************************************
kernels.h -- device data structures shared by the kernels and the host
engine, and the host-side launch functions of every kernel.
******************************************************************************/
#pragma once

#include "common.cuh"
#include "field.cuh"
#include "mass.h"

#include <algorithm>

namespace ccf
{

constexpr int MAX_NBR = 8;    /* include/tree_node.cuh:23 */
constexpr int MAX_M2L = 27;   /* include/tree_node.cuh:24 */
constexpr int MAX_P2L = 5;    /* include/tree_node.cuh:25 */

/* quadtree nodes, structure of arrays; nodes of a level are contiguous */
struct TreeDev
{
	double2* center;
	double* half;
	int* level;
	int* parent;
	int* child;        /* first of four contiguous children, -1 for a leaf */
	int* star_start;
	int* star_count;
	int* nbr;          /* [node * MAX_NBR + j] */
	int* nbr_count;
	int* m2l;          /* [node * MAX_M2L + j] */
	int* m2l_count;
	int* p2l;          /* [node * MAX_P2L + j] */
	int* p2l_count;
	int* flag;         /* split flag of the level being built */
	int* rank;         /* exclusive scan of flag */
};

/* one row of the root solver: all roots of one branch centre (initial
   solve) or of one (centre, side) continuation */
struct RowDesc
{
	int field;         /* index into the launch's FieldView / FieldOut arrays */
	int branch;        /* c, the branch whose centre the row starts from */
	int side;          /* -1: initial solve at the branch centre; 0: phi decreasing; 1: increasing */
	int steps;         /* continuation rows: phi steps j = 1 .. steps (row_slots maps them to outputs) */
	long long base;    /* offset of the row in master / snapshot / fin / list */
	long long cont_base; /* initial rows: offset of the (branch, side 0) continuation row;
	                        tracked continuation rows: offset of the row's column tables */
};

/* phase of a whole step of the phi grid: cos, sin in FP64 and double-float */
struct PhaseEntry
{
	double2 cs;
	float4 cs_df;      /* (cos hi, sin hi, cos lo, sin lo) */
};

/* per-field outputs and statistics of a solver launch */
struct FieldOut
{
	double2* ccs;          /* file layout, rows = R * nb, cols */
	double2* caustics;     /* may be null */
	double* errs;
	double* mu;            /* may be null */
	int nb;
	int nphi;
	int cols;
	int half;              /* nphi / (2 nb) */
	int step_first;        /* continuation steps to run: [step_first, step_last] */
	int step_last;
	int max_iters_init;
	int max_iters_step;
	int seg;               /* branches per solved centre: the initial solve runs at the centres
	                          c = 0, seg, 2 seg, ... and the continuation rows from a centre cover
	                          seg branches (1: every centre, the reference's scheme) */
	const PhaseEntry* phase;   /* [nphi]: the phase of global step P (below) */
	/* continuation arrays that the initial solve fills for both sides */
	double2* cont_master;
	float4* cont_snap32;
	double2* cont_snap64;
	/* the output window: the arrays hold branches w_b0 .. w_b0 + w_nb - 1
	   (mod nb) and columns w_k0 .. w_k0 + w_cols - 1 of each, in the file
	   layout's order; the whole field is (0, nb, 0, cols) */
	int w_b0, w_nb, w_k0, w_cols;
	/* tracker: 1 when the outputs lie in host memory, where the column check
	   runs inside the tracking launch; else a launch of its own reads the
	   stored roots back (track_check_kernel) */
	int check_inline;
	/* statistics */
	unsigned long long* stats;   /* STATS_WORDS words: [0] max_err bits, [1] nan flag, [2] updates,
	                                [3] terms, [4] unconverged, [5] max sweeps init, [6] max sweeps
	                                step, [7] updates in the initial solve, [8] terms in the initial
	                                solve, [9] continuation rows re-run by the full-sum solver, [10]
	                                tracker sub-step halvings, [11] TRACK_* flags of the re-run rows,
	                                [12] rows tracked again with fine sub-steps; [16] .. [20] the
	                                FP64 polish (STAT_POLISHED_*) */
};

/* slot of root a, branch b, column k in the window's arrays; NO_OUT when
   the window does not hold that column */
constexpr size_t NO_OUT = ~(size_t)0;
CCF_HD size_t out_slot(const FieldOut& O, int a, int b, int k)
{
	int bi = b - O.w_b0;
	if (bi < 0) bi += O.nb;
	const int ki = k - O.w_k0;
	if (bi >= O.w_nb || ki < 0 || ki >= O.w_cols) return NO_OUT;
	return ((size_t)a * O.w_nb + bi) * O.w_cols + ki;
}
CCF_HD void full_window(FieldOut& O)
{
	O.w_b0 = 0;
	O.w_nb = O.nb;
	O.w_k0 = 0;
	O.w_cols = O.cols;
}

/* statistics words of a field (FieldOut::stats) */
constexpr int STATS_WORDS = 24;
constexpr int STAT_POLISHED_MAX_ERR = 16;   /* largest 1/mu error after the polish (double bits) */
constexpr int STAT_POLISHED_NAN = 17;       /* a non-finite 1/mu error after the polish */
constexpr int STAT_POLISHED = 18;           /* points the polish worked on */
constexpr int STAT_POLISHED_UNCONV = 19;    /* unconverged points the polish could not converge */
constexpr int STAT_POLISHED_ABOVE = 20;     /* polished points whose 1/mu error stays above POLISH_ERR with
                                               |f| above the FP64 floor (below) */
constexpr int STAT_POLISHED_FLOOR = 21;     /* polished points above POLISH_ERR at the FP64 floor: |f| within
                                               four times |f'| times half the FP64 spacing of the root, which no
                                               FP64 root can improve on */

/* FP64 polish (polish.cu) */
constexpr double POLISH_ERR = 0.000000001;       /* the reference's 1/mu target (include/ccf_functions.cuh:207-211) */
constexpr double POLISH_STEP_TOL = 0.000000001;  /* theta_star: the reference's step test (ccf_functions.cuh:385) */
constexpr double POLISH_MOVE = 1e-4;             /* theta_star: the most a converged, flagged point may move */
constexpr double POLISH_MOVE_LISTED = 1e-2;      /* theta_star: the same for an unconverged point */

/* The solvers store -1 - err in the 1/mu slot of a point they left
   unconverged; the polish, which always follows them, removes the mark. */
CCF_HD double unconverged_mark(double err) { return isfinite(err) && err >= 0 ? -1 - err : err; }

/* the fields of a polish launch: every point of every field's output
   window, or (nbs > 0) the columns [k0, k0 + nks) of branches
   [b0, b0 + nbs), which the window must hold */
struct PolishArgs
{
	const FieldView* fields;
	const FieldOut* outs;
	int num_fields;
	int b0, nbs, k0, nks;
	unsigned long long* list;        /* flagged points: field << 48 | output slot */
	unsigned long long* list_count;  /* zeroed before the launch */
	long long list_cap;
};

/* Outputs of step j of the continuation row (c, side).  Global step
   P = c 2 half +/- j (mod nphi) is the phase phi0 + P 2 pi / nphi; it is
   column k = (P + half) mod 2 half of branch b = (P + half) / (2 half),
   and at a branch boundary (k = 0) also column 2 half of branch b - 1 --
   except the slot of the neighbouring solved centre's own row when every
   centre is solved (seg = 1: the reference's layout, where row (c, 1) ends
   in column 2 half of branch c and row (c + 1, 0) in column 0 of branch
   c + 1).  Returns the number of slots (1 or 2) in b[], k[]. */
CCF_HD int row_slots(int nb, int half, int seg, int c, int side, int j, int* b, int* k)
{
	const int period = 2 * half;
	const int nphi = nb * period;
	int P = c * period + (side ? j : -j);
	P = ((P % nphi) + nphi) % nphi;
	const int v = P + half;
	int bb = v / period;
	const int kk = v - bb * period;
	bb %= nb;
	int n = 0;
	const int nbr = side ? (c + seg) % nb : (c - seg + nb) % nb;   /* the next solved centre that way */
	if (!(kk == 0 && side == 1 && seg == 1 && bb == nbr))
	{
		b[n] = bb;
		k[n] = kk;
		n++;
	}
	if (kk == 0)
	{
		const int bp = (bb - 1 + nb) % nb;
		if (!(side == 0 && seg == 1 && bp == nbr))
		{
			b[n] = bp;
			k[n] = period;
			n++;
		}
	}
	return n;
}

/* global step of step j of row (c, side), in [0, nphi) */
CCF_HD int row_global_step(int nb, int half, int c, int side, int j)
{
	const int nphi = nb * 2 * half;
	const int P = c * 2 * half + (side ? j : -j);
	return ((P % nphi) + nphi) % nphi;
}

struct SolveArgs
{
	const FieldView* fields;
	const FieldOut* outs;
	const RowDesc* rows;
	int num_rows;
	int cluster;           /* CTAs per row */
	double2* master;
	float4* snap32;
	double2* snap64;
	unsigned char* fin;
	int* list;
	double2* fval;         /* [2 (row base + root) + {0, 1}]: f and f' of the sweep's active roots */
	const float4* const* star_hilo;   /* per field, FP32 hi/lo stars (mixed) */
	int* error;
	const int* num_rows_dev;   /* when set, the rows to run are rows[0 .. *num_rows_dev), at most num_rows */
};

/* Per-root tracking of the continuation rows (solver.cu, track_kernel).
   Row statistics, TRACK_ROW_STATS per row: [0] largest 1/mu bound (double
   bits), [1] TRACK_* flags, [2] most evaluations one root needed for one phi
   step, [3] points kept unconverged (the corrector stalled next to a zero). */
constexpr int TRACK_ROW_STATS = 4;
constexpr int TRACK_TSUB = 64;        /* a whole phi step in the tracker's sub-step units */
constexpr int TRACK_FINE_SUB = 8;     /* longest sub-step when a failed row is tracked again */
constexpr unsigned long long TRACK_DUPLICATE = 1;    /* two roots of a column on one zero */
constexpr unsigned long long TRACK_LOST = 2;         /* a root that did not converge */
constexpr unsigned long long TRACK_NONFINITE = 4;    /* a non-finite 1/mu bound */
constexpr unsigned long long TRACK_TABLE_FULL = 8;   /* the column table probe limit was reached */

struct TrackArgs
{
	const FieldView* fields;
	const FieldOut* outs;
	const RowDesc* rows;        /* continuation rows; cont_base = offset of the row's column tables */
	int num_rows;
	const double2* master;      /* start roots (the branch centre), master[row.base + root]; read only */
	unsigned long long* table;  /* column tables: 2 R slots per phi step, zeroed before the launch */
	unsigned long long* row_stats;   /* TRACK_ROW_STATS per row, zeroed before the launch */
	const int* item_start;      /* [num_rows]: first work item (32 roots) of each row */
	int num_items;
	int* counter;               /* [0] next solo root, [1] next item in order; zeroed before the launch */
	int2* solo;                 /* (row, root) of the roots that start off the root box: one warp each, first ... */
	int* num_solo;              /* ... their number (zeroed before the marking launch) */
	unsigned char* is_solo;     /* [master index]: the root runs solo, not in its item */
	const int* item_order;      /* [num_items]: the queue's order of the items; null: in order */
	/* re-tracking of rows that failed the check: the rows are a device-side
	   list of *num_rows_dev rows, items_per_row fixed-size items each (no
	   solo roots), and a phi sub-step never longer than max_sub */
	const int* num_rows_dev;    /* when set: the number of rows, on the device */
	int items_per_row;          /* when > 0: item = row * items_per_row + chunk */
	int max_sub;                /* longest sub-step (TSUB = a whole phi step) */
};

/* stars.cu */
void launch_generate_stars(cudaStream_t s, int n, int seed, int rectangular, double2 corner, double corner_abs,
	const MassTable& mt, double2* pos, double* mass);
void launch_star_stats(cudaStream_t s, int n, const double* mass, double* out);
void launch_seed_roots(cudaStream_t s, int nstars, int nroots, int nrows, const double2* pos, const double* mass,
	double corner_abs, double theta, double a_lin, double gamma, int nb, int seg, double2* master, float4* snap32,
	double2* snap64);
void launch_star_hilo(cudaStream_t s, int n, const double2* pos, float4* out, const double* mass = nullptr,
	float2* mass_out = nullptr);

/* One field of a batched setup (tree.cu tree_batch_kernel, fmm.cu
   fmm_batch_kernel and leaf_batch_kernel, stars.cu stars_batch_kernel): one
   CTA per field does what the per-level launches do for one field. */
constexpr int TREE_MAX_LEVELS = 40;
constexpr int BATCH_INFO_INTS = 3 + 2 * (TREE_MAX_LEVELS + 1) + 4;   /* tree info, then the leaf info */
struct BatchSeg
{
	/* stars (generated when gen is set) */
	int n;
	int gen;
	int seed;
	int rectangular;
	double2 corner;
	double corner_abs;
	MassTable mt;
	double2* star_gen;
	double2* pos;
	double* mass;
	double2* tpos;
	double* tmass;
	double* stats5;
	/* tree */
	TreeDev T;
	int node_cap;
	int limit;
	double root_half;
	/* info: [0] levels, [1] nodes, [2] error bits (1 a neighbour list overflowed, 2 the node
	   capacity ran out), [3 ..] level starts, [3 + TREE_MAX_LEVELS + 1 ..] level counts,
	   then [LEAF_INFO + 0] leaves, [+1] the sum of the near-list lengths, [+2] error bits
	   (2 a leaf has more than MAX_NEAR near stars) */
	int* info;
	/* FMM */
	int P;
	const double* B;
	double2* multi;
	double2* local;
	int* leaf_flag;
	int* leaf_index;
	/* leaf records */
	double theta2;
	int num_leaves;
	double2* leaf_center;
	double* leaf_inv_half;
	int* leaf_near_count;
	NearStar* leaf_near;
	double2* leaf_loc;
	float2* leaf_loc3f;
	int* node_leaf;
	float4* leaf_near_df;   /* null: no double-float copies (FP64 precision) */
	float2* leaf_mass_df;
	float4* leaf_loc_df;
	float2* leaf_ih_df;
	float4* star_hilo;
	float2* star_mass_df;
};
constexpr int LEAF_INFO = 3 + 2 * (TREE_MAX_LEVELS + 1);

/* exclusive scan of n ints by the calling block (every thread calls it;
   n up to a few million); returns the total */
CCF_D int block_exclusive_scan(const int* __restrict__ in, int* __restrict__ out, int n)
{
	__shared__ int s_warp[32];
	__shared__ int s_carry;
	if (threadIdx.x == 0) s_carry = 0;
	__syncthreads();
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (int base = 0; base < n; base += blockDim.x)
	{
		int i = base + threadIdx.x;
		int v = i < n ? in[i] : 0;
		int x = v;
		for (int o = 1; o < 32; o <<= 1)
		{
			int y = __shfl_up_sync(0xffffffffu, x, o);
			if (lane >= o) x += y;
		}
		if (lane == 31) s_warp[warp] = x;
		__syncthreads();
		if (warp == 0)
		{
			int w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0;
			for (int o = 1; o < 32; o <<= 1)
			{
				int y = __shfl_up_sync(0xffffffffu, w, o);
				if (lane >= o) w += y;
			}
			s_warp[lane] = w;
		}
		__syncthreads();
		int prefix = s_carry + (warp > 0 ? s_warp[warp - 1] : 0) + x - v;
		if (i < n) out[i] = prefix;
		__syncthreads();
		if (threadIdx.x == blockDim.x - 1) s_carry = prefix + v;
		__syncthreads();
	}
	const int total = s_carry;
	__syncthreads();
	return total;
}


void launch_stars_batch(cudaStream_t s, const BatchSeg* segs, int nseg);

/* the root seeds of one field's solved centres (stars.cu seed_root) */
struct SeedSeg
{
	int nstars, nroots, nrows, nb, seg;
	const double2* pos;
	const double* mass;
	double corner_abs, theta, a_lin, gamma;
	double2* master;
	float4* snap32;
	double2* snap64;
};
void launch_seed_roots_batch(cudaStream_t s, const SeedSeg* segs, int nseg, long long max_seeds);

/* tree.cu */
void launch_tree_batch(cudaStream_t s, const BatchSeg* segs, int nseg);
void launch_tree_root(cudaStream_t s, const TreeDev& T, double half, int nstars);
void launch_tree_flag(cudaStream_t s, const TreeDev& T, int start, int count, int limit, int* out);
void launch_scan(cudaStream_t s, const int* in, int* out, int n);
void launch_tree_children(cudaStream_t s, const TreeDev& T, int start, int count, int child_start);
void launch_tree_partition(cudaStream_t s, const TreeDev& T, int start, int count, double2* pos, double* mass,
	double2* tpos, double* tmass);
void launch_tree_neighbors(cudaStream_t s, const TreeDev& T, int start, int count, int* err);
void launch_leaf_flag(cudaStream_t s, const TreeDev& T, int num_nodes, int* flag);

/* fmm.cu */
void launch_fmm_batch(cudaStream_t s, const BatchSeg* segs, int nseg, int max_levels, int max_level_nodes,
	long long max_coefficients);
void launch_leaf_batch(cudaStream_t s, const BatchSeg* segs, int nseg);
void launch_fmm_upward(cudaStream_t s, const TreeDev& T, int start, int count, int P, const double2* pos, const double* mass,
	double2* multi, const double* B);
void launch_fmm_downward(cudaStream_t s, const TreeDev& T, int start, int count, int P, const double2* pos, const double* mass,
	const double2* multi, double2* local, const double* B);
void launch_leaf_build(cudaStream_t s, const TreeDev& T, int num_nodes, const int* leaf_index, int P, double theta2,
	const double2* pos, const double* mass, const double2* local, double2* leaf_center, double* leaf_inv_half,
	int* leaf_near_count, NearStar* leaf_near, double2* leaf_loc, float2* leaf_loc3f, int* node_leaf, int* err);

void launch_leaf_df(cudaStream_t s, int num_leaves, int P, const double2* leaf_center, const double* leaf_inv_half,
	const int* near_count, const NearStar* near, const double2* loc, float4* near_df, float2* mass_df, float4* loc_df,
	float2* ih_df);
void launch_fold_smooth(cudaStream_t s, int num_leaves, int P, const double2* leaf_center, const double* leaf_inv_half,
	const double2* loc, const double2* ef, int nf, const double2* er, int nr, const double2* eq, int nq, double radius,
	float4* loc_df, float2* loc3f, double2* loc64, unsigned char* fold);

/* solver.cu */
int solver_blocks_per_sm(bool mixed);
cudaError_t launch_solve(cudaStream_t s, const SolveArgs& a, bool mixed, bool initial);
cudaError_t launch_track_mark(cudaStream_t s, const TrackArgs& a);
cudaError_t launch_track_item_order(cudaStream_t s, const TrackArgs& a, int* work, int* order);
constexpr int TRACK_WARPS_PER_SM = 12;   /* resident tracker warps per SM (3 CTAs of 4 warps) */
cudaError_t launch_phase_table(cudaStream_t s, int nb, int nphi, PhaseEntry* out);
cudaError_t launch_track(cudaStream_t s, const TrackArgs& a, bool mixed);
cudaError_t launch_track_check(cudaStream_t s, const TrackArgs& a, long long max_row_points);
cudaError_t launch_collect_rerun(cudaStream_t s, const TrackArgs& a, RowDesc* rerun, int* count);
cudaError_t launch_clear_tables(cudaStream_t s, const TrackArgs& a);
cudaError_t launch_eval_points(cudaStream_t s, const FieldView* F_dev, int npts, const double2* z, const double* phi,
	double2* f, double2* df, double2* w, double* err, double* mu);

/* fmm_check.cu: largest far-field error over one point per leaf (double bits
   into *out, which must be zero) */
cudaError_t launch_fmm_error(cudaStream_t s, const FieldView* F_dev, int num_leaves, unsigned long long* out);

/* polish.cu: two launches (scan, list) on s; max_points = the largest field's
   point count (or box); list_count must be zero when they start */
cudaError_t launch_polish(cudaStream_t s, const PolishArgs& a, long long max_points, int num_sms);

} /* namespace ccf */
