/******************************************************************************
ccf_oracle.h -- TEST INFRASTRUCTURE ONLY.

C interface of the CPU oracle: a plain FP64 restatement of the reference's
critical-curve / caustic algorithm (weisluke/ccf), used by tests/, by
__graft_entry__.smoke() and by bench.py's CPU baseline leg as the checker.
The product never links, loads or calls anything here.
******************************************************************************/
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

/* mass function ids, registry of include/mass_functions.cuh:17-25 */
enum oracle_mass_function
{
	ORACLE_MF_EQUAL = 0,
	ORACLE_MF_UNIFORM = 1,
	ORACLE_MF_SALPETER = 2,
	ORACLE_MF_KROUPA = 3,
	ORACLE_MF_OPTICAL_DEPTH = 4
};

typedef struct oracle_params
{
	/* public fields of CCF<T> (include/ccf.cuh:42-62) */
	double kappa_tot;
	double shear;
	double kappa_star;
	double theta_star;
	double m_solar;
	double m_lower;
	double m_upper;
	double safety_scale;
	int mass_function;
	int rectangular;
	int approx;
	int num_stars;
	int num_phi;
	int num_branches;
	int random_seed;
	int write_mu_length_scales;

	/* optional star field given by the caller (exchanged star file);
	   stars_in holds num_stars triples (x1, x2, mass) */
	const double* stars_in;
	int stars_in_rectangular;
	double stars_in_corner_re;
	double stars_in_corner_im;
	double stars_in_theta;

	/* solver controls */
	int num_threads;      /* OpenMP threads; 1 = serial, deterministic */
	int init_iters;       /* Aberth sweeps at the branch centres; reference 30 */
	int step_iters;       /* Aberth sweeps per phi step; reference 20 */
	int early_out;        /* 1 = reference's 1/mu < 1e-9 early return */
	double polish_tol;    /* > 0: after the run, iterate every column until
	                         all steps are < polish_tol * theta_star */
	int polish_max_iters;
	int exact_binomials;  /* 1 = exact binomials instead of the reference's
	                         int32 Pascal table */
	int max_steps;        /* > 0: stop the continuation after this many phi
	                         steps (bounded CPU-baseline sample) */
	int max_branches;     /* > 0: solve only max_branches branches: first_branch,
	                         first_branch + branch_stride, ... (mod num_branches) */
	int first_branch;
	int branch_stride;    /* 0 = 1 */
	int polish_newton;    /* with polish_tol > 0: 1 = polish each root alone by
	                         FP64 Newton steps z <- z - f / f' on the oracle's
	                         own f (two evaluations per point); 0 = full Aberth
	                         sweeps of every column without the early return */
	int jacobi;           /* 1: every sweep updates a row's roots from the row
	                         as it stood before the sweep, the roots split over
	                         the threads (rows one after another: large rows);
	                         0: the reference's in-place order, rows split over
	                         the threads.  Both converge to the zeros of f; the
	                         order of the updates only changes the path. */
	int seed_curves;      /* 1: the branch centres' seeds on each star's own
	                         critical curve, z_i +/- theta sqrt(m) / sqrt(a e^{-i phi}
	                         - gamma) (the CUDA path's seeds), instead of the
	                         reference's z_i +/- 1 */
} oracle_params;

typedef struct oracle_info
{
	int num_stars;
	int num_roots;
	int taylor_smooth;
	int tree_levels;
	int expansion_order;
	int num_nodes;
	int rectangular;
	int random_seed;
	double corner_re;
	double corner_im;
	double theta_star;
	double kappa_star;
	double mu_ave;
	double alpha_error;
	double root_half_length;
	double mean_mass;
	double mean_mass2;
	double mean_mass2_ln_mass;
	double kappa_star_actual;
	double m_lower_actual;
	double m_upper_actual;
	double mean_mass_actual;
	double mean_mass2_actual;
	double mean_mass2_ln_mass_actual;
	double m_lower;
	double m_upper;
	double max_error;
	int has_nan;
	long long root_updates;   /* executed Aberth updates */
	long long root_terms;     /* executed reciprocal-sum terms */
	double t_stars;
	double t_tree;
	double t_init_roots;
	double t_ccs;
	double t_caustics;
	char error[256];
} oracle_info;

/* defaults of CCF<T> plus the reference's solver constants */
void oracle_default_params(oracle_params* p);

/* derived parameters only (no star field, no tree); returns 0 on success */
int oracle_derive(const oracle_params* p, oracle_info* info);

/* the full pipeline.  Output arrays use the reference's file layout
   (include/ccf.cuh:1214-1257): rows = num_roots * num_branches,
   cols = num_phi / num_branches + 1, row = root * num_branches + branch.
   stars_out: num_stars * 3 doubles in tree order (may be NULL);
   ccs, caustics: rows*cols complex as interleaved doubles (may be NULL);
   errs, mu_length_scales: rows*cols doubles (may be NULL).
   Returns 0 on success. */
int oracle_run(const oracle_params* p, oracle_info* info, double* stars_out,
	double* ccs, double* caustics, double* errs, double* mu_length_scales);

/* evaluate the deflection field of the star field described by p (after the
   tree and FMM are built exactly as the reference builds them) at npts
   points z (interleaved complex).  Outputs (interleaved complex, may be NULL):
   alpha = alpha_star + alpha_local + alpha_smooth, f = parametric critical
   curve function at phase phi[i], df = its z-derivative, w = lens map.
   Returns 0 on success. */
int oracle_eval(const oracle_params* p, oracle_info* info, int npts, const double* z,
	const double* phi, double* alpha, double* f, double* df, double* w);

/* match two root sets column by column: a and b are rows*cols complex in the
   output layout; for every column the rows of a are matched to the rows of b
   by nearest neighbour.  Writes the largest matched distance, the number of
   columns where the nearest-neighbour map is not a permutation, and the
   number of non-finite entries.  nb groups rows by branch (row % nb).
   Returns 0 on success. */
int oracle_match_sets(int rows, int cols, int nb, const double* a, const double* b,
	double* max_dist, long long* non_bijective_cols, long long* non_finite);

/* as oracle_match_sets, and also writes for every entry of a the row of b it
   matched (idx: rows*cols ints, -1 where unmatched) and its distance (dist). */
int oracle_match_index(int rows, int cols, int nb, const double* a, const double* b, int* idx, double* dist);

#ifdef __cplusplus
}
#endif
