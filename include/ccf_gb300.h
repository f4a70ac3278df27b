/******************************************************************************
ccf_gb300.h -- C ABI of the GB300-native critical-curve and caustic finder.

The reference (weisluke/ccf) exports no extern "C" surface: its operator API
is the header-only class template CCF<T> (include/ccf.cuh:34-1289) and the
main_ccf command line (src/main_ccf.cu).  Every entry point below states the
reference interface it replaces.  Signatures use plain C types and pointers
only, so that C, C++, Python ctypes/cffi or any other FFI can bind them.

Thread safety: one handle must not be used from two threads at once;
different handles are independent.  All work runs on CUDA device 0 (the
reference's choice, include/ccf.cuh:205-212) unless ccf_params.device says
otherwise.  The library never resets the CUDA context (the reference calls
cudaDeviceReset on every run, include/ccf.cuh:151, which a long-lived caller
cannot afford).
******************************************************************************/
#ifndef CCF_GB300_H
#define CCF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CCF_GB300_ABI_VERSION 2

/* Status codes.  The reference returns bool from every stage and prints the
   reason to std::cerr (include/ccf.cuh:1265-1287); here the reason is kept
   per handle and returned by ccf_last_error(). */
typedef enum ccf_status
{
	CCF_OK = 0,
	CCF_ERR_INVALID_ARGUMENT = 1, /* input check failed (include/ccf.cuh:218-346) */
	CCF_ERR_CUDA = 2,             /* a CUDA call failed (include/util.cuh:156-190) */
	CCF_ERR_NO_DEVICE = 3,        /* no CUDA device (include/ccf.cuh:185-189) */
	CCF_ERR_OUT_OF_MEMORY = 4,
	CCF_ERR_IO = 5,               /* star file or output file problem */
	CCF_ERR_NOT_RUN = 6,          /* results asked for before a successful run */
	CCF_ERR_NUMERIC = 7,          /* non-finite 1/mu errors (include/ccf.cuh:963-967) */
	CCF_ERR_TIMEOUT = 8,          /* a bounded device-side wait ran out */
	CCF_ERR_BUDGET = 9            /* request larger than the device-memory budget */
} ccf_status;

/* Arithmetic used by the root solver. */
typedef enum ccf_precision
{
	CCF_PRECISION_FP64 = 0,  /* all solver arithmetic in FP64 */
	CCF_PRECISION_MIXED = 1  /* FP32 Aberth correction sums; critical-curve
	                            function, residual and caustic map in double-float
	                            (two FP32 numbers, ~48 bits) within the corner
	                            circle and FP64 outside; length scales in FP64 */
} ccf_precision;

/* How the roots are carried from one phi step to the next. */
typedef enum ccf_continuation
{
	CCF_CONTINUATION_TRACK = 0,  /* default: every root follows its own path in
	                                phi with a quartic predictor (the polynomial
	                                through its last five positions; the secant
	                                after sub-steps) and a corrector whose Aberth
	                                correction keeps the poles of the leaf's near
	                                stars only; every column is checked for two
	                                roots on one zero.  A row that fails the check
	                                (or loses a root) is tracked again from its
	                                centre with sub-steps of at most 1/8 phi step,
	                                and a row that fails again is run by the
	                                full-sum continuation */
	CCF_CONTINUATION_ABERTH = 1  /* the full Aberth step of the reference for every
	                                root of a row (include/ccf_functions.cuh:261-394) */
} ccf_continuation;

/* Parameters.  The first block mirrors the public fields of CCF<T> with the
   same names, meanings and defaults (include/ccf.cuh:42-62); the second block
   is specific to this implementation.  Fill with ccf_default_params(). */
typedef struct ccf_params
{
	double kappa_tot;            /* default 0.3  */
	double shear;                /* default 0.3  */
	double kappa_star;           /* default 0.27 */
	double theta_star;           /* default 1    */
	char mass_function[32];      /* "equal", "uniform", "salpeter", "kroupa", "optical_depth" */
	double m_solar;              /* default 1    */
	double m_lower;              /* default 0.01 */
	double m_upper;              /* default 50   */
	int rectangular;             /* default 0    */
	int approx;                  /* default 1    */
	double safety_scale;         /* default 1.37 */
	int num_stars;               /* default 137  */
	char starfile[1024];         /* default ""   */
	int num_phi;                 /* default 100  */
	int num_branches;            /* default 1    */
	int random_seed;             /* default 0 (= draw from the clock) */
	int write_stars;             /* default 1    */
	int write_critical_curves;   /* default 1    */
	int write_caustics;          /* default 1    */
	int write_mu_length_scales;  /* default 0    */
	char outfile_prefix[1024];   /* default "./" */

	int precision;               /* ccf_precision, default CCF_PRECISION_MIXED */
	int output_float;            /* 1: write files in single precision, as the
	                                reference built with -D is_float does */
	int max_iters_init;          /* cap on Aberth sweeps at a branch centre (default 300) */
	int max_iters_step;          /* cap on Aberth sweeps per phi step (default 60) */
	int exact_binomials;         /* 1: exact binomials in the FMM translations;
	                                0 (default): the reference's int32 table */
	int device;                  /* CUDA device ordinal, default 0 */
	int continuation;            /* ccf_continuation, default CCF_CONTINUATION_TRACK */
	int solved_centres;          /* tracker: branch centres solved by the initial Aberth solve,
	                                a divisor of num_branches (the others are reached by
	                                tracking); 0 (default): as few as fill the GPU */
	int expansion_order;         /* FMM expansion order P: 0 (default) = the reference's formula
	                                (include/ccf.cuh:840-852); 3 .. 31 = this order.  Another
	                                order than the reference's changes the far field within its
	                                error target (1e-7 theta_star, include/ccf.cuh:439) and the
	                                roots with it */
	int leaf_max_stars;          /* tree split rule: a node is split while its stars and its
	                                neighbours' exceed this; 0 (default) = 32, the reference's
	                                (include/tree_node.cuh:14, :321-345); 4 .. 32 (a smaller
	                                leaf makes the near sums shorter and the tree deeper; it
	                                changes the far field as expansion_order does) */
	int init_cluster;            /* CTAs per branch-centre row of the initial Aberth solve:
	                                0 (default) = as many as fill the GPU once; 1, 2, 4, 8, 16 */
	int autotune;                /* 1: ccf_run applies the settings ccf_autotune found for fields
	                                of this shape (init_cluster, solved_centres), tuning on the
	                                first run of a shape; 2: also expansion_order and
	                                leaf_max_stars.  0 (default): the settings as given */
	int host_outputs;            /* where the outputs (roots, caustics, 1/mu errors, length
	                                scales) are kept: 0 (default) device memory; 1 page-locked
	                                host memory that the library holds, mapped into the GPU's
	                                address space, written by the kernels directly (on GB300 over
	                                NVLink-C2C): no device memory for them, no copy after the
	                                run; 2 the same host memory, filled one group of branches at
	                                a time from two device chunk buffers (about 2 GiB each) by
	                                bulk copies that overlap the next group's computation (a
	                                single field per run; batches write as with 1) */
	int reserved[1];
} ccf_params;

/* Derived parameters, statistics and timings of a run.  Names follow the keys
   of ccf_parameter_info.txt (include/ccf.cuh:1142-1191). */
typedef struct ccf_info
{
	int num_stars;
	int num_roots;
	int taylor_smooth;
	int tree_levels;
	int expansion_order;
	int num_nodes;
	int num_leaves;
	int rectangular;
	int random_seed;
	int has_nan;
	double kappa_star;
	double theta_star;
	double corner_x1;
	double corner_x2;
	double mu_ave;
	double alpha_error;
	double root_half_length;
	double mean_mass;
	double mean_mass2;
	double mean_mass2_ln_mass;
	double kappa_star_actual;
	double m_lower;
	double m_upper;
	double m_lower_actual;
	double m_upper_actual;
	double mean_mass_actual;
	double mean_mass2_actual;
	double mean_mass2_ln_mass_actual;
	double max_error;            /* max_error_1/mu, after the FP64 polish */
	long long num_points;        /* num_roots * (num_phi + num_branches) */
	long long root_updates;      /* executed Aberth updates */
	long long sum_terms;         /* executed reciprocal-sum terms */
	long long unconverged;       /* output points the solvers left unconverged (sweep cap
	                                reached, tracker stalled) that the FP64 polish could not
	                                converge either */
	int max_sweeps_init;         /* most sweeps any branch centre needed */
	int max_sweeps_step;         /* most sweeps any phi step needed */
	double t_stars;              /* seconds, CUDA events */
	double t_tree;               /* tree build + FMM coefficients */
	double t_init_roots;
	double t_ccs;
	double t_caustics;           /* the FP64 polish (the residual, caustic map and length
	                                scales are formed in the solvers' epilogues) */
	double t_total;              /* star generation -> caustics on the device */
	long long kernel_launches;   /* CUDA kernels this field's run launched */
	long long root_updates_init; /* the part of root_updates done at the branch centres */
	long long sum_terms_init;    /* the part of sum_terms done at the branch centres */
	long long rows_rerun;        /* continuation rows the tracker handed to the full-sum solver */
	long long step_halvings;     /* phi sub-step halvings of the tracker */
	long long rerun_flags;       /* why rows were re-run: 1 two roots on one zero, 2 a
	                                root lost, 4 a non-finite 1/mu bound, 8 a full
	                                column table (bits OR-ed over the rows) */
	double near_mean;            /* mean number of stars in a leaf's near list */
	int centres_solved;          /* branch centres solved by the initial Aberth solve (the
	                                tracker solves every seg-th one and tracks the others) */
	int rows_retracked;          /* tracker rows that failed the check and were tracked again
	                                with sub-steps of 1/8 phi step (rows_rerun: those that
	                                failed again and went to the full-sum solver) */
	int leaves_folded;           /* leaves whose expansion carries the smooth-mass Taylor
	                                series (mixed precision, rectangular Taylor form), so
	                                that the continuation skips the series there */
	/* FP64 polish: every output point whose 1/mu error is above 1e-9, or that
	   the solvers left unconverged, takes FP64 Newton steps with the near-pole
	   Aberth correction until the reference's stopping rules hold
	   (include/ccf_functions.cuh:207-211, :385) */
	double max_error_unpolished;       /* max_error_1/mu before the polish */
	long long unconverged_unpolished;  /* unconverged points before the polish */
	long long points_polished;         /* points the polish worked on */
	long long points_above_target;     /* polished points whose FP64 1/mu error stays above
	                                      1e-9 although |f| is above the FP64 floor (below) */
	int init_cluster;                  /* CTAs per row of the initial Aberth solve */
	int leaf_max_stars;                /* the tree's leaf limit (32: the reference's rule) */
	long long points_at_fp64_floor;    /* polished points whose 1/mu error stays above 1e-9
	                                      because |f| is within four times |f'| times half the
	                                      FP64 spacing of the root: no FP64 root does better (the
	                                      reference's own FP64 roots carry the same floor) */
} ccf_info;

typedef struct ccf_handle ccf_handle;

/* Library version and ABI check. */
int ccf_abi_version(void);

/* Fill p with the reference's defaults (include/ccf.cuh:42-62). */
void ccf_default_params(ccf_params* p);

/* Replaces the CCF<T> default constructor (include/ccf.cuh:68-71). */
ccf_status ccf_create(ccf_handle** out);

/* Releases all device and host memory of the handle. */
void ccf_destroy(ccf_handle* h);

/* Replaces assignment to the public fields of CCF<T> (include/ccf.cuh:42-62). */
ccf_status ccf_set_params(ccf_handle* h, const ccf_params* p);
ccf_status ccf_get_params(const ccf_handle* h, ccf_params* p);

/* Supply a star field in memory instead of a star file: the in-memory form of
   -sf/--starfile (include/star.cuh:175-320).  xym holds n triples
   (x1, x2, mass).  Pass n = 0 to go back to generated fields. */
ccf_status ccf_set_stars(ccf_handle* h, int n, const double* xym, int rectangular,
	double corner_x1, double corner_x2, double theta_star);

/* Replaces bool CCF<T>::run(int verbose) (include/ccf.cuh:1265-1280):
   star field, tree and FMM, initial roots, phi continuation, 1/mu errors,
   caustics and (if requested) length scales, all resident on the device. */
ccf_status ccf_run(ccf_handle* h, int verbose);

/* Replaces bool CCF<T>::save(int verbose) (include/ccf.cuh:1282-1287):
   writes ccf_parameter_info.txt and the requested .bin files with the
   reference's layout (include/ccf.cuh:1123-1260). */
ccf_status ccf_save(ccf_handle* h, int verbose);

/* Derived parameters, statistics and timings of the last run. */
ccf_status ccf_get_info(const ccf_handle* h, ccf_info* info);

/* Copy results to host memory, in the reference's file layout
   (include/ccf.cuh:1214-1257): rows = num_roots * num_branches,
   cols = num_phi / num_branches + 1, row = root * num_branches + branch.
   Complex arrays are interleaved (re, im) doubles.  Any pointer may be NULL.
   stars: num_stars triples (x1, x2, mass) in tree order, as ccf_stars.bin. */
ccf_status ccf_get_results(ccf_handle* h, double* ccs, double* caustics, double* errs,
	double* mu_length_scales, double* stars);

/* Device pointers of the same arrays (valid until the next run or destroy);
   a pointer is NULL when that output was not requested.  With
   ccf_params.host_outputs they address page-locked host memory, which the
   host can read through the same pointers. */
ccf_status ccf_get_device_results(ccf_handle* h, const double** ccs, const double** caustics,
	const double** errs, const double** mu_length_scales);

/* Page-locked host memory for the destinations of ccf_get_results (copies
   into it run at the full host-device bandwidth; pageable destinations are
   staged).  An addition of this library, with no counterpart in the
   reference.  CCF_ERR_NO_DEVICE without a CUDA device. */
ccf_status ccf_host_alloc(size_t bytes, void** out);
ccf_status ccf_host_free(void* p);

/* Message of the last failure on this handle ("" if none). */
const char* ccf_last_error(const ccf_handle* h);

/* Checks p and computes the derived parameters (corner, taylor_smooth,
   num_roots, mass-function moments) on the host; needs no GPU.
   Restates include/ccf.cuh:218-497.  msg (may be NULL) receives the reason
   of a CCF_ERR_INVALID_ARGUMENT. */
ccf_status ccf_derive_params(const ccf_params* p, ccf_info* info, char* msg, size_t msg_len);

/* Run several independent fields as one batch: their rows share persistent
   solver launches (the reference handles one field per process).  handles[i]
   carries the parameters of field i; results and info land in each handle. */
ccf_status ccf_run_batch(ccf_handle** handles, int n, int verbose);

/* Write the star file of the last run (include/star.cuh:498-534) to an
   explicit path. */
ccf_status ccf_write_star_file(const ccf_handle* h, const char* path);

/* Evaluate the field of the last run at n host points z (interleaved
   complex) with phases phi: the critical-curve function f and its
   z-derivative (include/ccf_functions.cuh:69-121), the lens map w
   (ccf_functions.cuh:33-45), the 1/mu error bound (ccf_functions.cuh:457-463)
   and the length scale (ccf_functions.cuh:144-166).  These are the device
   functions the reference's kernels call, exposed for checks and for
   callers that need the map at arbitrary points.  Any output may be NULL. */
ccf_status ccf_eval_points(ccf_handle* h, int n, const double* z, const double* phi, double* f, double* df,
	double* w, double* err, double* mu_length);

/* Continue one (branch, side) of the field built by the last ccf_run on h,
   from caller-supplied starting roots, without allocating any device memory.
   This entry point has no counterpart in the reference.  It exists for
   callers that cannot call cudaMalloc where they need the extra phi steps: a
   host framework that owns all device memory through its own pool, or a
   real-time loop that must not take the allocator's locks or synchronise
   implicitly.  The solver's per-row scratch sits in a fixed 8 MiB device
   array built into the library (held by every GPU that loads it until the
   process exits), which limits a row to about 120 000 roots; larger rows are
   rejected with CCF_ERR_INVALID_ARGUMENT.
   start_roots: num_roots complex roots (device memory) at the branch centre.
   ccs, errs, caustics: device arrays in the ccf_get_results layout of the
   field; only the columns of steps 1..num_steps on this side are written
   (caustics may be NULL), after the same FP64 polish as ccf_run.  errs holds
   each written point's 1/mu error: a point meets the reference's target when
   it is at most 1e-9; the run's statistics are not returned.  stream: a
   cudaStream_t, or NULL for the default stream; the call only enqueues work
   on it and reads no host memory once it has returned.  The caller's
   current device is unchanged on return.  The first call on a device looks
   up the scratch's device address; make that first call before any stream
   capture.  The address stays valid for the CUDA context it was looked up
   in: after a cudaDeviceReset the entry point must not be called again in
   that process.  All calls share the scratch and it keeps the last call's
   contents: calls whose work overlaps on the GPU race and must be
   serialised by the caller. */
ccf_status ccf_continue_branch_noalloc(ccf_handle* h, int branch, int side, int num_steps, const double* start_roots,
	double* ccs, double* errs, double* caustics, void* stream);

/* The largest far-field error of the field built by the last ccf_run: at
   one point in every leaf, the deflection of the stars from the leaf's near
   sum and local expansion against the direct sum over every star
   (include/alpha_star.cuh:18-115 over all stars).  The reference chooses its
   expansion order so that this stays below alpha_error = 1e-7 theta_star
   (include/ccf.cuh:439, :840-852).  No reference counterpart. */
ccf_status ccf_fmm_error(ccf_handle* h, double* max_error);

/* Autotuner: times candidate solver settings on h's field -- init_cluster,
   solved_centres and, with fmm = 1, leaf_max_stars and expansion_order -- and
   returns in *best h's parameters with the fastest settings whose runs are
   as good as the defaults' (no non-finite 1/mu error, no more unconverged
   points or points above the 1/mu target; for the FMM settings a far-field
   error within alpha_error or the default's own).  The result is cached per
   field shape (GPU, precision, continuation, geometry, num_branches, buckets
   of num_stars and phi steps) in memory and in $CCF_GB300_AUTOTUNE_CACHE
   (else ~/.cache/ccf_gb300/autotune.txt).  h keeps its parameters; its
   results are those of the last trial and must be rerun.  best_seconds (may
   be NULL) receives the tuned field's device time.  No reference counterpart
   (the reference fixes its launch shapes, leaf size and order). */
ccf_status ccf_autotune(ccf_handle* h, int fmm, int verbose, ccf_params* best, double* best_seconds);

/* Device memory a run with parameters p will hold (stars, tree, FMM and leaf
   records, solver rows, outputs), an upper estimate used for admission.  No
   reference counterpart (the reference allocates managed memory as it goes,
   include/ccf.cuh:131-143). */
ccf_status ccf_estimate_device_bytes(const ccf_params* p, unsigned long long* bytes);

/* ---------------- asynchronous batches ----------------
   ccf_run_batch on a host thread: submit returns at once, poll / wait read
   the outcome.  The handles must stay alive and untouched until the batch is
   waited for.  No reference counterpart (one field per process there). */
typedef struct ccf_batch ccf_batch;
ccf_status ccf_batch_submit(ccf_handle** handles, int n, int verbose, ccf_batch** out);
/* *done = 1 once the batch has finished */
ccf_status ccf_batch_poll(ccf_batch* b, int* done);
/* waits and returns the batch's ccf_run_batch status */
ccf_status ccf_batch_wait(ccf_batch* b);
/* waits if needed, then frees the batch object (not the handles) */
void ccf_batch_destroy(ccf_batch* b);

/* ---------------- serving ----------------
   A request loop over one GPU.  Requests (parameter sets) are queued in
   arrival order and admitted while a slot is free and the device memory the
   admitted requests hold (ccf_estimate_device_bytes, counted from admission
   until ccf_server_release) stays within hbm_budget.  Each admitted request
   runs on its own handle, engine and CUDA stream, so the work of concurrent
   requests overlaps on the device; its stars, tree, roots and results stay
   resident until released.  A request larger than the whole budget is
   rejected (CCF_ERR_BUDGET); one that had to wait at the head of the queue
   for memory is counted as deferred.  No reference counterpart: the
   reference resets the device on every run (include/ccf.cuh:151). */
typedef struct ccf_server ccf_server;

typedef struct ccf_server_config
{
	int device;                    /* CUDA device ordinal */
	int slots;                     /* requests running at once (>= 1) */
	unsigned long long hbm_budget; /* bytes admitted requests may hold */
	int verbose;                   /* passed to each run */
	int reserved[7];
} ccf_server_config;

typedef enum ccf_request_state
{
	CCF_REQUEST_QUEUED = 0,
	CCF_REQUEST_RUNNING = 1,
	CCF_REQUEST_DONE = 2,
	CCF_REQUEST_FAILED = 3,
	CCF_REQUEST_REJECTED = 4
} ccf_request_state;

typedef struct ccf_request_info
{
	int state;                 /* ccf_request_state */
	int status;                /* ccf_status of the run once done, failed or rejected */
	int deferred;              /* 1 if it waited at the head of the queue for memory */
	int reserved0;
	unsigned long long bytes;  /* admission estimate */
	double t_submit;           /* seconds since the server was created */
	double t_start;
	double t_end;
	double reserved[4];
} ccf_request_info;

typedef struct ccf_server_stats
{
	long long submitted, admitted, completed, failed, rejected, deferred, queued, running;
	unsigned long long bytes_in_use, hbm_budget;
	double reserved[4];
} ccf_server_stats;

ccf_status ccf_server_create(const ccf_server_config* cfg, ccf_server** out);
/* queue a request; *id identifies it in the calls below */
ccf_status ccf_server_submit(ccf_server* s, const ccf_params* p, long long* id);
/* wait until the request is done, failed or rejected (timeout_seconds < 0:
   no limit); CCF_ERR_TIMEOUT if it is still queued or running */
ccf_status ccf_server_wait(ccf_server* s, long long id, double timeout_seconds);
ccf_status ccf_server_request_info(ccf_server* s, long long id, ccf_request_info* out);
/* the handle holding a finished request's field and results (owned by the
   server until ccf_server_release; use ccf_get_results, ccf_get_info,
   ccf_save, ccf_last_error on it) */
ccf_status ccf_server_handle(ccf_server* s, long long id, ccf_handle** h);
/* free a finished request's device memory and return it to the budget */
ccf_status ccf_server_release(ccf_server* s, long long id);
ccf_status ccf_server_get_stats(ccf_server* s, ccf_server_stats* out);
/* waits for running requests, drops queued ones, frees everything */
void ccf_server_destroy(ccf_server* s);

#ifdef __cplusplus
}
#endif

#endif /* CCF_GB300_H */
