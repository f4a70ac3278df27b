/******************************************************************************
noalloc.cu -- the continuation of one (branch, side) row with no device
allocation: ccf_continue_branch_noalloc.

Some callers cannot call cudaMalloc at the point where they need more phi
steps of a branch: code that runs while a host framework owns every byte of
device memory through its own pool, or a real-time loop that must not take
the allocator's locks or trigger implicit synchronisation.  For them the
solver's per-row scratch (root positions, their FP32 snapshot, convergence
flags, the active-root list and the launch descriptors) lives in the
file-scope device array below instead of in buffers the engine allocates.
The array holds NOALLOC_SCRATCH_BYTES (8 MiB); every GPU that loads the
library keeps it until the process exits.  A row of R roots needs about
69 R bytes plus 8 KiB, so R may be up to about 120 000; larger rows are
rejected with CCF_ERR_INVALID_ARGUMENT.

All calls share the one array and it keeps the last call's contents; calls
whose work overlaps on the GPU (two streams, or two host threads) race on it
and must be serialised by the caller.  The launch descriptors reach the
scratch through the parameters of a small set-up kernel enqueued on the
caller's stream, so a call reads no host memory after it returns.  The
continuation is followed by the same FP64 polish as ccf_run (polish.cu) over
the columns this call wrote.
******************************************************************************/
#include "../../include/ccf_gb300.h"
#include "engine.h"

#include <mutex>
#include <string>

namespace
{

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)8 << 20;
constexpr int MAX_DEVICES = 64;

/* The scratch.  In host code this name is only a stand-in for the symbol:
   its device address comes from cudaGetSymbolAddress, per device. */
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[MAX_DEVICES] = {};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

/* device address of the scratch on the current device, looked up once per
   device (a cudaDeviceReset by the caller invalidates it: the entry point is
   documented as needing the context it first ran in) */
cudaError_t scratch_address(int dev, unsigned char** out)
{
	std::lock_guard<std::mutex> lock(g_setup_mutex);
	if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
	if (!g_scratch_addr[dev])
	{
		void* p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess) return e;
		g_scratch_addr[dev] = (unsigned char*)p;
	}
	*out = g_scratch_addr[dev];
	return cudaSuccess;
}

/* writes the launch descriptors into the scratch and clears the statistics:
   everything arrives as kernel parameters, none of it from host memory */
__global__ void noalloc_setup_kernel(const ccf::FieldView v, const ccf::FieldOut o, const ccf::RowDesc r, const float4* hilo,
	unsigned char* base, size_t o_view, size_t o_out, size_t o_row, size_t o_hilo, size_t o_stats, size_t o_plist)
{
	if (blockIdx.x == 0 && threadIdx.x == 0) *(unsigned long long*)(base + o_plist) = 0;   /* polish list count */
	if (blockIdx.x != 0) return;
	if (threadIdx.x == 0)
	{
		*(ccf::FieldView*)(base + o_view) = v;
		*(ccf::FieldOut*)(base + o_out) = o;
		*(ccf::RowDesc*)(base + o_row) = r;
		*(const float4**)(base + o_hilo) = hilo;
	}
	unsigned long long* st = (unsigned long long*)(base + o_stats);
	for (int i = threadIdx.x; i < ccf::STATS_WORDS; i += blockDim.x) st[i] = 0;
}

} /* namespace */

/* the handle layout is private to capi.cu; these accessors are defined there */
ccf::Field* ccf_internal_field(ccf_handle* h);
ccf::Engine* ccf_internal_engine(ccf_handle* h);
void ccf_internal_set_error(ccf_handle* h, const std::string& msg);

extern "C" ccf_status ccf_continue_branch_noalloc(ccf_handle* h, int branch, int side, int num_steps,
	const double* start_roots, double* ccs, double* errs, double* caustics, void* stream)
{
	if (!h) return CCF_ERR_INVALID_ARGUMENT;
	ccf::Field& f = *ccf_internal_field(h);
	ccf::Engine& eng = *ccf_internal_engine(h);
	if (!f.ran)
	{
		ccf_internal_set_error(h, "Error. The field has not been built: call ccf_run first.");
		return CCF_ERR_NOT_RUN;
	}
	const ccf_params& p = f.params;
	const int R = f.d.num_roots, nb = p.num_branches, half = p.num_phi / (2 * nb);
	if (branch < 0 || branch >= nb || (side != 0 && side != 1) || num_steps < 1 || num_steps > half)
	{
		ccf_internal_set_error(h, "Error. branch must be in [0, num_branches), side 0 or 1, num_steps in [1, num_phi / (2 num_branches)].");
		return CCF_ERR_INVALID_ARGUMENT;
	}
	if (!start_roots || !ccs || !errs)
	{
		ccf_internal_set_error(h, "Error. start_roots, ccs and errs must be device pointers.");
		return CCF_ERR_INVALID_ARGUMENT;
	}
	const bool mixed = p.precision == CCF_PRECISION_MIXED;
	/* scratch layout: descriptors, statistics, then the row arrays */
	const size_t o_view = 0;
	const size_t o_out = align256(o_view + sizeof(ccf::FieldView));
	const size_t o_row = align256(o_out + sizeof(ccf::FieldOut));
	const size_t o_hilo = align256(o_row + sizeof(ccf::RowDesc));
	const size_t o_stats = align256(o_hilo + sizeof(const float4*));
	const size_t o_master = align256(o_stats + ccf::STATS_WORDS * sizeof(unsigned long long));
	const size_t o_snap = align256(o_master + (size_t)R * sizeof(double2));
	const size_t o_fin = align256(o_snap + (size_t)R * (mixed ? sizeof(float4) : sizeof(double2)));
	const size_t o_list = align256(o_fin + (size_t)R);
	const size_t o_fval = align256(o_list + (size_t)R * sizeof(int));
	const size_t o_plist = align256(o_fval + 2 * (size_t)R * sizeof(double2));
	const size_t need = o_plist + 256;
	if (need > NOALLOC_SCRATCH_BYTES)
	{
		ccf_internal_set_error(h, "Error. A row of " + std::to_string(R) + " roots needs " + std::to_string(need) +
			" bytes of scratch; ccf_continue_branch_noalloc has " + std::to_string(NOALLOC_SCRATCH_BYTES) + ".");
		return CCF_ERR_INVALID_ARGUMENT;
	}
	/* the caller's current device is put back before returning */
	int caller_dev = -1;
	cudaError_t e = cudaGetDevice(&caller_dev);
	if (e == cudaSuccess && caller_dev != eng.device) e = cudaSetDevice(eng.device);
	auto restore = [&]() {
		if (caller_dev >= 0 && caller_dev != eng.device) cudaSetDevice(caller_dev);
	};
	unsigned char* base = nullptr;
	if (e == cudaSuccess) e = scratch_address(eng.device, &base);
	if (e != cudaSuccess)
	{
		restore();
		ccf_internal_set_error(h, std::string("CUDA error in ccf_continue_branch_noalloc setup: ") + cudaGetErrorString(e));
		return CCF_ERR_CUDA;
	}
	cudaStream_t s = (cudaStream_t)stream;

	ccf::FieldOut o;
	std::memset(&o, 0, sizeof(o));
	o.ccs = (double2*)ccs;
	o.caustics = (double2*)caustics;
	o.errs = errs;
	o.mu = nullptr;
	o.nb = nb;
	o.nphi = p.num_phi;
	o.cols = p.num_phi / nb + 1;
	o.half = half;
	o.step_first = 1;
	o.step_last = num_steps;
	ccf::full_window(o);
	o.seg = 1;
	o.max_iters_init = p.max_iters_init;
	o.max_iters_step = p.max_iters_step;
	o.stats = (unsigned long long*)(base + o_stats);
	ccf::RowDesc r;
	r.field = 0;
	r.branch = branch;
	r.side = side;
	r.steps = num_steps;
	r.base = 0;
	r.cont_base = 0;
	const float4* hilo = mixed ? f.star_hilo.ptr : nullptr;

	noalloc_setup_kernel<<<1, 32, 0, s>>>(f.view, o, r, hilo, base, o_view, o_out, o_row, o_hilo, o_stats, o_plist);
	e = cudaGetLastError();
	if (e == cudaSuccess) e = cudaMemcpyAsync(base + o_master, start_roots, (size_t)R * sizeof(double2), cudaMemcpyDeviceToDevice, s);
	if (e == cudaSuccess)
	{
		if (mixed) ccf::launch_star_hilo(s, R, (const double2*)(base + o_master), (float4*)(base + o_snap));
		else e = cudaMemcpyAsync(base + o_snap, start_roots, (size_t)R * sizeof(double2), cudaMemcpyDeviceToDevice, s);
	}
	if (e == cudaSuccess) e = cudaGetLastError();
	if (e != cudaSuccess)
	{
		restore();
		ccf_internal_set_error(h, std::string("CUDA error in ccf_continue_branch_noalloc: ") + cudaGetErrorString(e));
		return CCF_ERR_CUDA;
	}
	ccf::SolveArgs A;
	std::memset(&A, 0, sizeof(A));
	A.fields = (const ccf::FieldView*)(base + o_view);
	A.outs = (const ccf::FieldOut*)(base + o_out);
	A.rows = (const ccf::RowDesc*)(base + o_row);
	A.num_rows = 1;
	int cl = 1;
	while (cl < 8 && R / (cl * 2) >= 256) cl *= 2;
	A.cluster = cl;
	A.master = (double2*)(base + o_master);
	A.snap32 = mixed ? (float4*)(base + o_snap) : nullptr;
	A.snap64 = mixed ? nullptr : (double2*)(base + o_snap);
	A.fin = base + o_fin;
	A.list = (int*)(base + o_list);
	A.fval = (double2*)(base + o_fval);
	A.star_hilo = (const float4* const*)(base + o_hilo);
	A.error = nullptr;
	e = ccf::launch_solve(s, A, mixed, false);
	if (e == cudaSuccess)
	{
		/* the FP64 polish of ccf_run, over the columns written here */
		ccf::PolishArgs PA;
		PA.fields = A.fields;
		PA.outs = A.outs;
		PA.num_fields = 1;
		PA.b0 = branch;
		PA.nbs = 1;
		PA.k0 = side == 0 ? half - num_steps : half + 1;
		PA.nks = num_steps;
		/* the rest of the scratch lists the points to polish (count first) */
		PA.list_count = (unsigned long long*)(base + o_plist);
		PA.list = PA.list_count + 32;
		PA.list_cap = (long long)((NOALLOC_SCRATCH_BYTES - o_plist) / sizeof(unsigned long long)) - 32;
		e = ccf::launch_polish(s, PA, (long long)R * num_steps, eng.num_sms);
	}
	restore();
	if (e != cudaSuccess)
	{
		ccf_internal_set_error(h, std::string("CUDA error in ccf_continue_branch_noalloc launch: ") + cudaGetErrorString(e));
		return CCF_ERR_CUDA;
	}
	return CCF_OK;
}
