/******************************************************************************
capi.cu -- the extern "C" entry points declared in include/ccf_gb300.h.
A handle owns one field (its parameters, device data and results) and an
engine (its stream and solver buffers).
******************************************************************************/
#include "../../include/ccf_gb300.h"
#include "engine.h"

#include <cstring>
#include <new>
#include <string>

struct ccf_handle
{
	ccf::Field field;
	ccf::Engine engine;
	std::string last_error;
};

bool ccf_internal_autotune_apply(ccf_handle* h);   /* autotune.cpp */
ccf::Field* ccf_internal_field(ccf_handle* h) { return &h->field; }
ccf::Engine* ccf_internal_engine(ccf_handle* h) { return &h->engine; }
void ccf_internal_set_error(ccf_handle* h, const std::string& msg) { h->last_error = msg; }

static ccf_status fail(ccf_handle* h, ccf_status s, const std::string& msg)
{
	if (h) h->last_error = msg;
	return s;
}

extern "C" {

int ccf_abi_version(void) { return CCF_GB300_ABI_VERSION; }

void ccf_default_params(ccf_params* p)
{
	if (!p) return;
	std::memset(p, 0, sizeof(*p));
	/* include/ccf.cuh:42-62 */
	p->kappa_tot = 0.3;
	p->shear = 0.3;
	p->kappa_star = 0.27;
	p->theta_star = 1;
	std::strcpy(p->mass_function, "equal");
	p->m_solar = 1;
	p->m_lower = 0.01;
	p->m_upper = 50;
	p->rectangular = 0;
	p->approx = 1;
	p->safety_scale = 1.37;
	p->num_stars = 137;
	p->starfile[0] = 0;
	p->num_phi = 100;
	p->num_branches = 1;
	p->random_seed = 0;
	p->write_stars = 1;
	p->write_critical_curves = 1;
	p->write_caustics = 1;
	p->write_mu_length_scales = 0;
	std::strcpy(p->outfile_prefix, "./");
	p->precision = CCF_PRECISION_MIXED;
	p->output_float = 0;
	p->max_iters_init = 300;
	p->max_iters_step = 60;
	p->exact_binomials = 0;
	p->device = 0;
	p->continuation = CCF_CONTINUATION_TRACK;
	p->solved_centres = 0;
}

ccf_status ccf_create(ccf_handle** out)
{
	if (!out) return CCF_ERR_INVALID_ARGUMENT;
	ccf_handle* h = new (std::nothrow) ccf_handle();
	if (!h) return CCF_ERR_OUT_OF_MEMORY;
	ccf_default_params(&h->field.params);
	*out = h;
	return CCF_OK;
}

void ccf_destroy(ccf_handle* h) { delete h; }

ccf_status ccf_set_params(ccf_handle* h, const ccf_params* p)
{
	if (!h || !p) return fail(h, CCF_ERR_INVALID_ARGUMENT, "Error. Null argument.");
	/* results stay valid when only the file-writing fields change, so that
	   run(); set prefix; save() works as with the reference's public fields */
	ccf_params a = h->field.params, b = *p;
	std::memset(a.outfile_prefix, 0, sizeof(a.outfile_prefix));
	std::memset(b.outfile_prefix, 0, sizeof(b.outfile_prefix));
	a.write_stars = b.write_stars = 0;
	a.write_critical_curves = b.write_critical_curves = 0;
	a.output_float = b.output_float = 0;
	a.random_seed = b.random_seed = 0;
	bool same = std::memcmp(&a, &b, sizeof(a)) == 0;
	int seed = h->field.params.random_seed;
	h->field.params = *p;
	h->field.params.mass_function[sizeof(p->mass_function) - 1] = 0;
	h->field.params.starfile[sizeof(p->starfile) - 1] = 0;
	h->field.params.outfile_prefix[sizeof(p->outfile_prefix) - 1] = 0;
	if (!same || (p->random_seed != 0 && p->random_seed != seed)) h->field.ran = false;
	return CCF_OK;
}

ccf_status ccf_get_params(const ccf_handle* h, ccf_params* p)
{
	if (!h || !p) return CCF_ERR_INVALID_ARGUMENT;
	*p = h->field.params;
	return CCF_OK;
}

ccf_status ccf_set_stars(ccf_handle* h, int n, const double* xym, int rectangular, double corner_x1, double corner_x2,
	double theta_star)
{
	if (!h) return CCF_ERR_INVALID_ARGUMENT;
	h->field.ran = false;
	if (n == 0)
	{
		h->field.user_stars.reset();
		return CCF_OK;
	}
	if (n < 0 || !xym) return fail(h, CCF_ERR_INVALID_ARGUMENT, "Error. Invalid num_stars input. num_stars must be an integer > 0");
	if (rectangular != 0 && rectangular != 1)
		return fail(h, CCF_ERR_INVALID_ARGUMENT, "Error. Invalid rectangular input. rectangular must be 1 (rectangular) or 0 (circular).");
	auto sf = std::make_unique<ccf::StarField>();
	sf->n = n;
	sf->rectangular = rectangular;
	sf->corner_x1 = corner_x1;
	sf->corner_x2 = corner_x2;
	sf->theta = theta_star;
	sf->xym.assign(xym, xym + (size_t)3 * n);
	h->field.user_stars = std::move(sf);
	return CCF_OK;
}

ccf_status ccf_run(ccf_handle* h, int verbose)
{
	if (!h) return CCF_ERR_INVALID_ARGUMENT;
	h->last_error.clear();
	if (h->field.params.autotune > 0 && !ccf_internal_autotune_apply(h))
		return fail(h, CCF_ERR_CUDA, "Error. The autotuner could not run the field: " + h->engine.error);
	std::vector<ccf::Field*> fs{&h->field};
	ccf_status rc = h->engine.run(fs, verbose);
	if (rc != CCF_OK) h->last_error = h->engine.error;
	return rc;
}

ccf_status ccf_run_batch(ccf_handle** handles, int n, int verbose)
{
	if (!handles || n < 1) return CCF_ERR_INVALID_ARGUMENT;
	std::vector<ccf::Field*> fs;
	for (int i = 0; i < n; i++)
	{
		if (!handles[i]) return CCF_ERR_INVALID_ARGUMENT;
		handles[i]->last_error.clear();
		fs.push_back(&handles[i]->field);
	}
	ccf_status rc = handles[0]->engine.run(fs, verbose);
	if (rc != CCF_OK)
	{
		for (int i = 0; i < n; i++) handles[i]->last_error = fs[i]->error.empty() ? handles[0]->engine.error : fs[i]->error;
	}
	return rc;
}

ccf_status ccf_save(ccf_handle* h, int verbose)
{
	if (!h) return CCF_ERR_INVALID_ARGUMENT;
	ccf_status rc = h->engine.save(h->field, verbose);
	if (rc != CCF_OK) h->last_error = h->engine.error;
	return rc;
}

ccf_status ccf_get_info(const ccf_handle* h, ccf_info* info)
{
	if (!h || !info) return CCF_ERR_INVALID_ARGUMENT;
	*info = h->field.info;
	return h->field.ran ? CCF_OK : CCF_ERR_NOT_RUN;
}

ccf_status ccf_get_results(ccf_handle* h, double* ccs, double* caustics, double* errs, double* mu_length_scales, double* stars)
{
	if (!h) return CCF_ERR_INVALID_ARGUMENT;
	ccf_status rc = h->engine.copy_results(h->field, ccs, caustics, errs, mu_length_scales, stars);
	if (rc != CCF_OK) h->last_error = h->engine.error;
	return rc;
}

ccf_status ccf_get_device_results(ccf_handle* h, const double** ccs, const double** caustics, const double** errs,
	const double** mu_length_scales)
{
	if (!h) return CCF_ERR_INVALID_ARGUMENT;
	if (!h->field.ran) return fail(h, CCF_ERR_NOT_RUN, "Error. No results: run() has not completed.");
	if (ccs) *ccs = (const double*)h->field.out_ccs;
	if (errs) *errs = h->field.out_errs;
	if (caustics) *caustics = (const double*)h->field.out_caustics;
	if (mu_length_scales) *mu_length_scales = h->field.out_mu;
	return CCF_OK;
}

ccf_status ccf_host_alloc(size_t bytes, void** out)
{
	if (!out) return CCF_ERR_INVALID_ARGUMENT;
	*out = nullptr;
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
	{
		cudaGetLastError();
		return CCF_ERR_NO_DEVICE;
	}
	/* mapped and portable: the library's copy kernel can write it from any device */
	if (cudaHostAlloc(out, bytes > 0 ? bytes : 1, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess)
	{
		cudaGetLastError();
		*out = nullptr;
		return CCF_ERR_OUT_OF_MEMORY;
	}
	return CCF_OK;
}

ccf_status ccf_host_free(void* p)
{
	if (!p) return CCF_OK;
	return cudaFreeHost(p) == cudaSuccess ? CCF_OK : CCF_ERR_CUDA;
}

const char* ccf_last_error(const ccf_handle* h)
{
	if (!h) return "null handle";
	return h->last_error.c_str();
}

ccf_status ccf_derive_params(const ccf_params* p, ccf_info* info, char* msg, size_t msg_len)
{
	if (!p || !info) return CCF_ERR_INVALID_ARGUMENT;
	std::string m;
	ccf::StarField sf;
	const ccf::StarField* sfp = nullptr;
	if (p->starfile[0])
	{
		if (!ccf::read_star_file(p->starfile, sf, m))
		{
			if (msg && msg_len) std::snprintf(msg, msg_len, "%s", m.c_str());
			return CCF_ERR_IO;
		}
		sfp = &sf;
	}
	ccf::Derived d;
	if (!ccf::derive_params(*p, sfp, d, m))
	{
		if (msg && msg_len) std::snprintf(msg, msg_len, "%s", m.c_str());
		return CCF_ERR_INVALID_ARGUMENT;
	}
	std::memset(info, 0, sizeof(*info));
	info->num_stars = d.num_stars;
	info->num_roots = d.num_roots;
	info->taylor_smooth = d.taylor_smooth;
	info->rectangular = d.rectangular;
	info->random_seed = d.random_seed;
	info->kappa_star = d.kappa_star;
	info->theta_star = d.theta;
	info->corner_x1 = d.corner_x1;
	info->corner_x2 = d.corner_x2;
	info->mu_ave = d.mu_ave;
	info->alpha_error = d.alpha_error;
	info->mean_mass = d.mean_mass;
	info->mean_mass2 = d.mean_mass2;
	info->mean_mass2_ln_mass = d.mean_mass2_ln_mass;
	info->m_lower = d.m_lower;
	info->m_upper = d.m_upper;
	info->num_points = (long long)d.num_roots * (p->num_phi + p->num_branches);
	if (msg && msg_len) msg[0] = 0;
	return CCF_OK;
}

ccf_status ccf_eval_points(ccf_handle* h, int n, const double* z, const double* phi, double* f, double* df,
	double* w, double* err, double* mu_length)
{
	if (!h || n < 0 || (n > 0 && (!z || !phi))) return CCF_ERR_INVALID_ARGUMENT;
	if (!h->field.ran) return fail(h, CCF_ERR_NOT_RUN, "Error. No results: run() has not completed.");
	if (n == 0) return CCF_OK;
	cudaStream_t s = h->engine.stream;
	ccf::DBuf<double2> dz, df_, dd, dw;
	ccf::DBuf<double> dphi, de, dm;
	if (dz.ensure(n) || df_.ensure(n) || dd.ensure(n) || dw.ensure(n) || dphi.ensure(n) || de.ensure(n) || dm.ensure(n))
		return fail(h, CCF_ERR_OUT_OF_MEMORY, "Error. cudaMalloc failed in ccf_eval_points");
	cudaMemcpyAsync(dz.ptr, z, n * sizeof(double2), cudaMemcpyHostToDevice, s);
	cudaMemcpyAsync(dphi.ptr, phi, n * sizeof(double), cudaMemcpyHostToDevice, s);
	cudaError_t e = ccf::launch_eval_points(s, h->field.view_dev.ptr, n, dz.ptr, dphi.ptr, df_.ptr, dd.ptr, dw.ptr, de.ptr, dm.ptr);
	if (e == cudaSuccess && f) e = cudaMemcpyAsync(f, df_.ptr, n * sizeof(double2), cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess && df) e = cudaMemcpyAsync(df, dd.ptr, n * sizeof(double2), cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess && w) e = cudaMemcpyAsync(w, dw.ptr, n * sizeof(double2), cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess && err) e = cudaMemcpyAsync(err, de.ptr, n * sizeof(double), cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess && mu_length) e = cudaMemcpyAsync(mu_length, dm.ptr, n * sizeof(double), cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	if (e != cudaSuccess) return fail(h, CCF_ERR_CUDA, std::string("CUDA error in ccf_eval_points: ") + cudaGetErrorString(e));
	return CCF_OK;
}

ccf_status ccf_fmm_error(ccf_handle* h, double* max_error)
{
	if (!h || !max_error) return CCF_ERR_INVALID_ARGUMENT;
	if (!h->field.ran) return fail(h, CCF_ERR_NOT_RUN, "Error. No results: run() has not completed.");
	cudaStream_t s = h->engine.stream;
	ccf::DBuf<unsigned long long> out;
	if (out.ensure(1)) return fail(h, CCF_ERR_OUT_OF_MEMORY, "Error. cudaMalloc failed in ccf_fmm_error");
	unsigned long long bits = 0;
	cudaError_t e = cudaMemsetAsync(out.ptr, 0, sizeof(unsigned long long), s);
	if (e == cudaSuccess) e = ccf::launch_fmm_error(s, h->field.view_dev.ptr, h->field.num_leaves, out.ptr);
	if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, out.ptr, sizeof(bits), cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	if (e != cudaSuccess) return fail(h, CCF_ERR_CUDA, std::string("CUDA error in ccf_fmm_error: ") + cudaGetErrorString(e));
	std::memcpy(max_error, &bits, sizeof(double));
	return CCF_OK;
}

ccf_status ccf_write_star_file(const ccf_handle* h, const char* path)
{
	if (!h || !path) return CCF_ERR_INVALID_ARGUMENT;
	ccf_handle* hh = const_cast<ccf_handle*>(h);
	ccf::StarField sf;
	sf.n = h->field.d.num_stars;
	sf.rectangular = h->field.d.rectangular;
	sf.corner_x1 = h->field.d.corner_x1;
	sf.corner_x2 = h->field.d.corner_x2;
	sf.theta = h->field.d.theta;
	sf.xym.resize((size_t)3 * sf.n);
	ccf_status rc = hh->engine.copy_results(hh->field, nullptr, nullptr, nullptr, nullptr, sf.xym.data());
	if (rc != CCF_OK) return rc;
	if (!ccf::write_star_file(path, sf, h->field.params.output_float != 0)) return CCF_ERR_IO;
	return CCF_OK;
}

} /* extern "C" */
