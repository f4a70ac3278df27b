/******************************************************************************
ccf_gb300.hpp -- header-only C++ class with the public surface of the
reference's CCF<T> (include/ccf.cuh:34-1289): the same public fields with the
same defaults (:42-62), a default constructor (:68-71), bool run(int) (:1265)
and bool save(int) (:1282).  Code written against the reference compiles
against this header by replacing #include "ccf.cuh" with
#include "ccf_gb300.hpp"; the work runs through the C ABI of ccf_gb300.h.

T selects the precision of the output files (float: single, as the reference
built with -D is_float; double: double).  The roots themselves are always
solved to the FP64 function (mixed-precision solver by default).
******************************************************************************/
#pragma once

#include "ccf_gb300.h"

#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <type_traits>
#include <vector>

template <typename T>
class CCF
{
	static_assert(std::is_same_v<T, float> || std::is_same_v<T, double>, "CCF<T>: T must be float or double");

public:
	/* include/ccf.cuh:42-62 */
	T kappa_tot = static_cast<T>(0.3);
	T shear = static_cast<T>(0.3);
	T kappa_star = static_cast<T>(0.27);
	T theta_star = static_cast<T>(1);
	std::string mass_function_str = "equal";
	T m_solar = static_cast<T>(1);
	T m_lower = static_cast<T>(0.01);
	T m_upper = static_cast<T>(50);
	int rectangular = 0;
	int approx = 1;
	T safety_scale = static_cast<T>(1.37);
	int num_stars = 137;
	std::string starfile = "";
	int num_phi = 100;
	int num_branches = 1;
	int random_seed = 0;
	int write_stars = 1;
	int write_critical_curves = 1;
	int write_caustics = 1;
	int write_mu_length_scales = 0;
	std::string outfile_prefix = "./";

	/* additions: solver precision (CCF_PRECISION_MIXED or CCF_PRECISION_FP64),
	   device and continuation (CCF_CONTINUATION_TRACK or CCF_CONTINUATION_ABERTH) */
	int precision = CCF_PRECISION_MIXED;
	int device = 0;
	int continuation = CCF_CONTINUATION_TRACK;

	CCF()
	{
		ccf_create(&h_);
	}
	~CCF()
	{
		ccf_destroy(h_);
	}
	CCF(const CCF&) = delete;
	CCF& operator=(const CCF&) = delete;

	bool run(int verbose)
	{
		if (!push()) return false;
		ccf_status s = ccf_run(h_, verbose);
		if (s != CCF_OK)
		{
			std::cerr << ccf_last_error(h_) << "\n";
			return false;
		}
		ccf_info info;
		ccf_get_info(h_, &info);
		random_seed = info.random_seed;
		return true;
	}

	bool save(int verbose)
	{
		if (!push()) return false;
		ccf_status s = ccf_save(h_, verbose);
		if (s != CCF_OK)
		{
			std::cerr << ccf_last_error(h_) << "\n";
			return false;
		}
		return true;
	}

	/* the underlying handle, for ccf_get_results / ccf_get_device_results */
	ccf_handle* handle() { return h_; }

private:
	ccf_handle* h_ = nullptr;

	bool push()
	{
		if (!h_) return false;
		ccf_params p;
		ccf_default_params(&p);
		p.kappa_tot = kappa_tot;
		p.shear = shear;
		p.kappa_star = kappa_star;
		p.theta_star = theta_star;
		std::snprintf(p.mass_function, sizeof(p.mass_function), "%s", mass_function_str.c_str());
		p.m_solar = m_solar;
		p.m_lower = m_lower;
		p.m_upper = m_upper;
		p.rectangular = rectangular;
		p.approx = approx;
		p.safety_scale = safety_scale;
		p.num_stars = num_stars;
		std::snprintf(p.starfile, sizeof(p.starfile), "%s", starfile.c_str());
		p.num_phi = num_phi;
		p.num_branches = num_branches;
		p.random_seed = random_seed;
		p.write_stars = write_stars;
		p.write_critical_curves = write_critical_curves;
		p.write_caustics = write_caustics;
		p.write_mu_length_scales = write_mu_length_scales;
		std::snprintf(p.outfile_prefix, sizeof(p.outfile_prefix), "%s", outfile_prefix.c_str());
		p.precision = precision;
		p.output_float = std::is_same_v<T, float> ? 1 : 0;
		p.device = device;
		p.continuation = continuation;
		return ccf_set_params(h_, &p) == CCF_OK;
	}
};
