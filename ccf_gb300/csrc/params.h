/******************************************************************************
params.h -- host-side parameter checks, derived parameters, smooth-mass
polynomials, binomial tables and the reference's file formats.
******************************************************************************/
#pragma once

#include "../../include/ccf_gb300.h"

#include <complex>
#include <string>
#include <vector>

namespace ccf
{

struct StarField
{
	int n = 0;
	int rectangular = 0;
	double corner_x1 = 0;
	double corner_x2 = 0;
	double theta = 1;
	std::vector<double> xym;   /* n triples (x1, x2, mass) */
};

/* everything derived on the host before any device work */
struct Derived
{
	int num_stars = 0;
	int num_roots = 0;
	int taylor_smooth = 0;
	int rectangular = 0;
	int mass_kind = 0;
	int random_seed = 0;
	bool star_input = false;      /* stars come from a file or from ccf_set_stars */
	double kappa_star = 0;
	double theta = 1;
	double m_lower = 0;
	double m_upper = 0;
	double mean_mass = 0;
	double mean_mass2 = 0;
	double mean_mass2_ln_mass = 0;
	double mu_ave = 0;
	double alpha_error = 0;
	double corner_x1 = 0;
	double corner_x2 = 0;
};

/* include/ccf.cuh:218-346; returns false with the reference's message */
bool check_params(const ccf_params& p, bool star_input, std::string& msg);

/* include/ccf.cuh:348-497 (with the star field already read if given) */
bool derive_params(const ccf_params& p, const StarField* stars, Derived& d, std::string& msg);

/* corner after the star statistics are known, include/ccf.cuh:686-700 */
void update_corner(const ccf_params& p, Derived& d, double mean_mass_actual);

/* polynomial forms of the rectangular Taylor alpha_smooth (see smooth.cpp) */
struct SmoothPoly
{
	int m = 0;
	double k1 = 0;
	std::vector<std::complex<double>> d1, d2, a;
	std::complex<double> inv_corner, inv_corner2;
};
SmoothPoly smooth_polynomials(double kappa_star, double cx, double cy, int taylor_smooth);

/* Pascal triangle to row n as doubles; reference_int32 reproduces the
   reference's int32 table (include/binomial_coefficients.cuh:11-44) whose
   entries wrap modulo 2^32 above n = 33 */
std::vector<double> binomial_table(int n, bool reference_int32);

/* files (include/star.cuh:175-534, include/array_functions.cuh:280-306,
   include/ccf.cuh:1123-1192) */
bool read_star_file(const std::string& path, StarField& out, std::string& msg);
bool write_star_file(const std::string& path, const StarField& f, bool single);
bool write_array_complex(const std::string& path, const double* z, int nrows, int ncols, bool single);
bool write_array_real(const std::string& path, const double* v, int nrows, int ncols, bool single);
bool write_parameter_info(const std::string& path, const ccf_params& p, const ccf_info& info, bool star_input);

} /* namespace ccf */
