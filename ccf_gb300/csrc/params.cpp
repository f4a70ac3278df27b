/******************************************************************************
params.cpp -- host-side parameter checks, derived parameters, smooth-mass
polynomials, binomial tables and the reference's file formats.
******************************************************************************/
#include "params.h"
#include "common.cuh"
#include "mass.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <limits>
#include <sstream>

namespace ccf
{

namespace
{
constexpr double PI_D = 3.141592653589793238462643383279502884;
constexpr double INV_PI_D = 0.318309886183790671537767526745028724;
constexpr int MAX_TS = 101;   /* include/ccf.cuh:79 */

double dmin() { return std::numeric_limits<double>::min(); }

std::string num(double v)
{
	std::ostringstream s;
	s << v;
	return s.str();
}
}

bool check_params(const ccf_params& p, bool star_input, std::string& msg)
{
	const bool sf = star_input;
	if (p.kappa_tot < dmin()) { msg = "Error. kappa_tot must be >= " + num(dmin()); return false; }
	if (p.kappa_star < dmin()) { msg = "Error. kappa_star must be >= " + num(dmin()); return false; }
	if (!sf && p.kappa_star > p.kappa_tot) { msg = "Error. kappa_star must be <= kappa_tot"; return false; }
	if (!sf && p.theta_star < dmin()) { msg = "Error. theta_star must be >= " + num(dmin()); return false; }
	if (!sf && mass_function_kind(p.mass_function) < 0)
	{
		msg = "Error. mass_function must be equal, uniform, Salpeter, Kroupa, or optical_depth.";
		return false;
	}
	if (!sf && p.m_solar < dmin()) { msg = "Error. m_solar must be >= " + num(dmin()); return false; }
	if (!sf && p.m_lower < dmin()) { msg = "Error. m_lower must be >= " + num(dmin()); return false; }
	if (!sf && p.m_upper < p.m_lower) { msg = "Error. m_upper must be >= m_lower."; return false; }
	if (!sf && p.rectangular != 0 && p.rectangular != 1)
	{
		msg = "Error. rectangular must be 1 (rectangular) or 0 (circular).";
		return false;
	}
	if (p.approx != 0 && p.approx != 1) { msg = "Error. approx must be 1 (approximate) or 0 (exact)."; return false; }
	if (p.safety_scale < 1.1) { msg = "Error. safety_scale must be >= 1.1"; return false; }
	if (p.num_stars < 1) { msg = "Error. num_stars must be an integer > 0"; return false; }
	if (p.num_phi < 1 || p.num_phi % 2 != 0) { msg = "Error. num_phi must be an even integer > 0"; return false; }
	if (p.num_branches < 1) { msg = "Error. num_branches must be an integer > 0"; return false; }
	if (p.num_phi % (2 * p.num_branches) != 0) { msg = "Error. num_phi must be a multiple of 2 * num_branches"; return false; }
	if (p.write_stars != 0 && p.write_stars != 1) { msg = "Error. write_stars must be 1 (true) or 0 (false)."; return false; }
	if (p.write_critical_curves != 0 && p.write_critical_curves != 1)
	{
		msg = "Error. write_critical_curves must be 1 (true) or 0 (false).";
		return false;
	}
	if (p.write_caustics != 0 && p.write_caustics != 1) { msg = "Error. write_caustics must be 1 (true) or 0 (false)."; return false; }
	if (p.write_mu_length_scales != 0 && p.write_mu_length_scales != 1)
	{
		msg = "Error. write_mu_length_scales must be 1 (true) or 0 (false).";
		return false;
	}
	if (p.precision != CCF_PRECISION_FP64 && p.precision != CCF_PRECISION_MIXED)
	{
		msg = "Error. precision must be 0 (fp64) or 1 (mixed).";
		return false;
	}
	if (p.max_iters_init < 1 || p.max_iters_step < 1) { msg = "Error. sweep caps must be >= 1."; return false; }
	if (p.continuation != CCF_CONTINUATION_TRACK && p.continuation != CCF_CONTINUATION_ABERTH)
	{
		msg = "Error. continuation must be 0 (track) or 1 (aberth).";
		return false;
	}
	if (p.solved_centres < 0 || (p.solved_centres > 0 && (p.num_branches <= 0 || p.num_branches % p.solved_centres != 0)))
	{
		msg = "Error. solved_centres must be 0 or a divisor of num_branches.";
		return false;
	}
	if (p.expansion_order != 0 && (p.expansion_order < 3 || p.expansion_order > MAX_ORDER))
	{
		msg = "Error. expansion_order must be 0 (the reference's formula) or in [3, " + std::to_string(MAX_ORDER) + "].";
		return false;
	}
	if (p.leaf_max_stars != 0 && (p.leaf_max_stars < 4 || p.leaf_max_stars > MAX_NEAR))
	{
		msg = "Error. leaf_max_stars must be 0 (the reference's 32) or in [4, " + std::to_string(MAX_NEAR) + "].";
		return false;
	}
	if (p.init_cluster != 0 && p.init_cluster != 1 && p.init_cluster != 2 && p.init_cluster != 4 && p.init_cluster != 8 &&
		p.init_cluster != 16)
	{
		msg = "Error. init_cluster must be 0 (automatic), 1, 2, 4, 8 or 16.";
		return false;
	}
	if (p.host_outputs < 0 || p.host_outputs > 2)
	{
		msg = "Error. host_outputs must be 0, 1 or 2.";
		return false;
	}
	if (p.autotune < 0 || p.autotune > 2)
	{
		msg = "Error. autotune must be 0, 1 or 2.";
		return false;
	}
	return true;
}

/* star statistics of include/star.cuh:124-161, on the host for star input */
static void host_star_stats(const StarField& f, double& kappastar, double& ml, double& mu, double& m1, double& m2, double& m2l)
{
	ml = std::numeric_limits<double>::max();
	mu = std::numeric_limits<double>::min();
	double mt = 0, m2t = 0, mlt = 0;
	for (int i = 0; i < f.n; i++)
	{
		double m = f.xym[3 * i + 2];
		mt += m;
		m2t += m * m;
		mlt += m * m * std::log(m);
		ml = std::min(ml, m);
		mu = std::max(mu, m);
	}
	m1 = mt / f.n;
	m2 = m2t / f.n;
	m2l = mlt / f.n;
	if (f.rectangular) kappastar = mt * PI_D * f.theta * f.theta / (4 * f.corner_x1 * f.corner_x2);
	else
	{
		double a = std::hypot(f.corner_x1, f.corner_x2);
		kappastar = mt * f.theta * f.theta / (a * a);
	}
}

bool derive_params(const ccf_params& p, const StarField* stars, Derived& d, std::string& msg)
{
	d = Derived();
	d.star_input = stars != nullptr;
	if (!check_params(p, d.star_input, msg)) return false;
	d.num_stars = p.num_stars;
	d.rectangular = p.rectangular;
	d.kappa_star = p.kappa_star;
	d.theta = p.theta_star;
	d.random_seed = p.random_seed;
	double cx = 0, cy = 0;
	if (!d.star_input)
	{
		d.mass_kind = mass_function_kind(p.mass_function);
		if (d.mass_kind == MF_EQUAL)
		{
			d.m_lower = 1;
			d.m_upper = 1;
		}
		else
		{
			d.m_lower = p.m_lower * p.m_solar;
			d.m_upper = p.m_upper * p.m_solar;
		}
		MassTable mt = make_mass_table(d.mass_kind, d.m_lower, d.m_upper, p.m_solar);
		mass_moments(mt, d.mean_mass, d.mean_mass2, d.mean_mass2_ln_mass);
	}
	else
	{
		d.num_stars = stars->n;
		d.rectangular = stars->rectangular;
		d.theta = stars->theta;
		cx = stars->corner_x1;
		cy = stars->corner_x2;
		if (stars->n < 1) { msg = "Error. Invalid num_stars input. num_stars must be an integer > 0"; return false; }
		if (cx < 0 || cy < 0) { msg = "Error. Real and imaginary parts of the corner of the star field must both be >= 0"; return false; }
		if (d.theta < dmin()) { msg = "Error. theta_star must be >= " + num(dmin()); return false; }
		host_star_stats(*stars, d.kappa_star, d.m_lower, d.m_upper, d.mean_mass, d.mean_mass2, d.mean_mass2_ln_mass);
		d.random_seed = 0;
	}
	d.mu_ave = 1 / ((1 - p.kappa_tot) * (1 - p.kappa_tot) - p.shear * p.shear);
	if (!d.star_input)
	{
		cx = 1 / std::abs(1 - p.kappa_tot + p.shear);
		cy = 1 / std::abs(1 - p.kappa_tot - p.shear);
		double f;
		if (d.rectangular)
		{
			double ax = std::sqrt(cx / cy), ay = std::sqrt(cy / cx);
			f = std::sqrt(PI_D * d.theta * d.theta * d.num_stars * d.mean_mass / (4 * d.kappa_star));
			cx = ax * f;
			cy = ay * f;
		}
		else
		{
			double a = std::hypot(cx, cy);
			cx /= a;
			cy /= a;
			f = std::sqrt(d.theta * d.theta * d.num_stars * d.mean_mass / d.kappa_star);
			cx *= f;
			cy *= f;
		}
	}
	d.corner_x1 = cx;
	d.corner_x2 = cy;
	d.alpha_error = d.theta * 0.0000001;
	const double cabs = std::hypot(cx, cy);
	const double carg = std::atan2(cy, cx);
	int ts = 1;
	while ((d.kappa_star * INV_PI_D * 4 / (ts + 1) * cabs * (p.safety_scale + 1) / (p.safety_scale - 1)
		* std::pow(1 / p.safety_scale, ts + 1) > d.alpha_error) && ts <= MAX_TS)
	{
		ts += 2;
	}
	while ((std::fmod(carg * (ts - 1), PI_D) < 0.1 * PI_D || std::fmod(carg * (ts - 1), PI_D) > 0.9 * PI_D) && ts <= MAX_TS)
	{
		ts += 2;
	}
	d.taylor_smooth = ts;
	if (d.rectangular && ts > MAX_TS) { msg = "Error. taylor_smooth must be <= " + std::to_string(MAX_TS); return false; }
	if (d.rectangular) d.num_roots = p.approx ? 2 * d.num_stars + ts - 1 : 2 * d.num_stars;
	else d.num_roots = p.approx ? 2 * d.num_stars : 2 * d.num_stars + 2;
	return true;
}

void update_corner(const ccf_params& p, Derived& d, double mean_mass_actual)
{
	if (d.star_input) return;
	double cx = d.corner_x1, cy = d.corner_x2;
	if (d.rectangular)
	{
		double ax = std::sqrt(cx / cy), ay = std::sqrt(cy / cx);
		double f = std::sqrt(PI_D * d.theta * d.theta * d.num_stars * mean_mass_actual / (4 * d.kappa_star));
		d.corner_x1 = ax * f;
		d.corner_x2 = ay * f;
	}
	else
	{
		double a = std::hypot(cx, cy);
		double f = std::sqrt(d.theta * d.theta * d.num_stars * mean_mass_actual / d.kappa_star);
		d.corner_x1 = cx / a * f;
		d.corner_x2 = cy / a * f;
	}
	(void)p;
}

/* The rectangular Taylor form of alpha_smooth (include/alpha_smooth.cuh:63-92,
   186-209, 252-276) rewritten as polynomials in zbar with fixed coefficients:
     d alpha_s/dzbar   = sum_{m=1..M} D1_m u^m + k1,           u = (zbar/c)^2
     d2 alpha_s/dzbar2 = (zbar / c^2) sum_{m=1..M} D2_m u^(m-1)
     alpha_s           = (0, -kappa/pi) sum_{n=0..ts+1} A_n zbar^n - 2 kappa (c.re + z.re)
   with M = (ts - 1)/2, e_i = 1 - exp(2 i i arg c):
     D1_m = 2 (0, -kappa/pi) e_{2m} / (2m),  D2_m = 2 (0, -kappa/pi) e_{2m},
     k1 = kappa - 4 kappa arg(c) / pi,
   and A_n the coefficients of sum_k s_k (c_k - w)(log c_k - sum_{i=1..ts} (w/c_k)^i / i)
   over the corners c_k = c, conj c, -c, -conj c with signs +, -, +, -:
     A_0 = sum s_k c_k log c_k,  A_1 = -sum s_k (log c_k + 1),
     A_n = sum s_k / (n (n - 1) c_k^(n-1)) for 2 <= n <= ts,  A_(ts+1) = sum s_k / (ts c_k^ts).
   Coefficients are formed in long double. */
SmoothPoly smooth_polynomials(double kappa_star, double cx, double cy, int ts)
{
	using CL = std::complex<long double>;
	SmoothPoly s;
	s.m = std::max(0, (ts - 1) / 2);
	const long double k = kappa_star;
	const long double pi = 3.141592653589793238462643383279502884L;
	const long double arg = std::atan2((long double)cy, (long double)cx);
	const CL mk(0, -k / pi);
	for (int m = 1; m <= s.m; m++)
	{
		long double i = 2 * m;
		CL e(1 - std::cos(2 * i * arg), -std::sin(2 * i * arg));
		CL d1 = 2.0L * mk * e / i;
		CL d2 = 2.0L * mk * e;
		s.d1.push_back(std::complex<double>((double)d1.real(), (double)d1.imag()));
		s.d2.push_back(std::complex<double>((double)d2.real(), (double)d2.imag()));
	}
	s.k1 = (double)(k - 4 * k * arg / pi);
	const CL c(cx, cy);
	const CL corners[4] = {c, std::conj(c), -c, -std::conj(c)};
	const long double sign[4] = {1, -1, 1, -1};
	s.a.assign(ts + 2, 0);
	std::vector<CL> A(ts + 2, CL(0, 0));
	for (int q = 0; q < 4; q++)
	{
		CL ck = corners[q];
		CL lk(std::log(std::abs(ck)), std::atan2(ck.imag(), ck.real()));
		A[0] += sign[q] * ck * lk;
		A[1] += sign[q] * (-lk - 1.0L);
		CL ick = 1.0L / ck;
		CL pw = ick;   /* 1 / c_k^(n-1) for n = 2 */
		for (int n = 2; n <= ts; n++)
		{
			A[n] += sign[q] * pw / (long double)(n * (n - 1));
			pw *= ick;
		}
		A[ts + 1] += sign[q] * pw / (long double)ts;
	}
	for (int n = 0; n < ts + 2; n++) s.a[n] = std::complex<double>((double)A[n].real(), (double)A[n].imag());
	s.inv_corner = std::complex<double>(1.0, 0.0) / std::complex<double>(cx, cy);
	s.inv_corner2 = s.inv_corner * s.inv_corner;
	return s;
}

std::vector<double> binomial_table(int n, bool reference_int32)
{
	std::vector<double> out((size_t)(n + 1) * (n + 2) / 2, 0);
	std::vector<int32_t> bi(out.size(), 0);
	std::vector<double> be(out.size(), 0);
	for (int r = 0; r <= n; r++)
	{
		int rs = r * (r + 1) / 2, ps = (r - 1) * r / 2;
		for (int i = 0; i <= r; i++)
		{
			if (i == 0 || i == r)
			{
				bi[rs + i] = 1;
				be[rs + i] = 1;
			}
			else
			{
				bi[rs + i] = (int32_t)((uint32_t)bi[ps + i - 1] + (uint32_t)bi[ps + i]);
				be[rs + i] = be[ps + i - 1] + be[ps + i];
			}
		}
	}
	for (size_t i = 0; i < out.size(); i++) out[i] = reference_int32 ? (double)bi[i] : be[i];
	return out;
}

/* ---------------- files ---------------- */

bool read_star_file(const std::string& path, StarField& out, std::string& msg)
{
	std::filesystem::path fp = path;
	if (fp.extension() == ".bin")
	{
		/* include/star.cuh:175-320 */
		std::error_code ec;
		uintmax_t fsize = std::filesystem::file_size(path, ec);
		if (ec) { msg = "Error determining size of star input file " + path; return false; }
		std::ifstream in(path, std::ios::binary);
		if (!in.is_open()) { msg = "Error. Failed to open file " + path; return false; }
		int32_t n = 0, rect = 0;
		in.read((char*)&n, 4);
		if (!in || n < 1) { msg = "Error. Invalid num_stars input. num_stars must be an integer > 0"; return false; }
		in.read((char*)&rect, 4);
		if (rect != 0 && rect != 1) { msg = "Error. Invalid rectangular input. rectangular must be 1 (rectangular) or 0 (circular)."; return false; }
		out.n = n;
		out.rectangular = rect;
		out.xym.assign((size_t)3 * n, 0);
		if (fsize == 8 + 16 + 8 + (uintmax_t)n * 24)
		{
			double c[2], th;
			in.read((char*)c, 16);
			in.read((char*)&th, 8);
			in.read((char*)out.xym.data(), (size_t)n * 24);
			out.corner_x1 = c[0];
			out.corner_x2 = c[1];
			out.theta = th;
		}
		else if (fsize == 8 + 8 + 4 + (uintmax_t)n * 12)
		{
			float c[2], th;
			in.read((char*)c, 8);
			in.read((char*)&th, 4);
			std::vector<float> tmp((size_t)3 * n);
			in.read((char*)tmp.data(), (size_t)n * 12);
			for (size_t i = 0; i < tmp.size(); i++) out.xym[i] = tmp[i];
			out.corner_x1 = c[0];
			out.corner_x2 = c[1];
			out.theta = th;
		}
		else
		{
			msg = "Error. Star input file " + path + " does not contain validly formatted single or double precision stars and accompanying information.";
			return false;
		}
		if (!in) { msg = "Error. Truncated star input file " + path; return false; }
		if (out.corner_x1 < 0 || out.corner_x2 < 0) { msg = "Error. Real and imaginary parts of the corner of the star field must both be >= 0"; return false; }
		if (out.theta < dmin()) { msg = "Error. theta_star must be >= " + num(dmin()); return false; }
		return true;
	}
	if (fp.extension() == ".txt")
	{
		/* include/star.cuh:334-434 */
		std::ifstream in(path);
		if (!in.is_open()) { msg = "Error. Failed to open file " + path; return false; }
		double x1, x2, m;
		out.xym.clear();
		while (in >> x1 >> x2 >> m)
		{
			out.xym.push_back(x1);
			out.xym.push_back(x2);
			out.xym.push_back(m);
		}
		out.n = (int)(out.xym.size() / 3);
		if (out.n < 1) { msg = "Error. Invalid num_stars input. num_stars must be an integer > 0"; return false; }
		double max_x1 = 0, max_x2 = 0, max_rad = 0, total = 0, I = 0;
		for (int i = 0; i < out.n; i++)
		{
			x1 = out.xym[3 * i];
			x2 = out.xym[3 * i + 1];
			m = out.xym[3 * i + 2];
			total += m;
			I += m * (x1 * x1 + x2 * x2);
			max_x1 = std::max(max_x1, std::abs(x1));
			max_x2 = std::max(max_x2, std::abs(x2));
			max_rad = std::max(max_rad, std::hypot(x1, x2));
		}
		double I_circ = total * max_rad * max_rad / 2;
		double I_rect = total * (max_x1 * max_x1 + max_x2 * max_x2) / 3;
		if (I / I_circ > I / I_rect)
		{
			out.rectangular = 0;
			out.corner_x1 = max_rad;
			out.corner_x2 = 0;
		}
		else
		{
			out.rectangular = 1;
			out.corner_x1 = max_x1;
			out.corner_x2 = max_x2;
		}
		out.theta = 1;
		return true;
	}
	msg = "Error. Star input file " + path + " is not a .bin or .txt file.";
	return false;
}

bool write_star_file(const std::string& path, const StarField& f, bool single)
{
	/* include/star.cuh:498-534 */
	std::ofstream out(path, std::ios::binary);
	if (!out.is_open()) return false;
	int32_t n = f.n, rect = f.rectangular;
	out.write((char*)&n, 4);
	out.write((char*)&rect, 4);
	double c[2] = {f.corner_x1, f.corner_x2};
	if (!rect)
	{
		c[0] = std::hypot(f.corner_x1, f.corner_x2);
		c[1] = 0;
	}
	if (single)
	{
		float cf[2] = {(float)c[0], (float)c[1]}, th = (float)f.theta;
		out.write((char*)cf, 8);
		out.write((char*)&th, 4);
		std::vector<float> tmp(f.xym.begin(), f.xym.end());
		out.write((char*)tmp.data(), (std::streamsize)(tmp.size() * 4));
	}
	else
	{
		out.write((char*)c, 16);
		out.write((char*)&f.theta, 8);
		out.write((char*)f.xym.data(), (std::streamsize)(f.xym.size() * 8));
	}
	return (bool)out;
}

static bool write_array_impl(const std::string& path, const double* v, size_t count, int nrows, int ncols, bool single)
{
	/* include/array_functions.cuh:280-306 */
	if (std::filesystem::path(path).extension() != ".bin") return false;
	std::ofstream out(path, std::ios::binary);
	if (!out.is_open()) return false;
	int32_t r = nrows, c = ncols;
	out.write((char*)&r, 4);
	out.write((char*)&c, 4);
	if (single)
	{
		const size_t block = 1 << 20;
		std::vector<float> tmp;
		for (size_t i = 0; i < count; i += block)
		{
			size_t n = std::min(block, count - i);
			tmp.resize(n);
			for (size_t j = 0; j < n; j++) tmp[j] = (float)v[i + j];
			out.write((char*)tmp.data(), (std::streamsize)(n * 4));
		}
	}
	else
	{
		out.write((const char*)v, (std::streamsize)(count * 8));
	}
	return (bool)out;
}

bool write_array_complex(const std::string& path, const double* z, int nrows, int ncols, bool single)
{
	return write_array_impl(path, z, (size_t)nrows * ncols * 2, nrows, ncols, single);
}

bool write_array_real(const std::string& path, const double* v, int nrows, int ncols, bool single)
{
	return write_array_impl(path, v, (size_t)nrows * ncols, nrows, ncols, single);
}

bool write_parameter_info(const std::string& path, const ccf_params& p, const ccf_info& i, bool star_input)
{
	/* include/ccf.cuh:1129-1192, same keys, order and precision */
	std::ofstream out(path);
	if (!out.is_open()) return false;
	out.precision(9);
	out << "kappa_tot " << p.kappa_tot << "\n";
	out << "shear " << p.shear << "\n";
	out << "mu_ave " << i.mu_ave << "\n";
	out << "smooth_fraction " << (1 - i.kappa_star / p.kappa_tot) << "\n";
	out << "kappa_star " << i.kappa_star << "\n";
	if (!star_input) out << "kappa_star_actual " << i.kappa_star_actual << "\n";
	out << "theta_star " << i.theta_star << "\n";
	out << "random_seed " << i.random_seed << "\n";
	if (!star_input)
	{
		std::string mf = p.mass_function;
		out << "mass_function " << mf << "\n";
		if (mf == "salpeter" || mf == "kroupa") out << "m_solar " << p.m_solar << "\n";
		out << "m_lower " << i.m_lower << "\n";
		out << "m_upper " << i.m_upper << "\n";
		out << "mean_mass " << i.mean_mass << "\n";
		out << "mean_mass2 " << i.mean_mass2 << "\n";
		out << "mean_mass2_ln_mass " << i.mean_mass2_ln_mass << "\n";
	}
	out << "m_lower_actual " << i.m_lower_actual << "\n";
	out << "m_upper_actual " << i.m_upper_actual << "\n";
	out << "mean_mass_actual " << i.mean_mass_actual << "\n";
	out << "mean_mass2_actual " << i.mean_mass2_actual << "\n";
	out << "mean_mass2_ln_mass_actual " << i.mean_mass2_ln_mass_actual << "\n";
	out << "num_stars " << i.num_stars << "\n";
	if (i.rectangular)
	{
		out << "corner_x1 " << i.corner_x1 << "\n";
		out << "corner_x2 " << i.corner_x2 << "\n";
		if (p.approx) out << "taylor_smooth " << i.taylor_smooth << "\n";
	}
	else
	{
		out << "rad " << std::hypot(i.corner_x1, i.corner_x2) << "\n";
	}
	out << "num_roots " << i.num_roots << "\n";
	out << "num_phi " << p.num_phi << "\n";
	out << "num_branches " << p.num_branches << "\n";
	out << "max_error_1/mu " << i.max_error << "\n";
	out << "t_init_roots " << i.t_init_roots << "\n";
	out << "t_ccs " << i.t_ccs << "\n";
	out << "t_caustics " << i.t_caustics << "\n";
	return (bool)out;
}

} /* namespace ccf */
