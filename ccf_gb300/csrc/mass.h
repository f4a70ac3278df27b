/******************************************************************************
mass.h -- mass functions of the point-mass lenses, host and device.

The five laws of the reference (include/mass_functions.cuh:17-25):
equal, uniform (power law of slope 0), Salpeter (slope -2.35), Kroupa (broken
power law, slopes -0.3 / -1.3 / -2.3 with breaks at 0.08 and 0.5 solar
masses) and optical_depth (two masses contributing equal convergence).

Power laws are held as up to three segments, each with its lower edge, slope,
normalisation b and the cumulative probability before it; a draw inverts the
segment's integral of b m^a (the reference's invert_power_integral,
include/mass_functions/power_law.cuh:87-101).  The segment table is built
once on the host with the reference's formulas
(include/mass_functions/kroupa.cuh:53-123) and evaluated per star on the
device.
******************************************************************************/
#pragma once

#include <cmath>
#include <cstring>
#include <string>

#ifdef __CUDACC__
#define CCF_MF_HD __host__ __device__
#else
#define CCF_MF_HD
#endif

namespace ccf
{

enum MassFunctionKind
{
	MF_EQUAL = 0,
	MF_UNIFORM = 1,
	MF_SALPETER = 2,
	MF_KROUPA = 3,
	MF_OPTICAL_DEPTH = 4
};

struct MassTable
{
	int kind;
	int nseg;            /* power-law segments used (1..3) */
	double m_lower;      /* in the units the stars carry (m_solar applied) */
	double m_upper;
	double x0[3];        /* lower edge of each segment */
	double slope[3];
	double b[3];         /* normalisation of b m^slope in the segment */
	double cum[3];       /* probability mass of segments before this one */
	double prob[3];      /* probability of the segment */
};

inline int mass_function_kind(const std::string& s)
{
	if (s == "equal") return MF_EQUAL;
	if (s == "uniform") return MF_UNIFORM;
	if (s == "salpeter") return MF_SALPETER;
	if (s == "kroupa") return MF_KROUPA;
	if (s == "optical_depth") return MF_OPTICAL_DEPTH;
	return -1;
}

/* integral of b x^a over [x1, x2] (power_law.cuh:30-44) */
CCF_MF_HD inline double mf_power_integral(double x1, double x2, double a, double b = 1)
{
	if (a != -1) return b * (pow(x2, a + 1) - pow(x1, a + 1)) / (a + 1);
	return b * (log(x2) - log(x1));
}
/* integral of b x^a ln x over [x1, x2] (power_law.cuh:59-73) */
inline double mf_power_log_integral(double x1, double x2, double a, double b = 1)
{
	if (a != -1)
	{
		return b * (std::pow(x2, a + 1) * ((a + 1) * std::log(x2) - 1) - std::pow(x1, a + 1) * ((a + 1) * std::log(x1) - 1)) / ((a + 1) * (a + 1));
	}
	return b * (std::log(x2) * std::log(x2) - std::log(x1) * std::log(x1)) / 2;
}
/* x with integral of b m^a over [x1, x] equal to p (power_law.cuh:87-101) */
CCF_MF_HD inline double mf_invert(double p, double x1, double a, double b)
{
	if (a != -1) return pow(p * (a + 1) / b + pow(x1, a + 1), 1 / (a + 1));
	return x1 * exp(p / b);
}

/* Build the segment table.  ml, mu already carry m_solar, as after
   include/ccf.cuh:359-368. */
inline MassTable make_mass_table(int kind, double ml, double mu, double ms)
{
	MassTable t;
	std::memset(&t, 0, sizeof(t));
	t.kind = kind;
	t.m_lower = ml;
	t.m_upper = mu;
	if (kind == MF_UNIFORM || kind == MF_SALPETER)
	{
		double a = kind == MF_SALPETER ? -2.35 : 0.0;
		t.nseg = 1;
		t.x0[0] = ml;
		t.slope[0] = a;
		t.prob[0] = 1;
		if (ml != mu) t.b[0] = 1 / mf_power_integral(ml, mu, a);
	}
	else if (kind == MF_KROUPA)
	{
		const double s[3] = {-0.3, -1.3, -2.3};
		const double m0 = 0.08 * ms, m1 = 0.5 * ms;
		/* segments present between ml and mu, with continuity factors */
		double lo[3] = {ml, m0, m1}, hi[3] = {m0, m1, mu};
		int first = ml < m0 ? 0 : (ml < m1 ? 1 : 2);
		int last = mu < m0 ? 0 : (mu < m1 ? 1 : 2);
		double pr[3] = {0, 0, 0}, cont[3] = {1, 1, 1};
		for (int k = first + 1; k <= last; k++)
		{
			double brk = k == 1 ? m0 : m1;
			cont[k] = cont[k - 1] * std::pow(brk, s[k - 1] - s[k]);
		}
		for (int k = first; k <= last; k++)
		{
			double a = (k == first) ? ml : lo[k];
			double bnd = (k == last) ? mu : hi[k];
			pr[k] = mf_power_integral(a, bnd, s[k]) * cont[k];
		}
		double tot = 0;
		for (int k = first; k <= last; k++) tot += pr[k];
		double b0 = 1 / tot;
		double cum = 0;
		t.nseg = 3;
		for (int k = 0; k < 3; k++)
		{
			t.slope[k] = s[k];
			t.x0[k] = (k == first) ? ml : lo[k];
			t.b[k] = (k >= first && k <= last) ? b0 * cont[k] : 0;
			t.prob[k] = (k >= first && k <= last) ? pr[k] * b0 : 0;
			t.cum[k] = cum;
			cum += t.prob[k];
		}
	}
	return t;
}

/* one mass from a uniform deviate p in (0, 1] (mass functions' mass()) */
CCF_MF_HD inline double mass_draw(const MassTable& t, double p)
{
	switch (t.kind)
	{
	case MF_EQUAL:
		return 1;
	case MF_OPTICAL_DEPTH:
		if (t.m_lower == t.m_upper) return t.m_lower;
		return (p <= t.m_upper / (t.m_lower + t.m_upper)) ? t.m_lower : t.m_upper;
	case MF_KROUPA:
	{
		if (t.m_lower == t.m_upper) return t.m_lower;
		int k;
		if (p < t.prob[0]) k = 0;
		else if (p < t.prob[0] + t.prob[1]) k = 1;
		else k = 2;
		return mf_invert(p - t.cum[k], t.x0[k], t.slope[k], t.b[k]);
	}
	default:
		if (t.m_lower == t.m_upper) return t.m_lower;
		return mf_invert(p, t.x0[0], t.slope[0], t.b[0]);
	}
}

/* <m>, <m^2>, <m^2 ln m> of the law (the mass functions' mean_mass*()) */
inline void mass_moments(const MassTable& t, double& m1, double& m2, double& m2ln)
{
	const double ml = t.m_lower, mu = t.m_upper;
	if (t.kind == MF_EQUAL)
	{
		m1 = 1; m2 = 1; m2ln = 0;
		return;
	}
	if (ml == mu)
	{
		m1 = ml; m2 = ml * ml; m2ln = ml * ml * std::log(ml);
		return;
	}
	if (t.kind == MF_OPTICAL_DEPTH)
	{
		m1 = 2 * ml * mu / (ml + mu);
		m2 = ml * mu;
		m2ln = ml * mu * (ml * std::log(ml) + mu * std::log(mu)) / (ml + mu);
		return;
	}
	m1 = m2 = m2ln = 0;
	for (int k = 0; k < t.nseg; k++)
	{
		if (t.b[k] == 0) continue;
		double lo = t.x0[k];
		double hi = (k + 1 < t.nseg && t.b[k + 1] != 0) ? t.x0[k + 1] : mu;
		m1 += mf_power_integral(lo, hi, t.slope[k] + 1, t.b[k]);
		m2 += mf_power_integral(lo, hi, t.slope[k] + 2, t.b[k]);
		m2ln += mf_power_log_integral(lo, hi, t.slope[k] + 2, t.b[k]);
	}
}

} /* namespace ccf */
