/******************************************************************************
ccf_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the checker, never the product).

A plain FP64 CPU restatement of the reference's critical-curve and caustic
algorithm (weisluke/ccf, include/*.cuh).  Every arithmetic step keeps the
reference's operation order (Smith division, hypot-based modulus, repeated
multiplication for integer powers, the reference's int32 binomial table,
in-place Gauss-Seidel Aberth sweeps in index order), so that a serial run
equals the reference compiled for the host bit for bit.  Each function cites
the reference file:line it restates.

Parallelism: independent (branch, side) rows and independent output points
are spread over OpenMP threads; within a row the sweep order is the serial
one, so results do not depend on the thread count.

Star fields are drawn with curand's XORWOW generator through its host code
path in the CUDA headers (called, not re-implemented), exactly as the
reference's kernels draw them on the device.
******************************************************************************/
#include "ccf_oracle.h"

#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <numbers>
#include <vector>

namespace
{

constexpr double PI = std::numbers::pi_v<double>;
constexpr double INV_PI = std::numbers::inv_pi_v<double>;

double now_s()
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

/******************************************************************************
complex arithmetic with the semantics of include/complex.cuh:10-312
******************************************************************************/
struct Cx
{
	double re = 0;
	double im = 0;
};

inline Cx cx(double r, double i) { return Cx{r, i}; }
inline Cx conj(Cx a) { return Cx{a.re, -a.im}; }                                  /* :73-76 */
inline double cabs(Cx a) { return std::hypot(a.re, a.im); }                      /* :81-84 */
inline double carg(Cx a) { return std::atan2(a.im, a.re); }                      /* :89-92 */
inline Cx cexp(Cx a) { return Cx{std::exp(a.re) * std::cos(a.im), std::exp(a.re) * std::sin(a.im)}; } /* :97-100 */
inline Cx clog(Cx a) { return Cx{std::log(cabs(a)), carg(a)}; }                  /* :105-111 */
inline Cx neg(Cx a) { return Cx{-a.re, -a.im}; }
inline Cx add(Cx a, Cx b) { return Cx{a.re + b.re, a.im + b.im}; }               /* :139-142 */
inline Cx addr(Cx a, double x) { return Cx{a.re + x, a.im}; }                    /* :143-146 */
inline Cx sub(Cx a, Cx b) { return Cx{a.re - b.re, a.im - b.im}; }               /* :166-169 */
inline Cx subr(Cx a, double x) { return Cx{a.re - x, a.im}; }                    /* :170-173 */
inline Cx rsub(double x, Cx a) { return Cx{x - a.re, -a.im}; }                   /* :174-177 */
inline Cx mul(Cx a, Cx b) { return Cx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; } /* :198-201 */
inline Cx mulr(Cx a, double x) { return Cx{a.re * x, a.im * x}; }                /* :202-205 */
inline Cx rmul(double x, Cx a) { return Cx{x * a.re, x * a.im}; }                /* :206-209 */
inline Cx divr(Cx a, double x) { return Cx{a.re / x, a.im / x}; }                /* :263-266 */
inline Cx div(Cx a, Cx b)                                                         /* :247-262 Smith */
{
	if (std::abs(b.im) < std::abs(b.re))
	{
		double f = b.im / b.re;
		return Cx{(a.re + a.im * f) / (b.re + b.im * f), (a.im - a.re * f) / (b.re + b.im * f)};
	}
	double f = b.re / b.im;
	return Cx{(a.re * f + a.im) / (b.re * f + b.im), (a.im * f - a.re) / (b.re * f + b.im)};
}
inline Cx rdiv(double num, Cx b)                                                  /* :267-280 */
{
	if (std::abs(b.im) < std::abs(b.re))
	{
		double f = b.im / b.re;
		return Cx{num / (b.re + b.im * f), (-num * f) / (b.re + b.im * f)};
	}
	double f = b.re / b.im;
	return Cx{(num * f) / (b.re * f + b.im), -num / (b.re * f + b.im)};
}
inline Cx cpowi(Cx a, int n)                                                      /* :285-306 */
{
	Cx res = cx(1, 0);
	if (n > 0)
	{
		for (int i = 0; i < n; i++) res = mul(res, a);
	}
	else if (n < 0)
	{
		for (int i = 0; i > n; i--) res = mul(res, a);
		res = rdiv(1, res);
	}
	return res;
}

/******************************************************************************
mass functions: include/mass_functions/*.cuh
******************************************************************************/
/* include/mass_functions/power_law.cuh:30-44 */
double power_integral(double x1, double x2, double a, double b = 1)
{
	if (a != -1) return b * (std::pow(x2, a + 1) - std::pow(x1, a + 1)) / (a + 1);
	return b * (std::log(x2) - std::log(x1));
}
/* include/mass_functions/power_law.cuh:59-73 */
double power_log_integral(double x1, double x2, double a, double b = 1)
{
	if (a != -1)
	{
		return b * (std::pow(x2, a + 1) * ((a + 1) * std::log(x2) - 1) - std::pow(x1, a + 1) * ((a + 1) * std::log(x1) - 1)) / ((a + 1) * (a + 1));
	}
	return b * (std::log(x2) * std::log(x2) - std::log(x1) * std::log(x1)) / 2;
}
/* include/mass_functions/power_law.cuh:87-101 */
double invert_power_integral(double p, double x1, double a, double b)
{
	if (a != -1) return std::pow(p * (a + 1) / b + std::pow(x1, a + 1), 1 / (a + 1));
	return x1 * std::exp(p / b);
}

double slope_of(int mf)
{
	if (mf == ORACLE_MF_SALPETER) return -2.35;   /* include/mass_functions/salpeter.cuh:22 */
	return 0;                                     /* include/mass_functions/uniform.cuh:22 */
}

/* Kroupa segment probabilities and normalisations,
   include/mass_functions/kroupa.cuh:53-123 (the same case analysis is repeated
   in each of its four methods) */
struct KroupaSetup
{
	double probs[3] = {0, 0, 0};
	double b[3] = {0, 0, 0};
	double m0, m1;
};
const double KROUPA_SLOPES[3] = {-0.3, -1.3, -2.3};  /* kroupa.cuh:27-29 */
const double KROUPA_BREAKS[2] = {0.08, 0.5};          /* kroupa.cuh:31-32 */

KroupaSetup kroupa_setup(double ml, double mu, double ms)
{
	KroupaSetup k;
	const double* s = KROUPA_SLOPES;
	k.m0 = KROUPA_BREAKS[0] * ms;
	k.m1 = KROUPA_BREAKS[1] * ms;
	double m0 = k.m0, m1 = k.m1;
	if (mu < m0)
	{
		k.probs[0] = power_integral(ml, mu, s[0]);
		k.b[0] = 1 / k.probs[0];
		k.probs[0] *= k.b[0];
	}
	else if (mu < m1)
	{
		if (ml < m0)
		{
			k.probs[0] = power_integral(ml, m0, s[0]);
			k.probs[1] = power_integral(m0, mu, s[1]) * std::pow(m0, s[0] - s[1]);
			k.b[0] = 1 / (k.probs[0] + k.probs[1]);
			k.probs[0] *= k.b[0];
			k.probs[1] *= k.b[0];
			k.b[1] = k.b[0] * std::pow(m0, s[0] - s[1]);
		}
		else
		{
			k.probs[1] = power_integral(ml, mu, s[1]);
			k.b[1] = 1 / k.probs[1];
			k.probs[1] *= k.b[1];
		}
	}
	else
	{
		if (ml < m0)
		{
			k.probs[0] = power_integral(ml, m0, s[0]);
			k.probs[1] = power_integral(m0, m1, s[1]) * std::pow(m0, s[0] - s[1]);
			k.probs[2] = power_integral(m1, mu, s[2]) * std::pow(m0, s[0] - s[1]) * std::pow(m1, s[1] - s[2]);
			k.b[0] = 1 / (k.probs[0] + k.probs[1] + k.probs[2]);
			k.probs[0] *= k.b[0];
			k.probs[1] *= k.b[0];
			k.probs[2] *= k.b[0];
			k.b[1] = k.b[0] * std::pow(m0, s[0] - s[1]);
			k.b[2] = k.b[1] * std::pow(m1, s[1] - s[2]);
		}
		else if (ml < m1)
		{
			k.probs[1] = power_integral(ml, m1, s[1]);
			k.probs[2] = power_integral(m1, mu, s[2]) * std::pow(m1, s[1] - s[2]);
			k.b[1] = 1 / (k.probs[1] + k.probs[2]);
			k.probs[1] *= k.b[1];
			k.probs[2] *= k.b[1];
			k.b[2] = k.b[1] * std::pow(m1, s[1] - s[2]);
		}
		else
		{
			k.probs[2] = power_integral(ml, mu, s[2]);
			k.b[2] = 1 / k.probs[2];
			k.probs[2] *= k.b[2];
		}
	}
	return k;
}

/* moment of order q (q = 1: <m>, 2: <m^2>; log = <m^2 ln m>) of the Kroupa law,
   include/mass_functions/kroupa.cuh:171-502 */
double kroupa_moment(double ml, double mu, double ms, int q, bool log_moment)
{
	KroupaSetup k = kroupa_setup(ml, mu, ms);
	const double* s = KROUPA_SLOPES;
	auto I = [&](double x1, double x2, double a, double b) {
		return log_moment ? power_log_integral(x1, x2, a + q, b) : power_integral(x1, x2, a + q, b);
	};
	double m0 = k.m0, m1 = k.m1;
	if (mu < m0) return I(ml, mu, s[0], k.b[0]);
	if (mu < m1)
	{
		if (ml < m0) return I(ml, m0, s[0], k.b[0]) + I(m0, mu, s[1], k.b[1]);
		return I(ml, mu, s[1], k.b[1]);
	}
	if (ml < m0) return I(ml, m0, s[0], k.b[0]) + I(m0, m1, s[1], k.b[1]) + I(m1, mu, s[2], k.b[2]);
	if (ml < m1) return I(ml, m1, s[1], k.b[1]) + I(m1, mu, s[2], k.b[2]);
	return I(ml, mu, s[2], k.b[2]);
}

/* include/mass_functions/kroupa.cuh:43-162 */
double kroupa_mass(double p, double ml, double mu, double ms)
{
	if (ml == mu) return ml;
	KroupaSetup k = kroupa_setup(ml, mu, ms);
	const double* s = KROUPA_SLOPES;
	double m0 = k.m0, m1 = k.m1;
	if (p < k.probs[0]) return invert_power_integral(p, ml, s[0], k.b[0]);
	if (p < (k.probs[0] + k.probs[1]))
	{
		if (ml < m0) return invert_power_integral(p - k.probs[0], m0, s[1], k.b[1]);
		return invert_power_integral(p, ml, s[1], k.b[1]);
	}
	if (ml < m0) return invert_power_integral(p - k.probs[0] - k.probs[1], m1, s[2], k.b[2]);
	if (ml < m1) return invert_power_integral(p - k.probs[1], m1, s[2], k.b[2]);
	return invert_power_integral(p, ml, s[2], k.b[2]);
}

double mf_mass(int mf, double p, double ml, double mu, double ms)
{
	switch (mf)
	{
	case ORACLE_MF_EQUAL: return 1;                                  /* equal.cuh:41-44 */
	case ORACLE_MF_KROUPA: return kroupa_mass(p, ml, mu, ms);
	case ORACLE_MF_OPTICAL_DEPTH:                                   /* optical_depth.cuh:27-39 */
		if (ml == mu) return ml;
		if (p <= mu / (ml + mu)) return ml;
		return mu;
	default:                                                        /* power_law.cuh:126-144 */
	{
		if (ml == mu) return ml;
		double a = slope_of(mf);
		double b = 1 / power_integral(ml, mu, a);
		return invert_power_integral(p, ml, a, b);
	}
	}
}

void mf_moments(int mf, double ml, double mu, double ms, double& m1, double& m2, double& m2ln)
{
	switch (mf)
	{
	case ORACLE_MF_EQUAL:                                             /* equal.cuh:55-74 */
		m1 = 1; m2 = 1; m2ln = 0;
		return;
	case ORACLE_MF_KROUPA:
		if (ml == mu) { m1 = ml; m2 = ml * ml; m2ln = ml * ml * std::log(ml); return; }
		m1 = kroupa_moment(ml, mu, ms, 1, false);
		m2 = kroupa_moment(ml, mu, ms, 2, false);
		m2ln = kroupa_moment(ml, mu, ms, 2, true);
		return;
	case ORACLE_MF_OPTICAL_DEPTH:                                    /* optical_depth.cuh:48-93 */
		if (ml == mu) { m1 = ml; m2 = ml * ml; m2ln = ml * ml * std::log(ml); return; }
		m1 = 2 * ml * mu / (ml + mu);
		m2 = ml * mu;
		m2ln = ml * mu * (ml * std::log(ml) + mu * std::log(mu)) / (ml + mu);
		return;
	default:                                                        /* power_law.cuh:153-226 */
	{
		if (ml == mu) { m1 = ml; m2 = ml * ml; m2ln = ml * ml * std::log(ml); return; }
		double a = slope_of(mf);
		double b = 1 / power_integral(ml, mu, a);
		m1 = power_integral(ml, mu, a + 1, b);
		m2 = power_integral(ml, mu, a + 2, b);
		m2ln = power_log_integral(ml, mu, a + 2, b);
	}
	}
}

/******************************************************************************
quadtree: include/tree_node.cuh
******************************************************************************/
constexpr int MAX_DIRECT = 32;      /* tree_node.cuh:14 */
constexpr int MAX_ORDER = 31;       /* tree_node.cuh:20 */

struct Star
{
	Cx pos;
	double mass;
};

struct Node
{
	Cx center;
	double half_length = 0;
	int level = 0;
	int parent = -1;
	int children[4] = {-1, -1, -1, -1};
	int num_children = 0;
	int neighbors[8];
	int num_neighbors = 0;
	int m2l[27];
	int num_m2l = 0;
	int p2l[5];
	int num_p2l = 0;
	int stars = 0;
	int numstars = 0;
	int expansion_order = 0;
	Cx multipole[MAX_ORDER + 1];
	Cx local[MAX_ORDER + 1];
};

struct Field
{
	/* configuration */
	double kappa_tot, shear, kappa_star, theta;
	int rectangular, approx, taylor_smooth;
	Cx corner;
	/* stars in tree order, tree nodes level by level */
	std::vector<Star> stars;
	std::vector<Node> nodes;
	std::vector<int> level_start, level_count;
	int tree_levels = 0;
	int expansion_order = 0;
	double root_half_length = 0;
	std::vector<int> binom;
};

int nstars_with_neighbors(const Field& F, const Node& n)
{
	int s = n.numstars;
	for (int j = 0; j < n.num_neighbors; j++) s += F.nodes[n.neighbors[j]].numstars;
	return s;
}

/* tree_node.cuh:183-267 */
void set_neighbors(Field& F, int idx)
{
	Node& n = F.nodes[idx];
	if (n.level == 0) return;
	const Node& parent = F.nodes[n.parent];
	for (int i = 0; i < parent.num_children; i++)
	{
		int c = parent.children[i];
		if (F.nodes[c].numstars == 0) continue;
		if (c != idx) n.neighbors[n.num_neighbors++] = c;
	}
	for (int i = 0; i < parent.num_neighbors; i++)
	{
		int nb = parent.neighbors[i];
		const Node& neighbor = F.nodes[nb];
		if (neighbor.numstars == 0) continue;
		if (neighbor.num_children == 0)
		{
			if (std::fabs(neighbor.center.re - n.center.re) < 3.5 * n.half_length
				&& std::fabs(neighbor.center.im - n.center.im) < 3.5 * n.half_length)
			{
				n.neighbors[n.num_neighbors++] = nb;
			}
			else
			{
				n.p2l[n.num_p2l++] = nb;
			}
		}
		else
		{
			for (int j = 0; j < neighbor.num_children; j++)
			{
				int c = neighbor.children[j];
				const Node& node = F.nodes[c];
				if (node.numstars == 0) continue;
				if (std::fabs(node.center.re - n.center.re) < 3 * n.half_length
					&& std::fabs(node.center.im - n.center.im) < 3 * n.half_length)
				{
					n.neighbors[n.num_neighbors++] = c;
				}
				else
				{
					n.m2l[n.num_m2l++] = c;
				}
			}
		}
	}
}

/* level loop of include/ccf.cuh:781-829 with the serial execution order of
   the kernels in include/tree_node.cuh:321-519 */
void build_tree(Field& F, std::vector<Star>& stars)
{
	F.nodes.clear();
	F.level_start.clear();
	F.level_count.clear();
	Node root;
	root.center = cx(0, 0);
	root.half_length = F.root_half_length;
	root.level = 0;
	root.numstars = (int)stars.size();
	F.nodes.push_back(root);
	F.level_start.push_back(0);
	F.level_count.push_back(1);
	F.tree_levels = 0;
	std::vector<Star> temp(stars.size());
	int maxn;
	do
	{
		int L = F.tree_levels;
		int start = F.level_start[L], count = F.level_count[L];
		maxn = 0;
		int nonempty = 0;
		std::vector<char> flag(count, 0);
		for (int i = 0; i < count; i++)                      /* tree_node.cuh:321-345 */
		{
			int ns = nstars_with_neighbors(F, F.nodes[start + i]);
			if (ns > MAX_DIRECT) { nonempty++; flag[i] = 1; }
			maxn = std::max(maxn, ns);
		}
		if (maxn <= MAX_DIRECT) break;
		int child_start = (int)F.nodes.size();
		F.nodes.resize(child_start + 4 * nonempty);
		int slot = nonempty - 1;                             /* ccf.cuh:809 */
		for (int i = 0; i < count; i++)                      /* tree_node.cuh:355-381 */
		{
			if (!flag[i]) continue;
			int base = child_start + 4 * slot;
			slot--;
			Node& n = F.nodes[start + i];
			static const double off[4][2] = {{1, 1}, {-1, 1}, {-1, -1}, {1, -1}};  /* tree_node.cuh:155-161 */
			double hl = n.half_length / 2;
			for (int c = 0; c < 4; c++)
			{
				Node ch;
				ch.center = add(n.center, rmul(hl, cx(off[c][0], off[c][1])));
				ch.half_length = hl;
				ch.level = n.level + 1;
				ch.parent = start + i;
				F.nodes[base + c] = ch;
				n.children[c] = base + c;
			}
			n.num_children = 4;
		}
		for (int i = 0; i < count; i++)                      /* tree_node.cuh:392-501 */
		{
			Node& n = F.nodes[start + i];
			if (n.numstars == 0 || n.num_children == 0) continue;
			int s = n.stars, ns = n.numstars;
			int top = 0, bottom = 0, ch[4] = {0, 0, 0, 0};
			for (int k = 0; k < ns; k++)
			{
				if (stars[s + k].pos.im >= n.center.im) temp[s + top++] = stars[s + k];
				else temp[s + ns - 1 - bottom++] = stars[s + k];
			}
			for (int k = 0; k < ns; k++)
			{
				if (k < top)
				{
					if (temp[s + k].pos.re >= n.center.re) stars[s + ch[0]++] = temp[s + k];
					else stars[s + top - 1 - ch[1]++] = temp[s + k];
				}
				else
				{
					if (temp[s + k].pos.re < n.center.re) stars[s + top + ch[2]++] = temp[s + k];
					else stars[s + ns - 1 - ch[3]++] = temp[s + k];
				}
			}
			F.nodes[n.children[0]].stars = s;
			F.nodes[n.children[0]].numstars = ch[0];
			for (int c = 1; c < 4; c++)
			{
				Node& prev = F.nodes[n.children[c - 1]];
				F.nodes[n.children[c]].stars = prev.stars + prev.numstars;
				F.nodes[n.children[c]].numstars = ch[c];
			}
		}
		F.tree_levels++;
		F.level_start.push_back(child_start);
		F.level_count.push_back(4 * nonempty);
		for (int i = 0; i < 4 * nonempty; i++) set_neighbors(F, child_start + i);   /* tree_node.cuh:509-519 */
	} while (true);
}

/* include/binomial_coefficients.cuh:11-44: the reference's Pascal triangle is
   held in int32, whose additions wrap for n > 33; that wrapped table is what
   the reference's FMM translations use */
void binomials(std::vector<int>& b, int n)
{
	b.assign((n + 1) * (n + 2) / 2 + 1, 0);
	for (int r = 0; r <= n; r++)
	{
		int rs = r * (r + 1) / 2, ps = (r - 1) * r / 2;
		for (int i = 0; i <= r; i++)
		{
			if (i == 0 || i == r) b[rs + i] = 1;
			else b[rs + i] = (int)((uint32_t)b[ps + i - 1] + (uint32_t)b[ps + i]);
		}
	}
}
inline double binom(const Field& F, int n, int k)  /* binomial_coefficients.cuh:53-64 */
{
	if (n < k) return 0;
	return F.binom[n * (n + 1) / 2 + k];
}

/* exact binomial as a double, for the exact_binomials option */
std::vector<double> g_exact_binom;
bool g_use_exact = false;

inline double binom_any(const Field& F, int n, int k)
{
	if (n < k) return 0;
	if (g_use_exact) return g_exact_binom[n * (n + 1) / 2 + k];
	return (double)F.binom[n * (n + 1) / 2 + k];
}

/* FMM passes: include/fmm.cuh */
void fmm_build(Field& F)
{
	const int P = F.expansion_order;
	std::vector<Cx> buf(27 * (MAX_ORDER + 1));
	for (int L = F.tree_levels; L >= 0; L--)                    /* ccf.cuh:866-875 */
	{
		int s = F.level_start[L], c = F.level_count[L];
		for (int i = 0; i < c; i++)                                /* fmm.cuh:59-98 (P2M) */
		{
			Node& n = F.nodes[s + i];
			if (n.num_children != 0 || n.numstars == 0) continue;
			for (int p = 0; p <= P; p++)
			{
				Cx r;
				if (p == 0)                                          /* fmm.cuh:26-35 */
				{
					for (int k = 0; k < n.numstars; k++) r = addr(r, F.stars[n.stars + k].mass);
				}
				else                                                 /* fmm.cuh:36-46 */
				{
					for (int k = 0; k < n.numstars; k++)
					{
						const Star& st = F.stars[n.stars + k];
						r = sub(r, mulr(cpowi(divr(sub(st.pos, n.center), n.half_length), p), st.mass));
					}
					r = divr(r, p);
				}
				n.multipole[p] = r;
			}
			n.expansion_order = std::max(n.expansion_order, P);
		}
		for (int i = 0; i < c; i++)                                /* fmm.cuh:150-192 (M2M) */
		{
			Node& n = F.nodes[s + i];
			for (int j = 0; j < n.num_children; j++)
			{
				const Node& ch = F.nodes[n.children[j]];
				for (int p = 0; p <= P; p++)                       /* fmm.cuh:109-139 */
				{
					Cx r;
					if (p == 0) r = ch.multipole[0];
					else
					{
						Cx dz = divr(sub(ch.center, n.center), ch.half_length);
						for (int k = p; k >= 1; k--)
						{
							r = add(r, mulr(ch.multipole[k], binom_any(F, p - 1, k - 1)));
							r = div(r, dz);
						}
						r = sub(r, divr(ch.multipole[0], p));
						r = mul(r, cpowi(dz, p));
						r = divr(r, (double)(1 << p));
					}
					buf[j * (MAX_ORDER + 1) + p] = r;
				}
			}
			for (int j = 0; j < n.num_children; j++)
			{
				for (int p = 0; p <= P; p++) n.multipole[p] = add(n.multipole[p], buf[j * (MAX_ORDER + 1) + p]);
				n.expansion_order = std::max(n.expansion_order, P);
			}
		}
	}
	for (int L = 2; L <= F.tree_levels; L++)                      /* ccf.cuh:880-893 */
	{
		int s = F.level_start[L], c = F.level_count[L];
		for (int i = 0; i < c; i++)                                /* fmm.cuh:235-268 (L2L) */
		{
			Node& n = F.nodes[s + i];
			const Node& par = F.nodes[n.parent];
			for (int p = 0; p <= P; p++)                           /* fmm.cuh:204-223 */
			{
				Cx r;
				Cx dz = divr(sub(n.center, par.center), par.half_length);
				for (int k = P; k >= 1; k--)
				{
					r = add(r, mulr(par.local[k], binom_any(F, k, p)));
					r = mul(r, dz);
				}
				r = div(r, cpowi(dz, p));
				r = divr(r, (double)(1 << p));
				buf[p] = r;
			}
			for (int p = 0; p <= P; p++) n.local[p] = buf[p];
			n.expansion_order = std::max(n.expansion_order, P);
		}
		for (int i = 0; i < c; i++)                                /* fmm.cuh:333-374 (M2L) */
		{
			Node& n = F.nodes[s + i];
			for (int j = 0; j < n.num_m2l; j++)
			{
				const Node& from = F.nodes[n.m2l[j]];
				Cx dz = divr(sub(from.center, n.center), from.half_length);
				for (int p = 0; p <= P; p++)                       /* fmm.cuh:281-322 */
				{
					Cx r;
					if (p == 0)
					{
						for (int k = P; k >= 1; k--)
						{
							r = add(r, from.multipole[k]);
							r = div(r, neg(dz));
						}
						r = add(r, mul(from.multipole[0], clog(neg(dz))));
						r = add(r, mulr(from.multipole[0], std::log(from.half_length)));
					}
					else
					{
						for (int k = P; k >= 1; k--)
						{
							r = add(r, mulr(from.multipole[k], binom_any(F, p + k - 1, k - 1)));
							r = div(r, neg(dz));
						}
						r = sub(r, divr(from.multipole[0], p));
						r = div(r, cpowi(dz, p));
					}
					buf[j * (MAX_ORDER + 1) + p] = r;
				}
			}
			for (int j = 0; j < n.num_m2l; j++)
			{
				for (int p = 0; p <= P; p++) n.local[p] = add(n.local[p], buf[j * (MAX_ORDER + 1) + p]);
				n.expansion_order = std::max(n.expansion_order, P);
			}
		}
		for (int i = 0; i < c; i++)                                /* fmm.cuh:423-464 (P2L) */
		{
			Node& n = F.nodes[s + i];
			for (int j = 0; j < n.num_p2l; j++)
			{
				const Node& from = F.nodes[n.p2l[j]];
				for (int p = 0; p <= P; p++)                       /* fmm.cuh:387-413 */
				{
					Cx r;
					for (int k = 0; k < from.numstars; k++)
					{
						const Star& st = F.stars[from.stars + k];
						Cx dz = divr(sub(st.pos, n.center), n.half_length);
						if (p == 0)
						{
							r = add(r, rmul(st.mass, clog(neg(dz))));
							r = addr(r, st.mass * std::log(n.half_length));
						}
						else
						{
							r = sub(r, rdiv(st.mass, rmul((double)p, cpowi(dz, p))));
						}
					}
					buf[j * (MAX_ORDER + 1) + p] = r;
				}
			}
			for (int j = 0; j < n.num_p2l; j++)
			{
				for (int p = 0; p <= P; p++) n.local[p] = add(n.local[p], buf[j * (MAX_ORDER + 1) + p]);
				n.expansion_order = std::max(n.expansion_order, P);
			}
		}
	}
}

/* include/tree_node.cuh:529-561 */
const Node& nearest_node(const Field& F, Cx z)
{
	const Node* n = &F.nodes[0];
	while (n->num_children > 0)
	{
		if (std::fabs(z.re - n->center.re) > n->half_length || std::fabs(z.im - n->center.im) > n->half_length) return *n;
		if (z.re >= n->center.re && z.im >= n->center.im) n = &F.nodes[n->children[0]];
		else if (z.re < n->center.re && z.im >= n->center.im) n = &F.nodes[n->children[1]];
		else if (z.re < n->center.re && z.im < n->center.im) n = &F.nodes[n->children[2]];
		else n = &F.nodes[n->children[3]];
	}
	return *n;
}

/******************************************************************************
deflection field: include/alpha_star.cuh, alpha_local.cuh, alpha_smooth.cuh
******************************************************************************/
template <class Fn>
inline void for_near_stars(const Field& F, const Node& n, Fn fn)
{
	for (int j = 0; j < n.num_neighbors; j++)
	{
		const Node& nb = F.nodes[n.neighbors[j]];
		for (int i = 0; i < nb.numstars; i++) fn(F.stars[nb.stars + i]);
	}
	for (int i = 0; i < n.numstars; i++) fn(F.stars[n.stars + i]);
}

Cx alpha_star(const Field& F, Cx z, const Node& n)                 /* alpha_star.cuh:18-41 */
{
	Cx a;
	for_near_stars(F, n, [&](const Star& s) { a = add(a, rdiv(s.mass, sub(z, s.pos))); });
	a = mulr(a, F.theta * F.theta);
	return conj(a);
}
Cx d_alpha_star_d_zbar(const Field& F, Cx z, const Node& n)        /* alpha_star.cuh:54-77 */
{
	Cx a;
	for_near_stars(F, n, [&](const Star& s) { Cx d = sub(z, s.pos); a = add(a, rdiv(s.mass, mul(d, d))); });
	a = mulr(a, -F.theta * F.theta);
	return conj(a);
}
Cx d2_alpha_star_d_zbar2(const Field& F, Cx z, const Node& n)      /* alpha_star.cuh:90-115 */
{
	Cx a;
	for_near_stars(F, n, [&](const Star& s) { Cx d = sub(z, s.pos); a = add(a, rdiv(s.mass, mul(mul(d, d), d))); });
	a = mulr(a, 2 * F.theta * F.theta);
	return conj(a);
}
Cx alpha_local(const Field& F, Cx z, const Node& n)                /* alpha_local.cuh:19-36 */
{
	Cx a;
	Cx dz = divr(sub(z, n.center), n.half_length);
	for (int i = n.expansion_order; i >= 1; i--)
	{
		a = mul(a, dz);
		a = add(a, mulr(n.local[i], i));
	}
	a = mulr(a, F.theta * F.theta);
	a = divr(a, n.half_length);
	return conj(a);
}
Cx d_alpha_local_d_zbar(const Field& F, Cx z, const Node& n)       /* alpha_local.cuh:52-69 */
{
	Cx a;
	Cx dz = divr(sub(z, n.center), n.half_length);
	for (int i = n.expansion_order; i >= 2; i--)
	{
		a = mul(a, dz);
		a = add(a, mulr(mulr(n.local[i], i), i - 1));
	}
	a = mulr(a, F.theta * F.theta);
	a = divr(a, n.half_length * n.half_length);
	return conj(a);
}
Cx d2_alpha_local_d_zbar2(const Field& F, Cx z, const Node& n)     /* alpha_local.cuh:85-102 */
{
	Cx a;
	Cx dz = divr(sub(z, n.center), n.half_length);
	for (int i = n.expansion_order; i >= 3; i--)
	{
		a = mul(a, dz);
		a = add(a, mulr(mulr(mulr(n.local[i], i), i - 1), i - 2));
	}
	a = mulr(a, F.theta * F.theta);
	a = divr(a, n.half_length * n.half_length * n.half_length);
	return conj(a);
}

inline double heaviside(double x) { return x >= 0 ? 1 : 0; }        /* alpha_smooth.cuh:16-26 */
inline double boxcar(Cx z, Cx c)                                      /* alpha_smooth.cuh:38-48 */
{
	return (-c.re <= z.re && z.re <= c.re && -c.im <= z.im && z.im <= c.im) ? 1 : 0;
}

Cx alpha_smooth(const Field& F, Cx z)                                /* alpha_smooth.cuh:63-127 */
{
	const double ks = F.kappa_star;
	const Cx c = F.corner;
	Cx a;
	if (F.rectangular)
	{
		if (F.approx)
		{
			Cx s1, s2, s3, s4;
			for (int i = F.taylor_smooth; i >= 1; i--)
			{
				Cx t = divr(cx(1, 0), i);
				s1 = add(s1, t);
				s2 = add(s2, t);
				s3 = add(s3, t);
				s4 = add(s4, t);
				s1 = mul(s1, div(conj(z), c));
				s2 = mul(s2, div(conj(z), conj(c)));
				s3 = mul(s3, div(conj(z), neg(c)));
				s4 = mul(s4, div(conj(z), neg(conj(c))));
			}
			a = add(sub(mul(sub(c, conj(z)), sub(clog(c), s1)), mul(sub(conj(c), conj(z)), sub(clog(conj(c)), s2))),
				mul(sub(neg(c), conj(z)), sub(clog(neg(c)), s3)));
			a = sub(a, mul(sub(neg(conj(c)), conj(z)), sub(clog(conj(neg(c))), s4)));
			a = mul(a, cx(0, -ks * INV_PI));
			a = subr(a, ks * 2 * (c.re + z.re));
		}
		else
		{
			Cx c1 = sub(c, conj(z));
			Cx c2 = sub(conj(c), conj(z));
			Cx c3 = sub(neg(c), conj(z));
			Cx c4 = sub(neg(conj(c)), conj(z));
			a = sub(add(sub(mul(c1, clog(c1)), mul(c2, clog(c2))), mul(c3, clog(c3))), mul(c4, clog(c4)));
			a = mul(a, cx(0, -ks * INV_PI));
			a = subr(a, ks * 2 * (c.re + z.re) * boxcar(z, c));
			a = subr(a, ks * 4 * c.re * heaviside(c.im + z.im) * heaviside(c.im - z.im) * heaviside(z.re - c.re));
		}
	}
	else
	{
		if (F.approx) a = rmul(-ks, z);
		else
		{
			if (cabs(z) <= cabs(c)) a = rmul(-ks, z);
			else a = rdiv(-ks * cabs(c) * cabs(c), conj(z));
		}
	}
	return a;
}

double d_alpha_smooth_d_z(const Field& F, Cx z)                      /* alpha_smooth.cuh:142-170 */
{
	const double ks = F.kappa_star;
	if (F.rectangular) return F.approx ? -ks : -ks * boxcar(z, F.corner);
	return F.approx ? -ks : -ks * heaviside(cabs(F.corner) - cabs(z));
}

Cx d_alpha_smooth_d_zbar(const Field& F, Cx z)                       /* alpha_smooth.cuh:186-236 */
{
	const double ks = F.kappa_star;
	const Cx c = F.corner;
	Cx d;
	if (F.rectangular)
	{
		if (F.approx)
		{
			Cx r = div(conj(z), c);
			Cx phase = cx(0, carg(c));
			for (int i = F.taylor_smooth - 1; i >= 2; i -= 2)
			{
				d = add(d, divr(rsub(1, cexp(mulr(rmul(2, phase), i))), i));
				d = mul(d, mul(r, r));
			}
			d = mulr(d, 2);
			d = mul(d, cx(0, -ks * INV_PI));
			d = addr(d, ks - 4 * ks * carg(c) * INV_PI);
		}
		else
		{
			Cx c1 = sub(conj(c), conj(z));
			Cx c2 = sub(c, conj(z));
			Cx c3 = sub(neg(c), conj(z));
			Cx c4 = sub(neg(conj(c)), conj(z));
			d = add(sub(sub(clog(c1), clog(c2)), clog(c3)), clog(c4));
			d = mul(d, cx(0, -ks * INV_PI));
			d = subr(d, ks * boxcar(z, c));
		}
	}
	else
	{
		if (F.approx) d = cx(0, 0);
		else d = rdiv(ks * cabs(c) * cabs(c), cpowi(conj(z), 2));
	}
	return d;
}

Cx d2_alpha_smooth_d_zbar2(const Field& F, Cx z)                     /* alpha_smooth.cuh:252-301 */
{
	const double ks = F.kappa_star;
	const Cx c = F.corner;
	Cx d;
	if (F.rectangular)
	{
		if (F.approx)
		{
			Cx r = div(conj(z), c);
			Cx phase = cx(0, carg(c));
			for (int i = F.taylor_smooth - 1; i >= 2; i -= 2)
			{
				d = add(d, rsub(1, cexp(mulr(rmul(2, phase), i))));
				d = mul(d, mul(r, r));
			}
			d = div(d, conj(z));
			d = mulr(d, 2);
			d = mul(d, cx(0, -ks * INV_PI));
		}
		else
		{
			Cx c1 = sub(conj(c), conj(z));
			Cx c2 = sub(c, conj(z));
			Cx c3 = sub(neg(c), conj(z));
			Cx c4 = sub(neg(conj(c)), conj(z));
			d = sub(add(add(rdiv(-1, c1), rdiv(1, c2)), rdiv(1, c3)), rdiv(1, c4));
			d = mul(d, cx(0, -ks * INV_PI));
		}
	}
	else
	{
		if (F.approx) d = cx(0, 0);
		else d = rdiv(-2 * ks * cabs(c) * cabs(c), cpowi(conj(z), 3));
	}
	return d;
}

/* include/ccf_functions.cuh:33-45 */
Cx image_to_source(const Field& F, Cx z, const Node& n)
{
	Cx as = alpha_star(F, z, n), al = alpha_local(F, z, n), sm = alpha_smooth(F, z);
	return sub(sub(sub(add(rmul(1 - F.kappa_tot, z), rmul(F.shear, conj(z))), as), al), sm);
}
/* include/ccf_functions.cuh:69-86 */
Cx parametric_cc(const Field& F, Cx z, const Node& n, double phi)
{
	Cx a = d_alpha_star_d_zbar(F, z, n);
	Cx b = d_alpha_local_d_zbar(F, z, n);
	double sz = d_alpha_smooth_d_z(F, z);
	Cx c = d_alpha_smooth_d_zbar(F, z);
	Cx r = rsub(F.shear, conj(a));
	r = sub(r, conj(b));
	r = sub(r, conj(c));
	r = sub(r, rmul(1 - F.kappa_tot - sz, cx(std::cos(phi), -std::sin(phi))));
	return r;
}
/* include/ccf_functions.cuh:108-121 */
Cx d_parametric_cc_dz(const Field& F, Cx z, const Node& n)
{
	Cx a = d2_alpha_star_d_zbar2(F, z, n);
	Cx b = d2_alpha_local_d_zbar2(F, z, n);
	Cx c = d2_alpha_smooth_d_zbar2(F, z);
	return sub(sub(neg(conj(a)), conj(b)), conj(c));
}
/* include/ccf_functions.cuh:144-166 */
double mu_length_scale(const Field& F, Cx z, const Node& n)
{
	Cx a = d_alpha_star_d_zbar(F, z, n);
	Cx b = d_alpha_local_d_zbar(F, z, n);
	double sz = d_alpha_smooth_d_z(F, z);
	Cx c = d_alpha_smooth_d_zbar(F, z);
	double dwdz = 1 - F.kappa_tot - sz;
	Cx dwdzb = sub(sub(rsub(F.shear, a), b), c);
	Cx a2 = d2_alpha_star_d_zbar2(F, z, n);
	Cx b2 = d2_alpha_local_d_zbar2(F, z, n);
	Cx c2 = d2_alpha_smooth_d_zbar2(F, z);
	Cx d2w = sub(sub(neg(a2), b2), c2);
	Cx cct = mul(mul(cx(0, -2), conj(dwdzb)), d2w);
	Cx ct = add(rmul(dwdz, cct), mul(dwdzb, conj(cct)));
	return 1 / (2 * cabs(ct));
}

/* include/ccf_functions.cuh:193-243.  Returns the updated root; counts the
   reciprocal-sum terms it executed. */
Cx aberth_update(const Field& F, int k, Cx z, double phi, const Cx* roots, int nroots, bool early_out, long long& terms)
{
	const Node& node = nearest_node(F, z);
	Cx f0 = parametric_cc(F, z, node, phi);
	double sz = d_alpha_smooth_d_z(F, z);
	if (early_out)
	{
		if (std::fabs(cabs(f0) * (cabs(f0) + 2 * (1 - F.kappa_tot - sz))) < 0.000000001 &&
			std::fabs(cabs(f0) * (cabs(f0) - 2 * (1 - F.kappa_tot - sz))) < 0.000000001)
		{
			return z;
		}
	}
	Cx f1 = d_parametric_cc_dz(F, z, node);
	Cx p_sum;
	const int nstars = (int)F.stars.size();
	for (int i = 0; i < nstars; i++) p_sum = add(p_sum, rdiv(1, sub(z, F.stars[i].pos)));
	if (!F.rectangular && !F.approx) p_sum = add(p_sum, rdiv(1, z));
	p_sum = mulr(p_sum, 2);
	Cx root_sum;
	for (int i = 0; i < nroots; i++)
	{
		if (i != k) root_sum = add(root_sum, rdiv(1, sub(z, roots[i])));
	}
	terms += nstars + nroots - 1;
	Cx result = add(f1, mul(f0, sub(p_sum, root_sum)));
	return sub(z, div(f0, result));
}

/* one in-place sweep over a row (include/ccf_functions.cuh:346-390) */
int sweep_row(const Field& F, Cx* row, int nroots, char* fin, double phi, bool early_out, double tol,
	long long& updates, long long& terms)
{
	int active = 0;
	for (int a = 0; a < nroots; a++)
	{
		if (fin[a]) continue;
		Cx res = aberth_update(F, a, row[a], phi, row, nroots, early_out, terms);
		updates++;
		double norm = cabs(sub(res, row[a])) / F.theta;
		if (norm < tol) fin[a] = 1;
		else active++;
		row[a] = res;
	}
	return active;
}

/* The same Aberth step (include/ccf_functions.cuh:193-243) applied to every
   root of the row from the row as it stood before the sweep, the roots split
   over nt threads (Jacobi order; the reference updates in place while other
   threads read, include/ccf_functions.cuh:374-389). */
int sweep_row_jacobi(const Field& F, Cx* row, int nroots, char* fin, double phi, bool early_out, double tol, int nt,
	long long& updates, long long& terms)
{
	std::vector<Cx> next(row, row + nroots);
	int active = 0;
	long long u = 0, t = 0;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 16) reduction(+ : active, u, t)
	for (int a = 0; a < nroots; a++)
	{
		if (fin[a]) continue;
		long long ta = 0;
		Cx res = aberth_update(F, a, row[a], phi, row, nroots, early_out, ta);
		t += ta;
		u++;
		double norm = cabs(sub(res, row[a])) / F.theta;
		if (norm < tol) fin[a] = 1;
		else active++;
		next[a] = res;
	}
	std::copy(next.begin(), next.end(), row);
	updates += u;
	terms += t;
	return active;
}

inline double center_phi(int c, int nb) { return PI / nb + c * 2 * PI / nb; }   /* ccf_functions.cuh:344 */

struct Run
{
	Field F;
	int num_stars = 0, num_roots = 0;
	int rectangular = 0;
	Cx corner;
	double theta = 1, kappa_star = 0;
	oracle_info info;
	std::vector<Star> stars_gen;  /* generation order */
};

void fail(oracle_info* info, const char* msg)
{
	std::snprintf(info->error, sizeof(info->error), "%s", msg);
}

/* include/ccf.cuh:218-346 (the checks that do not depend on the star file) */
bool check_params(const oracle_params* p, oracle_info* info)
{
	bool sf = p->stars_in != nullptr;
	if (p->kappa_tot < std::numeric_limits<double>::min()) { fail(info, "kappa_tot must be >= min"); return false; }
	if (p->kappa_star < std::numeric_limits<double>::min()) { fail(info, "kappa_star must be >= min"); return false; }
	if (!sf && p->kappa_star > p->kappa_tot) { fail(info, "kappa_star must be <= kappa_tot"); return false; }
	if (!sf && p->theta_star < std::numeric_limits<double>::min()) { fail(info, "theta_star must be >= min"); return false; }
	if (!sf && (p->mass_function < 0 || p->mass_function > 4)) { fail(info, "bad mass function"); return false; }
	if (!sf && p->m_solar < std::numeric_limits<double>::min()) { fail(info, "m_solar must be >= min"); return false; }
	if (!sf && p->m_lower < std::numeric_limits<double>::min()) { fail(info, "m_lower must be >= min"); return false; }
	if (!sf && p->m_upper < p->m_lower) { fail(info, "m_upper must be >= m_lower"); return false; }
	if (!sf && p->rectangular != 0 && p->rectangular != 1) { fail(info, "rectangular must be 0 or 1"); return false; }
	if (p->approx != 0 && p->approx != 1) { fail(info, "approx must be 0 or 1"); return false; }
	if (p->safety_scale < 1.1) { fail(info, "safety_scale must be >= 1.1"); return false; }
	if (p->num_stars < 1) { fail(info, "num_stars must be > 0"); return false; }
	if (p->num_phi < 1 || p->num_phi % 2 != 0) { fail(info, "num_phi must be an even integer > 0"); return false; }
	if (p->num_branches < 1) { fail(info, "num_branches must be > 0"); return false; }
	if (p->num_phi % (2 * p->num_branches) != 0) { fail(info, "num_phi must be a multiple of 2 * num_branches"); return false; }
	return true;
}

/* include/ccf.cuh:348-497, plus the star-field part of :602-730 */
bool derive(const oracle_params* p, Run& R, bool make_stars)
{
	oracle_info& info = R.info;
	if (!check_params(p, &info)) return false;
	Field& F = R.F;
	F.kappa_tot = p->kappa_tot;
	F.shear = p->shear;
	F.approx = p->approx;
	double kappa_star = p->kappa_star, theta = p->theta_star;
	double ml = p->m_lower, mu = p->m_upper;
	int nstars = p->num_stars, rect = p->rectangular;
	Cx corner;
	double mean_mass = 0, mean_mass2 = 0, mean_mass2_ln_mass = 0;
	bool sf = p->stars_in != nullptr;
	if (!sf)
	{
		if (p->mass_function == ORACLE_MF_EQUAL) { ml = 1; mu = 1; }
		else { ml = ml * p->m_solar; mu = mu * p->m_solar; }
		mf_moments(p->mass_function, ml, mu, p->m_solar, mean_mass, mean_mass2, mean_mass2_ln_mass);
	}
	else
	{
		/* star-file branch: include/star.cuh:454-484 + :124-161 */
		rect = p->stars_in_rectangular;
		corner = cx(p->stars_in_corner_re, p->stars_in_corner_im);
		theta = p->stars_in_theta;
		R.stars_gen.resize(nstars);
		for (int i = 0; i < nstars; i++)
		{
			R.stars_gen[i].pos = cx(p->stars_in[3 * i], p->stars_in[3 * i + 1]);
			R.stars_gen[i].mass = p->stars_in[3 * i + 2];
		}
	}
	info.mu_ave = 1 / ((1 - p->kappa_tot) * (1 - p->kappa_tot) - p->shear * p->shear);
	auto star_stats = [&](double& ks, double& mlo, double& mhi, double& m1, double& m2, double& m2l) {
		/* include/star.cuh:124-161 */
		mlo = std::numeric_limits<double>::max();
		mhi = std::numeric_limits<double>::min();
		double mt = 0, m2t = 0, m2lt = 0;
		for (int i = 0; i < nstars; i++)
		{
			double m = R.stars_gen[i].mass;
			mt += m;
			m2t += m * m;
			m2lt += m * m * std::log(m);
			mlo = std::min(mlo, m);
			mhi = std::max(mhi, m);
		}
		m1 = mt / nstars;
		m2 = m2t / nstars;
		m2l = m2lt / nstars;
		if (rect) ks = mt * PI * theta * theta / (4 * corner.re * corner.im);
		else ks = mt * theta * theta / (cabs(corner) * cabs(corner));
	};
	if (sf)
	{
		star_stats(kappa_star, ml, mu, mean_mass, mean_mass2, mean_mass2_ln_mass);
	}
	if (!sf)
	{
		corner = cx(1 / std::abs(1 - p->kappa_tot + p->shear), 1 / std::abs(1 - p->kappa_tot - p->shear));
		if (rect)
		{
			corner = cx(std::sqrt(corner.re / corner.im), std::sqrt(corner.im / corner.re));
			corner = mulr(corner, std::sqrt(PI * theta * theta * nstars * mean_mass / (4 * kappa_star)));
		}
		else
		{
			corner = divr(corner, cabs(corner));
			corner = mulr(corner, std::sqrt(theta * theta * nstars * mean_mass / kappa_star));
		}
	}
	double alpha_error = theta * 0.0000001;
	int ts = 1;
	const int MAX_TS = 101;
	while ((kappa_star * INV_PI * 4 / (ts + 1) * cabs(corner) * (p->safety_scale + 1) / (p->safety_scale - 1)
		* std::pow(1 / p->safety_scale, ts + 1) > alpha_error) && ts <= MAX_TS)
	{
		ts += 2;
	}
	while ((std::fmod(carg(corner) * (ts - 1), PI) < 0.1 * PI || std::fmod(carg(corner) * (ts - 1), PI) > 0.9 * PI) && ts <= MAX_TS)
	{
		ts += 2;
	}
	if (rect && ts > MAX_TS) { fail(&info, "taylor_smooth must be <= 101"); return false; }
	int nroots;
	if (rect) nroots = p->approx ? 2 * nstars + ts - 1 : 2 * nstars;
	else nroots = p->approx ? 2 * nstars : 2 * nstars + 2;

	info.num_stars = nstars;
	info.num_roots = nroots;
	info.taylor_smooth = ts;
	info.rectangular = rect;
	info.alpha_error = alpha_error;
	info.theta_star = theta;
	info.kappa_star = kappa_star;
	info.mean_mass = mean_mass;
	info.mean_mass2 = mean_mass2;
	info.mean_mass2_ln_mass = mean_mass2_ln_mass;
	info.m_lower = ml;
	info.m_upper = mu;
	info.random_seed = sf ? 0 : p->random_seed;
	R.num_stars = nstars;
	R.num_roots = nroots;
	R.rectangular = rect;
	R.theta = theta;
	R.kappa_star = kappa_star;
	F.kappa_star = kappa_star;
	F.theta = theta;
	F.rectangular = rect;
	F.taylor_smooth = ts;

	if (make_stars)
	{
		double t0 = now_s();
		if (!sf)
		{
			/* include/star.cuh:40-107 */
			R.stars_gen.resize(nstars);
			int nt = std::max(1, p->num_threads);
#pragma omp parallel for num_threads(nt) schedule(static)
			for (int i = 0; i < nstars; i++)
			{
				curandState st;
				curand_init(p->random_seed, i, 0, &st);
				double x1, x2;
				if (rect)
				{
					x1 = curand_uniform_double(&st) * 2 * corner.re - corner.re;
					x2 = curand_uniform_double(&st) * 2 * corner.im - corner.im;
				}
				else
				{
					double a = curand_uniform_double(&st) * 2 * PI;
					double r = std::sqrt(curand_uniform_double(&st)) * cabs(corner);
					x1 = r * std::cos(a);
					x2 = r * std::sin(a);
				}
				R.stars_gen[i].pos = cx(x1, x2);
				R.stars_gen[i].mass = mf_mass(p->mass_function, curand_uniform_double(&st), ml, mu, p->m_solar);
			}
		}
		star_stats(info.kappa_star_actual, info.m_lower_actual, info.m_upper_actual,
			info.mean_mass_actual, info.mean_mass2_actual, info.mean_mass2_ln_mass_actual);
		if (!sf)
		{
			/* include/ccf.cuh:686-700 */
			if (rect)
			{
				corner = cx(std::sqrt(corner.re / corner.im), std::sqrt(corner.im / corner.re));
				corner = mulr(corner, std::sqrt(PI * theta * theta * nstars * info.mean_mass_actual / (4 * kappa_star)));
			}
			else
			{
				corner = divr(corner, cabs(corner));
				corner = mulr(corner, std::sqrt(theta * theta * nstars * info.mean_mass_actual / kappa_star));
			}
		}
		info.t_stars = now_s() - t0;
	}
	R.corner = corner;
	F.corner = corner;
	info.corner_re = corner.re;
	info.corner_im = corner.im;
	return true;
}

/* include/ccf.cuh:732-904 */
bool make_tree(const oracle_params* p, Run& R)
{
	Field& F = R.F;
	oracle_info& info = R.info;
	double t0 = now_s();
	double rhl = R.rectangular ? (R.corner.re > R.corner.im ? R.corner.re : R.corner.im) : cabs(R.corner);
	F.root_half_length = rhl * 1.1;
	F.stars = R.stars_gen;
	build_tree(F, F.stars);
	int P = (int)std::ceil(2 * std::log2(R.theta) + F.tree_levels - std::log2(F.root_half_length) - std::log2(info.alpha_error));
	if (P < 3) { fail(&info, "Expansion order needs to be >= 3"); return false; }
	if (P > MAX_ORDER) { fail(&info, "Maximum allowed expansion order is 31"); return false; }
	F.expansion_order = P;
	binomials(F.binom, 2 * P);
	g_use_exact = p->exact_binomials != 0;
	if (g_use_exact)
	{
		int n = 2 * P;
		g_exact_binom.assign((n + 1) * (n + 2) / 2 + 1, 0);
		for (int r = 0; r <= n; r++)
			for (int i = 0; i <= r; i++)
				g_exact_binom[r * (r + 1) / 2 + i] = (i == 0 || i == r) ? 1 :
					g_exact_binom[(r - 1) * r / 2 + i - 1] + g_exact_binom[(r - 1) * r / 2 + i];
	}
	fmm_build(F);
	info.tree_levels = F.tree_levels;
	info.expansion_order = P;
	info.num_nodes = (int)F.nodes.size();
	info.root_half_length = F.root_half_length;
	info.t_tree = now_s() - t0;
	return true;
}

} /* namespace */

extern "C" {

void oracle_default_params(oracle_params* p)
{
	std::memset(p, 0, sizeof(*p));
	p->kappa_tot = 0.3;
	p->shear = 0.3;
	p->kappa_star = 0.27;
	p->theta_star = 1;
	p->m_solar = 1;
	p->m_lower = 0.01;
	p->m_upper = 50;
	p->safety_scale = 1.37;
	p->mass_function = ORACLE_MF_EQUAL;
	p->rectangular = 0;
	p->approx = 1;
	p->num_stars = 137;
	p->num_phi = 100;
	p->num_branches = 1;
	p->random_seed = 0;
	p->num_threads = 1;
	p->init_iters = 30;
	p->step_iters = 20;
	p->early_out = 1;
	p->polish_tol = 0;
	p->polish_max_iters = 50;
	p->exact_binomials = 0;
}

int oracle_derive(const oracle_params* p, oracle_info* info)
{
	Run R;
	std::memset(&R.info, 0, sizeof(R.info));
	bool ok = derive(p, R, false);
	*info = R.info;
	return ok ? 0 : 1;
}

int oracle_eval(const oracle_params* p, oracle_info* info, int npts, const double* z,
	const double* phi, double* alpha, double* f, double* df, double* w)
{
	Run R;
	std::memset(&R.info, 0, sizeof(R.info));
	if (!derive(p, R, true) || !make_tree(p, R)) { *info = R.info; return 1; }
	const Field& F = R.F;
	int nt = std::max(1, p->num_threads);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 64)
	for (int i = 0; i < npts; i++)
	{
		Cx zz = cx(z[2 * i], z[2 * i + 1]);
		const Node& n = nearest_node(F, zz);
		if (alpha)
		{
			Cx a = add(add(alpha_star(F, zz, n), alpha_local(F, zz, n)), alpha_smooth(F, zz));
			alpha[2 * i] = a.re; alpha[2 * i + 1] = a.im;
		}
		if (f)
		{
			Cx v = parametric_cc(F, zz, n, phi ? phi[i] : 0);
			f[2 * i] = v.re; f[2 * i + 1] = v.im;
		}
		if (df)
		{
			Cx v = d_parametric_cc_dz(F, zz, n);
			df[2 * i] = v.re; df[2 * i + 1] = v.im;
		}
		if (w)
		{
			Cx v = image_to_source(F, zz, n);
			w[2 * i] = v.re; w[2 * i + 1] = v.im;
		}
	}
	*info = R.info;
	return 0;
}

int oracle_run(const oracle_params* p, oracle_info* info, double* stars_out,
	double* ccs, double* caustics, double* errs, double* mu_length_scales)
{
	Run R;
	std::memset(&R.info, 0, sizeof(R.info));
	if (!derive(p, R, true) || !make_tree(p, R)) { *info = R.info; return 1; }
	const Field& F = R.F;
	const int nroots = R.num_roots, nstars = R.num_stars;
	const int nphi = p->num_phi, nb = p->num_branches;
	const int half = nphi / (2 * nb);
	const int nb_solve = (p->max_branches > 0 && p->max_branches < nb) ? p->max_branches : nb;
	/* the solved branches: first_branch + i branch_stride (all of them by default) */
	std::vector<int> branch_of(nb_solve);
	std::vector<char> solved_branch(nb, 0);
	for (int i = 0; i < nb_solve; i++)
	{
		const int st = p->branch_stride > 0 ? p->branch_stride : 1;
		branch_of[i] = nb_solve == nb ? i : (((p->first_branch + i * st) % nb) + nb) % nb;
		solved_branch[branch_of[i]] = 1;
	}
	const bool jac = p->jacobi != 0;
	const int nsteps = (p->max_steps > 0 && p->max_steps < half) ? p->max_steps : half;
	const int nt = std::max(1, p->num_threads);
	const size_t npts = (size_t)(nphi + nb) * nroots;
	const bool early = p->early_out != 0;
	const double tol = 0.000000001;

	/* ccs_init layout of include/ccf.cuh:526: (nphi + nb) rows of nroots */
	std::vector<Cx> z(npts);
	std::vector<char> fin((size_t)nb * 2 * nroots, 0);
	auto center_row = [&](int c) { return (size_t)(half + c * nphi / nb + c); };   /* ccf_functions.cuh:373 */

	/* include/ccf.cuh:711-726; or (seed_curves) the two zeros of f for the
	   star alone at the centre's phase, theta^2 m / (z - z_i)^2 = a e^{-i phi}
	   - gamma with a = 1 - kappa_tot + kappa_star */
	for (int c = 0; c < nb; c++)
	{
		Cx* row = &z[center_row(c) * nroots];
		const double phi = center_phi(c, nb);
		const double a_lin = 1 - F.kappa_tot + F.kappa_star;
		const double dx = a_lin * std::cos(phi) - F.shear, dy = -a_lin * std::sin(phi);
		const double rd = std::hypot(dx, dy), half_arg = -0.5 * std::atan2(dy, dx);
		for (int i = 0; i < nstars; i++)
		{
			if (p->seed_curves && rd > 1e-6 && R.stars_gen[i].mass > 0)
			{
				const double r = F.theta * std::sqrt(R.stars_gen[i].mass / rd);
				const Cx w = cx(r * std::cos(half_arg), r * std::sin(half_arg));
				row[i] = add(R.stars_gen[i].pos, w);
				row[i + nstars] = sub(R.stars_gen[i].pos, w);
			}
			else
			{
				row[i] = addr(R.stars_gen[i].pos, 1);
				row[i + nstars] = subr(R.stars_gen[i].pos, 1);
			}
		}
		int extra = nroots - 2 * nstars;
		for (int i = 0; i < extra; i++)
		{
			row[2 * nstars + i] = rmul(cabs(R.corner), cx(std::cos(2 * PI / extra * i), std::sin(2 * PI / extra * i)));
		}
	}

	long long upd = 0, terms = 0;
	/* include/ccf.cuh:906-940: at j = 0 both sides sweep the same centre row */
	double t0 = now_s();
#pragma omp parallel for num_threads(jac ? 1 : nt) schedule(dynamic, 1) reduction(+ : upd, terms)
	for (int ci = 0; ci < nb_solve; ci++)
	{
		const int c = branch_of[ci];
		Cx* row = &z[center_row(c) * nroots];
		double phi = center_phi(c, nb);
		for (int it = 0; it < p->init_iters; it++)
		{
			for (int b = 0; b < 2; b++)
			{
				char* fl = &fin[((size_t)c * 2 + b) * nroots];
				if (jac) sweep_row_jacobi(F, row, nroots, fl, phi, early, tol, nt, upd, terms);
				else sweep_row(F, row, nroots, fl, phi, early, tol, upd, terms);
			}
		}
	}
	double t1 = now_s();
	/* include/ccf.cuh:1001-1033 with ccf_functions.cuh:261-295 and :321-394 */
#pragma omp parallel for num_threads(jac ? 1 : nt) schedule(dynamic, 1) reduction(+ : upd, terms)
	for (int cb = 0; cb < 2 * nb_solve; cb++)
	{
		int c = branch_of[cb / 2], b = cb % 2;
		int sgn = (b == 0 ? -1 : 1);
		char* fn = &fin[((size_t)c * 2 + b) * nroots];
		for (int j = 1; j <= nsteps; j++)
		{
			Cx* row = &z[(center_row(c) + sgn * j) * nroots];
			const Cx* prev = &z[(center_row(c) + sgn * (j - 1)) * nroots];
			for (int a = 0; a < nroots; a++) { row[a] = prev[a]; fn[a] = 0; }
			double phi = center_phi(c, nb) + sgn * (2 * PI / nphi * j);
			for (int it = 0; it < p->step_iters; it++)
			{
				if (jac) sweep_row_jacobi(F, row, nroots, fn, phi, early, tol, nt, upd, terms);
				else sweep_row(F, row, nroots, fn, phi, early, tol, upd, terms);
			}
		}
	}
	double t2 = now_s();

	/* optional polish: every (branch, step) row iterated without the early
	   return until each root's step is below polish_tol */
	if (p->polish_tol > 0 && p->polish_newton)
	{
		/* every solved point alone: FP64 Newton on the oracle's own f and f'
		   (include/ccf_functions.cuh:69-121) until the step is below
		   polish_tol theta_star */
#pragma omp parallel for num_threads(nt) schedule(dynamic, 256)
		for (long long q = 0; q < (long long)npts; q++)
		{
			const int r = (int)(q / nroots);
			const int c = r / (nphi / nb + 1), k = r % (nphi / nb + 1);
			const int jj = k - half;
			if (!solved_branch[c] || jj < -nsteps || jj > nsteps) continue;
			const double phi = center_phi(c, nb) + (jj < 0 ? -1 : 1) * (2 * PI / nphi * std::abs(jj));
			Cx zz = z[q];
			for (int it = 0; it < p->polish_max_iters; it++)
			{
				const Node& n = nearest_node(F, zz);
				const Cx step = div(parametric_cc(F, zz, n, phi), d_parametric_cc_dz(F, zz, n));
				if (!(std::isfinite(step.re) && std::isfinite(step.im))) break;
				zz = sub(zz, step);
				if (cabs(step) < p->polish_tol * F.theta) break;
			}
			z[q] = zz;
		}
	}
	else if (p->polish_tol > 0)
	{
#pragma omp parallel for num_threads(jac ? 1 : nt) schedule(dynamic, 1)
		for (int r = 0; r < nphi + nb; r++)
		{
			int c = r / (nphi / nb + 1);
			int k = r % (nphi / nb + 1);
			if (!solved_branch[c]) continue;
			int jj = k - half;
			if (jj < -nsteps || jj > nsteps) continue;
			double phi = center_phi(c, nb) + (jj < 0 ? -1 : 1) * (2 * PI / nphi * std::abs(jj));
			std::vector<char> fl(nroots, 0);
			long long u = 0, t = 0;
			for (int it = 0; it < p->polish_max_iters; it++)
			{
				Cx* row = &z[(size_t)r * nroots];
				const int left = jac ? sweep_row_jacobi(F, row, nroots, fl.data(), phi, false, p->polish_tol, nt, u, t)
				                     : sweep_row(F, row, nroots, fl.data(), phi, false, p->polish_tol, u, t);
				if (left == 0) break;
			}
		}
	}

	/* errors, caustics, length scales per point (include/ccf_functions.cuh:419-467,
	   :510-526, :547-563), stored in the output layout of include/ccf.cuh:1077 */
	const int cols = nphi / nb + 1;
	double max_error = 0;
	int has_nan = 0;
	double t3 = now_s();
#pragma omp parallel for num_threads(nt) schedule(dynamic, 256) reduction(max : max_error) reduction(| : has_nan)
	for (long long q = 0; q < (long long)npts; q++)
	{
		int r = (int)(q / nroots), a = (int)(q % nroots);
		int c = r / cols, k = r % cols;
		int jj = k - half;
		bool solved = solved_branch[c] && jj >= -nsteps && jj <= nsteps;
		Cx zz = z[q];
		size_t out = ((size_t)a * nb + c) * cols + k;
		if (ccs) { ccs[2 * out] = zz.re; ccs[2 * out + 1] = zz.im; }
		if (!solved)
		{
			if (errs) errs[out] = 0;
			if (caustics) { caustics[2 * out] = 0; caustics[2 * out + 1] = 0; }
			if (mu_length_scales) mu_length_scales[out] = 0;
			continue;
		}
		const Node& n = nearest_node(F, zz);
		double phi = center_phi(c, nb) + (jj < 0 ? -1 : 1) * (2 * PI / nphi * std::abs(jj));
		Cx f0 = parametric_cc(F, zz, n, phi);
		double sz = d_alpha_smooth_d_z(F, zz);
		double e1 = std::fabs(cabs(f0) * (cabs(f0) + 2 * (1 - F.kappa_tot - sz)));
		double e2 = std::fabs(cabs(f0) * (cabs(f0) - 2 * (1 - F.kappa_tot - sz)));
		double e = std::fmax(e1, e2);
		if (!std::isfinite(e)) has_nan = 1;
		else max_error = std::max(max_error, e);
		if (errs) errs[out] = e;
		if (caustics)
		{
			Cx w = image_to_source(F, zz, n);
			caustics[2 * out] = w.re;
			caustics[2 * out + 1] = w.im;
		}
		if (mu_length_scales && p->write_mu_length_scales) mu_length_scales[out] = mu_length_scale(F, zz, n);
	}
	double t4 = now_s();
	if (stars_out)
	{
		for (int i = 0; i < nstars; i++)
		{
			stars_out[3 * i] = F.stars[i].pos.re;
			stars_out[3 * i + 1] = F.stars[i].pos.im;
			stars_out[3 * i + 2] = F.stars[i].mass;
		}
	}
	R.info.max_error = max_error;
	R.info.has_nan = has_nan;
	R.info.root_updates = upd;
	R.info.root_terms = terms;
	R.info.t_init_roots = t1 - t0;
	R.info.t_ccs = t2 - t1;
	R.info.t_caustics = t4 - t3;
	*info = R.info;
	return 0;
}

int oracle_match_index(int rows, int cols, int nb, const double* a, const double* b, int* idx, double* dist)
{
	if (rows % nb != 0) return 1;
	const int R = rows / nb;
#pragma omp parallel for schedule(dynamic, 4)
	for (long long ck = 0; ck < (long long)nb * cols; ck++)
	{
		int c = (int)(ck / cols), k = (int)(ck % cols);
		std::vector<std::pair<double, int>> bx(R);
		std::vector<double> byy(R);
		for (int r = 0; r < R; r++)
		{
			size_t ib = ((size_t)r * nb + c) * cols + k;
			bx[r] = {b[2 * ib], r};
			byy[r] = b[2 * ib + 1];
		}
		std::sort(bx.begin(), bx.end());
		for (int r = 0; r < R; r++)
		{
			size_t ia = ((size_t)r * nb + c) * cols + k;
			double ax = a[2 * ia], ay = a[2 * ia + 1];
			int pos = (int)(std::lower_bound(bx.begin(), bx.end(), std::make_pair(ax, -1)) - bx.begin());
			double best = std::numeric_limits<double>::infinity();
			int bi = -1;
			for (int dir = -1; dir <= 1; dir += 2)
			{
				for (int q = (dir < 0 ? pos - 1 : pos); q >= 0 && q < R; q += dir)
				{
					double dx = bx[q].first - ax;
					if (dx * dx > best) break;
					int j = bx[q].second;
					double d2 = dx * dx + (byy[j] - ay) * (byy[j] - ay);
					if (d2 < best) { best = d2; bi = j; }
				}
			}
			idx[ia] = bi < 0 ? -1 : (int)((size_t)bi * nb + c);
			dist[ia] = std::sqrt(best);
		}
	}
	return 0;
}

int oracle_match_sets(int rows, int cols, int nb, const double* a, const double* b,
	double* max_dist, long long* non_bijective_cols, long long* non_finite)
{
	if (rows % nb != 0) return 1;
	const int R = rows / nb;
	double md = 0;
	long long nbij = 0, nfin = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(max : md) reduction(+ : nbij, nfin)
	for (long long ck = 0; ck < (long long)nb * cols; ck++)
	{
		int c = (int)(ck / cols), k = (int)(ck % cols);
		std::vector<std::pair<double, int>> bx(R);
		std::vector<double> ax(R), ay(R), bxx(R), byy(R);
		for (int r = 0; r < R; r++)
		{
			size_t ia = ((size_t)r * nb + c) * cols + k;
			ax[r] = a[2 * ia]; ay[r] = a[2 * ia + 1];
			bxx[r] = b[2 * ia]; byy[r] = b[2 * ia + 1];
			if (!std::isfinite(ax[r]) || !std::isfinite(ay[r]) || !std::isfinite(bxx[r]) || !std::isfinite(byy[r])) nfin++;
			bx[r] = {bxx[r], r};
		}
		std::sort(bx.begin(), bx.end());
		std::vector<int> used(R, 0);
		bool bij = true;
		for (int r = 0; r < R; r++)
		{
			/* nearest neighbour by an expanding window over the x-sorted list */
			int pos = (int)(std::lower_bound(bx.begin(), bx.end(), std::make_pair(ax[r], -1)) - bx.begin());
			double best = std::numeric_limits<double>::infinity();
			int bi = -1;
			for (int dir = -1; dir <= 1; dir += 2)
			{
				for (int q = (dir < 0 ? pos - 1 : pos); q >= 0 && q < R; q += dir)
				{
					double dx = bx[q].first - ax[r];
					if (dx * dx > best) break;
					int j = bx[q].second;
					double d2 = dx * dx + (byy[j] - ay[r]) * (byy[j] - ay[r]);
					if (d2 < best) { best = d2; bi = j; }
				}
			}
			if (bi < 0) { bij = false; continue; }
			if (used[bi]++) bij = false;
			if (std::isfinite(best)) md = std::max(md, std::sqrt(best));
		}
		if (!bij) nbij++;
	}
	*max_dist = md;
	*non_bijective_cols = nbij;
	*non_finite = nfin;
	return 0;
}

} /* extern "C" */
