/******************************************************************************
stars.cu -- seeded star-field generation, star statistics and root seeds.

Random numbers: curand's XORWOW generator, one subsequence per star
(curand_init(seed, i, 0)), three uniform doubles per star in the order
(x1 or angle, x2 or radius, mass) -- the stream the reference draws
(include/star.cuh:40-107), so a seed gives the reference's star field.
The state lives in registers for the one thread that draws the star; nothing
is written back.
******************************************************************************/
#include "kernels.h"

#include <curand_kernel.h>

namespace ccf
{

CCF_D void generate_star(int i, int seed, int rectangular, double2 corner, double corner_abs, const MassTable& mt,
	double2* __restrict__ pos, double* __restrict__ mass)
{
	curandStateXORWOW_t st;
	curand_init(seed, i, 0, &st);
	double x1, x2;
	if (rectangular)
	{
		x1 = curand_uniform_double(&st) * 2 * corner.x - corner.x;
		x2 = curand_uniform_double(&st) * 2 * corner.y - corner.y;
	}
	else
	{
		double a = curand_uniform_double(&st) * 2 * PI;
		double r = sqrt(curand_uniform_double(&st)) * corner_abs;
		double s, c;
		sincos(a, &s, &c);
		x1 = r * c;
		x2 = r * s;
	}
	pos[i] = make_double2(x1, x2);
	mass[i] = mass_draw(mt, curand_uniform_double(&st));
}

__global__ void __launch_bounds__(256) generate_stars_kernel(int n, int seed, int rectangular, double2 corner, double corner_abs,
	MassTable mt, double2* __restrict__ pos, double* __restrict__ mass)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) generate_star(i, seed, rectangular, corner, corner_abs, mt, pos, mass);
}

/* Deterministic reduction of the star statistics of include/star.cuh:124-161
   by one block of 1024 threads (the summation order is fixed by the block
   size): total mass, sum m^2, sum m^2 ln m, min, max. */
CCF_D void star_stats_block(int n, const double* __restrict__ mass, double* out)
{
	__shared__ double s_m[1024], s_m2[1024], s_l[1024], s_lo[1024], s_hi[1024];
	double m1 = 0, m2 = 0, ml = 0, lo = 1.7976931348623157e308, hi = 2.2250738585072014e-308;
	for (int i = threadIdx.x; i < n; i += blockDim.x)
	{
		double m = mass[i];
		m1 += m;
		m2 += m * m;
		ml += m * m * log(m);
		lo = fmin(lo, m);
		hi = fmax(hi, m);
	}
	s_m[threadIdx.x] = m1;
	s_m2[threadIdx.x] = m2;
	s_l[threadIdx.x] = ml;
	s_lo[threadIdx.x] = lo;
	s_hi[threadIdx.x] = hi;
	__syncthreads();
	for (int s = blockDim.x / 2; s > 0; s >>= 1)
	{
		if (threadIdx.x < s)
		{
			s_m[threadIdx.x] += s_m[threadIdx.x + s];
			s_m2[threadIdx.x] += s_m2[threadIdx.x + s];
			s_l[threadIdx.x] += s_l[threadIdx.x + s];
			s_lo[threadIdx.x] = fmin(s_lo[threadIdx.x], s_lo[threadIdx.x + s]);
			s_hi[threadIdx.x] = fmax(s_hi[threadIdx.x], s_hi[threadIdx.x + s]);
		}
		__syncthreads();
	}
	if (threadIdx.x == 0)
	{
		out[0] = s_m[0];
		out[1] = s_m2[0];
		out[2] = s_l[0];
		out[3] = s_lo[0];
		out[4] = s_hi[0];
	}
}

__global__ void __launch_bounds__(1024) star_stats_kernel(int n, const double* __restrict__ mass, double* out)
{
	star_stats_block(n, mass, out);
}

/* The star field of one field per CTA of 1024 threads, for batches: the
   generated (or uploaded) stars in generation order, their copy that the
   tree build reorders, and the statistics -- what generate_stars_kernel, the
   copy and star_stats_kernel do for one field. */
__global__ void __launch_bounds__(1024) stars_batch_kernel(const BatchSeg* __restrict__ segs)
{
	const BatchSeg& S = segs[blockIdx.x];
	if (S.gen)
		for (int i = threadIdx.x; i < S.n; i += blockDim.x)
			generate_star(i, S.seed, S.rectangular, S.corner, S.corner_abs, S.mt, S.star_gen, S.mass);
	__syncthreads();
	for (int i = threadIdx.x; i < S.n; i += blockDim.x) S.pos[i] = S.star_gen[i];
	star_stats_block(S.n, S.mass, S.stats5);
}

void launch_stars_batch(cudaStream_t s, const BatchSeg* segs, int nseg)
{
	if (nseg > 0) stars_batch_kernel<<<nseg, 1024, 0, s>>>(segs);
}

/* Initial roots of the rows of solved branch centres (row r is the centre
   of branch r seg).  Each star gets two seeds at the critical curve of the
   star alone at the row's phase: with the star's own term the only one,
   f = 0 reads theta^2 m / (z - z_i)^2 = a e^{-i phi} - gamma (a = 1 - kappa
   - d alpha_smooth / dz, include/ccf_functions.cuh:69-86), so
   z = z_i +/- theta sqrt(m) / sqrt(a e^{-i phi} - gamma).  The reference
   seeds z_i +/- 1 (include/ccf.cuh:711-726); both lead the simultaneous
   Aberth iteration to the same set of zeros, these in fewer sweeps.  The
   extra roots of the rectangular Taylor form sit evenly on the circle of
   radius |corner|, as in the reference.  Stars in tree order. */
CCF_D void seed_root(long long q, int nstars, int nroots, const double2* __restrict__ pos, const double* __restrict__ mass,
	double corner_abs, double theta, double a_lin, double gamma, int nb, int seg, double2* __restrict__ master,
	float4* __restrict__ snap32, double2* __restrict__ snap64)
{
	const int extra = nroots - 2 * nstars;
	const int row = (int)(q / nroots);
	const int a = (int)(q % nroots);
	double2 z;
	if (a < 2 * nstars)
	{
		const int i = a < nstars ? a : a - nstars;
		const double phi = PI / nb + (row * seg) * 2 * PI / nb;
		double sp, cp;
		sincos(phi, &sp, &cp);
		/* D = a e^{-i phi} - gamma; w = theta sqrt(m) / sqrt(D) */
		const double dx = a_lin * cp - gamma, dy = -a_lin * sp;
		const double rd = hypot(dx, dy);
		double2 w = make_double2(1, 0);
		if (rd > 1e-6 && mass[i] > 0)
		{
			const double r = theta * sqrt(mass[i] / rd), t = -0.5 * atan2(dy, dx);
			w = make_double2(r * cos(t), r * sin(t));
		}
		const double sg = a < nstars ? 1.0 : -1.0;
		z = make_double2(pos[i].x + sg * w.x, pos[i].y + sg * w.y);
	}
	else
	{
		const int k = a - 2 * nstars;
		const double t = 2 * PI / extra * k;
		z = make_double2(corner_abs * cos(t), corner_abs * sin(t));
	}
	master[q] = z;
	if (snap32) snap32[q] = split_hilo(z);
	if (snap64) snap64[q] = z;
}

__global__ void seed_roots_kernel(int nstars, int nroots, int nrows, const double2* __restrict__ pos,
	const double* __restrict__ mass, double corner_abs, double theta, double a_lin, double gamma, int nb, int seg,
	double2* __restrict__ master, float4* __restrict__ snap32, double2* __restrict__ snap64)
{
	const long long total = (long long)nrows * nroots;
	for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x)
		seed_root(q, nstars, nroots, pos, mass, corner_abs, theta, a_lin, gamma, nb, seg, master, snap32, snap64);
}

/* the seeds of every field of a batch in one launch: blockIdx.y is the field */
__global__ void seed_roots_batch_kernel(const SeedSeg* __restrict__ segs)
{
	const SeedSeg& S = segs[blockIdx.y];
	const long long total = (long long)S.nrows * S.nroots;
	for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x)
		seed_root(q, S.nstars, S.nroots, S.pos, S.mass, S.corner_abs, S.theta, S.a_lin, S.gamma, S.nb, S.seg, S.master,
			S.snap32, S.snap64);
}

/* FP32 hi/lo form of the star positions (the poles of the Aberth sums) and,
   when mass is given, of the masses */
__global__ void star_hilo_kernel(int n, const double2* __restrict__ pos, float4* __restrict__ out,
	const double* __restrict__ mass, float2* __restrict__ mass_out)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	out[i] = split_hilo(pos[i]);
	if (mass)
	{
		float h = __double2float_rn(mass[i]);
		mass_out[i] = make_float2(h, __double2float_rn(mass[i] - (double)h));
	}
}

void launch_generate_stars(cudaStream_t s, int n, int seed, int rectangular, double2 corner, double corner_abs,
	const MassTable& mt, double2* pos, double* mass)
{
	generate_stars_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, seed, rectangular, corner, corner_abs, mt, pos, mass);
}

void launch_star_stats(cudaStream_t s, int n, const double* mass, double* out)
{
	star_stats_kernel<<<1, 1024, 0, s>>>(n, mass, out);
}

void launch_seed_roots(cudaStream_t s, int nstars, int nroots, int nrows, const double2* pos, const double* mass,
	double corner_abs, double theta, double a_lin, double gamma, int nb, int seg, double2* master, float4* snap32,
	double2* snap64)
{
	long long total = (long long)nrows * nroots;
	int blocks = (int)std::min<long long>((total + 255) / 256, 152 * 16);
	seed_roots_kernel<<<blocks, 256, 0, s>>>(nstars, nroots, nrows, pos, mass, corner_abs, theta, a_lin, gamma, nb, seg,
		master, snap32, snap64);
}

void launch_seed_roots_batch(cudaStream_t s, const SeedSeg* segs, int nseg, long long max_seeds)
{
	if (nseg <= 0) return;
	const int gx = (int)std::min<long long>((max_seeds + 255) / 256, 152 * 4);
	seed_roots_batch_kernel<<<dim3(gx, nseg), 256, 0, s>>>(segs);
}

void launch_star_hilo(cudaStream_t s, int n, const double2* pos, float4* out, const double* mass, float2* mass_out)
{
	star_hilo_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, pos, out, mass, mass_out);
}

} /* namespace ccf */
