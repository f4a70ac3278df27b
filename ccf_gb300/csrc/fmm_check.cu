/******************************************************************************
fmm_check.cu -- the far-field error of a built field: at one point in every
leaf, the deflection of the stars from the leaf's near sum and local
expansion against the direct sum over every star,

    alpha_stars(z) = theta^2 sum_i m_i / conj(z - z_i)

(include/alpha_star.cuh:18-115 over all stars).  The reference chooses the
expansion order so that this error stays below alpha_error = 1e-7 theta_star
(include/ccf.cuh:439, :840-852); the check measures it for an explicit
expansion order or leaf size, and for the autotuner's candidates.
******************************************************************************/
#include "kernels.h"

namespace ccf
{

namespace
{

/* one warp per leaf: lanes split the direct sum over all stars; the point is
   a fixed offset from the leaf centre, inside the leaf */
__global__ void fmm_error_kernel(const FieldView* __restrict__ Fp, unsigned long long* out)
{
	const FieldView& F = *Fp;
	const unsigned full = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	const int leaf = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
	if (leaf >= F.num_leaves) return;
	const double2 c = F.leaf_center[leaf];
	const double h = 1.0 / F.leaf_inv_half[leaf];
	const double2 z = make_double2(c.x + 0.37 * h, c.y - 0.61 * h);
	/* direct: sum over every star of m / (z - z_i), lane-strided */
	double sx = 0, sy = 0;
	for (int i = lane; i < F.num_stars; i += 32)
	{
		const double2 p = F.star_pos[i];
		const double2 id = cinv(make_double2(z.x - p.x, z.y - p.y));
		sx = fma(F.star_mass[i], id.x, sx);
		sy = fma(F.star_mass[i], id.y, sy);
	}
	for (int o = 16; o > 0; o >>= 1)
	{
		sx += __shfl_xor_sync(full, sx, o);
		sy += __shfl_xor_sync(full, sy, o);
	}
	if (lane != 0) return;
	/* the field's evaluation: near stars directly, the rest from the local
	   expansion (alpha_star = theta^2 conj(s1), alpha_local = conj(H1)) */
	const int lf = find_leaf(F, z);
	if (lf < 0) return;
	const NearSums S = leaf_sums<true, false>(F, lf, z);
	const int P = F.order;
	const double2 al = local_horner(F.leaf_loc + (size_t)lf * 3 * (P + 1), P, 1, leaf_dz(F, lf, z));
	/* both as conj(alpha): theta^2 s1 + H1 against theta^2 sum m / (z - z_i) */
	const double ex = F.theta2 * S.s1.x + al.x - F.theta2 * sx;
	const double ey = F.theta2 * S.s1.y + al.y - F.theta2 * sy;
	const double e = hypot(ex, ey);
	if (isfinite(e)) atomicMax(out, (unsigned long long)__double_as_longlong(e));
	else atomicMax(out, 0x7ff0000000000000ull);
}

} /* namespace */

cudaError_t launch_fmm_error(cudaStream_t s, const FieldView* F_dev, int num_leaves, unsigned long long* out)
{
	if (num_leaves <= 0) return cudaSuccess;
	const int warps = 8;
	fmm_error_kernel<<<(num_leaves + warps - 1) / warps, warps * 32, 0, s>>>(F_dev, out);
	return cudaGetLastError();
}

} /* namespace ccf */
