/******************************************************************************
ref_harness.cpp -- TEST INFRASTRUCTURE ONLY (oracle side, never product code).

Runs the reference's own FP64 functions (weisluke/ccf include/*.cuh, compiled
as host C++ through ref_shim.h) in the order CCF<T>::run uses them
(include/ccf.cuh:1265-1280), serially on one CPU core, and writes the
reference's output files plus a few extra diagnostics.  The reference drives
its kernels with <<<>>> launches that a host compiler cannot parse, so this
file restates that driver sequence; every numerical step is a call into the
reference's own headers.

Built by oracle/Makefile into oracle/_ref/ccf_ref_host only where the
reference sources are present.  Used to pin the oracle restatement
(oracle/ccf_oracle.cpp) and to generate the committed golden fixtures.

Usage: ccf_ref_host  -k K -y G -ks KS -t T -mf MF -ms MS -ml ML -mh MH
                      -r R -a A -ss SS -ns N -np NP -nb NB -rs SEED
                      [-sf starfile.bin] [-wls 0|1] -o prefix
******************************************************************************/
#include "ref_shim.h"

#include "array_functions.cuh"
#include "binomial_coefficients.cuh"
#include "ccf_functions.cuh"
#include "complex.cuh"
#include "fmm.cuh"
#include "mass_functions.cuh"
#include "star.cuh"
#include "tree_node.cuh"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <numbers>
#include <string>
#include <vector>

/* storage for the reference kernels' extern __shared__ arrays (serial run) */
namespace treenode { int shared_memory[6 * 1024]; }
namespace fmm { Complex<double> coeffs[(treenode::MAX_EXPANSION_ORDER + 1) * 32]; }

using T = double;

static double now_s()
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char** argv)
{
	/* defaults of include/ccf.cuh:42-62 */
	T kappa_tot = 0.3, shear = 0.3, kappa_star = 0.27, theta_star = 1;
	std::string mass_function_str = "equal";
	T m_solar = 1, m_lower = 0.01, m_upper = 50;
	int rectangular = 0, approx = 1;
	T safety_scale = 1.37;
	int num_stars = 137;
	std::string starfile = "";
	int num_phi = 100, num_branches = 1, random_seed = 0, write_mu_length_scales = 0;
	std::string prefix = "./";

	for (int i = 1; i + 1 < argc; i += 2)
	{
		std::string o = argv[i], v = argv[i + 1];
		if (o == "-k") kappa_tot = std::stod(v);
		else if (o == "-y") shear = std::stod(v);
		else if (o == "-ks") kappa_star = std::stod(v);
		else if (o == "-t") theta_star = std::stod(v);
		else if (o == "-mf") mass_function_str = v;
		else if (o == "-ms") m_solar = std::stod(v);
		else if (o == "-ml") m_lower = std::stod(v);
		else if (o == "-mh") m_upper = std::stod(v);
		else if (o == "-r") rectangular = std::stoi(v);
		else if (o == "-a") approx = std::stoi(v);
		else if (o == "-ss") safety_scale = std::stod(v);
		else if (o == "-ns") num_stars = std::stoi(v);
		else if (o == "-sf") starfile = v;
		else if (o == "-np") num_phi = std::stoi(v);
		else if (o == "-nb") num_branches = std::stoi(v);
		else if (o == "-rs") random_seed = std::stoi(v);
		else if (o == "-wls") write_mu_length_scales = std::stoi(v);
		else if (o == "-o") prefix = v;
		else { std::cerr << "unknown option " << o << "\n"; return 1; }
	}
	if (num_phi % (2 * num_branches) != 0 || num_phi % 2 != 0)
	{
		std::cerr << "num_phi must be a multiple of 2 * num_branches\n";
		return 1;
	}

	/* calculate_derived_params: include/ccf.cuh:348-497 */
	const int MAX_TAYLOR_SMOOTH = 101;
	std::shared_ptr<massfunctions::MassFunction<T>> mass_function;
	T mean_mass = 0, mean_mass2 = 0, mean_mass2_ln_mass = 0;
	Complex<T> corner;
	star<T>* stars = nullptr;
	if (starfile == "")
	{
		if (mass_function_str != "equal")
		{
			m_lower = m_lower * m_solar;
			m_upper = m_upper * m_solar;
		}
		else
		{
			m_lower = 1;
			m_upper = 1;
		}
		mass_function = massfunctions::MASS_FUNCTIONS<T>.at(mass_function_str);
		mean_mass = mass_function->mean_mass(m_lower, m_upper, m_solar);
		mean_mass2 = mass_function->mean_mass2(m_lower, m_upper, m_solar);
		mean_mass2_ln_mass = mass_function->mean_mass2_ln_mass(m_lower, m_upper, m_solar);
	}
	else
	{
		if (!read_star_file<T>(num_stars, rectangular, corner, theta_star, stars,
			kappa_star, m_lower, m_upper, mean_mass, mean_mass2, mean_mass2_ln_mass, starfile))
		{
			std::cerr << "cannot read star file\n";
			return 1;
		}
	}
	T mu_ave = 1 / ((1 - kappa_tot) * (1 - kappa_tot) - shear * shear);
	if (starfile == "")
	{
		corner = Complex<T>(1 / std::abs(1 - kappa_tot + shear), 1 / std::abs(1 - kappa_tot - shear));
		if (rectangular)
		{
			corner = Complex<T>(std::sqrt(corner.re / corner.im), std::sqrt(corner.im / corner.re));
			corner *= std::sqrt(std::numbers::pi_v<T> * theta_star * theta_star * num_stars * mean_mass / (4 * kappa_star));
		}
		else
		{
			corner = corner / corner.abs();
			corner *= std::sqrt(theta_star * theta_star * num_stars * mean_mass / kappa_star);
		}
	}
	T alpha_error = theta_star * 0.0000001;
	int taylor_smooth = 1;
	while ((kappa_star * std::numbers::inv_pi_v<T> * 4 / (taylor_smooth + 1) * corner.abs() * (safety_scale + 1) / (safety_scale - 1)
		* std::pow(1 / safety_scale, taylor_smooth + 1) > alpha_error)
		&& taylor_smooth <= MAX_TAYLOR_SMOOTH)
	{
		taylor_smooth += 2;
	}
	while ((std::fmod(corner.arg() * (taylor_smooth - 1), std::numbers::pi_v<T>) < 0.1 * std::numbers::pi_v<T>
		|| std::fmod(corner.arg() * (taylor_smooth - 1), std::numbers::pi_v<T>) > 0.9 * std::numbers::pi_v<T>)
		&& taylor_smooth <= MAX_TAYLOR_SMOOTH)
	{
		taylor_smooth += 2;
	}
	if (rectangular && taylor_smooth > MAX_TAYLOR_SMOOTH)
	{
		std::cerr << "taylor_smooth too large\n";
		return 1;
	}
	int num_roots;
	if (rectangular) num_roots = approx ? 2 * num_stars + taylor_smooth - 1 : 2 * num_stars;
	else num_roots = approx ? 2 * num_stars : 2 * num_stars + 2;

	/* allocate_initialize_memory: include/ccf.cuh:499-600 */
	curandState* states = (curandState*)std::calloc(num_stars, sizeof(curandState));
	if (stars == nullptr) stars = (star<T>*)std::calloc(num_stars, sizeof(star<T>));
	star<T>* temp_stars = (star<T>*)std::calloc(num_stars, sizeof(star<T>));
	int* binomial_coeffs = (int*)std::calloc(2 * treenode::MAX_EXPANSION_ORDER * (2 * treenode::MAX_EXPANSION_ORDER + 3) / 2 + 1, sizeof(int));
	size_t npts = (size_t)(num_phi + num_branches) * num_roots;
	Complex<T>* ccs_init = new Complex<T>[npts];
	Complex<T>* ccs = new Complex<T>[npts];
	bool* fin = (bool*)std::calloc((size_t)num_branches * 2 * num_roots, sizeof(bool));
	T* errs = (T*)std::calloc(npts, sizeof(T));
	Complex<T>* caustics = new Complex<T>[npts];
	T* mu_length_scales = (T*)std::calloc(npts, sizeof(T));
	int has_nan = 0;

	double t0 = now_s();
	/* populate_star_array: include/ccf.cuh:602-730 */
	if (starfile == "")
	{
		initialize_curand_states_kernel<T>(states, num_stars, random_seed);
		if (mass_function_str == "equal")
			generate_star_field_kernel<T, massfunctions::Equal<T>>(states, stars, num_stars, rectangular, corner, m_lower, m_upper, m_solar);
		else if (mass_function_str == "uniform")
			generate_star_field_kernel<T, massfunctions::Uniform<T>>(states, stars, num_stars, rectangular, corner, m_lower, m_upper, m_solar);
		else if (mass_function_str == "salpeter")
			generate_star_field_kernel<T, massfunctions::Salpeter<T>>(states, stars, num_stars, rectangular, corner, m_lower, m_upper, m_solar);
		else if (mass_function_str == "kroupa")
			generate_star_field_kernel<T, massfunctions::Kroupa<T>>(states, stars, num_stars, rectangular, corner, m_lower, m_upper, m_solar);
		else if (mass_function_str == "optical_depth")
			generate_star_field_kernel<T, massfunctions::OpticalDepth<T>>(states, stars, num_stars, rectangular, corner, m_lower, m_upper, m_solar);
		else { std::cerr << "bad mass function\n"; return 1; }
	}
	else
	{
		random_seed = 0;
	}
	T kappa_star_actual, m_lower_actual, m_upper_actual, mean_mass_actual, mean_mass2_actual, mean_mass2_ln_mass_actual;
	calculate_star_params<T>(num_stars, rectangular, corner, theta_star, stars,
		kappa_star_actual, m_lower_actual, m_upper_actual, mean_mass_actual, mean_mass2_actual, mean_mass2_ln_mass_actual);
	if (starfile == "")
	{
		if (rectangular)
		{
			corner = Complex<T>(std::sqrt(corner.re / corner.im), std::sqrt(corner.im / corner.re));
			corner *= std::sqrt(std::numbers::pi_v<T> * theta_star * theta_star * num_stars * mean_mass_actual / (4 * kappa_star));
		}
		else
		{
			corner = corner / corner.abs();
			corner *= std::sqrt(theta_star * theta_star * num_stars * mean_mass_actual / kappa_star);
		}
	}
	/* write the generated (unsorted) star field too, for exchange with other implementations */
	write_star_file<T>(num_stars, rectangular, corner, theta_star, stars, prefix + "ccf_stars_unsorted.bin");
	for (int j = 0; j < num_branches; j++)
	{
		int center = (num_phi / (2 * num_branches) + j * num_phi / num_branches + j) * num_roots;
		for (int i = 0; i < num_stars; i++)
		{
			ccs_init[center + i] = stars[i].position + 1;
			ccs_init[center + i + num_stars] = stars[i].position - 1;
		}
		int nroots_extra = num_roots - 2 * num_stars;
		for (int i = 0; i < nroots_extra; i++)
		{
			ccs_init[center + 2 * num_stars + i] = corner.abs() *
				Complex<T>(std::cos(2 * std::numbers::pi_v<T> / nroots_extra * i),
					std::sin(2 * std::numbers::pi_v<T> / nroots_extra * i));
		}
	}

	/* create_tree: include/ccf.cuh:732-904 */
	T root_half_length = rectangular ? (corner.re > corner.im ? corner.re : corner.im) : corner.abs();
	root_half_length = root_half_length * 1.1;
	int tree_levels = 0;
	std::vector<TreeNode<T>*> tree;
	std::vector<int> num_nodes;
	tree.push_back(new TreeNode<T>[1]);
	num_nodes.push_back(1);
	tree[0][0] = TreeNode<T>(Complex<T>(0, 0), root_half_length, 0);
	tree[0][0].numstars = num_stars;
	int max_num_stars_in_level, min_num_stars_in_level, num_nonempty_nodes;
	do
	{
		max_num_stars_in_level = 0;
		min_num_stars_in_level = num_stars;
		num_nonempty_nodes = 0;
		treenode::get_node_star_info_kernel<T>(tree[tree_levels], num_nodes[tree_levels],
			&num_nonempty_nodes, &min_num_stars_in_level, &max_num_stars_in_level);
		if (max_num_stars_in_level > treenode::MAX_NUM_STARS_DIRECT)
		{
			int nchild = num_nonempty_nodes * treenode::MAX_NUM_CHILDREN;
			tree.push_back(new TreeNode<T>[nchild > 0 ? nchild : 1]);
			num_nodes.push_back(nchild);
			num_nonempty_nodes--;
			treenode::create_children_kernel<T>(tree[tree_levels], num_nodes[tree_levels], &num_nonempty_nodes, tree[tree_levels + 1]);
			treenode::sort_stars_kernel<T>(tree[tree_levels], num_nodes[tree_levels], stars, temp_stars);
			tree_levels++;
			treenode::set_neighbors_kernel<T>(tree[tree_levels], num_nodes[tree_levels]);
		}
	} while (max_num_stars_in_level > treenode::MAX_NUM_STARS_DIRECT);

	int expansion_order = std::ceil(2 * std::log2(theta_star) + tree_levels
		- std::log2(root_half_length) - std::log2(alpha_error));
	if (expansion_order < 3 || expansion_order > treenode::MAX_EXPANSION_ORDER)
	{
		std::cerr << "bad expansion order " << expansion_order << "\n";
		return 1;
	}
	calculate_binomial_coeffs(binomial_coeffs, 2 * expansion_order);
	for (int i = tree_levels; i >= 0; i--)
	{
		fmm::calculate_multipole_coeffs_kernel<T>(tree[i], num_nodes[i], expansion_order, stars);
		fmm::calculate_M2M_coeffs_kernel<T>(tree[i], num_nodes[i], expansion_order, binomial_coeffs);
	}
	for (int i = 2; i <= tree_levels; i++)
	{
		fmm::calculate_L2L_coeffs_kernel<T>(tree[i], num_nodes[i], expansion_order, binomial_coeffs);
		fmm::calculate_M2L_coeffs_kernel<T>(tree[i], num_nodes[i], expansion_order, binomial_coeffs);
		fmm::calculate_P2L_coeffs_kernel<T>(tree[i], num_nodes[i], expansion_order, binomial_coeffs, stars);
	}
	double t1 = now_s();

	/* find_initial_roots: include/ccf.cuh:906-977 */
	for (int i = 0; i < 30; i++)
	{
		find_critical_curve_roots_kernel<T>(kappa_tot, shear, theta_star, stars, kappa_star, tree[0],
			rectangular, corner, approx, taylor_smooth, ccs_init, num_roots, 0, num_phi, num_branches, fin);
	}
	double t2 = now_s();
	find_errors_kernel<T>(ccs_init, num_roots, kappa_tot, shear, theta_star, stars, kappa_star, tree[0],
		rectangular, corner, approx, taylor_smooth, 0, num_phi, num_branches, errs);
	T max_error_init = 0;
	for (size_t i = 0; i < npts; i++) max_error_init = std::max(max_error_init, errs[i]);

	/* find_ccs: include/ccf.cuh:979-1083 */
	for (int j = 1; j <= num_phi / (2 * num_branches); j++)
	{
		prepare_roots_kernel<T>(ccs_init, num_roots, j, num_phi, num_branches, fin);
		for (int i = 0; i < 20; i++)
		{
			find_critical_curve_roots_kernel<T>(kappa_tot, shear, theta_star, stars, kappa_star, tree[0],
				rectangular, corner, approx, taylor_smooth, ccs_init, num_roots, j, num_phi, num_branches, fin);
		}
	}
	double t3 = now_s();
	for (int j = 0; j <= num_phi / (2 * num_branches); j++)
	{
		find_errors_kernel<T>(ccs_init, num_roots, kappa_tot, shear, theta_star, stars, kappa_star, tree[0],
			rectangular, corner, approx, taylor_smooth, j, num_phi, num_branches, errs);
	}
	has_nan_err_kernel<T>(errs, (int)npts, &has_nan);
	T max_error = 0;
	for (size_t i = 0; i < npts; i++) max_error = std::max(max_error, errs[i]);
	transpose_array_kernel<Complex<T>>(ccs_init, num_phi + num_branches, num_roots, ccs);

	/* find_caustics / find_mu_length_scales: include/ccf.cuh:1085-1121 */
	find_caustics_kernel<T>(ccs, (int)npts, kappa_tot, shear, theta_star, stars, kappa_star, tree[0],
		rectangular, corner, approx, taylor_smooth, caustics);
	double t4 = now_s();
	if (write_mu_length_scales)
	{
		find_mu_length_scales_kernel<T>(ccs, (int)npts, kappa_tot, shear, theta_star, stars, kappa_star, tree[0],
			rectangular, corner, approx, taylor_smooth, mu_length_scales);
	}

	/* outputs, written with the reference's own writers (include/ccf.cuh:1123-1260) */
	write_star_file<T>(num_stars, rectangular, corner, theta_star, stars, prefix + "ccf_stars.bin");
	write_array<Complex<T>>(ccs, num_roots * num_branches, num_phi / num_branches + 1, prefix + "ccf_ccs.bin");
	write_array<Complex<T>>(caustics, num_roots * num_branches, num_phi / num_branches + 1, prefix + "ccf_caustics.bin");
	if (write_mu_length_scales)
	{
		write_array<T>(mu_length_scales, num_roots * num_branches, num_phi / num_branches + 1, prefix + "ccf_mu_length_scales.bin");
	}
	/* errs in the transposed output order, for point-wise residual checks */
	T* errs_t = (T*)std::calloc(npts, sizeof(T));
	transpose_array_kernel<T>(errs, num_phi + num_branches, num_roots, errs_t);
	write_array<T>(errs_t, num_roots * num_branches, num_phi / num_branches + 1, prefix + "ccf_errs.bin");

	std::ofstream info(prefix + "ccf_ref_info.txt");
	info.precision(17);
	info << "num_stars " << num_stars << "\n";
	info << "num_roots " << num_roots << "\n";
	info << "rectangular " << rectangular << "\n";
	info << "corner_x1 " << corner.re << "\n";
	info << "corner_x2 " << corner.im << "\n";
	info << "theta_star " << theta_star << "\n";
	info << "kappa_star " << kappa_star << "\n";
	info << "kappa_star_actual " << kappa_star_actual << "\n";
	info << "mean_mass " << mean_mass << "\n";
	info << "mean_mass2 " << mean_mass2 << "\n";
	info << "mean_mass2_ln_mass " << mean_mass2_ln_mass << "\n";
	info << "mean_mass_actual " << mean_mass_actual << "\n";
	info << "mean_mass2_actual " << mean_mass2_actual << "\n";
	info << "mean_mass2_ln_mass_actual " << mean_mass2_ln_mass_actual << "\n";
	info << "m_lower_actual " << m_lower_actual << "\n";
	info << "m_upper_actual " << m_upper_actual << "\n";
	info << "mu_ave " << mu_ave << "\n";
	info << "taylor_smooth " << taylor_smooth << "\n";
	info << "root_half_length " << root_half_length << "\n";
	info << "tree_levels " << tree_levels << "\n";
	info << "expansion_order " << expansion_order << "\n";
	for (int i = 0; i <= tree_levels; i++) info << "num_nodes_" << i << " " << num_nodes[i] << "\n";
	info << "max_error_init " << max_error_init << "\n";
	info << "max_error " << max_error << "\n";
	info << "has_nan " << has_nan << "\n";
	info << "t_tree_fmm " << (t1 - t0) << "\n";
	info << "t_init_roots " << (t2 - t1) << "\n";
	info << "t_ccs " << (t3 - t2) << "\n";
	info << "t_caustics " << (t4 - t3) << "\n";
	info.close();
	return 0;
}
