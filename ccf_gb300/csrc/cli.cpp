/******************************************************************************
cli.cpp -- ccf_gpu, the command line of the reference's main_ccf
(src/main_ccf.cu) over the C ABI: the same 24 option pairs with the same
meanings, defaults, messages and exit codes, plus three additive options,
-pr/--precision (mixed or fp64), -ct/--continuation (track or aberth) and
-d/--device.
******************************************************************************/
#include "ccf_gb300.hpp"

#include <algorithm>
#include <cctype>
#include <iostream>
#include <string>
#include <vector>

namespace
{

/* src/main_ccf.cu:29-56, plus the three additions */
const std::vector<std::string> OPTS = {
	"-h", "--help", "-v", "--verbose", "-k", "--kappa_tot", "-y", "--shear", "-s", "--smooth_fraction",
	"-ks", "--kappa_star", "-t", "--theta_star", "-mf", "--mass_function", "-ms", "--m_solar",
	"-ml", "--m_lower", "-mh", "--m_upper", "-r", "--rectangular", "-a", "--approx", "-ss", "--safety_scale",
	"-ns", "--num_stars", "-sf", "--starfile", "-np", "--num_phi", "-nb", "--num_branches",
	"-rs", "--random_seed", "-ws", "--write_stars", "-wcc", "--write_critical_curves", "-wc", "--write_caustics",
	"-wls", "--write_length_scales", "-o", "--outfile_prefix", "-pr", "--precision", "-ct", "--continuation", "-d", "--device"};

bool exists(char** b, char** e, const std::string& o) { return std::find(b, e, o) != e; }

char* value(char** b, char** e, const std::string& o)
{
	char** it = std::find(b, e, o);
	if (it != e && ++it != e) return *it;
	return nullptr;
}

std::string lower(std::string s)
{
	std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return (char)std::tolower(c); });
	return s;
}

template <typename T, typename U>
void set_param(const std::string& name, T& param, U what, int verbose)
{
	param = static_cast<T>(what);
	if (verbose >= 2) std::cout << name << " set to: " << param << "\n";
}

}  // namespace

CCF<double> ccf;
int verbose = 1;
double smooth_fraction = 1 - ccf.kappa_star / ccf.kappa_tot;

static void display_usage(char* name)
{
	std::cout << "Usage: " << (name ? name : "programname") << " opt1 val1 opt2 val2 opt3 val3 ...\n"
		<< "                                                                               \n"
		<< "Options:\n"
		<< "  -h,--help                  Show this help message\n"
		<< "  -v,--verbose               Specify verbosity of output from 0 (none) to 1, 2,\n"
		<< "                             or 3 (low, medium, high). Default value: " << verbose << "\n"
		<< "  -k,--kappa_tot             Specify the total convergence. Default value: " << ccf.kappa_tot << "\n"
		<< "  -y,--shear                 Specify the shear. Default value: " << ccf.shear << "\n"
		<< "  -s,--smooth_fraction       Specify the fraction of convergence due to\n"
		<< "                             smoothly distributed mass. Default value: " << smooth_fraction << "\n"
		<< "  -ks,--kappa_star           Specify the convergence in point mass lenses. If\n"
		<< "                             provided, this overrides any supplied value for\n"
		<< "                             the smooth fraction. Default value: " << ccf.kappa_star << "\n"
		<< "  -t,--theta_star            Specify the size of the Einstein radius of a unit\n"
		<< "                             mass point lens in arbitrary units.\n"
		<< "                             Default value: " << ccf.theta_star << "\n"
		<< "  -mf,--mass_function        Specify the mass function to use for the point\n"
		<< "                             mass lenses. Options are: equal, uniform,\n"
		<< "                             Salpeter, and, Kroupa, or optical_depth.\n"
		<< "                             Default value: " << ccf.mass_function_str << "\n"
		<< "  -ms,--m_solar              Specify the solar mass in arbitrary units.\n"
		<< "                             Default value: " << ccf.m_solar << "\n"
		<< "  -ml,--m_lower              Specify the lower mass cutoff in solar mass units.\n"
		<< "                             Default value: " << ccf.m_lower << "\n"
		<< "  -mh,--m_upper              Specify the upper mass cutoff in solar mass units.\n"
		<< "                             Default value: " << ccf.m_upper << "\n"
		<< "  -r,--rectangular           Specify whether the star field should be\n"
		<< "                             rectangular (1) or circular (0). Default value: " << ccf.rectangular << "\n"
		<< "  -a,--approx                Specify whether terms for alpha_smooth should be\n"
		<< "                             approximated (1) or exact (0). Default value: " << ccf.approx << "\n"
		<< "  -ss,--safety_scale         Specify the ratio of the size of the star field to\n"
		<< "                             the radius of convergence for alpha_smooth.\n"
		<< "                             Default value: " << ccf.safety_scale << "\n"
		<< "  -ns,--num_stars            Specify the number of stars desired.\n"
		<< "                             Default value: " << ccf.num_stars << "\n"
		<< "  -sf,--starfile             Specify the location of a binary file containing\n"
		<< "                             values for num_stars, rectangular, corner,\n"
		<< "                             theta_star, and the star positions and masses.\n"
		<< "                             A whitespace delimited text file where each line\n"
		<< "                             contains the x1 and x2 coordinates and the mass of\n"
		<< "                             a microlens, in units where theta_star = 1, is\n"
		<< "                             also accepted. If provided, this takes precedence\n"
		<< "                             for all star information.\n"
		<< "  -np,--num_phi              Specify the number of steps used to vary phi in\n"
		<< "                             the range [0, 2*pi]. Default value: " << ccf.num_phi << "\n"
		<< "  -nb,--num_branches         Specify the number of branches to use for phi in\n"
		<< "                             the range [0, 2*pi]. Default value: " << ccf.num_branches << "\n"
		<< "  -rs,--random_seed          Specify the random seed for star field generation.\n"
		<< "                             A value of 0 is reserved for star input files.\n"
		<< "  -ws,--write_stars          Specify whether to write stars (1) or not (0).\n"
		<< "                             Default value: " << ccf.write_stars << "\n"
		<< "  -wcc,                      Specify whether to write critical curves (1) or\n"
		<< "   --write_critical_curves   not (0). Default value: " << ccf.write_critical_curves << "\n"
		<< "  -wc,--write_caustics       Specify whether to write caustics (1) or not (0).\n"
		<< "                             Default value: " << ccf.write_caustics << "\n"
		<< "  -wls,                      Specify whether to write magnification length\n"
		<< "   --write_length_scales     scales (1) or not (0). Default value: " << ccf.write_mu_length_scales << "\n"
		<< "  -o,--outfile_prefix        Specify the prefix to be used in output\n"
		<< "                             filenames. Default value: " << ccf.outfile_prefix << "\n"
		<< "  -pr,--precision            Root solver arithmetic: mixed (FP32 correction sums,\n"
		<< "                             double-float critical-curve function) or fp64.\n"
		<< "                             Default value: mixed\n"
		<< "  -ct,--continuation         Phi continuation: track (each root on its own,\n"
		<< "                             checked, full-sum re-run of failing rows) or\n"
		<< "                             aberth (full Aberth step for every root).\n"
		<< "                             Default value: track\n"
		<< "  -d,--device                CUDA device ordinal. Default value: 0\n";
}

int main(int argc, char* argv[])
{
	char** b = argv;
	char** e = argv + argc;
	if (exists(b, e, "-h") || exists(b, e, "--help"))
	{
		display_usage(argv[0]);
		return -1;
	}
	if ((argc - 1) % 2 != 0)
	{
		std::cerr << "Error. Invalid input syntax.\n";
		display_usage(argv[0]);
		return -1;
	}
	for (int i = 1; i < argc; i += 2)
	{
		if (std::find(OPTS.begin(), OPTS.end(), std::string(argv[i])) == OPTS.end())
		{
			std::cerr << "Error. Invalid input syntax. Unknown option " << argv[i] << "\n";
			display_usage(argv[0]);
			return -1;
		}
		if (argv[i] == std::string("-v") || argv[i] == std::string("--verbose"))
		{
			try
			{
				int v = std::stoi(value(b, e, argv[i]));
				set_param("verbose", verbose, v, v);
			}
			catch (...)
			{
				std::cerr << "Error. Invalid verbose input.\n";
				return -1;
			}
		}
	}
	const bool sf = exists(b, e, "-sf") || exists(b, e, "--starfile");
	const bool ks = exists(b, e, "-ks") || exists(b, e, "--kappa_star");
	for (int i = 1; i < argc; i += 2)
	{
		const std::string o = argv[i];
		char* in = value(b, e, o);
		auto is = [&](const char* s, const char* l) { return o == s || o == l; };
		try
		{
			if (is("-k", "--kappa_tot")) set_param("kappa_tot", ccf.kappa_tot, std::stod(in), verbose);
			else if (is("-y", "--shear")) set_param("shear", ccf.shear, std::stod(in), verbose);
			else if (is("-s", "--smooth_fraction"))
			{
				if (sf || ks) continue;
				set_param("smooth_fraction", smooth_fraction, std::stod(in), verbose);
				if (smooth_fraction < 0)
				{
					std::cerr << "Error. Invalid smooth_fraction input. smooth_fraction must be >= 0\n";
					return -1;
				}
				if (smooth_fraction >= 1)
				{
					std::cerr << "Error. Invalid smooth_fraction input. smooth_fraction must be < 1\n";
					return -1;
				}
			}
			else if (is("-ks", "--kappa_star")) { if (!sf) set_param("kappa_star", ccf.kappa_star, std::stod(in), verbose); }
			else if (is("-t", "--theta_star")) { if (!sf) set_param("theta_star", ccf.theta_star, std::stod(in), verbose); }
			else if (is("-mf", "--mass_function")) { if (!sf) set_param("mass_function", ccf.mass_function_str, lower(in), verbose); }
			else if (is("-ms", "--m_solar")) set_param("m_solar", ccf.m_solar, std::stod(in), verbose);
			else if (is("-ml", "--m_lower")) { if (!sf) set_param("m_lower", ccf.m_lower, std::stod(in), verbose); }
			else if (is("-mh", "--m_upper")) { if (!sf) set_param("m_upper", ccf.m_upper, std::stod(in), verbose); }
			else if (is("-r", "--rectangular")) { if (!sf) set_param("rectangular", ccf.rectangular, std::stoi(in), verbose); }
			else if (is("-a", "--approx")) set_param("approx", ccf.approx, std::stoi(in), verbose);
			else if (is("-ss", "--safety_scale")) set_param("safety_scale", ccf.safety_scale, std::stod(in), verbose);
			else if (is("-ns", "--num_stars")) { if (!sf) set_param("num_stars", ccf.num_stars, std::stoi(in), verbose); }
			else if (is("-sf", "--starfile")) set_param("starfile", ccf.starfile, std::string(in), verbose);
			else if (is("-np", "--num_phi")) set_param("num_phi", ccf.num_phi, std::stoi(in), verbose);
			else if (is("-nb", "--num_branches")) set_param("num_branches", ccf.num_branches, std::stoi(in), verbose);
			else if (is("-rs", "--random_seed")) { if (!sf) set_param("random_seed", ccf.random_seed, std::stoi(in), verbose); }
			else if (is("-ws", "--write_stars")) set_param("write_stars", ccf.write_stars, std::stoi(in), verbose);
			else if (is("-wcc", "--write_critical_curves")) set_param("write_critical_curves", ccf.write_critical_curves, std::stoi(in), verbose);
			else if (is("-wc", "--write_caustics")) set_param("write_caustics", ccf.write_caustics, std::stoi(in), verbose);
			else if (is("-wls", "--write_length_scales")) set_param("write_length_scales", ccf.write_mu_length_scales, std::stoi(in), verbose);
			else if (is("-o", "--outfile_prefix")) set_param("outfile_prefix", ccf.outfile_prefix, std::string(in), verbose);
			else if (is("-pr", "--precision"))
			{
				std::string pr = lower(in);
				if (pr != "mixed" && pr != "fp64") throw std::invalid_argument("precision");
				set_param("precision", ccf.precision, pr == "mixed" ? CCF_PRECISION_MIXED : CCF_PRECISION_FP64, verbose);
			}
			else if (is("-ct", "--continuation"))
			{
				std::string ct = lower(in);
				if (ct != "track" && ct != "aberth") throw std::invalid_argument("continuation");
				set_param("continuation", ccf.continuation, ct == "track" ? CCF_CONTINUATION_TRACK : CCF_CONTINUATION_ABERTH, verbose);
			}
			else if (is("-d", "--device")) set_param("device", ccf.device, std::stoi(in), verbose);
		}
		catch (...)
		{
			/* the message names the long form of the option, as the reference's does */
			size_t k = std::find(OPTS.begin(), OPTS.end(), o) - OPTS.begin();
			std::string name = OPTS[k | 1].substr(2);
			std::cerr << "Error. Invalid " << name << " input.\n";
			return -1;
		}
	}
	/* src/main_ccf.cu:497-502 */
	if (!sf && !ks && (exists(b, e, "-s") || exists(b, e, "--smooth_fraction")))
	{
		set_param("kappa_star", ccf.kappa_star, (1 - smooth_fraction) * ccf.kappa_tot, verbose);
	}
	if (verbose >= 2) std::cout << "\n";
	if (!ccf.run(verbose)) return -1;
	if (!ccf.save(verbose)) return -1;
	return 0;
}
