// tdvmc_run -- native host driver of the GB300 TDVP path.
//
// The GPU counterpart of the reference's main program for the BosonsBulk
// system (mainMPI, src/TDVMC.cpp:3004-4059): reads a reference JSON config
// (the keys registered in RegisterAllConfigItems, TDVMC.cpp:297-349),
// initialises the walkers on a jittered lattice (InitCoordinateConfiguration,
// TDVMC.cpp:672-785), runs the time loop through the C ABI of
// include/tdvmc_gpu.h (TDVMC.cpp:3419-3926) and writes the same per-step
// files (AppendDataToFile calls, TDVMC.cpp:3833-3839) and end-of-run files
// (TDVMC.cpp:3939-3953) with 15 significant digits in 24-character columns
// (Utils.h:25-28).
//
// With CALCULATE_ADDITIONAL_DATA_EVERY_NTH_STEP > 0 it appends g(r) and S(k)
// to gr.dat and sk.dat and the time to timesAdditional.dat
// (TDVMC.cpp:3471-3520), after MC_NADDITIONALTHERMSTEPS moves per walker;
// the k shells are the first 50 of kVectors{D}D.json next to the config file
// (BosonsBulk.cpp:55, 124-139).
//
// Files as the reference: the config must carry CONFIG_VERSION "0.24"
// (TDVMC.cpp:133, 3039-3043); walkers start from
// <config dir>/coords/particleconfiguration_<N>_<DIM>D_<k>.csv when such files
// exist (the last line, comma-separated x y z per particle;
// LoadLastPositionsFromFile, TDVMC.cpp:640-670; walker w takes file w mod the
// number of consecutive files k = 0, 1, ...), else from the jittered lattice;
// at the end the driver writes AAFinish_particleconfiguration_<N>_<DIM>D.dat
// (walker 0) and coords/particleconfiguration_<N>_<DIM>D_<k>.dat for the first
// GPU_COORDS_FILES walkers (default 1) (TDVMC.cpp:4010-4018), and
// AAFinish_tVMC.config: the input config with the final parameters
// (WriteConfig, TDVMC.cpp:387-407, 4027-4034; numbers with 17 significant
// digits where the reference prints 6).
//
// Random-number state for a successive run, as the reference keeps its
// generators' states (random/state_*_<rank>.dat read from the config directory
// at the start when present and written to the output directory at the end,
// Utils.cpp:48-78, TDVMC.cpp:515-525, 3958-3964): the Philox streams are keyed
// by (GPU_SEED, epoch) with the epoch in the key's upper 32 bits;
// random/state_philox.dat holds "seed epoch", a run that finds it in the config
// directory continues with that seed at the next epoch (fresh streams, none of
// the previous run's repeated), and every run writes its own pair at the end.
//
// Parameter acceptance (USE_PARAMETER_ACCEPTANCE_CHECK = 1, TDVMC.cpp:3648-
// 3800, AcceptNewParams 2585-2630): a step is tried at most twice, the second
// time with twice the sampling effort; PARAMETER_ACCEPTANCE_CHECK_TYPE 0
// rejects a non-positive-definite S, 1 also non-finite new parameters, 2 also a
// relative change of any uR_k above 0.1 from the step's start.  A step that
// needed its second trial sets the run back 5 steps (SetBackNSteps,
// TDVMC.cpp:2746-2784, 3876-3880, 3909-3916): time, records and parameters of
// the last 5 steps are dropped and the walkers restart from their initial
// configuration with MC_VERY_FIRST_NINITIALIZATIONSTEPS moves.  Check types 3
// and above are refused.
//
// Extra keys (all optional): GPU_WALKERS (default MC_NSTEPS), GPU_PRECISION
// ("mixed" or "fp64"), POTENTIAL ("square" as BosonsBulk, "gauss", "lj"),
// HBAR2_2M (default 1.0, the reference's constant), GPU_ADJOINT (0/1),
// GPU_SEED (its low 32 bits key the Philox streams), GPU_COORDS_FILES.
//
// usage: tdvmc_run <config file> [output directory]
#include "tdvmc_gpu.h"

#include <sys/stat.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <memory>
#include <random>
#include <sstream>
#include <string>
#include <vector>

namespace {

// ---------------------------------------------------------------- JSON ----
struct Json {
	enum Kind { NUL, NUM, STR, BOOL, ARR, OBJ } kind = NUL;
	double num = 0.0;
	bool b = false;
	std::string str;
	std::vector<Json> arr;
	std::map<std::string, Json> obj;
};

struct Parser {
	const std::string& s;
	size_t i = 0;
	explicit Parser(const std::string& src) : s(src) {}
	void ws() {
		while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
	}
	bool fail(const char* what) {
		std::fprintf(stderr, "config: JSON error near offset %zu: %s\n", i, what);
		return false;
	}
	bool value(Json& out) {
		ws();
		if (i >= s.size()) return fail("unexpected end");
		char c = s[i];
		if (c == '{') {
			out.kind = Json::OBJ;
			i++;
			ws();
			if (i < s.size() && s[i] == '}') {
				i++;
				return true;
			}
			while (true) {
				ws();
				Json key;
				if (!string(key)) return false;
				ws();
				if (i >= s.size() || s[i] != ':') return fail("expected ':'");
				i++;
				Json v;
				if (!value(v)) return false;
				out.obj[key.str] = v;
				ws();
				if (i < s.size() && s[i] == ',') {
					i++;
					continue;
				}
				if (i < s.size() && s[i] == '}') {
					i++;
					return true;
				}
				return fail("expected ',' or '}'");
			}
		}
		if (c == '[') {
			out.kind = Json::ARR;
			i++;
			ws();
			if (i < s.size() && s[i] == ']') {
				i++;
				return true;
			}
			while (true) {
				Json v;
				if (!value(v)) return false;
				out.arr.push_back(v);
				ws();
				if (i < s.size() && s[i] == ',') {
					i++;
					continue;
				}
				if (i < s.size() && s[i] == ']') {
					i++;
					return true;
				}
				return fail("expected ',' or ']'");
			}
		}
		if (c == '"') return string(out);
		if (s.compare(i, 4, "true") == 0) {
			out.kind = Json::BOOL;
			out.b = true;
			i += 4;
			return true;
		}
		if (s.compare(i, 5, "false") == 0) {
			out.kind = Json::BOOL;
			i += 5;
			return true;
		}
		if (s.compare(i, 4, "null") == 0) {
			i += 4;
			return true;
		}
		char* end = nullptr;
		out.num = std::strtod(s.c_str() + i, &end);
		if (end == s.c_str() + i) return fail("bad value");
		out.kind = Json::NUM;
		i = end - s.c_str();
		return true;
	}
	bool string(Json& out) {
		if (s[i] != '"') return fail("expected string");
		out.kind = Json::STR;
		i++;
		while (i < s.size() && s[i] != '"') {
			if (s[i] == '\\' && i + 1 < s.size()) i++;
			out.str.push_back(s[i++]);
		}
		if (i >= s.size()) return fail("unterminated string");
		i++;
		return true;
	}
};

struct Config {
	Json root;
	double num(const char* k, double def) const {
		auto it = root.obj.find(k);
		return (it != root.obj.end() && it->second.kind == Json::NUM) ? it->second.num : def;
	}
	std::string str(const char* k, const std::string& def) const {
		auto it = root.obj.find(k);
		return (it != root.obj.end() && it->second.kind == Json::STR) ? it->second.str : def;
	}
	std::vector<double> vec(const char* k) const {
		std::vector<double> v;
		auto it = root.obj.find(k);
		if (it != root.obj.end() && it->second.kind == Json::ARR)
			for (auto& e : it->second.arr) v.push_back(e.num);
		return v;
	}
};

// -------------------------------------------------------------- output ----
std::string g_out;

void append_line(const std::string& name, const std::vector<double>& v) {
	std::ofstream f(g_out + name + ".dat", std::ios::app);
	f.precision(15);
	f << std::scientific;
	for (double x : v) f << std::setw(24) << x;
	f << "\n";
}

// A file of one header line and rows (every nth row from the nth on): a single
// header as its own line, several as 24-wide columns (Utils.cpp:809-858).
void write_table(const std::string& name, const std::vector<std::string>& header,
                 const std::vector<std::vector<double>>& rows, int nth = 1) {
	std::ofstream f(g_out + name + ".dat");
	f.precision(15);
	f << std::scientific;
	if (header.size() == 1) {
		f << header[0];
	} else {
		for (auto& h : header) f << std::setw(24) << h;
	}
	f << "\n";
	for (size_t i = (size_t)nth - 1; i < rows.size(); i += (size_t)nth) {
		for (double x : rows[i]) f << std::setw(24) << x;
		f << "\n";
	}
}

// k shells: rows of the "data" array of kVectors{D}D.json, scaled by 2 pi / L
bool read_k_shells(const std::string& path, int dim, double L, int nshell, std::vector<int32_t>& off,
                   std::vector<double>& kvec) {
	std::ifstream in(path);
	if (!in) return false;
	std::stringstream ss;
	ss << in.rdbuf();
	std::string text = ss.str();
	Json j;
	Parser ps(text);
	if (!ps.value(j) || j.kind != Json::OBJ) return false;
	auto it = j.obj.find("data");
	if (it == j.obj.end() || it->second.kind != Json::ARR) return false;
	off.assign(1, 0);
	kvec.clear();
	const double f = 2.0 * M_PI / L;
	for (size_t k = 0; k < it->second.arr.size() && (int)k < nshell; k++) {
		for (auto& v : it->second.arr[k].arr) {
			if (v.kind != Json::ARR || (int)v.arr.size() < dim) return false;
			for (int a = 0; a < dim; a++) kvec.push_back(v.arr[a].num * f);
		}
		off.push_back((int32_t)(kvec.size() / dim));
	}
	return true;
}

// JSON text of a value (numbers with 17 significant digits)
std::string json_text(const Json& j) {
	std::ostringstream o;
	o.precision(17);
	switch (j.kind) {
	case Json::NUM:
		o << j.num;
		break;
	case Json::STR:
		o << '"' << j.str << '"';
		break;
	case Json::BOOL:
		o << (j.b ? "true" : "false");
		break;
	case Json::ARR:
		o << "\n\t[\n\t\t ";
		for (size_t i = 0; i < j.arr.size(); i++) o << (i ? ", " : "") << json_text(j.arr[i]);
		o << "\n\t]";
		break;
	case Json::OBJ: {
		o << "{";
		size_t i = 0;
		for (auto& kv : j.obj) o << (i++ ? ", " : "") << '"' << kv.first << "\" : " << json_text(kv.second);
		o << "}";
		break;
	}
	default:
		o << "null";
	}
	return o.str();
}

Json json_array(const std::vector<double>& v) {
	Json j;
	j.kind = Json::ARR;
	for (double x : v) {
		Json e;
		e.kind = Json::NUM;
		e.num = x;
		j.arr.push_back(e);
	}
	return j;
}

// the last non-empty line of a coordinate file, numbers separated by commas
// (LoadLastPositionsFromFile) or white space
bool read_last_positions(const std::string& path, int n, int dim, std::vector<double>& xyz) {
	std::ifstream f(path);
	if (!f) return false;
	std::string line, last;
	while (std::getline(f, line))
		if (line.find_first_not_of(" \t\r") != std::string::npos) last = line;
	if (last.empty()) return false;
	for (char& c : last)
		if (c == ',') c = ' ';
	std::istringstream in(last);
	xyz.clear();
	double v;
	while (in >> v) xyz.push_back(v);
	return (int)xyz.size() >= n * dim;
}

// one line of N x DIM coordinates, particle-major, in the data-file format
// (WriteParticleInputFile: WriteDataToFile without a header)
void write_positions(const std::string& path, const std::vector<double>& x, int64_t w, int n, int dim) {
	std::ofstream f(path);
	f.precision(15);
	f << std::scientific;
	for (int i = 0; i < n; i++)
		for (int a = 0; a < dim; a++) f << std::setw(24) << x[((size_t)w * dim + a) * n + i];
	f << "\n";
}

bool file_exists(const std::string& p) {
	struct stat st;
	return stat(p.c_str(), &st) == 0;
}

int die(const char* what, int code) {
	std::fprintf(stderr, "tdvmc_run: %s: %s (%d)\n", what, tdvmc_status_string(code), code);
	return 1;
}

}  // namespace

int main(int argc, char** argv) {
	if (argc < 2) {
		std::fprintf(stderr, "usage: %s <config> [output directory]\n", argv[0]);
		return 2;
	}
	std::ifstream in(argv[1]);
	if (!in) {
		std::fprintf(stderr, "cannot read %s\n", argv[1]);
		return 2;
	}
	std::stringstream ss;
	ss << in.rdbuf();
	std::string text = ss.str();
	Config cfg;
	Parser ps(text);
	if (!ps.value(cfg.root) || cfg.root.kind != Json::OBJ) return 2;
	// the reference refuses configs of another version (TDVMC.cpp:133, 3039-3043)
	const std::string required_version = "0.24";
	if (cfg.str("CONFIG_VERSION", "") != required_version) {
		std::fprintf(stderr, "Config file is out of date.\nrequired: \"%s\"\nfound: \"%s\"\n",
		             required_version.c_str(), cfg.str("CONFIG_VERSION", "").c_str());
		return 1;
	}
	// BosonsBulk (TDVMC.cpp:2843-2850) or NUBosonsBulkPB (2953-2960)
	const std::string system = cfg.str("SYSTEM_TYPE", "BosonsBulk");
	if (system != "BosonsBulk" && system != "NUBosonsBulkPB") {
		std::fprintf(stderr, "only SYSTEM_TYPE BosonsBulk and NUBosonsBulkPB are implemented on the GPU\n");
		return 2;
	}
	const bool pb = system == "NUBosonsBulkPB";
	if (pb && (int)cfg.num("USE_NURBS", 0) != 1) {
		// NUBosonsBulkPB reads r_max from the knot vector before it would build default
		// knots (NUBosonsBulkPB.cpp:76, 91-97): the reference program crashes without them
		std::fprintf(stderr, "SYSTEM_TYPE NUBosonsBulkPB needs USE_NURBS = 1 and its NURBS_GRID\n");
		return 2;
	}
	g_out = argc > 2 ? std::string(argv[2]) : cfg.str("OUTPUT_DIRECTORY", "./");
	if (!g_out.empty() && g_out.back() != '/') g_out += "/";
	mkdir(g_out.c_str(), 0755);

	const int N = (int)cfg.num("N", 2), DIM = (int)cfg.num("DIM", 3), P = (int)cfg.num("N_PARAM", 10);
	const double LBOX = cfg.num("LBOX", 1.0);
	const int MC_NSTEPS = (int)cfg.num("MC_NSTEPS", 1);
	const int MC_NTHERMSTEPS = (int)cfg.num("MC_NTHERMSTEPS", N);
	const int MC_VERY_FIRST = (int)cfg.num("MC_VERY_FIRST_NINITIALIZATIONSTEPS", 0);
	const double MC_STEP = cfg.num("MC_STEP", 0.5);
	const double TIMESTEP = cfg.num("TIMESTEP", 1e-3), TOTALTIME = cfg.num("TOTALTIME", 0.0);
	const int WRITE_NTH = std::max(1, (int)cfg.num("WRITE_EVERY_NTH_STEP_TO_FILE", 1));
	const int64_t walkers = (int64_t)cfg.num("GPU_WALKERS", MC_NSTEPS);
	const std::string prec = cfg.str("GPU_PRECISION", "mixed");
	const std::string pot = cfg.str("POTENTIAL", "square");
	uint64_t seed_base = (uint64_t)cfg.num("GPU_SEED", 1) & 0xFFFFFFFFull;
	uint64_t epoch = 0;
	const int ADD_NTH = (int)cfg.num("CALCULATE_ADDITIONAL_DATA_EVERY_NTH_STEP", 0);
	const int ADD_THERM = (int)cfg.num("MC_NADDITIONALTHERMSTEPS", 0);
	const int GR_BINS = (int)cfg.num("GR_BIN_COUNT", 50);
	std::string cfg_dir = argv[1];
	cfg_dir = cfg_dir.find_last_of("\\/") == std::string::npos ? "./" : cfg_dir.substr(0, cfg_dir.find_last_of("\\/")) + "/";

	{
		// the previous run's random-number state, when the config directory holds it
		std::ifstream fs(cfg_dir + "random/state_philox.dat");
		uint64_t sb = 0, ep = 0;
		if (fs >> sb >> ep) {
			seed_base = sb & 0xFFFFFFFFull;
			epoch = (ep + 1) & 0xFFFFFFFFull;
			std::printf("random state from %srandom/state_philox.dat: seed %llu, epoch %llu\n", cfg_dir.c_str(),
			            (unsigned long long)seed_base, (unsigned long long)epoch);
		}
	}
	const uint64_t seed = (epoch << 32) | seed_base;

	tdvmc_system_desc d{};
	d.dim = DIM;
	d.n = N;
	d.p = P;
	std::vector<double> grid = cfg.vec("NURBS_GRID");
	if ((int)cfg.num("USE_NURBS", 0) == 1) {
		d.n_user_knots = (int)grid.size();
		d.user_knots = grid.data();
	}
	d.box_length = LBOX;
	d.pot_kind = pot == "lj" ? TDVMC_POT_LJ : (pot == "gauss" ? TDVMC_POT_GAUSS : TDVMC_POT_SQUARE);
	if (pb) {
		// its square well (NUBosonsBulkPB.cpp:347-350); GPU_PB_EXACT_DERIVATIVES = 1 selects the
		// exact derivatives of the mirrored pair term instead of the reference's form
		d.pot_kind = TDVMC_POT_SQUARE;
		d.system_type = (int)cfg.num("GPU_PB_EXACT_DERIVATIVES", 0) == 1 ? TDVMC_SYS_NU_BOSONS_BULK_PB_EXACT
		                                                                  : TDVMC_SYS_NU_BOSONS_BULK_PB;
	}
	// NUBosonsBulkPB reports 9 + GR_BIN_COUNT other expectation values (400 bins when the
	// count is 0), the g(r) entries never filled (NUBosonsBulkPB.cpp:55-61, 578-582)
	const int pb_gr = pb ? ((int)cfg.num("GR_BIN_COUNT", 0) > 0 ? (int)cfg.num("GR_BIN_COUNT", 0) : 400) : 0;
	std::vector<double> sp = cfg.vec("SYSTEM_PARAMS");
	d.n_pot = (int)std::min<size_t>(5, sp.size());
	for (int i = 0; i < d.n_pot; i++) d.pot[i] = sp[i];
	d.hbar2_2m = cfg.num("HBAR2_2M", 1.0);
	d.precision = prec == "fp64" ? TDVMC_PREC_FP64 : TDVMC_PREC_MIXED;
	d.n_walkers = walkers;
	tdvmc_ctx* ctx = nullptr;
	int rc = tdvmc_create(&d, &ctx);
	if (rc) return die("tdvmc_create", rc);

	std::vector<double> uR = cfg.vec("PARAMS_REAL"), uI = cfg.vec("PARAMS_IMAGINARY");
	uR.resize(P, 0.0);
	uI.resize(P, 0.0);
	double phiR = cfg.num("PARAM_PHIR", 0.0), phiI = cfg.num("PARAM_PHII", 0.0);
	if ((rc = tdvmc_set_params(ctx, uR.data(), uI.data(), phiR, phiI))) return die("tdvmc_set_params", rc);
	{
		// start parameters, one per line, and the per-step files with their headers
		// (TDVMC.cpp:3117-3128)
		std::vector<std::vector<double>> cR, cI;
		for (int k = 0; k < P; k++) {
			cR.push_back({uR[k]});
			cI.push_back({uI[k]});
		}
		write_table("ParametersR0", {"uR_k..."}, cR);
		write_table("ParametersI0", {"uI_k..."}, cI);
		const std::vector<std::vector<double>> none;
		write_table("LocalEnergyR", {"E^R"}, none);
		write_table("LocalEnergyI", {"E^I"}, none);
		write_table("LocalOperators", {"<O_k>..."}, none);
		write_table("OtherExpectationValues", {"kinetic, potential, wf, g(r)"}, none);
		write_table("ParametersR", {"uR_k..."}, none);
		write_table("ParametersI", {"uI_k..."}, none);
		write_table("times", {"t"}, none);
	}

	// initial walkers (InitCoordinateConfiguration, TDVMC.cpp:672-785): the last line of
	// coords/particleconfiguration_<N>_<DIM>D_<k>.csv for k = 0, 1, ... (walker w takes
	// file w mod K), else the lattice with 1/10 jitter, one generator per walker
	std::vector<double> x0((size_t)walkers * DIM * N);
	std::vector<std::vector<double>> files;
	{
		const std::string stem = cfg_dir + "coords/particleconfiguration_" + std::to_string(N) + "_" +
		                         std::to_string(DIM) + "D_";
		std::vector<double> xyz;
		while (read_last_positions(stem + std::to_string(files.size()) + ".csv", N, DIM, xyz)) files.push_back(xyz);
	}
	if (!files.empty()) {
		std::printf("init coordinates from %zu file(s) coords/particleconfiguration_%d_%dD_*.csv\n", files.size(), N,
		            DIM);
		for (int64_t w = 0; w < walkers; w++) {
			const std::vector<double>& f = files[(size_t)(w % (int64_t)files.size())];
			for (int i = 0; i < N; i++)
				for (int a = 0; a < DIM; a++) x0[((size_t)w * DIM + a) * N + i] = f[(size_t)i * DIM + a];
		}
	} else {
		const int m = (int)std::lround(std::pow((double)N, 1.0 / DIM));
		const double l = LBOX / m;
		for (int64_t w = 0; w < walkers; w++) {
			std::mt19937_64 gen((uint64_t)w + 1);
			std::uniform_real_distribution<double> U(0.0, 1.0);
			for (int i = 0; i < N; i++) {
				int idx[3] = {0, 0, 0}, rem = i;
				for (int a = DIM - 1; a >= 0; a--) {
					idx[a] = rem % m;
					rem /= m;
				}
				for (int a = 0; a < DIM; a++) {
					double v = idx[a] * l + (U(gen) - 0.5) * l / 10.0;
					if (DIM == 1) v -= LBOX / 2.0;
					x0[((size_t)w * DIM + a) * N + i] = v;
				}
			}
		}
	}
	// the start configuration (of walker 0), as the reference writes its chain's (TDVMC.cpp:3095-3098)
	write_positions(g_out + "particleconfiguration.dat", x0, 0, N, DIM);
	int64_t acc = 0;
	uint32_t restarts = 0;
	// walkers from their initial configuration, thermalised (also after a set-back)
	auto init_walkers = [&]() -> int {
		int r = tdvmc_set_walkers(ctx, x0.data(), walkers);
		if (r) return r;
		if (MC_VERY_FIRST > 0) r = tdvmc_sample(ctx, MC_VERY_FIRST, MC_STEP, seed, 0xFFFFFFF0u - restarts, &acc);
		restarts++;
		return r;
	};
	if ((rc = init_walkers())) return die("initial walkers", rc);

	tdvmc_step_opts o{};
	o.dt = TIMESTEP;
	o.imaginary_time = (int)cfg.num("IMAGINARY_TIME", 0);
	o.ode_solver = (int)cfg.num("ODE_SOLVER_TYPE", 2);
	o.lin_solver = (int)cfg.num("LINEAR_EQUATION_SOLVER_TYPE", 0);
	o.precondition = (int)cfg.num("USE_PRECONDITIONING", 0);
	o.normalize_wf = (int)cfg.num("USE_NORMALIZE_WF", 0);
	o.moves_per_stage = MC_NTHERMSTEPS;
	o.mc_step = MC_STEP;
	o.seed = seed;
	o.use_adjoint = (int)cfg.num("GPU_ADJOINT", 0);
	// ODE_SOLVER_TYPE 3 and 5: samples are refreshed on every step after the first
	// whenever UPDATE_SAMPLES_EVERY_NTH_STEP > 0, because the reference's
	// condition (TDVMC.cpp:3665) also holds for every parameter trial
	o.update_every = (int)cfg.num("UPDATE_SAMPLES_EVERY_NTH_STEP", 0) > 0 ? 1 : 0;
	o.update_percent = cfg.num("UPDATE_SAMPLES_PERCENT", 100.0);
	if (o.ode_solver != 0 && o.ode_solver != 2 && o.ode_solver != 3 && o.ode_solver != 5) {
		std::fprintf(stderr, "ODE_SOLVER_TYPE %d is not implemented on the GPU (0, 2, 3 and 5 are)\n", o.ode_solver);
		return 2;
	}
	const bool acceptance_check = (int)cfg.num("USE_PARAMETER_ACCEPTANCE_CHECK", 0) == 1;
	const int check_type = (int)cfg.num("PARAMETER_ACCEPTANCE_CHECK_TYPE", 0);
	if (acceptance_check && (check_type < 0 || check_type > 2)) {
		std::fprintf(stderr, "PARAMETER_ACCEPTANCE_CHECK_TYPE %d is not implemented on the GPU (0, 1 and 2 are)\n",
		             check_type);
		return 2;
	}
	const int coords_files = std::max(0, (int)cfg.num("GPU_COORDS_FILES", 1));

	std::vector<std::vector<double>> allER, allEI, allO, allOther, allPR, allPI;
	std::vector<double> times;
	std::vector<double> O(P);
	std::vector<int32_t> k_off;
	std::vector<double> k_vec;
	if (ADD_NTH > 0) {
		const std::string kp = cfg_dir + "kVectors" + std::to_string(DIM) + "D.json";
		if (!read_k_shells(kp, DIM, LBOX, 50, k_off, k_vec)) {
			std::fprintf(stderr, "cannot read the k vectors %s; S(k) is skipped\n", kp.c_str());
			k_off.assign(1, 0);
		}
	}
	// parameters at the start of the last steps (uRList etc., TDVMC.cpp:3437-3460)
	std::vector<std::vector<double>> histR, histI;
	std::vector<double> histPR, histPI;
	int step = 0;
	for (double t = 0.0; t <= TOTALTIME; t += TIMESTEP, step++) {
		if ((rc = tdvmc_set_time(ctx, t))) return die("tdvmc_set_time", rc);
		if (ADD_NTH > 0 && step % ADD_NTH == 0) {
			// additional system properties of the current parameters (TDVMC.cpp:3471-3520)
			if (ADD_THERM > 0 && (rc = tdvmc_sample(ctx, ADD_THERM, MC_STEP, seed, 0xFFFF0000u + (uint32_t)step, &acc)))
				return die("tdvmc_sample", rc);
			const int nshell = (int)k_off.size() - 1;
			std::vector<double> gr(GR_BINS), sk(std::max(nshell, 1));
			int32_t ngr = 0;
			if ((rc = tdvmc_observables(ctx, GR_BINS, nshell, k_off.data(), k_vec.empty() ? nullptr : k_vec.data(),
			                            gr.data(), &ngr, sk.data())))
				return die("tdvmc_observables", rc);
			gr.resize(ngr);
			sk.resize(nshell);
			append_line("timesAdditional", {t});
			append_line("gr", gr);
			if (nshell > 0) append_line("sk", sk);
		}
		std::vector<double> pR(P), pI(P);
		double p0R, p0I;
		tdvmc_get_params(ctx, pR.data(), pI.data(), &p0R, &p0I);
		histR.push_back(pR);
		histI.push_back(pI);
		histPR.push_back(p0R);
		histPI.push_back(p0I);
		if (histR.size() > 105) {
			histR.erase(histR.begin());
			histI.erase(histI.begin());
			histPR.erase(histPR.begin());
			histPI.erase(histPI.begin());
		}
		tdvmc_stats st{};
		tdvmc_step_opts oo = o;
		// up to two trials, the second with twice the sampling effort (TDVMC.cpp:3648-3651);
		// a trial is rejected by a non-positive-definite S (doNotAcceptStep,
		// TDVMC.cpp:1583-1588) and, by check type, by non-finite or too large changes of
		// the new parameters (AcceptNewParams, TDVMC.cpp:2585-2630)
		int trial = 0;
		bool accepted = false;
		while (!accepted && trial < 2) {
			trial++;
			oo.moves_per_stage = o.moves_per_stage * trial;
			rc = tdvmc_step(ctx, &oo, &st);
			if (rc && rc != TDVMC_ERR_NOT_PD && rc != TDVMC_ERR_NONFINITE) return die("tdvmc_step", rc);
			if (!acceptance_check) {
				accepted = true;
				break;
			}
			std::vector<double> nR(P), nI(P);
			double nPR, nPI;
			tdvmc_get_params(ctx, nR.data(), nI.data(), &nPR, &nPI);
			accepted = rc != TDVMC_ERR_NOT_PD;
			if (accepted && check_type >= 1 && histR.size() > 1)
				for (int k = 0; k < P && accepted; k++) {
					if (!std::isfinite(nR[k])) accepted = false;
					else if (check_type == 2 && std::fabs(1.0 - nR[k] / pR[k]) > 0.1) accepted = false;
				}
			if (!accepted) {
				std::fprintf(stderr, "PARAMETERS NOT ACCEPTED (t=%g, trial %d)\n", t, trial);
				tdvmc_set_params(ctx, pR.data(), pI.data(), p0R, p0I);
			}
		}
		// the reference's setback condition: a step that needed its second trial
		// (TDVMC.cpp:3876-3880) rewinds 5 steps (SetBackNSteps, TDVMC.cpp:2746-2784)
		const bool set_back = acceptance_check && trial == 2;
		tdvmc_get_step_operators(ctx, O.data());
		std::vector<double> other(st.other, st.other + 9);
		other.resize(9 + pb_gr, 0.0);
		std::vector<double> parR = pR, parI = pI;
		parR.push_back(p0R);
		parI.push_back(p0I);
		times.push_back(t);
		allER.push_back({st.energy_re});
		allEI.push_back({st.energy_im});
		allO.push_back(O);
		allOther.push_back(other);
		allPR.push_back(parR);
		allPI.push_back(parI);
		if (step % WRITE_NTH == 0) {
			append_line("timesSystem", {t});
			append_line("LocalEnergyR", {st.energy_re});
			append_line("LocalEnergyI", {st.energy_im});
			append_line("LocalOperators", O);
			append_line("OtherExpectationValues", other);
			append_line("ParametersR", parR);
			append_line("ParametersI", parI);
			std::printf("t=%g  E/N=%.10g (kin %.6g, pot %.6g)  acceptance %.1f%%\n", t, st.energy_re / N,
			            st.other[0] / N, st.other[1] / N, 100.0 * st.accept_rate);
			if (file_exists("./stop")) {
				std::printf("Detected stop-file!\n");
				break;
			}
		}
		if (!std::isfinite(st.energy_re)) {
			std::fprintf(stderr, "Energy not finite\n");
			break;
		}
		if (set_back) {
			std::fprintf(stderr, "Parameters not accepted: SetBackNSteps(5) at t=%g\n", t);
			for (int k = 0; k < 5 && !histR.empty() && !times.empty(); k++) {
				t -= TIMESTEP;
				step--;
				times.pop_back();
				allER.pop_back();
				allEI.pop_back();
				allO.pop_back();
				allOther.pop_back();
				allPR.pop_back();
				allPI.pop_back();
				pR = histR.back();
				pI = histI.back();
				p0R = histPR.back();
				p0I = histPI.back();
				histR.pop_back();
				histI.pop_back();
				histPR.pop_back();
				histPI.pop_back();
			}
			if ((rc = tdvmc_set_params(ctx, pR.data(), pI.data(), p0R, p0I))) return die("tdvmc_set_params", rc);
			if ((rc = init_walkers())) return die("walkers after the set-back", rc);
		}
	}
	// the run's series (TDVMC.cpp:3939-3953)
	for (int nth : {1, 100}) {
		const std::string sfx = nth == 1 ? "" : "_every100th";
		write_table("AllLocalEnergyR" + sfx, {"ER"}, allER, nth);
		write_table("AllLocalEnergyI" + sfx, {"EI"}, allEI, nth);
		write_table("AllLocalOperators" + sfx, {"<O_k>", "..."}, allO, nth);
		write_table("AllOtherExpectationValues" + sfx, {"kinetic", "potential", "wf", "g(r)"}, allOther, nth);
		write_table("AllParametersR" + sfx, {"uR_k", "..."}, allPR, nth);
		write_table("AllParametersI" + sfx, {"uI_k", "..."}, allPI, nth);
	}
	std::vector<std::vector<double>> tt;
	for (double t : times) tt.push_back({t});
	write_table("Alltimes", {"t"}, tt);

	// files for successive runs (TDVMC.cpp:4010-4034)
	std::vector<double> xf((size_t)walkers * DIM * N);
	if ((rc = tdvmc_get_walkers(ctx, xf.data(), walkers))) return die("tdvmc_get_walkers", rc);
	mkdir((g_out + "coords").c_str(), 0755);
	for (int k = 0; k < coords_files && k < walkers; k++)
		write_positions(g_out + "coords/particleconfiguration_" + std::to_string(N) + "_" + std::to_string(DIM) + "D_" +
		                    std::to_string(k) + ".dat",
		                xf, k, N, DIM);
	write_positions(g_out + "AAFinish_particleconfiguration_" + std::to_string(N) + "_" + std::to_string(DIM) + "D.dat",
	                xf, 0, N, DIM);
	{
		mkdir((g_out + "random").c_str(), 0755);
		std::ofstream fs(g_out + "random/state_philox.dat");
		fs << seed_base << " " << epoch << "\n";
	}
	{
		std::vector<double> fR(P), fI(P);
		double fPR, fPI;
		tdvmc_get_params(ctx, fR.data(), fI.data(), &fPR, &fPI);
		Json fin = cfg.root;
		fin.obj["PARAMS_REAL"] = json_array(fR);
		fin.obj["PARAMS_IMAGINARY"] = json_array(fI);
		fin.obj["PARAM_PHIR"].kind = Json::NUM;
		fin.obj["PARAM_PHIR"].num = fPR;
		fin.obj["PARAM_PHII"].kind = Json::NUM;
		fin.obj["PARAM_PHII"].num = fPI;
		std::ofstream f(g_out + "AAFinish_tVMC.config");
		f << "{\n";
		size_t i = 0;
		for (auto& kv : fin.obj)
			f << "\t\"" << kv.first << "\" : " << json_text(kv.second) << (++i < fin.obj.size() ? ",\n" : "\n");
		f << "}";
	}
	tdvmc_destroy(ctx);
	return 0;
}
