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
// Extra keys (all optional): GPU_WALKERS (default MC_NSTEPS), GPU_PRECISION
// ("mixed" or "fp64"), POTENTIAL ("square" as BosonsBulk, "gauss", "lj"),
// HBAR2_2M (default 1.0, the reference's constant), GPU_ADJOINT (0/1),
// GPU_SEED.
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

void write_table(const std::string& name, const std::string& header, const std::vector<std::vector<double>>& rows) {
	std::ofstream f(g_out + name + ".dat");
	f.precision(15);
	f << std::scientific;
	f << std::setw(24) << header << "\n";
	for (auto& r : rows) {
		for (double x : r) f << std::setw(24) << x;
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
	if (cfg.str("SYSTEM_TYPE", "BosonsBulk") != "BosonsBulk") {
		std::fprintf(stderr, "only SYSTEM_TYPE BosonsBulk is implemented on the GPU\n");
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
	const uint64_t seed = (uint64_t)cfg.num("GPU_SEED", 1);
	const int ADD_NTH = (int)cfg.num("CALCULATE_ADDITIONAL_DATA_EVERY_NTH_STEP", 0);
	const int ADD_THERM = (int)cfg.num("MC_NADDITIONALTHERMSTEPS", 0);
	const int GR_BINS = (int)cfg.num("GR_BIN_COUNT", 50);
	std::string cfg_dir = argv[1];
	cfg_dir = cfg_dir.find_last_of("\\/") == std::string::npos ? "./" : cfg_dir.substr(0, cfg_dir.find_last_of("\\/")) + "/";

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

	// lattice start with 1/10 jitter per walker (TDVMC.cpp:713-760), one generator per walker
	std::vector<double> x((size_t)walkers * DIM * N);
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
				x[((size_t)w * DIM + a) * N + i] = v;
			}
		}
	}
	if ((rc = tdvmc_set_walkers(ctx, x.data(), walkers))) return die("tdvmc_set_walkers", rc);
	int64_t acc = 0;
	if (MC_VERY_FIRST > 0 && (rc = tdvmc_sample(ctx, MC_VERY_FIRST, MC_STEP, seed, 0xFFFFFFF0u, &acc)))
		return die("tdvmc_sample", rc);

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
		tdvmc_stats st{};
		tdvmc_step_opts oo = o;
		// a non-positive-definite S rejects the step (doNotAcceptStep, TDVMC.cpp:1583-1588,
		// 2588-2591); retry once with twice the sampling effort (TDVMC.cpp:3648-3651)
		for (int trial = 1; trial <= 2; trial++) {
			oo.moves_per_stage = o.moves_per_stage * trial;
			rc = tdvmc_step(ctx, &oo, &st);
			if (rc == TDVMC_OK || !acceptance_check || rc != TDVMC_ERR_NOT_PD) break;
			std::fprintf(stderr, "PARAMETERS NOT ACCEPTED (t=%g), retrying\n", t);
			tdvmc_set_params(ctx, pR.data(), pI.data(), p0R, p0I);
		}
		if (rc && rc != TDVMC_ERR_NOT_PD) return die("tdvmc_step", rc);
		tdvmc_get_step_operators(ctx, O.data());
		std::vector<double> other(st.other, st.other + 9);
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
	}
	write_table("AllLocalEnergyR", "ER", allER);
	write_table("AllLocalEnergyI", "EI", allEI);
	write_table("AllLocalOperators", "<O_k>", allO);
	write_table("AllOtherExpectationValues", "kinetic", allOther);
	write_table("AllParametersR", "uR_k", allPR);
	write_table("AllParametersI", "uI_k", allPI);
	std::vector<std::vector<double>> tt;
	for (double t : times) tt.push_back({t});
	write_table("Alltimes", "t", tt);
	tdvmc_destroy(ctx);
	return 0;
}
