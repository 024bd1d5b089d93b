// Golden-vector harness around the reference implementation.
//
// TEST INFRASTRUCTURE ONLY.  This file is linked against the unmodified
// reference sources (compiled in place by oracle/ref/build_ref.sh, with the
// reference's `main` renamed) and drives the reference's own physics plugin
// `PhysicalSystems::BosonsBulk` (src/PhysicalSystems/BosonsBulk.cpp) and its
// driver routines in src/TDVMC.cpp on fixed inputs, printing the results with
// 17 significant digits.  tests/golden/make_golden.py turns those outputs into
// the committed fixtures that pin oracle/tdvmc_oracle.c.
//
// Commands (whitespace-separated text on stdin):
//   SYSTEM dim n p L nuser [user knots..] nsp [system params..] time
//   SYSTEMPB (same arguments)   -> the same with PhysicalSystems::NUBosonsBulkPB
//   PARAMS uR[p] uI[p] phiR phiI
//   WEIGHTS                      -> knot vector and SplineFactory weights
//   EVAL ncfg [cfg: n*dim]...    -> lnpsi, wf, O[p], E_R, E_I, other[9], LJ sum
//   MOVE ncase [cfg, particle, newpos(dim)]... -> exponent, exponentNew, quotient
//   SOLVE imag precond solver O[p] ER EI OO[p*p] OER[p] OEI[p]
//                                -> uDotR[p] uDotI[p] phiDotR phiDotI rejected
//   SAMPLE seed step nwarm nsamp ntherm nblock [cfg] -> per block averages
//   NIC dim L ncase [ri rj]...   -> |d| and d (generic VectorDisplacementNIC)
//   GRBINS nbins                 -> GR_BIN_COUNT of the next SYSTEM (default 50)
//   ADDITIONAL ncfg [cfg]...     -> g(r) values, S(k) values and the k grid
//                                   (BosonsBulk::CalculateAdditionalSystemProperties)
#include "Constants.h"
#include "SplineFactory.h"
#include "Utils.h"
#include "PhysicalSystems/BosonsBulk.h"
#include "PhysicalSystems/NUBosonsBulkPB.h"
#include "Potentials/LJ.h"
#include "Observables/ObservableVsOnGrid.h"

#include <cstdio>
#include <iostream>
#include <random>
#include <string>
#include <vector>

using namespace std;

// Globals and driver routines defined in the reference's src/TDVMC.cpp.
extern PhysicalSystems::IPhysicalSystem* sys;
extern string configDirectory;
extern int USE_PARAM_START, USE_PARAM_END, USED_PARAM_COUNT;
extern int MC_NSTEPS, MC_NTHERMSTEPS, MC_NINITIALIZATIONSTEPS;
extern int LINEAR_EQUATION_SOLVER_TYPE, USE_PRECONDITIONING, ODE_SOLVER_TYPE;
extern int WRITE_EVERY_NTH_STEP_TO_FILE, MC_NSTEP_MULTIPLICATION_FACTOR_FOR_WRITE_DATA;
extern int UPDATE_SAMPLES_EVERY_NTH_STEP, GR_BIN_COUNT;
extern double MC_STEP;
extern bool isRootRank;
extern bool doNotAcceptStep;
extern long long nAcceptances, nTrials;
extern vector<double> localOperators;
extern double localEnergyR, localEnergyI;
extern vector<vector<double> > localOperatorsMatrix;
extern vector<double> localOperatorlocalEnergyR, localOperatorlocalEnergyI;
extern vector<double> otherExpectationValues;
extern mt19937_64 generator;

void Init();
void PostSystemInit();
void DoMetropolisStep(vector<vector<double> >& R, vector<double>& uR, vector<double>& uI, double phiR, double phiI);
void UpdateExpectationValues(vector<vector<double> >& R, vector<double>& uR, vector<double>& uI, double phiR, double phiI, bool intermediateStep);
void SolveForParametersDot(vector<double>& uDotR, vector<double>& uDotI, double* phiDotR, double* phiDotI);

static int g_grbins = 50;
static vector<double> g_nodes;
static double g_rmax = 0.0;
static vector<double> g_uR, g_uI;
static double g_phiR = 0.0, g_phiI = 0.0;

static void out(double v) { printf("%.17g ", v); }
static void endl_() { printf("\n"); fflush(stdout); }

static vector<vector<double> > read_cfg()
{
	vector<vector<double> > R(N, vector<double>(DIM));
	for (int i = 0; i < N; i++)
		for (int a = 0; a < DIM; a++)
			cin >> R[i][a];
	return R;
}

static void cmd_system(bool pb)
{
	int nuser, nsp;
	double t;
	cin >> DIM >> N >> N_PARAM >> LBOX >> nuser;
	vector<double> user(nuser);
	for (auto& v : user) cin >> v;
	cin >> nsp;
	vector<double> sp(nsp);
	for (auto& v : sp) cin >> v;
	cin >> t;

	USE_PARAM_START = 0;
	USE_PARAM_END = 0;
	MC_NSTEPS = 1;
	MC_NTHERMSTEPS = 1;
	MC_NINITIALIZATIONSTEPS = 0;
	WRITE_EVERY_NTH_STEP_TO_FILE = 1;
	MC_NSTEP_MULTIPLICATION_FACTOR_FOR_WRITE_DATA = 1;
	UPDATE_SAMPLES_EVERY_NTH_STEP = 0;
	GR_BIN_COUNT = g_grbins;
	isRootRank = true;

	if (sys) delete sys;
	if (pb)
	{
		auto* b = new PhysicalSystems::NUBosonsBulkPB(sp, configDirectory);
		if (nuser > 0) b->SetNodes(user);
		b->SetGrBinCount(GR_BIN_COUNT);
		sys = b;
	}
	else
	{
		auto* b = new PhysicalSystems::BosonsBulk(sp, configDirectory);
		if (nuser > 0) b->SetNodes(user);
		b->SetPairDistributionBinCount(GR_BIN_COUNT);
		sys = b;
	}
	Init();
	sys->InitSystem();
	PostSystemInit();
	sys->SetTime(t);

	// Same knot construction as BosonsBulk::InitSystem / SetNodes.
	g_nodes.clear();
	if (nuser > 0)
	{
		g_nodes = user;
		for (int i = 0; i < 3; i++)
		{
			g_nodes.insert(g_nodes.begin(), -user[i + 1]);
			g_nodes.push_back(2.0 * user[user.size() - 1] - user[user.size() - 2 - i]);
		}
	}
	else
	{
		double half = LBOX / 2.0;
		for (int i = -3; i < N_PARAM + 3; i++) g_nodes.push_back((i * half) / ((double)N_PARAM - 1));
	}
	g_rmax = g_nodes[g_nodes.size() - 4];
	g_uR.assign(N_PARAM, 0.0);
	g_uI.assign(N_PARAM, 0.0);
	printf("OK SYSTEM\n");
	fflush(stdout);
}

static void cmd_params()
{
	g_uR.resize(N_PARAM);
	g_uI.resize(N_PARAM);
	for (auto& v : g_uR) cin >> v;
	for (auto& v : g_uI) cin >> v;
	cin >> g_phiR >> g_phiI;
	printf("OK PARAMS\n");
	fflush(stdout);
}

static void cmd_weights()
{
	auto w = SplineFactory::GetWeights(g_nodes);
	printf("NODES %d ", (int)g_nodes.size());
	for (double v : g_nodes) out(v);
	endl_();
	printf("WEIGHTS %d ", (int)w.size());
	for (auto& s : w)
		for (auto& p : s)
			for (double c : p) out(c);
	endl_();
}

static double lj_sum(vector<vector<double> >& R)
{
	Potentials::LJ lj;
	vector<double> d(DIM);
	double v = 0.0;
	for (int n = 0; n < N; n++)
		for (int i = 0; i < n; i++)
		{
			double r = VectorDisplacementNIC_DIM(R[n], R[i], d);
			if (r <= g_rmax) v += lj.GetPotential(r);
		}
	return v;
}

static void cmd_eval()
{
	int ncfg;
	cin >> ncfg;
	for (int c = 0; c < ncfg; c++)
	{
		auto R = read_cfg();
		sys->CalculateWavefunction(R, g_uR, g_uI, g_phiR, g_phiI);
		sys->CalculateExpectationValues(R, g_uR, g_uI, g_phiR, g_phiI);
		printf("EVAL ");
		out(sys->GetExponent());
		out(sys->GetWf());
		for (double v : sys->GetLocalOperators()) out(v);
		out(sys->GetLocalEnergyR());
		out(sys->GetLocalEnergyI());
		for (double v : sys->GetOtherExpectationValues()) out(v);
		out(lj_sum(R));
		endl_();
	}
}

static void cmd_move()
{
	int ncase;
	cin >> ncase;
	for (int c = 0; c < ncase; c++)
	{
		auto R = read_cfg();
		int p;
		cin >> p;
		vector<double> np(DIM);
		for (auto& v : np) cin >> v;
		sys->CalculateWavefunction(R, g_uR, g_uI, g_phiR, g_phiI);
		double e0 = sys->GetExponent();
		vector<double> old = R[p];
		R[p] = np;
		double q = sys->CalculateWFQuotient(R, g_uR, g_uI, g_phiR, g_phiI, p, old);
		printf("MOVE ");
		out(e0);
		out(sys->GetExponentNew());
		out(q);
		endl_();
	}
}

static void cmd_solve()
{
	int imag, precond, solver;
	cin >> imag >> precond >> solver;
	IMAGINARY_TIME = imag;
	USE_PRECONDITIONING = precond;
	LINEAR_EQUATION_SOLVER_TYPE = solver;
	USED_PARAM_COUNT = N_PARAM;
	localOperators.assign(N_PARAM, 0.0);
	localOperatorsMatrix.assign(N_PARAM, vector<double>(N_PARAM, 0.0));
	localOperatorlocalEnergyR.assign(N_PARAM, 0.0);
	localOperatorlocalEnergyI.assign(N_PARAM, 0.0);
	for (auto& v : localOperators) cin >> v;
	cin >> localEnergyR >> localEnergyI;
	for (auto& row : localOperatorsMatrix)
		for (auto& v : row) cin >> v;
	for (auto& v : localOperatorlocalEnergyR) cin >> v;
	for (auto& v : localOperatorlocalEnergyI) cin >> v;
	doNotAcceptStep = false;
	vector<double> dR, dI;
	double pR = 0.0, pI = 0.0;
	SolveForParametersDot(dR, dI, &pR, &pI);
	printf("SOLVE ");
	for (double v : dR) out(v);
	for (double v : dI) out(v);
	out(pR);
	out(pI);
	out(doNotAcceptStep ? 1.0 : 0.0);
	endl_();
	doNotAcceptStep = false;
}

static void cmd_sample()
{
	unsigned long long seed;
	int nwarm, nsamp, ntherm, nblock;
	cin >> seed >> MC_STEP >> nwarm >> nsamp >> ntherm >> nblock;
	auto R = read_cfg();
	generator = mt19937_64(seed);
	MC_NSTEPS = nsamp;
	MC_NTHERMSTEPS = ntherm;
	MC_NINITIALIZATIONSTEPS = 0;
	sys->CalculateWavefunction(R, g_uR, g_uI, g_phiR, g_phiI);
	for (int i = 0; i < nwarm; i++) DoMetropolisStep(R, g_uR, g_uI, g_phiR, g_phiI);
	for (int b = 0; b < nblock; b++)
	{
		nAcceptances = 0;
		nTrials = 0;
		UpdateExpectationValues(R, g_uR, g_uI, g_phiR, g_phiI, true);
		printf("BLOCK ");
		out((double)nAcceptances / (double)nTrials);
		out(localEnergyR);
		out(localEnergyI);
		for (double v : localOperators) out(v);
		for (double v : otherExpectationValues) out(v);
		endl_();
	}
}

static void cmd_nic()
{
	int dim, ncase;
	double L;
	cin >> dim >> L >> ncase;
	LBOX = L;
	LBOX_R = 1.0 / LBOX;
	LBOX_2 = LBOX / 2.0;
	for (int c = 0; c < ncase; c++)
	{
		vector<double> ri(dim), rj(dim), d(dim);
		for (auto& v : ri) cin >> v;
		for (auto& v : rj) cin >> v;
		double r = VectorDisplacementNIC(ri, rj, d);
		printf("NIC ");
		out(r);
		for (double v : d) out(v);
		endl_();
	}
}

static void cmd_additional()
{
	int ncfg;
	cin >> ncfg;
	for (int c = 0; c < ncfg; c++)
	{
		auto R = read_cfg();
		sys->CalculateAdditionalSystemProperties(R, g_uR, g_uI, g_phiR, g_phiI);
		auto oc = sys->GetAdditionalObservablesClone();
		printf("ADD ");
		for (int o = 0; o < 2; o++)
		{
			auto* g = dynamic_cast<Observables::ObservableVsOnGrid*>(oc.observables[o]);
			const vector<double>& v = g->observablesV[0].values;
			printf("%d ", (int)v.size());
			for (double x : v) out(x);
		}
		auto* k = dynamic_cast<Observables::ObservableVsOnGrid*>(oc.observables[1]);
		printf("%d ", (int)k->grid.grid.size());
		for (double x : k->grid.grid) out(x);
		endl_();
		oc.Destroy();
	}
}

// the reference's own entry point (src/TDVMC.cpp main, renamed by build_ref.sh)
int tdvmc_reference_main(int argc, char** argv);

int main(int argc, char** argv)
{
	// "--run <config file>": the reference's full program on that config (its time
	// loop and output files), as main(argc = 2) runs it (TDVMC.cpp:4307 ff.)
	if (argc > 2 && string(argv[1]) == "--run")
	{
		char* args[2] = {argv[0], argv[2]};
		return tdvmc_reference_main(2, args);
	}
	configDirectory = argc > 1 ? string(argv[1]) : string("./");
	OUT_DIR = "./";
	string cmd;
	while (cin >> cmd)
	{
		if (cmd == "SYSTEM") cmd_system(false);
		else if (cmd == "SYSTEMPB") cmd_system(true);
		else if (cmd == "PARAMS") cmd_params();
		else if (cmd == "WEIGHTS") cmd_weights();
		else if (cmd == "EVAL") cmd_eval();
		else if (cmd == "MOVE") cmd_move();
		else if (cmd == "SOLVE") cmd_solve();
		else if (cmd == "SAMPLE") cmd_sample();
		else if (cmd == "NIC") cmd_nic();
		else if (cmd == "GRBINS") cin >> g_grbins;
		else if (cmd == "ADDITIONAL") cmd_additional();
		else
		{
			fprintf(stderr, "unknown command %s\n", cmd.c_str());
			return 2;
		}
	}
	return 0;
}
