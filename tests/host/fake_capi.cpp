// A CPU stand-in for the C ABI of include/tdvmc_gpu.h, for testing the host
// driver's control logic (tdvmc_run) without a GPU.  Only the calls the
// driver makes are implemented.  Scripted behaviour:
//   every tdvmc_step call k (k = 1, 2, ...) adds k * dt to every uR and sets
//   the energy to k; FAKE_NOT_PD="k1,k2,..." makes those calls return
//   TDVMC_ERR_NOT_PD; FAKE_BIG="k,..." makes those calls change uR by a
//   factor 2 (a change above the 10 % of acceptance check type 2).
// Each call appends one line to $FAKE_LOG.
#include "tdvmc_gpu.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <sstream>
#include <string>
#include <vector>

struct tdvmc_ctx {
	int n = 0, dim = 0, p = 0;
	int64_t nw = 0;
	std::vector<double> uR, uI, x;
	double phiR = 0, phiI = 0;
	int calls = 0;
};

static std::set<int> parse(const char* env) {
	std::set<int> s;
	const char* v = std::getenv(env);
	if (!v) return s;
	std::stringstream ss(v);
	std::string tok;
	while (std::getline(ss, tok, ',')) s.insert(std::atoi(tok.c_str()));
	return s;
}

static void logf(const char* fmt, double a = 0, double b = 0) {
	const char* path = std::getenv("FAKE_LOG");
	if (!path) return;
	FILE* f = std::fopen(path, "a");
	if (!f) return;
	std::fprintf(f, fmt, a, b);
	std::fputc('\n', f);
	std::fclose(f);
}

extern "C" {

const char* tdvmc_status_string(int s) { return s == 0 ? "ok" : "error"; }

int tdvmc_create(const tdvmc_system_desc* d, tdvmc_ctx** out) {
	tdvmc_ctx* c = new tdvmc_ctx();
	c->n = d->n;
	c->dim = d->dim;
	c->p = d->p;
	c->nw = d->n_walkers;
	c->uR.assign(c->p, 0.0);
	c->uI.assign(c->p, 0.0);
	*out = c;
	logf("create system %.0f pot %.0f", d->system_type, d->pot_kind);
	return 0;
}

int tdvmc_destroy(tdvmc_ctx* c) {
	delete c;
	return 0;
}

int tdvmc_set_time(tdvmc_ctx*, double t) {
	logf("time %.6f", t);
	return 0;
}

int tdvmc_set_params(tdvmc_ctx* c, const double* uR, const double* uI, double phiR, double phiI) {
	c->uR.assign(uR, uR + c->p);
	c->uI.assign(uI, uI + c->p);
	c->phiR = phiR;
	c->phiI = phiI;
	logf("set_params %.6f", uR[0]);
	return 0;
}

int tdvmc_get_params(tdvmc_ctx* c, double* uR, double* uI, double* phiR, double* phiI) {
	std::memcpy(uR, c->uR.data(), c->p * sizeof(double));
	std::memcpy(uI, c->uI.data(), c->p * sizeof(double));
	*phiR = c->phiR;
	*phiI = c->phiI;
	return 0;
}

int tdvmc_set_walkers(tdvmc_ctx* c, const double* x, int64_t nw) {
	c->x.assign(x, x + (size_t)nw * c->dim * c->n);
	logf("set_walkers %.6f", x[0]);
	return 0;
}

int tdvmc_get_walkers(tdvmc_ctx* c, double* x, int64_t nw) {
	std::memcpy(x, c->x.data(), (size_t)nw * c->dim * c->n * sizeof(double));
	return 0;
}

int tdvmc_sample(tdvmc_ctx*, int32_t moves, double, uint64_t seed, uint32_t, int64_t* accepted) {
	if (accepted) *accepted = 0;
	logf("sample %.0f seed %.0f", moves, (double)seed);
	return 0;
}

int tdvmc_observables(tdvmc_ctx*, int32_t, int32_t, const int32_t*, const double*, double*, int32_t* cnt, double*) {
	*cnt = 0;
	return 0;
}

int tdvmc_step(tdvmc_ctx* c, const tdvmc_step_opts* o, tdvmc_stats* st) {
	c->calls++;
	const int k = c->calls;
	const bool big = parse("FAKE_BIG").count(k) > 0;
	for (int i = 0; i < c->p; i++) c->uR[i] = big ? 2.0 * c->uR[i] : c->uR[i] + k * o->dt;
	std::memset(st, 0, sizeof(*st));
	st->energy_re = k;
	st->n_walkers = c->nw;
	logf("step %.0f moves %.0f", k, o->moves_per_stage);
	return parse("FAKE_NOT_PD").count(k) ? TDVMC_ERR_NOT_PD : TDVMC_OK;
}

int tdvmc_get_step_operators(tdvmc_ctx* c, double* O) {
	for (int i = 0; i < c->p; i++) O[i] = 0.0;
	return 0;
}

}  // extern "C"
