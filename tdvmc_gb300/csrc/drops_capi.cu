// C ABI of the batched trapped drops (declarations in include/tdvmc_gpu.h):
// context, device tables, persistent work queues, per-drop reductions and
// solves, CUDA-graph capture of the RK stages.
#include "../../include/tdvmc_gpu.h"

#include "common.cuh"
#include "k_drops.cuh"
#include "k_solve.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>

using namespace tdvmc;

namespace {

struct DropGraphKey {
	double dt, mc_step;
	int imag, ode, lin, pre, norm, moves, adj;
	uint64_t seed;
	int ts, te;
	bool operator<(const DropGraphKey& o) const {
		return std::tie(dt, mc_step, imag, ode, lin, pre, norm, moves, adj, seed, ts, te) <
		       std::tie(o.dt, o.mc_step, o.imag, o.ode, o.lin, o.pre, o.norm, o.moves, o.adj, o.seed, o.ts, o.te);
	}
};

// local B-spline pieces of a uniform knot vector [q][c]: spline j+3-q on interval
// j in t = (r - k_{j+3}) / h, the same for every interval (Cox-de Boor, as
// piece_local of the bulk context for equal widths)
void uniform_pieces(double* loc) {
	const double L[4][4] = {{0.0, 0.0, 0.0, 1.0 / 6.0},
	                        {1.0 / 6.0, 0.5, 0.5, -0.5},
	                        {4.0 / 6.0, 0.0, -1.0, 0.5},
	                        {1.0 / 6.0, -0.5, 0.5, -1.0 / 6.0}};
	for (int q = 0; q < 4; q++)
		for (int c = 0; c < 4; c++) loc[q * 4 + c] = L[q][c];
}

}  // namespace

struct tdvmc_drops {
	int prec = TDVMC_PREC_FP64;
	int S = 0;  // drops
	int p = 0, p1 = 0, ns = 0, np = 0;
	int64_t nws = 0;
	int nmax = 0;
	int device = 0, nsm = 0;
	cudaStream_t st = nullptr;
	std::vector<int> n;
	std::vector<int64_t> pos_off;
	int64_t total_coords = 0;
	DropConst dc{};
	int tpb_s = 128, tpb_e = 64;  // threads (walkers) per block of the sampler and the evaluation
	// device
	DropSys* sys = nullptr;
	int4 *items_s = nullptr, *items_e = nullptr;
	int nitems_s = 0, nitems_e = 0;
	int* counters = nullptr;  // [0] sampler, [1] evaluation
	void *pos = nullptr, *lnpsi = nullptr, *O = nullptr, *eloc = nullptr, *other7 = nullptr, *dE = nullptr;
	int* acc = nullptr;
	double *base = nullptr, *stage = nullptr, *kdot = nullptr, *rhs = nullptr;
	double *fold_d = nullptr, *loc_d = nullptr;
	void *coefU = nullptr, *coefC = nullptr;
	DynState* dyn = nullptr;
	double *means = nullptr, *means0 = nullptr, *Sm = nullptr, *cov = nullptr;
	bool have_walkers = false, have_eval = false, last_adj = false;
	int64_t launches = 0;
	std::map<DropGraphKey, cudaGraphExec_t> graphs;
	std::map<DropGraphKey, int> graph_kernels;
	std::vector<cudaEvent_t>* prof = nullptr;
	std::vector<const char*>* prof_names = nullptr;
	std::string err;
};

namespace {

#define DK(call)                                                                         \
	do {                                                                                 \
		cudaError_t e_ = (call);                                                         \
		if (e_ != cudaSuccess) {                                                         \
			if (ctx) ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);      \
			return TDVMC_ERR_CUDA;                                                       \
		}                                                                                \
	} while (0)

size_t tsz(const tdvmc_drops* c) { return c->prec == TDVMC_PREC_FP64 ? sizeof(double) : sizeof(float); }

void dmark(tdvmc_drops* ctx, const char* name) {
	if (!ctx->prof) return;
	cudaEvent_t e;
	cudaEventCreate(&e);
	cudaEventRecord(e, ctx->st);
	ctx->prof->push_back(e);
	ctx->prof_names->push_back(name);
}

// work items (drop, first walker, count) of `tpb` walkers, drops with more
// particles first (their walkers cost ~n^2)
std::vector<int4> make_items(const tdvmc_drops* c, int tpb) {
	std::vector<int> order(c->S);
	std::iota(order.begin(), order.end(), 0);
	std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return c->n[a] > c->n[b]; });
	std::vector<int4> it;
	for (int s : order)
		for (int64_t w = 0; w < c->nws; w += tpb)
			it.push_back(make_int4(s, (int)w, (int)std::min<int64_t>(tpb, c->nws - w), 0));
	return it;
}

int set_items(tdvmc_drops* ctx, int tpb_s, int tpb_e) {
	std::vector<int4> a = make_items(ctx, tpb_s), b = make_items(ctx, tpb_e);
	if (ctx->items_s) cudaFree(ctx->items_s);
	if (ctx->items_e) cudaFree(ctx->items_e);
	ctx->items_s = ctx->items_e = nullptr;
	DK(cudaMalloc(&ctx->items_s, a.size() * sizeof(int4)));
	DK(cudaMalloc(&ctx->items_e, b.size() * sizeof(int4)));
	DK(cudaMemcpy(ctx->items_s, a.data(), a.size() * sizeof(int4), cudaMemcpyHostToDevice));
	DK(cudaMemcpy(ctx->items_e, b.data(), b.size() * sizeof(int4), cudaMemcpyHostToDevice));
	ctx->nitems_s = (int)a.size();
	ctx->nitems_e = (int)b.size();
	ctx->tpb_s = tpb_s;
	ctx->tpb_e = tpb_e;
	for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
	ctx->graphs.clear();
	ctx->graph_kernels.clear();
	return TDVMC_OK;
}

// persistent grid: resident blocks per SM x SMs, at most one block per item
int pgrid(tdvmc_drops* ctx, const void* fn, int threads, size_t smem, int nitems) {
	int per_sm = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
	if (per_sm < 1) per_sm = 1;
	return std::max(1, std::min(nitems, per_sm * ctx->nsm));
}

template <typename T>
int dl_prep(tdvmc_drops* ctx) {
	k_drop_prep<T><<<ctx->S, 128, 0, ctx->st>>>(ctx->dc, ctx->sys, ctx->stage, ctx->fold_d, ctx->loc_d,
	                                              (T*)ctx->coefU, (T*)ctx->coefC);
	ctx->launches++;
	dmark(ctx, "k_drop_prep");
	DK(cudaGetLastError());
	return TDVMC_OK;
}

template <typename T>
int dl_sample(tdvmc_drops* ctx, int moves_pp, double step, uint64_t seed) {
	const int B = ctx->tpb_s;
	const size_t smem = (size_t)ctx->dc.ncoef * sizeof(Q4<T>) + (size_t)3 * ctx->nmax * B * sizeof(T);
	const void* fn = (const void*)k_drop_sample<T>;
	DK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	DK(cudaMemsetAsync(ctx->counters, 0, sizeof(int), ctx->st));
	const int grid = pgrid(ctx, fn, B, smem, ctx->nitems_s);
	const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
	k_drop_sample<T><<<grid, B, smem, ctx->st>>>(ctx->dc, ctx->sys, ctx->items_s, ctx->nitems_s, ctx->counters,
	                                             (const T*)ctx->coefU, ctx->stage, (T*)ctx->pos, moves_pp, (T)step, key,
	                                             ctx->dyn, ctx->nmax, ctx->acc);
	ctx->launches++;
	dmark(ctx, "k_drop_sample");
	DK(cudaGetLastError());
	return TDVMC_OK;
}

constexpr size_t kDropSmemMax = 227 * 1024;

// shared memory of the evaluation kernel with B threads
size_t eval_smem(const tdvmc_drops* ctx, int B, bool adj) {
	const size_t t = tsz(ctx);
	return (size_t)3 * ctx->dc.nbin_max * 4 * t + (size_t)drop_eval_rows(ctx->nmax, ctx->ns, adj) * B * t;
}

template <typename T>
int dl_eval(tdvmc_drops* ctx, bool adj) {
	const int B = ctx->tpb_e;
	const size_t smem = eval_smem(ctx, B, adj);
	if (smem > kDropSmemMax) return TDVMC_ERR_ARG;
	const void* fn = adj ? (const void*)k_drop_eval<T, true> : (const void*)k_drop_eval<T, false>;
	DK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	DK(cudaMemsetAsync(ctx->counters + 1, 0, sizeof(int), ctx->st));
	const int grid = pgrid(ctx, fn, B, smem, ctx->nitems_e);
	if (adj)
		k_drop_eval<T, true><<<grid, B, smem, ctx->st>>>(ctx->dc, ctx->sys, ctx->items_e, ctx->nitems_e,
		                                                 ctx->counters + 1, (const T*)ctx->coefC, ctx->stage,
		                                                 ctx->fold_d, ctx->loc_d, (const T*)ctx->pos, ctx->nmax,
		                                                 (T*)ctx->lnpsi, (T*)ctx->O, (T*)ctx->eloc, (T*)ctx->other7,
		                                                 (T*)ctx->dE);
	else
		k_drop_eval<T, false><<<grid, B, smem, ctx->st>>>(ctx->dc, ctx->sys, ctx->items_e, ctx->nitems_e,
		                                                  ctx->counters + 1, (const T*)ctx->coefC, ctx->stage,
		                                                  ctx->fold_d, ctx->loc_d, (const T*)ctx->pos, ctx->nmax,
		                                                  (T*)ctx->lnpsi, (T*)ctx->O, (T*)ctx->eloc, (T*)ctx->other7,
		                                                  (T*)ctx->dE);
	ctx->launches++;
	dmark(ctx, "k_drop_eval");
	DK(cudaGetLastError());
	return TDVMC_OK;
}

template <typename T>
int dl_reduce(tdvmc_drops* ctx, bool adj) {
	// the staged chunk: kDropRedStage walkers x the column count
	const size_t smem = (size_t)kDropRedStage * DropCols{ctx->p1}.count() * sizeof(T);
	DK(cudaFuncSetAttribute((const void*)k_drop_reduce<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	k_drop_reduce<T><<<ctx->S, kDropReduceThreads, smem, ctx->st>>>(ctx->dc, (const T*)ctx->O, (const T*)ctx->eloc,
	                                                              (const T*)ctx->other7, ctx->acc, (const T*)ctx->dE,
	                                                              adj ? 1 : 0, ctx->means, ctx->Sm, ctx->cov);
	ctx->launches++;
	dmark(ctx, "k_drop_reduce");
	DK(cudaGetLastError());
	return TDVMC_OK;
}

template <typename T>
int dl_solve(tdvmc_drops* ctx, int imag, int pre, int lin, int mode, int norm, double dt, int adj_force) {
	SolveArgs a;
	a.p = ctx->p1;
	a.imag = imag;
	a.precond = pre;
	a.solver = lin;
	a.mode = mode;
	a.normalize = norm;
	a.ldS = ctx->p1;
	a.ldC = 2;
	a.adj_force = adj_force;
	a.dE_col = DropCols{ctx->p1}.dE();
	a.dt = dt;
	const size_t smem = solve_smem_bytes(ctx->p1);
	DK(cudaFuncSetAttribute((const void*)k_solve_systems<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	k_solve_systems<T><<<ctx->S, 256, smem, ctx->st>>>(a, ctx->dyn, ctx->means, ctx->Sm, ctx->cov, (const T*)ctx->lnpsi,
	                                                   ctx->nws, ctx->base, ctx->stage, ctx->kdot, ctx->rhs,
	                                                   ctx->means0, DropCols{ctx->p1}.count());
	ctx->launches++;
	dmark(ctx, "k_solve_systems");
	DK(cudaGetLastError());
	return TDVMC_OK;
}

template <typename T>
int dl_stage(tdvmc_drops* ctx, const tdvmc_step_opts* o) {
	int rc;
	const bool adj = o->use_adjoint != 0;
	if ((rc = dl_prep<T>(ctx))) return rc;
	if (o->moves_per_stage > 0 && (rc = dl_sample<T>(ctx, o->moves_per_stage, o->mc_step, o->seed))) return rc;
	if ((rc = dl_eval<T>(ctx, adj))) return rc;
	if ((rc = dl_reduce<T>(ctx, adj))) return rc;
	return dl_solve<T>(ctx, o->imaginary_time, o->precondition, o->lin_solver, o->ode_solver == 0 ? 2 : 1,
	                   o->normalize_wf, o->dt, (o->use_adjoint == 2 && o->imaginary_time) ? 1 : 0);
}

int dl_stage_any(tdvmc_drops* ctx, const tdvmc_step_opts* o) {
	return ctx->prec == TDVMC_PREC_FP64 ? dl_stage<double>(ctx, o) : dl_stage<float>(ctx, o);
}

int check_drop_opts(const tdvmc_step_opts* o) {
	if (!o || !(o->dt > 0) || o->moves_per_stage < 0 || !(o->mc_step >= 0)) return TDVMC_ERR_ARG;
	if (o->ode_solver != 0 && o->ode_solver != 2) return TDVMC_ERR_ARG;
	if (o->lin_solver != 0 && o->lin_solver != 1) return TDVMC_ERR_ARG;
	return TDVMC_OK;
}

int drop_graph(tdvmc_drops* ctx, const tdvmc_step_opts* o, cudaGraphExec_t* out, int* kernels) {
	DropGraphKey k{o->dt, o->mc_step, o->imaginary_time, o->ode_solver, o->lin_solver, o->precondition,
	               o->normalize_wf, o->moves_per_stage, o->use_adjoint, o->seed, ctx->tpb_s, ctx->tpb_e};
	auto it = ctx->graphs.find(k);
	if (it != ctx->graphs.end()) {
		*out = it->second;
		*kernels = ctx->graph_kernels[k];
		return TDVMC_OK;
	}
	cudaGraph_t g;
	DK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
	const int64_t l0 = ctx->launches;
	const int rc = dl_stage_any(ctx, o);
	const cudaError_t e = cudaStreamEndCapture(ctx->st, &g);
	const int nk = (int)(ctx->launches - l0);
	ctx->launches = l0;
	if (rc) return rc;
	if (e != cudaSuccess) {
		ctx->err = cudaGetErrorString(e);
		return TDVMC_ERR_CUDA;
	}
	cudaGraphExec_t ex;
	DK(cudaGraphInstantiate(&ex, g, 0));
	cudaGraphDestroy(g);
	ctx->graphs[k] = ex;
	ctx->graph_kernels[k] = nk;
	*out = ex;
	*kernels = nk;
	return TDVMC_OK;
}

int drop_enqueue(tdvmc_drops* ctx, const tdvmc_step_opts* o, int nsteps) {
	cudaGraphExec_t g;
	int nk = 0, rc;
	if ((rc = drop_graph(ctx, o, &g, &nk))) return rc;
	const int nst = o->ode_solver == 0 ? 1 : 4;
	for (int s = 0; s < nsteps; s++)
		for (int k = 0; k < nst; k++) {
			DK(cudaGraphLaunch(g, ctx->st));
			ctx->launches += nk;
		}
	return TDVMC_OK;
}

int drop_status(tdvmc_drops* ctx, int32_t* status) {
	std::vector<DynState> d(ctx->S);
	DK(cudaMemcpyAsync(d.data(), ctx->dyn, d.size() * sizeof(DynState), cudaMemcpyDeviceToHost, ctx->st));
	DK(cudaStreamSynchronize(ctx->st));
	int any = 0;
	for (int s = 0; s < ctx->S; s++) {
		const int v = d[s].status;
		if (status) status[s] = (v & kStatusNonFinite) ? TDVMC_ERR_NONFINITE : (v & kStatusNotPD) ? TDVMC_ERR_NOT_PD : 0;
		any |= v;
		d[s].status = 0;
	}
	DK(cudaMemcpyAsync(ctx->dyn, d.data(), d.size() * sizeof(DynState), cudaMemcpyHostToDevice, ctx->st));
	DK(cudaStreamSynchronize(ctx->st));
	return (any & kStatusNonFinite) ? TDVMC_ERR_NONFINITE : (any & kStatusNotPD) ? TDVMC_ERR_NOT_PD : TDVMC_OK;
}

template <typename T>
int dcopy_out(tdvmc_drops* ctx, const void* d, double* h, size_t count) {
	if (!h) return TDVMC_OK;
	std::vector<T> tmp(count);
	DK(cudaMemcpyAsync(tmp.data(), d, count * sizeof(T), cudaMemcpyDeviceToHost, ctx->st));
	DK(cudaStreamSynchronize(ctx->st));
	for (size_t i = 0; i < count; i++) h[i] = (double)tmp[i];
	return TDVMC_OK;
}
int dcopy_any(tdvmc_drops* ctx, const void* d, double* h, size_t count) {
	return ctx->prec == TDVMC_PREC_FP64 ? dcopy_out<double>(ctx, d, h, count) : dcopy_out<float>(ctx, d, h, count);
}

void free_all(tdvmc_drops* c) {
	for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
	void* bufs[] = {c->sys, c->items_s, c->items_e, c->counters, c->pos, c->lnpsi, c->O, c->eloc, c->other7,
	                c->dE, c->acc, c->base, c->stage, c->kdot, c->rhs, c->fold_d, c->loc_d, c->coefU, c->coefC,
	                c->dyn, c->means, c->means0, c->Sm, c->cov};
	for (void* b : bufs)
		if (b) cudaFree(b);
	if (c->st) cudaStreamDestroy(c->st);
}

}  // namespace

extern "C" {

int tdvmc_drops_create(const tdvmc_drops_desc* d, tdvmc_drops** out) {
	if (!d || !out) return TDVMC_ERR_ARG;
	*out = nullptr;
	if (d->n_systems < 1 || !d->n || !d->rmax || d->p < 4 || d->p > kDropMaxP || d->walkers_per_system < 1 ||
	    d->walkers_per_system > 0x7fffffffLL / d->n_systems || !(d->hbar2_2m > 0) || !(d->sigma > 0) ||
	    (d->precision != TDVMC_PREC_FP64 && d->precision != TDVMC_PREC_MIXED))
		return TDVMC_ERR_ARG;
	for (int s = 0; s < d->n_systems; s++)
		if (d->n[s] < 2 || d->n[s] > kDropMaxN || !(d->rmax[s] > 0)) return TDVMC_ERR_ARG;
	tdvmc_drops* ctx = new tdvmc_drops();
	tdvmc_drops& c = *ctx;
	c.prec = d->precision;
	c.S = d->n_systems;
	c.p = d->p;
	c.p1 = d->p + 1;
	c.ns = d->p + 2;
	c.np = 2 * c.p1 + 2;
	c.nws = d->walkers_per_system;
	c.n.assign(d->n, d->n + c.S);
	c.nmax = *std::max_element(c.n.begin(), c.n.end());
	std::vector<DropSys> sys(c.S);
	int64_t off = 0;
	for (int s = 0; s < c.S; s++) {
		DropSys& y = sys[s];
		y.n = c.n[s];
		y.nbin = c.p - 1;
		y.rmax = d->rmax[s];
		y.hinv = (double)(c.p - 1) / d->rmax[s];
		y.hf = (float)y.hinv;
		y.hf_lo = (float)(y.hinv - (double)y.hf);
		y.rcut_lo = (float)(y.rmax * (1.0 - 4e-6));
		y.rcut_hi = (float)(y.rmax * (1.0 + 4e-6));
		y.pos_off = off;
		c.pos_off.push_back(off);
		off += c.nws * 3 * y.n;
	}
	c.total_coords = off;
	DropConst& k = c.dc;
	k.p = c.p;
	k.p1 = c.p1;
	k.ns = c.ns;
	k.np = c.np;
	k.ncoef = c.p;  // nbin + 1
	k.nbin_max = c.p - 1;
	k.nws = c.nws;
	k.v0 = d->v0;
	k.inv2s2 = 1.0 / (2.0 * d->sigma * d->sigma);
	k.kappa = d->omega * d->omega / (4.0 * d->hbar2_2m);
	k.hbar2_2m = d->hbar2_2m;

	cudaGetDevice(&c.device);
	cudaDeviceGetAttribute(&c.nsm, cudaDevAttrMultiProcessorCount, c.device);
	if (cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking) != cudaSuccess) {
		free_all(ctx);
		delete ctx;
		return TDVMC_ERR_CUDA;
	}
	const size_t ts = tsz(ctx);
	const int64_t nwt = (int64_t)c.S * c.nws;
	const int K = DropCols{c.p1}.count();
	bool ok = true;
	auto A = [&](void** p, size_t bytes) {
		if (!ok) return;
		if (cudaMalloc(p, bytes) != cudaSuccess) ok = false;
	};
	A((void**)&c.sys, c.S * sizeof(DropSys));
	A((void**)&c.counters, 2 * sizeof(int));
	A(&c.pos, (size_t)c.total_coords * ts);
	A(&c.lnpsi, (size_t)nwt * ts);
	A(&c.O, (size_t)nwt * c.p1 * ts);
	A(&c.eloc, (size_t)nwt * 2 * ts);
	A(&c.other7, (size_t)nwt * 7 * ts);
	A(&c.dE, (size_t)nwt * 2 * c.p1 * ts);
	A((void**)&c.acc, (size_t)nwt * sizeof(int));
	A((void**)&c.base, (size_t)c.S * c.np * sizeof(double));
	A((void**)&c.stage, (size_t)c.S * c.np * sizeof(double));
	A((void**)&c.kdot, (size_t)c.S * 4 * c.np * sizeof(double));
	A((void**)&c.rhs, (size_t)c.S * c.np * sizeof(double));
	A((void**)&c.fold_d, (size_t)c.p * c.ns * sizeof(double));
	A((void**)&c.loc_d, 16 * sizeof(double));
	A(&c.coefU, (size_t)c.S * k.ncoef * 4 * ts);
	A(&c.coefC, (size_t)c.S * k.nbin_max * 12 * ts);
	A((void**)&c.dyn, (size_t)c.S * sizeof(DynState));
	A((void**)&c.means, (size_t)c.S * K * sizeof(double));
	A((void**)&c.means0, (size_t)c.S * K * sizeof(double));
	A((void**)&c.Sm, (size_t)c.S * c.p1 * c.p1 * sizeof(double));
	A((void**)&c.cov, (size_t)c.S * c.p1 * 2 * sizeof(double));
	if (!ok) {
		free_all(ctx);
		delete ctx;
		return TDVMC_ERR_NOMEM;
	}
	// boundary-condition fold of the pair spline (uniform factors, as the bulk system:
	// SplineFactory.cpp:423-439, 563-579)
	std::vector<double> fold((size_t)c.p * c.ns, 0.0);
	const double bcs[2][3] = {{0, 1, 0}, {1, 0, 1}};
	const double bce[2][3] = {{1, 0, 1}, {0, 1, 0}};
	for (int i = 0; i < 2; i++)
		for (int j = 0; j < 3; j++) fold[(size_t)i * c.ns + j] = bcs[i][j];
	for (int i = 2, sp = 3; i < c.p - 2; i++, sp++) fold[(size_t)i * c.ns + sp] = 1.0;
	for (int i = c.p - 2, idx = 0; i < c.p; i++, idx++)
		for (int j = 0; j < 3; j++) fold[(size_t)i * c.ns + c.ns - 3 + j] = bce[idx][j];
	double loc[16];
	uniform_pieces(loc);
	std::vector<DynState> dy(c.S);
	for (auto& v : dy) {
		v.pa = v.pb = 0.0;
		v.pass = 0;
		v.stage = 0;
		v.status = 0;
		v.cs_start = 0;
	}
	std::vector<double> zeros((size_t)c.S * 4 * c.np, 0.0);
	const bool cp =
	    cudaMemcpy(c.sys, sys.data(), sys.size() * sizeof(DropSys), cudaMemcpyHostToDevice) == cudaSuccess &&
	    cudaMemcpy(c.fold_d, fold.data(), fold.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
	    cudaMemcpy(c.loc_d, loc, sizeof(loc), cudaMemcpyHostToDevice) == cudaSuccess &&
	    cudaMemcpy(c.dyn, dy.data(), dy.size() * sizeof(DynState), cudaMemcpyHostToDevice) == cudaSuccess &&
	    cudaMemcpy(c.base, zeros.data(), (size_t)c.S * c.np * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
	    cudaMemcpy(c.stage, zeros.data(), (size_t)c.S * c.np * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
	    cudaMemcpy(c.kdot, zeros.data(), zeros.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
	    cudaMemset(c.acc, 0, (size_t)nwt * sizeof(int)) == cudaSuccess &&
	    cudaMemset(c.dE, 0, (size_t)nwt * 2 * c.p1 * ts) == cudaSuccess;
	if (!cp) {
		free_all(ctx);
		delete ctx;
		return TDVMC_ERR_CUDA;
	}
	// default tiles: 128 walkers per sampler block; the evaluation takes 64 where its
	// shared-memory rows fit, else 32
	const int rc = set_items(ctx, 128, eval_smem(ctx, 64, true) <= kDropSmemMax ? 64 : 32);
	if (rc) {
		free_all(ctx);
		delete ctx;
		return rc;
	}
	*out = ctx;
	return TDVMC_OK;
}

int tdvmc_drops_destroy(tdvmc_drops* ctx) {
	if (!ctx) return TDVMC_ERR_ARG;
	cudaStreamSynchronize(ctx->st);
	free_all(ctx);
	delete ctx;
	return TDVMC_OK;
}

int tdvmc_drops_get_stream(tdvmc_drops* ctx, void** stream) {
	if (!ctx || !stream) return TDVMC_ERR_ARG;
	*stream = (void*)ctx->st;
	return TDVMC_OK;
}

int tdvmc_drops_set_params(tdvmc_drops* ctx, const double* uR, const double* uI, const double* phiR,
                           const double* phiI) {
	if (!ctx || !uR || !uI) return TDVMC_ERR_ARG;
	std::vector<double> v((size_t)ctx->S * ctx->np, 0.0);
	for (int s = 0; s < ctx->S; s++) {
		double* q = &v[(size_t)s * ctx->np];
		for (int k = 0; k < ctx->p1; k++) {
			q[k] = uR[(size_t)s * ctx->p1 + k];
			q[ctx->p1 + k] = uI[(size_t)s * ctx->p1 + k];
		}
		q[2 * ctx->p1] = phiR ? phiR[s] : 0.0;
		q[2 * ctx->p1 + 1] = phiI ? phiI[s] : 0.0;
		for (int k = 0; k < ctx->np; k++)
			if (!std::isfinite(q[k])) return TDVMC_ERR_ARG;
	}
	DK(cudaMemcpyAsync(ctx->base, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
	DK(cudaMemcpyAsync(ctx->stage, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
	// a new step starts at stage 0
	std::vector<DynState> d(ctx->S);
	DK(cudaMemcpyAsync(d.data(), ctx->dyn, d.size() * sizeof(DynState), cudaMemcpyDeviceToHost, ctx->st));
	DK(cudaStreamSynchronize(ctx->st));
	for (auto& x : d) x.stage = 0;
	DK(cudaMemcpyAsync(ctx->dyn, d.data(), d.size() * sizeof(DynState), cudaMemcpyHostToDevice, ctx->st));
	DK(cudaStreamSynchronize(ctx->st));
	ctx->have_eval = false;
	return TDVMC_OK;
}

int tdvmc_drops_get_params(tdvmc_drops* ctx, double* uR, double* uI, double* phiR, double* phiI) {
	if (!ctx) return TDVMC_ERR_ARG;
	std::vector<double> v((size_t)ctx->S * ctx->np);
	DK(cudaMemcpyAsync(v.data(), ctx->base, v.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
	DK(cudaStreamSynchronize(ctx->st));
	for (int s = 0; s < ctx->S; s++) {
		const double* q = &v[(size_t)s * ctx->np];
		for (int k = 0; k < ctx->p1; k++) {
			if (uR) uR[(size_t)s * ctx->p1 + k] = q[k];
			if (uI) uI[(size_t)s * ctx->p1 + k] = q[ctx->p1 + k];
		}
		if (phiR) phiR[s] = q[2 * ctx->p1];
		if (phiI) phiI[s] = q[2 * ctx->p1 + 1];
	}
	return TDVMC_OK;
}

int tdvmc_drops_set_walkers(tdvmc_drops* ctx, const double* x) {
	if (!ctx || !x) return TDVMC_ERR_ARG;
	const size_t m = (size_t)ctx->total_coords;
	for (size_t i = 0; i < m; i++)
		if (!std::isfinite(x[i])) return TDVMC_ERR_ARG;
	if (ctx->prec == TDVMC_PREC_FP64) {
		DK(cudaMemcpyAsync(ctx->pos, x, m * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
		DK(cudaStreamSynchronize(ctx->st));
	} else {
		std::vector<float> f(m);
		for (size_t i = 0; i < m; i++) f[i] = (float)x[i];
		DK(cudaMemcpyAsync(ctx->pos, f.data(), m * sizeof(float), cudaMemcpyHostToDevice, ctx->st));
		DK(cudaStreamSynchronize(ctx->st));
	}
	ctx->have_walkers = true;
	ctx->have_eval = false;
	return TDVMC_OK;
}

int tdvmc_drops_get_walkers(tdvmc_drops* ctx, double* x) {
	if (!ctx || !x) return TDVMC_ERR_ARG;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	return dcopy_any(ctx, ctx->pos, x, (size_t)ctx->total_coords);
}

int tdvmc_drops_sample(tdvmc_drops* ctx, int32_t moves_per_particle, double mc_step, uint64_t seed, uint32_t pass,
                       int64_t* accepted) {
	if (!ctx || moves_per_particle < 0 || !(mc_step >= 0)) return TDVMC_ERR_ARG;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	// the pass counter of drop 0 feeds the Philox counter
	DynState d0;
	DK(cudaMemcpyAsync(&d0, ctx->dyn, sizeof(d0), cudaMemcpyDeviceToHost, ctx->st));
	DK(cudaStreamSynchronize(ctx->st));
	d0.pass = pass;
	DK(cudaMemcpyAsync(ctx->dyn, &d0, sizeof(d0), cudaMemcpyHostToDevice, ctx->st));
	int rc = ctx->prec == TDVMC_PREC_FP64 ? dl_prep<double>(ctx) : dl_prep<float>(ctx);
	if (rc) return rc;
	rc = ctx->prec == TDVMC_PREC_FP64 ? dl_sample<double>(ctx, moves_per_particle, mc_step, seed)
	                                  : dl_sample<float>(ctx, moves_per_particle, mc_step, seed);
	if (rc) return rc;
	DK(cudaStreamSynchronize(ctx->st));
	if (accepted) {
		std::vector<int> a((size_t)ctx->S * ctx->nws);
		DK(cudaMemcpy(a.data(), ctx->acc, a.size() * sizeof(int), cudaMemcpyDeviceToHost));
		int64_t t = 0;
		for (int v : a) t += v;
		*accepted = t;
	}
	ctx->have_eval = false;
	return TDVMC_OK;
}

int tdvmc_drops_eval(tdvmc_drops* ctx, double* lnpsi, double* O, double* eloc, double* other7, double* dE) {
	if (!ctx) return TDVMC_ERR_ARG;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	const bool adj = dE != nullptr;
	int rc = ctx->prec == TDVMC_PREC_FP64 ? dl_prep<double>(ctx) : dl_prep<float>(ctx);
	if (rc) return rc;
	rc = ctx->prec == TDVMC_PREC_FP64 ? dl_eval<double>(ctx, adj) : dl_eval<float>(ctx, adj);
	if (rc) return rc;
	DK(cudaStreamSynchronize(ctx->st));
	ctx->have_eval = true;
	ctx->last_adj = adj;
	const size_t nwt = (size_t)ctx->S * ctx->nws;
	if ((rc = dcopy_any(ctx, ctx->lnpsi, lnpsi, nwt))) return rc;
	if ((rc = dcopy_any(ctx, ctx->O, O, nwt * ctx->p1))) return rc;
	if ((rc = dcopy_any(ctx, ctx->eloc, eloc, nwt * 2))) return rc;
	if ((rc = dcopy_any(ctx, ctx->other7, other7, nwt * 7))) return rc;
	if (adj && (rc = dcopy_any(ctx, ctx->dE, dE, nwt * 2 * ctx->p1))) return rc;
	return TDVMC_OK;
}

int tdvmc_drops_reduce(tdvmc_drops* ctx, double* O_mean, double* energy, double* S, double* cov_OER,
                       double* cov_OEI, double* dE_mean, double* accepted_mean) {
	if (!ctx) return TDVMC_ERR_ARG;
	if (!ctx->have_eval) return TDVMC_ERR_STATE;
	int rc = ctx->prec == TDVMC_PREC_FP64 ? dl_reduce<double>(ctx, ctx->last_adj) : dl_reduce<float>(ctx, ctx->last_adj);
	if (rc) return rc;
	const int p1 = ctx->p1;
	const DropCols cl{p1};
	const int K = cl.count();
	std::vector<double> m((size_t)ctx->S * K), Sh((size_t)ctx->S * p1 * p1), cv((size_t)ctx->S * p1 * 2);
	DK(cudaMemcpyAsync(m.data(), ctx->means, m.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
	DK(cudaMemcpyAsync(Sh.data(), ctx->Sm, Sh.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
	DK(cudaMemcpyAsync(cv.data(), ctx->cov, cv.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
	DK(cudaStreamSynchronize(ctx->st));
	for (int s = 0; s < ctx->S; s++) {
		const double* q = &m[(size_t)s * K];
		for (int k = 0; k < p1; k++) {
			if (O_mean) O_mean[(size_t)s * p1 + k] = q[k];
			if (cov_OER) cov_OER[(size_t)s * p1 + k] = cv[((size_t)s * p1 + k) * 2];
			if (cov_OEI) cov_OEI[(size_t)s * p1 + k] = cv[((size_t)s * p1 + k) * 2 + 1];
			if (dE_mean) {
				dE_mean[((size_t)s * p1 + k) * 2] = q[cl.dE() + 2 * k];
				dE_mean[((size_t)s * p1 + k) * 2 + 1] = q[cl.dE() + 2 * k + 1];
			}
		}
		if (energy) {
			energy[2 * s] = q[cl.ER()];
			energy[2 * s + 1] = q[cl.EI()];
		}
		if (accepted_mean) accepted_mean[s] = q[cl.acc()];
	}
	if (S) std::memcpy(S, Sh.data(), Sh.size() * sizeof(double));
	return TDVMC_OK;
}

int tdvmc_drops_tdvp_rhs(tdvmc_drops* ctx, int32_t imaginary_time, int32_t precondition, int32_t lin_solver,
                         double* uDotR, double* uDotI, double* phiDotR, double* phiDotI, int32_t* status) {
	if (!ctx || (lin_solver != 0 && lin_solver != 1)) return TDVMC_ERR_ARG;
	if (!ctx->have_eval) return TDVMC_ERR_STATE;
	int rc = ctx->prec == TDVMC_PREC_FP64 ? dl_reduce<double>(ctx, ctx->last_adj) : dl_reduce<float>(ctx, ctx->last_adj);
	if (rc) return rc;
	rc = ctx->prec == TDVMC_PREC_FP64 ? dl_solve<double>(ctx, imaginary_time, precondition, lin_solver, 0, 0, 0.0, 0)
	                                  : dl_solve<float>(ctx, imaginary_time, precondition, lin_solver, 0, 0, 0.0, 0);
	if (rc) return rc;
	std::vector<double> r((size_t)ctx->S * ctx->np);
	DK(cudaMemcpyAsync(r.data(), ctx->rhs, r.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
	DK(cudaStreamSynchronize(ctx->st));
	for (int s = 0; s < ctx->S; s++) {
		const double* q = &r[(size_t)s * ctx->np];
		for (int k = 0; k < ctx->p1; k++) {
			if (uDotR) uDotR[(size_t)s * ctx->p1 + k] = q[k];
			if (uDotI) uDotI[(size_t)s * ctx->p1 + k] = q[ctx->p1 + k];
		}
		if (phiDotR) phiDotR[s] = q[2 * ctx->p1];
		if (phiDotI) phiDotI[s] = q[2 * ctx->p1 + 1];
	}
	return drop_status(ctx, status);
}

int tdvmc_drops_run_steps(tdvmc_drops* ctx, const tdvmc_step_opts* o, int32_t nsteps, double* energy,
                          int32_t* status) {
	if (!ctx || nsteps < 0) return TDVMC_ERR_ARG;
	int rc = check_drop_opts(o);
	if (rc) return rc;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	if ((rc = drop_enqueue(ctx, o, nsteps))) return rc;
	DK(cudaStreamSynchronize(ctx->st));
	ctx->have_eval = true;
	ctx->last_adj = o->use_adjoint != 0;
	if (energy) {
		const DropCols cl{ctx->p1};
		const int K = cl.count();
		std::vector<double> m((size_t)ctx->S * K);
		// RK4 keeps the first stage's means; the Euler step has only one
		DK(cudaMemcpy(m.data(), o->ode_solver == 0 ? ctx->means : ctx->means0, m.size() * sizeof(double),
		              cudaMemcpyDeviceToHost));
		for (int s = 0; s < ctx->S; s++) {
			energy[2 * s] = m[(size_t)s * K + cl.ER()];
			energy[2 * s + 1] = m[(size_t)s * K + cl.EI()];
		}
	}
	return drop_status(ctx, status);
}

int tdvmc_drops_time_steps(tdvmc_drops* ctx, const tdvmc_step_opts* o, int32_t nsteps, float* ms) {
	if (!ctx || nsteps < 1 || !ms) return TDVMC_ERR_ARG;
	int rc = check_drop_opts(o);
	if (rc) return rc;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	cudaGraphExec_t g;
	int nk = 0;
	if ((rc = drop_graph(ctx, o, &g, &nk))) return rc;
	cudaEvent_t a, b;
	DK(cudaEventCreate(&a));
	if (cudaEventCreate(&b) != cudaSuccess) {
		cudaEventDestroy(a);
		return TDVMC_ERR_CUDA;
	}
	cudaEventRecord(a, ctx->st);
	rc = drop_enqueue(ctx, o, nsteps);
	cudaEventRecord(b, ctx->st);
	const cudaError_t e = cudaEventSynchronize(b);
	if (!rc && e == cudaSuccess) cudaEventElapsedTime(ms, a, b);
	cudaEventDestroy(a);
	cudaEventDestroy(b);
	if (rc) return rc;
	DK(e);
	ctx->have_eval = true;
	ctx->last_adj = o->use_adjoint != 0;
	return drop_status(ctx, nullptr);
}

int tdvmc_drops_profile_stage(tdvmc_drops* ctx, const tdvmc_step_opts* o, float* ms, const char** names,
                              int32_t* count) {
	if (!ctx || !ms || !count) return TDVMC_ERR_ARG;
	int rc = check_drop_opts(o);
	if (rc) return rc;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	std::vector<cudaEvent_t> ev;
	std::vector<const char*> nm;
	cudaEvent_t e0;
	DK(cudaEventCreate(&e0));
	cudaEventRecord(e0, ctx->st);
	ctx->prof = &ev;
	ctx->prof_names = &nm;
	rc = dl_stage_any(ctx, o);
	ctx->prof = nullptr;
	ctx->prof_names = nullptr;
	cudaStreamSynchronize(ctx->st);
	if (!rc) {
		// back to the step boundary: every drop's next step starts at stage 0 from its
		// unchanged base parameters
		std::vector<DynState> d(ctx->S);
		if (cudaMemcpyAsync(ctx->stage, ctx->base, (size_t)ctx->S * ctx->np * sizeof(double), cudaMemcpyDeviceToDevice,
		                    ctx->st) != cudaSuccess ||
		    cudaMemcpyAsync(d.data(), ctx->dyn, d.size() * sizeof(DynState), cudaMemcpyDeviceToHost, ctx->st) !=
		        cudaSuccess ||
		    cudaStreamSynchronize(ctx->st) != cudaSuccess) {
			rc = TDVMC_ERR_CUDA;
		} else {
			for (auto& x : d) x.stage = 0;
			if (cudaMemcpyAsync(ctx->dyn, d.data(), d.size() * sizeof(DynState), cudaMemcpyHostToDevice, ctx->st) !=
			        cudaSuccess ||
			    cudaStreamSynchronize(ctx->st) != cudaSuccess)
				rc = TDVMC_ERR_CUDA;
		}
	}
	const int k = (int)std::min<size_t>(ev.size(), 16);
	cudaEvent_t prev = e0;
	for (int i = 0; i < k; i++) {
		ms[i] = 0.f;
		cudaEventElapsedTime(&ms[i], prev, ev[i]);
		if (names) names[i] = nm[i];
		prev = ev[i];
	}
	*count = k;
	cudaEventDestroy(e0);
	for (auto e : ev) cudaEventDestroy(e);
	if (rc) return rc;
	ctx->have_eval = true;
	ctx->last_adj = o->use_adjoint != 0;
	return drop_status(ctx, nullptr);
}

int tdvmc_drops_autotune(tdvmc_drops* ctx, int32_t moves_per_particle, double mc_step) {
	if (!ctx || moves_per_particle < 0) return TDVMC_ERR_ARG;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	// candidates are timed on a copy of the walkers, which are restored afterwards
	const size_t bytes = (size_t)ctx->total_coords * tsz(ctx);
	void* save = nullptr;
	DK(cudaMalloc(&save, bytes));
	cudaEvent_t a = nullptr, b = nullptr;
	int rc = TDVMC_OK;
	const int ts0 = ctx->tpb_s, te0 = ctx->tpb_e;
	int best_s = ts0, best_e = te0;
	float tbest_s = 1e30f, tbest_e = 1e30f;
	auto fail = [&](int code) {
		rc = code;
		return code;
	};
	do {
		if (cudaMemcpyAsync(save, ctx->pos, bytes, cudaMemcpyDeviceToDevice, ctx->st) != cudaSuccess ||
		    cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
			fail(TDVMC_ERR_CUDA);
			break;
		}
		if ((rc = ctx->prec == TDVMC_PREC_FP64 ? dl_prep<double>(ctx) : dl_prep<float>(ctx))) break;
		for (int tpb : {32, 64, 128}) {
			const bool eval_fits = eval_smem(ctx, tpb, true) <= kDropSmemMax;
			if ((rc = set_items(ctx, tpb, eval_fits ? tpb : te0))) break;
			for (int rep = 0; rep < 2 && !rc; rep++) {
				cudaEventRecord(a, ctx->st);
				rc = ctx->prec == TDVMC_PREC_FP64 ? dl_sample<double>(ctx, moves_per_particle, mc_step, 7)
				                                  : dl_sample<float>(ctx, moves_per_particle, mc_step, 7);
				cudaEventRecord(b, ctx->st);
				if (cudaEventSynchronize(b) != cudaSuccess) fail(TDVMC_ERR_CUDA);
				float t = 0.f;
				cudaEventElapsedTime(&t, a, b);
				if (rep == 1 && t < tbest_s) {
					tbest_s = t;
					best_s = tpb;
				}
			}
			if (rc || !eval_fits) continue;
			for (int rep = 0; rep < 2 && !rc; rep++) {
				cudaEventRecord(a, ctx->st);
				rc = ctx->prec == TDVMC_PREC_FP64 ? dl_eval<double>(ctx, true) : dl_eval<float>(ctx, true);
				cudaEventRecord(b, ctx->st);
				if (cudaEventSynchronize(b) != cudaSuccess) fail(TDVMC_ERR_CUDA);
				float t = 0.f;
				cudaEventElapsedTime(&t, a, b);
				if (rep == 1 && t < tbest_e) {
					tbest_e = t;
					best_e = tpb;
				}
			}
			if (rc) break;
		}
	} while (false);
	// restore the walkers and keep the best tiles (the starting tiles on error)
	if (save) {
		cudaMemcpyAsync(ctx->pos, save, bytes, cudaMemcpyDeviceToDevice, ctx->st);
		cudaStreamSynchronize(ctx->st);
		cudaFree(save);
	}
	if (a) cudaEventDestroy(a);
	if (b) cudaEventDestroy(b);
	const int rs = rc ? set_items(ctx, ts0, te0) : set_items(ctx, best_s, best_e);
	ctx->have_eval = false;
	return rc ? rc : rs;
}

int tdvmc_drops_get_tiles(tdvmc_drops* ctx, int32_t* sample_threads, int32_t* eval_threads) {
	if (!ctx) return TDVMC_ERR_ARG;
	if (sample_threads) *sample_threads = ctx->tpb_s;
	if (eval_threads) *eval_threads = ctx->tpb_e;
	return TDVMC_OK;
}

int64_t tdvmc_drops_launch_count(tdvmc_drops* ctx) { return ctx ? ctx->launches : -1; }

}  // extern "C"
