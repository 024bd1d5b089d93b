// C ABI of the GB300 TDVP hot path: context, device tables, kernel dispatch,
// CUDA-graph capture of the RK stages.  Declarations and the reference
// interface each entry point replaces: include/tdvmc_gpu.h.
#include "../../include/tdvmc_gpu.h"

#include "common.cuh"
#include "dispatch.cuh"
#include "k_cs.cuh"
#include "k_eloc.cuh"
#include "k_gram_tf32.cuh"
#include "k_obs.cuh"
#include "k_sample.cuh"
#include "k_solve.cuh"
#include "k_stats.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

using namespace tdvmc;

namespace {

struct Tiles {
	int sg = 32;     // sampler lanes per walker
	int sgpb = 4;    // sampler walkers per block
	int eg = 32;     // evaluation lanes per walker
	int egpb = 0;    // evaluation walkers per block; 0: per kernel, the most walkers resident per SM
	int hist = 0;    // histogram update mode of the evaluation kernel (full-warp groups)
};

struct GraphKey {
	double dt, mc_step;
	int imag, ode, lin, pre, norm, moves, adj;
	uint64_t seed;
	int kind;       // stage kind of the stored-sample solver (CsStage), 0 otherwise
	int64_t count;  // walkers refreshed by a CsStage::kRefresh stage
	bool operator<(const GraphKey& o) const {
		return std::tie(dt, mc_step, imag, ode, lin, pre, norm, moves, adj, seed, kind, count) <
		       std::tie(o.dt, o.mc_step, o.imag, o.ode, o.lin, o.pre, o.norm, o.moves, o.adj, o.seed, o.kind, o.count);
	}
};

// Stages of ODE_SOLVER_TYPE 3 (RK4 on stored samples)
enum CsStage : int {
	kCsFull = 1,     // sample every walker, store, evaluate the stored samples
	kCsRefresh = 2,  // sample and store a rotating window of walkers, evaluate all
	kCsReuse = 3,    // evaluate the stored samples at the stage parameters
};

}  // namespace

struct tdvmc_ctx {
	SysConst sc{};
	int prec = TDVMC_PREC_FP64;
	int64_t nw = 0;
	int device = 0;
	int nsm = 0;
	cudaStream_t st = nullptr;
	std::vector<double> knots, loc, fold, pot;
	std::vector<double> locc;  // the pieces in the FP32 kernels' local coordinate (loc for FP64)
	int npot = 0;
	double time = 0.0;
	Tiles tiles;
	bool have_walkers = false;
	bool have_eval = false;
	bool last_adj = false;
	int last_moves = 0;
	int64_t launches = 0;
	// device buffers (T = float or double by precision)
	void *pos = nullptr, *lnpsi = nullptr, *O = nullptr, *eloc = nullptr, *other7 = nullptr, *dE = nullptr;
	int* acc = nullptr;
	double *base = nullptr, *stage = nullptr, *kdot = nullptr, *rhs = nullptr;
	double *loc_d = nullptr, *fold_d = nullptr;
	void *coefU = nullptr, *coefC = nullptr, *uout = nullptr, *kb = nullptr, *hv = nullptr, *locT = nullptr;
	int* lut = nullptr;
	double *part1 = nullptr, *means1 = nullptr, *means0 = nullptr, *part2 = nullptr, *C2 = nullptr;
	float* partS = nullptr;
	double* Sg = nullptr;
	void* gramws = nullptr;
	DynState* dyn = nullptr;
	int nblk1 = 0, nblk2 = 0, chunk2 = 0, nblkS = 0;
	bool gram_tc = false;  // S on the tensor cores (mixed precision only)
	bool packed_sampler = true;  // FP32 uniform-knot sampler with f32x2 pair arithmetic
	bool shared_coords = false;  // its variant with the lane's coordinates in shared memory
	std::map<GraphKey, cudaGraphExec_t> graphs;
	std::map<GraphKey, int> graph_kernels;  // kernels launched by one replay
	// stored samples (correlated-sampling reuse), allocated on first use
	void *csD = nullptr, *csD2 = nullptr, *csO = nullptr, *csV = nullptr, *cs_piece = nullptr;
	bool cs_uni = false;          // every interval has the same piece row (equal widths)
	double cs_pu[kCsPiece] = {};  // that row
	void* gbuf = nullptr;  // per-particle gradients [w][6][n] passed to the reverse (adjoint) kernel
	// sampling / evaluation pipeline over walker chunks: the sampler runs on st,
	// the evaluation of the previous chunk on st2 beside it.  Off by default:
	// at N=343, 65,536 walkers it measured 380-416 ms per step (2-8 chunks)
	// against 328 ms back to back, because the evaluation kernels lose more to
	// the block slots left to the sampler than the sampler gains.
	static constexpr int kMaxChunks = 16;
	int pipeline = 1;  // chunks per stage; 1 runs sampling and evaluation back to back
	cudaStream_t st2 = nullptr;
	cudaEvent_t ev_s[kMaxChunks] = {};
	cudaEvent_t ev_e = nullptr;
	int32_t* chunk_starts = nullptr;  // device: first walker of every chunk
	int32_t* csN = nullptr;
	bool cs_valid = false;      // the store matches the walkers
	int64_t cs_steps = 0;       // stored-sample steps since the last full store
	int64_t cs_last_count = 0;  // walkers sampled by the last refresh
	std::string err;
	// status limit of the bounded hardware waits (k_gram_tf32, k_cs_eval_st);
	// TDVMC_TEST_WAIT_NS at creation overrides it (0: give up at once, to test
	// the failure path)
	uint64_t wait_ns = kWaitStatusNs;
	// eager profiling: events recorded after every kernel when set
	std::vector<cudaEvent_t>* prof = nullptr;
	std::vector<const char*>* prof_names = nullptr;
};

namespace {

#define CK(call)                                                                  \
	do {                                                                          \
		cudaError_t e_ = (call);                                                  \
		if (e_ != cudaSuccess) {                                                  \
			if (ctx) ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_); \
			return TDVMC_ERR_CUDA;                                                \
		}                                                                         \
	} while (0)

// ---------------------------------------------------------------------------
// host-side spline tables (same construction as BosonsBulk::InitSystem and
// SplineFactory::GetWeights3, evaluated in local interval coordinates)
// ---------------------------------------------------------------------------
void poly_lin(const double* a, double c0, double c1, double* out) {
	double o[4] = {0, 0, 0, 0};
	for (int i = 0; i < 4; i++) {
		o[i] += a[i] * c0;
		if (i + 1 < 4) o[i + 1] += a[i] * c1;
	}
	for (int i = 0; i < 4; i++) out[i] = o[i];
}

// polynomial in t of B-spline N_{s,3} on knot interval b
void piece_local(const std::vector<double>& k, int s, int b, double* out) {
	double N[4][4][4];
	std::memset(N, 0, sizeof(N));
	const double h = k[b + 1] - k[b];
	for (int i = 0; i < 4; i++)
		if (s + i == b) N[0][i][0] = 1.0;
	for (int d = 1; d <= 3; d++)
		for (int i = 0; i + d <= 3; i++) {
			const int ii = s + i;
			double acc[4] = {0, 0, 0, 0}, tmp[4];
			const double den1 = k[ii + d] - k[ii], den2 = k[ii + d + 1] - k[ii + 1];
			if (den1 != 0.0) {
				poly_lin(N[d - 1][i], (k[b] - k[ii]) / den1, h / den1, tmp);
				for (int c = 0; c < 4; c++) acc[c] += tmp[c];
			}
			if (den2 != 0.0) {
				poly_lin(N[d - 1][i + 1], (k[ii + d + 1] - k[b]) / den2, -h / den2, tmp);
				for (int c = 0; c < 4; c++) acc[c] += tmp[c];
			}
			std::memcpy(N[d][i], acc, sizeof(acc));
		}
	std::memcpy(out, N[3][0], 4 * sizeof(double));
}

size_t tsize(int prec) { return prec == TDVMC_PREC_FP64 ? sizeof(double) : sizeof(float); }

void apply_quench(tdvmc_ctx* c, double& a, double& b) {
	a = c->npot > 0 ? c->pot[0] : 0.0;
	b = c->npot > 1 ? c->pot[1] : 0.0;
	if (c->npot > 4 && c->time >= c->pot[2]) {
		a = c->pot[3];
		b = c->pot[4];
	}
}

// ---------------------------------------------------------------------------
// kernel dispatch (instantiations in inst_*.cu)
// ---------------------------------------------------------------------------
int slots_for(int n, int G) { return sample_slots_for(n, G); }

void mark(tdvmc_ctx* ctx, const char* name) {
	if (!ctx->prof) return;
	cudaEvent_t e;
	cudaEventCreate(&e);
	cudaEventRecord(e, ctx->st);
	ctx->prof->push_back(e);
	ctx->prof_names->push_back(name);
}

// Persistent grid: resident blocks per SM x SMs, at most one block per work
// group; free > 0 leaves that many block slots per SM to a concurrent kernel.
int grid_for(tdvmc_ctx* ctx, const void* fn, int threads, size_t smem, int64_t work_groups, int gpb, int free = 0) {
	int per_sm = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
	per_sm -= free;
	if (per_sm < 1) per_sm = 1;
	int64_t need = (work_groups + gpb - 1) / gpb;
	int64_t g = (int64_t)per_sm * ctx->nsm;
	return (int)std::max<int64_t>(1, std::min(need, g));
}

template <typename T>
int launch_prep(tdvmc_ctx* ctx) {
	k_prep<T><<<1, 128, 0, ctx->st>>>(ctx->sc.p, ctx->sc.ns, ctx->sc.nbin, ctx->sc.ncoef, ctx->sc.uniform, ctx->sc.hinv,
	                                  (const T*)ctx->hv, ctx->stage, ctx->fold_d, ctx->loc_d, (T*)ctx->coefU,
	                                  (T*)ctx->coefC, (T*)ctx->uout);
	ctx->launches++;
	mark(ctx, "k_prep");
	CK(cudaGetLastError());
	return TDVMC_OK;
}

// Samples walkers (start + w) mod nw, w < count; start = *wstart (device) or 0.
template <typename T>
int launch_sample(tdvmc_ctx* ctx, int moves, double step, uint64_t seed, int64_t count = -1,
                  const int32_t* wstart = nullptr) {
	if (count < 0) count = ctx->nw;
	const int G = ctx->tiles.sg, gpb = ctx->tiles.sgpb;
	const int slots = slots_for(ctx->sc.n, G);
	SampleFn<T> fn = nullptr;
	if constexpr (std::is_same<T, float>::value)
		if (ctx->packed_sampler && ctx->sc.uniform) {
			if (ctx->sc.mirror) {
				fn = pick_sample_f32_packed_pb(G, slots);
			} else {
				if (ctx->shared_coords) fn = pick_sample_f32_packed_shared(G, slots);
				if (!fn) fn = pick_sample_f32_packed(G, slots);
			}
		}
	const bool packed = fn != nullptr;
	if (!fn) fn = ctx->sc.mirror ? pick_sample_pb<T>(G, slots) : pick_sample<T>(G, slots);
	if (!fn) return TDVMC_ERR_ARG;
	const int threads = G * gpb;
	const size_t smem =
	    sample_smem_bytes<T>(ctx->sc.ncoef, ctx->sc.nbin, ctx->sc.ncell, ctx->sc.n, gpb, packed ? kCoefCopies : 1);
	CK(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	const int grid = grid_for(ctx, (const void*)fn, threads, smem, count, gpb);
	uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
	fn<<<grid, threads, smem, ctx->st>>>(ctx->sc, (const Q4<T>*)ctx->coefU, (const T*)ctx->uout, (const T*)ctx->kb,
	                                     (const T*)ctx->hv, ctx->lut, (T*)ctx->pos, count, ctx->nw, wstart, moves,
	                                     (T)step, key, &ctx->dyn->pass, ctx->acc);
	ctx->launches++;
	mark(ctx, "k_sample");
	CK(cudaGetLastError());
	return TDVMC_OK;
}

// shared memory of the forward (k_eloc) and, for adj, the larger of it and the reverse kernel
template <typename T>
size_t eloc_smem(tdvmc_ctx* ctx, int G, int gpb, bool adj) {
	const SysConst& s = ctx->sc;
	const size_t f = eloc_cta_bytes<T>(s.nbin, s.ncell) + (size_t)gpb * eloc_group_bytes<T>(s.n, s.nbin, s.ns, G);
	if (!adj) return f;
	const size_t r =
	    rev_cta_bytes<T>(s.nbin, s.ncell) + (size_t)gpb * rev_group_bytes<T>(s.n, s.nbin, s.ns, G, G == 32 ? ctx->tiles.hist : 0);
	return std::max(f, r);
}

// Walkers per block of an evaluation kernel (cta + gpb * grp bytes of shared
// memory, G lanes per walker): `want` when positive, fewer where the shared
// memory would not fit; else the count in {1, 2, 4} that keeps the most walkers
// resident per SM (the smaller on a tie).  Sets the kernel's shared memory
// attributes for the largest request; 0 if no count fits.
int pick_gpb(const void* fn, int G, int want, size_t cta, size_t grp) {
	constexpr size_t kSmemMax = 227 * 1024;
	if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax) != cudaSuccess ||
	    cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared) !=
	        cudaSuccess)
		return 0;
	cudaFuncAttributes fa;
	if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) return 0;
	const int max_threads = fa.maxThreadsPerBlock < 128 ? fa.maxThreadsPerBlock : 128;
	if (want > 0) {
		int g = want;
		while (g > 1 && (cta + (size_t)g * grp > kSmemMax || G * g > max_threads)) g--;
		return cta + (size_t)g * grp <= kSmemMax ? g : 0;
	}
	int best = 0, best_w = 0;
	for (int g : {1, 2, 4}) {
		if (G * g > max_threads || cta + (size_t)g * grp > kSmemMax) continue;
		int blocks = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, G * g, cta + (size_t)g * grp) != cudaSuccess)
			return 0;
		if (blocks * g > best_w) {
			best_w = blocks * g;
			best = g;
		}
	}
	return best;
}

// Gradient scratch (nw x 6 x n): the partner sums of the 32-lane forward
// kernel and the adjoint's input, allocated on the first evaluation and
// always before a stream capture (allocation is not capturable).
int ensure_gbuf(tdvmc_ctx* ctx) {
	if (ctx->gbuf) return TDVMC_OK;
	const size_t bytes = (size_t)ctx->nw * 6 * ctx->sc.n * tsize(ctx->prec);
	if (cudaMalloc(&ctx->gbuf, bytes) != cudaSuccess) {
		ctx->gbuf = nullptr;
		cudaGetLastError();  // out of memory is not sticky
		return TDVMC_ERR_NOMEM;
	}
	return TDVMC_OK;
}

// Forward evaluation; with adj also the reverse (adjoint) kernel, which reads
// the per-particle gradients the forward kernel leaves in ctx->gbuf.
// Walkers [w0, w0 + count) on stream st; free block slots per SM as in grid_for.
template <typename T>
int launch_eloc(tdvmc_ctx* ctx, bool adj, int64_t w0 = 0, int64_t count = -1, cudaStream_t st = nullptr,
                int free = 0) {
	if (count < 0) count = ctx->nw;
	if (!st) st = ctx->st;
	const int G = ctx->tiles.eg;
	const int hist = G == 32 ? ctx->tiles.hist : 0;
	const bool pb = ctx->sc.mirror != 0;
	ElocFn<T> fn = pb ? pick_eloc_pb<T>(G, adj, hist) : pick_eloc<T>(G, adj, hist);
	RevFn<T> fr = !adj ? nullptr : pb ? pick_eloc_rev_pb<T>(G, hist) : pick_eloc_rev<T>(G, hist);
	if (!fn || (adj && !fr)) return TDVMC_ERR_ARG;
	const SysConst& s = ctx->sc;
	// the gradient scratch: the adjoint's input, and the 32-lane forward's partner sums
	const bool need_g = adj || G == 32;
	if (need_g && !ctx->gbuf) return TDVMC_ERR_STATE;  // ensure_gbuf was not called
	const size_t fcta = eloc_cta_bytes<T>(s.nbin, s.ncell), fgrp = eloc_group_bytes<T>(s.n, s.nbin, s.ns, G);
	const int gpb = pick_gpb((const void*)fn, G, ctx->tiles.egpb, fcta, fgrp);
	if (gpb < 1) return TDVMC_ERR_CUDA;
	const int threads = G * gpb;
	const size_t smem = fcta + (size_t)gpb * fgrp;
	const int grid = grid_for(ctx, (const void*)fn, threads, smem, count, gpb, free);
	const size_t P = (size_t)s.p, dn = (size_t)s.dim * s.n;
	T* gb = need_g ? (T*)ctx->gbuf + (size_t)w0 * 6 * s.n : nullptr;
	fn<<<grid, threads, smem, st>>>(s, ctx->dyn, (const Q4<T>*)ctx->coefC, (const T*)ctx->kb, (const T*)ctx->hv, ctx->lut,
	                                (const T*)ctx->locT, ctx->fold_d, ctx->stage, (const T*)ctx->pos + w0 * dn, count,
	                                (T*)ctx->lnpsi + w0, (T*)ctx->O + w0 * P, (T*)ctx->eloc + 2 * w0,
	                                (T*)ctx->other7 + 7 * w0, (T*)ctx->dE + 2 * P * w0, gb);
	ctx->launches++;
	mark(ctx, "k_eloc");
	CK(cudaGetLastError());
	if (!adj) return TDVMC_OK;
	const size_t rcta = rev_cta_bytes<T>(s.nbin, s.ncell), rgrp = rev_group_bytes<T>(s.n, s.nbin, s.ns, G, hist);
	const int gpr = pick_gpb((const void*)fr, G, ctx->tiles.egpb, rcta, rgrp);
	if (gpr < 1) return TDVMC_ERR_CUDA;
	const int threads_r = G * gpr;
	const size_t smr = rcta + (size_t)gpr * rgrp;
	const int gridr = grid_for(ctx, (const void*)fr, threads_r, smr, count, gpr, free);
	fr<<<gridr, threads_r, smr, st>>>(s, (const T*)ctx->kb, (const T*)ctx->hv, ctx->lut, (const T*)ctx->locT, ctx->fold_d,
	                                 (const T*)ctx->pos + w0 * dn, gb, count, (T*)ctx->dE + 2 * P * w0);
	ctx->launches++;
	mark(ctx, "k_eloc_rev");
	CK(cudaGetLastError());
	return TDVMC_OK;
}

template <typename T>
int launch_reduce(tdvmc_ctx* ctx, bool adj) {
	const int P = ctx->sc.p;
	Cols1 c{P};
	const int K1 = c.count();
	k_reduce1<T><<<ctx->nblk1, 256, 0, ctx->st>>>(P, ctx->nw, (const T*)ctx->O, (const T*)ctx->eloc,
	                                               (const T*)ctx->other7, (const T*)ctx->lnpsi, ctx->acc,
	                                               (const T*)ctx->dE, adj ? 1 : 0, ctx->stage, ctx->part1);
	mark(ctx, "k_reduce1");
	k_finalize<<<finalize_blocks(K1), kFinalizeThreads, 0, ctx->st>>>(K1, ctx->nblk1, ctx->part1, 1.0 / (double)ctx->nw,
	                                                                 ctx->means1);
	mark(ctx, "k_finalize1");
	ctx->launches += 2;
	CK(cudaGetLastError());
	const bool tc = ctx->gram_tc;
	const size_t sm2 = (size_t)ctx->chunk2 * (P + 2) * sizeof(double);
	CK(cudaFuncSetAttribute((const void*)k_reduce2<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2));
	k_reduce2<T><<<ctx->nblk2, 256, sm2, ctx->st>>>(P, ctx->nw, ctx->chunk2, (const T*)ctx->O, (const T*)ctx->eloc,
	                                                 ctx->means1, tc ? 0 : 1, ctx->part2);
	mark(ctx, "k_reduce2");
	k_finalize<<<finalize_blocks(P * (P + 2)), kFinalizeThreads, 0, ctx->st>>>(P * (P + 2), ctx->nblk2, ctx->part2,
	                                                                           1.0 / (double)ctx->nw, ctx->C2);
	mark(ctx, "k_finalize2");
	ctx->launches += 2;
	CK(cudaGetLastError());
	if (tc) {
		int rc = launch_gram_tf32(ctx->st, P, ctx->nw, (const float*)ctx->O, ctx->means1, ctx->nblkS, ctx->partS,
		                          ctx->Sg, ctx->nsm, ctx->wait_ns);
		ctx->launches += 2;
		mark(ctx, "k_gram_tf32+finalize");
		if (rc) {
			ctx->err = "gram launch failed";
			return TDVMC_ERR_CUDA;
		}
		CK(cudaGetLastError());
	}
	return TDVMC_OK;
}

template <typename T>
int launch_solve(tdvmc_ctx* ctx, int imag, int pre, int lin, int mode, int norm, double dt, int adj_force = 0) {
	const int P = ctx->sc.p;
	SolveArgs a;
	a.adj_force = adj_force;
	a.dE_col = Cols1{P}.dE();
	a.p = P;
	a.imag = imag;
	a.precond = pre;
	a.solver = lin;
	a.mode = mode;
	a.normalize = norm;
	a.dt = dt;
	const bool tc = ctx->gram_tc;
	const double* S = tc ? ctx->Sg : ctx->C2;
	a.ldS = tc ? P : P + 2;
	a.ldC = P + 2;
	const size_t smem = (size_t)(P * (P + 2) + 6 * P + 8) * sizeof(double);
	CK(cudaFuncSetAttribute((const void*)k_solve<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	Cols1 c{P};
	k_solve<T><<<1, 256, smem, ctx->st>>>(a, ctx->dyn, ctx->means1, S, ctx->C2 + P, (const T*)ctx->lnpsi, ctx->base,
	                                       ctx->stage, ctx->kdot, ctx->rhs, ctx->means0, c.count());
	ctx->launches++;
	mark(ctx, "k_solve");
	CK(cudaGetLastError());
	return TDVMC_OK;
}

// ---- stored samples (correlated-sampling reuse, ODE_SOLVER_TYPE 3) --------
int cs_alloc(tdvmc_ctx* ctx) {
	if (ctx->csD) return TDVMC_OK;
	const size_t ts = tsize(ctx->prec);
	const size_t nw = (size_t)ctx->nw, ns = (size_t)ctx->sc.ns, n = (size_t)ctx->sc.n, P = (size_t)ctx->sc.p;
	const size_t dbytes = nw * ns * 3 * (size_t)cs_npad((int)n) * ts;
	bool ok = cudaMalloc(&ctx->csD, dbytes) == cudaSuccess &&
	          cudaMalloc(&ctx->csD2, nw * ns * ts) == cudaSuccess && cudaMalloc(&ctx->csO, nw * P * ts) == cudaSuccess &&
	          cudaMalloc(&ctx->csV, nw * ts) == cudaSuccess &&
	          cudaMalloc((void**)&ctx->csN, nw * sizeof(int32_t)) == cudaSuccess;
	if (!ok) {
		void* b[] = {ctx->csD, ctx->csD2, ctx->csO, ctx->csV, ctx->csN};
		for (void* x : b)
			if (x) cudaFree(x);
		ctx->csD = ctx->csD2 = ctx->csO = ctx->csV = nullptr;
		ctx->csN = nullptr;
		cudaGetLastError();  // out of memory is not sticky
		return TDVMC_ERR_NOMEM;
	}
	// the row padding of D must read as zero; the store writes rows < n only
	CK(cudaMemsetAsync(ctx->csD, 0, dbytes, ctx->st));
	return TDVMC_OK;
}

// Stores walkers (start + w) mod nw, w < count (start = *wstart or 0).
template <typename T>
int launch_cs_store(tdvmc_ctx* ctx, int64_t count, const int32_t* wstart) {
	constexpr int G = 32;
	const SysConst& s = ctx->sc;
	// up to four walkers per block share the piece table
	const size_t cta = cs_cta_bytes<T>(s.nbin, s.ncell), grp = cs_group_bytes<T>(s.n, s.ns, G);
	int gpb = 4;
	while (gpb > 1 && cta + gpb * grp > 200 * 1024) gpb--;
	const size_t smem = cta + gpb * grp;
	auto fn = s.mirror ? (ctx->cs_uni ? k_cs_store<T, G, true, true> : k_cs_store<T, G, false, true>)
	                   : (ctx->cs_uni ? k_cs_store<T, G, true> : k_cs_store<T, G, false>);
	CsPieceRow<T> pu;
	for (int k = 0; k < kCsPiece; k++) pu.c[k] = (T)ctx->cs_pu[k];
	CK(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	const int grid = grid_for(ctx, (const void*)fn, G * gpb, smem, count, gpb);
	fn<<<grid, G * gpb, smem, ctx->st>>>(s, pu, ctx->dyn, (const T*)ctx->cs_piece, (const T*)ctx->kb, (const T*)ctx->hv, ctx->lut,
	                               ctx->fold_d, (const T*)ctx->pos, count, ctx->nw, wstart, (T*)ctx->csD,
	                               (T*)ctx->csD2, (T*)ctx->csO, (T*)ctx->csV, ctx->csN);
	ctx->launches++;
	mark(ctx, "k_cs_store");
	CK(cudaGetLastError());
	return TDVMC_OK;
}

template <typename T>
int launch_cs_eval(tdvmc_ctx* ctx, bool adj) {
	const SysConst& s = ctx->sc;
	const int threads = 128, wpb = threads / 32;
	if constexpr (sizeof(T) == 4) {
		if (s.ns <= kCsStNs) {
			constexpr int wst = kCsStWarps;
			const size_t smem = cs_eval_st_smem_bytes(s.ns, wst) + 8 * wst;
			auto fn = adj ? k_cs_eval_st<true> : k_cs_eval_st<false>;
			CK(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
			const int grid = grid_for(ctx, (const void*)fn, 32 * wst, smem, ctx->nw, wst);
			fn<<<grid, 32 * wst, smem, ctx->st>>>(s, ctx->stage, ctx->fold_d, (const float*)ctx->csD,
			                                     (const float*)ctx->csD2, (const float*)ctx->csO, (const float*)ctx->csV,
			                                     ctx->csN, ctx->nw, (float*)ctx->lnpsi, (float*)ctx->O, (float*)ctx->eloc,
			                                     (float*)ctx->other7, (float*)ctx->dE, ctx->wait_ns);
			ctx->launches++;
			mark(ctx, adj ? "k_cs_eval_st_adjoint" : "k_cs_eval_st");
			CK(cudaGetLastError());
			return TDVMC_OK;
		}
	}
	const size_t smem = cs_eval_smem_bytes<T>(s.n, s.ns, wpb);
	auto fn = adj ? k_cs_eval<T, true> : k_cs_eval<T, false>;
	CK(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	const int grid = grid_for(ctx, (const void*)fn, threads, smem, ctx->nw, wpb);
	fn<<<grid, threads, smem, ctx->st>>>(s, ctx->stage, ctx->fold_d, (const T*)ctx->csD, (const T*)ctx->csD2,
	                                     (const T*)ctx->csO, (const T*)ctx->csV, ctx->csN, ctx->nw, (T*)ctx->lnpsi,
	                                     (T*)ctx->O, (T*)ctx->eloc, (T*)ctx->other7, (T*)ctx->dE);
	ctx->launches++;
	mark(ctx, adj ? "k_cs_eval_adjoint" : "k_cs_eval");
	CK(cudaGetLastError());
	return TDVMC_OK;
}

// One RK stage on stored samples (CalculateNextParametersRK4ReuseSamples,
// TDVMC.cpp:2037-2103, with the sample update of TDVMC.cpp:3654-3677 at the
// first stage of a step).
// Solvers on stored samples: RK4 (ODE_SOLVER_TYPE 3) and the predictor-corrector (5).
inline bool cs_ode(int ode) { return ode == 3 || ode == 5; }
// Stages per step of the time integrators (RK4 4, Euler 1, predictor + correctors).
inline int stages_per_step(int ode) { return ode == 0 ? 1 : ode == 5 ? 1 + kPcCorrectors : 4; }

template <typename T>
int run_cs_stage(tdvmc_ctx* ctx, const tdvmc_step_opts* o, int kind, int64_t count) {
	int rc;
	const bool adj = o->use_adjoint != 0;
	if (kind == kCsFull || kind == kCsRefresh) {
		const bool all = kind == kCsFull;
		const int64_t cnt = all ? ctx->nw : count;
		const int32_t* ws = all ? nullptr : &ctx->dyn->cs_start;
		if ((rc = launch_prep<T>(ctx))) return rc;
		if (!all) CK(cudaMemsetAsync(ctx->acc, 0, (size_t)ctx->nw * sizeof(int), ctx->st));
		if (o->moves_per_stage > 0 && (rc = launch_sample<T>(ctx, o->moves_per_stage, o->mc_step, o->seed, cnt, ws)))
			return rc;
		if ((rc = launch_cs_store<T>(ctx, cnt, ws))) return rc;
		if (!all) {
			k_cs_advance<<<1, 32, 0, ctx->st>>>(ctx->dyn, cnt, ctx->nw);
			ctx->launches++;
			mark(ctx, "k_cs_advance");
			CK(cudaGetLastError());
		}
	}
	if ((rc = launch_cs_eval<T>(ctx, adj))) return rc;
	if ((rc = launch_reduce<T>(ctx, adj))) return rc;
	return launch_solve<T>(ctx, o->imaginary_time, o->precondition, o->lin_solver, o->ode_solver == 5 ? 3 : 1,
	                       o->normalize_wf, o->dt, (o->use_adjoint == 2 && o->imaginary_time) ? 1 : 0);
}

template <typename T>
int run_stage(tdvmc_ctx* ctx, const tdvmc_step_opts* o) {
	int rc;
	const int K = (int)std::min<int64_t>(ctx->pipeline, ctx->nw);
	if (K > 1 && o->moves_per_stage > 0 && !ctx->prof) {
		// chunk k is evaluated on st2 while st samples chunk k+1; the evaluation
		// kernels leave two block slots per SM to the sampler
		if ((rc = launch_prep<T>(ctx))) return rc;
		const bool adj = o->use_adjoint != 0;
		for (int k = 0; k < K; k++) {
			const int64_t a = ctx->nw * k / K, b = ctx->nw * (k + 1) / K;
			if ((rc = launch_sample<T>(ctx, o->moves_per_stage, o->mc_step, o->seed, b - a, ctx->chunk_starts + k)))
				return rc;
			CK(cudaEventRecord(ctx->ev_s[k], ctx->st));
			CK(cudaStreamWaitEvent(ctx->st2, ctx->ev_s[k], 0));
			if ((rc = launch_eloc<T>(ctx, adj, a, b - a, ctx->st2, 2))) return rc;
		}
		CK(cudaEventRecord(ctx->ev_e, ctx->st2));
		CK(cudaStreamWaitEvent(ctx->st, ctx->ev_e, 0));
		if ((rc = launch_reduce<T>(ctx, adj))) return rc;
		return launch_solve<T>(ctx, o->imaginary_time, o->precondition, o->lin_solver, o->ode_solver == 0 ? 2 : 1,
		                       o->normalize_wf, o->dt, (o->use_adjoint == 2 && o->imaginary_time) ? 1 : 0);
	}
	if ((rc = launch_prep<T>(ctx))) return rc;
	if (o->moves_per_stage > 0 && (rc = launch_sample<T>(ctx, o->moves_per_stage, o->mc_step, o->seed))) return rc;
	if ((rc = launch_eloc<T>(ctx, o->use_adjoint != 0))) return rc;
	if ((rc = launch_reduce<T>(ctx, o->use_adjoint != 0))) return rc;
	return launch_solve<T>(ctx, o->imaginary_time, o->precondition, o->lin_solver, o->ode_solver == 0 ? 2 : 1,
	                       o->normalize_wf, o->dt, (o->use_adjoint == 2 && o->imaginary_time) ? 1 : 0);
}

int run_stage_any(tdvmc_ctx* ctx, const tdvmc_step_opts* o, int kind = 0, int64_t count = 0) {
	if (kind)
		return ctx->prec == TDVMC_PREC_FP64 ? run_cs_stage<double>(ctx, o, kind, count)
		                                    : run_cs_stage<float>(ctx, o, kind, count);
	return ctx->prec == TDVMC_PREC_FP64 ? run_stage<double>(ctx, o) : run_stage<float>(ctx, o);
}

int check_opts(const tdvmc_step_opts* o) {
	if (!o || !(o->dt == o->dt)) return TDVMC_ERR_ARG;
	if (o->ode_solver != 0 && o->ode_solver != 2 && !cs_ode(o->ode_solver)) return TDVMC_ERR_ARG;
	if (cs_ode(o->ode_solver) &&
	    (o->update_every < 0 || !(o->update_percent >= 0.0 && o->update_percent <= 100.0)))
		return TDVMC_ERR_ARG;
	if (o->lin_solver != 0 && o->lin_solver != 1) return TDVMC_ERR_ARG;
	if (o->moves_per_stage < 0) return TDVMC_ERR_ARG;
	if (o->use_adjoint < 0 || o->use_adjoint > 2) return TDVMC_ERR_ARG;
	return TDVMC_OK;
}

// Graph of one stage; `kernels` = kernels one replay launches.
int get_graph(tdvmc_ctx* ctx, const tdvmc_step_opts* o, cudaGraphExec_t* out, int* kernels, int kind = 0,
              int64_t count = 0) {
	GraphKey k{o->dt, o->mc_step, o->imaginary_time, o->ode_solver, o->lin_solver, o->precondition,
	           o->normalize_wf, o->moves_per_stage, o->use_adjoint, o->seed, kind, count};
	auto it = ctx->graphs.find(k);
	if (it != ctx->graphs.end()) {
		*out = it->second;
		*kernels = ctx->graph_kernels[k];
		return TDVMC_OK;
	}
	{
		const int ra = ensure_gbuf(ctx);  // gradient scratch of the forward and adjoint kernels
		if (ra) return ra;
	}
	cudaGraph_t g;
	CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
	const int64_t l0 = ctx->launches;
	int rc = run_stage_any(ctx, o, kind, count);
	cudaError_t e = cudaStreamEndCapture(ctx->st, &g);
	const int nk = (int)(ctx->launches - l0);
	ctx->launches = l0;  // counted when the graph runs
	if (rc) return rc;
	if (e != cudaSuccess) {
		ctx->err = cudaGetErrorString(e);
		return TDVMC_ERR_CUDA;
	}
	cudaGraphExec_t ex;
	CK(cudaGraphInstantiate(&ex, g, 0));
	cudaGraphDestroy(g);
	ctx->graphs[k] = ex;
	ctx->graph_kernels[k] = nk;
	*out = ex;
	*kernels = nk;
	return TDVMC_OK;
}

// Stage kind of the first stage of the next stored-sample step and the size of
// its refresh window.  UPDATE_SAMPLES_EVERY_NTH_STEP = 0 samples every walker
// each step (TDVMC.cpp:3654); otherwise every update_every-th step refreshes
// floor(nw * UPDATE_SAMPLES_PERCENT / 100) consecutive walkers
// (UpdateSamplesConsecutive, TDVMC.cpp:975-983, 3406-3408, 3665-3675).
void cs_plan(tdvmc_ctx* ctx, const tdvmc_step_opts* o, int* kind, int64_t* count) {
	int64_t c = (int64_t)std::floor((double)ctx->nw * o->update_percent / 100.0);
	c = std::max<int64_t>(0, std::min<int64_t>(c, ctx->nw));
	*count = 0;
	if (!ctx->cs_valid || o->update_every <= 0) *kind = kCsFull;
	else if (ctx->cs_steps % o->update_every == 0 && c > 0) {
		*kind = c >= ctx->nw ? kCsFull : kCsRefresh;
		if (*kind == kCsRefresh) *count = c;
	} else
		*kind = kCsReuse;
}

// Enqueues nsteps steps (graph replays) on the context's stream.
int enqueue_steps(tdvmc_ctx* ctx, const tdvmc_step_opts* o, int32_t nsteps) {
	int rc;
	if (!cs_ode(o->ode_solver)) {
		cudaGraphExec_t g;
		int nk = 0;
		if ((rc = get_graph(ctx, o, &g, &nk))) return rc;
		const int nst = stages_per_step(o->ode_solver);
		for (int s = 0; s < nsteps; s++)
			for (int k = 0; k < nst; k++) {
				CK(cudaGraphLaunch(g, ctx->st));
				ctx->launches += nk;
			}
		if (nsteps > 0 && o->moves_per_stage > 0) ctx->cs_valid = false;
		return TDVMC_OK;
	}
	if ((rc = cs_alloc(ctx))) return rc;
	cudaGraphExec_t gr;
	int nkr = 0;
	if ((rc = get_graph(ctx, o, &gr, &nkr, kCsReuse))) return rc;
	for (int s = 0; s < nsteps; s++) {
		int kind;
		int64_t cnt;
		cs_plan(ctx, o, &kind, &cnt);
		cudaGraphExec_t g0 = gr;
		int nk0 = nkr;
		if (kind != kCsReuse && (rc = get_graph(ctx, o, &g0, &nk0, kind, cnt))) return rc;
		CK(cudaGraphLaunch(g0, ctx->st));
		ctx->launches += nk0;
		for (int k = 1; k < stages_per_step(o->ode_solver); k++) {
			CK(cudaGraphLaunch(gr, ctx->st));
			ctx->launches += nkr;
		}
		if (kind == kCsFull) {
			ctx->cs_valid = true;
			ctx->cs_steps = 1;
			ctx->cs_last_count = ctx->nw;
		} else {
			ctx->cs_steps++;
			if (kind == kCsRefresh) ctx->cs_last_count = cnt;
		}
	}
	return TDVMC_OK;
}

template <typename T>
int copy_out(tdvmc_ctx* ctx, const void* dsrc, double* host, size_t count) {
	if (!host) return TDVMC_OK;
	std::vector<T> tmp(count);
	CK(cudaMemcpyAsync(tmp.data(), dsrc, count * sizeof(T), cudaMemcpyDeviceToHost, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	for (size_t i = 0; i < count; i++) host[i] = (double)tmp[i];
	return TDVMC_OK;
}

int copy_out_any(tdvmc_ctx* ctx, const void* d, double* h, size_t n) {
	return ctx->prec == TDVMC_PREC_FP64 ? copy_out<double>(ctx, d, h, n) : copy_out<float>(ctx, d, h, n);
}

void fill_stats(tdvmc_ctx* ctx, const std::vector<double>& m, int moves, tdvmc_stats* s) {
	const int P = ctx->sc.p;
	Cols1 c{P};
	s->n_walkers = ctx->nw;
	s->energy_re = m[c.ER()];
	s->energy_im = m[c.EI()];
	const int o = c.other();
	s->other[0] = m[o + 0];  // kineticR
	s->other[1] = m[o + 1];  // V_int
	s->other[2] = m[c.wf()];
	s->other[3] = m[c.lnpsi()];
	s->other[4] = m[o + 2];
	s->other[5] = m[o + 3];
	s->other[6] = m[o + 4];
	s->other[7] = m[o + 5];
	s->other[8] = m[o + 6];
	s->accept_rate = moves > 0 ? m[c.acc()] / (double)moves : 0.0;
}

int read_status(tdvmc_ctx* ctx, int32_t* status) {
	DynState d;
	CK(cudaMemcpyAsync(&d, ctx->dyn, sizeof(DynState), cudaMemcpyDeviceToHost, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	*status = d.status;
	if (d.status) {
		int32_t zero = 0;
		CK(cudaMemcpyAsync(&ctx->dyn->status, &zero, sizeof(int32_t), cudaMemcpyHostToDevice, ctx->st));
		CK(cudaStreamSynchronize(ctx->st));
	}
	return TDVMC_OK;
}

int status_code(int32_t st) {
	if (st & kStatusNonFinite) return TDVMC_ERR_NONFINITE;
	if (st & kStatusNotPD) return TDVMC_ERR_NOT_PD;
	return TDVMC_OK;
}

}  // namespace

extern "C" {

const char* tdvmc_status_string(int s) {
	switch (s) {
	case TDVMC_OK: return "ok";
	case TDVMC_ERR_ARG: return "invalid argument";
	case TDVMC_ERR_CUDA: return "CUDA error";
	case TDVMC_ERR_NOMEM: return "out of device memory";
	case TDVMC_ERR_STATE: return "invalid call order";
	case TDVMC_ERR_NOT_PD: return "S matrix not positive definite";
	case TDVMC_ERR_NONFINITE: return "non-finite parameters";
	}
	return "unknown status";
}

int tdvmc_create(const tdvmc_system_desc* d, tdvmc_ctx** out) {
	tdvmc_ctx* ctx = nullptr;
	if (!d || !out) return TDVMC_ERR_ARG;
	*out = nullptr;
	if (d->dim < 1 || d->dim > 3 || d->n < 2 || d->n > 1024 || d->p < 4 || d->p > kMaxP || d->n_walkers < 1 ||
	    !(d->box_length > 0) || (d->precision != TDVMC_PREC_FP64 && d->precision != TDVMC_PREC_MIXED) ||
	    d->n_walkers > 0x7fffffffLL)
		return TDVMC_ERR_ARG;
	if (d->n_user_knots > 0 && (d->user_knots == nullptr || d->n_user_knots != d->p)) return TDVMC_ERR_ARG;
	if (d->n_pot < 0 || d->n_pot > 5) return TDVMC_ERR_ARG;
	if (d->system_type != TDVMC_SYS_BOSONS_BULK && d->system_type != TDVMC_SYS_NU_BOSONS_BULK_PB &&
	    d->system_type != TDVMC_SYS_NU_BOSONS_BULK_PB_EXACT)
		return TDVMC_ERR_ARG;
	const bool pb = d->system_type != TDVMC_SYS_BOSONS_BULK;
	// NUBosonsBulkPB reads r_max from its knot vector before it builds default knots
	// (NUBosonsBulkPB.cpp:76, 91-97), and its potential is the square well (347-350)
	if (pb && (d->n_user_knots == 0 || d->pot_kind != TDVMC_POT_SQUARE)) return TDVMC_ERR_ARG;
	ctx = new tdvmc_ctx();
	tdvmc_ctx& c = *ctx;
	c.prec = d->precision;
	c.nw = d->n_walkers;
	c.pot.assign(d->pot, d->pot + 5);
	c.npot = d->n_pot;
	const int P = d->p;
	// knots: BosonsBulk.cpp:61-67 (uniform) or SetNodes mirroring (35-44)
	if (d->n_user_knots > 0) {
		const int K = d->n_user_knots;
		for (int i = 0; i < 3; i++) c.knots.push_back(-d->user_knots[3 - i]);
		for (int i = 0; i < K; i++) c.knots.push_back(d->user_knots[i]);
		for (int i = 0; i < 3; i++) c.knots.push_back(2.0 * d->user_knots[K - 1] - d->user_knots[K - 2 - i]);
		for (size_t i = 1; i < c.knots.size(); i++)
			if (!(c.knots[i] > c.knots[i - 1])) {
				delete ctx;
				return TDVMC_ERR_ARG;
			}
	} else {
		const double half = d->box_length / 2.0;
		for (int i = -3; i < P + 3; i++) c.knots.push_back(((double)i * half) / ((double)P - 1.0));
	}
	const int nk = (int)c.knots.size();
	SysConst& s = c.sc;
	s.n = d->n;
	s.dim = d->dim;
	s.p = P;
	s.ns = nk - 4;
	s.nbin = nk - 7;
	s.rmax = c.knots[nk - 4];
	s.L = d->box_length;
	s.Lr = 1.0 / d->box_length;
	s.hbar2_2m = d->hbar2_2m;
	s.pot_kind = d->pot_kind;
	s.mirror = d->system_type == TDVMC_SYS_NU_BOSONS_BULK_PB ? 1 : pb ? 2 : 0;
	// r_max below 1.5 L: the samplers' phantom slots (kPhantomBoxes) lie beyond it.
	// Mirrored distances 2 r_max - r stay non-negative for every pair (the largest
	// minimum-image distance is sqrt(dim) L / 2; a margin of 1e-5 covers rounding).
	if (s.ns - 2 != P || s.nbin > kMaxBins || !(s.rmax < 1.5 * s.L) ||
	    (pb && !(2.0 * s.rmax >= std::sqrt((double)s.dim) * s.L / 2.0 * (1.0 + 1e-5)))) {
		delete ctx;
		return TDVMC_ERR_ARG;
	}
	// local piece polynomials loc[j][q][c]: spline j+3-q on interval j (knot j+3)
	c.loc.assign((size_t)s.nbin * 16, 0.0);
	for (int j = 0; j < s.nbin; j++)
		for (int q = 0; q < 4; q++) piece_local(c.knots, j + 3 - q, j + 3, &c.loc[((size_t)j * 4 + q) * 4]);
	// boundary-condition fold (uniform factors: SplineFactory.cpp:423-439, 563-579)
	c.fold.assign((size_t)P * s.ns, 0.0);
	const double bcs[2][3] = {{0, 1, 0}, {1, 0, 1}};
	const double bce[2][3] = {{1, 0, 1}, {0, 1, 0}};
	for (int i = 0; i < 2; i++)
		for (int j = 0; j < 3; j++) c.fold[(size_t)i * s.ns + j] = bcs[i][j];
	for (int i = 2, sp = 3; i < P - 2; i++, sp++) c.fold[(size_t)i * s.ns + sp] = 1.0;
	for (int i = P - 2, idx = 0; i < P; i++, idx++)
		for (int j = 0; j < 3; j++) c.fold[(size_t)i * s.ns + s.ns - 3 + j] = bce[idx][j];
	if (pb) {
		// NUBosonsBulkPB::RefreshLocalOperators (NUBosonsBulkPB.cpp:219-228):
		// O_k = S_{k+1}, O_1 += S_0, O_{p-1} += S_{p+1} (the system declares a further
		// spline S_{p+2} that no pair ever fills)
		std::fill(c.fold.begin(), c.fold.end(), 0.0);
		for (int k = 0; k < P; k++) c.fold[(size_t)k * s.ns + k + 1] = 1.0;
		c.fold[(size_t)1 * s.ns + 0] += 1.0;
		c.fold[(size_t)(P - 1) * s.ns + s.ns - 1] += 1.0;
	}
	// interval geometry
	std::vector<double> kb(s.nbin), hv(s.nbin);
	double hmin = 1e300, hmaxw = 0.0;
	for (int j = 0; j < s.nbin; j++) {
		kb[j] = c.knots[j + 3];
		const double h = c.knots[j + 4] - c.knots[j + 3];
		hv[j] = 1.0 / h;
		hmin = std::min(hmin, h);
		hmaxw = std::max(hmaxw, h);
	}
	s.uniform = (hmaxw - hmin) <= 1e-12 * hmaxw ? 1 : 0;
	s.hinv = hv[0];
	s.hf = (float)s.hinv;
	s.hf_lo = (float)(s.hinv - (double)s.hf);
	// the FP32 distance of an FP32 pair is within about 2.5e-7 (relative) of its FP64
	// distance (the rounding of the differences and of r^2, the first-order box
	// remainder, the Newton-refined square root); the band of 1e-6 keeps a margin of
	// about four
	s.rcut_band = (float)(s.rmax * 1e-6);
	s.lc = (float)(-2.0 * (s.L - (double)(float)s.L));
	std::vector<int> lut;
	if (!s.uniform) {
		const double span = s.rmax - kb[0];
		double cell = hmin / 2.0;
		int ncell = (int)std::ceil(s.rmax / cell) + 1;
		if (ncell > kMaxLut || kb[0] < 0.0 || span <= 0) {
			delete ctx;
			return TDVMC_ERR_ARG;
		}
		s.ncell = ncell;
		s.cell_inv = 1.0 / cell;
		lut.resize(ncell);
		for (int ci = 0; ci < ncell; ci++) {
			const double r = ci * cell;
			int j = 0;
			while (j + 1 < s.nbin && kb[j + 1] <= r) j++;
			lut[ci] = j;
		}
	} else {
		s.ncell = 0;
		s.cell_inv = 0.0;
	}
	// sampler table: the nbin cubics, then the outer-pair constant
	s.ncoef = s.nbin + 1;

	cudaGetDevice(&c.device);
	cudaDeviceGetAttribute(&c.nsm, cudaDevAttrMultiProcessorCount, c.device);
	if (cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking) != cudaSuccess ||
	    cudaStreamCreateWithFlags(&c.st2, cudaStreamNonBlocking) != cudaSuccess) {
		tdvmc_destroy(ctx);
		return TDVMC_ERR_CUDA;
	}
	for (int k = 0; k < tdvmc_ctx::kMaxChunks; k++)
		if (cudaEventCreateWithFlags(&c.ev_s[k], cudaEventDisableTiming) != cudaSuccess) {
			tdvmc_destroy(ctx);
			return TDVMC_ERR_CUDA;
		}
	if (cudaEventCreateWithFlags(&c.ev_e, cudaEventDisableTiming) != cudaSuccess) {
		tdvmc_destroy(ctx);
		return TDVMC_ERR_CUDA;
	}
	// TDVMC_PIPELINE=k splits every sampling stage into k walker chunks (1 = off)
	if (const char* pl = std::getenv("TDVMC_PIPELINE"))
		c.pipeline = std::max(1, std::min(tdvmc_ctx::kMaxChunks, std::atoi(pl)));
	const size_t ts = tsize(c.prec);
	const int64_t nw = c.nw;
	const int np = 2 * P + 2;
	Cols1 cols{P};
	const int K1 = cols.count();
	// at most kReduce1MaxWalkers walkers per block: enough blocks for every walker
	c.nblk1 = (int)std::max<int64_t>(std::min<int64_t>(std::max<int64_t>(1, (nw + 31) / 32), 8 * (int64_t)c.nsm),
	                                 (nw + kReduce1MaxWalkers - 1) / kReduce1MaxWalkers);
	c.chunk2 = (int)std::max<int64_t>(1, std::min<int64_t>(128, (96 * 1024) / ((P + 2) * 8)));
	c.nblk2 = (int)((nw + c.chunk2 - 1) / c.chunk2);
	c.nblkS = gram_blocks(nw, c.nsm);
	{
		// S = Oc^T Oc on the tensor cores in mixed precision (TDVMC_GRAM=fp64 selects
		// the FP64 CUDA-core contraction instead)
		const char* g = std::getenv("TDVMC_GRAM");
		const bool want_tc = !(g && std::strcmp(g, "fp64") == 0);
		c.gram_tc = (c.prec == TDVMC_PREC_MIXED) && want_tc && gram_supported(P);
	}
	bool ok = true;
	auto A = [&](void** p, size_t bytes) {
		if (!ok) return;
		if (cudaMalloc(p, bytes) != cudaSuccess) ok = false;
	};
	A(&c.pos, (size_t)nw * d->dim * d->n * ts);
	A(&c.lnpsi, (size_t)nw * ts);
	A(&c.O, (size_t)nw * P * ts);
	A(&c.eloc, (size_t)nw * 2 * ts);
	A(&c.other7, (size_t)nw * 7 * ts);
	A(&c.dE, (size_t)nw * 2 * P * ts);
	A((void**)&c.acc, (size_t)nw * sizeof(int));
	A((void**)&c.base, np * sizeof(double));
	A((void**)&c.stage, np * sizeof(double));
	A((void**)&c.kdot, 4 * np * sizeof(double));
	A((void**)&c.rhs, np * sizeof(double));
	A((void**)&c.loc_d, c.loc.size() * sizeof(double));
	A((void**)&c.fold_d, c.fold.size() * sizeof(double));
	A(&c.coefU, (size_t)s.ncoef * 4 * ts);
	A(&c.coefC, (size_t)s.nbin * 12 * ts);
	A(&c.uout, 32);
	A(&c.kb, (size_t)s.nbin * ts);
	A(&c.hv, (size_t)s.nbin * ts);
	A(&c.locT, c.loc.size() * ts);
	A(&c.cs_piece, (size_t)s.nbin * kCsPiece * ts);
	A((void**)&c.lut, (size_t)std::max(1, s.ncell) * sizeof(int));
	A((void**)&c.part1, (size_t)c.nblk1 * K1 * sizeof(double));
	A((void**)&c.means1, K1 * sizeof(double));
	A((void**)&c.means0, K1 * sizeof(double));
	A((void**)&c.part2, (size_t)c.nblk2 * P * (P + 2) * sizeof(double));
	A((void**)&c.C2, (size_t)P * (P + 2) * sizeof(double));
	A((void**)&c.partS, (size_t)c.nblkS * P * P * sizeof(float));
	A((void**)&c.Sg, (size_t)P * P * sizeof(double));
	A((void**)&c.dyn, sizeof(DynState));
	A((void**)&c.chunk_starts, tdvmc_ctx::kMaxChunks * sizeof(int32_t));
	if (!ok) {
		tdvmc_destroy(ctx);
		return TDVMC_ERR_NOMEM;
	}
	// Local pieces as the FP32 kernels evaluate them.  Their local coordinate is
	// t_f = r hf - j (equal widths, hf = 1/h rounded to FP32) or (r - kb_f) hv_f with
	// the FP32-rounded interval tables; the true coordinate is the affine
	// t = a_j t_f + b_j, a_j = hv / hv_f, b_j = j (a_j - 1) or (kb_f - kb) hv.  The
	// pieces composed with that map (coefficients in t_f) keep the rounding of 1/h
	// and of the knots, a bias shared by every pair of an interval, out of the
	// spline values without an extra operation per pair; the derivatives in r are
	// hv_f d/dt_f.  FP64 contexts use the pieces as they are.
	c.locc = c.loc;
	if (c.prec == TDVMC_PREC_MIXED)
		for (int j = 0; j < s.nbin; j++) {
			double a, b;
			if (s.uniform) {
				a = s.hinv / (double)s.hf;
				b = (a - 1.0) * j;
			} else {
				a = hv[j] / (double)(float)hv[j];
				b = ((double)(float)kb[j] - kb[j]) * hv[j];
			}
			const double binom[4][4] = {{1, 0, 0, 0}, {1, 1, 0, 0}, {1, 2, 1, 0}, {1, 3, 3, 1}};
			for (int q = 0; q < 4; q++) {
				const double* l = &c.loc[((size_t)j * 4 + q) * 4];
				double* o = &c.locc[((size_t)j * 4 + q) * 4];
				for (int k = 0; k < 4; k++) {
					double v = 0.0;
					for (int cc = k; cc < 4; cc++) v += l[cc] * binom[cc][k] * std::pow(a, k) * std::pow(b, cc - k);
					o[k] = v;
				}
			}
		}
	// static tables
	std::vector<char> kbT(s.nbin * ts), hvT(s.nbin * ts), locT(c.loc.size() * ts);
	for (int j = 0; j < s.nbin; j++) {
		if (c.prec == TDVMC_PREC_FP64) {
			((double*)kbT.data())[j] = kb[j];
			((double*)hvT.data())[j] = hv[j];
		} else {
			((float*)kbT.data())[j] = (float)kb[j];
			((float*)hvT.data())[j] = (float)hv[j];
		}
	}
	for (size_t i = 0; i < c.loc.size(); i++) {
		if (c.prec == TDVMC_PREC_FP64) ((double*)locT.data())[i] = c.loc[i];
		else ((float*)locT.data())[i] = (float)c.locc[i];
	}
	// stored-sample piece table: dB/dr, B and d2B/dr2 of the four pieces per interval
	std::vector<double> piece((size_t)s.nbin * kCsPiece, 0.0);
	for (int j = 0; j < s.nbin; j++)
		for (int q = 0; q < 4; q++) {
			const double* l = &c.loc[((size_t)j * 4 + q) * 4];
			const double h = hv[j];
			double* pc = &piece[(size_t)j * kCsPiece];
			pc[3 * q + 0] = h * l[1];
			pc[3 * q + 1] = 2.0 * h * l[2];
			pc[3 * q + 2] = 3.0 * h * l[3];
			for (int cc = 0; cc < 4; cc++) pc[12 + 4 * q + cc] = l[cc];
			pc[28 + 2 * q + 0] = 2.0 * h * h * l[2];
			pc[28 + 2 * q + 1] = 6.0 * h * h * l[3];
		}
	{
		// equal widths: one row for all intervals when the rows agree to rounding
		double scale = 0.0;
		for (int k = 0; k < kCsPiece; k++) scale = std::max(scale, std::fabs(piece[k]));
		bool same = s.uniform != 0;
		for (int j = 1; same && j < s.nbin; j++)
			for (int k = 0; k < kCsPiece; k++)
				if (std::fabs(piece[(size_t)j * kCsPiece + k] - piece[k]) > 1e-12 * scale) same = false;
		c.cs_uni = same;
		for (int k = 0; k < kCsPiece; k++) c.cs_pu[k] = piece[k];
	}
	std::vector<char> pieceT(piece.size() * ts);
	for (size_t i = 0; i < piece.size(); i++) {
		if (c.prec == TDVMC_PREC_FP64) ((double*)pieceT.data())[i] = piece[i];
		else ((float*)pieceT.data())[i] = (float)piece[i];
	}
	DynState dy{};
	std::vector<int32_t> starts(tdvmc_ctx::kMaxChunks, 0);
	{
		const int K = (int)std::min<int64_t>(c.pipeline, nw);
		for (int k = 0; k < tdvmc_ctx::kMaxChunks; k++) starts[k] = (int32_t)(k < K ? nw * k / K : 0);
	}
	c.time = 0.0;
	apply_quench(ctx, dy.pa, dy.pb);
	std::vector<double> zeros((size_t)4 * np, 0.0);
	bool cp = cudaMemcpy(c.kb, kbT.data(), kbT.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
	          cudaMemcpy(c.hv, hvT.data(), hvT.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
	          cudaMemcpy(c.locT, locT.data(), locT.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
	          cudaMemcpy(c.cs_piece, pieceT.data(), pieceT.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
	          cudaMemcpy(c.loc_d, c.locc.data(), c.locc.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
	          cudaMemcpy(c.fold_d, c.fold.data(), c.fold.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
	          cudaMemcpy(c.dyn, &dy, sizeof(dy), cudaMemcpyHostToDevice) == cudaSuccess &&
	          cudaMemcpy(c.chunk_starts, starts.data(), starts.size() * sizeof(int32_t), cudaMemcpyHostToDevice) ==
	              cudaSuccess &&
	          cudaMemcpy(c.base, zeros.data(), np * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
	          cudaMemcpy(c.stage, zeros.data(), np * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
	          cudaMemcpy(c.kdot, zeros.data(), 4 * np * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
	          cudaMemset(c.acc, 0, (size_t)nw * sizeof(int)) == cudaSuccess &&
	          cudaMemset(c.dE, 0, (size_t)nw * 2 * P * ts) == cudaSuccess;
	if (cp && s.ncell > 0) cp = cudaMemcpy(c.lut, lut.data(), lut.size() * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess;
	if (!cp) {
		tdvmc_destroy(ctx);
		return TDVMC_ERR_CUDA;
	}
	// default tiles: a full warp per walker from 64 particles up
	c.tiles.sg = d->n >= 64 ? 32 : (d->n >= 24 ? 16 : 8);
	if (slots_for(d->n, c.tiles.sg) < 0) c.tiles.sg = 32;
	if (slots_for(d->n, c.tiles.sg) < 0) {
		tdvmc_destroy(ctx);
		return TDVMC_ERR_ARG;
	}
	c.tiles.eg = c.tiles.sg;
	// FP32 sampler with uniform knots: where a full warp per walker needs 11 register
	// slots, two walkers per warp (16 lanes, 22 slots) share each move's bookkeeping
	// (1.5 % faster at N = 343); the evaluation keeps the full warp
	if (c.prec == TDVMC_PREC_MIXED && c.sc.uniform && c.tiles.sg == 32 && slots_for(d->n, 32) == 11 &&
	    slots_for(d->n, 16) == 22)
		c.tiles.sg = 16;
	// NUBosonsBulkPB: its kernels are built for a full warp per walker
	if (pb) c.tiles.sg = c.tiles.eg = 32;
	// TDVMC_SAMPLE_LANES overrides the sampler's lanes per walker (8, 16 or 32)
	if (const char* sl = std::getenv("TDVMC_SAMPLE_LANES"); sl && !pb) {
		const int g = std::atoi(sl);
		if ((g == 8 || g == 16 || g == 32) && slots_for(d->n, g) > 0) c.tiles.sg = g;
	}
	c.tiles.sgpb = 128 / c.tiles.sg;
	c.tiles.egpb = c.tiles.eg == 32 ? 0 : 32 / c.tiles.eg;
	// TDVMC_EVAL_WALKERS_PER_BLOCK overrides the evaluation kernels' walkers per block
	if (const char* e = std::getenv("TDVMC_EVAL_WALKERS_PER_BLOCK"))
		c.tiles.egpb = std::max(1, std::min(128 / c.tiles.eg, std::atoi(e)));
	if (const char* h = std::getenv("TDVMC_HIST"); h && !pb) c.tiles.hist = std::max(0, std::min(2, std::atoi(h)));
	if (const char* wt = std::getenv("TDVMC_TEST_WAIT_NS")) c.wait_ns = (uint64_t)std::strtoull(wt, nullptr, 10);
	// TDVMC_SAMPLER=scalar selects the scalar FP32 sampler
	if (const char* sm = std::getenv("TDVMC_SAMPLER")) {
		c.packed_sampler = std::strcmp(sm, "scalar") != 0;
		c.shared_coords = std::strcmp(sm, "shared") == 0;
	}
	*out = ctx;
	return TDVMC_OK;
}

int tdvmc_destroy(tdvmc_ctx* ctx) {
	if (!ctx) return TDVMC_ERR_ARG;
	if (ctx->st) cudaStreamSynchronize(ctx->st);
	for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
	void* bufs[] = {ctx->pos, ctx->lnpsi, ctx->O, ctx->eloc, ctx->other7, ctx->dE, ctx->acc, ctx->base, ctx->stage,
	                ctx->kdot, ctx->rhs, ctx->loc_d, ctx->fold_d, ctx->coefU, ctx->coefC, ctx->uout, ctx->kb, ctx->hv,
	                ctx->locT, ctx->lut, ctx->part1, ctx->means1, ctx->means0, ctx->part2, ctx->C2, ctx->partS, ctx->Sg,
	                ctx->dyn, ctx->gramws, ctx->csD, ctx->csD2, ctx->csO, ctx->csV, ctx->csN, ctx->cs_piece, ctx->gbuf,
	                ctx->chunk_starts};
	for (void* b : bufs)
		if (b) cudaFree(b);
	if (ctx->st) cudaStreamDestroy(ctx->st);
	if (ctx->st2) cudaStreamDestroy(ctx->st2);
	for (int k = 0; k < tdvmc_ctx::kMaxChunks; k++)
		if (ctx->ev_s[k]) cudaEventDestroy(ctx->ev_s[k]);
	if (ctx->ev_e) cudaEventDestroy(ctx->ev_e);
	delete ctx;
	return TDVMC_OK;
}

int tdvmc_get_stream(tdvmc_ctx* ctx, void** stream) {
	if (!ctx || !stream) return TDVMC_ERR_ARG;
	*stream = (void*)ctx->st;
	return TDVMC_OK;
}

int tdvmc_set_time(tdvmc_ctx* ctx, double time) {
	if (!ctx) return TDVMC_ERR_ARG;
	ctx->time = time;
	double ab[2];
	apply_quench(ctx, ab[0], ab[1]);
	CK(cudaMemcpyAsync(ctx->dyn, ab, 2 * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	return TDVMC_OK;
}

int tdvmc_set_params(tdvmc_ctx* ctx, const double* uR, const double* uI, double phiR, double phiI) {
	if (!ctx || !uR || !uI) return TDVMC_ERR_ARG;
	const int P = ctx->sc.p;
	std::vector<double> v(2 * P + 2);
	std::copy(uR, uR + P, v.begin());
	std::copy(uI, uI + P, v.begin() + P);
	v[2 * P] = phiR;
	v[2 * P + 1] = phiI;
	CK(cudaMemcpyAsync(ctx->base, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
	CK(cudaMemcpyAsync(ctx->stage, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
	uint32_t zero = 0;
	CK(cudaMemcpyAsync(&ctx->dyn->stage, &zero, sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	return TDVMC_OK;
}

int tdvmc_get_params(tdvmc_ctx* ctx, double* uR, double* uI, double* phiR, double* phiI) {
	if (!ctx) return TDVMC_ERR_ARG;
	const int P = ctx->sc.p;
	std::vector<double> v(2 * P + 2);
	CK(cudaMemcpyAsync(v.data(), ctx->base, v.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	if (uR) std::copy(v.begin(), v.begin() + P, uR);
	if (uI) std::copy(v.begin() + P, v.begin() + 2 * P, uI);
	if (phiR) *phiR = v[2 * P];
	if (phiI) *phiI = v[2 * P + 1];
	return TDVMC_OK;
}

int tdvmc_set_walkers(tdvmc_ctx* ctx, const double* x, int64_t nw) {
	if (!ctx || !x || nw != ctx->nw) return TDVMC_ERR_ARG;
	const size_t cnt = (size_t)nw * ctx->sc.dim * ctx->sc.n;
	if (ctx->prec == TDVMC_PREC_FP64) {
		CK(cudaMemcpyAsync(ctx->pos, x, cnt * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
		CK(cudaStreamSynchronize(ctx->st));
	} else {
		std::vector<float> f(cnt);
		for (size_t i = 0; i < cnt; i++) f[i] = (float)x[i];
		CK(cudaMemcpyAsync(ctx->pos, f.data(), cnt * sizeof(float), cudaMemcpyHostToDevice, ctx->st));
		CK(cudaStreamSynchronize(ctx->st));
	}
	ctx->have_walkers = true;
	ctx->cs_valid = false;
	return TDVMC_OK;
}

int tdvmc_get_walkers(tdvmc_ctx* ctx, double* x, int64_t nw) {
	if (!ctx || !x || nw != ctx->nw) return TDVMC_ERR_ARG;
	return copy_out_any(ctx, ctx->pos, x, (size_t)nw * ctx->sc.dim * ctx->sc.n);
}

int tdvmc_sample(tdvmc_ctx* ctx, int32_t moves, double mc_step, uint64_t seed, uint32_t pass, int64_t* accepted) {
	if (!ctx || moves < 0) return TDVMC_ERR_ARG;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	CK(cudaMemcpyAsync(&ctx->dyn->pass, &pass, sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->st));
	int rc = ctx->prec == TDVMC_PREC_FP64 ? launch_prep<double>(ctx) : launch_prep<float>(ctx);
	if (rc) return rc;
	rc = ctx->prec == TDVMC_PREC_FP64 ? launch_sample<double>(ctx, moves, mc_step, seed)
	                                  : launch_sample<float>(ctx, moves, mc_step, seed);
	if (rc) return rc;
	if (moves > 0) ctx->cs_valid = false;
	ctx->last_moves = moves;
	std::vector<int> a((size_t)ctx->nw);
	CK(cudaMemcpyAsync(a.data(), ctx->acc, a.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	if (accepted) {
		int64_t t = 0;
		for (int v : a) t += v;
		*accepted = t;
	}
	return TDVMC_OK;
}

static int eval_common(tdvmc_ctx* ctx, bool adj) {
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	{
		const int ra = ensure_gbuf(ctx);
		if (ra) return ra;
	}
	int rc = ctx->prec == TDVMC_PREC_FP64 ? launch_prep<double>(ctx) : launch_prep<float>(ctx);
	if (rc) return rc;
	rc = ctx->prec == TDVMC_PREC_FP64 ? launch_eloc<double>(ctx, adj) : launch_eloc<float>(ctx, adj);
	if (rc) return rc;
	ctx->have_eval = true;
	ctx->last_adj = adj;
	return TDVMC_OK;
}

int tdvmc_eval_local(tdvmc_ctx* ctx, double* lnpsi, double* O, double* eloc, double* other7) {
	if (!ctx) return TDVMC_ERR_ARG;
	int rc = eval_common(ctx, false);
	if (rc) return rc;
	const size_t nw = (size_t)ctx->nw;
	if ((rc = copy_out_any(ctx, ctx->lnpsi, lnpsi, nw))) return rc;
	if ((rc = copy_out_any(ctx, ctx->O, O, nw * ctx->sc.p))) return rc;
	if ((rc = copy_out_any(ctx, ctx->eloc, eloc, nw * 2))) return rc;
	if ((rc = copy_out_any(ctx, ctx->other7, other7, nw * 7))) return rc;
	CK(cudaStreamSynchronize(ctx->st));
	return TDVMC_OK;
}

int tdvmc_store_samples(tdvmc_ctx* ctx) {
	if (!ctx) return TDVMC_ERR_ARG;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	int rc = cs_alloc(ctx);
	if (rc) return rc;
	rc = ctx->prec == TDVMC_PREC_FP64 ? launch_cs_store<double>(ctx, ctx->nw, nullptr)
	                                  : launch_cs_store<float>(ctx, ctx->nw, nullptr);
	if (rc) return rc;
	CK(cudaStreamSynchronize(ctx->st));
	ctx->cs_valid = true;
	ctx->cs_steps = 0;
	return TDVMC_OK;
}

int tdvmc_eval_stored(tdvmc_ctx* ctx, double* lnpsi, double* O, double* eloc, double* other7, double* dE) {
	if (!ctx) return TDVMC_ERR_ARG;
	if (!ctx->cs_valid) return TDVMC_ERR_STATE;
	const bool adj = dE != nullptr;
	int rc = ctx->prec == TDVMC_PREC_FP64 ? launch_cs_eval<double>(ctx, adj) : launch_cs_eval<float>(ctx, adj);
	if (rc) return rc;
	ctx->have_eval = true;
	ctx->last_adj = adj;
	const size_t nw = (size_t)ctx->nw;
	if ((rc = copy_out_any(ctx, ctx->lnpsi, lnpsi, nw))) return rc;
	if ((rc = copy_out_any(ctx, ctx->O, O, nw * ctx->sc.p))) return rc;
	if ((rc = copy_out_any(ctx, ctx->eloc, eloc, nw * 2))) return rc;
	if ((rc = copy_out_any(ctx, ctx->other7, other7, nw * 7))) return rc;
	if (adj && (rc = copy_out_any(ctx, ctx->dE, dE, nw * 2 * ctx->sc.p))) return rc;
	CK(cudaStreamSynchronize(ctx->st));
	return TDVMC_OK;
}

int tdvmc_observables(tdvmc_ctx* ctx, int32_t gr_bins, int32_t nshell, const int32_t* shell_off, const double* kvec,
                      double* gr, int32_t* gr_count, double* sk) {
	if (!ctx || gr_bins < 1 || gr_bins > 8192 || nshell < 0 || !gr || !gr_count) return TDVMC_ERR_ARG;
	if (nshell > 0 && (!shell_off || !kvec || !sk)) return TDVMC_ERR_ARG;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	const SysConst& s = ctx->sc;
	const int D = s.dim, N = s.n;
	const int nvec = nshell > 0 ? shell_off[nshell] : 0;
	if (nshell > 0) {
		if (shell_off[0] != 0) return TDVMC_ERR_ARG;
		for (int k = 0; k < nshell; k++)
			if (shell_off[k + 1] < shell_off[k]) return TDVMC_ERR_ARG;
		if (nvec > 4096) return TDVMC_ERR_ARG;
	}
	// grid of BosonsBulk.cpp:145 (Grid::Init: count = (max - min) / spacing, truncated)
	const double spacing = s.rmax / gr_bins;
	const int count = (int)((s.rmax - 0.0) / spacing);
	std::vector<double> scale(std::max(count, 1));
	for (int i = 0; i < count; i++) {
		if (D == 1) scale[i] = spacing;
		else if (D == 3) scale[i] = 4.0 * M_PI * std::pow(spacing * (i + 1), 3.0) / 3.0;
		else scale[i] = M_PI * std::pow(spacing * (i + 1), 2.0);
	}
	if (D > 1)
		for (int i = count - 1; i > 0; i--) scale[i] = scale[i] - scale[i - 1];
	// NUBosonsBulkPB adds 1.0 per pair (NUBosonsBulkPB.cpp:602-612)
	const double weight = s.mirror ? 1.0 : 1.0 / ((double)(N - 1)) * D;
	// k vectors padded to 3 components, in the working precision
	const bool f64 = ctx->prec == TDVMC_PREC_FP64;
	const size_t ts = tsize(ctx->prec);
	std::vector<char> kv((size_t)std::max(nvec, 1) * 3 * ts, 0);
	for (int v = 0; v < nvec; v++)
		for (int a = 0; a < 3; a++) {
			const double x = a < D ? kvec[(size_t)v * D + a] : 0.0;
			if (f64) ((double*)kv.data())[v * 3 + a] = x;
			else ((float*)kv.data())[v * 3 + a] = (float)x;
		}
	void *d_k = nullptr, *d_off = nullptr, *d_cnt = nullptr, *d_sk = nullptr;
	auto release = [&]() {
		void* b[] = {d_k, d_off, d_cnt, d_sk};
		for (void* x : b)
			if (x) cudaFree(x);
	};
	const size_t skn = (size_t)ctx->nw * std::max(nshell, 1);
	if (cudaMalloc(&d_k, kv.size()) != cudaSuccess || cudaMalloc(&d_off, (size_t)(nshell + 1) * sizeof(int)) != cudaSuccess ||
	    cudaMalloc(&d_cnt, (size_t)count * sizeof(unsigned long long) + 8) != cudaSuccess ||
	    cudaMalloc(&d_sk, skn * sizeof(double)) != cudaSuccess) {
		release();
		cudaGetLastError();
		return TDVMC_ERR_NOMEM;
	}
	std::vector<int> off(nshell + 1, 0);
	for (int k = 0; k <= nshell && nshell > 0; k++) off[k] = shell_off[k];
	int rc = TDVMC_OK;
	const int threads = 128, wpb = threads / 32;
	const size_t smem = f64 ? obs_smem_bytes<double>(N, count, nvec, wpb) : obs_smem_bytes<float>(N, count, nvec, wpb);
	const void* fn = f64 ? (const void*)k_observables<double> : (const void*)k_observables<float>;
	if (smem > 220 * 1024) rc = TDVMC_ERR_ARG;
	if (!rc) {
		bool ok = cudaMemcpyAsync(d_k, kv.data(), kv.size(), cudaMemcpyHostToDevice, ctx->st) == cudaSuccess &&
		          cudaMemcpyAsync(d_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->st) ==
		              cudaSuccess &&
		          cudaMemsetAsync(d_cnt, 0, (size_t)count * sizeof(unsigned long long) + 8, ctx->st) == cudaSuccess &&
		          cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
		if (!ok) rc = TDVMC_ERR_CUDA;
	}
	if (!rc) {
		const int grid = grid_for(ctx, fn, threads, smem, ctx->nw, wpb);
		if (f64)
			k_observables<double><<<grid, threads, smem, ctx->st>>>(
			    s, (const double*)ctx->pos, ctx->nw, count, spacing, (const double*)d_k, nvec, (const int*)d_off,
			    nshell, (unsigned long long*)d_cnt, (double*)d_sk);
		else
			k_observables<float><<<grid, threads, smem, ctx->st>>>(
			    s, (const float*)ctx->pos, ctx->nw, count, spacing, (const float*)d_k, nvec, (const int*)d_off, nshell,
			    (unsigned long long*)d_cnt, (double*)d_sk);
		ctx->launches++;
		if (cudaGetLastError() != cudaSuccess) rc = TDVMC_ERR_CUDA;
	}
	std::vector<unsigned long long> cnt(std::max(count, 1));
	std::vector<double> skw(nshell > 0 ? skn : 0);
	if (!rc) {
		bool ok = cudaMemcpyAsync(cnt.data(), d_cnt, (size_t)count * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
		                          ctx->st) == cudaSuccess;
		if (ok && nshell > 0)
			ok = cudaMemcpyAsync(skw.data(), d_sk, skn * sizeof(double), cudaMemcpyDeviceToHost, ctx->st) == cudaSuccess;
		ok = ok && cudaStreamSynchronize(ctx->st) == cudaSuccess;
		if (!ok) rc = TDVMC_ERR_CUDA;
	}
	release();
	if (rc) return rc;
	// mean over walkers; each walker is one sample of the reference's running mean
	const double inv = 1.0 / (double)ctx->nw;
	for (int b = 0; b < count; b++) gr[b] = (double)cnt[b] * (weight / scale[b]) * inv;
	*gr_count = count;
	for (int k = 0; k < nshell; k++) {
		double acc = 0.0;
		for (int64_t w = 0; w < ctx->nw; w++) acc += skw[(size_t)w * nshell + k];
		sk[k] = acc * inv;
	}
	return TDVMC_OK;
}

int tdvmc_eval_local_adjoint(tdvmc_ctx* ctx, double* dE) {
	if (!ctx) return TDVMC_ERR_ARG;
	int rc = eval_common(ctx, true);
	if (rc) return rc;
	if ((rc = copy_out_any(ctx, ctx->dE, dE, (size_t)ctx->nw * 2 * ctx->sc.p))) return rc;
	CK(cudaStreamSynchronize(ctx->st));
	return TDVMC_OK;
}

int tdvmc_reduce_stats(tdvmc_ctx* ctx, tdvmc_stats* stats, double* O_mean, double* S, double* cov_OER,
                       double* cov_OEI, double* dE_mean) {
	if (!ctx) return TDVMC_ERR_ARG;
	if (!ctx->have_eval) return TDVMC_ERR_STATE;
	int rc = ctx->prec == TDVMC_PREC_FP64 ? launch_reduce<double>(ctx, ctx->last_adj)
	                                      : launch_reduce<float>(ctx, ctx->last_adj);
	if (rc) return rc;
	const int P = ctx->sc.p;
	Cols1 c{P};
	std::vector<double> m(c.count()), c2((size_t)P * (P + 2)), sg((size_t)P * P);
	CK(cudaMemcpyAsync(m.data(), ctx->means1, m.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
	CK(cudaMemcpyAsync(c2.data(), ctx->C2, c2.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
	CK(cudaMemcpyAsync(sg.data(), ctx->Sg, sg.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	const bool tc = ctx->gram_tc;
	if (stats) {
		fill_stats(ctx, m, ctx->last_moves, stats);
		stats->status = 0;
	}
	for (int k = 0; k < P; k++) {
		if (O_mean) O_mean[k] = m[k];
		if (cov_OER) cov_OER[k] = c2[(size_t)k * (P + 2) + P];
		if (cov_OEI) cov_OEI[k] = c2[(size_t)k * (P + 2) + P + 1];
		if (S)
			for (int l = 0; l < P; l++) S[(size_t)k * P + l] = tc ? sg[(size_t)k * P + l] : c2[(size_t)k * (P + 2) + l];
		if (dE_mean) {
			dE_mean[2 * k] = ctx->last_adj ? m[c.dE() + 2 * k] : 0.0;
			dE_mean[2 * k + 1] = ctx->last_adj ? m[c.dE() + 2 * k + 1] : 0.0;
		}
	}
	return TDVMC_OK;
}

int tdvmc_tdvp_rhs(tdvmc_ctx* ctx, int32_t imag, int32_t pre, int32_t lin, double* uDotR, double* uDotI,
                   double* phiDotR, double* phiDotI) {
	if (!ctx || (lin != 0 && lin != 1)) return TDVMC_ERR_ARG;
	if (!ctx->have_eval) return TDVMC_ERR_STATE;
	int rc = ctx->prec == TDVMC_PREC_FP64 ? launch_solve<double>(ctx, imag, pre, lin, 0, 0, 0.0)
	                                      : launch_solve<float>(ctx, imag, pre, lin, 0, 0, 0.0);
	if (rc) return rc;
	const int P = ctx->sc.p;
	std::vector<double> v(2 * P + 2);
	CK(cudaMemcpyAsync(v.data(), ctx->rhs, v.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	if (uDotR) std::copy(v.begin(), v.begin() + P, uDotR);
	if (uDotI) std::copy(v.begin() + P, v.begin() + 2 * P, uDotI);
	if (phiDotR) *phiDotR = v[2 * P];
	if (phiDotI) *phiDotI = v[2 * P + 1];
	int32_t st = 0;
	if ((rc = read_status(ctx, &st))) return rc;
	return status_code(st);
}

int tdvmc_run_steps(tdvmc_ctx* ctx, const tdvmc_step_opts* o, int32_t nsteps, tdvmc_stats* stats) {
	if (!ctx || nsteps < 0) return TDVMC_ERR_ARG;
	int rc = check_opts(o);
	if (rc) return rc;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	if ((rc = enqueue_steps(ctx, o, nsteps))) return rc;
	ctx->have_eval = true;
	ctx->last_adj = o->use_adjoint != 0;
	ctx->last_moves = o->moves_per_stage;
	int32_t st = 0;
	if (stats) {
		const int P = ctx->sc.p;
		Cols1 c{P};
		std::vector<double> m(c.count());
		CK(cudaMemcpyAsync(m.data(), ctx->means0, m.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
		CK(cudaStreamSynchronize(ctx->st));
		fill_stats(ctx, m, o->moves_per_stage, stats);
		// stored samples: the rate of the walkers the last refresh moved
		if (cs_ode(o->ode_solver) && ctx->cs_last_count > 0)
			stats->accept_rate *= (double)ctx->nw / (double)ctx->cs_last_count;
	}
	if ((rc = read_status(ctx, &st))) return rc;
	if (stats) stats->status = status_code(st);
	return status_code(st);
}

int tdvmc_get_step_operators(tdvmc_ctx* ctx, double* O_mean) {
	if (!ctx || !O_mean) return TDVMC_ERR_ARG;
	CK(cudaMemcpyAsync(O_mean, ctx->means0, ctx->sc.p * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	return TDVMC_OK;
}

int tdvmc_step(tdvmc_ctx* ctx, const tdvmc_step_opts* o, tdvmc_stats* stats) {
	return tdvmc_run_steps(ctx, o, 1, stats);
}

int tdvmc_time_steps(tdvmc_ctx* ctx, const tdvmc_step_opts* o, int32_t nsteps, float* ms) {
	if (!ctx || !ms || nsteps < 0) return TDVMC_ERR_ARG;
	int rc = check_opts(o);
	if (rc) return rc;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	if (cs_ode(o->ode_solver)) {
		// build the graphs (and the store) outside the timed region
		if ((rc = cs_alloc(ctx))) return rc;
		cudaGraphExec_t g;
		int nk;
		int kind;
		int64_t cnt;
		cs_plan(ctx, o, &kind, &cnt);
		if ((rc = get_graph(ctx, o, &g, &nk, kCsReuse))) return rc;
		if (kind != kCsReuse && (rc = get_graph(ctx, o, &g, &nk, kind, cnt))) return rc;
	} else {
		cudaGraphExec_t g;
		int nk;
		if ((rc = get_graph(ctx, o, &g, &nk))) return rc;
	}
	cudaEvent_t e0, e1;
	CK(cudaEventCreate(&e0));
	CK(cudaEventCreate(&e1));
	CK(cudaStreamSynchronize(ctx->st));
	CK(cudaEventRecord(e0, ctx->st));
	if ((rc = enqueue_steps(ctx, o, nsteps))) return rc;
	CK(cudaEventRecord(e1, ctx->st));
	CK(cudaEventSynchronize(e1));
	CK(cudaEventElapsedTime(ms, e0, e1));
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	ctx->have_eval = true;
	ctx->last_adj = o->use_adjoint != 0;
	ctx->last_moves = o->moves_per_stage;
	return TDVMC_OK;
}

int tdvmc_profile_stage(tdvmc_ctx* ctx, const tdvmc_step_opts* o, float* ms, const char** names, int32_t* count) {
	if (!ctx || !ms || !count) return TDVMC_ERR_ARG;
	int rc = check_opts(o);
	if (rc) return rc;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	std::vector<cudaEvent_t> ev;
	std::vector<const char*> nm;
	cudaEvent_t e0;
	CK(cudaEventCreate(&e0));
	CK(cudaStreamSynchronize(ctx->st));
	CK(cudaEventRecord(e0, ctx->st));
	if ((rc = ensure_gbuf(ctx))) return rc;
	ctx->prof = &ev;
	ctx->prof_names = &nm;
	if (cs_ode(o->ode_solver)) {
		// one first stage of the next stored-sample step (the store is not advanced)
		int kind;
		int64_t cnt;
		rc = cs_alloc(ctx);
		if (!rc) {
			cs_plan(ctx, o, &kind, &cnt);
			rc = run_stage_any(ctx, o, kind, cnt);
			if (!rc && kind == kCsFull) {
				ctx->cs_valid = true;
				ctx->cs_steps = 0;
			}
		}
	} else {
		rc = run_stage_any(ctx, o);
		if (o->moves_per_stage > 0) ctx->cs_valid = false;
	}
	ctx->prof = nullptr;
	ctx->prof_names = nullptr;
	if (!rc) {
		// the stage's solve left the context inside a step (the next stage's parameters
		// and stage index): back to the step boundary, so that the next step starts at
		// stage 0 from the unchanged base parameters
		const uint32_t zero = 0;
		const size_t pb = (size_t)(2 * ctx->sc.p + 2) * sizeof(double);
		if (cudaMemcpyAsync(ctx->stage, ctx->base, pb, cudaMemcpyDeviceToDevice, ctx->st) != cudaSuccess ||
		    cudaMemcpyAsync(&ctx->dyn->stage, &zero, sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->st) != cudaSuccess)
			rc = TDVMC_ERR_CUDA;
	}
	cudaError_t se = cudaStreamSynchronize(ctx->st);
	int nk = 0;
	cudaEvent_t prev = e0;
	for (size_t i = 0; i < ev.size() && nk < 16; i++, nk++) {
		float t = 0.f;
		cudaEventElapsedTime(&t, prev, ev[i]);
		ms[nk] = t;
		if (names) names[nk] = nm[i];
		prev = ev[i];
	}
	for (auto e : ev) cudaEventDestroy(e);
	cudaEventDestroy(e0);
	*count = nk;
	if (rc) return rc;
	CK(se);
	ctx->have_eval = true;
	ctx->last_adj = o->use_adjoint != 0;
	ctx->last_moves = o->moves_per_stage;
	return TDVMC_OK;
}

int tdvmc_autotune(tdvmc_ctx* ctx, int32_t moves, double mc_step) {
	if (!ctx || moves < 1) return TDVMC_ERR_ARG;
	if (!ctx->have_walkers) return TDVMC_ERR_STATE;
	// every candidate is timed twice (the second time counts) on the current walkers,
	// which are restored after each sampling candidate; on any error the context keeps
	// its starting tiles, and the copy and the events are released on every path
	const size_t bytes = (size_t)ctx->nw * ctx->sc.dim * ctx->sc.n * tsize(ctx->prec);
	const Tiles start = ctx->tiles;
	Tiles best = start;
	float best_s = 1e30f, best_e = 1e30f;
	void* save = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	int rc = TDVMC_OK;
	auto timed = [&](auto&& launch, float& ms) -> int {
		if (cudaEventRecord(e0, ctx->st) != cudaSuccess) return TDVMC_ERR_CUDA;
		const int r = launch();
		if (cudaEventRecord(e1, ctx->st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
			return TDVMC_ERR_CUDA;
		if (r) return r;
		return cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess ? TDVMC_OK : TDVMC_ERR_CUDA;
	};
	do {
		if (cudaMalloc(&save, bytes) != cudaSuccess) {
			save = nullptr;
			cudaGetLastError();
			rc = TDVMC_ERR_NOMEM;
			break;
		}
		if (cudaMemcpyAsync(save, ctx->pos, bytes, cudaMemcpyDeviceToDevice, ctx->st) != cudaSuccess ||
		    cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
			rc = TDVMC_ERR_CUDA;
			break;
		}
		if ((rc = ensure_gbuf(ctx))) break;
		const int n = ctx->sc.n;
		for (int G : {8, 16, 32}) {
			if (slots_for(n, G) < 0 || (G > 8 && n < G / 2)) continue;
			for (int gpb : {1, 2, 4, 8}) {
				if (G * gpb > 128) continue;
				ctx->tiles.sg = G;
				ctx->tiles.sgpb = gpb;
				if ((rc = ctx->prec == TDVMC_PREC_FP64 ? launch_prep<double>(ctx) : launch_prep<float>(ctx))) break;
				float ms = 0.f;
				for (int rep = 0; rep < 2 && !rc; rep++) {
					rc = timed([&] {
						return ctx->prec == TDVMC_PREC_FP64 ? launch_sample<double>(ctx, moves, mc_step, 7)
						                                    : launch_sample<float>(ctx, moves, mc_step, 7);
					}, ms);
					if (!rc && cudaMemcpyAsync(ctx->pos, save, bytes, cudaMemcpyDeviceToDevice, ctx->st) != cudaSuccess)
						rc = TDVMC_ERR_CUDA;
				}
				if (rc == TDVMC_ERR_ARG) {  // no kernel for this tile: not a candidate
					rc = TDVMC_OK;
					continue;
				}
				if (rc) break;
				if (ms < best_s) {
					best_s = ms;
					best.sg = G;
					best.sgpb = gpb;
				}
			}
			if (rc) break;
			for (int gpb : {0, 1, 2, 4})
				for (int hist : {0, 1, 2}) {
					if (G * gpb > 128 || (G != 32 && hist != 0) || rc) continue;
					ctx->tiles.eg = G;
					ctx->tiles.egpb = gpb;
					ctx->tiles.hist = hist;
					const size_t smem = ctx->prec == TDVMC_PREC_FP64 ? eloc_smem<double>(ctx, G, gpb, true)
					                                                 : eloc_smem<float>(ctx, G, gpb, true);
					if (smem > 220 * 1024) continue;
					float ms = 0.f;
					for (int rep = 0; rep < 2 && !rc; rep++)
						rc = timed([&] {
							return ctx->prec == TDVMC_PREC_FP64 ? launch_eloc<double>(ctx, true)
							                                    : launch_eloc<float>(ctx, true);
						}, ms);
					if (rc == TDVMC_ERR_ARG) {
						rc = TDVMC_OK;
						continue;
					}
					if (!rc && ms < best_e) {
						best_e = ms;
						best.eg = G;
						best.egpb = gpb;
						best.hist = hist;
					}
				}
			if (rc) break;
		}
	} while (false);
	if (save) {
		cudaMemcpyAsync(ctx->pos, save, bytes, cudaMemcpyDeviceToDevice, ctx->st);
		cudaStreamSynchronize(ctx->st);
		cudaFree(save);
	}
	if (e0) cudaEventDestroy(e0);
	if (e1) cudaEventDestroy(e1);
	ctx->tiles = rc ? start : best;
	for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
	ctx->graphs.clear();
	ctx->graph_kernels.clear();
	ctx->have_eval = false;
	if (!rc && cudaStreamSynchronize(ctx->st) != cudaSuccess) rc = TDVMC_ERR_CUDA;
	return rc;
}

int tdvmc_get_tiles(tdvmc_ctx* ctx, int32_t* sl, int32_t* sw, int32_t* el, int32_t* ew) {
	if (!ctx) return TDVMC_ERR_ARG;
	if (sl) *sl = ctx->tiles.sg;
	if (sw) *sw = ctx->tiles.sgpb;
	if (el) *el = ctx->tiles.eg;
	if (ew) *ew = ctx->tiles.egpb;
	return TDVMC_OK;
}

int64_t tdvmc_launch_count(tdvmc_ctx* ctx) { return ctx ? ctx->launches : -1; }

}  // extern "C"
