// Correlated-sampling reuse: per-walker data that does not depend on the
// variational parameters, stored once per sample and re-evaluated at other
// parameters without resampling (BosonsBulk::FillCorrelatedSamplingData and
// CalculateExpectationValues(ICorrelatedSamplingData*), BosonsBulk.cpp:468-472,
// 675-681; CSDataBulkSplines.h:9-16; used by CalculateNextParametersRK4ReuseSamples,
// TDVMC.cpp:2037-2103, and UpdateExpectationValuesForGivenSamples, 1222-1293).
//
// Stored per walker, at spline level (s = 0..ns-1, before the boundary fold):
//   D[s][a][n] = sum_{i != n, r <= r_max} B_s'(r_ni) (x_n - x_i)_a / r_ni
//                chunk-major: particle n at chunk n / 32, column n % 32, each chunk
//                one contiguous block [3 s + a][32] (n padded to npad = n rounded
//                up to 32; the padding is zero)
//   D2[s]      = sum_n sum_{i != n, r <= r_max} (B_s''(r_ni) + (D-1)/r_ni B_s'(r_ni))
//   O[k]       = BC-folded sum_{i < n, r <= r_max} B_s(r_ni)
//   V          = pair potential over i < n, r <= r_max;  n_out = #pairs beyond r_max
// With per-spline complex weights w_s = sum_k alpha_k fold[k][s]:
//   G_n = sum_s w_s D[s][.][n],  sum_n L_n = sum_s w_s D2[s],
// which gives the same local energy, kinetic sums and adjoint as k_eloc.
#pragma once

#include "common.cuh"
#include "k_eloc.cuh"

namespace tdvmc {

// piece table per knot interval j (36 values): for q = 0..3 (spline j+3-q)
//   [0..11]  h l1, 2h l2, 3h l3        (dB/dr = a0 + t (a1 + t a2))
//   [12..27] l0, l1, l2, l3            (B in the local coordinate t)
//   [28..35] 2h^2 l2, 6h^2 l3          (d2B/dr2 = c0 + t c1)
constexpr int kCsPiece = 36;
// Row stride of the piece table in shared memory: odd, so that lanes reading the
// same entry of different intervals hit different banks (up to 32 intervals)
constexpr int kCsPieceS = 37;

__host__ __device__ inline int cs_npad(int n) { return (n + 31) & ~31; }
// offset of D[e = 3 s + a][n] within one walker's block (ne = 3 ns rows)
__host__ __device__ inline size_t cs_doff(int ne, int e, int n) {
	return ((size_t)(n >> 5) * ne + e) * 32 + (n & 31);
}

// Shared memory of k_cs_store.
//   CTA:   piece[nbin][37] (36 used) | kb[nbin] | hv[nbin] | lut[ncell]
//   group: xs[n] | drow[ns*3*G] | oacc[ns*G] | d2acc[ns*G]   (lane-private columns)
template <typename T>
__host__ __device__ inline size_t cs_cta_bytes(int nbin, int ncell) {
	size_t b = (size_t)nbin * kCsPieceS * sizeof(T) + 2 * (size_t)nbin * sizeof(T) + (size_t)ncell * sizeof(int);
	return (b + 31) & ~(size_t)31;
}
template <typename T>
__host__ __device__ inline size_t cs_group_bytes(int n, int ns, int G) {
	size_t b = (size_t)n * sizeof(Q4<T>) + (size_t)ns * 5 * G * sizeof(T);
	return (b + 31) & ~(size_t)31;
}

// With equal interval widths every interval has the same piece row (the
// B-spline basis is translation invariant); it is passed as a kernel parameter,
// so the polynomial evaluations take their coefficients from the constant bank.
template <typename T> struct CsPieceRow {
	T c[kCsPiece];
};

// Geometry of one (row, partner) pair: minimum-image difference, distance,
// interval and local coordinate (no shared-memory writes, so the geometry of
// several partners can be computed before any of their accumulations).
template <typename T> struct CsGeom {
	T dx, dy, dz, r, rinv, t, sr;
	int j;
	bool in, out;  // within r_max (and not the self pair); beyond r_max
};
// FP32: r <= r_max from the FP32 distance; nearmin collects |r - r_max|, and the
// pairs within rounding of r_max are decided again in FP64 after the slot
// (cs_fix_slot).  force: the pair as within r_max whatever r is (the fix-up).
// MIR: the distances of NUBosonsBulkPB (mirror_r).
template <typename T, bool MIR = false>
__device__ __forceinline__ CsGeom<T> cs_geom(const SysConst& sc, const Q4<T>& xr, const Q4<T>& xi, bool ok,
                                             const T* __restrict__ kb, const T* __restrict__ hv,
                                             const int* __restrict__ lut, T& nearmin, bool force = false) {
	CsGeom<T> g;
	const T L = (T)sc.L, Lr = (T)sc.Lr;
	if constexpr (sizeof(T) == 4) {
		// FP32: the evaluation kernels' distance (box remainder in r^2, one Newton step)
		float dx = xr.x - xi.x, dy = xr.y - xi.y, dz = xr.z - xi.z;
		const float r2 = pair_r2_f32(sc.lc, L, Lr, dx, dy, dz);
		g.dx = dx;
		g.dy = dy;
		g.dz = dz;
		g.rinv = rsqrt_(r2);
		g.r = pair_r_newton(r2, g.rinv);
	} else {
		g.dx = nic(xr.x - xi.x, L, Lr);
		g.dy = nic(xr.y - xi.y, L, Lr);
		g.dz = nic(xr.z - xi.z, L, Lr);
		const T r2 = fma(g.dz, g.dz, fma(g.dy, g.dy, g.dx * g.dx));
		g.rinv = rsqrt_(r2);
		g.r = r2 * g.rinv;
	}
	bool cut;
	if constexpr (MIR) {
		// NUBosonsBulkPB: the mirrored distance, counted iff r' < r_max (no second look;
		// FP32: an r' rounded onto r_max counted inside, as in the evaluation kernels)
		mirror_r((T)(2.0 * sc.rmax), g.r, g.rinv, sc.mirror == 2);
		cut = sizeof(T) == 4 ? g.r <= (T)sc.rmax : g.r < (T)sc.rmax;
	} else {
		cut = force || g.r <= (T)sc.rmax;
		if constexpr (sizeof(T) == 4) nearmin = fminf(nearmin, fabsf(g.r - (T)sc.rmax));
	}
	g.in = ok && cut;
	g.out = ok && !cut;
	T t;
	if (sizeof(T) == 4 && sc.uniform) {  // (dead code for T = double)
		// t = r / h - j with one rounding, r (hf + hf_lo) - j: the store's piece table
		// is the plain one (its rows are equal, so one row serves every interval)
		float jf;
		g.j = floor_clamp((float)g.r * sc.hf, sc.nbin - 1, jf);
		t = (T)fmaf((float)g.r, sc.hf_lo, fmaf((float)g.r, sc.hf, -jf));
	} else {
		g.j = locate<T>(sc, g.r, kb, hv, lut, t);
	}
	g.t = g.in ? t : T(0);  // t is NaN for the self pair
	g.sr = g.in ? g.rinv : T(0);
	return g;
}

// The accumulations of one pair: the row's D columns always; with STATS also
// the pair's O, D2, potential and outer count (unordered pairs, counted once).
// UNI: the piece row is pu for every interval, else row j of the shared table.
template <typename T, int G, bool STATS, bool UNI>
__device__ __forceinline__ void cs_accum(const SysConst& sc, const CsGeom<T>& g, const CsPieceRow<T>& pu,
                                         const T* __restrict__ piece, T* __restrict__ drow, T* __restrict__ oacc,
                                         T* __restrict__ d2acc, int lane, T pa, T pb, KSum<T>& vs, int& nout) {
	const T dx = g.dx, dy = g.dy, dz = g.dz, r = g.r, rinv = g.rinv, t = g.t, sr = g.sr;
	const bool in = g.in;
	const int j = g.j;
	const T* pj = piece + (size_t)j * kCsPieceS;
	auto pc = [&](int k) -> T {
		if constexpr (UNI) return pu.c[k];
		else return pj[k];
	};
	const int s0 = j + 3;  // spline of piece q is s0 - q
	// the 12 (spline, axis) slots of the pair are distinct: all loads first, then
	// the stores, so the shared-memory round trips overlap
	T b1[4], cur[4][3];
	T* dq[4];
#pragma unroll
	for (int q = 0; q < 4; q++) {
		b1[q] = fma(t, fma(t, pc(3 * q + 2), pc(3 * q + 1)), pc(3 * q));  // B'(r)
		dq[q] = drow + (size_t)(s0 - q) * 3 * G + lane;
		cur[q][0] = dq[q][0];
		cur[q][1] = dq[q][G];
		cur[q][2] = dq[q][2 * G];
	}
#pragma unroll
	for (int q = 0; q < 4; q++) {
		const T bs = b1[q] * sr;  // B'(r) / r
		dq[q][0] = fma(bs, dx, cur[q][0]);
		dq[q][G] = fma(bs, dy, cur[q][1]);
		dq[q][2 * G] = fma(bs, dz, cur[q][2]);
	}
	if (STATS) {
		const T on = in ? T(1) : T(0);
		const T dm1 = (T)(sc.dim - 1);
		T ov[4], dv[4];
#pragma unroll
		for (int q = 0; q < 4; q++) {
			ov[q] = oacc[(size_t)(s0 - q) * G + lane];
			dv[q] = d2acc[(size_t)(s0 - q) * G + lane];
		}
#pragma unroll
		for (int q = 0; q < 4; q++) {
			const int l = 12 + 4 * q;
			const T b = fma(t, fma(t, fma(t, pc(l + 3), pc(l + 2)), pc(l + 1)), pc(l)) * on;
			const T b2 = fma(t, pc(28 + 2 * q + 1), pc(28 + 2 * q));
			const T lap = (b2 + dm1 * b1[q] * sr) * on;
			oacc[(size_t)(s0 - q) * G + lane] = ov[q] + b;
			d2acc[(size_t)(s0 - q) * G + lane] = dv[q] + T(2) * lap;  // both orderings of the pair
		}
		vs.add(in ? pair_pot<T>(sc.pot_kind, r, rinv, pa, pb) : T(0));
		nout += g.out ? 1 : 0;
	}
}

template <typename T, int G, bool STATS, bool UNI, bool MIR = false>
__device__ __forceinline__ void cs_pair(const SysConst& sc, const Q4<T>& xr, const Q4<T>& xi, bool ok,
                                        const CsPieceRow<T>& pu, const T* __restrict__ piece, const T* __restrict__ kb,
                                        const T* __restrict__ hv, const int* __restrict__ lut, T* __restrict__ drow,
                                        T* __restrict__ oacc, T* __restrict__ d2acc, int lane, T pa, T pb, KSum<T>& vs,
                                        int& nout, T& nearmin) {
	cs_accum<T, G, STATS, UNI>(sc, cs_geom<T, MIR>(sc, xr, xi, ok, kb, hv, lut, nearmin), pu, piece, drow, oacc, d2acc, lane, pa, pb,
	                           vs, nout);
}

// kCsBatch partners [i, i + kCsBatch): all geometries first, then the accumulations
// in partner order.
constexpr int kCsBatch = 4;
template <typename T, int G, bool STATS, bool UNI, bool MIR = false>
__device__ __forceinline__ void cs_batch(const SysConst& sc, const Q4<T>& xr, const Q4<T>* __restrict__ xs, int i,
                                         bool ok, const CsPieceRow<T>& pu, const T* __restrict__ piece,
                                         const T* __restrict__ kb, const T* __restrict__ hv,
                                         const int* __restrict__ lut, T* __restrict__ drow, T* __restrict__ oacc,
                                         T* __restrict__ d2acc, int lane, T pa, T pb, KSum<T>& vs, int& nout,
                                         T& nearmin) {
	CsGeom<T> g[kCsBatch];
#pragma unroll
	for (int u = 0; u < kCsBatch; u++) g[u] = cs_geom<T, MIR>(sc, xr, xs[i + u], ok, kb, hv, lut, nearmin);
#pragma unroll
	for (int u = 0; u < kCsBatch; u++)
		cs_accum<T, G, STATS, UNI>(sc, g[u], pu, piece, drow, oacc, d2acc, lane, pa, pb, vs, nout);
}

// Cutoff fix-up of one row (FP32, the row's lane alone): the pairs whose FP32
// distance lies within rounding of r_max (sc.rcut_band) are decided again in
// FP64 from the FP32 coordinates, as the evaluation kernels decide them; where
// that differs from the sweep's decision the pair's terms are added (FP64 in)
// or removed (FP64 out): the row's D columns, and for counted pairs (i < nrow)
// O, D2, the potential and the outer count.  Rare; a separate function so the
// sweep's code and registers do not carry it.
struct CsFix {
	float v;
	int nout;
};
template <int G, bool UNI>
__device__ __noinline__ CsFix cs_fix_slot(SysConst sc, CsPieceRow<float> pu, const float* piece, const float* kb,
                                          const float* hv, const int* lut, const Q4<float>* xs, float* drow,
                                          float* oacc, float* d2acc, int n, int nrow, int lane, float pa, float pb) {
	CsFix f = {0.f, 0};
	const Q4<float> xr = xs[nrow];
	const float rmax = (float)sc.rmax, dm1 = (float)(sc.dim - 1);
	for (int i = 0; i < n; i++) {
		if (i == nrow) continue;
		float nm = 3.0e38f;
		const CsGeom<float> g = cs_geom<float>(sc, xr, xs[i], true, kb, hv, lut, nm, true);
		if (!(fabsf(g.r - rmax) < sc.rcut_band)) continue;
		const bool in32 = g.r <= rmax, in64 = cut_fp64(sc, xr, xs[i]);
		if (in64 == in32) continue;
		const float sgn = in64 ? 1.f : -1.f;
		const float* pj = piece + (size_t)g.j * kCsPieceS;
		auto pc = [&](int k) -> float {
			if constexpr (UNI) return pu.c[k];
			else return pj[k];
		};
		const int s0 = g.j + 3;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			const float b1 = fmaf(g.t, fmaf(g.t, pc(3 * q + 2), pc(3 * q + 1)), pc(3 * q));
			const float bs = sgn * b1 * g.sr;
			float* dq = drow + (size_t)(s0 - q) * 3 * G + lane;
			dq[0] = fmaf(bs, g.dx, dq[0]);
			dq[G] = fmaf(bs, g.dy, dq[G]);
			dq[2 * G] = fmaf(bs, g.dz, dq[2 * G]);
			if (i < nrow) {
				const int l = 12 + 4 * q;
				const float b = fmaf(g.t, fmaf(g.t, fmaf(g.t, pc(l + 3), pc(l + 2)), pc(l + 1)), pc(l));
				const float b2 = fmaf(g.t, pc(28 + 2 * q + 1), pc(28 + 2 * q));
				oacc[(size_t)(s0 - q) * G + lane] += sgn * b;
				d2acc[(size_t)(s0 - q) * G + lane] += sgn * 2.f * (b2 + dm1 * b1 * g.sr);
			}
		}
		if (i < nrow) {
			f.v += sgn * pair_pot<float>(sc.pot_kind, g.r, g.rinv, pa, pb);
			f.nout -= in64 ? 1 : -1;
		}
	}
	return f;
}

// Stores the correlated-sampling data of walkers (start + w) mod nw_total,
// w < count (start from *wstart when given, else 0).
// MIR: NUBosonsBulkPB (mirrored distances; no cutoff fix-up).
template <typename T, int G, bool UNI, bool MIR = false>
__global__ void __launch_bounds__(128, 2) k_cs_store(SysConst sc, const CsPieceRow<T> pu, const DynState* __restrict__ dyn,
                                                  const T* __restrict__ piece_g, const T* __restrict__ kb_g,
                                                  const T* __restrict__ hv_g, const int* __restrict__ lut_g,
                                                  const double* __restrict__ fold_g, const T* __restrict__ pos,
                                                  int64_t count, int64_t nw_total, const int32_t* __restrict__ wstart,
                                                  T* __restrict__ D_o, T* __restrict__ D2_o, T* __restrict__ O_o,
                                                  T* __restrict__ V_o, int32_t* __restrict__ nout_o) {
	extern __shared__ __align__(32) unsigned char smem_raw[];
	const int nbin = sc.nbin, n = sc.n, ns = sc.ns, P = sc.p;
	T* piece = reinterpret_cast<T*>(smem_raw);
	T* kb = piece + (size_t)nbin * kCsPieceS;
	T* hv = kb + nbin;
	int* lut = reinterpret_cast<int*>(hv + nbin);
	for (int i = threadIdx.x; i < nbin * kCsPiece; i += blockDim.x)
		piece[(i / kCsPiece) * kCsPieceS + i % kCsPiece] = piece_g[i];
	for (int i = threadIdx.x; i < nbin; i += blockDim.x) {
		kb[i] = kb_g[i];
		hv[i] = hv_g[i];
	}
	for (int i = threadIdx.x; i < sc.ncell; i += blockDim.x) lut[i] = lut_g[i];

	const int tid = threadIdx.x;
	const int lane = tid & (G - 1);
	const int gib = tid / G;
	const int gpb = blockDim.x / G;
	const unsigned wl = tid & 31;
	const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (wl & ~(unsigned)(G - 1)));
	unsigned char* gbase = smem_raw + cs_cta_bytes<T>(nbin, sc.ncell) + (size_t)gib * cs_group_bytes<T>(n, ns, G);
	// disjoint regions: the compiler may move position loads across accumulator stores
	Q4<T>* __restrict__ xs = reinterpret_cast<Q4<T>*>(gbase);
	T* __restrict__ drow = reinterpret_cast<T*>(xs + n);
	T* __restrict__ oacc = drow + (size_t)ns * 3 * G;
	T* __restrict__ d2acc = oacc + (size_t)ns * G;
	__syncthreads();

	const T pa = (T)dyn->pa, pb = (T)dyn->pb;
	const T L = (T)sc.L, Lr = (T)sc.Lr;
	const int64_t w0 = wstart ? (int64_t)*wstart : 0;
	const int nslot = (n + G - 1) / G;

	for (int64_t wi = (int64_t)blockIdx.x * gpb + gib; wi < count; wi += (int64_t)gridDim.x * gpb) {
		int64_t w = w0 + wi;
		if (w >= nw_total) w -= nw_total;
		const T* pw = pos + (size_t)w * sc.dim * n;
		for (int i = lane; i < n; i += G) {
			const T x0 = nic(pw[i], L, Lr);
			const T x1 = sc.dim > 1 ? nic(pw[n + i], L, Lr) : T(0);
			const T x2 = sc.dim > 2 ? nic(pw[2 * n + i], L, Lr) : T(0);
			xs[i] = Q4<T>{x0, x1, x2, T(0)};
		}
		for (int e = lane; e < ns * G; e += G) {
			oacc[e] = T(0);
			d2acc[e] = T(0);
		}
		__syncwarp(gmask);
		KSum<T> vs;
		int nout = 0;
		const int npad = cs_npad(n);
		T* Dw = D_o + (size_t)w * ns * 3 * npad;
		for (int s = 0; s < nslot; s++) {
			const int nrow = s * G + lane;
			const bool rowok = nrow < n;
			const Q4<T> xr = rowok ? xs[nrow] : Q4<T>{T(0), T(0), T(0), T(0)};
			for (int e = lane; e < ns * 3 * G; e += G) drow[e] = T(0);
			T nearmin = T(3.0e38);
			const int base = s * G;
			const int dend = (base + G < n) ? base + G : n;
			// partners below the slot: every lane's pair is counted once (i < nrow);
			// base is a multiple of G, so of kCsBatch
			for (int i = 0; i < base; i += kCsBatch)
				cs_batch<T, G, true, UNI, MIR>(sc, xr, xs, i, rowok, pu, piece, kb, hv, lut, drow, oacc, d2acc, lane, pa, pb,
				                          vs, nout, nearmin);
			// the slot's own block: counted iff i < nrow
			for (int i = base; i < dend; i++) {
				if (i < nrow)
					cs_pair<T, G, true, UNI, MIR>(sc, xr, xs[i], rowok, pu, piece, kb, hv, lut, drow, oacc, d2acc, lane, pa, pb, vs,
					                    nout, nearmin);
				else
					cs_pair<T, G, false, UNI, MIR>(sc, xr, xs[i], rowok && i != nrow, pu, piece, kb, hv, lut, drow, oacc, d2acc, lane,
					                     pa, pb, vs, nout, nearmin);
			}
			// partners above the slot: D only
			int i = dend;
			for (; i + kCsBatch <= n; i += kCsBatch)
				cs_batch<T, G, false, UNI, MIR>(sc, xr, xs, i, rowok, pu, piece, kb, hv, lut, drow, oacc, d2acc, lane, pa, pb,
				                           vs, nout, nearmin);
			for (; i < n; i++)
				cs_pair<T, G, false, UNI, MIR>(sc, xr, xs[i], rowok, pu, piece, kb, hv, lut, drow, oacc, d2acc, lane, pa, pb,
				                          vs, nout, nearmin);
			if constexpr (sizeof(T) == 4 && !MIR) {
				if (rowok && nearmin < sc.rcut_band) {
					const CsFix f = cs_fix_slot<G, UNI>(sc, pu, piece, kb, hv, lut, xs, drow, oacc, d2acc, n, nrow, lane,
					                                    pa, pb);
					vs.add(f.v);
					nout += f.nout;
				}
			}
			if (rowok)
				for (int e = 0; e < ns * 3; e++) Dw[cs_doff(ns * 3, e, nrow)] = drow[(size_t)e * G + lane];
		}
		__syncwarp(gmask);
		// lane-ordered sums of the lane-private accumulators
		for (int sp = lane; sp < ns; sp += G) {
			T so = T(0), s2 = T(0);
			for (int l = 0; l < G; l++) {
				so += oacc[(size_t)sp * G + l];
				s2 += d2acc[(size_t)sp * G + l];
			}
			drow[sp] = so;
			drow[ns + sp] = s2;
			D2_o[(size_t)w * ns + sp] = s2;
		}
		__syncwarp(gmask);
		for (int k = lane; k < P; k += G) {
			double o = 0.0;
			for (int sp = 0; sp < ns; sp++) {
				const double f = fold_g[(size_t)k * ns + sp];
				if (!fold_zero(f)) o += f * (double)drow[sp];
			}
			O_o[(size_t)w * P + k] = (T)o;
		}
		const T v = group_sum<T, G>(vs.value(), gmask);
		int nall = nout;
#pragma unroll
		for (int o = G / 2; o > 0; o >>= 1) nall += __shfl_xor_sync(gmask, nall, o, G);
		if (lane == 0) {
			V_o[w] = v;
			nout_o[w] = nall;
		}
		__syncwarp(gmask);
	}
}

// Local quantities of every stored walker at the current stage parameters:
// same outputs as k_eloc (ln psi, O, E_loc, kinetic sums, dE/d alpha).
// One warp per walker; each lane takes V consecutive particles per 16-byte
// load, 32 V particles per chunk.  D is streamed once for G_n; with ADJ each
// chunk's G_n . D[s][.][n] follows right after its G_n (a second read of the
// chunk's D: with a whole GPU of warps streaming, most of it comes from HBM
// again), and the per-lane sums over the chunks stay in shared memory
// (part[s][lane], complex) and are added over the lanes once per walker
// instead of one butterfly per spline.
template <typename T> struct Vec16;
template <> struct Vec16<float> {
	using type = float4;
	static constexpr int V = 4;
	__device__ static void get(const type& v, float* o) {
		o[0] = v.x;
		o[1] = v.y;
		o[2] = v.z;
		o[3] = v.w;
	}
};
template <> struct Vec16<double> {
	using type = double2;
	static constexpr int V = 2;
	__device__ static void get(const type& v, double* o) {
		o[0] = v.x;
		o[1] = v.y;
	}
};

// Shared memory of k_cs_eval: wR, wI [ns each, padded to 4] | per warp:
// part[ns][33][2] (lane-private complex partial sums; the row of 33 keeps the
// per-spline sums over the lanes free of bank conflicts) | A[2*ns, padded to 4]
__host__ __device__ inline int cs_ns2(int ns) { return (2 * ns + 3) & ~3; }
constexpr int kCsPartRow = 33;
template <typename T>
__host__ __device__ inline size_t cs_eval_smem_bytes(int n, int ns, int warps) {
	(void)n;
	return ((size_t)cs_ns2(ns) + (size_t)warps * ((size_t)2 * kCsPartRow * ns + cs_ns2(ns))) * sizeof(T);
}

// The end of one walker's stored-sample evaluation: the Laplacian sums from D2,
// ln psi, O, E_loc, the kinetic sums and, with ADJ, dE/d alpha from
// asum[2s + {0, 1}] = sum_n G_n . D[s][.][n] (complex).  One warp.
template <typename T, bool ADJ>
__device__ __forceinline__ void cs_finish_walker(const SysConst& sc, const double* __restrict__ params,
                                 const double* __restrict__ fold_g, const T* __restrict__ D2,
                                 const T* __restrict__ Os, const T* __restrict__ Vs,
                                 const int32_t* __restrict__ nouts, int64_t w, const T* wR, const T* wI,
                                 const T* asum, const KSum<T>& r1, const KSum<T>& i1, const KSum<T>& r1i1,
                                 T* __restrict__ lnpsi_o, T* __restrict__ O_o, T* __restrict__ eloc_o,
                                 T* __restrict__ other_o, T* __restrict__ dE_o) {
	const int ns = sc.ns, P = sc.p;
	const int lane = threadIdx.x & 31;
	const double c = sc.hbar2_2m;
	T l2r = T(0), l2i = T(0);
	for (int s = lane; s < ns; s += 32) {
		const T v = D2[(size_t)w * ns + s];
		l2r = fma(wR[s], v, l2r);
		l2i = fma(wI[s], v, l2i);
	}
	const T sR1 = group_sum<T, 32>(r1.value(), 0xffffffffu);
	const T sI1 = group_sum<T, 32>(i1.value(), 0xffffffffu);
	const T sR1I1 = group_sum<T, 32>(r1i1.value(), 0xffffffffu);
	const T sR2 = group_sum<T, 32>(l2r, 0xffffffffu);
	const T sI2 = group_sum<T, 32>(l2i, 0xffffffffu);
	const T vint = Vs[w];
	double lnp = 0.0;
	for (int k = lane; k < P; k += 32) {
		const T o = Os[(size_t)w * P + k];
		O_o[(size_t)w * P + k] = o;
		lnp += params[k] * (double)o;
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) lnp += __shfl_xor_sync(0xffffffffu, lnp, o);
	if (lane == 0) {
		lnp += params[P - 1] * (double)nouts[w];
		const double kinR = -((double)sR1 - (double)sI1 + (double)sR2) * c;
		const double kinI = -((double)sR1I1 + (double)sI2) * c;
		lnpsi_o[w] = (T)lnp;
		eloc_o[2 * w + 0] = (T)(kinR + (double)vint);
		eloc_o[2 * w + 1] = (T)kinI;
		T* ot = other_o + (size_t)w * 7;
		ot[0] = (T)kinR;
		ot[1] = vint;
		ot[2] = sR1;
		ot[3] = sI1;
		ot[4] = sR2;
		ot[5] = sI2;
		ot[6] = sR1I1;
	}
	if (ADJ) {
		__syncwarp();
		for (int k = lane; k < P; k += 32) {
			double dR = 0.0, dI = 0.0;
			for (int s = 0; s < ns; s++) {
				const double f = fold_g[(size_t)k * ns + s];
				if (fold_zero(f)) continue;
				dR += f * (2.0 * (double)asum[2 * s] + (double)D2[(size_t)w * ns + s]);
				dI += f * (2.0 * (double)asum[2 * s + 1]);
			}
			dE_o[((size_t)w * P + k) * 2 + 0] = (T)(-c * dR);
			dE_o[((size_t)w * P + k) * 2 + 1] = (T)(-c * dI);
		}
	}
}

template <typename T, bool ADJ>
__global__ void __launch_bounds__(128) k_cs_eval(SysConst sc, const double* __restrict__ params,
                                                 const double* __restrict__ fold_g, const T* __restrict__ D,
                                                 const T* __restrict__ D2, const T* __restrict__ Os,
                                                 const T* __restrict__ Vs, const int32_t* __restrict__ nouts,
                                                 int64_t nw, T* __restrict__ lnpsi_o, T* __restrict__ O_o,
                                                 T* __restrict__ eloc_o, T* __restrict__ other_o, T* __restrict__ dE_o) {
	using VT = typename Vec16<T>::type;
	constexpr int V = Vec16<T>::V;
	extern __shared__ __align__(32) unsigned char smem_raw[];
	const int n = sc.n, ns = sc.ns, P = sc.p;
	const int npad = cs_npad(n);
	T* wR = reinterpret_cast<T*>(smem_raw);
	T* wI = wR + ns;
	T* gs_all = wR + cs_ns2(ns);  // per warp: part[ns][33][2] (adjoint), then [2*ns] spline sums
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int wpb = blockDim.x >> 5;
	for (int s = threadIdx.x; s < ns; s += blockDim.x) {
		double r = 0.0, im = 0.0;
		for (int k = 0; k < P; k++) {
			const double f = fold_g[(size_t)k * ns + s];
			r += params[k] * f;
			im += params[P + k] * f;
		}
		wR[s] = (T)r;
		wI[s] = (T)im;
	}
	__syncthreads();
	T* part = gs_all + (size_t)warp * ((size_t)2 * kCsPartRow * ns + cs_ns2(ns));
	T* asum = part + (size_t)2 * kCsPartRow * ns;

	for (int64_t w = (int64_t)blockIdx.x * wpb + warp; w < nw; w += (int64_t)gridDim.x * wpb) {
		const T* Dw = D + (size_t)w * ns * 3 * npad;
		KSum<T> r1, i1, r1i1;
		if (ADJ)
			for (int s = 0; s < ns; s++) {
				part[((size_t)s * kCsPartRow + lane) * 2] = T(0);
				part[((size_t)s * kCsPartRow + lane) * 2 + 1] = T(0);
			}
		for (int c0 = lane * V; c0 < n; c0 += 32 * V) {
			T gr[3][V], gi[3][V];
#pragma unroll
			for (int a = 0; a < 3; a++)
#pragma unroll
				for (int v = 0; v < V; v++) gr[a][v] = gi[a][v] = T(0);
			for (int s = 0; s < ns; s++) {
				const T a_ = wR[s], b_ = wI[s];
#pragma unroll
				for (int a = 0; a < 3; a++) {
					T d[V];
					Vec16<T>::get(*reinterpret_cast<const VT*>(Dw + cs_doff(3 * ns, 3 * s + a, c0)), d);
#pragma unroll
					for (int v = 0; v < V; v++) {
						gr[a][v] = fma(a_, d[v], gr[a][v]);
						gi[a][v] = fma(b_, d[v], gi[a][v]);
					}
				}
			}
#pragma unroll
			for (int v = 0; v < V; v++) {
				if (c0 + v < n) {
					r1.add(gr[0][v] * gr[0][v] + gr[1][v] * gr[1][v] + gr[2][v] * gr[2][v]);
					i1.add(gi[0][v] * gi[0][v] + gi[1][v] * gi[1][v] + gi[2][v] * gi[2][v]);
					r1i1.add(T(2) * (gr[0][v] * gi[0][v] + gr[1][v] * gi[1][v] + gr[2][v] * gi[2][v]));
				}
			}
			if (ADJ) {
				// this chunk's G_n . D[s][.][n] (the padding of D is zero)
				for (int s = 0; s < ns; s++) {
					T cr = T(0), ci = T(0);
#pragma unroll
					for (int a = 0; a < 3; a++) {
						T d[V];
						Vec16<T>::get(*reinterpret_cast<const VT*>(Dw + cs_doff(3 * ns, 3 * s + a, c0)), d);
#pragma unroll
						for (int v = 0; v < V; v++) {
							cr = fma(gr[a][v], d[v], cr);
							ci = fma(gi[a][v], d[v], ci);
						}
					}
					T* pp = part + ((size_t)s * kCsPartRow + lane) * 2;
					pp[0] += cr;
					pp[1] += ci;
				}
			}
		}
		if (ADJ) {
			__syncwarp();
			// A_s = sum_n G_n . D[s][.][n] (complex): the lanes' partial sums in lane order
			for (int s = lane; s < ns; s += 32) {
				T ar = T(0), ai = T(0);
				const T* pp = part + (size_t)s * kCsPartRow * 2;
				for (int l = 0; l < 32; l++) {
					ar += pp[2 * l];
					ai += pp[2 * l + 1];
				}
				asum[2 * s] = ar;
				asum[2 * s + 1] = ai;
			}
		}
		cs_finish_walker<T, ADJ>(sc, params, fold_g, D2, Os, Vs, nouts, w, wR, wI, asum, r1, i1, r1i1, lnpsi_o, O_o,
		                         eloc_o, other_o, dE_o);
		__syncwarp();
	}
}

// Stored-sample evaluation in FP32 for ns <= 32: one warp per walker, the
// walker's D streamed through shared memory one contiguous 32-particle chunk at
// a time by a TMA bulk copy (each byte of D leaves HBM once; one buffer per warp
// keeps 16 warps on an SM, and the other warps' copies overlap this warp's
// arithmetic), then one particle per lane: G_n from the chunk, and with ADJ the per-spline
// partial sums of G_n . D[s][.][n] kept in registers.  At the walker's end the
// lanes' sums pass through the buffer just used (row of 2 ns + 1 floats per
// lane) and are added in lane order.
constexpr int kCsStNs = 32;
__host__ __device__ inline int cs_st_warp_floats(int ns) {
	const int chunk = ns * 3 * 32, tr = 32 * (2 * ns + 1);
	return (((chunk > tr) ? chunk : tr) + 3) & ~3;
}
__host__ __device__ inline size_t cs_eval_st_smem_bytes(int ns, int warps) {
	return ((size_t)cs_ns2(ns) + (size_t)warps * ((size_t)cs_st_warp_floats(ns) + cs_ns2(ns))) * sizeof(float);
}

// Each chunk is one TMA bulk copy (cp.async.bulk) issued by lane 0 and
// completed on the warp's mbarrier.  Every wait is bounded in time
// (mbar_wait_ns): when the status limit runs out the walker's E_loc is written
// as NaN (the statistics then report a non-finite value), the warp waits for
// its own copy with the drain limit and returns.
// lane 0: order this warp's earlier generic accesses of dst before the async
// write, arm the barrier with the byte count and start the copy
__device__ __forceinline__ void cs_bulk_copy(uint32_t mbar, float* dst, const float* src, uint32_t bytes) {
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
	                 (uint32_t)__cvta_generic_to_shared(dst)),
	             "l"(src), "r"(bytes), "r"(mbar)
	             : "memory");
}

constexpr int kCsStWarps = 4;  // warps per block: 4 blocks (16 warps) per SM at 32 splines
template <bool ADJ>
__global__ void __launch_bounds__(32 * kCsStWarps, 4) k_cs_eval_st(
    SysConst sc, const double* __restrict__ params, const double* __restrict__ fold_g, const float* __restrict__ D,
    const float* __restrict__ D2, const float* __restrict__ Os, const float* __restrict__ Vs,
    const int32_t* __restrict__ nouts, int64_t nw, float* __restrict__ lnpsi_o, float* __restrict__ O_o,
    float* __restrict__ eloc_o, float* __restrict__ other_o, float* __restrict__ dE_o, uint64_t wait_ns) {
	extern __shared__ __align__(32) unsigned char smem_raw[];
	const int n = sc.n, ns = sc.ns, P = sc.p;
	const int npad = cs_npad(n), nrow = 3 * ns, nch = npad / 32;
	float* wR = reinterpret_cast<float*>(smem_raw);
	float* wI = wR + ns;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int wpb = blockDim.x >> 5;
	for (int s = threadIdx.x; s < ns; s += blockDim.x) {
		double r = 0.0, im = 0.0;
		for (int k = 0; k < P; k++) {
			const double f = fold_g[(size_t)k * ns + s];
			r += params[k] * f;
			im += params[P + k] * f;
		}
		wR[s] = (float)r;
		wI[s] = (float)im;
	}
	__syncthreads();
	const int wfl = cs_st_warp_floats(ns);
	float* chunk = wR + cs_ns2(ns) + (size_t)warp * (wfl + cs_ns2(ns));  // [row = 3 s + a][32]
	float* asum = chunk + wfl;
	const size_t wstride = (size_t)nrow * npad;
	// one mbarrier per warp after the warps' regions
	const uint32_t mbar = (uint32_t)__cvta_generic_to_shared(smem_raw + cs_eval_st_smem_bytes(ns, wpb)) + 8u * warp;
	const uint32_t cbytes = (uint32_t)nrow * 32u * 4u;
	uint32_t phase = 0;
	if (lane == 0) {
		asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncwarp();

	for (int64_t w = (int64_t)blockIdx.x * wpb + warp; w < nw; w += (int64_t)gridDim.x * wpb) {
		const float* Dw = D + (size_t)w * wstride;
		KSum<float> r1, i1, r1i1;
		float pr[kCsStNs], pi[kCsStNs];
#pragma unroll
		for (int s = 0; s < kCsStNs; s++) pr[s] = pi[s] = 0.f;
		for (int c = 0; c < nch; c++) {
			if (lane == 0) cs_bulk_copy(mbar, chunk, Dw + (size_t)c * nrow * 32, cbytes);
			const bool ok = mbar_wait_ns(mbar, phase, wait_ns);
			phase ^= 1u;
			if (!__all_sync(0xffffffffu, ok)) {
				if (lane == 0) {
					eloc_o[2 * w] = __int_as_float(0x7fc00000);
					eloc_o[2 * w + 1] = __int_as_float(0x7fc00000);
				}
				mbar_wait_ns(mbar, phase ^ 1u, kWaitDrainNs);  // the copy still in flight
				return;
			}
			__syncwarp();
			const int c0 = c * 32;
			float gr0 = 0.f, gr1 = 0.f, gr2 = 0.f, gi0 = 0.f, gi1 = 0.f, gi2 = 0.f;
#pragma unroll
			for (int s = 0; s < kCsStNs; s++) {
				if (s < ns) {
					const float a_ = wR[s], b_ = wI[s];
					const float d0 = chunk[(3 * s) * 32 + lane], d1 = chunk[(3 * s + 1) * 32 + lane],
					            d2 = chunk[(3 * s + 2) * 32 + lane];
					gr0 = fmaf(a_, d0, gr0);
					gr1 = fmaf(a_, d1, gr1);
					gr2 = fmaf(a_, d2, gr2);
					gi0 = fmaf(b_, d0, gi0);
					gi1 = fmaf(b_, d1, gi1);
					gi2 = fmaf(b_, d2, gi2);
				}
			}
			if (c0 + lane < n) {
				r1.add(gr0 * gr0 + gr1 * gr1 + gr2 * gr2);
				i1.add(gi0 * gi0 + gi1 * gi1 + gi2 * gi2);
				r1i1.add(2.f * (gr0 * gi0 + gr1 * gi1 + gr2 * gi2));
			}
			if (ADJ) {
#pragma unroll
				for (int s = 0; s < kCsStNs; s++) {
					if (s < ns) {
						const float d0 = chunk[(3 * s) * 32 + lane], d1 = chunk[(3 * s + 1) * 32 + lane],
						            d2 = chunk[(3 * s + 2) * 32 + lane];
						pr[s] = fmaf(gr0, d0, fmaf(gr1, d1, fmaf(gr2, d2, pr[s])));
						pi[s] = fmaf(gi0, d0, fmaf(gi1, d1, fmaf(gi2, d2, pi[s])));
					}
				}
			}
			__syncwarp();  // every lane is done with the chunk before the next copy
		}
		if (ADJ) {
			const int rl = 2 * ns + 1;
#pragma unroll
			for (int s = 0; s < kCsStNs; s++) {
				if (s < ns) {
					chunk[lane * rl + 2 * s] = pr[s];
					chunk[lane * rl + 2 * s + 1] = pi[s];
				}
			}
			__syncwarp();
			for (int s = lane; s < ns; s += 32) {
				float ar = 0.f, ai = 0.f;
				for (int l = 0; l < 32; l++) {
					ar += chunk[l * rl + 2 * s];
					ai += chunk[l * rl + 2 * s + 1];
				}
				asum[2 * s] = ar;
				asum[2 * s + 1] = ai;
			}
		}
		cs_finish_walker<float, ADJ>(sc, params, fold_g, D2, Os, Vs, nouts, w, wR, wI, asum, r1, i1, r1i1, lnpsi_o,
		                             O_o, eloc_o, other_o, dE_o);
		__syncwarp();
	}
}

// Next refresh window: start <- (start + count) mod nw.
__global__ void k_cs_advance(DynState* dyn, int64_t count, int64_t nw) {
	if (threadIdx.x == 0 && blockIdx.x == 0) {
		int64_t s = (int64_t)dyn->cs_start + count;
		dyn->cs_start = (int32_t)(s % nw);
	}
}

}  // namespace tdvmc
