// Per-walker local quantities of the pair-spline Jastrow wave function:
// ln psi, O_k = d ln psi / d uR_k (BC-folded spline sums), the complex local
// energy with its kinetic partial sums, and optionally the adjoint
// dE_loc / d alpha_k.  Follows BosonsBulk::CalculateLocalOperators,
// CalculateOtherLocalOperators and CalculateExpectationValues
// (BosonsBulk.cpp:179-218, 220-336, 349-458, 522-545).
//
// One group of G lanes owns one walker.  Forward sweep: lane l owns row
// particle n = s*G + l of slot s and loops over all partners i (the partner
// coordinate is a shared-memory broadcast), accumulating the complex
// gradient G_n and Laplacian of ln psi in registers with compensated block
// sums.  Pair statistics that are linear in the spline basis (O_k, and for
// the adjoint the alpha-independent Laplacian of O_k) are accumulated as
// per-interval moments sum t^c (and sum t^c / r) in lane-private shared
// histograms; partners below the slot base are counted once per unordered
// pair with warp-uniform control flow (the diagonal block is the only mixed
// region).  Reverse sweep (adjoint): one pass over unordered pairs that
// recomputes minimum-image distances and accumulates sum t^c g with
// g = (G_n - G_i) . rhat_ni; no pair table is stored.  Moments are turned
// into spline values with the local piece polynomials and folded to the p
// parameters at the end.
#pragma once

#include "common.cuh"
#include "k_sample.cuh"

namespace tdvmc {

constexpr int kFwdMoments = 4;     // sum t^c, c = 0..3
constexpr int kFwdMomentsAdj = 7;  // + sum t^c / r, c = 0..2
constexpr int kRevMoments = 6;     // complex sum g t^c, c = 0..2
constexpr int kHistSlots = 8;      // histogram slots per interval and lane in the float4 mode
// slots per interval and lane: the largest moment count (7), or 8 for the float4 mode
template <int HIST> struct HistSlots { static constexpr int value = HIST == 1 ? 8 : 7; };

// Histogram update modes of the lane-private moment histograms:
//   0  scalar read-modify-write      hist[(j*8 + m)*G + lane]
//   1  float4 read-modify-write      hist4[(j*2 + m/4)*G + lane].{x,y,z,w}[m%4]
//   2  shared-memory atomic add      same layout as 0 (no contention: lane-private)
template <int HIST, typename T, int G>
__device__ __forceinline__ void hist_add8(T* __restrict__ hist, int j, int lane, const T (&v)[8], int nv) {
	if (HIST == 1) {
		Q4<T>* h4 = reinterpret_cast<Q4<T>*>(hist) + ((size_t)j * 2) * G + lane;
		Q4<T> a = h4[0];
		a.x += v[0];
		a.y += v[1];
		a.z += v[2];
		a.w += v[3];
		h4[0] = a;
		if (nv > 4) {
			Q4<T> b = h4[G];
			b.x += v[4];
			b.y += v[5];
			b.z += v[6];
			if (nv > 7) b.w += v[7];
			h4[G] = b;
		}
	} else {
		T* hp = hist + (size_t)j * HistSlots<HIST>::value * G + lane;
#pragma unroll
		for (int m = 0; m < 8; m++) {
			if (m >= nv) break;
			if (HIST == 2) atomicAdd(hp + m * G, v[m]);
			else hp[m * G] += v[m];
		}
	}
}

// value of moment m of interval j summed over the group's lanes
template <int HIST, typename T, int G>
__device__ __forceinline__ T hist_sum(const T* __restrict__ hist, int j, int m) {
	T s = T(0);
	if (HIST == 1) {
		const T* h = hist + (((size_t)j * 2 + m / 4) * G) * 4 + (m & 3);
#pragma unroll 8
		for (int l = 0; l < G; l++) s += h[l * 4];
	} else {
		const T* h = hist + ((size_t)j * HistSlots<HIST>::value + m) * G;
#pragma unroll 8
		for (int l = 0; l < G; l++) s += h[l];
	}
	return s;
}

// Shared memory layout:
//   CTA:   coefC[2*nbin] (uR, uI cubics) | kb[nbin] | hv[nbin] | lut[ncell]
//   group: xs[n] | Gs[n*6] (adjoint) | hist[nbin*NM*G] | red[nbin*NMtot] | spl[ns*4] | misc[16]
template <typename T>
__host__ __device__ inline size_t eloc_cta_bytes(int nbin, int ncell) {
	size_t b = 2 * (size_t)nbin * sizeof(Q4<T>) + 2 * (size_t)nbin * sizeof(T) + (size_t)ncell * sizeof(int);
	return (b + 31) & ~(size_t)31;
}
template <typename T>
__host__ __device__ inline size_t eloc_group_bytes(int n, int nbin, int ns, int G, bool adj, int hist_mode = 0) {
	int nm = adj ? kFwdMomentsAdj : kFwdMoments;
	int nmh = hist_mode == 1 ? 8 : 7;
	size_t b = (size_t)n * sizeof(Q4<T>);
	if (adj) b += (size_t)((n * 6 + 7) & ~7) * sizeof(T);  // keeps the histogram 32-byte aligned
	b += (size_t)nbin * nmh * G * sizeof(T);
	b += (size_t)nbin * (nm + (adj ? kRevMoments : 0)) * sizeof(T);
	b += (size_t)ns * 4 * sizeof(T) + 16 * sizeof(T);
	return (b + 31) & ~(size_t)31;
}

template <typename T, int G>
__device__ __forceinline__ T group_sum(T v, unsigned gmask) {
#pragma unroll
	for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gmask, v, o, G);
	return v;
}

// Geometry and spline derivatives of one (row, partner) pair of the forward sweep.
template <typename T> struct FwdPair {
	T dx, dy, dz, r, rinv, t;
	T gR, gI, lR, lI;
	int j;
	bool in;
};

template <typename T>
__device__ __forceinline__ FwdPair<T> fwd_pair(const SysConst& sc, const Q4<T>& xr, const Q4<T>& xi, bool ok,
                                               const Q4<T>* __restrict__ coefC, const T* __restrict__ kb,
                                               const T* __restrict__ hv, const int* __restrict__ lut) {
	FwdPair<T> q;
	const T L = (T)sc.L, Lr = (T)sc.Lr;
	q.dx = nic(xr.x - xi.x, L, Lr);
	q.dy = nic(xr.y - xi.y, L, Lr);
	q.dz = nic(xr.z - xi.z, L, Lr);
	const T r2 = q.dx * q.dx + q.dy * q.dy + q.dz * q.dz;
	q.rinv = rsqrt_(r2);
	q.r = r2 * q.rinv;
	q.in = ok && (q.r <= (T)sc.rmax);
	q.j = locate<T>(sc, q.r, kb, hv, lut, q.t);
	const Q4<T> cR = coefC[2 * q.j];
	const Q4<T> cI = coefC[2 * q.j + 1];
	const T hj = sc.uniform ? (T)sc.hinv : hv[q.j];
	const T t = q.t;
	const T d1R = (cR.y + t * (T(2) * cR.z + T(3) * t * cR.w)) * hj;
	const T d1I = (cI.y + t * (T(2) * cI.z + T(3) * t * cI.w)) * hj;
	const T d2R = (T(2) * cR.z + T(6) * t * cR.w) * (hj * hj);
	const T d2I = (T(2) * cI.z + T(6) * t * cI.w) * (hj * hj);
	const T dm1 = (T)(sc.dim - 1);
	q.gR = q.in ? d1R * q.rinv : T(0);
	q.gI = q.in ? d1I * q.rinv : T(0);
	q.lR = q.in ? d2R + dm1 * q.gR : T(0);
	q.lI = q.in ? d2I + dm1 * q.gI : T(0);
	return q;
}

// Pair statistics of one counted (unordered) pair: moments and potential.
template <typename T, int G, bool ADJ, int HIST>
__device__ __forceinline__ void fwd_stats(const SysConst& sc, const FwdPair<T>& q, bool on, T* __restrict__ hist,
                                          int lane, T pa, T pb, T& vb) {
	const T ts = on ? q.t : T(0);  // t is NaN for the self pair
	const T t2 = ts * ts;
	const T qq = on ? q.rinv : T(0);
	T v[8] = {on ? T(1) : T(0), ts, t2, t2 * ts, qq, qq * ts, qq * t2, T(0)};
	hist_add8<HIST, T, G>(hist, q.j, lane, v, ADJ ? kFwdMomentsAdj : kFwdMoments);
	vb += on ? pair_pot<T>(sc.pot_kind, q.r, q.rinv, pa, pb) : T(0);
}

// Forward sweep of row nrow against partners [i0, i1), kNp partners per
// iteration so their dependency chains overlap (one warp per SM sub-partition
// is all the shared memory allows).
// ON: 0 = no pair statistics, 1 = all lanes count the pair, 2 = count iff i < nrow.
constexpr int kNp = 4;
template <typename T, int G, int ON, bool ADJ, int HIST>
__device__ __forceinline__ void fwd_region(const SysConst& sc, int i0, int i1, int nrow, bool rowok, const Q4<T>& xr,
                                           const Q4<T>* __restrict__ xs, const Q4<T>* __restrict__ coefC,
                                           const T* __restrict__ kb, const T* __restrict__ hv,
                                           const int* __restrict__ lut, T* __restrict__ hist, int lane, T pa, T pb,
                                           KSum<T>* acc /* gRx gRy gRz gIx gIy gIz lR lI */, KSum<T>& vsum, int& nout) {
	const T rmax = (T)sc.rmax;
	for (int c0 = i0; c0 < i1; c0 += 32) {
		const int c1 = (c0 + 32 < i1) ? c0 + 32 : i1;
		T a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
		T vb = T(0);
		for (int i = c0; i < c1; i += kNp) {
			FwdPair<T> q[kNp];
			int ii[kNp];
			bool have[kNp];
#pragma unroll
			for (int h = 0; h < kNp; h++) {
				have[h] = i + h < c1;
				ii[h] = have[h] ? i + h : i;
			}
			Q4<T> xp[kNp];
#pragma unroll
			for (int h = 0; h < kNp; h++) xp[h] = xs[ii[h]];
#pragma unroll
			for (int h = 0; h < kNp; h++)
				q[h] = fwd_pair<T>(sc, xr, xp[h], have[h] && rowok && ii[h] != nrow, coefC, kb, hv, lut);
#pragma unroll
			for (int h = 0; h < kNp; h++) {
				a[0] += q[h].gR * q[h].dx;
				a[1] += q[h].gR * q[h].dy;
				a[2] += q[h].gR * q[h].dz;
				a[3] += q[h].gI * q[h].dx;
				a[4] += q[h].gI * q[h].dy;
				a[5] += q[h].gI * q[h].dz;
				a[6] += q[h].lR;
				a[7] += q[h].lI;
			}
			if (ON != 0) {
#pragma unroll
				for (int h = 0; h < kNp; h++) {
					const bool c = have[h] && ((ON == 1) ? true : (ii[h] < nrow));
					fwd_stats<T, G, ADJ, HIST>(sc, q[h], q[h].in && c, hist, lane, pa, pb, vb);
					nout += (rowok && ii[h] != nrow && c && !(q[h].r <= rmax)) ? 1 : 0;
				}
			}
		}
#pragma unroll
		for (int k = 0; k < 8; k++) acc[k].add(a[k]);
		if (ON != 0) vsum.add(vb);
	}
}

// Reverse sweep over unordered pairs (i < nrow) for partners [i0, i1), kNp
// partners per iteration.
template <typename T, int G, bool DIAG, int HIST>
__device__ __forceinline__ void rev_region(const SysConst& sc, int i0, int i1, int nrow, bool rowok, const Q4<T>& xr,
                                           const T* gn, const Q4<T>* __restrict__ xs, const T* __restrict__ Gs,
                                           const T* __restrict__ kb, const T* __restrict__ hv,
                                           const int* __restrict__ lut, T* __restrict__ hist, int lane) {
	const T L = (T)sc.L, Lr = (T)sc.Lr, rmax = (T)sc.rmax;
	for (int i = i0; i < i1; i += kNp) {
		T v[kNp][8];
		int jj[kNp];
#pragma unroll
		for (int h = 0; h < kNp; h++) {
			const bool have = i + h < i1;
			const int ii = have ? i + h : i;
			const Q4<T> xi = xs[ii];
			const T* gi = Gs + (size_t)ii * 6;
			const T dx = nic(xr.x - xi.x, L, Lr), dy = nic(xr.y - xi.y, L, Lr), dz = nic(xr.z - xi.z, L, Lr);
			const T r2 = dx * dx + dy * dy + dz * dz;
			const T rinv = rsqrt_(r2);
			const T r = r2 * rinv;
			const bool on = have && rowok && (r <= rmax) && (DIAG ? (ii < nrow) : true);
			T t;
			jj[h] = locate<T>(sc, r, kb, hv, lut, t);
			t = on ? t : T(0);  // t is NaN for the self pair
			const T sr = on ? rinv : T(0);
			const T gR = ((gn[0] - gi[0]) * dx + (gn[1] - gi[1]) * dy + (gn[2] - gi[2]) * dz) * sr;
			const T gI = ((gn[3] - gi[3]) * dx + (gn[4] - gi[4]) * dy + (gn[5] - gi[5]) * dz) * sr;
			const T t2 = t * t;
			v[h][0] = gR;
			v[h][1] = gR * t;
			v[h][2] = gR * t2;
			v[h][3] = gI;
			v[h][4] = gI * t;
			v[h][5] = gI * t2;
			v[h][6] = v[h][7] = T(0);
		}
#pragma unroll
		for (int h = 0; h < kNp; h++) hist_add8<HIST, T, G>(hist, jj[h], lane, v[h], kRevMoments);
	}
}

// Sum lane-private histograms into red[nbin*nm] and clear them.
template <typename T, int G, int HIST>
__device__ __forceinline__ void hist_reduce(T* hist, T* red, int nbin, int nm, int lane, unsigned gmask) {
	__syncwarp(gmask);
	for (int e = lane; e < nbin * nm; e += G) red[e] = hist_sum<HIST, T, G>(hist, e / nm, e % nm);
	__syncwarp(gmask);
	for (int e = lane; e < nbin * HistSlots<HIST>::value * G; e += G) hist[e] = T(0);
	__syncwarp(gmask);
}

template <typename T, int G, bool ADJ, int HIST>
__global__ void __launch_bounds__(128, 1) k_eloc(SysConst sc, const DynState* __restrict__ dyn, const Q4<T>* __restrict__ coefC_g,
                                              const T* __restrict__ kb_g, const T* __restrict__ hv_g,
                                              const int* __restrict__ lut_g, const T* __restrict__ loc_g,
                                              const double* __restrict__ fold_g, const double* __restrict__ params,
                                              const T* __restrict__ pos, int64_t nw, T* __restrict__ lnpsi_o,
                                              T* __restrict__ O_o, T* __restrict__ eloc_o, T* __restrict__ other_o,
                                              T* __restrict__ dE_o) {
	constexpr int NM = ADJ ? kFwdMomentsAdj : kFwdMoments;
	constexpr int NMH = HistSlots<HIST>::value;
	extern __shared__ __align__(32) unsigned char smem_raw[];
	const int nbin = sc.nbin, n = sc.n, ns = sc.ns, P = sc.p;
	Q4<T>* coefC = reinterpret_cast<Q4<T>*>(smem_raw);
	T* kb = reinterpret_cast<T*>(coefC + 2 * nbin);
	T* hv = kb + nbin;
	int* lut = reinterpret_cast<int*>(hv + nbin);
	const size_t cta_b = eloc_cta_bytes<T>(nbin, sc.ncell);
	const size_t grp_b = eloc_group_bytes<T>(n, nbin, ns, G, ADJ, HIST);

	for (int i = threadIdx.x; i < 2 * nbin; i += blockDim.x) coefC[i] = coefC_g[i];
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
	unsigned char* gbase = smem_raw + cta_b + (size_t)gib * grp_b;
	Q4<T>* xs = reinterpret_cast<Q4<T>*>(gbase);
	T* Gs = reinterpret_cast<T*>(xs + n);
	T* hist = Gs + (ADJ ? (size_t)((n * 6 + 7) & ~7) : 0);
	T* red = hist + (size_t)nbin * NMH * G;
	T* redr = red + (size_t)nbin * NM;
	T* spl = redr + (ADJ ? (size_t)nbin * kRevMoments : 0);  // [ns][4]: S, Lsp, AR, AI
	T* misc = spl + (size_t)ns * 4;

	for (int e = lane; e < nbin * NMH * G; e += G) hist[e] = T(0);
	__syncthreads();

	const T pa = (T)dyn->pa, pb = (T)dyn->pb;
	const int nslot = (n + G - 1) / G;

	for (int64_t w = (int64_t)blockIdx.x * gpb + gib; w < nw; w += (int64_t)gridDim.x * gpb) {
		const T* pw = pos + (size_t)w * sc.dim * n;
		for (int i = lane; i < n; i += G) {
			T x0 = pw[i];
			T x1 = sc.dim > 1 ? pw[n + i] : T(0);
			T x2 = sc.dim > 2 ? pw[2 * n + i] : T(0);
			xs[i] = Q4<T>{x0, x1, x2, T(0)};
		}
		__syncwarp(gmask);

		KSum<T> e_r1, e_i1, e_r1i1, e_lR, e_lI, e_v;
		int nout = 0;
		for (int s = 0; s < nslot; s++) {
			const int nrow = s * G + lane;
			const bool rowok = nrow < n;
			const Q4<T> xr = rowok ? xs[nrow] : Q4<T>{T(0), T(0), T(0), T(0)};
			KSum<T> acc[8];
			const int base = s * G;
			const int dend = (base + G < n) ? base + G : n;
			fwd_region<T, G, 1, ADJ, HIST>(sc, 0, base, nrow, rowok, xr, xs, coefC, kb, hv, lut, hist, lane, pa, pb, acc, e_v, nout);
			fwd_region<T, G, 2, ADJ, HIST>(sc, base, dend, nrow, rowok, xr, xs, coefC, kb, hv, lut, hist, lane, pa, pb, acc, e_v, nout);
			fwd_region<T, G, 0, ADJ, HIST>(sc, dend, n, nrow, rowok, xr, xs, coefC, kb, hv, lut, hist, lane, pa, pb, acc, e_v, nout);
			const T gRx = acc[0].value(), gRy = acc[1].value(), gRz = acc[2].value();
			const T gIx = acc[3].value(), gIy = acc[4].value(), gIz = acc[5].value();
			if (rowok) {
				e_r1.add(gRx * gRx + gRy * gRy + gRz * gRz);
				e_i1.add(gIx * gIx + gIy * gIy + gIz * gIz);
				e_r1i1.add(T(2) * (gRx * gIx + gRy * gIy + gRz * gIz));
				e_lR.add(acc[6].value());
				e_lI.add(acc[7].value());
				if (ADJ) {
					T* g = Gs + (size_t)nrow * 6;
					g[0] = gRx;
					g[1] = gRy;
					g[2] = gRz;
					g[3] = gIx;
					g[4] = gIy;
					g[5] = gIz;
				}
			}
		}
		// group totals (compensated per lane, then a butterfly over lanes)
		T sR1 = group_sum<T, G>(e_r1.value(), gmask);
		T sI1 = group_sum<T, G>(e_i1.value(), gmask);
		T sR1I1 = group_sum<T, G>(e_r1i1.value(), gmask);
		T sR2 = group_sum<T, G>(e_lR.value(), gmask);
		T sI2 = group_sum<T, G>(e_lI.value(), gmask);
		T vint = group_sum<T, G>(e_v.value(), gmask);
		int nout_all = nout;
#pragma unroll
		for (int o = G / 2; o > 0; o >>= 1) nout_all += __shfl_xor_sync(gmask, nout_all, o, G);

		hist_reduce<T, G, HIST>(hist, red, nbin, NM, lane, gmask);

		if (ADJ) {
			for (int s = 0; s < nslot; s++) {
				const int nrow = s * G + lane;
				const bool rowok = nrow < n;
				const Q4<T> xr = rowok ? xs[nrow] : Q4<T>{T(0), T(0), T(0), T(0)};
				T gn[6] = {0, 0, 0, 0, 0, 0};
				if (rowok)
					for (int k = 0; k < 6; k++) gn[k] = Gs[(size_t)nrow * 6 + k];
				const int base = s * G;
				const int dend = (base + G < n) ? base + G : n;
				rev_region<T, G, false, HIST>(sc, 0, base, nrow, rowok, xr, gn, xs, Gs, kb, hv, lut, hist, lane);
				rev_region<T, G, true, HIST>(sc, base, dend, nrow, rowok, xr, gn, xs, Gs, kb, hv, lut, hist, lane);
			}
			hist_reduce<T, G, HIST>(hist, redr, nbin, kRevMoments, lane, gmask);
		}

		// moments -> spline values: spline sp = j + 3 - q on interval j
		const T dm1 = (T)(sc.dim - 1);
		for (int sp = lane; sp < ns; sp += G) {
			T S = T(0), Lsp = T(0), AR = T(0), AI = T(0);
#pragma unroll
			for (int q = 0; q < 4; q++) {
				const int j = sp - 3 + q;
				if (j < 0 || j >= nbin) continue;
				const T* l = loc_g + ((size_t)j * 4 + q) * 4;
				const T l0 = l[0], l1 = l[1], l2 = l[2], l3 = l[3];
				const T* m = red + (size_t)j * NM;
				S += l0 * m[0] + l1 * m[1] + l2 * m[2] + l3 * m[3];
				if (ADJ) {
					const T hj = sc.uniform ? (T)sc.hinv : hv[j];
					Lsp += T(2) * (hj * hj * (T(2) * l2 * m[0] + T(6) * l3 * m[1]) +
					               dm1 * hj * (l1 * m[4] + T(2) * l2 * m[5] + T(3) * l3 * m[6]));
					const T* g = redr + (size_t)j * kRevMoments;
					AR += hj * (l1 * g[0] + T(2) * l2 * g[1] + T(3) * l3 * g[2]);
					AI += hj * (l1 * g[3] + T(2) * l2 * g[4] + T(3) * l3 * g[5]);
				}
			}
			spl[sp * 4 + 0] = S;
			spl[sp * 4 + 1] = Lsp;
			spl[sp * 4 + 2] = AR;
			spl[sp * 4 + 3] = AI;
		}
		__syncwarp(gmask);
		// fold to the p parameters; ln psi in FP64 (BosonsBulk.cpp:522-539)
		const double c = sc.hbar2_2m;
		double lnp = 0.0;
		for (int k = lane; k < P; k += G) {
			double Ok = 0.0, dR = 0.0, dI = 0.0;
			for (int sp = 0; sp < ns; sp++) {
				const double f = fold_g[(size_t)k * ns + sp];
				if (f == 0.0) continue;
				Ok += f * (double)spl[sp * 4 + 0];
				if (ADJ) {
					dR += f * (2.0 * (double)spl[sp * 4 + 2] + (double)spl[sp * 4 + 1]);
					dI += f * (2.0 * (double)spl[sp * 4 + 3]);
				}
			}
			O_o[(size_t)w * P + k] = (T)Ok;
			if (ADJ) {
				dE_o[((size_t)w * P + k) * 2 + 0] = (T)(-c * dR);
				dE_o[((size_t)w * P + k) * 2 + 1] = (T)(-c * dI);
			}
			lnp += params[k] * Ok;
		}
#pragma unroll
		for (int o = G / 2; o > 0; o >>= 1) lnp += __shfl_xor_sync(gmask, lnp, o, G);
		if (lane == 0) {
			lnp += params[P - 1] * (double)nout_all;
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
		__syncwarp(gmask);
	}
	(void)misc;
}

}  // namespace tdvmc
