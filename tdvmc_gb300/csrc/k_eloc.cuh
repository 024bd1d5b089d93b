// Per-walker local quantities of the pair-spline Jastrow wave function:
// ln psi, O_k = d ln psi / d uR_k (BC-folded spline sums), the complex local
// energy with its kinetic partial sums, and optionally the adjoint
// dE_loc / d alpha_k.  Follows BosonsBulk::CalculateLocalOperators,
// CalculateOtherLocalOperators and CalculateExpectationValues
// (BosonsBulk.cpp:179-218, 220-336, 349-458, 522-545).
//
// One group of G lanes owns one walker.  Rows n = s*G + lane (slot s) are
// lane-owned; each lane walks the half shell of partners i = n + t (mod N),
// t = 1..(N-1)/2 (N even: t = N/2 only for n < N/2), so every unordered pair
// is visited exactly once.  The row's complex gradient G_n and the Laplacian
// accumulate in registers with compensated block sums.  The partner's share
// -g d of G_i travels systolically: the partner accumulator of lane l holds
// the sum for target base + l + t, shifts one lane down per step, and lane 0
// flushes the completed target to shared memory, so no two lanes ever write
// the same entry.  Pair statistics that are linear in the spline basis
// (O_k, and for the adjoint the alpha-independent Laplacian of O_k) are
// accumulated as per-interval moments sum t^c (and sum t^c / r) in
// lane-private shared histograms.  Reverse sweep (adjoint): the same half
// shell once more, recomputing minimum-image distances and accumulating
// sum t^c g with g = (G_n - G_i) . rhat_ni; no pair table is stored.
// Moments are turned into spline values with the local piece polynomials
// and folded to the p parameters at the end.
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
	b += (size_t)n * 8 * sizeof(T);  // G_n: (Re xyz, pad, Im xyz, pad)
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

// Forward sweep of one slot over the half shell (see the file comment).
template <typename T, int G, bool ADJ, int HIST>
__device__ __forceinline__ void fwd_slot(const SysConst& sc, int base, int lane, unsigned gmask,
                                         const Q4<T>* __restrict__ xs, Q4<T>* __restrict__ Gs,
                                         const Q4<T>* __restrict__ coefC, const T* __restrict__ kb,
                                         const T* __restrict__ hv, const int* __restrict__ lut,
                                         T* __restrict__ hist, T pa, T pb, KSum<T>& e_lR, KSum<T>& e_lI,
                                         KSum<T>& e_v, int& nout) {
	const int n = sc.n;
	const int nrow = base + lane;
	const bool rowok = nrow < n;
	const int nr = rowok ? nrow : 0;
	const bool even = (n & 1) == 0;
	const int tmax = even ? n / 2 : (n - 1) / 2;
	const int trow = even ? (nrow < n / 2 ? n / 2 : n / 2 - 1) : tmax;
	const T L = (T)sc.L, Lr = (T)sc.Lr, rmax = (T)sc.rmax, dm1 = (T)(sc.dim - 1);
	const T hu = (T)sc.hinv;
	const Q4<T> xr = xs[nr];
	KSum<T> acc[8];
	// systolic partner accumulator: target index base + lane + t (mod n)
	T p0 = 0, p1 = 0, p2 = 0, p3 = 0, p4 = 0, p5 = 0;
	for (int c0 = 1; c0 <= tmax; c0 += 32) {
		const int c1 = (c0 + 31 < tmax) ? c0 + 31 : tmax;
		T a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
		T vb = T(0);
		for (int t = c0; t <= c1; t++) {
			int i = nr + t;
			i -= (i >= n) ? n : 0;
			const bool valid = rowok && (t <= trow);
			const Q4<T> xi = xs[i];
			const T dx = nic(xr.x - xi.x, L, Lr), dy = nic(xr.y - xi.y, L, Lr), dz = nic(xr.z - xi.z, L, Lr);
			const T r2 = dx * dx + dy * dy + dz * dz;
			const T rinv = rsqrt_(r2);
			const T r = r2 * rinv;
			const bool in = valid && (r <= rmax);
			T tl;
			const int j = locate<T>(sc, r, kb, hv, lut, tl);
			const Q4<T> cR = coefC[2 * j];
			const Q4<T> cI = coefC[2 * j + 1];
			const T hj = sc.uniform ? hu : hv[j];
			const T d1R = (cR.y + tl * (T(2) * cR.z + T(3) * tl * cR.w)) * hj;
			const T d1I = (cI.y + tl * (T(2) * cI.z + T(3) * tl * cI.w)) * hj;
			const T d2R = (T(2) * cR.z + T(6) * tl * cR.w) * (hj * hj);
			const T d2I = (T(2) * cI.z + T(6) * tl * cI.w) * (hj * hj);
			const T gR = in ? d1R * rinv : T(0);
			const T gI = in ? d1I * rinv : T(0);
			const T gRx = gR * dx, gRy = gR * dy, gRz = gR * dz;
			const T gIx = gI * dx, gIy = gI * dy, gIz = gI * dz;
			a[0] += gRx;
			a[1] += gRy;
			a[2] += gRz;
			a[3] += gIx;
			a[4] += gIy;
			a[5] += gIz;
			a[6] += in ? d2R + dm1 * gR : T(0);
			a[7] += in ? d2I + dm1 * gI : T(0);
			p0 -= gRx;
			p1 -= gRy;
			p2 -= gRz;
			p3 -= gIx;
			p4 -= gIy;
			p5 -= gIz;
			// lane 0 holds the completed target base + t: flush it
			if (lane == 0) {
				int k = base + t;
				k -= (k >= n) ? n : 0;
				k -= (k >= n) ? n : 0;
				Q4<T> gr = Gs[2 * k], gi = Gs[2 * k + 1];
				gr.x += p0;
				gr.y += p1;
				gr.z += p2;
				gi.x += p3;
				gi.y += p4;
				gi.z += p5;
				Gs[2 * k] = gr;
				Gs[2 * k + 1] = gi;
			}
			// shift down one lane; lane G-1 starts a fresh target
			p0 = __shfl_down_sync(gmask, p0, 1, G);
			p1 = __shfl_down_sync(gmask, p1, 1, G);
			p2 = __shfl_down_sync(gmask, p2, 1, G);
			p3 = __shfl_down_sync(gmask, p3, 1, G);
			p4 = __shfl_down_sync(gmask, p4, 1, G);
			p5 = __shfl_down_sync(gmask, p5, 1, G);
			if (lane == G - 1) p0 = p1 = p2 = p3 = p4 = p5 = T(0);
			// pair statistics (every visited pair is an unordered pair)
			const T ts = in ? tl : T(0);  // tl is not meaningful outside the cut-off
			const T t2 = ts * ts;
			const T q = in ? rinv : T(0);
			T v[8] = {in ? T(1) : T(0), ts, t2, t2 * ts, q, q * ts, q * t2, T(0)};
			hist_add8<HIST, T, G>(hist, j, lane, v, ADJ ? kFwdMomentsAdj : kFwdMoments);
			vb += in ? pair_pot<T>(sc.pot_kind, r, rinv, pa, pb) : T(0);
			nout += (valid && !(r <= rmax)) ? 1 : 0;
		}
#pragma unroll
		for (int k = 0; k < 8; k++) acc[k].add(a[k]);
		e_v.add(vb);
	}
	// the remaining partner targets base + lane + tmax + 1 (mod n), and the row
	// itself; the targets are distinct across lanes when G <= n, otherwise the
	// lanes flush one after the other
	__syncwarp(gmask);
	{
		int k = base + lane + tmax + 1;
		while (k >= n) k -= n;
		for (int l = (G <= n ? lane : 0); l < (G <= n ? lane + 1 : G); l++) {
			if (l == lane) {
				Q4<T> gr = Gs[2 * k], gi = Gs[2 * k + 1];
				gr.x += p0;
				gr.y += p1;
				gr.z += p2;
				gi.x += p3;
				gi.y += p4;
				gi.z += p5;
				Gs[2 * k] = gr;
				Gs[2 * k + 1] = gi;
			}
			if (G > n) __syncwarp(gmask);
		}
	}
	__syncwarp(gmask);
	if (rowok) {
		Q4<T> gr = Gs[2 * nrow], gi = Gs[2 * nrow + 1];
		gr.x += acc[0].value();
		gr.y += acc[1].value();
		gr.z += acc[2].value();
		gi.x += acc[3].value();
		gi.y += acc[4].value();
		gi.z += acc[5].value();
		Gs[2 * nrow] = gr;
		Gs[2 * nrow + 1] = gi;
		// each unordered pair adds the same Laplacian term to both particles
		e_lR.add(T(2) * acc[6].value());
		e_lI.add(T(2) * acc[7].value());
	}
	__syncwarp(gmask);
}

// Reverse (adjoint) sweep of one slot over the half shell.
template <typename T, int G, int HIST>
__device__ __forceinline__ void rev_slot(const SysConst& sc, int base, int lane, const Q4<T>* __restrict__ xs,
                                         const Q4<T>* __restrict__ Gs, const T* __restrict__ kb,
                                         const T* __restrict__ hv, const int* __restrict__ lut,
                                         T* __restrict__ hist) {
	const int n = sc.n;
	const int nrow = base + lane;
	const bool rowok = nrow < n;
	const int nr = rowok ? nrow : 0;
	const bool even = (n & 1) == 0;
	const int tmax = even ? n / 2 : (n - 1) / 2;
	const int trow = even ? (nrow < n / 2 ? n / 2 : n / 2 - 1) : tmax;
	const T L = (T)sc.L, Lr = (T)sc.Lr, rmax = (T)sc.rmax;
	const Q4<T> xr = xs[nr];
	const Q4<T> gnr = Gs[2 * nr], gni = Gs[2 * nr + 1];
	for (int t = 1; t <= tmax; t++) {
		int i = nr + t;
		i -= (i >= n) ? n : 0;
		const Q4<T> xi = xs[i];
		const Q4<T> gir = Gs[2 * i], gii = Gs[2 * i + 1];
		const T dx = nic(xr.x - xi.x, L, Lr), dy = nic(xr.y - xi.y, L, Lr), dz = nic(xr.z - xi.z, L, Lr);
		const T r2 = dx * dx + dy * dy + dz * dz;
		const T rinv = rsqrt_(r2);
		const T r = r2 * rinv;
		const bool on = rowok && (t <= trow) && (r <= rmax);
		T tl;
		const int j = locate<T>(sc, r, kb, hv, lut, tl);
		tl = on ? tl : T(0);
		const T sr = on ? rinv : T(0);
		const T gR = ((gnr.x - gir.x) * dx + (gnr.y - gir.y) * dy + (gnr.z - gir.z) * dz) * sr;
		const T gI = ((gni.x - gii.x) * dx + (gni.y - gii.y) * dy + (gni.z - gii.z) * dz) * sr;
		const T t2 = tl * tl;
		T v[8] = {gR, gR * tl, gR * t2, gI, gI * tl, gI * t2, T(0), T(0)};
		hist_add8<HIST, T, G>(hist, j, lane, v, kRevMoments);
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
__global__ void __launch_bounds__(128) k_eloc(SysConst sc, const DynState* __restrict__ dyn, const Q4<T>* __restrict__ coefC_g,
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
	Q4<T>* Gs = xs + n;  // 2 per particle: (Re xyz, -), (Im xyz, -)
	T* hist = reinterpret_cast<T*>(Gs + 2 * n);
	T* red = hist + (size_t)nbin * NMH * G;
	T* redr = red + (size_t)nbin * NM;
	T* spl = redr + (ADJ ? (size_t)nbin * kRevMoments : 0);  // [ns][4]: S, Lsp, AR, AI

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
			Gs[2 * i] = Q4<T>{T(0), T(0), T(0), T(0)};
			Gs[2 * i + 1] = Q4<T>{T(0), T(0), T(0), T(0)};
		}
		__syncwarp(gmask);

		KSum<T> e_lR, e_lI, e_v;
		int nout = 0;
		for (int s = 0; s < nslot; s++)
			fwd_slot<T, G, ADJ, HIST>(sc, s * G, lane, gmask, xs, Gs, coefC, kb, hv, lut, hist, pa, pb, e_lR, e_lI,
			                          e_v, nout);
		// kinetic sums of the final gradients (BosonsBulk.cpp:418-420)
		KSum<T> e_r1, e_i1, e_r1i1;
		for (int i = lane; i < n; i += G) {
			const Q4<T> gr = Gs[2 * i], gi = Gs[2 * i + 1];
			e_r1.add(gr.x * gr.x + gr.y * gr.y + gr.z * gr.z);
			e_i1.add(gi.x * gi.x + gi.y * gi.y + gi.z * gi.z);
			e_r1i1.add(T(2) * (gr.x * gi.x + gr.y * gi.y + gr.z * gi.z));
		}
		const T sR1 = group_sum<T, G>(e_r1.value(), gmask);
		const T sI1 = group_sum<T, G>(e_i1.value(), gmask);
		const T sR1I1 = group_sum<T, G>(e_r1i1.value(), gmask);
		const T sR2 = group_sum<T, G>(e_lR.value(), gmask);
		const T sI2 = group_sum<T, G>(e_lI.value(), gmask);
		const T vint = group_sum<T, G>(e_v.value(), gmask);
		int nout_all = nout;
#pragma unroll
		for (int o = G / 2; o > 0; o >>= 1) nout_all += __shfl_xor_sync(gmask, nout_all, o, G);

		hist_reduce<T, G, HIST>(hist, red, nbin, NM, lane, gmask);

		if (ADJ) {
			for (int s = 0; s < nslot; s++) rev_slot<T, G, HIST>(sc, s * G, lane, xs, Gs, kb, hv, lut, hist);
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
}

}  // namespace tdvmc
