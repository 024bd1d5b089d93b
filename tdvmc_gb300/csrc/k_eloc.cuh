// Per-walker local quantities of the pair-spline Jastrow wave function:
// ln psi, O_k = d ln psi / d uR_k (BC-folded spline sums), the complex local
// energy with its kinetic partial sums, and optionally the adjoint
// dE_loc / d alpha_k.  Follows BosonsBulk::CalculateLocalOperators,
// CalculateOtherLocalOperators and CalculateExpectationValues
// (BosonsBulk.cpp:179-218, 220-336, 349-458, 522-545).
//
// One group of G lanes owns one walker; lane l owns row particle n = s*G + l
// of slot s.  Forward sweep with 32-lane groups (half_block_f32 in FP32,
// half_block_s in FP64): every
// unordered pair once in a rotation schedule; the row's complex gradient G_n
// is accumulated in registers with compensated block sums and the partner's
// share travels along the lanes back to the partner's row (the Laplacian of
// ln psi enters only as a total).  Forward sweep otherwise (fwd_region_f2 in
// FP32, fwd_region): each row loops over all partners i (a shared-memory
// broadcast) and counts
// the statistics of the pairs i < n.  O_k is linear in the spline basis and
// is accumulated as per-interval moments sum t^c in lane-private shared
// histograms.  Reverse sweep (adjoint): one pass over unordered pairs that
// recomputes minimum-image distances and accumulates sum t^c g with
// g = (G_n - G_i) . rhat_ni, plus the (D-1)/r term of the Laplacian of O_k,
// which enters the adjoint in the same B' combination; no pair table is
// stored.  Moments are turned into spline values with the local piece
// polynomials and folded to the p parameters at the end.
#pragma once

#include "common.cuh"
#include "k_sample.cuh"

#include <type_traits>

namespace tdvmc {

constexpr int kFwdMoments = 4;  // sum t^c, c = 0..3
constexpr int G32 = 32;
constexpr int kRevMoments = 6;  // complex sum g t^c, c = 0..2 (real part with (D-1)/r)
// slots per interval and lane: the largest moment count of the kernel's
// sweeps (4, or 6 with the adjoint), rounded to whole float4s in that mode
template <int HIST, bool ADJ> struct HistSlots {
	static constexpr int value = ADJ ? (HIST == 1 ? 8 : 6) : 4;
};

// Histogram update modes of the lane-private moment histograms (NMH slots):
//   0  per-lane records, 2-vector read-modify-write   hist[(j*G + lane)*NMH + m]
//   1  float4 read-modify-write      hist4[(j*NMH/4 + m/4)*G + lane].{x,y,z,w}[m%4]
//   2  shared-memory atomic add      layout of 0 (no contention: lane-private)
// In mode 0 a lane's NMH moments of one interval are contiguous (NMH even), so
// they move as 8-byte (FP32) or 16-byte (FP64) vectors; records of 24 or 48
// bytes map the lanes of each access phase to distinct banks.  FP32 records
// of 4 moments move as one float4; FP32 records of 6 moments are split per
// interval into a float4 block and a float2 block,
//   hist[j*6G + lane*4 + m] (m < 4),  hist[j*6G + 4G + lane*2 + m - 4] (m >= 4),
// two accesses instead of three, still one bank group per lane.
template <typename T> struct V2;
template <> struct V2<float> {
	using type = float2;
};
template <> struct V2<double> {
	using type = double2;
};
// A16: the record starts on a 16-byte boundary (FP32 records of 4k values move as float4)
template <int NV, typename T, bool A16 = false>
__device__ __forceinline__ void rec_load(const T* p, T* v) {
	if constexpr (A16 && sizeof(T) == 4 && NV % 4 == 0) {
#pragma unroll
		for (int m = 0; m < NV; m += 4) {
			const float4 a = *reinterpret_cast<const float4*>(p + m);
			v[m] = a.x;
			v[m + 1] = a.y;
			v[m + 2] = a.z;
			v[m + 3] = a.w;
		}
	} else {
		using VT = typename V2<T>::type;
#pragma unroll
		for (int m = 0; m < NV; m += 2) {
			const VT a = *reinterpret_cast<const VT*>(p + m);
			v[m] = a.x;
			v[m + 1] = a.y;
		}
	}
}
template <int NV, typename T, bool A16 = false>
__device__ __forceinline__ void rec_store(T* p, const T* v) {
	if constexpr (A16 && sizeof(T) == 4 && NV % 4 == 0) {
#pragma unroll
		for (int m = 0; m < NV; m += 4) *reinterpret_cast<float4*>(p + m) = float4{v[m], v[m + 1], v[m + 2], v[m + 3]};
	} else {
		using VT = typename V2<T>::type;
#pragma unroll
		for (int m = 0; m < NV; m += 2) *reinterpret_cast<VT*>(p + m) = VT{v[m], v[m + 1]};
	}
}

template <int G>
__device__ __forceinline__ void rec6_load(const float* hist, int j, int lane, float* v) {
	const float* b = hist + (size_t)j * 6 * G;
	const float4 a = *reinterpret_cast<const float4*>(b + lane * 4);
	const float2 c = *reinterpret_cast<const float2*>(b + 4 * G + lane * 2);
	v[0] = a.x;
	v[1] = a.y;
	v[2] = a.z;
	v[3] = a.w;
	v[4] = c.x;
	v[5] = c.y;
}
template <int G>
__device__ __forceinline__ void rec6_store(float* hist, int j, int lane, const float* v) {
	float* b = hist + (size_t)j * 6 * G;
	*reinterpret_cast<float4*>(b + lane * 4) = float4{v[0], v[1], v[2], v[3]};
	*reinterpret_cast<float2*>(b + 4 * G + lane * 2) = float2{v[4], v[5]};
}
// FP32 six-moment records in mode 0 use the split layout
template <int HIST, int NMH, typename T>
constexpr bool kSplit6 = HIST == 0 && NMH == 6 && sizeof(T) == 4;

template <int HIST, int NMH, typename T, int G>
__device__ __forceinline__ void hist_add8(T* __restrict__ hist, int j, int lane, const T (&v)[8], int nv) {
	if (HIST == 1) {
		Q4<T>* h4 = reinterpret_cast<Q4<T>*>(hist) + ((size_t)j * (NMH / 4)) * G + lane;
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
	} else if (HIST == 2) {
		T* hp = hist + ((size_t)j * G + lane) * NMH;
#pragma unroll
		for (int m = 0; m < 8; m++) {
			if (m >= nv) break;
			atomicAdd(hp + m, v[m]);
		}
	} else if constexpr (kSplit6<HIST, NMH, T>) {
		float a[6];
		rec6_load<G>(hist, j, lane, a);
#pragma unroll
		for (int m = 0; m < 6; m++) a[m] += m < nv ? v[m] : 0.f;
		rec6_store<G>(hist, j, lane, a);
	} else {
		T* hp = hist + ((size_t)j * G + lane) * NMH;
		T a[8];
		if (nv == kRevMoments) {
			rec_load<kRevMoments>(hp, a);
#pragma unroll
			for (int m = 0; m < kRevMoments; m++) a[m] += v[m];
			rec_store<kRevMoments>(hp, a);
		} else {
			rec_load<kFwdMoments, T, NMH % 4 == 0>(hp, a);
#pragma unroll
			for (int m = 0; m < kFwdMoments; m++) a[m] += v[m];
			rec_store<kFwdMoments, T, NMH % 4 == 0>(hp, a);
		}
	}
}

// Two partners' moments into lane-private histogram slots (scalar mode): both
// intervals' slots are loaded before anything is stored, so the loads overlap;
// B's record starts from A's updated record when the intervals coincide and is
// stored last, so that one store holds both partners' moments.
template <int NMH, int NV, typename T, int G>
__device__ __forceinline__ void hist_add_pair(T* __restrict__ hist, int jA, const T (&vA)[8], int jB,
                                              const T (&vB)[8], int lane) {
	if constexpr (kSplit6<0, NMH, T> && NV == 6) {
		float a[6], b[6];
		rec6_load<G>(hist, jA, lane, a);
		rec6_load<G>(hist, jB, lane, b);
		const bool same = jA == jB;
#pragma unroll
		for (int m = 0; m < 6; m++) {
			a[m] += vA[m];
			b[m] = (same ? a[m] : b[m]) + vB[m];
		}
		rec6_store<G>(hist, jA, lane, a);
		rec6_store<G>(hist, jB, lane, b);
		return;
	}
	T* hA = hist + ((size_t)jA * G + lane) * NMH;
	T* hB = hist + ((size_t)jB * G + lane) * NMH;
	constexpr bool A16 = NMH % 4 == 0;  // hist starts on a 16-byte boundary
	T a[NV], b[NV];
	rec_load<NV, T, A16>(hA, a);
	rec_load<NV, T, A16>(hB, b);
	const bool same = jA == jB;
#pragma unroll
	for (int m = 0; m < NV; m++) {
		a[m] += vA[m];
		b[m] = (same ? a[m] : b[m]) + vB[m];
	}
	rec_store<NV, T, A16>(hA, a);
	rec_store<NV, T, A16>(hB, b);
}

// value of moment m of interval j summed over the group's lanes
template <int HIST, int NMH, typename T, int G>
__device__ __forceinline__ T hist_sum(const T* __restrict__ hist, int j, int m) {
	T s = T(0);
	if (HIST == 1) {
		const T* h = hist + (((size_t)j * (NMH / 4) + m / 4) * G) * 4 + (m & 3);
#pragma unroll 8
		for (int l = 0; l < G; l++) s += h[l * 4];
	} else if constexpr (kSplit6<HIST, NMH, T>) {
		const T* h = hist + (size_t)j * 6 * G + (m < 4 ? m : 4 * G + (m - 4));
		const int st = m < 4 ? 4 : 2;
#pragma unroll 8
		for (int l = 0; l < G; l++) s += h[l * st];
	} else {
		const T* h = hist + (size_t)j * G * NMH + m;
#pragma unroll 8
		for (int l = 0; l < G; l++) s += h[(size_t)l * NMH];
	}
	return s;
}

// Shared memory layout of the forward kernel k_eloc:
//   CTA:   coefC[3*nbin] (u', u'' coefficients) | kb[nbin] | hv[nbin] | lut[ncell]
//   group: xs[n] {x, y, z, 0} | hist[nbin*4*G] | red[nbin*4]
//   (32-lane groups: xs[n].w holds gRx of the half sweep's rows; gRy..gIz
//   accumulate in the global gradient scratch)
// and of the reverse (adjoint) kernel k_eloc_rev:
//   CTA:   kb[nbin] | hv[nbin] | lut[ncell]
//   group: xs[n] {x, y, z, gRx} | g4[n] {gRy, gRz, gIx, gIy} | gz[n] {gIz} | hist[nbin*NMH*G] | redr[nbin*6]
// The spline values [ns][4] of the last step borrow the start of the (then
// empty) histogram and are cleared after use.
template <typename T>
__host__ __device__ inline size_t eloc_cta_bytes(int nbin, int ncell) {
	size_t b = 3 * (size_t)nbin * sizeof(Q4<T>) + 2 * (size_t)nbin * sizeof(T) + (size_t)ncell * sizeof(int);
	return (b + 31) & ~(size_t)31;
}
__host__ __device__ inline int eloc_hist_slots(bool adj, int hist_mode) {
	return adj ? (hist_mode == 1 ? 8 : 6) : 4;
}
__host__ __device__ inline size_t eloc_hist_len(int nbin, int ns, int G, int slots) {
	size_t h = (size_t)nbin * slots * G;
	return h < (size_t)ns * 4 ? (size_t)ns * 4 : h;
}
template <typename T>
__host__ __device__ inline size_t eloc_group_bytes(int n, int nbin, int ns, int G) {
	size_t b = (size_t)n * sizeof(Q4<T>);
	b += eloc_hist_len(nbin, ns, G, 4) * sizeof(T);
	b += (size_t)nbin * kFwdMoments * sizeof(T);
	return (b + 31) & ~(size_t)31;
}
template <typename T>
__host__ __device__ inline size_t rev_cta_bytes(int nbin, int ncell) {
	size_t b = 2 * (size_t)nbin * sizeof(T) + (size_t)ncell * sizeof(int);
	return (b + 31) & ~(size_t)31;
}
template <typename T>
__host__ __device__ inline size_t rev_group_bytes(int n, int nbin, int ns, int G, int hist_mode) {
	size_t b = 2 * (size_t)n * sizeof(Q4<T>) + (size_t)((n + 7) & ~7) * sizeof(T);  // keeps the histogram 32-byte aligned
	b += eloc_hist_len(nbin, ns, G, eloc_hist_slots(true, hist_mode)) * sizeof(T);
	b += (size_t)nbin * kRevMoments * sizeof(T);
	return (b + 31) & ~(size_t)31;
}

template <typename T, int G>
__device__ __forceinline__ T group_sum(T v, unsigned gmask) {
#pragma unroll
	for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gmask, v, o, G);
	return v;
}

// Cutoff r <= r_max of one pair.  FP32: decided from the FP32 distance except
// within rounding of r_max (rcut_lo < r < rcut_hi), where the distance of the
// same FP32 coordinates is computed again in FP64, as the FP64 path computes
// it.  A pair that crosses r_max moves a whole spline value between O_k and
// the outer-pair count, so a rounding flip there would exceed every FP32
// tolerance; at N = 1000 a few pairs per walker fall in the band.
__device__ __forceinline__ bool cut_fp64(const SysConst& sc, const Q4<float>& a, const Q4<float>& b) {
	const double dx = nic((double)a.x - (double)b.x, sc.L, sc.Lr);
	const double dy = nic((double)a.y - (double)b.y, sc.L, sc.Lr);
	const double dz = nic((double)a.z - (double)b.z, sc.L, sc.Lr);
	return sqrt(fma(dz, dz, fma(dy, dy, dx * dx))) <= sc.rmax;
}
template <typename T>
__device__ __forceinline__ bool within_rmax(const SysConst& sc, T r, const Q4<T>& a, const Q4<T>& b) {
	if constexpr (sizeof(T) == 4) {
		if (fabsf(r - (float)sc.rmax) < sc.rcut_band) return cut_fp64(sc, a, b);
	}
	return r <= (T)sc.rmax;
}
// The same for the pairs (a, b0) and (a, b1) of one f32x2 stream, rows a, b0,
// b1 of xs (indices below n when `valid`).  The coordinates are read again
// from shared memory on the rare FP64 branch, so the hot path keeps no extra
// registers alive for it.
__device__ __forceinline__ void within_rmax2(const SysConst& sc, float r0, float r1, const Q4<float>* xs, int a,
                                             int b0, int b1, bool valid, bool& in0, bool& in1) {
	const float rmax = (float)sc.rmax;
	in0 = r0 <= rmax;
	in1 = r1 <= rmax;
	float d0, d1;
	f2_split(f2_sub(f2_make(r0, r1), f2_make(rmax, rmax)), d0, d1);
	const bool n0 = fabsf(d0) < sc.rcut_band, n1 = fabsf(d1) < sc.rcut_band;
	if (valid && (n0 || n1)) {
		const Q4<float> xa = xs[a];
		if (n0) in0 = cut_fp64(sc, xa, xs[b0]);
		if (n1) in1 = cut_fp64(sc, xa, xs[b1]);
	}
}

// Geometry and spline derivatives of one (row, partner) pair of the forward sweep.
template <typename T> struct FwdPair {
	T dx, dy, dz, r, rinv, t;
	T gR, gI, lR, lI;
	int j;
	bool in;   // counted: a valid pair within r_max
	bool cut;  // within r_max
};

// MIR: the mirrored distance of NUBosonsBulkPB (mirror_r), counted iff r' < r_max.
template <typename T, bool MIR = false>
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
	if constexpr (MIR) {
		mirror_r((T)(2.0 * sc.rmax), q.r, q.rinv, sc.mirror == 2);
		q.cut = q.r < (T)sc.rmax;
	} else {
		q.cut = within_rmax<T>(sc, q.r, xr, xi);
	}
	q.in = ok && q.cut;
	q.j = locate<T>(sc, q.r, kb, hv, lut, q.t);
	const Q4<T> cR = coefC[3 * q.j];
	const Q4<T> cI = coefC[3 * q.j + 1];
	const Q4<T> c2 = coefC[3 * q.j + 2];
	const T t = q.t;
	const T d1R = fma(t, fma(t, cR.z, cR.y), cR.x);
	const T d1I = fma(t, fma(t, cI.z, cI.y), cI.x);
	const T d2R = fma(t, c2.x, cR.w);
	const T d2I = fma(t, c2.y, cI.w);
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
	T v[8] = {on ? T(1) : T(0), ts, t2, t2 * ts, T(0), T(0), T(0), T(0)};
	hist_add8<HIST, HistSlots<HIST, false>::value, T, G>(hist, q.j, lane, v, kFwdMoments);
	vb += on ? pair_pot<T>(sc.pot_kind, q.r, q.rinv, pa, pb) : T(0);
}

// Forward sweep of row nrow against partners [i0, i1), kNp partners per
// iteration so their dependency chains overlap (one warp per SM sub-partition
// is all the shared memory allows).
// ON: 0 = no pair statistics, 1 = all lanes count the pair, 2 = count iff i < nrow.
constexpr int kNp = 2;
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
					nout += (rowok && ii[h] != nrow && c && !q[h].cut) ? 1 : 0;
				}
			}
		}
#pragma unroll
		for (int k = 0; k < 8; k++) acc[k].add(a[k]);
		if (ON != 0) vsum.add(vb);
	}
}

// FP32 forward sweep with partner pairs in f32x2 arithmetic (same pairs,
// masks and statistics as fwd_region): kF2 pairs of partners per iteration,
// each pair one packed instruction stream (differences, minimum image, r^2,
// r, the interval coordinate, the gradient products and the accumulators);
// the pairs are independent chains for the scheduler.  The table-dependent
// derivative polynomials stay scalar.  The local coordinate of a pair outside
// the support (NaN for the self pair) is zeroed before the masks multiply.
// FP32 distances of two pairs in one f32x2 stream (each half of an f32x2
// operation rounds as the scalar one does, so sweep_r reproduces r).  FWD, the
// forward sweeps: pair_r2_f32 (the box length's remainder in r^2) and
// pair_r_newton; the O_k moments, E_loc and the gradients that the adjoint reads
// all come from these.  The adjoint sweeps keep the plain minimum image with Lf
// and r^2 q: at N = 1000, P = 64 on a lattice with a shell of pairs at r_max,
// dE/d alpha agrees with FP64 to 4e-6 relative either way, and the plain form
// costs 8 % less adjoint time (measured).
struct F2Box {
	f2_t Lr, mL, R, lc;
};
__device__ __forceinline__ F2Box f2_box(const SysConst& sc) {
	const float L = (float)sc.L, Lr = (float)sc.Lr;
	return F2Box{f2_make(Lr, Lr), f2_make(-L, -L), f2_make(kRoundF, kRoundF), f2_make(sc.lc, sc.lc)};
}
template <bool FWD>
__device__ __forceinline__ f2_t pair_r_f2(const F2Box& b, f2_t& dx, f2_t& dy, f2_t& dz, float& qa, float& qb) {
	const f2_t kx = f2_sub(f2_fma(dx, b.Lr, b.R), b.R);
	const f2_t ky = f2_sub(f2_fma(dy, b.Lr, b.R), b.R);
	const f2_t kz = f2_sub(f2_fma(dz, b.Lr, b.R), b.R);
	dx = f2_fma(kx, b.mL, dx);
	dy = f2_fma(ky, b.mL, dy);
	dz = f2_fma(kz, b.mL, dz);
	f2_t r2;
	if (FWD) {
		const f2_t kd = f2_fma(kz, dz, f2_fma(ky, dy, f2_mul(kx, dx)));
		r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_fma(dx, dx, f2_mul(kd, b.lc))));
	} else {
		r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
	}
	float ra, rb;
	f2_split(r2, ra, rb);
	qa = rsqrt_(ra);
	qb = rsqrt_(rb);
	if (!FWD) return f2_mul(r2, f2_make(qa, qb));
	return f2_make(pair_r_newton(ra, qa), pair_r_newton(rb, qb));
}

constexpr int kF2 = 2;
template <int G, int ON, bool ADJ, int HIST>
__device__ __forceinline__ void fwd_region_f2(const SysConst& sc, int i0, int i1, int nrow, bool rowok,
                                              const Q4<float>& xr, const Q4<float>* __restrict__ xs,
                                              const Q4<float>* __restrict__ coefC, const float* __restrict__ kb,
                                              const float* __restrict__ hv, const int* __restrict__ lut,
                                              float* __restrict__ hist, int lane, float pa, float pb,
                                              KSum<float>* acc, KSum<float>& vsum, int& nout) {
	const f2_t X2 = f2_make(xr.x, xr.x), Y2 = f2_make(xr.y, xr.y), Z2 = f2_make(xr.z, xr.z);
	const f2_t R2 = f2_make(kRoundF, kRoundF);
	const F2Box box = f2_box(sc);
	const f2_t H2 = f2_make(sc.hf, sc.hf), mh2 = f2_make(-0.5f, -0.5f);
	const float dm1 = (float)(sc.dim - 1);
	const f2_t dm12 = f2_make(dm1, dm1);
	const float ymax = kRoundF + (float)(sc.nbin - 1);
	constexpr int kChunk = 16 * kF2;  // partners per compensated block sum, whole iterations
	for (int c0 = i0; c0 < i1; c0 += kChunk) {
		const int c1 = (c0 + kChunk < i1) ? c0 + kChunk : i1;
		f2_t a2[8];
#pragma unroll
		for (int k = 0; k < 8; k++) a2[k] = f2_make(0.f, 0.f);
		float vb = 0.f;
		for (int i = c0; i < c1; i += 2 * kF2) {
#pragma unroll
			for (int h = 0; h < kF2; h++) {
				const int iA = i + 2 * h, iB = iA + 1;
				const bool haveA = iA < c1, haveB = iB < c1;
				const int ia = haveA ? iA : i, ib = haveB ? iB : i;
				const Q4<float> pA = xs[ia], pB = xs[ib];
				f2_t dx = f2_sub(X2, f2_make(pA.x, pB.x));
				f2_t dy = f2_sub(Y2, f2_make(pA.y, pB.y));
				f2_t dz = f2_sub(Z2, f2_make(pA.z, pB.z));
				float qa, qb;
				const f2_t r = pair_r_f2<true>(box, dx, dy, dz, qa, qb);
				float rA, rB;
				f2_split(r, rA, rB);
				const bool okA = haveA && rowok && ia != nrow, okB = haveB && rowok && ib != nrow;
				bool wA, wB;
				within_rmax2(sc, rA, rB, xs, nrow, ia, ib, rowok, wA, wB);
				const bool inA = okA && wA, inB = okB && wB;
				float tA, tB;
				int jA, jB;
				if (sc.uniform) {
					// floor(x) = round(x - 1/2), x = r / h, clamped to the last interval
					const f2_t x = f2_mul(r, H2);
					float ya, yb;
					f2_split(f2_add(f2_add(x, mh2), R2), ya, yb);
					ya = fminf(ya, ymax);
					yb = fminf(yb, ymax);
					float xa, xb;
					f2_split(f2_sub(x, f2_sub(f2_make(ya, yb), R2)), xa, xb);
					tA = xa;
					tB = xb;
					jA = __float_as_int(ya) - __float_as_int(kRoundF);
					jB = __float_as_int(yb) - __float_as_int(kRoundF);
				} else {
					jA = locate<float>(sc, rA, kb, hv, lut, tA);
					jB = locate<float>(sc, rB, kb, hv, lut, tB);
				}
				tA = inA ? tA : 0.f;
				tB = inB ? tB : 0.f;
				const Q4<float> cRA = coefC[3 * jA], cIA = coefC[3 * jA + 1], c2A = coefC[3 * jA + 2];
				const Q4<float> cRB = coefC[3 * jB], cIB = coefC[3 * jB + 1], c2B = coefC[3 * jB + 2];
				const f2_t d1R =
				    f2_make(fmaf(tA, fmaf(tA, cRA.z, cRA.y), cRA.x), fmaf(tB, fmaf(tB, cRB.z, cRB.y), cRB.x));
				const f2_t d1I =
				    f2_make(fmaf(tA, fmaf(tA, cIA.z, cIA.y), cIA.x), fmaf(tB, fmaf(tB, cIB.z, cIB.y), cIB.x));
				const f2_t d2R = f2_make(fmaf(tA, c2A.x, cRA.w), fmaf(tB, c2B.x, cRB.w));
				const f2_t d2I = f2_make(fmaf(tA, c2A.y, cIA.w), fmaf(tB, c2B.y, cIB.w));
				const f2_t sr = f2_make(inA ? qa : 0.f, inB ? qb : 0.f);
				const f2_t on = f2_make(inA ? 1.f : 0.f, inB ? 1.f : 0.f);
				const f2_t gR = f2_mul(d1R, sr), gI = f2_mul(d1I, sr);
				const f2_t lR = f2_fma(dm12, gR, f2_mul(d2R, on)), lI = f2_fma(dm12, gI, f2_mul(d2I, on));
				a2[0] = f2_fma(gR, dx, a2[0]);
				a2[1] = f2_fma(gR, dy, a2[1]);
				a2[2] = f2_fma(gR, dz, a2[2]);
				a2[3] = f2_fma(gI, dx, a2[3]);
				a2[4] = f2_fma(gI, dy, a2[4]);
				a2[5] = f2_fma(gI, dz, a2[5]);
				a2[6] = f2_add(a2[6], lR);
				a2[7] = f2_add(a2[7], lI);
				if (ON != 0) {
					const bool cA = haveA && ((ON == 1) ? true : (ia < nrow));
					const bool cB = haveB && ((ON == 1) ? true : (ib < nrow));
					const bool sA = inA && cA, sB = inB && cB;
					if (HIST == 0) {
						// moments sum t^c of both counted pairs, one paired update
						const float t2A = tA * tA, t2B = tB * tB;
						const float vA[8] = {sA ? 1.f : 0.f, sA ? tA : 0.f, sA ? t2A : 0.f, sA ? t2A * tA : 0.f,
						                     0.f, 0.f, 0.f, 0.f};
						const float vB[8] = {sB ? 1.f : 0.f, sB ? tB : 0.f, sB ? t2B : 0.f, sB ? t2B * tB : 0.f,
						                     0.f, 0.f, 0.f, 0.f};
						hist_add_pair<HistSlots<HIST, false>::value, kFwdMoments, float, G>(hist, jA, vA, jB, vB, lane);
						vb += sA ? pair_pot<float>(sc.pot_kind, rA, qa, pa, pb) : 0.f;
						vb += sB ? pair_pot<float>(sc.pot_kind, rB, qb, pa, pb) : 0.f;
					} else {
						FwdPair<float> q;
						q.t = tA;
						q.j = jA;
						q.r = rA;
						q.rinv = qa;
						fwd_stats<float, G, ADJ, HIST>(sc, q, sA, hist, lane, pa, pb, vb);
						q.t = tB;
						q.j = jB;
						q.r = rB;
						q.rinv = qb;
						fwd_stats<float, G, ADJ, HIST>(sc, q, sB, hist, lane, pa, pb, vb);
					}
					nout += (okA && cA && !wA) ? 1 : 0;
					nout += (okB && cB && !wB) ? 1 : 0;
				}
			}
		}
#pragma unroll
		for (int k = 0; k < 8; k++) {
			float lo, hi;
			f2_split(a2[k], lo, hi);
			acc[k].add(lo + hi);
		}
		if (ON != 0) vsum.add(vb);
	}
}

// FP32 half sweep of the forward kernel for 32-lane groups: every unordered
// pair once.  Rows come in slots of 32 (row s*32 + lane).  Slot s meets each
// earlier slot sp in 32 rotation steps (at step k lane l pairs with row
// sp*32 + (l + k) mod 32) and its own slot in steps 1..16 (step 16 for lanes
// below 16 only), which meets every unordered pair exactly once.  The row's
// gradient g d stays in registers; the partner's share (-g d) is collected in
// a travelling sum trav that moves down the lanes with the rotation: before
// step k lane l holds the sum for partner (l + k) mod 32, so after the 32
// steps of a block it is back in the partner's lane (own slot: after 16 steps
// it sits 17 lanes on).  kHalfSteps steps per iteration in two f32x2 streams;
// the sum moves once per iteration, fed by one shuffle per step (p_j from
// lane l + kHalfSteps - j), so its dependency chain is one shuffle long.  The
// partners' rows of the next iteration are loaded one iteration ahead.  The
// Laplacian enters the energy only as a total, twice the sum over pairs; the
// pairs beyond r_max are not counted here (the caller takes all pairs less
// the moment-0 total).
constexpr int kHalfSteps = 4;

// Potential of two pairs into vb (pair_pot; Lennard-Jones in f32x2 with the
// same operation order, the other kinds per pair).
__device__ __forceinline__ void pair_pot2(int kind, float rA, float rB, float qa, float qb, bool inA, bool inB,
                                          float pa, float pb, float& vb) {
	float vA, vB;
	if (kind == 3) {
		f2_t s2 = f2_mul(f2_make(pa, pa), f2_make(qa, qb));
		s2 = f2_mul(s2, s2);
		const f2_t s6 = f2_mul(f2_mul(s2, s2), s2);
		const float b4 = 4.f * pb;
		f2_split(f2_mul(f2_mul(f2_make(b4, b4), s6), f2_sub(s6, f2_make(1.f, 1.f))), vA, vB);
	} else {
		vA = pair_pot<float>(kind, rA, qa, pa, pb);
		vB = pair_pot<float>(kind, rB, qb, pa, pb);
	}
	vb += inA ? vA : 0.f;
	vb += inB ? vB : 0.f;
}
template <bool DIAG, bool ADJ, int HIST, bool MIR = false>
__device__ __forceinline__ void half_block_f32(const SysConst& sc, int sp, int n, int lane, int nrow, bool rowok,
                                               const Q4<float>& xr, const Q4<float>* __restrict__ xs,
                                               const Q4<float>* __restrict__ coefC, const float* __restrict__ kb,
                                               const float* __restrict__ hv, const int* __restrict__ lut,
                                               float* __restrict__ hist, float pa, float pb, KSum<float>* own,
                                               float* trav, KSum<float>& elR, KSum<float>& elI, KSum<float>& vsum,
                                               float& nearmin) {
	const float rmax = (float)sc.rmax, m2 = (float)(2.0 * sc.rmax);
	const f2_t RM2 = f2_make(rmax, rmax);
	const f2_t X2 = f2_make(xr.x, xr.x), Y2 = f2_make(xr.y, xr.y), Z2 = f2_make(xr.z, xr.z);
	const f2_t R2 = f2_make(kRoundF, kRoundF);
	const F2Box box = f2_box(sc);
	const f2_t H2 = f2_make(sc.hf, sc.hf), mh2 = f2_make(-0.5f, -0.5f);
	const float dm1 = (float)(sc.dim - 1);
	const f2_t dm12 = f2_make(dm1, dm1);
	const float ymax = kRoundF + (float)(sc.nbin - 1);
	f2_t a2[6], l2R = f2_make(0.f, 0.f), l2I = f2_make(0.f, 0.f);
#pragma unroll
	for (int c = 0; c < 6; c++) a2[c] = f2_make(0.f, 0.f);
	float vb = 0.f;
	constexpr int k0 = DIAG ? 1 : 0, k1 = DIAG ? 17 : 32;
	// partner rows of the next iteration are loaded one iteration ahead
	Q4<float> nxt[kHalfSteps];
#pragma unroll
	for (int j = 0; j < kHalfSteps; j++) {
		const int i = sp * 32 + ((lane + k0 + j) & 31);
		nxt[j] = xs[DIAG && i >= n ? 0 : i];
	}
	for (int k = k0; k < k1; k += kHalfSteps) {
		float pj[kHalfSteps][6];  // g d of each step, R then I, x y z
		Q4<float> cur[kHalfSteps];
#pragma unroll
		for (int j = 0; j < kHalfSteps; j++) cur[j] = nxt[j];
		if (k + kHalfSteps < k1) {
#pragma unroll
			for (int j = 0; j < kHalfSteps; j++) {
				const int i = sp * 32 + ((lane + k + kHalfSteps + j) & 31);
				nxt[j] = xs[DIAG && i >= n ? 0 : i];
			}
		}
#pragma unroll
		for (int h = 0; h < kHalfSteps / 2; h++) {
			const int kA = k + 2 * h, kB = kA + 1;
			// an earlier slot is full; the own slot may be the last, partial one
			const int ia = sp * 32 + ((lane + kA) & 31), ib = sp * 32 + ((lane + kB) & 31);
			const bool okA = DIAG ? (rowok && ia < n && (kA < 16 || (kA == 16 && lane < 16))) : rowok;
			const bool okB = DIAG ? (rowok && ib < n && (kB < 16 || (kB == 16 && lane < 16))) : rowok;
			const Q4<float> pA = cur[2 * h], pB = cur[2 * h + 1];
			f2_t dx = f2_sub(X2, f2_make(pA.x, pB.x));
			f2_t dy = f2_sub(Y2, f2_make(pA.y, pB.y));
			f2_t dz = f2_sub(Z2, f2_make(pA.z, pB.z));
			float qa, qb;
			f2_t r = pair_r_f2<true>(box, dx, dy, dz, qa, qb);
			float rA, rB;
			f2_split(r, rA, rB);
			bool inA, inB;
			if constexpr (MIR) {
				// mirrored distances: no second look.  r' = r_max, where the reference counts
				// the pair outside, has measure zero in FP64; an FP32 r' rounded onto r_max
				// is counted inside, as FP64 counts the pair with probability one
				mirror_r(m2, rA, qa, sc.mirror == 2);
				mirror_r(m2, rB, qb, sc.mirror == 2);
				r = f2_make(rA, rB);
				inA = okA && (rA <= rmax);
				inB = okB && (rB <= rmax);
			} else {
				inA = okA && (rA <= rmax);
				inB = okB && (rB <= rmax);
				// distance to r_max: pairs within rounding of it are decided again after the block
				float da, db;
				f2_split(f2_sub(r, RM2), da, db);
				nearmin = fminf(nearmin, fminf(fabsf(da), fabsf(db)));
			}
			float tA, tB;
			int jA, jB;
			if (sc.uniform) {
				const f2_t x = f2_mul(r, H2);
				float ya, yb;
				f2_split(f2_add(f2_add(x, mh2), R2), ya, yb);
				ya = fminf(ya, ymax);
				yb = fminf(yb, ymax);
				float xa, xb;
				f2_split(f2_sub(x, f2_sub(f2_make(ya, yb), R2)), xa, xb);
				tA = xa;
				tB = xb;
				jA = __float_as_int(ya) - __float_as_int(kRoundF);
				jB = __float_as_int(yb) - __float_as_int(kRoundF);
			} else {
				jA = locate<float>(sc, rA, kb, hv, lut, tA);
				jB = locate<float>(sc, rB, kb, hv, lut, tB);
			}
			tA = inA ? tA : 0.f;
			tB = inB ? tB : 0.f;
			const Q4<float> cRA = coefC[3 * jA], cIA = coefC[3 * jA + 1], c2A = coefC[3 * jA + 2];
			const Q4<float> cRB = coefC[3 * jB], cIB = coefC[3 * jB + 1], c2B = coefC[3 * jB + 2];
			const f2_t d1R = f2_make(fmaf(tA, fmaf(tA, cRA.z, cRA.y), cRA.x), fmaf(tB, fmaf(tB, cRB.z, cRB.y), cRB.x));
			const f2_t d1I = f2_make(fmaf(tA, fmaf(tA, cIA.z, cIA.y), cIA.x), fmaf(tB, fmaf(tB, cIB.z, cIB.y), cIB.x));
			const f2_t d2R = f2_make(fmaf(tA, c2A.x, cRA.w), fmaf(tB, c2B.x, cRB.w));
			const f2_t d2I = f2_make(fmaf(tA, c2A.y, cIA.w), fmaf(tB, c2B.y, cIB.w));
			const f2_t sr = f2_make(inA ? qa : 0.f, inB ? qb : 0.f);
			const f2_t on = f2_make(inA ? 1.f : 0.f, inB ? 1.f : 0.f);
			const f2_t gR = f2_mul(d1R, sr), gI = f2_mul(d1I, sr);
			l2R = f2_add(l2R, f2_fma(dm12, gR, f2_mul(d2R, on)));
			l2I = f2_add(l2I, f2_fma(dm12, gI, f2_mul(d2I, on)));
			const f2_t q[6] = {f2_mul(gR, dx), f2_mul(gR, dy), f2_mul(gR, dz),
			                   f2_mul(gI, dx), f2_mul(gI, dy), f2_mul(gI, dz)};
#pragma unroll
			for (int c = 0; c < 6; c++) {
				a2[c] = f2_add(a2[c], q[c]);
				f2_split(q[c], pj[2 * h][c], pj[2 * h + 1][c]);
			}
			// pair statistics: every pair met here is an unordered pair, counted once
			if (HIST == 0) {
				const float t2A = tA * tA, t2B = tB * tB;
				const float vA[8] = {inA ? 1.f : 0.f, tA, t2A, t2A * tA, 0.f, 0.f, 0.f, 0.f};
				const float vB[8] = {inB ? 1.f : 0.f, tB, t2B, t2B * tB, 0.f, 0.f, 0.f, 0.f};
				hist_add_pair<HistSlots<HIST, false>::value, kFwdMoments, float, G32>(hist, jA, vA, jB, vB, lane);
				pair_pot2(sc.pot_kind, rA, rB, qa, qb, inA, inB, pa, pb, vb);
			} else {
				FwdPair<float> fq;
				fq.t = tA;
				fq.j = jA;
				fq.r = rA;
				fq.rinv = qa;
				fwd_stats<float, G32, ADJ, HIST>(sc, fq, inA, hist, lane, pa, pb, vb);
				fq.t = tB;
				fq.j = jB;
				fq.r = rB;
				fq.rinv = qb;
				fwd_stats<float, G32, ADJ, HIST>(sc, fq, inB, hist, lane, pa, pb, vb);
			}
			// pairs beyond r_max are counted by the caller (all pairs less those in moment 0)
		}
		// trav(l) <- trav(l + S) + p_0(l + S) + p_1(l + S - 1) + ... + p_{S-1}(l + 1), S = kHalfSteps
#pragma unroll
		for (int c = 0; c < 6; c++) {
			float t = __shfl_sync(0xffffffffu, trav[c] + pj[0][c], (lane + kHalfSteps) & 31);
#pragma unroll
			for (int j = 1; j < kHalfSteps; j++) t += __shfl_sync(0xffffffffu, pj[j][c], (lane + kHalfSteps - j) & 31);
			trav[c] = t;
		}
	}
#pragma unroll
	for (int c = 0; c < 6; c++) {
		float lo, hi;
		f2_split(a2[c], lo, hi);
		own[c].add(lo + hi);
	}
	float lo, hi;
	f2_split(l2R, lo, hi);
	elR.add(2.f * (lo + hi));
	f2_split(l2I, lo, hi);
	elI.add(2.f * (lo + hi));
	vsum.add(vb);
}

// The half sweep of half_block_f32 in scalar arithmetic (FP64): the same
// rotation schedule, travelling partner sums and statistics, two steps per
// iteration as independent pairs.
template <typename T, bool DIAG, bool ADJ, int HIST, bool MIR = false>
__device__ __forceinline__ void half_block_s(const SysConst& sc, int sp, int n, int lane, bool rowok,
                                             const Q4<T>& xr, const Q4<T>* __restrict__ xs,
                                             const Q4<T>* __restrict__ coefC, const T* __restrict__ kb,
                                             const T* __restrict__ hv, const int* __restrict__ lut,
                                             T* __restrict__ hist, T pa, T pb, KSum<T>* own, T* trav, KSum<T>& elR,
                                             KSum<T>& elI, KSum<T>& vsum) {
	constexpr int S = 2;  // steps per iteration
	T a[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
	T l2R = T(0), l2I = T(0), vb = T(0);
	constexpr int k0 = DIAG ? 1 : 0, k1 = DIAG ? 17 : 32;
	for (int k = k0; k < k1; k += S) {
		T pj[S][6];
		FwdPair<T> q[S];
#pragma unroll
		for (int h = 0; h < S; h++) {
			const int kk = k + h;
			const int i = sp * 32 + ((lane + kk) & 31);
			const bool ok = DIAG ? (rowok && i < n && (kk < 16 || (kk == 16 && lane < 16))) : rowok;
			q[h] = fwd_pair<T, MIR>(sc, xr, xs[DIAG && i >= n ? 0 : i], ok, coefC, kb, hv, lut);
		}
#pragma unroll
		for (int h = 0; h < S; h++) {
			pj[h][0] = q[h].gR * q[h].dx;
			pj[h][1] = q[h].gR * q[h].dy;
			pj[h][2] = q[h].gR * q[h].dz;
			pj[h][3] = q[h].gI * q[h].dx;
			pj[h][4] = q[h].gI * q[h].dy;
			pj[h][5] = q[h].gI * q[h].dz;
#pragma unroll
			for (int c = 0; c < 6; c++) a[c] += pj[h][c];
			l2R += q[h].lR;
			l2I += q[h].lI;
			fwd_stats<T, G32, ADJ, HIST>(sc, q[h], q[h].in, hist, lane, pa, pb, vb);
		}
		// trav(l) <- trav(l + S) + p_0(l + S) + p_1(l + S - 1) + ... + p_{S-1}(l + 1)
#pragma unroll
		for (int c = 0; c < 6; c++) {
			T t = __shfl_sync(0xffffffffu, trav[c] + pj[0][c], (lane + S) & 31);
#pragma unroll
			for (int j = 1; j < S; j++) t += __shfl_sync(0xffffffffu, pj[j][c], (lane + S - j) & 31);
			trav[c] = t;
		}
	}
#pragma unroll
	for (int c = 0; c < 6; c++) own[c].add(a[c]);
	elR.add(T(2) * l2R);
	elI.add(T(2) * l2I);
	vsum.add(vb);
}

template <typename T, bool DIAG, bool ADJ, int HIST, bool MIR = false>
__device__ __forceinline__ void half_block(const SysConst& sc, int sp, int n, int lane, int nrow, bool rowok,
                                           float& nearmin, const Q4<T>& xr,
                                           const Q4<T>* __restrict__ xs, const Q4<T>* __restrict__ coefC,
                                           const T* __restrict__ kb, const T* __restrict__ hv,
                                           const int* __restrict__ lut, T* __restrict__ hist, T pa, T pb,
                                           KSum<T>* own, T* trav, KSum<T>& elR, KSum<T>& elI, KSum<T>& vsum) {
	if constexpr (std::is_same<T, float>::value)
		half_block_f32<DIAG, ADJ, HIST, MIR>(sc, sp, n, lane, nrow, rowok, xr, xs, coefC, kb, hv, lut, hist, pa, pb, own,
		                                trav, elR, elI, vsum, nearmin);
	else
		half_block_s<T, DIAG, ADJ, HIST, MIR>(sc, sp, n, lane, rowok, xr, xs, coefC, kb, hv, lut, hist, pa, pb, own, trav,
		                                 elR, elI, vsum);
}

// The FP32 distance of a pair exactly as the f32x2 sweeps form it (each half of
// an f32x2 operation rounds like the scalar one), so that a second look at a
// pair sees the decision the sweep took; fwd as in pair_r_f2.
__device__ __forceinline__ float sweep_r(const SysConst& sc, const Q4<float>& a, const Q4<float>& b, float& q,
                                         float& dx, float& dy, float& dz, bool fwd) {
	const float L = (float)sc.L, Lr = (float)sc.Lr;
	if (!fwd) {
		dx = nic(__fsub_rn(a.x, b.x), L, Lr);
		dy = nic(__fsub_rn(a.y, b.y), L, Lr);
		dz = nic(__fsub_rn(a.z, b.z), L, Lr);
		const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
		q = rsqrt_(r2);
		return __fmul_rn(r2, q);
	}
	dx = __fsub_rn(a.x, b.x);
	dy = __fsub_rn(a.y, b.y);
	dz = __fsub_rn(a.z, b.z);
	const float r2 = pair_r2_f32(sc.lc, L, Lr, dx, dy, dz);
	q = rsqrt_(r2);
	return pair_r_newton(r2, q);
}
// interval and local coordinate as the f32x2 sweeps form them (equal widths)
__device__ __forceinline__ int sweep_t(const SysConst& sc, float r, const float* kb, const float* hv, const int* lut,
                                       float& t) {
	if (!sc.uniform) return locate<float>(sc, r, kb, hv, lut, t);
	const float x = __fmul_rn(r, sc.hf);
	const float y = fminf(__fadd_rn(__fadd_rn(x, -0.5f), kRoundF), kRoundF + (float)(sc.nbin - 1));
	t = __fsub_rn(x, __fsub_rn(y, kRoundF));
	return __float_as_int(y) - __float_as_int(kRoundF);
}

// Cutoff fix-up of one block of the FP32 half sweep (half_block_f32): the sweep
// decides r <= r_max from the FP32 distance and records how close any pair
// came to r_max; when a lane's block had a pair within rounding of it, the
// group looks at the block's pairs again, decides those near r_max in FP64 from
// the FP32 coordinates (as the FP64 path does) and, where that decision
// differs, adds or removes the pair's terms.  Rare (a few pairs per walker at
// N = 1000), and a separate function: the sweep's code and registers do not
// carry it.  Phase 1 returns the row's gradient, Laplacian and potential terms
// and updates the moments (lane-private records); phase 2 (after the rows'
// gradients are stored) corrects the partner's gradient, atomically, since
// several lanes may correct one partner (gRx in xs[].w, gRy..gIz in
// gacc[(c-1) n + i]).
struct FixTerms {
	float g[6];
	float lR, lI, v;
};
template <bool DIAG, int HIST>
__device__ __noinline__ FixTerms half_block_fix(SysConst sc, int sp, int n, int lane, int nrow, bool rowok,
                                                Q4<float>* xs, float* gacc, const Q4<float>* coefC, const float* kb,
                                                const float* hv, const int* lut, float* hist, float pa, float pb,
                                                int phase) {
	FixTerms out = {{0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, 0.f, 0.f, 0.f};
	if (!rowok) return out;
	const float rmax = (float)sc.rmax;
	const float dm1 = (float)(sc.dim - 1);
	const Q4<float> xr = xs[nrow];
	constexpr int k0 = DIAG ? 1 : 0, k1 = DIAG ? 17 : 32;
	for (int k = k0; k < k1; k++) {
		const int i = sp * 32 + ((lane + k) & 31);
		if (DIAG && !(i < n && (k < 16 || (k == 16 && lane < 16)))) continue;
		const Q4<float> xi = xs[i];
		float q, dx, dy, dz;
		const float r = sweep_r(sc, xr, xi, q, dx, dy, dz, true);
		if (!(fabsf(__fsub_rn(r, rmax)) < sc.rcut_band)) continue;
		const bool in32 = r <= rmax;
		if (cut_fp64(sc, xr, xi) == in32) continue;
		const float sgn = in32 ? -1.f : 1.f;
		float t;
		const int j = sweep_t(sc, r, kb, hv, lut, t);
		const Q4<float> cR = coefC[3 * j], cI = coefC[3 * j + 1], c2 = coefC[3 * j + 2];
		const float gR = fmaf(t, fmaf(t, cR.z, cR.y), cR.x) * q;
		const float gI = fmaf(t, fmaf(t, cI.z, cI.y), cI.x) * q;
		const float g6[6] = {gR * dx, gR * dy, gR * dz, gI * dx, gI * dy, gI * dz};
		if (phase == 1) {
#pragma unroll
			for (int c = 0; c < 6; c++) out.g[c] += sgn * g6[c];
			out.lR += sgn * 2.f * fmaf(dm1, gR, fmaf(t, c2.x, cR.w));
			out.lI += sgn * 2.f * fmaf(dm1, gI, fmaf(t, c2.y, cI.w));
			out.v += sgn * pair_pot<float>(sc.pot_kind, r, q, pa, pb);
			const float t2 = t * t;
			const float v[8] = {sgn, sgn * t, sgn * t2, sgn * t2 * t, 0.f, 0.f, 0.f, 0.f};
			hist_add8<HIST, HistSlots<HIST, false>::value, float, 32>(hist, j, lane, v, kFwdMoments);
		} else {
			atomicAdd(&xs[i].w, -sgn * g6[0]);
#pragma unroll
			for (int c = 1; c < 6; c++) atomicAdd(&gacc[(size_t)(c - 1) * n + i], -sgn * g6[c]);
		}
	}
	return out;
}

// Cutoff fix-up of one region of the FP32 reverse sweep (rev_region_f2): the
// pairs near r_max whose FP64 decision differs from the sweep's have their
// moment terms added or removed (lane-private histogram records).
struct Grad6 {
	float v[6];
};
template <int G, bool DIAG, int HIST, bool ROT>
__device__ __noinline__ void rev_region_fix(SysConst sc, int i0, int i1, int nrow, bool rowok, Grad6 gn,
                                            const Q4<float>* xs, const Q4<float>* g4, const float* gz,
                                            const float* kb, const float* hv, const int* lut, float* hist, int lane) {
	if (!rowok) return;
	const float rmax = (float)sc.rmax;
	const float dm1 = (float)(sc.dim - 1);
	const Q4<float> xr = xs[nrow];
	const int kend = ROT ? 17 : i1;
	for (int k = ROT ? 1 : i0; k < kend; k++) {
		int i = k;
		if (ROT) {
			i = i0 + ((lane + k) & 31);
			if (!(i < i1 && (k < 16 || lane < 16))) continue;
		} else if (DIAG && !(i < nrow)) {
			continue;
		}
		const Q4<float> xi = xs[i];
		float q, dx, dy, dz;
		const float r = sweep_r(sc, xr, xi, q, dx, dy, dz, false);
		if (!(fabsf(__fsub_rn(r, rmax)) < sc.rcut_band)) continue;
		const bool in32 = r <= rmax;
		if (cut_fp64(sc, xr, xi) == in32) continue;
		const float sgn = in32 ? -1.f : 1.f;
		float t;
		const int j = sweep_t(sc, r, kb, hv, lut, t);
		const Q4<float> gi = g4[i];
		const float gR = ((gn.v[0] - xi.w) * dx + (gn.v[1] - gi.x) * dy + (gn.v[2] - gi.y) * dz + dm1) * q;
		const float gI = ((gn.v[3] - gi.z) * dx + (gn.v[4] - gi.w) * dy + (gn.v[5] - gz[i]) * dz) * q;
		const float t2 = t * t;
		const float v[8] = {sgn * gR, sgn * gR * t, sgn * gR * t2, sgn * gI, sgn * gI * t, sgn * gI * t2, 0.f, 0.f};
		hist_add8<HIST, HistSlots<HIST, true>::value, float, G>(hist, j, lane, v, kRevMoments);
	}
}

// Reverse sweep over unordered pairs (i < nrow) for partners [i0, i1), kNp
// partners per iteration.
template <typename T, int G, bool DIAG, int HIST, bool MIR = false>
__device__ __forceinline__ void rev_region(const SysConst& sc, int i0, int i1, int nrow, bool rowok, const Q4<T>& xr,
                                           const T* gn, const Q4<T>* __restrict__ xs, const Q4<T>* __restrict__ g4,
                                           const T* __restrict__ gz, const T* __restrict__ kb,
                                           const T* __restrict__ hv, const int* __restrict__ lut,
                                           T* __restrict__ hist, int lane) {
	const T L = (T)sc.L, Lr = (T)sc.Lr, rmax = (T)sc.rmax;
	const T dm1 = (T)(sc.dim - 1);
	for (int i = i0; i < i1; i += kNp) {
		T v[kNp][8];
		int jj[kNp];
#pragma unroll
		for (int h = 0; h < kNp; h++) {
			const bool have = i + h < i1;
			const int ii = have ? i + h : i;
			const Q4<T> xi = xs[ii];  // .w = gRx of the partner
			const Q4<T> gi = g4[ii];
			const T giz = gz[ii];
			const T dx = nic(xr.x - xi.x, L, Lr), dy = nic(xr.y - xi.y, L, Lr), dz = nic(xr.z - xi.z, L, Lr);
			const T r2 = dx * dx + dy * dy + dz * dz;
			T rinv = rsqrt_(r2);
			T r = r2 * rinv;
			bool cut;
			if constexpr (MIR) {
				mirror_r((T)(2.0 * sc.rmax), r, rinv, sc.mirror == 2);
				cut = r < rmax;
			} else {
				cut = within_rmax<T>(sc, r, xr, xi);
			}
			const bool on = have && rowok && cut && (DIAG ? (ii < nrow) : true);
			T t;
			jj[h] = locate<T>(sc, r, kb, hv, lut, t);
			t = on ? t : T(0);  // t is NaN for the self pair
			const T sr = on ? rinv : T(0);
			// (G_n - G_i) . rhat plus the (D-1)/r of the Laplacian of B (real part only)
			const T gR = ((gn[0] - xi.w) * dx + (gn[1] - gi.x) * dy + (gn[2] - gi.y) * dz + dm1) * sr;
			const T gI = ((gn[3] - gi.z) * dx + (gn[4] - gi.w) * dy + (gn[5] - giz) * dz) * sr;
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
		for (int h = 0; h < kNp; h++) hist_add8<HIST, HistSlots<HIST, true>::value, T, G>(hist, jj[h], lane, v[h], kRevMoments);
	}
}

// FP32 reverse sweep with partner pairs in f32x2 arithmetic (same pairs and
// moments as rev_region): kF2 packed pairs per iteration.
// ROT (own slot, 32-lane groups): instead of the partners i < nrow of the
// slot [i0, i1), lane l meets row i0 + (l + k) mod 32 at steps k = 1..16
// (step 16 for lanes below 16 only), every unordered pair of the slot once
// with no idle lanes; the pair terms do not depend on which row is first.
template <int G, bool DIAG, int HIST, bool ROT = false, bool MIR = false>
__device__ __forceinline__ void rev_region_f2(const SysConst& sc, int i0, int i1, int nrow, bool rowok,
                                              const Q4<float>& xr, const float* gn, const Q4<float>* __restrict__ xs,
                                              const Q4<float>* __restrict__ g4, const float* __restrict__ gz,
                                              const float* __restrict__ kb, const float* __restrict__ hv,
                                              const int* __restrict__ lut, float* __restrict__ hist, int lane,
                                              float& nearmin) {
	const float rmax = (float)sc.rmax, m2 = (float)(2.0 * sc.rmax);
	const f2_t RM2 = f2_make(rmax, rmax);
	const f2_t X2 = f2_make(xr.x, xr.x), Y2 = f2_make(xr.y, xr.y), Z2 = f2_make(xr.z, xr.z);
	const f2_t R2 = f2_make(kRoundF, kRoundF);
	const F2Box box = f2_box(sc);
	const f2_t H2 = f2_make(sc.hf, sc.hf), mh2 = f2_make(-0.5f, -0.5f);
	const float dm1 = (float)(sc.dim - 1);
	const f2_t dm12 = f2_make(dm1, dm1);
	const float ymax = kRoundF + (float)(sc.nbin - 1);
	f2_t GN[6];
#pragma unroll
	for (int k = 0; k < 6; k++) GN[k] = f2_make(gn[k], gn[k]);
	static_assert(!ROT || (DIAG && G == 32), "rotation only for the own slot of 32-lane groups");
	for (int i = ROT ? 1 : i0; i < (ROT ? 17 : i1); i += 2 * kF2) {
#pragma unroll
		for (int h = 0; h < kF2; h++) {
			int ia, ib;
			bool haveA, haveB;
			if (ROT) {
				const int kA = i + 2 * h, kB = kA + 1;
				ia = i0 + ((lane + kA) & 31);
				ib = i0 + ((lane + kB) & 31);
				haveA = ia < i1 && (kA < 16 || lane < 16);
				haveB = ib < i1 && (kB < 16 || lane < 16);
				ia = haveA ? ia : i0;
				ib = haveB ? ib : i0;
			} else {
				// the off-diagonal range [0, s*G) is a whole number of iterations
				const int iA = i + 2 * h, iB = iA + 1;
				haveA = DIAG ? iA < i1 : true;
				haveB = DIAG ? iB < i1 : true;
				ia = haveA ? iA : i;
				ib = haveB ? iB : i;
			}
			const Q4<float> pA = xs[ia], pB = xs[ib];  // .w = gRx of the partner
			const Q4<float> gA = g4[ia], gB = g4[ib];
			const float zA = gz[ia], zB = gz[ib];
			f2_t dx = f2_sub(X2, f2_make(pA.x, pB.x));
			f2_t dy = f2_sub(Y2, f2_make(pA.y, pB.y));
			f2_t dz = f2_sub(Z2, f2_make(pA.z, pB.z));
			float qa, qb;
			f2_t r = pair_r_f2<false>(box, dx, dy, dz, qa, qb);
			float rA, rB;
			f2_split(r, rA, rB);
			bool cA, cB;
			if constexpr (MIR) {
				// mirrored distances (no second look; r' rounded onto r_max counted inside,
				// as in the forward sweep)
				mirror_r(m2, rA, qa, sc.mirror == 2);
				mirror_r(m2, rB, qb, sc.mirror == 2);
				r = f2_make(rA, rB);
				cA = rA <= rmax;
				cB = rB <= rmax;
			} else {
				cA = rA <= rmax;
				cB = rB <= rmax;
				// distance to r_max: pairs within rounding of it are decided again after the region
				float da, db;
				f2_split(f2_sub(r, RM2), da, db);
				nearmin = fminf(nearmin, fminf(fabsf(da), fabsf(db)));
			}
			const bool onA = haveA && rowok && cA && ((DIAG && !ROT) ? (ia < nrow) : true);
			const bool onB = haveB && rowok && cB && ((DIAG && !ROT) ? (ib < nrow) : true);
			float tA, tB;
			int jA, jB;
			if (sc.uniform) {
				const f2_t x = f2_mul(r, H2);
				float ya, yb;
				f2_split(f2_add(f2_add(x, mh2), R2), ya, yb);
				ya = fminf(ya, ymax);
				yb = fminf(yb, ymax);
				float xa, xb;
				f2_split(f2_sub(x, f2_sub(f2_make(ya, yb), R2)), xa, xb);
				tA = xa;
				tB = xb;
				jA = __float_as_int(ya) - __float_as_int(kRoundF);
				jB = __float_as_int(yb) - __float_as_int(kRoundF);
			} else {
				jA = locate<float>(sc, rA, kb, hv, lut, tA);
				jB = locate<float>(sc, rB, kb, hv, lut, tB);
			}
			const f2_t t = f2_make(onA ? tA : 0.f, onB ? tB : 0.f);  // t is NaN for the self pair
			const f2_t sr = f2_make(onA ? qa : 0.f, onB ? qb : 0.f);
			// (G_n - G_i) . rhat plus the (D-1)/r of the Laplacian of B (real part only)
			const f2_t gR = f2_mul(
			    f2_fma(f2_sub(GN[2], f2_make(gA.y, gB.y)), dz,
			           f2_fma(f2_sub(GN[1], f2_make(gA.x, gB.x)), dy,
			                  f2_fma(f2_sub(GN[0], f2_make(pA.w, pB.w)), dx, dm12))),
			    sr);
			const f2_t gI = f2_mul(
			    f2_fma(f2_sub(GN[5], f2_make(zA, zB)), dz,
			           f2_fma(f2_sub(GN[4], f2_make(gA.w, gB.w)), dy, f2_mul(f2_sub(GN[3], f2_make(gA.z, gB.z)), dx))),
			    sr);
			const f2_t t2 = f2_mul(t, t);
			float v[2][8];
			f2_split(gR, v[0][0], v[1][0]);
			f2_split(f2_mul(gR, t), v[0][1], v[1][1]);
			f2_split(f2_mul(gR, t2), v[0][2], v[1][2]);
			f2_split(gI, v[0][3], v[1][3]);
			f2_split(f2_mul(gI, t), v[0][4], v[1][4]);
			f2_split(f2_mul(gI, t2), v[0][5], v[1][5]);
			v[0][6] = v[0][7] = v[1][6] = v[1][7] = 0.f;
			if (HIST == 0) {
				hist_add_pair<HistSlots<HIST, true>::value, kRevMoments, float, G>(hist, jA, v[0], jB, v[1], lane);
			} else {
				hist_add8<HIST, HistSlots<HIST, true>::value, float, G>(hist, jA, lane, v[0], kRevMoments);
				hist_add8<HIST, HistSlots<HIST, true>::value, float, G>(hist, jB, lane, v[1], kRevMoments);
			}
		}
	}
}

// Sum lane-private histograms into red[nbin*nm] and clear them.
template <typename T, int G, int HIST, int NMH>
__device__ __forceinline__ void hist_reduce(T* hist, T* red, int nbin, int nm, int lane, unsigned gmask) {
	__syncwarp(gmask);
	for (int e = lane; e < nbin * nm; e += G) red[e] = hist_sum<HIST, NMH, T, G>(hist, e / nm, e % nm);
	__syncwarp(gmask);
	for (int e = lane; e < nbin * NMH * G; e += G) hist[e] = T(0);
	__syncwarp(gmask);
}

// Forward kernel: ln psi, O_k, E_loc and the kinetic sums of every walker.
// With ADJ it also writes every particle's complex gradient G_n to
// gout[w][6][n] (gRx gRy gRz gIx gIy gIz) for k_eloc_rev and the B'' part of
// dE_loc/d alpha to dE_o, which k_eloc_rev completes.
// FP32 32-lane groups: at most 2 walkers (64 threads) per block and 5 blocks
// per SM, so that registers (<= 204) and shared memory both allow 10 resident walkers.
// MIR: NUBosonsBulkPB (mirrored distances; 32-lane groups only).
template <typename T, int G, bool ADJ, int HIST, bool MIR = false>
__global__ void __launch_bounds__((G == 32 && sizeof(T) == 4) ? 64 : 128, (G == 32 && sizeof(T) == 4) ? 5 : 1)
    k_eloc(SysConst sc, const DynState* __restrict__ dyn, const Q4<T>* __restrict__ coefC_g,
                                              const T* __restrict__ kb_g, const T* __restrict__ hv_g,
                                              const int* __restrict__ lut_g, const T* __restrict__ loc_g,
                                              const double* __restrict__ fold_g, const double* __restrict__ params,
                                              const T* __restrict__ pos, int64_t nw, T* __restrict__ lnpsi_o,
                                              T* __restrict__ O_o, T* __restrict__ eloc_o, T* __restrict__ other_o,
                                              T* __restrict__ dE_o, T* __restrict__ gout) {
	static_assert(!MIR || G == 32, "mirrored distances: 32-lane groups");
	constexpr int NM = kFwdMoments;
	constexpr int NMH = HistSlots<HIST, false>::value;
	extern __shared__ __align__(32) unsigned char smem_raw[];
	const int nbin = sc.nbin, n = sc.n, ns = sc.ns, P = sc.p;
	Q4<T>* coefC = reinterpret_cast<Q4<T>*>(smem_raw);
	T* kb = reinterpret_cast<T*>(coefC + 3 * nbin);
	T* hv = kb + nbin;
	int* lut = reinterpret_cast<int*>(hv + nbin);
	const size_t cta_b = eloc_cta_bytes<T>(nbin, sc.ncell);
	const size_t grp_b = eloc_group_bytes<T>(n, nbin, ns, G);

	for (int i = threadIdx.x; i < 3 * nbin; i += blockDim.x) coefC[i] = coefC_g[i];
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
	T* hist = reinterpret_cast<T*>(xs + n);
	const size_t hist_len = eloc_hist_len(nbin, ns, G, NMH);
	T* red = hist + hist_len;
	T* spl = hist;  // [ns][4]: S, Lsp, -, -, while the histogram is empty

	for (size_t e = lane; e < hist_len; e += G) hist[e] = T(0);
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
		T* gw = (ADJ || G == 32) ? gout + (size_t)w * 6 * n : nullptr;
		if constexpr (G == 32) {
			// half sweep; row gradients: gRx in xs[row].w, gRy..gIz in the walker's gradient
			// scratch gw[c][row], c = 1..5 (L2-resident while the walker runs).  Lane l only
			// touches rows = l mod 32, so its own reads see its own writes.
			T* gacc = gw + n;
			for (int i = lane; i < n; i += 32)
#pragma unroll
				for (int c = 0; c < 5; c++) gacc[c * n + i] = T(0);
			for (int s = 0; s < nslot; s++) {
				const int nrow = s * 32 + lane;
				const bool rowok = nrow < n;
				const Q4<T> xr = rowok ? xs[nrow] : Q4<T>{T(0), T(0), T(0), T(0)};
				KSum<T> own[6];
				for (int sp = 0; sp < s; sp++) {
					const int pr = sp * 32 + lane;  // an earlier slot is full: pr < n
					T pacc[5];  // the partner row's sums so far, loaded before the block
#pragma unroll
					for (int c = 0; c < 5; c++) pacc[c] = gacc[c * n + pr];
					T trav[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
					float nearmin = 3.0e38f;
					half_block<T, false, ADJ, HIST, MIR>(sc, sp, n, lane, nrow, rowok, nearmin, xr, xs, coefC, kb, hv, lut,
					                                hist, pa, pb, own, trav, e_lR, e_lI, e_v);
					// the partners' shares are home
					xs[pr].w -= trav[0];
#pragma unroll
					for (int c = 0; c < 5; c++) gacc[c * n + pr] = pacc[c] - trav[c + 1];
					if constexpr (std::is_same<T, float>::value) {
						if (__any_sync(0xffffffffu, nearmin < sc.rcut_band)) {
							__syncwarp();
							const FixTerms f = half_block_fix<false, HIST>(sc, sp, n, lane, nrow, rowok, xs, gacc, coefC,
							                                              kb, hv, lut, hist, pa, pb, 1);
#pragma unroll
							for (int c = 0; c < 6; c++) own[c].add(f.g[c]);
							e_lR.add(f.lR);
							e_lI.add(f.lI);
							e_v.add(f.v);
							half_block_fix<false, HIST>(sc, sp, n, lane, nrow, rowok, xs, gacc, coefC, kb, hv, lut, hist,
							                            pa, pb, 2);
							__syncwarp();
						}
					}
				}
				T trav[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
				float nearmin = 3.0e38f;
				half_block<T, true, ADJ, HIST, MIR>(sc, s, n, lane, nrow, rowok, nearmin, xr, xs, coefC, kb, hv, lut, hist,
				                               pa, pb, own, trav, e_lR, e_lI, e_v);
#pragma unroll
				for (int c = 0; c < 6; c++) own[c].add(-__shfl_sync(0xffffffffu, trav[c], (lane + 15) & 31));
				bool fix = false;
				if constexpr (std::is_same<T, float>::value) {
					fix = __any_sync(0xffffffffu, nearmin < sc.rcut_band);
					if (fix) {
						const FixTerms f = half_block_fix<true, HIST>(sc, s, n, lane, nrow, rowok, xs, gacc, coefC, kb,
						                                             hv, lut, hist, pa, pb, 1);
#pragma unroll
						for (int c = 0; c < 6; c++) own[c].add(f.g[c]);
						e_lR.add(f.lR);
						e_lI.add(f.lI);
						e_v.add(f.v);
					}
				}
				if (rowok) {  // later slots add their shares
					xs[nrow].w = own[0].value();
#pragma unroll
					for (int c = 1; c < 6; c++) gacc[(c - 1) * n + nrow] = own[c].value();
				}
				if constexpr (std::is_same<T, float>::value) {
					if (fix) {
						__syncwarp();
						half_block_fix<true, HIST>(sc, s, n, lane, nrow, rowok, xs, gacc, coefC, kb, hv, lut, hist, pa,
						                           pb, 2);
						__syncwarp();
					}
				}
			}
			for (int r = lane; r < n; r += 32) {
				const T gRx = xs[r].w, gRy = gacc[r], gRz = gacc[n + r];
				const T gIx = gacc[2 * n + r], gIy = gacc[3 * n + r], gIz = gacc[4 * n + r];
				e_r1.add(gRx * gRx + gRy * gRy + gRz * gRz);
				e_i1.add(gIx * gIx + gIy * gIy + gIz * gIz);
				e_r1i1.add(T(2) * (gRx * gIx + gRy * gIy + gRz * gIz));
				if (ADJ) gw[r] = gRx;  // gRy..gIz are in place
			}
		} else
		for (int s = 0; s < nslot; s++) {
			const int nrow = s * G + lane;
			const bool rowok = nrow < n;
			const Q4<T> xr = rowok ? xs[nrow] : Q4<T>{T(0), T(0), T(0), T(0)};
			KSum<T> acc[8];
			const int base = s * G;
			const int dend = (base + G < n) ? base + G : n;
			if constexpr (std::is_same<T, float>::value) {
				fwd_region_f2<G, 1, ADJ, HIST>(sc, 0, base, nrow, rowok, xr, xs, coefC, kb, hv, lut, hist, lane, pa, pb, acc, e_v, nout);
				fwd_region_f2<G, 2, ADJ, HIST>(sc, base, dend, nrow, rowok, xr, xs, coefC, kb, hv, lut, hist, lane, pa, pb, acc, e_v, nout);
				fwd_region_f2<G, 0, ADJ, HIST>(sc, dend, n, nrow, rowok, xr, xs, coefC, kb, hv, lut, hist, lane, pa, pb, acc, e_v, nout);
			} else {
				fwd_region<T, G, 1, ADJ, HIST>(sc, 0, base, nrow, rowok, xr, xs, coefC, kb, hv, lut, hist, lane, pa, pb, acc, e_v, nout);
				fwd_region<T, G, 2, ADJ, HIST>(sc, base, dend, nrow, rowok, xr, xs, coefC, kb, hv, lut, hist, lane, pa, pb, acc, e_v, nout);
				fwd_region<T, G, 0, ADJ, HIST>(sc, dend, n, nrow, rowok, xr, xs, coefC, kb, hv, lut, hist, lane, pa, pb, acc, e_v, nout);
			}
			const T gRx = acc[0].value(), gRy = acc[1].value(), gRz = acc[2].value();
			const T gIx = acc[3].value(), gIy = acc[4].value(), gIz = acc[5].value();
			if (rowok) {
				e_r1.add(gRx * gRx + gRy * gRy + gRz * gRz);
				e_i1.add(gIx * gIx + gIy * gIy + gIz * gIz);
				e_r1i1.add(T(2) * (gRx * gIx + gRy * gIy + gRz * gIz));
				e_lR.add(acc[6].value());
				e_lI.add(acc[7].value());
				if (ADJ) {
					gw[nrow] = gRx;
					gw[n + nrow] = gRy;
					gw[2 * n + nrow] = gRz;
					gw[3 * n + nrow] = gIx;
					gw[4 * n + nrow] = gIy;
					gw[5 * n + nrow] = gIz;
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

		hist_reduce<T, G, HIST, NMH>(hist, red, nbin, NM, lane, gmask);
		if constexpr (G == 32) {
			// half sweep: pairs beyond r_max are all pairs less those in moment 0
			// (integer counts below 2^24, exact in FP32)
			T m0 = T(0);
			for (int j = 0; j < nbin; j++) m0 += red[j * NM];
			nout_all = n * (n - 1) / 2 - (int)m0;
		}

		// moments -> spline values: spline sp = j + 3 - q on interval j
		for (int sp = lane; sp < ns; sp += G) {
			T S = T(0), Lsp = T(0);
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
					// B'' part of the Laplacian of O_k; its (D-1)/r B' part comes from k_eloc_rev
					Lsp += T(2) * hj * hj * (T(2) * l2 * m[0] + T(6) * l3 * m[1]);
				}
			}
			spl[sp * 4 + 0] = S;
			spl[sp * 4 + 1] = Lsp;
		}
		__syncwarp(gmask);
		// fold to the p parameters; ln psi in FP64 (BosonsBulk.cpp:522-539)
		const double c = sc.hbar2_2m;
		double lnp = 0.0;
		for (int k = lane; k < P; k += G) {
			double Ok = 0.0, dR = 0.0;
			for (int sp = 0; sp < ns; sp++) {
				const double f = fold_g[(size_t)k * ns + sp];
				if (fold_zero(f)) continue;
				Ok += f * (double)spl[sp * 4 + 0];
				if (ADJ) dR += f * (double)spl[sp * 4 + 1];
			}
			O_o[(size_t)w * P + k] = (T)Ok;
			if (ADJ) {
				dE_o[((size_t)w * P + k) * 2 + 0] = (T)(-c * dR);
				dE_o[((size_t)w * P + k) * 2 + 1] = T(0);
			}
			lnp += params[k] * Ok;
		}
		__syncwarp(gmask);
		for (int e = lane; e < ns * 4; e += G) spl[e] = T(0);  // the histogram starts empty
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

// Reverse (adjoint) kernel: one pass over unordered pairs with the gradients
// of k_eloc, accumulating sum t^c ((G_n - G_i) . rhat_ni + (D-1)/r) per
// interval, then adds 2 sum_n G_n . sD_k + the (D-1)/r B' part of the
// Laplacian of O_k to the dE_o that k_eloc started.
template <typename T, int G, int HIST, bool MIR = false>
__global__ void __launch_bounds__(128, 1) k_eloc_rev(SysConst sc, const T* __restrict__ kb_g, const T* __restrict__ hv_g,
                                                  const int* __restrict__ lut_g, const T* __restrict__ loc_g,
                                                  const double* __restrict__ fold_g, const T* __restrict__ pos,
                                                  const T* __restrict__ gin, int64_t nw, T* __restrict__ dE_o) {
	static_assert(!MIR || G == 32, "mirrored distances: 32-lane groups");
	constexpr int NMH = HistSlots<HIST, true>::value;
	extern __shared__ __align__(32) unsigned char smem_raw[];
	const int nbin = sc.nbin, n = sc.n, ns = sc.ns, P = sc.p;
	T* kb = reinterpret_cast<T*>(smem_raw);
	T* hv = kb + nbin;
	int* lut = reinterpret_cast<int*>(hv + nbin);
	const size_t cta_b = rev_cta_bytes<T>(nbin, sc.ncell);
	const int hist_mode = HIST;
	const size_t grp_b = rev_group_bytes<T>(n, nbin, ns, G, hist_mode);
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
	Q4<T>* g4 = xs + n;
	T* gz = reinterpret_cast<T*>(xs + 2 * n);
	T* hist = gz + (size_t)((n + 7) & ~7);
	const size_t hist_len = eloc_hist_len(nbin, ns, G, NMH);
	T* redr = hist + hist_len;
	T* spl = hist;  // [ns][4]: -, -, AR, AI, while the histogram is empty

	for (size_t e = lane; e < hist_len; e += G) hist[e] = T(0);
	__syncthreads();
	const int nslot = (n + G - 1) / G;

	for (int64_t w = (int64_t)blockIdx.x * gpb + gib; w < nw; w += (int64_t)gridDim.x * gpb) {
		const T* pw = pos + (size_t)w * sc.dim * n;
		const T* gw = gin + (size_t)w * 6 * n;
		for (int i = lane; i < n; i += G) {
			T x0 = pw[i];
			T x1 = sc.dim > 1 ? pw[n + i] : T(0);
			T x2 = sc.dim > 2 ? pw[2 * n + i] : T(0);
			xs[i] = Q4<T>{x0, x1, x2, gw[i]};
			g4[i] = Q4<T>{gw[n + i], gw[2 * n + i], gw[3 * n + i], gw[4 * n + i]};
			gz[i] = gw[5 * n + i];
		}
		__syncwarp(gmask);
		for (int s = 0; s < nslot; s++) {
			const int nrow = s * G + lane;
			const bool rowok = nrow < n;
			const Q4<T> xr = rowok ? xs[nrow] : Q4<T>{T(0), T(0), T(0), T(0)};
			T gn[6] = {0, 0, 0, 0, 0, 0};
			if (rowok) {
				const Q4<T> a = g4[nrow];
				gn[0] = xr.w;
				gn[1] = a.x;
				gn[2] = a.y;
				gn[3] = a.z;
				gn[4] = a.w;
				gn[5] = gz[nrow];
			}
			const int base = s * G;
			const int dend = (base + G < n) ? base + G : n;
			if constexpr (std::is_same<T, float>::value) {
				float nm0 = 3.0e38f, nm1 = 3.0e38f;
				rev_region_f2<G, false, HIST, false, MIR>(sc, 0, base, nrow, rowok, xr, gn, xs, g4, gz, kb, hv, lut, hist,
				                                          lane, nm0);
				rev_region_f2<G, true, HIST, G == 32, MIR>(sc, base, dend, nrow, rowok, xr, gn, xs, g4, gz, kb, hv, lut,
				                                           hist, lane, nm1);
				// pairs within rounding of r_max, decided again in FP64 (rev_region_fix)
				if (__any_sync(gmask, nm0 < sc.rcut_band || nm1 < sc.rcut_band)) {
					const Grad6 g6 = {{gn[0], gn[1], gn[2], gn[3], gn[4], gn[5]}};
					if (__any_sync(gmask, nm0 < sc.rcut_band))
						rev_region_fix<G, false, HIST, false>(sc, 0, base, nrow, rowok, g6, xs, g4, gz, kb, hv, lut, hist,
						                                      lane);
					if (__any_sync(gmask, nm1 < sc.rcut_band))
						rev_region_fix<G, true, HIST, G == 32>(sc, base, dend, nrow, rowok, g6, xs, g4, gz, kb, hv, lut,
						                                       hist, lane);
				}
			} else {
				rev_region<T, G, false, HIST, MIR>(sc, 0, base, nrow, rowok, xr, gn, xs, g4, gz, kb, hv, lut, hist, lane);
				rev_region<T, G, true, HIST, MIR>(sc, base, dend, nrow, rowok, xr, gn, xs, g4, gz, kb, hv, lut, hist, lane);
			}
		}
		hist_reduce<T, G, HIST, NMH>(hist, redr, nbin, kRevMoments, lane, gmask);

		for (int sp = lane; sp < ns; sp += G) {
			T AR = T(0), AI = T(0);
#pragma unroll
			for (int q = 0; q < 4; q++) {
				const int j = sp - 3 + q;
				if (j < 0 || j >= nbin) continue;
				const T* l = loc_g + ((size_t)j * 4 + q) * 4;
				const T l1 = l[1], l2 = l[2], l3 = l[3];
				const T hj = sc.uniform ? (T)sc.hinv : hv[j];
				const T* g = redr + (size_t)j * kRevMoments;
				AR += hj * (l1 * g[0] + T(2) * l2 * g[1] + T(3) * l3 * g[2]);
				AI += hj * (l1 * g[3] + T(2) * l2 * g[4] + T(3) * l3 * g[5]);
			}
			spl[sp * 4 + 2] = AR;
			spl[sp * 4 + 3] = AI;
		}
		__syncwarp(gmask);
		const double c = sc.hbar2_2m;
		for (int k = lane; k < P; k += G) {
			double dR = 0.0, dI = 0.0;
			for (int sp = 0; sp < ns; sp++) {
				const double f = fold_g[(size_t)k * ns + sp];
				if (fold_zero(f)) continue;
				dR += f * (2.0 * (double)spl[sp * 4 + 2]);
				dI += f * (2.0 * (double)spl[sp * 4 + 3]);
			}
			T* d = dE_o + ((size_t)w * P + k) * 2;
			d[0] = (T)((double)d[0] - c * dR);
			d[1] = (T)(-c * dI);
		}
		__syncwarp(gmask);
		for (int e = lane; e < ns * 4; e += G) spl[e] = T(0);  // the histogram starts empty
		__syncwarp(gmask);
	}
}

}  // namespace tdvmc
