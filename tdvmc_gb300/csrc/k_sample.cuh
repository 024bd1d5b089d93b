// Batched single-particle Metropolis sampling of the pair-spline Jastrow
// |psi|^2 (DoMetropolisStep, TDVMC.cpp:858-916; ratio from
// BosonsBulk::CalculateWFChange / CalculateWFQuotient, BosonsBulk.cpp:553-657).
//
// One group of G lanes owns one walker at a time (persistent grid-stride
// loop over walkers).  Particle i of the walker lives in lane i % G, slot
// i / G, in registers; a shared-memory mirror serves the random reads of the
// moved particle.  Per move every lane evaluates u(r) at the old and new
// position against its own particles; a butterfly reduction gives
// delta = ln psi_new - ln psi_old on every lane (bitwise identical), and the
// whole group takes the same decision.
//
// u(r) = sum_s w_s B_s(r) is the BC-folded spline pair function, stored per
// knot interval as one cubic in the local coordinate t (coefU); beyond r_max
// every pair contributes uR[p-1], the reference's outer-pair term
// (BosonsBulk.cpp:531-534, 641-643).
#pragma once

#include "common.cuh"

namespace tdvmc {

template <typename T> struct alignas(4 * sizeof(T)) Q4 {
	T x, y, z, w;
};

// Pair function at squared distance r2.  coef holds nbin + 1 cubics in the
// centred local coordinate tau = t - 1/2 (better conditioned and one
// operation shorter); entry nbin is the constant outer-pair value uR[p-1]
// (coefficients (u, 0, 0, 0)), selected for r >= r_max by the clamp of the
// interval index.
template <typename T>
__device__ __forceinline__ T pair_u(const SysConst& sc, T r2, const Q4<T>* __restrict__ coef,
                                    const T* __restrict__ kb, const T* __restrict__ hv,
                                    const int* __restrict__ lut) {
	const T rinv = rsqrt_(r2);
	const T r = r2 * rinv;
	T tau;
	int j;
	if (sc.uniform) {
		// floor(x) = round(x - 1/2), x = r / h, without conversions (see nic)
		const T xm = fma(r, (T)sc.hinv, T(-0.5));
		const T R = sizeof(T) == 4 ? (T)kRoundF : (T)kRoundD;
		T y = xm + R;
		y = fmin(y, R + (T)sc.nbin);
		const T jf = y - R;
		tau = xm - jf;
		if (sizeof(T) == 4) j = __float_as_int((float)y) - __float_as_int(kRoundF);
		else j = (int)(__double_as_longlong((double)y) - __double_as_longlong(kRoundD));
	} else {
		T t;
		j = locate<T>(sc, r, kb, hv, lut, t);
		j = r < (T)sc.rmax ? j : sc.nbin;
		tau = t - T(0.5);
	}
	const Q4<T> c = coef[j];
	return c.x + tau * (c.y + tau * (c.z + tau * c.w));
}

// squared minimum-image distance of two positions inside [-L/2, L/2]:
// per axis min(|d|, L - |d|), exact for |d| <= L (Sterbenz)
template <typename T>
__device__ __forceinline__ T mi_r2(T dx, T dy, T dz, T L) {
	const T ax = fabs(dx), ay = fabs(dy), az = fabs(dz);
	const T mx = fmin(ax, L - ax), my = fmin(ay, L - ay), mz = fmin(az, L - az);
	return mx * mx + my * my + mz * mz;
}

// Shared memory: coef[nbin] | kb[nbin] | hv[nbin] | lut[ncell] | mirror[groups][n]
template <typename T>
__host__ __device__ inline size_t sample_smem_bytes(int nbin, int ncell, int n, int groups) {
	size_t b = (size_t)(nbin + 1) * sizeof(Q4<T>) + 2 * (size_t)nbin * sizeof(T) + (size_t)ncell * sizeof(int);
	b = (b + 31) & ~(size_t)31;
	return b + (size_t)groups * n * sizeof(Q4<T>);
}

template <typename T, int G, int SLOTS>
__global__ void __launch_bounds__(128) k_sample(SysConst sc, const Q4<T>* __restrict__ coef_g, const T* __restrict__ uout_g,
                                                const T* __restrict__ kb_g, const T* __restrict__ hv_g,
                                                const int* __restrict__ lut_g, T* __restrict__ pos, int64_t nw, int moves,
                                                T step, uint2 key, const uint32_t* __restrict__ pass_ptr,
                                                int* __restrict__ acc_out) {
	extern __shared__ __align__(32) unsigned char smem_raw[];
	Q4<T>* coef = reinterpret_cast<Q4<T>*>(smem_raw);
	T* kb = reinterpret_cast<T*>(coef + sc.nbin + 1);
	T* hv = kb + sc.nbin;
	int* lut = reinterpret_cast<int*>(hv + sc.nbin);
	size_t off = (size_t)(sc.nbin + 1) * sizeof(Q4<T>) + 2 * (size_t)sc.nbin * sizeof(T) + (size_t)sc.ncell * sizeof(int);
	off = (off + 31) & ~(size_t)31;
	Q4<T>* mirror_all = reinterpret_cast<Q4<T>*>(smem_raw + off);

	for (int i = threadIdx.x; i <= sc.nbin; i += blockDim.x) coef[i] = coef_g[i];
	for (int i = threadIdx.x; i < sc.nbin; i += blockDim.x) {
		kb[i] = kb_g[i];
		hv[i] = hv_g[i];
	}
	for (int i = threadIdx.x; i < sc.ncell; i += blockDim.x) lut[i] = lut_g[i];
	__syncthreads();

	const int n = sc.n;
	const int tid = threadIdx.x;
	const int lane = tid & (G - 1);
	const int gib = tid / G;
	const int gpb = blockDim.x / G;
	const unsigned wl = tid & 31;
	const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (wl & ~(unsigned)(G - 1)));
	Q4<T>* xs = mirror_all + (size_t)gib * n;
	const T L = (T)sc.L, Lr = (T)sc.Lr;
	const uint32_t pass = *pass_ptr;
	(void)uout_g;

	for (int64_t w = (int64_t)blockIdx.x * gpb + gib; w < nw; w += (int64_t)gridDim.x * gpb) {
		T* pw = pos + (size_t)w * sc.dim * n;
		T x[SLOTS], y[SLOTS], z[SLOTS];
#pragma unroll
		for (int s = 0; s < SLOTS; s++) {
			int i = s * G + lane;
			x[s] = y[s] = z[s] = T(0);
			if (i < n) {
				// positions into [-L/2, L/2] (AlignCoordinates, TDVMC.cpp:2569-2582)
				x[s] = nic(pw[i], L, Lr);
				if (sc.dim > 1) y[s] = nic(pw[n + i], L, Lr);
				if (sc.dim > 2) z[s] = nic(pw[2 * n + i], L, Lr);
				xs[i] = Q4<T>{x[s], y[s], z[s], T(0)};
			}
		}
		__syncwarp(gmask);
		int nacc = 0;
		for (int mb = 0; mb < moves; mb += G) {
			// lane l draws the random numbers of move mb + l
			MoveRand<T> rl;
			rl.part = 0;
			rl.u = T(1);
			rl.z0 = rl.z1 = rl.z2 = T(0);
			if (mb + lane < moves) rl = move_rand<T>((uint32_t)(mb + lane), (uint32_t)w, pass, key, n, sc.dim);
			T lu = log(rl.u);
			T dz0 = step * rl.z0, dz1 = step * rl.z1, dz2 = step * rl.z2;
			const int nb = (moves - mb) < G ? (moves - mb) : G;
			for (int jm = 0; jm < nb; jm++) {
				const int p = __shfl_sync(gmask, rl.part, jm, G);
				const T lum = __shfl_sync(gmask, lu, jm, G);
				const T e0 = __shfl_sync(gmask, dz0, jm, G);
				const T e1 = __shfl_sync(gmask, dz1, jm, G);
				const T e2 = __shfl_sync(gmask, dz2, jm, G);
				const Q4<T> xo = xs[p];
				const T xn0 = nic(xo.x + e0, L, Lr);
				const T xn1 = nic(xo.y + e1, L, Lr);
				const T xn2 = nic(xo.z + e2, L, Lr);
				// the moved particle's own slot in this lane, -1 elsewhere
				const int self_slot = (lane == (p & (G - 1))) ? p / G : -1;
				T dsum = T(0);
#pragma unroll
				for (int s = 0; s < SLOTS; s++) {
					bool valid = (s != self_slot);
					if (s == SLOTS - 1) valid = valid && (s * G + lane < n);
					const T r2n = mi_r2(x[s] - xn0, y[s] - xn1, z[s] - xn2, L);
					const T r2o = mi_r2(x[s] - xo.x, y[s] - xo.y, z[s] - xo.z, L);
					const T un = pair_u<T>(sc, r2n, coef, kb, hv, lut);
					const T uo = pair_u<T>(sc, r2o, coef, kb, hv, lut);
					dsum += valid ? (un - uo) : T(0);
				}
#pragma unroll
				for (int o = G / 2; o > 0; o >>= 1) dsum += __shfl_xor_sync(gmask, dsum, o, G);
				// exp(2 delta) >= U; a non-finite or overflowing quotient rejects (TDVMC.cpp:886-915)
				const T two = T(2) * dsum;
				const bool accept = isfinite(two) && (two >= lum) && ((double)two < kLogDblMax);
				if (accept) {
					const int owner = p & (G - 1);
					const int sp = p / G;
					if (lane == owner) {
						xs[p] = Q4<T>{xn0, xn1, xn2, T(0)};
#pragma unroll
						for (int s = 0; s < SLOTS; s++)
							if (s == sp) {
								x[s] = xn0;
								y[s] = xn1;
								z[s] = xn2;
							}
					}
					nacc++;
				}
				__syncwarp(gmask);
			}
		}
#pragma unroll
		for (int s = 0; s < SLOTS; s++) {
			int i = s * G + lane;
			if (i < n) {
				pw[i] = x[s];
				if (sc.dim > 1) pw[n + i] = y[s];
				if (sc.dim > 2) pw[2 * n + i] = z[s];
			}
		}
		if (lane == 0) acc_out[w] = nacc;
		__syncwarp(gmask);
	}
}

}  // namespace tdvmc
