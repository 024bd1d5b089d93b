// Batched single-particle Metropolis sampling of the pair-spline Jastrow
// |psi|^2 (DoMetropolisStep, TDVMC.cpp:858-916; ratio from
// BosonsBulk::CalculateWFChange / CalculateWFQuotient, BosonsBulk.cpp:553-657).
//
// One group of G lanes owns one walker at a time (persistent grid-stride
// loop over walkers (start + w) mod nw_total, w < nw, start = *wstart or 0).  Particle i of the walker lives in lane i % G, slot
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

// Pair function at squared distance r2.  coef holds the nbin cubics in the
// centred local coordinate tau = t - 1/2 (better conditioned and one
// operation shorter); entries nbin .. ncoef-1 are the constant outer-pair
// value uR[p-1] (coefficients (u, 0, 0, 0)), selected for r >= r_max.
// MIR (NUBosonsBulkPB): r enters as r' = min(r, 2 r_max - r) (mirror_r), held
// at 0 and above for the phantom slots, whose two terms of a move then read
// the same entry and still cancel exactly.
template <typename T, bool MIR = false>
__device__ __forceinline__ T pair_u(const SysConst& sc, T r2, const Q4<T>* __restrict__ coef,
                                    const T* __restrict__ kb, const T* __restrict__ hv,
                                    const int* __restrict__ lut) {
	T r = pair_r(r2);
	if constexpr (MIR) r = fmax(fmin(r, (T)(2.0 * sc.rmax) - r), T(0));
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

// The samplers hold the particles of a walker in register slots of G lanes
// (particle s*G + lane in slot s), compiled for a few slot counts, so the
// slots past n (a partial slot, and whole slots where the count was rounded
// up) hold no particle.  They hold a phantom three box lengths away on every
// axis instead: per axis min(|d|, L - |d|) is then below -1.5 L, so its
// distance to any position in the box exceeds r_max (at most L/2), both of its
// pair terms in a move read the constant outer-pair entry, and they cancel
// exactly in the move's difference (u - u with finite tau).
constexpr float kPhantomBoxes = 3.0f;

// squared minimum-image distance of two positions inside [-L/2, L/2]:
// per axis min(|d|, L - |d|), exact for |d| <= L (Sterbenz)
template <typename T>
__device__ __forceinline__ T mi_r2(T dx, T dy, T dz, T L) {
	const T ax = fabs(dx), ay = fabs(dy), az = fabs(dz);
	const T mx = fmin(ax, L - ax), my = fmin(ay, L - ay), mz = fmin(az, L - az);
	return fma(mz, mz, fma(my, my, mx * mx));
}

// Shared memory: coef[ncoef][copies] | kb[nbin] | hv[nbin] | lut[ncell] | mirror[groups][n]
// (copies: 1 for k_sample, kCoefCopies for k_sample_f2)
template <typename T>
__host__ __device__ inline size_t sample_smem_bytes(int ncoef, int nbin, int ncell, int n, int groups, int copies = 1) {
	size_t b = (size_t)ncoef * copies * sizeof(Q4<T>) + 2 * (size_t)nbin * sizeof(T) + (size_t)ncell * sizeof(int);
	b = (b + 31) & ~(size_t)31;
	return b + (size_t)groups * n * sizeof(Q4<T>);
}

template <typename T, int G, int SLOTS, bool MIR = false>
__global__ void __launch_bounds__(128) k_sample(SysConst sc, const Q4<T>* __restrict__ coef_g, const T* __restrict__ uout_g,
                                                const T* __restrict__ kb_g, const T* __restrict__ hv_g,
                                                const int* __restrict__ lut_g, T* __restrict__ pos, int64_t nw,
                                                int64_t nw_total, const int32_t* __restrict__ wstart, int moves,
                                                T step, uint2 key, const uint32_t* __restrict__ pass_ptr,
                                                int* __restrict__ acc_out) {
	extern __shared__ __align__(32) unsigned char smem_raw[];
	Q4<T>* coef = reinterpret_cast<Q4<T>*>(smem_raw);
	T* kb = reinterpret_cast<T*>(coef + sc.ncoef);
	T* hv = kb + sc.nbin;
	int* lut = reinterpret_cast<int*>(hv + sc.nbin);
	size_t off = (size_t)sc.ncoef * sizeof(Q4<T>) + 2 * (size_t)sc.nbin * sizeof(T) + (size_t)sc.ncell * sizeof(int);
	off = (off + 31) & ~(size_t)31;
	Q4<T>* mirror_all = reinterpret_cast<Q4<T>*>(smem_raw + off);

	for (int i = threadIdx.x; i < sc.ncoef; i += blockDim.x) coef[i] = coef_g[i];
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
	const int64_t w0 = wstart ? (int64_t)*wstart : 0;
	(void)uout_g;

	for (int64_t wi = (int64_t)blockIdx.x * gpb + gib; wi < nw; wi += (int64_t)gridDim.x * gpb) {
		int64_t w = w0 + wi;
		if (w >= nw_total) w -= nw_total;
		T* pw = pos + (size_t)w * sc.dim * n;
		T x[SLOTS], y[SLOTS], z[SLOTS];
#pragma unroll
		for (int s = 0; s < SLOTS; s++) {
			int i = s * G + lane;
			// slots past n hold the phantom (see kPhantomBoxes)
			x[s] = y[s] = z[s] = (T)kPhantomBoxes * L;
			if (i < n) {
				// positions into [-L/2, L/2] (AlignCoordinates, TDVMC.cpp:2569-2582)
				x[s] = nic(pw[i], L, Lr);
				y[s] = sc.dim > 1 ? nic(pw[n + i], L, Lr) : T(0);
				z[s] = sc.dim > 2 ? nic(pw[2 * n + i], L, Lr) : T(0);
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
					const T un = pair_u<T, MIR>(sc, r2n, coef, kb, hv, lut);
					const T uo = pair_u<T, MIR>(sc, r2o, coef, kb, hv, lut);
					dsum += valid ? (un - uo) : T(0);
				}
#pragma unroll
				for (int o = G / 2; o > 0; o >>= 1) dsum += __shfl_xor_sync(gmask, dsum, o, G);
				// exp(2 delta) >= U; a non-finite or overflowing quotient rejects (TDVMC.cpp:886-915)
				const T two = T(2) * dsum;
				// the bound in T: no float lies between log(DBL_MAX) and its nearest float,
				// so the comparison decides as the double one does
				const bool accept = isfinite(two) && (two >= lum) && (two < (T)kLogDblMax);
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

// ---- packed FP32 pairs (f32x2 arithmetic of sm_100 and later) --------------
// One 64-bit register holds two floats; add/sub/mul/fma.rn.f32x2 round each
// half exactly like the scalar instruction, in one issue slot.
typedef unsigned long long f2_t;
__device__ __forceinline__ f2_t f2_make(float lo, float hi) {
	f2_t r;
	asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
	return r;
}
__device__ __forceinline__ void f2_split(f2_t v, float& lo, float& hi) {
	asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2_t f2_add(f2_t a, f2_t b) {
	f2_t d;
	asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
	return d;
}
__device__ __forceinline__ f2_t f2_sub(f2_t a, f2_t b) {
	f2_t d;
	asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
	return d;
}
__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b) {
	f2_t d;
	asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
	return d;
}
// a * b + c
__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c) {
	f2_t d;
	asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
	return d;
}
__device__ __forceinline__ Q4<float> lds_q4(uint32_t addr) {
	Q4<float> c;
	asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(c.x), "=f"(c.y), "=f"(c.z), "=f"(c.w) : "r"(addr));
	return c;
}

// The packed sampler holds its pair-function table in kCoefCopies interleaved
// copies (entry j of copy c at [j][c]) and lane l reads copy l mod kCoefCopies:
// the 8 lanes of each quarter-warp 16-byte load then hit 8 different bank
// groups whatever entries they read, so the table loads have no bank conflicts.
constexpr int kCoefCopies = 8;

// FP32 sampler for uniform knots with packed pair arithmetic.  It walks the
// same chain as k_sample<float>, bit for bit: same random numbers, moves and
// acceptance rule, and every pair term and partial sum rounded the same way.
// Per register slot the distances of the slot's particle to the proposed and
// to the old position of the moved particle are one f32x2 instruction stream
// from r^2 on (r^2, r, the interval index by the float-rounding trick, the
// local coordinate).  The lane's own coordinates are held once, in slot pairs,
// so the differences of two slots to the moved particle are one f32x2
// subtraction; the per-axis minimum image min(|d|, L - |d|) stays scalar, so
// the min runs on the ALU pipe beside the FMA pipe.  Up to 11 slots the kernel
// is compiled for 5 blocks per SM (a few spilled registers cost less than the
// fifth block gains).  The interval
// index is clamped to the outer-pair entry nbin with one integer min on the
// float's bit pattern, so every pair beyond r_max reads the same (broadcast)
// table entry.  The moved particle's own slot (old distance 0, kept finite by
// a 1e-30 floor on r^2, which is below the rounding of any other r^2) and
// slots past n are left out of the sum by predication.  Every table read is
// in range for any input (r >= 0 puts the rounded index at 0 or above, the
// integer min maps larger, infinite and NaN indices to entry nbin).  A walker
// with a coordinate outside [-L/2, L/2] after wrapping (non-finite or too large
// to wrap exactly) makes no moves, as in the scalar sampler where every
// quotient of such a walker is rejected, and a proposal outside is rejected.
//
// CS (coordinates in shared memory): the lane's own coordinates are read from
// the shared mirror at each move (two 16-byte loads per slot pair) instead of
// being held in registers, for slot counts whose coordinates would not fit in
// registers (32 slots: 96 registers); same arithmetic, same chain.
// MIR (NUBosonsBulkPB): both distances enter as r' = min(r, 2 r_max - r), held
// at 0 and above (pair_u).
template <int G, int SLOTS, bool CS = false, bool MIR = false>
__global__ void __launch_bounds__(128, CS ? (SLOTS > 16 ? 3 : 4) : (SLOTS <= 11 ? 5 : 3)) k_sample_f2(SysConst sc, const Q4<float>* __restrict__ coef_g,
                                                   const float* __restrict__ uout_g, const float* __restrict__ kb_g,
                                                   const float* __restrict__ hv_g, const int* __restrict__ lut_g,
                                                   float* __restrict__ pos, int64_t nw, int64_t nw_total,
                                                   const int32_t* __restrict__ wstart, int moves, float step, uint2 key,
                                                   const uint32_t* __restrict__ pass_ptr, int* __restrict__ acc_out) {
	extern __shared__ __align__(32) unsigned char smem_raw[];
	Q4<float>* coef = reinterpret_cast<Q4<float>*>(smem_raw);
	size_t off = (size_t)sc.ncoef * kCoefCopies * sizeof(Q4<float>) + 2 * (size_t)sc.nbin * sizeof(float) +
	             (size_t)sc.ncell * sizeof(int);
	off = (off + 31) & ~(size_t)31;
	Q4<float>* mirror_all = reinterpret_cast<Q4<float>*>(smem_raw + off);
	for (int i = threadIdx.x; i < sc.ncoef * kCoefCopies; i += blockDim.x) coef[i] = coef_g[i / kCoefCopies];
	__syncthreads();
	(void)uout_g;
	(void)kb_g;
	(void)hv_g;
	(void)lut_g;

	const int n = sc.n;
	const int tid = threadIdx.x;
	const int lane = tid & (G - 1);
	// byte address of entry j of this lane's copy is coef_a + (bits(y) << 7), y = kRoundF + j
	// (128 bytes per entry: the kCoefCopies copies of 16 bytes)
	const uint32_t coef_a = (uint32_t)__cvta_generic_to_shared(coef) + ((uint32_t)(tid & (kCoefCopies - 1)) << 4) -
	                        ((uint32_t)__float_as_uint(kRoundF) << 7);
	const int gib = tid / G;
	const int gpb = blockDim.x / G;
	const unsigned wl = tid & 31;
	const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (wl & ~(unsigned)(G - 1)));
	Q4<float>* xs = mirror_all + (size_t)gib * n;
	const float L = (float)sc.L, Lr = (float)sc.Lr;
	const f2_t R2 = f2_make(kRoundF, kRoundF);
	const f2_t H2 = f2_make((float)sc.hinv, (float)sc.hinv), mhalf2 = f2_make(-0.5f, -0.5f);
	const f2_t tiny2 = f2_make(1e-30f, 1e-30f);
	const uint32_t ymax = __float_as_uint(kRoundF) + (uint32_t)sc.nbin;  // bit pattern of kRoundF + nbin
	const uint32_t pass = *pass_ptr;
	const bool last_ok = (SLOTS - 1) * G + lane < n;
	const float half = 0.5f * L * (1.f + 1e-5f);
	const float m2 = (float)(2.0 * sc.rmax);
	const int64_t w0 = wstart ? (int64_t)*wstart : 0;

	for (int64_t wi = (int64_t)blockIdx.x * gpb + gib; wi < nw; wi += (int64_t)gridDim.x * gpb) {
		int64_t w = w0 + wi;
		if (w >= nw_total) w -= nw_total;
		float* pw = pos + (size_t)w * sc.dim * n;
		// own particles in slot pairs (slot s: pair s / 2, half s % 2), so the
		// differences of two slots to a moving particle are one f32x2 subtraction
		constexpr int NP = (SLOTS + 1) / 2;
		constexpr int NR = CS ? 1 : NP;  // register slot pairs
		f2_t PX[NR], PY[NR], PZ[NR];
		bool inside = true;
		const float ph = kPhantomBoxes * L;
		if (CS) {
			for (int i = lane; i < n; i += G) {
				const float x = nic(pw[i], L, Lr);
				const float y = sc.dim > 1 ? nic(pw[n + i], L, Lr) : 0.f;
				const float z = sc.dim > 2 ? nic(pw[2 * n + i], L, Lr) : 0.f;
				inside = inside && fabsf(x) <= half && fabsf(y) <= half && fabsf(z) <= half;
				xs[i] = Q4<float>{x, y, z, 0.f};
			}
		}
#pragma unroll
		for (int k = 0; k < (CS ? 0 : NP); k++) {
			// slots past n hold the phantom (see kPhantomBoxes)
			float x[2] = {ph, ph}, y[2] = {ph, ph}, z[2] = {ph, ph};
#pragma unroll
			for (int h = 0; h < 2; h++) {
				const int i = (2 * k + h) * G + lane;
				if (2 * k + h < SLOTS && i < n) {
					// positions into [-L/2, L/2] (AlignCoordinates, TDVMC.cpp:2569-2582)
					x[h] = nic(pw[i], L, Lr);
					y[h] = sc.dim > 1 ? nic(pw[n + i], L, Lr) : 0.f;
					z[h] = sc.dim > 2 ? nic(pw[2 * n + i], L, Lr) : 0.f;
					inside = inside && fabsf(x[h]) <= half && fabsf(y[h]) <= half && fabsf(z[h]) <= half;
					xs[i] = Q4<float>{x[h], y[h], z[h], 0.f};
				}
			}
			PX[CS ? 0 : k] = f2_make(x[0], x[1]);
			PY[CS ? 0 : k] = f2_make(y[0], y[1]);
			PZ[CS ? 0 : k] = f2_make(z[0], z[1]);
		}
		const bool walker_ok = __all_sync(gmask, inside);
		__syncwarp(gmask);
		int nacc = 0;
		for (int mb = 0; walker_ok && mb < moves; mb += G) {
			MoveRand<float> rl;
			rl.part = 0;
			rl.u = 1.f;
			rl.z0 = rl.z1 = rl.z2 = 0.f;
			if (mb + lane < moves) rl = move_rand<float>((uint32_t)(mb + lane), (uint32_t)w, pass, key, n, sc.dim);
			const float lu = logf(rl.u);
			const float dz0 = step * rl.z0, dz1 = step * rl.z1, dz2 = step * rl.z2;
			const int nb = (moves - mb) < G ? (moves - mb) : G;
			for (int jm = 0; jm < nb; jm++) {
				const int p = __shfl_sync(gmask, rl.part, jm, G);
				const float lum = __shfl_sync(gmask, lu, jm, G);
				const float e0 = __shfl_sync(gmask, dz0, jm, G);
				const float e1 = __shfl_sync(gmask, dz1, jm, G);
				const float e2 = __shfl_sync(gmask, dz2, jm, G);
				const Q4<float> xo = xs[p];
				const float xn0 = nic(xo.x + e0, L, Lr);
				const float xn1 = nic(xo.y + e1, L, Lr);
				const float xn2 = nic(xo.z + e2, L, Lr);
				if (!(fabsf(xn0) <= half && fabsf(xn1) <= half && fabsf(xn2) <= half)) continue;  // uniform over the group
				const int self_slot = (lane == (p & (G - 1))) ? p / G : -1;
				float dsum = 0.f;
				const f2_t N0 = f2_make(xn0, xn0), N1 = f2_make(xn1, xn1), N2 = f2_make(xn2, xn2);
				const f2_t O0 = f2_make(xo.x, xo.x), O1 = f2_make(xo.y, xo.y), O2 = f2_make(xo.z, xo.z);
				f2_t CX, CY, CZ;  // CS: the slot pair's coordinates, loaded at its first slot
#pragma unroll
				for (int s = 0; s < SLOTS; s++) {
					if (CS && (s & 1) == 0) {
						const int i0 = s * G + lane, i1 = i0 + G;
						const Q4<float> c0 = xs[i0 < n ? i0 : 0];
						const Q4<float> c1 = xs[i1 < n ? i1 : 0];
						CX = f2_make(i0 < n ? c0.x : ph, i1 < n ? c1.x : ph);
						CY = f2_make(i0 < n ? c0.y : ph, i1 < n ? c1.y : ph);
						CZ = f2_make(i0 < n ? c0.z : ph, i1 < n ? c1.z : ph);
					}
					const f2_t SX = CS ? CX : PX[CS ? 0 : s / 2], SY = CS ? CY : PY[CS ? 0 : s / 2];
					const f2_t SZ = CS ? CZ : PZ[CS ? 0 : s / 2];
					float an, ao, bn, bo, cn, co;
					{
						float d[2];
						f2_split(f2_sub(SX, N0), d[0], d[1]);
						an = d[s & 1];
						f2_split(f2_sub(SX, O0), d[0], d[1]);
						ao = d[s & 1];
						f2_split(f2_sub(SY, N1), d[0], d[1]);
						bn = d[s & 1];
						f2_split(f2_sub(SY, O1), d[0], d[1]);
						bo = d[s & 1];
						f2_split(f2_sub(SZ, N2), d[0], d[1]);
						cn = d[s & 1];
						f2_split(f2_sub(SZ, O2), d[0], d[1]);
						co = d[s & 1];
					}
					const f2_t mx = f2_make(fminf(fabsf(an), L - fabsf(an)), fminf(fabsf(ao), L - fabsf(ao)));
					const f2_t my = f2_make(fminf(fabsf(bn), L - fabsf(bn)), fminf(fabsf(bo), L - fabsf(bo)));
					const f2_t mz = f2_make(fminf(fabsf(cn), L - fabsf(cn)), fminf(fabsf(co), L - fabsf(co)));
					const f2_t r2 = f2_fma(mz, mz, f2_fma(my, my, f2_fma(mx, mx, tiny2)));
					float ra, rb;
					f2_split(r2, ra, rb);
					float sa = pair_r(ra), sb = pair_r(rb);
					if constexpr (MIR) {
						sa = fmaxf(fminf(sa, m2 - sa), 0.f);
						sb = fmaxf(fminf(sb, m2 - sb), 0.f);
					}
					const f2_t r = f2_make(sa, sb);
					// floor(x) = round(x - 1/2), x = r / h (see nic)
					const f2_t xm = f2_fma(r, H2, mhalf2);
					const f2_t yv = f2_add(xm, R2);
					const f2_t tau = f2_sub(xm, f2_sub(yv, R2));
					float ya, yb, ta, tb;
					f2_split(yv, ya, yb);
					f2_split(tau, ta, tb);
					const Q4<float> ca = lds_q4(coef_a + (min(__float_as_uint(ya), ymax) << 7));
					const Q4<float> cb = lds_q4(coef_a + (min(__float_as_uint(yb), ymax) << 7));
					const float un = fmaf(ta, fmaf(ta, fmaf(ta, ca.w, ca.z), ca.y), ca.x);
					const float uo = fmaf(tb, fmaf(tb, fmaf(tb, cb.w, cb.z), cb.y), cb.x);
					const bool ok = (s == SLOTS - 1) ? (last_ok && s != self_slot) : (s != self_slot);
					const float du = un - uo;
					if (ok) dsum += du;
				}
#pragma unroll
				for (int o = G / 2; o > 0; o >>= 1) dsum += __shfl_xor_sync(gmask, dsum, o, G);
				// exp(2 delta) >= U; a non-finite or overflowing quotient rejects (TDVMC.cpp:886-915)
				const float two = 2.f * dsum;
				const bool accept = isfinite(two) && (two >= lum) && (two < (float)kLogDblMax);
				if (accept) {
					if constexpr (CS) {
						if (lane == (p & (G - 1))) xs[p] = Q4<float>{xn0, xn1, xn2, 0.f};
					} else if (lane == (p & (G - 1))) {
						xs[p] = Q4<float>{xn0, xn1, xn2, 0.f};
						const float nx = xn0, ny = xn1, nz = xn2;
						switch (p / G) {
#define TDVMC_SET_SLOT(S)                                              \
	case S:                                                            \
		if (S < SLOTS) {                                               \
			constexpr int k = S < SLOTS ? S / 2 : 0;                   \
			float a0, a1;                                              \
			f2_split(PX[k], a0, a1);                                   \
			PX[k] = (S & 1) ? f2_make(a0, nx) : f2_make(nx, a1);       \
			f2_split(PY[k], a0, a1);                                   \
			PY[k] = (S & 1) ? f2_make(a0, ny) : f2_make(ny, a1);       \
			f2_split(PZ[k], a0, a1);                                   \
			PZ[k] = (S & 1) ? f2_make(a0, nz) : f2_make(nz, a1);       \
		}                                                              \
		break;
							TDVMC_SET_SLOT(0) TDVMC_SET_SLOT(1) TDVMC_SET_SLOT(2) TDVMC_SET_SLOT(3)
							TDVMC_SET_SLOT(4) TDVMC_SET_SLOT(5) TDVMC_SET_SLOT(6) TDVMC_SET_SLOT(7)
							TDVMC_SET_SLOT(8) TDVMC_SET_SLOT(9) TDVMC_SET_SLOT(10) TDVMC_SET_SLOT(11)
							TDVMC_SET_SLOT(12) TDVMC_SET_SLOT(13) TDVMC_SET_SLOT(14) TDVMC_SET_SLOT(15)
							TDVMC_SET_SLOT(16) TDVMC_SET_SLOT(17) TDVMC_SET_SLOT(18) TDVMC_SET_SLOT(19)
							TDVMC_SET_SLOT(20) TDVMC_SET_SLOT(21)
#undef TDVMC_SET_SLOT
						}
					}
					nacc++;
				}
				__syncwarp(gmask);
			}
		}
		if (CS && walker_ok) {
			__syncwarp(gmask);
			for (int i = lane; i < n; i += G) {
				const Q4<float> c = xs[i];
				pw[i] = c.x;
				if (sc.dim > 1) pw[n + i] = c.y;
				if (sc.dim > 2) pw[2 * n + i] = c.z;
			}
		}
#pragma unroll
		for (int s = 0; s < SLOTS && walker_ok && !CS; s++) {
			const int i = s * G + lane;
			if (i < n) {
				float d[2];
				f2_split(PX[s / 2], d[0], d[1]);
				pw[i] = d[s & 1];
				f2_split(PY[s / 2], d[0], d[1]);
				if (sc.dim > 1) pw[n + i] = d[s & 1];
				f2_split(PZ[s / 2], d[0], d[1]);
				if (sc.dim > 2) pw[2 * n + i] = d[s & 1];
			}
		}
		if (lane == 0) acc_out[w] = nacc;
		__syncwarp(gmask);
	}
}

}  // namespace tdvmc
