// Device building blocks shared by the TDVP kernels: system constants,
// minimum image, knot-interval location, Philox random numbers and
// compensated sums.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tdvmc {

constexpr int kMaxBins = 128;   // knot intervals on [0, r_max] (p - 1 for uniform knots)
constexpr int kMaxSplines = 130;
constexpr int kMaxP = 128;
constexpr int kMaxLut = 1024;   // non-uniform knots: interval lookup cells
constexpr double kLogDblMax = 709.782712893384;  // log(DBL_MAX): exp(2 delta) overflows beyond

// Static description of a system, passed by value to every kernel.
struct SysConst {
	int n;        // particles per walker
	int dim;      // 1..3 (coordinates beyond dim are zero)
	int p;        // parameters
	int ns;       // splines = p + 2
	int nbin;     // knot intervals on [0, r_max]
	int uniform;  // 1: equal interval widths
	int ncell;    // non-uniform: lookup cells
	int pot_kind;
	int ncoef;    // entries of the sampler's pair-function table (>= nbin + 1)
	double L, Lr;
	double rmax;
	double hinv;      // uniform: 1 / interval width
	double cell_inv;  // non-uniform: 1 / lookup cell width
	double hbar2_2m;
	// 1 / interval width as hf + hf_lo (FP32): hf is what the FP32 kernels use; the
	// stored-sample store forms t = r (hf + hf_lo) - j with one rounding (its piece
	// table is the plain one), the evaluation kernels use pieces composed with the
	// map from their t to the true one
	float hf, hf_lo;
	// FP32 distances with |r - r_max| < rcut_band lie within rounding of r_max:
	// the cutoff of such a pair is decided again in FP64 from its FP32 coordinates
	float rcut_band;
	// -2 (L - Lf), Lf the FP32 box length: the first-order share of the FP32 box
	// length's remainder in the r^2 of a wrapped pair (see pair_r2_f32)
	float lc;
	// NUBosonsBulkPB, a pair at r >= r_max enters at r' = 2 r_max - r (mirror_r):
	// 1 the reference's derivative terms, 2 the exact ones; 0 BosonsBulk
	int mirror;
};

// Values that change between stages or steps live in device memory so a
// captured CUDA graph stays valid: stage parameters, derived spline
// coefficients, potential branch and the Philox pass counter.
struct DynState {
	double pa, pb;      // active potential parameters (after the quench rule)
	uint32_t pass;      // Philox pass counter of the next sampling pass
	uint32_t stage;     // RK stage being computed
	int32_t status;     // OR of TDVMC_ERR_* flags of the solves since last read
	int32_t cs_start;   // first walker of the next stored-sample refresh
};

// Minimum image of one Cartesian difference: d - L * round(d / L)
// (Utils.cpp:266-281).  The rounding uses the float-add trick
// round(x) = (x + 1.5*2^23) - 1.5*2^23 (|x| < 2^22), which keeps the work on
// the FMA pipe instead of the quarter-rate conversion pipe.  It rounds
// exact halves to even where the reference rounds them away from zero, and
// the reference's 1e-10 nudge at exactly +-L/2 is not applied: both differ
// only on a set of measure zero, where the two images are equidistant.
constexpr float kRoundF = 12582912.0f;             // 1.5 * 2^23
constexpr double kRoundD = 6755399441055744.0;     // 1.5 * 2^52
__device__ __forceinline__ float nic(float d, float L, float Lr) {
	const float k = __fadd_rn(__fmaf_rn(d, Lr, kRoundF), -kRoundF);
	return __fmaf_rn(-k, L, d);
}
__device__ __forceinline__ double nic(double d, double L, double Lr) {
	const double k = __dadd_rn(__fma_rn(d, Lr, kRoundD), -kRoundD);
	return __fma_rn(-k, L, d);
}

// FP32 squared pair distance from the raw differences d of two FP32 positions.
// Minimum image d - k Lf, k = rint(d / L), with the FP32 box length Lf.  The
// remainder L - Lf is not subtracted from d: a shifted difference d - k Lf is
// exact on the FP32 grid, so rounding d - k L back to FP32 would move every
// wrapped pair by the same fraction of an ulp, a bias that the splines next to
// r_max = L/2 sum coherently over a dense shell of pairs.  It enters r^2 at
// first order instead, as -2 (L - Lf) sum_a k_a d_a, where the rounding of r^2
// is unbiased.  dx, dy, dz return the shifted differences (the pair direction).
__device__ __forceinline__ float pair_r2_f32(float lc, float L, float Lr, float& dx, float& dy, float& dz) {
	const float kx = __fadd_rn(__fmaf_rn(dx, Lr, kRoundF), -kRoundF);
	const float ky = __fadd_rn(__fmaf_rn(dy, Lr, kRoundF), -kRoundF);
	const float kz = __fadd_rn(__fmaf_rn(dz, Lr, kRoundF), -kRoundF);
	dx = __fmaf_rn(-kx, L, dx);
	dy = __fmaf_rn(-ky, L, dy);
	dz = __fmaf_rn(-kz, L, dz);
	const float kd = __fmaf_rn(kz, dz, __fmaf_rn(ky, dy, __fmul_rn(kx, dx)));
	return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, __fmul_rn(kd, lc))));
}
// FP32 distance from r^2 and q ~ 1/r (hardware rsqrt): r^2 q and one Newton step
// r + (r^2 - r r) q / 2.  The relative error of rsqrt.approx (below 2^-22.9) is
// correlated over a narrow range of r, so without the step it too would enter
// the sums over a shell of pairs coherently; after it r is within about one
// rounding of sqrt(r^2).
__device__ __forceinline__ float pair_r_newton(float r2, float q) {
	const float r = __fmul_rn(r2, q);
	return __fmaf_rn(__fmaf_rn(-r, r, r2), __fmul_rn(0.5f, q), r);
}

// floor(x) for 0 <= x < 2^22 clamped to jmax, as (integer, float), without
// conversion instructions (see nic).
__device__ __forceinline__ int floor_clamp(float x, int jmax, float& jf) {
	float y = __fadd_rn(__fadd_rn(x, -0.5f), kRoundF);
	y = fminf(y, kRoundF + (float)jmax);
	jf = __fadd_rn(y, -kRoundF);
	return __float_as_int(y) - __float_as_int(kRoundF);
}
__device__ __forceinline__ int floor_clamp(double x, int jmax, double& jf) {
	double y = __dadd_rn(__dadd_rn(x, -0.5), kRoundD);
	y = fmin(y, kRoundD + (double)jmax);
	jf = __dadd_rn(y, -kRoundD);
	return (int)(__double_as_longlong(y) - __double_as_longlong(kRoundD));
}

// FP32: the hardware reciprocal square root (PTX rsqrt.approx.ftz.f32) without
// handling for subnormal arguments: squared pair distances are either normal
// or exactly 0 (a masked self pair, giving +inf as before).
__device__ __forceinline__ float rsqrt_(float x) {
	float r;
	asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
	return r;
}
__device__ __forceinline__ double rsqrt_(double x) { return rsqrt(x); }
// Pair distance from its square in the samplers: FP32 the hardware square root
// (PTX sqrt.approx.ftz.f32, one instruction; r^2 is never subnormal there),
// FP64 r^2 / sqrt(r^2) as r^2 * rsqrt(r^2).
__device__ __forceinline__ float pair_r(float r2) {
	float r;
	asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(r2));
	return r;
}
__device__ __forceinline__ double pair_r(double r2) { return r2 * rsqrt_(r2); }

// NUBosonsBulkPB (NUBosonsBulkPB.cpp:249-253, 333-336, 690-693): a pair at
// r >= r_max enters at the mirrored distance r' = 2 r_max - r (m2 = 2 r_max).
// q ~ 1/r is what the derivative terms scale the displacement d and (D-1) by.
// The reference's form: q = 1/r' (correctly rounded), the direction keeping the
// sign of d (its first-derivative factor stays 1, outsideL2 is never set, :387).
// exact: the derivatives of u(2 r_max - r) itself, q = -1/r (d r'/d r = -1).
// Branch-free (about half of the pairs of a bulk system are mirrored); FP32 takes
// the hardware reciprocal (PTX rcp.approx.ftz.f32, as q ~ 1/r is the hardware
// rsqrt), FP64 the correctly rounded one.
__device__ __forceinline__ float rcp_approx(float x) {
	float r;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
	return r;
}
__device__ __forceinline__ void mirror_r(float m2, float& r, float& q, bool exact) {
	const float rm = __fsub_rn(m2, r);
	const bool mir = rm < r;
	const float qm = exact ? -q : rcp_approx(rm);
	r = mir ? rm : r;
	q = mir ? qm : q;
}
__device__ __forceinline__ void mirror_r(double m2, double& r, double& q, bool exact) {
	const double rm = __dsub_rn(m2, r);
	const bool mir = rm < r;
	const double qm = exact ? -q : __drcp_rn(rm);
	r = mir ? rm : r;
	q = mir ? qm : q;
}

// A fold entry that is exactly +0.0, tested on its bit pattern: the ALU's integer
// compare instead of an FP64 compare (the FP64 pipe issues a small fraction of the
// FP32 rate on this GPU); the fold tables hold +0.0, never -0.0, for absent entries.
__device__ __forceinline__ bool fold_zero(double f) { return __double_as_longlong(f) == 0; }

// Interval lookup over [0, r_max]: returns j (interval index; knot k_{j+3})
// and the local coordinate t in [0, 1].  kb[j] = left knot, hv[j] = 1/width,
// lut[c] = first candidate interval of lookup cell c (non-uniform grids).
template <typename T>
__device__ __forceinline__ int locate(const SysConst& s, T r, const T* kb, const T* hv, const int* lut, T& t) {
	if (s.uniform) {
		const T x = r * (T)s.hinv;
		T jf;
		const int j = floor_clamp(x, s.nbin - 1, jf);
		t = x - jf;
		return j;
	}
	int c = (int)(r * (T)s.cell_inv);
	c = c < s.ncell - 1 ? c : s.ncell - 1;
	int j = lut[c];
	if (j + 1 < s.nbin && r >= kb[j + 1]) j++;
	if (j + 1 < s.nbin && r >= kb[j + 1]) j++;
	t = (r - kb[j]) * hv[j];
	return j;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
__device__ __forceinline__ uint4 philox(uint4 c, uint2 k) {
#pragma unroll
	for (int r = 0; r < 10; r++) {
		uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
		uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
		c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
		k.x += 0x9E3779B9u;
		k.y += 0xBB67AE85u;
	}
	return c;
}

// uniform (0,1) from 32 random bits
__device__ __forceinline__ double u01d(uint32_t x) { return ((double)x + 0.5) * (1.0 / 4294967296.0); }
__device__ __forceinline__ float u01f(uint32_t x) { return ((float)(x >> 9) + 0.5f) * (1.0f / 8388608.0f); }

// Random numbers of one Metropolis move: particle, acceptance uniform and
// three standard normals (Box-Muller); the same assignment of Philox words
// as the oracle.
template <typename T> struct MoveRand {
	int part;
	T u, z0, z1, z2;
};

__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, double& c, double& s) {
	double rho = sqrt(-2.0 * log(u01d(a)));
	double sn, cs;
	sincospi(2.0 * u01d(b), &sn, &cs);
	c = rho * cs;
	s = rho * sn;
}
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float& c, float& s) {
	float rho = sqrtf(-2.0f * logf(u01f(a)));
	float sn, cs;
	sincospif(2.0f * u01f(b), &sn, &cs);
	c = rho * cs;
	s = rho * sn;
}
__device__ __forceinline__ double uacc(uint32_t x, double) { return u01d(x); }
__device__ __forceinline__ float uacc(uint32_t x, float) { return u01f(x); }

template <typename T>
__device__ __forceinline__ MoveRand<T> move_rand(uint32_t move, uint32_t walker, uint32_t pass, uint2 key, int n, int dim) {
	MoveRand<T> m;
	uint4 a = philox(make_uint4(move, walker, pass, 0u), key);
	m.part = (int)__umulhi(a.x, (uint32_t)n);
	m.u = uacc(a.y, T(0));
	T c, s;
	box_muller(a.z, a.w, c, s);
	m.z0 = c;
	m.z1 = dim > 1 ? s : T(0);
	m.z2 = T(0);
	if (dim > 2) {
		uint4 b = philox(make_uint4(move, walker, pass, 1u), key);
		T c2, s2;
		box_muller(b.x, b.y, c2, s2);
		m.z2 = c2;
	}
	return m;
}

// Bounded waits on an mbarrier phase (tensor-core commits, TMA bulk copies).
// The bound is wall time from the %globaltimer nanosecond clock, read every 64
// polls, so it does not depend on how long one try_wait suspends.  A kernel
// waits for a completion first with its status limit; if that runs out it
// records the failure and waits again, with the drain limit, for the same
// completion, so no copy or MMA is left in flight when the block moves on or
// exits.  A status limit of 0 gives up without polling (test of the failure
// path).
constexpr uint64_t kWaitStatusNs = 2000000000ull;  // 2 s
constexpr uint64_t kWaitDrainNs = 4000000000ull;   // 4 s
__device__ __forceinline__ uint64_t globaltimer_ns() {
	uint64_t t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
	uint32_t done;
	asm volatile(
	    "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
	    "selp.u32 %0, 1, 0, p;\n\t}\n"
	    : "=r"(done)
	    : "r"(mbar), "r"(parity)
	    : "memory");
	return done != 0;
}
__device__ __forceinline__ bool mbar_wait_ns(uint32_t mbar, uint32_t parity, uint64_t limit_ns) {
	if (limit_ns == 0) return false;
	const uint64_t t0 = globaltimer_ns();
	for (unsigned it = 1;; it++) {
		if (mbar_try_wait(mbar, parity)) return true;
		if ((it & 63u) == 0 && globaltimer_ns() - t0 > limit_ns) return false;
	}
}

// Kahan-compensated running sum.
template <typename T> struct KSum {
	T s, c;
	__device__ __forceinline__ KSum() : s(0), c(0) {}
	__device__ __forceinline__ void add(T x) {
		T y = x - c;
		T t = s + y;
		c = (t - s) - y;
		s = t;
	}
	__device__ __forceinline__ T value() const { return s - c; }
};

// pair potential (a, b from the quench rule): BosonsBulk.cpp:263-271, LJ.cpp:16-22
template <typename T>
__device__ __forceinline__ T pair_pot(int kind, T r, T rinv, T a, T b) {
	if (kind == 1) return r < a ? b : T(0);
	if (kind == 2) {
		T x = r / a;
		return b * exp(-(x * x) * T(0.5));
	}
	if (kind == 3) {
		T s2 = a * rinv;
		s2 = s2 * s2;
		T s6 = s2 * s2 * s2;
		return T(4) * b * s6 * (s6 - T(1));
	}
	return T(0);
}

}  // namespace tdvmc
