// Pair distribution g(r) and static structure factor S(k) of every walker
// (BosonsBulk::CalculateAdditionalSystemProperties, BosonsBulk.cpp:474-520).
//
// One warp per walker.  g(r): the pairs i < j with r < r_max are counted per
// bin floor(r / spacing) in a warp-private shared histogram of 32-bit integer
// counts (exact, order independent) that is added to 64-bit global counts once
// per warp; the host applies the reference's weight D/(N-1) and shell volumes.
// S(k): lanes over particles, per shell the sums of cos and sin of k.r over
// the shell's vectors and the particles, then (C^2 + S^2) / (N * vectors) per
// walker; the host averages the walkers in a fixed order.
#pragma once

#include "common.cuh"

namespace tdvmc {

// Shared memory: kvec[nvec][3] | per warp: xs[n] | hist[count]
template <typename T>
__host__ __device__ inline size_t obs_smem_bytes(int n, int count, int nvec, int warps) {
	size_t b = (size_t)nvec * 3 * sizeof(T);
	b = (b + 15) & ~(size_t)15;
	size_t per = (size_t)n * sizeof(Q4<T>) + (size_t)count * sizeof(uint32_t);
	per = (per + 15) & ~(size_t)15;
	return b + (size_t)warps * per;
}

template <typename T>
__global__ void __launch_bounds__(128) k_observables(SysConst sc, const T* __restrict__ pos, int64_t nw, int count,
                                                     double spacing, const T* __restrict__ kvec_g, int nvec,
                                                     const int* __restrict__ shell_off, int nshell,
                                                     unsigned long long* __restrict__ gr_counts,
                                                     double* __restrict__ sk_w) {
	extern __shared__ __align__(32) unsigned char smem_raw[];
	const int n = sc.n;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
	T* kvec = reinterpret_cast<T*>(smem_raw);
	size_t off = ((size_t)nvec * 3 * sizeof(T) + 15) & ~(size_t)15;
	size_t per = (size_t)n * sizeof(Q4<T>) + (size_t)count * sizeof(uint32_t);
	per = (per + 15) & ~(size_t)15;
	Q4<T>* xs = reinterpret_cast<Q4<T>*>(smem_raw + off + (size_t)warp * per);
	uint32_t* hist = reinterpret_cast<uint32_t*>(xs + n);
	for (int i = threadIdx.x; i < nvec * 3; i += blockDim.x) kvec[i] = kvec_g[i];
	for (int b = lane; b < count; b += 32) hist[b] = 0u;
	__syncthreads();

	const T L = (T)sc.L, Lr = (T)sc.Lr, rmax = (T)sc.rmax, h = (T)spacing;
	for (int64_t w = (int64_t)blockIdx.x * wpb + warp; w < nw; w += (int64_t)gridDim.x * wpb) {
		const T* pw = pos + (size_t)w * sc.dim * n;
		for (int i = lane; i < n; i += 32) {
			const T x0 = nic(pw[i], L, Lr);
			const T x1 = sc.dim > 1 ? nic(pw[n + i], L, Lr) : T(0);
			const T x2 = sc.dim > 2 ? nic(pw[2 * n + i], L, Lr) : T(0);
			xs[i] = Q4<T>{x0, x1, x2, T(0)};
		}
		__syncwarp();
		// g(r): row i (lane-strided) against partners j < i
		for (int i = lane; i < n; i += 32) {
			const Q4<T> a = xs[i];
			for (int j = 0; j < i; j++) {
				const Q4<T> b = xs[j];
				const T dx = nic(a.x - b.x, L, Lr), dy = nic(a.y - b.y, L, Lr), dz = nic(a.z - b.z, L, Lr);
				const T r = sqrt(fma(dz, dz, fma(dy, dy, dx * dx)));
				if (r < rmax) {
					const int bin = (int)floor(r / h);  // Grid::GetIndex
					if (bin < count) atomicAdd(&hist[bin], 1u);
				}
			}
		}
		// S(k): per shell sums over its vectors and the particles
		for (int k = 0; k < nshell; k++) {
			T cs = T(0), sn = T(0);
			for (int v = shell_off[k]; v < shell_off[k + 1]; v++) {
				const T kx = kvec[3 * v], ky = kvec[3 * v + 1], kz = kvec[3 * v + 2];
				for (int i = lane; i < n; i += 32) {
					const Q4<T> a = xs[i];
					T s, c;
					sincos(fma(kz, a.z, fma(ky, a.y, kx * a.x)), &s, &c);
					cs += c;
					sn += s;
				}
			}
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) {
				cs += __shfl_xor_sync(0xffffffffu, cs, o);
				sn += __shfl_xor_sync(0xffffffffu, sn, o);
			}
			if (lane == 0) {
				const int nv = shell_off[k + 1] - shell_off[k];
				const double C = (double)cs, S = (double)sn;
				sk_w[(size_t)w * nshell + k] = nv > 0 ? (C * C + S * S) / ((double)n * (double)nv) : 0.0;
			}
		}
		__syncwarp();
	}
	__syncwarp();
	for (int b = lane; b < count; b += 32)
		if (hist[b]) atomicAdd(&gr_counts[b], (unsigned long long)hist[b]);
}

}  // namespace tdvmc
