// S = Oc^T Oc / N_w on the 5th-generation tensor cores, split-precision
// 3xTF32 with FP32 accumulation in tensor memory (TMEM).
//
// Oc[w][k] = O[w][k] - <O_k> is formed in FP64 from the FP32 per-walker O_k
// and the FP64 walker means (the "FP64 centring"), rounded to FP32 and split
// as Oc = hi + lo with hi, lo TF32.  Then S ~= hi.hi + hi.lo + lo.hi
// (the lo.lo term is below FP32 resolution).
//
// Mapping: one CTA (128 threads) per SM walks over tiles of 32 walkers.  A
// tile is staged in shared memory parameter-major / walker-contiguous, which
// is the K-major canonical layout (no swizzle) for both MMA operands:
// A = tile rows 0..127 (M = 128, parameters padded with zeros) and
// B = tile rows 0..N-1 (N = p rounded up to 16).  One elected thread issues
// 4 x 3 tcgen05.mma (K = 8 each) per tile and commits them to an mbarrier;
// the next tile is staged into the other buffer meanwhile.  At the end the
// accumulator D (row k = TMEM lane k, column l) is read back with
// tcgen05.ld and written as the CTA's FP32 partial; a second kernel adds the
// partials in FP64 in fixed order and symmetrises.
//
// Every mbarrier wait is bounded in time (mbar_wait_ns): a commit not seen
// within the status limit marks the CTA failed and is then waited for with the
// drain limit, so no MMA still reads a buffer that is restaged or writes the
// accumulator that is read and freed; a failed CTA writes NaN partials (the
// solve then reports TDVMC_ERR_NONFINITE) instead of hanging.
#include "common.cuh"
#include "k_gram_tf32.cuh"

namespace tdvmc {

namespace {

constexpr int kTileK = 32;                    // walkers per tile (MMA K total per tile)
constexpr int kM = 128;                       // MMA M: parameter rows (padded)
constexpr int kLBO = 128;                     // bytes between core matrices along K
constexpr int kSBO = (kTileK / 4) * 128;      // bytes between 8-row groups
constexpr int kTileBytes = (kM / 8) * kSBO;   // 16 KB per operand tile
constexpr int kThreads = 128;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
	return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor: start, LBO, SBO (all >> 4),
// descriptor version 1 (bits 46-47), no swizzle, base offset 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
	uint64_t d = 0;
	d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
	d |= (uint64_t)((kLBO >> 4) & 0x3FFFu) << 16;
	d |= (uint64_t)((kSBO >> 4) & 0x3FFFu) << 32;
	d |= (uint64_t)1u << 46;
	return d;
}

// instruction descriptor, kind::tf32: D f32, A/B tf32, both K-major
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
	return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
	uint32_t r;
	asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
	return r;
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
	asm volatile(
	    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
	    "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t* mbar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
	             : "memory");
}

// the commit of phase `parity`: status limit, then the drain limit on time-out;
// false when the status limit ran out
__device__ __forceinline__ bool wait_parity(uint64_t* mbar, uint32_t parity, uint64_t status_ns) {
	const uint32_t a = smem_u32(mbar);
	if (mbar_wait_ns(a, parity, status_ns)) return true;
	mbar_wait_ns(a, parity, kWaitDrainNs);
	return false;
}

// byte offset of element (row m, walker kk) in a K-major no-swizzle tile
__device__ __forceinline__ uint32_t tile_off(int m, int kk) {
	return (uint32_t)((m >> 3) * kSBO + (kk >> 2) * kLBO + (m & 7) * 16 + (kk & 3) * 4);
}

__global__ void __launch_bounds__(kThreads, 1) k_gram_tf32(int p, int npad, int64_t nw, const float* __restrict__ O,
                                                           const double* __restrict__ means, float* __restrict__ partial,
                                                           uint64_t wait_ns) {
	extern __shared__ __align__(1024) unsigned char smem_raw[];
	// 1024-byte aligned operand buffers: [buf][hi, lo]
	unsigned char* base = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
	__shared__ __align__(8) uint64_t mbar[2];
	__shared__ uint32_t tmem_slot;
	__shared__ int failed;

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const uint32_t ncols = npad <= 32 ? 32u : (npad <= 64 ? 64u : 128u);
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
		             "r"(ncols));
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
	}
	if (tid == 0) {
		asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[0])));
		asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[1])));
		asm volatile("fence.mbarrier_init.release.cluster;");
		failed = 0;
	}
	asm volatile("tcgen05.fence::before_thread_sync;");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;");
	const uint32_t tmem = tmem_slot;
	const uint32_t idesc = instr_desc(kM, npad);
	const double mean = tid < p ? means[tid] : 0.0;

	const int64_t ntiles = (nw + kTileK - 1) / kTileK;
	int it = 0;
	for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, it++) {
		const int b = it & 1;
		if (it >= 2 && !wait_parity(&mbar[b], (uint32_t)(((it - 2) >> 1) & 1), wait_ns)) failed = 1;
		unsigned char* hi = base + b * 2 * kTileBytes;
		unsigned char* lo = hi + kTileBytes;
		// stage: thread tid owns parameter row m = tid, 32 walkers of the tile
		const int m = tid;
		const int64_t w0 = tile * kTileK;
#pragma unroll
		for (int g = 0; g < kTileK / 4; g++) {
			uint32_t h[4], l[4];
#pragma unroll
			for (int q = 0; q < 4; q++) {
				const int64_t w = w0 + g * 4 + q;
				float x = 0.f;
				if (m < p && w < nw) x = (float)((double)O[(size_t)w * p + m] - mean);
				h[q] = to_tf32(x);
				l[q] = to_tf32(x - __uint_as_float(h[q]));
			}
			const uint32_t off = tile_off(m, g * 4);
			*reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
			*reinterpret_cast<uint4*>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
		}
		asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
		__syncthreads();
		if (tid == 0) {
			asm volatile("tcgen05.fence::after_thread_sync;");
			const uint32_t ah = smem_u32(hi), al = smem_u32(lo);
#pragma unroll
			for (int kc = 0; kc < kTileK / 8; kc++) {
				const uint32_t o = kc * 2 * kLBO;
				const uint64_t dh = smem_desc(ah + o), dl = smem_desc(al + o);
				mma_tf32(tmem, dh, dh, idesc, (it > 0 || kc > 0) ? 1u : 0u);
				mma_tf32(tmem, dh, dl, idesc, 1u);
				mma_tf32(tmem, dl, dh, idesc, 1u);
			}
			commit(&mbar[b]);
		}
	}
	// drain: the last commit of each buffer
	if (it >= 1 && !wait_parity(&mbar[(it - 1) & 1], (uint32_t)(((it - 1) >> 1) & 1), wait_ns)) failed = 1;
	if (it >= 2 && !wait_parity(&mbar[(it - 2) & 1], (uint32_t)(((it - 2) >> 1) & 1), wait_ns)) failed = 1;
	asm volatile("tcgen05.fence::after_thread_sync;");
	__syncthreads();

	// read D: warp w owns TMEM lanes 32w..32w+31 (= parameter rows)
	const int row = warp * 32 + lane;
	for (int c0 = 0; c0 < npad; c0 += 32) {
		uint32_t v[32];
		const uint32_t addr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
		asm volatile(
		    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
		    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
		    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
		      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
		      "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
		      "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
		      "=r"(v[30]), "=r"(v[31])
		    : "r"(addr));
		asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
		if (row < p) {
			float* dst = partial + ((size_t)blockIdx.x * p + row) * p;
#pragma unroll
			for (int j = 0; j < 32; j++)
				if (c0 + j < p) dst[c0 + j] = failed ? __int_as_float(0x7fc00000) : __uint_as_float(v[j]);
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;");
	__syncthreads();
	if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// S[k][l] = (sum_b partial[b][k][l] + partial[b][l][k]) / (2 nw), FP64, fixed
// order: one warp per entry, lane l adding blocks l, l + 32, ..., then a fixed
// butterfly.
constexpr int kGramFinThreads = 256;
__global__ void __launch_bounds__(kGramFinThreads) k_gram_finalize(int p, int nblk, const float* __restrict__ partial,
                                                                   double inv_nw, double* __restrict__ S) {
	const int lane = threadIdx.x & 31;
	const int e = blockIdx.x * (kGramFinThreads / 32) + (threadIdx.x >> 5);
	if (e >= p * p) return;  // whole warps
	const int k = e / p, l = e % p;
	double s = 0.0;
	for (int b = lane; b < nblk; b += 32)
		s += (double)partial[((size_t)b * p + k) * p + l] + (double)partial[((size_t)b * p + l) * p + k];
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
	if (lane == 0) S[e] = 0.5 * s * inv_nw;
}

}  // namespace

bool gram_supported(int p) { return p >= 1 && p <= 128; }

int gram_blocks(int64_t nw, int nsm) {
	const int64_t tiles = (nw + kTileK - 1) / kTileK;
	return (int)(tiles < nsm ? tiles : nsm);
}

size_t gram_smem_bytes() { return (size_t)4 * kTileBytes + 1024; }

int launch_gram_tf32(cudaStream_t st, int p, int64_t nw, const float* O, const double* means, int nblk, float* partial,
                     double* S, int, uint64_t wait_ns) {
	if (!gram_supported(p) || nblk < 1) return 1;
	const int npad = (p + 15) / 16 * 16;
	const size_t smem = gram_smem_bytes();
	if (cudaFuncSetAttribute(k_gram_tf32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 1;
	k_gram_tf32<<<nblk, kThreads, smem, st>>>(p, npad, nw, O, means, partial, wait_ns);
	k_gram_finalize<<<(p * p + kGramFinThreads / 32 - 1) / (kGramFinThreads / 32), kGramFinThreads, 0, st>>>(
	    p, nblk, partial, 1.0 / (double)nw, S);
	return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace tdvmc
