// S = Oc^T Oc / N_w on the tensor cores (3xTF32 with FP32 accumulation in
// tensor memory).  Oc = O - <O> is formed from the FP32 per-walker O_k and the
// FP64 walker means before the split into TF32 high and low parts.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tdvmc {

// true when the tensor-core path handles p parameters
bool gram_supported(int p);
// number of CTAs (walker chunks) the contraction uses for nw walkers
int gram_blocks(int64_t nw, int nsm);
// partial[nblk][p*p] (FP32) then S[p*p] = sum / nw (FP64); returns 0 on success.
// wait_ns: status limit of the waits for the tensor-core commits (kWaitStatusNs)
int launch_gram_tf32(cudaStream_t st, int p, int64_t nw, const float* O, const double* means, int nblk, float* partial,
                     double* S, int nsm, uint64_t wait_ns);

}  // namespace tdvmc
