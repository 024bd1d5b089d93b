#include "dispatch.cuh"
#define TDVMC_T double
#define TDVMC_FN pick_sample_f64
#include "inst_sample.inc"
