#include "dispatch.cuh"
#include "k_eloc.cuh"
#define TDVMC_T float
#define TDVMC_FN pick_eloc_f32
#include "inst_eloc.inc"
