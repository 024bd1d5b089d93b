#include "dispatch.cuh"
#include "k_eloc.cuh"
#define TDVMC_T float
#define TDVMC_FN pick_eloc_f32
#define TDVMC_REV_FN pick_eloc_rev_f32
#include "inst_eloc.inc"
