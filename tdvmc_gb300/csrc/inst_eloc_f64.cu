#include "dispatch.cuh"
#include "k_eloc.cuh"
#define TDVMC_T double
#define TDVMC_FN pick_eloc_f64
#define TDVMC_REV_FN pick_eloc_rev_f64
#include "inst_eloc.inc"
