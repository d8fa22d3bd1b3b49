// Batched flux kernels: FP64, no FMA contraction (built with -fmad=false); class group 2.
#define GBNS_REAL double
#define GBNS_TAG 64
#define GBNS_FP32 0
#define GBNS_BATCH_GROUP 2
#define GBNS_BATCH_FN launch_flux_batch_f64x_c
#define GBNS_BATCH_BOX_FN launch_flux_batch_f64x_c_box
#include "batch_flux.cuh"
