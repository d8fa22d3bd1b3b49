// Batched flux kernels: FP32 flux arithmetic, FP64 accumulation; class group 2.
#define GBNS_REAL float
#define GBNS_TAG 65
#define GBNS_FP32 1
#define GBNS_BATCH_GROUP 2
#define GBNS_BATCH_FN launch_flux_batch_f32_c
#define GBNS_BATCH_BOX_FN launch_flux_batch_f32_c_box
#include "batch_flux.cuh"
