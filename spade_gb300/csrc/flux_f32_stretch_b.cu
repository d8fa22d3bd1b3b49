// Flux-divergence kernels: FP32 flux arithmetic, FP64 accumulation; stretch coordinates; convective group b.
#define GBNS_REAL float
#define GBNS_STRETCH true
#define GBNS_GROUP 1
#define GBNS_FP32 1
#define GBNS_TAG 11
#define GBNS_FN flux_f32_stretch_b
#include "flux_inst.cuh"
