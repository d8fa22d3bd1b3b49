// Flux-divergence kernels: FP32 flux arithmetic, FP64 accumulation; stretch coordinates; convective group c (hybrid).
#define GBNS_REAL float
#define GBNS_STRETCH true
#define GBNS_GROUP 2
#define GBNS_FP32 1
#define GBNS_TAG 10
#define GBNS_FN flux_f32_stretch_c
#include "flux_inst.cuh"
