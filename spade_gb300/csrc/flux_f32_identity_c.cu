// Flux-divergence kernels: FP32 flux arithmetic, FP64 accumulation; identity coordinates; convective group c (hybrid).
#define GBNS_REAL float
#define GBNS_STRETCH false
#define GBNS_GROUP 2
#define GBNS_FP32 1
#define GBNS_TAG 8
#define GBNS_FN flux_f32_identity_c
#include "flux_inst.cuh"
