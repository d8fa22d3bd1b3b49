// Flux-divergence kernels: FP64 with FMA contraction; stretch coordinates; convective group c (hybrid).
#define GBNS_REAL double
#define GBNS_STRETCH true
#define GBNS_GROUP 2
#define GBNS_FP32 0
#define GBNS_TAG 6
#define GBNS_FN flux_f64_stretch_c
#include "flux_inst.cuh"
