// Flux-divergence kernels: FP64 with FMA contraction; identity coordinates; convective group c (hybrid).
#define GBNS_REAL double
#define GBNS_STRETCH false
#define GBNS_GROUP 2
#define GBNS_FP32 0
#define GBNS_TAG 4
#define GBNS_FN flux_f64_identity_c
#include "flux_inst.cuh"
