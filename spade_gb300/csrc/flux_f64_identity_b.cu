// Flux-divergence kernels: FP64 with FMA contraction; identity coordinates; convective group b.
#define GBNS_REAL double
#define GBNS_STRETCH false
#define GBNS_GROUP 1
#define GBNS_FP32 0
#define GBNS_TAG 5
#define GBNS_FN flux_f64_identity_b
#include "flux_inst.cuh"
