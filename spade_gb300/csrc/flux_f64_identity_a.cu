// Flux-divergence kernels: FP64 with FMA contraction; identity coordinates; convective group a.
#define GBNS_REAL double
#define GBNS_STRETCH false
#define GBNS_GROUP 0
#define GBNS_FP32 0
#define GBNS_TAG 4
#define GBNS_FN flux_f64_identity_a
#include "flux_inst.cuh"
