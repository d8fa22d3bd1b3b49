// Flux-divergence kernels: FP64 with FMA contraction; stretch coordinates; convective group b.
#define GBNS_REAL double
#define GBNS_STRETCH true
#define GBNS_GROUP 1
#define GBNS_FP32 0
#define GBNS_TAG 7
#define GBNS_FN flux_f64_stretch_b
#include "flux_inst.cuh"
