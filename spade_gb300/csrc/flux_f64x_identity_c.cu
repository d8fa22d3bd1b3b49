// Flux-divergence kernels: FP64, no FMA contraction (bit-compatible with the reference's CPU arithmetic; built with -fmad=false); identity coordinates; convective group c (hybrid).
#define GBNS_REAL double
#define GBNS_STRETCH false
#define GBNS_GROUP 2
#define GBNS_FP32 0
#define GBNS_TAG 0
#define GBNS_FN flux_f64x_identity_c
#include "flux_inst.cuh"
