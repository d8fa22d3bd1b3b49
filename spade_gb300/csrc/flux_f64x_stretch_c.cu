// Flux-divergence kernels: FP64, no FMA contraction (bit-compatible with the reference's CPU arithmetic; built with -fmad=false); stretch coordinates; convective group c (hybrid).
#define GBNS_REAL double
#define GBNS_STRETCH true
#define GBNS_GROUP 2
#define GBNS_FP32 0
#define GBNS_TAG 2
#define GBNS_FN flux_f64x_stretch_c
#include "flux_inst.cuh"
