// Batched form: many independent grids advanced together.
//
// Every active grid ("instance") has a descriptor InstK in device memory.
// Work is described by device work-lists that the host rebuilds when the set
// of instances changes:
//   * tile items (instance, block, tile), grouped by kernel class (the
//     compile-time flux configuration: convective scheme, coordinates);
//   * block items (instance, block) for the RK stage and the ghost fill.
// Persistent kernels (one CTA per SM slot) walk the lists; counts and
// offsets are read from device memory, so a captured CUDA graph of one step
// stays valid while instances come and go.
#pragma once

#include "gbns_internal.cuh"

namespace gbns
{
    struct BcK
    {
        int kind[6];
        double t_wall[6];
    };

    struct InstK
    {
        GeomK G;
        SchemeK S;
        BcK bc;
        double* q;          // primitive state, AoS5 with ghosts
        double* R[3];       // R0, R1 and the second state buffer of the fused stages
        double dt;
        int ytab;           // index into the Y-metric table array, -1 for identity
        int pad;
    };

    struct TileItem { int inst, lb, tile, pad; };
    struct BlockItem { int inst, lb; };

    // Kernel classes of the batched flux launch.
    enum batch_class
    {
        BCLASS_CK2_ID = 0,     // cent_keep<2>, identity coordinates (Taylor-Green)
        BCLASS_TOTANI_ID,      // totani_lr, identity
        BCLASS_FWENO_ID,       // fweno_t, identity
        BCLASS_WENO5_ST,       // WENO5, stretched y (channel)
        BCLASS_WENO5_ID,       // WENO5, identity
        BCLASS_HYB2_ID,        // hybrid_scheme_t(cent_keep<2>, fweno_t), identity
        BCLASS_COUNT
    };

    // Returns the class of a (grid, scheme) pair or -1 if it has no batched kernel.
    int batch_class_of(const gbns_grid_desc* g, const gbns_scheme_desc* s);

    // Tile variants of a class: how many, and the tile shape of one (for
    // counting tiles per block on the host).
    int batch_class_variants(int cls, int precision);
    void batch_class_tile(int cls, int precision, int variant, int tile[3]);

    // Flux launch of one class (tile variant v) for one SSPRK3 stage: one
    // CTA per item.  `offsets` and `counts` (device, BCLASS_COUNT ints) locate
    // the class's items; `nitems` is the host's copy of its count (the grid).
    // One function per precision and class group (a: cent_keep<2>,
    // totani_lr, fweno_t; b: WENO5; c: hybrid).  `left` (device, one per
    // slot): steps an instance still has to do before it idles (-1: no
    // limit); items of instances at 0 are skipped.
    // `tmaps` (device, two per slot: q and R[2]; may be NULL): tensor maps
    // the FP64 tiles stage their box from, for the items whose `pad` is set.
    // The *_box functions give a variant's TMA box (cells along x, y, z; zeros
    // when the variant stages no FP64 box by TMA), which the maps must use.
#define GBNS_BATCH_DECL(NAME) \
    int NAME(int cls, int v, const TileItem* items, const int* offsets, const int* counts, \
             const InstK* insts, const YTabK* ytabs, const long long* left, const CUtensorMap* tmaps, \
             int stage, int nitems, cudaStream_t st); \
    int NAME##_box(int cls, int v, int box[3]);
    GBNS_BATCH_DECL(launch_flux_batch_f64x_a)
    GBNS_BATCH_DECL(launch_flux_batch_f64x_b)
    GBNS_BATCH_DECL(launch_flux_batch_f64x_c)
    GBNS_BATCH_DECL(launch_flux_batch_f32_a)
    GBNS_BATCH_DECL(launch_flux_batch_f32_b)
    GBNS_BATCH_DECL(launch_flux_batch_f32_c)
#undef GBNS_BATCH_DECL

    // Batched ghost fill (mode 0: q, 1: R[2], 2: copy R[2] into q and fill
    // q's ghosts); the RK stage update runs in the flux launch's epilogue.
    int launch_ghost_batch(const BlockItem* items, const int* count, const InstK* insts, const long long* left,
                           int mode, cudaStream_t st);
    // per-slot step counters: one step done by every limited instance; set one
    int launch_steps_tick(long long* left, int n, cudaStream_t st);
    int launch_steps_set(long long* left, int slot, long long value, cudaStream_t st);

    int persistent_grid(int ctas_per_sm);
}
