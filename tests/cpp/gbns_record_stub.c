/* A stand-in for libgbns.so that records the C-ABI calls the C++ drop-in
 * (include/spade_gb300.h) makes instead of running them: every
 * gbns_flux_div_host call is appended to the file named by GBNS_RECORD as
 *   u64 sizeof(gbns_grid_desc), the descriptor bytes,
 *   u64 sizeof(gbns_scheme_desc), the descriptor bytes,
 *   i32 increment, u64 count, count doubles of prims, count doubles of rhs,
 * with count = gbns_array_size(grid).  Test infrastructure: the recorded
 * calls are replayed through the real library on a GPU
 * (tests/test_gpu_dropin_replay.py). */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gbns.h"

static size_t array_doubles(const gbns_grid_desc* g)
{
    size_t n = (size_t)g->nblk[0]*g->nblk[1]*g->nblk[2];
    n *= (size_t)(g->ncell[0] + 2*g->ng)*(g->ncell[1] + 2*g->ng)*(g->ncell[2] + 2*g->ng);
    return 5*n;
}

int gbns_flux_div_host(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                       const double* host_prims, double* host_rhs, int increment, void* stream)
{
    (void)stream;
    const char* path = getenv("GBNS_RECORD");
    if (!path) return GBNS_ERR_INVALID;
    FILE* f = fopen(path, "ab");
    if (!f) return GBNS_ERR_INVALID;
    const unsigned long long gs = sizeof(*grid), ss = sizeof(*scheme);
    const unsigned long long n = array_doubles(grid);
    const int incr = increment;
    fwrite(&gs, 8, 1, f); fwrite(grid, 1, gs, f);
    fwrite(&ss, 8, 1, f); fwrite(scheme, 1, ss, f);
    fwrite(&incr, 4, 1, f); fwrite(&n, 8, 1, f);
    fwrite(host_prims, 8, n, f); fwrite(host_rhs, 8, n, f);
    fclose(f);
    return GBNS_OK;
}

int gbns_last_error(char* buf, size_t len)
{
    if (buf && len) snprintf(buf, len, "recording stand-in");
    return 0;
}

/* gbns_flux_div_blocks_host calls (refined layouts) go to the file named by
 * GBNS_RECORD_BLOCKS as the record above with, after the increment flag,
 *   u64 nblocks, 6*nblocks doubles of block bounds,
 * then count and the two arrays. */
int gbns_flux_div_blocks_host(const gbns_grid_desc* grid, const gbns_scheme_desc* scheme, const double* block_bounds,
                              const double* host_prims, double* host_rhs, int increment, void* stream)
{
    (void)stream;
    const char* path = getenv("GBNS_RECORD_BLOCKS");
    if (!path) return GBNS_ERR_INVALID;
    FILE* f = fopen(path, "ab");
    if (!f) return GBNS_ERR_INVALID;
    const unsigned long long gs = sizeof(*grid), ss = sizeof(*scheme);
    const unsigned long long nb = (unsigned long long)grid->nblk[0];
    const unsigned long long n = array_doubles(grid);
    const int incr = increment;
    fwrite(&gs, 8, 1, f); fwrite(grid, 1, gs, f);
    fwrite(&ss, 8, 1, f); fwrite(scheme, 1, ss, f);
    fwrite(&incr, 4, 1, f);
    fwrite(&nb, 8, 1, f); fwrite(block_bounds, 8, 6*nb, f);
    fwrite(&n, 8, 1, f);
    fwrite(host_prims, 8, n, f); fwrite(host_rhs, 8, n, f);
    fclose(f);
    return GBNS_OK;
}
