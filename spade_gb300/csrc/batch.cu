// Host side of the batched form: instance table, HBM-budget arena, work-list
// construction, CUDA-graph capture of one SSPRK3 step, and the C ABI.
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "gbns_internal.cuh"
#include "batch_internal.cuh"

namespace gbns
{
    int batch_class_of(const gbns_grid_desc* g, const gbns_scheme_desc* s)
    {
        const bool id = g->coords == GBNS_COORDS_IDENTITY;
        if (s->convective == GBNS_CONV_CENT_KEEP && s->order == 2 && id) return BCLASS_CK2_ID;
        if (s->convective == GBNS_CONV_TOTANI && id) return BCLASS_TOTANI_ID;
        if (s->convective == GBNS_CONV_FWENO && id) return BCLASS_FWENO_ID;
        if (s->convective == GBNS_CONV_WENO5) return id ? BCLASS_WENO5_ID : BCLASS_WENO5_ST;
        if (s->convective == GBNS_CONV_HYBRID && s->order == 2 && id) return BCLASS_HYB2_ID;
        return -1;
    }

    // Tile shapes of the variants in batch_flux.cuh (same order).
    int batch_class_variants(int cls, int precision)
    {
        if (cls == BCLASS_HYB2_ID && precision == GBNS_PREC_FP32_FLUX) return 2;
        return 3;
    }

    void batch_class_tile(int cls, int precision, int variant, int tile[3])
    {
        const bool fp32 = precision == GBNS_PREC_FP32_FLUX;
        const bool weno5 = cls == BCLASS_WENO5_ST || cls == BCLASS_WENO5_ID;
        // 8x8x4 tiles: variant 1 of the centred and fweno classes and of FP64
        // WENO5, variant 0 of FP32 WENO5 and of the hybrid
        bool thin;
        if (cls == BCLASS_HYB2_ID) thin = variant == 0;
        else if (weno5 && fp32) thin = variant == 0;
        else thin = variant == 1;
        tile[0] = 8; tile[1] = 8; tile[2] = thin ? 4 : 8;
    }

    int launch_flux_batch(int cls, int v, int precision, const TileItem* items, const int* offsets, const int* counts,
                          const InstK* insts, const YTabK* ytabs, const long long* left, const CUtensorMap* tmaps,
                          int stage, int nitems, cudaStream_t st)
    {
        const int group = cls == BCLASS_HYB2_ID ? 2 : ((cls == BCLASS_WENO5_ST || cls == BCLASS_WENO5_ID) ? 1 : 0);
        if (precision == GBNS_PREC_FP32_FLUX)
        {
            if (group == 0) return launch_flux_batch_f32_a(cls, v, items, offsets, counts, insts, ytabs, left, nullptr, stage, nitems, st);
            if (group == 1) return launch_flux_batch_f32_b(cls, v, items, offsets, counts, insts, ytabs, left, nullptr, stage, nitems, st);
            return launch_flux_batch_f32_c(cls, v, items, offsets, counts, insts, ytabs, left, nullptr, stage, nitems, st);
        }
        if (group == 0) return launch_flux_batch_f64x_a(cls, v, items, offsets, counts, insts, ytabs, left, tmaps, stage, nitems, st);
        if (group == 1) return launch_flux_batch_f64x_b(cls, v, items, offsets, counts, insts, ytabs, left, tmaps, stage, nitems, st);
        return launch_flux_batch_f64x_c(cls, v, items, offsets, counts, insts, ytabs, left, tmaps, stage, nitems, st);
    }

    // The FP64 TMA box of a class's variant (zeros: no TMA staging).
    int batch_box(int cls, int v, int precision, int box[3])
    {
        box[0] = box[1] = box[2] = 0;
        if (precision == GBNS_PREC_FP32_FLUX) return GBNS_OK;
        const int group = cls == BCLASS_HYB2_ID ? 2 : ((cls == BCLASS_WENO5_ST || cls == BCLASS_WENO5_ID) ? 1 : 0);
        if (group == 0) return launch_flux_batch_f64x_a_box(cls, v, box);
        if (group == 1) return launch_flux_batch_f64x_b_box(cls, v, box);
        return launch_flux_batch_f64x_c_box(cls, v, box);
    }

    // First-fit allocator over one device allocation (offsets in bytes).
    class Arena
    {
        std::map<size_t, size_t> free_;   // offset -> size
    public:
        size_t size = 0, used = 0;
        void init(size_t n) { free_.clear(); free_[0] = n; size = n; used = 0; }
        bool alloc(size_t n, size_t* off)
        {
            n = (n + 255) & ~size_t(255);
            for (auto it = free_.begin(); it != free_.end(); ++it)
            {
                if (it->second < n) continue;
                *off = it->first;
                const size_t rest = it->second - n;
                const size_t roff = it->first + n;
                free_.erase(it);
                if (rest) free_[roff] = rest;
                used += n;
                return true;
            }
            return false;
        }
        void release(size_t off, size_t n)
        {
            n = (n + 255) & ~size_t(255);
            used -= n;
            auto it = free_.emplace(off, n).first;
            auto nx = std::next(it);
            if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
            if (it != free_.begin())
            {
                auto pv = std::prev(it);
                if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
            }
        }
    };

    struct Slot
    {
        bool active = false;
        gbns_grid_desc g;
        gbns_scheme_desc s;
        gbns_bc_desc bc;
        double dt = 0.0;
        size_t off = 0;          // arena offset of q, R0, R1, R2 (contiguous)
        size_t arr_bytes = 0;
        int cls = -1;
        long long steps = 0;
        long long cells = 0;
        long long left = -1;     // steps still to do before it idles (-1: no limit); mirrors d_left
    };
}

using namespace gbns;

struct gbns_batch
{
    int device = 0;
    int precision = GBNS_PREC_FP64;
    int use_graph = 1;
    cudaStream_t stream = nullptr;      // the batch's own stream (capturable)
    cudaStream_t caller = nullptr;      // the caller's stream; ordered with events
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    char* arena_base = nullptr;
    Arena arena;
    std::vector<Slot> slots;
    InstK* d_insts = nullptr;
    long long* d_left = nullptr;        // per-slot step counters (device)
    int inst_cap = 0;
    YTabK* d_ytabs = nullptr;
    TileItem* d_tiles = nullptr;
    size_t tile_cap = 0;
    BlockItem* d_blocks = nullptr;
    size_t block_cap = 0;
    int* d_meta = nullptr;     // offsets[BCLASS_COUNT], counts[BCLASS_COUNT], nblocks
    // FP64: per slot the tensor maps of q and R[2] for the TMA staging of its
    // class's current tile variant (rebuilt with the lists)
    CUtensorMap* d_tmaps = nullptr;
    size_t tmap_cap = 0;
    std::vector<CUtensorMap> h_tmaps;
    std::vector<TileItem> h_tiles;
    std::vector<BlockItem> h_blocks;
    int h_meta[2*BCLASS_COUNT + 1];
    int variant[BCLASS_COUNT] = {0, 0, 0, 0, 0, 0};   // tile variant per class (gbns_batch_autotune)
    unsigned class_mask = 0;
    bool dirty = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    unsigned graph_mask = 0;
    int graph_counts[BCLASS_COUNT] = {0, 0, 0, 0, 0, 0};   // items per class the graph's launch grids cover
    bool graph_valid = false;
};

namespace
{
    // Work of a call runs on the batch stream after everything already queued
    // on the caller's stream, and the caller's stream waits for it.
    int enter(gbns_batch* b)
    {
        int rc = check_cuda(cudaEventRecord(b->ev_in, b->caller), "batch order (record)");
        if (!rc) rc = check_cuda(cudaStreamWaitEvent(b->stream, b->ev_in, 0), "batch order (wait)");
        return rc;
    }

    int leave(gbns_batch* b, int rc)
    {
        int r2 = check_cuda(cudaEventRecord(b->ev_out, b->stream), "batch order (record)");
        if (!r2) r2 = check_cuda(cudaStreamWaitEvent(b->caller, b->ev_out, 0), "batch order (wait)");
        return rc ? rc : r2;
    }

    int grow_insts(gbns_batch* b, int need)
    {
        if (need <= b->inst_cap) return GBNS_OK;
        int cap = b->inst_cap ? b->inst_cap : 16;
        while (cap < need) cap *= 2;
        InstK* ni = nullptr;
        YTabK* ny = nullptr;
        long long* nl = nullptr;
        int rc = check_cuda(cudaMalloc(&ni, sizeof(InstK)*cap), "batch instance table");
        if (rc) return rc;
        rc = check_cuda(cudaMalloc(&ny, sizeof(YTabK)*cap), "batch metric tables");
        if (rc) { cudaFree(ni); return rc; }
        rc = check_cuda(cudaMalloc(&nl, sizeof(long long)*cap), "batch step counters");
        if (rc) { cudaFree(ni); cudaFree(ny); return rc; }
        // new slots start idle (0) until an instance takes them
        rc = check_cuda(cudaMemsetAsync(nl, 0, sizeof(long long)*cap, b->stream), "batch step counters");
        if (rc) { cudaFree(ni); cudaFree(ny); cudaFree(nl); return rc; }
        if (b->d_insts)
        {
            cudaMemcpyAsync(ni, b->d_insts, sizeof(InstK)*b->inst_cap, cudaMemcpyDeviceToDevice, b->stream);
            cudaMemcpyAsync(ny, b->d_ytabs, sizeof(YTabK)*b->inst_cap, cudaMemcpyDeviceToDevice, b->stream);
            cudaMemcpyAsync(nl, b->d_left, sizeof(long long)*b->inst_cap, cudaMemcpyDeviceToDevice, b->stream);
            cudaStreamSynchronize(b->stream);
            cudaFree(b->d_insts);
            cudaFree(b->d_ytabs);
            cudaFree(b->d_left);
        }
        b->d_insts = ni;
        b->d_ytabs = ny;
        b->d_left = nl;
        b->inst_cap = cap;
        b->graph_valid = false;
        return GBNS_OK;
    }

    template <class T>
    int grow_list(T** dptr, size_t* cap, size_t need, gbns_batch* b, const char* what)
    {
        if (need <= *cap && *dptr) return GBNS_OK;
        size_t c = *cap ? *cap : 1024;
        while (c < need) c *= 2;
        T* p = nullptr;
        int rc = check_cuda(cudaMalloc(&p, sizeof(T)*c), what);
        if (rc) return rc;
        if (*dptr)
        {
            cudaStreamSynchronize(b->stream);
            cudaFree(*dptr);
        }
        *dptr = p;
        *cap = c;
        b->graph_valid = false;
        return GBNS_OK;
    }

    // Encodes slot si's tensor maps (q and R[2]) for the TMA box of its
    // class's current variant; false when that variant stages no FP64 box by
    // TMA or the layout does not allow it (padded rows must hold an even
    // number of cells for the 16-byte rule; the arena keeps the arrays
    // 256-byte aligned).
    bool slot_tma(gbns_batch* b, size_t si)
    {
        const Slot& S = b->slots[si];
        if (b->h_tmaps.size() < 2*(si + 1)) b->h_tmaps.resize(2*(si + 1));
        int box[3];
        if (batch_box(S.cls, b->variant[S.cls], b->precision, box) || box[0] == 0) return false;
        GeomK G;
        if (make_geom(&S.g, G) || G.ni % 2 != 0) return false;
        double* q = reinterpret_cast<double*>(b->arena_base + S.off);
        double* r2 = reinterpret_cast<double*>(b->arena_base + S.off + 3*S.arr_bytes);
        if (encode_prims_tmap(&b->h_tmaps[2*si], q, G, box[0], box[1], box[2])) return false;
        if (encode_prims_tmap(&b->h_tmaps[2*si + 1], r2, G, box[0], box[1], box[2])) return false;
        return true;
    }

    int rebuild_lists(gbns_batch* b)
    {
        b->h_tiles.clear();
        b->h_blocks.clear();
        b->class_mask = 0;
        b->h_tmaps.assign(2*b->slots.size(), CUtensorMap{});
        for (int c = 0; c < BCLASS_COUNT; ++c)
        {
            b->h_meta[c] = int(b->h_tiles.size());
            int t[3];
            batch_class_tile(c, b->precision, b->variant[c], t);
            for (size_t si = 0; si < b->slots.size(); ++si)
            {
                const Slot& S = b->slots[si];
                if (!S.active || S.cls != c) continue;
                const int nt = ((S.g.ncell[0] + t[0] - 1)/t[0])*((S.g.ncell[1] + t[1] - 1)/t[1])*((S.g.ncell[2] + t[2] - 1)/t[2]);
                const int nblk = S.g.nblk[0]*S.g.nblk[1]*S.g.nblk[2];
                const int tma = slot_tma(b, si) ? 1 : 0;
                for (int lb = 0; lb < nblk; ++lb)
                    for (int tile = 0; tile < nt; ++tile)
                        b->h_tiles.push_back(TileItem{int(si), lb, tile, tma});
            }
            b->h_meta[BCLASS_COUNT + c] = int(b->h_tiles.size()) - b->h_meta[c];
            if (b->h_meta[BCLASS_COUNT + c]) b->class_mask |= 1u << c;
        }
        for (size_t si = 0; si < b->slots.size(); ++si)
        {
            const Slot& S = b->slots[si];
            if (!S.active) continue;
            const int nblk = S.g.nblk[0]*S.g.nblk[1]*S.g.nblk[2];
            for (int lb = 0; lb < nblk; ++lb) b->h_blocks.push_back(BlockItem{int(si), lb});
        }
        b->h_meta[2*BCLASS_COUNT] = int(b->h_blocks.size());
        int rc = grow_list(&b->d_tiles, &b->tile_cap, b->h_tiles.size(), b, "batch tile list");
        if (rc) return rc;
        rc = grow_list(&b->d_blocks, &b->block_cap, b->h_blocks.size(), b, "batch block list");
        if (rc) return rc;
        if (!b->h_tiles.empty())
            rc = check_cuda(cudaMemcpyAsync(b->d_tiles, b->h_tiles.data(), sizeof(TileItem)*b->h_tiles.size(),
                                            cudaMemcpyHostToDevice, b->stream), "upload tile list");
        if (rc) return rc;
        if (!b->h_blocks.empty())
            rc = check_cuda(cudaMemcpyAsync(b->d_blocks, b->h_blocks.data(), sizeof(BlockItem)*b->h_blocks.size(),
                                            cudaMemcpyHostToDevice, b->stream), "upload block list");
        if (rc) return rc;
        if (b->precision != GBNS_PREC_FP32_FLUX && !b->h_tmaps.empty())
        {
            rc = grow_list(&b->d_tmaps, &b->tmap_cap, b->h_tmaps.size(), b, "batch tensor maps");
            if (rc) return rc;
            rc = check_cuda(cudaMemcpyAsync(b->d_tmaps, b->h_tmaps.data(), sizeof(CUtensorMap)*b->h_tmaps.size(),
                                            cudaMemcpyHostToDevice, b->stream), "upload tensor maps");
            if (rc) return rc;
        }
        rc = check_cuda(cudaMemcpyAsync(b->d_meta, b->h_meta, sizeof(b->h_meta), cudaMemcpyHostToDevice, b->stream),
                        "upload list counts");
        if (rc) return rc;
        // pageable sources: keep them alive until the copies have been consumed
        rc = check_cuda(cudaStreamSynchronize(b->stream), "batch list upload");
        b->dirty = false;
        return rc;
    }

    int launch_step(gbns_batch* b)
    {
        const int* offs = b->d_meta;
        const int* cnts = b->d_meta + BCLASS_COUNT;
        const int* nblk = b->d_meta + 2*BCLASS_COUNT;
        for (int stage = 0; stage < 3; ++stage)
        {
            for (int c = 0; c < BCLASS_COUNT; ++c)
            {
                if (!(b->class_mask & (1u << c))) continue;
                int rc = launch_flux_batch(c, b->variant[c], b->precision, b->d_tiles, offs, cnts, b->d_insts,
                                           b->d_ytabs, b->d_left, b->d_tmaps, stage, b->h_meta[BCLASS_COUNT + c],
                                           b->stream);
                if (rc) return rc;
            }
            // the stage update ran in the flux launch's epilogue; fill the
            // ghosts of the state it wrote (stage 2: copy it back into q)
            int rc = launch_ghost_batch(b->d_blocks, nblk, b->d_insts, b->d_left, stage == 0 ? 1 : (stage == 1 ? 0 : 2),
                                        b->stream);
            if (rc) return rc;
        }
        // one step done by every instance that still had steps to do
        return launch_steps_tick(b->d_left, b->inst_cap, b->stream);
    }

    int capture(gbns_batch* b)
    {
        if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
        if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
        int rc = check_cuda(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        if (rc) return rc;
        const int lrc = launch_step(b);
        cudaGraph_t g = nullptr;
        rc = check_cuda(cudaStreamEndCapture(b->stream, &g), "end capture");
        if (lrc) { if (g) cudaGraphDestroy(g); return lrc; }
        if (rc) return rc;
        rc = check_cuda(cudaGraphInstantiate(&b->gexec, g, 0), "graph instantiate");
        if (rc) { cudaGraphDestroy(g); return rc; }
        b->graph = g;
        b->graph_mask = b->class_mask;
        for (int c = 0; c < BCLASS_COUNT; ++c) b->graph_counts[c] = b->h_meta[BCLASS_COUNT + c];
        b->graph_valid = true;
        return GBNS_OK;
    }

    // The flux launches' grids are the classes' item counts: a graph captured
    // for other counts is captured again.
    bool graph_current(const gbns_batch* b)
    {
        if (!b->graph_valid || b->graph_mask != b->class_mask) return false;
        for (int c = 0; c < BCLASS_COUNT; ++c)
            if (b->graph_counts[c] != b->h_meta[BCLASS_COUNT + c]) return false;
        return true;
    }
}

extern "C"
{
    int gbns_batch_create(gbns_batch** out, size_t hbm_budget_bytes, int precision, int use_graph, void* stream)
    {
        if (!out) return set_error(GBNS_ERR_INVALID, "out is NULL");
        if (precision != GBNS_PREC_FP64 && precision != GBNS_PREC_FP32_FLUX)
            return set_error(GBNS_ERR_UNSUPPORTED, "batched form runs GBNS_PREC_FP64 or GBNS_PREC_FP32_FLUX");
        if (hbm_budget_bytes < (size_t(1) << 20)) return set_error(GBNS_ERR_INVALID, "HBM budget below 1 MiB");
        gbns_batch* b = new gbns_batch();
        b->precision = precision;
        b->use_graph = use_graph ? 1 : 0;
        b->caller = static_cast<cudaStream_t>(stream);
        int rc = check_cuda(cudaGetDevice(&b->device), "cudaGetDevice");
        if (!rc) rc = check_cuda(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "batch stream");
        if (!rc) rc = check_cuda(cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming), "batch event");
        if (!rc) rc = check_cuda(cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming), "batch event");
        if (!rc) rc = check_cuda(cudaMalloc(&b->arena_base, hbm_budget_bytes), "batch arena (HBM budget)");
        if (!rc) rc = check_cuda(cudaMalloc(&b->d_meta, sizeof(b->h_meta)), "batch list counts");
        if (rc)
        {
            if (b->arena_base) cudaFree(b->arena_base);
            if (b->stream) cudaStreamDestroy(b->stream);
            if (b->ev_in) cudaEventDestroy(b->ev_in);
            if (b->ev_out) cudaEventDestroy(b->ev_out);
            delete b;
            return rc;
        }
        b->arena.init(hbm_budget_bytes);
        std::memset(b->h_meta, 0, sizeof(b->h_meta));
        // FP64 starts every class on its 8x8x8 / 576-thread tile (variant 2:
        // products and quotients on the integer pipes), the fastest on the
        // measured mixes; gbns_batch_autotune re-times them on the instances
        if (precision == GBNS_PREC_FP64)
            for (int c = 0; c < BCLASS_COUNT; ++c) b->variant[c] = 2;
        *out = b;
        return GBNS_OK;
    }

    int gbns_batch_destroy(gbns_batch* b)
    {
        if (!b) return GBNS_OK;
        cudaStreamSynchronize(b->stream);
        if (b->gexec) cudaGraphExecDestroy(b->gexec);
        if (b->graph) cudaGraphDestroy(b->graph);
        cudaFree(b->arena_base);
        cudaFree(b->d_insts);
        cudaFree(b->d_ytabs);
        cudaFree(b->d_left);
        cudaFree(b->d_tiles);
        cudaFree(b->d_blocks);
        cudaFree(b->d_tmaps);
        cudaFree(b->d_meta);
        cudaEventDestroy(b->ev_in);
        cudaEventDestroy(b->ev_out);
        cudaStreamDestroy(b->stream);
        delete b;
        return GBNS_OK;
    }

    static int batch_add_impl(gbns_batch* b, const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                              const gbns_bc_desc* bc, double dt, const double* prims, int* slot_out);

    int gbns_batch_add(gbns_batch* b, const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                       const gbns_bc_desc* bc, double dt, const double* prims, int* slot_out)
    {
        if (!b || !grid || !scheme || !bc || !prims || !slot_out) return set_error(GBNS_ERR_INVALID, "NULL argument");
        int rc = enter(b);
        if (rc) return rc;
        return leave(b, batch_add_impl(b, grid, scheme, bc, dt, prims, slot_out));
    }

    static int batch_add_impl(gbns_batch* b, const gbns_grid_desc* grid, const gbns_scheme_desc* scheme,
                              const gbns_bc_desc* bc, double dt, const double* prims, int* slot_out)
    {
        GeomK G;
        SchemeK S;
        int rc = make_geom(grid, G);
        if (rc) return rc;
        rc = make_scheme(scheme, S);
        if (rc) return rc;
        if (scheme->precision != b->precision) return set_error(GBNS_ERR_INVALID, "scheme precision differs from the batch's");
        const int cls = batch_class_of(grid, scheme);
        if (cls < 0) return set_error(GBNS_ERR_UNSUPPORTED, "no batched kernel for this scheme/coordinates");
        if (scheme_halo(scheme) > G.ng) return set_error(GBNS_ERR_INVALID, "scheme stencil needs more ghost layers");
        if (!(dt > 0.0)) return set_error(GBNS_ERR_INVALID, "dt must be positive");
        for (int f = 0; f < 6; ++f)
            if (bc->kind[f] < GBNS_BC_PERIODIC || bc->kind[f] > GBNS_BC_SLIP_ADIABATIC) return set_error(GBNS_ERR_INVALID, "unknown boundary kind");
        const size_t arr = size_t(G.bstride)*G.nblk*sizeof(double);
        const size_t per = (arr + 255) & ~size_t(255);
        size_t off = 0;
        if (!b->arena.alloc(4*per, &off))
            return set_error(GBNS_ERR_CAPACITY, "HBM budget exhausted: instance needs " + std::to_string(4*per) +
                             " bytes, " + std::to_string(b->arena.size - b->arena.used) + " free (fragmented or full)");
        int si = -1;
        for (size_t i = 0; i < b->slots.size(); ++i) if (!b->slots[i].active) { si = int(i); break; }
        if (si < 0) { si = int(b->slots.size()); b->slots.emplace_back(); }
        rc = grow_insts(b, int(b->slots.size()));
        if (rc) { b->arena.release(off, 4*per); return rc; }
        Slot& sl = b->slots[si];
        sl.active = true;
        sl.g = *grid;
        sl.s = *scheme;
        sl.bc = *bc;
        sl.dt = dt;
        sl.off = off;
        sl.arr_bytes = per;
        sl.cls = cls;
        sl.steps = 0;
        sl.cells = (long long)G.n[0]*G.n[1]*G.n[2]*G.nblk;
        InstK I;
        std::memset(&I, 0, sizeof(I));
        I.G = G;
        I.S = S;
        for (int f = 0; f < 6; ++f) { I.bc.kind[f] = bc->kind[f]; I.bc.t_wall[f] = bc->t_wall[f]; }
        char* base = b->arena_base + off;
        I.q = reinterpret_cast<double*>(base);
        for (int r = 0; r < 3; ++r) I.R[r] = reinterpret_cast<double*>(base + (r + 1)*per);
        I.dt = dt;
        I.ytab = -1;
        if (grid->coords != GBNS_COORDS_IDENTITY)
        {
            static thread_local YTabK ytab;
            rc = make_ytab(grid, G, ytab);
            if (!rc) rc = check_cuda(cudaMemcpyAsync(b->d_ytabs + si, &ytab, sizeof(YTabK), cudaMemcpyHostToDevice, b->stream), "upload metric table");
            if (!rc) rc = check_cuda(cudaStreamSynchronize(b->stream), "upload metric table");
            I.ytab = si;
        }
        if (!rc) rc = check_cuda(cudaMemcpyAsync(I.q, prims, arr, cudaMemcpyDefault, b->stream), "copy initial state");
        if (!rc) rc = check_cuda(cudaMemcpyAsync(b->d_insts + si, &I, sizeof(InstK), cudaMemcpyHostToDevice, b->stream), "upload instance");
        if (!rc) rc = launch_steps_set(b->d_left, si, -1, b->stream);
        sl.left = -1;
        if (!rc) rc = launch_fill_ghosts(G, bc, I.q, b->stream);
        if (!rc) rc = check_cuda(cudaStreamSynchronize(b->stream), "batch add");
        if (rc) { sl.active = false; b->arena.release(off, 4*per); return rc; }
        b->dirty = true;
        *slot_out = si;
        return GBNS_OK;
    }

    int gbns_batch_remove(gbns_batch* b, int slot)
    {
        if (!b || slot < 0 || slot >= int(b->slots.size()) || !b->slots[slot].active)
            return set_error(GBNS_ERR_INVALID, "no active instance in that slot");
        // the caller's queued work may still read this instance
        int rc = enter(b);
        if (!rc) rc = check_cuda(cudaStreamSynchronize(b->stream), "batch remove");
        if (rc) return rc;
        Slot& sl = b->slots[slot];
        rc = launch_steps_set(b->d_left, slot, 0, b->stream);
        if (rc) return rc;
        b->arena.release(sl.off, 4*sl.arr_bytes);
        sl.active = false;
        sl.left = 0;
        b->dirty = true;
        return leave(b, GBNS_OK);
    }

    static int batch_step_impl(gbns_batch* b, int nsteps);

    int gbns_batch_step(gbns_batch* b, int nsteps)
    {
        if (!b || nsteps < 0) return set_error(GBNS_ERR_INVALID, "bad batch or step count");
        int rc = enter(b);
        if (rc) return rc;
        return leave(b, batch_step_impl(b, nsteps));
    }

    static int batch_step_impl(gbns_batch* b, int nsteps)
    {
        int rc = GBNS_OK;
        if (b->dirty) rc = rebuild_lists(b);
        if (rc) return rc;
        if (b->h_blocks.empty() || nsteps == 0) return GBNS_OK;
        if (b->use_graph)
        {
            if (!graph_current(b)) rc = capture(b);
            if (rc) return rc;
            for (int n = 0; n < nsteps; ++n)
            {
                rc = check_cuda(cudaGraphLaunch(b->gexec, b->stream), "graph launch");
                if (rc) return rc;
            }
        }
        else
        {
            for (int n = 0; n < nsteps && !rc; ++n) rc = launch_step(b);
            if (rc) return rc;
        }
        for (auto& sl : b->slots)
        {
            if (!sl.active) continue;
            if (sl.left < 0) { sl.steps += nsteps; continue; }
            const long long done = sl.left < nsteps ? sl.left : nsteps;
            sl.steps += done;
            sl.left -= done;
        }
        return GBNS_OK;
    }

    int gbns_batch_set_steps(gbns_batch* b, int slot, long long nsteps)
    {
        if (!b || slot < 0 || slot >= int(b->slots.size()) || !b->slots[slot].active)
            return set_error(GBNS_ERR_INVALID, "no active instance in that slot");
        int rc = enter(b);
        if (rc) return rc;
        const long long v = nsteps < 0 ? -1 : nsteps;
        rc = launch_steps_set(b->d_left, slot, v, b->stream);
        if (!rc) b->slots[slot].left = v;
        return leave(b, rc);
    }

    int gbns_batch_steps_left(gbns_batch* b, int slot, long long* left)
    {
        if (!b || !left || slot < 0 || slot >= int(b->slots.size()) || !b->slots[slot].active)
            return set_error(GBNS_ERR_INVALID, "no active instance in that slot");
        *left = b->slots[slot].left;
        return GBNS_OK;
    }

    int gbns_batch_state(gbns_batch* b, int slot, double** prims, long long* steps_done)
    {
        if (!b || slot < 0 || slot >= int(b->slots.size()) || !b->slots[slot].active)
            return set_error(GBNS_ERR_INVALID, "no active instance in that slot");
        const Slot& sl = b->slots[slot];
        if (prims) *prims = reinterpret_cast<double*>(b->arena_base + sl.off);
        if (steps_done) *steps_done = sl.steps;
        return GBNS_OK;
    }

    int gbns_batch_usage(gbns_batch* b, size_t* bytes_used, size_t* bytes_budget, int* active, long long* cells)
    {
        if (!b) return set_error(GBNS_ERR_INVALID, "NULL batch");
        int n = 0;
        long long c = 0;
        for (const auto& sl : b->slots) if (sl.active) { ++n; c += sl.cells; }
        if (bytes_used) *bytes_used = b->arena.used;
        if (bytes_budget) *bytes_budget = b->arena.size;
        if (active) *active = n;
        if (cells) *cells = c;
        return GBNS_OK;
    }

    int gbns_batch_autotune(gbns_batch* b, int reps, int* variants_out)
    {
        if (!b || reps < 1) return set_error(GBNS_ERR_INVALID, "bad batch or repetition count");
        int rc = enter(b);
        if (rc) return rc;
        if (b->dirty) rc = rebuild_lists(b);
        const unsigned active = b->class_mask;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (!rc) rc = check_cuda(cudaEventCreate(&e0), "autotune event");
        if (!rc) rc = check_cuda(cudaEventCreate(&e1), "autotune event");
        for (int c = 0; c < BCLASS_COUNT && !rc; ++c)
        {
            if (!(active & (1u << c))) continue;
            // stage 0 reads q and writes only R0 and the second state buffer,
            // so timing it leaves every instance's state as it was
            float best_ms = 0.0f;
            int best = 0;
            for (int v = 0; v < batch_class_variants(c, b->precision) && !rc; ++v)
            {
                b->variant[c] = v;
                rc = rebuild_lists(b);
                const int* offs = b->d_meta;
                const int* cnts = b->d_meta + BCLASS_COUNT;
                if (!rc) rc = launch_flux_batch(c, v, b->precision, b->d_tiles, offs, cnts, b->d_insts, b->d_ytabs,
                                                b->d_left, b->d_tmaps, 0, b->h_meta[BCLASS_COUNT + c], b->stream);
                if (!rc) rc = check_cuda(cudaEventRecord(e0, b->stream), "autotune event");
                for (int r = 0; r < reps && !rc; ++r)
                    rc = launch_flux_batch(c, v, b->precision, b->d_tiles, offs, cnts, b->d_insts, b->d_ytabs,
                                           b->d_left, b->d_tmaps, 0, b->h_meta[BCLASS_COUNT + c], b->stream);
                if (!rc) rc = check_cuda(cudaEventRecord(e1, b->stream), "autotune event");
                if (!rc) rc = check_cuda(cudaEventSynchronize(e1), "autotune sync");
                float ms = 0.0f;
                if (!rc) rc = check_cuda(cudaEventElapsedTime(&ms, e0, e1), "autotune elapsed");
                if (!rc && (v == 0 || ms < best_ms)) { best_ms = ms; best = v; }
            }
            b->variant[c] = best;
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (!rc) rc = rebuild_lists(b);
        b->graph_valid = false;
        if (!rc && variants_out)
            for (int c = 0; c < BCLASS_COUNT; ++c) variants_out[c] = (active & (1u << c)) ? b->variant[c] : -1;
        return leave(b, rc);
    }

    int gbns_batch_set_variant(gbns_batch* b, int cls, int variant)
    {
        if (!b || cls < 0 || cls >= BCLASS_COUNT) return set_error(GBNS_ERR_INVALID, "bad batch or kernel class");
        if (variant < 0 || variant >= batch_class_variants(cls, b->precision))
            return set_error(GBNS_ERR_INVALID, "tile variant out of range for this class");
        b->variant[cls] = variant;
        b->dirty = true;
        b->graph_valid = false;
        return GBNS_OK;
    }

    int gbns_batch_class_count(void) { return BCLASS_COUNT; }

    int gbns_batch_class_variant_info(int cls, int precision, int variant, int* tile_xyz)
    {
        if (cls < 0 || cls >= BCLASS_COUNT || variant < 0 || variant >= batch_class_variants(cls, precision))
            return set_error(GBNS_ERR_INVALID, "bad kernel class or variant");
        if (tile_xyz) batch_class_tile(cls, precision, variant, tile_xyz);
        return GBNS_OK;
    }

    size_t gbns_batch_instance_bytes(const gbns_grid_desc* grid)
    {
        GeomK G;
        if (make_geom(grid, G)) return 0;
        const size_t arr = size_t(G.bstride)*G.nblk*sizeof(double);
        return 4*((arr + 255) & ~size_t(255));
    }
}
