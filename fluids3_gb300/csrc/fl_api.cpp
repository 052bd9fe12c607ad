// Host runtime behind the C ABI (include/fluids_gb300.h): allocation, data
// movement, the phase sequence of FluidSystem::Run and graph replay.
//
// Reference counterparts (fluids4.0/fluid_system.cpp):
//   Initialize/Start/AllocateParticles/AllocateGrid   92-168, 218-272
//   TransferToCUDA / TransferFromCUDA                 2312-2330
//   InsertParticlesCUDA ... AdvanceCUDA               2334-2531
//   Run (RUN_GPU_FULL) / AdvanceTime                  475-542
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <vector>

#include "fl_internal.h"

// Pairs the density pass records per point for the force pass (HBM: 4 B
// per entry, 512 B per point of capacity).
static const int kPairListCap = 128;

// ---------------------------------------------------------------------------
// errors

static thread_local char g_err[512] = "";

int fl_fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

extern "C" const char *fl_last_error(void) { return g_err; }
extern "C" int fl_abi_version(void) { return FL_ABI_VERSION; }

// ---------------------------------------------------------------------------
// parameters

void fl_make_dev_params(const fl_params &p, DevParams *d) {
    memset(d, 0, sizeof(*d));
    d->gridMin = make_float3(p.gridMin[0], p.gridMin[1], p.gridMin[2]);
    d->gridDelta = make_float3(p.gridDelta[0], p.gridDelta[1], p.gridDelta[2]);
    d->gridRes = make_int3(p.gridRes[0], p.gridRes[1], p.gridRes[2]);
    d->gridScanMax = make_int3(p.gridScanMax[0], p.gridScanMax[1], p.gridScanMax[2]);
    d->gridSrch = p.gridSrch;
    d->gridAdjCnt = p.gridAdjCnt;
    d->ncells = p.gridTotal;
    d->nadj = (1 * p.gridRes[2] + 1) * p.gridRes[0] + 1;   // fluid_kernels.cu:120
    d->rd2 = p.rd2; d->d2 = p.d2; d->pmass = p.pmass; d->poly6kern = p.poly6kern;
    d->psmoothradius = p.psmoothradius; d->prest_dens = p.prest_dens;
    d->pintstiff = p.pintstiff; d->sim_scale = p.sim_scale;
    d->spikykern = p.spikykern; d->vterm = p.vterm; d->lapkern = p.lapkern;
    d->pradius = p.pradius; d->bound_slope = p.bound_slope; d->bound_stiff = p.bound_stiff;
    d->bound_damp = p.bound_damp; d->bound_friction = p.bound_friction;
    d->bound_wall_force = p.bound_wall_force; d->bound_wall_freq = p.bound_wall_freq;
    d->bound_min = make_float3(p.bound_min[0], p.bound_min[1], p.bound_min[2]);
    d->bound_max = make_float3(p.bound_max[0], p.bound_max[1], p.bound_max[2]);
    d->gravity = make_float3(p.gravity[0], p.gravity[1], p.gravity[2]);
    d->AL = p.AL; d->AL2 = p.AL2; d->VL = p.VL; d->VL2 = p.VL2;
    for (int c = 0; c < p.gridAdjCnt && c < 216; c++) d->adj[c] = p.gridAdj[c];
    // search-block pruning: cell edge 1/gridDelta per axis; band = h (1 + 1e-4)
    // plus 1e-3 of the smallest edge, orders of magnitude above the rounding
    // of the cell computation (see band_code in fl_kernels.cu)
    d->cellw = make_float3(1.0f / p.gridDelta[0], 1.0f / p.gridDelta[1], 1.0f / p.gridDelta[2]);
    float wmin = d->cellw.x;
    if (d->cellw.y < wmin) wmin = d->cellw.y;
    if (d->cellw.z < wmin) wmin = d->cellw.z;
    d->band = sqrtf(p.rd2) * 1.0001f + 1.0e-3f * wmin;
    d->prune = (p.gridSrch == 2) ? 1 : 0;
}

static int check_derived(const fl_params *p) {
    if (p->gridTotal <= 0 || p->gridSrch < 2 || p->gridSrch > FL_MAX_GRID_SRCH ||
        p->gridAdjCnt != p->gridSrch * p->gridSrch * p->gridSrch)
        return fl_fail(FL_ERR_PARAMS, "parameters are not derived (call fl_params_derive)");
    if ((long long)p->gridRes[0] * p->gridRes[1] * p->gridRes[2] != p->gridTotal)
        return fl_fail(FL_ERR_PARAMS, "gridTotal disagrees with gridRes");
    return FL_OK;
}

// ---------------------------------------------------------------------------
// allocation

int fl_dalloc(void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fl_fail(e == cudaErrorMemoryAllocation ? FL_ERR_NOMEM : FL_ERR_CUDA,
                       "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    }
    return FL_OK;
}

static void free_grid(fl_system *s) {
    cudaFree(s->cnt);
    cudaFree(s->off);
    cudaFree(s->tasks);
    s->codes_valid = 0;
    s->cnt = s->off = nullptr;
    s->tasks = nullptr;
    s->task_cap = 0;
    s->scan_ticket = nullptr;
    s->task_counters = nullptr;
    s->scan_status = nullptr;
}

// Grid block: [cnt (grid_pad) | ticket (256 B) | descriptors] in one
// allocation so one memset clears all of it; off is separate.
static size_t grid_block_bytes(const fl_system *s) {
    return s->grid_pad * sizeof(uint32_t) + fl_scan_scratch_bytes(s->scan_tiles);
}

static int alloc_grid(fl_system *s) {
    const size_t tile = fl_scan_tile();
    const size_t entries = (size_t)s->gcells;
    s->scan_tiles = (int)((entries + tile - 1) / tile);
    s->grid_pad = (size_t)s->scan_tiles * tile;
    void *blk = nullptr, *off = nullptr, *tasks = nullptr;
    FL_TRY(fl_dalloc(&blk, grid_block_bytes(s)));
    int r = fl_dalloc(&off, s->grid_pad * sizeof(uint32_t));
    if (r != FL_OK) { cudaFree(blk); return r; }
    s->task_cap = fl_task_cap(s->max_points, s->gcells);
    r = fl_dalloc(&tasks, s->task_cap * sizeof(uint2));
    if (r != FL_OK) { cudaFree(blk); cudaFree(off); return r; }
    s->tasks = (uint2 *)tasks;
    s->cnt = (uint32_t *)blk;
    s->scan_ticket = (uint32_t *)((char *)blk + s->grid_pad * sizeof(uint32_t));
    s->task_counters = s->scan_ticket + 1;   // same 256-byte slot as the ticket
    s->crowd_dev = s->scan_ticket + 4;       // cleared with it every step
    s->scan_status = (uint64_t *)((char *)s->scan_ticket + 256);
    s->off = (uint32_t *)off;
    s->scan_epoch = 1;
    s->codes_valid = 0;
    FL_CUDA_TRY(cudaMemsetAsync(blk, 0, grid_block_bytes(s), s->stream));
    FL_CUDA_TRY(cudaMemsetAsync(off, 0, s->grid_pad * sizeof(uint32_t), s->stream));
    return FL_OK;
}

static int ensure_side(fl_system *s);
static int reset_auto(fl_system *s);

static void destroy_graph(fl_system *s) {
    if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
    s->graph_exec = nullptr;
    s->graph_steps = 0;
}

static void free_all(fl_system *s) {
    destroy_graph(s);
    if (s->crowd_host) cudaFreeHost(s->crowd_host);
    fl_tape_free(s);
    for (int k = 0; k < F_COUNT; k++)
        for (int c = 0; c < 2; c++) cudaFree(s->f[k].p[c]);
    cudaFree(s->cell_pre); cudaFree(s->rank_tmp); cudaFree(s->src); cudaFree(s->upbits);
    cudaFree(s->hitlist); cudaFree(s->hitcnt); cudaFree(s->pairdata);
    cudaFree(s->big_cells); cudaFree(s->big_count);
    cudaFree(s->d_scenes); cudaFree(s->point_scene); cudaFree(s->cell_scene);
    free(s->scene_point_base); free(s->scene_n); free(s->scene_cell_base); free(s->scene_ncells);
    free(s->scene_params);
    free_grid(s);
    cudaFree(s->dev_err);
    cudaFree(s->time_dev);
    cudaFree(s->stage);
    for (int c = 0; c <= FL_MAX_CHECKPOINTS; c++) {
        for (int k = 0; k < F_COUNT; k++) cudaFree(s->ckpt[c][k]);
        cudaFree(s->ckpt_time[c]);
    }
    for (int k = 0; k < 8; k++)
        if (s->ev[k]) cudaEventDestroy(s->ev[k]);
    if (s->ev_early) cudaEventDestroy(s->ev_early);
    if (s->ev_late) cudaEventDestroy(s->ev_late);
    if (s->ev_crowd) cudaEventDestroy(s->ev_crowd);
    if (s->ev_crowd_done) cudaEventDestroy(s->ev_crowd_done);
    for (int k = 0; k < 2; k++)
        if (s->ev_auto[k]) cudaEventDestroy(s->ev_auto[k]);
    cudaFree(s->crowd_epoch);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->stream) cudaStreamDestroy(s->stream);
}

struct TimingState {
    std::vector<cudaEvent_t> events;   // 7 per timed step
    int steps = 0;
};
static TimingState *detach_timing(fl_system *s);

extern "C" int fl_create(const fl_params *p, int max_points, fl_system **out) {
    if (!p || !out) return fl_fail(FL_ERR_ARG, "fl_create: null argument");
    *out = nullptr;
    if (max_points < 0) return fl_fail(FL_ERR_ARG, "fl_create: max_points < 0");
    FL_TRY(check_derived(p));
    fl_system *s = (fl_system *)calloc(1, sizeof(fl_system));
    if (!s) return fl_fail(FL_ERR_NOMEM, "fl_create: host allocation failed");
    s->passes = FL_PASSES_AUTO;   // per-point passes, cell tasks once cells crowd (fl_set_neighbour_passes)
    int r = FL_OK;
    do {
        if (cudaGetDevice(&s->device) != cudaSuccess) {
            r = fl_fail(FL_ERR_CUDA, "fl_create: no CUDA device");
            break;
        }
        if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
            r = fl_fail(FL_ERR_CUDA, "fl_create: cudaStreamCreate failed");
            break;
        }
        if (cudaHostAlloc((void **)&s->crowd_host, 64, cudaHostAllocDefault) != cudaSuccess) {
            s->crowd_host = nullptr;
            r = fl_fail(FL_ERR_NOMEM, "fl_create: page-locked allocation failed");
            break;
        }
        s->crowd_host[0] = s->crowd_host[1] = 0;
        if ((r = fl_dalloc((void **)&s->crowd_epoch, 256)) != FL_OK) break;
        if (cudaMemset(s->crowd_epoch, 0, 256) != cudaSuccess) {
            r = fl_fail(FL_ERR_CUDA, "fl_create: memset failed");
            break;
        }
        if ((r = ensure_side(s)) != FL_OK) break;
        s->P = *p;
        fl_make_dev_params(*p, &s->D);
        s->max_points = max_points;
        s->ncells = p->gridTotal;
        s->gcells = p->gridTotal + 1;
        s->nscenes = 1;
        const size_t np = (size_t)(max_points > 0 ? max_points : 1);
        const size_t esz[F_COUNT] = {16, 16, 16, 16, 4, 4, 4, 4};
        for (int k = 0; k < F_COUNT && r == FL_OK; k++) {
            s->f[k].esz = esz[k];
            for (int c = 0; c < 2 && r == FL_OK; c++) r = fl_dalloc(&s->f[k].p[c], esz[k] * np);
        }
        if (r != FL_OK) break;
        if ((r = fl_dalloc((void **)&s->cell_pre, 4 * np)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&s->rank_tmp, 4 * np)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&s->src, 4 * np)) != FL_OK) break;
        s->D.upwords = (int)((np + 31) / 32 + 1);
        // rows 0-2: upper-band flags; rows 3-5: lower-band flags (adjoint only)
        if ((r = fl_dalloc((void **)&s->upbits, 2 * fl_upbits_bytes(s))) != FL_OK) break;
        s->D.hcap = kPairListCap;
        if ((r = fl_dalloc((void **)&s->hitlist, 4 * ((np + 31) / 32) * 32 * (size_t)kPairListCap)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&s->hitcnt, 4 * np)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&s->pairdata, 2 * sizeof(float4) * np)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&s->big_cells, 4 * fl_big_cells_cap(max_points))) != FL_OK) break;
        if ((r = fl_dalloc((void **)&s->big_count, 256)) != FL_OK) break;
        if (cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, s->device) != cudaSuccess ||
            s->num_sms < 1) {
            r = fl_fail(FL_ERR_CUDA, "fl_create: SM count");
            break;
        }
        if ((r = fl_kernels_init(s)) != FL_OK) break;
        if ((r = fl_cells_init(s)) != FL_OK) break;
        if ((r = fl_pairs_init()) != FL_OK) break;
        if ((r = fl_dalloc((void **)&s->dev_err, 256)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&s->time_dev, 256)) != FL_OK) break;
        if ((r = alloc_grid(s)) != FL_OK) break;
        if (cudaMemsetAsync(s->dev_err, 0, 256, s->stream) != cudaSuccess ||
            cudaMemsetAsync(s->time_dev, 0, 256, s->stream) != cudaSuccess ||
            cudaMemsetAsync(s->big_count, 0, 256, s->stream) != cudaSuccess) {
            r = fl_fail(FL_ERR_CUDA, "fl_create: memset failed");
            break;
        }
        for (int k = 0; k < F_COUNT && r == FL_OK; k++)
            for (int c = 0; c < 2; c++)
                if (cudaMemsetAsync(s->f[k].p[c], 0, s->f[k].esz * np, s->stream) != cudaSuccess)
                    r = fl_fail(FL_ERR_CUDA, "fl_create: memset failed");
        if (r != FL_OK) break;
        for (int k = 0; k < 8; k++)
            if (cudaEventCreate(&s->ev[k]) != cudaSuccess) r = fl_fail(FL_ERR_CUDA, "fl_create: event");
        if (r != FL_OK) break;
        s->time = 0.0f;
        s->time_host_valid = 1;
        if (cudaStreamSynchronize(s->stream) != cudaSuccess) {
            r = fl_fail(FL_ERR_CUDA, "fl_create: %s", cudaGetErrorString(cudaGetLastError()));
            break;
        }
    } while (0);
    if (r != FL_OK) {
        free_all(s);
        free(s);
        return r;
    }
    *out = s;
    return FL_OK;
}

// ---------------------------------------------------------------------------
// batched systems

extern "C" int fl_batch_create(const fl_params *params, const int *counts, int nscenes, fl_system **out) {
    if (!params || !counts || !out) return fl_fail(FL_ERR_ARG, "fl_batch_create: null argument");
    *out = nullptr;
    if (nscenes < 1 || nscenes > 65535)
        return fl_fail(FL_ERR_ARG, "fl_batch_create: %d scenes (1..65535)", nscenes);
    long long npts = 0, ncell = 0, gcell = 0;
    int all_prune = 1;
    for (int k = 0; k < nscenes; k++) {
        FL_TRY(check_derived(&params[k]));
        if (counts[k] < 0) return fl_fail(FL_ERR_ARG, "fl_batch_create: scene %d count < 0", k);
        if (params[k].dt != params[0].dt)
            return fl_fail(FL_ERR_PARAMS, "fl_batch_create: scene %d has dt %g, scene 0 %g (the batch shares one clock)",
                           k, (double)params[k].dt, (double)params[0].dt);
        npts += counts[k];
        ncell += params[k].gridTotal;
        gcell += params[k].gridTotal + 1;
        if (params[k].gridSrch != 2) all_prune = 0;
    }
    if (npts > (1LL << 31) - 1 || gcell > (1LL << 30))
        return fl_fail(FL_ERR_PARAMS, "fl_batch_create: %lld points / %lld cell entries exceed the limits", npts, gcell);

    // allocate as one big system over the concatenation, then install the scene table
    fl_params p0 = params[0];
    p0.gridTotal = (int)ncell;                      // reference-layout cells (all scenes)
    p0.gridRes[0] = (int)ncell; p0.gridRes[1] = 1; p0.gridRes[2] = 1;
    fl_system *s = nullptr;
    FL_TRY(fl_create(&p0, (int)npts, &s));
    int r = FL_OK;
    do {
        s->P = params[0];
        s->batched = 1;
        s->nscenes = nscenes;
        if ((r = fl_cells_init(s)) != FL_OK) break;
        if ((r = fl_pairs_init()) != FL_OK) break;
        free_grid(s);
        s->ncells = (int)ncell;
        s->gcells = (int)gcell;
        if ((r = alloc_grid(s)) != FL_OK) break;
        s->scene_point_base = (int *)calloc(nscenes, sizeof(int));
        s->scene_n = (int *)calloc(nscenes, sizeof(int));
        s->scene_cell_base = (int *)calloc(nscenes, sizeof(int));
        s->scene_ncells = (int *)calloc(nscenes, sizeof(int));
        s->scene_params = (fl_params *)calloc(nscenes, sizeof(fl_params));
        if (s->scene_params) memcpy(s->scene_params, params, sizeof(fl_params) * nscenes);
        std::vector<DevParams> tab(nscenes);
        std::vector<uint16_t> pscene((size_t)(npts > 0 ? npts : 1)), cscene((size_t)gcell);
        if (!s->scene_point_base || !s->scene_n || !s->scene_cell_base || !s->scene_ncells || !s->scene_params) {
            r = fl_fail(FL_ERR_NOMEM, "fl_batch_create: host allocation failed");
            break;
        }
        long long pb = 0, cb = 0;
        for (int k = 0; k < nscenes; k++) {
            fl_make_dev_params(params[k], &tab[k]);
            tab[k].cell_base = (int)cb;
            tab[k].upwords = s->D.upwords;
            tab[k].hcap = s->D.hcap;
            tab[k].prune = all_prune;
            s->scene_point_base[k] = (int)pb;
            s->scene_n[k] = counts[k];
            s->scene_cell_base[k] = (int)cb;
            s->scene_ncells[k] = params[k].gridTotal;
            for (long long i = 0; i < counts[k]; i++) pscene[(size_t)(pb + i)] = (uint16_t)k;
            for (long long c = 0; c <= params[k].gridTotal; c++) cscene[(size_t)(cb + c)] = (uint16_t)k;
            pb += counts[k];
            cb += params[k].gridTotal + 1;
        }
        // launch-wide constants come from scene 0's block
        const int upwords = s->D.upwords, hcap = s->D.hcap;
        s->D = tab[0];
        s->D.upwords = upwords;
        s->D.hcap = hcap;
        s->D.prune = all_prune;
        if ((r = fl_dalloc((void **)&s->d_scenes, sizeof(DevParams) * nscenes)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&s->point_scene, sizeof(uint16_t) * pscene.size())) != FL_OK) break;
        if ((r = fl_dalloc((void **)&s->cell_scene, sizeof(uint16_t) * cscene.size())) != FL_OK) break;
        if (cudaMemcpy(s->d_scenes, tab.data(), sizeof(DevParams) * nscenes, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(s->point_scene, pscene.data(), sizeof(uint16_t) * pscene.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(s->cell_scene, cscene.data(), sizeof(uint16_t) * cscene.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
            r = fl_fail(FL_ERR_CUDA, "fl_batch_create: scene table upload failed");
            break;
        }
        if (cudaStreamSynchronize(s->stream) != cudaSuccess) {
            r = fl_fail(FL_ERR_CUDA, "fl_batch_create: %s", cudaGetErrorString(cudaGetLastError()));
            break;
        }
    } while (0);
    if (r != FL_OK) {
        fl_destroy(s);
        return r;
    }
    *out = s;
    return FL_OK;
}

extern "C" int fl_batch_scene_info(const fl_system *s, int scene, int *point_base, int *n, int *cell_base,
                                   int *ncells) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_batch_scene_info: null system");
    if (scene < 0 || scene >= s->nscenes) return fl_fail(FL_ERR_ARG, "fl_batch_scene_info: scene %d", scene);
    int pb = 0, np = s->n, cb = 0, nc = s->ncells;
    if (s->batched) {
        pb = s->scene_point_base[scene];
        np = s->scene_n[scene];
        nc = s->scene_ncells[scene];
        cb = 0;
        for (int k = 0; k < scene; k++) cb += s->scene_ncells[k];   // reference-layout position
    }
    if (point_base) *point_base = pb;
    if (n) *n = np;
    if (cell_base) *cell_base = cb;
    if (ncells) *ncells = nc;
    return FL_OK;
}

extern "C" int fl_num_scenes(const fl_system *s) { return s ? s->nscenes : 0; }

extern "C" int fl_batch_get_params(const fl_system *s, int scene, fl_params *p) {
    if (!s || !p) return fl_fail(FL_ERR_ARG, "fl_batch_get_params: null argument");
    if (scene < 0 || scene >= s->nscenes) return fl_fail(FL_ERR_ARG, "fl_batch_get_params: scene %d", scene);
    *p = s->batched ? s->scene_params[scene] : s->P;
    return FL_OK;
}

extern "C" int fl_batch_set_params(fl_system *s, int scene, const fl_params *p) {
    if (!s || !p) return fl_fail(FL_ERR_ARG, "fl_batch_set_params: null argument");
    if (scene < 0 || scene >= s->nscenes) return fl_fail(FL_ERR_ARG, "fl_batch_set_params: scene %d", scene);
    if (!s->batched) return fl_set_params(s, p);
    FL_TRY(check_derived(p));
    const fl_params &o = s->scene_params[scene];
    bool same = p->gridSrch == o.gridSrch && p->gridTotal == o.gridTotal && p->dt == o.dt;
    for (int k = 0; k < 3; k++)
        same = same && p->gridRes[k] == o.gridRes[k] && p->gridMin[k] == o.gridMin[k] &&
               p->gridDelta[k] == o.gridDelta[k] && p->gridScanMax[k] == o.gridScanMax[k];
    if (!same)
        return fl_fail(FL_ERR_PARAMS, "fl_batch_set_params: scene %d: the new block changes the scene's grid or dt",
                       scene);
    DevParams d;
    fl_make_dev_params(*p, &d);
    d.cell_base = s->scene_cell_base[scene];
    d.upwords = s->D.upwords;
    d.hcap = s->D.hcap;
    d.prune = s->D.prune;
    FL_CUDA_TRY(cudaMemcpyAsync(s->d_scenes + scene, &d, sizeof(d), cudaMemcpyHostToDevice, s->stream));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->scene_params[scene] = *p;
    if (scene == 0) {   // scene 0's block also serves as the launch-wide one
        const int upwords = s->D.upwords, hcap = s->D.hcap, prune = s->D.prune;
        s->D = d;
        s->D.cell_base = 0;
        s->D.upwords = upwords;
        s->D.hcap = hcap;
        s->D.prune = prune;
        s->P = *p;
        destroy_graph(s);
    }
    fl_tape_touch(s);
    return FL_OK;
}

extern "C" int fl_destroy(fl_system *s) {
    if (!s) return FL_OK;
    cudaStreamSynchronize(s->stream);
    TimingState *t = detach_timing(s);
    if (t) {
        for (cudaEvent_t e : t->events) cudaEventDestroy(e);
        delete t;
    }
    free_all(s);
    free(s);
    return FL_OK;
}

// Timing state lives beside the system (kept out of the plain-C struct).
static std::map<fl_system *, TimingState *> g_timing;
static TimingState *detach_timing(fl_system *s) {
    auto it = g_timing.find(s);
    if (it == g_timing.end()) return nullptr;
    TimingState *t = it->second;
    g_timing.erase(it);
    return t;
}

void fl_reset_progress(fl_system *s) {
    fl_tape_touch(s);
    s->have_insert = s->have_offsets = s->have_grid = 0;
    s->codes_valid = 0;
    s->lists_valid = 0;
    s->offsets_inclusive = 0;
}

extern "C" int fl_set_params(fl_system *s, const fl_params *p) {
    if (!s || !p) return fl_fail(FL_ERR_ARG, "fl_set_params: null argument");
    FL_TRY(check_derived(p));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (s->batched)
        return fl_fail(FL_ERR_STATE, "fl_set_params: a batched system keeps the parameters it was created with");
    if (p->gridTotal != s->ncells) {
        free_grid(s);
        s->ncells = p->gridTotal;
        s->gcells = p->gridTotal + 1;
        FL_TRY(alloc_grid(s));
    }
    const int upwords = s->D.upwords, hcap = s->D.hcap;
    s->P = *p;
    fl_make_dev_params(*p, &s->D);
    s->D.upwords = upwords;
    s->D.hcap = hcap;
    destroy_graph(s);
    fl_reset_progress(s);
    return FL_OK;
}

extern "C" int fl_get_params(const fl_system *s, fl_params *p) {
    if (!s || !p) return fl_fail(FL_ERR_ARG, "fl_get_params: null argument");
    *p = s->P;
    return FL_OK;
}

extern "C" int fl_num_points(const fl_system *s) { return s ? s->n : 0; }
extern "C" int fl_grid_total(const fl_system *s) { return s ? s->ncells : 0; }

static int sync_time_to_host(fl_system *s) {
    if (s->time_host_valid) return FL_OK;
    FL_CUDA_TRY(cudaMemcpyAsync(&s->time, s->time_dev + s->time_slot, sizeof(float),
                                cudaMemcpyDeviceToHost, s->stream));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->time_host_valid = 1;
    return FL_OK;
}

extern "C" int fl_get_time(const fl_system *cs, float *t) {
    fl_system *s = const_cast<fl_system *>(cs);
    if (!s || !t) return fl_fail(FL_ERR_ARG, "fl_get_time: null argument");
    FL_TRY(sync_time_to_host(s));
    *t = s->time;
    return FL_OK;
}

extern "C" int fl_set_time(fl_system *s, float t) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_set_time: null system");
    s->time = t;
    s->time_host_valid = 1;
    FL_CUDA_TRY(cudaMemcpyAsync(s->time_dev + s->time_slot, &s->time, sizeof(float),
                                cudaMemcpyHostToDevice, s->stream));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return FL_OK;
}

extern "C" void *fl_stream(fl_system *s) { return s ? (void *)s->stream : nullptr; }

// ---------------------------------------------------------------------------
// data movement

int fl_ensure_stage(fl_system *s, size_t bytes) {
    if (bytes <= s->stage_bytes) return FL_OK;
    cudaFree(s->stage);
    s->stage = nullptr;
    s->stage_bytes = 0;
    FL_TRY(fl_dalloc(&s->stage, bytes));
    s->stage_bytes = bytes;
    return FL_OK;
}

extern "C" int fl_host_alloc(size_t bytes, void **out) {
    if (!out) return fl_fail(FL_ERR_ARG, "fl_host_alloc: null argument");
    *out = nullptr;
    cudaError_t e = cudaHostAlloc(out, bytes ? bytes : 16, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        *out = nullptr;
        return fl_fail(FL_ERR_NOMEM, "cudaHostAlloc(%zu): %s", bytes, cudaGetErrorString(e));
    }
    return FL_OK;
}

extern "C" int fl_host_free(void *p) {
    if (p) FL_CUDA_TRY(cudaFreeHost(p));
    return FL_OK;
}

// Page-locked host memory (fl_host_alloc, cudaHostAlloc) is mapped into the
// device's address space: kernels read and write it directly over the
// host link, so a transfer needs no staging copy. Returns the device-side
// address of such memory, or null for pageable memory.
static void *mapped_device_ptr(const void *host) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost) ? a.devicePointer : nullptr;
}

extern "C" int fl_set_particles(fl_system *s, int n, const float *pos, const float *vel,
                                const float *veval, const float *force, const float *press,
                                const uint32_t *clr) {
    if (!s || !pos) return fl_fail(FL_ERR_ARG, "fl_set_particles: null system or pos");
    if (n < 0) return fl_fail(FL_ERR_ARG, "fl_set_particles: n < 0");
    if (n > s->max_points)
        return fl_fail(FL_ERR_CAPACITY, "fl_set_particles: %d points exceed capacity %d", n, s->max_points);
    if (s->batched && n != s->max_points)
        return fl_fail(FL_ERR_ARG, "fl_set_particles: a batched system takes all %d points (scenes concatenated)",
                       s->max_points);
    destroy_graph(s);
    FL_TRY(reset_auto(s));
    s->n = n;
    if (n > 0) {
        // one staging slice per float3 field, then unpack to float4 on device
        const size_t v3 = 12 * (size_t)n;
        FL_TRY(fl_ensure_stage(s, 4 * v3));
        const float *src3[4] = {pos, vel, veval, force};
        const int fid[4] = {F_POS, F_VEL, F_VEVAL, F_FORCE};
        const float *msrc[4];
        float4 *mdst[4];
        int nm = 0;
        for (int k = 0; k < 4; k++) {
            float4 *dst = s->f[fid[k]].cur<float4>();
            if (!src3[k]) {
                FL_CUDA_TRY(cudaMemsetAsync(dst, 0, sizeof(float4) * (size_t)n, s->stream));
                continue;
            }
            if (const void *mapped = mapped_device_ptr(src3[k])) {   // read over the host link, below
                msrc[nm] = (const float *)mapped;
                mdst[nm++] = dst;
                continue;
            }
            float *slice = (float *)((char *)s->stage + k * v3);
            FL_CUDA_TRY(cudaMemcpyAsync(slice, src3[k], v3, cudaMemcpyHostToDevice, s->stream));
            FL_TRY(fl_launch_unpack3(s, slice, dst, n));
        }
        FL_TRY(fl_launch_unpack3_set(s, nm, msrc, mdst, n));
        const void *src1[2] = {press, clr};
        const int fid1[2] = {F_PRESS, F_CLR};
        for (int k = 0; k < 2; k++) {
            void *dst = s->f[fid1[k]].cur<void>();
            if (!src1[k]) FL_CUDA_TRY(cudaMemsetAsync(dst, 0, 4 * (size_t)n, s->stream));
            else FL_CUDA_TRY(cudaMemcpyAsync(dst, src1[k], 4 * (size_t)n, cudaMemcpyHostToDevice, s->stream));
        }
    }
    // the caller may reuse its host arrays on return
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    fl_reset_progress(s);
    return FL_OK;
}

// AddParticle (fluids4.0/fluid_system.cpp:274-290) k times with the given
// values: the points go after the live ones, force and density start at 0.
extern "C" int fl_add_particles(fl_system *s, int k, const float *pos, const float *vel, const float *veval,
                                const uint32_t *clr) {
    if (!s || (k > 0 && !pos)) return fl_fail(FL_ERR_ARG, "fl_add_particles: null system or pos");
    if (k < 0) return fl_fail(FL_ERR_ARG, "fl_add_particles: k < 0");
    if (s->batched) return fl_fail(FL_ERR_STATE, "fl_add_particles: a batched system has fixed scene sizes");
    if ((long long)s->n + k > s->max_points)
        return fl_fail(FL_ERR_CAPACITY, "fl_add_particles: %d + %d points exceed capacity %d", s->n, k, s->max_points);
    if (k == 0) return FL_OK;
    destroy_graph(s);
    const int base = s->n;
    const size_t v3 = 12 * (size_t)k;
    FL_TRY(fl_ensure_stage(s, 3 * v3));
    const float *src3[3] = {pos, vel, veval};
    const int fid[3] = {F_POS, F_VEL, F_VEVAL};
    for (int q = 0; q < 3; q++) {
        float4 *dst = s->f[fid[q]].cur<float4>() + base;
        if (!src3[q]) {
            FL_CUDA_TRY(cudaMemsetAsync(dst, 0, sizeof(float4) * (size_t)k, s->stream));
            continue;
        }
        float *slice = (float *)((char *)s->stage + q * v3);
        FL_CUDA_TRY(cudaMemcpyAsync(slice, src3[q], v3, cudaMemcpyHostToDevice, s->stream));
        FL_TRY(fl_launch_unpack3(s, slice, dst, k));
    }
    FL_CUDA_TRY(cudaMemsetAsync(s->f[F_FORCE].cur<float4>() + base, 0, sizeof(float4) * (size_t)k, s->stream));
    FL_CUDA_TRY(cudaMemsetAsync(s->f[F_PRESS].cur<float>() + base, 0, 4 * (size_t)k, s->stream));
    uint32_t *cdst = s->f[F_CLR].cur<uint32_t>() + base;
    if (clr) FL_CUDA_TRY(cudaMemcpyAsync(cdst, clr, 4 * (size_t)k, cudaMemcpyHostToDevice, s->stream));
    else FL_CUDA_TRY(cudaMemsetAsync(cdst, 0, 4 * (size_t)k, s->stream));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->n = base + k;
    fl_reset_progress(s);
    return FL_OK;
}

static int buffer_bytes(const fl_system *s, int id, size_t *bytes) {
    switch (id) {
    case FL_FPOS: case FL_FVEL: case FL_FVEVAL: case FL_FFORCE: *bytes = 12 * (size_t)s->n; return FL_OK;
    case FL_FPRESS: case FL_FCLR: case FL_FGCELL: case FL_FGNDX: case FL_FGRID:
        *bytes = 4 * (size_t)s->n; return FL_OK;
    case FL_FGRIDCNT: case FL_FGRIDOFF: *bytes = 4 * (size_t)s->ncells; return FL_OK;
    default: return fl_fail(FL_ERR_ARG, "unknown buffer id %d", id);
    }
}

static int field_of(int id) {
    switch (id) {
    case FL_FPOS: return F_POS; case FL_FVEL: return F_VEL; case FL_FVEVAL: return F_VEVAL;
    case FL_FFORCE: return F_FORCE; case FL_FPRESS: return F_PRESS; case FL_FCLR: return F_CLR;
    case FL_FGCELL: return F_GCELL; case FL_FGNDX: return F_GNDX;
    default: return -1;
    }
}

// Produce buffer `id` in fluid.h layout at device address dev (async).
static int export_to_device(fl_system *s, int id, void *dev) {
    const int fi = field_of(id);
    if (id == FL_FPOS || id == FL_FVEL || id == FL_FVEVAL || id == FL_FFORCE)
        return fl_launch_pack3(s, s->f[fi].cur<float4>(), (float *)dev, s->n);
    if (id == FL_FGCELL && s->batched) return fl_launch_gcell_ref(s, (uint32_t *)dev);
    if (fi >= 0) {
        FL_CUDA_TRY(cudaMemcpyAsync(dev, s->f[fi].cur<void>(), 4 * (size_t)s->n,
                                    cudaMemcpyDeviceToDevice, s->stream));
        return FL_OK;
    }
    if (id == FL_FGRIDCNT || id == FL_FGRIDOFF) {
        // reference layout: each scene's C cells, without its out-of-range bin
        const uint32_t *srcg = (id == FL_FGRIDCNT) ? s->cnt : s->off;
        size_t at = 0;
        for (int sc = 0; sc < s->nscenes; sc++) {
            const int base = s->batched ? s->scene_cell_base[sc] : 0;
            const int c = s->batched ? s->scene_ncells[sc] : s->ncells;
            FL_CUDA_TRY(cudaMemcpyAsync((uint32_t *)dev + at, srcg + base, 4 * (size_t)c,
                                        cudaMemcpyDeviceToDevice, s->stream));
            at += (size_t)c;
        }
        return FL_OK;
    }
    if (id == FL_FGRID) {
        // identity over the in-range sorted slots (countingSortFull sets FGRID[s] = s, cu:83)
        return fl_launch_grid_identity(s, (uint32_t *)dev, s->n,
                                       s->have_grid ? s->f[F_GCELL].cur<uint32_t>() : nullptr);
    }
    return fl_fail(FL_ERR_ARG, "unknown buffer id %d", id);
}

extern "C" int fl_get_buffer(fl_system *s, int id, void *host, size_t bytes) {
    if (!s || !host) return fl_fail(FL_ERR_ARG, "fl_get_buffer: null argument");
    size_t need = 0;
    FL_TRY(buffer_bytes(s, id, &need));
    if (bytes < need) return fl_fail(FL_ERR_ARG, "fl_get_buffer: %zu bytes < %zu needed", bytes, need);
    if (need == 0) return FL_OK;
    // Packed on the device, then one copy-engine transfer: into page-locked
    // memory this beats the pack kernel writing over the host link (191 vs
    // ~150 GB/s on GB300), unlike uploads, where kernels reading page-locked
    // memory directly beat staging.
    FL_TRY(fl_ensure_stage(s, need));
    FL_TRY(export_to_device(s, id, s->stage));
    FL_CUDA_TRY(cudaMemcpyAsync(host, s->stage, need, cudaMemcpyDeviceToHost, s->stream));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (id == FL_FGRIDOFF && s->offsets_inclusive) {
        // zero_offsets = 0 asks for the inclusive scan: off[c] + cnt[c]
        std::vector<uint32_t> cnt(s->ncells);
        FL_TRY(export_to_device(s, FL_FGRIDCNT, s->stage));
        FL_CUDA_TRY(cudaMemcpyAsync(cnt.data(), s->stage, 4 * (size_t)s->ncells, cudaMemcpyDeviceToHost,
                                    s->stream));
        FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
        uint32_t *o = (uint32_t *)host;
        for (int c = 0; c < s->ncells; c++) o[c] += cnt[c];
    }
    return FL_OK;
}

extern "C" int fl_export_device(fl_system *s, int id, void *dev, size_t bytes) {
    if (!s || !dev) return fl_fail(FL_ERR_ARG, "fl_export_device: null argument");
    size_t need = 0;
    FL_TRY(buffer_bytes(s, id, &need));
    if (bytes < need) return fl_fail(FL_ERR_ARG, "fl_export_device: %zu bytes < %zu needed", bytes, need);
    if (need == 0) return FL_OK;
    if (id == FL_FGRIDOFF && s->offsets_inclusive)
        return fl_fail(FL_ERR_STATE, "fl_export_device: inclusive offsets are host-readback only");
    return export_to_device(s, id, dev);
}

extern "C" int fl_import_device(fl_system *s, int n, const void *dev_pos, const void *dev_vel,
                                const void *dev_veval) {
    if (!s || !dev_pos) return fl_fail(FL_ERR_ARG, "fl_import_device: null system or pos");
    if (n < 0 || n > s->max_points)
        return fl_fail(FL_ERR_CAPACITY, "fl_import_device: %d points (capacity %d)", n, s->max_points);
    if (s->batched && n != s->max_points)
        return fl_fail(FL_ERR_ARG, "fl_import_device: a batched system takes all %d points", s->max_points);
    destroy_graph(s);
    s->n = n;
    FL_TRY(fl_launch_unpack3(s, (const float *)dev_pos, s->f[F_POS].cur<float4>(), n));
    if (dev_vel) FL_TRY(fl_launch_unpack3(s, (const float *)dev_vel, s->f[F_VEL].cur<float4>(), n));
    else FL_CUDA_TRY(cudaMemsetAsync(s->f[F_VEL].cur<void>(), 0, 16 * (size_t)n, s->stream));
    if (dev_veval) FL_TRY(fl_launch_unpack3(s, (const float *)dev_veval, s->f[F_VEVAL].cur<float4>(), n));
    else FL_CUDA_TRY(cudaMemsetAsync(s->f[F_VEVAL].cur<void>(), 0, 16 * (size_t)n, s->stream));
    fl_reset_progress(s);
    return FL_OK;
}

// ---------------------------------------------------------------------------
// phases

static int clear_grid(fl_system *s) {
    // InsertParticlesCUDA clears FGRIDCNT/FGRIDOFF (cpp:2336-2337); here one
    // memset clears the counts, the scan ticket and the scan descriptors.
    FL_CUDA_TRY(cudaMemsetAsync(s->cnt, 0, grid_block_bytes(s), s->stream));
    return FL_OK;
}

static int readback(fl_system *s, void *host, const void *dev, size_t bytes) {
    if (!host || bytes == 0) return FL_OK;
    FL_CUDA_TRY(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s->stream));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return FL_OK;
}

extern "C" int fl_insert_particles(fl_system *s, uint32_t *gcell, uint32_t *gndx, uint32_t *gcnt) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_insert_particles: null system");
    fl_tape_touch(s);
    FL_TRY(clear_grid(s));
    FL_TRY(fl_launch_insert(s, s->f[F_GCELL].cur<uint32_t>()));
    // canonical gndx: offsets, arrival-order index scatter, per-cell sort
    FL_TRY(fl_launch_scan(s, s->gcells, 0));
    FL_TRY(fl_launch_scatter_index(s));
    FL_TRY(fl_launch_sort_cells(s, 0));
    s->codes_valid = 0;
    s->lists_valid = 0;
    s->have_insert = 1;
    s->have_offsets = 0;
    s->have_grid = 0;
    FL_TRY(readback(s, gcell, s->f[F_GCELL].cur<void>(), 4 * (size_t)s->n));
    FL_TRY(readback(s, gndx, s->f[F_GNDX].cur<void>(), 4 * (size_t)s->n));
    if (gcnt) FL_TRY(fl_get_buffer(s, FL_FGRIDCNT, gcnt, 4 * (size_t)s->ncells));
    return FL_OK;
}

extern "C" int fl_prefix_sum_cells(fl_system *s, uint32_t *goff, int zero_offsets) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_prefix_sum_cells: null system");
    fl_tape_touch(s);
    if (!s->have_insert) return fl_fail(FL_ERR_STATE, "fl_prefix_sum_cells before fl_insert_particles");
    FL_TRY(fl_launch_scan(s, s->gcells, 1));
    s->have_offsets = 1;
    s->offsets_inclusive = zero_offsets ? 0 : 1;
    if (goff) FL_TRY(fl_get_buffer(s, FL_FGRIDOFF, goff, 4 * (size_t)s->ncells));
    return FL_OK;
}

static void flip(fl_system *s, int k) { s->f[k].live ^= 1; }

extern "C" int fl_counting_sort_full(fl_system *s, float *ppos) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_counting_sort_full: null system");
    fl_tape_touch(s);
    if (!s->have_insert || !s->have_offsets)
        return fl_fail(FL_ERR_STATE, "fl_counting_sort_full before insert and prefix sum");
    FL_TRY(fl_launch_gather_all(s));
    for (int k = 0; k < F_COUNT; k++) flip(s, k);
    s->lists_valid = 0;
    FL_TRY(fl_launch_band_codes(s));
    s->have_grid = 1;
    s->have_insert = 0;   // the pre-sort cell list no longer matches the order
    if (ppos) FL_TRY(fl_get_buffer(s, FL_FPOS, ppos, 12 * (size_t)s->n));
    return FL_OK;
}

extern "C" int fl_compute_pressure(fl_system *s) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_compute_pressure: null system");
    fl_tape_touch(s);
    if (!s->have_grid) return fl_fail(FL_ERR_STATE, "fl_compute_pressure before fl_counting_sort_full");
    return fl_launch_density(s);
}

extern "C" int fl_compute_force(fl_system *s) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_compute_force: null system");
    fl_tape_touch(s);
    if (!s->have_grid) return fl_fail(FL_ERR_STATE, "fl_compute_force before fl_counting_sort_full");
    return fl_launch_force(s);
}

extern "C" int fl_advance(fl_system *s, float time, float dt, float ss) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_advance: null system");
    fl_tape_touch(s);
    if (!s->have_grid) return fl_fail(FL_ERR_STATE, "fl_advance before fl_counting_sort_full");
    s->codes_valid = 0;   // positions move; their band codes and pair lists no longer hold
    s->lists_valid = 0;
    return fl_launch_advance(s, time, dt, ss);
}

// ---------------------------------------------------------------------------
// Run: the fused step

static int record(fl_system *s, TimingState *t, int k) {
    if (!t) return FL_OK;
    FL_CUDA_TRY(cudaEventRecord(t->events[(size_t)t->steps * 7 + k], s->stream));
    return FL_OK;
}

// The cell-task passes (fl_cells.cu) need the pruned search (gridSrch 2 in
// every scene) with band codes from this step's sort. A recording tape keeps
// the per-point passes (its hooks keep each step's pair lists).
static bool cells_selected(const fl_system *s) {
    return s->passes == FL_PASSES_CELL_TASKS || (s->passes == FL_PASSES_AUTO && s->auto_cells);
}

static bool use_cell_passes(const fl_system *s, bool taped) {
    return cells_selected(s) && s->D.prune && s->codes_valid && !taped && s->n > 0;
}

// FL_PASSES_AUTO: measured on GB300 (4M-point wave tank, 10-step runs as it
// clumps, the largest cell read after each run), the cell tasks take 1.19x
// the per-point step time by a largest cell of 489, 1.04x at 581, 0.91x at
// 691 and 0.75-0.86x from 789 to 14,935 points (1.69x at the start, 61).
// The cells grow during a run, so the switch sits a little below where the
// run-end figures cross. Every step's sort records the
// largest in-range cell above 128 points and sends it to page-locked host
// memory; the next call reads whatever copy has arrived (a step or two
// old, no wait) and switches with hysteresis. The passes give identical
// results, so when the switch happens changes no result.
constexpr uint32_t kAutoCellsOn = 512, kAutoCellsOff = 384;

static void update_auto(fl_system *s) {
    if (s->passes != FL_PASSES_AUTO || !s->crowd_host) return;
    volatile const uint32_t *h = s->crowd_host;
    if (h[1] != s->auto_epoch) return;   // no count of the current state has arrived yet
    const uint32_t big = h[0];
    if (!s->auto_cells && big >= kAutoCellsOn) s->auto_cells = 1;
    else if (s->auto_cells && big < kAutoCellsOff) s->auto_cells = 0;
}

// The state was replaced (particles set, checkpoint restored): back to the
// per-point passes until a count of the new state arrives (the counts
// carry the state's epoch, so an older count in flight is ignored).
static int reset_auto(fl_system *s) {
    s->auto_cells = 0;
    s->auto_epoch++;
    return fl_launch_set_word(s, s->crowd_epoch, s->auto_epoch);
}

// After the sort: the count and the epoch go to the host on the side stream,
// off the step's critical path; join_crowd makes the step's end wait for
// them (the next step's memset clears the count).
static int send_crowd(fl_system *s) {
    if (s->passes != FL_PASSES_AUTO || !s->crowd_host) return FL_OK;
    FL_CUDA_TRY(cudaEventRecord(s->ev_crowd, s->stream));
    FL_CUDA_TRY(cudaStreamWaitEvent(s->side, s->ev_crowd, 0));
    FL_CUDA_TRY(cudaMemcpyAsync(s->crowd_host, s->crowd_dev, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->side));
    FL_CUDA_TRY(cudaMemcpyAsync(s->crowd_host + 1, s->crowd_epoch, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                s->side));
    FL_CUDA_TRY(cudaEventRecord(s->ev_crowd_done, s->side));
    return FL_OK;
}

static int join_crowd(fl_system *s) {
    if (s->passes != FL_PASSES_AUTO || !s->crowd_host) return FL_OK;
    FL_CUDA_TRY(cudaStreamWaitEvent(s->stream, s->ev_crowd_done, 0));
    return FL_OK;
}

static int run_step(fl_system *s, TimingState *t) {
    // InsertParticles, PrefixSumCells, CountingSortFull, ComputePressure,
    // ComputeForce + Advance (cpp:507-515) as eight launches (the sort is a
    // cell sort of the point indices, one for crowded cells, and a gather).
    const bool taped = fl_tape_recording(s) != 0;
    if (taped) FL_TRY(fl_tape_pre_step(s));
    FL_TRY(record(s, t, 0));
    FL_TRY(clear_grid(s));
    FL_TRY(fl_launch_insert(s, nullptr));
    FL_TRY(record(s, t, 1));
    FL_TRY(fl_launch_scan(s, s->gcells, 0));
    FL_TRY(record(s, t, 2));
    FL_TRY(fl_launch_scatter_index(s));
    FL_TRY(record(s, t, 3));
    FL_TRY(fl_launch_sort_cells(s, 1));
    FL_TRY(send_crowd(s));
    flip(s, F_POS); flip(s, F_VEL); flip(s, F_VEVAL); flip(s, F_CLR); flip(s, F_GCELL); flip(s, F_GNDX);
    const bool cells = use_cell_passes(s, taped);
    s->last_step_cells = cells;
    if (!s->capturing) s->passes_steps[cells ? 1 : 0]++;
    if (cells) FL_TRY(fl_launch_make_tasks(s));
    FL_TRY(record(s, t, 4));
    FL_TRY(cells ? fl_launch_density_cells(s) : fl_launch_density(s));
    FL_TRY(record(s, t, 5));
    FL_TRY(cells ? fl_launch_force_cells(s, s->P.dt, nullptr) : fl_launch_force_advance(s, s->P.dt));
    FL_TRY(join_crowd(s));
    flip(s, F_POS); flip(s, F_VEVAL);
    s->codes_valid = 0;
    s->lists_valid = 0;
    FL_TRY(record(s, t, 6));
    s->time_slot ^= 1;
    if (t) t->steps++;
    if (taped) FL_TRY(fl_tape_post_step(s));
    return FL_OK;
}

int fl_step_fused(fl_system *s) { return run_step(s, nullptr); }

int fl_rebuild_grid(fl_system *s) {
    FL_TRY(clear_grid(s));
    FL_TRY(fl_launch_insert(s, nullptr));
    FL_TRY(fl_launch_scan(s, s->gcells, 0));
    FL_TRY(fl_launch_scatter_index(s));
    FL_TRY(fl_launch_sort_cells(s, 2));
    flip(s, F_POS); flip(s, F_VEL); flip(s, F_VEVAL); flip(s, F_CLR); flip(s, F_GCELL); flip(s, F_GNDX);
    s->lists_valid = 0;
    return FL_OK;
}

int fl_recompute_step(fl_system *s) {
    FL_TRY(fl_rebuild_grid(s));
    if (use_cell_passes(s, false)) {   // the cell-task density, writing the same pair lists
        FL_TRY(fl_launch_make_tasks(s));
        FL_TRY(fl_launch_density_cells(s, true));
        return FL_OK;
    }
    FL_TRY(fl_launch_density(s));
    return FL_OK;
}

static TimingState *active_timing(fl_system *s) {
    if (!s->timing) return nullptr;
    auto it = g_timing.find(s);
    if (it == g_timing.end()) return nullptr;
    TimingState *t = it->second;
    if (t->steps >= 4096) return nullptr;
    const size_t need = (size_t)(t->steps + 1) * 7;
    while (t->events.size() < need) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        t->events.push_back(e);
    }
    return t;
}

static int begin_run(fl_system *s) {
    if (!s->time_host_valid) return FL_OK;
    // host time is authoritative: publish it to the slot the next step reads
    // (as a kernel argument: a copy from pageable host memory could make the
    // host wait for the stream)
    return fl_launch_set_time(s, s->time_slot, s->time);
}

extern "C" int fl_run(fl_system *s) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_run: null system");
    update_auto(s);
    FL_TRY(begin_run(s));
    FL_TRY(run_step(s, active_timing(s)));
    if (s->time_host_valid) s->time += s->P.dt;   // AdvanceTime (cpp:529), same float add
    s->have_insert = 0;
    s->have_offsets = 1;
    s->have_grid = 1;
    return FL_OK;
}

// The step of fl_run_from_host: run_step with the velocities, evaluated
// velocities and colours gathered late, from the staging the side stream
// fills (ev_late), just before the force pass, their first reader (the
// density pass reads only positions; the evaluated-velocity half of its
// pair records is completed by the late gather).
static int run_step_late(fl_system *s, const float *vel3, const float *veval3, const uint32_t *clr,
                         float *pos_out) {
    FL_TRY(clear_grid(s));
    FL_TRY(fl_launch_insert(s, nullptr));
    FL_TRY(fl_launch_scan(s, s->gcells, 0));
    FL_TRY(fl_launch_scatter_index(s));
    FL_TRY(fl_launch_sort_cells(s, 1, true));
    FL_TRY(send_crowd(s));
    flip(s, F_POS); flip(s, F_VEL); flip(s, F_VEVAL); flip(s, F_CLR); flip(s, F_GCELL); flip(s, F_GNDX);
    const bool cells = use_cell_passes(s, false);
    s->last_step_cells = cells;
    s->passes_steps[cells ? 1 : 0]++;
    if (cells) FL_TRY(fl_launch_make_tasks(s));
    FL_TRY(cells ? fl_launch_density_cells(s) : fl_launch_density(s));
    FL_CUDA_TRY(cudaStreamWaitEvent(s->stream, s->ev_late, 0));
    FL_TRY(fl_launch_gather_late(s, vel3, veval3, clr));
    if (cells) {
        // the force pass also writes the new positions into the caller's
        // page-locked array as it goes (no separate readback)
        FL_TRY(fl_launch_force_cells(s, s->P.dt, pos_out ? (float *)mapped_device_ptr(pos_out) : nullptr));
    } else {
        // the force pass writes the new positions into the caller's
        // page-locked array as it goes (no separate readback)
        FL_TRY(fl_launch_force_advance(s, s->P.dt, 0, -1, pos_out ? (float *)mapped_device_ptr(pos_out) : nullptr));
    }
    FL_TRY(join_crowd(s));
    flip(s, F_POS); flip(s, F_VEVAL);
    s->codes_valid = 0;
    s->lists_valid = 0;
    s->time_slot ^= 1;
    return FL_OK;
}

static int ensure_side(fl_system *s) {
    if (!s->side) FL_CUDA_TRY(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));   // the input copies
    if (!s->ev_early) FL_CUDA_TRY(cudaEventCreateWithFlags(&s->ev_early, cudaEventDisableTiming));
    if (!s->ev_late) FL_CUDA_TRY(cudaEventCreateWithFlags(&s->ev_late, cudaEventDisableTiming));
    if (!s->ev_crowd) FL_CUDA_TRY(cudaEventCreateWithFlags(&s->ev_crowd, cudaEventDisableTiming));
    if (!s->ev_crowd_done) FL_CUDA_TRY(cudaEventCreateWithFlags(&s->ev_crowd_done, cudaEventDisableTiming));
    for (int k = 0; k < 2; k++)
        if (!s->ev_auto[k]) FL_CUDA_TRY(cudaEventCreateWithFlags(&s->ev_auto[k], cudaEventDisableTiming));
    return FL_OK;
}

// TransferToCUDA + Run (fluids4.0/fluid_system.cpp:2312-2321, 506-524) in one
// call, for a state kept in host memory between steps. With the point fields
// in page-locked memory, the positions are read over the host link first;
// velocities, evaluated velocities and colours, first needed by the force
// pass, follow on a copy engine (side stream) while insert, sort and density
// run, and k_gather_late puts them in sorted order; the force pass writes
// the new positions into pos_out itself as it computes them. Results equal
// fl_set_particles followed by fl_run, bit for bit; other host memory, a
// batched system, a recording tape or phase timing take that path.
extern "C" int fl_run_from_host(fl_system *s, int n, const float *pos, const float *vel, const float *veval,
                                const uint32_t *clr, float *pos_out) {
    if (!s || !pos) return fl_fail(FL_ERR_ARG, "fl_run_from_host: null system or pos");
    if (n < 0) return fl_fail(FL_ERR_ARG, "fl_run_from_host: n < 0");
    if (n > s->max_points)
        return fl_fail(FL_ERR_CAPACITY, "fl_run_from_host: %d points exceed capacity %d", n, s->max_points);
    const void *mpos = mapped_device_ptr(pos);
    const void *mvev = veval ? mapped_device_ptr(veval) : nullptr;
    const bool pinned = mpos && (!veval || mvev) && (!vel || mapped_device_ptr(vel)) &&
                        (!clr || mapped_device_ptr(clr)) && (!pos_out || mapped_device_ptr(pos_out));
    if (n == 0 || !pinned || s->batched || s->timing || fl_tape_recording(s)) {
        FL_TRY(fl_set_particles(s, n, pos, vel, veval, nullptr, nullptr, clr));
        FL_TRY(fl_run(s));
        if (pos_out) FL_TRY(fl_get_buffer(s, FL_FPOS, pos_out, 12 * (size_t)n));
        FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
        return FL_OK;
    }
    destroy_graph(s);
    update_auto(s);
    FL_TRY(ensure_side(s));
    const size_t n3 = 12 * (size_t)n;
    FL_TRY(fl_ensure_stage(s, 2 * n3 + 4 * (size_t)n));
    s->n = n;
    // early: positions over the link; force and density cleared
    // (fl_set_particles with those absent)
    const float *msrc[1] = {(const float *)mpos};
    float4 *mdst[1] = {s->f[F_POS].cur<float4>()};
    FL_TRY(fl_launch_unpack3_set(s, 1, msrc, mdst, n));
    FL_CUDA_TRY(cudaMemsetAsync(s->f[F_FORCE].cur<float4>(), 0, 16 * (size_t)n, s->stream));
    FL_CUDA_TRY(cudaMemsetAsync(s->f[F_PRESS].cur<float>(), 0, 4 * (size_t)n, s->stream));
    // late: the other fields on the copy engine once the link is free
    float *stage_vel = vel ? (float *)s->stage : nullptr;
    float *stage_vev = veval ? (float *)((char *)s->stage + n3) : nullptr;
    uint32_t *stage_clr = clr ? (uint32_t *)((char *)s->stage + 2 * n3) : nullptr;
    FL_CUDA_TRY(cudaEventRecord(s->ev_early, s->stream));
    FL_CUDA_TRY(cudaStreamWaitEvent(s->side, s->ev_early, 0));
    if (vel) FL_CUDA_TRY(cudaMemcpyAsync(stage_vel, vel, n3, cudaMemcpyHostToDevice, s->side));
    if (veval) FL_CUDA_TRY(cudaMemcpyAsync(stage_vev, veval, n3, cudaMemcpyHostToDevice, s->side));
    if (clr) FL_CUDA_TRY(cudaMemcpyAsync(stage_clr, clr, 4 * (size_t)n, cudaMemcpyHostToDevice, s->side));
    FL_CUDA_TRY(cudaEventRecord(s->ev_late, s->side));
    fl_reset_progress(s);
    FL_TRY(begin_run(s));
    const int r = run_step_late(s, stage_vel, stage_vev, stage_clr, pos_out);
    // the host arrays are the caller's again once the step (and the
    // input copies on the side stream) are done
    cudaError_t e = cudaStreamSynchronize(s->stream);
    const cudaError_t e2 = cudaStreamSynchronize(s->side);
    if (e == cudaSuccess) e = e2;
    FL_TRY(r);
    if (e != cudaSuccess) return fl_fail(FL_ERR_CUDA, "fl_run_from_host: %s", cudaGetErrorString(e));
    if (s->time_host_valid) s->time += s->P.dt;   // AdvanceTime (cpp:529), same float add
    s->have_insert = 0;
    s->have_offsets = 1;
    s->have_grid = 1;
    return FL_OK;
}

// A captured pair of steps returns every field's live copy and the time
// slot to where they started, so the same graph replays any number of times.
static int capture_pair(fl_system *s) {
    destroy_graph(s);
    int live[F_COUNT];
    for (int k = 0; k < F_COUNT; k++) live[k] = s->f[k].live;
    const int slot = s->time_slot;
    cudaGraph_t g = nullptr;
    FL_CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    s->capturing = 1;
    int r = run_step(s, nullptr);
    if (r == FL_OK) r = run_step(s, nullptr);
    s->capturing = 0;
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    for (int k = 0; k < F_COUNT; k++) s->f[k].live = live[k];
    s->time_slot = slot;
    if (r != FL_OK) { if (g) cudaGraphDestroy(g); return r; }
    if (e != cudaSuccess) return fl_fail(FL_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&s->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        s->graph_exec = nullptr;
        return fl_fail(FL_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    }
    s->graph_steps = 2;
    s->graph_cells = (int)cells_selected(s);
    s->graph_ran_cells = s->last_step_cells;
    for (int k = 0; k < F_COUNT; k++) s->graph_live[k] = live[k];
    return FL_OK;
}

static int run_steps_graph(fl_system *s, int nsteps);

// With FL_PASSES_AUTO a long call runs in chunks of kAutoChunk steps, each
// chunk's passes chosen from the counts of the chunk two before it (waited
// for, so one chunk stays queued and the GPU never idles).
constexpr int kAutoChunk = 32;

extern "C" int fl_run_steps(fl_system *s, int nsteps) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_run_steps: null system");
    if (nsteps < 0) return fl_fail(FL_ERR_ARG, "fl_run_steps: nsteps < 0");
    if (s->timing || fl_tape_recording(s)) {   // timed or taped steps stay eager (per-step hooks)
        for (int k = 0; k < nsteps; k++) FL_TRY(fl_run(s));
        return FL_OK;
    }
    if (s->passes != FL_PASSES_AUTO || nsteps <= kAutoChunk) return run_steps_graph(s, nsteps);
    int left = nsteps;
    for (int k = 0; left > 0; k++) {
        const int c = left < kAutoChunk ? left : kAutoChunk;
        if (k >= 2) FL_CUDA_TRY(cudaEventSynchronize(s->ev_auto[k & 1]));
        FL_TRY(run_steps_graph(s, c));
        FL_CUDA_TRY(cudaEventRecord(s->ev_auto[k & 1], s->stream));
        left -= c;
    }
    return FL_OK;
}

static int run_steps_graph(fl_system *s, int nsteps) {
    update_auto(s);
    const int pairs = nsteps / 2;
    if (pairs > 0) {
        bool match = s->graph_exec != nullptr && s->graph_cells == (int)cells_selected(s);
        for (int k = 0; k < F_COUNT && match; k++) match = s->graph_live[k] == s->f[k].live;
        if (!match) FL_TRY(capture_pair(s));
        FL_TRY(begin_run(s));
        for (int p = 0; p < pairs; p++) FL_CUDA_TRY(cudaGraphLaunch(s->graph_exec, s->stream));
        s->passes_steps[s->graph_ran_cells ? 1 : 0] += 2 * (int64_t)pairs;
        s->time_host_valid = 0;   // the device slot now holds the time
        s->have_insert = 0;
        s->have_offsets = 1;
        s->have_grid = 1;
    }
    if (nsteps & 1) {
        if (!s->time_host_valid) {
            // the eager step must read the device time, not a stale host copy
            FL_TRY(run_step(s, nullptr));
            s->have_insert = 0; s->have_offsets = 1; s->have_grid = 1;
        } else {
            FL_TRY(fl_run(s));
        }
    }
    return FL_OK;
}

static int save_slot(fl_system *s, int slot);
static int restore_slot(fl_system *s, int slot);

extern "C" int fl_checkpoint_save(fl_system *s, int slot) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_checkpoint_save: null system");
    if (slot < 0 || slot >= FL_MAX_CHECKPOINTS)
        return fl_fail(FL_ERR_ARG, "fl_checkpoint_save: slot %d outside [0, %d)", slot, FL_MAX_CHECKPOINTS);
    return save_slot(s, slot);
}

static int save_slot(fl_system *s, int slot) {
    const size_t np = (size_t)(s->max_points > 0 ? s->max_points : 1);
    if (!s->ckpt_time[slot]) {
        for (int k = 0; k < F_COUNT; k++) FL_TRY(fl_dalloc(&s->ckpt[slot][k], s->f[k].esz * np));
        FL_TRY(fl_dalloc((void **)&s->ckpt_time[slot], 256));
    }
    for (int k = 0; k < F_COUNT; k++)
        if (s->n > 0)
            FL_CUDA_TRY(cudaMemcpyAsync(s->ckpt[slot][k], s->f[k].cur<void>(), s->f[k].esz * (size_t)s->n,
                                        cudaMemcpyDeviceToDevice, s->stream));
    FL_CUDA_TRY(cudaMemcpyAsync(s->ckpt_time[slot], s->time_dev + s->time_slot, sizeof(float),
                                cudaMemcpyDeviceToDevice, s->stream));
    s->ckpt_n[slot] = s->n;
    s->ckpt_host_time[slot] = s->time;
    s->ckpt_host_valid[slot] = s->time_host_valid;
    return FL_OK;
}

extern "C" int fl_checkpoint_restore(fl_system *s, int slot) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_checkpoint_restore: null system");
    if (slot < 0 || slot >= FL_MAX_CHECKPOINTS || !s->ckpt_time[slot])
        return fl_fail(FL_ERR_ARG, "fl_checkpoint_restore: slot %d holds no checkpoint", slot);
    return restore_slot(s, slot);
}

static int restore_slot(fl_system *s, int slot) {
    s->n = s->ckpt_n[slot];
    FL_TRY(reset_auto(s));
    for (int k = 0; k < F_COUNT; k++)
        if (s->n > 0)
            FL_CUDA_TRY(cudaMemcpyAsync(s->f[k].cur<void>(), s->ckpt[slot][k], s->f[k].esz * (size_t)s->n,
                                        cudaMemcpyDeviceToDevice, s->stream));
    FL_CUDA_TRY(cudaMemcpyAsync(s->time_dev + s->time_slot, s->ckpt_time[slot], sizeof(float),
                                cudaMemcpyDeviceToDevice, s->stream));
    s->time = s->ckpt_host_time[slot];
    s->time_host_valid = s->ckpt_host_valid[slot];
    fl_reset_progress(s);
    return FL_OK;
}

// Launch-shape autotuner: for each knob in turn (density, force and sort
// block sizes, then the cell sort's cells per warp) every candidate is timed
// over `steps` eager steps from the same saved state, the others held at
// their best so far; the state is restored at the end. Shapes change no
// result: each point's work is one thread's (a cell's sort one warp's)
// whatever the block, the thread order within it or the cells per warp.
extern "C" int fl_autotune(fl_system *s, int steps, int *chosen) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_autotune: null system");
    if (steps < 1) return fl_fail(FL_ERR_ARG, "fl_autotune: steps < 1");
    if (fl_tape_recording(s)) return fl_fail(FL_ERR_STATE, "fl_autotune: a tape is recording (fl_tape_end first)");
    if (s->n == 0) return FL_OK;
    const int slot = FL_MAX_CHECKPOINTS;   // the tuner's own checkpoint slot
    FL_TRY(save_slot(s, slot));
    int *knob[4] = {&s->blk_density, &s->blk_force, &s->blk_sort, &s->sort_cells};
    const int cand[4][4] = {{128, 256, 512, 1024}, {32, 64, 128, 0}, {64, 128, 256, 0}, {2, 4, 8, 0}};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    FL_CUDA_TRY(cudaEventCreate(&e0));
    cudaError_t ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) { cudaEventDestroy(e0); return fl_fail(FL_ERR_CUDA, "fl_autotune: event"); }
    // one knob at a time; its candidates timed in three interleaved rounds,
    // each keeping its fastest (shapes differ by a few percent, about the
    // spread of a single short measurement)
    int r = FL_OK;
    for (int k = 0; k < 4 && r == FL_OK; k++) {
        float min_ms[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int round = 0; round < 3 && r == FL_OK; round++) {
            for (int c = 0; c < 4 && cand[k][c] && r == FL_OK; c++) {
                *knob[k] = cand[k][c];
                destroy_graph(s);
                if ((r = restore_slot(s, slot)) != FL_OK) break;
                if (round == 0 && (r = fl_run(s)) != FL_OK) break;   // warm: first launch of this shape
                if (round == 0 && (r = restore_slot(s, slot)) != FL_OK) break;
                cudaEventRecord(e0, s->stream);
                for (int t = 0; t < steps && r == FL_OK; t++) r = fl_run(s);
                cudaEventRecord(e1, s->stream);
                if (cudaEventSynchronize(e1) != cudaSuccess) { r = fl_fail(FL_ERR_CUDA, "fl_autotune: timing"); break; }
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (round == 0 || ms < min_ms[c]) min_ms[c] = ms;
            }
        }
        int best = 0;
        for (int c = 0; c < 4 && cand[k][c]; c++)
            if (best == 0 || min_ms[c] < min_ms[best - 1]) best = c + 1;
        *knob[k] = cand[k][best - 1];
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    destroy_graph(s);
    if (r == FL_OK) r = restore_slot(s, slot);
    if (r == FL_OK && chosen) {
        chosen[0] = s->blk_density; chosen[1] = s->blk_force; chosen[2] = s->blk_sort;
    }
    return r;
}

extern "C" int fl_set_launch_shapes(fl_system *s, const int *shapes) {
    if (!s || !shapes) return fl_fail(FL_ERR_ARG, "fl_set_launch_shapes: null argument");
    const int d = shapes[0], f = shapes[1], so = shapes[2], c = shapes[3];
    auto block_ok = [](int v, int hi) { return v == 0 || (v >= 32 && v <= hi && v % 32 == 0); };
    if (!block_ok(d, 1024) || !block_ok(f, 128) || !block_ok(so, 256) || !(c == 0 || c == 2 || c == 4 || c == 8))
        return fl_fail(FL_ERR_ARG, "fl_set_launch_shapes: density 32..1024, force 32..128, sort 32..256 threads "
                                   "(multiples of 32), 2, 4 or 8 cells per warp (0: default)");
    s->blk_density = d;
    s->blk_force = f;
    s->blk_sort = so;
    s->sort_cells = c;
    destroy_graph(s);   // the captured step holds the old shapes
    return FL_OK;
}

extern "C" int fl_set_neighbour_passes(fl_system *s, int mode) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_set_neighbour_passes: null system");
    if (mode != FL_PASSES_PER_POINT && mode != FL_PASSES_CELL_TASKS && mode != FL_PASSES_POINT_PAIRS &&
        mode != FL_PASSES_AUTO)
        return fl_fail(FL_ERR_ARG, "fl_set_neighbour_passes: mode %d is none of %d, %d, %d, %d", mode,
                       FL_PASSES_PER_POINT, FL_PASSES_CELL_TASKS, FL_PASSES_POINT_PAIRS, FL_PASSES_AUTO);
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->passes = mode;
    s->auto_cells = 0;
    destroy_graph(s);   // the captured step holds the other passes
    return FL_OK;
}

extern "C" int fl_set_reverse_lists(fl_system *s, int mode) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_set_reverse_lists: null system");
    if (mode != FL_REVERSE_AUTO && mode != FL_REVERSE_WALK && mode != FL_REVERSE_TRANSPOSE)
        return fl_fail(FL_ERR_ARG, "fl_set_reverse_lists: mode %d is none of %d, %d, %d", mode, FL_REVERSE_AUTO,
                       FL_REVERSE_WALK, FL_REVERSE_TRANSPOSE);
    s->adj_revmode = mode;
    return FL_OK;
}

extern "C" int fl_neighbour_passes(const fl_system *s) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_neighbour_passes: null system");
    return s->passes;
}

extern "C" int fl_passes_steps(const fl_system *s, int64_t *counts) {
    if (!s || !counts) return fl_fail(FL_ERR_ARG, "fl_passes_steps: null argument");
    counts[0] = s->passes_steps[0];
    counts[1] = s->passes_steps[1];
    return FL_OK;
}

extern "C" int fl_neighbour_passes_in_use(fl_system *s) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_neighbour_passes_in_use: null system");
    if (s->passes != FL_PASSES_AUTO) return s->passes;
    update_auto(s);   // the latest count that has reached the host
    return s->auto_cells ? FL_PASSES_CELL_TASKS : FL_PASSES_PER_POINT;
}

extern "C" int fl_launch_shapes(fl_system *s, int *shapes) {
    if (!s || !shapes) return fl_fail(FL_ERR_ARG, "fl_launch_shapes: null argument");
    shapes[0] = s->blk_density ? s->blk_density : 256;
    shapes[1] = s->blk_force ? s->blk_force : 128;
    shapes[2] = s->blk_sort ? s->blk_sort : 256;
    shapes[3] = s->sort_cells ? s->sort_cells : 4;
    return FL_OK;
}

extern "C" int fl_conservation(fl_system *s, double *out) {
    if (!s || !out) return fl_fail(FL_ERR_ARG, "fl_conservation: null argument");
    const int ns = s->nscenes;
    int most = s->n;
    std::vector<int> base(ns), cnt(ns);
    for (int k = 0; k < ns; k++) {
        base[k] = s->batched ? s->scene_point_base[k] : 0;
        cnt[k] = s->batched ? s->scene_n[k] : s->n;
        if (s->batched && k == 0) most = 0;
        if (s->batched && cnt[k] > most) most = cnt[k];
    }
    const int nchunks = fl_conservation_chunks(most);
    const size_t vals = (size_t)ns * nchunks * FL_CONSERVATION_VALUES;
    const size_t bytes = sizeof(double) * vals + 2 * sizeof(int) * (size_t)ns + 64;
    FL_TRY(fl_ensure_stage(s, bytes));
    double *partial = (double *)s->stage;
    int *dbase = (int *)(partial + vals), *dcnt = dbase + ns;
    FL_CUDA_TRY(cudaMemcpyAsync(dbase, base.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s->stream));
    FL_CUDA_TRY(cudaMemcpyAsync(dcnt, cnt.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s->stream));
    FL_TRY(fl_launch_conservation(s, dbase, dcnt, nchunks, partial));
    std::vector<double> h(vals);
    FL_CUDA_TRY(cudaMemcpyAsync(h.data(), partial, sizeof(double) * vals, cudaMemcpyDeviceToHost, s->stream));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (int k = 0; k < ns; k++)
        for (int v = 0; v < FL_CONSERVATION_VALUES; v++) {
            double t = 0.0;
            for (int c = 0; c < nchunks; c++) t += h[((size_t)k * nchunks + c) * FL_CONSERVATION_VALUES + v];
            out[(size_t)k * FL_CONSERVATION_VALUES + v] = t;
        }
    return FL_OK;
}

extern "C" int fl_device_status(fl_system *s, uint32_t *flags) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_device_status: null system");
    uint32_t v = 0;
    FL_CUDA_TRY(cudaMemcpyAsync(&v, s->dev_err, 4, cudaMemcpyDeviceToHost, s->stream));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (flags) *flags = v;
    return FL_OK;
}

extern "C" int fl_sync(fl_system *s) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_sync: null system");
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    uint32_t v = 0;
    FL_TRY(fl_device_status(s, &v));
    if (v) {
        FL_CUDA_TRY(cudaMemsetAsync(s->dev_err, 0, 4, s->stream));
        FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
        return fl_fail(FL_ERR_DEVICE, "device error word 0x%x%s%s%s", v,
                       (v & FL_DEV_SPIN_TIMEOUT) ? " (scan look-back timed out)" : "",
                       (v & FL_DEV_BAD_CELL) ? " (cell index out of range)" : "",
                       (v & FL_DEV_NONFINITE) ? " (non-finite position)" : "");
    }
    return FL_OK;
}

extern "C" int fl_integrity_check(fl_system *s, int64_t *bad) {
    if (!s || !bad) return fl_fail(FL_ERR_ARG, "fl_integrity_check: null argument");
    if (!s->have_grid) return fl_fail(FL_ERR_STATE, "fl_integrity_check needs a sorted grid");
    FL_TRY(fl_ensure_stage(s, 16));
    FL_CUDA_TRY(cudaMemsetAsync(s->stage, 0, 8, s->stream));
    FL_TRY(fl_launch_integrity(s, (unsigned long long *)s->stage));
    unsigned long long v = 0;
    FL_TRY(readback(s, &v, s->stage, 8));
    *bad = (int64_t)v;
    return FL_OK;
}

extern "C" int fl_set_timing(fl_system *s, int enable) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_set_timing: null system");
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    TimingState *t = detach_timing(s);
    if (t) {
        for (cudaEvent_t e : t->events) cudaEventDestroy(e);
        delete t;
    }
    s->timing = enable ? 1 : 0;
    if (enable) g_timing[s] = new TimingState();
    return FL_OK;
}

extern "C" int fl_time_steps(fl_system *s, int nsteps, int use_graph, int restart_every,
                             int restart_slot, double *ms) {
    if (!s || !ms) return fl_fail(FL_ERR_ARG, "fl_time_steps: null argument");
    if (nsteps < 0) return fl_fail(FL_ERR_ARG, "fl_time_steps: nsteps < 0");
    if (restart_every > 0 && (restart_slot < 0 || restart_slot >= FL_MAX_CHECKPOINTS ||
                              !s->ckpt_time[restart_slot]))
        return fl_fail(FL_ERR_ARG, "fl_time_steps: restart slot %d holds no checkpoint", restart_slot);
    FL_CUDA_TRY(cudaEventRecord(s->ev[0], s->stream));
    for (int done = 0; done < nsteps;) {
        const int chunk = restart_every > 0 ? (nsteps - done < restart_every ? nsteps - done : restart_every)
                                            : nsteps - done;
        if (restart_every > 0) FL_TRY(fl_checkpoint_restore(s, restart_slot));
        if (use_graph) {
            FL_TRY(fl_run_steps(s, chunk));
        } else {
            for (int k = 0; k < chunk; k++) FL_TRY(fl_run(s));
        }
        done += chunk;
    }
    FL_CUDA_TRY(cudaEventRecord(s->ev[1], s->stream));
    FL_CUDA_TRY(cudaEventSynchronize(s->ev[1]));
    float v = 0.0f;
    FL_CUDA_TRY(cudaEventElapsedTime(&v, s->ev[0], s->ev[1]));
    *ms = v;
    return FL_OK;
}

extern "C" int fl_get_phase_times(fl_system *s, double ms[8], int *steps) {
    if (!s || !ms) return fl_fail(FL_ERR_ARG, "fl_get_phase_times: null argument");
    for (int k = 0; k < 8; k++) ms[k] = 0.0;
    if (steps) *steps = 0;
    auto it = g_timing.find(s);
    if (it == g_timing.end()) return FL_OK;
    TimingState *t = it->second;
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (int st = 0; st < t->steps; st++)
        for (int k = 0; k < 6; k++) {
            float v = 0.0f;
            FL_CUDA_TRY(cudaEventElapsedTime(&v, t->events[(size_t)st * 7 + k],
                                             t->events[(size_t)st * 7 + k + 1]));
            ms[k] += v;
        }
    if (t->steps > 0)
        for (int k = 0; k < 6; k++) ms[k] /= t->steps;
    if (steps) *steps = t->steps;
    return FL_OK;
}
