/*
 * ref_wrap.cpp -- TEST INFRASTRUCTURE ONLY (oracle tier 1: the reference's
 * own kernel arithmetic, run on the host).
 *
 * Compiles the reference kernel source fluids4.0/fluid_kernels.cu unchanged
 * (force-including ref_shim.h) and runs each __global__ body once per
 * particle in index order. Serial atomics make gndx the canonical
 * within-cell order. The host orchestration mirrors FluidSystem::Run,
 * RUN_GPU_FULL (fluids4.0/fluid_system.cpp:506-524): memset of the grid
 * counts and offsets (cpp:2336-2337), insert, an exclusive scan (the serial
 * scan of the reference's CPU_SUMS branch, cpp:2356-2370), the copy into the
 * temp buffers (cpp:2458-2465), counting sort, pressure, force, advance.
 *
 * Built by oracle/build_ref.sh into oracle/_ref/; only tests/, bench.py's
 * reference arm and the smoke check load it, never the product.
 */
#include <stddef.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>

#include "fluid_kernels.cu"          /* the reference source, found via -I */
#include "../include/fluids_gb300.h"

thread_local uint3 blockIdx;
thread_local uint3 blockDim;
thread_local uint3 threadIdx;

static inline void set_thread(int i) {
    blockDim = make_uint3(1, 1, 1);
    threadIdx = make_uint3(0, 0, 0);
    blockIdx = make_uint3((unsigned)i, 0, 0);
}

static FBufs g_tmp_host;   /* host storage behind ftemp */
static int g_ncells = 0;

extern "C" {

/* Fill the kernels' __constant__ parameter block from a derived fl_params. */
int ref_set_params(const fl_params *p) {
    memset(&fparam, 0, sizeof(fparam));
    fparam.sim_scale = p->sim_scale;
    fparam.pmass = p->pmass;
    fparam.prest_dens = p->prest_dens;
    fparam.pintstiff = p->pintstiff;
    fparam.pradius = p->pradius;
    fparam.psmoothradius = p->psmoothradius;
    fparam.r2 = p->r2;
    fparam.pvisc = p->pvisc;
    fparam.AL = p->AL; fparam.AL2 = p->AL2;
    fparam.VL = p->VL; fparam.VL2 = p->VL2;
    fparam.d2 = p->d2; fparam.rd2 = p->rd2; fparam.vterm = p->vterm;
    fparam.poly6kern = p->poly6kern; fparam.spikykern = p->spikykern; fparam.lapkern = p->lapkern;
    fparam.grid_size = p->grid_size; fparam.grid_density = p->grid_density;
    fparam.gridSize = make_float3(p->gridSize[0], p->gridSize[1], p->gridSize[2]);
    fparam.gridDelta = make_float3(p->gridDelta[0], p->gridDelta[1], p->gridDelta[2]);
    fparam.gridMin = make_float3(p->gridMin[0], p->gridMin[1], p->gridMin[2]);
    fparam.gridMax = make_float3(p->gridMax[0], p->gridMax[1], p->gridMax[2]);
    fparam.gridRes = make_int3(p->gridRes[0], p->gridRes[1], p->gridRes[2]);
    fparam.gridScanMax = make_int3(p->gridScanMax[0], p->gridScanMax[1], p->gridScanMax[2]);
    fparam.gridSrch = p->gridSrch;
    fparam.gridTotal = p->gridTotal;
    fparam.gridAdjCnt = p->gridAdjCnt;
    if (p->gridAdjCnt > 64) return -1;   /* FParams.gridAdj holds 64 entries */
    for (int c = 0; c < p->gridAdjCnt; c++) fparam.gridAdj[c] = p->gridAdj[c];
    fparam.bound_slope = p->bound_slope; fparam.bound_stiff = p->bound_stiff;
    fparam.bound_friction = p->bound_friction; fparam.bound_damp = p->bound_damp;
    fparam.bound_wall_force = p->bound_wall_force; fparam.bound_wall_freq = p->bound_wall_freq;
    fparam.bound_min = make_float3(p->bound_min[0], p->bound_min[1], p->bound_min[2]);
    fparam.bound_max = make_float3(p->bound_max[0], p->bound_max[1], p->bound_max[2]);
    fparam.gravity = make_float3(p->gravity[0], p->gravity[1], p->gravity[2]);
    g_ncells = p->gridTotal;
    return 0;
}

/* Point buffer `id` of the kernels' fbuf table at caller-owned host memory. */
void ref_bind(int id, void *host) { fbuf.mgpu[id] = (char *)host; }

static void ensure_temp(int n) {
    static int cap = 0;
    if (n <= cap) return;
    const int ids[8] = {FPOS, FVEL, FVEVAL, FFORCE, FPRESS, FCLR, FGCELL, FGNDX};
    const size_t esz[8] = {12, 12, 12, 12, 4, 4, 4, 4};
    for (int k = 0; k < 8; k++) {
        free(g_tmp_host.mgpu[ids[k]]);
        g_tmp_host.mgpu[ids[k]] = (char *)malloc(esz[k] * (size_t)n);
        ftemp.mgpu[ids[k]] = g_tmp_host.mgpu[ids[k]];
    }
    cap = n;
}

void ref_insert(int n) {
    memset(fbuf.mgpu[FGRIDCNT], 0, (size_t)g_ncells * 4);
    memset(fbuf.mgpu[FGRIDOFF], 0, (size_t)g_ncells * 4);
    for (int i = 0; i < n; i++) { set_thread(i); insertParticles(n); }
}

void ref_prefix_sum(int zero_offsets) {
    const uint *cnt = (const uint *)fbuf.mgpu[FGRIDCNT];
    uint *off = (uint *)fbuf.mgpu[FGRIDOFF];
    uint sum = 0;
    for (int c = 0; c < g_ncells; c++) {
        if (zero_offsets) { off[c] = sum; sum += cnt[c]; }
        else { sum += cnt[c]; off[c] = sum; }
    }
}

void ref_counting_sort(int n) {
    ensure_temp(n);
    const int ids[8] = {FPOS, FVEL, FVEVAL, FFORCE, FPRESS, FCLR, FGCELL, FGNDX};
    const size_t esz[8] = {12, 12, 12, 12, 4, 4, 4, 4};
    for (int k = 0; k < 8; k++) memcpy(ftemp.mgpu[ids[k]], fbuf.mgpu[ids[k]], esz[k] * (size_t)n);
    for (int i = 0; i < n; i++) { set_thread(i); countingSortFull(n); }
}

void ref_compute_pressure(int n, int threads) {
    #pragma omp parallel for schedule(dynamic, 1024) num_threads(threads) if (threads > 1)
    for (int i = 0; i < n; i++) { set_thread(i); computePressure(n); }
}

void ref_compute_force(int n, int threads) {
    #pragma omp parallel for schedule(dynamic, 1024) num_threads(threads) if (threads > 1)
    for (int i = 0; i < n; i++) { set_thread(i); computeForce(n); }
}

void ref_advance(float time, float dt, float ss, int n, int threads) {
    #pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
    for (int i = 0; i < n; i++) { set_thread(i); advanceParticles(time, dt, ss, n); }
}

/* sampleParticles (fluid_kernels.cu:263-308) once per voxel, blockIdx = the
 * voxel (blockDim 1). gausskern as UpdateParamsCUDA derives it (cpp:2302).
 * The kernel stores an out-of-range voxel at another index than an
 * in-range one; callers keep the box inside the scan range. */
void ref_sample_particles(float *brick, int rx, int ry, int rz, const float *bmin, const float *bmax, int n,
                          float scalar) {
    const float sr = fparam.psmoothradius;
    fparam.gausskern = 1.0f / pow(3.141592f * 2.0f * sr * sr, 3.0f / 2.0f);
    const uint3 res = make_uint3((unsigned)rx, (unsigned)ry, (unsigned)rz);
    const float3 lo = make_float3(bmin[0], bmin[1], bmin[2]);
    const float3 hi = make_float3(bmax[0], bmax[1], bmax[2]);
    blockDim = make_uint3(1, 1, 1);
    threadIdx = make_uint3(0, 0, 0);
    for (int z = 0; z < rz; z++)
        for (int y = 0; y < ry; y++)
            for (int x = 0; x < rx; x++) {
                blockIdx = make_uint3((unsigned)x, (unsigned)y, (unsigned)z);
                sampleParticles(brick, res, lo, hi, n, scalar);
            }
}

/* `steps` RUN_GPU_FULL steps starting at *time; *time advances by dt each step. */
void ref_run(int n, int steps, float *time, float dt, int threads) {
    for (int s = 0; s < steps; s++) {
        ref_insert(n);
        ref_prefix_sum(1);
        ref_counting_sort(n);
        ref_compute_pressure(n, threads);
        ref_compute_force(n, threads);
        ref_advance(*time, dt, fparam.sim_scale, n, threads);
        *time += dt;
    }
}

int ref_sizeof_fparams(void) { return (int)sizeof(FParams); }

/* Byte offset of FParams field `name` as the reference header lays it out
 * (fluids4.0/fluid.h:155-192); "sizeof FParams", "sizeof FBufs" and
 * "FBufs.mgpu" give those; -1 for an unknown name. Lets a test check the
 * field-by-field restatement that drives the reference's GPU module. */
long ref_layout(const char *name) {
#define L(f) if (!strcmp(name, #f)) return (long)offsetof(FParams, f);
    L(mode) L(example) L(sim_scale) L(capture) L(numThreads) L(numBlocks) L(gridThreads) L(gridBlocks)
    L(szPnts) L(szHash) L(szGrid) L(stride) L(pnum) L(chk) L(pdist) L(pmass) L(prest_dens) L(pintstiff)
    L(pradius) L(psmoothradius) L(pspacing) L(r2) L(pvisc) L(AL) L(AL2) L(VL) L(VL2) L(d2) L(rd2) L(vterm)
    L(poly6kern) L(spikykern) L(lapkern) L(gausskern) L(grid_size) L(grid_density) L(gridSize) L(gridDelta)
    L(gridMin) L(gridMax) L(gridRes) L(gridScanMax) L(gridSrch) L(gridTotal) L(gridAdjCnt) L(gridActive)
    L(gridAdj) L(bound_slope) L(bound_stiff) L(bound_friction) L(bound_damp) L(bound_wall_force)
    L(bound_wall_freq) L(bound_min) L(bound_max) L(init_min) L(init_max) L(grav_dir) L(grav_pos) L(gravity)
    L(grav_amt) L(emit_rate) L(emit_pos) L(emit_ang) L(emit_dang) L(emit_spread) L(brickRes) L(pemit) L(pmem)
#undef L
    if (!strcmp(name, "sizeof FParams")) return (long)sizeof(FParams);
    if (!strcmp(name, "sizeof FBufs")) return (long)sizeof(FBufs);
    if (!strcmp(name, "FBufs.mgpu")) return (long)offsetof(FBufs, mgpu);
    return -1;
}

} /* extern "C" */
