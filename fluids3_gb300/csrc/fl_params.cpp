// Parameter defaults and derivation for the SPH step (host code).
//
// Restates, in the reference's own FP32 operation order, the host functions
// that turn the user-facing inputs into the derived FParams block the
// kernels read (fluids4.0/fluid.h:155-192):
//   SetupDefaultParams   fluids4.0/fluid_system.cpp:1953-2041
//   SetupExampleParams   fluids4.0/fluid_system.cpp:2043-2097 (example 3 box)
//   SetupSpacing         fluids4.0/fluid_system.cpp:2099-2117 (grid part)
//   SetupGrid            fluids4.0/fluid_system.cpp:793-846
//   FluidSetupCUDA       fluids4.0/fluid_system.cpp:2249-2287
//   UpdateParamsCUDA     fluids4.0/fluid_system.cpp:2289-2310
// Rounding matters: e.g. a 0.02 m cell at sim_scale 0.004 is 4.9999995
// world units in FP32, so an 80-unit span needs 17 cells, not 16. This file
// is compiled with -ffp-contract=off so no expression is fused.
#include <math.h>
#include <string.h>

#include "fl_internal.h"

extern "C" int fl_params_default(fl_params *p) {
    if (!p) return fl_fail(FL_ERR_ARG, "fl_params_default: null params");
    memset(p, 0, sizeof(*p));
    p->dt = 0.003f;
    p->sim_scale = 0.004f;
    p->pvisc = 0.35f;
    p->prest_dens = 400.0f;
    p->pmass = 0.00020543f;
    p->pradius = 0.015f;
    p->pdist = 0.0059f;
    p->psmoothradius = 0.015f;
    p->pintstiff = 1.5f;
    p->bound_stiff = 50000.0f;
    p->bound_damp = 150.0f;
    p->AL = 150.0f;
    p->VL = 50.0f;
    p->bound_slope = 0.0f;
    p->bound_friction = 0.0f;
    p->bound_wall_force = 0.0f;
    p->bound_wall_freq = 0.0f;
    p->grav_amt = 1.0f;
    p->grav_dir[0] = 0.0f; p->grav_dir[1] = -9.8f; p->grav_dir[2] = 0.0f;
    p->grid_density = 2.0f;
    // example 3, "small dam break" (cpp:2081-2088)
    p->bound_min[0] = -40.0f; p->bound_min[1] = 0.0f;  p->bound_min[2] = -40.0f;
    p->bound_max[0] = 40.0f;  p->bound_max[1] = 60.0f; p->bound_max[2] = 40.0f;
    return FL_OK;
}

extern "C" int fl_params_derive(fl_params *p) {
    if (!p) return fl_fail(FL_ERR_ARG, "fl_params_derive: null params");
    if (!(p->sim_scale > 0.0f) || !(p->psmoothradius > 0.0f) || !(p->grid_density > 0.0f))
        return fl_fail(FL_ERR_PARAMS, "fl_params_derive: sim_scale, psmoothradius and grid_density must be > 0");

    // SetupSpacing, grid part (cpp:2101, 2114-2116). 1.5 and 2.0 are double
    // literals upstream, so those products are formed in double and rounded.
    p->grid_size = (float)(1.5 * (double)p->psmoothradius / (double)p->grid_density);
    const float border = (float)(2.0 * (double)(p->grid_size / p->sim_scale));
    for (int k = 0; k < 3; k++) {
        p->gridMin[k] = p->bound_min[k] - border;
        p->gridMax[k] = p->bound_max[k] + border;
    }

    // SetupGrid (cpp:793-846)
    const float world_cellsize = p->grid_size / p->sim_scale;
    for (int k = 0; k < 3; k++) {
        const float span = p->gridMax[k] - p->gridMin[k];
        const float cells = ceilf(span / world_cellsize);
        if (!(cells >= 1.0f) || !(cells < 1.0e6f))
            return fl_fail(FL_ERR_PARAMS, "fl_params_derive: grid resolution out of range on axis %d", k);
        p->gridRes[k] = (int)cells;
        p->gridSize[k] = (float)p->gridRes[k] * p->grid_size / p->sim_scale;
    }
    for (int k = 0; k < 3; k++) p->gridDelta[k] = (float)p->gridRes[k] / p->gridSize[k];
    const long long total = (long long)p->gridRes[0] * p->gridRes[1] * p->gridRes[2];
    if (total > (1LL << 30))
        return fl_fail(FL_ERR_PARAMS, "fl_params_derive: %lld cells exceed the 2^30 limit", total);
    p->gridTotal = (int)total;

    int srch = (int)(floorf(2.0f * (p->psmoothradius / p->sim_scale) / world_cellsize) + 1.0f);
    if (srch < 2) srch = 2;
    if (srch > FL_MAX_GRID_SRCH)
        return fl_fail(FL_ERR_PARAMS, "fl_params_derive: neighbour search needs %d cells per axis (> 6)", srch);
    p->gridSrch = srch;
    p->gridAdjCnt = srch * srch * srch;

    // FluidSetupCUDA (cpp:2249-2287): scan limits and the y,z,x-ordered
    // adjacency of the search block.
    for (int k = 0; k < 3; k++) p->gridScanMax[k] = p->gridRes[k] - srch;
    int cell = 0;
    for (int y = 0; y < srch; y++)
        for (int z = 0; z < srch; z++)
            for (int x = 0; x < srch; x++)
                p->gridAdj[cell++] = (y * p->gridRes[2] + z) * p->gridRes[0] + x;
    for (int c = cell; c < 216; c++) p->gridAdj[c] = 0;

    // UpdateParamsCUDA (cpp:2289-2310)
    for (int k = 0; k < 3; k++) p->gravity[k] = p->grav_dir[k] * p->grav_amt;
    p->AL2 = p->AL * p->AL;
    p->VL2 = p->VL * p->VL;
    const float sr = p->psmoothradius;
    p->r2 = sr * sr;
    p->pdist = powf(p->pmass / p->prest_dens, 1 / 3.0f);
    p->poly6kern = 315.0f / (64.0f * 3.141592f * powf(sr, 9.0f));
    p->spikykern = -45.0f / (3.141592f * powf(sr, 6.0f));
    p->lapkern = 45.0f / (3.141592f * powf(sr, 6.0f));
    p->d2 = p->sim_scale * p->sim_scale;
    p->rd2 = p->r2 / p->d2;
    p->vterm = p->lapkern * p->pvisc;
    return FL_OK;
}
