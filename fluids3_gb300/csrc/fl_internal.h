// Internal declarations shared by the host runtime and the kernels.
#pragma once

#include <stdint.h>
#include <cuda_runtime.h>

#include "../../include/fluids_gb300.h"

// Record a failure message for fl_last_error() and return `code`.
int fl_fail(int code, const char *fmt, ...);

#define FL_CUDA_TRY(expr)                                                       \
    do {                                                                        \
        cudaError_t _e = (expr);                                                \
        if (_e != cudaSuccess)                                                  \
            return fl_fail(FL_ERR_CUDA, "%s: %s (%s:%d)", #expr,                \
                           cudaGetErrorString(_e), __FILE__, __LINE__);         \
    } while (0)

#define FL_TRY(expr)                                                            \
    do {                                                                        \
        int _r = (expr);                                                        \
        if (_r != FL_OK) return _r;                                             \
    } while (0)

// ---------------------------------------------------------------------------
// Kernel-side parameter block, passed by value (__grid_constant__) to every
// launch: the FParams fields the step reads (fluids4.0/fluid.h:155-192).
struct DevParams {
    float3 gridMin, gridDelta;
    int3 gridRes, gridScanMax;
    int gridSrch, gridAdjCnt;
    int ncells;          // C; cell index C is the bin for out-of-range points
    int nadj;            // (resZ + 1) * resX + 1: corner offset of the search block
    float rd2, d2, pmass, poly6kern;
    float psmoothradius, prest_dens, pintstiff, sim_scale, spikykern, vterm;
    float lapkern;       // viscosity Laplacian constant (vterm = lapkern * visc); the adjoint's visc partial
    float pradius, bound_slope, bound_stiff, bound_damp, bound_friction;
    float bound_wall_force, bound_wall_freq;
    float3 bound_min, bound_max, gravity;
    float AL, AL2, VL, VL2;
    // search-block pruning (gridSrch == 2 only): world-unit cell edge per
    // axis and the band width (h plus a safety margin) within which a point
    // can reach into the lower neighbour cell
    float3 cellw;
    float band;
    int prune;           // 1 when gridSrch == 2
    int upwords;         // words per axis row of the upper-band slot flags
    int hcap;            // pair-list capacity per point
    int cell_base;       // first internal cell entry of this scene (0 for a single scene)
    int adj[216];
};

void fl_make_dev_params(const fl_params &p, DevParams *d);

// Scene table of a batched system: per-scene parameter blocks and the
// scene of every point slot and internal cell entry. `params` is null for a
// single-scene system, whose kernels take their parameters by value.
struct SceneTab {
    const DevParams *params;
    const uint16_t *point_scene;
    const uint16_t *cell_scene;
};

// One particle field held twice in HBM. Gathers (the counting sort) and the
// fused force+advance pass write the copy that is not live and then flip,
// so no kernel overwrites a value that another thread may still read.
struct Field {
    void *p[2];
    int live;
    size_t esz;          // bytes per element in HBM
    template <class T> T *cur() const { return (T *)p[live]; }
    template <class T> T *nxt() const { return (T *)p[live ^ 1]; }
};

enum { F_POS, F_VEL, F_VEVAL, F_FORCE, F_PRESS, F_CLR, F_GCELL, F_GNDX, F_COUNT };

struct fl_system {
    int device;
    cudaStream_t stream;
    fl_params P;
    DevParams D;
    int max_points;
    int n;                 // live point count
    int ncells;            // C (reference-layout cells; summed over scenes when batched)
    int gcells;            // internal cell entries: C + 1 per scene (the extra one: out-of-range bin)
    float time;

    // batched systems: nscenes > 1 or batched != 0
    int batched;
    int nscenes;
    DevParams *d_scenes;   // device table, one block per scene
    uint16_t *point_scene, *cell_scene;
    int *scene_point_base, *scene_n, *scene_cell_base, *scene_ncells;   // host copies
    fl_params *scene_params;   // host copy of every scene's parameter block

    Field f[F_COUNT];      // pos/vel/veval/force: float4; press: float; clr/gcell/gndx: uint

    // insert / sort scratch, indexed by pre-sort point index unless noted
    uint32_t *cell_pre;    // cell of point i (C when out of range)
    uint32_t *rank_tmp;    // arrival rank from the counting atomics; reused by the dense-cell path
    uint32_t *src;         // sorted slot -> pre-sort index

    // grid: C + 1 entries (entry C is the out-of-range bin), padded to whole
    // scan tiles. One allocation holds [cnt | scan ticket | scan descriptors]
    // so a single memset clears all three at the start of a step.
    uint32_t *cnt;
    uint32_t *off;
    size_t grid_pad;
    uint32_t *scan_ticket; // dynamic tile counter (256 B slot)
    uint64_t *scan_status; // decoupled look-back tile descriptors
    int scan_tiles;
    uint32_t scan_epoch;

    uint32_t *dev_err;     // device error word (FL_DEV_*)

    // per sorted slot and axis: is the point within `band` of its cell's
    // upper face (rows 0-2 of upwords 32-bit words); valid together with the
    // band codes in pos.w while codes_valid is set. Rows 3-5: the same for
    // the lower face, filled only by the adjoint's rebuilt steps (sort mode 2)
    uint32_t *upbits;
    int codes_valid;

    // pairs found by the density pass, reused by the force pass while the
    // positions and grid are unchanged (lists_valid)
    uint32_t *big_cells;   // cell entries above 128 points, listed by the cell sort (fl_big_cells_cap)
    uint32_t *big_count;   // [0] their number, [1] k_sort_big's sign-off count (256 B slot, zeroed at creation)
    int num_sms;

    // cell tasks of the fused step's neighbour passes (fl_cells.cu): (first slot, cell entry)
    // per 64 slots of a cell, listed every step; counters in the scan
    // ticket's slot (cleared with the counts)
    uint2 *tasks;
    size_t task_cap;
    uint32_t *task_counters;
    int passes;            // FL_PASSES_*: the neighbour passes of the fused step
    int auto_cells;        // FL_PASSES_AUTO: the cell tasks are in use (hysteresis state)
    int graph_cells;       // the captured step pair runs the cell tasks
    int capturing;         // run_step is being captured into the step-pair graph
    int last_step_cells;   // the last issued (or captured) step took the cell tasks
    int graph_ran_cells;   // the captured step pair takes the cell tasks
    int64_t passes_steps[2]; // fused steps issued with the per-point passes / the cell tasks
    uint32_t *crowd_dev;   // largest in-range cell above 128 points, this step (0: none)
    uint32_t *crowd_epoch; // device: the state's epoch (bumped when the state is replaced)
    uint32_t *crowd_host;  // page-locked [count, epoch], sent after each step's sort
    uint32_t auto_epoch;   // host: the current state's epoch
    int adj_revmode;       // FL_REVERSE_*: how the adjoint finds its reverse pair lists
    int cells_grid[2];     // blocks of the cell-task density and force passes (all resident)

    uint32_t *hitlist;     // ceil(N/32) * hcap * 32 entries
    uint32_t *hitcnt;      // per point
    // per slot, written with the lists: (pos.xyz, density), (veval.xyz, 0),
    // so the force pass reads a neighbour's data from one 32-byte sector
    float4 *pairdata;
    int lists_valid;

    // m_Time on the device, double-buffered by step parity so a captured
    // graph replays with the time advancing: step k reads time_dev[k & 1]
    // and writes time_dev[(k + 1) & 1] = time + dt (AdvanceTime, cpp:527-531).
    float *time_dev;
    int time_slot;
    int time_host_valid;   // host `time` mirrors the device value

    void *stage;           // device staging for fluid.h-layout import/export
    size_t stage_bytes;

    // phase-API progress, in the order Run issues the phases. have_grid: the
    // sorted copies, counts and offsets come from one completed sort.
    int have_insert, have_offsets, have_grid;
    int offsets_inclusive;

    // threads per block of the sort, density and force passes (0: the
    // compiled default); set by fl_autotune, results do not depend on them
    int blk_sort, blk_density, blk_force;
    int sort_cells;        // cell entries per warp of the cell sort (0: the compiled default)

    // graph replay for fl_run_steps
    cudaGraphExec_t graph_exec;
    int graph_steps;
    int graph_live[F_COUNT];

    // checkpoints: per slot, one copy of every field's live buffer + time
    // one more slot than the caller's: the autotuner's own
    void *ckpt[FL_MAX_CHECKPOINTS + 1][F_COUNT];
    float *ckpt_time[FL_MAX_CHECKPOINTS + 1];
    int ckpt_n[FL_MAX_CHECKPOINTS + 1];
    float ckpt_host_time[FL_MAX_CHECKPOINTS + 1];
    int ckpt_host_valid[FL_MAX_CHECKPOINTS + 1];

    // adjoint tape (fl_tape.cpp), null until fl_tape_begin
    struct fl_tape *tape;

    // fl_run_from_host: the copy-engine stream that brings velocities and
    // colours in while the step's first kernels run, and its two events
    // (created on first use)
    cudaStream_t side;
    cudaEvent_t ev_early, ev_late, ev_crowd, ev_crowd_done, ev_auto[2];

    // per-phase event timing (PERF_PUSH/PERF_POP of Run, cpp:507-515)
    int timing;
    cudaEvent_t ev[8];
    double phase_ms[8];
    int phase_runs;
};

inline SceneTab fl_scene_tab(const fl_system *s) {
    SceneTab t;
    t.params = s->batched ? s->d_scenes : nullptr;
    t.point_scene = s->point_scene;
    t.cell_scene = s->cell_scene;
    return t;
}

#define FL_LAUNCH_CHECK(name)                                                   \
    do {                                                                        \
        cudaError_t _e = cudaGetLastError();                                    \
        if (_e != cudaSuccess)                                                  \
            return fl_fail(FL_ERR_CUDA, "%s launch: %s", name, cudaGetErrorString(_e)); \
    } while (0)

// ---- host runtime entry points shared with the adjoint (fl_api.cpp) -------
int fl_dalloc(void **p, size_t bytes);
int fl_ensure_stage(fl_system *s, size_t bytes);
void fl_reset_progress(fl_system *s);
// One fused Run step reading the device time slot (no timing events).
int fl_step_fused(fl_system *s);
// The forward state of one step up to its densities: insert, scan, sort
// (gathering pos/vel/veval/clr, publishing both band-flag sets) and density
// (with pair lists) into the live copies.
int fl_recompute_step(fl_system *s);
// The same without the density pass: insert, scan, sort (mode 2) only.
int fl_rebuild_grid(fl_system *s);

// ---- adjoint tape (fl_tape.cpp) --------------------------------------------
int fl_tape_recording(const fl_system *s);
int fl_tape_pre_step(fl_system *s);
int fl_tape_post_step(fl_system *s);
// A state change outside Run (new particles, parameters, a restore, a phase
// call): the tape no longer describes the steps that led to the state.
void fl_tape_touch(fl_system *s);
void fl_tape_free(fl_system *s);

// ---- launch wrappers (fl_kernels.cu, fl_scan.cu, fl_adjoint.cu) ------------
int fl_launch_adj_advance(fl_system *s, const float *time_ptr, const float4 *force, const float4 *xo_b,
                          const float4 *vo_b, const float4 *eo_b, float4 *xa, float4 *ea, float4 *fb, float4 *v_out,
                          float2 *rr);
// crowd / crowd_count: the list of points whose pair lists overflowed
// (capacity n; the count starts at zero); revlong / revlong_count: the
// points whose transposed reverse lists are walked again (capacity n; the
// count starts at zero)
int fl_launch_adj_force(fl_system *s, const float2 *rr, const float4 *fb, float4 *xa, const float4 *ea, float *rb,
                        float4 *pc, float4 *e_out, uint32_t *revlist, uint32_t *revcnt, uint32_t *crowd,
                        uint32_t *crowd_count, uint32_t *revlong, uint32_t *revlong_count);
int fl_launch_adj_density(fl_system *s, const uint32_t *revlist, const uint32_t *revcnt, const float *rb,
                          const float4 *xa, float4 *x_out, uint32_t *crowd, uint32_t *crowd_count);
int fl_param_chunks(int max_scene_points);
// acc += partial sums x 2^gexp (gexp null: x 1)
int fl_launch_param_reduce(fl_system *s, const float4 *pc, const int *sbase, const int *sn, int nchunks,
                           double *partial, const int *gexp, double *acc);
// per scene: cotangents above 2^40 scaled by 2^-k, gexp += k (gmax zero on entry, left zero)
int fl_launch_adj_rescale(fl_system *s, float4 *gx, float4 *gv, float4 *ge, uint32_t *gmax, int *gexp);
// the cotangents times 2^gexp of their scene
int fl_launch_adj_apply_exponent(fl_system *s, float4 *gx, float4 *gv, float4 *ge, const int *gexp);
int fl_launch_compose(fl_system *s, int n, const uint32_t *src, const uint32_t *in, uint32_t *out);
// dst[k][0..n) = src[k][0..n) for k < count (<= 3), one kernel pass
int fl_launch_copy3(fl_system *s, int n, int count, const float4 *const *src, float4 *const *dst);
int fl_launch_insert(fl_system *s, uint32_t *gcell_pre_or_null);
int fl_launch_scan(fl_system *s, int count, int clear_status);
int fl_launch_scatter_index(fl_system *s);
// mode 0: rank only (sorted src + canonical gndx into f[F_GNDX].cur, pre-sort order)
// mode 1: sorted src, then a gather of pos/vel/veval/clr/gcell/gndx into the
//         nxt copies with band codes and the upper-band slot flags (rows 0-2)
// mode 2: mode 1 that also writes the lower-band slot flags (upbits rows 3-5)
// late (mode 1, plain systems): the gather moves positions only and leaves
// velocities, evaluated velocities and colours to fl_launch_gather_late
int fl_launch_sort_cells(fl_system *s, int mode, bool late = false);
// velocity, evaluated velocity (packed float3) and colour staging -> the
// sorted live copies through src (null source: zeros), and the evaluated
// velocity half of every pair record; after the density pass
int fl_launch_gather_late(fl_system *s, const float *vel3, const float *veval3, const uint32_t *clr);
// one-time kernel attributes (shared memory of the crowded-cell sort)
int fl_kernels_init(fl_system *s);
// entries of the crowded-cell list for max_points points (cells above 128)
size_t fl_big_cells_cap(int max_points);
// gather every field cur -> nxt through src (phase-API counting sort)
int fl_launch_gather_all(fl_system *s);
int fl_launch_band_codes(fl_system *s);
int fl_launch_density(fl_system *s);
int fl_launch_force(fl_system *s);
// slots [begin, end) (end < 0: n); both whole blocks of fl_force_block(s)
// threads, except end == n
int fl_launch_force_advance(fl_system *s, float dt, int begin = 0, int end = -1, float *host_pos = nullptr);
int fl_force_block(const fl_system *s);
int fl_launch_advance(fl_system *s, float time, float dt, float ss);
int fl_launch_pack3(fl_system *s, const float4 *src, float *dst, int n, cudaStream_t stream = nullptr);
int fl_launch_set_time(fl_system *s, int slot, float value);
int fl_launch_set_word(fl_system *s, uint32_t *word, uint32_t value);
int fl_launch_unpack3(fl_system *s, const float *src, float4 *dst, int n);
// up to 4 float3 -> float4 fields in one pass (src[k] may be host-mapped)
int fl_launch_unpack3_set(fl_system *s, int count, const float *const *src, float4 *const *dst, int n);
int fl_launch_grid_identity(fl_system *s, uint32_t *dst, int n, const uint32_t *gcell);
int fl_launch_gcell_ref(fl_system *s, uint32_t *dst);
int fl_launch_integrity(fl_system *s, unsigned long long *bad_dev);
int fl_conservation_chunks(int max_scene_points);
int fl_launch_conservation(fl_system *s, const int *sbase, const int *sn, int nchunks, double *partial);
int fl_launch_sample_volume(fl_system *s, const int res[3], const float bmin[3], const float bmax[3],
                            float scalar, float gausskern, float h2, float *out);
// cell-task passes of the fused step (fl_cells.cu)
size_t fl_task_cap(int max_points, int gcells);
int fl_cells_init(fl_system *s);   // after num_sms and batched are set
int fl_launch_make_tasks(fl_system *s);
// densities and pair records, plus the force pass's hit masks or (lists) the
// per-point pair lists and counts in the per-point pass's layout
int fl_launch_density_cells(fl_system *s, bool lists = false);
int fl_launch_density_pairs(fl_system *s);
int fl_pairs_init();   // once per process is enough; outside any stream capture
// force + advance over the tasks from the hit masks; host_pos (a
// device-usable pointer to page-locked host memory, or null) also receives
// the new positions as float x3
int fl_launch_force_cells(fl_system *s, float dt, float *host_pos);
size_t fl_scan_tile();
size_t fl_upbits_bytes(const fl_system *s);
size_t fl_scan_scratch_bytes(int ntiles);
