/*
 * fluids_gb300.h -- C ABI of the GB300 (sm_103a) SPH time step.
 *
 * Drop-in for the GPU pathway of the reference's FluidSystem
 * (fluids4.0/fluid_system.h:145-353): the same phases, the same buffer ids
 * and host layouts (fluids4.0/fluid.h:45-70), the same derived parameters
 * (fluids4.0/fluid.h:155-192), behind plain pointers and status codes.
 *
 *   reference (fluids4.0)                          this ABI
 *   -------------------------------------------    ---------------------------
 *   FluidSystem::Initialize + Start (cpp:92-168)   fl_params_default/derive, fl_create
 *   SetupSpacing/SetupGrid/FluidSetupCUDA/
 *     UpdateParamsCUDA (cpp:2099,793,2249,2289)    fl_params_derive, fl_set_params
 *   TransferToCUDA (cpp:2312-2321)                 fl_set_particles
 *   TransferFromCUDA (cpp:2323-2330)               fl_get_buffer
 *   InsertParticlesCUDA (cpp:2334-2350)            fl_insert_particles
 *   PrefixSumCellsCUDA (cpp:2354-2424)             fl_prefix_sum_cells
 *   CountingSortFullCUDA (cpp:2455-2479)           fl_counting_sort_full
 *   ComputePressureCUDA (cpp:2515-2519)            fl_compute_pressure
 *   ComputeForceCUDA (cpp:2521-2525)               fl_compute_force
 *   AdvanceCUDA (cpp:2527-2531)                    fl_advance
 *   Run, case RUN_GPU_FULL (cpp:506-524)           fl_run / fl_run_steps
 *   TransferToCUDA + Run + TransferFromCUDA        fl_run_from_host
 *   IntegrityCheck (cpp:2426-2453)                 fl_integrity_check
 *
 * Errors: every call returns FL_OK (0) or a negative FL_ERR_* code and never
 * exits the process (the reference prints and calls exit(-1), cpp:26-55).
 * fl_last_error() gives a message for the calling thread's last failure.
 *
 * Threading: one fl_system is driven by one host thread at a time. All
 * device work of a system is issued on its own CUDA stream; calls that hand
 * results to host memory synchronise that stream before returning.
 */
#ifndef FLUIDS_GB300_H
#define FLUIDS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FL_ABI_VERSION 1

/* Buffer ids, numbered as in fluids4.0/fluid.h:45-70. */
#define FL_FPOS      0   /* float3 [N] position, world units          */
#define FL_FVEL      1   /* float3 [N] velocity v(t+1/2)               */
#define FL_FVEVAL    2   /* float3 [N] evaluated velocity v(t)         */
#define FL_FFORCE    3   /* float3 [N] SPH force (before mass scaling) */
#define FL_FPRESS    4   /* float  [N] density (named press upstream)  */
#define FL_FCLR      5   /* uint   [N] RGBA8 colour                    */
#define FL_FGCELL    6   /* uint   [N] grid cell or FL_GRID_UNDEF      */
#define FL_FGNDX     7   /* uint   [N] index within the cell           */
#define FL_FGRID     12  /* uint   [N] sorted-slot lookup (identity)   */
#define FL_FGRIDCNT  13  /* uint   [C] particles per cell              */
#define FL_FGRIDOFF  14  /* uint   [C] first sorted slot of each cell  */

#define FL_GRID_UNDEF 0xFFFFFFFFu   /* GRID_UNDEF, fluids4.0/fluid_kernels.cuh:19 */
#define FL_MAX_GRID_SRCH 6          /* fatal above this, fluids4.0/fluid_system.cpp:830-833 */

/* Status codes. */
#define FL_OK             0
#define FL_ERR_ARG       -1   /* null pointer, bad id, size out of range        */
#define FL_ERR_CUDA      -2   /* a CUDA runtime call failed                      */
#define FL_ERR_PARAMS    -3   /* parameters give an unusable grid (gridSrch > 6) */
#define FL_ERR_CAPACITY  -4   /* more points than the system was created for    */
#define FL_ERR_DEVICE    -5   /* a kernel raised its device error word           */
#define FL_ERR_STATE     -6   /* phase called before the phase it depends on     */
#define FL_ERR_NOMEM     -7   /* device allocation failed                        */
#define FL_ERR_IO        -8   /* a point file could not be read or written       */

/* Device error word bits (fl_device_status). */
#define FL_DEV_SPIN_TIMEOUT  0x1u  /* a look-back wait hit its iteration limit */
#define FL_DEV_BAD_CELL      0x2u  /* a cell index outside [0, C] was seen     */
#define FL_DEV_NONFINITE     0x4u  /* a non-finite position was advanced       */

/*
 * Simulation parameters: inputs (first block) and the fields that
 * fl_params_derive computes from them (second block). Names follow FParams
 * (fluids4.0/fluid.h:155-192). All float arithmetic of the derivation is
 * FP32 in the reference's own operation order, so grids and kernels match
 * the reference bit for bit on the same inputs.
 */
typedef struct fl_params {
    /* inputs: SetupDefaultParams / SetupExampleParams (fluid_system.cpp:1953-2097) */
    float sim_scale;          /* world units -> metres                       */
    float pvisc;              /* viscosity                                   */
    float prest_dens;         /* rest density                                */
    float pmass;              /* particle mass                               */
    float pradius;            /* collision radius used by the walls          */
    float psmoothradius;      /* SPH support radius h (metres)               */
    float pintstiff;          /* pressure stiffness                          */
    float bound_stiff;        /* wall stiffness                              */
    float bound_damp;         /* wall damping                                */
    float bound_slope;        /* Y- wall slope along x                       */
    float bound_friction;     /* friction on the Y walls                     */
    float bound_wall_force;   /* amplitude of the moving X- wall             */
    float bound_wall_freq;    /* frequency of the moving X- wall             */
    float AL;                 /* acceleration limit                          */
    float VL;                 /* velocity limit                              */
    float grav_dir[3];        /* gravity direction * magnitude               */
    float grav_amt;           /* gravity multiplier                          */
    float bound_min[3];       /* domain walls, world units                   */
    float bound_max[3];
    float grid_density;       /* cell = 1.5 * h / grid_density (cpp:2101)    */
    float dt;                 /* time step m_DT                              */

    /* derived: SetupSpacing (grid part), SetupGrid, FluidSetupCUDA, UpdateParamsCUDA */
    float grid_size;          /* cell edge in metres                         */
    float r2, d2, rd2;        /* h^2, sim_scale^2, h^2/sim_scale^2           */
    float poly6kern, spikykern, lapkern, vterm;
    float AL2, VL2;
    float gravity[3];
    float pdist;
    float gridMin[3], gridMax[3], gridSize[3], gridDelta[3];
    int   gridRes[3];
    int   gridScanMax[3];
    int   gridSrch;           /* cells searched per axis, 2..6               */
    int   gridTotal;          /* C = resX*resY*resZ                          */
    int   gridAdjCnt;         /* gridSrch^3                                  */
    int   gridAdj[216];       /* cell offsets of the search block            */
} fl_params;

typedef struct fl_system fl_system;

/* ---- parameters ---------------------------------------------------------- */

/* SetupDefaultParams (fluid_system.cpp:1953-2041) with grid_density 2.0
 * (cpp:125) and the example-3 "small dam break" box (cpp:2081-2088). */
int fl_params_default(fl_params *p);

/* Fill the derived block from the inputs: SetupSpacing's grid bounds
 * (cpp:2101,2114-2116), SetupGrid (cpp:793-846), FluidSetupCUDA's scan
 * limits and adjacency (cpp:2249-2287), UpdateParamsCUDA (cpp:2289-2310).
 * Returns FL_ERR_PARAMS when gridSrch > 6 or the grid is empty. */
int fl_params_derive(fl_params *p);

/* ---- lifetime ------------------------------------------------------------ */

/* Initialize + AllocateParticles + AllocateGrid (cpp:92-130, 218-272) on the
 * current CUDA device. `p` must already be derived. */
int fl_create(const fl_params *p, int max_points, fl_system **out);
int fl_destroy(fl_system *s);

/* UpdateParamsCUDA (cpp:2289-2310): replace the parameter block. A block
 * with a different grid reallocates the grid buffers. */
int fl_set_params(fl_system *s, const fl_params *p);
int fl_get_params(const fl_system *s, fl_params *p);

int fl_num_points(const fl_system *s);
int fl_grid_total(const fl_system *s);
/* Simulation time m_Time, advanced by dt on every fl_run (AdvanceTime, cpp:527-531). */
int fl_get_time(const fl_system *s, float *t);
int fl_set_time(fl_system *s, float t);

/* ---- batched systems ------------------------------------------------------
 * Many independent scenes -- each with its own domain, grid and parameters
 * -- stepped together: every phase is one launch over the concatenation of
 * all scenes' points (scene 0 first), each scene owning a contiguous range
 * of cell entries, so one scan over all of them yields every scene's sorted
 * segment. counts[k] points of scene k, params[k] derived; all scenes share
 * dt (one clock). The handle works with every call above and below: buffers
 * read back as the scenes' arrays concatenated (FGRIDCNT/FGRIDOFF: each
 * scene's C cells in turn; FGCELL indexes that concatenated grid; FGRIDOFF
 * holds offsets into the concatenated point order). fl_set_particles/fl_import_device take all points at once.
 * Each scene's results are bit-identical to stepping it alone. */
int fl_batch_create(const fl_params *params, const int *counts, int nscenes, fl_system **out);
int fl_num_scenes(const fl_system *s);
/* Where scene `scene` lives: first point and point count in the
 * concatenated point order, first cell and cell count in the concatenated
 * reference-layout grid. A single-scene system is scene 0. */
int fl_batch_scene_info(const fl_system *s, int scene, int *point_base, int *n, int *cell_base,
                        int *ncells);
/* One scene's parameter block. fl_batch_set_params replaces the physical
 * parameters of scene `scene` (e.g. its viscosity or IntStiff during a
 * parameter fit) without rebuilding the batch: the new block (derived) must
 * keep the scene's grid -- gridRes, gridMin, gridDelta, gridSrch -- and the
 * batch's dt, else FL_ERR_PARAMS. Like fl_set_params it invalidates an
 * open tape. A single-scene system takes scene 0 through fl_set_params. */
int fl_batch_get_params(const fl_system *s, int scene, fl_params *p);
int fl_batch_set_params(fl_system *s, int scene, const fl_params *p);

/* ---- data movement (fluid.h host layout: float3 packed 12 B, uint 4 B) --- */

/* TransferToCUDA (cpp:2312-2321): n points from host SoA arrays. pos is
 * required; any other pointer may be NULL (zero-filled). */
int fl_set_particles(fl_system *s, int n, const float *pos, const float *vel,
                     const float *veval, const float *force, const float *press,
                     const uint32_t *clr);

/* AddParticle (cpp:274-290), k at a time, for emitters (AddEmit, cpp:336-361):
 * k points from host arrays appended after the live ones (vel, veval and
 * clr may be NULL: zero); force and density start at zero. FL_ERR_CAPACITY
 * beyond max_points; single-scene systems only. Like fl_set_particles it
 * invalidates an open tape. */
int fl_add_particles(fl_system *s, int k, const float *pos, const float *vel, const float *veval,
                     const uint32_t *clr);

/* TransferToCUDA + Run + TransferFromCUDA's positions (cpp:2312-2330,
 * 506-524) in one call, for a state kept in host memory between steps: n
 * points from host SoA arrays (pos required; vel, veval, clr may be NULL:
 * zero), one step, and, when pos_out is given, the new positions into it
 * (n x float3, what fl_get_buffer(FL_FPOS) returns; it may be pos itself,
 * which is read in full before any new position is written). Returns when
 * all of it is done, so the arrays may be reused at once. Results equal
 * fl_set_particles (force and density absent), fl_run and fl_get_buffer,
 * bit for bit. With every given array in page-locked memory (fl_host_alloc)
 * on a single-scene system, the positions are read over the host link
 * first, velocities, evaluated velocities and colours follow on a copy
 * engine while the insert, sort and density kernels run, and the force
 * pass writes the new positions into pos_out as it computes them. */
int fl_run_from_host(fl_system *s, int n, const float *pos, const float *vel, const float *veval,
                     const uint32_t *clr, float *pos_out);

/* Copy buffer `buf_id` (FL_F* id) into host memory in fluid.h layout.
 * `bytes` must be at least the buffer size (N or C elements). */
int fl_get_buffer(fl_system *s, int buf_id, void *host_dst, size_t bytes);

/* Page-locked host memory for the transfer calls above. It is mapped into
 * the device's address space: fl_set_particles reads float3 fields from it
 * in one kernel pass (no staging copy), and fl_get_buffer fills it with one
 * copy-engine transfer of the packed field. */
int fl_host_alloc(size_t bytes, void **out);
int fl_host_free(void *p);

/* Device-side export/import in fluid.h layout (headless stand-in for the
 * reference's CUDA-GL interop buffers, cpp:196-204). `dev` is a device
 * pointer on the system's device; the copy is ordered on the system stream. */
int fl_export_device(fl_system *s, int buf_id, void *dev, size_t bytes);
int fl_import_device(fl_system *s, int n, const void *dev_pos, const void *dev_vel,
                     const void *dev_veval);

/* ---- point files ---------------------------------------------------------
 * The .pts format of SavePoints / RunPlayback (cpp:1511-1545, 1787-1841):
 * int N, int nfields, then per field {int type (0 char, 2 float), int
 * channels, N x channels values}: position float x3, velocity float x3,
 * colour char x4 (RGBA8), and -- written here when asked -- a fourth field,
 * evaluated velocity float x3, so a run resumes bit for bit (readers that
 * stop after three fields, like the reference's, are unaffected). Host byte
 * order. fl_pts_read with all arrays NULL only fills *n and *nfields; a
 * missing fourth field reads as zeros. Malformed files give FL_ERR_IO. */
int fl_pts_write(const char *path, int n, const float *pos, const float *vel, const uint32_t *clr,
                 const float *veval);
int fl_pts_read(const char *path, int *n, int *nfields, float *pos, float *vel, uint32_t *clr, float *veval);
/* SavePoints: the system's points to `path` (veval as well when with_veval).
 * RunPlayback: the file's points into the system (fl_set_particles). */
int fl_save_points(fl_system *s, const char *path, int with_veval);
int fl_load_points(fl_system *s, const char *path);

/* SampleParticlesCUDA (cpp:2497-2507; kernel fluid_kernels.cu:263-308), the
 * volume sampling behind SaveBricks (cpp:1597-1752): at every voxel of a
 * res[0] x res[1] x res[2] lattice over [bmin, bmax) (voxel i at bmin + i /
 * res * (bmax - bmin)), scalar x the sum over the particles of its search
 * block within the smoothing radius of gausskern * exp(-r^2 / h2) (r in
 * simulation units, h2 = r2 / 4). Written to out[(z * res[1] + y) * res[0]
 * + x] (host or device memory); voxels outside the scan range are 0. With
 * sort_first the points are first binned and sorted (InsertParticles,
 * PrefixSumCells, CountingSortFull, as SaveBricks does), else the grid of
 * the last sort is used. Single-scene systems. */
int fl_sample_volume(fl_system *s, float *out, const int res[3], const float bmin[3], const float bmax[3],
                     float scalar, int sort_first);

/* ---- phases (fluid_system.h:249-256) ------------------------------------- */

/* InsertParticlesCUDA (cpp:2334-2350; kernel fluid_kernels.cu:22-53).
 * gcell/gndx (N) and gcnt (C) are optional host readbacks. gndx is the
 * canonical within-cell index: the number of lower-indexed points in the
 * same cell (the serial reference's cnt++ order, fluids3.9 cpp:489). */
int fl_insert_particles(fl_system *s, uint32_t *gcell, uint32_t *gndx, uint32_t *gcnt);

/* PrefixSumCellsCUDA (cpp:2354-2424; kernels fluid_kernels.cu:423-467):
 * zero_offsets=1 gives the exclusive scan of FGRIDCNT into FGRIDOFF,
 * zero_offsets=0 the inclusive scan. goff (C) is an optional readback. */
int fl_prefix_sum_cells(fl_system *s, uint32_t *goff, int zero_offsets);

/* CountingSortFullCUDA (cpp:2455-2479; kernel fluid_kernels.cu:56-87):
 * permutes all particle buffers to slot FGRIDOFF[cell]+gndx. Points outside
 * the scan range go to the tail in index order (upstream leaves stale
 * copies there). ppos (N float3) is an optional readback. */
int fl_counting_sort_full(fl_system *s, float *ppos);

/* ComputePressureCUDA (cpp:2515-2519; kernel fluid_kernels.cu:112-149). */
int fl_compute_pressure(fl_system *s);
/* ComputeForceCUDA (cpp:2521-2525; kernel fluid_kernels.cu:180-217). */
int fl_compute_force(fl_system *s);
/* AdvanceCUDA (cpp:2527-2531; kernel fluid_kernels.cu:332-420). */
int fl_advance(fl_system *s, float time, float dt, float ss);

/* Run (cpp:475-525, RUN_GPU_FULL): one full step on the fused kernel
 * sequence, then time += dt. Asynchronous: no host sync. */
int fl_run(fl_system *s);
/* nsteps consecutive Run steps replayed from a captured CUDA graph. */
int fl_run_steps(fl_system *s, int nsteps);

/* Device-side checkpoints of the particle state (every per-point buffer
 * and the simulation time) in one of FL_MAX_CHECKPOINTS slots, e.g. to
 * replay a segment of steps. A slot's storage (80 B per point) is
 * allocated on its first save and kept until fl_destroy. Restoring leaves
 * the grid to be rebuilt by the next fl_run / fl_insert_particles. */
#define FL_MAX_CHECKPOINTS 4
int fl_checkpoint_save(fl_system *s, int slot);
int fl_checkpoint_restore(fl_system *s, int slot);

/* Global conservation sums per scene, in FP64 on the device (rollouts are
 * chaotic, so they are judged by these drifts rather than by trajectories):
 * out[10 * scene + k] = count of points not parked outside the domain,
 * mass, momentum x/y/z (pmass * vel), kinetic energy (1/2 pmass |vel|^2),
 * gravitational potential energy (-pmass gravity . pos * sim_scale), and
 * the sum of positions x/y/z (world units; / count = centre of mass). No
 * counterpart in the reference. */
#define FL_CONSERVATION_VALUES 10
int fl_conservation(fl_system *s, double *out);

/* Launch-shape autotuner (no counterpart in the reference): times the
 * density pass at 128..1024 threads per block, the force and sort passes at
 * three block sizes each and the cell sort at 2, 4 and 8 cells per warp,
 * over `steps` steps from the current state (restored afterwards), and
 * keeps the fastest; chosen (nullable, 3 ints) gets the threads per block
 * of density, force, sort. Results are identical for every shape.
 * FL_ERR_STATE while a tape is recording. */
int fl_autotune(fl_system *s, int steps, int *chosen);

/* The launch shapes in use (no counterpart in the reference): shapes[0..3]
 * = threads per block of the density, force and sort passes, cell entries
 * per warp of the cell sort. */
int fl_launch_shapes(fl_system *s, int *shapes);

/* Pin the launch shapes (no counterpart in the reference), e.g. ones an
 * earlier fl_autotune chose: the same four values, 0 for the compiled
 * default; density 32..1024, force 32..128, sort 32..256 threads per block
 * (multiples of 32), 2, 4 or 8 cells per warp, else FL_ERR_ARG. Results are
 * identical for every shape. */
int fl_set_launch_shapes(fl_system *s, const int *shapes);

/* Which neighbour passes the fused step (fl_run, fl_run_steps,
 * fl_run_from_host) uses; all give bit-identical densities, forces and
 * states. FL_PASSES_PER_POINT (the faster step while cells are small): one thread
 * per point walks its own search block (fluids4.0/fluid_kernels.cu:112-149
 * as written) and records its pair list, which the force pass drains.
 * FL_PASSES_CELL_TASKS: one warp per 64 points of a cell walks their shared
 * search block once, in lockstep, staged in shared memory, recording hit
 * masks; the force pass walks the block again and evaluates the hits
 * pair-parallel. Used where the pruned search applies (gridSrch 2 in every
 * scene) and no tape is recording; the phase entry points and recording
 * tapes always use the per-point passes. FL_PASSES_POINT_PAIRS: the
 * per-point passes, except that where the pruned search applies one thread
 * walks the search block once for two points of a cell with the same
 * lower-band bits (which visit the same candidates in the same order); this
 * one holds for every density pass of the system (fused step, phase entry
 * points, tapes). FL_PASSES_AUTO (the default): the per-point passes until
 * the largest in-range cell reaches 512 points, the cell tasks from then
 * until it falls below 384 (each step's sort records the largest cell; a
 * fused-step call acts on the last value that has reached the host, a
 * step or two old). No counterpart in the reference (which has only the
 * per-point walk). fl_neighbour_passes returns the mode set;
 * fl_neighbour_passes_in_use the passes the next fused step takes
 * (FL_PASSES_AUTO resolved with the latest count on the host: after
 * fl_sync, the last step's). */
#define FL_PASSES_PER_POINT   0
#define FL_PASSES_CELL_TASKS  1
#define FL_PASSES_POINT_PAIRS 2
#define FL_PASSES_AUTO        3
int fl_set_neighbour_passes(fl_system *s, int mode);
int fl_neighbour_passes(const fl_system *s);
int fl_neighbour_passes_in_use(fl_system *s);
/* Fused steps issued since creation with the per-point passes (counts[0])
 * and with the cell tasks (counts[1]) -- what FL_PASSES_AUTO chose. */
int fl_passes_steps(const fl_system *s, int64_t *counts);

/* Wait for the system stream; returns FL_ERR_DEVICE if a kernel raised the
 * device error word since the last fl_sync (bits in *dev_flags if non-NULL). */
int fl_sync(fl_system *s);
int fl_device_status(fl_system *s, uint32_t *dev_flags);

/* IntegrityCheck (cpp:2426-2453): number of sorted slots whose cell/index
 * disagree with FGRIDOFF/FGRIDCNT (0 when the grid is consistent). */
int fl_integrity_check(fl_system *s, int64_t *bad);

/* Per-phase device timing, the counterpart of the PERF_PUSH/PERF_POP pairs
 * around each phase of Run (cpp:507-515). While enabled, fl_run brackets
 * every launch with CUDA events on the system stream (up to 4096 steps).
 * fl_get_phase_times synchronises and returns the mean milliseconds per
 * step of each phase: [0] clear+insert, [1] scan, [2] index scatter,
 * [3] canonical sort+gather, [4] density, [5] force+advance; *steps gets
 * the number of timed steps. Enabling again resets the accumulators. */
int fl_set_timing(fl_system *s, int enable);
/* Run nsteps steps (graph replay when use_graph != 0, else eager fl_run)
 * between two CUDA events on the system stream; synchronises and stores the
 * elapsed device time in *ms. With restart_every > 0 the steps run as
 * segments of at most restart_every steps, each starting from checkpoint
 * `restart_slot` (the restore is inside the timed interval). */
int fl_time_steps(fl_system *s, int nsteps, int use_graph, int restart_every, int restart_slot,
                  double *ms);
int fl_get_phase_times(fl_system *s, double ms[8], int *steps);

/* ---- adjoint of the fused step -------------------------------------------
 * No counterpart in the reference (its step has no derivative). The
 * reverse-mode derivative of a run of fl_run / fl_run_steps steps with
 * respect to the particle state at its start and to three parameters
 * (pvisc, prest_dens, pintstiff), for optimisation and inverse problems
 * over the same simulation. The integer structure of each step (cells, the
 * sort, which pairs interact, which walls and limits act) is piecewise
 * constant and carries no derivative.
 *
 * fl_tape_begin opens a tape for up to max_steps steps (a tape already
 * open with the same max_steps and every starts over in its storage,
 * without reallocating; another shape is freed first): every Run step
 * from then on saves the state before it every `every` steps (48 B per
 * point each; every > 1 trades memory for a replay of each segment during
 * fl_backward) and its time. Changing the state outside Run while recording
 * (fl_set_particles, fl_import_device, fl_set_params, fl_checkpoint_restore,
 * a phase call) invalidates the tape; fl_set_time does not. A step beyond
 * max_steps fails with FL_ERR_CAPACITY. Steps run eagerly while recording.
 *
 * fl_backward takes dL/d(final FPOS, FVEL, FVEVAL) in the current slot
 * order (fluid.h float3 layout, n x 3 floats; NULL = zero) and returns
 * dL/d(initial FPOS, FVEL, FVEVAL) in the order the points had when
 * recording began (NULL = not wanted) and, per scene, dL/d(pvisc,
 * prest_dens, pintstiff) as 3 doubles (gparams[3 * scene + k]; NULL = not
 * wanted). Vector arguments may be host or device memory. The live state is
 * left as it was, except that the phase API needs a fresh
 * fl_insert_particles. The result is deterministic (no atomics).
 * fl_tape_order gives, per current slot, the point's index when recording
 * began (n uint32, host or device). fl_tape_steps: steps recorded. */
int fl_tape_begin(fl_system *s, int max_steps, int every);
/* fl_tape_begin with flags. FL_TAPE_KEEP_LISTS: each step's pair lists,
 * pair counts and densities are kept (~520 B per point per step: 512 B of
 * pair list) -- for every step of the tape when every = 1, for the steps of
 * the segment being replayed when every > 1 -- so its reverse step skips
 * the density pass: memory for time, same gradients. */
#define FL_TAPE_KEEP_LISTS 1
int fl_tape_begin_ex(fl_system *s, int max_steps, int every, int flags);
int fl_tape_steps(const fl_system *s);
int fl_tape_order(fl_system *s, uint32_t *order);
/* fl_backward_scaled: fl_backward for long rollouts, whose exact gradient
 * grows about 1.4x per step (nearby trajectories diverge) and leaves the
 * FP32 range after a few hundred steps. The reverse pass scales each
 * scene's cotangents by a power of two whenever their largest component
 * passes 2^40 (exact: every reverse operation is linear in them), so
 * nothing overflows; gpos/gvel/gveval receive the mantissas and
 * exponents[scene] (nscenes ints, host) the binary exponent: the gradient
 * is mantissa * 2^exponent. gparams are the full FP64 values. fl_backward
 * itself returns mantissa * 2^exponent in float (infinite where that
 * overflows); both give identical bits wherever no scaling happened. */
int fl_backward_scaled(fl_system *s, const float *dpos, const float *dvel, const float *dveval,
                       float *gpos, float *gvel, float *gveval, double *gparams, int *exponents);
int fl_backward(fl_system *s, const float *dpos, const float *dvel, const float *dveval,
                float *gpos, float *gvel, float *gveval, double *gparams);
int fl_tape_end(fl_system *s);

/* ---- allocation-free scan ------------------------------------------------
 * No counterpart in the reference. For host applications that cannot let a
 * library allocate device memory -- an engine or plugin host that owns the
 * whole device budget, or a real-time loop where cudaMalloc/cudaFree would
 * synchronise the device and stall its other streams: the cell prefix sum
 * of fl_prefix_sum_cells over caller-owned device buffers, without a
 * fl_system. d_counts[n] in, d_offsets[n] out (exclusive scan when
 * zero_offsets != 0, inclusive otherwise); the two ranges must not overlap
 * (the scan is not in place; overlapping ranges are rejected with
 * FL_ERR_ARG). d_status (one device uint32, required: FL_ERR_ARG if NULL)
 * gets FL_DEV_SPIN_TIMEOUT OR-ed in if a look-back wait gave up, in which
 * case the offsets are wrong; it is the only report of that, since the
 * call does not wait for its work. Work is queued on `stream` (a
 * cudaStream_t; NULL = default stream).
 * The scan's scratch is a fixed ~8.5 KB device array inside the library,
 * held by every GPU that loads it until the process exits, so n is limited
 * to FL_NOALLOC_MAX_COUNTS (larger n is rejected with FL_ERR_ARG). The first
 * call on each device looks up that array's device address with the device
 * current; make that first call before any stream capture. Later calls look
 * it up again unless their stream is capturing, so the array is found again
 * after a cudaDeviceReset. All calls share the one array: calls whose GPU
 * work overlaps (other streams, other host threads) race on it and must be
 * ordered by the caller. Nothing is allocated: no cudaMalloc, cudaFree or
 * allocating library routine. */
#define FL_NOALLOC_MAX_COUNTS 4194304
int fl_prefix_sum_noalloc(const uint32_t *d_counts, uint32_t *d_offsets, int n, int zero_offsets,
                          uint32_t *d_status, void *stream);

/* ---- test hooks for the bounded look-back waits ----------------------------
 * No counterpart in the reference. Each runs a scan with tile 0 withheld --
 * one CTA fewer, the tile ticket starting at 1, so every index stays in
 * bounds -- and a short spin limit (1 .. 2^20 polls): tile 1's wait for
 * tile 0's descriptor runs out, the kernel records FL_DEV_SPIN_TIMEOUT and
 * returns. fl_test_scan_timeout scans the system's cell counts (at least
 * two 4096-entry tiles; fl_sync then returns FL_ERR_DEVICE), and
 * fl_test_scan_noalloc_timeout runs fl_prefix_sum_noalloc's scan (n > 4096;
 * the flag lands in d_status). The offsets they write are not a scan; they
 * exist to test the error path. */
int fl_test_scan_timeout(fl_system *s, int spin_limit);
int fl_test_scan_noalloc_timeout(const uint32_t *d_counts, uint32_t *d_offsets, int n, uint32_t *d_status,
                                 int spin_limit, void *stream);

/* How fl_backward finds each point's reverse pairs (no counterpart in the
 * reference): FL_REVERSE_WALK walks the point's reverse block (one launch);
 * FL_REVERSE_TRANSPOSE transposes the density pass's pair lists (atomics,
 * then a per-list sort: less work, more launches); FL_REVERSE_AUTO (the
 * default) transposes from FL_REVERSE_TRANSPOSE_MIN points (all scenes of
 * a batch together) and walks below. All give the same lists, so the same
 * gradients bit for bit. */
#define FL_REVERSE_AUTO      0
#define FL_REVERSE_WALK      1
#define FL_REVERSE_TRANSPOSE 2
#define FL_REVERSE_TRANSPOSE_MIN (1 << 20)
int fl_set_reverse_lists(fl_system *s, int mode);

/* The CUDA stream (cudaStream_t) the system issues its work on. */
void *fl_stream(fl_system *s);

/* Message for the calling thread's most recent failed call. */
const char *fl_last_error(void);
int fl_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* FLUIDS_GB300_H */
