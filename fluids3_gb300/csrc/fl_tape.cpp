// Adjoint tape and reverse pass of the fused step (no counterpart in the
// reference, whose step has no derivative).
//
// While a tape is open every Run step (fl_run, fl_run_steps) saves what
// its reverse needs: the state before the step (position, velocity,
// evaluated velocity: 48 B per point) every `every` steps, the step's time,
// and with every = 1 the step's SPH force (16 B per point). fl_backward
// then walks the steps last to first. With every > 1 it first replays each
// checkpoint segment's fused steps, saving every step's state and force in
// segment buffers. For each step it rebuilds the sort and the densities
// (with their pair lists) from the saved state and runs the adjoint kernels
// (fl_adjoint.cu). Everything is deterministic, so the rebuilt values are
// the recorded step's, bit for bit.
//
// Device memory: ceil(max_steps / every) checkpoints of 48 B per point;
// with every = 1, 16 B per point per step of forces, else `every` segment
// slots of 64 B per point; and ~450 B per point of adjoint buffers,
// reverse-pair lists, identity maps and the saved final state.
#include <stdlib.h>
#include <string.h>

#include <math.h>
#include <vector>

#include "fl_internal.h"

struct fl_tape {
    int max_steps, every, steps, n, cap;
    int broken, recording;
    int nck;
    float4 *ck;             // nck x {pos, vel, veval} x cap
    float4 *seg;            // every x {pos, vel, veval} x cap (every > 1)
    float4 *force;          // per step of the tape (every = 1) or of a segment: the step's SPH force
    float *time;            // per recorded step: the time it read
    uint32_t *ident[2];     // per current slot: the point's index when recording began
    int ident_cur;
    float4 *g[2][3];        // adjoint of (pos, vel, veval), ping-pong across steps
    int gcur;
    float4 *xa, *ea, *fb, *pc;
    float *rb;
    float2 *rr;                   // per slot: density and its reciprocal
    uint32_t *revlist, *revcnt;   // reverse pairs (transposed pair lists), for both pair adjoints
    uint32_t *crowd, *crowd_count; // points whose pair lists overflowed (count cleared per reverse step)
    uint32_t *revlong;             // points whose reverse lists are walked (count: crowd_count[1])
    int nchunks;
    double *partial, *acc;  // per-scene parameter gradients (visc, rest density, IntStiff)
    uint32_t *gmax;         // per scene: largest cotangent component of the last reverse step (float bits)
    int *gexp;              // per scene: the cotangents are the gradient times 2^-gexp
    int *sbase, *sn;
    void *save[F_COUNT];    // the live state when fl_backward starts, restored at its end
    float *save_time;
    // FL_TAPE_KEEP_LISTS (every > 1): per segment slot, the replayed step's
    // pair lists, pair counts and densities, so its reverse step skips the
    // density pass
    int keep_lists;
    size_t list_words;
    uint32_t *seg_list, *seg_cnt;
    float *seg_rho;
    uint32_t *own_list, *own_cnt;   // the system's own lists while a recorded step writes into a slot
};

static void tape_release(fl_tape *t) {
    if (!t) return;
    cudaFree(t->ck); cudaFree(t->seg); cudaFree(t->force); cudaFree(t->time);
    for (int k = 0; k < 2; k++) {
        cudaFree(t->ident[k]);
        for (int j = 0; j < 3; j++) cudaFree(t->g[k][j]);
    }
    cudaFree(t->xa); cudaFree(t->ea); cudaFree(t->fb); cudaFree(t->pc); cudaFree(t->rb);
    cudaFree(t->revlist); cudaFree(t->revcnt); cudaFree(t->rr);
    cudaFree(t->crowd); cudaFree(t->crowd_count); cudaFree(t->revlong);
    cudaFree(t->partial); cudaFree(t->acc); cudaFree(t->sbase); cudaFree(t->sn);
    cudaFree(t->gmax); cudaFree(t->gexp);
    for (int k = 0; k < F_COUNT; k++) cudaFree(t->save[k]);
    cudaFree(t->save_time);
    cudaFree(t->seg_list); cudaFree(t->seg_cnt); cudaFree(t->seg_rho);
    delete t;
}

void fl_tape_free(fl_system *s) {
    if (!s || !s->tape) return;
    cudaStreamSynchronize(s->stream);
    if (s->tape->own_list) {   // a recorded step stopped while writing into a slot
        s->hitlist = s->tape->own_list;
        s->hitcnt = s->tape->own_cnt;
    }
    tape_release(s->tape);
    s->tape = nullptr;
}

int fl_tape_recording(const fl_system *s) { return s->tape && s->tape->recording && !s->tape->broken; }

void fl_tape_touch(fl_system *s) {
    if (s && s->tape && s->tape->steps > 0) s->tape->broken = 1;
}

// The live (pos, vel, veval) copies to / from a {pos, vel, veval} x cap
// block, in one kernel pass.
static int save_state(fl_system *s, const fl_tape *t, float4 *dst) {
    const float4 *src[3] = {s->f[F_POS].cur<float4>(), s->f[F_VEL].cur<float4>(), s->f[F_VEVAL].cur<float4>()};
    float4 *out[3] = {dst, dst + t->cap, dst + 2 * (size_t)t->cap};
    return fl_launch_copy3(s, s->n, 3, src, out);
}

static int load_state(fl_system *s, const fl_tape *t, const float4 *blk) {
    const float4 *src[3] = {blk, blk + t->cap, blk + 2 * (size_t)t->cap};
    float4 *out[3] = {s->f[F_POS].cur<float4>(), s->f[F_VEL].cur<float4>(), s->f[F_VEVAL].cur<float4>()};
    return fl_launch_copy3(s, s->n, 3, src, out);
}

static int save_force(fl_system *s, float4 *dst) {
    const float4 *src[1] = {s->f[F_FORCE].cur<float4>()};
    float4 *out[1] = {dst};
    return fl_launch_copy3(s, s->n, 1, src, out);
}

extern "C" int fl_tape_begin(fl_system *s, int max_steps, int every) {
    return fl_tape_begin_ex(s, max_steps, every, 0);
}

extern "C" int fl_tape_begin_ex(fl_system *s, int max_steps, int every, int flags) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_tape_begin: null system");
    if (flags & ~FL_TAPE_KEEP_LISTS) return fl_fail(FL_ERR_ARG, "fl_tape_begin_ex: unknown flags 0x%x", flags);
    const int keep = (flags & FL_TAPE_KEEP_LISTS) ? 1 : 0;
    if (max_steps < 1 || every < 1 || every > max_steps)
        return fl_fail(FL_ERR_ARG, "fl_tape_begin: max_steps %d, every %d (need 1 <= every <= max_steps)",
                       max_steps, every);
    if (s->tape && s->tape->max_steps == max_steps && s->tape->every == every && s->tape->keep_lists == keep &&
        s->tape->cap == (s->max_points > 0 ? s->max_points : 1)) {
        // same shape: start over in the storage already held
        fl_tape *t = s->tape;
        FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
        t->steps = 0;
        t->n = 0;
        t->broken = 0;
        t->ident_cur = 0;
        t->gcur = 0;
        t->recording = 1;
        return FL_OK;
    }
    fl_tape_free(s);
    fl_tape *t = new fl_tape();
    memset(t, 0, sizeof(*t));
    t->max_steps = max_steps;
    t->every = every;
    t->cap = s->max_points > 0 ? s->max_points : 1;
    t->nck = (max_steps + every - 1) / every;
    int most = s->max_points;
    if (s->batched) {
        most = 0;
        for (int k = 0; k < s->nscenes; k++) most = s->scene_n[k] > most ? s->scene_n[k] : most;
    }
    t->nchunks = fl_param_chunks(most);
    const size_t cap = (size_t)t->cap;
    int r = FL_OK;
    do {
        if ((r = fl_dalloc((void **)&t->ck, 48 * cap * (size_t)t->nck)) != FL_OK) break;
        if (every > 1 && (r = fl_dalloc((void **)&t->seg, 48 * cap * (size_t)every)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->force, 16 * cap * (size_t)(every > 1 ? every : max_steps))) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->time, 4 * (size_t)max_steps)) != FL_OK) break;
        for (int k = 0; k < 2 && r == FL_OK; k++) {
            r = fl_dalloc((void **)&t->ident[k], 4 * cap);
            for (int j = 0; j < 3 && r == FL_OK; j++) r = fl_dalloc((void **)&t->g[k][j], 16 * cap);
        }
        if (r != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->xa, 16 * cap)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->ea, 16 * cap)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->fb, 16 * cap)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->pc, 16 * cap)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->rb, 4 * cap)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->revcnt, 4 * cap)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->crowd, 4 * cap)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->revlong, 4 * cap)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->crowd_count, 256)) != FL_OK) break;
        if (cudaMemsetAsync(t->crowd_count, 0, 256, s->stream) != cudaSuccess) {
            r = fl_fail(FL_ERR_CUDA, "tape: memset failed");
            break;
        }
        if ((r = fl_dalloc((void **)&t->rr, 8 * cap)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->revlist, 4 * ((cap + 31) / 32) * 32 * (size_t)s->D.hcap)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->partial, 24 * (size_t)s->nscenes * t->nchunks)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->acc, 24 * (size_t)s->nscenes)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->sbase, 4 * (size_t)s->nscenes)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->sn, 4 * (size_t)s->nscenes)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->gmax, 4 * (size_t)s->nscenes)) != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->gexp, 4 * (size_t)s->nscenes)) != FL_OK) break;
        for (int k = 0; k < F_COUNT && r == FL_OK; k++) r = fl_dalloc(&t->save[k], s->f[k].esz * cap);
        if (r != FL_OK) break;
        if ((r = fl_dalloc((void **)&t->save_time, 256)) != FL_OK) break;
        if (keep) {   // slots: every step of a segment (every > 1) or of the whole tape (every = 1)
            t->keep_lists = 1;
            const size_t slots = (size_t)(every > 1 ? every : max_steps);
            t->list_words = ((cap + 31) / 32) * 32 * (size_t)s->D.hcap;
            if ((r = fl_dalloc((void **)&t->seg_list, 4 * t->list_words * slots)) != FL_OK) break;
            if ((r = fl_dalloc((void **)&t->seg_cnt, 4 * cap * slots)) != FL_OK) break;
            r = fl_dalloc((void **)&t->seg_rho, 4 * cap * slots);
        }
    } while (0);
    if (r != FL_OK) {
        tape_release(t);
        return r;
    }
    t->recording = 1;
    s->tape = t;
    return FL_OK;
}

extern "C" int fl_tape_end(fl_system *s) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_tape_end: null system");
    fl_tape_free(s);
    return FL_OK;
}

extern "C" int fl_tape_steps(const fl_system *s) {
    if (!s || !s->tape) return 0;
    return s->tape->steps;
}

int fl_tape_pre_step(fl_system *s) {
    fl_tape *t = s->tape;
    const int k = t->steps;
    if (k >= t->max_steps)
        return fl_fail(FL_ERR_CAPACITY, "tape full: it holds %d steps (fl_tape_begin max_steps)", t->max_steps);
    if (k == 0) t->n = s->n;
    else if (s->n != t->n) { t->broken = 1; return FL_OK; }
    if (k % t->every == 0) FL_TRY(save_state(s, t, t->ck + (size_t)(k / t->every) * 3 * t->cap));
    FL_CUDA_TRY(cudaMemcpyAsync(t->time + k, s->time_dev + s->time_slot, sizeof(float),
                                cudaMemcpyDeviceToDevice, s->stream));
    if (t->keep_lists && t->every == 1) {   // this step's density pass writes into slot k
        t->own_list = s->hitlist;
        t->own_cnt = s->hitcnt;
        s->hitlist = t->seg_list + (size_t)k * t->list_words;
        s->hitcnt = t->seg_cnt + (size_t)k * t->cap;
    }
    return FL_OK;
}

int fl_tape_post_step(fl_system *s) {
    fl_tape *t = s->tape;
    if (t->own_list) {
        s->hitlist = t->own_list;
        s->hitcnt = t->own_cnt;
        t->own_list = t->own_cnt = nullptr;
        if (!t->broken && s->n)
            FL_CUDA_TRY(cudaMemcpyAsync(t->seg_rho + (size_t)t->steps * t->cap, s->f[F_PRESS].cur<void>(),
                                        4 * (size_t)s->n, cudaMemcpyDeviceToDevice, s->stream));
    }
    if (t->broken) return FL_OK;
    // every = 1: keep the step's force (sorted order) so the reverse pass
    // need not recompute it
    if (t->every == 1) FL_TRY(save_force(s, t->force + (size_t)t->steps * t->cap));
    FL_TRY(fl_launch_compose(s, s->n, s->src, t->steps == 0 ? nullptr : t->ident[t->ident_cur],
                             t->ident[t->ident_cur ^ 1]));
    t->ident_cur ^= 1;
    t->steps++;
    return FL_OK;
}

extern "C" int fl_tape_order(fl_system *s, uint32_t *order) {
    if (!s || !order) return fl_fail(FL_ERR_ARG, "fl_tape_order: null argument");
    fl_tape *t = s->tape;
    if (!t) return fl_fail(FL_ERR_STATE, "fl_tape_order: no tape (fl_tape_begin)");
    if (s->n == 0) return FL_OK;
    const size_t bytes = 4 * (size_t)s->n;
    const uint32_t *from = t->ident[t->ident_cur];
    if (t->steps == 0) {
        FL_TRY(fl_ensure_stage(s, bytes));
        FL_TRY(fl_launch_compose(s, s->n, nullptr, nullptr, (uint32_t *)s->stage));
        from = (const uint32_t *)s->stage;
    }
    FL_CUDA_TRY(cudaMemcpyAsync(order, from, bytes, cudaMemcpyDefault, s->stream));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return FL_OK;
}

// fluid.h-layout (float3) adjoint in, float4 out; null means zero.
static int upload_vec3(fl_system *s, const float *src, float4 *dst) {
    const size_t n = (size_t)s->n;
    if (!src) {
        FL_CUDA_TRY(cudaMemsetAsync(dst, 0, 16 * n, s->stream));
        return FL_OK;
    }
    FL_TRY(fl_ensure_stage(s, 12 * n));
    FL_CUDA_TRY(cudaMemcpyAsync(s->stage, src, 12 * n, cudaMemcpyDefault, s->stream));
    return fl_launch_unpack3(s, (const float *)s->stage, dst, (int)n);
}

static int download_vec3(fl_system *s, const float4 *src, float *dst) {
    if (!dst) return FL_OK;
    const size_t n = (size_t)s->n;
    FL_TRY(fl_ensure_stage(s, 12 * n));
    FL_TRY(fl_launch_pack3(s, src, (float *)s->stage, (int)n));
    FL_CUDA_TRY(cudaMemcpyAsync(dst, s->stage, 12 * n, cudaMemcpyDefault, s->stream));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return FL_OK;
}

// The reverse of recorded step k from its saved state and force; with
// `slot` >= 0 the step's pair lists, counts and densities come from that
// segment slot instead of a density pass.
static int backward_step(fl_system *s, fl_tape *t, const float4 *state, const float4 *force, int k,
                         int slot = -1) {
    FL_TRY(load_state(s, t, state));
    uint32_t *own_list = s->hitlist, *own_cnt = s->hitcnt;
    if (slot >= 0) {
        FL_TRY(fl_rebuild_grid(s));
        if (s->n)
            FL_CUDA_TRY(cudaMemcpyAsync(s->f[F_PRESS].cur<void>(), t->seg_rho + (size_t)slot * t->cap,
                                        4 * (size_t)s->n, cudaMemcpyDeviceToDevice, s->stream));
        s->hitlist = t->seg_list + (size_t)slot * t->list_words;
        s->hitcnt = t->seg_cnt + (size_t)slot * t->cap;
        s->lists_valid = 1;
    } else {
        FL_TRY(fl_recompute_step(s));
    }
    const int c = t->gcur, x = c ^ 1;
    const int r = [&]() {
        FL_CUDA_TRY(cudaMemsetAsync(t->crowd_count, 0, 2 * sizeof(uint32_t), s->stream));
        FL_TRY(fl_launch_adj_advance(s, t->time + k, force, t->g[c][0], t->g[c][1], t->g[c][2], t->xa, t->ea,
                                     t->fb, t->g[x][1], t->rr));
        FL_TRY(fl_launch_adj_force(s, t->rr, t->fb, t->xa, t->ea, t->rb, t->pc, t->g[x][2], t->revlist,
                                   t->revcnt, t->crowd, t->crowd_count, t->revlong, t->crowd_count + 1));
        FL_TRY(fl_launch_adj_density(s, t->revlist, t->revcnt, t->rb, t->xa, t->g[x][0], t->crowd,
                                     t->crowd_count));
        FL_TRY(fl_launch_param_reduce(s, t->pc, t->sbase, t->sn, t->nchunks, t->partial, t->gexp, t->acc));
        FL_TRY(fl_launch_adj_rescale(s, t->g[x][0], t->g[x][1], t->g[x][2], t->gmax, t->gexp));
        return FL_OK;
    }();
    s->hitlist = own_list;
    s->hitcnt = own_cnt;
    if (slot >= 0) s->lists_valid = 0;   // the live lists (and pair records) are not this state's
    if (r != FL_OK) return r;
    t->gcur = x;
    return FL_OK;
}

static int run_reverse(fl_system *s, fl_tape *t) {
    const size_t blk = 3 * (size_t)t->cap;
    const int nseg = (t->steps + t->every - 1) / t->every;
    for (int g = nseg - 1; g >= 0; g--) {
        const int t0 = g * t->every;
        const int t1 = (t0 + t->every < t->steps) ? t0 + t->every : t->steps;
        const float4 *ck = t->ck + (size_t)g * blk;
        if (t->every == 1) {
            FL_TRY(backward_step(s, t, ck, t->force + (size_t)t0 * t->cap, t0, t->keep_lists ? t0 : -1));
            continue;
        }
        // replay the segment's fused steps from its checkpoint, saving the
        // state before each step and the force it computed
        FL_TRY(load_state(s, t, ck));
        for (int k = t0; k < t1; k++) {
            FL_TRY(save_state(s, t, t->seg + (size_t)(k - t0) * blk));
            FL_CUDA_TRY(cudaMemcpyAsync(s->time_dev + s->time_slot, t->time + k, sizeof(float),
                                        cudaMemcpyDeviceToDevice, s->stream));
            uint32_t *own_list = s->hitlist, *own_cnt = s->hitcnt;
            const int own_passes = s->passes;
            if (t->keep_lists) {   // the step's density pass (one that writes pair lists) fills the slot
                s->hitlist = t->seg_list + (size_t)(k - t0) * t->list_words;
                s->hitcnt = t->seg_cnt + (size_t)(k - t0) * t->cap;
                if (s->passes == FL_PASSES_CELL_TASKS || s->passes == FL_PASSES_AUTO) s->passes = FL_PASSES_PER_POINT;
            }
            const int r = fl_step_fused(s);
            s->hitlist = own_list;
            s->hitcnt = own_cnt;
            s->passes = own_passes;
            FL_TRY(r);
            FL_TRY(save_force(s, t->force + (size_t)(k - t0) * t->cap));
            if (t->keep_lists && s->n)
                FL_CUDA_TRY(cudaMemcpyAsync(t->seg_rho + (size_t)(k - t0) * t->cap, s->f[F_PRESS].cur<void>(),
                                            4 * (size_t)s->n, cudaMemcpyDeviceToDevice, s->stream));
        }
        for (int k = t1 - 1; k >= t0; k--)
            FL_TRY(backward_step(s, t, t->seg + (size_t)(k - t0) * blk, t->force + (size_t)(k - t0) * t->cap, k,
                                 t->keep_lists ? k - t0 : -1));
    }
    return FL_OK;
}

// The reverse pass; the state gradients come back as mantissas with a
// per-scene binary exponent in `exps` (host, nscenes entries).
// With apply_exponent the mantissas are multiplied by 2^exponent on the
// device first (in float: infinite where the gradient overflows it).
static int backward_impl(fl_system *s, const float *dpos, const float *dvel, const float *dveval, float *gpos,
                         float *gvel, float *gveval, double *gparams, int *exps, bool apply_exponent) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_backward: null system");
    fl_tape *t = s->tape;
    if (!t) return fl_fail(FL_ERR_STATE, "fl_backward: no tape (fl_tape_begin)");
    if (t->broken)
        return fl_fail(FL_ERR_STATE, "fl_backward: the state changed outside Run while recording; the tape "
                                     "no longer describes it");
    if (t->steps == 0) return fl_fail(FL_ERR_STATE, "fl_backward: no recorded steps");
    if (s->n != t->n) return fl_fail(FL_ERR_STATE, "fl_backward: point count changed since recording");
    const size_t n = (size_t)s->n;

    // keep the live state: the reverse pass rebuilds every step in place
    for (int k = 0; k < F_COUNT; k++)
        if (n) FL_CUDA_TRY(cudaMemcpyAsync(t->save[k], s->f[k].cur<void>(), s->f[k].esz * n,
                                           cudaMemcpyDeviceToDevice, s->stream));
    FL_CUDA_TRY(cudaMemcpyAsync(t->save_time, s->time_dev + s->time_slot, sizeof(float),
                                cudaMemcpyDeviceToDevice, s->stream));
    const int slot = s->time_slot, host_valid = s->time_host_valid;
    const float host_time = s->time;

    // per-scene point ranges for the parameter sums
    {
        const int ns = s->nscenes;
        int *hb = (int *)calloc((size_t)ns, sizeof(int)), *hn = (int *)calloc((size_t)ns, sizeof(int));
        if (!hb || !hn) { free(hb); free(hn); return fl_fail(FL_ERR_NOMEM, "fl_backward: host memory"); }
        for (int k = 0; k < ns; k++) {
            hb[k] = s->batched ? s->scene_point_base[k] : 0;
            hn[k] = s->batched ? s->scene_n[k] : s->n;
        }
        cudaError_t e1 = cudaMemcpyAsync(t->sbase, hb, 4 * (size_t)ns, cudaMemcpyHostToDevice, s->stream);
        cudaError_t e2 = cudaMemcpyAsync(t->sn, hn, 4 * (size_t)ns, cudaMemcpyHostToDevice, s->stream);
        cudaError_t e3 = cudaStreamSynchronize(s->stream);
        free(hb); free(hn);
        if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
            return fl_fail(FL_ERR_CUDA, "fl_backward: scene ranges: %s",
                           cudaGetErrorString(e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3)));
    }
    FL_CUDA_TRY(cudaMemsetAsync(t->acc, 0, 24 * (size_t)s->nscenes, s->stream));
    FL_CUDA_TRY(cudaMemsetAsync(t->gmax, 0, 4 * (size_t)s->nscenes, s->stream));
    FL_CUDA_TRY(cudaMemsetAsync(t->gexp, 0, 4 * (size_t)s->nscenes, s->stream));
    t->gcur = 0;
    FL_TRY(upload_vec3(s, dpos, t->g[0][0]));
    FL_TRY(upload_vec3(s, dvel, t->g[0][1]));
    FL_TRY(upload_vec3(s, dveval, t->g[0][2]));

    const int rec = t->recording;
    t->recording = 0;
    int r = run_reverse(s, t);
    t->recording = rec;

    // the live state back as it was (the grid stays from the rebuilt steps,
    // so the phase API needs a fresh insert)
    for (int k = 0; k < F_COUNT; k++)
        if (n) FL_CUDA_TRY(cudaMemcpyAsync(s->f[k].cur<void>(), t->save[k], s->f[k].esz * n,
                                           cudaMemcpyDeviceToDevice, s->stream));
    s->time_slot = slot;
    FL_CUDA_TRY(cudaMemcpyAsync(s->time_dev + slot, t->save_time, sizeof(float), cudaMemcpyDeviceToDevice,
                                s->stream));
    s->time = host_time;
    s->time_host_valid = host_valid;
    s->have_insert = s->have_offsets = s->have_grid = 0;
    s->codes_valid = s->lists_valid = 0;
    if (r != FL_OK) return r;

    if (apply_exponent)
        FL_TRY(fl_launch_adj_apply_exponent(s, t->g[t->gcur][0], t->g[t->gcur][1], t->g[t->gcur][2], t->gexp));
    FL_TRY(download_vec3(s, t->g[t->gcur][0], gpos));
    FL_TRY(download_vec3(s, t->g[t->gcur][1], gvel));
    FL_TRY(download_vec3(s, t->g[t->gcur][2], gveval));
    if (gparams)
        FL_CUDA_TRY(cudaMemcpyAsync(gparams, t->acc, 24 * (size_t)s->nscenes, cudaMemcpyDeviceToHost, s->stream));
    FL_CUDA_TRY(cudaMemcpyAsync(exps, t->gexp, 4 * (size_t)s->nscenes, cudaMemcpyDeviceToHost, s->stream));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return FL_OK;
}

extern "C" int fl_backward_scaled(fl_system *s, const float *dpos, const float *dvel, const float *dveval,
                                  float *gpos, float *gvel, float *gveval, double *gparams, int *exponents) {
    if (!s || !exponents) return fl_fail(FL_ERR_ARG, "fl_backward_scaled: null system or exponents");
    return backward_impl(s, dpos, dvel, dveval, gpos, gvel, gveval, gparams, exponents, false);
}

extern "C" int fl_backward(fl_system *s, const float *dpos, const float *dvel, const float *dveval,
                           float *gpos, float *gvel, float *gveval, double *gparams) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_backward: null system");
    std::vector<int> e((size_t)(s->nscenes > 0 ? s->nscenes : 1), 0);
    return backward_impl(s, dpos, dvel, dveval, gpos, gvel, gveval, gparams, e.data(), true);
}
