// Point files, volume sampling and particle emission: the data either side
// of the step.
//
// .pts files follow SavePoints / RunPlayback (fluids4.0/fluid_system.cpp:
// 1511-1545, 1787-1841): int N, int nfields, then per field
// {int type (0 char, 1 int, 2 float, 3 double), int channels, N x channels
// values}, in the order position (float x3), velocity (float x3), colour
// (char x4). This writer may add a fourth field, the evaluated velocity
// (float x3), so a run resumes exactly; a reader that stops after three
// fields (the reference's) reads such a file unchanged. Host byte order.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fl_internal.h"

namespace {

struct FileCloser {
    FILE *f;
    ~FileCloser() { if (f) fclose(f); }
};

bool put_field(FILE *f, int type, int channels, const void *data, size_t bytes) {
    return fwrite(&type, sizeof(int), 1, f) == 1 && fwrite(&channels, sizeof(int), 1, f) == 1 &&
           (bytes == 0 || fwrite(data, 1, bytes, f) == bytes);
}

// Reads one field's header and data (or skips the data when dst is null).
int get_field(FILE *f, const char *path, const char *what, int want_type, int want_channels, int n, void *dst,
              size_t elem) {
    int type = -1, channels = -1;
    if (fread(&type, sizeof(int), 1, f) != 1 || fread(&channels, sizeof(int), 1, f) != 1)
        return fl_fail(FL_ERR_IO, "%s: truncated before the %s field", path, what);
    if (type != want_type || channels != want_channels)
        return fl_fail(FL_ERR_IO, "%s: %s field has type %d x %d (want %d x %d)", path, what, type, channels,
                       want_type, want_channels);
    const size_t bytes = (size_t)n * elem;
    if (dst) {
        if (bytes && fread(dst, 1, bytes, f) != bytes)
            return fl_fail(FL_ERR_IO, "%s: truncated in the %s field", path, what);
    } else if (bytes && fseek(f, (long)bytes, SEEK_CUR) != 0) {
        return fl_fail(FL_ERR_IO, "%s: truncated in the %s field", path, what);
    }
    return FL_OK;
}

}  // namespace

extern "C" int fl_pts_write(const char *path, int n, const float *pos, const float *vel, const uint32_t *clr,
                            const float *veval) {
    if (!path || n < 0 || (n > 0 && (!pos || !vel || !clr)))
        return fl_fail(FL_ERR_ARG, "fl_pts_write: null path or array, or n < 0");
    FileCloser fc{fopen(path, "wb")};
    if (!fc.f) return fl_fail(FL_ERR_IO, "fl_pts_write: cannot create %s", path);
    const int nfields = veval ? 4 : 3;
    const size_t v3 = 12 * (size_t)n;
    bool ok = fwrite(&n, sizeof(int), 1, fc.f) == 1 && fwrite(&nfields, sizeof(int), 1, fc.f) == 1 &&
              put_field(fc.f, 2, 3, pos, v3) && put_field(fc.f, 2, 3, vel, v3) &&
              put_field(fc.f, 0, 4, clr, 4 * (size_t)n);
    if (ok && veval) ok = put_field(fc.f, 2, 3, veval, v3);
    if (!ok) return fl_fail(FL_ERR_IO, "fl_pts_write: writing %s failed", path);
    if (fclose(fc.f) != 0) { fc.f = nullptr; return fl_fail(FL_ERR_IO, "fl_pts_write: closing %s failed", path); }
    fc.f = nullptr;
    return FL_OK;
}

extern "C" int fl_pts_read(const char *path, int *n, int *nfields, float *pos, float *vel, uint32_t *clr,
                           float *veval) {
    if (!path || !n) return fl_fail(FL_ERR_ARG, "fl_pts_read: null path or n");
    FileCloser fc{fopen(path, "rb")};
    if (!fc.f) return fl_fail(FL_ERR_IO, "fl_pts_read: cannot open %s", path);
    int cnt = 0, nf = 0;
    if (fread(&cnt, sizeof(int), 1, fc.f) != 1 || fread(&nf, sizeof(int), 1, fc.f) != 1)
        return fl_fail(FL_ERR_IO, "%s: truncated header", path);
    if (cnt < 0 || nf < 3) return fl_fail(FL_ERR_IO, "%s: %d points, %d fields (need >= 0 and >= 3)", path, cnt, nf);
    *n = cnt;
    if (nfields) *nfields = nf;
    if (!pos && !vel && !clr && !veval) return FL_OK;   // header query
    FL_TRY(get_field(fc.f, path, "position", 2, 3, cnt, pos, 12));
    FL_TRY(get_field(fc.f, path, "velocity", 2, 3, cnt, vel, 12));
    FL_TRY(get_field(fc.f, path, "colour", 0, 4, cnt, clr, 4));
    if (veval) {
        if (nf >= 4) FL_TRY(get_field(fc.f, path, "evaluated velocity", 2, 3, cnt, veval, 12));
        else memset(veval, 0, 12 * (size_t)cnt);
    }
    return FL_OK;
}

extern "C" int fl_save_points(fl_system *s, const char *path, int with_veval) {
    if (!s || !path) return fl_fail(FL_ERR_ARG, "fl_save_points: null argument");
    const int n = s->n;
    const size_t v3 = 12 * (size_t)(n > 0 ? n : 1);
    float *pos = (float *)malloc(v3), *vel = (float *)malloc(v3), *ve = with_veval ? (float *)malloc(v3) : nullptr;
    uint32_t *clr = (uint32_t *)malloc(4 * (size_t)(n > 0 ? n : 1));
    int r = (!pos || !vel || !clr || (with_veval && !ve)) ? fl_fail(FL_ERR_NOMEM, "fl_save_points: host memory")
                                                          : FL_OK;
    if (r == FL_OK && n > 0) r = fl_get_buffer(s, FL_FPOS, pos, 12 * (size_t)n);
    if (r == FL_OK && n > 0) r = fl_get_buffer(s, FL_FVEL, vel, 12 * (size_t)n);
    if (r == FL_OK && n > 0) r = fl_get_buffer(s, FL_FCLR, clr, 4 * (size_t)n);
    if (r == FL_OK && n > 0 && ve) r = fl_get_buffer(s, FL_FVEVAL, ve, 12 * (size_t)n);
    if (r == FL_OK) r = fl_pts_write(path, n, pos, vel, clr, ve);
    free(pos); free(vel); free(ve); free(clr);
    return r;
}

extern "C" int fl_load_points(fl_system *s, const char *path) {
    if (!s || !path) return fl_fail(FL_ERR_ARG, "fl_load_points: null argument");
    int n = 0, nf = 0;
    FL_TRY(fl_pts_read(path, &n, &nf, nullptr, nullptr, nullptr, nullptr));
    if (n > s->max_points)
        return fl_fail(FL_ERR_CAPACITY, "fl_load_points: %s holds %d points (capacity %d)", path, n, s->max_points);
    const size_t v3 = 12 * (size_t)(n > 0 ? n : 1);
    float *pos = (float *)malloc(v3), *vel = (float *)malloc(v3), *ve = (float *)malloc(v3);
    uint32_t *clr = (uint32_t *)malloc(4 * (size_t)(n > 0 ? n : 1));
    int r = (!pos || !vel || !ve || !clr) ? fl_fail(FL_ERR_NOMEM, "fl_load_points: host memory") : FL_OK;
    if (r == FL_OK) r = fl_pts_read(path, &n, &nf, pos, vel, clr, ve);
    // RunPlayback (cpp:1787-1841) loads positions, velocities and colours;
    // a fourth field restores the evaluated velocity (else zero)
    if (r == FL_OK) r = fl_set_particles(s, n, pos, vel, ve, nullptr, nullptr, clr);
    free(pos); free(vel); free(ve); free(clr);
    return r;
}

// SampleParticlesCUDA (cpp:2497-2507) with SaveBricks' preparation
// (cpp:1597-1612): optionally insert + prefix sum + counting sort first,
// then one launch over the voxel lattice. gausskern and h2 as the reference
// derives them (UpdateParamsCUDA cpp:2302; fluid_kernels.cu:268, where
// 2.0 * r2 / 8.0 is evaluated in double).
extern "C" int fl_sample_volume(fl_system *s, float *out, const int res[3], const float bmin[3],
                                const float bmax[3], float scalar, int sort_first) {
    if (!s || !out || !res || !bmin || !bmax) return fl_fail(FL_ERR_ARG, "fl_sample_volume: null argument");
    if (s->batched) return fl_fail(FL_ERR_STATE, "fl_sample_volume: a batched system samples no single volume");
    if (res[0] < 1 || res[1] < 1 || res[2] < 1 || (long long)res[0] * res[1] * res[2] > (1LL << 31))
        return fl_fail(FL_ERR_ARG, "fl_sample_volume: resolution %d x %d x %d", res[0], res[1], res[2]);
    if (sort_first) {
        FL_TRY(fl_insert_particles(s, nullptr, nullptr, nullptr));
        FL_TRY(fl_prefix_sum_cells(s, nullptr, 1));
        FL_TRY(fl_counting_sort_full(s, nullptr));
    } else if (!s->have_grid || s->offsets_inclusive) {
        return fl_fail(FL_ERR_STATE, "fl_sample_volume: no sorted grid (sort_first = 1, or the phase calls first)");
    }
    const float sr = s->P.psmoothradius;
    const float gausskern = 1.0f / powf(3.141592f * 2.0f * sr * sr, 3.0f / 2.0f);
    const float h2 = (float)(2.0 * (double)s->P.r2 / 8.0);
    const size_t bytes = sizeof(float) * (size_t)res[0] * res[1] * res[2];
    cudaPointerAttributes attr;
    const bool on_device = cudaPointerGetAttributes(&attr, out) == cudaSuccess && attr.type == cudaMemoryTypeDevice;
    cudaGetLastError();
    if (on_device) {
        FL_TRY(fl_launch_sample_volume(s, res, bmin, bmax, scalar, gausskern, h2, out));
        FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
        return FL_OK;
    }
    FL_TRY(fl_ensure_stage(s, bytes));
    FL_TRY(fl_launch_sample_volume(s, res, bmin, bmax, scalar, gausskern, h2, (float *)s->stage));
    FL_CUDA_TRY(cudaMemcpyAsync(out, s->stage, bytes, cudaMemcpyDefault, s->stream));
    FL_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return FL_OK;
}
