/*
 * fluids_oracle.c -- TEST INFRASTRUCTURE ONLY: CPU oracle of the SPH step.
 *
 * A serial C restatement of the reference GPU step (fluids4.0, RUN_GPU_FULL)
 * on fluid.h-layout host arrays (float3 packed 12 B, uint 4 B). Tier 2 of
 * the oracle: FP32 in the reference kernels' own operation order (compiled
 * with -ffp-contract=off, so nothing is fused), plus FP64 restatements of
 * the density and force formulas. Tier 1 is the reference source itself
 * built on the host (ref_wrap.cpp); the tests pin this file against it.
 *
 * Within-cell order is canonical: gndx = number of lower-indexed points in
 * the same cell (serial cnt++, fluids3.9/fluid_system.cpp:489). Points
 * outside the scan range take bin C: they are placed after all in-range
 * points in index order, with gcell = GRID_UNDEF and gndx = their rank
 * there, density 0 and force 0 (upstream leaves those slots stale).
 *
 * Only tests/, bench.py's CPU arm and the smoke check load this library.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "../include/fluids_gb300.h"

#define UNDEF 0xFFFFFFFFu
#define EPS 0.00001f   /* EPSILON, fluids4.0/fluid_kernels.cuh:17 */

/* Cell of a position or C: insertParticles, fluids4.0/fluid_kernels.cu:39-43. */
static uint32_t cell_of(const fl_params *p, const float *x) {
    int gc[3];
    for (int k = 0; k < 3; k++) {
        const float g = (x[k] - p->gridMin[k]) * p->gridDelta[k];
        /* C's (int) is undefined out of range; clamp first (any value
         * outside [1, scanmax] is rejected the same way) */
        gc[k] = (g >= 2.0e9f || g != g) ? -1 : (g <= -2.0e9f ? -1 : (int)g);
    }
    if (gc[0] >= 1 && gc[0] <= p->gridScanMax[0] && gc[1] >= 1 && gc[1] <= p->gridScanMax[1] &&
        gc[2] >= 1 && gc[2] <= p->gridScanMax[2])
        return (uint32_t)((gc[1] * p->gridRes[2] + gc[2]) * p->gridRes[0] + gc[0]);
    return (uint32_t)p->gridTotal;
}

/* InsertParticles: cnt has C + 1 entries (entry C counts out-of-range points). */
void orc_insert(const fl_params *p, int n, const float *pos, uint32_t *gcell, uint32_t *gndx,
                uint32_t *cnt) {
    const uint32_t C = (uint32_t)p->gridTotal;
    memset(cnt, 0, sizeof(uint32_t) * (C + 1));
    for (int i = 0; i < n; i++) {
        const uint32_t c = cell_of(p, pos + 3 * i);
        gcell[i] = (c == C) ? UNDEF : c;
        gndx[i] = cnt[c]++;
    }
}

/* PrefixSumCells: exclusive scan over `entries` counts (fluids3.9 cpp:1059-1073). */
void orc_prefix_sum(int entries, const uint32_t *cnt, uint32_t *off) {
    uint32_t sum = 0;
    for (int c = 0; c < entries; c++) { off[c] = sum; sum += cnt[c]; }
}

/* CountingSortFull (fluids4.0/fluid_kernels.cu:56-87) over every field. */
void orc_counting_sort(const fl_params *p, int n, const uint32_t *off,
                       const float *pos, const float *vel, const float *veval, const float *force,
                       const float *press, const uint32_t *clr, const uint32_t *gcell,
                       const uint32_t *gndx,
                       float *pos_o, float *vel_o, float *veval_o, float *force_o, float *press_o,
                       uint32_t *clr_o, uint32_t *gcell_o, uint32_t *gndx_o) {
    const uint32_t C = (uint32_t)p->gridTotal;
    for (int i = 0; i < n; i++) {
        const uint32_t c = gcell[i] == UNDEF ? C : gcell[i];
        const uint32_t s = off[c] + gndx[i];
        memcpy(pos_o + 3 * s, pos + 3 * i, 12);
        memcpy(vel_o + 3 * s, vel + 3 * i, 12);
        memcpy(veval_o + 3 * s, veval + 3 * i, 12);
        memcpy(force_o + 3 * s, force + 3 * i, 12);
        press_o[s] = press[i];
        clr_o[s] = clr[i];
        gcell_o[s] = gcell[i];
        gndx_o[s] = gndx[i];
    }
}

/* computePressure (fluids4.0/fluid_kernels.cu:112-149) for sorted point i,
 * FGRID = identity. */
static float density_point(const fl_params *p, int nadj, int i, const float *pos, const uint32_t *gcell,
                           const uint32_t *off, const uint32_t *cnt) {
    if (gcell[i] == UNDEF) return 0.0f;
    const int base = (int)gcell[i] - nadj;
    const float *xi = pos + 3 * i;
    float sum = 0.0f;
    for (int c = 0; c < p->gridAdjCnt; c++) {
        const int cell = base + p->gridAdj[c];
        const uint32_t j1 = off[cell] + cnt[cell];
        for (uint32_t j = off[cell]; j < j1; j++) {
            const float *xj = pos + 3 * j;
            const float dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
            float dsq = dx * dx + dy * dy + dz * dz;
            if (dsq < p->rd2 && dsq > 0.0f) {
                dsq = (p->rd2 - dsq) * p->d2;
                sum += dsq * dsq * dsq;
            }
        }
    }
    sum = sum * p->pmass * p->poly6kern;
    if (sum == 0.0f) sum = 1.0f;
    return sum;
}

void orc_density(const fl_params *p, int n, const float *pos, const uint32_t *gcell,
                 const uint32_t *off, const uint32_t *cnt, float *press, int threads) {
    const int nadj = (1 * p->gridRes[2] + 1) * p->gridRes[0] + 1;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(threads) if (threads > 1)
    for (int i = 0; i < n; i++) press[i] = density_point(p, nadj, i, pos, gcell, off, cnt);
}

/* The same at m chosen sorted slots: out[k] is slot idx[k]'s density (a
 * sample of a large state; every other slot is still read as a neighbour). */
void orc_density_at(const fl_params *p, int m, const uint32_t *idx, const float *pos, const uint32_t *gcell,
                    const uint32_t *off, const uint32_t *cnt, float *out, int threads) {
    const int nadj = (1 * p->gridRes[2] + 1) * p->gridRes[0] + 1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads) if (threads > 1)
    for (int k = 0; k < m; k++) out[k] = density_point(p, nadj, (int)idx[k], pos, gcell, off, cnt);
}

/* The pairs computePressure's loop accepts (0 < d^2 < rd2), per sorted
 * point in visiting order, as CSR: point i's neighbour slots are
 * nbr[poff[i] .. poff[i+1]). With nbr null only poff is filled (a counting
 * pass); the frozen structure of the FP64 adjoint model (adjoint64.c). */
void orc_pairs(const fl_params *p, int n, const float *pos, const uint32_t *gcell,
               const uint32_t *off, const uint32_t *cnt, uint32_t *poff, uint32_t *nbr) {
    const int nadj = (1 * p->gridRes[2] + 1) * p->gridRes[0] + 1;
    uint32_t k = 0;
    for (int i = 0; i < n; i++) {
        poff[i] = k;
        if (gcell[i] == UNDEF) continue;
        const int base = (int)gcell[i] - nadj;
        const float *xi = pos + 3 * i;
        for (int c = 0; c < p->gridAdjCnt; c++) {
            const int cell = base + p->gridAdj[c];
            const uint32_t j1 = off[cell] + cnt[cell];
            for (uint32_t j = off[cell]; j < j1; j++) {
                const float *xj = pos + 3 * j;
                const float dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
                const float dsq = dx * dx + dy * dy + dz * dz;
                if (dsq < p->rd2 && dsq > 0.0f) {
                    if (nbr) nbr[k] = j;
                    k++;
                }
            }
        }
    }
    poff[n] = k;
}

/* sampleParticles (fluids4.0/fluid_kernels.cu:263-308) over a sorted state
 * (FGRID = identity): voxel (x, y, z) at bmin + i / res * (bmax - bmin),
 * out[(z * res[1] + y) * res[0] + x] = scalar * sum gausskern * exp(-r^2 / h2)
 * over the search block's particles within the smoothing radius; 0 where
 * the voxel lies outside the scan range. FP32 in the reference's order
 * (libm expf here, CUDA's expf on the device: the sums agree to ~1e-6). */
void orc_sample_volume(const fl_params *p, const float *pos, const uint32_t *off, const uint32_t *cnt,
                       const int *res, const float *bmin, const float *bmax, float scalar, float gausskern,
                       float h2, float *out) {
    const int nadj = (1 * p->gridRes[2] + 1) * p->gridRes[0] + 1;
    for (int z = 0; z < res[2]; z++)
        for (int y = 0; y < res[1]; y++)
            for (int x = 0; x < res[0]; x++) {
                float q[3];
                const int ix[3] = {x, y, z};
                for (int k = 0; k < 3; k++) q[k] = bmin[k] + ((float)ix[k] / (float)res[k]) * (bmax[k] - bmin[k]);
                const size_t idx = ((size_t)z * res[1] + y) * res[0] + x;
                const uint32_t c = cell_of(p, q);
                if (c == (uint32_t)p->gridTotal) { out[idx] = 0.0f; continue; }
                const int base = (int)c - nadj;
                float v = 0.0f;
                for (int a = 0; a < p->gridAdjCnt; a++) {
                    const int cell = base + p->gridAdj[a];
                    for (uint32_t j = off[cell]; j < off[cell] + cnt[cell]; j++) {
                        const float dx = q[0] - pos[3 * j], dy = q[1] - pos[3 * j + 1], dz = q[2] - pos[3 * j + 2];
                        float dsq = dx * dx + dy * dy + dz * dz;
                        if (dsq < p->rd2 && dsq > 0.0f) {
                            dsq = sqrtf(dsq * p->d2);
                            v += gausskern * expf(-(dsq * dsq) / h2);
                        }
                    }
                }
                out[idx] = v * scalar;
            }
}

/* computeForce (fluids4.0/fluid_kernels.cu:180-217) for sorted point i; the
 * float3 operators of cutil_math.h expand component-wise, and '/ s' is
 * '* (1.0f / s)'. */
static void force_point(const fl_params *p, int nadj, int i, const float *pos, const float *veval,
                        const float *press, const uint32_t *gcell, const uint32_t *off,
                        const uint32_t *cnt, float *fo) {
    if (gcell[i] == UNDEF) { fo[0] = fo[1] = fo[2] = 0.0f; return; }
    const int base = (int)gcell[i] - nadj;
    const float *xi = pos + 3 * i, *vi = veval + 3 * i;
    const float di = press[i];
    const float pi = (di - p->prest_dens) * p->pintstiff;
    float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f;
    for (int c = 0; c < p->gridAdjCnt; c++) {
        const int cell = base + p->gridAdj[c];
        const uint32_t j1 = off[cell] + cnt[cell];
        for (uint32_t j = off[cell]; j < j1; j++) {
            const float *xj = pos + 3 * j, *vj = veval + 3 * j;
            const float dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
            const float dsq = dx * dx + dy * dy + dz * dz;
            if (dsq < p->rd2 && dsq > 0.0f) {
                const float r = sqrtf(dsq * p->d2);
                const float dj = press[j];
                const float pj = (dj - p->prest_dens) * p->pintstiff;
                const float cr = p->psmoothradius - r;
                const float pterm = p->sim_scale * -0.5f * cr * p->spikykern * (pi + pj) / r;
                const float sx = dx * pterm + (vj[0] - vi[0]) * p->vterm;
                const float sy = dy * pterm + (vj[1] - vi[1]) * p->vterm;
                const float sz = dz * pterm + (vj[2] - vi[2]) * p->vterm;
                const float inv = 1.0f / (di * dj);
                f0 += (sx * cr) * inv;
                f1 += (sy * cr) * inv;
                f2 += (sz * cr) * inv;
            }
        }
    }
    fo[0] = f0; fo[1] = f1; fo[2] = f2;
}

void orc_force(const fl_params *p, int n, const float *pos, const float *veval,
               const float *press, const uint32_t *gcell, const uint32_t *off,
               const uint32_t *cnt, float *force, int threads) {
    const int nadj = (1 * p->gridRes[2] + 1) * p->gridRes[0] + 1;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(threads) if (threads > 1)
    for (int i = 0; i < n; i++) force_point(p, nadj, i, pos, veval, press, gcell, off, cnt, force + 3 * i);
}

/* The same at m chosen sorted slots: out[3k..3k+2] is slot idx[k]'s force. */
void orc_force_at(const fl_params *p, int m, const uint32_t *idx, const float *pos, const float *veval,
                  const float *press, const uint32_t *gcell, const uint32_t *off, const uint32_t *cnt,
                  float *out, int threads) {
    const int nadj = (1 * p->gridRes[2] + 1) * p->gridRes[0] + 1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads) if (threads > 1)
    for (int k = 0; k < m; k++) force_point(p, nadj, (int)idx[k], pos, veval, press, gcell, off, cnt, out + 3 * k);
}

/* advanceParticles (fluids4.0/fluid_kernels.cu:332-420), in place. The
 * moving-wall term is evaluated like the reference source: sin of a float,
 * then '* 0.5 + 0.5' and the amplitude product in double. */
void orc_advance(const fl_params *p, int n, float time, float dt, float ss,
                 const uint32_t *gcell, const float *force, float *pos, float *vel,
                 float *veval, int threads) {
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
    for (int i = 0; i < n; i++) {
        float *x = pos + 3 * i, *v = vel + 3 * i, *e = veval + 3 * i;
        if (gcell[i] == UNDEF) {
            x[0] = x[1] = x[2] = -1000.0f;
            v[0] = v[1] = v[2] = 0.0f;
            continue;
        }
        float ax = force[3 * i] * p->pmass, ay = force[3 * i + 1] * p->pmass, az = force[3 * i + 2] * p->pmass;
        const float px = x[0], py = x[1], pz = x[2];
        const float ex = e[0], ey = e[1], ez = e[2];
        float diff, adj, nx, ny, nz;
        /* Y- with slope */
        diff = p->pradius - (py - (p->bound_min[1] + (px - p->bound_min[0]) * p->bound_slope)) * ss;
        if (diff > EPS) {
            nx = -p->bound_slope; ny = 1.0f - p->bound_slope; nz = 0.0f;
            adj = p->bound_stiff * diff - p->bound_damp * (nx * ex + ny * ey + nz * ez);
            nx *= adj; ny *= adj; nz *= adj;
            ax += nx - ex * p->bound_friction;
            ay += ny - ey * p->bound_friction;
            az += nz - ez * p->bound_friction;
        }
        /* Y+ */
        diff = p->pradius - (p->bound_max[1] - py) * ss;
        if (diff > EPS) {
            nx = 0.0f; ny = -1.0f; nz = 0.0f;
            adj = p->bound_stiff * diff - p->bound_damp * (nx * ex + ny * ey + nz * ez);
            nx *= adj; ny *= adj; nz *= adj;
            ax += nx - ex * p->bound_friction;
            ay += ny - ey * p->bound_friction;
            az += nz - ez * p->bound_friction;
        }
        /* X- moving wall */
        const float wall = (float)(((double)sinf(time * p->bound_wall_freq + pz / 400.f) * 0.5 + 0.5) *
                                   (double)p->bound_wall_force);
        diff = p->pradius - (px - (p->bound_min[0] + wall)) * ss;
        if (diff > EPS) {
            nx = 1.0f; ny = 0.0f; nz = 0.0f;
            adj = wall * p->bound_stiff * diff - p->bound_damp * (nx * ex + ny * ey + nz * ez);
            ax += nx * adj; ay += ny * adj; az += nz * adj;
        }
        /* X+ */
        diff = p->pradius - (p->bound_max[0] - px) * ss;
        if (diff > EPS) {
            nx = -1.0f; ny = 0.0f; nz = 0.0f;
            adj = p->bound_stiff * diff - p->bound_damp * (nx * ex + ny * ey + nz * ez);
            ax += nx * adj; ay += ny * adj; az += nz * adj;
        }
        /* Z- */
        diff = p->pradius - (pz - p->bound_min[2]) * ss;
        if (diff > EPS) {
            nx = 0.0f; ny = 0.0f; nz = 1.0f;
            adj = p->bound_stiff * diff - p->bound_damp * (nx * ex + ny * ey + nz * ez);
            ax += nx * adj; ay += ny * adj; az += nz * adj;
        }
        /* Z+ */
        diff = p->pradius - (p->bound_max[2] - pz) * ss;
        if (diff > EPS) {
            nx = 0.0f; ny = 0.0f; nz = -1.0f;
            adj = p->bound_stiff * diff - p->bound_damp * (nx * ex + ny * ey + nz * ez);
            ax += nx * adj; ay += ny * adj; az += nz * adj;
        }
        ax += p->gravity[0]; ay += p->gravity[1]; az += p->gravity[2];
        float speed = ax * ax + ay * ay + az * az;
        if (speed > p->AL2) {
            const float k = p->AL / sqrtf(speed);
            ax *= k; ay *= k; az *= k;
        }
        float vx = v[0], vy = v[1], vz = v[2];
        speed = vx * vx + vy * vy + vz * vz;
        if (speed > p->VL2) {
            const float k = p->VL / sqrtf(speed);
            vx *= k; vy *= k; vz *= k;
        }
        const float nvx = ax * dt + vx, nvy = ay * dt + vy, nvz = az * dt + vz;
        e[0] = (vx + nvx) * 0.5f; e[1] = (vy + nvy) * 0.5f; e[2] = (vz + nvz) * 0.5f;
        v[0] = nvx; v[1] = nvy; v[2] = nvz;
        const float dts = dt / ss;
        x[0] = px + nvx * dts; x[1] = py + nvy * dts; x[2] = pz + nvz * dts;
    }
}

/* ---- FP64 restatements ---------------------------------------------------
 * Same candidate cells, same formulas (poly6 density; spiky pressure plus
 * viscosity-Laplacian force), every operation in double. The force takes
 * the densities as input so that it checks the force pass alone. */
static double density_point_f64(const fl_params *p, int nadj, int i, const float *pos, const uint32_t *gcell,
                                const uint32_t *off, const uint32_t *cnt) {
    const double ss = p->sim_scale, h = p->psmoothradius;
    const double rd2 = (h * h) / (ss * ss), d2 = ss * ss;
    const double poly6 = 315.0 / (64.0 * M_PI * pow(h, 9.0));
    if (gcell[i] == UNDEF) return 0.0;
    const int base = (int)gcell[i] - nadj;
    double sum = 0.0;
    for (int c = 0; c < p->gridAdjCnt; c++) {
        const int cell = base + p->gridAdj[c];
        const uint32_t j1 = off[cell] + cnt[cell];
        for (uint32_t j = off[cell]; j < j1; j++) {
            const double dx = (double)pos[3 * i] - pos[3 * j];
            const double dy = (double)pos[3 * i + 1] - pos[3 * j + 1];
            const double dz = (double)pos[3 * i + 2] - pos[3 * j + 2];
            const double dsq = dx * dx + dy * dy + dz * dz;
            if (dsq < rd2 && dsq > 0.0) {
                const double t = (rd2 - dsq) * d2;
                sum += t * t * t;
            }
        }
    }
    const double rho = sum * (double)p->pmass * poly6;
    return (rho == 0.0) ? 1.0 : rho;
}

void orc_density_f64(const fl_params *p, int n, const float *pos, const uint32_t *gcell,
                     const uint32_t *off, const uint32_t *cnt, double *press, int threads) {
    const int nadj = (1 * p->gridRes[2] + 1) * p->gridRes[0] + 1;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(threads) if (threads > 1)
    for (int i = 0; i < n; i++) press[i] = density_point_f64(p, nadj, i, pos, gcell, off, cnt);
}

void orc_density_f64_at(const fl_params *p, int m, const uint32_t *idx, const float *pos,
                        const uint32_t *gcell, const uint32_t *off, const uint32_t *cnt, double *out,
                        int threads) {
    const int nadj = (1 * p->gridRes[2] + 1) * p->gridRes[0] + 1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads) if (threads > 1)
    for (int k = 0; k < m; k++) out[k] = density_point_f64(p, nadj, (int)idx[k], pos, gcell, off, cnt);
}

/* scale (nullable): per point, the sum of the magnitudes of its pair terms --
 * the bound that an FP32 evaluation's error is proportional to. */
static void force_point_f64(const fl_params *p, int nadj, int i, const float *pos, const float *veval,
                            const float *press, const uint32_t *gcell, const uint32_t *off,
                            const uint32_t *cnt, double *fo, double *scale) {
    const double ss = p->sim_scale, h = p->psmoothradius;
    const double rd2 = (h * h) / (ss * ss), d2 = ss * ss;
    const double spiky = -45.0 / (M_PI * pow(h, 6.0));
    const double vterm = 45.0 / (M_PI * pow(h, 6.0)) * (double)p->pvisc;
    const double rest = p->prest_dens, stiff = p->pintstiff;
    double sc = 0.0;
    fo[0] = fo[1] = fo[2] = 0.0;
    if (scale) *scale = 0.0;
    if (gcell[i] == UNDEF) return;
    const int base = (int)gcell[i] - nadj;
    const double di = press[i], pi = (di - rest) * stiff;
    for (int c = 0; c < p->gridAdjCnt; c++) {
        const int cell = base + p->gridAdj[c];
        const uint32_t j1 = off[cell] + cnt[cell];
        for (uint32_t j = off[cell]; j < j1; j++) {
            double d[3], dsq = 0.0;
            for (int k = 0; k < 3; k++) {
                d[k] = (double)pos[3 * i + k] - pos[3 * j + k];
                dsq += d[k] * d[k];
            }
            if (dsq < rd2 && dsq > 0.0) {
                const double r = sqrt(dsq * d2);
                const double dj = press[j], pj = (dj - rest) * stiff;
                const double cr = h - r;
                const double pterm = -0.5 * ss * cr * spiky * (pi + pj) / r;
                double t2 = 0.0;
                for (int k = 0; k < 3; k++) {
                    const double t = (d[k] * pterm + ((double)veval[3 * j + k] - veval[3 * i + k]) * vterm) *
                                     cr / (di * dj);
                    fo[k] += t;
                    t2 += t * t;
                }
                sc += sqrt(t2);
            }
        }
    }
    if (scale) *scale = sc;
}

void orc_force_f64(const fl_params *p, int n, const float *pos, const float *veval,
                   const float *press, const uint32_t *gcell, const uint32_t *off,
                   const uint32_t *cnt, double *force, double *scale, int threads) {
    const int nadj = (1 * p->gridRes[2] + 1) * p->gridRes[0] + 1;
#pragma omp parallel for schedule(dynamic, 1024) num_threads(threads) if (threads > 1)
    for (int i = 0; i < n; i++)
        force_point_f64(p, nadj, i, pos, veval, press, gcell, off, cnt, force + 3 * i, scale ? scale + i : NULL);
}

void orc_force_f64_at(const fl_params *p, int m, const uint32_t *idx, const float *pos, const float *veval,
                      const float *press, const uint32_t *gcell, const uint32_t *off, const uint32_t *cnt,
                      double *force, double *scale, int threads) {
    const int nadj = (1 * p->gridRes[2] + 1) * p->gridRes[0] + 1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads) if (threads > 1)
    for (int k = 0; k < m; k++)
        force_point_f64(p, nadj, (int)idx[k], pos, veval, press, gcell, off, cnt, force + 3 * k,
                        scale ? scale + k : NULL);
}

/* ---- one full step -------------------------------------------------------
 * Run, RUN_GPU_FULL (fluids4.0/fluid_system.cpp:506-524) on host arrays.
 * `a` holds the state and receives the result; `t` is same-sized scratch.
 * cnt/off need C + 1 entries. *time advances by dt (AdvanceTime, cpp:529). */
typedef struct orc_bufs {
    float *pos, *vel, *veval, *force, *press;
    uint32_t *clr, *gcell, *gndx;
} orc_bufs;

void orc_step(const fl_params *p, int n, orc_bufs *a, orc_bufs *t, uint32_t *cnt, uint32_t *off,
              float *time, int threads) {
    orc_insert(p, n, a->pos, a->gcell, a->gndx, cnt);
    orc_prefix_sum(p->gridTotal + 1, cnt, off);
    orc_counting_sort(p, n, off, a->pos, a->vel, a->veval, a->force, a->press, a->clr, a->gcell,
                      a->gndx, t->pos, t->vel, t->veval, t->force, t->press, t->clr, t->gcell,
                      t->gndx);
    orc_bufs tmp = *a; *a = *t; *t = tmp;
    orc_density(p, n, a->pos, a->gcell, off, cnt, a->press, threads);
    orc_force(p, n, a->pos, a->veval, a->press, a->gcell, off, cnt, a->force, threads);
    orc_advance(p, n, *time, p->dt, p->sim_scale, a->gcell, a->force, a->pos, a->vel, a->veval, threads);
    *time += p->dt;
}

/* `steps` steps on caller-owned fluid.h arrays; results land in the first
 * set (`x*`), the second set is scratch. For timing the CPU baseline. */
void orc_run(const fl_params *p, int n, int steps, float *time, int threads,
             float *pos, float *vel, float *veval, float *force, float *press,
             uint32_t *clr, uint32_t *gcell, uint32_t *gndx,
             float *pos2, float *vel2, float *veval2, float *force2, float *press2,
             uint32_t *clr2, uint32_t *gcell2, uint32_t *gndx2,
             uint32_t *cnt, uint32_t *off) {
    orc_bufs a = {pos, vel, veval, force, press, clr, gcell, gndx};
    orc_bufs b = {pos2, vel2, veval2, force2, press2, clr2, gcell2, gndx2};
    const orc_bufs first = a;
    for (int s = 0; s < steps; s++) orc_step(p, n, &a, &b, cnt, off, time, threads);
    if (a.pos != first.pos) {
        /* an odd number of swaps left the result in the scratch set */
        memcpy(first.pos, a.pos, 12 * (size_t)n); memcpy(first.vel, a.vel, 12 * (size_t)n);
        memcpy(first.veval, a.veval, 12 * (size_t)n); memcpy(first.force, a.force, 12 * (size_t)n);
        memcpy(first.press, a.press, 4 * (size_t)n); memcpy(first.clr, a.clr, 4 * (size_t)n);
        memcpy(first.gcell, a.gcell, 4 * (size_t)n); memcpy(first.gndx, a.gndx, 4 * (size_t)n);
    }
}
