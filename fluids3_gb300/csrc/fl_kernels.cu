// SPH step kernels for sm_103a.
//
// Compiled with --fmad=false: every float expression rounds exactly as
// written, in the order the reference kernels write it
// (fluids4.0/fluid_kernels.cu), so grid cells are bit-identical and the
// density/force/advance sums match a host evaluation of the same order.
// Math is IEEE (no fast-math): sqrtf and '/' are correctly rounded.
//
// HBM layout: positions, velocities, evaluated velocities and forces are
// float4 (16 B aligned, one vector load per particle); density, colour,
// cell and within-cell index are 4-byte scalars. All particle fields are
// held twice (see Field in fl_internal.h).
#include <stdio.h>

#include "fl_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr uint32_t kUndef = FL_GRID_UNDEF;
constexpr float kEpsilon = 0.00001f;   // EPSILON, fluids4.0/fluid_kernels.cuh:17

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// ---------------------------------------------------------------------------
// Grid cell of a position: insertParticles, fluids4.0/fluid_kernels.cu:39-43.
// Returns C (the out-of-range bin) when the cell is outside [1, gridScanMax].
__device__ __forceinline__ uint32_t cell_of(const DevParams &P, float4 p) {
    const float gx = (p.x - P.gridMin.x) * P.gridDelta.x;
    const float gy = (p.y - P.gridMin.y) * P.gridDelta.y;
    const float gz = (p.z - P.gridMin.z) * P.gridDelta.z;
    const int cx = __float2int_rz(gx), cy = __float2int_rz(gy), cz = __float2int_rz(gz);
    if (cx >= 1 && cx <= P.gridScanMax.x && cy >= 1 && cy <= P.gridScanMax.y &&
        cz >= 1 && cz <= P.gridScanMax.z)
        return (uint32_t)((cy * P.gridRes.z + cz) * P.gridRes.x + cx);
    return (uint32_t)P.ncells;
}

// insertParticles (fluids4.0/fluid_kernels.cu:22-53) with warp-aggregated
// counting: lanes of a warp that land in the same cell elect one leader,
// which adds the group size with a single atomic; each lane's arrival rank is
// the group's base plus its position among the group's lanes. The rank is
// only an intermediate: the canonical within-cell order is fixed later by
// k_sort_cells.
__global__ void __launch_bounds__(kThreads)
k_insert(const __grid_constant__ DevParams P, int n, const float4 *__restrict__ pos,
         uint32_t *__restrict__ cell_out, uint32_t *__restrict__ rank_out,
         uint32_t *__restrict__ gcell_out, uint32_t *__restrict__ cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    uint32_t cell = 0;
    if (valid) {
        cell = cell_of(P, pos[i]);
        cell_out[i] = cell;
        if (gcell_out) gcell_out[i] = (cell == (uint32_t)P.ncells) ? kUndef : cell;
    }
    const unsigned active = __ballot_sync(0xffffffffu, valid);
    if (!valid) return;
    const unsigned peers = __match_any_sync(active, cell);
    const int leader = __ffs(peers) - 1;
    const unsigned lane = lane_id();
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(&cnt[cell], (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    rank_out[i] = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

// Place each point's index at its arrival slot inside its cell's segment.
__global__ void __launch_bounds__(kThreads)
k_scatter_index(int n, const uint32_t *__restrict__ cell_pre, const uint32_t *__restrict__ rank,
                const uint32_t *__restrict__ off, uint32_t *__restrict__ src) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    src[off[cell_pre[i]] + rank[i]] = (uint32_t)i;
}

// ---------------------------------------------------------------------------
// Canonical within-cell order. Each warp owns one cell segment of src and
// sorts its point indices ascending, so slot off[c]+k holds the k-th lowest
// index in cell c -- the order a serial insert (gndx = cnt[cell]++) yields.
// Segments up to 1024 points are sorted in registers by a warp bitonic
// network (K keys per lane, element e = lane*K + r); larger ones take a
// counting-rank path.
template <int K>
__device__ __forceinline__ void warp_bitonic(uint32_t (&v)[K]) {
    const unsigned lane = lane_id();
#pragma unroll
    for (int size = 2; size <= 32 * K; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= K) {
                const int lstride = stride / K;
#pragma unroll
                for (int r = 0; r < K; r++) {
                    const unsigned e = lane * K + r;
                    const uint32_t other = __shfl_xor_sync(0xffffffffu, v[r], lstride);
                    const bool up = (e & size) == 0;
                    const bool lower = (e & stride) == 0;
                    v[r] = (lower == up) ? min(v[r], other) : max(v[r], other);
                }
            } else {
#pragma unroll
                for (int r = 0; r < K; r++) {
                    if ((r & stride) == 0) {
                        const int r2 = r | stride;
                        const unsigned e = lane * K + r;
                        const bool up = (e & size) == 0;
                        const uint32_t a = v[r], b = v[r2];
                        if ((a > b) == up) { v[r] = b; v[r2] = a; }
                    }
                }
            }
        }
    }
}

struct SortArgs {
    const uint32_t *off, *cnt;
    uint32_t *src, *scratch;
    uint32_t *gndx_pre;                // mode 0: canonical gndx by pre-sort index
    // mode 1 gather
    const float4 *pos_in, *vel_in, *veval_in;
    const uint32_t *clr_in;
    float4 *pos_out, *vel_out, *veval_out;
    uint32_t *clr_out, *gcell_out, *gndx_out;
    int ncells;
};

template <int MODE>
__device__ __forceinline__ void emit_slot(const SortArgs &a, int c, uint32_t o, uint32_t k, uint32_t i) {
    if (MODE == 0) {
        a.gndx_pre[i] = k;
    } else {
        const uint32_t s = o + k;
        a.pos_out[s] = a.pos_in[i];
        a.vel_out[s] = a.vel_in[i];
        a.veval_out[s] = a.veval_in[i];
        a.clr_out[s] = a.clr_in[i];
        a.gcell_out[s] = (c == a.ncells) ? kUndef : (uint32_t)c;
        a.gndx_out[s] = k;
    }
}

template <int MODE, int K>
__device__ __forceinline__ void sort_segment(const SortArgs &a, int c, uint32_t o, uint32_t m) {
    const unsigned lane = lane_id();
    uint32_t v[K];
#pragma unroll
    for (int r = 0; r < K; r++) {
        const uint32_t e = lane * K + r;
        v[r] = (e < m) ? a.src[o + e] : 0xffffffffu;
    }
    warp_bitonic<K>(v);
    if constexpr (K == 1) {
        if (lane < m) {
            if (MODE == 0) a.src[o + lane] = v[0];
            emit_slot<MODE>(a, c, o, lane, v[0]);
        }
    } else {
#pragma unroll
        for (int r = 0; r < K; r++) {
            const uint32_t e = lane * K + r;
            if (e < m) a.src[o + e] = v[r];
        }
        __syncwarp();
        for (uint32_t k = lane; k < m; k += 32) emit_slot<MODE>(a, c, o, k, a.src[o + k]);
    }
}

template <int MODE>
__device__ void sort_segment_dense(const SortArgs &a, int c, uint32_t o, uint32_t m) {
    // rank of each key = number of smaller keys in the segment (keys are distinct)
    const unsigned lane = lane_id();
    for (uint32_t k = lane; k < m; k += 32) {
        const uint32_t key = a.src[o + k];
        uint32_t rank = 0;
        for (uint32_t u = 0; u < m; u++) rank += (a.src[o + u] < key);
        a.scratch[o + rank] = key;
    }
    __syncwarp();
    for (uint32_t k = lane; k < m; k += 32) a.src[o + k] = a.scratch[o + k];
    __syncwarp();
    for (uint32_t k = lane; k < m; k += 32) emit_slot<MODE>(a, c, o, k, a.src[o + k]);
}

template <int MODE>
__global__ void __launch_bounds__(kThreads)
k_sort_cells(const __grid_constant__ SortArgs a) {
    const int c = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
    if (c > a.ncells) return;
    const uint32_t m = a.cnt[c];
    if (m == 0) return;
    const uint32_t o = a.off[c];
    if (m <= 32) sort_segment<MODE, 1>(a, c, o, m);
    else if (m <= 64) sort_segment<MODE, 2>(a, c, o, m);
    else if (m <= 128) sort_segment<MODE, 4>(a, c, o, m);
    else if (m <= 256) sort_segment<MODE, 8>(a, c, o, m);
    else if (m <= 512) sort_segment<MODE, 16>(a, c, o, m);
    else if (m <= 1024) sort_segment<MODE, 32>(a, c, o, m);
    else sort_segment_dense<MODE>(a, c, o, m);
}

// Phase-API counting sort (countingSortFull, fluids4.0/fluid_kernels.cu:56-87)
// as a gather through the canonical src: every field moves cur -> nxt.
__global__ void __launch_bounds__(kThreads)
k_gather_all(int n, const uint32_t *__restrict__ src,
             const float4 *__restrict__ pos, const float4 *__restrict__ vel,
             const float4 *__restrict__ veval, const float4 *__restrict__ force,
             const float *__restrict__ press, const uint32_t *__restrict__ clr,
             const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ gndx,
             float4 *__restrict__ pos_o, float4 *__restrict__ vel_o,
             float4 *__restrict__ veval_o, float4 *__restrict__ force_o,
             float *__restrict__ press_o, uint32_t *__restrict__ clr_o,
             uint32_t *__restrict__ gcell_o, uint32_t *__restrict__ gndx_o) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t i = src[s];
    pos_o[s] = pos[i];
    vel_o[s] = vel[i];
    veval_o[s] = veval[i];
    force_o[s] = force[i];
    press_o[s] = press[i];
    clr_o[s] = clr[i];
    gcell_o[s] = gcell[i];
    gndx_o[s] = gndx[i];
}

// ---------------------------------------------------------------------------
// computePressure (fluids4.0/fluid_kernels.cu:112-149). FGRID is the
// identity after a full sort (cu:83), so neighbour slots are read directly.
__global__ void __launch_bounds__(kThreads)
k_density(const __grid_constant__ DevParams P, int n, const float4 *__restrict__ pos,
          const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off,
          const uint32_t *__restrict__ cnt, float *__restrict__ press) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t gc = gcell[i];
    if (gc == kUndef) { press[i] = 0.0f; return; }
    const int base = (int)gc - P.nadj;
    const float4 p = pos[i];
    float sum = 0.0f;
    for (int c = 0; c < P.gridAdjCnt; c++) {
        const int cell = base + P.adj[c];
        const uint32_t j0 = off[cell], j1 = j0 + cnt[cell];
        for (uint32_t j = j0; j < j1; j++) {
            const float4 q = pos[j];
            const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
            float dsq = dx * dx + dy * dy + dz * dz;
            if (dsq < P.rd2 && dsq > 0.0f) {
                dsq = (P.rd2 - dsq) * P.d2;
                sum += dsq * dsq * dsq;
            }
        }
    }
    sum = sum * P.pmass * P.poly6kern;
    if (sum == 0.0f) sum = 1.0f;
    press[i] = sum;
}

// computeForce's pair loop (fluids4.0/fluid_kernels.cu:180-217), same
// operation order; returns the SPH force on point i.
__device__ __forceinline__ float3 force_sum(const DevParams &P, int i, uint32_t gc,
                                            const float4 *__restrict__ pos,
                                            const float4 *__restrict__ veval,
                                            const float *__restrict__ press,
                                            const uint32_t *__restrict__ off,
                                            const uint32_t *__restrict__ cnt) {
    const int base = (int)gc - P.nadj;
    const float4 p = pos[i];
    const float4 vi = veval[i];
    const float di = press[i];
    const float pi = (di - P.prest_dens) * P.pintstiff;
    float3 f = make_float3(0.0f, 0.0f, 0.0f);
    for (int c = 0; c < P.gridAdjCnt; c++) {
        const int cell = base + P.adj[c];
        const uint32_t j0 = off[cell], j1 = j0 + cnt[cell];
        for (uint32_t j = j0; j < j1; j++) {
            const float4 q = pos[j];
            const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
            const float dsq = dx * dx + dy * dy + dz * dz;
            if (dsq < P.rd2 && dsq > 0.0f) {
                const float r = sqrtf(dsq * P.d2);
                const float dj = press[j];
                const float pj = (dj - P.prest_dens) * P.pintstiff;
                const float cr = P.psmoothradius - r;
                const float pterm = P.sim_scale * -0.5f * cr * P.spikykern * (pi + pj) / r;
                const float4 vj = veval[j];
                const float sx = dx * pterm + (vj.x - vi.x) * P.vterm;
                const float sy = dy * pterm + (vj.y - vi.y) * P.vterm;
                const float sz = dz * pterm + (vj.z - vi.z) * P.vterm;
                const float inv = 1.0f / (di * dj);
                f.x += (sx * cr) * inv;
                f.y += (sy * cr) * inv;
                f.z += (sz * cr) * inv;
            }
        }
    }
    return f;
}

__global__ void __launch_bounds__(kThreads)
k_force(const __grid_constant__ DevParams P, int n, const float4 *__restrict__ pos,
        const float4 *__restrict__ veval, const float *__restrict__ press,
        const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off,
        const uint32_t *__restrict__ cnt, float4 *__restrict__ force) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t gc = gcell[i];
    if (gc == kUndef) { force[i] = make_float4(0.f, 0.f, 0.f, 0.f); return; }
    const float3 f = force_sum(P, i, gc, pos, veval, press, off, cnt);
    force[i] = make_float4(f.x, f.y, f.z, 0.0f);
}

// advanceParticles body (fluids4.0/fluid_kernels.cu:343-419) for an
// in-range point: walls, gravity, limits, leapfrog. `accel` enters as the
// SPH force; returns the new position, velocity and evaluated velocity.
__device__ __forceinline__ void advance_point(const DevParams &P, float time, float dt, float ss,
                                              float3 accel, float3 pos, float3 vel, float3 veval,
                                              float3 &pos_o, float3 &vel_o, float3 &veval_o) {
    accel.x *= P.pmass; accel.y *= P.pmass; accel.z *= P.pmass;
    float diff, adj;
    // Y- wall with slope (cu:356-361)
    diff = P.pradius - (pos.y - (P.bound_min.y + (pos.x - P.bound_min.x) * P.bound_slope)) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(-P.bound_slope, 1.0f - P.bound_slope, 0.0f);
        adj = P.bound_stiff * diff - P.bound_damp * (nrm.x * veval.x + nrm.y * veval.y + nrm.z * veval.z);
        nrm.x *= adj; nrm.y *= adj; nrm.z *= adj;
        accel.x += nrm.x - veval.x * P.bound_friction;
        accel.y += nrm.y - veval.y * P.bound_friction;
        accel.z += nrm.z - veval.z * P.bound_friction;
    }
    // Y+ (cu:363-368)
    diff = P.pradius - (P.bound_max.y - pos.y) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(0.0f, -1.0f, 0.0f);
        adj = P.bound_stiff * diff - P.bound_damp * (nrm.x * veval.x + nrm.y * veval.y + nrm.z * veval.z);
        nrm.x *= adj; nrm.y *= adj; nrm.z *= adj;
        accel.x += nrm.x - veval.x * P.bound_friction;
        accel.y += nrm.y - veval.y * P.bound_friction;
        accel.z += nrm.z - veval.z * P.bound_friction;
    }
    // X- moving wall (cu:371-377): stiffness scaled by the wall term
    const float wall = (sinf(time * P.bound_wall_freq + pos.z / 400.f) * 0.5f + 0.5f) * P.bound_wall_force;
    diff = P.pradius - (pos.x - (P.bound_min.x + wall)) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(1.0f, 0.0f, 0.0f);
        adj = wall * P.bound_stiff * diff - P.bound_damp * (nrm.x * veval.x + nrm.y * veval.y + nrm.z * veval.z);
        accel.x += nrm.x * adj; accel.y += nrm.y * adj; accel.z += nrm.z * adj;
    }
    // X+ (cu:378-383)
    diff = P.pradius - (P.bound_max.x - pos.x) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(-1.0f, 0.0f, 0.0f);
        adj = P.bound_stiff * diff - P.bound_damp * (nrm.x * veval.x + nrm.y * veval.y + nrm.z * veval.z);
        accel.x += nrm.x * adj; accel.y += nrm.y * adj; accel.z += nrm.z * adj;
    }
    // Z- (cu:386-391)
    diff = P.pradius - (pos.z - P.bound_min.z) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(0.0f, 0.0f, 1.0f);
        adj = P.bound_stiff * diff - P.bound_damp * (nrm.x * veval.x + nrm.y * veval.y + nrm.z * veval.z);
        accel.x += nrm.x * adj; accel.y += nrm.y * adj; accel.z += nrm.z * adj;
    }
    // Z+ (cu:392-397)
    diff = P.pradius - (P.bound_max.z - pos.z) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(0.0f, 0.0f, -1.0f);
        adj = P.bound_stiff * diff - P.bound_damp * (nrm.x * veval.x + nrm.y * veval.y + nrm.z * veval.z);
        accel.x += nrm.x * adj; accel.y += nrm.y * adj; accel.z += nrm.z * adj;
    }
    accel.x += P.gravity.x; accel.y += P.gravity.y; accel.z += P.gravity.z;
    // accel limit (cu:403-406)
    float speed = accel.x * accel.x + accel.y * accel.y + accel.z * accel.z;
    if (speed > P.AL2) {
        const float k = P.AL / sqrtf(speed);
        accel.x *= k; accel.y *= k; accel.z *= k;
    }
    // velocity limit (cu:409-413)
    speed = vel.x * vel.x + vel.y * vel.y + vel.z * vel.z;
    if (speed > P.VL2) {
        const float k = P.VL / sqrtf(speed);
        vel.x *= k; vel.y *= k; vel.z *= k;
    }
    // leapfrog (cu:416-419)
    const float3 vnext = make_float3(accel.x * dt + vel.x, accel.y * dt + vel.y, accel.z * dt + vel.z);
    veval_o = make_float3((vel.x + vnext.x) * 0.5f, (vel.y + vnext.y) * 0.5f, (vel.z + vnext.z) * 0.5f);
    vel_o = vnext;
    const float dts = dt / ss;
    pos_o = make_float3(pos.x + vnext.x * dts, pos.y + vnext.y * dts, pos.z + vnext.z * dts);
}

__device__ __forceinline__ float3 xyz(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float4 f4(float3 v) { return make_float4(v.x, v.y, v.z, 0.0f); }

// advanceParticles (fluids4.0/fluid_kernels.cu:332-420), in place.
__global__ void __launch_bounds__(kThreads)
k_advance(const __grid_constant__ DevParams P, int n, float time, float dt, float ss,
          const uint32_t *__restrict__ gcell, const float4 *__restrict__ force,
          float4 *__restrict__ pos, float4 *__restrict__ vel, float4 *__restrict__ veval) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (gcell[i] == kUndef) {
        pos[i] = make_float4(-1000.f, -1000.f, -1000.f, 0.f);
        vel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    float3 po, vo, eo;
    advance_point(P, time, dt, ss, xyz(force[i]), xyz(pos[i]), xyz(vel[i]), xyz(veval[i]), po, vo, eo);
    pos[i] = f4(po);
    vel[i] = f4(vo);
    veval[i] = f4(eo);
}

// Force then advance for one point: the last two phases of Run fused.
// Neighbour reads come from pos_in/veval_in; the new position and evaluated
// velocity go to the other copies, velocity and force are updated in place.
__global__ void __launch_bounds__(kThreads)
k_force_advance(const __grid_constant__ DevParams P, int n, float *time_dev, int slot, float dt,
                const float4 *__restrict__ pos_in, const float4 *__restrict__ veval_in,
                const float *__restrict__ press, const uint32_t *__restrict__ gcell,
                const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt,
                float4 *__restrict__ vel, float4 *__restrict__ force,
                float4 *__restrict__ pos_out, float4 *__restrict__ veval_out,
                uint32_t *__restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const float time = time_dev[slot];
    if (i == 0) time_dev[slot ^ 1] = time + dt;
    if (i >= n) return;
    const uint32_t gc = gcell[i];
    if (gc == kUndef) {
        force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        pos_out[i] = make_float4(-1000.f, -1000.f, -1000.f, 0.f);
        vel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        veval_out[i] = veval_in[i];
        return;
    }
    const float3 f = force_sum(P, i, gc, pos_in, veval_in, press, off, cnt);
    force[i] = f4(f);
    float3 po, vo, eo;
    advance_point(P, time, dt, P.sim_scale, f, xyz(pos_in[i]), xyz(vel[i]), xyz(veval_in[i]), po, vo, eo);
    if (!(isfinite(po.x) && isfinite(po.y) && isfinite(po.z))) atomicOr(err, FL_DEV_NONFINITE);
    pos_out[i] = f4(po);
    vel[i] = f4(vo);
    veval_out[i] = f4(eo);
}

// ---------------------------------------------------------------------------
__global__ void k_pack3(int n, const float4 *__restrict__ src, float *__restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = src[i];
    dst[3 * i + 0] = v.x; dst[3 * i + 1] = v.y; dst[3 * i + 2] = v.z;
}

__global__ void k_unpack3(int n, const float *__restrict__ src, float4 *__restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[i] = make_float4(src[3 * i + 0], src[3 * i + 1], src[3 * i + 2], 0.0f);
}

__global__ void k_grid_identity(int n, int n_in, uint32_t *__restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[i] = (i < n_in) ? (uint32_t)i : kUndef;
}

// IntegrityCheck (fluids4.0/fluid_system.cpp:2426-2453): every sorted slot of
// cell g must carry gcell == g and gndx == its rank; tail slots must be UNDEF.
__global__ void k_integrity(int ncells, int n, const uint32_t *__restrict__ off,
                            const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ gcell,
                            const uint32_t *__restrict__ gndx, unsigned long long *bad) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g > ncells) return;
    const uint32_t o = off[g], m = cnt[g];
    unsigned long long b = 0;
    for (uint32_t k = 0; k < m; k++) {
        const uint32_t s = o + k;
        if (s >= (uint32_t)n) { b++; continue; }
        const uint32_t want = (g == ncells) ? kUndef : (uint32_t)g;
        if (gcell[s] != want || gndx[s] != k) b++;
    }
    if (b) atomicAdd(bad, b);
}

inline int blocks_for(long long n, int threads) { return (int)((n + threads - 1) / threads); }

}  // namespace

// ---------------------------------------------------------------------------
// Launch wrappers.

#define FL_LAUNCH_CHECK(name)                                                   \
    do {                                                                        \
        cudaError_t _e = cudaGetLastError();                                    \
        if (_e != cudaSuccess)                                                  \
            return fl_fail(FL_ERR_CUDA, "%s launch: %s", name, cudaGetErrorString(_e)); \
    } while (0)

int fl_launch_insert(fl_system *s, uint32_t *gcell_pre_or_null) {
    if (s->n == 0) return FL_OK;
    k_insert<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(
        s->D, s->n, s->f[F_POS].cur<float4>(), s->cell_pre, s->rank_tmp, gcell_pre_or_null, s->cnt);
    FL_LAUNCH_CHECK("insert");
    return FL_OK;
}

int fl_launch_scatter_index(fl_system *s) {
    if (s->n == 0) return FL_OK;
    k_scatter_index<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(
        s->n, s->cell_pre, s->rank_tmp, s->off, s->src);
    FL_LAUNCH_CHECK("scatter_index");
    return FL_OK;
}

int fl_launch_sort_cells(fl_system *s, int mode) {
    SortArgs a = {};
    a.off = s->off; a.cnt = s->cnt; a.src = s->src; a.scratch = s->rank_tmp;
    a.ncells = s->ncells;
    const int warps_per_block = kThreads / 32;
    const int grid = blocks_for((long long)s->ncells + 1, warps_per_block);
    if (mode == 0) {
        a.gndx_pre = s->f[F_GNDX].cur<uint32_t>();
        k_sort_cells<0><<<grid, kThreads, 0, s->stream>>>(a);
    } else {
        a.pos_in = s->f[F_POS].cur<float4>(); a.pos_out = s->f[F_POS].nxt<float4>();
        a.vel_in = s->f[F_VEL].cur<float4>(); a.vel_out = s->f[F_VEL].nxt<float4>();
        a.veval_in = s->f[F_VEVAL].cur<float4>(); a.veval_out = s->f[F_VEVAL].nxt<float4>();
        a.clr_in = s->f[F_CLR].cur<uint32_t>(); a.clr_out = s->f[F_CLR].nxt<uint32_t>();
        a.gcell_out = s->f[F_GCELL].nxt<uint32_t>();
        a.gndx_out = s->f[F_GNDX].nxt<uint32_t>();
        k_sort_cells<1><<<grid, kThreads, 0, s->stream>>>(a);
    }
    FL_LAUNCH_CHECK("sort_cells");
    return FL_OK;
}

int fl_launch_gather_all(fl_system *s) {
    if (s->n == 0) return FL_OK;
    k_gather_all<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(
        s->n, s->src,
        s->f[F_POS].cur<float4>(), s->f[F_VEL].cur<float4>(), s->f[F_VEVAL].cur<float4>(),
        s->f[F_FORCE].cur<float4>(), s->f[F_PRESS].cur<float>(), s->f[F_CLR].cur<uint32_t>(),
        s->f[F_GCELL].cur<uint32_t>(), s->f[F_GNDX].cur<uint32_t>(),
        s->f[F_POS].nxt<float4>(), s->f[F_VEL].nxt<float4>(), s->f[F_VEVAL].nxt<float4>(),
        s->f[F_FORCE].nxt<float4>(), s->f[F_PRESS].nxt<float>(), s->f[F_CLR].nxt<uint32_t>(),
        s->f[F_GCELL].nxt<uint32_t>(), s->f[F_GNDX].nxt<uint32_t>());
    FL_LAUNCH_CHECK("gather_all");
    return FL_OK;
}

int fl_launch_density(fl_system *s) {
    if (s->n == 0) return FL_OK;
    k_density<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(
        s->D, s->n, s->f[F_POS].cur<float4>(), s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt,
        s->f[F_PRESS].cur<float>());
    FL_LAUNCH_CHECK("density");
    return FL_OK;
}

int fl_launch_force(fl_system *s) {
    if (s->n == 0) return FL_OK;
    k_force<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(
        s->D, s->n, s->f[F_POS].cur<float4>(), s->f[F_VEVAL].cur<float4>(),
        s->f[F_PRESS].cur<float>(), s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt,
        s->f[F_FORCE].cur<float4>());
    FL_LAUNCH_CHECK("force");
    return FL_OK;
}

int fl_launch_force_advance(fl_system *s, float dt) {
    k_force_advance<<<blocks_for(s->n > 0 ? s->n : 1, kThreads), kThreads, 0, s->stream>>>(
        s->D, s->n, s->time_dev, s->time_slot, dt, s->f[F_POS].cur<float4>(), s->f[F_VEVAL].cur<float4>(),
        s->f[F_PRESS].cur<float>(), s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt,
        s->f[F_VEL].cur<float4>(), s->f[F_FORCE].cur<float4>(),
        s->f[F_POS].nxt<float4>(), s->f[F_VEVAL].nxt<float4>(), s->dev_err);
    FL_LAUNCH_CHECK("force_advance");
    return FL_OK;
}

int fl_launch_advance(fl_system *s, float time, float dt, float ss) {
    if (s->n == 0) return FL_OK;
    k_advance<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(
        s->D, s->n, time, dt, ss, s->f[F_GCELL].cur<uint32_t>(), s->f[F_FORCE].cur<float4>(),
        s->f[F_POS].cur<float4>(), s->f[F_VEL].cur<float4>(), s->f[F_VEVAL].cur<float4>());
    FL_LAUNCH_CHECK("advance");
    return FL_OK;
}

int fl_launch_pack3(fl_system *s, const float4 *src, float *dst, int n) {
    if (n == 0) return FL_OK;
    k_pack3<<<blocks_for(n, kThreads), kThreads, 0, s->stream>>>(n, src, dst);
    FL_LAUNCH_CHECK("pack3");
    return FL_OK;
}

int fl_launch_unpack3(fl_system *s, const float *src, float4 *dst, int n) {
    if (n == 0) return FL_OK;
    k_unpack3<<<blocks_for(n, kThreads), kThreads, 0, s->stream>>>(n, src, dst);
    FL_LAUNCH_CHECK("unpack3");
    return FL_OK;
}

int fl_launch_grid_identity(fl_system *s, uint32_t *dst, int n, int n_in) {
    if (n == 0) return FL_OK;
    k_grid_identity<<<blocks_for(n, kThreads), kThreads, 0, s->stream>>>(n, n_in, dst);
    FL_LAUNCH_CHECK("grid_identity");
    return FL_OK;
}

int fl_launch_integrity(fl_system *s, unsigned long long *bad_dev) {
    k_integrity<<<blocks_for((long long)s->ncells + 1, kThreads), kThreads, 0, s->stream>>>(
        s->ncells, s->n, s->off, s->cnt, s->f[F_GCELL].cur<uint32_t>(),
        s->f[F_GNDX].cur<uint32_t>(), bad_dev);
    FL_LAUNCH_CHECK("integrity");
    return FL_OK;
}
