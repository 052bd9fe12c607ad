// Cell-task neighbour passes of the fused step (FL_PASSES_CELL_TASKS, and
// FL_PASSES_AUTO once a cell crowds; gridSrch 2, band codes set), and the
// cell-task density of the adjoint's rebuilt steps.
//
// computePressure and computeForce (fluids4.0/fluid_kernels.cu:112-149,
// 180-217) walk, for every point, the 2x2x2 search block c-1..c of its cell
// c. Every point of a cell shares that block, so here the unit of work is a
// task: up to 64 sorted slots of one cell, taken by one warp (two points per
// lane: slot s0 + lane and s0 + 32 + lane). The warp walks the block once
// for all of its points, in lockstep:
//
//  * the walk visits the adjacency entries in the reference's order, each
//    entry only if some point of the task lies within the band of every
//    lower face that entry reaches across (the same pruning as the
//    per-thread walk: lower-band bits in pos.w), and within an entry the
//    members whose upper-band flags cover those faces, in ascending slot
//    order -- the "union" sequence of the task;
//  * each 32-slot flag word is staged with one coalesced load per lane into
//    a per-warp ring in shared memory, and every staged candidate is then
//    tested by all lanes at once (a broadcast read), 32 at a time;
//  * a pair that some other point of the task needed but this point's own
//    pruning would have skipped has |d| >= band > h, so it fails the test
//    0 < d^2 < rd2: each point's sums still see exactly the reference's
//    terms in the reference's order, and densities and forces stay
//    bit-identical to the per-point walk.
//
// The density pass evaluates two points per lane in packed f32x2
// arithmetic (sub/mul.rn.f32x2: IEEE round-to-nearest per element, the same
// results as scalar operations) when a task has more than 32 points; no
// packed add ever takes two packed products (see density_group2). It
// records hit masks for the force pass, or pair lists for the adjoint. The
// force pass is described above k_force_cells.
//
// Tasks are listed once per step by k_make_tasks (one entry per 64 slots of
// a cell, out-of-range bins included, in any order: no result depends on
// it). Both passes run a grid sized to the resident warps, each warp taking
// tasks from a ticket.
#include <algorithm>

#include "fl_internal.h"

namespace {

#include "fl_device.cuh"
#include "fl_step.cuh"

constexpr int kTaskPoints = 64;    // slots per task: two per lane
constexpr int kCellThreads = 128;  // threads per block of both passes (4 warps, one task each at a time)
constexpr uint32_t kRing = 64;     // staged candidates per warp (at most 63 are pending)
constexpr uint32_t kMaskWords = 16; // hit-mask words kept per point: unions of up to 512 candidates
constexpr uint32_t kPairCap = 512; // hit pairs of one group evaluated pair-parallel (else per lane)

// ---- tasks ------------------------------------------------------------------
// counters (in the grid block, cleared with the counts every step):
// [0] tasks listed, [1] density pass ticket, [2] force pass ticket.
// One task per kTaskPoints slots of every non-empty cell entry (an entry's
// tasks are its slots off + 64 k); a task is (first slot, cell entry).
__global__ void __launch_bounds__(256)
k_make_tasks(int gcells, const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt,
             uint2 *__restrict__ tasks, uint32_t cap, uint32_t *counters, uint32_t *err) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned lane = lane_id();
    const uint32_t m = (c < gcells) ? cnt[c] : 0u;
    const uint32_t k = (m + kTaskPoints - 1) / kTaskPoints;
    uint32_t incl = k;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= (unsigned)d) incl += y;
    }
    uint32_t base = 0;
    if (lane == 31 && incl) base = atomicAdd(&counters[0], incl);
    base = __shfl_sync(0xffffffffu, base, 31);
    if (!k) return;
    const uint32_t o = off[c];
    uint32_t t = base + incl - k;
    for (uint32_t q = 0; q < k; q++, t++) {
        if (t < cap) tasks[t] = make_uint2(o + q * kTaskPoints, (uint32_t)c);
        else atomicOr(err, FL_DEV_BAD_CELL);
    }
}

// The adjacency entries (bit k) the task's points reach: entry k is needed
// when some point lies within the band of every lower face the entry
// crosses (lower-band bits 3-5 of its code).
__device__ __forceinline__ uint32_t needed_entries(bool va, uint32_t ca, bool vb, uint32_t cb) {
    const uint32_t la = (ca >> 3) & 7u, lb = (cb >> 3) & 7u;
    uint32_t need = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const uint32_t U = lower_axes(k);
        if (__any_sync(0xffffffffu, (va && (la & U) == U) || (vb && (lb & U) == U))) need |= 1u << k;
    }
    return need;
}

// The union walk of a task in cell c: for each needed adjacency entry in
// order, the members of that neighbour cell whose upper-band flags cover the
// faces the entry crosses, in ascending slot order. stage(r, j) (called by
// the lanes that hold candidate j) puts slot j's data into ring slot r;
// group(g, count) evaluates the `count` candidates staged from union index
// g (g a multiple of 32; count 32 except for the last group). All lanes
// call this with the same arguments.
template <class Stage, class Group>
__device__ __forceinline__ void walk_union(const DevParams &P, int c, uint32_t need,
                                           const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt,
                                           const uint32_t *__restrict__ upbits, Stage stage, Group group) {
    const unsigned lane = lane_id();
    const unsigned below = (1u << lane) - 1u;
    const int base = c - P.nadj;
    uint32_t staged = 0, head = 0;
    for (int k = 0; k < 8; k++) {
        if (!((need >> k) & 1u)) continue;
        const int cn = base + P.adj[k];
        const uint32_t mn = cnt[cn];
        if (mn == 0) continue;
        const uint32_t lo = off[cn], hi = lo + mn;
        const uint32_t U = lower_axes(k);
        const uint32_t w_lo = lo >> 5, w_hi = (hi - 1) >> 5;
        for (uint32_t wd = w_lo; wd <= w_hi; wd++) {
            uint32_t bits = 0xffffffffu;
            if (U & 1u) bits &= upbits[wd];
            if (U & 2u) bits &= upbits[(size_t)P.upwords + wd];
            if (U & 4u) bits &= upbits[2 * (size_t)P.upwords + wd];
            if (wd == w_lo) bits &= 0xffffffffu << (lo & 31u);
            if (wd == w_hi && (hi & 31u)) bits &= 0xffffffffu >> (32u - (hi & 31u));
            if (!bits) continue;
            if ((bits >> lane) & 1u) stage((staged + __popc(bits & below)) & (kRing - 1u), (wd << 5) + lane);
            staged += __popc(bits);
            if (staged - head >= 32u) {
                __syncwarp();
                group(head, 32u);
                __syncwarp();
                head += 32u;
            }
        }
    }
    if (staged > head) {
        __syncwarp();
        group(head, staged - head);
        __syncwarp();
    }
}

// ---- density ----------------------------------------------------------------
// Candidates of one group against one point per lane (a), in order. A
// candidate that fails the test adds +0, which leaves the (non-negative)
// sum unchanged.
// Returns the group's hit mask (bit u: candidate g + u passed the test).
__device__ __forceinline__ uint32_t density_group1(const DevParams &P, const float4 *ring, uint32_t g,
                                                   uint32_t count, float4 pa, float &sa) {
    uint32_t ma = 0;
#pragma unroll 4
    for (uint32_t u = 0; u < count; u++) {
        const float4 q = ring[(g + u) & (kRing - 1u)];
        const float dx = pa.x - q.x, dy = pa.y - q.y, dz = pa.z - q.z;
        const float dsq = dx * dx + dy * dy + dz * dz;
        const float t = (P.rd2 - dsq) * P.d2;
        const float t3 = t * t * t;
        const bool hit = dsq < P.rd2 && dsq > 0.0f;
        sa += hit ? t3 : 0.0f;
        ma |= (hit ? 1u : 0u) << u;
    }
    return ma;
}

// The same for two points per lane (a, b), in packed f32x2 arithmetic.
__device__ __forceinline__ void density_group2(const DevParams &P, const float4 *ring, uint32_t g, uint32_t count,
                                               uint64_t px, uint64_t py, uint64_t pz, uint64_t &sab,
                                               uint32_t &ma, uint32_t &mb) {
    ma = mb = 0;
    const uint64_t rd2 = pk2(P.rd2, P.rd2), d2 = pk2(P.d2, P.d2);
#pragma unroll 4
    for (uint32_t u = 0; u < count; u++) {
        const float4 q = ring[(g + u) & (kRing - 1u)];
        const uint64_t dx = sub2(px, pk2(q.x, q.x));
        const uint64_t dy = sub2(py, pk2(q.y, q.y));
        const uint64_t dz = sub2(pz, pk2(q.z, q.z));
        // The squares are summed in scalar: ptxas contracts a packed add of
        // two packed products into a packed fused multiply-add (one rounding
        // fewer), explicit .rn notwithstanding; the scalar adds of the
        // unpacked squares round exactly as the reference's expression.
        float xa, xb, ya, yb, za, zb;
        up2(mul2(dx, dx), xa, xb);
        up2(mul2(dy, dy), ya, yb);
        up2(mul2(dz, dz), za, zb);
        const float da = xa + ya + za, db = xb + yb + zb;
        const uint64_t t = mul2(sub2(rd2, pk2(da, db)), d2);
        const uint64_t t3 = mul2(mul2(t, t), t);
        float ta, tb;
        up2(t3, ta, tb);
        const bool ha = da < P.rd2 && da > 0.0f, hb = db < P.rd2 && db > 0.0f;
        ta = ha ? ta : 0.0f;
        tb = hb ? tb : 0.0f;
        sab = add2(sab, pk2(ta, tb));
        ma |= (ha ? 1u : 0u) << u;
        mb |= (hb ? 1u : 0u) << u;
    }
}

// Pair lists in the per-point passes' layout (list_at: the first hcap hits
// of a point in visiting order; hitcnt: the count of all of them) from one
// group's hit mask. The slot of each staged candidate rides in its .w.
__device__ __forceinline__ void list_hits(const DevParams &P, const float4 *ring, uint32_t g, uint32_t h, uint32_t i,
                                          uint32_t &nh, uint32_t *__restrict__ hitlist) {
    while (h) {
        const uint32_t u = (uint32_t)(__ffs(h) - 1);
        h &= h - 1u;
        if (nh < (uint32_t)P.hcap) hitlist[list_at(P, (int)i, nh)] = __float_as_uint(ring[(g + u) & (kRing - 1u)].w);
        nh++;
    }
}

// Besides the densities and the pair records, LIST = false (the fused step)
// writes each point's hit masks for the force pass: word w of point i, at
// masks[w * mstride + i], holds bit u set when union candidate 32 w + u
// passed the test (the first kMaskWords words). LIST = true (the adjoint's
// rebuilt steps) writes each point's pair list and count (hitlist,
// hitcnt) exactly as the per-point density pass does, for the reverse
// kernels, which drain those lists. Both share the pair-list buffer.
template <bool BATCH, bool LIST>
__global__ void __launch_bounds__(kCellThreads)
k_density_cells(const __grid_constant__ DevParams P0, const SceneTab T, const uint2 *__restrict__ tasks,
                uint32_t cap, uint32_t *counters, const float4 *__restrict__ pos, const uint32_t *__restrict__ off,
                const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ upbits,
                const float4 *__restrict__ veval, float *__restrict__ press, float4 *__restrict__ pairdata,
                uint32_t *__restrict__ hitlist, uint32_t *__restrict__ hitcnt, size_t mstride) {
    __shared__ float4 s_ring[kCellThreads / 32][kRing];
    const unsigned lane = lane_id();
    float4 *ring = s_ring[threadIdx.x >> 5];
    const uint32_t ntasks = min(counters[0], cap);   // k_make_tasks flags an overflow
    for (;;) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(&counters[1], 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= ntasks) return;
        const uint2 task = tasks[t];
        const int c = (int)task.y;
        const DevParams &P = BATCH ? T.params[T.cell_scene[c]] : P0;
        const uint32_t mt = min((uint32_t)kTaskPoints, off[c] + cnt[c] - task.x);
        const uint32_t ia = task.x + lane, ib = ia + 32u;
        const bool va = lane < mt, vb = lane + 32u < mt;
        if (c - P.cell_base == P.ncells) {   // the out-of-range bin: density 0
            if (va) press[ia] = 0.0f;
            if (vb) press[ib] = 0.0f;
            if (LIST && va) hitcnt[ia] = 0;
            if (LIST && vb) hitcnt[ib] = 0;
            continue;
        }
        const float4 pa = va ? pos[ia] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 pb = vb ? pos[ib] : make_float4(0.f, 0.f, 0.f, 0.f);
        const uint32_t need = needed_entries(va, __float_as_uint(pa.w), vb, __float_as_uint(pb.w));
        auto stage = [&](uint32_t r, uint32_t j) {
            float4 q = pos[j];
            q.w = __uint_as_float(j);   // the slot (band codes are not needed here)
            ring[r] = q;
        };
        float sa = 0.0f, sb = 0.0f;
        uint32_t na = 0, nb = 0;
        if (mt > 32u) {   // two points per lane
            const uint64_t px = pk2(pa.x, pb.x), py = pk2(pa.y, pb.y), pz = pk2(pa.z, pb.z);
            uint64_t sab = pk2(0.0f, 0.0f);
            walk_union(P, c, need, off, cnt, upbits, stage, [&](uint32_t g, uint32_t count) {
                uint32_t ma, mb;
                density_group2(P, ring, g, count, px, py, pz, sab, ma, mb);
                if (LIST) {
                    if (va) list_hits(P, ring, g, ma, ia, na, hitlist);
                    if (vb) list_hits(P, ring, g, mb, ib, nb, hitlist);
                } else if ((g >> 5) < kMaskWords) {
                    uint32_t *row = hitlist + (size_t)(g >> 5) * mstride;
                    if (va) row[ia] = ma;
                    if (vb) row[ib] = mb;
                }
            });
            up2(sab, sa, sb);
        } else {
            walk_union(P, c, need, off, cnt, upbits, stage, [&](uint32_t g, uint32_t count) {
                const uint32_t ma = density_group1(P, ring, g, count, pa, sa);
                if (LIST) {
                    if (va) list_hits(P, ring, g, ma, ia, na, hitlist);
                } else if ((g >> 5) < kMaskWords && va) {
                    hitlist[(size_t)(g >> 5) * mstride + ia] = ma;
                }
            });
        }
        // fluid_kernels.cu:146-148, and the pair records the force pass reads
        if (va) {
            sa = sa * P.pmass * P.poly6kern;
            if (sa == 0.0f) sa = 1.0f;
            press[ia] = sa;
            const float4 e = veval[ia];
            pairdata[2 * (size_t)ia] = make_float4(pa.x, pa.y, pa.z, sa);
            pairdata[2 * (size_t)ia + 1] = make_float4(e.x, e.y, e.z, 0.0f);
            if (LIST) hitcnt[ia] = na;
        }
        if (vb) {
            sb = sb * P.pmass * P.poly6kern;
            if (sb == 0.0f) sb = 1.0f;
            press[ib] = sb;
            const float4 e = veval[ib];
            pairdata[2 * (size_t)ib] = make_float4(pb.x, pb.y, pb.z, sb);
            pairdata[2 * (size_t)ib + 1] = make_float4(e.x, e.y, e.z, 0.0f);
            if (LIST) hitcnt[ib] = nb;
        }
    }
}


// ---- force + advance ----------------------------------------------------------
// The force pass walks the same union as the density pass (same codes,
// flags and counts, so the same sequence), staging each candidate's 32-byte
// pair record (position and density; evaluated velocity). For each group of
// 32 candidates the hits of the task's points come from the density pass's
// masks (past kMaskWords words the test is repeated). The hits of a group
// are then evaluated pair-parallel: they are listed point by point, in
// candidate order, in shared memory; 32 lanes compute 32 pair terms at a
// time (pair_term, the reference's arithmetic); and each lane adds its own
// points' terms in list order -- the reference's pair order -- so every
// force is the same sum, bit for bit. Groups with more than kPairCap hits
// (crowded cells) are drained per lane instead, each lane adding its hits
// as it finds them.
struct ForceOut {
    float4 *vel, *force, *pos_out, *veval_out;
    float *host_pos;      // optional page-locked host copy of the new positions (float x3)
    uint32_t *err;
};

struct ForceShared {
    float4 ring[kRing][2];        // staged pair records
    float4 pts[kTaskPoints][2];   // the task's points: (p.xyz, pressure term), (veval.xyz, density)
    float4 terms[32];             // one batch of pair terms
    uint16_t pairs[kPairCap];     // the group's hits: point << 5 | candidate
};

__device__ __forceinline__ uint32_t hit_bits(const DevParams &P, const float4 (*ring)[2], uint32_t g, uint32_t count,
                                             float4 p) {
    uint32_t h = 0;
#pragma unroll 4
    for (uint32_t u = 0; u < count; u++) {
        const float4 q = ring[(g + u) & (kRing - 1u)][0];
        const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
        const float dsq = dx * dx + dy * dy + dz * dz;
        h |= (dsq < P.rd2 && dsq > 0.0f) ? (1u << u) : 0u;
    }
    return h;
}

// One point's hits of a group, added in candidate order (the per-lane drain).
__device__ __forceinline__ void drain_hits(const DevParams &P, const ForceShared &sh, uint32_t g, uint32_t h,
                                           const float4 pt[2], float3 &f) {
    while (h) {
        const uint32_t u = (uint32_t)(__ffs(h) - 1);
        h &= h - 1u;
        const float4 *rec = sh.ring[(g + u) & (kRing - 1u)];
        const float3 t = pair_term(P, pt[0], pt[0].w, pt[1], pt[1].w, rec[0], rec[1], rec[0].w);
        f.x += t.x; f.y += t.y; f.z += t.z;
    }
}

// Adds the terms of list entries [lo, hi) that fall in the batch [bs, bs + 32).
__device__ __forceinline__ void take_terms(const ForceShared &sh, uint32_t lo, uint32_t hi, uint32_t bs, float3 &f) {
    const uint32_t a = max(lo, bs), b = min(hi, bs + 32u);
    for (uint32_t e = a; e < b; e++) {
        const float4 t = sh.terms[e - bs];
        f.x += t.x; f.y += t.y; f.z += t.z;
    }
}

// The advance of one in-range point from its force (fluid_kernels.cu:332-420).
__device__ __forceinline__ float3 finish_point(const DevParams &P, float time, float dt, uint32_t i, float4 p,
                                               float4 vi, float3 f, const ForceOut &o) {
    o.force[i] = f4(f);
    float3 po, vo, eo;
    advance_point(P, time, dt, P.sim_scale, f, xyz(p), xyz(o.vel[i]), xyz(vi), po, vo, eo);
    if (!(isfinite(po.x) && isfinite(po.y) && isfinite(po.z))) atomicOr(o.err, FL_DEV_NONFINITE);
    o.pos_out[i] = f4(po);
    o.vel[i] = f4(vo);
    o.veval_out[i] = f4(eo);
    return po;
}

// An out-of-range point: no force, parked at (-1000, -1000, -1000) with zero
// velocity (advanceParticles, cu:339-342).
__device__ __forceinline__ float3 park_point(uint32_t i, const float4 *__restrict__ veval, const ForceOut &o) {
    o.force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    o.pos_out[i] = make_float4(-1000.f, -1000.f, -1000.f, 0.f);
    o.vel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    o.veval_out[i] = veval[i];
    return make_float3(-1000.f, -1000.f, -1000.f);
}

// The new positions of `count` (<= 32) consecutive slots from s, packed
// float x3 into page-locked host memory, staged in shared memory so that
// each store instruction of the warp writes 128 contiguous bytes.
__device__ __forceinline__ void host_store(float *host, uint32_t s, uint32_t count, float3 v, float *stage) {
    const unsigned lane = lane_id();
    __syncwarp();
    stage[3 * lane] = v.x; stage[3 * lane + 1] = v.y; stage[3 * lane + 2] = v.z;
    __syncwarp();
    for (uint32_t e = lane; e < 3u * count; e += 32u) host[3 * (size_t)s + e] = stage[e];
    __syncwarp();
}

template <bool BATCH>
__global__ void __launch_bounds__(kCellThreads)
k_force_cells(const __grid_constant__ DevParams P0, const SceneTab T, const uint2 *__restrict__ tasks,
              uint32_t cap, uint32_t *counters, float *time_dev, int slot, float dt, const float4 *__restrict__ pos_in,
              const float4 *__restrict__ veval_in, const float *__restrict__ press,
              const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt,
              const uint32_t *__restrict__ upbits, const float4 *__restrict__ pairdata,
              const uint32_t *__restrict__ masks, size_t mstride, const __grid_constant__ ForceOut o) {
    __shared__ ForceShared s_sh[kCellThreads / 32];
    const unsigned lane = lane_id();
    ForceShared &sh = s_sh[threadIdx.x >> 5];
    const float time = time_dev[slot];
    if (blockIdx.x == 0 && threadIdx.x == 0) time_dev[slot ^ 1] = time + dt;
    const uint32_t ntasks = min(counters[0], cap);   // k_make_tasks flags an overflow
    for (;;) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(&counters[2], 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= ntasks) return;
        const uint2 task = tasks[t];
        const int c = (int)task.y;
        const DevParams &P = BATCH ? T.params[T.cell_scene[c]] : P0;
        const uint32_t mt = min((uint32_t)kTaskPoints, off[c] + cnt[c] - task.x);
        const uint32_t ia = task.x + lane, ib = ia + 32u;
        const bool va = lane < mt, vb = lane + 32u < mt;
        float3 na = make_float3(0.f, 0.f, 0.f), nb = na;
        if (c - P.cell_base == P.ncells) {   // the out-of-range bin
            if (va) na = park_point(ia, veval_in, o);
            if (vb) nb = park_point(ib, veval_in, o);
        } else {
            // the task's points: (position, pressure term), (veval, density)
            float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = make_float4(0.f, 0.f, 0.f, 1.f), b0 = a0, b1 = a1;
            uint32_t code_a = 0, code_b = 0;
            if (va) {
                const float4 p = pos_in[ia], e = veval_in[ia];
                const float d = press[ia];
                code_a = __float_as_uint(p.w);
                a0 = make_float4(p.x, p.y, p.z, (d - P.prest_dens) * P.pintstiff);
                a1 = make_float4(e.x, e.y, e.z, d);
            }
            if (vb) {
                const float4 p = pos_in[ib], e = veval_in[ib];
                const float d = press[ib];
                code_b = __float_as_uint(p.w);
                b0 = make_float4(p.x, p.y, p.z, (d - P.prest_dens) * P.pintstiff);
                b1 = make_float4(e.x, e.y, e.z, d);
            }
            __syncwarp();
            sh.pts[lane][0] = a0; sh.pts[lane][1] = a1;
            sh.pts[32 + lane][0] = b0; sh.pts[32 + lane][1] = b1;
            const float4 pa[2] = {a0, a1}, pb[2] = {b0, b1};
            const uint32_t need = needed_entries(va, code_a, vb, code_b);
            const bool dual = mt > 32u;
            float3 fa = make_float3(0.f, 0.f, 0.f), fb = fa;
            auto stage = [&](uint32_t r, uint32_t j) {
                sh.ring[r][0] = pairdata[2 * (size_t)j];
                sh.ring[r][1] = pairdata[2 * (size_t)j + 1];
            };
            walk_union(P, c, need, off, cnt, upbits, stage, [&](uint32_t g, uint32_t count) {
                uint32_t ha = 0, hb = 0;
                if ((g >> 5) < kMaskWords) {   // the density pass's record of this group
                    const uint32_t *row = masks + (size_t)(g >> 5) * mstride;
                    if (va) ha = row[ia];
                    if (dual && vb) hb = row[ib];
                } else {                       // beyond it: the same test again
                    if (va) ha = hit_bits(P, sh.ring, g, count, a0);
                    if (dual && vb) hb = hit_bits(P, sh.ring, g, count, b0);
                }
                // list offsets: point a of lane l, then point b of lane l
                const uint32_t ca = __popc(ha), cb = __popc(hb);
                uint32_t xa = ca, xb = cb;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t ya = __shfl_up_sync(0xffffffffu, xa, d);
                    const uint32_t yb = __shfl_up_sync(0xffffffffu, xb, d);
                    if (lane >= (unsigned)d) { xa += ya; xb += yb; }
                }
                const uint32_t total_a = __shfl_sync(0xffffffffu, xa, 31);
                const uint32_t total = total_a + __shfl_sync(0xffffffffu, xb, 31);
                if (total == 0) return;
                if (total > kPairCap) {   // crowded: each lane drains its own hits
                    drain_hits(P, sh, g, ha, pa, fa);
                    drain_hits(P, sh, g, hb, pb, fb);
                    return;
                }
                const uint32_t lo_a = xa - ca, lo_b = total_a + xb - cb;
                for (uint32_t h = ha, e = lo_a; h; h &= h - 1u, e++)
                    sh.pairs[e] = (uint16_t)((lane << 5) | (uint32_t)(__ffs(h) - 1));
                for (uint32_t h = hb, e = lo_b; h; h &= h - 1u, e++)
                    sh.pairs[e] = (uint16_t)(((32u + lane) << 5) | (uint32_t)(__ffs(h) - 1));
                __syncwarp();
                for (uint32_t bs = 0; bs < total; bs += 32u) {
                    const uint32_t e = bs + lane;
                    if (e < total) {
                        const uint32_t pr = sh.pairs[e];
                        const float4 *pt = sh.pts[pr >> 5];
                        const float4 *rec = sh.ring[(g + (pr & 31u)) & (kRing - 1u)];
                        const float3 tm = pair_term(P, pt[0], pt[0].w, pt[1], pt[1].w, rec[0], rec[1], rec[0].w);
                        sh.terms[lane] = make_float4(tm.x, tm.y, tm.z, 0.f);
                    }
                    __syncwarp();
                    take_terms(sh, lo_a, lo_a + ca, bs, fa);
                    take_terms(sh, lo_b, lo_b + cb, bs, fb);
                    __syncwarp();
                }
            });
            if (va) na = finish_point(P, time, dt, ia, a0, a1, fa, o);
            if (vb) nb = finish_point(P, time, dt, ib, b0, b1, fb, o);
        }
        if (o.host_pos) {
            float *st = reinterpret_cast<float *>(sh.ring);   // free once the walk is done
            host_store(o.host_pos, task.x, min(mt, 32u), na, st);
            if (mt > 32u) host_store(o.host_pos, task.x + 32u, mt - 32u, nb, st);
        }
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// Launch wrappers.

size_t fl_task_cap(int max_points, int gcells) {
    const size_t n = (size_t)(max_points > 0 ? max_points : 1);
    return n / kTaskPoints + std::min(n, (size_t)gcells) + 32;
}

static int resident_blocks(const void *kern) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCellThreads, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return per_sm;
}

// Grid of the pass: every block resident at once (queried once, at system
// creation, outside any stream capture).
int fl_cells_init(fl_system *s) {
    const int d = s->batched ? resident_blocks((const void *)k_density_cells<true, false>)
                             : resident_blocks((const void *)k_density_cells<false, false>);
    const int f = s->batched ? resident_blocks((const void *)k_force_cells<true>)
                             : resident_blocks((const void *)k_force_cells<false>);
    s->cells_grid[0] = d * s->num_sms;
    s->cells_grid[1] = f * s->num_sms;
    return FL_OK;
}

// The hit masks share the per-point pass's pair-list buffer (128 words per
// point; the masks take at most kMaskWords): row w holds word w of every slot.
static size_t mask_stride(const fl_system *s) {
    return ((size_t)(s->max_points > 0 ? s->max_points : 1) + 31) & ~(size_t)31;
}
static_assert(kMaskWords <= 128, "the hit masks must fit in the pair-list buffer");

int fl_launch_make_tasks(fl_system *s) {
    k_make_tasks<<<blocks_for((long long)s->gcells, 256), 256, 0, s->stream>>>(
        s->gcells, s->off, s->cnt, s->tasks, (uint32_t)s->task_cap, s->task_counters, s->dev_err);
    FL_LAUNCH_CHECK("make_tasks");
    return FL_OK;
}

int fl_launch_density_cells(fl_system *s, bool lists) {
    if (s->n == 0) return FL_OK;
    auto kern = lists ? (s->batched ? k_density_cells<true, true> : k_density_cells<false, true>)
                      : (s->batched ? k_density_cells<true, false> : k_density_cells<false, false>);
    const int grid = s->cells_grid[0];
    kern<<<grid, kCellThreads, 0, s->stream>>>(s->D, fl_scene_tab(s), s->tasks, (uint32_t)s->task_cap,
                                                s->task_counters, s->f[F_POS].cur<float4>(), s->off, s->cnt, s->upbits,
                                                s->f[F_VEVAL].cur<float4>(), s->f[F_PRESS].cur<float>(),
                                                s->pairdata, s->hitlist, s->hitcnt, mask_stride(s));
    FL_LAUNCH_CHECK("density_cells");
    s->lists_valid = lists ? 1 : 0;   // without lists the buffer holds the force pass's hit masks
    return FL_OK;
}

int fl_launch_force_cells(fl_system *s, float dt, float *host_pos) {
    auto kern = s->batched ? k_force_cells<true> : k_force_cells<false>;
    ForceOut o;
    o.vel = s->f[F_VEL].cur<float4>();
    o.force = s->f[F_FORCE].cur<float4>();
    o.pos_out = s->f[F_POS].nxt<float4>();
    o.veval_out = s->f[F_VEVAL].nxt<float4>();
    o.host_pos = host_pos;
    o.err = s->dev_err;
    kern<<<s->cells_grid[1], kCellThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->tasks, (uint32_t)s->task_cap, s->task_counters, s->time_dev, s->time_slot, dt,
        s->f[F_POS].cur<float4>(), s->f[F_VEVAL].cur<float4>(), s->f[F_PRESS].cur<float>(), s->off, s->cnt,
        s->upbits, s->pairdata, s->hitlist, mask_stride(s), o);
    FL_LAUNCH_CHECK("force_cells");
    return FL_OK;
}
