// Paired density pass (FL_PASSES_POINT_PAIRS; gridSrch 2 with band codes).
//
// computePressure (fluids4.0/fluid_kernels.cu:112-149) walks, for every
// point, the search block of its cell. With pruning, the candidates a point
// visits depend only on its cell and its lower-band bits (pos.w bits 3-5):
// two points of one cell with the same bits visit the same candidates in
// the same order. Here one thread takes such a pair and walks its candidates
// once, testing each against both points: one load and one pass of the
// enumeration serve two sums. Each point's sum still adds the reference's
// terms in the reference's order, in scalar FP32 without contraction, so
// densities, pair lists, counts and pair records are bit-identical to the
// per-point pass (k_density).
//
// A block takes kPairSlots consecutive sorted slots:
//  1. its walking points are ordered by lower-band bits, ascending slot
//     within equal bits (a counting sort), which puts the points of one cell
//     with equal bits next to each other;
//  2. every run of equal (cell, bits) is cut into pairs, an odd run ending in
//     a single point; the pairs and singles are the block's items, kept in
//     that order, so neighbouring items reach into the same adjacency
//     entries;
//  3. the block's warps take the items 32 at a time from a counter in shared
//     memory until none are left.
// Points in the out-of-range bin get density 0 and no pairs, as in
// k_density.
#include <algorithm>

#include "fl_internal.h"

namespace {

#include "fl_device.cuh"

constexpr int kPairThreads = 128;
constexpr int kPairSlots = 512;                     // sorted slots per block
constexpr int kPer = kPairSlots / kPairThreads;     // slots per thread in steps 1-2
constexpr int kPairWarps = kPairThreads / 32;
constexpr int kGroups = kPairSlots / 32;            // 32-slot groups of the counting sort
constexpr uint32_t kWalkKeys = 8;                   // lower-band bit patterns
constexpr uint32_t kSkipKey = kWalkKeys;            // out-of-range bin or past n: no walk
constexpr uint32_t kAlone = 0xffffu;                // an item's second point: none

struct PairShared {
    uint32_t item[kPairSlots];                      // local slot a | local slot b << 16
    uint32_t cnt[(kWalkKeys + 1) * kGroups];        // (key, group) counts, then offsets
    uint16_t sorted[kPairSlots];                    // walking local slots in (bits, slot) order
    uint8_t key[kPairSlots];                        // by local slot
    uint32_t wtot[kPairWarps];
    uint32_t next;                                  // first item not yet taken
};

// Exclusive scan over the block's threads, one value each (MAX: running
// maximum, identity 0; else running sum); `total` receives the reduction
// of all values. All threads call it.
template <bool MAX>
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t *wtot, uint32_t &total) {
    const unsigned lane = lane_id(), w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= (unsigned)d) x = MAX ? max(x, y) : x + y;
    }
    const uint32_t before = __shfl_up_sync(0xffffffffu, x, 1);
    if (lane == 31) wtot[w] = x;
    __syncthreads();
    uint32_t pre = 0, tot = 0;
#pragma unroll
    for (int k = 0; k < kPairWarps; k++) {
        const uint32_t t = wtot[k];
        if ((unsigned)k < w) pre = MAX ? max(pre, t) : pre + t;
        tot = MAX ? max(tot, t) : tot + t;
    }
    __syncthreads();   // wtot is free again
    total = tot;
    if (lane == 0) return pre;
    return MAX ? max(pre, before) : pre + before;
}

template <bool BATCH>
__global__ void __launch_bounds__(kPairThreads, 4)
k_density_pairs(const __grid_constant__ DevParams P0, const SceneTab T, int n, const float4 *__restrict__ pos,
                const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off,
                const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ upbits,
                const float4 *__restrict__ veval, float *__restrict__ press, uint32_t *__restrict__ hitlist,
                uint32_t *__restrict__ hitcnt, float4 *__restrict__ pairdata) {
    __shared__ PairShared sh;
    const int base = blockIdx.x * kPairSlots;
    const unsigned lane = lane_id(), w = threadIdx.x >> 5;

    // 1. counting sort of the block's slots by lower-band bits
    uint32_t key[kPer], rank[kPer];
#pragma unroll
    for (int h = 0; h < kPer; h++) {
        const int e = h * kPairThreads + (int)threadIdx.x;
        const int i = base + e;
        uint32_t k = kSkipKey;
        if (i < n) {
            const uint32_t gc = gcell[i];
            if (gc == kUndef) {
                press[i] = 0.0f;
                hitcnt[i] = 0;
            } else {
                k = (__float_as_uint(pos[i].w) >> 3) & 7u;
            }
        }
        sh.key[e] = (uint8_t)k;
        key[h] = k;
        rank[h] = 0;
        const unsigned below = (1u << lane) - 1u;
        const int g = h * kPairWarps + (int)w;   // group of slots e - lane .. e - lane + 31
#pragma unroll
        for (uint32_t kk = 0; kk <= kWalkKeys; kk++) {
            const unsigned b = __ballot_sync(0xffffffffu, k == kk);
            if (lane == 0) sh.cnt[kk * kGroups + g] = __popc(b);
            if (k == kk) rank[h] = __popc(b & below);
        }
    }
    if (threadIdx.x == 0) sh.next = 0;
    __syncthreads();
    if (w == 0) {   // exclusive scan of the (key, group) counts, key-major
        constexpr uint32_t total = (kWalkKeys + 1) * kGroups;
        uint32_t run = 0;
        for (uint32_t c0 = 0; c0 < total; c0 += 32) {
            const uint32_t e = c0 + lane;
            const uint32_t v = (e < total) ? sh.cnt[e] : 0u;
            uint32_t x = v;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= (unsigned)d) x += y;
            }
            if (e < total) sh.cnt[e] = run + x - v;
            run += __shfl_sync(0xffffffffu, x, 31);
        }
    }
    __syncthreads();
#pragma unroll
    for (int h = 0; h < kPer; h++)
        if (key[h] < kWalkKeys)
            sh.sorted[sh.cnt[key[h] * kGroups + h * kPairWarps + w] + rank[h]] =
                (uint16_t)(h * kPairThreads + (int)threadIdx.x);
    const uint32_t nvalid = sh.cnt[kSkipKey * kGroups];   // walking points: the keys below kSkipKey
    __syncthreads();

    // 2. runs of equal (cell, bits) cut into pairs; thread t looks at sorted
    //    positions kPer t .. kPer t + kPer - 1
    auto same_run = [&](uint32_t k1, uint32_t k2) {   // k1 < k2 < nvalid
        const uint32_t e1 = sh.sorted[k1], e2 = sh.sorted[k2];
        return sh.key[e1] == sh.key[e2] && gcell[base + e1] == gcell[base + e2];
    };
    const uint32_t k0 = threadIdx.x * kPer;
    bool head[kPer];
    uint32_t heads = 0;
#pragma unroll
    for (int h = 0; h < kPer; h++) {
        const uint32_t k = k0 + h;
        head[h] = k < nvalid && (k == 0 || !same_run(k - 1, k));
        if (head[h]) heads = k;
    }
    uint32_t unused;
    uint32_t run_start = block_exclusive<true>(heads, sh.wtot, unused);
    bool first[kPer], partner[kPer];
    uint32_t nfirst = 0;
#pragma unroll
    for (int h = 0; h < kPer; h++) {
        const uint32_t k = k0 + h;
        if (head[h]) run_start = k;
        first[h] = k < nvalid && ((k - run_start) & 1u) == 0;
        partner[h] = first[h] && k + 1 < nvalid && same_run(k, k + 1);
        nfirst += first[h] ? 1u : 0u;
    }
    uint32_t nitems;
    uint32_t idx = block_exclusive<false>(nfirst, sh.wtot, nitems);
#pragma unroll
    for (int h = 0; h < kPer; h++) {
        if (!first[h]) continue;
        const uint32_t k = k0 + h;
        const uint32_t b = partner[h] ? (uint32_t)sh.sorted[k + 1] : kAlone;
        sh.item[idx++] = (uint32_t)sh.sorted[k] | (b << 16);
    }
    __syncthreads();

    // 3. the walks: one per item, 32 items per warp at a time
    for (;;) {
        uint32_t c0 = 0;
        if (lane == 0) c0 = atomicAdd(&sh.next, 32u);
        c0 = __shfl_sync(0xffffffffu, c0, 0);
        if (c0 >= nitems) break;
        const uint32_t it = c0 + lane;
        if (it >= nitems) continue;
        const uint32_t v = sh.item[it];
        const uint32_t ea = v & 0xffffu, eb = v >> 16;
        const bool two = eb != kAlone;
        const int a = base + (int)ea;
        const int b = two ? base + (int)eb : a;
        const DevParams &P = BATCH ? T.params[T.point_scene[a]] : P0;
        const int cbase = (int)gcell[a] - P.nadj;
        const float4 pa = pos[a], pb = pos[b];
        const uint32_t code = __float_as_uint(pa.w);
        const float rd2 = P.rd2, d2 = P.d2;
        const uint32_t cap = (uint32_t)P.hcap;
        uint32_t *const la = hitlist + list_at(P, a, 0);
        uint32_t *const lb = hitlist + list_at(P, b, 0);
        float sa = 0.0f, sb = 0.0f;
        uint32_t na = 0, nb = 0;
        auto visit = [&](uint32_t j) {
            const float4 q = pos[j];
            const float ax = pa.x - q.x, ay = pa.y - q.y, az = pa.z - q.z;
            const float bx = pb.x - q.x, by = pb.y - q.y, bz = pb.z - q.z;
            float da = ax * ax + ay * ay + az * az;
            float db = bx * bx + by * by + bz * bz;
            if (da < rd2 && da > 0.0f) {
                da = (rd2 - da) * d2;
                sa += da * da * da;
                if (na < cap) la[(size_t)na * 32u] = j;
                na++;
            }
            if (two && db < rd2 && db > 0.0f) {
                db = (rd2 - db) * d2;
                sb += db * db * db;
                if (nb < cap) lb[(size_t)nb * 32u] = j;
                nb++;
            }
        };
        for (int c = 0; c < P.gridAdjCnt; c++) {
            CandIter ci;
            cand_begin<true>(ci, P, c, cbase + P.adj[c], code, true, off, cnt, upbits);
            if (ci.U == 0u) {   // the own cell: no flags to consult, every slot in order
                for (uint32_t j = ci.lo; j < ci.hi; j++) visit(j);
                continue;
            }
            uint32_t j;
            while (cand_next<true>(ci, P, upbits, j)) visit(j);
        }
        auto finish = [&](int i, float4 p, float sum, uint32_t nh) {
            sum = sum * P.pmass * P.poly6kern;
            if (sum == 0.0f) sum = 1.0f;
            press[i] = sum;
            hitcnt[i] = nh;
            const float4 e = veval[i];
            pairdata[2 * (size_t)i] = make_float4(p.x, p.y, p.z, sum);
            pairdata[2 * (size_t)i + 1] = make_float4(e.x, e.y, e.z, 0.0f);
        };
        finish(a, pa, sa, na);
        if (two) finish(b, pb, sb, nb);
    }
}

}  // namespace

// The pass's blocks are bound by registers, not shared memory: ask for the
// smallest shared-memory carveout that still holds every resident block, so
// the rest of the SM's unified L1 caches the candidate positions (queried
// once, at system creation, outside any stream capture).
template <typename K>
static int set_carveout(K kern) {
    int per_sm = 0, dev = 0, smem_sm = 0;
    cudaFuncAttributes fa;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPairThreads, 0) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, kern) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        per_sm < 1 || smem_sm < 1) {
        cudaGetLastError();
        return FL_OK;   // keep the driver's choice
    }
    const long long need = (long long)per_sm * ((long long)fa.sharedSizeBytes + 1024);   // + the driver's 1 KB
    const int pct = (int)std::min(100LL, (need * 100 + smem_sm - 1) / smem_sm);
    FL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
    return FL_OK;
}

int fl_pairs_init() {
    FL_TRY(set_carveout(k_density_pairs<false>));
    return set_carveout(k_density_pairs<true>);
}

int fl_launch_density_pairs(fl_system *s) {
    if (s->n == 0) return FL_OK;
    auto kern = s->batched ? k_density_pairs<true> : k_density_pairs<false>;
    kern<<<blocks_for(s->n, kPairSlots), kPairThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->n, s->f[F_POS].cur<float4>(), s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt,
        s->upbits, s->f[F_VEVAL].cur<float4>(), s->f[F_PRESS].cur<float>(), s->hitlist, s->hitcnt, s->pairdata);
    FL_LAUNCH_CHECK("density_pairs");
    s->lists_valid = 1;
    return FL_OK;
}
