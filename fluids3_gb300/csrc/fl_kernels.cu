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
#include <algorithm>
#include <stdio.h>

#include "fl_internal.h"

namespace {

#include "fl_device.cuh"
#include "fl_step.cuh"

// insertParticles (fluids4.0/fluid_kernels.cu:22-53) with warp-aggregated
// counting: a run of consecutive lanes that land in the same cell elects its
// first lane, which adds the run's length with a single atomic; each lane's
// arrival rank is the run's base plus its position in the run. The rank is
// only an intermediate: the canonical within-cell order is fixed later by
// k_sort_cells.
// Batched systems: a point's cell is offset by its scene's cell_base, so
// every scene owns a contiguous range of cell entries (its out-of-range bin
// last) and one scan over all of them yields each scene's segments.
template <bool BATCH>
__global__ void __launch_bounds__(kThreads)
k_insert(const __grid_constant__ DevParams P0, const SceneTab T, int n, const float4 *__restrict__ pos,
         uint32_t *__restrict__ cell_out, uint32_t *__restrict__ rank_out,
         uint32_t *__restrict__ gcell_out, uint32_t *__restrict__ cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    uint32_t cell = 0;
    if (valid) {
        const DevParams &P = BATCH ? T.params[T.point_scene[i]] : P0;
        const uint32_t local = cell_of(P, pos[i]);
        cell = (uint32_t)P.cell_base + local;
        cell_out[i] = cell;
        if (gcell_out) gcell_out[i] = (local == (uint32_t)P.ncells) ? kUndef : cell;
    }
    // Points come in the previous step's sorted order, so equal cells sit in
    // runs of consecutive lanes: each run reserves its slots with one atomic
    // (valid lanes are a prefix of the warp).
    const unsigned active = __ballot_sync(0xffffffffu, valid);
    if (!valid) return;
    const unsigned lane = lane_id();
    const uint32_t prev = __shfl_up_sync(active, cell, 1);
    const bool head = lane == 0 || prev != cell;
    const unsigned heads = __ballot_sync(active, head);
    const unsigned upto = (lane == 31) ? 0xffffffffu : ((2u << lane) - 1u);   // lanes 0..lane
    const int first = 31 - __clz(heads & upto);                              // this run's head
    const unsigned later = heads & ~upto;
    const int end = later ? __ffs(later) - 1 : 32 - __clz(active);            // one past the run
    uint32_t base = 0;
    if (head) base = atomicAdd(&cnt[cell], (uint32_t)(end - (int)lane));
    base = __shfl_sync(active, base, first);
    rank_out[i] = base + (uint32_t)((int)lane - first);
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
// Canonical within-cell order. A warp sorts the point indices of one cell
// segment of src at a time, ascending, so slot off[c]+k holds the k-th lowest
// index in cell c -- the order a serial insert (gndx = cnt[cell]++) yields.
// Segments up to 128 points are sorted in registers by a warp bitonic
// network (K keys per lane, element e = lane*K + r); larger ones by a block
// each (k_sort_big).
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

// Mode 0 (phase API) also records each point's rank within its cell by
// pre-sort index (gndx_pre); mode 1 (fused step) only orders src, and
// k_gather_sorted then moves the points.
struct SortArgs {
    const uint32_t *off, *cnt;
    uint32_t *src, *scratch;
    uint32_t *gndx_pre;                // mode 0: canonical gndx by pre-sort index
    uint32_t *big_cells, *big_count;   // cell entries above 128 points, for k_sort_big
    uint32_t big_cap;
    int gcells;                        // internal cell entries (all scenes, bins included)
    uint32_t *crowd_max;               // largest in-range cell above 128 points (atomic max)
    const DevParams *scenes;           // batched: the scene table (bins at cell_base + ncells)
    const uint16_t *cell_scene;
    int ncells0;                       // single scene: its bin's entry
};

// Whether cell entry c is a scene's out-of-range bin.
__device__ __forceinline__ bool is_bin(const SortArgs &a, int c) {
    if (!a.scenes) return c == a.ncells0;
    const DevParams &P = a.scenes[a.cell_scene[c]];
    return c - P.cell_base == P.ncells;
}

template <int MODE, int K>
__device__ __forceinline__ void sort_segment(const SortArgs &a, uint32_t o, uint32_t m) {
    const unsigned lane = lane_id();
    uint32_t v[K];
#pragma unroll
    for (int r = 0; r < K; r++) {
        const uint32_t e = lane * K + r;
        v[r] = (e < m) ? a.src[o + e] : 0xffffffffu;
    }
    warp_bitonic<K>(v);
#pragma unroll
    for (int r = 0; r < K; r++) {
        const uint32_t e = lane * K + r;
        if (e < m) {
            a.src[o + e] = v[r];
            if (MODE == 0) a.gndx_pre[v[r]] = e;
        }
    }
}

// Each warp owns CELLS consecutive cell entries (2, 4 or 8; the autotuner's
// cells-per-warp knob, 4 by default): one read of their
// counts and offsets, then the cells that need ordering (a single point is
// in order already, but mode 0 still records its rank). Cells of up to 64
// points go through one pipeline, the next cell's keys loading while the
// current one sorts; cells of 65-128 points are sorted on their own
// afterwards; larger ones are listed for k_sort_big.
constexpr int kSortCells = 4;

template <int MODE, int CELLS>
__global__ void __launch_bounds__(kThreads)
k_sort_cells(const __grid_constant__ SortArgs a) {
    const int c0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * CELLS;
    if (c0 >= a.gcells) return;
    const unsigned lane = lane_id();
    const int c = c0 + (int)lane;
    const bool owned = lane < (unsigned)CELLS && c < a.gcells;
    const uint32_t my_m = owned ? a.cnt[c] : 0u;
    const uint32_t my_o = owned ? a.off[c] : 0u;
    const unsigned todo_all = __ballot_sync(0xffffffffu, my_m > (MODE == 0 ? 0u : 1u));
    const unsigned large = __ballot_sync(0xffffffffu, my_m > 64u);
    unsigned todo = todo_all & ~large;

    uint32_t m = 0, o = 0, w0 = 0xffffffffu, w1 = 0xffffffffu;
    auto fetch = [&]() {   // next small cell's size, offset and keys (element e = 2 lane + r)
        if (!todo) { m = 0; return; }
        const int k = __ffs(todo) - 1;
        todo &= todo - 1u;
        m = __shfl_sync(0xffffffffu, my_m, k);
        o = __shfl_sync(0xffffffffu, my_o, k);
        const uint32_t e = 2 * lane;
        w0 = (e < m) ? a.src[o + e] : 0xffffffffu;
        w1 = (e + 1 < m) ? a.src[o + e + 1] : 0xffffffffu;
    };
    fetch();
    while (m) {
        uint32_t v[2] = {w0, w1};
        const uint32_t cm = m, co = o;
        fetch();
        // the insert hands out a cell's slots in ascending runs (one per
        // insert warp), so a segment is often in order already
        const uint32_t next = __shfl_down_sync(0xffffffffu, v[0], 1);
        const bool in_order = __all_sync(0xffffffffu, v[0] <= v[1] && (lane == 31 || v[1] <= next));
        if (in_order && MODE != 0) continue;
        if (!in_order) warp_bitonic<2>(v);
#pragma unroll
        for (int r = 0; r < 2; r++) {
            const uint32_t e = 2 * lane + r;
            if (e < cm) {
                a.src[co + e] = v[r];
                if (MODE == 0) a.gndx_pre[v[r]] = e;
            }
        }
    }
    unsigned rest = todo_all & large;
    while (rest) {
        const int k = __ffs(rest) - 1;
        rest &= rest - 1u;
        const uint32_t lm = __shfl_sync(0xffffffffu, my_m, k);
        const uint32_t lo = __shfl_sync(0xffffffffu, my_o, k);
        if (lm <= 128) {
            sort_segment<MODE, 4>(a, lo, lm);
        } else if (lane == 0) {
            const uint32_t slot = atomicAdd(a.big_count, 1u);
            if (slot < a.big_cap) a.big_cells[slot] = (uint32_t)(c0 + k);
            if (!is_bin(a, c0 + k)) atomicMax(a.crowd_max, lm);
        }
    }
}

// Cells above 128 points (crowded regions: a collapsing scene can hold
// thousands of points in one cell), one block of kBigThreads per cell: up
// to kBigChunk keys are sorted by a block bitonic network in shared memory;
// a larger cell is sorted in chunks of kBigChunk, then every key is placed
// at its rank -- its index in its own chunk plus, for each other chunk, the
// number of smaller keys there (a binary search) -- through the scratch
// array. Keys are distinct point indices. Needs kBigChunk * 4 bytes of
// dynamic shared memory.
constexpr int kBigThreads = 1024;
constexpr uint32_t kBigChunk = 16384;

__device__ __forceinline__ void block_bitonic(uint32_t *s, uint32_t p2) {   // p2: a power of two
    for (uint32_t size = 2; size <= p2; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t t = threadIdx.x; t < p2 / 2; t += blockDim.x) {
                const uint32_t i = ((t & ~(stride - 1u)) << 1) | (t & (stride - 1u));
                const uint32_t j = i + stride;
                const uint32_t x = s[i], y = s[j];
                if ((x > y) == ((i & size) == 0)) { s[i] = y; s[j] = x; }
            }
            __syncthreads();
        }
    }
}

// Sorts src[o, o+len) in place through shared memory (all threads call it).
__device__ __forceinline__ void block_sort_range(uint32_t *s_keys, uint32_t *src, uint32_t o, uint32_t len) {
    uint32_t p2 = 256;
    while (p2 < len) p2 <<= 1;
    for (uint32_t e = threadIdx.x; e < p2; e += blockDim.x) s_keys[e] = (e < len) ? src[o + e] : 0xffffffffu;
    __syncthreads();
    block_bitonic(s_keys, p2);
    for (uint32_t e = threadIdx.x; e < len; e += blockDim.x) src[o + e] = s_keys[e];
    __syncthreads();
}

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t *a, uint32_t len, uint32_t key) {
    uint32_t lo = 0, hi = len;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

template <int MODE>
__global__ void __launch_bounds__(kBigThreads)
k_sort_big(const __grid_constant__ SortArgs a) {
    extern __shared__ uint32_t s_keys[];
    __shared__ uint32_t s_nbig;
    if (threadIdx.x == 0) s_nbig = min(*(volatile uint32_t *)a.big_count, a.big_cap);
    __syncthreads();
    const uint32_t nbig = s_nbig;
    for (uint32_t b = blockIdx.x; b < nbig; b += gridDim.x) {
        const uint32_t c = a.big_cells[b];
        const uint32_t m = a.cnt[c], o = a.off[c];
        for (uint32_t cb = 0; cb < m; cb += kBigChunk) block_sort_range(s_keys, a.src, o + cb, min(kBigChunk, m - cb));
        if (m > kBigChunk) {
            const uint32_t nch = (m + kBigChunk - 1) / kBigChunk;
            for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) {
                const uint32_t key = a.src[o + k];
                const uint32_t mine = k / kBigChunk;
                uint32_t rank = k - mine * kBigChunk;
                for (uint32_t ch = 0; ch < nch; ch++) {
                    if (ch == mine) continue;
                    const uint32_t lo = ch * kBigChunk;
                    rank += lower_bound_u32(a.src + o + lo, min(kBigChunk, m - lo), key);
                }
                a.scratch[o + rank] = key;
            }
            __syncthreads();
            for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) a.src[o + k] = a.scratch[o + k];
            __syncthreads();
        }
        if (MODE == 0)
            for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) a.gndx_pre[a.src[o + k]] = k;
        __syncthreads();
    }
    // the last block to finish clears the list for the next sort (every
    // block has read the count before it signs off)
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(a.big_count + 1, 1u) == gridDim.x - 1) {
            a.big_count[0] = 0;
            a.big_count[1] = 0;
        }
    }
}

// The cell a warp owns: its scene's parameters, its entry index (global),
// its index within the scene's grid, and whether it is the scene's
// out-of-range bin.
struct CellCtx {
    const DevParams *P;
    int c, local;
    bool overflow;
};

template <bool BATCH>
__device__ __forceinline__ CellCtx cell_ctx(const DevParams &P0, const SceneTab &T, int c) {
    CellCtx cx;
    cx.P = BATCH ? &T.params[T.cell_scene[c]] : &P0;
    cx.c = c;
    cx.local = c - cx.P->cell_base;
    cx.overflow = cx.local == cx.P->ncells;
    return cx;
}

// The move of the fused step's sort, one thread per sorted slot s: the point
// src[s] (canonical order, set by k_sort_cells in mode 1) goes to slot s
// with its band code in pos.w, its cell in gcell and its rank within the
// cell in gndx (countingSortFull, fluids4.0/fluid_kernels.cu:56-87, with
// the canonical within-cell order). The 32 slots of a warp are one word of
// each slot-flag row, so the warp stores the words whole: rows 0-2 the
// upper-band flags (ROWS >= 1), rows 3-5 the lower-band flags (ROWS == 2).
template <bool BATCH, int ROWS, bool LATE = false>
__global__ void __launch_bounds__(kThreads)
k_gather_sorted(const __grid_constant__ DevParams P0, const SceneTab T, int n, const uint32_t *__restrict__ src,
                const uint32_t *__restrict__ cell_pre, const uint32_t *__restrict__ off,
                const float4 *__restrict__ pos_in, const float4 *__restrict__ vel_in,
                const float4 *__restrict__ veval_in, const uint32_t *__restrict__ clr_in,
                float4 *__restrict__ pos_out, float4 *__restrict__ vel_out, float4 *__restrict__ veval_out,
                uint32_t *__restrict__ clr_out, uint32_t *__restrict__ gcell_out,
                uint32_t *__restrict__ gndx_out, uint32_t *__restrict__ upbits) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x * blockDim.x + (threadIdx.x & ~31u) >= (unsigned)n) return;   // whole warp past n
    const bool valid = s < n;
    uint32_t code = 0, upwords = 0;
    if (valid) {
        const uint32_t i = src[s];
        const uint32_t c = cell_pre[i];
        const DevParams &P = BATCH ? T.params[T.cell_scene[c]] : P0;
        const int local = (int)c - P.cell_base;
        float4 p = pos_in[i];
        if (ROWS >= 1) code = band_code(P, local, p);
        p.w = __uint_as_float(code);
        pos_out[s] = p;
        if (!LATE) {   // LATE: velocities, evaluated velocities, colours come from k_gather_late
            vel_out[s] = vel_in[i];
            veval_out[s] = veval_in[i];
            clr_out[s] = clr_in[i];
        }
        gcell_out[s] = (local == P.ncells) ? kUndef : c;
        gndx_out[s] = (uint32_t)s - off[c];
        upwords = (uint32_t)P.upwords;
    }
    if constexpr (ROWS >= 1) {
        const size_t word = (size_t)(s >> 5);
        const unsigned lane = lane_id();
        upwords = __shfl_sync(0xffffffffu, upwords, 0);   // lane 0 holds a point (s0 < n)
#pragma unroll
        for (int row = 0; row < 3 * ROWS; row++) {
            const unsigned b = __ballot_sync(0xffffffffu, valid && ((code >> row) & 1u));
            if (lane == 0) upbits[(size_t)row * upwords + word] = b;
        }
    }
}

// The velocities, evaluated velocities and colours of a step whose state
// came from host memory (fl_run_from_host), gathered into sorted order once
// the copy engine has delivered them: packed float3 and uint staging (null:
// zeros, as fl_set_particles clears an absent field), read through src. The
// evaluated velocity also completes slot s's pair record (the density pass
// ran before it arrived and wrote only the record's first half correctly).
__device__ __forceinline__ float4 load3_or_zero(const float *__restrict__ a, uint32_t i) {
    return a ? make_float4(a[3 * (size_t)i], a[3 * (size_t)i + 1], a[3 * (size_t)i + 2], 0.0f)
             : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void __launch_bounds__(kThreads)
k_gather_late(int n, const uint32_t *__restrict__ src, const float *__restrict__ vel3,
              const float *__restrict__ veval3, const uint32_t *__restrict__ clr, float4 *__restrict__ vel_out,
              float4 *__restrict__ veval_out, uint32_t *__restrict__ clr_out, float4 *__restrict__ pairdata) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t i = src[s];
    vel_out[s] = load3_or_zero(vel3, i);
    const float4 e = load3_or_zero(veval3, i);
    veval_out[s] = e;
    pairdata[2 * (size_t)s + 1] = e;
    clr_out[s] = clr ? clr[i] : 0u;
}

// Band codes and upper-band slot flags for an already sorted grid
// (phase-API path, after k_gather_all): warp per cell, codes into pos.w.
template <bool BATCH>
__global__ void __launch_bounds__(kThreads)
k_band_codes(const __grid_constant__ DevParams P0, const SceneTab T, int gcells,
             const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt,
             float4 *__restrict__ pos, uint32_t *__restrict__ upbits) {
    const int c = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
    if (c >= gcells) return;
    const uint32_t m = cnt[c];
    if (m == 0) return;
    const uint32_t o = off[c];
    const CellCtx cx = cell_ctx<BATCH>(P0, T, c);
    const DevParams &P = *cx.P;
    const unsigned lane = lane_id();
    for (uint32_t kb = 0; kb < m; kb += 32) {
        const uint32_t k = kb + lane;
        const bool valid = k < m;
        uint32_t code = 0;
        if (valid) {
            float4 p = pos[o + k];
            code = band_code(P, cx.local, p);
            p.w = __uint_as_float(code);
            pos[o + k] = p;
        }
        publish_upbits(P, upbits, o + kb, code, valid);
    }
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

constexpr int kDensityMaxThreads = 1024;

// computePressure (fluids4.0/fluid_kernels.cu:112-149). FGRID is the
// identity after a full sort (cu:83), so neighbour slots are read directly.
// With LIST the slots of the pairs that pass 0 < d^2 < rd2 are recorded, in
// visiting order, for the force pass (same positions, same test), together
// with each point's pair record (position and density, evaluated velocity).
template <bool PRUNE, bool LIST, bool BATCH>
__global__ void __launch_bounds__(kDensityMaxThreads, 2)
k_density(const __grid_constant__ DevParams P0, const SceneTab T, int n, const float4 *__restrict__ pos,
          const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off,
          const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ upbits,
          const float4 *__restrict__ veval, float *__restrict__ press, uint32_t *__restrict__ hitlist,
          uint32_t *__restrict__ hitcnt, float4 *__restrict__ pairdata) {
    // pruned: the lanes of a warp take points with the same lower-band bits,
    // which decide the entries of the search block a point visits
    extern __shared__ uint32_t s_dyn[];
    const int i = PRUNE ? band_grouped_slot(n, pos, gcell, 3, s_dyn) : (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) return;
    const DevParams &P = BATCH ? T.params[T.point_scene[i]] : P0;
    const uint32_t gc = gcell[i];
    if (gc == kUndef) {
        press[i] = 0.0f;
        if (LIST) hitcnt[i] = 0;
        return;
    }
    const int base = (int)gc - P.nadj;
    const float4 p = pos[i];
    const uint32_t my_code = __float_as_uint(p.w);
    float sum = 0.0f;
    uint32_t nh = 0;
    // Branch-free: every candidate's term is formed and a miss adds +0.0,
    // which leaves the sum's bits unchanged (the sum starts at +0.0 and its
    // terms are positive), so the sum is the reference's; the list store
    // is predicated. Without the divergent branch the warp skips the
    // convergence bookkeeping around it (6% faster than branching at 4M).
    uint32_t *const lrow = hitlist + list_at(P, i, 0);
    const uint32_t cap = (uint32_t)P.hcap;
    const float rd2 = P.rd2, d2 = P.d2;
    auto visit = [&](uint32_t j) {
        const float4 q = pos[j];
        const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
        const float dsq = dx * dx + dy * dy + dz * dz;
        const bool hit = dsq < rd2 && dsq > 0.0f;
        float t = (rd2 - dsq) * d2;
        t = t * t * t;
        sum += hit ? t : 0.0f;
        if (LIST) {
            if (hit && nh < cap) lrow[(size_t)nh * 32u] = j;
            nh += hit ? 1u : 0u;
        }
    };
    for (int c = 0; c < P.gridAdjCnt; c++) {
        CandIter it;
        cand_begin<PRUNE>(it, P, c, base + P.adj[c], my_code, true, off, cnt, upbits);
        if (PRUNE && it.U == 0u) {   // the own cell: no flags to consult, every slot in order
            for (uint32_t j = it.lo; j < it.hi; j++) visit(j);
            continue;
        }
        uint32_t j;
        while (cand_next<PRUNE>(it, P, upbits, j)) visit(j);
    }
    sum = sum * P.pmass * P.poly6kern;
    if (sum == 0.0f) sum = 1.0f;
    press[i] = sum;
    if (LIST) {
        hitcnt[i] = nh;
        const float4 e = veval[i];
        pairdata[2 * (size_t)i] = make_float4(p.x, p.y, p.z, sum);
        pairdata[2 * (size_t)i + 1] = make_float4(e.x, e.y, e.z, 0.0f);
    }
}

// computeForce (fluids4.0/fluid_kernels.cu:180-217) in two stages per warp:
// lanes first walk their candidates with the cheap distance test and push
// each hit's slot onto a per-thread list in shared memory; whenever some
// lane's list is full (and at the end) the warp drains every list, each
// lane evaluating its own hits in the order found. The long pair-force
// arithmetic (sqrt, two IEEE divisions) then runs with every lane busy
// instead of inside a branch few lanes take, and each point still adds its
// pair terms in the reference's order.
constexpr int kForceThreads = 128;
constexpr int kHitCap = 32;
constexpr uint32_t kPairsInFlight = 4;   // pairs of a list drained per round of loads

// Neighbour j's data from the field arrays.
__device__ __forceinline__ void add_pair_force(const DevParams &P, ForcePoint &fp, uint32_t j,
                                               const float4 *__restrict__ pos,
                                               const float4 *__restrict__ veval,
                                               const float *__restrict__ press) {
    add_pair_terms(P, fp, pos[j], veval[j], press[j]);
}

// Neighbour j's data from its pair record (the same values, one sector).
__device__ __forceinline__ void add_pair_force_rec(const DevParams &P, ForcePoint &fp, uint32_t j,
                                                   const float4 *__restrict__ pairdata) {
    const float4 q = pairdata[2 * (size_t)j];
    add_pair_terms(P, fp, q, pairdata[2 * (size_t)j + 1], q.w);
}

__device__ __forceinline__ void drain_hits(const DevParams &P, ForcePoint &fp, uint32_t &nhits,
                                           const uint32_t *hits, const float4 *__restrict__ pos,
                                           const float4 *__restrict__ veval,
                                           const float *__restrict__ press) {
    const uint32_t most = __reduce_max_sync(0xffffffffu, nhits);
    for (uint32_t t = 0; t < most; t++)
        if (t < nhits) add_pair_force(P, fp, hits[t * kForceThreads], pos, veval, press);
    nhits = 0;
}

// The force on point i (all 32 lanes of the warp must call this). With
// LIST the pairs come from the density pass's list (every lane draining its
// own list in step); a point whose pairs overflowed the list walks its
// candidates again. Without LIST (no density pass since the last sort) the
// warp walks and drains per-lane hit lists in shared memory.
template <bool PRUNE, bool LIST>
__device__ __forceinline__ float3 force_of(const DevParams &P, int i, bool active, uint32_t gc,
                                           const float4 *__restrict__ pos,
                                           const float4 *__restrict__ veval,
                                           const float *__restrict__ press,
                                           const uint32_t *__restrict__ off,
                                           const uint32_t *__restrict__ cnt,
                                           const uint32_t *__restrict__ upbits,
                                           const uint32_t *__restrict__ hitlist,
                                           const uint32_t *__restrict__ hitcnt,
                                           const float4 *__restrict__ pairdata) {
    ForcePoint fp;
    fp.f = make_float3(0.0f, 0.0f, 0.0f);
    uint32_t my_code = 0;
    int base = 0;
    if (active) {
        fp.p = pos[i];
        fp.vi = veval[i];
        fp.di = press[i];
        fp.pi = (fp.di - P.prest_dens) * P.pintstiff;
        my_code = __float_as_uint(fp.p.w);
        base = (int)gc - P.nadj;
    }
    if constexpr (LIST) {
        // No shared memory here, so the whole unified L1 caches the
        // neighbour reads. A lane whose list overflowed (rare with 128
        // entries) walks its candidates and adds each pair as found, in the
        // same order.
        const uint32_t nh = active ? hitcnt[i] : 0u;
        const bool over = nh > (uint32_t)P.hcap;
        if (!__any_sync(0xffffffffu, over)) {
            // Four pairs in flight: their records are all requested before
            // the first of them is evaluated, and the next four list entries
            // while they are, so the drain (bound by these dependent loads,
            // not by arithmetic) waits one round trip per four pairs. Each
            // point still adds its pairs in list order; a lane past its
            // list's end adds +0.0, which leaves a force sum's bits unchanged
            // (a sum that starts at +0.0 never becomes -0.0), so the adds
            // need no branch.
            const uint32_t most = __reduce_max_sync(0xffffffffu, nh);
            uint32_t t = 0;
            uint32_t jn[kPairsInFlight];
#pragma unroll
            for (uint32_t k = 0; k < kPairsInFlight; k++) jn[k] = (k < nh) ? hitlist[list_at(P, i, k)] : 0u;
            for (; t + kPairsInFlight <= most; t += kPairsInFlight) {
                float4 q[kPairsInFlight], v[kPairsInFlight];
#pragma unroll
                for (uint32_t k = 0; k < kPairsInFlight; k++) {
                    q[k] = make_float4(0.f, 0.f, 0.f, 1.f);
                    v[k] = q[k];
                    if (t + k < nh) {
                        q[k] = pairdata[2 * (size_t)jn[k]];
                        v[k] = pairdata[2 * (size_t)jn[k] + 1];
                    }
                }
#pragma unroll
                for (uint32_t k = 0; k < kPairsInFlight; k++) {
                    const uint32_t tn = t + kPairsInFlight + k;
                    jn[k] = (tn < nh) ? hitlist[list_at(P, i, tn)] : 0u;
                }
#pragma unroll
                for (uint32_t k = 0; k < kPairsInFlight; k++) {
                    const float3 tk = pair_term(P, fp.p, fp.pi, fp.vi, fp.di, q[k], v[k], q[k].w);
                    const bool ok = t + k < nh;
                    fp.f.x += ok ? tk.x : 0.0f;
                    fp.f.y += ok ? tk.y : 0.0f;
                    fp.f.z += ok ? tk.z : 0.0f;
                }
            }
            for (; t < most; t++)
                if (t < nh) add_pair_force_rec(P, fp, hitlist[list_at(P, i, t)], pairdata);
            return fp.f;
        }
        if (!over) {
            for (uint32_t t = 0; t < nh; t++) add_pair_force_rec(P, fp, hitlist[list_at(P, i, t)], pairdata);
            return fp.f;
        }
        for (int c = 0; c < P.gridAdjCnt; c++) {
            CandIter it;
            cand_begin<PRUNE>(it, P, c, base + P.adj[c], my_code, true, off, cnt, upbits);
            uint32_t j;
            while (cand_next<PRUNE>(it, P, upbits, j)) {
                const float4 q = pos[j];
                const float dx = fp.p.x - q.x, dy = fp.p.y - q.y, dz = fp.p.z - q.z;
                const float dsq = dx * dx + dy * dy + dz * dz;
                if (dsq < P.rd2 && dsq > 0.0f) add_pair_force(P, fp, j, pos, veval, press);
            }
        }
        return fp.f;
    }
    __shared__ uint32_t s_hits[kHitCap * kForceThreads];
    uint32_t *hits = s_hits + threadIdx.x;
    uint32_t nhits = 0;
    for (int c = 0; c < P.gridAdjCnt; c++) {
        CandIter it;
        cand_begin<PRUNE>(it, P, c, base + P.adj[c], my_code, active, off, cnt, upbits);
        for (;;) {
            uint32_t j = 0;
            const bool have = cand_next<PRUNE>(it, P, upbits, j);
            if (!__any_sync(0xffffffffu, have)) break;
            if (have) {
                const float4 q = pos[j];
                const float dx = fp.p.x - q.x, dy = fp.p.y - q.y, dz = fp.p.z - q.z;
                const float dsq = dx * dx + dy * dy + dz * dz;
                if (dsq < P.rd2 && dsq > 0.0f) hits[(nhits++) * kForceThreads] = j;
            }
            if (__any_sync(0xffffffffu, nhits == kHitCap))
                drain_hits(P, fp, nhits, hits, pos, veval, press);
        }
    }
    drain_hits(P, fp, nhits, hits, pos, veval, press);
    return fp.f;
}

template <bool PRUNE, bool LIST, bool BATCH>
__global__ void __launch_bounds__(kForceThreads)
k_force(const __grid_constant__ DevParams P0, const SceneTab T, int n, const float4 *__restrict__ pos,
        const float4 *__restrict__ veval, const float *__restrict__ press,
        const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off,
        const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ upbits,
        const uint32_t *__restrict__ hitlist, const uint32_t *__restrict__ hitcnt,
        const float4 *__restrict__ pairdata, float4 *__restrict__ force) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const DevParams &P = (BATCH && i < n) ? T.params[T.point_scene[i]] : P0;
    const uint32_t gc = (i < n) ? gcell[i] : kUndef;
    const bool active = gc != kUndef;
    const float3 f = force_of<PRUNE, LIST>(P, i, active, gc, pos, veval, press, off, cnt, upbits,
                                           hitlist, hitcnt, pairdata);
    if (i < n) force[i] = active ? make_float4(f.x, f.y, f.z, 0.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
}

// advanceParticles (fluids4.0/fluid_kernels.cu:332-420), in place.
template <bool BATCH>
__global__ void __launch_bounds__(kThreads)
k_advance(const __grid_constant__ DevParams P0, const SceneTab T, int n, float time, float dt, float ss,
          const uint32_t *__restrict__ gcell, const float4 *__restrict__ force,
          float4 *__restrict__ pos, float4 *__restrict__ vel, float4 *__restrict__ veval) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevParams &P = BATCH ? T.params[T.point_scene[i]] : P0;
    if (BATCH) ss = P.sim_scale;   // each scene advances with its own scale
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
// At least 6 blocks of 128 per SM (64 registers used): the list drain keeps
// four pairs' loads in flight, which measured faster than more resident
// warps at 40 registers (0.375 vs 0.460 ms at 4M points; one, two and
// eight pairs in flight, and other register bounds, were slower).
template <bool PRUNE, bool LIST, bool BATCH>
__global__ void __launch_bounds__(kForceThreads, 6)
k_force_advance(const __grid_constant__ DevParams P0, const SceneTab T, int n, float *time_dev, int slot,
                float dt,
                const float4 *__restrict__ pos_in, const float4 *__restrict__ veval_in,
                const float *__restrict__ press, const uint32_t *__restrict__ gcell,
                const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt,
                const uint32_t *__restrict__ upbits,
                const uint32_t *__restrict__ hitlist, const uint32_t *__restrict__ hitcnt,
                const float4 *__restrict__ pairdata, float4 *__restrict__ vel, float4 *__restrict__ force,
                float4 *__restrict__ pos_out, float4 *__restrict__ veval_out,
                uint32_t *__restrict__ err, int base, float *__restrict__ host_pos) {
    // host_pos (fl_run_from_host): the new positions also go straight into
    // the caller's page-locked float3 array, in slot order, while the pass
    // runs (each warp's 384 contiguous bytes over the host link)
    const int i = base + blockIdx.x * blockDim.x + threadIdx.x;   // base: a whole number of blocks
    const float time = time_dev[slot];
    if (i == 0) time_dev[slot ^ 1] = time + dt;
    const DevParams &P = (BATCH && i < n) ? T.params[T.point_scene[i]] : P0;
    const uint32_t gc = (i < n) ? gcell[i] : kUndef;
    const bool active = gc != kUndef;
    const float3 f = force_of<PRUNE, LIST>(P, i, active, gc, pos_in, veval_in, press, off, cnt, upbits,
                                           hitlist, hitcnt, pairdata);
    if (i >= n) return;
    if (!active) {
        force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        pos_out[i] = make_float4(-1000.f, -1000.f, -1000.f, 0.f);
        vel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        veval_out[i] = veval_in[i];
        if (host_pos) {
            host_pos[3 * (size_t)i] = -1000.f;
            host_pos[3 * (size_t)i + 1] = -1000.f;
            host_pos[3 * (size_t)i + 2] = -1000.f;
        }
        return;
    }
    force[i] = f4(f);
    float3 po, vo, eo;
    advance_point(P, time, dt, P.sim_scale, f, xyz(pos_in[i]), xyz(vel[i]), xyz(veval_in[i]), po, vo, eo);
    if (!(isfinite(po.x) && isfinite(po.y) && isfinite(po.z))) atomicOr(err, FL_DEV_NONFINITE);
    pos_out[i] = f4(po);
    vel[i] = f4(vo);
    veval_out[i] = f4(eo);
    if (host_pos) {
        host_pos[3 * (size_t)i] = po.x;
        host_pos[3 * (size_t)i + 1] = po.y;
        host_pos[3 * (size_t)i + 2] = po.z;
    }
}

// ---------------------------------------------------------------------------
__global__ void k_set_time(float *time_dev, float value) { *time_dev = value; }
__global__ void k_set_word(uint32_t *word, uint32_t value) { *word = value; }

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

// Up to four float3 fields at once (uploads read straight from page-locked
// host memory: one pass keeps more of the link's requests in flight).
struct Unpack3Set {
    const float *src[4];
    float4 *dst[4];
    int count;
};

__global__ void k_unpack3_set(int n, const __grid_constant__ Unpack3Set u) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 v[4];
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (k < u.count) v[k] = make_float3(u.src[k][3 * i + 0], u.src[k][3 * i + 1], u.src[k][3 * i + 2]);
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (k < u.count) u.dst[k][i] = make_float4(v[k].x, v[k].y, v[k].z, 0.0f);
}

// FGCELL readback of a batched system: internal cell entries count one
// out-of-range bin per earlier scene; the reference layout does not.
__global__ void k_gcell_ref(int n, const uint32_t *__restrict__ gcell, const uint16_t *__restrict__ scene,
                            uint32_t *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t g = gcell[i];
    out[i] = (g == kUndef) ? kUndef : g - (uint32_t)scene[i];
}

__global__ void k_grid_identity(int n, const uint32_t *__restrict__ gcell, uint32_t *__restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[i] = gcell ? ((gcell[i] != kUndef) ? (uint32_t)i : kUndef) : kUndef;
}

// sampleParticles (fluids4.0/fluid_kernels.cu:263-308): a Gaussian-weighted
// particle count at every voxel of a res.x x res.y x res.z lattice over
// [bmin, bmax), read from the sorted grid. Voxel (x, y, z) sits at
// bmin + (x / res.x, y / res.y, z / res.z) * (bmax - bmin) and writes
// out[(z * res.y + y) * res.x + x] (the reference's final store; its
// out-of-range store uses another order, an upstream slip not kept here);
// voxels outside the scan range read 0.
__global__ void __launch_bounds__(512)
k_sample_volume(const __grid_constant__ DevParams P, int3 res, float3 bmin, float3 bmax, float scalar,
                float gausskern, float h2, const float4 *__restrict__ pos, const uint32_t *__restrict__ off,
                const uint32_t *__restrict__ cnt, float *__restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= res.x || y >= res.y || z >= res.z) return;
    const float px = bmin.x + ((float)x / (float)res.x) * (bmax.x - bmin.x);
    const float py = bmin.y + ((float)y / (float)res.y) * (bmax.y - bmin.y);
    const float pz = bmin.z + ((float)z / (float)res.z) * (bmax.z - bmin.z);
    const size_t idx = ((size_t)z * res.y + y) * res.x + x;
    const uint32_t cell = cell_of(P, make_float4(px, py, pz, 0.0f));
    if (cell == (uint32_t)P.ncells) {
        out[idx] = 0.0f;
        return;
    }
    const int base = (int)cell - P.nadj;
    float v = 0.0f;
    for (int c = 0; c < P.gridAdjCnt; c++) {
        const int cl = base + P.adj[c];
        const uint32_t j0 = off[cl], j1 = j0 + cnt[cl];
        for (uint32_t j = j0; j < j1; j++) {
            const float4 q = pos[j];
            const float dx = px - q.x, dy = py - q.y, dz = pz - q.z;
            float dsq = dx * dx + dy * dy + dz * dz;
            if (dsq < P.rd2 && dsq > 0.0f) {
                dsq = sqrtf(dsq * P.d2);
                v += gausskern * expf(-(dsq * dsq) / h2);
            }
        }
    }
    out[idx] = v * scalar;
}

// Global conservation sums in FP64, per scene: block (chunk, scene) adds up
// kConsChunk points of its scene into kConsVals partial sums (the only FP64
// work of the library). Points parked outside the domain (-1000, -1000,
// -1000) are left out. Values: count, mass, momentum (3), kinetic energy,
// gravitational potential energy, and the first moment of position (3,
// world units; divided by the count on the host for the centre of mass).
constexpr int kConsVals = 10;
constexpr int kConsChunk = 8192;
constexpr int kConsThreads = 256;

__global__ void __launch_bounds__(kConsThreads)
k_conservation(const __grid_constant__ DevParams P0, const SceneTab T, const int *__restrict__ sbase,
               const int *__restrict__ sn, int nchunks, const float4 *__restrict__ pos,
               const float4 *__restrict__ vel, double *__restrict__ partial) {
    const int chunk = blockIdx.x, scene = blockIdx.y;
    const DevParams &P = T.params ? T.params[scene] : P0;
    const int b = sbase[scene], m = sn[scene];
    const double mass = P.pmass, ss = P.sim_scale;
    double acc[kConsVals];
#pragma unroll
    for (int k = 0; k < kConsVals; k++) acc[k] = 0.0;
    const int lo = chunk * kConsChunk;
    for (int k = lo + (int)threadIdx.x; k < lo + kConsChunk && k < m; k += kConsThreads) {
        const float4 x = pos[b + k];
        if (x.x == -1000.0f && x.y == -1000.0f && x.z == -1000.0f) continue;
        const float4 v = vel[b + k];
        acc[0] += 1.0;
        acc[1] += mass;
        acc[2] += mass * v.x; acc[3] += mass * v.y; acc[4] += mass * v.z;
        acc[5] += 0.5 * mass * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
        acc[6] -= mass * ss * ((double)P.gravity.x * x.x + (double)P.gravity.y * x.y + (double)P.gravity.z * x.z);
        acc[7] += x.x; acc[8] += x.y; acc[9] += x.z;
    }
    __shared__ double sm[kConsVals][kConsThreads / 32];
    const int w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kConsVals; k++) {
        double t = acc[k];
        for (int d = 16; d > 0; d >>= 1) t += __shfl_down_sync(0xffffffffu, t, d);
        if ((threadIdx.x & 31u) == 0) sm[k][w] = t;
    }
    __syncthreads();
    if (threadIdx.x < kConsVals) {
        double t = 0.0;
        for (int q = 0; q < kConsThreads / 32; q++) t += sm[threadIdx.x][q];
        partial[((size_t)scene * nchunks + chunk) * kConsVals + threadIdx.x] = t;
    }
}

// IntegrityCheck (fluids4.0/fluid_system.cpp:2426-2453): every sorted slot of
// cell g must carry gcell == g and gndx == its rank; tail slots must be UNDEF.
template <bool BATCH>
__global__ void k_integrity(const __grid_constant__ DevParams P0, const SceneTab T, int gcells, int n,
                            const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt,
                            const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ gndx,
                            unsigned long long *bad) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= gcells) return;
    const CellCtx cx = cell_ctx<BATCH>(P0, T, g);
    const uint32_t o = off[g], m = cnt[g];
    unsigned long long b = 0;
    for (uint32_t k = 0; k < m; k++) {
        const uint32_t s = o + k;
        if (s >= (uint32_t)n) { b++; continue; }
        const uint32_t want = cx.overflow ? kUndef : (uint32_t)g;
        if (gcell[s] != want || gndx[s] != k) b++;
    }
    if (b) atomicAdd(bad, b);
}

}  // namespace

// ---------------------------------------------------------------------------
// Launch wrappers.


int fl_launch_insert(fl_system *s, uint32_t *gcell_pre_or_null) {
    if (s->n == 0) return FL_OK;
    auto kern = s->batched ? k_insert<true> : k_insert<false>;
    kern<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->n, s->f[F_POS].cur<float4>(), s->cell_pre, s->rank_tmp, gcell_pre_or_null,
        s->cnt);
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

int fl_kernels_init(fl_system *s) {
    (void)s;
    const int smem = (int)(kBigChunk * sizeof(uint32_t));
    FL_CUDA_TRY(cudaFuncSetAttribute(k_sort_big<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    FL_CUDA_TRY(cudaFuncSetAttribute(k_sort_big<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    return FL_OK;
}

size_t fl_big_cells_cap(int max_points) { return (size_t)(max_points > 0 ? max_points : 1) / 129 + 1; }

int fl_launch_sort_cells(fl_system *s, int mode, bool late) {
    SortArgs a = {};
    a.off = s->off; a.cnt = s->cnt; a.src = s->src; a.scratch = s->rank_tmp;
    a.big_cells = s->big_cells; a.big_count = s->big_count;
    a.big_cap = (uint32_t)fl_big_cells_cap(s->max_points);
    a.gcells = s->gcells;
    a.crowd_max = s->crowd_dev;
    a.scenes = s->batched ? s->d_scenes : nullptr;
    a.cell_scene = s->cell_scene;
    a.ncells0 = s->ncells;
    if (mode == 0) a.gndx_pre = s->f[F_GNDX].cur<uint32_t>();
    const int bs = s->blk_sort ? s->blk_sort : kThreads;
    const int cells = s->sort_cells ? s->sort_cells : kSortCells;
    const int grid = blocks_for((long long)s->gcells, (bs / 32) * cells);
    auto sort_kernel = [&](int mode) {
        if (cells == 2) return mode == 0 ? k_sort_cells<0, 2> : k_sort_cells<1, 2>;
        if (cells == 8) return mode == 0 ? k_sort_cells<0, 8> : k_sort_cells<1, 8>;
        return mode == 0 ? k_sort_cells<0, 4> : k_sort_cells<1, 4>;
    };
    // crowded cells: at most n / 129 of them, one block each, a block per SM;
    // the list count (big_count[0]) and the blocks' sign-off count
    // (big_count[1]) start at zero and k_sort_big leaves them so
    const int big_grid = (int)std::min<size_t>((size_t)s->num_sms, fl_big_cells_cap(s->n));
    const size_t big_smem = kBigChunk * sizeof(uint32_t);
    if (mode == 0) {
        sort_kernel(0)<<<grid, bs, 0, s->stream>>>(a);
        FL_LAUNCH_CHECK("sort_cells");
        k_sort_big<0><<<big_grid, kBigThreads, big_smem, s->stream>>>(a);
        FL_LAUNCH_CHECK("sort_big");
        return FL_OK;
    }
    sort_kernel(1)<<<grid, bs, 0, s->stream>>>(a);
    FL_LAUNCH_CHECK("sort_cells");
    k_sort_big<1><<<big_grid, kBigThreads, big_smem, s->stream>>>(a);
    FL_LAUNCH_CHECK("sort_big");
    if (s->n > 0) {
        const int rows = s->D.prune ? mode : 0;
        if (late && (s->batched || rows == 2))
            return fl_fail(FL_ERR_STATE, "sort: late velocities only on a plain system's step");
        auto gather = late ? (rows == 1 ? k_gather_sorted<false, 1, true> : k_gather_sorted<false, 0, true>)
                      : s->batched ? (rows == 2 ? k_gather_sorted<true, 2>
                                                : rows == 1 ? k_gather_sorted<true, 1> : k_gather_sorted<true, 0>)
                                   : (rows == 2 ? k_gather_sorted<false, 2>
                                                : rows == 1 ? k_gather_sorted<false, 1> : k_gather_sorted<false, 0>);
        gather<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(
            s->D, fl_scene_tab(s), s->n, s->src, s->cell_pre, s->off, s->f[F_POS].cur<float4>(),
            s->f[F_VEL].cur<float4>(), s->f[F_VEVAL].cur<float4>(), s->f[F_CLR].cur<uint32_t>(),
            s->f[F_POS].nxt<float4>(), s->f[F_VEL].nxt<float4>(), s->f[F_VEVAL].nxt<float4>(),
            s->f[F_CLR].nxt<uint32_t>(), s->f[F_GCELL].nxt<uint32_t>(), s->f[F_GNDX].nxt<uint32_t>(), s->upbits);
        FL_LAUNCH_CHECK("gather_sorted");
    }
    s->codes_valid = s->D.prune;
    return FL_OK;
}

int fl_launch_gather_late(fl_system *s, const float *vel3, const float *veval3, const uint32_t *clr) {
    if (s->n == 0) return FL_OK;
    k_gather_late<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(
        s->n, s->src, vel3, veval3, clr, s->f[F_VEL].cur<float4>(), s->f[F_VEVAL].cur<float4>(),
        s->f[F_CLR].cur<uint32_t>(), s->pairdata);
    FL_LAUNCH_CHECK("gather_late");
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

size_t fl_upbits_bytes(const fl_system *s) { return 3 * sizeof(uint32_t) * (size_t)s->D.upwords; }

// Pruned neighbour passes need gridSrch == 2 (every scene of a batch) and
// band codes that match the live positions (set by the fused sort or
// fl_launch_band_codes).
static bool use_prune(const fl_system *s) { return s->D.prune && s->codes_valid; }

int fl_launch_band_codes(fl_system *s) {
    if (!s->D.prune) { s->codes_valid = 0; return FL_OK; }
    const int grid = blocks_for((long long)s->gcells, kThreads / 32);
    FL_CUDA_TRY(cudaMemsetAsync(s->upbits, 0, fl_upbits_bytes(s), s->stream));
    auto kern = s->batched ? k_band_codes<true> : k_band_codes<false>;
    kern<<<grid, kThreads, 0, s->stream>>>(s->D, fl_scene_tab(s), s->gcells, s->off, s->cnt,
                                          s->f[F_POS].cur<float4>(), s->upbits);
    FL_LAUNCH_CHECK("band_codes");
    s->codes_valid = 1;
    return FL_OK;
}

template <bool BATCH>
static auto density_kernel(bool prune) {
    return prune ? k_density<true, true, BATCH> : k_density<false, true, BATCH>;
}

int fl_launch_density(fl_system *s) {
    if (s->n == 0) return FL_OK;
    if (s->passes == FL_PASSES_POINT_PAIRS && use_prune(s)) return fl_launch_density_pairs(s);
    auto kern = s->batched ? density_kernel<true>(use_prune(s)) : density_kernel<false>(use_prune(s));
    const int bs = s->blk_density ? s->blk_density : kThreads;
    kern<<<blocks_for(s->n, bs), bs, grouping_smem(bs, kBandKeys), s->stream>>>(
        s->D, fl_scene_tab(s), s->n, s->f[F_POS].cur<float4>(), s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt,
        s->upbits, s->f[F_VEVAL].cur<float4>(), s->f[F_PRESS].cur<float>(), s->hitlist, s->hitcnt, s->pairdata);
    FL_LAUNCH_CHECK("density");
    s->lists_valid = 1;
    return FL_OK;
}

template <bool LIST, bool BATCH>
static auto force_kernel(bool prune) {
    return prune ? k_force<true, LIST, BATCH> : k_force<false, LIST, BATCH>;
}
template <bool LIST, bool BATCH>
static auto force_advance_kernel(bool prune) {
    return prune ? k_force_advance<true, LIST, BATCH> : k_force_advance<false, LIST, BATCH>;
}

int fl_launch_force(fl_system *s) {
    if (s->n == 0) return FL_OK;
    const bool pr = use_prune(s);
    auto kern = s->lists_valid ? (s->batched ? force_kernel<true, true>(pr) : force_kernel<true, false>(pr))
                               : (s->batched ? force_kernel<false, true>(pr) : force_kernel<false, false>(pr));
    const int bs = s->blk_force ? s->blk_force : kForceThreads;
    kern<<<blocks_for(s->n, bs), bs, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->n, s->f[F_POS].cur<float4>(), s->f[F_VEVAL].cur<float4>(),
        s->f[F_PRESS].cur<float>(), s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt, s->upbits,
        s->hitlist, s->hitcnt, s->pairdata, s->f[F_FORCE].cur<float4>());
    FL_LAUNCH_CHECK("force");
    return FL_OK;
}

int fl_force_block(const fl_system *s) { return s->blk_force ? s->blk_force : kForceThreads; }

int fl_launch_force_advance(fl_system *s, float dt, int begin, int end, float *host_pos) {
    const bool pr = use_prune(s);
    auto kern = s->lists_valid
                    ? (s->batched ? force_advance_kernel<true, true>(pr) : force_advance_kernel<true, false>(pr))
                    : (s->batched ? force_advance_kernel<false, true>(pr) : force_advance_kernel<false, false>(pr));
    const int bs = fl_force_block(s);
    if (end < 0) end = s->n;
    if (begin % bs != 0 || (end != s->n && end % bs != 0) || begin > end)
        return fl_fail(FL_ERR_ARG, "force_advance: slot range [%d, %d) not in whole blocks of %d", begin, end, bs);
    const int count = end - begin;
    kern<<<blocks_for(count > 0 ? count : 1, bs), bs, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->n, s->time_dev, s->time_slot, dt, s->f[F_POS].cur<float4>(),
        s->f[F_VEVAL].cur<float4>(), s->f[F_PRESS].cur<float>(), s->f[F_GCELL].cur<uint32_t>(), s->off,
        s->cnt, s->upbits, s->hitlist, s->hitcnt, s->pairdata,
        s->f[F_VEL].cur<float4>(), s->f[F_FORCE].cur<float4>(),
        s->f[F_POS].nxt<float4>(), s->f[F_VEVAL].nxt<float4>(), s->dev_err, begin, host_pos);
    FL_LAUNCH_CHECK("force_advance");
    return FL_OK;
}

int fl_launch_advance(fl_system *s, float time, float dt, float ss) {
    if (s->n == 0) return FL_OK;
    auto kern = s->batched ? k_advance<true> : k_advance<false>;
    kern<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->n, time, dt, ss, s->f[F_GCELL].cur<uint32_t>(), s->f[F_FORCE].cur<float4>(),
        s->f[F_POS].cur<float4>(), s->f[F_VEL].cur<float4>(), s->f[F_VEVAL].cur<float4>());
    FL_LAUNCH_CHECK("advance");
    return FL_OK;
}

int fl_launch_set_time(fl_system *s, int slot, float value) {
    k_set_time<<<1, 1, 0, s->stream>>>(s->time_dev + slot, value);
    FL_LAUNCH_CHECK("set_time");
    return FL_OK;
}

int fl_launch_set_word(fl_system *s, uint32_t *word, uint32_t value) {
    k_set_word<<<1, 1, 0, s->stream>>>(word, value);
    FL_LAUNCH_CHECK("set_word");
    return FL_OK;
}

int fl_launch_pack3(fl_system *s, const float4 *src, float *dst, int n, cudaStream_t stream) {
    if (n == 0) return FL_OK;
    k_pack3<<<blocks_for(n, kThreads), kThreads, 0, stream ? stream : s->stream>>>(n, src, dst);
    FL_LAUNCH_CHECK("pack3");
    return FL_OK;
}

int fl_launch_unpack3_set(fl_system *s, int count, const float *const *src, float4 *const *dst, int n) {
    if (n == 0 || count == 0) return FL_OK;
    Unpack3Set u = {};
    u.count = count;
    for (int k = 0; k < count; k++) { u.src[k] = src[k]; u.dst[k] = dst[k]; }
    k_unpack3_set<<<blocks_for(n, kThreads), kThreads, 0, s->stream>>>(n, u);
    FL_LAUNCH_CHECK("unpack3_set");
    return FL_OK;
}

int fl_launch_unpack3(fl_system *s, const float *src, float4 *dst, int n) {
    if (n == 0) return FL_OK;
    k_unpack3<<<blocks_for(n, kThreads), kThreads, 0, s->stream>>>(n, src, dst);
    FL_LAUNCH_CHECK("unpack3");
    return FL_OK;
}

int fl_launch_gcell_ref(fl_system *s, uint32_t *dst) {
    if (s->n == 0) return FL_OK;
    k_gcell_ref<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(s->n, s->f[F_GCELL].cur<uint32_t>(),
                                                                         s->point_scene, dst);
    FL_LAUNCH_CHECK("gcell_ref");
    return FL_OK;
}

// FGRID readback: the identity on in-range sorted slots, GRID_UNDEF elsewhere
// (gcell null: no sort yet, everything UNDEF).
int fl_launch_grid_identity(fl_system *s, uint32_t *dst, int n, const uint32_t *gcell) {
    if (n == 0) return FL_OK;
    k_grid_identity<<<blocks_for(n, kThreads), kThreads, 0, s->stream>>>(n, gcell, dst);
    FL_LAUNCH_CHECK("grid_identity");
    return FL_OK;
}

int fl_launch_sample_volume(fl_system *s, const int res[3], const float bmin[3], const float bmax[3],
                            float scalar, float gausskern, float h2, float *out) {
    const dim3 block(8, 8, 8);
    const dim3 grid((unsigned)((res[0] + 7) / 8), (unsigned)((res[1] + 7) / 8), (unsigned)((res[2] + 7) / 8));
    k_sample_volume<<<grid, block, 0, s->stream>>>(s->D, make_int3(res[0], res[1], res[2]),
                                                    make_float3(bmin[0], bmin[1], bmin[2]),
                                                    make_float3(bmax[0], bmax[1], bmax[2]), scalar, gausskern, h2,
                                                    s->f[F_POS].cur<float4>(), s->off, s->cnt, out);
    FL_LAUNCH_CHECK("sample_volume");
    return FL_OK;
}

int fl_conservation_chunks(int max_scene_points) {
    return max_scene_points <= 0 ? 1 : (max_scene_points + kConsChunk - 1) / kConsChunk;
}

int fl_launch_conservation(fl_system *s, const int *sbase, const int *sn, int nchunks, double *partial) {
    dim3 grid((unsigned)nchunks, (unsigned)s->nscenes);
    k_conservation<<<grid, kConsThreads, 0, s->stream>>>(s->D, fl_scene_tab(s), sbase, sn, nchunks,
                                                         s->f[F_POS].cur<float4>(), s->f[F_VEL].cur<float4>(),
                                                         partial);
    FL_LAUNCH_CHECK("conservation");
    return FL_OK;
}

int fl_launch_integrity(fl_system *s, unsigned long long *bad_dev) {
    auto kern = s->batched ? k_integrity<true> : k_integrity<false>;
    kern<<<blocks_for((long long)s->gcells, kThreads), kThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->gcells, s->n, s->off, s->cnt, s->f[F_GCELL].cur<uint32_t>(),
        s->f[F_GNDX].cur<uint32_t>(), bad_dev);
    FL_LAUNCH_CHECK("integrity");
    return FL_OK;
}
