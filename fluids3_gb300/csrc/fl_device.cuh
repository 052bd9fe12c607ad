// Device helpers shared by the forward kernels (fl_kernels.cu) and the
// adjoint kernels (fl_adjoint.cu): the grid cell of a position, band codes
// for search-block pruning, candidate enumeration over a search block, the
// pair-list layout. Included inside each file's anonymous namespace.
#pragma once

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

// ---------------------------------------------------------------------------
// Search-block pruning (gridSrch == 2). The search block of a point in cell
// c is the 2x2x2 cells c-1..c per axis (fluid_kernels.cu:120,129-131). Along
// an axis where the block takes the lower neighbour, a pair can only pass
// the 0 < d^2 < rd2 test if the point lies within h of its cell's lower
// face and the neighbour lies within h of that same face. Each sorted point
// carries a band code in pos.w:
//   bits 0-2  within `band` of its own cell's upper face (x, y, z)
//   bits 3-5  within `band` of its own cell's lower face (x, y, z)
// with band = h (1 + 1e-4) + 1e-3 * cell edge, far above the rounding of
// the cell computation. Skipping only pairs whose every FP32 distance is
// >= band > h leaves each sum's terms and order unchanged, so the pruned
// passes are bit-identical to the reference loop.
__device__ __forceinline__ uint32_t band_code(const DevParams &P, int c, float4 p) {
    if (c >= P.ncells) return 0u;
    const int cx = c % P.gridRes.x;
    const int t = c / P.gridRes.x;
    const int cz = t % P.gridRes.z;
    const int cy = t / P.gridRes.z;
    const float lx = P.gridMin.x + (float)cx * P.cellw.x;
    const float ly = P.gridMin.y + (float)cy * P.cellw.y;
    const float lz = P.gridMin.z + (float)cz * P.cellw.z;
    uint32_t code = 0;
    code |= ((lx + P.cellw.x) - p.x < P.band) ? 1u : 0u;
    code |= ((ly + P.cellw.y) - p.y < P.band) ? 2u : 0u;
    code |= ((lz + P.cellw.z) - p.z < P.band) ? 4u : 0u;
    code |= (p.x - lx < P.band) ? 8u : 0u;
    code |= (p.y - ly < P.band) ? 16u : 0u;
    code |= (p.z - lz < P.band) ? 32u : 0u;
    return code;
}

// Upper-band flags of the sorted slots, one bit per slot and axis:
// upbits[axis * upwords + (slot >> 5)] bit (slot & 31). Published by the
// 32 lanes of a warp for 32 consecutive slots base + lane (all lanes call).
// The adjoint's rebuilt steps also publish the lower-band flags (code bits
// 3-5) into rows 3-5 the same way (upbits + 3 * upwords, `code >> 3`).
__device__ __forceinline__ void publish_upbits(const DevParams &P, uint32_t *upbits, uint32_t base,
                                               uint32_t code, bool valid) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t w0 = base >> 5, sh = base & 31u;
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        const unsigned b = __ballot_sync(0xffffffffu, valid && ((code >> ax) & 1u));
        if (b) {
            uint32_t *row = upbits + (size_t)ax * P.upwords;
            if (lane == 0) atomicOr(&row[w0], b << sh);
            if (lane == 1 && sh) atomicOr(&row[w0 + 1], b >> (32u - sh));
        }
    }
}

// Axes (bit 0 x, 1 y, 2 z) along which adjacency entry k (y,z,x order,
// fluid_system.cpp:2266-2270) reaches into the lower neighbour cell.
__device__ __forceinline__ uint32_t lower_axes(int k) {
    return ((k & 1) ? 0u : 1u) | ((k & 4) ? 0u : 2u) | ((k & 2) ? 0u : 4u);
}


// ---------------------------------------------------------------------------
// Candidate enumeration for one adjacency entry of the search block.
//
// Unpruned: every member of the neighbour cell, in sorted order (the
// reference loop, fluid_kernels.cu:131-133). Pruned (gridSrch == 2 with
// valid band codes): the cell is skipped unless the point is within the band
// of its lower face on every axis where the entry reaches down, and only
// members within the band of their upper face on those axes are visited,
// read 32 slots at a time from the per-slot flag words. Visiting order is
// always ascending slot, so a point's sum sees the same terms in the same
// order as the reference loop.
struct CandIter {
    uint32_t w, w_last;   // current and last 32-slot word of the cell's range
    uint32_t lo, hi;      // slot range [lo, hi)
    uint32_t bits;        // candidates left in word w
    uint32_t U;           // axes whose upper-band flag a candidate must carry
};

template <bool PRUNE>
__device__ __forceinline__ uint32_t cand_word(const CandIter &it, const DevParams &P,
                                              const uint32_t *__restrict__ upbits, uint32_t w) {
    uint32_t v = 0xffffffffu;
    if (PRUNE) {
        if (it.U & 1u) v &= upbits[w];
        if (it.U & 2u) v &= upbits[(size_t)P.upwords + w];
        if (it.U & 4u) v &= upbits[2 * (size_t)P.upwords + w];
    }
    if (w == (it.lo >> 5)) v &= 0xffffffffu << (it.lo & 31u);
    if (w == it.w_last && (it.hi & 31u)) v &= 0xffffffffu >> (32u - (it.hi & 31u));
    return v;
}

template <bool PRUNE>
__device__ __forceinline__ void cand_begin(CandIter &it, const DevParams &P, int k, int cell,
                                           uint32_t my_code, bool active,
                                           const uint32_t *__restrict__ off,
                                           const uint32_t *__restrict__ cnt,
                                           const uint32_t *__restrict__ upbits) {
    it.bits = 0; it.w = 0; it.w_last = 0; it.lo = it.hi = 0; it.U = 0;
    if (!active) return;
    if (PRUNE) {
        it.U = lower_axes(k);
        if (((my_code >> 3) & it.U) != it.U) return;     // too far from those lower faces
    }
    const uint32_t m = cnt[cell];
    if (m == 0) return;
    it.lo = off[cell];
    it.hi = it.lo + m;
    it.w = it.lo >> 5;
    it.w_last = (it.hi - 1) >> 5;
    it.bits = cand_word<PRUNE>(it, P, upbits, it.w);
}

template <bool PRUNE>
__device__ __forceinline__ bool cand_next(CandIter &it, const DevParams &P,
                                          const uint32_t *__restrict__ upbits, uint32_t &j) {
    while (it.bits == 0) {
        if (it.w >= it.w_last) return false;
        it.w++;
        it.bits = cand_word<PRUNE>(it, P, upbits, it.w);
    }
    j = (it.w << 5) + (uint32_t)(__ffs(it.bits) - 1);
    it.bits &= it.bits - 1u;
    return true;
}

// ---------------------------------------------------------------------------
// Block-local thread orders. Each point's result is one thread's work in the
// reference's order, so which thread of a block takes which of the block's
// points changes no result; grouping points whose loops have the same shape
// into the same warps shortens the loops that run as long as their slowest
// lane. group_by_key() returns the slot this thread takes: the block's slots
// ordered by their threads' keys (< NKEYS), ascending slot within a key. All
// threads of the block call it; s_dyn holds grouping_smem(blockDim, NKEYS)
// bytes of scratch, which the caller may reuse once it has returned.
__host__ __device__ inline size_t grouping_smem(int threads, uint32_t nkeys) {
    return (size_t)nkeys * (threads / 32) * sizeof(uint32_t) + (size_t)threads * sizeof(uint16_t);
}

template <uint32_t NKEYS>
__device__ __forceinline__ int group_by_key(uint32_t key, uint32_t *s_dyn) {
    const unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t *s_cnt = s_dyn;                                               // (key, warp), key-major
    uint16_t *s_slot = reinterpret_cast<uint16_t *>(s_dyn + NKEYS * nw);
    const unsigned below = (1u << lane) - 1u;
    uint32_t rank = 0;
    __syncthreads();   // earlier users of the scratch are done
    if constexpr (NKEYS <= 16) {
#pragma unroll
        for (uint32_t k = 0; k < NKEYS; k++) {
            const unsigned b = __ballot_sync(0xffffffffu, key == k);
            if (lane == 0) s_cnt[k * nw + w] = __popc(b);
            if (key == k) rank = __popc(b & below);
        }
    } else {
        for (uint32_t e = threadIdx.x; e < NKEYS * nw; e += blockDim.x) s_cnt[e] = 0;
        __syncthreads();
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        rank = __popc(peers & below);
        if (rank == 0) s_cnt[key * nw + w] = __popc(peers);
    }
    __syncthreads();
    if (w == 0) {   // exclusive scan of the (key, warp) counts
        const uint32_t total = NKEYS * nw;
        uint32_t run = 0;
        for (uint32_t c0 = 0; c0 < total; c0 += 32) {
            const uint32_t e = c0 + lane;
            const uint32_t v = (e < total) ? s_cnt[e] : 0u;
            uint32_t x = v;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= (unsigned)d) x += y;
            }
            if (e < total) s_cnt[e] = run + x - v;
            run += __shfl_sync(0xffffffffu, x, 31);
        }
    }
    __syncthreads();
    s_slot[s_cnt[key * nw + w] + rank] = (uint16_t)threadIdx.x;
    __syncthreads();
    return (int)(blockIdx.x * blockDim.x) + s_slot[threadIdx.x];
}

// Points of one cell with the same band bits visit the same candidates of
// the pruned walks (lower-band bits, shift 3: the entries of the search
// block; upper-band bits, shift 0: the cells of the reverse block), so the
// walks group a block's points by those bits, then cells out of range, then
// slots past n. Needs grouping_smem(blockDim, kBandKeys) bytes of s_dyn.
constexpr uint32_t kBandKeys = 10;

__device__ __forceinline__ int band_grouped_slot(int n, const float4 *__restrict__ pos,
                                                 const uint32_t *__restrict__ gcell, int shift,
                                                 uint32_t *s_dyn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t key = kBandKeys - 1;
    if (i < n) key = (gcell[i] == kUndef) ? kBandKeys - 2 : ((__float_as_uint(pos[i].w) >> shift) & 7u);
    return group_by_key<kBandKeys>(key, s_dyn);
}

// Pair list written by the density pass: for point i (global thread i,
// warp w = i / 32, lane l = i % 32) entry t lives at
// ((w * hcap + t) * 32 + l), so a warp reading entry t of all its lanes
// touches one 128-byte line. Entries past hcap are not stored; the count
// still records every pair, and the force pass re-walks such warps.
__device__ __forceinline__ size_t list_at(const DevParams &P, int i, uint32_t t) {
    return ((size_t)(i >> 5) * (size_t)P.hcap + t) * 32u + (uint32_t)(i & 31);
}


__device__ __forceinline__ float3 xyz(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float4 f4(float3 v) { return make_float4(v.x, v.y, v.z, 0.0f); }

inline int blocks_for(long long n, int threads) { return (int)((n + threads - 1) / threads); }
