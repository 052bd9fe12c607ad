// Single-pass exclusive (or inclusive) scan of the cell counts with
// decoupled look-back; replaces the reference's 3-level prefixSum /
// prefixFixup launches (fluids4.0/fluid_kernels.cu:423-467, host driver
// fluids4.0/fluid_system.cpp:2354-2424) with one launch.
//
// Each CTA takes a tile of kTile counts (dynamic tile id from a ticket, so a
// tile's predecessors were all scheduled before it), scans it, publishes
// its aggregate, then walks back over predecessor descriptors until it
// meets an inclusive prefix. A descriptor is 64 bits:
//   [63:62] flag (1 = aggregate, 2 = inclusive prefix), [61:32] launch
//   epoch, [31:0] value.
// The host zeroes the descriptors and the ticket before every launch (one
// memset that also clears the counts in the fused step); the epoch field
// is a second guard against reading a descriptor left by another launch.
// Every wait is bounded: after `spin_limit` polls (kSpinLimit in the step)
// the CTA records FL_DEV_SPIN_TIMEOUT in the device error word and stops
// waiting. `first_tile` offsets the ticket (0 in the step); the test hook
// below uses it to withhold tile 0 so that the wait runs out.
#include "fl_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;   // 4096 counts per tile
constexpr uint64_t kFlagAgg = 1ull, kFlagPrefix = 2ull;
constexpr int kSpinLimit = 1 << 20;

__device__ __forceinline__ uint64_t ld_acquire(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint64_t *p, uint64_t v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t pack(uint64_t flag, uint32_t epoch, uint32_t value) {
    return (flag << 62) | ((uint64_t)(epoch & 0x3fffffffu) << 32) | value;
}

__global__ void __launch_bounds__(kThreads)
k_scan(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, uint64_t *status,
       uint32_t *ticket, int ntiles, uint32_t epoch, int inclusive, uint32_t *err, int spin_limit,
       uint32_t first_tile) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp[kThreads / 32];
    __shared__ uint32_t s_prefix;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;

    if (threadIdx.x == 0) {
        s_tile = first_tile + atomicAdd(ticket, 1u);
    }
    __syncthreads();
    const uint32_t tile = s_tile;

    // 16 consecutive counts per thread; buffers are padded to whole tiles.
    const size_t base = (size_t)tile * kTile + (size_t)threadIdx.x * kItems;
    uint32_t item[kItems], v[kItems];
    const uint4 *in4 = reinterpret_cast<const uint4 *>(in + base);
#pragma unroll
    for (int q = 0; q < kItems / 4; q++) {
        const uint4 w = in4[q];
        item[4 * q + 0] = w.x; item[4 * q + 1] = w.y; item[4 * q + 2] = w.z; item[4 * q + 3] = w.w;
    }
    uint32_t run = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) { run += item[k]; v[k] = run; }   // inclusive within thread
    const uint32_t thread_total = run;

    uint32_t x = thread_total;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (unsigned)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kThreads / 32 ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < kThreads / 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (unsigned)o) w += y;
        }
        if (lane < kThreads / 32) s_warp[lane] = w;
    }
    __syncthreads();
    const uint32_t tile_total = s_warp[kThreads / 32 - 1];
    const uint32_t thread_excl = (warp ? s_warp[warp - 1] : 0u) + x - thread_total;

    if (threadIdx.x == 0) {
        uint32_t prefix = 0;
        if (tile == 0) {
            st_release(&status[0], pack(kFlagPrefix, epoch, tile_total));
        } else {
            st_release(&status[tile], pack(kFlagAgg, epoch, tile_total));
            int j = (int)tile - 1;
            while (j >= 0) {
                uint64_t d;
                int spins = 0;
                for (;;) {
                    d = ld_acquire(&status[j]);
                    if ((d >> 62) != 0 && (uint32_t)((d >> 32) & 0x3fffffffu) == (epoch & 0x3fffffffu))
                        break;
                    if (++spins > spin_limit) {
                        atomicOr(err, FL_DEV_SPIN_TIMEOUT);
                        d = pack(kFlagPrefix, epoch, 0);
                        break;
                    }
                    __nanosleep(32);
                }
                prefix += (uint32_t)d;
                if ((d >> 62) == kFlagPrefix) break;
                j--;
            }
            st_release(&status[tile], pack(kFlagPrefix, epoch, prefix + tile_total));
        }
        s_prefix = prefix;
    }
    __syncthreads();
    const uint32_t start = s_prefix + thread_excl;
    uint4 *out4 = reinterpret_cast<uint4 *>(out + base);
#pragma unroll
    for (int q = 0; q < kItems / 4; q++) {
        const uint32_t k0 = inclusive ? 0u : 1u;   // exclusive drops the element itself
        uint4 w;
        w.x = start + v[4 * q + 0] - k0 * item[4 * q + 0];
        w.y = start + v[4 * q + 1] - k0 * item[4 * q + 1];
        w.z = start + v[4 * q + 2] - k0 * item[4 * q + 2];
        w.w = start + v[4 * q + 3] - k0 * item[4 * q + 3];
        out4[q] = w;
    }
}

}  // namespace

size_t fl_scan_tile() { return kTile; }

// Ticket (padded to 256 B) followed by one descriptor per tile.
size_t fl_scan_scratch_bytes(int ntiles) { return 256 + sizeof(uint64_t) * (size_t)ntiles; }

// Exclusive scan of s->cnt[0 .. count) into s->off. With clear_status the
// ticket and descriptors are zeroed first; otherwise the caller has
// already cleared them (together with the counts).
int fl_launch_scan(fl_system *s, int count, int clear_status) {
    const int ntiles = (int)((count + kTile - 1) / kTile);
    if (ntiles > s->scan_tiles)
        return fl_fail(FL_ERR_ARG, "scan: %d tiles exceed the %d allocated", ntiles, s->scan_tiles);
    if (clear_status)
        FL_CUDA_TRY(cudaMemsetAsync(s->scan_ticket, 0, fl_scan_scratch_bytes(s->scan_tiles), s->stream));
    k_scan<<<ntiles, kThreads, 0, s->stream>>>(s->cnt, s->off, s->scan_status, s->scan_ticket,
                                               ntiles, s->scan_epoch, /*inclusive=*/0,
                                               s->dev_err, kSpinLimit, 0u);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fl_fail(FL_ERR_CUDA, "scan launch: %s", cudaGetErrorString(e));
    return FL_OK;
}

// Test hook: the system scan with tile 0 withheld (ntiles - 1 CTAs take
// tiles 1 .. ntiles - 1, so every index stays in bounds) and a short spin
// limit, so tile 1's wait for tile 0's descriptor runs out: the kernel
// records FL_DEV_SPIN_TIMEOUT and returns, and fl_sync reports it.
extern "C" int fl_test_scan_timeout(fl_system *s, int spin_limit) {
    if (!s) return fl_fail(FL_ERR_ARG, "fl_test_scan_timeout: null system");
    if (spin_limit < 1 || spin_limit > kSpinLimit)
        return fl_fail(FL_ERR_ARG, "fl_test_scan_timeout: spin limit %d outside [1, %d]", spin_limit, kSpinLimit);
    const int ntiles = (int)((s->gcells + kTile - 1) / kTile);
    if (ntiles < 2) return fl_fail(FL_ERR_ARG, "fl_test_scan_timeout: needs at least two scan tiles");
    FL_CUDA_TRY(cudaMemsetAsync(s->scan_ticket, 0, fl_scan_scratch_bytes(s->scan_tiles), s->stream));
    k_scan<<<ntiles - 1, kThreads, 0, s->stream>>>(s->cnt, s->off, s->scan_status, s->scan_ticket, ntiles,
                                                   s->scan_epoch, 0, s->dev_err, spin_limit, 1u);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fl_fail(FL_ERR_CUDA, "scan launch: %s", cudaGetErrorString(e));
    fl_reset_progress(s);
    return FL_OK;
}
