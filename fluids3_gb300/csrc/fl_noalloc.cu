// Cell-count prefix sum that allocates nothing.
//
// Some host applications cannot let a library allocate device memory: a
// render engine or plugin host that owns the whole device budget and hands
// out every buffer itself, or a real-time loop where cudaMalloc/cudaFree
// would synchronise the device and stall the application's other streams.
// fl_prefix_sum_noalloc gives them the single-pass decoupled-look-back scan
// over buffers they own. The scan's own scratch -- a tile ticket and one
// look-back descriptor per 4096-element tile -- lives in the file-scope
// device array g_noalloc_scratch below, which every GPU that loads this
// library holds (about 8.5 KB) until the process exits.
//
// The array's host-side name is only a stand-in for the device symbol, so
// its device address is fetched once per device with cudaGetSymbolAddress
// (on that device's first call, with that device current) and cached.
// Every call shares the one array and it keeps the last call's contents:
// the ticket and descriptors are cleared at the start of each call, and two
// calls whose work overlaps on the same GPU race on them.
#include <mutex>

#include "fl_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;          // 4096 counts per tile
constexpr int kMaxTiles = 1024;                   // up to 4,194,304 counts per call
constexpr int kMaxDevices = 64;
constexpr int kSpinLimit = 1 << 20;
constexpr uint64_t kFlagAgg = 1ull, kFlagPrefix = 2ull;

// [0, 256): tile ticket; [256, 256 + 8 * kMaxTiles): look-back descriptors.
constexpr size_t kScratchBytes = 256 + sizeof(uint64_t) * kMaxTiles;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mutex;
void *g_scratch_addr[kMaxDevices] = {};

__device__ __forceinline__ uint64_t ld_acquire(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint64_t *p, uint64_t v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t desc(uint64_t flag, uint32_t value) {
    return (flag << 62) | value;
}

// Same algorithm as the system scan (fl_scan.cu), with bounds-checked scalar
// loads and stores so the caller's buffers need neither padding nor 16-byte
// alignment.
__global__ void __launch_bounds__(kThreads)
k_scan_noalloc(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, int n, int ntiles,
               int inclusive, unsigned char *scratch, uint32_t *status_word) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp[kThreads / 32];
    __shared__ uint32_t s_prefix;
    uint32_t *ticket = reinterpret_cast<uint32_t *>(scratch);
    uint64_t *status = reinterpret_cast<uint64_t *>(scratch + 256);
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;

    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const long long base = (long long)tile * kTile + (long long)threadIdx.x * kItems;

    uint32_t item[kItems], v[kItems];
    uint32_t run = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        item[k] = (base + k < n) ? in[base + k] : 0u;
        run += item[k];
        v[k] = run;
    }
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
            st_release(&status[0], desc(kFlagPrefix, tile_total));
        } else {
            st_release(&status[tile], desc(kFlagAgg, tile_total));
            for (int j = (int)tile - 1; j >= 0; j--) {
                uint64_t d;
                int spins = 0;
                // bounded wait: after kSpinLimit polls stop waiting and
                // report through the caller's status word
                while (((d = ld_acquire(&status[j])) >> 62) == 0) {
                    if (++spins > kSpinLimit) {
                        if (status_word) atomicOr(status_word, FL_DEV_SPIN_TIMEOUT);
                        d = desc(kFlagPrefix, 0);
                        break;
                    }
                    __nanosleep(32);
                }
                prefix += (uint32_t)d;
                if ((d >> 62) == kFlagPrefix) break;
            }
            st_release(&status[tile], desc(kFlagPrefix, prefix + tile_total));
        }
        s_prefix = prefix;
    }
    __syncthreads();
    const uint32_t start = s_prefix + thread_excl;
#pragma unroll
    for (int k = 0; k < kItems; k++)
        if (base + k < n) out[base + k] = start + (inclusive ? v[k] : v[k] - item[k]);
}

// Device address of the scratch array on the current device (fetched once).
int scratch_address(void **out) {
    int dev = -1;
    FL_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return fl_fail(FL_ERR_ARG, "fl_prefix_sum_noalloc: device %d beyond the %d supported", dev, kMaxDevices);
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fl_fail(FL_ERR_CUDA, "fl_prefix_sum_noalloc: cudaGetSymbolAddress: %s",
                           cudaGetErrorString(e));
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return FL_OK;
}

}  // namespace

extern "C" int fl_prefix_sum_noalloc(const uint32_t *d_counts, uint32_t *d_offsets, int n,
                                     int zero_offsets, uint32_t *d_status, void *stream) {
    if (n < 0) return fl_fail(FL_ERR_ARG, "fl_prefix_sum_noalloc: n < 0");
    if (n > FL_NOALLOC_MAX_COUNTS)
        return fl_fail(FL_ERR_ARG,
                       "fl_prefix_sum_noalloc: %d counts exceed the fixed scratch limit of %d "
                       "(use fl_prefix_sum_cells on a system for larger grids)", n, FL_NOALLOC_MAX_COUNTS);
    if (n == 0) return FL_OK;
    if (!d_counts || !d_offsets) return fl_fail(FL_ERR_ARG, "fl_prefix_sum_noalloc: null buffer");
    void *scratch = nullptr;
    FL_TRY(scratch_address(&scratch));
    cudaStream_t st = (cudaStream_t)stream;
    const int ntiles = (n + kTile - 1) / kTile;
    // the ticket must start at 0 and no descriptor may look published
    FL_CUDA_TRY(cudaMemsetAsync(scratch, 0, 256 + sizeof(uint64_t) * (size_t)ntiles, st));
    k_scan_noalloc<<<ntiles, kThreads, 0, st>>>(d_counts, d_offsets, n, ntiles, zero_offsets ? 0 : 1,
                                                (unsigned char *)scratch, d_status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return fl_fail(FL_ERR_CUDA, "fl_prefix_sum_noalloc launch: %s", cudaGetErrorString(e));
    return FL_OK;
}

static_assert(FL_NOALLOC_MAX_COUNTS == kTile * kMaxTiles, "header limit must match the scratch size");
