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
// its device address is looked up with cudaGetSymbolAddress, with the
// calling device current. The first call on a device does this set-up (it
// may load the module, so it should come before any stream capture); later
// calls look the address up again whenever their stream is not capturing,
// so a context torn down by cudaDeviceReset and rebuilt is picked up, and
// reuse the last address found while capturing.
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
// `spin_limit` bounds every look-back wait (kSpinLimit for callers) and
// `first_tile` offsets the ticket (0 for callers; the test hook withholds
// tile 0 with it).
__global__ void __launch_bounds__(kThreads)
k_scan_noalloc(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, int n, int ntiles,
               int inclusive, unsigned char *scratch, uint32_t *status_word, int spin_limit,
               uint32_t first_tile) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp[kThreads / 32];
    __shared__ uint32_t s_prefix;
    uint32_t *ticket = reinterpret_cast<uint32_t *>(scratch);
    uint64_t *status = reinterpret_cast<uint64_t *>(scratch + 256);
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;

    if (threadIdx.x == 0) s_tile = first_tile + atomicAdd(ticket, 1u);
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
                // bounded wait: after spin_limit polls stop waiting and
                // report through the caller's status word
                while (((d = ld_acquire(&status[j])) >> 62) == 0) {
                    if (++spins > spin_limit) {
                        atomicOr(status_word, FL_DEV_SPIN_TIMEOUT);
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

// Device address of the scratch array on the current device: looked up
// again unless `stream` is capturing (the lookup may load the module, which
// a capture forbids); while capturing, the address of the last lookup on
// this device.
int scratch_address(cudaStream_t stream, void **out) {
    int dev = -1;
    FL_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return fl_fail(FL_ERR_ARG, "fl_prefix_sum_noalloc: device %d beyond the %d supported", dev, kMaxDevices);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    FL_CUDA_TRY(cudaStreamIsCapturing(stream, &cap));
    std::lock_guard<std::mutex> lock(g_mutex);
    if (cap == cudaStreamCaptureStatusNone || !g_scratch_addr[dev]) {
        if (cap != cudaStreamCaptureStatusNone)
            return fl_fail(FL_ERR_STATE, "fl_prefix_sum_noalloc: the first call on a device must come before "
                                         "stream capture");
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

// Arguments shared by the entry point and its test hook.
int check_args(const char *who, const uint32_t *d_counts, const uint32_t *d_offsets, int n,
               const uint32_t *d_status) {
    if (n < 0) return fl_fail(FL_ERR_ARG, "%s: n < 0", who);
    if (n > FL_NOALLOC_MAX_COUNTS)
        return fl_fail(FL_ERR_ARG,
                       "%s: %d counts exceed the fixed scratch limit of %d "
                       "(use fl_prefix_sum_cells on a system for larger grids)", who, n, FL_NOALLOC_MAX_COUNTS);
    if (n == 0) return FL_OK;
    if (!d_counts || !d_offsets) return fl_fail(FL_ERR_ARG, "%s: null buffer", who);
    if (!d_status)
        return fl_fail(FL_ERR_ARG, "%s: d_status is required (the only report of a look-back wait that gave up)",
                       who);
    const uintptr_t c0 = (uintptr_t)d_counts, o0 = (uintptr_t)d_offsets, len = (uintptr_t)n * sizeof(uint32_t);
    if (c0 < o0 + len && o0 < c0 + len)
        return fl_fail(FL_ERR_ARG, "%s: d_counts and d_offsets overlap (the scan is not in place)", who);
    return FL_OK;
}

int launch(const uint32_t *d_counts, uint32_t *d_offsets, int n, int zero_offsets, uint32_t *d_status,
           cudaStream_t st, int spin_limit, uint32_t first_tile) {
    void *scratch = nullptr;
    FL_TRY(scratch_address(st, &scratch));
    const int ntiles = (n + kTile - 1) / kTile;
    // the ticket must start at 0 and no descriptor may look published
    FL_CUDA_TRY(cudaMemsetAsync(scratch, 0, 256 + sizeof(uint64_t) * (size_t)ntiles, st));
    k_scan_noalloc<<<ntiles - (int)first_tile, kThreads, 0, st>>>(d_counts, d_offsets, n, ntiles,
                                                                  zero_offsets ? 0 : 1, (unsigned char *)scratch,
                                                                  d_status, spin_limit, first_tile);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return fl_fail(FL_ERR_CUDA, "fl_prefix_sum_noalloc launch: %s", cudaGetErrorString(e));
    return FL_OK;
}

}  // namespace

extern "C" int fl_prefix_sum_noalloc(const uint32_t *d_counts, uint32_t *d_offsets, int n,
                                     int zero_offsets, uint32_t *d_status, void *stream) {
    FL_TRY(check_args("fl_prefix_sum_noalloc", d_counts, d_offsets, n, d_status));
    if (n == 0) return FL_OK;
    return launch(d_counts, d_offsets, n, zero_offsets, d_status, (cudaStream_t)stream, kSpinLimit, 0u);
}

// Test hook: the same scan with tile 0 withheld (one CTA fewer, the ticket
// starting at tile 1, so every index stays in bounds) and a short spin
// limit: tile 1's wait for tile 0 runs out and FL_DEV_SPIN_TIMEOUT lands in
// d_status. The offsets written are not a scan.
extern "C" int fl_test_scan_noalloc_timeout(const uint32_t *d_counts, uint32_t *d_offsets, int n,
                                            uint32_t *d_status, int spin_limit, void *stream) {
    FL_TRY(check_args("fl_test_scan_noalloc_timeout", d_counts, d_offsets, n, d_status));
    if (n <= kTile) return fl_fail(FL_ERR_ARG, "fl_test_scan_noalloc_timeout: needs at least two tiles");
    if (spin_limit < 1 || spin_limit > kSpinLimit)
        return fl_fail(FL_ERR_ARG, "fl_test_scan_noalloc_timeout: spin limit %d outside [1, %d]", spin_limit,
                       kSpinLimit);
    return launch(d_counts, d_offsets, n, 0, d_status, (cudaStream_t)stream, spin_limit, 1u);
}

static_assert(FL_NOALLOC_MAX_COUNTS == kTile * kMaxTiles, "header limit must match the scratch size");
