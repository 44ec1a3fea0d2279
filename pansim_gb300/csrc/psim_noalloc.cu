// psim_csr_build_noalloc: the location CSR of a caller-owned device array of
// agent locations, built without allocating any device memory.
//
// Some callers of this library cannot call cudaMalloc: code whose device
// memory belongs to another allocator (a framework's caching allocator or a
// pool set up once at start), plug-ins that must not grow the device
// footprint behind their host's back, and latency-sensitive loops in which a
// cudaMalloc/cudaFree would synchronize the device.  For them this entry
// point keeps its scratch (the per-location histogram, the per-location
// cursors and the per-tile sums) in one file-scope __device__ array of fixed
// size that every GPU loading the library holds until the process exits.
//
// The caller passes the input (locations) and the outputs (offsets, agents).
// Every call shares the scratch array and leaves its contents behind: the
// histogram is cleared at the start of each call; calls that overlap on the
// GPU (for example on two streams of the same device) race on it.
//
// The array's device address is looked up once per CUDA context (keyed by
// the context's process-unique id, cuCtxGetId): a device reset or another
// context made current on the same device loads the module again, possibly
// at another address, and the next call looks the address up afresh.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/pansim_gb300.h"

namespace {

constexpr uint32_t NA_THREADS = 256;
constexpr uint32_t NA_ITEMS = 8;
constexpr uint32_t NA_TILE = NA_THREADS * NA_ITEMS;
constexpr uint32_t NA_MAX_TILES = (PSIM_NOALLOC_MAX_LOCATIONS + NA_TILE - 1) / NA_TILE;
// histogram [MAX] | cursor [MAX] | tile sums [MAX_TILES]
constexpr size_t NA_WORDS = 2ull * PSIM_NOALLOC_MAX_LOCATIONS + NA_MAX_TILES;

__device__ __align__(256) uint32_t g_noalloc_scratch[NA_WORDS];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_setup_mutex;
// per device: the id of the context whose module the address belongs to
uint32_t* g_scratch_ptr[NA_MAX_DEVICES] = {};
unsigned long long g_scratch_ctx[NA_MAX_DEVICES] = {};
thread_local std::string g_noalloc_error;

// driver entry points taken through the runtime (the library does not link
// libcuda itself)
typedef CUresult (*ctx_get_current_fn)(CUcontext*);
typedef CUresult (*ctx_get_id_fn)(CUcontext, unsigned long long*);
ctx_get_current_fn g_ctx_get_current = nullptr;
ctx_get_id_fn g_ctx_get_id = nullptr;

int na_fail(int code, const std::string& msg) {
    g_noalloc_error = msg;
    return code;
}

// grid-stride loops count in 64 bits: with 32-bit indices an n_agents near
// 2^32 would wrap the index past the end and visit agents twice
__global__ void na_zero(uint32_t* counts, uint32_t L) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < L; l += stride) counts[l] = 0u;
}

__global__ void na_count(const uint32_t* loc, uint32_t N, uint32_t L, uint32_t* counts) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
        const uint32_t l = loc[i];
        if (l < L) atomicAdd(&counts[l], 1u);
    }
}

__device__ __forceinline__ uint32_t na_block_sum(uint32_t v, uint32_t* s_red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    uint32_t tot = 0;
    for (int q = 0; q < (int)(NA_THREADS / 32); ++q) tot += s_red[q];
    __syncthreads();
    return tot;
}

__global__ void __launch_bounds__(NA_THREADS) na_tile_sums(const uint32_t* counts, uint32_t L, uint32_t* tile_sums) {
    __shared__ uint32_t s_red[NA_THREADS / 32];
    const uint32_t base = blockIdx.x * NA_TILE;
    uint32_t v = 0;
    for (uint32_t q = 0; q < NA_ITEMS; ++q) {
        const uint32_t l = base + q * NA_THREADS + threadIdx.x;
        v += l < L ? counts[l] : 0u;
    }
    v = na_block_sum(v, s_red);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = v;
}

// exclusive scan of the histogram: offsets (output) and cursors (scratch)
__global__ void __launch_bounds__(NA_THREADS) na_scan(const uint32_t* counts, uint32_t L, const uint32_t* tile_sums,
                                                      uint32_t* offsets, uint32_t* cursor) {
    __shared__ uint32_t s_red[NA_THREADS / 32];
    __shared__ uint32_t s_warp[NA_THREADS / 32];
    const uint32_t tile = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t wbase = tile * NA_TILE + (uint32_t)warp * (32 * NA_ITEMS);
    uint32_t c[NA_ITEMS], ex[NA_ITEMS];
    for (uint32_t q = 0; q < NA_ITEMS; ++q) {
        const uint32_t l = wbase + q * 32 + lane;
        c[q] = l < L ? counts[l] : 0u;
    }
    uint32_t pre = 0;
    for (uint32_t j = threadIdx.x; j < tile; j += NA_THREADS) pre += tile_sums[j];
    const uint32_t prefix = na_block_sum(pre, s_red);
    uint32_t carry = 0;
    for (uint32_t q = 0; q < NA_ITEMS; ++q) {
        uint32_t x = c[q];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        ex[q] = carry + x - c[q];
        carry += __shfl_sync(0xffffffffu, x, 31);
    }
    if (lane == 0) s_warp[warp] = carry;
    __syncthreads();
    uint32_t woff = 0;
    for (int q = 0; q < warp; ++q) woff += s_warp[q];
    const uint32_t base = prefix + woff;
    for (uint32_t q = 0; q < NA_ITEMS; ++q) {
        const uint32_t l = wbase + q * 32 + lane;
        if (l < L) {
            offsets[l] = base + ex[q];
            cursor[l] = base + ex[q];
        }
        if (l + 1 == L) offsets[L] = base + ex[q] + c[q];
    }
}

__global__ void na_scatter(const uint32_t* loc, uint32_t N, uint32_t L, uint32_t* cursor, uint32_t* agents) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
        const uint32_t l = loc[i];
        if (l < L) {
            const uint32_t p = atomicAdd(&cursor[l], 1u);
            if (p < N) agents[p] = (uint32_t)i;
        }
    }
}

// The id of the current thread's CUDA context (0 and no error when the
// thread has none yet).
int current_context_id(unsigned long long* id) {
    *id = 0;
    if (!g_ctx_get_current || !g_ctx_get_id) {
        cudaDriverEntryPointQueryResult q1, q2;
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
            q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return na_fail(PSIM_ERR_CUDA, "cudaGetDriverEntryPointByVersion: cuCtxGetCurrent/cuCtxGetId unavailable");
        g_ctx_get_current = (ctx_get_current_fn)f1;
        g_ctx_get_id = (ctx_get_id_fn)f2;
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return na_fail(PSIM_ERR_CUDA, "cuCtxGetCurrent failed");
    if (ctx && g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return na_fail(PSIM_ERR_CUDA, "cuCtxGetId failed");
    return 0;
}

// Set-up, once per device and context, with that device current: the device
// address of the scratch array (its host-side name is only a stand-in).
int scratch_for_current_device(uint32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(PSIM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= NA_MAX_DEVICES) return na_fail(PSIM_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    unsigned long long ctx_id = 0;
    int rc = current_context_id(&ctx_id);
    if (rc) return rc;
    if (!g_scratch_ptr[dev] || ctx_id == 0 || ctx_id != g_scratch_ctx[dev]) {
        void* p = nullptr;
        // makes the device's primary context current if the thread had none
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return na_fail(PSIM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        rc = current_context_id(&ctx_id);
        if (rc) return rc;
        g_scratch_ptr[dev] = (uint32_t*)p;
        g_scratch_ctx[dev] = ctx_id;
    }
    *out = g_scratch_ptr[dev];
    return 0;
}

unsigned grid(uint32_t n) {
    unsigned g = (n + 255) / 256;
    if (g > 1216) g = 1216;
    return g ? g : 1u;
}

}  // namespace

extern "C" int psim_csr_build_noalloc(const uint32_t* d_location, uint32_t n_agents, uint32_t n_locations,
                                      uint32_t* d_offsets, uint32_t* d_agents, void* stream) {
    g_noalloc_error.clear();
    if (n_locations == 0 || n_locations > PSIM_NOALLOC_MAX_LOCATIONS)
        return na_fail(PSIM_ERR_ARG, "psim_csr_build_noalloc: n_locations must be 1.." +
                                         std::to_string(PSIM_NOALLOC_MAX_LOCATIONS) + ", got " +
                                         std::to_string(n_locations));
    if (n_agents > PSIM_NOALLOC_MAX_AGENTS)
        return na_fail(PSIM_ERR_ARG, "psim_csr_build_noalloc: n_agents must be <= " +
                                         std::to_string(PSIM_NOALLOC_MAX_AGENTS) + ", got " + std::to_string(n_agents));
    if ((n_agents && (!d_location || !d_agents)) || !d_offsets)
        return na_fail(PSIM_ERR_ARG, "psim_csr_build_noalloc: null device pointer");
    uint32_t* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    uint32_t* counts = scratch;
    uint32_t* cursor = scratch + PSIM_NOALLOC_MAX_LOCATIONS;
    uint32_t* tile_sums = scratch + 2ull * PSIM_NOALLOC_MAX_LOCATIONS;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned tiles = (n_locations + NA_TILE - 1) / NA_TILE;
    na_zero<<<grid(n_locations), 256, 0, s>>>(counts, n_locations);
    if (n_agents) na_count<<<grid(n_agents), 256, 0, s>>>(d_location, n_agents, n_locations, counts);
    na_tile_sums<<<tiles, NA_THREADS, 0, s>>>(counts, n_locations, tile_sums);
    na_scan<<<tiles, NA_THREADS, 0, s>>>(counts, n_locations, tile_sums, d_offsets, cursor);
    if (n_agents) na_scatter<<<grid(n_agents), 256, 0, s>>>(d_location, n_agents, n_locations, cursor, d_agents);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail(PSIM_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return 0;
}

extern "C" const char* psim_noalloc_last_error(void) { return g_noalloc_error.c_str(); }
