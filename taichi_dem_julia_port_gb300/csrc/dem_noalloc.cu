// dem_noalloc.cu — the broad-phase bucket sort for callers that cannot
// allocate device memory.
//
// Some embedders cannot call cudaMalloc: a host that pre-allocates every
// device buffer once and forbids allocation afterwards (a real-time or
// certified control loop), a process whose allocator is owned by another
// framework, or a step that runs while allocation is blocked.  They pass their
// own input and output buffers, and the temporary memory the sort needs lives
// in one file-scope device array below, reserved on every GPU that loads this
// library until the process exits.
//
// Limits: n <= 1,048,576 particles and hash_table_size <= 1,048,576 buckets;
// the array is 12.6 MB (counts, starts, tile sums, unsorted order).
#include <mutex>

#include "dem_device.cuh"
#include "dem_gb300.h"

namespace {

constexpr long long kMaxN = 1 << 20;
constexpr long long kMaxH = 1 << 20;
constexpr int kTile = 2048;
constexpr int kBlock = 256;
constexpr int kMaxTiles = (int)((kMaxH + kTile - 1) / kTile);
constexpr size_t kCountsOff = 0;
constexpr size_t kStartsOff = kCountsOff + kMaxH;
constexpr size_t kTilesOff = kStartsOff + kMaxH + 64;
constexpr size_t kUnsortedOff = kTilesOff + kMaxTiles;
constexpr size_t kWords = kUnsortedOff + kMaxN;
constexpr int kMaxDevices = 64;

// The scratch: bucket counts (zero at the start of every call), bucket starts,
// per-tile sums of the counts, and the bucket-grouped order before the
// within-bucket ordering.  Host code must not take this name as a device
// address; it uses the address from cudaGetSymbolAddress (see scratch_on()).
static __device__ __align__(256) uint32_t g_scratch[kWords];

struct Geometry {
    double dmin[3];
    double cell;
    uint32_t H;
    uint32_t mask;
};

__device__ __forceinline__ uint32_t na_bucket(int x, int y, int z, const Geometry& g) {
    const uint32_t m = dem::morton1(x, y, z);
    return g.mask ? (m & g.mask) : (m % g.H);
}

// cell + hashcode (src/utils.jl:1-2) and count_particles! (src/kernels.jl:7-13)
__global__ void k_na_hash(const double* __restrict__ px, const double* __restrict__ py,
                          const double* __restrict__ pz, int n, Geometry g, uint32_t* bucket_out,
                          uint32_t* counts) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double pos[3] = {px[i], py[i], pz[i]};
    int ijk[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
        ijk[c] = dem::ceil_i32(__ddiv_rn(__dsub_rn(pos[c], g.dmin[c]), g.cell));
    const uint32_t b = na_bucket(ijk[0], ijk[1], ijk[2], g);
    bucket_out[i] = b + 1u;  // the reference's 1-based hashcode
    atomicAdd(&counts[b], 1u);
}

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[kBlock / 32];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (unsigned)o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kBlock / 32 ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (unsigned)o) w += y;
        }
        if (lane < kBlock / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    *total = warp_sums[kBlock / 32 - 1];
    const uint32_t r = (warp ? warp_sums[warp - 1] : 0u) + x - v;
    __syncthreads();
    return r;
}

// accumulate! of the counts (src/executor.jl:50) in three passes without
// any inter-block waiting: tile sums, one-block scan of the sums, apply.
__global__ void k_na_tile_sums(const uint32_t* counts, long long H, uint32_t* tiles) {
    const long long base = (long long)blockIdx.x * kTile + threadIdx.x * (kTile / kBlock);
    uint32_t s = 0;
    for (int k = 0; k < kTile / kBlock; ++k)
        if (base + k < H) s += counts[base + k];
    uint32_t total;
    block_excl_scan(s, &total);
    if (threadIdx.x == 0) tiles[blockIdx.x] = total;
}

__global__ void k_na_scan_tiles(uint32_t* tiles, int ntiles) {
    uint32_t carry = 0;
    for (int base = 0; base < ntiles; base += kBlock) {
        const int t = base + threadIdx.x;
        const uint32_t v = t < ntiles ? tiles[t] : 0u;
        uint32_t total;
        const uint32_t e = block_excl_scan(v, &total);
        if (t < ntiles) tiles[t] = carry + e;
        carry += total;
    }
}

__global__ void k_na_apply(const uint32_t* counts, long long H, const uint32_t* tiles,
                           uint32_t* starts) {
    const long long base = (long long)blockIdx.x * kTile + threadIdx.x * (kTile / kBlock);
    uint32_t v[kTile / kBlock];
    uint32_t s = 0;
    for (int k = 0; k < kTile / kBlock; ++k) {
        v[k] = base + k < H ? counts[base + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = tiles[blockIdx.x] + block_excl_scan(s, &total);
    for (int k = 0; k < kTile / kBlock; ++k) {
        if (base + k < H) starts[base + k] = run;
        if (base + k == H - 1) starts[H] = run + v[k];
        run += v[k];
    }
}

// get_particle_id! (src/kernels.jl:15-22); the decrements return every count
// to zero.
__global__ void k_na_scatter(const uint32_t* bucket, int n, uint32_t* counts,
                             const uint32_t* starts, uint32_t* unsorted) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t b = bucket[i] - 1u;
    const uint32_t slot = atomicSub(&counts[b], 1u) - 1u;
    unsorted[starts[b] + slot] = (uint32_t)i;
}

// ascending particle index inside each bucket
__global__ void k_na_order(const uint32_t* bucket, const uint32_t* unsorted,
                           const uint32_t* starts, int n, uint32_t* sorted) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t i = unsorted[k];
    const uint32_t b = bucket[i] - 1u;
    const uint32_t s = starts[b], e = starts[b + 1];
    uint32_t rank = 0;
    for (uint32_t t = s; t < e; ++t) rank += unsorted[t] < i ? 1u : 0u;
    sorted[s + rank] = i;
}

std::mutex g_setup_mutex;
uint32_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_scratch on the current device, looked up once per
// device (the first call on each device does this, so that call should come
// before any stream capture on that device).
int scratch_on(int device, uint32_t** out) {
    if (device < 0 || device >= kMaxDevices) return DEM_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return DEM_ERR_CUDA;
        g_scratch_ptr[device] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch_ptr[device];
    return DEM_OK;
}

}  // namespace

extern "C" int dem_bucket_sort_noalloc(const double* px, const double* py, const double* pz,
                                       int64_t n, const double* domain_min, double cell_size,
                                       int64_t hash_table_size, uint32_t* bucket,
                                       uint32_t* sorted, void* stream) {
    if (n < 0 || !domain_min || !(cell_size > 0) || hash_table_size < 1) return DEM_ERR_INVALID;
    if (n > kMaxN || hash_table_size > kMaxH) return DEM_ERR_CAPACITY;
    if (n > 0 && (!px || !py || !pz || !bucket || !sorted)) return DEM_ERR_INVALID;
    if (n == 0) return DEM_OK;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return DEM_ERR_NO_DEVICE;
    uint32_t* scratch = nullptr;
    const int rc = scratch_on(device, &scratch);
    if (rc != DEM_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t* counts = scratch + kCountsOff;
    uint32_t* starts = scratch + kStartsOff;
    uint32_t* tiles = scratch + kTilesOff;
    uint32_t* unsorted = scratch + kUnsortedOff;
    Geometry g;
    for (int c = 0; c < 3; ++c) g.dmin[c] = domain_min[c];
    g.cell = cell_size;
    g.H = (uint32_t)hash_table_size;
    g.mask = (g.H & (g.H - 1)) == 0 ? g.H - 1 : 0u;
    const int nn = (int)n;
    const int nb = (nn + kBlock - 1) / kBlock;
    const int ntiles = (int)((hash_table_size + kTile - 1) / kTile);
    if (cudaMemsetAsync(counts, 0, sizeof(uint32_t) * (size_t)hash_table_size, s) != cudaSuccess)
        return DEM_ERR_CUDA;
    k_na_hash<<<nb, kBlock, 0, s>>>(px, py, pz, nn, g, bucket, counts);
    k_na_tile_sums<<<ntiles, kBlock, 0, s>>>(counts, hash_table_size, tiles);
    k_na_scan_tiles<<<1, kBlock, 0, s>>>(tiles, ntiles);
    k_na_apply<<<ntiles, kBlock, 0, s>>>(counts, hash_table_size, tiles, starts);
    k_na_scatter<<<nb, kBlock, 0, s>>>(bucket, nn, counts, starts, unsorted);
    k_na_order<<<nb, kBlock, 0, s>>>(bucket, unsorted, starts, nn, sorted);
    return cudaGetLastError() == cudaSuccess ? DEM_OK : DEM_ERR_CUDA;
}
