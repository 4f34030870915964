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
// The sort: cell + hashcode per particle (src/utils.jl:1-2), then a stable
// least-significant-digit radix sort of the particle indices by bucket, 10
// bits per pass (one pass for tables of up to 1,024 buckets, two above).
// Stability keeps ascending index inside each bucket, which is the order the
// library's regular broad phase gives (the reference leaves it free,
// src/kernels.jl:15-22).  The work is O(n + H) whatever the bucket
// occupancy: one bucket holding every particle costs the same as many small
// ones.
//
// Limits: n <= 1,048,576 particles and hash_table_size <= 1,048,576 buckets;
// the array is 12.6 MB (the first pass's keys and indices, the per-block
// digit counts, and the tile sums of their scan).
#include <mutex>

#include "dem_device.cuh"
#include "dem_gb300.h"

namespace {

constexpr long long kMaxN = 1 << 20;
constexpr long long kMaxH = 1 << 20;
constexpr int kBlock = 256;
constexpr int kItems = 4;
constexpr int kChunk = kBlock * kItems;  // particles per block of a radix pass
constexpr int kDigitBits = 10;
constexpr int kBins = 1 << kDigitBits;
constexpr long long kMaxBlocks = kMaxN / kChunk;
constexpr long long kHistWords = kBins * kMaxBlocks;
constexpr int kTile = 2048;  // counts per tile of the digit-count scan
constexpr int kMaxTiles = (int)((kHistWords + kTile - 1) / kTile);
constexpr size_t kKeysOff = 0;
constexpr size_t kValsOff = kKeysOff + kMaxN;
constexpr size_t kHistOff = kValsOff + kMaxN;
constexpr size_t kTilesOff = kHistOff + kHistWords;
constexpr size_t kWords = kTilesOff + kMaxTiles;
constexpr int kMaxDevices = 64;

// The scratch: the first pass's output keys (0-based buckets) and particle
// indices, the digit counts of every block (digit-major, scanned in place
// into each block's first slot per digit) and the per-tile sums of that scan.
// Every word a call reads is written earlier in the same call, so nothing
// needs clearing between calls.  Host code must not take this name as a
// device address; it uses the address from cudaGetSymbolAddress (see
// scratch_on()).
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

// cell + hashcode (src/utils.jl:1-2): the reference's 1-based bucket
__global__ void k_na_hash(const double* __restrict__ px, const double* __restrict__ py,
                          const double* __restrict__ pz, int n, Geometry g, uint32_t* bucket_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double pos[3] = {px[i], py[i], pz[i]};
    int ijk[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
        ijk[c] = dem::ceil_i32(__ddiv_rn(__dsub_rn(pos[c], g.dmin[c]), g.cell));
    bucket_out[i] = na_bucket(ijk[0], ijk[1], ijk[2], g) + 1u;
}

// Digit counts of one block's kChunk keys (key = in[k] - bias), written
// digit-major: hist[digit * nblk + block].
__global__ void k_na_digit_count(const uint32_t* __restrict__ keys, uint32_t bias, int n,
                                 int shift, int nblk, uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[kBins];
    for (int b = threadIdx.x; b < kBins; b += kBlock) h[b] = 0u;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kChunk;
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
        const long long k = base + q * kBlock + threadIdx.x;
        if (k < n) atomicAdd(&h[((keys[k] - bias) >> shift) & (kBins - 1)], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kBins; b += kBlock) hist[(size_t)b * nblk + blockIdx.x] = h[b];
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

// Exclusive scan of the digit counts, in place, in three passes without any
// inter-block waiting: tile sums, one-block scan of the sums, apply.
__global__ void k_na_tile_sums(const uint32_t* v, long long m, uint32_t* tiles) {
    const long long base = (long long)blockIdx.x * kTile + threadIdx.x * (kTile / kBlock);
    uint32_t s = 0;
    for (int k = 0; k < kTile / kBlock; ++k)
        if (base + k < m) s += v[base + k];
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

__global__ void k_na_apply(uint32_t* v, long long m, const uint32_t* tiles) {
    const long long base = (long long)blockIdx.x * kTile + threadIdx.x * (kTile / kBlock);
    uint32_t x[kTile / kBlock];
    uint32_t s = 0;
    for (int k = 0; k < kTile / kBlock; ++k) {
        x[k] = base + k < m ? v[base + k] : 0u;
        s += x[k];
    }
    uint32_t total;
    uint32_t run = tiles[blockIdx.x] + block_excl_scan(s, &total);
    for (int k = 0; k < kTile / kBlock; ++k) {
        if (base + k < m) v[base + k] = run;
        run += x[k];
    }
}

// Stable scatter of one block's kChunk (key, index) pairs by the digit at
// `shift`: an element's place is its block's first slot for that digit plus
// the number of elements of the block before it with the same digit.  The
// ranks are counted in element order by one warp, 32 elements per round
// (__match_any_sync groups equal digits), so the order inside a digit is
// the input order.  idx_in == nullptr: the indices are the positions.
__global__ void k_na_digit_scatter(const uint32_t* __restrict__ keys, uint32_t bias,
                                   const uint32_t* __restrict__ idx_in, int n, int shift, int nblk,
                                   const uint32_t* __restrict__ first,
                                   uint32_t* __restrict__ keys_out, uint32_t* __restrict__ idx_out) {
    __shared__ uint32_t s_key[kChunk], s_idx[kChunk], s_rank[kChunk], s_cnt[kBins];
    const long long base = (long long)blockIdx.x * kChunk;
    const int m = (int)min((long long)kChunk, (long long)n - base);
    for (int b = threadIdx.x; b < kBins; b += kBlock) s_cnt[b] = 0u;
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
        const int e = q * kBlock + threadIdx.x;
        if (e < m) {
            s_key[e] = keys[base + e] - bias;
            s_idx[e] = idx_in ? idx_in[base + e] : (uint32_t)(base + e);
        }
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const unsigned lane = threadIdx.x;
        for (int r = 0; r < kChunk / 32; ++r) {
            const int e = r * 32 + (int)lane;
            const bool valid = e < m;
            const uint32_t d = valid ? (s_key[e] >> shift) & (kBins - 1) : (uint32_t)kBins;
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            uint32_t before = 0;
            if (valid) before = s_cnt[d];
            __syncwarp();
            if (valid) {
                s_rank[e] = before + (uint32_t)__popc(peers & ((1u << lane) - 1u));
                if ((unsigned)(__ffs(peers) - 1) == lane) s_cnt[d] = before + (uint32_t)__popc(peers);
            }
            __syncwarp();
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
        const int e = q * kBlock + threadIdx.x;
        if (e < m) {
            const uint32_t d = (s_key[e] >> shift) & (kBins - 1);
            const uint32_t dst = first[(size_t)d * nblk + blockIdx.x] + s_rank[e];
            idx_out[dst] = s_idx[e];
            if (keys_out) keys_out[dst] = s_key[e];
        }
    }
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
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) {
            cudaGetLastError();  // this call's own failure
            return DEM_ERR_CUDA;
        }
        g_scratch_ptr[device] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch_ptr[device];
    return DEM_OK;
}

// The launch just queued: its configuration error, if any (a launch error is
// this call's own; the check at entry made sure none was pending before).
inline bool launched() { return cudaGetLastError() == cudaSuccess; }

}  // namespace

extern "C" int dem_bucket_sort_noalloc(const double* px, const double* py, const double* pz,
                                       int64_t n, const double* domain_min, double cell_size,
                                       int64_t hash_table_size, uint32_t* bucket,
                                       uint32_t* sorted, void* stream) {
    if (n < 0 || !domain_min || !(cell_size > 0) || hash_table_size < 1) return DEM_ERR_INVALID;
    if (n > kMaxN || hash_table_size > kMaxH) return DEM_ERR_CAPACITY;
    if (n > 0 && (!px || !py || !pz || !bucket || !sorted)) return DEM_ERR_INVALID;
    if (n == 0) return DEM_OK;
    // an error already pending on this thread belongs to someone else: it is
    // reported (DEM_ERR_CUDA) and left in place, and no work is queued
    if (cudaPeekAtLastError() != cudaSuccess) return DEM_ERR_CUDA;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return DEM_ERR_NO_DEVICE;
    uint32_t* scratch = nullptr;
    const int rc = scratch_on(device, &scratch);
    if (rc != DEM_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t* keys_tmp = scratch + kKeysOff;
    uint32_t* idx_tmp = scratch + kValsOff;
    uint32_t* hist = scratch + kHistOff;
    uint32_t* tiles = scratch + kTilesOff;
    Geometry g;
    for (int c = 0; c < 3; ++c) g.dmin[c] = domain_min[c];  // host memory
    g.cell = cell_size;
    g.H = (uint32_t)hash_table_size;
    g.mask = (g.H & (g.H - 1)) == 0 ? g.H - 1 : 0u;
    const int nn = (int)n;
    k_na_hash<<<(nn + kBlock - 1) / kBlock, kBlock, 0, s>>>(px, py, pz, nn, g, bucket);
    if (!launched()) return DEM_ERR_CUDA;
    // buckets are 0 .. H-1 < 2^20: one 10-bit pass for H <= 1,024, else two
    const int passes = hash_table_size <= kBins ? 1 : 2;
    const int nblk = (nn + kChunk - 1) / kChunk;
    const long long m = (long long)kBins * nblk;
    const int ntiles = (int)((m + kTile - 1) / kTile);
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = pass * kDigitBits;
        const bool last = pass == passes - 1;
        const uint32_t* kin = pass == 0 ? bucket : keys_tmp;
        const uint32_t bias = pass == 0 ? 1u : 0u;  // the outputs' buckets are 1-based
        const uint32_t* iin = pass == 0 ? nullptr : idx_tmp;
        k_na_digit_count<<<nblk, kBlock, 0, s>>>(kin, bias, nn, shift, nblk, hist);
        if (!launched()) return DEM_ERR_CUDA;
        k_na_tile_sums<<<ntiles, kBlock, 0, s>>>(hist, m, tiles);
        if (!launched()) return DEM_ERR_CUDA;
        k_na_scan_tiles<<<1, kBlock, 0, s>>>(tiles, ntiles);
        if (!launched()) return DEM_ERR_CUDA;
        k_na_apply<<<ntiles, kBlock, 0, s>>>(hist, m, tiles);
        if (!launched()) return DEM_ERR_CUDA;
        k_na_digit_scatter<<<nblk, kBlock, 0, s>>>(kin, bias, iin, nn, shift, nblk, hist,
                                                   last ? nullptr : keys_tmp,
                                                   last ? sorted : idx_tmp);
        if (!launched()) return DEM_ERR_CUDA;
    }
    return DEM_OK;
}
