// dem_kernels.cu — the DEM step as hand-written CUDA for sm_103a.
//
// One step (the reference's `simulate!`, src/executor.jl:162-172) is
//   k_hash       cell, Morton bucket, octant; warp-aggregated bucket counts
//   k_scan       exclusive scan of the H bucket counts (single pass, decoupled
//                look-back)                                   -> bucket starts
//   k_scatter    counting-sort scatter (warp-aggregated atomics; the counts
//                return to zero, so the table needs no clearing)
//   k_canon      ascending index inside each bucket + bucket-sorted copies of
//                the positions (FP64 and an FP32 copy for the pre-filter)
//   k_detect     cp_list enumeration fused with update_contacts!: existing
//                contacts decide survival, new touching pairs are stashed
//   k_scan       exclusive scan of the new row sizes          -> row_ptr
//   k_compact    rolling-array rebuild: surviving + new contacts, rows sorted
//                by j; incoming-contact lists for the force gather
//   k_force      resolve_collision! per contact (EBPM or Hertz-Mindlin)
//   k_integrate  per particle: contact force gather in a fixed order,
//                resolve_wall!, apply_body_force!, update!
// All of it is captured once in a CUDA graph per contact-buffer parity.
#include <cstdio>

#include "dem_device.cuh"

namespace dem {
namespace {

constexpr int kThreads = 256;
constexpr int kScanBlock = 1024;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;
constexpr unsigned long long kSpinLimit = 1ull << 24;
constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagIncl = 2ull << 62;
constexpr unsigned long long kValMask = (1ull << 62) - 1;

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }
// Row bound clamped to the buffer capacity: after a capacity overflow (which
// raises kErrCapacity) no kernel reads or writes past the contact buffers.
__device__ __forceinline__ int row_at(const int32_t* rp, int i, int cap) {
    const int v = rp[i];
    return v < 0 ? 0 : (v < cap ? v : cap);
}

// ---------------------------------------------------------------------------
// Exclusive scan, single pass with decoupled look-back.  Tiles are taken in
// launch order from a counter, so a tile only waits for tiles already running;
// every wait is bounded and raises kErrTimeout when the bound is hit.  The
// last tile to finish resets the tile states and counters for the next launch.
// out has count+1 entries; out[count] is the total.
// LIMITED: the bucket-count scan covers only [0, bmax] (bmax = largest bucket
// this step, from k_hash); tiles past it exit at once, cell_limit records the
// covered range and bmax is reset for the next step.
template <typename T, bool LIMITED>
__global__ void __launch_bounds__(kScanBlock)
    k_scan_excl(const T* __restrict__ in, T* __restrict__ out, long long count, int ntiles,
                unsigned long long* state, DevCounters* ctr) {
    __shared__ int s_tile;
    __shared__ int s_last;
    __shared__ unsigned long long s_warp[kScanBlock / 32];
    __shared__ unsigned long long s_prefix;
    if (LIMITED) {
        const long long lim = (long long)ctr->bmax + 1;
        count = lim < count ? lim : count;
    }
    const int ntiles_eff = (int)((count + kScanTile - 1) / kScanTile);
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(&ctr->scan_tiles, 1ull);
    __syncthreads();
    const int tile = s_tile;
    if (tile < ntiles_eff) {
        const long long base = (long long)tile * kScanTile + (long long)threadIdx.x * kScanItems;
        T v[kScanItems];
        unsigned long long sum = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            long long idx = base + k;
            v[k] = idx < count ? in[idx] : (T)0;
            sum += (unsigned long long)v[k];
        }
        unsigned long long x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane_id() >= (unsigned)o) x += y;
        }
        const int warp = threadIdx.x >> 5;
        if (lane_id() == 31) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            unsigned long long w = lane_id() < kScanBlock / 32 ? s_warp[lane_id()] : 0ull;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane_id() >= (unsigned)o) w += y;
            }
            if (lane_id() < kScanBlock / 32) s_warp[lane_id()] = w;
        }
        __syncthreads();
        const unsigned long long agg = s_warp[kScanBlock / 32 - 1];
        const unsigned long long texcl = (warp ? s_warp[warp - 1] : 0ull) + x - sum;
        if (threadIdx.x == 0) {
            cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> me(state[tile]);
            unsigned long long prefix = 0;
            if (tile == 0) {
                me.store(kFlagIncl | (agg & kValMask), cuda::memory_order_release);
            } else {
                me.store(kFlagAgg | (agg & kValMask), cuda::memory_order_release);
                for (int q = tile - 1; q >= 0; --q) {
                    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> pr(state[q]);
                    unsigned long long st = 0;
                    for (unsigned long long it = 0;; ++it) {
                        st = pr.load(cuda::memory_order_acquire);
                        if (st >> 62) break;
                        if (it > kSpinLimit) {
                            raise_error(ctr, kErrTimeout);
                            st = kFlagIncl;
                            break;
                        }
                        __nanosleep(64);
                    }
                    prefix += st & kValMask;
                    if ((st & ~kValMask) == kFlagIncl) break;
                }
                me.store(kFlagIncl | ((prefix + agg) & kValMask), cuda::memory_order_release);
            }
            s_prefix = prefix;
            if (tile == ntiles_eff - 1) out[count] = (T)(prefix + agg);
        }
        __syncthreads();
        unsigned long long run = s_prefix + texcl;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            long long idx = base + k;
            if (idx < count) out[idx] = (T)run;
            run += (unsigned long long)v[k];
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned long long done = atomicAdd(&ctr->scan_done, 1ull);
        s_last = (done == (unsigned long long)ntiles - 1) ? 1 : 0;
    }
    __syncthreads();
    if (s_last) {
        for (int t = threadIdx.x; t < ntiles_eff; t += kScanBlock) state[t] = 0ull;
        if (threadIdx.x == 0) {
            if (count == 0) out[0] = (T)0;
            if (LIMITED) {
                ctr->cell_limit = (unsigned int)count;
                ctr->bmax = 0u;
            }
            ctr->scan_tiles = 0ull;
            ctr->scan_done = 0ull;
        }
    }
}

// ---------------------------------------------------------------------------
// `cell`, `hashcode`, `center`, `neighbors` (src/utils.jl:1-16) and
// `count_particles!` (src/kernels.jl:7-13).
__global__ void __launch_bounds__(kThreads) k_hash(DemDev d, DemParams p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < p.n;
    uint32_t b = 0;
    if (act) {
        const double pos[3] = {d.px[i], d.py[i], d.pz[i]};
        int ijk[3];
        int oct = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            ijk[c] = ceil_i32(__ddiv_rn(__dsub_rn(pos[c], p.dmin[c]), p.cell));
            const double ctr =
                __dadd_rn(p.dmin[c], __dmul_rn(__dsub_rn((double)ijk[c], 0.5), p.cell));
            if (pos[c] > ctr) oct |= 1 << c;
        }
        b = bucket_of(ijk[0], ijk[1], ijk[2], p);
        d.cellinfo[i] = make_int4(ijk[0], ijk[1], ijk[2], oct);
        d.bucket[i] = b;
    }
    const unsigned mask = __ballot_sync(0xffffffffu, act);
    if (act) {
        const unsigned peers = __match_any_sync(mask, b);
        if (lane_id() == (unsigned)(__ffs(peers) - 1)) atomicAdd(&d.cell_count[b], __popc(peers));
        const unsigned wmax = __reduce_max_sync(mask, b);
        if (lane_id() == (unsigned)(__ffs(mask) - 1)) atomicMax(&d.ctr->bmax, wmax);
    }
}

// `get_particle_id!` (src/kernels.jl:15-22): counting-sort scatter.  The
// atomic decrements bring every count back to zero.
__global__ void __launch_bounds__(kThreads) k_scatter(DemDev d, DemParams p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < p.n;
    const unsigned mask = __ballot_sync(0xffffffffu, act);
    if (!act) return;
    const uint32_t b = d.bucket[i];
    const unsigned peers = __match_any_sync(mask, b);
    const int leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if (lane_id() == (unsigned)leader) old = atomicSub(&d.cell_count[b], (uint32_t)__popc(peers));
    old = __shfl_sync(peers, old, leader);
    const uint32_t slot = old - 1u - (uint32_t)__popc(peers & lanemask_lt());
    d.unsorted[d.cell_start[b] + slot] = (uint32_t)i;
}

// Canonical order inside a bucket (ascending particle index) and the sorted
// position copies used by the pair search.
__global__ void __launch_bounds__(kThreads) k_canon(DemDev d, DemParams p) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= p.n) return;
    const uint32_t i = d.unsorted[k];
    const uint32_t b = d.bucket[i];
    const uint32_t s = d.cell_start[b], e = d.cell_start[b + 1];
    uint32_t rank = 0;
    for (uint32_t t = s; t < e; ++t) rank += d.unsorted[t] < i ? 1u : 0u;
    const uint32_t pos = s + rank;
    d.sorted[pos] = i;
    const double x = d.px[i], y = d.py[i], z = d.pz[i], r = d.r[i];
    d.spos[pos] = make_double4_32a(x, y, z, r);
    d.spos32[pos] = make_float4((float)(x - p.dmin[0]), (float)(y - p.dmin[1]),
                                (float)(z - p.dmin[2]), (float)r);
}

// ---------------------------------------------------------------------------
// cp_list enumeration fused with `update_contacts!` (src/kernels.jl:87-120) or
// `init_bonds!` (src/kernels.jl:60-85).  Eight lanes per particle i (in
// bucket order), lane t taking the t-th of i's octant buckets in the order of
// `neighbors` (src/utils.jl:4-16); pairs (i, j) with j > i in those buckets are
// the reference's cp_list.  A bucket that repeats an earlier lane's bucket is
// skipped, so a pair listed twice in cp_list is handled once.
//  * existing Hertz contact (i, j): ends iff the pair is in cp_list and no
//    longer touching; bonded contacts survive (breakage is decided by the
//    force kernel); contacts broken last step are dropped.
//  * new contact: touching and not in row i.  Row membership is checked
//    before the FP64 distance test, so bonded neighbours cost no FP64 work.
constexpr int kLanes = 8;
__device__ __forceinline__ void bucket_range(const DemDev& d, uint32_t b, uint32_t lim,
                                             uint32_t* s, uint32_t* e) {
    if (b < lim) {
        *s = d.cell_start[b];
        *e = d.cell_start[b + 1];
    } else {
        *s = *e = 0u;
    }
}

template <bool INIT>
__global__ void __launch_bounds__(kThreads) k_detect(DemDev d, DemParams p, int cur) {
    __shared__ int s_new[kThreads / kLanes];
    const int lane = threadIdx.x & (kLanes - 1);
    const int g = threadIdx.x / kLanes;
    const int k = blockIdx.x * (kThreads / kLanes) + g;
    if (lane == 0) s_new[g] = 0;
    __syncwarp();
    if (k >= p.n) return;
    const unsigned gmask = 0xffu << (lane_id() & ~7u);
    const int i = (int)d.sorted[k];
    const double4_32a P = d.spos[k];
    const float4 P32 = d.spos32[k];
    const int4 ci = d.cellinfo[i];
    const int dx = (ci.w & 1) ? 1 : -1, dy = (ci.w & 2) ? 1 : -1, dz = (ci.w & 4) ? 1 : -1;
    const int ox = (lane == 1 || lane == 4 || lane == 5 || lane == 7) ? dx : 0;
    const int oy = (lane == 2 || lane == 4 || lane == 6 || lane == 7) ? dy : 0;
    const int oz = (lane == 3 || lane == 5 || lane == 6 || lane == 7) ? dz : 0;
    const uint32_t myB = bucket_of(ci.x + ox, ci.y + oy, ci.z + oz, p);
    uint32_t B[8];
    bool dup = false;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        B[u] = __shfl_sync(gmask, myB, u, kLanes);
        dup |= (u < lane) && (B[u] == myB);
    }
    const double ri = INIT ? d.r0[i] : P.w;

    const ContactSoA o = d.c[cur];
    const int e0 = row_at(d.row_ptr[cur], i, p.cap), e1 = row_at(d.row_ptr[cur], i + 1, p.cap);
    int nkeep = 0;
    int ended = 0;
    for (int e = e0 + lane; e < e1; e += kLanes) {
        const uint32_t fl = o.fl[e];
        int keep;
        if (!(fl & kActive)) {
            keep = 0;
        } else if (INIT || (fl & kBonded)) {
            keep = 1;
        } else {
            const int j = o.cj[e];
            const bool valid = touching_rn(P.x, P.y, P.z, d.px[j], d.py[j], d.pz[j], P.w, d.r[j]);
            const uint32_t bj = d.bucket[j];
            bool in_cp = false;
#pragma unroll
            for (int t = 0; t < 8; ++t) in_cp |= (B[t] == bj);
            keep = (valid || !in_cp) ? 1 : 0;
            ended += 1 - keep;
        }
        d.keep[e] = (uint8_t)keep;
        nkeep += keep;
    }
    nkeep = __reduce_add_sync(gmask, nkeep);
    ended = __reduce_add_sync(gmask, ended);

    int32_t* stash = d.stash + (size_t)i * p.kstash;
    uint32_t s, e;
    bucket_range(d, myB, d.ctr->cell_limit, &s, &e);
    if (dup) e = s;
    for (uint32_t q = s; q < e; ++q) {
        const int j = (int)d.sorted[q];
        const float4 Q32 = d.spos32[q];
        if (j <= i) continue;
        if (!INIT && !maybe_touching32(P32, Q32)) continue;
        bool found = false;
        for (int e2 = e0; e2 < e1 && !found; ++e2) found = (o.cj[e2] == j) && (o.fl[e2] & kActive);
        if (found) continue;
        const double4_32a Q = d.spos[q];
        const double rj = INIT ? d.r0[j] : Q.w;
        if (!touching_rn(P.x, P.y, P.z, Q.x, Q.y, Q.z, ri, rj)) continue;
        const int slot = atomicAdd(&s_new[g], 1);
        if (slot < p.kstash) stash[slot] = j;
    }
    __syncwarp(gmask);
    if (lane == 0) {
        int nnew = s_new[g];
        if (nnew > p.kstash) {
            raise_error(d.ctr, kErrCapacity);
            nnew = p.kstash;
        }
        for (int a2 = 1; a2 < nnew; ++a2) {  // new partners ascending
            const int v = stash[a2];
            int b2 = a2 - 1;
            while (b2 >= 0 && stash[b2] > v) {
                stash[b2 + 1] = stash[b2];
                --b2;
            }
            stash[b2 + 1] = v;
        }
        d.nnew[i] = nnew;
        d.cnt[i] = nkeep + nnew;
        if (ended) atomicAdd(&d.ctr->ended, (unsigned long long)ended);
        if (!INIT && nnew) atomicAdd(&d.ctr->created, (unsigned long long)nnew);
    }
}

// Rolling-array rebuild (the reference's remove_inactive_contact! + swap,
// src/kernels.jl:487-506, src/executor.jl:140-153): row i of buffer cur^1 is
// the merge, by j, of the surviving entries of row i and the sorted new
// partners.  One thread per old contact (coalesced copies) and one per
// particle for its new contacts; each computes its final slot directly.
template <bool INIT>
__global__ void __launch_bounds__(kThreads) k_compact(DemDev d, DemParams p, int cur) {
    const int nxt = cur ^ 1;
    const int total = d.row_ptr[nxt][p.n];
    if (total > p.cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) raise_error(d.ctr, kErrCapacity);
        return;
    }
    const int* rpo = d.row_ptr[cur];
    const int* rpn = d.row_ptr[nxt];
    const int cold = row_at(rpo, p.n, p.cap);
    const ContactSoA o = d.c[cur];
    const ContactSoA w = d.c[nxt];
    const int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < cold + p.n; t += stride) {
        if (t < cold) {
            if (!d.keep[t]) continue;
            const int i = o.ci[t], j = o.cj[t];
            int pos = rpn[i];
            for (int q = row_at(rpo, i, p.cap); q < t; ++q) pos += d.keep[q];
            const int nn = d.nnew[i];
            const int32_t* st = d.stash + (size_t)i * p.kstash;
            for (int u = 0; u < nn; ++u) pos += st[u] < j ? 1 : 0;
            w.ci[pos] = i;
            w.cj[pos] = j;
            w.fl[pos] = o.fl[t];
#pragma unroll
            for (int f = 0; f < 15; ++f) w.f[f][pos] = o.f[f][t];
            if (!INIT) {
                const int slot = atomicAdd(&d.in_cnt[j], 1);
                if (slot < p.kin) d.in_list[(size_t)j * p.kin + slot] = pos;
                else raise_error(d.ctr, kErrCapacity);
            }
        } else {
            const int i = t - cold;
            const int nn = d.nnew[i];
            if (!nn) continue;
            const int e0 = row_at(rpo, i, p.cap), e1 = row_at(rpo, i + 1, p.cap);
            const int32_t* st = d.stash + (size_t)i * p.kstash;
            for (int u = 0; u < nn; ++u) {
                const int j = st[u];
                int pos = rpn[i] + u;
                for (int q = e0; q < e1; ++q) pos += (d.keep[q] && o.cj[q] < j) ? 1 : 0;
                w.ci[pos] = i;
                w.cj[pos] = j;
                w.fl[pos] = INIT ? (kActive | kBonded) : kActive;
#pragma unroll
                for (int f = 0; f < 15; ++f) w.f[f][pos] = 0.0;
                if (!INIT) {
                    const int slot = atomicAdd(&d.in_cnt[j], 1);
                    if (slot < p.kin) d.in_list[(size_t)j * p.kin + slot] = pos;
                    else raise_error(d.ctr, kErrCapacity);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Contact frame of src/kernels.jl:145-165: the rotation taking the unit normal
// a = normalize(𝐤ⱼ - 𝐤ᵢ) to the local x axis.  For b = x̂ the reference's
// I + [v]ₓ + [v]ₓ² (1-c)/s² reduces to the rows
//   ( c, a₂, a₃ ), ( -a₂, 1 - a₂² f, -a₂a₃ f ), ( -a₃, -a₂a₃ f, 1 - a₃² f ),
// f = (1 - c)/s².  The branch s < tolerance is decided on exactly the
// reference's s and c (normalize and norm without contraction).  The matrix is
// orthonormal, so its inverse (src/kernels.jl:224, 298) is its transpose.
struct Frame {
    double r[3][3];
};
__device__ __forceinline__ Frame contact_frame(double ax, double ay, double az, double tol) {
    Frame F;
    // v = a × x̂ = (±0, a₃, -a₂); s = norm(v) evaluated as sqrt((0 + a₃²) + a₂²)
    const double s = norm_rn(0.0, az, -ay);
    const double c = ax;
    if (s < tol) {
        const double sg = c > 0.0 ? 1.0 : -1.0;
        F.r[0][0] = sg; F.r[0][1] = 0.0; F.r[0][2] = 0.0;
        F.r[1][0] = 0.0; F.r[1][1] = 1.0; F.r[1][2] = 0.0;
        F.r[2][0] = 0.0; F.r[2][1] = 0.0; F.r[2][2] = sg;
    } else {
        const double f = (1.0 - c) / (s * s);
        F.r[0][0] = c; F.r[0][1] = ay; F.r[0][2] = az;
        F.r[1][0] = -ay; F.r[1][1] = 1.0 - ay * ay * f; F.r[1][2] = -ay * az * f;
        F.r[2][0] = -az; F.r[2][1] = -ay * az * f; F.r[2][2] = 1.0 - az * az * f;
    }
    return F;
}
template <typename T>
__device__ __forceinline__ Vec3<T> rot(const Frame& F, Vec3<T> v) {  // R v
    return {(T)F.r[0][0] * v.x + (T)F.r[0][1] * v.y + (T)F.r[0][2] * v.z,
            (T)F.r[1][0] * v.x + (T)F.r[1][1] * v.y + (T)F.r[1][2] * v.z,
            (T)F.r[2][0] * v.x + (T)F.r[2][1] * v.y + (T)F.r[2][2] * v.z};
}
template <typename T>
__device__ __forceinline__ Vec3<T> rot_t(const Frame& F, Vec3<T> v) {  // Rᵀ v
    return {(T)F.r[0][0] * v.x + (T)F.r[1][0] * v.y + (T)F.r[2][0] * v.z,
            (T)F.r[0][1] * v.x + (T)F.r[1][1] * v.y + (T)F.r[2][1] * v.z,
            (T)F.r[0][2] * v.x + (T)F.r[1][2] * v.y + (T)F.r[2][2] * v.z};
}

__device__ __forceinline__ Vec3<double> ld3(const double* const* f, int base, int c) {
    return {f[base][c], f[base + 1][c], f[base + 2][c]};
}
__device__ __forceinline__ void st3(double* const* f, int base, int c, Vec3<double> v) {
    f[base][c] = v.x;
    f[base + 1][c] = v.y;
    f[base + 2][c] = v.z;
}
template <typename T>
__device__ __forceinline__ Vec3<double> to_d(Vec3<T> v) {
    return {(double)v.x, (double)v.y, (double)v.z};
}
template <typename T>
__device__ __forceinline__ Vec3<T> from_d(Vec3<double> v) {
    return {(T)v.x, (T)v.y, (T)v.z};
}

// The frame with the normal a already computed approximately (rsqrt).  Far
// from the degenerate case (s = |a × x̂| >= 2·tolerance) both branches of the
// reference are decided the same way and the general formula is used; near
// it, a and s are recomputed exactly as the reference does (normalize and norm
// without contraction) so the branch matches the reference bit for bit.
__device__ __forceinline__ Frame contact_frame_fast(double dx, double dy, double dz, double ax,
                                                    double ay, double az, double tol) {
    const double s2 = ay * ay + az * az;
    if (s2 < 4.0 * tol * tol) {
        const double L = norm_rn(dx, dy, dz);
        const double il = __ddiv_rn(1.0, L);
        return contact_frame(__dmul_rn(il, dx), __dmul_rn(il, dy), __dmul_rn(il, dz), tol);
    }
    Frame F;
    const double f = (1.0 - ax) / s2;
    F.r[0][0] = ax; F.r[0][1] = ay; F.r[0][2] = az;
    F.r[1][0] = -ay; F.r[1][1] = 1.0 - ay * ay * f; F.r[1][2] = -ay * az * f;
    F.r[2][0] = -az; F.r[2][1] = -ay * az * f; F.r[2][2] = 1.0 - az * az * f;
    return F;
}

// EBPM failure (src/kernels.jl:208-219):
//   σcᵢ = -Fₓ/A - (r/I)·sqrt(τᵢ₂²+τᵢ₃²), σc = -min(σcᵢ, σcⱼ), σt = max(σcᵢ, σcⱼ),
//   σs = |τᵢ₁|·r/2/I + 4/3/A·sqrt(F₂²+F₃²);  breaks if σc >= σc₀ or σt >= σt₀ or
//   σs >= σs₀.
// Each comparison is evaluated without its square root: sqrt(a)·k >= R is
// R <= 0 or a·k² >= R², and sqrt(a)·k <= R is R >= 0 and a·k² <= R² (k > 0).
// A NaN operand makes a comparison false, as in the reference.
__device__ __forceinline__ bool bond_breaks(const Vec3<double>& F, const Vec3<double>& ti,
                                            const Vec3<double>& tj, double invA, double rbI,
                                            const DemParams& p) {
    const double ai = ti.y * ti.y + ti.z * ti.z, aj = tj.y * tj.y + tj.z * tj.z;
    const double amax = jl_max(ai, aj), amin = jl_min(ai, aj);
    const double fa = F.x * invA, k2 = rbI * rbI;
    const double Rc = p.b_sc - fa;     // σc >= σc₀  <=>  rbI·sqrt(amax) >= Rc
    const double Rt = -(p.b_st + fa);  // σt >= σt₀  <=>  rbI·sqrt(amin) <= Rt
    const double Rs = p.b_ss - fabs(ti.x) * (0.5 * rbI);  // σs >= σs₀ <=> 4/3·invA·sqrt(b) >= Rs
    const double b = F.y * F.y + F.z * F.z;
    const double ks = (4.0 / 3.0) * invA;
    const bool comp = !isnan(amax) && (Rc <= 0.0 || amax * k2 >= Rc * Rc);
    const bool tens = !isnan(amin) && Rt >= 0.0 && amin * k2 <= Rt * Rt;
    const bool shear = !isnan(b) && !isnan(Rs) && (Rs <= 0.0 || b * (ks * ks) >= Rs * Rs);
    return comp || tens || shear;
}

// `resolve_collision!` for one active contact (src/kernels.jl:136-313).  T is
// the arithmetic type of the force model: double (DEM_FP64) or float
// (DEM_FP32_FORCE).  Relative quantities (overlap, relative displacement and
// rotation increments, relative velocity) are always formed in FP64 and then
// cast; the accumulated bond force/torques, the shear displacement 𝐬 and the
// bond-breakage test stay FP64 in both modes.
//
// EBPM in sum/difference form: with 𝚫 = 𝐝ᵢ - 𝐝ⱼ = 𝐑(𝐯ᵢ - 𝐯ⱼ)dt,
// 𝛉ₛ = 𝐑(𝛚ᵢ + 𝛚ⱼ)dt and 𝛉_d = 𝐑(𝛚ᵢ - 𝛚ⱼ)dt, the reference's increments
// k₅𝛉ᵢ + k₆𝛉ⱼ and k₆𝛉ᵢ + k₅𝛉ⱼ are k₊𝛉ₛ ± k₋𝛉_d with k₊ = (k₅+k₆)/2 =
// 3EI/L/(1+ϕ) and k₋ = (k₅-k₆)/2 = EI/L.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_force(DemDev d, DemParams p, int nxt) {
    int C = d.row_ptr[nxt][p.n];
    C = C < p.cap ? C : p.cap;
    const ContactSoA w = d.c[nxt];
    const int stride = gridDim.x * blockDim.x;
    const double dt = p.dt;
    const size_t cap = (size_t)p.cap;
    unsigned long long nbroken = 0, ngap = 0, ngamma = 0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += stride) {
        const uint32_t fl = w.fl[c];
        const int i = w.ci[c], j = w.cj[c];
        const Vec3<double> ki{d.px[i], d.py[i], d.pz[i]}, kj{d.px[j], d.py[j], d.pz[j]};
        const double ri = d.r[i], rj = d.r[j];
        // normal and length; the frame's branch is decided on the exact
        // reference values when the normal is within 2·tolerance of ±x̂
        const double dx = kj.x - ki.x, dy = kj.y - ki.y, dz = kj.z - ki.z;
        const double invL = rsqrt(dx * dx + dy * dy + dz * dz);
        const double L = (dx * dx + dy * dy + dz * dz) * invL;
        const double ax = dx * invL, ay = dy * invL, az = dz * invL;
        const Frame R = contact_frame_fast(dx, dy, dz, ax, ay, az, p.tol);
        const Vec3<double> vi{d.vx[i], d.vy[i], d.vz[i]}, vj{d.vx[j], d.vy[j], d.vz[j]};
        const Vec3<double> wi{d.wx[i], d.wy[i], d.wz[i]}, wj{d.wx[j], d.wy[j], d.wz[j]};
        Vec3<T> fig, mi, mj;
        if (fl & kBonded) {
            // EBPM (src/kernels.jl:170-239)
            const Vec3<double> Dd = rot<double>(R, {(vi.x - vj.x) * dt, (vi.y - vj.y) * dt, (vi.z - vj.z) * dt});
            const Vec3<double> Ts = rot<double>(R, {(wi.x + wj.x) * dt, (wi.y + wj.y) * dt, (wi.z + wj.z) * dt});
            const Vec3<double> Td = rot<double>(R, {(wi.x - wj.x) * dt, (wi.y - wj.y) * dt, (wi.z - wj.z) * dt});
            const Vec3<T> D = from_d<T>(Dd), S = from_d<T>(Ts), Q = from_d<T>(Td);
            const double rb = p.b_rho * jl_min(ri, rj);
            const double rb2 = rb * rb;
            const double Ib = rb2 * rb2 * (CUDART_PI / 4.0);
            const double Ab = rb2 * CUDART_PI;
            const T tinvL = (T)invL;
            const T phi = (T)(20.0 / 3.0 * (1.0 + p.b_nu) * rb2) * tinvL * tinvL;
            const T iphi = (T)1.0 / ((T)1.0 + phi);
            const T EIL = (T)(p.b_E * Ib) * tinvL;  // EI/L
            const T k1 = (T)(p.b_E * Ab) * tinvL;
            const T k3 = (T)6.0 * EIL * tinvL * iphi;
            const T k2 = (T)2.0 * k3 * tinvL;
            const T k4 = EIL * (T)p.b_inv1pnu;
            const T kp = (T)3.0 * EIL * iphi;
            const T km = EIL;
            const T dFx = k1 * D.x, dFy = k2 * D.y + k3 * S.z, dFz = k2 * D.z - k3 * S.y;
            const T ay_ = -k3 * D.z + kp * S.y, az_ = k3 * D.y + kp * S.z;
            const T dtix = k4 * Q.x, dtiy = ay_ + km * Q.y, dtiz = az_ + km * Q.z;
            const T dtjx = -k4 * Q.x, dtjy = ay_ - km * Q.y, dtjz = az_ - km * Q.z;
            Vec3<double> Fi = ld3(w.f, CF, c), ti = ld3(w.f, CTI, c), tj = ld3(w.f, CTJ, c);
            Fi = {Fi.x + (double)dFx, Fi.y + (double)dFy, Fi.z + (double)dFz};
            ti = {ti.x + (double)dtix, ti.y + (double)dtiy, ti.z + (double)dtiz};
            tj = {tj.x + (double)dtjx, tj.y + (double)dtjy, tj.z + (double)dtjz};
            // breakage test, FP64 (src/kernels.jl:208-222), see bond_breaks()
            const int small = ri <= rj ? i : j;  // rb = ρ·min(rᵢ, rⱼ)
            if (bond_breaks(Fi, ti, tj, d.b_invA[small], d.b_rbI[small], p)) {
                w.fl[c] = 0u;  // contact_active and contact_bonded bits cleared
                ++nbroken;
                fig = {(T)0, (T)0, (T)0};
                mi = fig;
                mj = fig;
            } else {
                const Vec3<double> fg = rot_t<double>(R, {-Fi.x, -Fi.y, -Fi.z});
                const Vec3<double> mg_i = rot_t<double>(R, {-ti.x, -ti.y, -ti.z});
                const Vec3<double> mg_j = rot_t<double>(R, {-tj.x, -tj.y, -tj.z});
                fig = from_d<T>(fg);
                mi = from_d<T>(mg_i);
                mj = from_d<T>(mg_j);
                st3(w.f, CK, c, {(ki.x + kj.x) * 0.5, (ki.y + kj.y) * 0.5, (ki.z + kj.z) * 0.5});
                st3(w.f, CF, c, Fi);
                st3(w.f, CTI, c, ti);
                st3(w.f, CTJ, c, tj);
                st3(w.f, CS, c, {0.0, 0.0, 0.0});
            }
        } else {
            // Hertz-Mindlin (src/kernels.jl:240-313)
            const double gap = L - ri - rj;
            if (gap > 0) ++ngap;
            const double ext = ri - fabs(gap);
            st3(w.f, CK, c, {ki.x + ax * ext, ki.y + ay * ext, ki.z + az * ext});
            const Vec3<T> kri{(T)(ax * ext), (T)(ay * ext), (T)(az * ext)};
            const Vec3<T> krj{kri.x - (T)dx, kri.y - (T)dy, kri.z - (T)dz};
            const Vec3<T> wci = cross3<T>(from_d<T>(wi), kri);
            const Vec3<T> wcj = cross3<T>(from_d<T>(wj), krj);
            const Vec3<T> dv{(T)(vj.x - vi.x) + (wcj.x - wci.x), (T)(vj.y - vi.y) + (wcj.y - wci.y),
                             (T)(vj.z - vi.z) + (wcj.z - wci.z)};
            const Vec3<T> vc = rot<T>(R, dv);
            const T tri = (T)ri, trj = (T)rj, tmi = (T)d.m[i], tmj = (T)d.m[j];
            const T Rs = tri * trj / (tri + trj);
            const T ms = tmi * tmj / (tmi + tmj);
            const T tgap = (T)gap;
            const T sq = sqrt(Rs * (T)fabs(gap));
            const T kn = (T)(4.0 / 3.0 * p.pp_Ys) * sq;
            const T kt = (T)(8.0 * p.pp_Gs) * sq;
            const T root = sqrt(ms * sq);
            const T gn = (T)p.pp_cgn * root;
            const T gt = (T)p.pp_cgt * root;
            if (gn < (T)0) ++ngamma;
            if (gt < (T)0) ++ngamma;
            Vec3<double> s = ld3(w.f, CS, c);
            s = {s.x + (double)vc.x * 0.0, s.y + (double)vc.y * dt, s.z + (double)vc.z * dt};
            const T F1 = -kn * tgap - gn * vc.x;
            const Vec3<T> Ft{-kt * (T)s.x, -kt * (T)s.y, -kt * (T)s.z};
            const T nFt = sqrt(Ft.x * Ft.x + Ft.y * Ft.y + Ft.z * Ft.z);
            const T muF1 = (T)p.pp_mu * F1;
            T F2, F3;
            if (nFt >= muF1) {
                const T ratio = muF1 / nFt;
                F2 = ratio * Ft.y;
                F3 = ratio * Ft.z;
                s = {s.x, (double)(F2 / kt), (double)(F3 / kt)};
            } else {
                F2 = Ft.y - gt * vc.y;
                F3 = Ft.z - gt * vc.z;
            }
            fig = rot_t<T>(R, {-F1, -F2, -F3});
            mi = cross3<T>(kri, fig);
            mj = cross3<T>(krj, {-fig.x, -fig.y, -fig.z});
            st3(w.f, CF, c, {(double)F1, (double)F2, (double)F3});
            st3(w.f, CS, c, s);
        }
        d.contrib[0 * cap + c] = (double)fig.x;
        d.contrib[1 * cap + c] = (double)fig.y;
        d.contrib[2 * cap + c] = (double)fig.z;
        d.contrib[3 * cap + c] = (double)mi.x;
        d.contrib[4 * cap + c] = (double)mi.y;
        d.contrib[5 * cap + c] = (double)mi.z;
        d.contrib[6 * cap + c] = (double)mj.x;
        d.contrib[7 * cap + c] = (double)mj.y;
        d.contrib[8 * cap + c] = (double)mj.z;
    }
    if (nbroken) atomicAdd(&d.ctr->broken, nbroken);
    if (ngap) atomicAdd(&d.ctr->warn_gap, ngap);
    if (ngamma) atomicAdd(&d.ctr->warn_damp, ngamma);
}

// Per particle: contact force gather in a fixed order (own row by j, then
// incoming contacts by contact index), `resolve_wall!` (src/kernels.jl:317-426),
// `apply_body_force!` (src/kernels.jl:428-443) and `update!`
// (src/kernels.jl:445-485).  For spheres 𝐈 = (2/5 m r²) I₃, so
// inv(𝐑)·inv(𝐈)·(𝐑𝛕 - 𝐑𝛚 × 𝐈𝐑𝛚) is 𝛕 / I exactly in real arithmetic and the
// quaternion only evolves as state.
constexpr int kMaxIncoming = 64;
constexpr int kRegIncoming = 16;
__global__ void __launch_bounds__(kThreads) k_integrate(DemDev d, DemParams p, int nxt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const size_t cap = (size_t)p.cap;
    const int* rp = d.row_ptr[nxt];
    double F[3] = {0.0, 0.0, 0.0}, M[3] = {0.0, 0.0, 0.0};
    const int c0 = row_at(rp, i, p.cap), c1 = row_at(rp, i + 1, p.cap);
    for (int c = c0; c < c1; ++c) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            F[q] += d.contrib[q * cap + c];
            M[q] += d.contrib[(3 + q) * cap + c];
        }
    }
    int nin = d.in_cnt[i];
    d.in_cnt[i] = 0;
    nin = nin < p.kin ? nin : p.kin;
    nin = nin < kMaxIncoming ? nin : kMaxIncoming;
    const int* il = d.in_list + (size_t)i * p.kin;
    if (nin <= kRegIncoming) {
        // ascending contact index, sorted in registers (odd-even transposition)
        int v[kRegIncoming];
#pragma unroll
        for (int t = 0; t < kRegIncoming; ++t) v[t] = t < nin ? il[t] : 0x7fffffff;
#pragma unroll
        for (int r = 0; r < kRegIncoming; ++r) {
#pragma unroll
            for (int t = r & 1; t + 1 < kRegIncoming; t += 2) {
                const int lo = min(v[t], v[t + 1]), hi = max(v[t], v[t + 1]);
                v[t] = lo;
                v[t + 1] = hi;
            }
        }
#pragma unroll
        for (int t = 0; t < kRegIncoming; ++t) {
            if (t < nin) {
                const int c = v[t];
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    F[q] += -d.contrib[q * cap + c];
                    M[q] += d.contrib[(6 + q) * cap + c];
                }
            }
        }
    } else {
        int inc[kMaxIncoming];
        for (int t = 0; t < nin; ++t) {
            const int v = il[t];
            int b = t - 1;
            while (b >= 0 && inc[b] > v) {
                inc[b + 1] = inc[b];
                --b;
            }
            inc[b + 1] = v;
        }
        for (int t = 0; t < nin; ++t) {
            const int c = inc[t];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                F[q] += -d.contrib[q * cap + c];
                M[q] += d.contrib[(6 + q) * cap + c];
            }
        }
    }
    const double x = d.px[i], y = d.py[i], z = d.pz[i];
    const double vx = d.vx[i], vy = d.vy[i], vz = d.vz[i];
    const double wx = d.wx[i], wy = d.wy[i], wz = d.wz[i];
    const double r = d.r[i], m = d.m[i];
    const double dt = p.dt;
    // resolve_wall!, one wall
    if (p.has_wall) {
        const double dotkn = __dadd_rn(__dadd_rn(__dmul_rn(x, p.wn[0]), __dmul_rn(y, p.wn[1])),
                                       __dmul_rn(z, p.wn[2]));
        const double L = __dsub_rn(dotkn, p.wd);
        if (fabs(L) < r) {
            const double gap = fabs(L) - r;
            const double dn = fabs(gap);
            const double sc = (fabs(L) + dn / 2.0) / fabs(L);
            const double kix = -L * p.wn[0] * sc, kiy = -L * p.wn[1] * sc, kiz = -L * p.wn[2] * sc;
            const double vcix = wy * kiz - wz * kiy + vx, vciy = wz * kix - wx * kiz + vy,
                         vciz = wx * kiy - wy * kix + vz;
            const double* Rw = p.wR;
            const double vcx = -(Rw[0] * vcix + Rw[1] * vciy + Rw[2] * vciz);
            const double vcy = -(Rw[3] * vcix + Rw[4] * vciy + Rw[5] * vciz);
            const double vcz = -(Rw[6] * vcix + Rw[7] * vciy + Rw[8] * vciz);
            const double sq = sqrt(r * dn);
            const double kn = 4.0 / 3.0 * p.pw_Ys * sq;
            const double kt = 8.0 * p.pw_Gs * sq;
            const double root = sqrt(m * sq);
            const double gn = p.pw_cgn * root;
            const double gt = p.pw_cgt * root;
            if (gn < 0) atomicAdd(&d.ctr->warn_damp, 1ull);
            if (gt < 0) atomicAdd(&d.ctr->warn_damp, 1ull);
            double sx = d.wsx[i] + vcx * 0.0, sy = d.wsy[i] + vcy * dt, sz = d.wsz[i] + vcz * dt;
            const double F1 = -kn * gap - gn * vcx;
            const double Ftx = -kt * sx, Fty = -kt * sy, Ftz = -kt * sz;
            const double nFt = sqrt(Ftx * Ftx + Fty * Fty + Ftz * Ftz);
            double F2, F3;
            if (nFt >= p.pw_mu * F1) {
                const double ratio = p.pw_mu * F1 / nFt;
                F2 = ratio * Fty;
                F3 = ratio * Ftz;
                sy = F2 / kt;
                sz = F3 / kt;
            } else {
                F2 = Fty - gt * vcy;
                F3 = Ftz - gt * vcz;
            }
            const double* Ri = p.wRinv;
            const double gx = -(Ri[0] * F1 + Ri[1] * F2 + Ri[2] * F3);
            const double gy = -(Ri[3] * F1 + Ri[4] * F2 + Ri[5] * F3);
            const double gz = -(Ri[6] * F1 + Ri[7] * F2 + Ri[8] * F3);
            F[0] += gx;
            F[1] += gy;
            F[2] += gz;
            M[0] += kiy * gz - kiz * gy;
            M[1] += kiz * gx - kix * gz;
            M[2] += kix * gy - kiy * gx;
            d.wsx[i] = sx;
            d.wsy[i] = sy;
            d.wsz[i] = sz;
        } else {
            d.wsx[i] = 0.0;
            d.wsy[i] = 0.0;
            d.wsz[i] = 0.0;
        }
    }
    // apply_body_force!
    F[0] += p.grav[0] * m;
    F[1] += p.grav[1] * m;
    F[2] += p.grav[2] * m;
    if (p.damping != 0.0) {
        const double v3[3] = {vx, vy, vz}, w3[3] = {wx, wy, wz};
        double dF[3], dM[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            dF[q] = -p.damping * fabs(F[q]) * jl_sign(v3[q]);
            dM[q] = -p.damping * fabs(M[q]) * jl_sign(w3[q]);
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            F[q] += dF[q];
            M[q] += dM[q];
        }
    }
    // update!
    const double invm = d.inv_m[i];
    const double ax = F[0] * invm, ay = F[1] * invm, az = F[2] * invm;
    const double hdt2 = 0.5 * (dt * dt);
    d.px[i] = x + vx * dt + ax * hdt2;
    d.py[i] = y + vy * dt + ay * hdt2;
    d.pz[i] = z + vz * dt + az * hdt2;
    d.vx[i] = vx + ax * dt;
    d.vy[i] = vy + ay * dt;
    d.vz[i] = vz + az * dt;
    const double qw = d.qw[i], qx = d.qx[i], qy = d.qy[i], qz = d.qz[i];
    const double dq0 = -0.5 * (qx * wx + qy * wy + qz * wz);
    const double dq1 = 0.5 * (qw * wx + qy * wz - qz * wy);
    const double dq2 = 0.5 * (qw * wy + qx * wz + qz * wx);
    const double dq3 = 0.5 * (qw * wz + qx * wy - qy * wx);
    const double nw = qw + dq0, nx = qx + dq1, ny = qy + dq2, nz = qz + dq3;
    const double inq = rsqrt(nw * nw + nx * nx + ny * ny + nz * nz);
    d.qw[i] = nw * inq;
    d.qx[i] = nx * inq;
    d.qy[i] = ny * inq;
    d.qz[i] = nz * inq;
    const double ii = d.inv_inertia[i];
    d.wx[i] = wx + M[0] * ii * dt;
    d.wy[i] = wy + M[1] * ii * dt;
    d.wz[i] = wz + M[2] * ii * dt;
    d.fx[i] = F[0];
    d.fy[i] = F[1];
    d.fz[i] = F[2];
    d.tx[i] = M[0];
    d.ty[i] = M[1];
    d.tz[i] = M[2];
}

// ---- inspection kernels (dem_debug_broadphase) -------------------------------
__global__ void k_morton(DemDev d, DemParams p, uint32_t* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const int4 c = d.cellinfo[i];
    out[i] = morton1(c.x, c.y, c.z);
}
// search_hash_table! (src/kernels.jl:24-37): pair count per i, multiplicity kept
__global__ void k_cp_count(DemDev d, DemParams p, int32_t* cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    uint32_t B[8];
    buckets8(d.cellinfo[i], p, B);
    const uint32_t lim = d.ctr->cell_limit;
    int c = 0;
    for (int t = 0; t < 8; ++t) {
        uint32_t s, e;
        bucket_range(d, B[t], lim, &s, &e);
        for (uint32_t q = s; q < e; ++q) c += (int)d.sorted[q] > i ? 1 : 0;
    }
    cnt[i] = c;
}
// update_cp_list! (src/kernels.jl:39-58)
__global__ void k_cp_fill(DemDev d, DemParams p, const int32_t* off, int32_t* cp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    uint32_t B[8];
    buckets8(d.cellinfo[i], p, B);
    const uint32_t lim = d.ctr->cell_limit;
    int o = off[i];
    for (int t = 0; t < 8; ++t) {
        uint32_t s, e;
        bucket_range(d, B[t], lim, &s, &e);
        for (uint32_t q = s; q < e; ++q) {
            const int j = (int)d.sorted[q];
            if (j > i) {
                cp[2 * o] = i;
                cp[2 * o + 1] = j;
                ++o;
            }
        }
    }
}

inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

int scan_tiles(int64_t n) { return (int)((n + kScanTile - 1) / kScanTile); }

void launch_scan_i32(const int32_t* in, int32_t* out, int64_t n, const DemDev& d, cudaStream_t s) {
    const int nt = scan_tiles(n);
    if (nt == 0) {
        cudaMemsetAsync(out, 0, sizeof(int32_t), s);
        return;
    }
    k_scan_excl<int32_t, false><<<nt, kScanBlock, 0, s>>>(in, out, n, nt, d.scan_state, d.ctr);
}

void launch_broadphase(const DemDev& d, const DemParams& p, int ntiles_cells, cudaStream_t s) {
    if (p.n == 0) return;
    const int nb = blocks_for(p.n, kThreads);
    k_hash<<<nb, kThreads, 0, s>>>(d, p);
    k_scan_excl<uint32_t, true><<<ntiles_cells, kScanBlock, 0, s>>>(d.cell_count, d.cell_start,
                                                               (long long)p.H, ntiles_cells,
                                                               d.scan_state, d.ctr);
    k_scatter<<<nb, kThreads, 0, s>>>(d, p);
    k_canon<<<nb, kThreads, 0, s>>>(d, p);
}

void launch_detect(const DemDev& d, const DemParams& p, int cur, bool init, cudaStream_t s) {
    if (p.n == 0) return;
    const int nb = blocks_for((long long)p.n * kLanes, kThreads);
    if (init) k_detect<true><<<nb, kThreads, 0, s>>>(d, p, cur);
    else k_detect<false><<<nb, kThreads, 0, s>>>(d, p, cur);
}

void launch_scan_rows(const DemDev& d, const DemParams& p, int nxt, cudaStream_t s) {
    launch_scan_i32(d.cnt, d.row_ptr[nxt], p.n, d, s);
}

void launch_compact(const DemDev& d, const DemParams& p, int cur, bool init, int grid,
                    cudaStream_t s) {
    if (p.n == 0) return;
    const int nb = min(blocks_for((long long)p.cap + p.n, kThreads), grid);
    if (init) k_compact<true><<<nb, kThreads, 0, s>>>(d, p, cur);
    else k_compact<false><<<nb, kThreads, 0, s>>>(d, p, cur);
}

void launch_force(const DemDev& d, const DemParams& p, int nxt, int grid, cudaStream_t s) {
    if (p.n == 0 || p.cap == 0) return;
    if (p.precision == 1) k_force<float><<<grid, kThreads, 0, s>>>(d, p, nxt);
    else k_force<double><<<grid, kThreads, 0, s>>>(d, p, nxt);
}

void launch_integrate(const DemDev& d, const DemParams& p, int nxt, cudaStream_t s) {
    if (p.n == 0) return;
    k_integrate<<<blocks_for(p.n, kThreads), kThreads, 0, s>>>(d, p, nxt);
}

void launch_cplist_count(const DemDev& d, const DemParams& p, int32_t* cnt, cudaStream_t s) {
    if (p.n == 0) return;
    k_cp_count<<<blocks_for(p.n, kThreads), kThreads, 0, s>>>(d, p, cnt);
}
void launch_cplist_fill(const DemDev& d, const DemParams& p, const int32_t* off, int32_t* cp,
                        cudaStream_t s) {
    if (p.n == 0) return;
    k_cp_fill<<<blocks_for(p.n, kThreads), kThreads, 0, s>>>(d, p, off, cp);
}
void launch_morton(const DemDev& d, const DemParams& p, uint32_t* morton, cudaStream_t s) {
    if (p.n == 0) return;
    k_morton<<<blocks_for(p.n, kThreads), kThreads, 0, s>>>(d, p, morton);
}

}  // namespace dem
