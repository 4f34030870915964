// dem_kernels.cu — the DEM step as hand-written CUDA for sm_103a.
//
// One step (the reference's `simulate!`, src/executor.jl:162-172) is
//   k_search     the contact update, one cooperative launch whose phases
//                are separated by grid barriers (the search phases run only
//                for scenes whose neighbour lists went stale):
//                  hash     cell, Morton bucket, octant; warp-aggregated counts
//                  scan     exclusive scan of the occupied bucket range
//                  scatter  counting-sort scatter (the counts return to zero,
//                           so the table needs no clearing)
//                  canon    ascending index inside each bucket + bucket-sorted
//                           copies of the positions (FP64 and FP32)
//                  detect   cp_list enumeration fused with update_contacts!:
//                           existing contacts decide survival, new touching
//                           pairs are found, neighbour lists are rebuilt
//                  lists    update_contacts! from the neighbour lists for
//                           the scenes that do not search this step (a
//                           single-scene handle runs only this phase then)
//                Both write each particle's next row where its contacts are
//                decided (the rolling-array rebuild: survivors + new contacts
//                sorted by j, placed by warp-aggregated atomics).
//   k_force      resolve_collision! per contact (EBPM or Hertz-Mindlin), and
//                each contact's entry in its partner's incoming list (the
//                integrator's gather)
//   k_integrate  per particle: contact force gather in a fixed order,
//                resolve_wall!, apply_body_force!, update!
// All of it is captured once in a CUDA graph per contact-buffer parity (three
// launches per step).  The standalone broad-phase kernels (k_hash,
// k_scan_excl, k_scatter, k_canon) serve the cp_list inspection entry point.
#include <type_traits>

#include "dem_device.cuh"

namespace dem {
namespace {

constexpr int kThreads = 256;
constexpr int kScanBlock = 1024;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;
constexpr unsigned long long kSpinLimit = 1ull << 24;
constexpr double kPi = 3.141592653589793;  // Julia's π rounded to binary64

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }

// Scene of a particle slot and its record: the kernel-parameter record for a
// single-scene handle, the HBM array for an arena (MULTI).
template <bool MULTI>
__device__ __forceinline__ int slot_scene(const DemDev& d, int i) {
    return MULTI ? d.scene_of[i] : 0;
}
template <bool MULTI>
__device__ __forceinline__ const SceneParams& scene_rec(const DemDev& d, const DemParams& p, int s) {
    if (MULTI) return d.sp[s];
    return p.s0;
}
// Does scene sc run the full pair search this step?  (Its rebuild flag is set,
// or it initialises bonds, or the caller hashes everything.)
__device__ __forceinline__ bool full_search(const DemDev& d, int cur, int sc, int mode, int all) {
    return all || mode == kModeInit || d.sflags[cur][sc] != 0u;
}

// particles placed in the bucket-sorted arrays this step
__device__ __forceinline__ int sorted_count(const DemDev& d) {
    return (int)d.cell_start[d.ctr->cell_limit];
}

// ---------------------------------------------------------------------------
// Exclusive scan, single pass with decoupled look-back.  Every CTA draws a
// ticket from its scan site's counter; a launch draws exactly `ntiles`
// tickets, so tile = ticket mod ntiles and the launch's epoch = ticket div
// ntiles + 1.  Tiles are processed in ticket order, so a tile only waits for
// tiles that are already running; each wait is bounded and raises
// kErrTimeout when the bound is hit.  Tile states carry the epoch, so nothing
// has to be reset between launches.
//   state word: epoch (30 bits) | flag (2 bits: 1 aggregate, 2 inclusive) | value (32 bits)
// out has count+1 entries; out[count] is the total.
// LIMITED: the bucket-count scan covers only [0, bmax] (bmax = largest bucket
// this step, from k_hash); tiles past it exit at once and cell_limit records
// the covered range.
constexpr unsigned long long kEpochMask = (1ull << 30) - 1;
__device__ __forceinline__ unsigned long long scan_word(unsigned long long epoch, unsigned flag,
                                                        unsigned long long v) {
    return ((epoch & kEpochMask) << 34) | ((unsigned long long)flag << 32) | (v & 0xffffffffull);
}

template <typename T, bool LIMITED>
__global__ void __launch_bounds__(kScanBlock)
    k_scan_excl(const T* __restrict__ in, T* __restrict__ out, long long count, int ntiles,
                unsigned long long* state, unsigned long long* tickets, DevCounters* ctr,
                unsigned long long spin_limit) {
    __shared__ unsigned long long s_ticket;
    __shared__ unsigned long long s_warp[kScanBlock / 32];
    dep_begin();
    __shared__ unsigned long long s_prefix;
    if (LIMITED) {
        const long long lim = (long long)ctr->bmax + 1;
        count = lim < count ? lim : count;
    }
    const int ntiles_eff = (int)((count + kScanTile - 1) / kScanTile);
    if (threadIdx.x == 0) s_ticket = atomicAdd(tickets, 1ull);
    __syncthreads();
    const int tile = (int)(s_ticket % (unsigned long long)ntiles);
    const unsigned long long epoch = (s_ticket / (unsigned long long)ntiles + 1ull) & kEpochMask;
    if (tile == 0 && threadIdx.x == 0) {
        if (LIMITED) ctr->cell_limit = (unsigned int)count;
        if (count == 0) out[0] = (T)0;
    }
    if (tile >= ntiles_eff) return;
    const long long base = (long long)tile * kScanTile + (long long)threadIdx.x * kScanItems;
    T v[kScanItems];
    unsigned long long sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const long long idx = base + k;
        v[k] = idx < count ? in[idx] : (T)0;
        sum += (unsigned long long)v[k];
    }
    unsigned long long x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane_id() >= (unsigned)o) x += y;
    }
    const int warp = threadIdx.x >> 5;
    if (lane_id() == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = s_warp[lane_id()];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane_id() >= (unsigned)o) w += y;
        }
        s_warp[lane_id()] = w;
    }
    __syncthreads();
    const unsigned long long agg = s_warp[kScanBlock / 32 - 1];
    const unsigned long long texcl = (warp ? s_warp[warp - 1] : 0ull) + x - sum;
    if (threadIdx.x == 0) {
        cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> me(state[tile]);
        unsigned long long prefix = 0;
        if (tile == 0) {
            me.store(scan_word(epoch, 2u, agg), cuda::memory_order_release);
        } else {
            me.store(scan_word(epoch, 1u, agg), cuda::memory_order_release);
            for (int q = tile - 1; q >= 0; --q) {
                cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> pr(state[q]);
                unsigned long long st = 0;
                unsigned flag = 0;
                for (unsigned long long it = 0;; ++it) {
                    st = pr.load(cuda::memory_order_acquire);
                    flag = (unsigned)(st >> 32) & 3u;
                    if ((st >> 34) == epoch && flag) break;
                    if (it > spin_limit) {
                        raise_error(ctr, kErrTimeout);
                        flag = 2u;
                        st = 0;
                        break;
                    }
                    __nanosleep(32);
                }
                prefix += st & 0xffffffffull;
                if (flag == 2u) break;
            }
            me.store(scan_word(epoch, 2u, prefix + agg), cuda::memory_order_release);
        }
        s_prefix = prefix;
        if (tile == ntiles_eff - 1) out[count] = (T)(prefix + agg);
    }
    __syncthreads();
    unsigned long long run = s_prefix + texcl;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const long long idx = base + k;
        if (idx < count) out[idx] = (T)run;
        run += (unsigned long long)v[k];
    }
}

// ---------------------------------------------------------------------------
// ceil(num / cell) with num / cell rounded as IEEE division (src/utils.jl:1).
// q = num·(1/cell) is within 2^-51·|q| of the rounded quotient; when no
// integer lies within 2^-49·|q| of q, both have the same ceiling.  Otherwise
// (rare: q must sit within ~10^-15 relative of an integer) the quotient is
// computed by the correctly rounded division.
__device__ __forceinline__ int32_t cell_index(double num, double cell, double inv_cell) {
    const double q = num * inv_cell;
    const double d = fabs(q) * 0x1p-49;
    const double lo = ceil(q - d), hi = ceil(q + d);
    if (lo == hi && lo > -2147483648.0 && lo < 2147483647.0) return (int32_t)lo;
    return ceil_i32(__ddiv_rn(num, cell));
}
// Cell ijk (1-based) and octant bits of a position for a given cell size
// (`cell` and the center comparison of `neighbors`, src/utils.jl:1-16), with
// an FP32 screen.  num = pos - dmin is formed exactly as the
// reference forms it; q' = fl32(num)·fl32(1/cell) lies within 4·2^-24·|q| of
// the exact quotient q = num/cell, and the reference's center
// dmin + (ijk - 1/2)·cell within 2^-51·(|dmin|/cell + |q| + 1) of its exact
// value (in cell units).  When the fraction of q' keeps a distance of
// m = 2^-20·(|q'| + |dmin|/cell + 1) from 0, 1/2 and 1, the exact ceiling and
// the exact octant side follow from q' alone; otherwise (and for NaN or huge
// values, which fail the test) the exact FP64 computation decides.
// One coordinate: the cell index and, with want_side, whether the coordinate
// lies above the cell's centre (*above; not computed otherwise).
__device__ __forceinline__ int cell_component(double x, double dmin, double cell,
                                              double inv_cell, float inv_cell32, float dmin_cells,
                                              bool want_side, bool* above) {
    const double num = __dsub_rn(x, dmin);
    const float q = d2f(num) * inv_cell32;
    const float fl = floorf(q);
    const float frac = q - fl;
    const float m = (fabsf(q) + dmin_cells + 1.0f) * 0x1p-20f;
    if (frac > m && frac < 1.0f - m && fabsf(frac - 0.5f) > m) {
        if (want_side) *above = frac > 0.5f;
        return (int)fl + 1;
    }
    const int ijk = cell_index(num, cell, inv_cell);
    if (want_side) {
        const double ctr = __dadd_rn(dmin, __dmul_rn(__dsub_rn((double)ijk, 0.5), cell));
        *above = x > ctr;
    }
    return ijk;
}
__device__ __forceinline__ int4 cell_of_screened(const double pos[3], const double dmin[3],
                                                 double cell, double inv_cell, float inv_cell32,
                                                 float dmin_cells) {
    int ijk[3];
    int oct = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        bool above = false;
        ijk[c] = cell_component(pos[c], dmin[c], cell, inv_cell, inv_cell32, dmin_cells, true,
                                &above);
        if (above) oct |= 1 << c;
    }
    return make_int4(ijk[0], ijk[1], ijk[2], oct);
}

// `cell`, `hashcode`, `center`, `neighbors` (src/utils.jl:1-16) and
// `count_particles!` (src/kernels.jl:7-13).
template <bool MULTI>
__device__ __forceinline__ void hash_particle(const DemDev& d, const DemParams& p, int cur, int all,
                                              int i, bool& act, uint32_t& b) {
    act = true;
    b = 0;
    const int sc = slot_scene<MULTI>(d, i);
    const int mode = MULTI ? (sc < 0 ? kModeFree : d.sp[sc].mode) : kModeStep;
    if (mode == kModeFree) {
        // free slot: not hashed, and no contact row in the next buffer
        d.bucket[i] = kNoBucket;
        d.row_len[cur ^ 1][i] = 0;
        d.row_start[cur ^ 1][i] = 0;
        d.path[i] = 0;  // kind 0 (free), mode Free
        act = false;
    } else if (!full_search(d, cur, sc, mode, all)) {
        d.bucket[i] = kNoBucket;  // this scene tests its neighbour lists
        d.path[i] = (uint8_t)(2 | (mode << 2));  // kind 2 (list)
        act = false;
    } else {
        d.path[i] = (uint8_t)(1 | (mode << 2));  // kind 1 (full search)
        const SceneParams& S = scene_rec<MULTI>(d, p, sc);
        const double pos[3] = {d.px[i], d.py[i], d.pz[i]};
        int4 ci = cell_of_screened(pos, S.dmin, S.cell, S.inv_cell, S.f_inv_cell, S.f_dmin_cells);
        b = bucket_of(ci.x, ci.y, ci.z, S);
        if (MULTI) ci.w |= sc << 3;
        d.cellinfo[i] = ci;
        d.bucket[i] = b;
        if (MULTI && !S.same_grid)
            d.refcell[i] = cell_of_screened(pos, S.dmin, S.cell_ref, S.inv_cell_ref,
                                            S.f_inv_cell_ref, S.f_dmin_cells_ref);
    }
}
// Bucket counts and the bucket maximum of a warp's hashed particles (every
// lane of the warp calls this); `hashed` (may be null) counts them.
__device__ __forceinline__ void hash_count(const DemDev& d, bool act, uint32_t b,
                                           unsigned int* hashed) {
    const unsigned mask = __ballot_sync(0xffffffffu, act);
    if (act) {
        const unsigned peers = __match_any_sync(mask, b);
        if (lane_id() == (unsigned)(__ffs(peers) - 1)) atomicAdd(&d.cell_count[b], __popc(peers));
        const unsigned wmax = __reduce_max_sync(mask, b);
        if (lane_id() == (unsigned)(__ffs(mask) - 1)) {
            atomicMax(&d.ctr->bmax, wmax);
            if (hashed) atomicAdd(hashed, __popc(mask));
        }
    }
}
template <bool MULTI>
__global__ void __launch_bounds__(kThreads) k_hash(DemDev d, DemParams p, int cur, int all) {
    dep_begin(p.dep == 2);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool act = false;
    uint32_t b = 0;
    if (i < p.n) hash_particle<MULTI>(d, p, cur, all, i, act, b);
    hash_count(d, act, b, nullptr);
}

// `get_particle_id!` (src/kernels.jl:15-22): counting-sort scatter.  The
// atomic decrements bring every count back to zero.
// (every lane of the warp calls scatter_warp; i >= n is inactive)
__device__ __forceinline__ void scatter_warp(const DemDev& d, const DemParams& p, int i) {
    const uint32_t b = i < p.n ? d.bucket[i] : kNoBucket;
    const bool act = b != kNoBucket;
    const unsigned mask = __ballot_sync(0xffffffffu, act);
    if (!act) return;
    const unsigned peers = __match_any_sync(mask, b);
    const int leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if (lane_id() == (unsigned)leader) old = atomicSub(&d.cell_count[b], (uint32_t)__popc(peers));
    old = __shfl_sync(peers, old, leader);
    const uint32_t slot = old - 1u - (uint32_t)__popc(peers & lanemask_lt());
    d.unsorted[d.cell_start[b] + slot] = (uint32_t)i;
}
__global__ void __launch_bounds__(kThreads) k_scatter(DemDev d, DemParams p) {
    dep_begin(p.dep == 2);
    scatter_warp(d, p, blockIdx.x * blockDim.x + threadIdx.x);
}

// Canonical order inside a bucket (ascending particle index) and the sorted
// copies the pair search reads at its own index (positions, the cell record,
// the current contact row), so its first loads do not wait on the particle
// index.  Also clears this step's bucket maximum (all its readers have
// finished).
template <bool MULTI>
__device__ __forceinline__ void canon_slot(const DemDev& d, const DemParams& p, int cur, int k) {
    const uint32_t i = d.unsorted[k];
    const uint32_t b = d.bucket[i];
    const uint32_t s = d.cell_start[b], e = d.cell_start[b + 1];
    uint32_t rank = 0;
    for (uint32_t t = s; t < e; ++t) rank += d.unsorted[t] < i ? 1u : 0u;
    const uint32_t pos = s + rank;
    d.sorted[pos] = i;
    const double x = d.px[i], y = d.py[i], z = d.pz[i], r = d.r[i];
    const SceneParams& S = scene_rec<MULTI>(d, p, slot_scene<MULTI>(d, (int)i));
    d.spos[pos] = make_double4_32a(x, y, z, r);
    const float fx = d2f(x - S.dmin[0]), fy = d2f(y - S.dmin[1]), fz = d2f(z - S.dmin[2]);
    d.spos32[pos] = make_float4(fx, fy, fz, reach32(fx, fy, fz, d2f(r)));
    d.scell[pos] = d.cellinfo[i];
    d.srow[pos] = make_int2(d.row_start[cur][i], d.row_len[cur][i]);
}
template <bool MULTI>
__global__ void __launch_bounds__(kThreads) k_canon(DemDev d, DemParams p, int cur) {
    dep_begin(p.dep == 2);
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) d.ctr->bmax = 0u;
    if (k >= sorted_count(d)) return;
    canon_slot<MULTI>(d, p, cur, k);
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
//  * new contact: touching and not in row i.  Row membership (from a shared
//    memory copy of row i) is checked before the FP64 distance test, so
//    bonded neighbours cost no FP64 work.
constexpr int kLanes = 8;
constexpr int kRowCache = 24;
constexpr int kBatch = 4;
__device__ __forceinline__ void bucket_range(const DemDev& d, uint32_t b, uint32_t lim,
                                             uint32_t* s, uint32_t* e) {
    if (b < lim) {
        *s = d.cell_start[b];
        *e = d.cell_start[b + 1];
    } else {
        *s = *e = 0u;
    }
}

// ---- next-buffer rows -------------------------------------------------------
// The rolling-array rebuild (the reference's remove_inactive_contact! + swap,
// src/kernels.jl:487-506, src/executor.jl:140-153) happens where a
// particle's contacts are decided: row i of buffer cur^1 is the merge, by j,
// of the surviving entries of row i (keep flags) and the sorted new partners.
// A row is placed by a warp-aggregated atomic on the buffer's allocator.

// One particle's decided row, held by every lane of its group.
struct RowJob {
    int i, mode;  // particle; its scene's mode (Step, Init or Frozen)
    int e0, e1;   // current row entries [e0, e1)
    int nnew;     // new partners (sorted, in the particle's stash)
    int len;      // next row length (survivors + new), 0 for no row
    int nb;       // bonds among them
};

// Places the rows of a warp's groups (L lanes each) in buffer nxt: every lane
// of the warp calls it with its group's (group-uniform) `len` and bond count
// `nb`; returns the group's row start and, in *bstart, the start of its bonds
// in the type-ordered list (its other contacts start at start - *bstart: the
// bonds placed before a row never outnumber the contacts placed before it,
// so both ranges lie inside [0, start + len)).  A row that would cross the
// capacity raises kErrCapacity and gets length 0.
template <int L>
__device__ __forceinline__ int place_rows(const DemDev& d, const DemParams& p, int nxt, int& len,
                                          int nb, int* bstart) {
    const unsigned lane = lane_id();
    const bool lead = lane % L == 0;
    const unsigned v = lead ? (unsigned)len : 0u, vb = lead ? (unsigned)nb : 0u;
    unsigned incl = v, inclb = vb;
#pragma unroll
    for (int o2 = 1; o2 < 32; o2 <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, o2);
        const unsigned yb = __shfl_up_sync(0xffffffffu, inclb, o2);
        if (lane >= (unsigned)o2) {
            incl += y;
            inclb += yb;
        }
    }
    // rows in the low word, bonds in the high word: the rows placed in a
    // step number at most the capacity plus kstash per particle, far below
    // 2^32, so the low word never carries
    unsigned long long base = 0ull;
    if (lane == 31 && incl)
        base = atomicAdd(reinterpret_cast<unsigned long long*>(&d.ctr->alloc[nxt]),
                         (unsigned long long)incl | ((unsigned long long)inclb << 32));
    base = __shfl_sync(0xffffffffu, base, 31);
    const int src = (int)(lane & ~(unsigned)(L - 1));
    const unsigned excl = __shfl_sync(0xffffffffu, incl - v, src);
    const unsigned exclb = __shfl_sync(0xffffffffu, inclb - vb, src);
    int start = (int)((unsigned)base + excl);
    *bstart = (int)((unsigned)(base >> 32) + exclb);
    if (len > 0 && (long long)start + len > (long long)p.cap) {
        if (lane % L == 0) raise_error(d.ctr, kErrCapacity);
        start = 0;
        len = 0;
    }
    return start;
}

__device__ __forceinline__ void add_incoming_entry(const DemDev& d, const DemParams& p, int j,
                                                   int pos, int i) {
    const int slot = atomicAdd(&d.in_cnt[j], 1);
    if (slot < p.kin) d.in_list[(size_t)j * p.kin + slot] = make_int2(pos, i);
    else raise_error(d.ctr, kErrCapacity);
}

// Writes the row of job `r` at [start, start + r.len) of buffer cur^1 (L
// lanes share it).  A stepping contact is
// written as its ids, flags and `src`, its slot in buffer cur: the force pass
// reads the carried state there (a bond's accumulated 𝐅, 𝛕ᵢ, 𝛕ⱼ, a Hertz
// contact's 𝐬) and writes the new state here, so the state is not copied
// (a bond's 𝐬 and a Hertz contact's torques are zero, reported as such by
// the host).  Contacts of scenes that do not step keep every field.
template <int L>
__device__ __forceinline__ void finish_row(const DemDev& d, const DemParams& p, int cur,
                                           const RowJob& r, int start, int bstart, int lane) {
    const ContactSoA o = d.c[cur];
    const ContactSoA w = d.c[cur ^ 1];
    const int32_t* st = d.stash + (size_t)r.i * p.kstash;
    const bool stepping = r.mode == kModeStep;
    const bool init = r.mode == kModeInit;  // new contacts are bonds
    const int hstart = start - bstart;
    const long long last = (long long)p.cap - 1;
    // the contact at row position pos, with nbb bonds before it in the row,
    // in the type-ordered list
    auto list_entry = [&](int pos, int nbb, bool bonded) {
        const long long k = bonded ? (long long)bstart + nbb
                                   : (long long)last - (hstart + (pos - start) - nbb);
        if (k >= 0 && k < (long long)p.cap) d.tlist[k] = pos;
    };
    for (int e = r.e0 + lane; e < r.e1; e += L) {
        if (!d.keep[e]) continue;
        const int j = o.cj[e];
        const uint32_t fl = o.fl[e];
        int pos = start, nbb = 0;
        for (int q = r.e0; q < e; ++q) {
            pos += d.keep[q];
            nbb += (d.keep[q] && (o.fl[q] & kBonded)) ? 1 : 0;
        }
        for (int u = 0; u < r.nnew; ++u) {
            const int before = st[u] < j ? 1 : 0;
            pos += before;
            if (init) nbb += before;
        }
        w.ci[pos] = r.i;
        w.cj[pos] = j;
        w.fl[pos] = fl;
        w.src[pos] = stepping ? e : -1;
        if (!stepping)
            for (int f = 0; f < 15; ++f) w.f[f][pos] = o.f[f][e];
        list_entry(pos, nbb, (fl & kBonded) != 0u);
    }
    for (int u = lane; u < r.nnew; u += L) {
        const int j = st[u];
        int pos = start + u, nbb = init ? u : 0;
        for (int q = r.e0; q < r.e1; ++q) {
            const bool before = d.keep[q] && o.cj[q] < j;
            pos += before ? 1 : 0;
            nbb += (before && (o.fl[q] & kBonded)) ? 1 : 0;
        }
        w.ci[pos] = r.i;
        w.cj[pos] = j;
        w.fl[pos] = init ? (kActive | kBonded) : kActive;
        w.src[pos] = -1;  // a new contact: zero carried state
        if (!stepping) {
#pragma unroll
            for (int f = 0; f < 15; ++f) w.f[f][pos] = 0.0;
        }
        list_entry(pos, nbb, init);
    }
}

// Places and writes the rows of a warp's groups: every lane of the warp
// calls it; `active` groups carry a decided job.
template <int L>
__device__ __forceinline__ void emit_rows(const DemDev& d, const DemParams& p, int cur, bool active,
                                          const RowJob& r, int lane) {
    int len = active ? r.len : 0, bstart = 0;
    const int start = place_rows<L>(d, p, cur ^ 1, len, active ? r.nb : 0, &bstart);
    if (!active) return;
    if (lane == 0) {
        d.row_start[cur ^ 1][r.i] = start;
        d.row_len[cur ^ 1][r.i] = len;
    }
    if (len > 0) finish_row<L>(d, p, cur, r, start, bstart, lane);
}

// Checksum term of a candidate pair (i, j) for the inspection of the pair
// search (a 64-bit finaliser of i·2^32 + j; summed with wrap-around).
__device__ __forceinline__ unsigned long long enum_mix(int i, int j) {
    unsigned long long z = ((unsigned long long)(unsigned)i << 32) | (unsigned)j;
    z ^= z >> 33;
    z *= 0xff51afd7ed558ccdull;
    z ^= z >> 33;
    z *= 0xc4ceb9fe1a85ec53ull;
    return z ^ (z >> 33);
}

// Shared memory of one 8-lane group of the pair search (k_search's detect phase).
struct DetectShared {
    int nnew;
    int nvl;                  // neighbour-list entries found
    int row[kRowCache];       // cached current row (partner or -1)
    uint32_t rb[kLanes];      // the reference's 8 octant buckets
    int2 seg[kLanes];         // (first sorted slot, prefix) per bucket
};

// The full pair search for the particle at sorted position k (one 8-lane group);
// lim = the buckets with valid starts this step.
template <bool INIT, bool MULTI>
__device__ __forceinline__ void detect_group(const DemDev& d, const DemParams& p, int cur, int k,
                                             int lane, unsigned gmask, uint32_t lim,
                                             DetectShared& sh, RowJob& job) {
    const int nxt = cur ^ 1;
    if (lane == 0) {
        sh.nnew = 0;
        sh.nvl = 0;
    }
    const int i = (int)d.sorted[k];
    const int4 ci = d.scell[k];
    const float4 P32 = d.spos32[k];
    const int2 row = d.srow[k];
    const int sc = MULTI ? (ci.w >> 3) : 0;
    const SceneParams& S = scene_rec<MULTI>(d, p, sc);
    const bool init = INIT || (MULTI && S.mode == kModeInit);
    const bool frozen = MULTI && S.mode == kModeFrozen;
    const int dx = (ci.w & 1) ? 1 : -1, dy = (ci.w & 2) ? 1 : -1, dz = (ci.w & 4) ? 1 : -1;
    const int ox = (lane == 1 || lane == 4 || lane == 5 || lane == 7) ? dx : 0;
    const int oy = (lane == 2 || lane == 4 || lane == 6 || lane == 7) ? dy : 0;
    const int oz = (lane == 3 || lane == 5 || lane == 6 || lane == 7) ? dz : 0;
    const uint32_t myB = bucket_of(ci.x + ox, ci.y + oy, ci.z + oz, S);
    // the reference's buckets decide cp_list membership (equal to the search
    // buckets for a single-scene handle)
    uint32_t myR = myB;
    if (MULTI) {
        const int4 rc = S.same_grid ? ci : d.refcell[i];
        const int rx = (rc.w & 1) ? 1 : -1, ry = (rc.w & 2) ? 1 : -1, rz = (rc.w & 4) ? 1 : -1;
        myR = ref_bucket_of(rc.x + (ox ? rx : 0), rc.y + (oy ? ry : 0), rc.z + (oz ? rz : 0), S);
    }
    bool dup = false;
#pragma unroll
    for (int u = 0; u < 7; ++u) {
        const uint32_t bu = __shfl_sync(gmask, myB, u, kLanes);  // every lane of the group
        dup |= (u < lane) && (bu == myB);
    }
    uint32_t s, e;
    bucket_range(d, myB, lim, &s, &e);
    if (dup || frozen) e = s;
    // a bucket lists its particles by ascending index: keep those above i
    // (cp_list holds the pairs i < j)
    {
        uint32_t lo = s, hi = e;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if ((int)d.sorted[mid] > i) hi = mid;
            else lo = mid + 1;
        }
        s = lo;
    }
    // the group's candidates: the concatenation of its 8 bucket ranges
    const int cnt = (int)(e - s);
    int incl = cnt;
#pragma unroll
    for (int o2 = 1; o2 < kLanes; o2 <<= 1) {
        const int y = __shfl_up_sync(gmask, incl, o2, kLanes);
        if (lane >= o2) incl += y;
    }
    const int total = __shfl_sync(gmask, incl, kLanes - 1, kLanes);
    sh.rb[lane] = myR;
    sh.seg[lane] = make_int2((int)s, incl - cnt);
    __syncwarp(gmask);

    // existing row: survival (update_contacts!, src/kernels.jl:87-101)
    const ContactSoA o = d.c[cur];
    const int e0 = row.x;
    const int e1 = e0 + row.y;
    const bool cached = e1 - e0 <= kRowCache;
    int nkeep = 0, ended = 0, nbond = 0;
    for (int e2 = e0 + lane; e2 < e1; e2 += kLanes) {
        const uint32_t fl = o.fl[e2];
        const int j = o.cj[e2];
        if (cached) sh.row[e2 - e0] = (fl & kActive) ? j : -1;
        int keep;
        if (!(fl & kActive)) {
            keep = 0;
        } else if (init || frozen || (fl & kBonded)) {
            keep = 1;
        } else {
            // FP64 position of i reloaded where needed (keeps registers free)
            const double4_32a P = d.spos[k];
            const bool valid = touching_rn(P.x, P.y, P.z, d.px[j], d.py[j], d.pz[j], P.w, d.r[j]);
            uint32_t bj;
            if (MULTI) {
                const int4 cj4 = S.same_grid ? d.cellinfo[j] : d.refcell[j];
                bj = ref_bucket_of(cj4.x, cj4.y, cj4.z, S);
            } else {
                bj = d.bucket[j];
            }
            bool in_cp = false;
#pragma unroll
            for (int t = 0; t < 8; ++t) in_cp |= (sh.rb[t] == bj);
            keep = (valid || !in_cp) ? 1 : 0;
            ended += 1 - keep;
        }
        d.keep[e2] = (uint8_t)keep;
        nkeep += keep;
        nbond += (keep && (fl & kBonded)) ? 1 : 0;
    }
    nkeep = __reduce_add_sync(gmask, nkeep);
    nbond = __reduce_add_sync(gmask, nbond);
    ended = __reduce_add_sync(gmask, ended);
    __syncwarp(gmask);

    // new contacts: lane t takes candidates t, t+8, ... of the concatenation,
    // so the group's lanes share the work evenly and read consecutive slots
    int32_t* stash = d.stash + (size_t)i * p.kstash;
    // current segment: its offset (first slot - prefix) and the next prefix
    int seg = 0, segoff = sh.seg[0].x, nextb = sh.seg[1].y;
    // the neighbour list is rebuilt with this search (not for held scenes)
    const bool build = !frozen;
    int32_t* vl = d.vl + (size_t)i * p.kvl;
    const float skin = S.f_skin;
    unsigned long long en = 0, eh = 0;  // inspection: pairs visited, their checksum
    for (int c0 = 0; c0 < total; c0 += kLanes * kBatch) {
        int jj[kBatch], qi[kBatch];
        float4 qq[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
            const int c = c0 + u * kLanes + lane;
            jj[u] = -1;
            qi[u] = 0;
            qq[u] = P32;
            if (c < total) {
                while (nextb <= c) {  // nextb of the last segment is total, > c
                    ++seg;
                    const int2 sg = sh.seg[seg];
                    segoff = sg.x - sg.y;
                    nextb = seg + 1 < kLanes ? sh.seg[seg + 1].y : total;
                }
                const int q = segoff + c;
                qi[u] = q;
                jj[u] = (int)d.sorted[q];
                qq[u] = d.spos32[q];
            }
        }
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
            const int j = jj[u];
            if (j <= i) continue;
            if (p.debug_enum) {
                ++en;
                eh += enum_mix(i, j);
            }
            // partners within rᵢ + rⱼ + skin join the neighbour list
            const bool near = maybe_touching32(P32, qq[u], skin);
            if (build && near) {
                const int vs = atomicAdd(&sh.nvl, 1);
                if (vs < p.kvl) vl[vs] = j;
            }
            // bond initialisation tests r₀ (no FP32 pre-filter); otherwise a
            // touching pair is near and passes the pre-filter
            if (!init && (!near || !maybe_touching32(P32, qq[u]))) continue;
            bool found = false;
            if (cached) {
                for (int t = 0; t < e1 - e0 && !found; ++t) found = sh.row[t] == j;
            } else {
                for (int e2 = e0; e2 < e1 && !found; ++e2)
                    found = (o.cj[e2] == j) && (o.fl[e2] & kActive);
            }
            if (found) continue;
            const double4_32a P = d.spos[k];
            const double4_32a Q = d.spos[qi[u]];
            const double ri = init ? d.r0[i] : P.w;
            const double rj = init ? d.r0[j] : Q.w;
            if (!touching_rn(P.x, P.y, P.z, Q.x, Q.y, Q.z, ri, rj)) continue;
            const int slot = atomicAdd(&sh.nnew, 1);
            if (slot < p.kstash) stash[slot] = j;
        }
    }
    if (p.debug_enum) {
        en = __reduce_add_sync(gmask, (unsigned)en);
#pragma unroll
        for (int o2 = kLanes / 2; o2 > 0; o2 >>= 1) eh += __shfl_xor_sync(gmask, eh, o2, kLanes);
        if (lane == 0) {
            atomicAdd(&d.ctr->enum_pairs, en);
            atomicAdd(&d.ctr->enum_hash, eh);
        }
    }
    __syncwarp(gmask);
    if (lane == 0) {
        if (build) {
            const int nv = sh.nvl;
            d.vl_len[i] = nv < p.kvl ? nv : p.kvl;
            d.xref[i] = P32;
            if (nv > p.kvl) atomicOr(&d.sflags[nxt][sc], 1u);  // list overflow: search again
        }
        int nnew = sh.nnew;
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
        sh.nnew = nnew;
        if (ended) atomicAdd(&d.sctr[sc].ended, (unsigned long long)ended);
        if (!init && nnew) atomicAdd(&d.sctr[sc].created, (unsigned long long)nnew);
    }
    __syncwarp(gmask);
    job.i = i;
    job.mode = init ? kModeInit : (frozen ? kModeFrozen : kModeStep);
    job.e0 = e0;
    job.e1 = e1;
    job.nnew = sh.nnew;
    job.len = nkeep + job.nnew;
    job.nb = nbond + (init ? job.nnew : 0);  // init_bonds!: every new contact is a bond
}

// cp_list membership of the pair (i, j), i < j, from the current positions:
// j's bucket among i's 8 octant buckets, in the reference's cells and table.
// Inlined: as a call it made the list kernels save and restore live registers
// around it (twice the spill traffic), and a warp whose particle had a contact
// to end waited about 16,000 cycles longer in its row loop (the 17,576-sphere
// cube: 53.8 -> 53.2 us per step; the 2,000,000-sphere bed 506 -> 497 us).
template <bool MULTI>
__device__ __forceinline__ bool in_cp_list(const DemDev& d, const SceneParams& S, int i, int j) {
    const double pi[3] = {d.px[i], d.py[i], d.pz[i]}, pj[3] = {d.px[j], d.py[j], d.pz[j]};
    const int4 ci = cell_of_screened(pi, S.dmin, S.cell_ref, S.inv_cell_ref, S.f_inv_cell_ref,
                                     S.f_dmin_cells_ref);
    const int4 cj = cell_of_screened(pj, S.dmin, S.cell_ref, S.inv_cell_ref, S.f_inv_cell_ref,
                                     S.f_dmin_cells_ref);
    const uint32_t bj = ref_bucket_of(cj.x, cj.y, cj.z, S);
    const int dx = (ci.w & 1) ? 1 : -1, dy = (ci.w & 2) ? 1 : -1, dz = (ci.w & 4) ? 1 : -1;
    bool in = false;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        const int ox = (t == 1 || t == 4 || t == 5 || t == 7) ? dx : 0;
        const int oy = (t == 2 || t == 4 || t == 6 || t == 7) ? dy : 0;
        const int oz = (t == 3 || t == 5 || t == 6 || t == 7) ? dz : 0;
        in |= ref_bucket_of(ci.x + ox, ci.y + oy, ci.z + oz, S) == bj;
    }
    return in;
}

// The same test with a particle's four lanes sharing it (every lane of the
// group calls it with the same i, j): lanes 0, 1, 2 compute one axis each of
// i's cell and side and of j's cell (j's side is not needed), so that the
// exact FP64 fallbacks of lattice-aligned coordinates run side by side
// instead of one after another on one lane.  The cells and sides are
// exchanged by shuffles and every lane returns the result.
__device__ __forceinline__ bool in_cp_list_group(const DemDev& d, const SceneParams& S, int i,
                                                 int j, int lane, unsigned gmask) {
    const int c = lane < 3 ? lane : 2;
    const double* P = c == 0 ? d.px : (c == 1 ? d.py : d.pz);
    bool above = false;
    const int ci = cell_component(P[i], S.dmin[c], S.cell_ref, S.inv_cell_ref, S.f_inv_cell_ref,
                                  S.f_dmin_cells_ref, true, &above);
    const int cj = cell_component(P[j], S.dmin[c], S.cell_ref, S.inv_cell_ref, S.f_inv_cell_ref,
                                  S.f_dmin_cells_ref, false, nullptr);
    const int base = (int)(lane_id() & ~3u);
    int CI[3], CJ[3], oct = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        CI[k] = __shfl_sync(gmask, ci, base + k);
        CJ[k] = __shfl_sync(gmask, cj, base + k);
        oct |= (__shfl_sync(gmask, above ? 1 : 0, base + k)) << k;
    }
    const uint32_t bj = ref_bucket_of(CJ[0], CJ[1], CJ[2], S);
    const int dx = (oct & 1) ? 1 : -1, dy = (oct & 2) ? 1 : -1, dz = (oct & 4) ? 1 : -1;
    bool in = false;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        const int ox = (t == 1 || t == 4 || t == 5 || t == 7) ? dx : 0;
        const int oy = (t == 2 || t == 4 || t == 6 || t == 7) ? dy : 0;
        const int oz = (t == 3 || t == 5 || t == 6 || t == 7) ? dz : 0;
        in |= ref_bucket_of(CI[0] + ox, CI[1] + oy, CI[2] + oz, S) == bj;
    }
    return in;
}

// `update_contacts!` from the neighbour lists, for the particles of scenes
// that do not run the full search this step (four lanes per particle,
// grid-stride over slots).  Survival of the current row is decided as in
// the full search; new contacts are the touching list partners that are not in the
// row.
constexpr int kVLanes = 4;
struct ListShared {
    int nnew;
    int row[kRowCache];
};
// The list update over slots [0, n), grid-stride (every thread of the launch
// calls it; a warp's groups move together).
// The list update of one particle whose row or list is not empty (one
// 4-lane group; `g` its ListShared slot): survival of the current row,
// the list partners' touching tests, the new partners in ascending order;
// fills `job` with the next row.
template <bool MULTI>
__device__ __forceinline__ void list_particle(const DemDev& d, const DemParams& p, int cur,
                                              ListShared* sh, int g, int lane, unsigned gmask,
                                              int i, int e0, int e1, int nv, bool frozen,
                                              RowJob& job) {
    const ContactSoA o = d.c[cur];
    if (lane == 0) sh[g].nnew = 0;
    const bool cached = e1 - e0 <= kRowCache;
    int nkeep = 0, ended = 0, nbond = 0;
    // a Hertz contact that no longer touches ends iff the pair is in the
    // cp_list: those entries wait (one bit per loop iteration of this lane)
    // for the group's shared membership test below
    unsigned pend = 0u;
    int it = 0;
    for (int e2 = e0 + lane; e2 < e1; e2 += kVLanes, ++it) {
        const uint32_t fl = o.fl[e2];
        const int j = o.cj[e2];
        if (cached) sh[g].row[e2 - e0] = (fl & kActive) ? j : -1;
        int keep;
        if (!(fl & kActive)) {
            keep = 0;
        } else if (frozen || (fl & kBonded)) {
            keep = 1;
        } else {
            const bool valid = touching_rn(d.px[i], d.py[i], d.pz[i], d.px[j], d.py[j],
                                           d.pz[j], d.r[i], d.r[j]);
            if (valid) {
                keep = 1;
            } else if (it < 32) {
                pend |= 1u << it;
                continue;
            } else {
                keep = in_cp_list<MULTI>(d, scene_rec<MULTI>(d, p, slot_scene<MULTI>(d, i)), i, j)
                           ? 0
                           : 1;
                ended += 1 - keep;
            }
        }
        d.keep[e2] = (uint8_t)keep;
        nkeep += keep;
        nbond += (keep && (fl & kBonded)) ? 1 : 0;
    }
    for (unsigned any = __ballot_sync(gmask, pend != 0u) & gmask; any;
         any = __ballot_sync(gmask, pend != 0u) & gmask) {
        const int src = __ffs(any) - 1;  // a lane of this group with a waiting entry
        const int sit = __ffs(__shfl_sync(gmask, pend, src)) - 1;
        const int e2 = e0 + (src & (kVLanes - 1)) + sit * kVLanes;
        const bool in = in_cp_list_group(d, scene_rec<MULTI>(d, p, slot_scene<MULTI>(d, i)), i,
                                         o.cj[e2], lane, gmask);
        if (lane == (src & (kVLanes - 1))) {
            pend &= ~(1u << sit);
            const int keep = in ? 0 : 1;
            d.keep[e2] = (uint8_t)keep;
            nkeep += keep;
            ended += 1 - keep;
        }
    }
    nkeep = __reduce_add_sync(gmask, nkeep);
    nbond = __reduce_add_sync(gmask, nbond);
    ended = __reduce_add_sync(gmask, ended);
    __syncwarp(gmask);
    int32_t* stash = d.stash + (size_t)i * p.kstash;
    if (!frozen) {
        const float4 Pi = d.pos32[i];
        const int32_t* vl = d.vl + (size_t)i * p.kvl;
        for (int v = lane; v < nv; v += kVLanes) {
            const int j = vl[v];
            // a partner already in the row (a bond, a Hertz contact)
            // needs no position: the row is checked first
            bool found = false;
            if (cached) {
                for (int t = 0; t < e1 - e0 && !found; ++t) found = sh[g].row[t] == j;
            } else {
                for (int e2 = e0; e2 < e1 && !found; ++e2)
                    found = (o.cj[e2] == j) && (o.fl[e2] & kActive);
            }
            if (found) continue;
            const float4 Pj = d.pos32[j];
            if (!maybe_touching32(Pi, Pj)) continue;
            if (!touching_rn(d.px[i], d.py[i], d.pz[i], d.px[j], d.py[j], d.pz[j], d.r[i],
                             d.r[j]))
                continue;
            const int slot = atomicAdd(&sh[g].nnew, 1);
            if (slot < p.kstash) stash[slot] = j;
        }
    }
    __syncwarp(gmask);
    if (lane == 0) {
        int nnew = sh[g].nnew;
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
        sh[g].nnew = nnew;
        if (ended || nnew) {
            const int sc = slot_scene<MULTI>(d, i);
            if (ended) atomicAdd(&d.sctr[sc].ended, (unsigned long long)ended);
            if (nnew) atomicAdd(&d.sctr[sc].created, (unsigned long long)nnew);
        }
    }
    __syncwarp(gmask);
    job.i = i;
    job.mode = frozen ? kModeFrozen : kModeStep;
    job.e0 = e0;
    job.e1 = e1;
    job.nnew = sh[g].nnew;
    job.len = nkeep + job.nnew;
    job.nb = nbond;
}

// The list update of one particle by one lane (the narrow layout): the same
// decisions as list_particle, with the row and the list walked by the lane
// itself (no shared row cache: a row's few entries are re-read from L1).
// Clearly touching pairs are accepted by an FP32 screen before the exact
// FP64 test (surely_touching32).  (The four-lane path keeps the FP64 test
// alone: on the 17,576-sphere cube the screen made its contact update 1.8 us
// faster and the force pass 2.8 us slower, because the FP64 position loads it
// saves were warming L2 for the force pass.)
template <bool MULTI>
__device__ __forceinline__ void list_particle1(const DemDev& d, const DemParams& p, int cur, int i,
                                               int e0, int e1, int nv, bool frozen, RowJob& job) {
    const ContactSoA o = d.c[cur];
    int nkeep = 0, ended = 0, nbond = 0;
    for (int e = e0; e < e1; ++e) {
        const uint32_t fl = o.fl[e];
        int keep;
        if (!(fl & kActive)) {
            keep = 0;
        } else if (frozen || (fl & kBonded)) {
            keep = 1;
        } else {
            const int j = o.cj[e];
            const bool valid =
                surely_touching32(d.pos32[i], d.rm32[i].z, d.pos32[j], d.rm32[j].z) ||
                touching_rn(d.px[i], d.py[i], d.pz[i], d.px[j], d.py[j], d.pz[j], d.r[i],
                            d.r[j]);
            keep = (valid ||
                    !in_cp_list<MULTI>(d, scene_rec<MULTI>(d, p, slot_scene<MULTI>(d, i)), i, j))
                       ? 1
                       : 0;
            ended += 1 - keep;
        }
        d.keep[e] = (uint8_t)keep;
        nkeep += keep;
        nbond += (keep && (fl & kBonded)) ? 1 : 0;
    }
    int32_t* stash = d.stash + (size_t)i * p.kstash;
    int nnew = 0;
    if (!frozen) {
        const float4 Pi = d.pos32[i];
        const int32_t* vl = d.vl + (size_t)i * p.kvl;
        for (int v = 0; v < nv; ++v) {
            const int j = vl[v];
            bool found = false;
            for (int e = e0; e < e1 && !found; ++e)
                found = (o.cj[e] == j) && (o.fl[e] & kActive);
            if (found) continue;
            const float4 Pj = d.pos32[j];
            if (!maybe_touching32(Pi, Pj)) continue;
            if (!surely_touching32(Pi, d.rm32[i].z, Pj, d.rm32[j].z) &&
                !touching_rn(d.px[i], d.py[i], d.pz[i], d.px[j], d.py[j], d.pz[j], d.r[i],
                             d.r[j]))
                continue;
            if (nnew < p.kstash) stash[nnew] = j;
            ++nnew;
        }
    }
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
    if (ended || nnew) {
        const int sc = slot_scene<MULTI>(d, i);
        if (ended) atomicAdd(&d.sctr[sc].ended, (unsigned long long)ended);
        if (nnew) atomicAdd(&d.sctr[sc].created, (unsigned long long)nnew);
    }
    job.i = i;
    job.mode = frozen ? kModeFrozen : kModeStep;
    job.e0 = e0;
    job.e1 = e1;
    job.nnew = nnew;
    job.len = nkeep + nnew;
    job.nb = nbond;
}

// The neighbour-list update with one lane per particle: in large scenes with
// few contacts and list partners per particle (a compacted bed, a pour) four
// lanes per particle leave most lanes idle and too few particles in flight
// to cover the chain of dependent loads; one lane per particle puts four
// times as many particles in flight.  A warp's rows are placed together
// (one atomic per warp).
// Warps take 32 consecutive particles in turn across the blocks (warp w of
// block b is the grid's warp w·gridDim + b): a cooperative launch places
// consecutive blocks on the same SM, so chunks by block would leave SMs idle
// whenever the particles do not fill the grid.
template <bool MULTI>
__device__ __forceinline__ void list_phase_narrow(const DemDev& d, const DemParams& p, int cur) {
    const int wslot = (int)(threadIdx.x >> 5) * (int)gridDim.x + (int)blockIdx.x;
    for (long long t0 = 0; t0 < p.n; t0 += (long long)gridDim.x * kThreads) {
        const int i0 = (int)(t0 + 32LL * wslot);
        const int i = i0 + (int)lane_id();
        bool act = i < p.n, frz = false;
        if (MULTI && act) {
            const uint8_t path = d.path[i];
            act = (path & 3) == 2;
            frz = (path >> 2) == kModeFrozen;
        }
        RowJob job{};
        if (act) {
            const int e0 = d.row_start[cur][i];
            const int e1 = e0 + d.row_len[cur][i];
            const int nv = frz ? 0 : d.vl_len[i];
            if (e1 == e0 && nv == 0) {  // no contact and no list partner: an empty row
                d.row_start[cur ^ 1][i] = 0;
                d.row_len[cur ^ 1][i] = 0;
                act = false;
            } else {
                list_particle1<MULTI>(d, p, cur, i, e0, e1, nv, frz, job);
            }
        }
        emit_rows<1>(d, p, cur, act, job, 0);
    }
}

// The neighbour-list update (a12, a13, a21 for scenes whose lists are valid):
// 4 lanes per particle.  A particle with no contact and no list partner gets
// an empty next row at once.  When the particles outnumber one pass of the
// grid's 4-lane groups and the contacts are sparse (fewer than one per four
// particles, as in a settling pour), each warp first reads 32 particles one
// lane each, writes the empty rows, and passes only the others to its groups,
// 8 at a time: a pass then costs one memory round trip per 32 particles
// instead of per 8 (2,000,000-sphere pour: 0.081 -> 0.054 ms).  With denser
// contacts the per-group layout is kept: measured on the mixed batch, the
// wide pass made the contact update and the force pass slower (0.633 vs
// 0.581 ms per step).
template <bool MULTI>
__device__ __forceinline__ void list_phase(const DemDev& d, const DemParams& p, int cur,
                                           ListShared* sh) {
    // one lane per particle when chosen, or by default when the particles
    // outnumber half the launch's threads
    if (p.list_lanes == 1 ||
        (p.list_lanes == 0 && 2LL * p.n > (long long)gridDim.x * kThreads)) {
        list_phase_narrow<MULTI>(d, p, cur);
        return;
    }
    const int lane = threadIdx.x & (kVLanes - 1);
    const int g = threadIdx.x / kVLanes;
    const unsigned gmask = 0xfu << (lane_id() & ~3u);
    // a warp's eight groups move together (their rows are placed per warp)
    const int gwarp = (int)(threadIdx.x >> 5) * (32 / kVLanes);
    // contacts in the current buffer: fixed while this kernel runs (rows are
    // placed in the other buffer), so every thread takes the same branch
    const long long ncur = (long long)__ldcg(&d.ctr->alloc[cur].rows);
    if (p.n > gridDim.x * (kThreads / kVLanes) && 4 * ncur < (long long)p.n) {
        const int gw = g - gwarp;  // the group within the warp, 0..7
        for (int base = blockIdx.x * kThreads + (int)(threadIdx.x & ~31u); base < p.n;
             base += gridDim.x * kThreads) {
            const int ip = base + (int)lane_id();
            bool act = ip < p.n, frz = false;
            if (MULTI && act) {
                const uint8_t path = d.path[ip];
                act = (path & 3) == 2;
                frz = (path >> 2) == kModeFrozen;
            }
            int e0 = 0, e1 = 0, nv = 0;
            if (act) {
                e0 = d.row_start[cur][ip];
                e1 = e0 + d.row_len[cur][ip];
                nv = frz ? 0 : d.vl_len[ip];
                if (e1 == e0 && nv == 0) {
                    d.row_start[cur ^ 1][ip] = 0;
                    d.row_len[cur ^ 1][ip] = 0;
                    act = false;
                }
            }
            unsigned need = __ballot_sync(0xffffffffu, act);
            while (need) {  // the same on every lane of the warp
                unsigned m = need;
                for (int t = 0; t < gw; ++t) m &= m - 1;  // this group's particle: set bit gw
                const int src = m ? __ffs(m) - 1 : 0;
                for (int t = 0; t < 32 / kVLanes; ++t) need &= need - 1;
                const int ge0 = __shfl_sync(0xffffffffu, e0, src);
                const int ge1 = __shfl_sync(0xffffffffu, e1, src);
                const int gnv = __shfl_sync(0xffffffffu, nv, src);
                const bool gfrz = __shfl_sync(0xffffffffu, frz, src);
                const bool active = m != 0u;
                RowJob job{};
                if (active)
                    list_particle<MULTI>(d, p, cur, sh, g, lane, gmask, base + src, ge0, ge1, gnv,
                                         gfrz, job);
                emit_rows<kVLanes>(d, p, cur, active, job, lane);
                __syncwarp();
            }
        }
        return;
    }
    // each block takes a contiguous share of the particles, a multiple of a
    // warp's 8 groups, so that every block of the cooperative grid (which
    // places consecutive blocks on the same SM) has work: on the
    // 17,576-sphere cube, 64 consecutive particles per block left half of
    // the SMs idle (54.5 -> 52.8 us per step with the even shares)
    const int per = (int)((((long long)p.n + gridDim.x - 1) / gridDim.x + 7) & ~7LL);
    const int lo = blockIdx.x * per;
    const int hi = min(lo + per, p.n);
    for (int i0 = lo + gwarp; i0 < hi; i0 += kThreads / kVLanes) {
        const int i = i0 + (g - gwarp);
        // which particles test their lists: the path byte the search wrote (arena)
        bool active = i < hi;
        bool frozen = false;
        if (MULTI && active) {
            const uint8_t path = d.path[i];
            active = (path & 3) == 2;
            frozen = (path >> 2) == kModeFrozen;
        }
        RowJob job{};
        int e0 = 0, e1 = 0, nv = 0;
        if (active) {
            e0 = d.row_start[cur][i];
            e1 = e0 + d.row_len[cur][i];
            nv = frozen ? 0 : d.vl_len[i];
            // no contact and no list partner: an empty next row, decided at once
            if (e1 == e0 && nv == 0) {
                job.i = i;
                job.mode = frozen ? kModeFrozen : kModeStep;
                job.e0 = job.e1 = e0;
                active = false;
                if (lane == 0) {
                    d.row_start[cur ^ 1][i] = 0;
                    d.row_len[cur ^ 1][i] = 0;
                }
            }
        }
        if (active) list_particle<MULTI>(d, p, cur, sh, g, lane, gmask, i, e0, e1, nv, frozen, job);
        emit_rows<kVLanes>(d, p, cur, active, job, lane);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// The contact update of a step in one cooperative launch: the full pair
// search (the broad phase kernels above: hash, bucket scan, counting sort,
// canonical order; then the cp_list enumeration), separated by grid
// barriers, and the neighbour-list update of the scenes that do not search.
// Every block of a cooperative launch is resident, so the barriers cannot
// wait on a block that has not started.  A single-scene handle whose lists
// are valid runs the list update only; an arena hashes (which also records
// each slot's path), runs the list update of its list scenes, and ends there
// when nothing was hashed.

// Grid barrier: arrival counter and generation word; a block waits for the
// generation to move on, with a bounded wait that raises kErrTimeout.
__device__ __forceinline__ void grid_sync(DevCounters* c,
                                          unsigned long long spin_limit = kSpinLimit) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* gen = &c->bar_gen;
        const unsigned int g = *gen;
        __threadfence();
        if (atomicAdd(&c->bar_count, 1u) == gridDim.x - 1) {
            atomicExch(&c->bar_count, 0u);
            __threadfence();
            atomicAdd(&c->bar_gen, 1u);
        } else {
            for (unsigned long long it = 0; *gen == g; ++it) {
                if (it > spin_limit) {
                    raise_error(c, kErrTimeout);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// Block-wide sum of one value per thread (kThreads threads).
__device__ __forceinline__ unsigned long long block_sum(unsigned long long v,
                                                        unsigned long long* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane_id() == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned long long t = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) t += red[w];
    __syncthreads();
    return t;
}

// Exclusive scan of cell_count[0, count) into cell_start (count = the
// buckets up to this step's largest, as the standalone scan), in tiles of
// kScanTile: tile sums, a barrier, then each tile's prefix from the sums.
// Ends with a barrier.
constexpr int kFusedItems = kScanTile / kThreads;
__device__ void scan_phase(const DemDev& d, const DemParams& p, unsigned long long* red) {
    // (values written by other blocks earlier in this launch are read past L1)
    const long long lim = (long long)__ldcg(&d.ctr->bmax) + 1;
    const long long count = lim < (long long)p.T ? lim : (long long)p.T;
    const int ntiles = (int)((count + kScanTile - 1) / kScanTile);
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const long long base = (long long)t * kScanTile + (long long)threadIdx.x * kFusedItems;
        unsigned long long v = 0;
#pragma unroll 8
        for (int k = 0; k < kFusedItems; ++k)
            if (base + k < count) v += d.cell_count[base + k];
        const unsigned long long tot = block_sum(v, red);
        if (threadIdx.x == 0) d.tile_sums[t] = (uint32_t)tot;
    }
    grid_sync(d.ctr);
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        unsigned long long pre = 0;
        for (int u = threadIdx.x; u < t; u += kThreads) pre += __ldcg(&d.tile_sums[u]);
        pre = block_sum(pre, red);
        const long long base = (long long)t * kScanTile + (long long)threadIdx.x * kFusedItems;
        unsigned long long mine = 0;
#pragma unroll 8
        for (int k = 0; k < kFusedItems; ++k)
            if (base + k < count) mine += d.cell_count[base + k];
        // exclusive prefix of `mine` across the block
        unsigned long long x = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane_id() >= (unsigned)o) x += y;
        }
        if (lane_id() == 31) red[threadIdx.x >> 5] = x;
        __syncthreads();
        unsigned long long wpre = 0;
        for (int w = 0; w < (int)(threadIdx.x >> 5); ++w) wpre += red[w];
        __syncthreads();
        unsigned long long run = pre + wpre + x - mine;
#pragma unroll 8
        for (int k = 0; k < kFusedItems; ++k) {
            if (base + k < count) {
                d.cell_start[base + k] = (uint32_t)run;
                run += d.cell_count[base + k];
            }
        }
        if (t == ntiles - 1 && threadIdx.x == kThreads - 1) d.cell_start[count] = (uint32_t)run;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) d.ctr->cell_limit = (unsigned int)count;
    grid_sync(d.ctr);
}

template <bool INIT, bool MULTI, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_search(DemDev d, DemParams p, int cur, int all) {
    __shared__ DetectShared sh[kThreads / kLanes];
    __shared__ ListShared lsh[kThreads / kVLanes];
    __shared__ unsigned long long red[kThreads / 32];
    dep_begin();
    if (!MULTI && !(all || INIT || d.sflags[cur][0] != 0u)) {
        list_phase<false>(d, p, cur, lsh);  // the scene tests its neighbour lists
        return;
    }
    const int stride = gridDim.x * kThreads;
    const int wbase = blockIdx.x * kThreads + (int)(threadIdx.x & ~31u);
    if (MULTI && blockIdx.x == 0 && threadIdx.x == 0) d.ctr->hashed[cur ^ 1] = 0u;
    // hash (`cell`, `hashcode`, `neighbors`, `count_particles!`)
    for (int i0 = wbase; i0 < p.n; i0 += stride) {
        const int i = i0 + (int)lane_id();
        bool act = false;
        uint32_t b = 0;
        if (i < p.n) hash_particle<MULTI>(d, p, cur, all, i, act, b);
        hash_count(d, act, b, MULTI ? &d.ctr->hashed[cur] : nullptr);
    }
    grid_sync(d.ctr);
    // the scenes that test their neighbour lists (path bytes written above):
    // independent of the search below (other particles and rows)
    if (MULTI && !INIT) list_phase<true>(d, p, cur, lsh);
    if (MULTI && *(volatile unsigned int*)&d.ctr->hashed[cur] == 0u) return;
    // `accumulate!` of the bucket counts
    scan_phase(d, p, red);
    // `get_particle_id!`
    for (int i0 = wbase; i0 < p.n; i0 += stride) scatter_warp(d, p, i0 + (int)lane_id());
    grid_sync(d.ctr);
    // canonical order; this step's bucket maximum is no longer read
    const uint32_t lim = __ldcg(&d.ctr->cell_limit);
    const int count = (int)__ldcg(&d.cell_start[lim]);
    if (blockIdx.x == 0 && threadIdx.x == 0) d.ctr->bmax = 0u;
    for (int k = blockIdx.x * kThreads + (int)threadIdx.x; k < count; k += stride)
        canon_slot<MULTI>(d, p, cur, k);
    grid_sync(d.ctr);
    // cp_list enumeration with update_contacts! / init_bonds!, then the next
    // rows; a warp's four groups move together (the rows are placed per warp)
    const int lane = threadIdx.x & (kLanes - 1);
    const int g = threadIdx.x / kLanes;
    const unsigned gmask = 0xffu << (lane_id() & ~7u);
    const int gwarp = (int)(threadIdx.x >> 5) * (32 / kLanes);  // the warp's first group
    for (int k0 = blockIdx.x * (kThreads / kLanes) + gwarp; k0 < count;
         k0 += gridDim.x * (kThreads / kLanes)) {
        const int k = k0 + (g - gwarp);
        RowJob job{};
        const bool active = k < count;
        if (active) detect_group<INIT, MULTI>(d, p, cur, k, lane, gmask, lim, sh[g], job);
        emit_rows<kLanes>(d, p, cur, active, job, lane);
        __syncwarp();
    }
}

// End of a step (run by k_integrate): the rebuild flags of this step are
// cleared; scenes that did not step keep theirs for their next step; scenes
// without a skin search in full every step.
template <bool MULTI>
__device__ __forceinline__ void scene_flags_one(const DemDev& d, const DemParams& p, int cur, int s) {
    const SceneParams& S = scene_rec<MULTI>(d, p, s);
    const int mode = MULTI ? S.mode : kModeStep;
    const int nxt = cur ^ 1;
    if (mode == kModeFree) {
        d.sflags[cur][s] = 0u;
        return;
    }
    if (mode == kModeStep && d.sflags[cur][s] != 0u) d.sctr[s].searches += 1ull;
    uint32_t carry = mode != kModeStep ? d.sflags[cur][s] : 0u;
    if (mode == kModeStep && !(S.f_half_skin > 0.0f)) carry = 1u;
    if (carry) atomicOr(&d.sflags[nxt][s], carry);
    d.sflags[cur][s] = 0u;
}


// ---------------------------------------------------------------------------
// Contact frame of src/kernels.jl:145-165: the rotation 𝐑 taking the unit
// normal a = normalize(𝐤ⱼ - 𝐤ᵢ) to the local x axis.  For b = x̂ the
// reference's I + [v]ₓ + [v]ₓ² (1-c)/s² has the rows
//   ( a₁, a₂, a₃ ), ( -a₂, 1 - a₂² f, -a₂a₃ f ), ( -a₃, -a₂a₃ f, 1 - a₃² f ),
// f = (1 - a₁)/s², s² = a₂² + a₃²; its degenerate branch (s < tolerance) is
// diag(±1, 1, ±1).  Both are kept as (a₁, a₂, a₃, f, neg3):
//   𝐑v  = ( a₁v₁ + w,  v₂ - a₂ t,  ±(v₃ - a₃ t) ),  w = a₂v₂ + a₃v₃, t = v₁ + f w
//   𝐑ᵀv = ( a₁v₁ - w,  v₂ + a₂ u,  ±(v₃ + a₃ u) ),  u = v₁ - f w
// (6 FP64 operations instead of 9).  𝐑 is orthonormal, so its inverse
// (src/kernels.jl:224, 298) is its transpose.  The branch is decided on the
// exact reference values of a and s when a is within 2·tolerance of ±x̂.
struct Frame {
    double a1, a2, a3, f;
    bool neg3;
};
__device__ __forceinline__ Frame frame_exact(double ax, double ay, double az, double tol) {
    // v = a × x̂ = (±0, a₃, -a₂); s = norm(v) evaluated as sqrt((0 + a₃²) + a₂²)
    const double s = norm_rn(0.0, az, -ay);
    Frame F;
    if (s < tol) {
        const double sg = ax > 0.0 ? 1.0 : -1.0;
        F.a1 = sg;
        F.a2 = 0.0;
        F.a3 = 0.0;
        F.f = 0.0;
        F.neg3 = sg < 0.0;
    } else {
        F.a1 = ax;
        F.a2 = ay;
        F.a3 = az;
        F.f = (1.0 - ax) / (s * s);
        F.neg3 = false;
    }
    return F;
}
// The degenerate branch without the exact recomputation: s² below tol² by a
// relative 2^-30 (far beyond the 1e-15 relative error of the fast normal)
// decides s < tol for the reference's exactly normalised a as well.
__device__ __forceinline__ Frame frame_degenerate(double ax) {
    const double sg = ax > 0.0 ? 1.0 : -1.0;
    Frame F;
    F.a1 = sg;
    F.a2 = 0.0;
    F.a3 = 0.0;
    F.f = 0.0;
    F.neg3 = sg < 0.0;
    return F;
}
static __device__ __noinline__ Frame frame_exact_from(double dx, double dy, double dz, double tol) {
    const double L = norm_rn(dx, dy, dz);
    const double il = __ddiv_rn(1.0, L);
    return frame_exact(__dmul_rn(il, dx), __dmul_rn(il, dy), __dmul_rn(il, dz), tol);
}
__device__ __forceinline__ Frame contact_frame(double dx, double dy, double dz, double ax,
                                               double ay, double az, const SceneParams& S) {
    const double s2 = ay * ay + az * az;
    // s² >= +0 (a sum of squares) and the tolerances are positive: compared
    // as bit patterns, off the FP64 pipe
    if (less_nonneg(s2, S.tol2_lo)) return frame_degenerate(ax);
    if (less_nonneg(s2, S.tol2_x4)) return frame_exact_from(dx, dy, dz, S.tol);
    Frame F;
    F.a1 = ax;
    F.a2 = ay;
    F.a3 = az;
    F.f = (1.0 - ax) * rcp_nr(s2);  // (1 - a₁)/s²
    F.neg3 = false;
    return F;
}
template <typename T>
__device__ __forceinline__ Vec3<T> rot(const Frame& R, Vec3<T> v) {  // 𝐑 v
    const T a1 = (T)R.a1, a2 = (T)R.a2, a3 = (T)R.a3, f = (T)R.f;
    const T w = a2 * v.y + a3 * v.z;
    const T t = v.x + f * w;
    const T z = v.z - a3 * t;
    return {a1 * v.x + w, v.y - a2 * t, R.neg3 ? -z : z};
}
template <typename T>
__device__ __forceinline__ Vec3<T> rot_t(const Frame& R, Vec3<T> v) {  // 𝐑ᵀ v
    const T a1 = (T)R.a1, a2 = (T)R.a2, a3 = (T)R.a3, f = (T)R.f;
    const T w = a2 * v.y + a3 * v.z;
    const T u = v.x - f * w;
    const T z = v.z + a3 * u;
    return {a1 * v.x - w, v.y + a2 * u, R.neg3 ? -z : z};
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
__device__ __forceinline__ Vec3<T> from_d(Vec3<double> v) {
    return {(T)v.x, (T)v.y, (T)v.z};
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
                                            double b_sc, double b_st, double b_ss) {
    const double ai = ti.y * ti.y + ti.z * ti.z, aj = tj.y * tj.y + tj.z * tj.z;
    const bool nan_a = isnan(ai) || isnan(aj);
    const double amax = fmax(ai, aj), amin = fmin(ai, aj);
    const double fa = F.x * invA, k2 = rbI * rbI;
    const double Rc = b_sc - fa;     // σc >= σc₀  <=>  rbI·sqrt(amax) >= Rc
    const double Rt = -(b_st + fa);  // σt >= σt₀  <=>  rbI·sqrt(amin) <= Rt
    const double Rs = b_ss - fabs(ti.x) * (0.5 * rbI);  // σs >= σs₀ <=> 4/3·invA·sqrt(b) >= Rs
    const double b = F.y * F.y + F.z * F.z;
    const double ks = (4.0 / 3.0) * invA;
    const bool comp = !nan_a && (Rc <= 0.0 || amax * k2 >= Rc * Rc);
    const bool tens = !nan_a && Rt >= 0.0 && amin * k2 <= Rt * Rt;
    const bool shear = !isnan(b) && !isnan(Rs) && (Rs <= 0.0 || b * (ks * ks) >= Rs * Rs);
    return comp || tens || shear;
}
__device__ __forceinline__ bool bond_breaks(const Vec3<double>& F, const Vec3<double>& ti,
                                            const Vec3<double>& tj, double invA, double rbI,
                                            const SceneParams& p) {
    return bond_breaks(F, ti, tj, invA, rbI, p.b_sc, p.b_st, p.b_ss);
}
// The breakage test of a bond between grains of a table scene (no FP32 screen).
static __device__ __noinline__ bool bond_breaks_tab(const Vec3<double>& F, const Vec3<double>& ti,
                                                    const Vec3<double>& tj, double invA,
                                                    double rbI, const PairConst& pc) {
    return bond_breaks(F, ti, tj, invA, rbI, pc.sc, pc.st, pc.ss);
}

// Breakage decision of bond_breaks behind an FP32 screen.  The three stresses
// σc = fa + rb/I·sqrt(amax), σt = -fa - rb/I·sqrt(amin) and
// σs = |τᵢ₁|·rb/2/I + 4/3/A·sqrt(F₂²+F₃²) are evaluated in FP32 from the FP64
// values; each FP32 result lies within 2^-20 (|terms| + |threshold|) of the
// exact one, so when every stress is below its threshold by 2^-16 of that
// scale the bond cannot break and the FP64 test is skipped.  Otherwise (and for
// NaN or out-of-range values, which fail every comparison) the FP64 test
// decides, so the outcome is always that of bond_breaks.
__device__ __forceinline__ double pair_value(float2 v) { return (double)v.x + (double)v.y; }

// bond_breaks on FP32 hi/lo pairs (out of line: the FP32 screen settles
// almost every bond without it)
static __device__ __noinline__ bool bond_breaks_pairs(const float2 (&F)[3], const float2 (&ti)[3],
                                                      const float2 (&tj)[3], double invA,
                                                      double rbI, const SceneParams& p) {
    const Vec3<double> Fd{pair_value(F[0]), pair_value(F[1]), pair_value(F[2])};
    const Vec3<double> tid{pair_value(ti[0]), pair_value(ti[1]), pair_value(ti[2])};
    const Vec3<double> tjd{pair_value(tj[0]), pair_value(tj[1]), pair_value(tj[2])};
    return bond_breaks(Fd, tid, tjd, invA, rbI, p);
}

__device__ __forceinline__ bool stress_clear(const Vec3<float>& Ff, const Vec3<float>& tif,
                                             const Vec3<float>& tjf, float iA, float rb,
                                             const SceneParams& p) {
    const float ai = tif.y * tif.y + tif.z * tif.z, aj = tjf.y * tjf.y + tjf.z * tjf.z;
    const float fa = Ff.x * iA;
    const float smax = rb * sqrtf(fmaxf(ai, aj)), smin = rb * sqrtf(fminf(ai, aj));
    const float s1 = fabsf(tif.x) * 0.5f * rb;
    const float s2 = (4.0f / 3.0f) * iA * sqrtf(Ff.y * Ff.y + Ff.z * Ff.z);
    const float sc = p.f_sc, st = p.f_st, ss = p.f_ss;
    const float afa = fabsf(fa);
    return (fa + smax + (afa + smax + fabsf(sc)) * 0x1p-16f < sc) &&
           (-fa - smin + (afa + smin + fabsf(st)) * 0x1p-16f < st) &&
           (s1 + s2 + (s1 + s2 + fabsf(ss)) * 0x1p-16f < ss);
}
__device__ __forceinline__ bool bond_breaks_screened(const float2 (&F)[3], const float2 (&ti)[3],
                                                     const float2 (&tj)[3], const Vec3<float>& Ff,
                                                     const Vec3<float>& tif, const Vec3<float>& tjf,
                                                     float iA, float rb, const DemDev& d, int small,
                                                     const SceneParams& p) {
    if (stress_clear(Ff, tif, tjf, iA, rb, p)) return false;
    return bond_breaks_pairs(F, ti, tj, d.b_invA[small], d.b_rbI[small], p);
}
// The FP64 force mode's breakage decision behind the same FP32 screen.
static __device__ __noinline__ bool bond_breaks_d(const Vec3<double>& F, const Vec3<double>& ti,
                                                  const Vec3<double>& tj, double invA, double rbI,
                                                  const SceneParams& p) {
    return bond_breaks(F, ti, tj, invA, rbI, p);
}
__device__ __forceinline__ bool bond_breaks_fp64(const Vec3<double>& F, const Vec3<double>& ti,
                                                 const Vec3<double>& tj, const DemDev& d,
                                                 int small, const SceneParams& p) {
    const Vec3<float> Ff{d2f(F.x), d2f(F.y), d2f(F.z)};
    const Vec3<float> tif{d2f(ti.x), d2f(ti.y), d2f(ti.z)};
    const Vec3<float> tjf{d2f(tj.x), d2f(tj.y), d2f(tj.z)};
    if (stress_clear(Ff, tif, tjf, d.bk32[small].w, d.rm32[small].x, p)) return false;
    return bond_breaks_d(F, ti, tj, d.b_invA[small], d.b_rbI[small], p);
}

// FP32 hi/lo pair accumulator (hi + lo carries about 48 bits): (hi, lo) + x
// by Knuth's two-sum and a fast renormalisation, all in FP32.
__device__ __forceinline__ float2 pair_add(float2 a, float x) {
    const float s = a.x + x;
    const float bp = s - a.x;
    const float e = (a.x - (s - bp)) + (x - bp) + a.y;
    const float h = s + e;
    return make_float2(h, e - (h - s));
}
__device__ __forceinline__ float2* pair_col(const ContactSoA& w, int f) {
    return reinterpret_cast<float2*>(w.f[f]);
}

// FP32 contact frame (same rows as Frame), from the FP32 unit normal; the
// degenerate branch is decided as in contact_frame, on FP64 values.
struct Frame32 {
    float a1, a2, a3, f;
    bool neg3;
};
static __device__ __noinline__ Frame32 frame32_exact(double dx, double dy, double dz, double tol) {
    const double L = norm_rn(dx, dy, dz);
    const double il = __ddiv_rn(1.0, L);
    const Frame F = frame_exact(__dmul_rn(il, dx), __dmul_rn(il, dy), __dmul_rn(il, dz), tol);
    return {(float)F.a1, (float)F.a2, (float)F.a3, (float)F.f, F.neg3};
}
__device__ __forceinline__ Frame32 contact_frame32(float ax, float ay, float az, double dx,
                                                   double dy, double dz, const SceneParams& S) {
    const float s2 = ay * ay + az * az;
    // s² below tol² by a relative 2^-10 (the FP32 normal is within 1e-6):
    // the reference's degenerate branch, decided without FP64
    if (s2 < S.f_tol1) {
        const float sg = ax > 0.0f ? 1.0f : -1.0f;
        return {sg, 0.0f, 0.0f, 0.0f, sg < 0.0f};
    }
    if (s2 < S.f_tol4) return frame32_exact(dx, dy, dz, S.tol);
    return {ax, ay, az, (1.0f - ax) / s2, false};
}
__device__ __forceinline__ Vec3<float> rot32(const Frame32& R, Vec3<float> v) {
    const float w = R.a2 * v.y + R.a3 * v.z;
    const float t = v.x + R.f * w;
    const float z = v.z - R.a3 * t;
    return {R.a1 * v.x + w, v.y - R.a2 * t, R.neg3 ? -z : z};
}
__device__ __forceinline__ Vec3<float> rot_t32(const Frame32& R, Vec3<float> v) {
    const float w = R.a2 * v.y + R.a3 * v.z;
    const float u = v.x - R.f * w;
    const float z = v.z + R.a3 * u;
    return {R.a1 * v.x - w, v.y + R.a2 * u, R.neg3 ? -z : z};
}

// `resolve_collision!` in the FP32 force mode (DEM_FP32_FORCE).  Differences
// of positions and velocities are formed in FP64 and then cast; the contact
// frame, stiffnesses, damping and friction run in FP32.  The shear
// displacement 𝐬 and the contact point stay FP64; the accumulated bond force
// and torques are FP32 hi/lo pairs (compensated sums, about 48 significant
// bits) stored in their FP64 slots, and the bond-breakage decision is the
// FP64 test's.  Contact forces are stored as (F, 0) pairs in this mode; the
// host decodes them, and a precision switch re-encodes the stored contacts
// (k_recode).  The FP64 differences are narrowed with d2f (integer pipe), so
// the FP64 pipe only forms the differences and the contact point.  The Hertz
// overlap is
// (L² - (rᵢ+rⱼ)²)/(L + rᵢ + rⱼ) with the numerator in FP64, which keeps the
// overlap's relative error at FP32 rounding even though L is FP32.
__device__ __forceinline__ void force32(const DemDev& d, const SceneParams& SP,
                                        const ContactSoA& w, const ContactSoA& o, int sidx, int c,
                                        uint32_t fl, int i, int j, int sc, size_t cap) {
    const double kix = d.px[i], kiy = d.py[i], kiz = d.pz[i];
    const double dxd = d.px[j] - kix, dyd = d.py[j] - kiy, dzd = d.pz[j] - kiz;
    const float dx = d2f(dxd), dy = d2f(dyd), dz = d2f(dzd);
    const float L2 = dx * dx + dy * dy + dz * dz;
    const float invL = rsqrtf(L2);
    const float ax = dx * invL, ay = dy * invL, az = dz * invL;
    const Frame32 R = contact_frame32(ax, ay, az, dxd, dyd, dzd, SP);
    const double ri = d.r[i], rj = d.r[j];
    Vec3<float> fig, mi, mj;
    if (fl & kBonded) {
        // EBPM (src/kernels.jl:170-239), increments in FP32
        const double wix = d.wx[i], wiy = d.wy[i], wiz = d.wz[i];
        const double wjx = d.wx[j], wjy = d.wy[j], wjz = d.wz[j];
        const Vec3<float> D = rot32(R, {d2f(d.vx[i] - d.vx[j]), d2f(d.vy[i] - d.vy[j]),
                                        d2f(d.vz[i] - d.vz[j])});
        const Vec3<float> Sv =
            rot32(R, {d2f(wix + wjx), d2f(wiy + wjy), d2f(wiz + wjz)});
        const Vec3<float> Q = rot32(R, {d2f(wix - wjx), d2f(wiy - wjy), d2f(wiz - wjz)});
        const float4 rmi = d.rm32[i], rmj = d.rm32[j];
        const bool i_small = rmi.z <= rmj.z;
        const int small = i_small ? i : j;   // rb = ρ·min(rᵢ, rⱼ)
        const float4 bk = d.bk32[small];     // (ϕ coefficient, E·I, E·A, 1/A)
        const float tdt = SP.f_dt;
        const float phi = bk.x * invL * invL;
        const float iphi = 1.0f / (1.0f + phi);
        const float EILdt = bk.y * invL * tdt;
        const float k1 = bk.z * invL * tdt;
        const float k3 = 6.0f * EILdt * invL * iphi;
        const float k2 = 2.0f * k3 * invL;
        const float k4 = EILdt * SP.f_inv1pnu;
        const float kp = 3.0f * EILdt * iphi;
        const float km = EILdt;
        const float dFx = k1 * D.x, dFy = k2 * D.y + k3 * Sv.z, dFz = k2 * D.z - k3 * Sv.y;
        const float ay_ = -k3 * D.z + kp * Sv.y, az_ = k3 * D.y + kp * Sv.z;
        const float dtix = k4 * Q.x, dtiy = ay_ + km * Q.y, dtiz = az_ + km * Q.z;
        const float dtjx = -k4 * Q.x, dtjy = ay_ - km * Q.y, dtjz = az_ - km * Q.z;
        // accumulated bond force and torques: FP32 hi/lo pairs in the FP64 slots
        float2 Fp[3], tip[3], tjp[3];
        const float dF[3] = {dFx, dFy, dFz}, dti[3] = {dtix, dtiy, dtiz};
        const float dtj[3] = {dtjx, dtjy, dtjz};
        const float2 z2 = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int q = 0; q < 3; ++q) {  // carried state from the other buffer
            Fp[q] = pair_add(sidx >= 0 ? pair_col(o, CF + q)[sidx] : z2, dF[q]);
            tip[q] = pair_add(sidx >= 0 ? pair_col(o, CTI + q)[sidx] : z2, dti[q]);
            tjp[q] = pair_add(sidx >= 0 ? pair_col(o, CTJ + q)[sidx] : z2, dtj[q]);
        }
        const Vec3<float> Ff{Fp[0].x, Fp[1].x, Fp[2].x};
        const Vec3<float> tif{tip[0].x, tip[1].x, tip[2].x};
        const Vec3<float> tjf{tjp[0].x, tjp[1].x, tjp[2].x};
        if (bond_breaks_screened(Fp, tip, tjp, Ff, tif, tjf, bk.w, (i_small ? rmi : rmj).x, d,
                                 small, SP)) {
            w.fl[c] = 0u;
            atomicAdd(&d.sctr[sc].broken, 1ull);
            fig = {0.0f, 0.0f, 0.0f};
            mi = fig;
            mj = fig;
        } else {
            fig = rot_t32(R, {-Ff.x, -Ff.y, -Ff.z});
            mi = rot_t32(R, {-tif.x, -tif.y, -tif.z});
            mj = rot_t32(R, {-tjf.x, -tjf.y, -tjf.z});
            st3(w.f, CK, c, {kix + 0.5 * dxd, kiy + 0.5 * dyd, kiz + 0.5 * dzd});
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                pair_col(w, CF + q)[c] = Fp[q];
                pair_col(w, CTI + q)[c] = tip[q];
                pair_col(w, CTJ + q)[c] = tjp[q];
            }
            // 𝐬 of a bond is zero from its creation on and is not stored again
        }
    } else {
        // Hertz-Mindlin (src/kernels.jl:240-313)
        const float4 rmi = d.rm32[i], rmj = d.rm32[j];  // (rb/I, m, r, 0)
        const double Rsum = ri + rj;
        const double num = (dxd * dxd + dyd * dyd + dzd * dzd) - Rsum * Rsum;
        const float L = L2 * invL;
        const float gap = d2f(num) / (L + d2f(Rsum));
        if (num > 0.0) atomicAdd(&d.sctr[sc].warn_gap, 1ull);
        const float ext = rmi.z - fabsf(gap);
        const Vec3<float> kri{ax * ext, ay * ext, az * ext};
        st3(w.f, CK, c, {kix + f2d(kri.x), kiy + f2d(kri.y), kiz + f2d(kri.z)});
        const Vec3<float> krj{kri.x - dx, kri.y - dy, kri.z - dz};
        const Vec3<float> wi{d2f(d.wx[i]), d2f(d.wy[i]), d2f(d.wz[i])};
        const Vec3<float> wj{d2f(d.wx[j]), d2f(d.wy[j]), d2f(d.wz[j])};
        const Vec3<float> wci = cross3<float>(wi, kri), wcj = cross3<float>(wj, krj);
        const Vec3<float> dv{d2f(d.vx[j] - d.vx[i]) + (wcj.x - wci.x),
                             d2f(d.vy[j] - d.vy[i]) + (wcj.y - wci.y),
                             d2f(d.vz[j] - d.vz[i]) + (wcj.z - wci.z)};
        const Vec3<float> vc = rot32(R, dv);
        const float fri = rmi.z, frj = rmj.z, tmi = rmi.y, tmj = rmj.y;
        const float Rs = fri * frj / (fri + frj);
        const float ms = tmi * tmj / (tmi + tmj);
        const float sq = sqrtf(Rs * fabsf(gap));
        const float kn = SP.f_kn * sq;
        const float kt = SP.f_kt * sq;
        const float root = sqrtf(ms * sq);
        const float gn = SP.f_cgn * root;
        const float gt = SP.f_cgt * root;
        if (gn < 0.0f || gt < 0.0f)
            atomicAdd(&d.sctr[sc].warn_damp, (unsigned long long)((gn < 0.0f) + (gt < 0.0f)));
        // 𝐬 += (0, vc₂, vc₃)·dt in FP64 (the normal component stays)
        Vec3<double> s = sidx >= 0 ? ld3(o.f, CS, sidx) : Vec3<double>{0.0, 0.0, 0.0};
        s = {s.x, s.y + f2d(vc.y * SP.f_dt), s.z + f2d(vc.z * SP.f_dt)};
        const float F1 = -kn * gap - gn * vc.x;
        const Vec3<float> Ft{-kt * d2f(s.x), -kt * d2f(s.y), -kt * d2f(s.z)};
        const float nFt = sqrtf(Ft.x * Ft.x + Ft.y * Ft.y + Ft.z * Ft.z);
        const float muF1 = SP.f_mu * F1;
        float F2, F3;
        if (nFt >= muF1) {
            const float ratio = muF1 / nFt;
            F2 = ratio * Ft.y;
            F3 = ratio * Ft.z;
            s = {s.x, f2d(F2 / kt), f2d(F3 / kt)};
        } else {
            F2 = Ft.y - gt * vc.y;
            F3 = Ft.z - gt * vc.z;
        }
        fig = rot_t32(R, {-F1, -F2, -F3});
        mi = cross3<float>(kri, fig);
        mj = cross3<float>(krj, {-fig.x, -fig.y, -fig.z});
        pair_col(w, CF + 0)[c] = make_float2(F1, 0.0f);
        pair_col(w, CF + 1)[c] = make_float2(F2, 0.0f);
        pair_col(w, CF + 2)[c] = make_float2(F3, 0.0f);
        st3(w.f, CS, c, s);
    }
    float* cb = d.contrib32;
    cb[0 * cap + c] = fig.x;
    cb[1 * cap + c] = fig.y;
    cb[2 * cap + c] = fig.z;
    cb[3 * cap + c] = mi.x;
    cb[4 * cap + c] = mi.y;
    cb[5 * cap + c] = mi.z;
    cb[6 * cap + c] = mj.x;
    cb[7 * cap + c] = mj.y;
    cb[8 * cap + c] = mj.z;
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
// 3EI/L/(1+ϕ) and k₋ = (k₅-k₆)/2 = EI/L; dt is folded into the stiffnesses.
// One contact, one thread: FP64 mode (T = double) or the FP32 force mode's
// Hertz and bond paths (T = float, via force32).
// TAB: a scene with material and wall tables (FP64 only): the pair's
// constants come from surfaces[midᵢ, midⱼ] and materials midᵢ, midⱼ, and the
// bond section of rb = ρ·min(rᵢ, rⱼ) is formed here from that surface.
template <typename T, bool TAB = false>
__device__ __forceinline__ void contact_one(const DemDev& d, const SceneParams& SP,
                                            const ContactSoA& w, const ContactSoA& o, int c,
                                            uint32_t fl, int i, int j, int sc, size_t cap) {
    const int sidx = w.src[c];  // carried state in the other buffer (-1: new, zero)
    if constexpr (std::is_same<T, float>::value) {
        force32(d, SP, w, o, sidx, c, fl, i, j, sc, cap);
        return;
    }
    const PairConst* pc = nullptr;
    if constexpr (TAB) pc = &d.mt->pair[d.mid[i] * d.mt->nmat + d.mid[j]];
    const double dt = SP.dt;
    const Vec3<double> ki{d.px[i], d.py[i], d.pz[i]}, kj{d.px[j], d.py[j], d.pz[j]};
    const double ri = d.r[i], rj = d.r[j];
    const Vec3<double> vi{d.vx[i], d.vy[i], d.vz[i]}, vj{d.vx[j], d.vy[j], d.vz[j]};
    const Vec3<double> wi{d.wx[i], d.wy[i], d.wz[i]}, wj{d.wx[j], d.wy[j], d.wz[j]};
    const double dx = kj.x - ki.x, dy = kj.y - ki.y, dz = kj.z - ki.z;
    const double L2 = dx * dx + dy * dy + dz * dz;
    const double invL = rsqrt(L2);
    const double L = L2 * invL;
    const double ax = dx * invL, ay = dy * invL, az = dz * invL;
    const Frame R = contact_frame(dx, dy, dz, ax, ay, az, SP);
    Vec3<T> fig, mi, mj;
    if (fl & kBonded) {
        // EBPM (src/kernels.jl:170-239)
        const Vec3<double> Dd = rot<double>(R, {vi.x - vj.x, vi.y - vj.y, vi.z - vj.z});
        const Vec3<double> Ts = rot<double>(R, {wi.x + wj.x, wi.y + wj.y, wi.z + wj.z});
        const Vec3<double> Td = rot<double>(R, {wi.x - wj.x, wi.y - wj.y, wi.z - wj.z});
        const Vec3<T> D = from_d<T>(Dd), Sv = from_d<T>(Ts), Q = from_d<T>(Td);
        const int small = !less_nonneg(rj, ri) ? i : j;  // rb = ρ·min(rᵢ, rⱼ); radii > 0
        // bond section (src/kernels.jl:178-184): per particle for the scene's
        // one surface, per pair from the surface table
        double b_phic, b_EI, b_EA, b_1pnu, b_invA = 0.0, b_rbI = 0.0;
        if constexpr (TAB) {
            const double rb = __dmul_rn(pc->ratio, d.r[small]);
            const double rb2 = __dmul_rn(rb, rb);
            const double Ab = __dmul_rn(rb2, kPi);
            const double Ib = __dmul_rn(__dmul_rn(rb2, rb2), kPi / 4.0);
            b_EA = __dmul_rn(pc->E, Ab);
            b_EI = __dmul_rn(pc->E, Ib);
            b_phic = __dmul_rn(__dmul_rn(20.0 / 3.0, __dadd_rn(1.0, pc->nu)), rb2);
            b_1pnu = pc->inv1pnu;
            b_invA = __ddiv_rn(1.0, Ab);
            b_rbI = __ddiv_rn(rb, Ib);
        } else {
            b_phic = d.b_phic[small];
            b_EI = d.b_EI[small];
            b_EA = d.b_EA[small];
            b_1pnu = SP.b_inv1pnu;
        }
        const T tinvL = (T)invL, tdt = (T)dt;
        const T phi = (T)b_phic * tinvL * tinvL;
        const T iphi = rcp_nr((T)1.0 + phi);  // 1/(1 + ϕ)
        const T EILdt = (T)b_EI * tinvL * tdt;  // EI/L·dt
        const T k1 = (T)b_EA * tinvL * tdt;
        const T k3 = (T)6.0 * EILdt * tinvL * iphi;
        const T k2 = (T)2.0 * k3 * tinvL;
        const T k4 = EILdt * (T)b_1pnu;
        const T kp = (T)3.0 * EILdt * iphi;
        const T km = EILdt;
        const T dFx = k1 * D.x, dFy = k2 * D.y + k3 * Sv.z, dFz = k2 * D.z - k3 * Sv.y;
        const T ay_ = -k3 * D.z + kp * Sv.y, az_ = k3 * D.y + kp * Sv.z;
        const T dtix = k4 * Q.x, dtiy = ay_ + km * Q.y, dtiz = az_ + km * Q.z;
        const T dtjx = -k4 * Q.x, dtjy = ay_ - km * Q.y, dtjz = az_ - km * Q.z;
        const Vec3<double> z3{0.0, 0.0, 0.0};
        Vec3<double> Fi = sidx >= 0 ? ld3(o.f, CF, sidx) : z3;
        Vec3<double> ti = sidx >= 0 ? ld3(o.f, CTI, sidx) : z3;
        Vec3<double> tj = sidx >= 0 ? ld3(o.f, CTJ, sidx) : z3;
        Fi = {Fi.x + (double)dFx, Fi.y + (double)dFy, Fi.z + (double)dFz};
        ti = {ti.x + (double)dtix, ti.y + (double)dtiy, ti.z + (double)dtiz};
        tj = {tj.x + (double)dtjx, tj.y + (double)dtjy, tj.z + (double)dtjz};
        // breakage test, FP64 (src/kernels.jl:208-222)
        bool broken;
        if constexpr (TAB) broken = bond_breaks_tab(Fi, ti, tj, b_invA, b_rbI, *pc);
        else broken = bond_breaks_fp64(Fi, ti, tj, d, small, SP);
        if (broken) {
            w.fl[c] = 0u;  // contact_active and contact_bonded bits cleared
            atomicAdd(&d.sctr[sc].broken, 1ull);
            fig = {(T)0, (T)0, (T)0};
            mi = fig;
            mj = fig;
        } else {
            fig = from_d<T>(rot_t<double>(R, {-Fi.x, -Fi.y, -Fi.z}));
            mi = from_d<T>(rot_t<double>(R, {-ti.x, -ti.y, -ti.z}));
            mj = from_d<T>(rot_t<double>(R, {-tj.x, -tj.y, -tj.z}));
            st3(w.f, CK, c, {half_exact(ki.x + kj.x), half_exact(ki.y + kj.y),
                             half_exact(ki.z + kj.z)});
            st3(w.f, CF, c, Fi);
            st3(w.f, CTI, c, ti);
            st3(w.f, CTJ, c, tj);  // a bond's 𝐬 stays zero and is not stored
        }
    } else {
        // Hertz-Mindlin (src/kernels.jl:240-313)
        const double gap = L - ri - rj;
        if (gap > 0) atomicAdd(&d.sctr[sc].warn_gap, 1ull);
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
        const double pYs = TAB ? pc->Ys : SP.pp_Ys, pGs = TAB ? pc->Gs : SP.pp_Gs;
        const double pcgn = TAB ? pc->cgn : SP.pp_cgn, pcgt = TAB ? pc->cgt : SP.pp_cgt;
        const double pmu = TAB ? pc->mu : SP.pp_mu;
        const T kn = (T)(4.0 / 3.0 * pYs) * sq;
        const T kt = (T)(8.0 * pGs) * sq;
        const T root = sqrt(ms * sq);
        const T gn = (T)pcgn * root;
        const T gt = (T)pcgt * root;
        if (gn < (T)0 || gt < (T)0)
            atomicAdd(&d.sctr[sc].warn_damp, (unsigned long long)((gn < (T)0) + (gt < (T)0)));
        Vec3<double> s = sidx >= 0 ? ld3(o.f, CS, sidx) : Vec3<double>{0.0, 0.0, 0.0};
        s = {s.x + (double)vc.x * 0.0, s.y + (double)vc.y * dt, s.z + (double)vc.z * dt};
        const T F1 = -kn * tgap - gn * vc.x;
        const Vec3<T> Ft{-kt * (T)s.x, -kt * (T)s.y, -kt * (T)s.z};
        const T nFt = sqrt(Ft.x * Ft.x + Ft.y * Ft.y + Ft.z * Ft.z);
        const T muF1 = (T)pmu * F1;
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

// With bonds and other contacts both present, threads take the contacts in
// the order of the type-ordered list that the rows' placement wrote (bonds
// first, then the others, the second part starting on a warp boundary), so
// that a warp runs one of the two force laws: a warp with both runs both in
// turn on the FP64 pipe, which spends the same time on a warp instruction
// whatever the number of active lanes.  With one type only, thread t takes
// contact t (no list read).  The list entry of a thread's next contact is
// read one iteration ahead, so that its latency overlaps the current one.
template <typename T, bool MULTI, bool TAB = false>
__device__ __forceinline__ void force_body(const DemDev& d, const DemParams& p, int nxt) {
    const RowCounter a = d.ctr->alloc[nxt];
    const int C = min((int)a.rows, p.cap);
    const int NB = min((int)a.bonds, C);
    const bool mixed = NB > 0 && NB < C;
    const int NBw = mixed ? (NB + 31) & ~31 : NB;
    const int total = mixed ? NBw + (C - NB) : C;
    const ContactSoA w = d.c[nxt];
    const ContactSoA o = d.c[nxt ^ 1];
    const int stride = gridDim.x * blockDim.x;
    const size_t cap = (size_t)p.cap;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        int c = t;
        if (mixed) {
            if (t >= NB && t < NBw) continue;  // padding up to the warp boundary
            c = t < NB ? d.tlist[t] : d.tlist[cap - 1 - (size_t)(t - NBw)];
            if ((unsigned)c >= (unsigned)C) continue;  // only after a capacity overflow
        }
        const uint32_t fl = w.fl[c];
        const int i = w.ci[c], j = w.cj[c];
        const int sc = slot_scene<MULTI>(d, i);
        if (MULTI && (sc < 0 || d.sp[sc].mode != kModeStep)) continue;
        // the contact in its partner's incoming list (the integrator's gather
        // sorts the list by owner, so the order of registration is free)
        add_incoming_entry(d, p, j, c, i);
        contact_one<T, TAB>(d, scene_rec<MULTI>(d, p, sc), w, o, c, fl, i, j, sc, cap);
    }
}

// The force pass with the compiler's register choice, and with a budget for
// four 256-thread blocks per SM (an autotuner choice for the FP32 mode).
template <typename T, bool MULTI>
__global__ void __launch_bounds__(kThreads) k_force(DemDev d, DemParams p, int nxt) {
    dep_begin(p.dep == 2);
    force_body<T, MULTI>(d, p, nxt);
}
template <typename T, bool MULTI>
__global__ void __launch_bounds__(kThreads, 4) k_force4(DemDev d, DemParams p, int nxt) {
    dep_begin(p.dep == 2);
    force_body<T, MULTI>(d, p, nxt);
}
// a single scene with material and wall tables (FP64)
__global__ void __launch_bounds__(kThreads) k_force_tab(DemDev d, DemParams p, int nxt) {
    dep_begin(p.dep == 2);
    force_body<double, false, true>(d, p, nxt);
}

// ---------------------------------------------------------------------------
// Per particle: contact force gather, `resolve_wall!` (src/kernels.jl:317-426),
// `apply_body_force!` (src/kernels.jl:428-443) and `update!`
// (src/kernels.jl:445-485).  One thread per particle, so every FP64
// instruction runs on full warps.  Contributions are added in a fixed order:
// the particle's own row (ordered by j), then its incoming contacts ordered by
// owner index i.  The order depends only on the contact set, not on where the
// contacts sit in the buffers, so results are reproducible.
// For spheres 𝐈 = (2/5 m r²) I₃, so inv(𝐑)·inv(𝐈)·(𝐑𝛕 - 𝐑𝛚 × 𝐈𝐑𝛚) is 𝛕/I
// exactly in real arithmetic; the quaternion only evolves as state.
constexpr int kMaxIncoming = 64;

// ascending .y, an odd-even transposition network on N register slots
template <int N>
__device__ __forceinline__ void sort_by_owner(int2 (&v)[N]) {
#pragma unroll
    for (int r = 0; r < N; ++r) {
#pragma unroll
        for (int u = r & 1; u + 1 < N; u += 2) {
            const bool sw = v[u].y > v[u + 1].y;
            const int2 a = v[u], b = v[u + 1];
            v[u] = sw ? b : a;
            v[u + 1] = sw ? a : b;
        }
    }
}
template <typename T>
__device__ __forceinline__ const T* contrib_of(const DemDev& d) {
    if constexpr (std::is_same<T, float>::value) return d.contrib32;
    else return d.contrib;
}
template <typename T, int N>
__device__ __forceinline__ void add_incoming(const DemDev& d, size_t cap, int2 (&v)[N], int nin,
                                             T* F, T* M) {
    const T* cb = contrib_of<T>(d);
    sort_by_owner<N>(v);
    T g[N][6];
#pragma unroll
    for (int u = 0; u < N; ++u) {
        if (u < nin) {
            const int c = v[u].x;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                g[u][q] = cb[q * cap + c];
                g[u][3 + q] = cb[(6 + q) * cap + c];
            }
        }
    }
#pragma unroll
    for (int u = 0; u < N; ++u) {
        if (u < nin) {
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                F[q] += -g[u][q];
                M[q] += g[u][3 + q];
            }
        }
    }
}

// Sum of the contact contributions on particle i in the fixed order: its own
// row (by j), then its incoming contacts by owner index.  T = double for the
// FP64 force mode, float for the FP32 force mode (its contributions are FP32).
// The caller loads the row (c0, len) and the incoming count with the rest of
// the particle's state; the first incoming entries are loaded here before the
// row's contributions, so the two chains of loads overlap.
template <typename T>
__device__ __forceinline__ void gather(const DemDev& d, const DemParams& p, int i, int c0, int len,
                                       int nin, T* F, T* M) {
    const size_t cap = (size_t)p.cap;
    const T* cb = contrib_of<T>(d);
    nin = nin < p.kin ? nin : p.kin;
    nin = nin < kMaxIncoming ? nin : kMaxIncoming;
    const int2* il = d.in_list + (size_t)i * p.kin;
    int2 v4[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v4[u] = u < nin ? il[u] : make_int2(0, 0x7fffffff);
    const int c1 = min(c0 + len, p.cap);
    int c = c0;
    for (; c + 1 < c1; c += 2) {
        T a[6], b[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            a[q] = cb[q * cap + c];
            b[q] = cb[q * cap + c + 1];
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            F[q] += a[q];
            M[q] += a[3 + q];
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            F[q] += b[q];
            M[q] += b[3 + q];
        }
    }
    if (c < c1) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            F[q] += cb[q * cap + c];
            M[q] += cb[(3 + q) * cap + c];
        }
    }
    if (nin <= 4) {
        add_incoming<T, 4>(d, cap, v4, nin, F, M);
    } else if (nin <= 8) {
        int2 v8[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v8[u] = u < 4 ? v4[u] : (u < nin ? il[u] : make_int2(0, 0x7fffffff));
        add_incoming<T, 8>(d, cap, v8, nin, F, M);
    } else {
        int2 inc[kMaxIncoming];
        for (int u = 0; u < nin; ++u) {
            const int2 v = il[u];
            int b = u - 1;
            while (b >= 0 && inc[b].y > v.y) {
                inc[b + 1] = inc[b];
                --b;
            }
            inc[b + 1] = v;
        }
        for (int u = 0; u < nin; ++u) {
            const int cc = inc[u].x;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                F[q] += -cb[q * cap + cc];
                M[q] += cb[(6 + q) * cap + cc];
            }
        }
    }
}

// Skin test: true once the FP32 position (fx, fy, fz) lies more than skin/2
// from xr, the position the scene's neighbour lists were built at (FP32
// rounding of both positions is taken off the allowance).
__device__ __forceinline__ bool left_skin(const SceneParams& S, float fx, float fy, float fz,
                                          float4 xr) {
    const float ex = fx - xr.x, ey = fy - xr.y, ez = fz - xr.z;
    const float M = fmaxf(fmaxf(fabsf(fx), fabsf(fy)), fabsf(fz)) +
                    fmaxf(fmaxf(fabsf(xr.x), fabsf(xr.y)), fabsf(xr.z));
    const float lim = S.f_half_skin - M * 0x1p-21f;
    return !(lim > 0.0f) || !(ex * ex + ey * ey + ez * ez <= lim * lim);
}

// One wall's constants as the wall contact reads them.
struct WallK {
    const double* wn;
    double wd;
    const double* wR;
    const double* wRinv;
    const float* f_wn;
    float f_wc0;
    double mu, Ys, Gs, cgn, cgt;
};
// resolve_wall! for one particle and one wall (src/kernels.jl:317-426):
// whether the wall touches the particle and, if so, the wall's force g and
// moment mw on it; updates the wall contact's shear history (*wsx, *wsy,
// *wsz; zero when not touching); `count`: this thread adds to the scene's
// warning counters.  An FP32 screen on the
// step's starting position (pos32, within 2^-24 of the FP64 one per
// coordinate) skips the exact test when |n·x - d| exceeds r by a margin that
// covers its rounding.
__device__ __forceinline__ bool wall_force(const DemDev& d, int sc, const WallK& W, double dt,
                                           float4 p32, float r32, double x, double y, double z,
                                           double vx, double vy, double vz, double wx, double wy,
                                           double wz, double r, double m, double* wsx, double* wsy,
                                           double* wsz, double g[3], double mw[3], bool count) {
    bool wall_near;
    {
        const float4 q = p32;
        const float Lf = q.x * W.f_wn[0] + q.y * W.f_wn[1] + q.z * W.f_wn[2] + W.f_wc0;
        const float rf = r32;
        const float mg = (fabsf(q.x) + fabsf(q.y) + fabsf(q.z) + fabsf(W.f_wc0) + rf) * 0x1p-20f;
        wall_near = !(fabsf(Lf) > rf + mg);
    }
    if (!wall_near) {
        *wsx = 0.0;
        *wsy = 0.0;
        *wsz = 0.0;
        return false;
    }
    const double dotkn = __dadd_rn(__dadd_rn(__dmul_rn(x, W.wn[0]), __dmul_rn(y, W.wn[1])),
                                   __dmul_rn(z, W.wn[2]));
    const double L = __dsub_rn(dotkn, W.wd);
    if (fabs(L) < r) {
        const double gap = fabs(L) - r;
        const double dn = fabs(gap);
        const double lsc = (fabs(L) + dn / 2.0) / fabs(L);
        const double kix = -L * W.wn[0] * lsc, kiy = -L * W.wn[1] * lsc, kiz = -L * W.wn[2] * lsc;
        const double vcix = wy * kiz - wz * kiy + vx, vciy = wz * kix - wx * kiz + vy,
                     vciz = wx * kiy - wy * kix + vz;
        const double* Rw = W.wR;
        const double vcx = -(Rw[0] * vcix + Rw[1] * vciy + Rw[2] * vciz);
        const double vcy = -(Rw[3] * vcix + Rw[4] * vciy + Rw[5] * vciz);
        const double vcz = -(Rw[6] * vcix + Rw[7] * vciy + Rw[8] * vciz);
        const double sq = sqrt(r * dn);
        const double kn = 4.0 / 3.0 * W.Ys * sq;
        const double kt = 8.0 * W.Gs * sq;
        const double root = sqrt(m * sq);
        const double gn = W.cgn * root;
        const double gt = W.cgt * root;
        if (count && gn < 0) atomicAdd(&d.sctr[sc].warn_damp, 1ull);
        if (count && gt < 0) atomicAdd(&d.sctr[sc].warn_damp, 1ull);
        double sx = *wsx + vcx * 0.0, sy = *wsy + vcy * dt, sz = *wsz + vcz * dt;
        const double F1 = -kn * gap - gn * vcx;
        const double Ftx = -kt * sx, Fty = -kt * sy, Ftz = -kt * sz;
        const double nFt = sqrt(Ftx * Ftx + Fty * Fty + Ftz * Ftz);
        double F2, F3;
        if (nFt >= W.mu * F1) {
            const double ratio = W.mu * F1 / nFt;
            F2 = ratio * Fty;
            F3 = ratio * Ftz;
            sy = F2 / kt;
            sz = F3 / kt;
        } else {
            F2 = Fty - gt * vcy;
            F3 = Ftz - gt * vcz;
        }
        const double* Ri = W.wRinv;
        const double gx = -(Ri[0] * F1 + Ri[1] * F2 + Ri[2] * F3);
        const double gy = -(Ri[3] * F1 + Ri[4] * F2 + Ri[5] * F3);
        const double gz = -(Ri[6] * F1 + Ri[7] * F2 + Ri[8] * F3);
        g[0] = gx;
        g[1] = gy;
        g[2] = gz;
        mw[0] = kiy * gz - kiz * gy;
        mw[1] = kiz * gx - kix * gz;
        mw[2] = kix * gy - kiy * gx;
        *wsx = sx;
        *wsy = sy;
        *wsz = sz;
        return true;
    }
    *wsx = 0.0;
    *wsy = 0.0;
    *wsz = 0.0;
    return false;
}
// resolve_wall! adding the wall's force and moment to F, M
__device__ __forceinline__ void wall_contact(const DemDev& d, int sc, const WallK& W, double dt,
                                             float4 p32, float r32, double x, double y, double z,
                                             double vx, double vy, double vz, double wx, double wy,
                                             double wz, double r, double m, double* wsx,
                                             double* wsy, double* wsz, double F[3], double M[3]) {
    double g[3], mw[3];
    if (wall_force(d, sc, W, dt, p32, r32, x, y, z, vx, vy, vz, wx, wy, wz, r, m, wsx, wsy, wsz, g,
                   mw, true)) {
        F[0] += g[0];
        F[1] += g[1];
        F[2] += g[2];
        M[0] += mw[0];
        M[1] += mw[1];
        M[2] += mw[2];
    }
}

// The fused download of an exchanged step (HostOut): the armed step count
// as this launch sees it (0 for arena kernels and unarmed handles; every
// block of a launch reads the same value, since it changes only after all
// of them have counted themselves out).
template <bool MULTI>
__device__ __forceinline__ int host_out_left(const DemDev& d) {
    if constexpr (MULTI) return 0;
    else return __ldcg(&d.ctr->hout.steps_left);
}
// One thread per block, after the block's records are written (`wrote`) or
// at any point (an integrator that writes none): the last block of the
// launch disarms one step and, after the last armed step's records, copies
// the device error word (no integrator raises one) to the host.
__device__ __forceinline__ void host_out_count(const DemDev& d, int left, bool wrote) {
    HostOut& H = d.ctr->hout;
    __threadfence();
    if (atomicAdd(&H.done, 1u) != gridDim.x - 1) return;
    __threadfence();
    if (left == 1 && wrote) *H.err = __ldcg(&d.ctr->error);
    H.done = 0u;
    H.steps_left = left - 1;
}

template <bool MULTI, bool F32, bool TAB = false>
__device__ __forceinline__ void integrate_body(const DemDev& d, const DemParams& p, int cur) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nxt = cur ^ 1;
    if (i == 0) d.ctr->alloc[cur] = RowCounter{0u, 0u};  // the free buffer is next step's target
    // an armed handle's step: this layout writes no records (the host reads
    // the state the usual way), it only counts the launch
    if (!MULTI && threadIdx.x == 0) {
        const int left = host_out_left<MULTI>(d);
        if (left > 0) host_out_count(d, left, false);
    }
    // the end-of-step rebuild-flag work of every scene (see scene_flags_one):
    // it only ORs into the next flags, as the particles' skin test does
    for (int s = i; s < p.ns; s += gridDim.x * blockDim.x) scene_flags_one<MULTI>(d, p, cur, s);
    if (i >= p.n) return;
    const int sc = slot_scene<MULTI>(d, i);
    if (MULTI && (sc < 0 || d.sp[sc].mode != kModeStep)) {
        d.in_cnt[i] = 0;
        return;
    }
    const SceneParams& S = scene_rec<MULTI>(d, p, sc);
    // every load of the particle's own state is issued before the gather's
    // dependent loads (nothing here is stored before the gather completes)
    const int row0 = d.row_start[nxt][i], rlen = d.row_len[nxt][i], nin = d.in_cnt[i];
    const double x = d.px[i], y = d.py[i], z = d.pz[i];
    const double vx = d.vx[i], vy = d.vy[i], vz = d.vz[i];
    const double wx = d.wx[i], wy = d.wy[i], wz = d.wz[i];
    const double r = d.r[i], m = d.m[i];
    const double invm = d.inv_m[i], ii = d.inv_inertia[i];
    const double qw = d.qw[i], qx = d.qx[i], qy = d.qy[i], qz = d.qz[i];
    const float4 p32 = d.pos32[i], xr = d.xref[i];
    const float r32 = d.rm32[i].z;
    // 𝐪 + Δ𝐪 with Δ𝐪 = ½ 𝛚 ⊗ 𝐪 (no dt, as the reference), the ½ folded into
    // 𝛚, as explicit FMA chains.  With 𝛚 = (+0, +0, +0) each fma(a, +0, c)
    // (a finite) returns c unless c is -0, so for a finite 𝐪 without a -0
    // component the chains return 𝐪 itself: a particle that does not spin
    // skips them, with identical results.  The normalisation always runs.
    // A spinless particle with the identity orientation (1, +0, +0, +0)
    // keeps it: |𝐪|² = 1 exactly, rsqrt(1) = 1 (checked by
    // dem_selftest_conversions) and 𝐪·1 = 𝐪, so nothing is computed or stored.
    auto update_quaternion = [&]() {
        double nw = qw, nx = qx, ny = qy, nz = qz;
        const bool spinless = (__double_as_longlong(wx) | __double_as_longlong(wy) |
                               __double_as_longlong(wz)) == 0ll;
        const bool identity = spinless && __double_as_longlong(qw) == 0x3ff0000000000000ll &&
                              (__double_as_longlong(qx) | __double_as_longlong(qy) |
                               __double_as_longlong(qz)) == 0ll;
        if (!identity) {
            if (!(spinless && finite_not_negzero(qw) && finite_not_negzero(qx) &&
                  finite_not_negzero(qy) && finite_not_negzero(qz))) {
                const double hx = half_exact(wx), hy = half_exact(wy), hz = half_exact(wz);
                nw = __fma_rn(-qz, hz, __fma_rn(-qy, hy, __fma_rn(-qx, hx, qw)));
                nx = __fma_rn(-qz, hy, __fma_rn(qy, hz, __fma_rn(qw, hx, qx)));
                ny = __fma_rn(qz, hx, __fma_rn(qx, hz, __fma_rn(qw, hy, qy)));
                nz = __fma_rn(-qy, hx, __fma_rn(qx, hy, __fma_rn(qw, hz, qz)));
            }
            const double inq = rsqrt(__fma_rn(nz, nz, __fma_rn(ny, ny, __fma_rn(nx, nx, nw * nw))));
            d.qw[i] = nw * inq;
            d.qx[i] = nx * inq;
            d.qy[i] = ny * inq;
            d.qz[i] = nz * inq;
        }
    };
    double F[3] = {0.0, 0.0, 0.0}, M[3] = {0.0, 0.0, 0.0};
    if constexpr (F32) {
        float Ff[3] = {0.0f, 0.0f, 0.0f}, Mf[3] = {0.0f, 0.0f, 0.0f};
        gather<float>(d, p, i, row0, rlen, nin, Ff, Mf);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            F[q] = f2d(Ff[q]);
            M[q] = f2d(Mf[q]);
        }
    } else {
        gather<double>(d, p, i, row0, rlen, nin, F, M);
    }
    d.in_cnt[i] = 0;
    const double dt = S.dt;
    // resolve_wall! (src/kernels.jl:317-426): the scene's one wall, or every
    // wall of a table scene in order (wall j's force and moment are added
    // after wall j-1's, as the reference's per-particle loop over j does)
    if constexpr (TAB) {
        const MatTables& T = *d.mt;
        const int a = d.mid[i];
        for (int wl = 0; wl < T.nwall; ++wl) {
            const WallConst& W = T.wall[wl];
            const WallK K{W.wn, W.wd, W.wR, W.wRinv, W.f_wn, W.f_wc0, W.mu[a], W.Ys[a], W.Gs[a],
                          W.cgn[a], W.cgt[a]};
            const size_t o = (size_t)wl * p.wstride + i;
            wall_contact(d, sc, K, dt, p32, r32, x, y, z, vx, vy, vz, wx, wy, wz, r, m, d.wsx + o,
                         d.wsy + o, d.wsz + o, F, M);
        }
    } else if (S.has_wall) {
        const WallK K{S.wn, S.wd, S.wR, S.wRinv, S.f_wn, S.f_wc0, S.pw_mu, S.pw_Ys, S.pw_Gs,
                      S.pw_cgn, S.pw_cgt};
        wall_contact(d, sc, K, dt, p32, r32, x, y, z, vx, vy, vz, wx, wy, wz, r, m, d.wsx + i,
                     d.wsy + i, d.wsz + i, F, M);
    }
    // apply_body_force!  A zero gravity component adds nothing: the force sum
    // starts at +0 and never becomes -0, so F + 0·m is F.
    if (nonzero_bits(S.grav[0])) F[0] += S.grav[0] * m;
    if (nonzero_bits(S.grav[1])) F[1] += S.grav[1] * m;
    if (nonzero_bits(S.grav[2])) F[2] += S.grav[2] * m;
    if (nonzero_bits(S.damping)) {
        const double v3[3] = {vx, vy, vz}, w3[3] = {wx, wy, wz};
        double dF[3], dM[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            dF[q] = -S.damping * fabs(F[q]) * jl_sign(v3[q]);
            dM[q] = -S.damping * fabs(M[q]) * jl_sign(w3[q]);
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            F[q] += dF[q];
            M[q] += dM[q];
        }
    }
    // update!
    const double ax = F[0] * invm, ay = F[1] * invm, az = F[2] * invm;
    const double hdt2 = S.hdt2;  // 0.5·(dt·dt)
    const double px1 = x + vx * dt + ax * hdt2, py1 = y + vy * dt + ay * hdt2,
                 pz1 = z + vz * dt + az * hdt2;
    d.px[i] = px1;
    d.py[i] = py1;
    d.pz[i] = pz1;
    // FP32 position for the neighbour-list search, and the skin test: the
    // scene searches in full next step once a particle has moved by skin/2
    // from where its list was built (FP32 rounding of both positions is
    // taken off the allowance)
    {
        const float fx = d2f(px1 - S.dmin[0]), fy = d2f(py1 - S.dmin[1]),
                    fz = d2f(pz1 - S.dmin[2]);
        d.pos32[i] = make_float4(fx, fy, fz, reach32(fx, fy, fz, r32));
        const bool moved = S.f_half_skin > 0.0f && left_skin(S, fx, fy, fz, xr);
        const unsigned am = __activemask();
        const unsigned peers = __match_any_sync(am, moved ? sc : -1);
        if (moved && lane_id() == (unsigned)(__ffs(peers) - 1) && d.sflags[nxt][sc] == 0u)
            atomicOr(&d.sflags[nxt][sc], 1u);
    }
    d.vx[i] = vx + ax * dt;
    d.vy[i] = vy + ay * dt;
    d.vz[i] = vz + az * dt;
    update_quaternion();
    // 𝛚 + 𝐌·I⁻¹dt: with 𝐌 = (+0, +0, +0) and a finite I⁻¹dt, fma(+0, I⁻¹dt, w)
    // is w unless w is -0, so a torque-free particle keeps its stored spin
    const bool torque_free = (__double_as_longlong(M[0]) | __double_as_longlong(M[1]) |
                              __double_as_longlong(M[2])) == 0ll;
    if (!(torque_free && product_finite(ii, dt) && not_negzero(wx) && not_negzero(wy) &&
          not_negzero(wz))) {
        const double iidt = ii * dt;
        d.wx[i] = __fma_rn(M[0], iidt, wx);
        d.wy[i] = __fma_rn(M[1], iidt, wy);
        d.wz[i] = __fma_rn(M[2], iidt, wz);
    }
    d.fx[i] = F[0];
    d.fy[i] = F[1];
    d.fz[i] = F[2];
    d.tx[i] = M[0];
    d.ty[i] = M[1];
    d.tz[i] = M[2];
}

// ---------------------------------------------------------------------------
// The same integration split over four warps per 32 particles, for scenes
// that leave most SM sub-partitions with at most one warp at one thread per
// particle.  An SM sub-partition retires one FP64 warp-instruction per ~64
// cycles whatever the number of active lanes, so a lone warp's FP64
// instructions, not its memory loads, set the pace there; the split divides
// them over four warps (on different sub-partitions) without repeating any:
// warps 0, 1, 2 own component q of the force and moment sums and of the
// position, velocity and spin updates of the block's 32 particles; warp 3
// evaluates the walls, then updates the quaternion while the others update
// the particles and, once the new position components are in shared memory,
// writes the FP32 position and runs the skin test.  Each component goes through the same operations in the same
// order as in integrate_body, so the results are bit-identical to it.
constexpr int kSplitThreads = 128;

template <typename P>
__device__ __forceinline__ P pick3(int q, P a, P b, P c) {
    return q == 0 ? a : (q == 1 ? b : c);
}
template <typename T, int N>
__device__ __forceinline__ void add_incoming_component(const T* cf, const T* cmj, int2 (&v)[N],
                                                       int nin, T& F, T& M) {
    sort_by_owner<N>(v);
    T gf[N], gm[N];
#pragma unroll
    for (int u = 0; u < N; ++u) {
        if (u < nin) {
            gf[u] = cf[v[u].x];
            gm[u] = cmj[v[u].x];
        }
    }
#pragma unroll
    for (int u = 0; u < N; ++u) {
        if (u < nin) {
            F += -gf[u];
            M += gm[u];
        }
    }
}
// component qc of gather(): the particle's own row, then its incoming
// contacts ordered by owner index
template <typename T>
__device__ __forceinline__ void gather_component(const DemDev& d, const DemParams& p, int i,
                                                 int c0, int len, int nin, int qc, T& F, T& M) {
    const size_t cap = (size_t)p.cap;
    const T* cb = contrib_of<T>(d);
    const T* cf = cb + (size_t)qc * cap;         // force on the owner
    const T* cmi = cb + (size_t)(3 + qc) * cap;  // the owner's moment
    const T* cmj = cb + (size_t)(6 + qc) * cap;  // the partner's moment
    nin = nin < p.kin ? nin : p.kin;
    nin = nin < kMaxIncoming ? nin : kMaxIncoming;
    const int2* il = d.in_list + (size_t)i * p.kin;
    int2 v4[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v4[u] = u < nin ? il[u] : make_int2(0, 0x7fffffff);
    const int c1 = min(c0 + len, p.cap);
    int c = c0;
    for (; c + 1 < c1; c += 2) {
        const T a0 = cf[c], a1 = cmi[c], b0 = cf[c + 1], b1 = cmi[c + 1];
        F += a0;
        M += a1;
        F += b0;
        M += b1;
    }
    if (c < c1) {
        F += cf[c];
        M += cmi[c];
    }
    if (nin <= 4) {
        add_incoming_component<T, 4>(cf, cmj, v4, nin, F, M);
    } else if (nin <= 8) {
        int2 v8[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v8[u] = u < 4 ? v4[u] : (u < nin ? il[u] : make_int2(0, 0x7fffffff));
        add_incoming_component<T, 8>(cf, cmj, v8, nin, F, M);
    } else {
        int2 inc[kMaxIncoming];
        for (int u = 0; u < nin; ++u) {
            const int2 v = il[u];
            int b = u - 1;
            while (b >= 0 && inc[b].y > v.y) {
                inc[b + 1] = inc[b];
                --b;
            }
            inc[b + 1] = v;
        }
        for (int u = 0; u < nin; ++u) {
            const int cc = inc[u].x;
            F += -cf[cc];
            M += cmj[cc];
        }
    }
}

template <bool MULTI, bool F32, bool TAB = false>
__device__ __forceinline__ void integrate_split(const DemDev& d, const DemParams& p, int cur) {
    constexpr int NW = TAB ? kMaxWalls : 1;
    __shared__ double s_wall[NW][6][32];  // each wall's force and moment on each particle
    __shared__ uint8_t s_touch[NW][32];
    __shared__ float s_pos[3][32];        // the new FP32 position components
    // an armed single-scene step: the new state of the block's particles, as
    // rows of the output records (HostOut), and the first armed step's
    // orientations and first-wall shear histories read from the caller's
    __shared__ double s_out[MULTI ? 1 : kHostOutRows][32];
    __shared__ uint8_t s_chg[MULTI ? 1 : kHostOutRows][32];  // value differs from the input
    __shared__ double s_in[MULTI ? 1 : 7][32];
    // 0, 1, 2: component; 3: walls and quaternion.  The roles rotate with
    // the block's round over the SMs: warp w of a block runs on SM
    // sub-partition w, and blocks are placed one per SM in turn (blocks b,
    // b + sms, b + 2·sms, ... share an SM), so rotating by b / sms gives the
    // blocks on one SM different sub-partitions for their wall and
    // quaternion warp, the one with the most FP64 instructions (a rotation by
    // b mod 4 would not: the SM count, 152, is a multiple of 4)
    const int q = ((int)(threadIdx.x >> 5) - (int)((blockIdx.x / (unsigned)max(p.sms, 1)) & 3u) -
                   1) & 3;
    const int l = (int)lane_id();
    const int i = blockIdx.x * 32 + l;
    const int nxt = cur ^ 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int left = host_out_left<MULTI>(d);
    const bool out = !MULTI && left == 1;  // this launch writes the caller's records
    const double* qin = nullptr;           // this launch reads these from the caller's
    const double* wsin = nullptr;
    if (!MULTI && left > 0 && left == __ldcg(&d.ctr->hout.steps_total)) {
        qin = d.ctr->hout.qin;
        wsin = d.ctr->hout.wsin;
    }
    if (t == 0) d.ctr->alloc[cur] = RowCounter{0u, 0u};  // the free buffer is next step's target
    for (int s2 = t; s2 < p.ns; s2 += gridDim.x * blockDim.x) scene_flags_one<MULTI>(d, p, cur, s2);
    // every thread reaches both barriers; `live`: a particle of a stepping scene
    const bool exists = i < p.n;
    int sc = 0;
    bool live = exists;
    if (live) {
        sc = slot_scene<MULTI>(d, i);
        if (MULTI && (sc < 0 || d.sp[sc].mode != kModeStep)) live = false;
    }
    const SceneParams& S = scene_rec<MULTI>(d, p, live ? sc : 0);
    const int nwall = TAB ? d.mt->nwall : (live && S.has_wall ? 1 : 0);
    double Fq = 0.0, Mq = 0.0, xq = 0.0, vq = 0.0, wq = 0.0, invm = 0.0, ii = 0.0, m = 0.0;
    if (q < 3) {
        if (live) {
            const int row0 = d.row_start[nxt][i], rlen = d.row_len[nxt][i], nin = d.in_cnt[i];
            xq = pick3(q, d.px, d.py, d.pz)[i];
            vq = pick3(q, d.vx, d.vy, d.vz)[i];
            wq = pick3(q, d.wx, d.wy, d.wz)[i];
            m = d.m[i];
            invm = d.inv_m[i];
            ii = d.inv_inertia[i];
            if constexpr (F32) {
                float Ff = 0.0f, Mf = 0.0f;
                gather_component<float>(d, p, i, row0, rlen, nin, q, Ff, Mf);
                Fq = f2d(Ff);
                Mq = f2d(Mf);
            } else {
                gather_component<double>(d, p, i, row0, rlen, nin, q, Fq, Mq);
            }
        }
    }
    if constexpr (!MULTI) {
        if (q == 3 && (qin || wsin)) {
            // the block's 32 particles are one contiguous range of each
            // record array: consecutive lanes read it, then each lane its own
            const int i0 = blockIdx.x * 32, m = min(32, p.n - i0);
            if (qin)
                for (int e = l; e < 4 * m; e += 32) s_in[e & 3][e >> 2] = qin[(size_t)4 * i0 + e];
            if (wsin)
                for (int e = l; e < 3 * m; e += 32) {
                    const int pq = e / 3;
                    s_in[4 + e - 3 * pq][pq] = wsin[(size_t)3 * i0 + e];
                }
            __syncwarp();
        }
    }
    // warp 3: the step's starting spin, for the walls now and the quaternion
    // after the first barrier (the component warps store the new spin after it)
    double wx = 0.0, wy = 0.0, wz = 0.0, qw = 1.0, qx = 0.0, qy = 0.0, qz = 0.0;
    if (q == 3 && live) {
        wx = d.wx[i];
        wy = d.wy[i];
        wz = d.wz[i];
        bool qhost = false;
        if constexpr (!MULTI) {
            if (qin) {
                qw = s_in[0][l];
                qx = s_in[1][l];
                qy = s_in[2][l];
                qz = s_in[3][l];
                qhost = true;
            }
            if (wsin) {  // the first wall's shear history, for wall_force below
                d.wsx[i] = s_in[4][l];
                d.wsy[i] = s_in[5][l];
                d.wsz[i] = s_in[6][l];
            }
        }
        if (!qhost) {
            qw = d.qw[i];  // loaded here: their latency hides behind the walls
            qx = d.qx[i];
            qy = d.qy[i];
            qz = d.qz[i];
        }
        const double x = d.px[i], y = d.py[i], z = d.pz[i];
        const double vx = d.vx[i], vy = d.vy[i], vz = d.vz[i];
        const double r = d.r[i];
        const float4 p32 = d.pos32[i];
        const float r32 = d.rm32[i].z;
        const double dt = S.dt;
        // resolve_wall!: each wall's force and moment, added by the component
        // warps in wall order
        for (int wl = 0; wl < nwall; ++wl) {
            size_t o = i;
            WallK K;
            if constexpr (TAB) {
                const MatTables& T = *d.mt;
                const int a = d.mid[i];
                const WallConst& W = T.wall[wl];
                K = WallK{W.wn, W.wd, W.wR, W.wRinv, W.f_wn, W.f_wc0, W.mu[a], W.Ys[a], W.Gs[a],
                          W.cgn[a], W.cgt[a]};
                o = (size_t)wl * p.wstride + i;
            } else {
                K = WallK{S.wn, S.wd, S.wR, S.wRinv, S.f_wn, S.f_wc0, S.pw_mu, S.pw_Ys, S.pw_Gs,
                          S.pw_cgn, S.pw_cgt};
            }
            double g[3], mw[3];
            if (out && wl == 0) {  // the first wall's shear history before the step
                s_out[19][l] = d.wsx[o];
                s_out[20][l] = d.wsy[o];
                s_out[21][l] = d.wsz[o];
            }
            const bool touch = wall_force(d, sc, K, dt, p32, r32, x, y, z, vx, vy, vz, wx, wy, wz,
                                          r, d.m[i], d.wsx + o, d.wsy + o, d.wsz + o, g, mw, true);
            s_touch[wl][l] = touch ? 1 : 0;
            if (touch) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    s_wall[wl][c][l] = g[c];
                    s_wall[wl][3 + c][l] = mw[c];
                }
            }
        }
        if (out) {  // the first wall's shear history as this thread left it
            const double* ws[3] = {d.wsx, d.wsy, d.wsz};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double v = ws[c][i];
                // without walls nothing changed it (the value before the
                // step is not staged then)
                s_chg[19 + c][l] = nwall > 0 && __double_as_longlong(v) !=
                                                    __double_as_longlong(s_out[19 + c][l]);
                s_out[19 + c][l] = v;
            }
        }
    }
    __syncthreads();  // walls in shared memory; every component thread has read in_cnt
    if (q == 3 && exists) d.in_cnt[i] = 0;
    // the quaternion (integrate_body's update, from the starting spin) runs
    // while the component warps update the position, velocity and spin
    if (q == 3 && live) {
        const bool spinless = (__double_as_longlong(wx) | __double_as_longlong(wy) |
                               __double_as_longlong(wz)) == 0ll;
        const bool identity = spinless && __double_as_longlong(qw) == 0x3ff0000000000000ll &&
                              (__double_as_longlong(qx) | __double_as_longlong(qy) |
                               __double_as_longlong(qz)) == 0ll;
        double ow = qw, ox = qx, oy = qy, oz = qz;
        if (!identity) {
            double nw = qw, nx = qx, ny = qy, nz = qz;
            if (!(spinless && finite_not_negzero(qw) && finite_not_negzero(qx) &&
                  finite_not_negzero(qy) && finite_not_negzero(qz))) {
                const double hx = half_exact(wx), hy = half_exact(wy), hz = half_exact(wz);
                nw = __fma_rn(-qz, hz, __fma_rn(-qy, hy, __fma_rn(-qx, hx, qw)));
                nx = __fma_rn(-qz, hy, __fma_rn(qy, hz, __fma_rn(qw, hx, qx)));
                ny = __fma_rn(qz, hx, __fma_rn(qx, hz, __fma_rn(qw, hy, qy)));
                nz = __fma_rn(-qy, hx, __fma_rn(qx, hy, __fma_rn(qw, hz, qz)));
            }
            const double inq = rsqrt(__fma_rn(nz, nz, __fma_rn(ny, ny, __fma_rn(nx, nx, nw * nw))));
            ow = nw * inq;
            ox = nx * inq;
            oy = ny * inq;
            oz = nz * inq;
            d.qw[i] = ow;
            d.qx[i] = ox;
            d.qy[i] = oy;
            d.qz[i] = oz;
        } else if (qin) {  // read from the caller's: the columns still hold the old ones
            d.qw[i] = ow;
            d.qx[i] = ox;
            d.qy[i] = oy;
            d.qz[i] = oz;
        }
        if (out) {
            s_out[9][l] = ow;
            s_out[10][l] = ox;
            s_out[11][l] = oy;
            s_out[12][l] = oz;
            s_chg[9][l] = __double_as_longlong(ow) != __double_as_longlong(qw);
            s_chg[10][l] = __double_as_longlong(ox) != __double_as_longlong(qx);
            s_chg[11][l] = __double_as_longlong(oy) != __double_as_longlong(qy);
            s_chg[12][l] = __double_as_longlong(oz) != __double_as_longlong(qz);
        }
    }
    if (q < 3 && live) {
        const double dt = S.dt;
        for (int wl = 0; wl < nwall; ++wl) {
            if (s_touch[wl][l]) {
                Fq += s_wall[wl][q][l];
                Mq += s_wall[wl][3 + q][l];
            }
        }
        // apply_body_force!
        if (nonzero_bits(S.grav[q])) Fq += S.grav[q] * m;
        if (nonzero_bits(S.damping)) {
            const double dF = -S.damping * fabs(Fq) * jl_sign(vq);
            const double dM = -S.damping * fabs(Mq) * jl_sign(wq);
            Fq += dF;
            Mq += dM;
        }
        // update!
        const double aq = Fq * invm;
        const double hdt2 = S.hdt2;
        const double pq1 = xq + vq * dt + aq * hdt2;
        pick3(q, d.px, d.py, d.pz)[i] = pq1;
        s_pos[q][l] = d2f(pq1 - S.dmin[q]);
        const double vq1 = vq + aq * dt;
        pick3(q, d.vx, d.vy, d.vz)[i] = vq1;
        // 𝛚 + 𝐌·I⁻¹dt; with Mq = +0, a finite I⁻¹dt and wq not -0 the sum
        // is wq and the stored spin stays
        double wq1 = wq;
        if (!(__double_as_longlong(Mq) == 0ll && product_finite(ii, dt) && not_negzero(wq))) {
            wq1 = __fma_rn(Mq, ii * dt, wq);
            pick3(q, d.wx, d.wy, d.wz)[i] = wq1;
        }
        pick3(q, d.fx, d.fy, d.fz)[i] = Fq;
        pick3(q, d.tx, d.ty, d.tz)[i] = Mq;
        if (out) {
            s_out[q][l] = pq1;
            s_out[3 + q][l] = vq1;
            s_out[6 + q][l] = wq1;
            s_out[13 + q][l] = Fq;
            s_out[16 + q][l] = Mq;
            s_chg[q][l] = __double_as_longlong(pq1) != __double_as_longlong(xq);
            s_chg[3 + q][l] = __double_as_longlong(vq1) != __double_as_longlong(vq);
            s_chg[6 + q][l] = __double_as_longlong(wq1) != __double_as_longlong(wq);
        }
    }
    __syncthreads();  // the new position components (and an armed step's rows) in shared memory
    if (q == 3 && live) {
        const float fx = s_pos[0][l], fy = s_pos[1][l], fz = s_pos[2][l];
        d.pos32[i] = make_float4(fx, fy, fz, reach32(fx, fy, fz, d.rm32[i].z));
        const bool moved = S.f_half_skin > 0.0f && left_skin(S, fx, fy, fz, d.xref[i]);
        const unsigned am = __activemask();
        const unsigned peers = __match_any_sync(am, moved ? sc : -1);
        if (moved && lane_id() == (unsigned)(__ffs(peers) - 1) && d.sflags[nxt][sc] == 0u)
            atomicOr(&d.sflags[nxt][sc], 1u);
    }
    if constexpr (!MULTI) {
        if (left > 0) {
            if (out) {
                // the block's 32 particles are one contiguous range of each
                // record array: k·32 values, written by consecutive threads
                const int i0 = blockIdx.x * 32, m = min(32, p.n - i0);
                const unsigned same = d.ctr->hout.same;
                int row = 0;
#pragma unroll
                for (int f = 0; f < kHostOutFields; ++f) {
                    const int k = f == 3 ? 4 : 3;
                    double* rec = d.ctr->hout.rec[f];
                    const bool keep = (same >> f) & 1u;  // unchanged values are there already
                    if (rec) {
                        for (int e = threadIdx.x; e < k * 32; e += kSplitThreads) {
                            const int pq = e / k, r = row + e - pq * k;
                            if (pq < m && (!keep || s_chg[r][pq])) rec[(size_t)k * i0 + e] = s_out[r][pq];
                        }
                    }
                    row += k;
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) host_out_count(d, left, out);
        }
    }
}

// The integrator with the compiler's register choice (FP64 force mode), and
// in the FP32 force mode with a budget for three 256-thread blocks per SM:
// its FP64 work per particle is small enough that more resident warps hide
// the state loads better than the extra registers would.
template <bool MULTI, bool F32>
__global__ void __launch_bounds__(kThreads) k_integrate(DemDev d, DemParams p, int cur) {
    dep_begin(p.dep == 2);
    integrate_body<MULTI, F32>(d, p, cur);
}
__global__ void __launch_bounds__(kThreads) k_integrate_tab(DemDev d, DemParams p, int cur) {
    dep_begin(p.dep == 2);
    integrate_body<false, false, true>(d, p, cur);
}
template <bool MULTI>
__global__ void __launch_bounds__(kThreads, 3) k_integrate3(DemDev d, DemParams p, int cur) {
    dep_begin(p.dep == 2);
    integrate_body<MULTI, true>(d, p, cur);
}
// four warps per 32 particles (integrate_split)
template <bool MULTI, bool F32>
__global__ void __launch_bounds__(kSplitThreads) k_integrate_split(DemDev d, DemParams p, int cur) {
    dep_begin(p.dep == 2);
    integrate_split<MULTI, F32>(d, p, cur);
}
__global__ void __launch_bounds__(kSplitThreads) k_integrate_split_tab(DemDev d, DemParams p,
                                                                       int cur) {
    dep_begin(p.dep == 2);
    integrate_split<false, false, true>(d, p, cur);
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
    buckets8(d.cellinfo[i], p.s0, B);
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
    buckets8(d.cellinfo[i], p.s0, B);
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

// Re-encodes the force and torque columns (𝐅ᵢ, 𝛕ᵢ, 𝛕ⱼ) of the first n
// entries of a contact buffer between FP64 values and FP32 hi/lo pairs.
__global__ void __launch_bounds__(kThreads) k_recode(ContactSoA w, int n, int to_pairs) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
#pragma unroll
    for (int f = CF; f < CS; ++f) {
        if (to_pairs) {
            const double v = w.f[f][c];
            const float hi = (float)v;
            reinterpret_cast<float2*>(w.f[f])[c] = make_float2(hi, (float)(v - (double)hi));
        } else {
            const float2 v = reinterpret_cast<const float2*>(w.f[f])[c];
            w.f[f][c] = (double)v.x + (double)v.y;
        }
    }
}
// block sizes of the grid-stride kernels: a multiple of 32 in [32, kThreads]
inline int clamp_block(int b) { return b < 32 ? 32 : (b > kThreads ? kThreads : (b / 32) * 32); }

// Launches a step kernel on `s`.  With `dep` it is a programmatic dependent
// launch: the grid may be scheduled while the previous kernel in the stream
// finishes, and every step kernel begins with dep_begin(), which waits for
// that kernel's completion before touching any state.  Inside a captured
// graph this becomes a programmatic edge; the order of effects is the same.
template <typename... KArgs, typename... Args>
void launch(bool dep, void (*kern)(KArgs...), int grid, int block, cudaStream_t s,
            Args... args) {
    if (!dep) {
        kern<<<grid, block, 0, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

}  // namespace

int scan_tiles(int64_t n) { return (int)((n + kScanTile - 1) / kScanTile); }

void launch_scan_i32(const int32_t* in, int32_t* out, int64_t n, const DemDev& d, int site,
                     cudaStream_t s) {
    const int nt = scan_tiles(n);
    if (nt == 0) {
        cudaMemsetAsync(out, 0, sizeof(int32_t), s);
        return;
    }
    k_scan_excl<int32_t, false><<<nt, kScanBlock, 0, s>>>(in, out, n, nt, d.scan_state[site],
                                                          &d.ctr->tickets[site], d.ctr, kSpinLimit);
}

void launch_broadphase(const DemDev& d, const DemParams& p, int cur, bool multi, bool all,
                       int ntiles_cells, cudaStream_t s) {
    if (p.n == 0) return;
    const int nb = blocks_for(p.n, kThreads);
    const bool dep = p.dep != 0;
    launch(dep, multi ? k_hash<true> : k_hash<false>, nb, kThreads, s, d, p, cur, all ? 1 : 0);
    launch(dep, k_scan_excl<uint32_t, true>, ntiles_cells, kScanBlock, s,
           (const uint32_t*)d.cell_count, d.cell_start, (long long)p.T, ntiles_cells,
           d.scan_state[kScanCells], &d.ctr->tickets[kScanCells], d.ctr, kSpinLimit);
    launch(dep, k_scatter, nb, kThreads, s, d, p);
    launch(dep, multi ? k_canon<true> : k_canon<false>, nb, kThreads, s, d, p, cur);
}

// Largest cooperative grid of one k_search instantiation (resident blocks per
// SM from the occupancy calculator, times the SMs).
template <bool INIT, bool MULTI, int MINB>
int search_grid_limit(int sms) {
    static int per_sm = -1;
    if (per_sm < 0) {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_search<INIT, MULTI, MINB>, kThreads,
                                                          0) != cudaSuccess)
            nb = 1;
        per_sm = nb > 0 ? nb : 1;
    }
    return per_sm * sms;
}

template <bool INIT, bool MULTI, int MINB>
void launch_search_t(const DemDev& d, const DemParams& p, int cur, bool all, cudaStream_t s) {
    // one 8-lane group per particle, within the resident limit
    const int want = max(1, blocks_for((long long)p.n * kLanes, kThreads));
    const int grid = max(1, min(want, search_grid_limit<INIT, MULTI, MINB>(p.sms)));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_search<INIT, MULTI, MINB>, d, p, cur, all ? 1 : 0);
}

template <int MINB>
void launch_search_b(const DemDev& d, const DemParams& p, int cur, bool init, bool multi, bool all,
                     cudaStream_t s) {
    if (multi) launch_search_t<false, true, MINB>(d, p, cur, all, s);
    else if (init) launch_search_t<true, false, MINB>(d, p, cur, all, s);
    else launch_search_t<false, false, MINB>(d, p, cur, all, s);
}

void launch_search(const DemDev& d, const DemParams& p, int cur, bool init, bool multi, bool all,
                   const LaunchShape& sh, cudaStream_t s) {
    if (p.n == 0) return;
    if (sh.detect_blocks_per_sm == 3) launch_search_b<3>(d, p, cur, init, multi, all, s);
    else launch_search_b<4>(d, p, cur, init, multi, all, s);
}

void launch_force(const DemDev& d, const DemParams& p, int nxt, bool multi, const LaunchShape& sh,
                  cudaStream_t s) {
    if (p.n == 0 || p.cap == 0) return;
    const int block = clamp_block(sh.force_block);
    const int grid = min(blocks_for(p.cap, block), max(sh.force_grid, 1));
    if (p.precision == 1) {
        // FP32 mode: register budget for 3 (default) or 4 blocks of 256 per SM
        if (sh.force_blocks_per_sm == 4)
            launch(p.dep != 0, multi ? k_force4<float, true> : k_force4<float, false>, grid, block,
                   s, d, p, nxt);
        else
            launch(p.dep != 0, multi ? k_force<float, true> : k_force<float, false>, grid, block, s,
                   d, p, nxt);
    } else if (p.tab) {
        launch(p.dep != 0, k_force_tab, grid, block, s, d, p, nxt);
    } else {
        launch(p.dep != 0, multi ? k_force<double, true> : k_force<double, false>, grid, block, s,
               d, p, nxt);
    }
}

void launch_integrate(const DemDev& d, const DemParams& p, int cur, bool multi,
                      const LaunchShape& sh, cudaStream_t s) {
    if (p.n == 0) return;
    const int block = clamp_block(sh.integrate_block);
    if (split_integrator(sh, p.n, p.sms)) {
        const int nb = blocks_for(p.n, 32);
        if (p.tab)
            launch(p.dep != 0, k_integrate_split_tab, nb, kSplitThreads, s, d, p, cur);
        else if (p.precision == 1)
            launch(p.dep != 0, multi ? k_integrate_split<true, true> : k_integrate_split<false, true>,
                   nb, kSplitThreads, s, d, p, cur);
        else
            launch(p.dep != 0,
                   multi ? k_integrate_split<true, false> : k_integrate_split<false, false>, nb,
                   kSplitThreads, s, d, p, cur);
        return;
    }
    const int nb = blocks_for(p.n, block);
    if (p.tab)
        launch(p.dep != 0, k_integrate_tab, nb, block, s, d, p, cur);
    else if (p.precision == 1)
        launch(p.dep != 0, multi ? k_integrate3<true> : k_integrate3<false>, nb, block, s, d, p,
               cur);
    else
        launch(p.dep != 0, multi ? k_integrate<true, false> : k_integrate<false, false>, nb, block,
               s, d, p, cur);
}

// Active entries of a slot's row (its contacts (i, j), j > i, sorted by j).
__device__ __forceinline__ void io_row(const DemDev& d, int cur, int cap, int i, int& e0,
                                       int& e1) {
    const int C = min((int)d.ctr->alloc[cur].rows, cap);
    e0 = max(d.row_start[cur][i], 0);
    e1 = min(d.row_start[cur][i] + d.row_len[cur][i], C);
}
__global__ void k_io_count(DemDev d, int cur, int cap, int p0, int n, int32_t* cnt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = p0 + t;
    int e0, e1, m = 0;
    io_row(d, cur, cap, i, e0, e1);
    const ContactSoA w = d.c[cur];
    for (int e = e0; e < e1; ++e) m += ((w.fl[e] & kActive) && w.ci[e] == i) ? 1 : 0;
    cnt[t] = m;
}
struct IORecord {
    int32_t i, j, bonded, pad;
    double k[3], F[3];
};
static_assert(sizeof(IORecord) == 64, "the DemIOContact layout");
__global__ void k_io_fill(DemDev d, int cur, int cap, int p0, int n, const int32_t* off,
                          int pairs, IORecord* out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = p0 + t;
    int e0, e1;
    io_row(d, cur, cap, i, e0, e1);
    const ContactSoA w = d.c[cur];
    int q = off[t];
    for (int e = e0; e < e1; ++e) {
        const uint32_t fl = w.fl[e];
        if (!(fl & kActive) || w.ci[e] != i) continue;
        IORecord r;
        r.i = t;
        r.j = w.cj[e] - p0;
        r.bonded = (fl & kBonded) ? 1 : 0;
        r.pad = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            r.k[c] = w.f[CK + c][e];
            if (pairs) {
                const float2 v = reinterpret_cast<const float2*>(w.f[CF + c])[e];
                r.F[c] = (double)v.x + (double)v.y;
            } else {
                r.F[c] = w.f[CF + c][e];
            }
        }
        out[q++] = r;
    }
}
// Active contacts and active bonds owned by slots [p0, p0 + n) (the scene
// counters of dem_get_stats), added into tot[0] and tot[1].
__global__ void k_range_counts(DemDev d, int cur, int cap, int p0, int n,
                               unsigned long long* tot) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned act = 0, bnd = 0;
    if (t < n) {
        const int i = p0 + t;
        int e0, e1;
        io_row(d, cur, cap, i, e0, e1);
        const ContactSoA w = d.c[cur];
        for (int e = e0; e < e1; ++e) {
            const uint32_t fl = w.fl[e];
            if ((fl & kActive) && w.ci[e] == i) {
                ++act;
                bnd += (fl & kBonded) ? 1u : 0u;
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        act += __shfl_down_sync(0xffffffffu, act, o);
        bnd += __shfl_down_sync(0xffffffffu, bnd, o);
    }
    if (lane_id() == 0 && (act | bnd)) {
        atomicAdd(&tot[0], (unsigned long long)act);
        atomicAdd(&tot[1], (unsigned long long)bnd);
    }
}
void launch_range_counts(const DemDev& d, int cur, int cap, int p0, int n,
                         unsigned long long* tot, cudaStream_t s) {
    if (n <= 0) return;
    k_range_counts<<<blocks_for(n, kThreads), kThreads, 0, s>>>(d, cur, cap, p0, n, tot);
}
void launch_io_count(const DemDev& d, int cur, int cap, int p0, int n, int32_t* cnt,
                     cudaStream_t s) {
    if (n <= 0) return;
    k_io_count<<<blocks_for(n, kThreads), kThreads, 0, s>>>(d, cur, cap, p0, n, cnt);
}
void launch_io_fill(const DemDev& d, int cur, int cap, int p0, int n, const int32_t* off,
                    bool pairs, void* out, cudaStream_t s) {
    if (n <= 0) return;
    k_io_fill<<<blocks_for(n, kThreads), kThreads, 0, s>>>(d, cur, cap, p0, n, off, pairs ? 1 : 0,
                                                           static_cast<IORecord*>(out));
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
// Self-test of d2f / f2d against the hardware conversions: thread t draws a
// binary64 value (random significand, exponents spread over and beyond the
// binary32 range, every 8th one a rounding tie) and a binary32 value, and
// counts results whose bits differ.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__global__ void k_selftest_conv(long long n, unsigned long long seed, unsigned long long* bad) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const unsigned long long r1 = mix64(seed ^ (unsigned long long)t);
    const unsigned long long r2 = mix64(r1);
    // exponent field within [1023-160, 1023+160]: subnormal, normal and overflowing results
    const unsigned long long ex = 1023ull - 160ull + (r2 % 321ull);
    unsigned long long sig = r1 & 0xfffffffffffffull;
    if ((t & 7) == 0) sig = (sig & ~0x3fffffffull) | 0x10000000ull;  // exact tie
    unsigned long long bits = ((r2 >> 63) << 63) | (ex << 52) | sig;
    if ((t & 15) == 1) bits &= 0x8000000000000000ull;  // ±0
    const double x = __longlong_as_double((long long)bits);
    const unsigned a = __float_as_uint(d2f(x)), b = __float_as_uint(__double2float_rn(x));
    const float f = __uint_as_float((t & 15) == 2 ? ((unsigned)r2 & 0x80000000u) : (unsigned)r2);
    const unsigned long long c = (unsigned long long)__double_as_longlong(f2d(f));
    const unsigned long long e = (unsigned long long)__double_as_longlong((double)f);
    if (a != b) atomicAdd(bad, 1ull);
    if (c != e && !isnan(f)) atomicAdd(bad + 1, 1ull);
    // rcp_nr on positive values across the normal FP32 range: within 2 ulp of
    // the correctly rounded reciprocal
    const double xr = __longlong_as_double((long long)(((1023ull - 100ull + (r2 % 201ull)) << 52) |
                                                       (r1 & 0xfffffffffffffull)));
    const long long u1 = __double_as_longlong(rcp_nr(xr)), u2 = __double_as_longlong(__drcp_rn(xr));
    const long long du = u1 > u2 ? u1 - u2 : u2 - u1;
    if (du > 2) atomicAdd(bad + 2, 1ull);
    // half_exact on the values drawn for d2f (zeros, subnormals, normals) and
    // on the FP32-widened ones: bit-identical to x * 0.5
    if (__double_as_longlong(half_exact(x)) != __double_as_longlong(x * 0.5)) atomicAdd(bad + 3, 1ull);
    const double xf = (double)f;
    if (!isnan(xf) && __double_as_longlong(half_exact(xf)) != __double_as_longlong(xf * 0.5))
        atomicAdd(bad + 3, 1ull);
    // and on the exponent fields at the edges: 0 (subnormal), 1, 2, 0x7fe, 0x7ff (inf)
    const unsigned long long edge[5] = {0ull, 1ull, 2ull, 0x7feull, 0x7ffull};
    const unsigned long long xe_bits = ((r1 >> 63) << 63) | (edge[(r2 >> 32) % 5ull] << 52) |
                                       ((t & 3) == 3 ? 0ull : (r2 & 0xfffffffffffffull));
    const double xe = __longlong_as_double((long long)xe_bits);
    if (!isnan(xe) && __double_as_longlong(half_exact(xe)) != __double_as_longlong(xe * 0.5))
        atomicAdd(bad + 3, 1ull);
    // the integrator's zero-spin and zero-torque skips: where they apply, the
    // quaternion chains with 𝛚 = +0 return 𝐪 and the spin update returns 𝛚
    // (z is +0 at run time, so no rule of the compiler's folds the products)
    const double z = (double)(t >> 62);
    const double q0 = x, q1 = xf, q2 = xe, q3 = (t & 2) ? -xr : 0.0;
    const unsigned long long bq[4] = {
        (unsigned long long)__double_as_longlong(q0), (unsigned long long)__double_as_longlong(q1),
        (unsigned long long)__double_as_longlong(q2), (unsigned long long)__double_as_longlong(q3)};
    if (finite_not_negzero(q0) && finite_not_negzero(q1) && finite_not_negzero(q2) &&
        finite_not_negzero(q3)) {
        const double n[4] = {__fma_rn(-q3, z, __fma_rn(-q2, z, __fma_rn(-q1, z, q0))),
                             __fma_rn(-q3, z, __fma_rn(q2, z, __fma_rn(q0, z, q1))),
                             __fma_rn(q3, z, __fma_rn(q1, z, __fma_rn(q0, z, q2))),
                             __fma_rn(-q2, z, __fma_rn(q1, z, __fma_rn(q0, z, q3)))};
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if ((unsigned long long)__double_as_longlong(n[k]) != bq[k]) atomicAdd(bad + 3, 1ull);
    }
    const double ia = fabs(xf), ib = fabs(xe);
    if (product_finite(ia, ib) && not_negzero(x) &&
        __double_as_longlong(__fma_rn(z, ia * ib, x)) != __double_as_longlong(x))
        atomicAdd(bad + 3, 1ull);
    // the identity orientation: |𝐪|² of (1, +0, +0, +0) as the integrator
    // forms it is 1, and rsqrt(1) is exactly 1
    const double one = 1.0 + z;
    const double nq2 = __fma_rn(z, z, __fma_rn(z, z, __fma_rn(z, z, one * one)));
    if (__double_as_longlong(rsqrt(nq2)) != 0x3ff0000000000000ll) atomicAdd(bad + 3, 1ull);
}

void launch_selftest_conv(long long n, unsigned long long seed, unsigned long long* bad,
                          cudaStream_t s) {
    if (n <= 0) return;
    k_selftest_conv<<<blocks_for(n, kThreads), kThreads, 0, s>>>(n, seed, bad);
}

// Bounded-wait self-test: two blocks meet at the grid barrier that the fused
// pair search uses; with `missing`, block 1 returns before it arrives, so
// block 0's wait must give up after `spin_limit` polls (kErrTimeout) and
// return.  Launched cooperatively, so both blocks are resident.
__global__ void k_selftest_barrier(DevCounters* c, int missing, unsigned long long spin_limit) {
    if (missing && blockIdx.x == 1) return;
    grid_sync(c, spin_limit);
}

cudaError_t launch_selftest_wait(int which, int missing, unsigned long long spin_limit,
                                 DevCounters* c, unsigned long long* state, uint32_t* io,
                                 cudaStream_t s) {
    if (which == 0) {
        void* args[] = {&c, &missing, &spin_limit};
        return cudaLaunchCooperativeKernel((const void*)k_selftest_barrier, dim3(2), dim3(32),
                                           args, 0, s);
    }
    // The scan of 2·kScanTile values in two tiles: every block draws a ticket
    // (tile = ticket mod 2).  With `missing`, one block runs: it draws ticket
    // 1 (the counter starts at 1), i.e. tile 1, whose look-back waits for
    // tile 0, which never publishes.  io holds 2·kScanTile inputs followed by
    // 2·kScanTile + 1 outputs.
    const long long count = 2LL * kScanTile;
    if (missing) {
        cudaError_t e = cudaMemsetAsync(&c->tickets[0], 0, sizeof(unsigned long long), s);
        if (e != cudaSuccess) return e;
        const unsigned long long one = 1ull;
        e = cudaMemcpyAsync(&c->tickets[0], &one, sizeof(one), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return e;
        e = cudaStreamSynchronize(s);  // `one` lives on this stack frame
        if (e != cudaSuccess) return e;
    }
    k_scan_excl<uint32_t, false><<<missing ? 1 : 2, kScanBlock, 0, s>>>(
        io, io + count, count, 2, state, &c->tickets[0], c, spin_limit);
    return cudaGetLastError();
}


// FP32 positions of slots [first, first + n) from the FP64 ones; with a
// flag buffer `fb` >= 0 (the one the next step reads), a scene with a particle
// now beyond skin/2 of its list position is flagged for a full search, as
// after an integration.
template <bool MULTI>
__global__ void k_refresh_pos32(DemDev d, DemParams p, int first, int n, int fb) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = first + t;
    const int sc = slot_scene<MULTI>(d, i);
    if (MULTI && sc < 0) return;
    const SceneParams& S = scene_rec<MULTI>(d, p, sc);
    const float fx = d2f(d.px[i] - S.dmin[0]), fy = d2f(d.py[i] - S.dmin[1]),
                fz = d2f(d.pz[i] - S.dmin[2]);
    d.pos32[i] = make_float4(fx, fy, fz, reach32(fx, fy, fz, d.rm32[i].z));
    if (fb >= 0 && (!(S.f_half_skin > 0.0f) || left_skin(S, fx, fy, fz, d.xref[i])) &&
        d.sflags[fb][sc] == 0u)
        atomicOr(&d.sflags[fb][sc], 1u);
}
void launch_refresh_pos32(const DemDev& d, const DemParams& p, bool multi, int first, int n,
                          int fb, cudaStream_t s) {
    if (n <= 0) return;
    const int g = blocks_for(n, kThreads);
    fb = fb == 0 || fb == 1 ? fb : -1;
    if (multi) k_refresh_pos32<true><<<g, kThreads, 0, s>>>(d, p, first, n, fb);
    else k_refresh_pos32<false><<<g, kThreads, 0, s>>>(d, p, first, n, fb);
}

// Particle state exchange: up to kXferFields fields, each a k-component
// record per particle (the host's layout) <-> k columns of the structure of
// arrays at slots [p0, p0 + n).  A record array is device-accessible caller
// memory (page-locked host or device) or the library's staging copy.
// A block moves kXferBlock particles, all fields at once: per field their
// k·kXferBlock record values are one contiguous range (whole 128-byte lines,
// which matters most for page-locked host memory across the chip-to-chip
// link), one value per thread, every field's loads issued before the first
// store, then transposed through shared memory and written column by column.
// Small blocks put a 17,576-particle scene on every SM.  REFRESH (an upload
// to a single-scene handle, field `posf` the positions): the FP32 position
// and the skin test of each slot, from the uploaded values, as
// k_refresh_pos32 does; with x.arm, it also arms the fused download
// (HostOut) of the exchanged step that follows.
constexpr int kXferBlock = 64;
static_assert(4 * kXferBlock <= kThreads, "one record value per thread and field");
template <bool REFRESH>
__global__ void __launch_bounds__(kThreads)
    k_xfer(XferSet x, int n, int p0, bool to_cols, DemDev d, DemParams p, int posf, int fb) {
    __shared__ double tile[kXferCols * kXferBlock];
    __shared__ double* s_col[kXferCols];
    __shared__ int s_off[kXferCols], s_k[kXferCols], s_foff[kXferFields], s_ncol;
    const int base = blockIdx.x * kXferBlock;
    const int m = min(kXferBlock, n - base);  // particles of this block
    const int t = threadIdx.x;
    if (t == 0) {
        int cc = 0, off = 0;
        for (int f = 0; f < x.nf; ++f) {
            s_foff[f] = off;
            for (int c = 0; c < x.k[f]; ++c, ++cc) {
                s_col[cc] = x.col[f][c];
                s_off[cc] = off + c;  // value c of particle q at off + k·q + c
                s_k[cc] = x.k[f];
            }
            off += x.k[f] * kXferBlock;
        }
        s_ncol = cc;
        if (x.err_dst && blockIdx.x == 0) *x.err_dst = __ldcg(x.err_src);
        // the step's integrators run after this kernel (stream order)
        if (REFRESH && x.arm && blockIdx.x == 0) d.ctr->hout = x.hout;
    }
    if (to_cols) {
        double v[kXferFields];
#pragma unroll
        for (int f = 0; f < kXferFields; ++f) {
            v[f] = 0.0;
            if (f < x.nf && t < x.k[f] * m) v[f] = x.rec[f][(size_t)x.k[f] * base + t];
        }
        __syncthreads();  // the column table
#pragma unroll
        for (int f = 0; f < kXferFields; ++f)
            if (f < x.nf && t < x.k[f] * m) tile[s_foff[f] + t] = v[f];
        __syncthreads();
        for (int e = t; e < s_ncol * kXferBlock; e += kThreads) {
            const int cc = e / kXferBlock, q = e % kXferBlock;
            if (q < m) s_col[cc][p0 + base + q] = tile[s_off[cc] + s_k[cc] * q];
        }
        if (REFRESH && t < m) {
            const int i = p0 + base + t;
            const SceneParams& S = scene_rec<false>(d, p, 0);
            const double* xp = tile + s_foff[posf] + 3 * t;
            const float fx = d2f(xp[0] - S.dmin[0]), fy = d2f(xp[1] - S.dmin[1]),
                        fz = d2f(xp[2] - S.dmin[2]);
            d.pos32[i] = make_float4(fx, fy, fz, reach32(fx, fy, fz, d.rm32[i].z));
            if (fb >= 0 && (!(S.f_half_skin > 0.0f) || left_skin(S, fx, fy, fz, d.xref[i])) &&
                d.sflags[fb][0] == 0u)
                atomicOr(&d.sflags[fb][0], 1u);
        }
    } else {
        __syncthreads();  // the column table
        for (int e = t; e < s_ncol * kXferBlock; e += kThreads) {
            const int cc = e / kXferBlock, q = e % kXferBlock;
            if (q < m) tile[s_off[cc] + s_k[cc] * q] = s_col[cc][p0 + base + q];
        }
        __syncthreads();
#pragma unroll
        for (int f = 0; f < kXferFields; ++f)
            if (f < x.nf && t < x.k[f] * m) x.rec[f][(size_t)x.k[f] * base + t] = tile[s_foff[f] + t];
    }
}
void launch_xfer(const XferSet& x, int n, int p0, bool to_cols, cudaStream_t s) {
    if (n <= 0 || x.nf <= 0) return;
    k_xfer<false><<<blocks_for(n, kXferBlock), kThreads, 0, s>>>(x, n, p0, to_cols, DemDev{},
                                                                  DemParams{}, -1, -1);
}
void launch_xfer_pos(const XferSet& x, int n, const DemDev& d, const DemParams& p, int posf,
                     int fb, cudaStream_t s) {
    if (posf < 0 || posf >= x.nf || x.k[posf] != 3) return launch_xfer(x, n, 0, true, s);
    if (n <= 0) return;
    fb = fb == 0 || fb == 1 ? fb : -1;
    k_xfer<true><<<blocks_for(n, kXferBlock), kThreads, 0, s>>>(x, n, 0, true, d, p, posf, fb);
}

void launch_recode(const DemDev& d, int buf, int n, bool to_pairs, cudaStream_t s) {
    if (n <= 0) return;
    k_recode<<<blocks_for(n, kThreads), kThreads, 0, s>>>(d.c[buf], n, to_pairs ? 1 : 0);
}
void launch_morton(const DemDev& d, const DemParams& p, uint32_t* morton, cudaStream_t s) {
    if (p.n == 0) return;
    k_morton<<<blocks_for(p.n, kThreads), kThreads, 0, s>>>(d, p, morton);
}

}  // namespace dem
