// dem_internal.h — device data layout and kernel launchers of libdem_sm100a.so.
//
// Layout in HBM.  A handle is an arena of particle slots holding one or more
// independent scenes (a single scene for dem_create; many for the batched and
// served modes).  Each scene owns a contiguous range of particle slots and a
// contiguous range of bucket-table entries; its constants live in a
// SceneParams record.
//  * particles: structure of arrays over all slots, FP64;
//  * broad phase: per-particle cell record (int4: ijk + octant bits), bucket
//    id, a bucket table of counts / starts (the reference's hash_table, one
//    range per scene), and particle copies in bucket-sorted order (double4
//    x,y,z,r and a float4 copy relative to the scene's domain_min for the
//    distance pre-filter);
//  * contacts: two buffers (the reference's contacts / contacts_temp rolling
//    pair), each a structure of arrays of rows — row i holds the contacts
//    (i, j) with j > i, sorted by j, at [row_start[i], row_start[i]+row_len[i]);
//    rows are placed by an atomic allocator, so the buffers need no scan;
//  * per-contact force contributions (9 FP64 values) and a per-particle list
//    of incoming contacts (those where the particle is j) used to sum forces
//    per particle in a fixed order, without floating-point atomics.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace dem {

constexpr uint32_t kActive = 1u;
constexpr uint32_t kBonded = 2u;

// error bits raised on the device (mapped to DEM_ERR_* on the host)
constexpr int kErrCapacity = 1;
constexpr int kErrTimeout = 2;
constexpr int kErrRange = 4;

// scene modes (SceneParams::mode)
constexpr int kModeFree = 0;    // slot range not in use: particles ignored, no contacts
constexpr int kModeFrozen = 1;  // state kept (contacts carried), no stepping
constexpr int kModeStep = 2;    // `simulate!`
constexpr int kModeInit = 3;    // `initialize!` (bonds from r₀), no integration

constexpr uint32_t kNoBucket = 0xffffffffu;

// Neighbour lists.  A full pair search (the reference's cp_list over the
// octant buckets) runs only for scenes whose rebuild flag is set; it also
// records, per particle, the partners j > i within rᵢ + rⱼ + skin (the
// neighbour list) and the particle's position.  Until any particle of the
// scene has moved by skin/2 from that position, every pair that can touch is
// on the list, so the other steps test only the list.  Contact ends still
// follow the reference's cells (computed from the current positions).

struct ContactSoA {
    int32_t* ci;
    int32_t* cj;
    uint32_t* fl;
    int32_t* src;   // slot of the contact in the other buffer (its carried state), -1 new
    double* f[15];  // kx ky kz | Fx Fy Fz | tix tiy tiz | tjx tjy tjz | sx sy sz
};
enum ContactField { CK = 0, CF = 3, CTI = 6, CTJ = 9, CS = 12 };

// Constants of one scene (host-derived).  For a single-scene handle the record
// travels in the kernel parameters; for an arena it is an array in HBM.
struct SceneParams {
    int mode;
    int p0, n;                // particle slots [p0, p0 + n)
    uint32_t t0, H, Hmask;    // search buckets [t0, t0 + H); Hmask = H-1 if H is a power of 2
    uint32_t Href, Href_mask; // the reference's hash-table size (src/executor.jl:266-267)
    int has_wall;
    int same_grid;            // search cells are the reference's cells (cell == cell_ref)
    double dmin[3];
    double cell, inv_cell;           // search cell size
    double cell_ref, inv_cell_ref;   // the reference's cell size 4 rₘₐₓ (src/executor.jl:265)
    double dt, tol;
    double grav[3];
    double damping;
    // particle-particle Hertz-Mindlin constants (surface [1,1], materials 1,1)
    // cgn = -2β·sqrt(5/3·Y*), cgt = -2β·sqrt(20/3·G*): γₙ = cgn·sqrt(m*·sqrt(R*Δn))
    double pp_mu, pp_Ys, pp_Gs, pp_cgn, pp_cgt;
    // EBPM bond constants (surface [1,1])
    double b_inv1pnu, b_sc, b_st, b_ss;
    // wall (wall_normal, wall_distance) and particle-wall constants
    double wn[3], wd;
    double wR[9], wRinv[9];  // contact frame of the wall and its inverse
    double pw_mu, pw_Ys, pw_Gs, pw_cgn, pw_cgt;
    // FP32 copies for the FP32 force mode (no conversions in the force kernel)
    float f_dt, f_inv1pnu, f_sc, f_st, f_ss;
    float f_mu, f_kn, f_kt, f_cgn, f_cgt;  // μ, 4/3·Y*, 8·G*, cgn, cgt (particle-particle)
    float f_tol4;                          // 4·tolerance² (degenerate frame test)
    float f_tol1;                          // tolerance²·(1 - 2^-10), rounded down
    // FP32 screen of the cell computation: 1/cell and max|dmin|/cell
    float f_inv_cell, f_dmin_cells, f_inv_cell_ref, f_dmin_cells_ref;
    // neighbour-list skin (0: a full search every step) and half of it in FP32
    double skin;
    float f_skin, f_half_skin;
    double hdt2;            // dt²/2
    double tol2_lo, tol2_x4;  // tolerance²·(1 - 2^-30) and 4·tolerance² (contact frame)
    float f_wn[3], f_wc0;   // FP32 wall normal and n·domain_min - wall_distance (wall screen)
};

// Material, surface and wall tables of a scene built with dem_create_tables
// (the reference's GlobalData.materials / surfaces / walls, src/types.jl:9-27,
// 58-62, which its `solve` fills with one particle material, one wall
// material and one wall, src/executor.jl:282-315).  Indices are 0-based
// (the reference's mid - 1).  Pair constants are surfaces[a, b] with
// materials a and b; wall constants hold, per particle material a, the
// particle-wall constants of surfaces[a, wall material].
constexpr int kMaxMaterials = 8;
constexpr int kMaxWalls = 8;
struct PairConst {
    double mu, Ys, Gs, cgn, cgt;              // Hertz-Mindlin: μ, Y*, G*, γ coefficients
    double ratio, E, nu, inv1pnu, sc, st, ss;  // EBPM: ρ, E, ν, 1/(1+ν), σc, σt, σs
};
struct WallConst {
    double wn[3], wd;
    double wR[9], wRinv[9];  // contact frame of the wall and its inverse
    float f_wn[3], f_wc0;    // FP32 normal and n·domain_min - distance (the wall screen)
    double mu[kMaxMaterials], Ys[kMaxMaterials], Gs[kMaxMaterials];
    double cgn[kMaxMaterials], cgt[kMaxMaterials];
};
struct MatTables {
    int nmat, nwall;
    PairConst pair[kMaxMaterials * kMaxMaterials];  // [a * nmat + b]
    WallConst wall[kMaxWalls];
};

struct SceneCounters {
    unsigned long long broken, ended, created, warn_gap, warn_damp;
    unsigned long long searches;  // steps that ran the full pair search
};

// Contacts placed in one contact buffer: all of them (rows) and, of them,
// the bonds.  One 64-bit word, so that a warp places its rows and its entries
// of the force pass's type-ordered list (DemDev::tlist) with one atomic.
struct alignas(8) RowCounter {
    unsigned int rows, bonds;
};

// The fused exchange of dem_step_exchange: the upload arms it, and the
// integrator of the last of `steps_left` steps writes the particle state
// straight into the caller's device-accessible page-locked records (the
// DemParticleState fields in their order: pos, vel, omega, quat, force,
// moment, wall_shear; nullptr: not written) and then the device error word
// into `err`.  With `qin` / `wsin` set, the upload left the orientations /
// the first wall's shear history out and the integrator of the first step
// (steps_left == steps_total) reads them from these records instead.  Every
// integrator launch of an armed handle counts its blocks in `done`; the last
// block out decrements `steps_left`, so the arming lasts exactly steps_total
// launches.  An integrator that cannot use the records (one thread per
// particle: the host then uploads every field) only counts, and `err` keeps
// the host's sentinel, so the host reads the state the usual way.
constexpr int kHostOutFields = 7;
constexpr int kHostOutRows = 22;  // 3+3+3+4+3+3+3 values per particle
struct HostOut {
    double* rec[kHostOutFields];
    const double* qin;   // orientations (4n), or nullptr: uploaded
    const double* wsin;  // first wall's shear history (3n), or nullptr: uploaded
    int* err;
    int steps_left, steps_total;
    unsigned int done;
    // bit f: record f is the same memory as the step's input of that field
    // (a one-step exchange in place), so values the step left bit for bit
    // unchanged are already there and are not written again
    unsigned int same;
};

struct DevCounters {
    int error;
    unsigned int bmax;        // largest bucket id of this step (k_hash), reset by k_canon
    unsigned int cell_limit;  // buckets [0, cell_limit) have valid starts this step
    unsigned int pad;
    RowCounter alloc[2];            // contacts placed in each contact buffer
    unsigned long long tickets[2];  // tile tickets of the scan sites (never reset)
    unsigned int bar_count, bar_gen;  // grid barrier of the fused search (arrivals, generation)
    unsigned int hashed[2];           // particles hashed by the step reading buffer cur
    // inspection of the fused pair search (DemParams::debug_enum): candidate
    // pairs (i, j > i) it visited and the wrapping sum of enum_mix(i, j)
    unsigned long long enum_pairs, enum_hash;
    HostOut hout;  // the fused download (zero: not armed)
};

// scan sites: each has its own ticket counter and tile-state array
constexpr int kScanCells = 0;
constexpr int kScanDebug = 1;

// Device pointers of one arena (passed by value to every kernel).
struct DemDev {
    // particles
    double *px, *py, *pz, *vx, *vy, *vz, *wx, *wy, *wz;
    double *qw, *qx, *qy, *qz;
    double *m, *inv_m, *r, *r0, *inv_inertia;
    double *b_invA, *b_rbI;        // bond section constants for rb = ρ·r (1/A, rb/I)
    double *b_EA, *b_EI, *b_phic;  // E·A, E·I and 20/3·(1+ν)·rb² for rb = ρ·r
    float4* bk32;                  // FP32 (b_phic, b_EI, b_EA, b_invA)
    float4* rm32;                  // FP32 (b_rbI, m, r, 0)
    double *fx, *fy, *fz, *tx, *ty, *tz;  // totals of the last step
    double *wsx, *wsy, *wsz;              // wall shear history: wall w of slot i at
                                          // [w * DemParams::wstride + i]
    const MatTables* mt;                  // tables of a dem_create_tables handle, else null
    const uint8_t* mid;                   // its grains' material indices, else null
    int32_t* scene_of;                    // arena: scene of each slot (-1 free); null otherwise
    // neighbour lists: kvl partners per slot, their count, the position at the
    // last full search and the current position (FP32, relative to the
    // scene's domain_min, .w = reach32); rebuild flags per scene and buffer
    int32_t* vl;
    int32_t* vl_len;
    float4* xref;
    float4* pos32;
    uint32_t* sflags[2];
    uint8_t* path;  // this step: kind (0 free, 1 full search, 2 list) | scene mode << 2
    SceneParams* sp;                      // arena: scene records; null otherwise
    SceneCounters* sctr;                  // per-scene event counters
    // broad phase
    int4* cellinfo;        // search cell ijk; .w = octant bits | scene index << 3
    int4* scell;           // cellinfo in sorted order
    int2* srow;            // (row_start, row_len) of the current buffer, sorted order
    int4* refcell;         // arena: the reference's cell ijk + octant (when grids differ)
    uint32_t* bucket;      // bucket of each particle (kNoBucket when not hashed)
    uint32_t* cell_count;  // table entries, zero between steps
    uint32_t* cell_start;  // table entries + 1
    uint32_t* tile_sums;   // bucket-count sums per scan tile (fused search)
    uint32_t* unsorted;    // bucket-grouped, arbitrary order inside a bucket
    uint32_t* sorted;      // bucket-grouped, ascending index inside a bucket
    double4_32a* spos;     // (x, y, z, r) in sorted order
    float4* spos32;        // (x-ox, y-oy, z-oz, r) in FP32, sorted order
    // contacts
    ContactSoA c[2];
    int32_t* row_start[2];  // first slot of each particle's row
    int32_t* row_len[2];    // entries in the row
    int32_t* stash;       // n * kstash new partners of this step
    uint8_t* keep;        // cap, survival flags of the current buffer
    int32_t* tlist;       // cap, the next buffer's contacts by type for the force pass:
                          // bonds at [0, bonds), the others at cap-1-k, k in
                          // [0, rows - bonds)
    int32_t* in_cnt;      // zero between steps
    int2* in_list;        // n * kin: (contact slot, owner i) of contacts where the particle is j
    // Contact columns 𝐅ᵢ, 𝛕ᵢ, 𝛕ⱼ hold FP64 values in the FP64 force mode and
    // FP32 (hi, lo) pairs in the FP32 force mode.
    double* contrib;      // 9 * cap, [field][contact]
    float* contrib32;     // 9 * cap, the FP32 force mode's contributions
    // scan scratch: tile states of each scan site
    unsigned long long* scan_state[2];
    DevCounters* ctr;
};

// Arena-wide constants (passed by value).
struct DemParams {
    int n;          // particle slots processed by a step (all in use lie below)
    int cap;        // contact capacity
    int kstash;     // new partners per particle per step
    int kin;        // incoming contacts per particle
    uint32_t T;     // bucket-table entries processed by a step (all in use lie below)
    int precision;  // 0 = FP64, 1 = FP32 force
    int kvl;        // neighbour-list capacity per particle
    int ns;         // scene records
    int sms;        // streaming multiprocessors (grid-stride launch sizes)
    int dep;        // a step's kernels: 0 ordinary launches, 1 programmatic dependent
                    // launches, 2 the same with the successor scheduled early
    int debug_enum; // 1: the pair search counts its candidate pairs (never in a graph)
    int tab;        // 1: a single scene with material / wall tables (DemDev::mt, mid)
    int list_lanes; // neighbour-list update: 0 auto, 1 or 4 lanes per particle
    int wstride;    // slots per wall-shear column
    SceneParams s0; // the scene of a single-scene handle
};

// Launch shape of the grid-stride kernels (block sizes are multiples of 32 up
// to 256; grids are upper bounds).  Results do not depend on it: every kernel
// computes the same values for any shape.
struct LaunchShape {
    int force_block, force_grid;
    int compact_block, compact_grid;
    int integrate_block;
    int detect_blocks_per_sm;  // register budget of the pair search and the list update:
                               // 3 or 4 blocks per SM
    int force_blocks_per_sm;   // register budget of the FP32 force kernel: 0 (none) or 4
    int dependent_launch;      // 0 ordinary, 1 programmatic dependent, 2 with early trigger
    int list_lanes;            // neighbour-list update: 0 auto, 1 or 4 lanes per particle
    int integrate_lanes;       // integrator: 0 auto, 1 or 4 lanes per particle
};

// The integrator layout: split over four warps per 32 particles
// (k_integrate_split) where one thread per particle would leave the SM
// sub-partitions with at most two warps each, or as the shape asks.
inline bool split_integrator(const LaunchShape& sh, long long n, int sms) {
    return sh.integrate_lanes == 4 || (sh.integrate_lanes == 0 && n <= (long long)sms * 256);
}

// ---- launchers (dem_kernels.cu) --------------------------------------------
// All launches go to `s`.  `cur` selects the contact buffer that holds the
// state at the start of the step; the step writes buffer cur^1.  `multi`
// selects the arena kernels (per-slot scene records) over the single-scene ones.
// `all`: hash every particle (otherwise only the scenes that search this step)
void launch_broadphase(const DemDev& d, const DemParams& p, int cur, bool multi, bool all,
                       int n_scan_tiles_cells, cudaStream_t s);

// The full pair search of the scenes that run it this step, fused into one
// cooperative launch (hash, bucket scan, counting sort, canonical order,
// cp_list enumeration with update_contacts! / init_bonds!); a step whose
// scenes all test their neighbour lists ends it at once.  `all`: every
// particle searches (bond initialisation).
void launch_search(const DemDev& d, const DemParams& p, int cur, bool init, bool multi, bool all,
                   const LaunchShape& sh, cudaStream_t s);
void launch_force(const DemDev& d, const DemParams& p, int nxt, bool multi, const LaunchShape& sh,
                  cudaStream_t s);
void launch_integrate(const DemDev& d, const DemParams& p, int cur, bool multi,
                      const LaunchShape& sh, cudaStream_t s);

// save_single's contact records (src/utils.jl:48-69): per slot of
// [p0, p0 + n) the number of active entries of its row in buffer `cur`
// (cnt[n]); then, from their exclusive scan `off` (n + 1 entries), the
// records themselves (64 bytes each: i, j, bonded, pad, 𝐤, 𝐅ᵢ; indices
// relative to p0; 𝐅ᵢ decoded from FP32 hi/lo pairs when `pairs`)
void launch_io_count(const DemDev& d, int cur, int cap, int p0, int n, int32_t* cnt,
                     cudaStream_t s);
// active contacts and bonds owned by slots [p0, p0 + n), added into tot[0..1]
void launch_range_counts(const DemDev& d, int cur, int cap, int p0, int n,
                         unsigned long long* tot, cudaStream_t s);
void launch_io_fill(const DemDev& d, int cur, int cap, int p0, int n, const int32_t* off,
                    bool pairs, void* out, cudaStream_t s);

// debug: cp_list materialisation on the current bucket arrays (single scene)
void launch_cplist_count(const DemDev& d, const DemParams& p, int32_t* cnt, cudaStream_t s);
void launch_cplist_fill(const DemDev& d, const DemParams& p, const int32_t* off, int32_t* cp,
                        cudaStream_t s);
void launch_morton(const DemDev& d, const DemParams& p, uint32_t* morton, cudaStream_t s);
// particle state exchange: per field, k-component records <-> k columns,
// slots [p0, p0 + n); to_cols: records -> columns
constexpr int kXferFields = 7;
constexpr int kXferCols = 22;  // columns of all exchangeable fields (3+3+3+4+3+3+3)
struct XferSet {
    double* rec[kXferFields];
    double* col[kXferFields][4];
    int k[kXferFields];
    int nf;
    const int* err_src;  // with err_dst (device-accessible): the kernel copies
    int* err_dst;        // the device error word (nullptr: no copy)
    int arm;             // an upload with positions: also arms the fused download
    HostOut hout;
};
void launch_xfer(const XferSet& x, int n, int p0, bool to_cols, cudaStream_t s);
// the upload of a single-scene handle whose field `posf` holds positions:
// also refreshes the FP32 positions of the uploaded slots and, with fb 0 or
// 1, flags a full search as launch_refresh_pos32 does
void launch_xfer_pos(const XferSet& x, int n, const DemDev& d, const DemParams& p, int posf,
                     int fb, cudaStream_t s);
// FP32 positions (pos32) of slots [first, first + n) from the FP64 positions;
// with fb 0 or 1, scenes with a particle beyond skin/2 of its list position
// are flagged for a full search in sflags[fb] (no test for fb < 0)
void launch_refresh_pos32(const DemDev& d, const DemParams& p, bool multi, int first, int n,
                          int fb, cudaStream_t s);
// re-encodes 𝐅ᵢ, 𝛕ᵢ, 𝛕ⱼ of contacts [0, n) of buffer `buf`: FP64 <-> FP32 hi/lo pairs
void launch_recode(const DemDev& d, int buf, int n, bool to_pairs, cudaStream_t s);
// exclusive scan of n int32 values into out[0..n] (out[n] = total)
void launch_scan_i32(const int32_t* in, int32_t* out, int64_t n, const DemDev& d, int site,
                     cudaStream_t s);

// self-test of the integer-pipe FP64<->FP32 conversions (bad[0]: narrowing,
// bad[1]: widening mismatches against the hardware)
void launch_selftest_conv(long long n, unsigned long long seed, unsigned long long* bad,
                          cudaStream_t s);
// self-test of the bounded device waits on the counters `c` (zeroed by the
// caller): which = 0 a grid barrier of two blocks, 1 a scan look-back over two
// tiles; `missing` = 1 leaves one party out (its block returns without
// arriving / its tile never publishes), so the wait must give up after
// `spin_limit` polls and raise kErrTimeout.
cudaError_t launch_selftest_wait(int which, int missing, unsigned long long spin_limit,
                                 DevCounters* c, unsigned long long* state, uint32_t* io,
                                 cudaStream_t s);

int scan_tiles(int64_t n);

}  // namespace dem
