// dem_internal.h — device data layout and kernel launchers of libdem_sm100a.so.
//
// Layout in HBM (one scene, n particles, contact capacity cap = n·max_coord):
//  * particles: structure of arrays in the caller's particle order, FP64;
//  * broad phase: per-particle cell record (int4: ijk + octant bits), bucket
//    id, a dense bucket table of H counts / H+1 starts (the reference's
//    hash_table), and particle copies in bucket-sorted order (double4 x,y,z,r
//    and a float4 copy relative to domain_min for the distance pre-filter);
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

struct ContactSoA {
    int32_t* ci;
    int32_t* cj;
    uint32_t* fl;
    double* f[15];  // kx ky kz | Fx Fy Fz | tix tiy tiz | tjx tjy tjz | sx sy sz
};
enum ContactField { CK = 0, CF = 3, CTI = 6, CTJ = 9, CS = 12 };

struct DevCounters {
    int error;
    unsigned int bmax;        // largest bucket id of this step (k_hash), reset by k_canon
    unsigned int cell_limit;  // buckets [0, cell_limit) have valid starts this step
    unsigned int pad;
    unsigned int row_alloc[2];  // contacts allocated in each contact buffer
    unsigned long long broken, ended, created, warn_gap, warn_damp;
    unsigned long long tickets[2];  // tile tickets of the scan sites (never reset)
};

// scan sites: each has its own ticket counter and tile-state array
constexpr int kScanCells = 0;
constexpr int kScanDebug = 1;

// Device pointers of one scene (passed by value to every kernel).
struct DemDev {
    // particles, caller order
    double *px, *py, *pz, *vx, *vy, *vz, *wx, *wy, *wz;
    double *qw, *qx, *qy, *qz;
    double *m, *inv_m, *r, *r0, *inv_inertia;
    double *b_invA, *b_rbI;  // bond section constants for rb = ρ·r (1/A, rb/I)
    double *b_EA, *b_EI, *b_phic;  // E·A, E·I and 20/3·(1+ν)·rb² for rb = ρ·r
    double *fx, *fy, *fz, *tx, *ty, *tz;  // totals of the last step
    double *wsx, *wsy, *wsz;              // wall shear history (one wall)
    // broad phase
    int4* cellinfo;
    uint32_t* bucket;      // 0-based bucket of each particle
    uint32_t* cell_count;  // H, zero between steps
    uint32_t* cell_start;  // H + 1
    uint32_t* unsorted;    // n, bucket-grouped, arbitrary order inside a bucket
    uint32_t* sorted;      // n, bucket-grouped, ascending index inside a bucket
    double4_32a* spos;        // n, (x, y, z, r) in sorted order
    float4* spos32;        // n, (x-ox, y-oy, z-oz, r) in FP32, sorted order
    // contacts
    ContactSoA c[2];
    int32_t* row_start[2];  // n, first slot of each particle's row
    int32_t* row_len[2];    // n, entries in the row
    int32_t* nnew;          // n
    int32_t* stash;       // n * kstash new partners of this step
    uint8_t* keep;        // cap, survival flags of the current buffer
    int32_t* in_cnt;      // n, zero between steps
    int2* in_list;        // n * kin: (contact slot, owner i) of contacts where the particle is j
    double* contrib;      // 9 * cap, [field][contact]
    // scan scratch: tile states of each scan site
    unsigned long long* scan_state[2];
    DevCounters* ctr;
};

// Scene constants (host-derived, passed by value).
struct DemParams {
    int n;
    int cap;        // contact capacity
    int kstash;     // new partners per particle per step
    int kin;        // incoming contacts per particle
    uint32_t H;     // hash table size
    uint32_t H_pow2_mask;  // H-1 when H is a power of two, else 0
    int has_wall;
    int precision;  // 0 = FP64, 1 = FP32 force
    double dmin[3];
    double cell, inv_cell;
    double dt, tol;
    double grav[3];
    double damping;
    // particle-particle Hertz-Mindlin constants (surface [1,1], materials 1,1)
    // cgn = -2β·sqrt(5/3·Y*), cgt = -2β·sqrt(20/3·G*): γₙ = cgn·sqrt(m*·sqrt(R*Δn))
    double pp_mu, pp_beta, pp_Ys, pp_Gs, pp_cgn, pp_cgt;
    // EBPM bond constants (surface [1,1])
    double b_rho, b_E, b_nu, b_inv1pnu, b_sc, b_st, b_ss;
    // wall (wall_normal, wall_distance) and particle-wall constants
    double wn[3], wd;
    double wR[9], wRinv[9];  // contact frame of the wall and its inverse
    double pw_mu, pw_beta, pw_Ys, pw_Gs, pw_cgn, pw_cgt;
};

// ---- launchers (dem_kernels.cu) --------------------------------------------
// All launches go to `s`.  `cur` selects the contact buffer that holds the
// state at the start of the step; the step writes buffer cur^1.
void launch_broadphase(const DemDev& d, const DemParams& p, int n_scan_tiles_cells,
                       cudaStream_t s);
void launch_detect(const DemDev& d, const DemParams& p, int cur, bool init, cudaStream_t s);
void launch_compact(const DemDev& d, const DemParams& p, int cur, bool init, int grid,
                    cudaStream_t s);
void launch_force(const DemDev& d, const DemParams& p, int nxt, int grid, cudaStream_t s);
void launch_integrate(const DemDev& d, const DemParams& p, int cur, cudaStream_t s);

// debug: cp_list materialisation on the current bucket arrays
void launch_cplist_count(const DemDev& d, const DemParams& p, int32_t* cnt, cudaStream_t s);
void launch_cplist_fill(const DemDev& d, const DemParams& p, const int32_t* off, int32_t* cp,
                        cudaStream_t s);
void launch_morton(const DemDev& d, const DemParams& p, uint32_t* morton, cudaStream_t s);
// exclusive scan of n int32 values into out[0..n] (out[n] = total)
void launch_scan_i32(const int32_t* in, int32_t* out, int64_t n, const DemDev& d, int site,
                     cudaStream_t s);

int scan_tiles(int64_t n);

}  // namespace dem
