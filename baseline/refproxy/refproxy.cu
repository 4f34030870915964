// Reference-structured GPU proxy of the DEMPort step — a labelled stand-in
// for timing, not part of the library.
//
// The reference's GPU path (Julia + CUDA.jl, src/executor.jl:31-172 and
// src/kernels.jl:1-506) cannot run on this machine: there is no Julia
// toolchain, and its CUDA.jl predates Blackwell.  This file restates that
// path in plain CUDA C++ with the reference's own structure, so that the
// library's step can be timed against it on the same GPU:
//   * array-of-structures records: the 272-byte Grain and the 136-byte
//     Contact of src/types.jl, walls' shear history as an nwall x n Contact
//     array;
//   * BitTables contact_active / contact_bonded of nextpow2(n)^2 bits,
//     indexed by i*n + j (src/utils.jl:18-28);
//   * the reference's kernel decomposition and launch order per step, one
//     thread per element in grid-stride loops of 256 threads, FP64 atomics
//     for the force scatter (src/kernels.jl:1-5), an inclusive scan for each
//     `accumulate!`, and the three device->host reads of src/executor.jl:64,
//     96 and 141;
//   * the same formulas in the same order (Rodrigues frame, EBPM with
//     breakage, Hertz-Mindlin, wall contact, body force, `update!`).
// It shares no code with the library.  Its one addition to the reference is
// bounds checks: a full contact list sets an error word instead of writing
// past its end.  Particle and contact indices are 0-based.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "dem_gb300.h"

namespace {

constexpr int kThreads = 256;  // `threads = 256` (src/executor.jl:319)
constexpr double kPi = 3.14159265358979323846;

struct V3 {
    double x, y, z;
};
__host__ __device__ inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
__host__ __device__ inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__host__ __device__ inline V3 operator/(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ inline double norm(V3 a) { return sqrt(dot(a, a)); }
__device__ inline V3 normalize(V3 a) { return a / norm(a); }

struct M3 {
    double a[3][3];
};
__device__ inline V3 mul(const M3& m, V3 v) {
    return {m.a[0][0] * v.x + m.a[0][1] * v.y + m.a[0][2] * v.z,
            m.a[1][0] * v.x + m.a[1][1] * v.y + m.a[1][2] * v.z,
            m.a[2][0] * v.x + m.a[2][1] * v.y + m.a[2][2] * v.z};
}
// General 3x3 inverse by cofactors (StaticArrays `inv`).
__device__ inline M3 inv3(const M3& m) {
    const double(*a)[3] = m.a;
    const double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
    const double c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
    const double c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
    const double det = a[0][0] * c00 + a[0][1] * c01 + a[0][2] * c02;
    const double id = 1.0 / det;
    M3 r;
    r.a[0][0] = c00 * id;
    r.a[1][0] = c01 * id;
    r.a[2][0] = c02 * id;
    r.a[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * id;
    r.a[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * id;
    r.a[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * id;
    r.a[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * id;
    r.a[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * id;
    r.a[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * id;
    return r;
}

// GrainDefault (src/types.jl): 3 x Int32 (+4 bytes of alignment), then FP64.
struct Grain {
    int32_t id, gid, mid, pad_;
    double V, m, r, r0;
    V3 k, v, a;
    double q[4];  // w, x, y, z
    V3 w, dw;
    M3 I;
};
static_assert(sizeof(Grain) == 272, "Grain record is 272 bytes");

// ContactDefault (src/types.jl)
struct Contact {
    int32_t i, j, midi, midj;
    V3 k, F, ti, tj, s;
};
static_assert(sizeof(Contact) == 136, "Contact record is 136 bytes");

struct Material {
    double rho, E, nu;
};
struct Surface {
    double mu, e, mur, rho, E, nu, sc, st, ss;
};
struct Wall {
    V3 n;
    double d;
    int32_t mid, pad_;
};

struct Int3 {
    int32_t x, y, z;
};
struct Vec8 {
    uint32_t b[8];
};

__device__ inline uint32_t spread10(uint32_t v) {
    uint32_t r = 0;
    for (int b = 0; b < 10; ++b) r |= ((v >> b) & 1u) << (3 * b);
    return r;
}
// cartesian3morton of a 1-based cell (x in bit 0), then `% H`: 0-based bucket
__device__ inline uint32_t hashcode(int32_t x, int32_t y, int32_t z, uint32_t H) {
    const uint32_t m = (spread10((uint32_t)(x - 1) & 0x3ffu) | (spread10((uint32_t)(y - 1) & 0x3ffu) << 1) |
                        (spread10((uint32_t)(z - 1) & 0x3ffu) << 2)) + 1u;
    return m % H;
}

__device__ inline bool get_bit(const uint32_t* bs, uint64_t idx) {
    return (bs[idx >> 5] & (1u << (idx & 31))) != 0u;
}
__device__ inline void set_bit(uint32_t* bs, uint64_t idx) { atomicOr(&bs[idx >> 5], 1u << (idx & 31)); }
__device__ inline void clear_bit(uint32_t* bs, uint64_t idx) {
    atomicAnd(&bs[idx >> 5], ~(1u << (idx & 31)));
}
__device__ inline void atomic_add_vec3(double* c, int i, V3 v) {
    atomicAdd(c + 3 * i, v.x);
    atomicAdd(c + 3 * i + 1, v.y);
    atomicAdd(c + 3 * i + 2, v.z);
}

#define GRID_STRIDE(i, n)                                                              \
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)(n); \
         i += (int64_t)gridDim.x * blockDim.x)

// ---- contact! preprocessing: four `map!` (src/executor.jl:39-43) -------------
__global__ void k_cell(const Grain* g, int n, V3 dmin, double cell, Int3* kid) {
    GRID_STRIDE(i, n) {
        const V3 k = g[i].k;
        kid[i] = {(int32_t)ceil((k.x - dmin.x) / cell), (int32_t)ceil((k.y - dmin.y) / cell),
                  (int32_t)ceil((k.z - dmin.z) / cell)};
    }
}
__global__ void k_hashcode(const Int3* kid, int n, uint32_t H, uint32_t* hid) {
    GRID_STRIDE(i, n) { hid[i] = hashcode(kid[i].x, kid[i].y, kid[i].z, H); }
}
__global__ void k_center(const Int3* kid, int n, V3 dmin, double cell, V3* kc) {
    GRID_STRIDE(i, n) {
        kc[i] = {dmin.x + (kid[i].x - 0.5) * cell, dmin.y + (kid[i].y - 0.5) * cell,
                 dmin.z + (kid[i].z - 0.5) * cell};
    }
}
__global__ void k_neighbors(const Grain* g, const Int3* kid, const V3* kc, int n, uint32_t H,
                            Vec8* nb) {
    GRID_STRIDE(i, n) {
        const V3 o = g[i].k, c = kc[i];
        const Int3 q = kid[i];
        const int dx = o.x > c.x ? 1 : -1, dy = o.y > c.y ? 1 : -1, dz = o.z > c.z ? 1 : -1;
        Vec8 r;
        r.b[0] = hashcode(q.x, q.y, q.z, H);
        r.b[1] = hashcode(q.x + dx, q.y, q.z, H);
        r.b[2] = hashcode(q.x, q.y + dy, q.z, H);
        r.b[3] = hashcode(q.x, q.y, q.z + dz, H);
        r.b[4] = hashcode(q.x + dx, q.y + dy, q.z, H);
        r.b[5] = hashcode(q.x + dx, q.y, q.z + dz, H);
        r.b[6] = hashcode(q.x, q.y + dy, q.z + dz, H);
        r.b[7] = hashcode(q.x + dx, q.y + dy, q.z + dz, H);
        nb[i] = r;
    }
}

// ---- hash table (src/kernels.jl:7-22) ---------------------------------------
__global__ void k_count_particles(uint32_t* ht, const uint32_t* hid, int n) {
    GRID_STRIDE(i, n) { atomicAdd(&ht[hid[i]], 1u); }
}
__global__ void k_get_particle_id(uint32_t* pid, uint32_t* htc, const uint32_t* hid, int n) {
    GRID_STRIDE(i, n) {
        const uint32_t id = atomicSub(&htc[hid[i]], 1u);  // 1-based end of the bucket
        pid[id - 1] = (uint32_t)i;
    }
}

// ---- `accumulate!(+, out, in)`: inclusive scan in three launches ------------
constexpr int kScanPer = 4;
constexpr int kScanTile = kThreads * kScanPer;

__device__ uint32_t block_exclusive(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[kThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t s = lane < kThreads / 32 ? warp_sums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kThreads / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t before = (w ? warp_sums[w - 1] : 0u) + x - v;
    *total = warp_sums[kThreads / 32 - 1];
    __syncthreads();
    return before;
}
__global__ void k_scan_tiles(const uint32_t* in, uint32_t* out, int64_t L, uint32_t* tile_sums) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
    uint32_t v[kScanPer], s = 0;
    for (int e = 0; e < kScanPer; ++e) {
        v[e] = base + e < L ? in[base + e] : 0u;
        s += v[e];
        v[e] = s;
    }
    uint32_t total;
    const uint32_t before = block_exclusive(s, &total);
    for (int e = 0; e < kScanPer; ++e)
        if (base + e < L) out[base + e] = v[e] + before;
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}
__global__ void k_scan_sums(uint32_t* sums, int64_t nt) {
    // one block: thread t scans its chunk of tile sums, then the chunks are offset
    const int64_t per = (nt + kThreads - 1) / kThreads;
    const int64_t b0 = threadIdx.x * per, b1 = b0 + per < nt ? b0 + per : nt;
    uint32_t s = 0;
    for (int64_t b = b0; b < b1; ++b) s += sums[b];
    uint32_t total;
    uint32_t run = block_exclusive(s, &total);
    for (int64_t b = b0; b < b1; ++b) {
        run += sums[b];
        sums[b] = run;  // inclusive
    }
}
__global__ void k_scan_add(uint32_t* out, int64_t L, const uint32_t* sums) {
    if (blockIdx.x == 0) return;
    const uint32_t add = sums[blockIdx.x - 1];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    for (int e = threadIdx.x; e < kScanTile; e += kThreads)
        if (base + e < L) out[base + e] += add;
}

// ---- pair search (src/kernels.jl:24-58) -------------------------------------
__global__ void k_search_hash_table(uint32_t* cp_range, const uint32_t* ht, const uint32_t* htc,
                                    const Vec8* nb, const uint32_t* pid, int n) {
    GRID_STRIDE(i, n) {
        const Vec8 b = nb[i];
        for (int q = 0; q < 8; ++q) {
            const uint32_t idx = b.b[q];
            for (uint32_t k = htc[idx]; k < htc[idx] + ht[idx]; ++k) {
                const uint32_t j = pid[k];
                if ((uint32_t)i < j) atomicAdd(&cp_range[i], 1u);
            }
        }
    }
}
__global__ void k_update_cp_list(int2* cp_list, uint32_t* cprc, const uint32_t* ht,
                                 const uint32_t* htc, const Vec8* nb, const uint32_t* pid, int n) {
    GRID_STRIDE(i, n) {
        const Vec8 b = nb[i];
        for (int q = 0; q < 8; ++q) {
            const uint32_t idx = b.b[q];
            for (uint32_t k = htc[idx]; k < htc[idx] + ht[idx]; ++k) {
                const uint32_t j = pid[k];
                if ((uint32_t)i < j) {
                    const uint32_t cur = atomicSub(&cprc[i], 1u);
                    cp_list[cur - 1] = make_int2((int)i, (int)j);
                }
            }
        }
    }
}

// ---- contact list (src/kernels.jl:60-120) -----------------------------------
__device__ inline void new_contact(Contact* contacts, uint32_t* cptr, int64_t cap, int* err, int i,
                                   int j, const Grain* g) {
    const uint32_t off = atomicAdd(&cptr[0], 1u);
    if ((int64_t)off >= cap) {
        atomicOr(err, 1);
        return;
    }
    Contact c;
    c.i = i;
    c.j = j;
    c.midi = g[i].mid;
    c.midj = g[j].mid;
    c.k = c.F = c.ti = c.tj = c.s = V3{0.0, 0.0, 0.0};
    contacts[off] = c;
}
__global__ void k_init_bonds(Contact* contacts, uint32_t* cptr, uint32_t* active, uint32_t* bonded,
                             const int2* cp_list, int64_t total, const Grain* g, int n, int64_t cap,
                             int* err) {
    GRID_STRIDE(idx, total) {
        const int i = cp_list[idx].x, j = cp_list[idx].y;
        if (norm(g[i].k - g[j].k) < g[i].r0 + g[j].r0) {
            const uint64_t ij = (uint64_t)i * n + j;
            set_bit(active, ij);
            set_bit(bonded, ij);
            new_contact(contacts, cptr, cap, err, i, j, g);
        }
    }
}
__global__ void k_update_contacts(Contact* contacts, uint32_t* cptr, uint32_t* active,
                                  const uint32_t* bonded, const int2* cp_list, int64_t total,
                                  const Grain* g, int n, int64_t cap, int* err) {
    GRID_STRIDE(idx, total) {
        const int i = cp_list[idx].x, j = cp_list[idx].y;
        const uint64_t ij = (uint64_t)i * n + j;
        if (!get_bit(bonded, ij)) {
            const bool valid = norm(g[i].k - g[j].k) < g[i].r + g[j].r;
            const bool exist = get_bit(active, ij);
            if (exist && !valid) {
                atomicAdd(&cptr[1], 1u);
                clear_bit(active, ij);
            } else if (!exist && valid) {
                set_bit(active, ij);
                new_contact(contacts, cptr, cap, err, i, j, g);
            }
        }
    }
}

// Rodrigues rotation taking the unit vector a onto the local x axis
// (src/kernels.jl:145-163, 331-350)
__device__ inline M3 frame(V3 a, double tol) {
    const V3 b{1.0, 0.0, 0.0};
    const V3 v = cross(a, b);
    const double s = norm(v), c = dot(a, b);
    M3 R;
    if (s < tol) {
        const double sg = c > 0.0 ? 1.0 : -1.0;
        R = M3{{{sg, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, sg}}};
    } else {
        const double vx[3][3] = {{0.0, -v.z, v.y}, {v.z, 0.0, -v.x}, {-v.y, v.x, 0.0}};
        const double f = (1.0 - c) / (s * s);
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) {
                double v2 = 0.0;
                for (int t = 0; t < 3; ++t) v2 += vx[r][t] * vx[t][q];
                R.a[r][q] = (r == q ? 1.0 : 0.0) + vx[r][q] + v2 * f;
            }
    }
    return R;
}

// ---- resolve_collision! (src/kernels.jl:122-315) ----------------------------
__global__ void k_resolve_collision(Contact* contacts, uint32_t* cptr, uint32_t* active,
                                    uint32_t* bonded, double* forces, double* moments,
                                    const Grain* g, const Material* mat, const Surface* surf,
                                    int nmat, int n, int64_t cap, double dt, double tol) {
    const int64_t total = (int64_t)cptr[0] < cap ? (int64_t)cptr[0] : cap;
    GRID_STRIDE(idx, total) {
        Contact c = contacts[idx];
        const int i = c.i, j = c.j;
        const uint64_t ij = (uint64_t)i * n + j;
        if (!get_bit(active, ij)) continue;
        const Grain& gi = g[i];
        const Grain& gj = g[j];
        const M3 R = frame(normalize(gj.k - gi.k), tol);
        const double Li = norm(gj.k - gi.k);
        const int midi = gi.mid, midj = gj.mid;
        const Surface sf = surf[midi * nmat + midj];
        if (get_bit(bonded, ij)) {
            const V3 k = (gi.k + gj.k) * 0.5;
            const V3 di = mul(R, gi.v) * dt, dj = mul(R, gj.v) * dt;
            const V3 thi = mul(R, gi.w) * dt, thj = mul(R, gj.w) * dt;
            const double rj = sf.rho * fmin(gi.r, gj.r);
            const double Lj = Li, Ej = sf.E, nu = sf.nu;
            const double Ij = rj * rj * rj * rj * kPi / 4.0;
            const double phi = 20.0 / 3.0 * (rj * rj) / (Lj * Lj) * (1.0 + nu);
            const double Aj = rj * rj * kPi;
            const double k1 = Ej * Aj / Lj;
            const double k2 = 12.0 * Ej * Ij / (Lj * Lj * Lj) / (1.0 + phi);
            const double k3 = 6.0 * Ej * Ij / (Lj * Lj) / (1.0 + phi);
            const double k4 = Ej * Ij / Lj / (1.0 + nu);
            const double k5 = Ej * Ij * (4.0 + phi) / Lj / (1.0 + phi);
            const double k6 = Ej * Ij * (2.0 - phi) / Lj / (1.0 + phi);
            const V3 dFi{k1 * (di.x - dj.x), k2 * (di.y - dj.y) + k3 * (thi.z + thj.z),
                         k2 * (di.z - dj.z) - k3 * (thi.y + thj.y)};
            const V3 dTi{k4 * (thi.x - thj.x), k3 * (dj.z - di.z) + k5 * thi.y + k6 * thj.y,
                         k3 * (di.y - dj.y) + k5 * thi.z + k6 * thj.z};
            const V3 dTj{k4 * (thj.x - thi.x), k3 * (dj.z - di.z) + k6 * thi.y + k5 * thj.y,
                         k3 * (di.y - dj.y) + k6 * thi.z + k5 * thj.z};
            const V3 Fi = c.F + dFi, Fj = -Fi;
            const V3 Ti = c.ti + dTi, Tj = c.tj + dTj;
            const double sci = Fj.x / Aj - rj / Ij * sqrt(Ti.y * Ti.y + Ti.z * Ti.z);
            const double scj = Fj.x / Aj - rj / Ij * sqrt(Tj.y * Tj.y + Tj.z * Tj.z);
            const double sc = -fmin(sci, scj);
            const double st = fmax(sci, scj);
            const double ss = fabs(Ti.x) * rj / 2.0 / Ij + 4.0 / 3.0 / Aj * sqrt(Fi.y * Fi.y + Fi.z * Fi.z);
            if (sc >= sf.sc || st >= sf.st || ss >= sf.ss) {
                atomicAdd(&cptr[1], 1u);
                clear_bit(active, ij);
                clear_bit(bonded, ij);
            } else {
                const M3 Ri = inv3(R);
                atomic_add_vec3(forces, i, mul(Ri, -Fi));
                atomic_add_vec3(forces, j, mul(Ri, -Fj));
                atomic_add_vec3(moments, i, mul(Ri, -Ti));
                atomic_add_vec3(moments, j, mul(Ri, -Tj));
                c.k = k;
                c.F = Fi;
                c.ti = Ti;
                c.tj = Tj;
                c.s = V3{0.0, 0.0, 0.0};
                contacts[idx] = c;
            }
        } else {  // Hertz-Mindlin
            const double gap = Li - gi.r - gj.r;
            const double dn = fabs(gap);
            const V3 k = gi.k + normalize(gj.k - gi.k) * (gi.r - dn);
            const V3 ki = k - gi.k, kj = k - gj.k;
            const V3 vci = cross(gi.w, ki) + gi.v, vcj = cross(gj.w, kj) + gj.v;
            const V3 vc = mul(R, vcj - vci);
            const double nui = mat[midi].nu, Ei = mat[midi].E, nuj = mat[midj].nu, Ej = mat[midj].E;
            const double Ys = 1.0 / ((1.0 - nui * nui) / Ei + (1.0 - nuj * nuj) / Ej);
            const double Gs = 1.0 / (2.0 * (2.0 - nui) * (1.0 + nui) / Ei +
                                     2.0 * (2.0 - nuj) * (1.0 + nuj) / Ej);
            const double Rs = 1.0 / (1.0 / gi.r + 1.0 / gj.r);
            const double ms = 1.0 / (1.0 / gi.m + 1.0 / gj.m);
            const double le = log(sf.e);
            const double beta = le / sqrt(le * le + kPi * kPi);
            const double Sn = 2.0 * Ys * sqrt(Rs * dn);
            const double St = 8.0 * Gs * sqrt(Rs * dn);
            const double kn = 4.0 / 3.0 * Ys * sqrt(Rs * dn);
            const double gn = -2.0 * beta * sqrt(5.0 / 6.0 * Sn * ms);
            const double kt = 8.0 * Gs * sqrt(Rs * dn);
            const double gt = -2.0 * beta * sqrt(5.0 / 6.0 * St * ms);
            V3 s = c.s + V3{vc.x * 0.0, vc.y * dt, vc.z * dt};
            const double F1 = -kn * gap - gn * vc.x;
            const V3 Ft = -kt * s;
            double F2, F3;
            if (norm(Ft) >= sf.mu * F1) {
                const double ratio = sf.mu * F1 / norm(Ft);
                F2 = ratio * Ft.y;
                F3 = ratio * Ft.z;
                s = V3{s.x, F2 / kt, F3 / kt};
            } else {
                F2 = Ft.y - gt * vc.y;
                F3 = Ft.z - gt * vc.z;
            }
            const V3 Fi{F1, F2, F3};
            const V3 Fig = mul(inv3(R), -Fi);
            atomic_add_vec3(forces, i, Fig);
            atomic_add_vec3(forces, j, -Fig);
            atomic_add_vec3(moments, i, cross(ki, Fig));
            atomic_add_vec3(moments, j, cross(kj, -Fig));
            c.k = k;
            c.F = Fi;
            c.s = s;
            contacts[idx] = c;
        }
    }
}

// ---- resolve_wall! (src/kernels.jl:317-426) ---------------------------------
__global__ void k_resolve_wall(Contact* wc, double* forces, double* moments, const Grain* g,
                               const Wall* walls, int nwall, const Material* mat,
                               const Surface* surf, int nmat, int n, double dt, double tol) {
    GRID_STRIDE(i, n) {
        const Grain& gi = g[i];
        for (int w = 0; w < nwall; ++w) {
            const Wall W = walls[w];
            Contact& C = wc[(int64_t)i * nwall + w];  // wall_contacts[j, i], column-major
            if (fabs(dot(gi.k, W.n) - W.d) < gi.r) {
                const M3 R = frame(W.n, tol);
                const double L = dot(gi.k, W.n) - W.d;
                const double gap = fabs(L) - gi.r;
                const double dn = fabs(gap);
                const V3 ki = -L * W.n / fabs(L) * (fabs(L) + dn / 2.0);
                const V3 k = gi.k + ki;
                const V3 vci = cross(gi.w, ki) + gi.v;
                const V3 vc = mul(R, -vci);
                const int midi = gi.mid, midj = W.mid;
                const Surface sf = surf[midi * nmat + midj];
                const double nui = mat[midi].nu, Ei = mat[midi].E, nuj = mat[midj].nu,
                             Ej = mat[midj].E;
                const double Ys = 1.0 / ((1.0 - nui * nui) / Ei + (1.0 - nuj * nuj) / Ej);
                const double Gs = 1.0 / (2.0 * (2.0 - nui) * (1.0 + nui) / Ei +
                                         2.0 * (2.0 - nuj) * (1.0 + nuj) / Ej);
                const double Rs = gi.r, ms = gi.m;
                const double le = log(sf.e);
                const double beta = le / sqrt(le * le + kPi * kPi);
                const double Sn = 2.0 * Ys * sqrt(Rs * dn);
                const double St = 8.0 * Gs * sqrt(Rs * dn);
                const double kn = 4.0 / 3.0 * Ys * sqrt(Rs * dn);
                const double gn = -2.0 * beta * sqrt(5.0 / 6.0 * Sn * ms);
                const double kt = 8.0 * Gs * sqrt(Rs * dn);
                const double gt = -2.0 * beta * sqrt(5.0 / 6.0 * St * ms);
                V3 s = C.s + V3{vc.x * 0.0, vc.y * dt, vc.z * dt};
                const double F1 = -kn * gap - gn * vc.x;
                const V3 Ft = -kt * s;
                double F2, F3;
                if (norm(Ft) >= sf.mu * F1) {
                    const double ratio = sf.mu * F1 / norm(Ft);
                    F2 = ratio * Ft.y;
                    F3 = ratio * Ft.z;
                    s = V3{s.x, F2 / kt, F3 / kt};
                } else {
                    F2 = Ft.y - gt * vc.y;
                    F3 = Ft.z - gt * vc.z;
                }
                const V3 Fi{F1, F2, F3};
                const V3 Fig = mul(inv3(R), -Fi);
                atomic_add_vec3(forces, (int)i, Fig);
                atomic_add_vec3(moments, (int)i, cross(ki, Fig));
                Contact nc;
                nc.i = (int)i;
                nc.j = -1;
                nc.midi = midi;
                nc.midj = midj;
                nc.k = k;
                nc.F = Fi;
                nc.ti = nc.tj = V3{0.0, 0.0, 0.0};
                nc.s = s;
                C = nc;
            } else {
                Contact z;
                memset(&z, 0, sizeof(z));
                C = z;
            }
        }
    }
}

// ---- apply_body_force! / update! (src/kernels.jl:428-485) -------------------
__device__ inline double sgn(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : x); }
__global__ void k_apply_body_force(double* forces, double* moments, const Grain* g, int n, V3 grav,
                                   double damping) {
    GRID_STRIDE(i, n) {
        atomic_add_vec3(forces, (int)i, grav * g[i].m);
        const V3 F{forces[3 * i], forces[3 * i + 1], forces[3 * i + 2]};
        const V3 T{moments[3 * i], moments[3 * i + 1], moments[3 * i + 2]};
        const V3 v = g[i].v, w = g[i].w;
        const V3 dF{-damping * fabs(F.x) * sgn(v.x), -damping * fabs(F.y) * sgn(v.y),
                    -damping * fabs(F.z) * sgn(v.z)};
        const V3 dT{-damping * fabs(T.x) * sgn(w.x), -damping * fabs(T.y) * sgn(w.y),
                    -damping * fabs(T.z) * sgn(w.z)};
        atomic_add_vec3(forces, (int)i, dF);
        atomic_add_vec3(moments, (int)i, dT);
    }
}
// Quaternionic.jl to_rotation_matrix for (w, x, y, z), divided by |q|^2
__device__ inline M3 quat_matrix(const double* q) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    const double s = 1.0 / (w * w + x * x + y * y + z * z);
    M3 R;
    R.a[0][0] = 1.0 - 2.0 * (y * y + z * z) * s;
    R.a[0][1] = 2.0 * (x * y - z * w) * s;
    R.a[0][2] = 2.0 * (x * z + y * w) * s;
    R.a[1][0] = 2.0 * (x * y + z * w) * s;
    R.a[1][1] = 1.0 - 2.0 * (x * x + z * z) * s;
    R.a[1][2] = 2.0 * (y * z - x * w) * s;
    R.a[2][0] = 2.0 * (x * z - y * w) * s;
    R.a[2][1] = 2.0 * (y * z + x * w) * s;
    R.a[2][2] = 1.0 - 2.0 * (x * x + y * y) * s;
    return R;
}
__global__ void k_update(Grain* g, const double* forces, const double* moments, int n, double dt) {
    GRID_STRIDE(i, n) {
        Grain G = g[i];
        const V3 F{forces[3 * i], forces[3 * i + 1], forces[3 * i + 2]};
        const V3 a = F / G.m;
        const V3 k = G.k + G.v * dt + 0.5 * a * (dt * dt);
        const V3 v = G.v + a * dt;
        const M3 R = quat_matrix(G.q);
        const V3 T{moments[3 * i], moments[3 * i + 1], moments[3 * i + 2]};
        const V3 Tl = mul(R, T), wl = mul(R, G.w);
        const V3 dwl = mul(inv3(G.I), Tl - cross(wl, mul(G.I, wl)));
        const V3 dw = mul(inv3(R), dwl);
        const double* q = G.q;
        const V3 w = G.w;
        const double d0 = -0.5 * (q[1] * w.x + q[2] * w.y + q[3] * w.z);
        const double d1 = 0.5 * (q[0] * w.x + q[2] * w.z - q[3] * w.y);
        const double d2 = 0.5 * (q[0] * w.y + q[1] * w.z + q[3] * w.x);
        const double d3 = 0.5 * (q[0] * w.z + q[1] * w.y - q[2] * w.x);
        double nq[4] = {q[0] + d0, q[1] + d1, q[2] + d2, q[3] + d3};
        const double qn = sqrt(nq[0] * nq[0] + nq[1] * nq[1] + nq[2] * nq[2] + nq[3] * nq[3]);
        for (int c = 0; c < 4; ++c) G.q[c] = nq[c] / qn;
        G.k = k;
        G.v = v;
        G.a = a;
        G.w = w + dw * dt;
        G.dw = dw;
        g[i] = G;
    }
}

// ---- remove_inactive_contact! (src/kernels.jl:487-506) ----------------------
__global__ void k_remove_inactive(const Contact* contacts, Contact* temp, uint32_t* cptr,
                                  const uint32_t* active, int64_t total, int n) {
    GRID_STRIDE(idx, total) {
        const Contact c = contacts[idx];
        if (get_bit(active, (uint64_t)c.i * n + c.j)) {
            const uint32_t off = atomicAdd(&cptr[0], 1u);
            temp[off] = c;
        }
    }
}

int blocks_for(int64_t n) { return (int)std::max<int64_t>(1, (n + kThreads - 1) / kThreads); }

}  // namespace

struct RefProxy {
    int n = 0, nwall = 1, nmat = 2;
    uint32_t H = 0;
    int64_t cp_cap = 0, c_cap = 0, bit_words = 0;
    V3 dmin{}, grav{};
    double cell = 0, dt = 0, tol = 0, damping = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    Grain* grains = nullptr;
    Int3* kid = nullptr;
    uint32_t* hid = nullptr;
    V3* kcenter = nullptr;
    Vec8* nb = nullptr;
    Material* mat = nullptr;
    Surface* surf = nullptr;
    Wall* walls = nullptr;
    Contact* wall_contacts = nullptr;
    double *forces = nullptr, *moments = nullptr;
    uint32_t *ht = nullptr, *htc = nullptr, *pid = nullptr;
    int2* cp_list = nullptr;
    uint32_t *cp_range = nullptr, *cprc = nullptr, *scan_sums = nullptr;
    Contact *contacts = nullptr, *contacts_temp = nullptr;
    uint32_t* cptr = nullptr;
    uint32_t *active = nullptr, *bonded = nullptr;
    int* err = nullptr;
    uint32_t* host_words = nullptr;  // page-locked: the per-step device->host reads
};

namespace {

#define RP_CU(x)                                   \
    do {                                           \
        if ((x) != cudaSuccess) return DEM_ERR_CUDA; \
    } while (0)

int scan(RefProxy* h, const uint32_t* in, uint32_t* out, int64_t L) {
    const int64_t nt = (L + kScanTile - 1) / kScanTile;
    k_scan_tiles<<<(int)nt, kThreads, 0, h->st>>>(in, out, L, h->scan_sums);
    k_scan_sums<<<1, kThreads, 0, h->st>>>(h->scan_sums, nt);
    k_scan_add<<<(int)nt, kThreads, 0, h->st>>>(out, L, h->scan_sums);
    RP_CU(cudaGetLastError());
    return DEM_OK;
}

// contact! up to the contact list (src/executor.jl:36-117)
int contact_phase(RefProxy* h, bool init) {
    const int n = h->n, b = blocks_for(n);
    cudaStream_t s = h->st;
    k_cell<<<b, kThreads, 0, s>>>(h->grains, n, h->dmin, h->cell, h->kid);
    k_hashcode<<<b, kThreads, 0, s>>>(h->kid, n, h->H, h->hid);
    k_center<<<b, kThreads, 0, s>>>(h->kid, n, h->dmin, h->cell, h->kcenter);
    k_neighbors<<<b, kThreads, 0, s>>>(h->grains, h->kid, h->kcenter, n, h->H, h->nb);
    RP_CU(cudaMemsetAsync(h->ht, 0, sizeof(uint32_t) * h->H, s));
    k_count_particles<<<b, kThreads, 0, s>>>(h->ht, h->hid, n);
    if (int rc = scan(h, h->ht, h->htc, h->H)) return rc;
    k_get_particle_id<<<b, kThreads, 0, s>>>(h->pid, h->htc, h->hid, n);
    RP_CU(cudaMemsetAsync(h->cp_range, 0, sizeof(uint32_t) * n, s));
    k_search_hash_table<<<b, kThreads, 0, s>>>(h->cp_range, h->ht, h->htc, h->nb, h->pid, n);
    if (int rc = scan(h, h->cp_range, h->cprc, n)) return rc;
    // host read 1: the pair total, the list grown by doubling
    RP_CU(cudaMemcpyAsync(h->host_words, h->cprc + (n - 1), sizeof(uint32_t),
                          cudaMemcpyDeviceToHost, s));
    RP_CU(cudaStreamSynchronize(s));
    const int64_t total = h->host_words[0];
    int64_t cap = h->cp_cap;
    while (cap < total) cap <<= 1;
    if (cap > h->cp_cap) {
        RP_CU(cudaFree(h->cp_list));
        h->cp_list = nullptr;
        RP_CU(cudaMalloc(&h->cp_list, sizeof(int2) * cap));
        h->cp_cap = cap;
    }
    k_update_cp_list<<<b, kThreads, 0, s>>>(h->cp_list, h->cprc, h->ht, h->htc, h->nb, h->pid, n);
    const int bt = blocks_for(total);
    if (init) {
        k_init_bonds<<<bt, kThreads, 0, s>>>(h->contacts, h->cptr, h->active, h->bonded, h->cp_list,
                                             total, h->grains, n, h->c_cap, h->err);
        RP_CU(cudaGetLastError());
        return DEM_OK;
    }
    k_update_contacts<<<bt, kThreads, 0, s>>>(h->contacts, h->cptr, h->active, h->bonded,
                                              h->cp_list, total, h->grains, n, h->c_cap, h->err);
    // host read 2: contact totals, forces only when a contact is active
    RP_CU(cudaMemcpyAsync(h->host_words, h->cptr, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    RP_CU(cudaStreamSynchronize(s));
    const int64_t tc = std::min<int64_t>(h->host_words[0], h->c_cap);
    const int64_t inactive = h->host_words[1];
    if (tc - inactive > 0)
        k_resolve_collision<<<blocks_for(tc), kThreads, 0, s>>>(
            h->contacts, h->cptr, h->active, h->bonded, h->forces, h->moments, h->grains, h->mat,
            h->surf, h->nmat, n, h->c_cap, h->dt, h->tol);
    RP_CU(cudaGetLastError());
    return DEM_OK;
}

int one_step(RefProxy* h) {
    cudaStream_t s = h->st;
    const int n = h->n, b = blocks_for(n);
    // clear_state!
    RP_CU(cudaMemsetAsync(h->forces, 0, sizeof(double) * 3 * n, s));
    RP_CU(cudaMemsetAsync(h->moments, 0, sizeof(double) * 3 * n, s));
    if (int rc = contact_phase(h, false)) return rc;
    k_resolve_wall<<<b, kThreads, 0, s>>>(h->wall_contacts, h->forces, h->moments, h->grains,
                                          h->walls, h->nwall, h->mat, h->surf, h->nmat, n, h->dt,
                                          h->tol);
    k_apply_body_force<<<b, kThreads, 0, s>>>(h->forces, h->moments, h->grains, n, h->grav,
                                              h->damping);
    k_update<<<b, kThreads, 0, s>>>(h->grains, h->forces, h->moments, n, h->dt);
    // late_clear_state!: host read 3, compaction only when a contact ended
    RP_CU(cudaMemcpyAsync(h->host_words, h->cptr, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    RP_CU(cudaStreamSynchronize(s));
    const int64_t tc = std::min<int64_t>(h->host_words[0], h->c_cap);
    if (h->host_words[1] > 0) {
        RP_CU(cudaMemsetAsync(h->cptr, 0, 2 * sizeof(uint32_t), s));
        k_remove_inactive<<<blocks_for(tc), kThreads, 0, s>>>(h->contacts, h->contacts_temp,
                                                             h->cptr, h->active, tc, n);
        std::swap(h->contacts, h->contacts_temp);
    }
    RP_CU(cudaGetLastError());
    return DEM_OK;
}

void free_all(RefProxy* h) {
    void* ptrs[] = {h->grains,   h->kid,      h->hid,      h->kcenter,  h->nb,       h->mat,
                    h->surf,     h->walls,    h->wall_contacts, h->forces, h->moments, h->ht,
                    h->htc,      h->pid,      h->cp_list,  h->cp_range, h->cprc,     h->scan_sums,
                    h->contacts, h->contacts_temp, h->cptr, h->active,  h->bonded,   h->err};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (h->host_words) cudaFreeHost(h->host_words);
    if (h->e0) cudaEventDestroy(h->e0);
    if (h->e1) cudaEventDestroy(h->e1);
    if (h->st) cudaStreamDestroy(h->st);
}

template <class T>
int dalloc(T** p, int64_t count) {
    RP_CU(cudaMalloc(p, sizeof(T) * (size_t)std::max<int64_t>(count, 1)));
    RP_CU(cudaMemset(*p, 0, sizeof(T) * (size_t)std::max<int64_t>(count, 1)));
    return DEM_OK;
}

int create(const DemConfigC* cfg, const DemParticlesIn* p, RefProxy* h) {
    const int64_t n = p->n;
    if (n < 1 || n > (1 << 22)) return DEM_ERR_INVALID;
    h->n = (int)n;
    // grain set-up of `solve` (src/executor.jl:217-243)
    std::vector<Grain> gs((size_t)n);
    double rmax = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        Grain& G = gs[(size_t)i];
        std::memset(&G, 0, sizeof(G));
        G.id = p->id ? p->id[i] : (int32_t)(i + 1);
        G.gid = p->gid ? p->gid[i] : 0;
        G.mid = 0;
        G.V = p->volume[i];
        G.m = p->mass[i];
        G.r = std::cbrt(G.V / (4.0 / 3.0 * kPi));
        G.r0 = G.r * cfg->particle_contact_radius_multiplier;
        G.k = {p->pos[3 * i], p->pos[3 * i + 1], p->pos[3 * i + 2]};
        G.v = {p->vel[3 * i], p->vel[3 * i + 1], p->vel[3 * i + 2]};
        G.q[0] = 1.0;
        const double Ii = 2.0 / 5.0 * G.m * G.r * G.r;
        G.I.a[0][0] = G.I.a[1][1] = G.I.a[2][2] = Ii;
        rmax = std::max(rmax, G.r);
    }
    const double density = gs.back().m / gs.back().V;
    const double r_search = rmax * cfg->particle_contact_radius_multiplier *
                            (1.0 + cfg->bond_tensile_strength / cfg->bond_elastic_modulus) *
                            cfg->neighboring_search_safety_factor;
    h->cell = 4.0 * r_search;
    if (!(h->cell > 0.0) || !std::isfinite(h->cell)) return DEM_ERR_INVALID;
    int64_t prod = 1;
    for (int c = 0; c < 3; ++c)
        prod *= (int64_t)std::ceil((cfg->domain_max[c] - cfg->domain_min[c]) / h->cell);
    h->H = (uint32_t)std::min<int64_t>(std::max<int64_t>(prod, 1 << 20), 1 << 22);
    h->dmin = {cfg->domain_min[0], cfg->domain_min[1], cfg->domain_min[2]};
    h->grav = {cfg->gravity[0], cfg->gravity[1], cfg->gravity[2]};
    h->dt = cfg->dt;
    h->tol = cfg->tolerance;
    h->damping = cfg->global_damping;
    h->cp_cap = std::max<int64_t>(1, n * cfg->collision_pair_init_capacity_factor);
    h->c_cap = std::max<int64_t>(1, n * cfg->max_coordinate_number);
    int64_t np2 = 1;
    while (np2 < n) np2 <<= 1;
    // the BitTables hold nextpow2(n)^2 bits each; above 2^16 particles they
    // pass 512 MiB and grow to the infeasible (2^21 particles: 512 GiB)
    if (np2 > (1 << 16)) return DEM_ERR_CAPACITY;
    h->bit_words = std::max<int64_t>((np2 * np2) >> 5, 1);
    // tables of src/executor.jl:282-315: material 0 = particles, 1 = wall
    const Material mats[2] = {{density, cfg->particle_elastic_modulus, cfg->particle_poisson_ratio},
                              {cfg->wall_density, cfg->wall_elastic_modulus, cfg->wall_poisson_ratio}};
    Surface surfs[4];
    std::memset(surfs, 0, sizeof(surfs));
    surfs[0] = {cfg->pp_coefficient_friction,  cfg->pp_coefficient_restitution,
                cfg->pp_coefficient_rolling_resistance, cfg->bond_radius_ratio,
                cfg->bond_elastic_modulus,     cfg->bond_poisson_ratio,
                cfg->bond_compressive_strength, cfg->bond_tensile_strength,
                cfg->bond_shear_strength};
    surfs[1] = surfs[2] = {cfg->pw_coefficient_friction, cfg->pw_coefficient_restitution,
                           cfg->pw_coefficient_rolling_resistance, 0, 0, 0, 0, 0, 0};
    Wall wall;
    std::memset(&wall, 0, sizeof(wall));
    wall.n = {cfg->wall_normal[0], cfg->wall_normal[1], cfg->wall_normal[2]};
    wall.d = cfg->wall_distance;
    wall.mid = 1;

    RP_CU(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    RP_CU(cudaEventCreate(&h->e0));
    RP_CU(cudaEventCreate(&h->e1));
    RP_CU(cudaMallocHost(&h->host_words, 64));
    int rc = DEM_OK;
    if (!rc) rc = dalloc(&h->grains, n);
    if (!rc) rc = dalloc(&h->kid, n);
    if (!rc) rc = dalloc(&h->hid, n);
    if (!rc) rc = dalloc(&h->kcenter, n);
    if (!rc) rc = dalloc(&h->nb, n);
    if (!rc) rc = dalloc(&h->mat, 2);
    if (!rc) rc = dalloc(&h->surf, 4);
    if (!rc) rc = dalloc(&h->walls, 1);
    if (!rc) rc = dalloc(&h->wall_contacts, n * h->nwall);
    if (!rc) rc = dalloc(&h->forces, 3 * n);
    if (!rc) rc = dalloc(&h->moments, 3 * n);
    if (!rc) rc = dalloc(&h->ht, h->H);
    if (!rc) rc = dalloc(&h->htc, h->H);
    if (!rc) rc = dalloc(&h->pid, n);
    if (!rc) rc = dalloc(&h->cp_list, h->cp_cap);
    if (!rc) rc = dalloc(&h->cp_range, n);
    if (!rc) rc = dalloc(&h->cprc, n);
    if (!rc) rc = dalloc(&h->scan_sums, (std::max<int64_t>(h->H, n) + kScanTile - 1) / kScanTile);
    if (!rc) rc = dalloc(&h->contacts, h->c_cap);
    if (!rc) rc = dalloc(&h->contacts_temp, h->c_cap);
    if (!rc) rc = dalloc(&h->cptr, 2);
    if (!rc) rc = dalloc(&h->active, h->bit_words);
    if (!rc) rc = dalloc(&h->bonded, h->bit_words);
    if (!rc) rc = dalloc(&h->err, 1);
    if (rc) return rc;
    RP_CU(cudaMemcpy(h->grains, gs.data(), sizeof(Grain) * n, cudaMemcpyHostToDevice));
    RP_CU(cudaMemcpy(h->mat, mats, sizeof(mats), cudaMemcpyHostToDevice));
    RP_CU(cudaMemcpy(h->surf, surfs, sizeof(surfs), cudaMemcpyHostToDevice));
    RP_CU(cudaMemcpy(h->walls, &wall, sizeof(wall), cudaMemcpyHostToDevice));
    RP_CU(cudaDeviceSynchronize());
    return DEM_OK;
}

}  // namespace

extern "C" {

// The grain set-up and buffers of `solve` (src/executor.jl:217-340).
// At most 65,536 particles (the BitTables' size).
int rp_create(const DemConfigC* cfg, const DemParticlesIn* p, RefProxy** out) {
    if (!cfg || !p || !out || !p->volume || !p->mass || !p->pos || !p->vel) return DEM_ERR_INVALID;
    RefProxy* h = new RefProxy();
    const int rc = create(cfg, p, h);
    if (rc) {
        free_all(h);
        delete h;
        return rc;
    }
    *out = h;
    return DEM_OK;
}

// initialize! (src/executor.jl:155-160)
int rp_init_bonds(RefProxy* h) {
    if (!h) return DEM_ERR_INVALID;
    const int rc = contact_phase(h, true);
    if (rc) return rc;
    RP_CU(cudaStreamSynchronize(h->st));
    return DEM_OK;
}

// simulate! x nsteps (src/executor.jl:162-172)
int rp_step(RefProxy* h, int64_t nsteps) {
    if (!h || nsteps < 0) return DEM_ERR_INVALID;
    for (int64_t k = 0; k < nsteps; ++k)
        if (int rc = one_step(h)) return rc;
    return DEM_OK;
}

// nsteps steps between two CUDA events on the proxy's stream (milliseconds)
int rp_step_timed(RefProxy* h, int64_t nsteps, float* ms) {
    if (!h || !ms) return DEM_ERR_INVALID;
    RP_CU(cudaStreamSynchronize(h->st));
    RP_CU(cudaEventRecord(h->e0, h->st));
    if (int rc = rp_step(h, nsteps)) return rc;
    RP_CU(cudaEventRecord(h->e1, h->st));
    RP_CU(cudaEventSynchronize(h->e1));
    RP_CU(cudaEventElapsedTime(ms, h->e0, h->e1));
    return DEM_OK;
}

// Positions and velocities (3n each, may be NULL); nonzero error word ->
// DEM_ERR_CAPACITY.
int rp_get_state(RefProxy* h, double* pos, double* vel) {
    if (!h) return DEM_ERR_INVALID;
    std::vector<Grain> gs((size_t)h->n);
    RP_CU(cudaStreamSynchronize(h->st));
    RP_CU(cudaMemcpy(gs.data(), h->grains, sizeof(Grain) * h->n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < h->n; ++i) {
        const Grain& G = gs[(size_t)i];
        if (pos) {
            pos[3 * i] = G.k.x;
            pos[3 * i + 1] = G.k.y;
            pos[3 * i + 2] = G.k.z;
        }
        if (vel) {
            vel[3 * i] = G.v.x;
            vel[3 * i + 1] = G.v.y;
            vel[3 * i + 2] = G.v.z;
        }
    }
    int err = 0;
    RP_CU(cudaMemcpy(&err, h->err, sizeof(int), cudaMemcpyDeviceToHost));
    return err ? DEM_ERR_CAPACITY : DEM_OK;
}

// Active contacts (i, j, bonded) in list order; `count` gets the number of
// active contacts (entries written: at most cap).
int rp_get_contacts(RefProxy* h, int32_t* ci, int32_t* cj, uint8_t* bonded, int64_t cap,
                    int64_t* count) {
    if (!h || !count) return DEM_ERR_INVALID;
    RP_CU(cudaStreamSynchronize(h->st));
    uint32_t ptr[2];
    RP_CU(cudaMemcpy(ptr, h->cptr, sizeof(ptr), cudaMemcpyDeviceToHost));
    const int64_t tc = std::min<int64_t>(ptr[0], h->c_cap);
    std::vector<Contact> cs((size_t)tc);
    std::vector<uint32_t> act((size_t)h->bit_words), bon((size_t)h->bit_words);
    if (tc) RP_CU(cudaMemcpy(cs.data(), h->contacts, sizeof(Contact) * tc, cudaMemcpyDeviceToHost));
    RP_CU(cudaMemcpy(act.data(), h->active, sizeof(uint32_t) * h->bit_words, cudaMemcpyDeviceToHost));
    RP_CU(cudaMemcpy(bon.data(), h->bonded, sizeof(uint32_t) * h->bit_words, cudaMemcpyDeviceToHost));
    auto bit = [](const std::vector<uint32_t>& b, uint64_t ij) {
        return (b[ij >> 5] >> (ij & 31)) & 1u;
    };
    int64_t m = 0;
    for (const Contact& c : cs) {
        const uint64_t ij = (uint64_t)c.i * h->n + c.j;
        if (!bit(act, ij)) continue;
        if (m < cap) {
            if (ci) ci[m] = c.i;
            if (cj) cj[m] = c.j;
            if (bonded) bonded[m] = (uint8_t)bit(bon, ij);
        }
        ++m;
    }
    *count = m;
    return DEM_OK;
}

int rp_destroy(RefProxy* h) {
    if (!h) return DEM_OK;
    cudaStreamSynchronize(h->st);
    free_all(h);
    delete h;
    return DEM_OK;
}

}  // extern "C"
