/*
 * dem_oracle.cpp — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement (C++17, FP64) of one DEM time step of the reference package
 * DEMPort (lucifer1004/taichi_dem_julia_port).  It is the checker for the
 * GB300 library and the timed CPU baseline.  Only tests/, the smoke check of
 * __graft_entry__.py and bench.py's CPU-baseline / reference legs may load it;
 * the product library never links, loads or calls it.
 *
 * What it restates (reference file:line):
 *   grain setup and derived sizes ..... src/executor.jl:217-315
 *   cell / hashcode / center / neighbors src/utils.jl:1-16
 *   BitTables (get/set/clear bit) ..... src/utils.jl:18-28
 *   count_particles!, get_particle_id!  src/kernels.jl:7-22
 *   search_hash_table!, update_cp_list!  src/kernels.jl:24-58
 *   init_bonds!, update_contacts! ...... src/kernels.jl:60-120
 *   resolve_collision! ................. src/kernels.jl:122-315
 *   resolve_wall! ...................... src/kernels.jl:317-426
 *   apply_body_force!, update! ......... src/kernels.jl:428-485
 *   remove_inactive_contact! + swap .... src/kernels.jl:487-506, src/executor.jl:140-153
 *   step order ......................... src/executor.jl:31-172
 *
 * Arithmetic follows Julia's evaluation order for each expression (n-ary `+`
 * and `*` fold left, `x^2` is x*x, `x^3` is (x*x)*x) and is compiled with
 * -ffp-contract=off so that no multiply-add is fused.  Cell indices, bucket
 * ids, octant signs and the contact / bond distance tests are therefore the
 * exact IEEE results of the reference's formulas.
 *
 * Order that the reference leaves free (atomics) is made canonical here:
 * particles within a bucket ascend by index, cp_list is emitted by ascending i,
 * contacts are processed in array order and the cleanup keeps array order.
 * Duplicate (i,j) pairs in cp_list (two octant cells hashing to one bucket)
 * are applied sequentially, so a pair is appended at most once; the reference
 * races there (src/kernels.jl:104-117).
 *
 * Parity status: pinned against the reference's own code where it runs here.
 *   - Morton code: dem.py's morton3d32 (dem.py:758-777) and README.md:23.
 *   - Quaternion-to-matrix formula: dem.py:317-344.
 *   - Contact physics: dem.py's DEMSolver.resolve (EBPM and Hertz-Mindlin,
 *     dem.py:1357-1606), evaluate_wall/resolve_wall (dem.py:1609-1743),
 *     apply_body_force (dem.py:1280-1305) and update (dem.py:1309-1354),
 *     executed from the reference's source on golden cases
 *     (tests/golden/make_physics_golden.py); the oracle agrees to 1e-12 of
 *     each vector's magnitude and takes identical breakage and wall-contact
 *     decisions.  dem.py states kernels.jl's formulas with a few sums
 *     associated differently, which is why the bound is not zero.
 * The broad phase and contact bookkeeping follow kernels.jl/executor.jl,
 * which dem.py does differently (0-based floor cells, per-particle contact
 * slots); those rows are checked against analytic properties (every touching
 * pair in cp_list) and the reference's scenes.  Third-party arithmetic with
 * no source in the reference (Morton.jl outside [1,1024], Quaternionic.jl,
 * StaticArrays' norm/inv, Julia's ^ and log) is restated from the published
 * algorithms.
 *
 * Modes: `threads` = 1 runs serially; > 1 runs the per-particle / per-pair /
 * per-contact loops with OpenMP and applies every order-dependent update
 * (appends, bit changes, force sums) sequentially, so both modes return
 * bit-identical results.
 */
#include "dem_gb300.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_set>
#include <vector>

#include <omp.h>

namespace {

constexpr double kPi = 3.141592653589793;

struct V3 {
    double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline double at(V3 a, int c) { return c == 0 ? a.x : (c == 1 ? a.y : a.z); }
// StaticArrays dot / cross: ((a1 b1 + a2 b2) + a3 b3)
inline double dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// StaticArrays `norm`: sqrt of the left-folded sum of squares; when the result
// is not in (0, Inf) it retries scaled by the largest magnitude.
double jl_norm(V3 a) {
    double l = std::sqrt((a.x * a.x + a.y * a.y) + a.z * a.z);
    if (l > 0.0 && l < INFINITY) return l;
    double sc = std::max(std::fabs(a.x), std::max(std::fabs(a.y), std::fabs(a.z)));
    if (sc == 0.0) return 0.0;
    double x = a.x / sc, y = a.y / sc, z = a.z / sc;
    return sc * std::sqrt((x * x + y * y) + z * z);
}
// StaticArrays `normalize(a) = inv(norm(a)) * a`
inline V3 jl_normalize(V3 a) { return (1.0 / jl_norm(a)) * a; }

inline double jl_min(double a, double b) {
    if (std::isnan(a) || std::isnan(b)) return NAN;
    return b < a ? b : a;
}
inline double jl_max(double a, double b) {
    if (std::isnan(a) || std::isnan(b)) return NAN;
    return b > a ? b : a;
}
// Julia sign(x): -1, +1, or x itself for ±0 and NaN
inline double jl_sign(double x) { return x < 0.0 ? -1.0 : (x > 0.0 ? 1.0 : x); }

// Julia 1.9 `^(x::Float64, n::Integer)` for n >= 4 (compensated power by
// squaring, Base.Math.pow_body).
double jl_pow(double x, int n) {
    double y = 1.0, xnlo = 0.0, ynlo = 0.0;
    while (n > 1) {
        if (n & 1) {
            double err = std::fma(y, xnlo, x * ynlo);
            double p = x * y;
            ynlo = std::fma(x, y, -p);
            y = p;
            ynlo += err;
        }
        double err = x * 2 * xnlo;
        double p = x * x;
        xnlo = std::fma(x, x, -p);
        x = p;
        xnlo += err;
        n >>= 1;
    }
    double err = std::fma(y, xnlo, x * ynlo);
    return (std::isfinite(x) && std::isfinite(err)) ? std::fma(x, y, err) : x * y;
}

struct M3 {
    double a[3][3];
};
M3 mmul(const M3& A, const M3& B) {
    M3 C;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            C.a[r][c] = (A.a[r][0] * B.a[0][c] + A.a[r][1] * B.a[1][c]) + A.a[r][2] * B.a[2][c];
    return C;
}
V3 mv(const M3& A, V3 v) {
    return {(A.a[0][0] * v.x + A.a[0][1] * v.y) + A.a[0][2] * v.z,
            (A.a[1][0] * v.x + A.a[1][1] * v.y) + A.a[1][2] * v.z,
            (A.a[2][0] * v.x + A.a[2][1] * v.y) + A.a[2][2] * v.z};
}
// StaticArrays 3x3 `inv`: rows of the inverse are cross products of the
// columns divided by the determinant.
M3 inv3(const M3& A) {
    V3 x0{A.a[0][0], A.a[1][0], A.a[2][0]};
    V3 x1{A.a[0][1], A.a[1][1], A.a[2][1]};
    V3 x2{A.a[0][2], A.a[1][2], A.a[2][2]};
    V3 y0 = cross(x1, x2);
    double d = dot(x0, y0);
    x0 = x0 / d;
    y0 = y0 / d;
    V3 y1 = cross(x2, x0);
    V3 y2 = cross(x0, x1);
    M3 R;
    R.a[0][0] = y0.x; R.a[0][1] = y0.y; R.a[0][2] = y0.z;
    R.a[1][0] = y1.x; R.a[1][1] = y1.y; R.a[1][2] = y1.z;
    R.a[2][0] = y2.x; R.a[2][1] = y2.y; R.a[2][2] = y2.z;
    return R;
}

// Rotation taking unit vector `a` to the local x axis (src/kernels.jl:145-165,
// same construction for walls at src/kernels.jl:332-352).
M3 frame_to_x(V3 a, double tol) {
    const V3 b{1.0, 0.0, 0.0};
    V3 v = cross(a, b);
    double s = jl_norm(v);
    double c = dot(a, b);
    M3 R;
    if (s < tol) {
        double sg = c > 0.0 ? 1.0 : -1.0;
        R = M3{{{sg, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, sg}}};
    } else {
        M3 vx{{{0.0, -v.z, v.y}, {v.z, 0.0, -v.x}, {-v.y, v.x, 0.0}}};
        M3 vx2 = mmul(vx, vx);
        double f = 1.0 - c, s2 = s * s;
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q)
                R.a[r][q] = ((r == q ? 1.0 : 0.0) + vx.a[r][q]) + (vx2.a[r][q] * f) / s2;
    }
    return R;
}

// Unit-quaternion rotation matrix (w,x,y,z), the formula of
// Quaternionic.jl `to_rotation_matrix` / dem.py:317-344.
M3 quat_to_matrix(const double* q) {
    double w = q[0], x = q[1], y = q[2], z = q[3];
    double n = 1.0 / (((w * w + x * x) + y * y) + z * z);
    M3 R;
    R.a[0][0] = 1.0 - 2.0 * (y * y + z * z) * n;
    R.a[0][1] = 2.0 * (x * y - z * w) * n;
    R.a[0][2] = 2.0 * (x * z + y * w) * n;
    R.a[1][0] = 2.0 * (x * y + z * w) * n;
    R.a[1][1] = 1.0 - 2.0 * (x * x + z * z) * n;
    R.a[1][2] = 2.0 * (y * z - x * w) * n;
    R.a[2][0] = 2.0 * (x * z - y * w) * n;
    R.a[2][1] = 2.0 * (y * z + x * w) * n;
    R.a[2][2] = 1.0 - 2.0 * (x * x + y * y) * n;
    return R;
}

// Morton.jl `cartesian3morton` for 1-based cells: interleave(ijk - 1) + 1 with
// x in bit 0 (README.md:23).  Coordinates keep their low 10 bits, as dem.py's
// morton3d32 does (dem.py:759-777); Morton.jl outside [1,1024] is unpinned.
uint32_t spread10(uint32_t v) {
    uint32_t r = 0;
    for (int b = 0; b < 10; ++b) r |= ((v >> b) & 1u) << (3 * b);
    return r;
}
uint32_t morton1(int32_t x, int32_t y, int32_t z) {
    uint32_t ux = (uint32_t)(x - 1) & 0x3ffu, uy = (uint32_t)(y - 1) & 0x3ffu,
             uz = (uint32_t)(z - 1) & 0x3ffu;
    return (spread10(ux) | (spread10(uy) << 1) | (spread10(uz) << 2)) + 1u;
}

struct Grain {
    int32_t id, gid, mid;  // mid is 0-based here (reference: 1)
    double V, m, r, r0;
    V3 k, v, a;
    double q[4];
    V3 w, dw;
    M3 I;
};

struct Contact {
    int32_t i, j, midi, midj;  // 0-based
    V3 k, F, ti, tj, s;
};

struct Material {
    double rho, E, nu;
};
struct Surface {
    double mu, e, mur, rho, E, nu, sc, st, ss;
};
struct Wall {
    V3 n;
    double d;
    int32_t mid;
};

// The BitTables of src/executor.jl:279-280: nextpow2(n)^2 bits addressed by
// ij = (i-1)*n + j with 1-based i, j.  Tables above 512 MiB are kept as a hash
// set with the same addressing (the dense table cannot be allocated there).
struct BitTable {
    bool dense = true;
    std::vector<uint32_t> words;
    std::unordered_set<uint64_t> set;
    void init(int64_t n) {
        uint64_t p = 1;
        while ((int64_t)p < std::max<int64_t>(n, 1)) p <<= 1;
        long double bits = (long double)p * (long double)p;
        dense = bits / 8 <= (long double)(1ull << 29);
        words.clear();
        set.clear();
        if (dense) words.assign((size_t)((p * p) >> 5) + 1, 0u);
    }
    bool get(uint64_t idx) const {
        if (dense) return (words[idx >> 5] >> (idx & 31)) & 1u;
        return set.count(idx) != 0;
    }
    void put(uint64_t idx) {
        if (dense) words[idx >> 5] |= 1u << (idx & 31);
        else set.insert(idx);
    }
    void clear(uint64_t idx) {
        if (dense) words[idx >> 5] &= ~(1u << (idx & 31));
        else set.erase(idx);
    }
};

struct ContactResult {
    int kind;  // 0 skip, 1 break, 2 apply
    Contact c;
    V3 fi, fj, mi, mj;
    int warn_gap, warn_gamma;
};

struct Scene {
    DemConfigC cfg;
    int64_t n = 0;
    int threads = 1;
    std::vector<Grain> g;
    double cell_size = 0, rmax = 0, material_density = 0;
    int64_t H = 0, total_steps = 0, save_per_steps = 0;
    // materials, surfaces ([a * nmat + b] = surfaces[a+1, b+1]) and walls
    // (src/types.jl:9-27, 58-62); wall_contacts[w * n + i] = wall_contacts[w+1, i+1]
    int nmat = 0;
    std::vector<Material> mat;
    std::vector<Surface> surf;
    std::vector<Wall> walls;
    std::vector<Contact> wall_contacts;  // nwall = 1
    std::vector<double> forces, moments;
    // broad phase
    std::vector<int32_t> kid;
    std::vector<uint32_t> morton, hid;  // hid 1-based
    std::vector<std::array<uint32_t, 8>> nbr;
    std::vector<uint32_t> ht, htc, pid;
    std::vector<int32_t> cp_i, cp_j;
    // contacts
    std::vector<Contact> contacts;
    uint32_t ptr_total = 0, ptr_inactive = 0;
    BitTable active, bonded;
    // statistics
    int64_t steps = 0, broken = 0, ended = 0, created = 0, warn_gap = 0, warn_gamma = 0;
    int error = DEM_OK;

    uint64_t bit(int32_t i, int32_t j) const { return (uint64_t)i * (uint64_t)n + (uint64_t)j + 1; }
};

// ---- setup (src/executor.jl:217-315) --------------------------------------
void set_tables(Scene& S);

void setup(Scene& S, const DemConfigC& cfg, const DemParticlesIn& p) {
    S.cfg = cfg;
    S.n = p.n;
    S.g.resize(S.n);
    double rmax_r = -INFINITY;
    for (int64_t i = 0; i < S.n; ++i) {
        Grain& G = S.g[i];
        G.id = p.id ? p.id[i] : (int32_t)(i + 1);
        G.gid = p.gid ? p.gid[i] : 0;
        G.mid = 0;
        G.V = p.volume[i];
        G.m = p.mass[i];
        G.r = std::cbrt(G.V / (4.0 / 3.0 * kPi));
        G.r0 = G.r * cfg.particle_contact_radius_multiplier;
        G.k = {p.pos[3 * i], p.pos[3 * i + 1], p.pos[3 * i + 2]};
        G.v = {p.vel[3 * i], p.vel[3 * i + 1], p.vel[3 * i + 2]};
        G.a = {0, 0, 0};
        G.q[0] = 1.0; G.q[1] = G.q[2] = G.q[3] = 0.0;
        G.w = {0, 0, 0};
        G.dw = {0, 0, 0};
        double I = 2.0 / 5.0 * G.m * (G.r * G.r);
        G.I = M3{{{I, 0.0, 0.0}, {0.0, I, 0.0}, {0.0, 0.0, I}}};
        rmax_r = std::max(rmax_r, G.r);
    }
    S.material_density = S.n ? S.g[S.n - 1].m / S.g[S.n - 1].V : 0.0;
    S.rmax = rmax_r * cfg.particle_contact_radius_multiplier *
             (1.0 + cfg.bond_tensile_strength / cfg.bond_elastic_modulus) *
             cfg.neighboring_search_safety_factor;
    S.cell_size = 4.0 * S.rmax;
    int64_t prod = 1;
    for (int c = 0; c < 3; ++c)
        prod *= (int64_t)std::ceil((cfg.domain_max[c] - cfg.domain_min[c]) / S.cell_size);
    S.H = std::min<int64_t>(std::max<int64_t>(prod, 1 << 20), 1 << 22);
    S.total_steps = (int64_t)std::trunc(cfg.target_time / cfg.dt);
    S.save_per_steps = (int64_t)std::trunc(cfg.saving_interval_time / cfg.dt);
    set_tables(S);
    S.wall_contacts.assign(S.n * S.walls.size(), Contact{});
    S.forces.assign(3 * S.n, 0.0);
    S.moments.assign(3 * S.n, 0.0);
    S.contacts.clear();
    S.contacts.reserve((size_t)std::max<int64_t>(S.n, 1) * 4);
    S.ptr_total = S.ptr_inactive = 0;
    S.active.init(S.n);
    S.bonded.init(S.n);
}

// Material, surface and wall tables of src/executor.jl:282-315 (one particle
// material, mid = 1; the wall material, mid = 2).
void set_tables(Scene& S) {
    const DemConfigC& cfg = S.cfg;
    S.nmat = 2;
    S.mat = {{S.material_density, cfg.particle_elastic_modulus, cfg.particle_poisson_ratio},
             {cfg.wall_density, cfg.wall_elastic_modulus, cfg.wall_poisson_ratio}};
    const Surface pp{cfg.pp_coefficient_friction, cfg.pp_coefficient_restitution,
                     cfg.pp_coefficient_rolling_resistance, cfg.bond_radius_ratio,
                     cfg.bond_elastic_modulus, cfg.bond_poisson_ratio,
                     cfg.bond_compressive_strength, cfg.bond_tensile_strength,
                     cfg.bond_shear_strength};
    const Surface pw{cfg.pw_coefficient_friction, cfg.pw_coefficient_restitution,
                     cfg.pw_coefficient_rolling_resistance, 0, 0, 0, 0, 0, 0};
    S.surf = {pp, pw, pw, Surface{0, 0, 0, 0, 0, 0, 0, 0, 0}};
    S.walls = {Wall{{cfg.wall_normal[0], cfg.wall_normal[1], cfg.wall_normal[2]}, cfg.wall_distance, 1}};
}

// ---- broad phase (src/executor.jl:38-78, src/utils.jl:1-16, src/kernels.jl:7-58)
int32_t ceil_i32(double t) {
    double c = std::ceil(t);
    if (!(c > -2147483648.0 && c < 2147483647.0)) return 0;  // NaN / overflow
    return (int32_t)c;
}

void broadphase(Scene& S) {
    const int64_t n = S.n;
    const uint64_t H = (uint64_t)S.H;
    const double cs = S.cell_size;
    const double* dmin = S.cfg.domain_min;
    S.kid.resize(3 * n);
    S.morton.resize(n);
    S.hid.resize(n);
    S.nbr.resize(n);
#pragma omp parallel for num_threads(S.threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const Grain& G = S.g[i];
        int32_t ijk[3];
        for (int c = 0; c < 3; ++c) ijk[c] = ceil_i32((at(G.k, c) - dmin[c]) / cs);
        int d[3];
        for (int c = 0; c < 3; ++c) {
            double ctr = dmin[c] + ((double)ijk[c] - 0.5) * cs;
            d[c] = at(G.k, c) > ctr ? 1 : -1;
        }
        auto hc = [&](int a, int b, int e) {
            return (uint32_t)((uint64_t)morton1(ijk[0] + a, ijk[1] + b, ijk[2] + e) % H) + 1u;
        };
        for (int c = 0; c < 3; ++c) S.kid[3 * i + c] = ijk[c];
        S.morton[i] = morton1(ijk[0], ijk[1], ijk[2]);
        S.hid[i] = hc(0, 0, 0);
        S.nbr[i] = {hc(0, 0, 0),       hc(d[0], 0, 0),    hc(0, d[1], 0),    hc(0, 0, d[2]),
                    hc(d[0], d[1], 0), hc(d[0], 0, d[2]), hc(0, d[1], d[2]), hc(d[0], d[1], d[2])};
    }
    // count_particles! + accumulate! + get_particle_id!  (canonical order)
    S.ht.assign(H, 0u);
    for (int64_t i = 0; i < n; ++i) S.ht[S.hid[i] - 1]++;
    S.htc.resize(H);
    uint32_t run = 0;
    for (uint64_t b = 0; b < H; ++b) {
        S.htc[b] = run;  // exclusive start = the value after get_particle_id!
        run += S.ht[b];
    }
    S.pid.resize(n);
    {
        std::vector<uint32_t> fill(S.htc);
        for (int64_t i = 0; i < n; ++i) S.pid[fill[S.hid[i] - 1]++] = (uint32_t)i;
    }
    // search_hash_table! / update_cp_list!: pairs i<j, j in one of i's 8 buckets
    std::vector<int64_t> cnt(n + 1, 0);
#pragma omp parallel for num_threads(S.threads) schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = 0;
        for (int b = 0; b < 8; ++b) {
            uint32_t idx = S.nbr[i][b] - 1;
            for (uint32_t k = S.htc[idx]; k < S.htc[idx] + S.ht[idx]; ++k)
                if ((int64_t)S.pid[k] > i) ++c;
        }
        cnt[i + 1] = c;
    }
    for (int64_t i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    S.cp_i.resize(cnt[n]);
    S.cp_j.resize(cnt[n]);
#pragma omp parallel for num_threads(S.threads) schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        int64_t o = cnt[i];
        for (int b = 0; b < 8; ++b) {
            uint32_t idx = S.nbr[i][b] - 1;
            for (uint32_t k = S.htc[idx]; k < S.htc[idx] + S.ht[idx]; ++k)
                if ((int64_t)S.pid[k] > i) {
                    S.cp_i[o] = (int32_t)i;
                    S.cp_j[o] = (int32_t)S.pid[k];
                    ++o;
                }
        }
    }
}

Contact zero_contact(const Scene& S, int32_t i, int32_t j) {
    Contact c{};
    c.i = i;
    c.j = j;
    c.midi = S.g[i].mid;
    c.midj = S.g[j].mid;
    return c;
}

bool append_contact(Scene& S, const Contact& c) {
    int64_t cap = S.n * S.cfg.max_coordinate_number;
    if ((int64_t)S.ptr_total >= cap) {
        S.error = DEM_ERR_CAPACITY;
        return false;
    }
    if (S.contacts.size() <= S.ptr_total) S.contacts.resize(S.ptr_total + 1);
    S.contacts[S.ptr_total++] = c;
    return true;
}

// init_bonds! (src/kernels.jl:60-85)
void init_bonds(Scene& S) {
    broadphase(S);
    const int64_t P = (int64_t)S.cp_i.size();
    std::vector<uint8_t> ok(P);
#pragma omp parallel for num_threads(S.threads) schedule(static)
    for (int64_t p = 0; p < P; ++p) {
        const Grain &gi = S.g[S.cp_i[p]], &gj = S.g[S.cp_j[p]];
        ok[p] = jl_norm(gi.k - gj.k) < gi.r0 + gj.r0;
    }
    for (int64_t p = 0; p < P; ++p) {
        if (!ok[p]) continue;
        uint64_t ij = S.bit(S.cp_i[p], S.cp_j[p]);
        if (S.active.get(ij)) continue;  // sequential application de-duplicates
        if (!append_contact(S, zero_contact(S, S.cp_i[p], S.cp_j[p]))) return;
        S.active.put(ij);
        S.bonded.put(ij);
    }
}

// update_contacts! (src/kernels.jl:87-120)
void update_contacts(Scene& S) {
    const int64_t P = (int64_t)S.cp_i.size();
    std::vector<int8_t> valid(P);
#pragma omp parallel for num_threads(S.threads) schedule(static)
    for (int64_t p = 0; p < P; ++p) {
        int32_t i = S.cp_i[p], j = S.cp_j[p];
        if (S.bonded.get(S.bit(i, j))) { valid[p] = -1; continue; }
        const Grain &gi = S.g[i], &gj = S.g[j];
        valid[p] = jl_norm(gi.k - gj.k) < gi.r + gj.r;
    }
    for (int64_t p = 0; p < P; ++p) {
        if (valid[p] < 0) continue;
        int32_t i = S.cp_i[p], j = S.cp_j[p];
        uint64_t ij = S.bit(i, j);
        bool exist = S.active.get(ij);
        if (exist && !valid[p]) {
            S.ptr_inactive++;
            S.active.clear(ij);
            S.ended++;
        } else if (!exist && valid[p]) {
            if (!append_contact(S, zero_contact(S, i, j))) return;
            S.active.put(ij);
            S.created++;
        }
    }
}

// resolve_collision! body for one active contact (src/kernels.jl:145-313)
ContactResult resolve_one(const Scene& S, const Contact& ct, bool is_bonded) {
    ContactResult out{};
    out.kind = 2;
    out.c = ct;
    const double dt = S.cfg.dt;
    const Grain &gi = S.g[ct.i], &gj = S.g[ct.j];
    V3 a = jl_normalize(gj.k - gi.k);
    M3 R = frame_to_x(a, S.cfg.tolerance);
    double Li = jl_norm(gj.k - gi.k);
    if (is_bonded) {
        V3 k = (gi.k + gj.k) * 0.5;
        V3 di = mv(R, gi.v) * dt, dj = mv(R, gj.v) * dt;
        V3 thi = mv(R, gi.w) * dt, thj = mv(R, gj.w) * dt;
        const Surface& sf = S.surf[gi.mid * S.nmat + gj.mid];
        double rj = sf.rho * jl_min(gi.r, gj.r);
        double Lj = Li;
        double Ej = sf.E, nu = sf.nu;
        double Ij = jl_pow(rj, 4) * kPi / 4;
        double phi = 20.0 / 3.0 * (rj * rj) / (Lj * Lj) * (1.0 + nu);
        double Aj = (rj * rj) * kPi;
        double k1 = Ej * Aj / Lj;
        double k2 = 12.0 * Ej * Ij / ((Lj * Lj) * Lj) / (1.0 + phi);
        double k3 = 6.0 * Ej * Ij / (Lj * Lj) / (1.0 + phi);
        double k4 = Ej * Ij / Lj / (1.0 + nu);
        double k5 = Ej * Ij * (4.0 + phi) / Lj / (1.0 + phi);
        double k6 = Ej * Ij * (2.0 - phi) / Lj / (1.0 + phi);
        V3 dF{k1 * (di.x - dj.x), k2 * (di.y - dj.y) + k3 * (thi.z + thj.z),
              k2 * (di.z - dj.z) - k3 * (thi.y + thj.y)};
        V3 dti{k4 * (thi.x - thj.x), (k3 * (dj.z - di.z) + k5 * thi.y) + k6 * thj.y,
               (k3 * (di.y - dj.y) + k5 * thi.z) + k6 * thj.z};
        V3 dtj{k4 * (thj.x - thi.x), (k3 * (dj.z - di.z) + k6 * thi.y) + k5 * thj.y,
               (k3 * (di.y - dj.y) + k6 * thi.z) + k5 * thj.z};
        V3 Fi = ct.F + dF;
        V3 Fj = -Fi;
        V3 ti = ct.ti + dti;
        V3 tj = ct.tj + dtj;
        double sci = Fj.x / Aj - rj / Ij * std::sqrt(ti.y * ti.y + ti.z * ti.z);
        double scj = Fj.x / Aj - rj / Ij * std::sqrt(tj.y * tj.y + tj.z * tj.z);
        double sc = -jl_min(sci, scj);
        double st = jl_max(sci, scj);
        double ss = std::fabs(ti.x) * rj / 2.0 / Ij + 4.0 / 3.0 / Aj * std::sqrt(Fi.y * Fi.y + Fi.z * Fi.z);
        if (sc >= sf.sc || st >= sf.st || ss >= sf.ss) {
            out.kind = 1;
            return out;
        }
        M3 Ri = inv3(R);
        out.fi = mv(Ri, -Fi);
        out.fj = mv(Ri, -Fj);
        out.mi = mv(Ri, -ti);
        out.mj = mv(Ri, -tj);
        out.c.k = k;
        out.c.F = Fi;
        out.c.ti = ti;
        out.c.tj = tj;
        out.c.s = {0, 0, 0};
        return out;
    }
    // Hertz-Mindlin (src/kernels.jl:240-313)
    double gap = Li - gi.r - gj.r;
    if (gap > 0) out.warn_gap = 1;
    double dn = std::fabs(gap);
    V3 k = gi.k + jl_normalize(gj.k - gi.k) * (gi.r - dn);
    V3 ki = k - gi.k, kj = k - gj.k;
    V3 vci = cross(gi.w, ki) + gi.v;
    V3 vcj = cross(gj.w, kj) + gj.v;
    V3 vc = mv(R, vcj - vci);
    const Material &mi = S.mat[gi.mid], &mj = S.mat[gj.mid];
    const Surface& sf = S.surf[gi.mid * S.nmat + gj.mid];
    double Ys = 1.0 / ((1.0 - mi.nu * mi.nu) / mi.E + (1.0 - mj.nu * mj.nu) / mj.E);
    double Gs = 1.0 / (2.0 * (2.0 - mi.nu) * (1.0 + mi.nu) / mi.E +
                       2.0 * (2.0 - mj.nu) * (1.0 + mj.nu) / mj.E);
    double Rs = 1.0 / (1.0 / gi.r + 1.0 / gj.r);
    double ms = 1.0 / (1.0 / gi.m + 1.0 / gj.m);
    double le = std::log(sf.e);
    double beta = le / std::sqrt(le * le + kPi * kPi);
    double Sn = 2.0 * Ys * std::sqrt(Rs * dn);
    double St = 8.0 * Gs * std::sqrt(Rs * dn);
    double kn = 4.0 / 3.0 * Ys * std::sqrt(Rs * dn);
    double gn = -2.0 * beta * std::sqrt(5.0 / 6.0 * Sn * ms);
    if (gn < 0) out.warn_gamma++;
    double kt = 8.0 * Gs * std::sqrt(Rs * dn);
    double gt = -2.0 * beta * std::sqrt(5.0 / 6.0 * St * ms);
    if (gt < 0) out.warn_gamma++;
    V3 ds{vc.x * 0.0, vc.y * dt, vc.z * dt};
    V3 s = ct.s + ds;
    double F1 = -kn * gap - gn * vc.x;
    V3 Ft = (-kt) * s;
    double F2, F3;
    double nFt = jl_norm(Ft);
    if (nFt >= sf.mu * F1) {
        double ratio = sf.mu * F1 / nFt;
        F2 = ratio * Ft.y;
        F3 = ratio * Ft.z;
        s = {s.x, F2 / kt, F3 / kt};
    } else {
        F2 = Ft.y - gt * vc.y;
        F3 = Ft.z - gt * vc.z;
    }
    V3 Fi{F1, F2, F3};
    V3 Fig = mv(inv3(R), -Fi);
    out.fi = Fig;
    out.fj = -Fig;
    out.mi = cross(ki, Fig);
    out.mj = cross(kj, -Fig);
    out.c.k = k;
    out.c.F = Fi;
    out.c.s = s;
    return out;
}

void add3(std::vector<double>& a, int64_t i, V3 v) {
    a[3 * i] += v.x;
    a[3 * i + 1] += v.y;
    a[3 * i + 2] += v.z;
}

void resolve_collision(Scene& S) {
    const int64_t C = S.ptr_total;
    std::vector<ContactResult> res(C);
#pragma omp parallel for num_threads(S.threads) schedule(static)
    for (int64_t c = 0; c < C; ++c) {
        const Contact& ct = S.contacts[c];
        uint64_t ij = S.bit(ct.i, ct.j);
        if (!S.active.get(ij)) { res[c].kind = 0; continue; }
        res[c] = resolve_one(S, ct, S.bonded.get(ij));
    }
    for (int64_t c = 0; c < C; ++c) {
        const ContactResult& r = res[c];
        if (r.kind == 0) continue;
        S.warn_gap += r.warn_gap;
        S.warn_gamma += r.warn_gamma;
        const Contact& ct = S.contacts[c];
        if (r.kind == 1) {
            uint64_t ij = S.bit(ct.i, ct.j);
            S.ptr_inactive++;
            S.active.clear(ij);
            S.bonded.clear(ij);
            S.broken++;
            continue;
        }
        add3(S.forces, ct.i, r.fi);
        add3(S.forces, ct.j, r.fj);
        add3(S.moments, ct.i, r.mi);
        add3(S.moments, ct.j, r.mj);
        S.contacts[c] = r.c;
    }
}

// resolve_wall! (src/kernels.jl:317-426): every wall j in order, per particle
void resolve_wall(Scene& S) {
    const double dt = S.cfg.dt, tol = S.cfg.tolerance;
    const int64_t nw = (int64_t)S.walls.size();
    int64_t warn = 0;
#pragma omp parallel for num_threads(S.threads) schedule(static) reduction(+ : warn)
    for (int64_t i = 0; i < S.n; ++i) {
      const Grain& G = S.g[i];
      for (int64_t w = 0; w < nw; ++w) {
        const Wall& W = S.walls[w];
        Contact& wc = S.wall_contacts[w * S.n + i];
        if (std::fabs(dot(G.k, W.n) - W.d) < G.r) {
            M3 R = frame_to_x(W.n, tol);
            double L = dot(G.k, W.n) - W.d;
            double gap = std::fabs(L) - G.r;
            double dn = std::fabs(gap);
            V3 ki{((-L) * W.n.x) / std::fabs(L) * (std::fabs(L) + dn / 2.0),
                  ((-L) * W.n.y) / std::fabs(L) * (std::fabs(L) + dn / 2.0),
                  ((-L) * W.n.z) / std::fabs(L) * (std::fabs(L) + dn / 2.0)};
            V3 k = G.k + ki;
            V3 vci = cross(G.w, ki) + G.v;
            V3 vc = mv(R, -vci);
            const Material &mi = S.mat[G.mid], &mj = S.mat[W.mid];
            const Surface& sf = S.surf[G.mid * S.nmat + W.mid];
            double Ys = 1.0 / ((1.0 - mi.nu * mi.nu) / mi.E + (1.0 - mj.nu * mj.nu) / mj.E);
            double Gs = 1.0 / (2.0 * (2.0 - mi.nu) * (1.0 + mi.nu) / mi.E +
                               2.0 * (2.0 - mj.nu) * (1.0 + mj.nu) / mj.E);
            double Rs = G.r, ms = G.m;
            double le = std::log(sf.e);
            double beta = le / std::sqrt(le * le + kPi * kPi);
            double Sn = 2.0 * Ys * std::sqrt(Rs * dn);
            double St = 8.0 * Gs * std::sqrt(Rs * dn);
            double kn = 4.0 / 3.0 * Ys * std::sqrt(Rs * dn);
            double gn = -2.0 * beta * std::sqrt(5.0 / 6.0 * Sn * ms);
            if (gn < 0) warn++;
            double kt = 8.0 * Gs * std::sqrt(Rs * dn);
            double gt = -2.0 * beta * std::sqrt(5.0 / 6.0 * St * ms);
            if (gt < 0) warn++;
            V3 ds{vc.x * 0.0, vc.y * dt, vc.z * dt};
            V3 s = wc.s + ds;
            double F1 = -kn * gap - gn * vc.x;
            V3 Ft = (-kt) * s;
            double F2, F3;
            double nFt = jl_norm(Ft);
            if (nFt >= sf.mu * F1) {
                double ratio = sf.mu * F1 / nFt;
                F2 = ratio * Ft.y;
                F3 = ratio * Ft.z;
                s = {s.x, F2 / kt, F3 / kt};
            } else {
                F2 = Ft.y - gt * vc.y;
                F3 = Ft.z - gt * vc.z;
            }
            V3 Fi{F1, F2, F3};
            V3 Fig = mv(inv3(R), -Fi);
            add3(S.forces, i, Fig);
            add3(S.moments, i, cross(ki, Fig));
            wc.i = (int32_t)i;
            wc.j = -1;
            wc.midi = G.mid;
            wc.midj = W.mid;
            wc.k = k;
            wc.F = Fi;
            wc.ti = wc.tj = {0, 0, 0};
            wc.s = s;
        } else {
            wc = Contact{};
        }
      }
    }
    S.warn_gamma += warn;
}

// apply_body_force! + update! (src/kernels.jl:428-485)
void body_and_update(Scene& S) {
    const double dt = S.cfg.dt, damp = S.cfg.global_damping;
    const V3 grav{S.cfg.gravity[0], S.cfg.gravity[1], S.cfg.gravity[2]};
#pragma omp parallel for num_threads(S.threads) schedule(static)
    for (int64_t i = 0; i < S.n; ++i) {
        Grain& G = S.g[i];
        add3(S.forces, i, grav * G.m);
        V3 F{S.forces[3 * i], S.forces[3 * i + 1], S.forces[3 * i + 2]};
        V3 T{S.moments[3 * i], S.moments[3 * i + 1], S.moments[3 * i + 2]};
        V3 dF{-damp * std::fabs(F.x) * jl_sign(G.v.x), -damp * std::fabs(F.y) * jl_sign(G.v.y),
              -damp * std::fabs(F.z) * jl_sign(G.v.z)};
        V3 dT{-damp * std::fabs(T.x) * jl_sign(G.w.x), -damp * std::fabs(T.y) * jl_sign(G.w.y),
              -damp * std::fabs(T.z) * jl_sign(G.w.z)};
        add3(S.forces, i, dF);
        add3(S.moments, i, dT);
    }
#pragma omp parallel for num_threads(S.threads) schedule(static)
    for (int64_t i = 0; i < S.n; ++i) {
        Grain& G = S.g[i];
        V3 F{S.forces[3 * i], S.forces[3 * i + 1], S.forces[3 * i + 2]};
        V3 a = F / G.m;
        V3 k = (G.k + G.v * dt) + (0.5 * a) * (dt * dt);
        V3 v = G.v + a * dt;
        const double* q = G.q;
        V3 w = G.w;
        M3 R = quat_to_matrix(q);
        V3 T{S.moments[3 * i], S.moments[3 * i + 1], S.moments[3 * i + 2]};
        V3 Tl = mv(R, T);
        V3 wl = mv(R, w);
        V3 dwl = mv(inv3(G.I), Tl - cross(wl, mv(G.I, wl)));
        V3 dw = mv(inv3(R), dwl);
        double dq1 = -0.5 * ((q[1] * w.x + q[2] * w.y) + q[3] * w.z);
        double dq2 = 0.5 * ((q[0] * w.x + q[2] * w.z) - q[3] * w.y);
        double dq3 = 0.5 * ((q[0] * w.y + q[1] * w.z) + q[3] * w.x);
        double dq4 = 0.5 * ((q[0] * w.z + q[1] * w.y) - q[2] * w.x);
        double nq[4] = {q[0] + dq1, q[1] + dq2, q[2] + dq3, q[3] + dq4};
        double nn = std::sqrt(((nq[0] * nq[0] + nq[1] * nq[1]) + nq[2] * nq[2]) + nq[3] * nq[3]);
        for (int c = 0; c < 4; ++c) G.q[c] = nq[c] / nn;
        G.w = w + dw * dt;
        G.k = k;
        G.v = v;
        G.a = a;
        G.dw = dw;
    }
}

// late_clear_state! (src/executor.jl:140-153)
void late_clear(Scene& S) {
    if (S.ptr_inactive == 0) return;
    uint32_t o = 0;
    for (uint32_t c = 0; c < S.ptr_total; ++c) {
        const Contact& ct = S.contacts[c];
        if (S.active.get(S.bit(ct.i, ct.j))) S.contacts[o++] = ct;
    }
    S.ptr_total = o;
    S.ptr_inactive = 0;
}

// simulate! (src/executor.jl:162-172)
void simulate(Scene& S) {
    std::fill(S.forces.begin(), S.forces.end(), 0.0);
    std::fill(S.moments.begin(), S.moments.end(), 0.0);
    broadphase(S);
    update_contacts(S);
    if (S.error) return;
    if (S.ptr_total - S.ptr_inactive > 0) resolve_collision(S);
    resolve_wall(S);
    body_and_update(S);
    late_clear(S);
    S.steps++;
}

}  // namespace

// ---- C interface used by the tests and bench.py ------------------------------
extern "C" {

void* oracle_create(const DemConfigC* cfg, const DemParticlesIn* p, int threads) {
    if (!cfg || !p || p->n < 0) return nullptr;
    Scene* S = new Scene();
    S->threads = threads > 0 ? threads : 1;
    setup(*S, *cfg, *p);
    return S;
}

// A scene with its own material, surface and wall tables (the reference's
// GlobalData.materials / surfaces / walls and Grain.mid); indices 0-based.
void* oracle_create_tables(const DemConfigC* cfg, const DemParticlesIn* p, const DemTables* t,
                           int threads) {
    if (!cfg || !p || p->n < 0 || !t || t->n_materials < 1) return nullptr;
    Scene* S = new Scene();
    S->threads = threads > 0 ? threads : 1;
    setup(*S, *cfg, *p);
    const int nm = (int)t->n_materials;
    S->nmat = nm;
    S->mat.clear();
    for (int a = 0; a < nm; ++a) {
        const DemMaterial& m = t->materials[a];
        S->mat.push_back({m.density, m.elastic_modulus, m.poisson_ratio});
    }
    S->surf.clear();
    for (int q = 0; q < nm * nm; ++q) {
        const DemSurface& f = t->surfaces[q];
        S->surf.push_back({f.friction, f.restitution, f.rolling_resistance, f.bond_radius_ratio,
                           f.bond_elastic_modulus, f.bond_poisson_ratio,
                           f.bond_compressive_strength, f.bond_tensile_strength,
                           f.bond_shear_strength});
    }
    S->walls.clear();
    for (int64_t w = 0; w < t->n_walls; ++w) {
        const DemWall& W = t->walls[w];
        S->walls.push_back({{W.normal[0], W.normal[1], W.normal[2]}, W.distance,
                            (int32_t)W.material});
    }
    S->wall_contacts.assign((size_t)S->n * S->walls.size(), Contact{});
    for (int64_t i = 0; i < S->n; ++i) S->g[i].mid = t->grain_material[i];
    return S;
}

void oracle_destroy(void* h) { delete static_cast<Scene*>(h); }

// wall_contacts[w+1, :].𝐬 (3n doubles)
int oracle_get_wall_shear(void* h, int w, double* out) {
    Scene& S = *static_cast<Scene*>(h);
    if (w < 0 || w >= (int)S.walls.size()) return DEM_ERR_INVALID;
    for (int64_t i = 0; i < S.n; ++i)
        for (int c = 0; c < 3; ++c) out[3 * i + c] = at(S.wall_contacts[w * S.n + i].s, c);
    return DEM_OK;
}
int oracle_set_wall_shear(void* h, int w, const double* in) {
    Scene& S = *static_cast<Scene*>(h);
    if (w < 0 || w >= (int)S.walls.size()) return DEM_ERR_INVALID;
    for (int64_t i = 0; i < S.n; ++i)
        S.wall_contacts[w * S.n + i].s = {in[3 * i], in[3 * i + 1], in[3 * i + 2]};
    return DEM_OK;
}

void oracle_set_threads(void* h, int threads) {
    static_cast<Scene*>(h)->threads = threads > 0 ? threads : 1;
}

int oracle_max_threads(void) { return omp_get_max_threads(); }

int oracle_init_bonds(void* h) {
    Scene& S = *static_cast<Scene*>(h);
    init_bonds(S);
    return S.error;
}

int oracle_step(void* h, int64_t nsteps) {
    Scene& S = *static_cast<Scene*>(h);
    for (int64_t s = 0; s < nsteps && !S.error; ++s) simulate(S);
    return S.error;
}

int oracle_get_derived(void* h, DemDerived* out) {
    Scene& S = *static_cast<Scene*>(h);
    out->cell_size = S.cell_size;
    out->r_max = S.rmax;
    out->hash_table_size = S.H;
    out->total_steps = S.total_steps;
    out->save_per_steps = S.save_per_steps;
    out->material_density = S.material_density;
    out->contact_capacity = S.n * S.cfg.max_coordinate_number;
    return DEM_OK;
}

int oracle_get_static(void* h, DemParticleStatic* out) {
    Scene& S = *static_cast<Scene*>(h);
    for (int64_t i = 0; i < S.n; ++i) {
        if (out->radius) out->radius[i] = S.g[i].r;
        if (out->radius0) out->radius0[i] = S.g[i].r0;
        if (out->mass) out->mass[i] = S.g[i].m;
        if (out->inertia) out->inertia[i] = S.g[i].I.a[0][0];
    }
    return DEM_OK;
}

int oracle_get_particles(void* h, DemParticleState* out) {
    Scene& S = *static_cast<Scene*>(h);
    for (int64_t i = 0; i < S.n; ++i) {
        const Grain& G = S.g[i];
        for (int c = 0; c < 3; ++c) {
            if (out->pos) out->pos[3 * i + c] = at(G.k, c);
            if (out->vel) out->vel[3 * i + c] = at(G.v, c);
            if (out->omega) out->omega[3 * i + c] = at(G.w, c);
            if (out->force) out->force[3 * i + c] = S.forces[3 * i + c];
            if (out->moment) out->moment[3 * i + c] = S.moments[3 * i + c];
            if (out->wall_shear)
                out->wall_shear[3 * i + c] = S.walls.empty() ? 0.0 : at(S.wall_contacts[i].s, c);
        }
        if (out->quat)
            for (int c = 0; c < 4; ++c) out->quat[4 * i + c] = G.q[c];
    }
    return DEM_OK;
}

int oracle_set_particles(void* h, const DemParticleState* in) {
    Scene& S = *static_cast<Scene*>(h);
    for (int64_t i = 0; i < S.n; ++i) {
        Grain& G = S.g[i];
        if (in->pos) G.k = {in->pos[3 * i], in->pos[3 * i + 1], in->pos[3 * i + 2]};
        if (in->vel) G.v = {in->vel[3 * i], in->vel[3 * i + 1], in->vel[3 * i + 2]};
        if (in->omega) G.w = {in->omega[3 * i], in->omega[3 * i + 1], in->omega[3 * i + 2]};
        if (in->quat)
            for (int c = 0; c < 4; ++c) G.q[c] = in->quat[4 * i + c];
        if (in->wall_shear && !S.walls.empty())
            S.wall_contacts[i].s = {in->wall_shear[3 * i], in->wall_shear[3 * i + 1],
                                    in->wall_shear[3 * i + 2]};
    }
    return DEM_OK;
}

int oracle_get_contacts(void* h, DemContacts* out, int64_t cap, int64_t* n_out) {
    Scene& S = *static_cast<Scene*>(h);
    std::vector<uint32_t> idx;
    for (uint32_t c = 0; c < S.ptr_total; ++c) {
        const Contact& ct = S.contacts[c];
        if (S.active.get(S.bit(ct.i, ct.j))) idx.push_back(c);
    }
    std::sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
        const Contact &x = S.contacts[a], &y = S.contacts[b];
        return x.i != y.i ? x.i < y.i : x.j < y.j;
    });
    *n_out = (int64_t)idx.size();
    if ((int64_t)idx.size() > cap) return DEM_ERR_CAPACITY;
    for (size_t t = 0; t < idx.size(); ++t) {
        const Contact& ct = S.contacts[idx[t]];
        if (out->i) out->i[t] = ct.i;
        if (out->j) out->j[t] = ct.j;
        if (out->bonded) out->bonded[t] = S.bonded.get(S.bit(ct.i, ct.j)) ? 1 : 0;
        for (int c = 0; c < 3; ++c) {
            if (out->point) out->point[3 * t + c] = at(ct.k, c);
            if (out->force) out->force[3 * t + c] = at(ct.F, c);
            if (out->torque_i) out->torque_i[3 * t + c] = at(ct.ti, c);
            if (out->torque_j) out->torque_j[3 * t + c] = at(ct.tj, c);
            if (out->shear) out->shear[3 * t + c] = at(ct.s, c);
        }
    }
    return DEM_OK;
}

int oracle_set_contacts(void* h, const DemContacts* in, int64_t n) {
    Scene& S = *static_cast<Scene*>(h);
    S.active.init(S.n);
    S.bonded.init(S.n);
    S.contacts.clear();
    S.ptr_total = S.ptr_inactive = 0;
    for (int64_t t = 0; t < n; ++t) {
        int32_t i = in->i[t], j = in->j[t];
        if (i < 0 || j <= i || j >= S.n) return DEM_ERR_INVALID;
        Contact c = zero_contact(S, i, j);
        auto g3 = [&](const double* a) { return a ? V3{a[3 * t], a[3 * t + 1], a[3 * t + 2]} : V3{0, 0, 0}; };
        c.k = g3(in->point);
        c.F = g3(in->force);
        c.ti = g3(in->torque_i);
        c.tj = g3(in->torque_j);
        c.s = g3(in->shear);
        if (!append_contact(S, c)) return DEM_ERR_CAPACITY;
        uint64_t ij = S.bit(i, j);
        S.active.put(ij);
        if (in->bonded && in->bonded[t]) S.bonded.put(ij);
    }
    return DEM_OK;
}

int oracle_get_stats(void* h, DemStats* out) {
    Scene& S = *static_cast<Scene*>(h);
    int64_t act = 0, bnd = 0;
    for (uint32_t c = 0; c < S.ptr_total; ++c) {
        const Contact& ct = S.contacts[c];
        uint64_t ij = S.bit(ct.i, ct.j);
        if (S.active.get(ij)) {
            ++act;
            if (S.bonded.get(ij)) ++bnd;
        }
    }
    std::memset(out, 0, sizeof(*out));
    out->n_particles = S.n;
    out->steps_done = S.steps;
    out->contacts = act;
    out->bonded = bnd;
    out->bonds_broken = S.broken;
    out->contacts_ended = S.ended;
    out->contacts_created = S.created;
    out->warn_gap = S.warn_gap;
    out->warn_damping = S.warn_gamma;
    out->error = S.error;
    out->precision = DEM_FP64;
    return DEM_OK;
}

// Broad phase only, on the current positions (see dem_debug_broadphase).
int oracle_broadphase(void* h, int32_t* cell, uint32_t* morton, uint32_t* bucket,
                      uint32_t* bucket_count, uint32_t* sorted, int32_t* cp, int64_t cp_cap,
                      int64_t* cp_n) {
    Scene& S = *static_cast<Scene*>(h);
    broadphase(S);
    for (int64_t i = 0; i < S.n; ++i) {
        if (cell)
            for (int c = 0; c < 3; ++c) cell[3 * i + c] = S.kid[3 * i + c];
        if (morton) morton[i] = S.morton[i];
        if (bucket) bucket[i] = S.hid[i];
        if (sorted) sorted[i] = S.pid[i];
    }
    if (bucket_count) std::memcpy(bucket_count, S.ht.data(), sizeof(uint32_t) * S.ht.size());
    *cp_n = (int64_t)S.cp_i.size();
    if (*cp_n > cp_cap) return cp ? DEM_ERR_CAPACITY : DEM_OK;
    if (cp)
        for (int64_t p = 0; p < *cp_n; ++p) {
            cp[2 * p] = S.cp_i[p];
            cp[2 * p + 1] = S.cp_j[p];
        }
    return DEM_OK;
}

// Pure helpers exposed for known-answer tests.
uint32_t oracle_morton1(int32_t x, int32_t y, int32_t z) { return morton1(x, y, z); }

void oracle_quat_to_matrix(const double* q, double* R9) {
    M3 R = quat_to_matrix(q);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R9[3 * r + c] = R.a[r][c];
}

void oracle_frame_to_x(const double* a, double tol, double* R9) {
    M3 R = frame_to_x(V3{a[0], a[1], a[2]}, tol);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R9[3 * r + c] = R.a[r][c];
}

double oracle_jl_norm(const double* a) { return jl_norm(V3{a[0], a[1], a[2]}); }

// Single-contact and single-particle evaluations through the oracle's own
// resolve_one / resolve_wall / body_and_update, for the golden vectors that
// tests/golden/make_physics_golden.py computes with the reference's dem.py
// (DEMSolver.resolve dem.py:1357-1606, evaluate_wall/resolve_wall
// dem.py:1609-1743, apply_body_force dem.py:1280-1305, update
// dem.py:1309-1354).  A grain record is 16 doubles:
//   r, m, k[3], v[3], w[3], q[4] (w,x,y,z), I (isotropic moment of inertia).
// Material 0 is the particles', material 1 the wall's; the tables come from
// `cfg` as in `solve` (the particle density does not enter any force).
static void load_grain(Grain& G, const double* g) {
    G.id = G.gid = G.mid = 0;
    G.r = g[0];
    G.m = g[1];
    G.V = 0.0;
    G.r0 = G.r;
    G.k = {g[2], g[3], g[4]};
    G.v = {g[5], g[6], g[7]};
    G.a = {0, 0, 0};
    G.w = {g[8], g[9], g[10]};
    for (int c = 0; c < 4; ++c) G.q[c] = g[11 + c];
    G.dw = {0, 0, 0};
    G.I = M3{{{g[15], 0.0, 0.0}, {0.0, g[15], 0.0}, {0.0, 0.0, g[15]}}};
}

static double* put3(double* o, V3 v) {
    o[0] = v.x; o[1] = v.y; o[2] = v.z;
    return o + 3;
}

// One particle-particle contact (i = grain 0, j = grain 1).  `state` is the
// contact's carried state F[3], ti[3], tj[3], s[3]; `bonded` selects EBPM.
// out (28): kind (1 bond broken, 2 forces applied), fi, fj, mi, mj, then the
// contact's new k, F, ti, tj, s.
int oracle_eval_pair(const DemConfigC* cfg, const double* gi, const double* gj,
                     const double* state, int bonded, double* out) {
    Scene S;
    S.cfg = *cfg;
    S.n = 2;
    S.g.resize(2);
    load_grain(S.g[0], gi);
    load_grain(S.g[1], gj);
    set_tables(S);
    Contact ct{};
    ct.i = 0; ct.j = 1;
    ct.F = {state[0], state[1], state[2]};
    ct.ti = {state[3], state[4], state[5]};
    ct.tj = {state[6], state[7], state[8]};
    ct.s = {state[9], state[10], state[11]};
    ContactResult r = resolve_one(S, ct, bonded != 0);
    out[0] = r.kind;
    double* o = out + 1;
    o = put3(o, r.fi); o = put3(o, r.fj); o = put3(o, r.mi); o = put3(o, r.mj);
    o = put3(o, r.c.k); o = put3(o, r.c.F); o = put3(o, r.c.ti); o = put3(o, r.c.tj);
    put3(o, r.c.s);
    return DEM_OK;
}

// One particle against the configured wall, with the wall contact's carried
// shear displacement `s_in`.  out (16): touching, force, moment, then the wall
// contact's k, F, s.
int oracle_eval_wall(const DemConfigC* cfg, const double* g, const double* s_in, double* out) {
    Scene S;
    S.cfg = *cfg;
    S.n = 1;
    S.threads = 1;
    S.g.resize(1);
    load_grain(S.g[0], g);
    set_tables(S);
    S.wall_contacts.assign(1, Contact{});
    S.wall_contacts[0].s = {s_in[0], s_in[1], s_in[2]};
    S.forces.assign(3, 0.0);
    S.moments.assign(3, 0.0);
    resolve_wall(S);
    const Contact& wc = S.wall_contacts[0];
    out[0] = wc.j == -1 ? 1.0 : 0.0;
    double* o = out + 1;
    o = put3(o, {S.forces[0], S.forces[1], S.forces[2]});
    o = put3(o, {S.moments[0], S.moments[1], S.moments[2]});
    o = put3(o, wc.k); o = put3(o, wc.F);
    put3(o, wc.s);
    return DEM_OK;
}

// apply_body_force! + update! for n particles whose contact force and moment
// sums are F, T (3n each).  out (19 per particle): k, v, q, w, then the force
// and moment after gravity and damping.
int oracle_eval_update(const DemConfigC* cfg, int64_t n, const double* g, const double* F,
                       const double* T, double* out) {
    Scene S;
    S.cfg = *cfg;
    S.n = n;
    S.threads = 1;
    S.g.resize(n);
    for (int64_t i = 0; i < n; ++i) load_grain(S.g[i], g + 16 * i);
    S.forces.assign(F, F + 3 * n);
    S.moments.assign(T, T + 3 * n);
    body_and_update(S);
    for (int64_t i = 0; i < n; ++i) {
        const Grain& G = S.g[i];
        double* o = out + 19 * i;
        o = put3(o, G.k); o = put3(o, G.v);
        for (int c = 0; c < 4; ++c) *o++ = G.q[c];
        o = put3(o, G.w);
        o = put3(o, {S.forces[3 * i], S.forces[3 * i + 1], S.forces[3 * i + 2]});
        put3(o, {S.moments[3 * i], S.moments[3 * i + 1], S.moments[3 * i + 2]});
    }
    return DEM_OK;
}

}  // extern "C"
