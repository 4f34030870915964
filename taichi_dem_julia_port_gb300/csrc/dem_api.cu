// dem_api.cu — the C ABI of libdem_sm100a.so (include/dem_gb300.h).
//
// Host responsibilities: the per-scene setup that `solve` performs before its
// loop (src/executor.jl:217-315), device buffers, the CUDA-graph step
// (`simulate!`, src/executor.jl:162-172), host<->device state exchange, and the
// arena of independent scenes (slot and bucket-range allocation, scene modes).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iterator>
#include <map>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "dem_gb300.h"
#include "dem_internal.h"

using namespace dem;

namespace {

constexpr double kPi = 3.141592653589793;
// Neighbour-list partners (j > i within reach) per particle: the scene's
// max_coordinate_number, at least 16 and at most 256.  A list that overflows
// makes its scene run the full pair search at the next step, so a dense
// polydisperse packing, whose large spheres have many small neighbours, needs
// room for them (measured: 100,000 spheres of radii 0.5-2 mm at solid
// fraction 0.45 overflowed 16-entry lists on every step).
constexpr int kListMin = 16, kListMax = 256;
inline int list_capacity(int64_t max_coordinate_number) {
    return (int)std::min<int64_t>(std::max<int64_t>(max_coordinate_number, kListMin), kListMax);
}

struct M3 {
    double a[3][3];
};
inline void cross(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
inline double dot3(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
double norm3(const double* a) {
    double l = std::sqrt((a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]);
    if (l > 0.0 && l < INFINITY) return l;
    if (std::isnan(a[0]) || std::isnan(a[1]) || std::isnan(a[2])) return NAN;
    double sc = std::max(std::fabs(a[0]), std::max(std::fabs(a[1]), std::fabs(a[2])));
    if (sc == 0.0) return 0.0;
    double x = a[0] / sc, y = a[1] / sc, z = a[2] / sc;
    return sc * std::sqrt((x * x + y * y) + z * z);
}
// Wall contact frame, built as src/kernels.jl:332-352 builds it.
M3 wall_frame(const double* n, double tol) {
    const double b[3] = {1.0, 0.0, 0.0};
    double v[3];
    cross(n, b, v);
    const double s = norm3(v), c = dot3(n, b);
    M3 R;
    if (s < tol) {
        const double sg = c > 0.0 ? 1.0 : -1.0;
        R = M3{{{sg, 0, 0}, {0, 1, 0}, {0, 0, sg}}};
        return R;
    }
    const M3 vx{{{0.0, -v[2], v[1]}, {v[2], 0.0, -v[0]}, {-v[1], v[0], 0.0}}};
    M3 vx2;
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q)
            vx2.a[r][q] = (vx.a[r][0] * vx.a[0][q] + vx.a[r][1] * vx.a[1][q]) + vx.a[r][2] * vx.a[2][q];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q)
            R.a[r][q] = ((r == q ? 1.0 : 0.0) + vx.a[r][q]) + (vx2.a[r][q] * (1.0 - c)) / (s * s);
    return R;
}
// 3x3 inverse by cofactors of the columns (as `inv` of StaticArrays).
M3 inverse3(const M3& A) {
    double x0[3] = {A.a[0][0], A.a[1][0], A.a[2][0]};
    double x1[3] = {A.a[0][1], A.a[1][1], A.a[2][1]};
    double x2[3] = {A.a[0][2], A.a[1][2], A.a[2][2]};
    double y0[3], y1[3], y2[3];
    cross(x1, x2, y0);
    const double d = dot3(x0, y0);
    for (int c = 0; c < 3; ++c) {
        x0[c] /= d;
        y0[c] /= d;
    }
    cross(x2, x0, y1);
    cross(x0, x1, y2);
    M3 R;
    for (int c = 0; c < 3; ++c) {
        R.a[0][c] = y0[c];
        R.a[1][c] = y1[c];
        R.a[2][c] = y2[c];
    }
    return R;
}

struct Hertz {
    double Ys, Gs, beta, cgn, cgt;
};
// Y*, G*, β of src/kernels.jl:261-266 (constant per material pair).
Hertz hertz_constants(double Ei, double nui, double Ej, double nuj, double e) {
    Hertz h;
    h.Ys = 1.0 / ((1.0 - nui * nui) / Ei + (1.0 - nuj * nuj) / Ej);
    h.Gs = 1.0 / (2.0 * (2.0 - nui) * (1.0 + nui) / Ei + 2.0 * (2.0 - nuj) * (1.0 + nuj) / Ej);
    const double le = std::log(e);
    h.beta = le / std::sqrt(le * le + kPi * kPi);
    h.cgn = -2.0 * h.beta * std::sqrt(5.0 / 3.0 * h.Ys);
    h.cgt = -2.0 * h.beta * std::sqrt(20.0 / 3.0 * h.Gs);
    return h;
}

thread_local char g_msg[512];
// what the last input check that returned DEM_ERR_INVALID on this thread found
// (cleared by the entry points that check their input)
thread_local char g_invalid[256];

// First-fit allocator of [start, start + len) ranges inside [0, cap).
struct FreeList {
    std::vector<std::pair<int64_t, int64_t>> free;  // (start, len), sorted by start
    void init(int64_t cap) {
        free.clear();
        if (cap > 0) free.push_back({0, cap});
    }
    bool take(int64_t len, int64_t* start) {
        if (len == 0) {
            *start = 0;
            return true;
        }
        for (size_t k = 0; k < free.size(); ++k) {
            if (free[k].second >= len) {
                *start = free[k].first;
                free[k].first += len;
                free[k].second -= len;
                if (free[k].second == 0) free.erase(free.begin() + (long)k);
                return true;
            }
        }
        return false;
    }
    void give(int64_t start, int64_t len) {
        if (len == 0) return;
        auto it = std::lower_bound(free.begin(), free.end(), std::make_pair(start, (int64_t)0));
        it = free.insert(it, {start, len});
        size_t k = (size_t)(it - free.begin());
        if (k + 1 < free.size() && free[k].first + free[k].second == free[k + 1].first) {
            free[k].second += free[k + 1].second;
            free.erase(free.begin() + (long)k + 1);
        }
        if (k > 0 && free[k - 1].first + free[k - 1].second == free[k].first) {
            free[k - 1].second += free[k].second;
            free.erase(free.begin() + (long)k);
        }
    }
};

struct SceneHost {
    int mode = kModeFree;
    DemConfigC cfg{};
    DemDerived der{};
    SceneParams sp{};
    double min_cell = 0.0;  // smallest search cell that finds every touching pair
    double rmax = 0.0;      // largest radius
    double cell_factor = 1.0;
    double skin_factor = 0.9;
    int64_t steps = 0, target = 0;
};

// Search cells of a scene for a cell factor f: f·(the reference's cell),
// clamped to [min_cell, the reference's cell].  The neighbour-list skin is
// skin_factor times the slack the octant search leaves for it: a pair found
// from i's octant buckets lies within cell/2, so the lists hold every pair
// within rᵢ + rⱼ + skin when skin <= cell/2 - 2·max r.
void set_search_cell(SceneParams& p, double f, double min_cell, bool empty, double rmax,
                     double skin_factor) {
    f = f > 0 ? f : 1.0;
    p.cell = empty ? p.cell_ref : std::min(p.cell_ref, std::max(f * p.cell_ref, min_cell));
    p.inv_cell = 1.0 / p.cell;
    p.same_grid = p.cell == p.cell_ref ? 1 : 0;
    const double slack = 0.5 * p.cell - 2.0 * rmax * (1.0 + 1e-6);
    p.skin = (!empty && slack > 0.0 && skin_factor > 0.0) ? std::min(skin_factor, 1.0) * slack : 0.0;
    p.f_skin = (float)(p.skin * (1.0 + 0x1p-20));
    p.f_half_skin = (float)(0.5 * p.skin * (1.0 - 0x1p-20));
    // the FP32 cell screen: 1/cell and max|dmin|/cell rounded up a little
    const double dm = std::max(std::fabs(p.dmin[0]), std::max(std::fabs(p.dmin[1]), std::fabs(p.dmin[2])));
    p.f_inv_cell = (float)p.inv_cell;
    p.f_inv_cell_ref = (float)p.inv_cell_ref;
    p.f_dmin_cells = (float)(dm * p.inv_cell * 1.001);
    p.f_dmin_cells_ref = (float)(dm * p.inv_cell_ref * 1.001);
}

// Per-particle arrays of one scene, derived on the host.
struct SceneArrays {
    std::vector<double> pos[3], vel[3];
    std::vector<double> m, inv_m, r, r0, inv_inertia, b_invA, b_rbI, b_EA, b_EI, b_phic;
};

uint32_t pow2_mask(uint32_t H) { return (H & (H - 1)) == 0 ? H - 1 : 0u; }

// The grain set-up and derived values of `solve` (src/executor.jl:217-315).
// The per-grain constants of `solve` (src/executor.jl:223-242) for grain i,
// and the largest radius so far.
static void grain_constants(const DemConfigC* cfg, const DemParticlesIn* pin, SceneArrays& A,
                            int i, double& rmax_r) {
    const double V = pin->volume[i], m = pin->mass[i];
    A.m[i] = m;
    A.r[i] = std::cbrt(V / (4.0 / 3.0 * kPi));
    A.r0[i] = A.r[i] * cfg->particle_contact_radius_multiplier;
    A.inv_inertia[i] = 1.0 / (2.0 / 5.0 * m * (A.r[i] * A.r[i]));
    A.inv_m[i] = 1.0 / m;
    // bond section of src/kernels.jl:178-184 for rb = ρ·rᵢ
    const double rb = cfg->bond_radius_ratio * A.r[i];
    const double Ab = rb * rb * kPi, Ib = rb * rb * (rb * rb) * (kPi / 4.0);
    A.b_invA[i] = 1.0 / Ab;
    A.b_rbI[i] = rb / Ib;
    A.b_EA[i] = cfg->bond_elastic_modulus * Ab;
    A.b_EI[i] = cfg->bond_elastic_modulus * Ib;
    A.b_phic[i] = 20.0 / 3.0 * (1.0 + cfg->bond_poisson_ratio) * (rb * rb);
    rmax_r = std::max(rmax_r, A.r[i]);
    for (int c = 0; c < 3; ++c) {
        A.pos[c][i] = pin->pos[3 * i + c];
        A.vel[c][i] = pin->vel[3 * i + c];
    }
}

int prepare_scene(const DemConfigC* cfg, const DemParticlesIn* pin, double cell_factor,
                  SceneHost& S, SceneArrays& A) {
    g_invalid[0] = 0;
    if (!cfg || !pin || pin->n < 0 || pin->n > 0x3fffffff) return DEM_ERR_INVALID;
    if (pin->n > 0 && (!pin->volume || !pin->mass || !pin->pos || !pin->vel)) return DEM_ERR_INVALID;
    if (!(cfg->dt > 0) || cfg->max_coordinate_number <= 0) return DEM_ERR_INVALID;
    const int n = (int)pin->n;
    S.cfg = *cfg;
    for (auto* v : {&A.m, &A.inv_m, &A.r, &A.r0, &A.inv_inertia, &A.b_invA, &A.b_rbI, &A.b_EA,
                    &A.b_EI, &A.b_phic})
        v->resize(n);
    for (int c = 0; c < 3; ++c) {
        A.pos[c].resize(n);
        A.vel[c].resize(n);
    }
    // per grain, independently: split over host threads for large scenes
    // (the results do not depend on the split)
    auto grains = [&](int i0, int i1, double& rmax, int& bad) {
        for (int i = i0; i < i1; ++i) {
            const double V = pin->volume[i], m = pin->mass[i];
            // a grain needs a positive finite volume and mass and a finite
            // position and velocity: anything else would make NaN cells and forces
            bool ok = V > 0 && m > 0 && std::isfinite(V) && std::isfinite(m);
            for (int c = 0; c < 3; ++c)
                ok = ok && std::isfinite(pin->pos[3 * i + c]) && std::isfinite(pin->vel[3 * i + c]);
            if (!ok) {
                bad = i;  // the first in this range
                return;
            }
            grain_constants(cfg, pin, A, i, rmax);
        }
    };
    const int nth = n < (1 << 16) ? 1
                                  : (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<double> rmaxs(nth, -INFINITY);
    std::vector<int> bads(nth, -1);
    {
        std::vector<std::thread> pool;
        const int64_t per = ((int64_t)n + nth - 1) / nth;
        for (int t = 1; t < nth; ++t) {
            const int i0 = (int)std::min<int64_t>(n, t * per);
            const int i1 = (int)std::min<int64_t>(n, (t + 1) * per);
            try {
                pool.emplace_back(grains, i0, i1, std::ref(rmaxs[t]), std::ref(bads[t]));
            } catch (...) {  // no thread to be had: this one does the range
                grains(i0, i1, rmaxs[t], bads[t]);
            }
        }
        grains(0, (int)std::min<int64_t>(n, per), rmaxs[0], bads[0]);
        for (auto& th : pool) th.join();
    }
    for (int t = 0; t < nth; ++t)
        if (bads[t] >= 0) {
            std::snprintf(g_invalid, sizeof(g_invalid),
                          "grain %d: volume, mass, position and velocity must be finite "
                          "(volume and mass > 0)", bads[t]);
            return DEM_ERR_INVALID;
        }
    double rmax_r = -INFINITY;
    for (double v : rmaxs) rmax_r = std::max(rmax_r, v);
    // derived sizes (src/executor.jl:244-267)
    DemDerived& D = S.der;
    D.material_density = n ? pin->mass[n - 1] / pin->volume[n - 1] : 0.0;
    D.r_max = rmax_r * cfg->particle_contact_radius_multiplier *
              (1.0 + cfg->bond_tensile_strength / cfg->bond_elastic_modulus) *
              cfg->neighboring_search_safety_factor;
    D.cell_size = 4.0 * D.r_max;
    int64_t prod = 1;
    for (int c = 0; c < 3; ++c)
        prod *= (int64_t)std::ceil((cfg->domain_max[c] - cfg->domain_min[c]) / D.cell_size);
    D.hash_table_size = std::min<int64_t>(std::max<int64_t>(prod, 1 << 20), 1 << 22);
    D.total_steps = (int64_t)std::trunc(cfg->target_time / cfg->dt);
    D.save_per_steps = (int64_t)std::trunc(cfg->saving_interval_time / cfg->dt);
    D.contact_capacity = (int64_t)n * cfg->max_coordinate_number;
    if (n > 0 && !(D.cell_size > 0 && std::isfinite(D.cell_size))) return DEM_ERR_INVALID;
    // device constants (materials / surfaces / wall of src/executor.jl:282-315)
    SceneParams& p = S.sp;
    std::memset(&p, 0, sizeof(p));
    p.n = n;
    p.Href = (uint32_t)D.hash_table_size;
    p.Href_mask = pow2_mask(p.Href);
    p.has_wall = 1;
    for (int c = 0; c < 3; ++c) {
        p.dmin[c] = cfg->domain_min[c];
        p.grav[c] = cfg->gravity[c];
        p.wn[c] = cfg->wall_normal[c];
    }
    p.cell_ref = D.cell_size;
    p.inv_cell_ref = 1.0 / D.cell_size;
    // Search cells.  A smaller cell still finds every touching pair with the
    // octant search as long as cell >= 2(rᵢ + rⱼ) for the radii in use, i.e.
    // 4·max r (stepping) and 4·max r₀ (bond initialisation).
    S.min_cell =
        4.0 * rmax_r * std::max(1.0, cfg->particle_contact_radius_multiplier) * (1.0 + 1e-9);
    S.rmax = n ? rmax_r : 0.0;
    S.cell_factor = cell_factor > 0 ? cell_factor : 1.0;
    set_search_cell(p, S.cell_factor, S.min_cell, n == 0, S.rmax, S.skin_factor);
    p.dt = cfg->dt;
    p.tol = cfg->tolerance;
    p.damping = cfg->global_damping;
    const Hertz pp = hertz_constants(cfg->particle_elastic_modulus, cfg->particle_poisson_ratio,
                                     cfg->particle_elastic_modulus, cfg->particle_poisson_ratio,
                                     cfg->pp_coefficient_restitution);
    p.pp_mu = cfg->pp_coefficient_friction;
    p.pp_Ys = pp.Ys;
    p.pp_Gs = pp.Gs;
    p.pp_cgn = pp.cgn;
    p.pp_cgt = pp.cgt;
    p.b_inv1pnu = 1.0 / (1.0 + cfg->bond_poisson_ratio);
    p.b_sc = cfg->bond_compressive_strength;
    p.b_st = cfg->bond_tensile_strength;
    p.b_ss = cfg->bond_shear_strength;
    p.wd = cfg->wall_distance;
    const M3 WR = wall_frame(cfg->wall_normal, cfg->tolerance);
    const M3 WRi = inverse3(WR);
    for (int r_ = 0; r_ < 3; ++r_)
        for (int c = 0; c < 3; ++c) {
            p.wR[3 * r_ + c] = WR.a[r_][c];
            p.wRinv[3 * r_ + c] = WRi.a[r_][c];
        }
    const Hertz pw = hertz_constants(cfg->particle_elastic_modulus, cfg->particle_poisson_ratio,
                                     cfg->wall_elastic_modulus, cfg->wall_poisson_ratio,
                                     cfg->pw_coefficient_restitution);
    p.pw_mu = cfg->pw_coefficient_friction;
    p.pw_Ys = pw.Ys;
    p.pw_Gs = pw.Gs;
    p.pw_cgn = pw.cgn;
    p.pw_cgt = pw.cgt;
    p.f_dt = (float)p.dt;
    p.f_inv1pnu = (float)p.b_inv1pnu;
    p.f_sc = (float)p.b_sc;
    p.f_st = (float)p.b_st;
    p.f_ss = (float)p.b_ss;
    p.f_mu = (float)p.pp_mu;
    p.f_kn = (float)(4.0 / 3.0 * p.pp_Ys);
    p.f_kt = (float)(8.0 * p.pp_Gs);
    p.f_cgn = (float)p.pp_cgn;
    p.f_cgt = (float)p.pp_cgt;
    p.f_tol4 = (float)(4.0 * p.tol * p.tol);
    p.f_tol1 = (float)(p.tol * p.tol * (1.0 - 0x1p-10));
    p.hdt2 = 0.5 * (p.dt * p.dt);
    p.tol2_lo = p.tol * p.tol * (1.0 - 0x1p-30);
    p.tol2_x4 = 4.0 * p.tol * p.tol;
    double c0 = -p.wd;
    for (int c = 0; c < 3; ++c) {
        p.f_wn[c] = (float)p.wn[c];
        c0 += p.wn[c] * p.dmin[c];
    }
    p.f_wc0 = (float)c0;
    return DEM_OK;
}

// Mode changes of up to 64 scenes, applied on the device in stream order.
struct ModeUpdates {
    int count;
    int idx[64];
    int mode[64];
};
__global__ void k_set_modes(SceneParams* sp, ModeUpdates u) {
    const int t = threadIdx.x;
    if (t < u.count) sp[u.idx[t]].mode = u.mode[t];
}
__global__ void k_fill_i32(int32_t* a, int64_t n, int32_t v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}
// A new scene's slots [p0, p0 + n) after its FP64 columns are uploaded: the
// identity orientation's w and the FP32 copies of the bond-section constants
// and of (rb/I, m, r) for the FP32 force mode, rounded to nearest as a host
// cast would round them.
__global__ void k_scene_columns(DemDev d, int64_t p0, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int64_t i = p0 + t;
    d.qw[i] = 1.0;
    d.bk32[i] = make_float4(__double2float_rn(d.b_phic[i]), __double2float_rn(d.b_EI[i]),
                            __double2float_rn(d.b_EA[i]), __double2float_rn(d.b_invA[i]));
    d.rm32[i] = make_float4(__double2float_rn(d.b_rbI[i]), __double2float_rn(d.m[i]),
                            __double2float_rn(d.r[i]), 0.0f);
}

}  // namespace

struct DemHandle {
    bool multi = false;
    bool tab = false;  // material / wall tables (dem_create_tables)
    int nwall = 1;     // wall-shear columns per slot
    int device = 0;
    int sm_count = 0;
    int n_cap = 0, c_cap = 0, s_cap = 0;
    uint32_t t_cap = 0;
    double cell_factor = 1.0;
    DemParams p{};
    DemDev d{};
    std::vector<SceneHost> scenes;
    FreeList pfree, tfree;
    int cur = 0;  // contact buffer holding the current state
    int64_t steps = 0;
    int64_t exchanges_direct = 0;  // fused downloads of dem_step_exchange
    int ntiles_cells = 0;
    LaunchShape shape{};
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    int graph_precision = -1;
    int enc = DEM_FP64;  // encoding of 𝐅ᵢ, 𝛕ᵢ, 𝛕ⱼ in the current contact buffer
    std::vector<void*> allocs;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double* xfer = nullptr;    // device staging: particle records in the host's layout
    int64_t xfer_n = 0;        // doubles
    int* err_host = nullptr;   // page-locked copy of the device error word
    int* err_dev = nullptr;    // its device address
    // the exchanged step of dem_step_exchange as one graph per contact-buffer
    // parity, for one set of caller buffers (key: their device addresses):
    // the position upload, then the contact update while a second stream
    // uploads velocities and spins, then forces and the integration (which
    // reads orientations and wall shear from the caller and writes the state
    // back into the caller's buffers)
    static constexpr int kXKey = 14;
    struct XGraph {
        cudaGraphExec_t exec = nullptr;
        const void* key[kXKey] = {};
    } xg[2];
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    // dem_step_profiled: the step's graph with an event before, between and
    // after its three kernels, per contact-buffer parity
    cudaGraphExec_t pg[2] = {nullptr, nullptr};
    cudaEvent_t pev[4] = {nullptr, nullptr, nullptr, nullptr};
    unsigned long long* counts = nullptr;  // dem_get_stats: a scene's active contacts, bonds
    int32_t* io_idx = nullptr;  // p4c records: per-slot counts and their scan (2n + 1)
    int64_t io_idx_n = 0;
    void* io_rec = nullptr;     // p4c records (64 bytes each)
    int64_t io_rec_n = 0;
};

#define CU(expr)                                                                            \
    do {                                                                                    \
        cudaError_t _e = (expr);                                                            \
        if (_e != cudaSuccess) {                                                            \
            std::snprintf(g_msg, sizeof(g_msg), "%s: %s", #expr, cudaGetErrorString(_e));   \
            return DEM_ERR_CUDA;                                                            \
        }                                                                                   \
    } while (0)

#define TRY(expr)                      \
    do {                               \
        int _rc = (expr);              \
        if (_rc != DEM_OK) return _rc; \
    } while (0)

namespace {

template <typename T>
int dalloc(DemHandle* h, T** ptr, size_t count) {
    void* p = nullptr;
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    CU(cudaMalloc(&p, bytes));
    h->allocs.push_back(p);
    CU(cudaMemsetAsync(p, 0, bytes, h->stream));
    *ptr = static_cast<T*>(p);
    return DEM_OK;
}

int check_device(int* dev, int* sms) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return DEM_ERR_NO_DEVICE;
    CU(cudaGetDevice(dev));
    cudaDeviceProp prop;
    CU(cudaGetDeviceProperties(&prop, *dev));
    if (prop.major != 10 || prop.minor != 3) {
        std::snprintf(g_msg, sizeof(g_msg), "device %d is sm_%d%d; this library is built for sm_103a",
                      *dev, prop.major, prop.minor);
        return DEM_ERR_NO_DEVICE;
    }
    *sms = prop.multiProcessorCount;
    return DEM_OK;
}

// Device buffers for n_cap particle slots, c_cap contacts, t_cap buckets.
int allocate(DemHandle* h) {
    const size_t n = (size_t)h->n_cap, cap = (size_t)h->c_cap, T = h->t_cap;
    DemDev& d = h->d;
    double** dbl[] = {&d.px, &d.py, &d.pz, &d.vx, &d.vy, &d.vz, &d.wx, &d.wy, &d.wz,
                      &d.qw, &d.qx, &d.qy, &d.qz, &d.m, &d.inv_m, &d.r, &d.r0, &d.inv_inertia,
                      &d.b_invA, &d.b_rbI, &d.b_EA, &d.b_EI, &d.b_phic,
                      &d.fx, &d.fy, &d.fz, &d.tx, &d.ty, &d.tz};
    for (double** a : dbl) TRY(dalloc(h, a, n));
    // wall shear: one column per wall, wall w of slot i at [w * n + i]
    for (double** a : {&d.wsx, &d.wsy, &d.wsz}) TRY(dalloc(h, a, n * (size_t)std::max(h->nwall, 1)));
    h->p.wstride = (int)n;
    TRY(dalloc(h, &d.cellinfo, n));
    TRY(dalloc(h, &d.scell, n));
    TRY(dalloc(h, &d.srow, n));
    TRY(dalloc(h, &d.bucket, n));
    TRY(dalloc(h, &d.cell_count, T));
    TRY(dalloc(h, &d.cell_start, T + 1));
    TRY(dalloc(h, &d.tile_sums, (size_t)scan_tiles((int64_t)T) + 1));
    TRY(dalloc(h, &d.unsorted, n));
    TRY(dalloc(h, &d.sorted, n));
    TRY(dalloc(h, &d.spos, n));
    TRY(dalloc(h, &d.spos32, n));
    for (int b = 0; b < 2; ++b) {
        TRY(dalloc(h, &d.c[b].ci, cap));
        TRY(dalloc(h, &d.c[b].cj, cap));
        TRY(dalloc(h, &d.c[b].fl, cap));
        TRY(dalloc(h, &d.c[b].src, cap));
        for (int f = 0; f < 15; ++f) TRY(dalloc(h, &d.c[b].f[f], cap));
        TRY(dalloc(h, &d.row_start[b], n));
        TRY(dalloc(h, &d.row_len[b], n));
    }
    TRY(dalloc(h, &d.stash, n * (size_t)h->p.kstash));
    TRY(dalloc(h, &d.keep, cap));
    TRY(dalloc(h, &d.tlist, cap));
    TRY(dalloc(h, &d.in_cnt, n));
    TRY(dalloc(h, &d.in_list, n * (size_t)h->p.kin));
    TRY(dalloc(h, &d.contrib, 9 * cap));
    TRY(dalloc(h, &d.contrib32, 9 * cap));
    TRY(dalloc(h, &d.bk32, n));
    TRY(dalloc(h, &d.rm32, n));
    TRY(dalloc(h, &d.scan_state[kScanCells], (size_t)scan_tiles((int64_t)T)));
    TRY(dalloc(h, &d.scan_state[kScanDebug], (size_t)scan_tiles((int64_t)n)));
    TRY(dalloc(h, &d.ctr, 1));
    TRY(dalloc(h, &d.sctr, (size_t)std::max(h->s_cap, 1)));
    TRY(dalloc(h, &d.vl, n * (size_t)h->p.kvl));
    TRY(dalloc(h, &d.vl_len, n));
    TRY(dalloc(h, &d.xref, n));
    TRY(dalloc(h, &d.pos32, n));
    TRY(dalloc(h, &d.path, n));
    for (int b = 0; b < 2; ++b) TRY(dalloc(h, &d.sflags[b], (size_t)std::max(h->s_cap, 1)));
    if (h->multi) {
        TRY(dalloc(h, &d.scene_of, n));
        TRY(dalloc(h, &d.sp, (size_t)h->s_cap));
        TRY(dalloc(h, &d.refcell, n));
        CU(cudaMemsetAsync(d.scene_of, 0xff, sizeof(int32_t) * std::max<size_t>(n, 1), h->stream));
    }
    return DEM_OK;
}

void drop_graphs(DemHandle* h);

void free_all(DemHandle* h) {
    drop_graphs(h);
    if (h->fork_ev) cudaEventDestroy(h->fork_ev);
    if (h->join_ev) cudaEventDestroy(h->join_ev);
    for (cudaEvent_t& e : h->pev) {
        if (e) cudaEventDestroy(e);
        e = nullptr;
    }
    if (h->side) cudaStreamDestroy(h->side);
    h->fork_ev = h->join_ev = nullptr;
    h->side = nullptr;
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->xfer) cudaFree(h->xfer);
    h->xfer = nullptr;
    if (h->io_idx) cudaFree(h->io_idx);
    h->io_idx = nullptr;
    if (h->counts) cudaFree(h->counts);
    h->counts = nullptr;
    if (h->io_rec) cudaFree(h->io_rec);
    h->io_rec = nullptr;
    if (h->err_host) cudaFreeHost(h->err_host);
    h->err_host = nullptr;
    h->err_dev = nullptr;
}

// Default launch shape: blocks of at most 256 threads, small enough that a
// single scene's particles give every SM at least four blocks (a
// 17,576-sphere scene in 256-thread blocks would leave half the SMs idle),
// and its expected ~3 contacts per particle at least eight: the hardware
// spreads many one-warp blocks more evenly over the SMs than fewer larger
// ones (measured on that scene's 50,700 bonds: 32-thread force blocks
// 46.9 us per step, 64-thread 48.0 us).  Arenas start at 256; the autotuner
// refines.
LaunchShape default_shape(const DemHandle* h) {
    auto block_for = [&](int64_t units, int per_sm) {
        int b = 256;
        while (b > 32 && units < (int64_t)b * per_sm * h->sm_count) b >>= 1;
        return b;
    };
    const int64_t n = h->multi ? INT64_MAX / 16 : h->n_cap;
    const int ib = block_for(n, 4), fb = block_for(3 * n, 8), cb = block_for(4 * n, 4);
    // a single scene's FP32 force kernel with the register budget for four
    // 256-thread blocks per SM (64 registers, a few bytes of spills): with
    // the compiler's choice (74 registers, three blocks) the 2,000,000-sphere
    // bed's force pass measured 215 us instead of 171 us.  The arena's keeps
    // the compiler's choice (the autotuner tries both).
    return LaunchShape{fb, h->sm_count * 16, cb, h->sm_count * 16, ib, 4, h->multi ? 0 : 4,
                       0, 0, 0};
}

int init_handle(DemHandle* h) {
    CU(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    CU(cudaEventCreate(&h->ev0));
    CU(cudaEventCreate(&h->ev1));
    TRY(allocate(h));
    h->ntiles_cells = std::max(1, scan_tiles((int64_t)h->p.T));
    h->shape = default_shape(h);
    h->p.dep = h->shape.dependent_launch;
    h->p.list_lanes = h->shape.list_lanes;
    return DEM_OK;
}

// Uploads a scene's particle arrays into slots [p0, p0 + n) and resets their
// dynamic state (ω = 0, q = 1, wall shear = 0, last forces = 0).
int upload_scene(DemHandle* h, const SceneArrays& A, int64_t p0) {
    const size_t n = A.r.size();
    if (!n) return DEM_OK;
    auto up = [&](double* dst, const std::vector<double>& src) {
        return cudaMemcpyAsync(dst + p0, src.data(), n * sizeof(double), cudaMemcpyHostToDevice,
                               h->stream);
    };
    DemDev& d = h->d;
    double* pd[3] = {d.px, d.py, d.pz};
    double* vd[3] = {d.vx, d.vy, d.vz};
    for (int c = 0; c < 3; ++c) {
        CU(up(pd[c], A.pos[c]));
        CU(up(vd[c], A.vel[c]));
    }
    const std::pair<double*, const std::vector<double>*> cols[] = {
        {d.m, &A.m},
        {d.inv_m, &A.inv_m},
        {d.r, &A.r},
        {d.r0, &A.r0},
        {d.inv_inertia, &A.inv_inertia},
        {d.b_invA, &A.b_invA},
        {d.b_rbI, &A.b_rbI},
        {d.b_EA, &A.b_EA},
        {d.b_EI, &A.b_EI},
        {d.b_phic, &A.b_phic}};
    for (const auto& c : cols) CU(up(c.first, *c.second));
    k_scene_columns<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(d, p0, (int64_t)n);
    CU(cudaGetLastError());
    for (double* z : {d.wx, d.wy, d.wz, d.qx, d.qy, d.qz, d.wsx, d.wsy, d.wsz, d.fx, d.fy, d.fz,
                      d.tx, d.ty, d.tz})
        CU(cudaMemsetAsync(z + p0, 0, n * sizeof(double), h->stream));
    // the host vectors above must outlive the copies
    CU(cudaStreamSynchronize(h->stream));
    return DEM_OK;
}

// The device form of a scene's material, surface and wall tables
// (dem_create_tables), checked: counts within the limits, every material
// index in range, finite constants.
int build_tables(const DemConfigC& cfg, const DemTables& t, int64_t n, MatTables& M,
                 std::vector<uint8_t>& mid) {
    g_invalid[0] = 0;
    auto bad = [](const char* what) {
        std::snprintf(g_invalid, sizeof(g_invalid), "tables: %s", what);
        return DEM_ERR_INVALID;
    };
    if (t.n_materials < 1 || t.n_materials > kMaxMaterials) return bad("n_materials not in 1..8");
    if (t.n_walls < 0 || t.n_walls > kMaxWalls) return bad("n_walls not in 0..8");
    if (!t.materials || !t.surfaces || (t.n_walls && !t.walls) || (n && !t.grain_material))
        return bad("missing array");
    const int nm = (int)t.n_materials;
    M.nmat = nm;
    M.nwall = (int)t.n_walls;
    for (int a = 0; a < nm; ++a) {
        const DemMaterial& m = t.materials[a];
        if (!(m.elastic_modulus > 0) || !std::isfinite(m.poisson_ratio)) return bad("material constants");
    }
    for (int a = 0; a < nm; ++a)
        for (int b = 0; b < nm; ++b) {
            const DemSurface& S = t.surfaces[a * nm + b];
            const DemMaterial &ma = t.materials[a], &mb = t.materials[b];
            const Hertz hc = hertz_constants(ma.elastic_modulus, ma.poisson_ratio,
                                             mb.elastic_modulus, mb.poisson_ratio, S.restitution);
            PairConst& P = M.pair[a * nm + b];
            P.mu = S.friction;
            P.Ys = hc.Ys;
            P.Gs = hc.Gs;
            P.cgn = hc.cgn;
            P.cgt = hc.cgt;
            P.ratio = S.bond_radius_ratio;
            P.E = S.bond_elastic_modulus;
            P.nu = S.bond_poisson_ratio;
            P.inv1pnu = 1.0 / (1.0 + S.bond_poisson_ratio);
            P.sc = S.bond_compressive_strength;
            P.st = S.bond_tensile_strength;
            P.ss = S.bond_shear_strength;
        }
    for (int w = 0; w < M.nwall; ++w) {
        const DemWall& W = t.walls[w];
        if (W.material < 0 || W.material >= nm) return bad("wall material out of range");
        WallConst& C = M.wall[w];
        double c0 = -W.distance;
        for (int c = 0; c < 3; ++c) {
            C.wn[c] = W.normal[c];
            C.f_wn[c] = (float)W.normal[c];
            c0 += W.normal[c] * cfg.domain_min[c];
        }
        C.wd = W.distance;
        C.f_wc0 = (float)c0;
        const M3 R = wall_frame(W.normal, cfg.tolerance);
        const M3 Ri = inverse3(R);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                C.wR[3 * r + c] = R.a[r][c];
                C.wRinv[3 * r + c] = Ri.a[r][c];
            }
        const DemMaterial& mw = t.materials[W.material];
        for (int a = 0; a < nm; ++a) {
            const DemSurface& S = t.surfaces[a * nm + W.material];
            const DemMaterial& ma = t.materials[a];
            const Hertz hc = hertz_constants(ma.elastic_modulus, ma.poisson_ratio,
                                             mw.elastic_modulus, mw.poisson_ratio, S.restitution);
            C.mu[a] = S.friction;
            C.Ys[a] = hc.Ys;
            C.Gs[a] = hc.Gs;
            C.cgn[a] = hc.cgn;
            C.cgt[a] = hc.cgt;
        }
    }
    mid.resize((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        const int32_t g = t.grain_material[i];
        if (g < 0 || g >= nm) {
            std::snprintf(g_invalid, sizeof(g_invalid), "tables: grain %lld material %d out of range",
                          (long long)i, (int)g);
            return DEM_ERR_INVALID;
        }
        mid[(size_t)i] = (uint8_t)g;
    }
    return DEM_OK;
}

int upload_tables(DemHandle* h, const MatTables& M, const std::vector<uint8_t>& mid) {
    MatTables* dm = nullptr;
    uint8_t* dmid = nullptr;
    TRY(dalloc(h, &dm, 1));
    TRY(dalloc(h, &dmid, std::max<size_t>(mid.size(), 1)));
    CU(cudaMemcpyAsync(dm, &M, sizeof(MatTables), cudaMemcpyHostToDevice, h->stream));
    if (!mid.empty())
        CU(cudaMemcpyAsync(dmid, mid.data(), mid.size(), cudaMemcpyHostToDevice, h->stream));
    h->d.mt = dm;
    h->d.mid = dmid;
    // every wall's shear history starts at zero
    const size_t cols = (size_t)h->nwall * (size_t)h->n_cap;
    for (double* z : {h->d.wsx, h->d.wsy, h->d.wsz})
        CU(cudaMemsetAsync(z, 0, cols * sizeof(double), h->stream));
    CU(cudaStreamSynchronize(h->stream));  // M and mid are the caller's stack and vector
    return DEM_OK;
}

// Marks scene s (every buffer parity) for a full pair search at its next step.
int flag_search(DemHandle* h, int s) {
    for (int b = 0; b < 2; ++b)
        CU(cudaMemsetAsync(h->d.sflags[b] + s, 1, sizeof(uint32_t), h->stream));
    return DEM_OK;
}

void record_step(DemHandle* h, int cur) {
    const int nxt = cur ^ 1;
    launch_search(h->d, h->p, cur, false, h->multi, false, h->shape, h->stream);
    launch_force(h->d, h->p, nxt, h->multi, h->shape, h->stream);
    launch_integrate(h->d, h->p, cur, h->multi, h->shape, h->stream);
}

void drop_graphs(DemHandle* h) {
    for (int b = 0; b < 2; ++b) {
        if (h->exec[b]) cudaGraphExecDestroy(h->exec[b]);
        h->exec[b] = nullptr;
        if (h->xg[b].exec) cudaGraphExecDestroy(h->xg[b].exec);
        h->xg[b].exec = nullptr;
        if (h->pg[b]) cudaGraphExecDestroy(h->pg[b]);
        h->pg[b] = nullptr;
    }
}

// Slots and buckets a step processes: up to the end of the highest range in
// use, rounded up, so the step's launches shrink with the arena's occupancy.
// The bucket scan's tickets and tile states restart when its tile count
// changes (its tile and epoch arithmetic assume a fixed count).
int update_bounds(DemHandle* h) {
    auto hi = [](const FreeList& fl, int64_t cap, int64_t grain) {
        int64_t top = cap;
        if (!fl.free.empty() && fl.free.back().first + fl.free.back().second == cap)
            top = fl.free.back().first;
        top = (top + grain - 1) / grain * grain;
        return std::min(std::max(top, grain), cap);
    };
    const int n = (int)hi(h->pfree, h->n_cap, 32768);
    const uint32_t T = (uint32_t)hi(h->tfree, h->t_cap, 65536);
    if (n == h->p.n && T == h->p.T) return DEM_OK;
    CU(cudaStreamSynchronize(h->stream));
    h->p.n = n;
    h->p.T = T;
    const int nt = std::max(1, scan_tiles((int64_t)T));
    if (nt != h->ntiles_cells) {
        h->ntiles_cells = nt;
        CU(cudaMemsetAsync(&h->d.ctr->tickets[kScanCells], 0, sizeof(unsigned long long),
                           h->stream));
        CU(cudaMemsetAsync(h->d.scan_state[kScanCells], 0,
                           sizeof(unsigned long long) * (size_t)scan_tiles((int64_t)h->t_cap),
                           h->stream));
    }
    drop_graphs(h);
    return DEM_OK;
}

int build_graphs(DemHandle* h) {
    if (h->graph_precision == h->p.precision && h->exec[0]) return DEM_OK;
    drop_graphs(h);
    for (int b = 0; b < 2; ++b) {
        if (h->exec[b]) {
            cudaGraphExecDestroy(h->exec[b]);
            h->exec[b] = nullptr;
        }
        cudaGraph_t g = nullptr;
        CU(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        record_step(h, b);
        CU(cudaStreamEndCapture(h->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&h->exec[b], g, 0);
        cudaGraphDestroy(g);
        CU(e);
    }
    h->graph_precision = h->p.precision;
    return DEM_OK;
}

int read_counters(DemHandle* h, DevCounters* out) {
    CU(cudaStreamSynchronize(h->stream));
    CU(cudaMemcpy(out, h->d.ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost));
    return DEM_OK;
}

int error_code(int bits) {
    if (bits & kErrCapacity) return DEM_ERR_CAPACITY;
    if (bits & kErrTimeout) return DEM_ERR_TIMEOUT;
    if (bits & kErrRange) return DEM_ERR_RANGE;
    return DEM_OK;
}

int device_error(DemHandle* h) {
    DevCounters c;
    TRY(read_counters(h, &c));
    return error_code(c.error);
}

int contact_count(DemHandle* h, int buf, int32_t* total) {
    unsigned int v = 0;
    CU(cudaMemcpyAsync(&v, &h->d.ctr->alloc[buf].rows, sizeof(v), cudaMemcpyDeviceToHost,
                       h->stream));
    CU(cudaStreamSynchronize(h->stream));
    *total = (int32_t)std::min<int64_t>((int64_t)v, (int64_t)h->c_cap);
    return DEM_OK;
}

// The FP32 force mode keeps 𝐅ᵢ, 𝛕ᵢ, 𝛕ⱼ as FP32 hi/lo pairs; re-encode the
// current buffer's contacts when the handle's precision changed.
int ensure_encoding(DemHandle* h) {
    if (h->enc == h->p.precision) return DEM_OK;
    int32_t C = 0;
    if (h->n_cap) TRY(contact_count(h, h->cur, &C));
    launch_recode(h->d, h->cur, C, h->p.precision == DEM_FP32_FORCE, h->stream);
    CU(cudaGetLastError());
    h->enc = h->p.precision;
    return DEM_OK;
}

// host side of the same encoding
inline double pair_decode(double slot) {
    float v[2];
    std::memcpy(v, &slot, sizeof(v));
    return (double)v[0] + (double)v[1];
}
inline double pair_encode(double x) {
    const float hi = (float)x;
    const float v[2] = {hi, (float)(x - (double)hi)};
    double slot;
    std::memcpy(&slot, v, sizeof(slot));
    return slot;
}

int get_dev(std::vector<double>& host, const double* dev, size_t n, cudaStream_t s) {
    host.resize(n);
    if (n) CU(cudaMemcpyAsync(host.data(), dev, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    return DEM_OK;
}

const SceneHost* scene_at(DemHandle* h, int32_t s) {
    if (!h || s < 0 || s >= (int32_t)h->scenes.size()) return nullptr;
    const SceneHost& S = h->scenes[s];
    return S.mode == kModeFree ? nullptr : &S;
}

int apply_modes(DemHandle* h, const std::vector<std::pair<int, int>>& upd) {
    for (size_t k = 0; k < upd.size(); k += 64) {
        ModeUpdates u{};
        u.count = (int)std::min<size_t>(64, upd.size() - k);
        for (int t = 0; t < u.count; ++t) {
            u.idx[t] = upd[k + t].first;
            u.mode[t] = upd[k + t].second;
        }
        k_set_modes<<<1, 64, 0, h->stream>>>(h->d.sp, u);
        CU(cudaGetLastError());
    }
    return DEM_OK;
}

// `initialize!` of newly added arena scenes: one launch in which they run in
// Init mode and every stepping scene is held (Frozen carries its state and
// contacts over unchanged), so it costs them no step.  Needs the graphs.
int launch_inits(DemHandle* h) {
    if (!h->multi) return DEM_OK;
    std::vector<std::pair<int, int>> hold, back;
    for (int k = 0; k < h->s_cap; ++k) {
        SceneHost& S = h->scenes[k];
        if (S.mode == kModeStep) {
            hold.push_back({k, kModeFrozen});
            back.push_back({k, kModeStep});
        } else if (S.mode == kModeInit) {
            back.push_back({k, kModeStep});
        }
    }
    if (back.size() == hold.size()) return DEM_OK;  // no scene to initialise
    for (auto& kv : back) h->scenes[kv.first].mode = kModeStep;
    TRY(apply_modes(h, hold));
    CU(cudaGraphLaunch(h->exec[h->cur], h->stream));
    h->cur ^= 1;
    return apply_modes(h, back);
}

// Scene bookkeeping after a step launch (stream-ordered, no host sync): step
// counts, and scenes that reached their target freeze.
int after_launch(DemHandle* h) {
    if (!h->multi) return DEM_OK;
    std::vector<std::pair<int, int>> upd;
    for (int k = 0; k < h->s_cap; ++k) {
        SceneHost& S = h->scenes[k];
        if (S.mode != kModeStep) continue;
        ++S.steps;
        if (S.target > 0 && S.steps >= S.target) {
            S.mode = kModeFrozen;
            upd.push_back({k, kModeFrozen});
        }
    }
    return upd.empty() ? DEM_OK : apply_modes(h, upd);
}

// Device staging for particle records, at least `doubles` long.
int xfer_buffer(DemHandle* h, int64_t doubles, double** out) {
    if (!h->xfer || h->xfer_n < doubles) {
        if (h->xfer) cudaFree(h->xfer);
        h->xfer = nullptr;
        h->xfer_n = 0;
        CU(cudaMalloc(&h->xfer, sizeof(double) * (size_t)std::max<int64_t>(doubles, 1)));
        h->xfer_n = std::max<int64_t>(doubles, 1);
    }
    *out = h->xfer;
    return DEM_OK;
}

// Page-locked ranges from dem_host_alloc: host base -> (bytes, device base),
// so that an exchange with them needs no pointer query.
struct HostRanges {
    std::mutex mu;
    std::map<uintptr_t, std::pair<size_t, uintptr_t>> r;
};
HostRanges& host_ranges() {
    static HostRanges* h = new HostRanges;  // never destroyed: used at exit by frees
    return *h;
}

// The device address of a caller buffer the GPU can access in place
// (page-locked host memory, or device memory), else nullptr.
double* device_view(const void* p) {
    {
        HostRanges& H = host_ranges();
        std::lock_guard<std::mutex> lk(H.mu);
        const uintptr_t u = reinterpret_cast<uintptr_t>(p);
        auto it = H.r.upper_bound(u);
        if (it != H.r.begin()) {
            --it;
            if (u - it->first < it->second.first)
                return reinterpret_cast<double*>(it->second.second + (u - it->first));
        }
    }
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeDevice)
        return static_cast<double*>(a.devicePointer);
    return nullptr;
}

// Can the host read the buffer (pageable or page-locked host memory)?
bool host_readable(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return a.type == cudaMemoryTypeUnregistered || a.type == cudaMemoryTypeHost;
}

// One particle state exchange between caller buffers (`host[f]`, k[f] doubles
// per particle, nullptr = field not exchanged) and the columns `cols[f]` at
// slots [p0, p0 + n): one kernel over all fields, which reads or writes
// device-accessible buffers in place; pageable buffers go through the
// library's staging copy with one cudaMemcpyAsync each.  Synchronises unless
// `sync` is false (uploads only: a pageable buffer is free once its copy call
// returns, a device-accessible one once the stream has passed the kernel);
// with `error`, also returns the device error word as of the exchange (copied
// by the kernel).  `posf` >= 0 (uploads to a single-scene handle): field posf
// holds positions; the kernel also refreshes the FP32 positions and, with
// `fb` 0 or 1, flags a full search when a particle left its skin.
int exchange(DemHandle* h, int64_t p0, int64_t n, const int* k, double* const* host,
             double* const (*cols)[4], int nfields, bool to_cols, int* error = nullptr,
             bool sync = true, int posf = -1, int fb = -1, const HostOut* arm = nullptr) {
    if (error && !h->err_host) {
        CU(cudaMallocHost(&h->err_host, 64));
        h->err_dev = reinterpret_cast<int*>(device_view(h->err_host));
    }
    XferSet x{};
    double* staged[kXferFields] = {};
    const double* src_host[kXferFields] = {};
    double* xf = nullptr;
    size_t off = 0;
    int xpos = -1;
    int ncol = 0;
    for (int f = 0; f < nfields && n > 0; ++f) {
        if (!host[f]) continue;
        if (k[f] < 1 || k[f] > 4 || (ncol += k[f]) > kXferCols) return DEM_ERR_INVALID;
        double* dv = device_view(host[f]);
        if (!dv) {
            if (!xf) TRY(xfer_buffer(h, 22 * n, &xf));
            dv = xf + off;
            off += (size_t)k[f] * n;
            staged[x.nf] = dv;
            src_host[x.nf] = host[f];
        }
        if (f == posf) xpos = x.nf;
        x.rec[x.nf] = dv;
        for (int c = 0; c < 4; ++c) x.col[x.nf][c] = cols[f][c];
        x.k[x.nf] = k[f];
        ++x.nf;
    }
    if (error) {
        if (n > 0 && x.nf > 0 && h->err_dev) {
            x.err_src = &h->d.ctr->error;
            x.err_dst = h->err_dev;
        } else {
            CU(cudaMemcpyAsync(h->err_host, &h->d.ctr->error, sizeof(int),
                               cudaMemcpyDeviceToHost, h->stream));
        }
    }
    if (n > 0 && x.nf > 0) {
        if (to_cols)
            for (int f = 0; f < x.nf; ++f)
                if (staged[f])
                    CU(cudaMemcpyAsync(staged[f], src_host[f], sizeof(double) * x.k[f] * n,
                                       cudaMemcpyHostToDevice, h->stream));
        if (arm && xpos >= 0) {
            x.arm = 1;
            x.hout = *arm;
        }
        if (xpos >= 0) launch_xfer_pos(x, (int)n, h->d, h->p, xpos, fb, h->stream);
        else launch_xfer(x, (int)n, (int)p0, to_cols, h->stream);
        CU(cudaGetLastError());
    }
    if (!to_cols)
        for (int f = 0; f < x.nf; ++f)
            if (staged[f])
                CU(cudaMemcpyAsync(const_cast<double*>(src_host[f]), staged[f],
                                   sizeof(double) * x.k[f] * n, cudaMemcpyDeviceToHost, h->stream));
    if (!sync && to_cols && !error) return DEM_OK;
    CU(cudaStreamSynchronize(h->stream));
    if (error) *error = *h->err_host;
    return DEM_OK;
}

// Particle state of slots [p0, p0 + n) to host arrays (scene-local order).
int get_particles_range(DemHandle* h, int64_t p0, int64_t n, DemParticleState* out) {
    const DemDev& d = h->d;
    const int k[] = {3, 3, 3, 4, 3, 3, 3};
    double* const host[] = {out->pos,   out->vel,    out->omega,     out->quat,
                            out->force, out->moment, out->wall_shear};
    double* const cols[][4] = {{d.px, d.py, d.pz},      {d.vx, d.vy, d.vz},
                               {d.wx, d.wy, d.wz},      {d.qw, d.qx, d.qy, d.qz},
                               {d.fx, d.fy, d.fz},      {d.tx, d.ty, d.tz},
                               {d.wsx, d.wsy, d.wsz}};
    int err = 0;
    TRY(exchange(h, p0, n, k, host, cols, 7, false, &err));
    return error_code(err);
}

// Contact entries of the current buffer whose owner lies in slots
// [p0, p0 + n): the rows of those slots, and the active entries among them.
struct RangeContacts {
    std::vector<int32_t> ci, cj, act;
    std::vector<uint32_t> fl;
    int32_t C = 0;
};
int range_contacts(DemHandle* h, int64_t p0, int64_t n, RangeContacts& R) {
    if (h->n_cap) TRY(contact_count(h, h->cur, &R.C));
    const int32_t C = R.C;
    const ContactSoA& s = h->d.c[h->cur];
    R.ci.resize(C);
    R.cj.resize(C);
    R.fl.resize(C);
    std::vector<int32_t> rs(n), rl(n);
    if (C) {
        CU(cudaMemcpyAsync(R.ci.data(), s.ci, (size_t)C * 4, cudaMemcpyDeviceToHost, h->stream));
        CU(cudaMemcpyAsync(R.cj.data(), s.cj, (size_t)C * 4, cudaMemcpyDeviceToHost, h->stream));
        CU(cudaMemcpyAsync(R.fl.data(), s.fl, (size_t)C * 4, cudaMemcpyDeviceToHost, h->stream));
    }
    if (n) {
        CU(cudaMemcpyAsync(rs.data(), h->d.row_start[h->cur] + p0, (size_t)n * 4,
                           cudaMemcpyDeviceToHost, h->stream));
        CU(cudaMemcpyAsync(rl.data(), h->d.row_len[h->cur] + p0, (size_t)n * 4,
                           cudaMemcpyDeviceToHost, h->stream));
    }
    CU(cudaStreamSynchronize(h->stream));
    R.act.clear();
    for (int64_t i = 0; i < n; ++i)
        for (int32_t c = std::max(rs[i], 0); c < std::min(rs[i] + rl[i], C); ++c)
            if ((R.fl[c] & kActive) && R.ci[c] == p0 + i) R.act.push_back(c);
    return DEM_OK;
}

// Active contacts whose owner lies in slots [p0, p0 + n), with scene-local
// indices, sorted by (i, j).
int get_contacts_range(DemHandle* h, int64_t p0, int64_t n, DemContacts* out, int64_t cap,
                       int64_t* n_out) {
    TRY(device_error(h));
    RangeContacts R;
    TRY(range_contacts(h, p0, n, R));
    const int32_t C = R.C;
    const ContactSoA& s = h->d.c[h->cur];
    const std::vector<int32_t>&ci = R.ci, &cj = R.cj;
    const std::vector<uint32_t>& fl = R.fl;
    std::vector<int32_t>& act = R.act;
    std::sort(act.begin(), act.end(), [&](int32_t a, int32_t b) {
        return ci[a] != ci[b] ? ci[a] < ci[b] : cj[a] < cj[b];
    });
    const int64_t na = (int64_t)act.size();
    *n_out = na;
    if (!out) return DEM_OK;
    if (na > cap) return DEM_ERR_CAPACITY;
    std::vector<double> f[15];
    if (na) {
        for (int q = 0; q < 15; ++q) TRY(get_dev(f[q], s.f[q], (size_t)C, h->stream));
        CU(cudaStreamSynchronize(h->stream));
        if (h->enc == DEM_FP32_FORCE)
            for (int q = CF; q < CS; ++q)
                for (int32_t c : act) f[q][c] = pair_decode(f[q][c]);
    }
    for (int64_t t = 0; t < na; ++t) {
        const int32_t c = act[t];
        if (out->i) out->i[t] = (int32_t)(ci[c] - p0);
        if (out->j) out->j[t] = (int32_t)(cj[c] - p0);
        const bool bonded = (fl[c] & kBonded) != 0;
        if (out->bonded) out->bonded[t] = bonded ? 1 : 0;
        // a bond's 𝐬 and a Hertz contact's torques are zero (not stored)
        for (int q = 0; q < 3; ++q) {
            if (out->point) out->point[3 * t + q] = f[CK + q][c];
            if (out->force) out->force[3 * t + q] = f[CF + q][c];
            if (out->torque_i) out->torque_i[3 * t + q] = bonded ? f[CTI + q][c] : 0.0;
            if (out->torque_j) out->torque_j[3 * t + q] = bonded ? f[CTJ + q][c] : 0.0;
            if (out->shear) out->shear[3 * t + q] = bonded ? 0.0 : f[CS + q][c];
        }
    }
    return DEM_OK;
}

// The active contacts of slots [p0, p0 + n) as p4c records in (i, j) order,
// compacted on the device: per-slot counts, their scan, then the records of
// each row in row order (rows are sorted by j); only the records cross to
// the host.
int get_io_contacts_range(DemHandle* h, int64_t p0, int64_t n, DemIOContact* out, int64_t cap,
                          int64_t* n_out) {
    TRY(device_error(h));
    *n_out = 0;
    if (n == 0) return DEM_OK;
    if (h->io_idx_n < 2 * n + 1) {
        if (h->io_idx) cudaFree(h->io_idx);
        h->io_idx = nullptr;
        h->io_idx_n = 0;
        CU(cudaMalloc(&h->io_idx, sizeof(int32_t) * (size_t)(2 * n + 1)));
        h->io_idx_n = 2 * n + 1;
    }
    int32_t* cnt = h->io_idx;
    int32_t* off = h->io_idx + n;
    launch_io_count(h->d, h->cur, h->c_cap, (int)p0, (int)n, cnt, h->stream);
    launch_scan_i32(cnt, off, n, h->d, kScanDebug, h->stream);
    CU(cudaGetLastError());
    int32_t total = 0;
    CU(cudaMemcpyAsync(&total, off + n, sizeof(total), cudaMemcpyDeviceToHost, h->stream));
    CU(cudaStreamSynchronize(h->stream));
    *n_out = total;
    if (!out || total == 0) return DEM_OK;
    if (total > cap) return DEM_ERR_CAPACITY;
    if (h->io_rec_n < total) {
        if (h->io_rec) cudaFree(h->io_rec);
        h->io_rec = nullptr;
        h->io_rec_n = 0;
        CU(cudaMalloc(&h->io_rec, sizeof(DemIOContact) * (size_t)total));
        h->io_rec_n = total;
    }
    launch_io_fill(h->d, h->cur, h->c_cap, (int)p0, (int)n, off, h->enc == DEM_FP32_FORCE,
                   h->io_rec, h->stream);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(out, h->io_rec, sizeof(DemIOContact) * (size_t)total,
                       cudaMemcpyDeviceToHost, h->stream));
    CU(cudaStreamSynchronize(h->stream));
    return DEM_OK;
}

int stats_of(DemHandle* h, int32_t s, const SceneHost& S, DemStats* out) {
    DevCounters c;
    TRY(read_counters(h, &c));
    SceneCounters sc{};
    CU(cudaMemcpy(&sc, h->d.sctr + s, sizeof(sc), cudaMemcpyDeviceToHost));
    // the scene's active contacts and bonds, counted on the device
    if (!h->counts) CU(cudaMalloc(&h->counts, 2 * sizeof(unsigned long long)));
    unsigned long long cnt[2] = {0ull, 0ull};
    CU(cudaMemsetAsync(h->counts, 0, sizeof(cnt), h->stream));
    launch_range_counts(h->d, h->cur, h->c_cap, (int)S.sp.p0, (int)S.sp.n, h->counts, h->stream);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(cnt, h->counts, sizeof(cnt), cudaMemcpyDeviceToHost, h->stream));
    CU(cudaStreamSynchronize(h->stream));
    const int64_t act = (int64_t)cnt[0], bnd = (int64_t)cnt[1];
    std::memset(out, 0, sizeof(*out));
    out->n_particles = S.sp.n;
    out->steps_done = h->multi ? S.steps : h->steps;
    out->contacts = act;
    out->bonded = bnd;
    out->bonds_broken = (int64_t)sc.broken;
    out->contacts_ended = (int64_t)sc.ended;
    out->contacts_created = (int64_t)sc.created;
    out->warn_gap = (int64_t)sc.warn_gap;
    out->warn_damping = (int64_t)sc.warn_damp;
    out->full_searches = (int64_t)sc.searches;
    out->exchanges_direct = h->multi ? 0 : h->exchanges_direct;
    out->error = error_code(c.error);
    out->precision = h->p.precision;
    return DEM_OK;
}

}  // namespace

extern "C" {

const char* dem_version(void) { return "dem_gb300 0.2.0 sm_103a"; }

const char* dem_strerror(int code) {
    switch (code) {
        case DEM_OK: return "ok";
        case DEM_ERR_INVALID: return g_invalid[0] ? g_invalid : "invalid argument or state";
        case DEM_ERR_CUDA: return g_msg[0] ? g_msg : "CUDA runtime error";
        case DEM_ERR_CAPACITY:
            return "capacity exceeded (contacts per particle, arena slots, buckets or scenes)";
        case DEM_ERR_TIMEOUT: return "a bounded device-side wait gave up";
        case DEM_ERR_NO_DEVICE: return g_msg[0] ? g_msg : "no sm_103 (GB300) CUDA device available";
        case DEM_ERR_RANGE: return "particle outside the representable cell range";
        default: return "unknown error";
    }
}

int dem_selftest_conversions(int64_t n, uint64_t seed, int64_t* mismatches) {
    if (n < 0 || !mismatches) return DEM_ERR_INVALID;
    int dev = 0, sms = 0;
    TRY(check_device(&dev, &sms));
    unsigned long long* bad = nullptr;
    CU(cudaMalloc(&bad, 4 * sizeof(unsigned long long)));
    unsigned long long hb[4] = {0, 0, 0, 0};
    cudaError_t e = cudaMemset(bad, 0, sizeof(hb));
    if (e == cudaSuccess) {
        launch_selftest_conv((long long)n, (unsigned long long)seed, bad, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost);
    cudaFree(bad);
    CU(e);
    mismatches[0] = (int64_t)hb[0];
    mismatches[1] = (int64_t)hb[1];
    mismatches[2] = (int64_t)hb[2];
    mismatches[3] = (int64_t)hb[3];
    return DEM_OK;
}

int dem_set_device(int device) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return DEM_ERR_NO_DEVICE;
    if (device < 0 || device >= ndev) return DEM_ERR_INVALID;
    CU(cudaSetDevice(device));
    return DEM_OK;
}

int create_single(const DemConfigC* cfg, const DemParticlesIn* pin, const DemTables* tables,
                  DemHandle** out) {
    if (!out) return DEM_ERR_INVALID;
    *out = nullptr;
    SceneHost S;
    SceneArrays A;
    TRY(prepare_scene(cfg, pin, 1.0, S, A));
    if (S.der.contact_capacity > 0x7fffffff) return DEM_ERR_CAPACITY;
    MatTables M{};
    std::vector<uint8_t> mid;
    if (tables) TRY(build_tables(*cfg, *tables, pin->n, M, mid));
    int dev = 0, sms = 0;
    TRY(check_device(&dev, &sms));
    DemHandle* h = new DemHandle();
    h->tab = tables != nullptr;
    h->nwall = tables ? std::max<int>(M.nwall, 1) : 1;
    h->p.tab = h->tab ? 1 : 0;
    h->device = dev;
    h->sm_count = sms;
    h->multi = false;
    h->n_cap = (int)pin->n;
    h->c_cap = (int)S.der.contact_capacity;
    h->t_cap = (uint32_t)S.der.hash_table_size;
    h->s_cap = 1;
    h->p.n = h->n_cap;
    h->p.cap = h->c_cap;
    h->p.kstash = (int)std::min<int64_t>(cfg->max_coordinate_number, 64);
    h->p.kin = h->p.kstash;
    h->p.kvl = list_capacity(cfg->max_coordinate_number);
    h->p.ns = 1;
    h->p.sms = sms;
    h->p.T = h->t_cap;
    h->p.precision = DEM_FP64;
    S.sp.mode = kModeStep;
    S.sp.p0 = 0;
    S.sp.t0 = 0;
    S.sp.H = S.sp.Href;
    S.sp.Hmask = S.sp.Href_mask;
    S.mode = kModeStep;
    h->p.s0 = S.sp;
    h->scenes.push_back(S);
    int rc = init_handle(h);
    if (rc == DEM_OK) rc = upload_scene(h, A, 0);
    if (rc == DEM_OK && h->tab) rc = upload_tables(h, M, mid);
    if (rc == DEM_OK) rc = flag_search(h, 0);
    if (rc == DEM_OK) {
        launch_refresh_pos32(h->d, h->p, false, 0, h->n_cap, -1, h->stream);
        if (cudaGetLastError() != cudaSuccess) rc = DEM_ERR_CUDA;
    }
    if (rc != DEM_OK) {
        free_all(h);
        delete h;
        return rc;
    }
    *out = h;
    return DEM_OK;
}

int dem_create(const DemConfigC* cfg, const DemParticlesIn* pin, DemHandle** out) {
    return create_single(cfg, pin, nullptr, out);
}

int dem_create_tables(const DemConfigC* cfg, const DemParticlesIn* pin, const DemTables* tables,
                      DemHandle** out) {
    if (!tables) return DEM_ERR_INVALID;
    return create_single(cfg, pin, tables, out);
}

int dem_arena_create(const DemArenaConfig* cfg, DemHandle** out) {
    if (!cfg || !out || cfg->max_particles <= 0 || cfg->max_particles > 0x3fffffff ||
        cfg->max_contacts <= 0 || cfg->max_contacts > 0x7fffffff || cfg->max_buckets <= 0 ||
        cfg->max_buckets > 0x7fffffff || cfg->max_scenes <= 0 || cfg->max_coordinate_number <= 0 ||
        (cfg->precision != DEM_FP64 && cfg->precision != DEM_FP32_FORCE) ||
        !(cfg->cell_factor >= 0) || cfg->cell_factor > 1)
        return DEM_ERR_INVALID;
    *out = nullptr;
    int dev = 0, sms = 0;
    TRY(check_device(&dev, &sms));
    DemHandle* h = new DemHandle();
    h->device = dev;
    h->sm_count = sms;
    h->multi = true;
    h->n_cap = (int)cfg->max_particles;
    h->c_cap = (int)cfg->max_contacts;
    h->t_cap = (uint32_t)cfg->max_buckets;
    h->s_cap = cfg->max_scenes;
    h->cell_factor = cfg->cell_factor > 0 ? cfg->cell_factor : 1.0;
    h->p.n = h->n_cap;
    h->p.cap = h->c_cap;
    h->p.kstash = std::min(cfg->max_coordinate_number, 64);
    h->p.kin = h->p.kstash;
    h->p.kvl = list_capacity(cfg->max_coordinate_number);
    h->p.ns = h->s_cap;
    h->p.sms = sms;
    h->p.T = h->t_cap;
    h->p.precision = cfg->precision;
    h->scenes.resize(h->s_cap);
    h->pfree.init(h->n_cap);
    h->tfree.init(h->t_cap);
    h->p.n = std::min(h->n_cap, 32768);
    h->p.T = std::min<uint32_t>(h->t_cap, 65536u);
    int rc = init_handle(h);
    if (rc == DEM_OK && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = DEM_ERR_CUDA;
    if (rc != DEM_OK) {
        free_all(h);
        delete h;
        return rc;
    }
    *out = h;
    return DEM_OK;
}

int dem_arena_add(DemHandle* h, const DemConfigC* cfg, const DemParticlesIn* pin, int init_bonds,
                  int64_t steps_target, int32_t* scene) {
    if (!h || !h->multi || !scene || steps_target < 0) return DEM_ERR_INVALID;
    SceneHost S;
    SceneArrays A;
    TRY(prepare_scene(cfg, pin, h->cell_factor, S, A));
    int idx = -1;
    for (int s = 0; s < h->s_cap; ++s)
        if (h->scenes[s].mode == kModeFree) {
            idx = s;
            break;
        }
    if (idx < 0) return DEM_ERR_CAPACITY;
    const int64_t n = pin->n;
    // search table of the scene: a power of two of at least 2 entries per particle
    uint32_t H = 1024;
    while ((int64_t)H < 2 * n && H < (1u << 30)) H <<= 1;
    int64_t p0 = 0, t0 = 0;
    if (!h->pfree.take(n, &p0)) return DEM_ERR_CAPACITY;
    if (!h->tfree.take(H, &t0)) {
        h->pfree.give(p0, n);
        return DEM_ERR_CAPACITY;
    }
    S.sp.p0 = (int)p0;
    S.sp.t0 = (uint32_t)t0;
    S.sp.H = H;
    S.sp.Hmask = H - 1;
    S.sp.mode = init_bonds ? kModeInit : kModeStep;
    S.mode = S.sp.mode;
    S.steps = 0;
    S.target = steps_target;
    int rc = upload_scene(h, A, p0);
    // the slots start with empty contact rows in both buffers
    for (int b = 0; b < 2 && rc == DEM_OK && n; ++b)
        if (cudaMemsetAsync(h->d.row_len[b] + p0, 0, (size_t)n * 4, h->stream) != cudaSuccess ||
            cudaMemsetAsync(h->d.row_start[b] + p0, 0, (size_t)n * 4, h->stream) != cudaSuccess)
            rc = DEM_ERR_CUDA;
    if (rc == DEM_OK && n) {
        const int nb = (int)((n + 255) / 256);
        k_fill_i32<<<nb, 256, 0, h->stream>>>(h->d.scene_of + p0, n, idx);
        if (cudaGetLastError() != cudaSuccess) rc = DEM_ERR_CUDA;
    }
    if (rc == DEM_OK) rc = flag_search(h, idx);
    if (rc == DEM_OK &&
        (cudaMemcpyAsync(h->d.sp + idx, &S.sp, sizeof(SceneParams), cudaMemcpyHostToDevice,
                         h->stream) != cudaSuccess ||
         cudaMemsetAsync(h->d.sctr + idx, 0, sizeof(SceneCounters), h->stream) != cudaSuccess ||
         cudaStreamSynchronize(h->stream) != cudaSuccess))
        rc = DEM_ERR_CUDA;
    if (rc == DEM_OK && n) {
        launch_refresh_pos32(h->d, h->p, true, (int)p0, (int)n, -1, h->stream);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(h->stream) != cudaSuccess)
            rc = DEM_ERR_CUDA;
    }
    if (rc != DEM_OK) {
        h->pfree.give(p0, n);
        h->tfree.give(t0, H);
        return rc;
    }
    h->scenes[idx] = S;
    *scene = idx;
    return update_bounds(h);
}

int dem_arena_remove(DemHandle* h, int32_t s) {
    if (!h || !h->multi || !scene_at(h, s)) return DEM_ERR_INVALID;
    SceneHost& S = h->scenes[s];
    const int64_t p0 = S.sp.p0, n = S.sp.n;
    TRY(apply_modes(h, {{s, kModeFree}}));
    if (n) {
        CU(cudaMemsetAsync(h->d.scene_of + p0, 0xff, (size_t)n * sizeof(int32_t), h->stream));
        // the scene's rows are emptied, so its contacts are not carried over
        for (int b = 0; b < 2; ++b)
            CU(cudaMemsetAsync(h->d.row_len[b] + p0, 0, (size_t)n * 4, h->stream));
    }
    h->pfree.give(p0, n);
    h->tfree.give(S.sp.t0, S.sp.H);
    S = SceneHost();
    return update_bounds(h);
}

int dem_arena_set_cell_factor(DemHandle* h, int32_t s, double f) {
    if (!h || !h->multi || !(f >= 0) || f > 1) return DEM_ERR_INVALID;
    if (s >= 0 && !scene_at(h, s)) return DEM_ERR_INVALID;
    for (int k = 0; k < h->s_cap; ++k) {
        if ((s >= 0 && k != s) || h->scenes[k].mode == kModeFree) continue;
        SceneHost& S = h->scenes[k];
        S.cell_factor = f > 0 ? f : 1.0;
        set_search_cell(S.sp, S.cell_factor, S.min_cell, S.sp.n == 0, S.rmax, S.skin_factor);
        // the record's mode on the device may differ from the host copy for
        // the length of dem_step only, so the host record is current here
        S.sp.mode = S.mode;
        CU(cudaMemcpyAsync(h->d.sp + k, &S.sp, sizeof(SceneParams), cudaMemcpyHostToDevice,
                           h->stream));
    }
    if (s < 0) h->cell_factor = f > 0 ? f : 1.0;
    CU(cudaStreamSynchronize(h->stream));
    return DEM_OK;
}

int dem_set_skin_factor(DemHandle* h, int32_t s, double f) {
    if (!h || !(f >= 0) || f > 1) return DEM_ERR_INVALID;
    if (s >= 0 && !scene_at(h, s)) return DEM_ERR_INVALID;
    for (int k = 0; k < (int)h->scenes.size(); ++k) {
        if ((s >= 0 && k != s) || h->scenes[k].mode == kModeFree) continue;
        SceneHost& S = h->scenes[k];
        S.skin_factor = f;
        set_search_cell(S.sp, S.cell_factor, S.min_cell, S.sp.n == 0, S.rmax, f);
        if (h->multi) {
            S.sp.mode = S.mode;
            CU(cudaMemcpyAsync(h->d.sp + k, &S.sp, sizeof(SceneParams), cudaMemcpyHostToDevice,
                               h->stream));
        } else {
            h->p.s0 = S.sp;  // kernel parameters: the step graphs are recaptured
            drop_graphs(h);
        }
        TRY(flag_search(h, k));
    }
    CU(cudaStreamSynchronize(h->stream));
    return DEM_OK;
}

int dem_set_launch_shape(DemHandle* h, const DemLaunchShape* sh) {
    if (!h || !sh || sh->force_block < 32 || sh->force_block > 256 || sh->force_block % 32 ||
        (sh->detect_blocks_per_sm != 0 && sh->detect_blocks_per_sm != 3 &&
         sh->detect_blocks_per_sm != 4) ||
        (sh->force_blocks_per_sm != 0 && sh->force_blocks_per_sm != 4) ||
        sh->compact_block < 32 || sh->compact_block > 256 || sh->compact_block % 32 ||
        sh->integrate_block < 32 || sh->integrate_block > 256 || sh->integrate_block % 32 ||
        sh->force_grid < 1 || sh->compact_grid < 1 ||
        sh->dependent_launch < 0 || sh->dependent_launch > 2 ||
        (sh->list_lanes != 0 && sh->list_lanes != 1 && sh->list_lanes != 4) ||
        (sh->integrate_lanes != 0 && sh->integrate_lanes != 1 && sh->integrate_lanes != 4))
        return DEM_ERR_INVALID;
    h->shape = LaunchShape{sh->force_block, sh->force_grid, sh->compact_block, sh->compact_grid,
                           sh->integrate_block,
                           sh->detect_blocks_per_sm ? sh->detect_blocks_per_sm : 4,
                           sh->force_blocks_per_sm, sh->dependent_launch, sh->list_lanes,
                           sh->integrate_lanes};
    h->p.dep = h->shape.dependent_launch;
    h->p.list_lanes = h->shape.list_lanes;
    drop_graphs(h);
    return DEM_OK;
}

int dem_get_launch_shape(DemHandle* h, DemLaunchShape* out) {
    if (!h || !out) return DEM_ERR_INVALID;
    *out = DemLaunchShape{h->shape.force_block,         h->shape.force_grid,
                          h->shape.compact_block,       h->shape.compact_grid,
                          h->shape.integrate_block,     h->shape.detect_blocks_per_sm,
                          h->shape.force_blocks_per_sm, h->shape.dependent_launch,
                          h->shape.list_lanes,          h->shape.integrate_lanes};
    return DEM_OK;
}

int dem_arena_scene_info(DemHandle* h, int32_t s, DemSceneInfo* out) {
    const SceneHost* S = scene_at(h, s);
    if (!S || !out) return DEM_ERR_INVALID;
    std::memset(out, 0, sizeof(*out));
    out->mode = S->mode;
    out->n = S->sp.n;
    out->first_slot = S->sp.p0;
    out->steps_done = h->multi ? S->steps : h->steps;
    out->steps_target = S->target;
    out->buckets = S->sp.H;
    return DEM_OK;
}

int dem_destroy(DemHandle* h) {
    if (!h) return DEM_ERR_INVALID;
    cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return DEM_OK;
}

int dem_set_precision(DemHandle* h, int mode) {
    if (!h || (mode != DEM_FP64 && mode != DEM_FP32_FORCE)) return DEM_ERR_INVALID;
    if (h->tab && mode != DEM_FP64) {
        std::snprintf(g_invalid, sizeof(g_invalid),
                      "a handle with material and wall tables computes in FP64 only");
        return DEM_ERR_INVALID;
    }
    h->p.precision = mode;
    return DEM_OK;
}

int dem_init_bonds(DemHandle* h) {
    if (!h || h->multi) return DEM_ERR_INVALID;
    if (h->n_cap == 0) return DEM_OK;
    TRY(ensure_encoding(h));
    const int cur = h->cur, nxt = cur ^ 1;
    launch_search(h->d, h->p, cur, true, false, true, h->shape, h->stream);
    // the old buffer becomes the next step's target: its allocator starts at 0
    CU(cudaMemsetAsync(&h->d.ctr->alloc[cur], 0, sizeof(RowCounter), h->stream));
    CU(cudaGetLastError());
    h->cur = nxt;
    return device_error(h);
}

int dem_step(DemHandle* h, int64_t nsteps) {
    if (!h || nsteps < 0) return DEM_ERR_INVALID;
    if (h->n_cap == 0 || nsteps == 0) {
        h->steps += nsteps;
        return DEM_OK;
    }
    TRY(ensure_encoding(h));
    TRY(build_graphs(h));
    TRY(launch_inits(h));
    for (int64_t s = 0; s < nsteps; ++s) {
        CU(cudaGraphLaunch(h->exec[h->cur], h->stream));
        h->cur ^= 1;
        TRY(after_launch(h));
    }
    h->steps += nsteps;
    return DEM_OK;
}

int dem_step_timed(DemHandle* h, int64_t nsteps, float* ms) {
    if (!h || !ms) return DEM_ERR_INVALID;
    TRY(build_graphs(h));
    CU(cudaEventRecord(h->ev0, h->stream));
    TRY(dem_step(h, nsteps));
    CU(cudaEventRecord(h->ev1, h->stream));
    CU(cudaEventSynchronize(h->ev1));
    CU(cudaEventElapsedTime(ms, h->ev0, h->ev1));
    return device_error(h);
}

int dem_step_profiled(DemHandle* h, float* phase_ms, int nphase) {
    if (!h || !phase_ms || nphase < 3) return DEM_ERR_INVALID;
    for (int k = 0; k < nphase; ++k) phase_ms[k] = 0.f;
    if (h->n_cap == 0) return DEM_OK;
    TRY(ensure_encoding(h));
    TRY(build_graphs(h));  // drops the profiled graphs too when the step graphs change
    if (h->multi) TRY(launch_inits(h));
    // the three kernels as the step graph runs them, with an event node
    // before, between and after them (one graph launch: no host launch
    // latency inside the timed phases)
    for (cudaEvent_t& e : h->pev)
        if (!e) CU(cudaEventCreate(&e));
    const int cur = h->cur, nxt = cur ^ 1;
    if (!h->pg[cur]) {
        CU(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaEventRecordWithFlags(h->pev[0], h->stream, cudaEventRecordExternal);
        if (e == cudaSuccess) {
            launch_search(h->d, h->p, cur, false, h->multi, false, h->shape, h->stream);
            e = cudaEventRecordWithFlags(h->pev[1], h->stream, cudaEventRecordExternal);
        }
        if (e == cudaSuccess) {
            launch_force(h->d, h->p, nxt, h->multi, h->shape, h->stream);
            e = cudaEventRecordWithFlags(h->pev[2], h->stream, cudaEventRecordExternal);
        }
        if (e == cudaSuccess) {
            launch_integrate(h->d, h->p, cur, h->multi, h->shape, h->stream);
            e = cudaEventRecordWithFlags(h->pev[3], h->stream, cudaEventRecordExternal);
        }
        if (e == cudaSuccess) e = cudaGetLastError();
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
        if (e == cudaSuccess) e = ec;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&h->pg[cur], g, 0);
        if (g) cudaGraphDestroy(g);
        CU(e);
    }
    CU(cudaGraphLaunch(h->pg[cur], h->stream));
    cudaError_t e = cudaEventSynchronize(h->pev[3]);
    for (int k = 0; k < 3 && e == cudaSuccess; ++k)
        e = cudaEventElapsedTime(&phase_ms[k], h->pev[k], h->pev[k + 1]);
    CU(e);
    h->cur = nxt;
    h->steps += 1;
    TRY(after_launch(h));
    return device_error(h);
}

int dem_sync(DemHandle* h) {
    if (!h) return DEM_ERR_INVALID;
    return device_error(h);
}

int dem_scene_get_derived(DemHandle* h, int32_t s, DemDerived* out) {
    const SceneHost* S = scene_at(h, s);
    if (!S || !out) return DEM_ERR_INVALID;
    *out = S->der;
    return DEM_OK;
}

int dem_get_derived(DemHandle* h, DemDerived* out) { return dem_scene_get_derived(h, 0, out); }

int dem_get_static(DemHandle* h, DemParticleStatic* out) {
    const SceneHost* S = scene_at(h, 0);
    if (!S || !out) return DEM_ERR_INVALID;
    const size_t n = (size_t)S->sp.n, p0 = (size_t)S->sp.p0;
    std::vector<double> r, r0, m, ii;
    TRY(get_dev(r, h->d.r + p0, n, h->stream));
    TRY(get_dev(r0, h->d.r0 + p0, n, h->stream));
    TRY(get_dev(m, h->d.m + p0, n, h->stream));
    TRY(get_dev(ii, h->d.inv_inertia + p0, n, h->stream));
    CU(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < n; ++i) {
        if (out->radius) out->radius[i] = r[i];
        if (out->radius0) out->radius0[i] = r0[i];
        if (out->mass) out->mass[i] = m[i];
        if (out->inertia) out->inertia[i] = 1.0 / ii[i];
    }
    return DEM_OK;
}

int dem_scene_get_particles(DemHandle* h, int32_t s, DemParticleState* out) {
    const SceneHost* S = scene_at(h, s);
    if (!S || !out) return DEM_ERR_INVALID;
    return get_particles_range(h, S->sp.p0, S->sp.n, out);
}

int dem_get_particles(DemHandle* h, DemParticleState* out) {
    return dem_scene_get_particles(h, 0, out);
}

int set_particles(DemHandle* h, const DemParticleState* in, bool sync,
                  const HostOut* arm = nullptr) {
    const SceneHost* S = scene_at(h, 0);
    if (!S || !in || h->multi) return DEM_ERR_INVALID;
    const int64_t n = S->sp.n;
    if (!n) return DEM_OK;
    const DemDev& d = h->d;
    const int k[] = {3, 3, 3, 4, 3};
    double* const host[] = {in->pos, in->vel, in->omega, in->quat, in->wall_shear};
    g_invalid[0] = 0;
    if (sync) {  // the synchronous upload checks its values (the exchange path does not)
        for (int f = 0; f < 5; ++f) {
            if (!host[f] || !host_readable(host[f])) continue;
            for (int64_t q = 0; q < k[f] * n; ++q)
                if (!std::isfinite(host[f][q])) {
                    std::snprintf(g_invalid, sizeof(g_invalid),
                                  "dem_set_particles: non-finite value in field %d, grain %lld",
                                  f, (long long)(q / k[f]));
                    return DEM_ERR_INVALID;
                }
        }
    }
    double* const cols[][4] = {{d.px, d.py, d.pz}, {d.vx, d.vy, d.vz}, {d.wx, d.wy, d.wz},
                               {d.qw, d.qx, d.qy, d.qz}, {d.wsx, d.wsy, d.wsz}};
    // new positions: the exchange kernel refreshes the FP32 positions; the
    // neighbour lists stay valid while every particle lies within skin/2 of
    // where they were built, else the next step searches in full
    return exchange(h, 0, n, k, host, cols, 5, true, nullptr, sync, 0, h->cur, arm);
}

int dem_set_particles(DemHandle* h, const DemParticleState* in) {
    return set_particles(h, in, true);  // the caller's buffers are free again on return
}

int dem_set_particles_async(DemHandle* h, const DemParticleState* in) {
    return set_particles(h, in, false);
}

// One exchanged step as a graph (DemHandle::XGraph): captured once per
// contact-buffer parity and set of caller buffers, replayed afterwards.
static int capture_exchange(DemHandle* h, int cur, double* pv, double* vv, double* ov, double* qv,
                            double* wv, const HostOut& ho, cudaGraphExec_t* exec) {
    if (!h->side) {
        CU(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
        CU(cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming));
        CU(cudaEventCreateWithFlags(&h->join_ev, cudaEventDisableTiming));
    }
    const DemDev& d = h->d;
    const int n = h->p.n;
    XferSet xp{};  // positions: FP32 copies, skin test, arming
    xp.rec[0] = pv;
    xp.col[0][0] = d.px;
    xp.col[0][1] = d.py;
    xp.col[0][2] = d.pz;
    xp.k[0] = 3;
    xp.nf = 1;
    xp.arm = 1;
    xp.hout = ho;
    // velocities, spins, orientations and the first wall's shear history,
    // beside the contact update (which reads none of them)
    XferSet xr{};
    double* const rv[4] = {vv, ov, qv, wv};
    double* const cv[4][4] = {{d.vx, d.vy, d.vz}, {d.wx, d.wy, d.wz}, {d.qw, d.qx, d.qy, d.qz},
                              {d.wsx, d.wsy, d.wsz}};
    const int kv[4] = {3, 3, 4, 3};
    for (int f = 0; f < 4; ++f) {
        if (!rv[f]) continue;
        xr.rec[xr.nf] = rv[f];
        for (int c = 0; c < kv[f]; ++c) xr.col[xr.nf][c] = cv[f][c];
        xr.k[xr.nf] = kv[f];
        ++xr.nf;
    }
    CU(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    auto ok = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
        return e == cudaSuccess;
    };
    // the positions first, with the host link to themselves (the contact
    // update waits for them); the rest from then on, beside the contact update
    launch_xfer_pos(xp, n, d, h->p, 0, cur, h->stream);
    ok(cudaGetLastError());
    if (e == cudaSuccess && xr.nf && ok(cudaEventRecord(h->fork_ev, h->stream)) &&
        ok(cudaStreamWaitEvent(h->side, h->fork_ev, 0))) {
        launch_xfer(xr, n, 0, true, h->side);
        if (ok(cudaGetLastError())) ok(cudaEventRecord(h->join_ev, h->side));
    }
    if (e == cudaSuccess) {
        launch_search(d, h->p, cur, false, false, false, h->shape, h->stream);
        if (ok(cudaGetLastError()) && xr.nf) ok(cudaStreamWaitEvent(h->stream, h->join_ev, 0));
        if (e == cudaSuccess) {
            launch_force(d, h->p, cur ^ 1, false, h->shape, h->stream);
            launch_integrate(d, h->p, cur, false, h->shape, h->stream);
            ok(cudaGetLastError());
        }
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
    if (e == cudaSuccess) e = ec;
    if (e == cudaSuccess) e = cudaGraphInstantiate(exec, g, 0);
    if (g) cudaGraphDestroy(g);
    CU(e);
    return DEM_OK;
}

// The fused exchange: the device addresses of the caller's output records
// (every non-null field must be device-accessible: page-locked host or
// device memory) and of the page-locked error word.
constexpr int kNoHostOut = INT_MIN;  // the error word's sentinel: no fused exchange ran
static bool fused_download(DemHandle* h, const DemParticleState* out, HostOut* ho) {
    double* const f[kHostOutFields] = {out->pos,   out->vel,    out->omega,     out->quat,
                                       out->force, out->moment, out->wall_shear};
    for (int q = 0; q < kHostOutFields; ++q) {
        ho->rec[q] = nullptr;
        if (f[q] && !(ho->rec[q] = device_view(f[q]))) return false;
    }
    if (!h->err_host) {
        if (cudaMallocHost(&h->err_host, 64) != cudaSuccess) {
            cudaGetLastError();
            h->err_host = nullptr;
            return false;
        }
        h->err_dev = reinterpret_cast<int*>(device_view(h->err_host));
    }
    ho->err = h->err_dev;
    ho->done = 0u;
    return h->err_dev != nullptr;
}

int dem_step_exchange(DemHandle* h, const DemParticleState* in, int64_t nsteps,
                      DemParticleState* out) {
    if (!h || nsteps < 0 || h->multi) return DEM_ERR_INVALID;
    HostOut ho{};
    const SceneHost* S = scene_at(h, 0);
    // the split integrator (the step graph's layout for this scene) writes
    // the state into `out` while it runs, instead of a separate read after
    // the step.  The upload before the step carries only the positions: in
    // the graph of a single step the other fields are uploaded on a second
    // stream beside the contact update; otherwise velocities and spins go
    // with the positions, and the integrator of the first step reads the
    // orientations and the first wall's shear history from `in` itself.
    if (in && in->pos && out && nsteps > 0 && nsteps <= INT_MAX && S && S->sp.n > 0 &&
        split_integrator(h->shape, h->p.n, h->p.sms) && fused_download(h, out, &ho)) {
        *reinterpret_cast<volatile int*>(h->err_host) = kNoHostOut;
        ho.steps_left = ho.steps_total = (int)nsteps;
        double* const pv = device_view(in->pos);
        double* const vv = in->vel ? device_view(in->vel) : nullptr;
        double* const ov = in->omega ? device_view(in->omega) : nullptr;
        double* const qv = in->quat ? device_view(in->quat) : nullptr;
        double* const wv = in->wall_shear ? device_view(in->wall_shear) : nullptr;
        // a one-step exchange in place: values the step leaves unchanged are
        // in `out` already (the step's input of that field came from there)
        const double* const inv[kHostOutFields] = {pv, vv, ov, qv, nullptr, nullptr, wv};
        ho.same = 0u;
        if (nsteps == 1)
            for (int q = 0; q < kHostOutFields; ++q)
                if (inv[q] && inv[q] == ho.rec[q]) ho.same |= 1u << q;
        ho.qin = qv;
        ho.wsin = wv;
        int rc = DEM_OK;
        if (nsteps == 1 && pv && (!in->vel || vv) && (!in->omega || ov) && (!in->quat || qv) &&
            (!in->wall_shear || wv)) {
            ho.qin = ho.wsin = nullptr;  // uploaded beside the contact update
            rc = ensure_encoding(h);
            if (rc == DEM_OK) rc = build_graphs(h);
            const void* key[DemHandle::kXKey] = {pv, vv, ov, qv, wv, ho.err,
                                                 reinterpret_cast<const void*>((uintptr_t)ho.same)};
            for (int q = 0; q < kHostOutFields; ++q) key[7 + q] = ho.rec[q];
            DemHandle::XGraph& X = h->xg[h->cur];
            if (rc == DEM_OK && (!X.exec || std::memcmp(X.key, key, sizeof(key)) != 0)) {
                if (X.exec) cudaGraphExecDestroy(X.exec);
                X.exec = nullptr;
                rc = capture_exchange(h, h->cur, pv, vv, ov, qv, wv, ho, &X.exec);
                if (rc == DEM_OK) std::memcpy(X.key, key, sizeof(key));
            }
            if (rc == DEM_OK) {
                if (cudaGraphLaunch(X.exec, h->stream) == cudaSuccess) {
                    h->cur ^= 1;
                    h->steps += 1;
                } else {
                    rc = DEM_ERR_CUDA;
                }
            }
        } else {
            DemParticleState up = *in;
            if (ho.qin) up.quat = nullptr;
            if (ho.wsin) up.wall_shear = nullptr;
            rc = set_particles(h, &up, false, &ho);
            if (rc == DEM_OK) rc = dem_step(h, nsteps);
        }
        if (rc != DEM_OK) {  // disarm before any later step can see it
            cudaMemsetAsync(&h->d.ctr->hout, 0, sizeof(HostOut), h->stream);
            cudaStreamSynchronize(h->stream);
            return rc;
        }
        CU(cudaStreamSynchronize(h->stream));
        const int err = *reinterpret_cast<volatile int*>(h->err_host);
        if (err != kNoHostOut) {
            ++h->exchanges_direct;
            return error_code(err);
        }
        // not expected (the split layout writes the records): the usual read
        return dem_get_particles(h, out);
    }
    if (in) TRY(set_particles(h, in, false));
    TRY(dem_step(h, nsteps));
    if (out) return dem_get_particles(h, out);
    return DEM_OK;
}

int dem_host_alloc(int64_t bytes, void** out) {
    if (!out || bytes < 0) return DEM_ERR_INVALID;
    *out = nullptr;
    const size_t nb = (size_t)std::max<int64_t>(bytes, 1);
    CU(cudaMallocHost(out, nb));
    double* dv = device_view(*out);  // before registration: the CUDA driver's answer
    if (dv) {
        HostRanges& H = host_ranges();
        std::lock_guard<std::mutex> lk(H.mu);
        H.r[reinterpret_cast<uintptr_t>(*out)] = {nb, reinterpret_cast<uintptr_t>(dv)};
    }
    return DEM_OK;
}

int dem_host_free(void* p) {
    if (!p) return DEM_OK;
    {
        HostRanges& H = host_ranges();
        std::lock_guard<std::mutex> lk(H.mu);
        H.r.erase(reinterpret_cast<uintptr_t>(p));
    }
    CU(cudaFreeHost(p));
    return DEM_OK;
}

int dem_scene_get_contacts(DemHandle* h, int32_t s, DemContacts* out, int64_t cap,
                           int64_t* n_out) {
    const SceneHost* S = scene_at(h, s);
    if (!S || !n_out) return DEM_ERR_INVALID;
    return get_contacts_range(h, S->sp.p0, S->sp.n, out, cap, n_out);
}

int dem_get_contacts(DemHandle* h, DemContacts* out, int64_t cap, int64_t* n_out) {
    return dem_scene_get_contacts(h, 0, out, cap, n_out);
}

int dem_get_wall_shear(DemHandle* h, int32_t wall, double* shear) {
    if (!h || h->multi || !shear || wall < 0 || wall >= h->nwall) return DEM_ERR_INVALID;
    const size_t o = (size_t)wall * (size_t)h->n_cap;
    const int k[] = {3};
    double* const host[] = {shear};
    double* const cols[][4] = {{h->d.wsx + o, h->d.wsy + o, h->d.wsz + o}};
    int err = 0;
    TRY(exchange(h, 0, h->n_cap, k, host, cols, 1, false, &err));
    return error_code(err);
}

int dem_set_wall_shear(DemHandle* h, int32_t wall, const double* shear) {
    if (!h || h->multi || !shear || wall < 0 || wall >= h->nwall) return DEM_ERR_INVALID;
    const size_t o = (size_t)wall * (size_t)h->n_cap;
    const int k[] = {3};
    double* const host[] = {const_cast<double*>(shear)};
    double* const cols[][4] = {{h->d.wsx + o, h->d.wsy + o, h->d.wsz + o}};
    return exchange(h, 0, h->n_cap, k, host, cols, 1, true);
}

int dem_scene_get_io_contacts(DemHandle* h, int32_t s, DemIOContact* out, int64_t cap,
                              int64_t* n_out) {
    const SceneHost* S = scene_at(h, s);
    if (!S || !n_out || cap < 0) return DEM_ERR_INVALID;
    return get_io_contacts_range(h, S->sp.p0, S->sp.n, out, cap, n_out);
}

int dem_get_io_contacts(DemHandle* h, DemIOContact* out, int64_t cap, int64_t* n_out) {
    return dem_scene_get_io_contacts(h, 0, out, cap, n_out);
}

int dem_set_contacts(DemHandle* h, const DemContacts* in, int64_t nc) {
    if (!h || h->multi || !in || nc < 0 || (nc > 0 && (!in->i || !in->j))) return DEM_ERR_INVALID;
    if (nc > h->p.cap) return DEM_ERR_CAPACITY;
    const int n = h->n_cap;
    std::vector<int64_t> order(nc);
    std::iota(order.begin(), order.end(), 0);
    for (int64_t t = 0; t < nc; ++t)
        if (in->i[t] < 0 || in->j[t] <= in->i[t] || in->j[t] >= n) return DEM_ERR_INVALID;
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        return in->i[a] != in->i[b] ? in->i[a] < in->i[b] : in->j[a] < in->j[b];
    });
    for (int64_t t = 1; t < nc; ++t)
        if (in->i[order[t]] == in->i[order[t - 1]] && in->j[order[t]] == in->j[order[t - 1]])
            return DEM_ERR_INVALID;
    std::vector<int32_t> rs(n, 0), rl(n, 0), ci(nc), cj(nc);
    std::vector<uint32_t> fl(nc);
    std::vector<double> f[15];
    for (int q = 0; q < 15; ++q) f[q].assign(nc, 0.0);
    for (int64_t t = 0; t < nc; ++t) {
        const int64_t s = order[t];
        ci[t] = in->i[s];
        cj[t] = in->j[s];
        fl[t] = kActive | ((in->bonded && in->bonded[s]) ? kBonded : 0u);
        rl[ci[t]]++;
        const double* src[5] = {in->point, in->force, in->torque_i, in->torque_j, in->shear};
        for (int g = 0; g < 5; ++g)
            if (src[g])
                for (int q = 0; q < 3; ++q) f[3 * g + q][t] = src[g][3 * s + q];
        if (h->enc == DEM_FP32_FORCE)
            for (int q = CF; q < CS; ++q) f[q][t] = pair_encode(f[q][t]);
    }
    for (int i = 1; i < n; ++i) rs[i] = rs[i - 1] + rl[i - 1];
    const ContactSoA& s = h->d.c[h->cur];
    if (nc) {
        CU(cudaMemcpyAsync(s.ci, ci.data(), nc * 4, cudaMemcpyHostToDevice, h->stream));
        CU(cudaMemcpyAsync(s.cj, cj.data(), nc * 4, cudaMemcpyHostToDevice, h->stream));
        CU(cudaMemcpyAsync(s.fl, fl.data(), nc * 4, cudaMemcpyHostToDevice, h->stream));
        for (int q = 0; q < 15; ++q)
            CU(cudaMemcpyAsync(s.f[q], f[q].data(), nc * 8, cudaMemcpyHostToDevice, h->stream));
    }
    if (n) {
        CU(cudaMemcpyAsync(h->d.row_start[h->cur], rs.data(), (size_t)n * 4,
                           cudaMemcpyHostToDevice, h->stream));
        CU(cudaMemcpyAsync(h->d.row_len[h->cur], rl.data(), (size_t)n * 4,
                           cudaMemcpyHostToDevice, h->stream));
    }
    // the uploaded buffer's bond count is not kept: the force pass reads the
    // type-ordered list of the buffer a step's rows are placed in
    RowCounter alloc[2] = {{0u, 0u}, {0u, 0u}};
    alloc[h->cur].rows = (unsigned)nc;
    CU(cudaMemcpyAsync(h->d.ctr->alloc, alloc, sizeof(alloc), cudaMemcpyHostToDevice,
                       h->stream));
    CU(cudaStreamSynchronize(h->stream));
    return DEM_OK;
}

int dem_scene_get_stats(DemHandle* h, int32_t s, DemStats* out) {
    const SceneHost* S = scene_at(h, s);
    if (!S || !out) return DEM_ERR_INVALID;
    return stats_of(h, s, *S, out);
}

int dem_get_stats(DemHandle* h, DemStats* out) { return dem_scene_get_stats(h, 0, out); }

int dem_debug_broadphase(DemHandle* h, int32_t* cell, uint32_t* morton, uint32_t* bucket,
                         uint32_t* bucket_count, uint32_t* sorted, int32_t* cp, int64_t cp_cap,
                         int64_t* cp_n) {
    if (!h || !cp_n || h->multi) return DEM_ERR_INVALID;
    const int n = h->n_cap;
    *cp_n = 0;
    if (n == 0) {
        if (bucket_count) std::memset(bucket_count, 0, sizeof(uint32_t) * h->t_cap);
        return DEM_OK;
    }
    launch_broadphase(h->d, h->p, h->cur, false, true, h->ntiles_cells, h->stream);
    uint32_t* dmorton = nullptr;
    int32_t *dcnt = nullptr, *doff = nullptr, *dcp = nullptr;
    auto cleanup = [&]() {
        cudaFree(dmorton);
        cudaFree(dcnt);
        cudaFree(doff);
        cudaFree(dcp);
    };
    if (cudaMalloc(&dmorton, (size_t)n * 4) != cudaSuccess ||
        cudaMalloc(&dcnt, (size_t)n * 4) != cudaSuccess ||
        cudaMalloc(&doff, ((size_t)n + 1) * 4) != cudaSuccess) {
        cleanup();
        return DEM_ERR_CUDA;
    }
    launch_morton(h->d, h->p, dmorton, h->stream);
    launch_cplist_count(h->d, h->p, dcnt, h->stream);
    launch_scan_i32(dcnt, doff, n, h->d, kScanDebug, h->stream);
    int32_t total = 0;
    cudaMemcpyAsync(&total, doff + n, 4, cudaMemcpyDeviceToHost, h->stream);
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
        cleanup();
        return DEM_ERR_CUDA;
    }
    *cp_n = total;
    int rc = DEM_OK;
    if (cp && total > cp_cap) rc = DEM_ERR_CAPACITY;
    if (cp && total <= cp_cap && total > 0) {
        if (cudaMalloc(&dcp, (size_t)total * 8) != cudaSuccess) {
            cleanup();
            return DEM_ERR_CUDA;
        }
        launch_cplist_fill(h->d, h->p, doff, dcp, h->stream);
        cudaMemcpyAsync(cp, dcp, (size_t)total * 8, cudaMemcpyDeviceToHost, h->stream);
    }
    std::vector<int4> ci(n);
    std::vector<uint32_t> bk(n), start;
    cudaMemcpyAsync(ci.data(), h->d.cellinfo, (size_t)n * sizeof(int4), cudaMemcpyDeviceToHost,
                    h->stream);
    cudaMemcpyAsync(bk.data(), h->d.bucket, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream);
    if (morton) cudaMemcpyAsync(morton, dmorton, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream);
    if (sorted) cudaMemcpyAsync(sorted, h->d.sorted, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream);
    if (bucket_count) {
        start.resize((size_t)h->t_cap + 1);
        cudaMemcpyAsync(start.data(), h->d.cell_start, start.size() * 4, cudaMemcpyDeviceToHost,
                        h->stream);
    }
    cudaError_t e = cudaStreamSynchronize(h->stream);
    cleanup();
    if (e != cudaSuccess) {
        std::snprintf(g_msg, sizeof(g_msg), "dem_debug_broadphase: %s", cudaGetErrorString(e));
        return DEM_ERR_CUDA;
    }
    for (int i = 0; i < n; ++i) {
        if (cell) {
            cell[3 * i] = ci[i].x;
            cell[3 * i + 1] = ci[i].y;
            cell[3 * i + 2] = ci[i].z;
        }
        if (bucket) bucket[i] = bk[i] + 1u;
    }
    DevCounters ctr;
    if (cudaMemcpy(&ctr, h->d.ctr, sizeof(ctr), cudaMemcpyDeviceToHost) != cudaSuccess)
        return DEM_ERR_CUDA;
    if (bucket_count)
        for (uint32_t b = 0; b < h->t_cap; ++b)
            bucket_count[b] = b < ctr.cell_limit ? start[b + 1] - start[b] : 0u;
    int err = device_error(h);
    return err != DEM_OK ? err : rc;
}

int dem_debug_step_enumeration(DemHandle* h, int64_t* pairs, uint64_t* checksum) {
    if (!h || !pairs || !checksum || h->multi) return DEM_ERR_INVALID;
    *pairs = 0;
    *checksum = 0;
    if (h->n_cap == 0) return DEM_OK;
    TRY(ensure_encoding(h));
    TRY(flag_search(h, 0));
    CU(cudaMemsetAsync(&h->d.ctr->enum_pairs, 0, 2 * sizeof(unsigned long long), h->stream));
    DemParams p = h->p;  // the captured graphs keep debug_enum = 0
    p.debug_enum = 1;
    const int cur = h->cur;
    launch_search(h->d, p, cur, false, false, false, h->shape, h->stream);
    launch_force(h->d, p, cur ^ 1, false, h->shape, h->stream);
    launch_integrate(h->d, p, cur, false, h->shape, h->stream);
    CU(cudaGetLastError());
    h->cur ^= 1;
    h->steps += 1;
    DevCounters c;
    TRY(read_counters(h, &c));
    *pairs = (int64_t)c.enum_pairs;
    *checksum = (uint64_t)c.enum_hash;
    return error_code(c.error);
}

int dem_selftest_wait_timeout(int which, int missing, int64_t spin_limit, int* status) {
    if (!status || (which != 0 && which != 1) || spin_limit < 1 || spin_limit > (1 << 20))
        return DEM_ERR_INVALID;
    int dev = 0, sms = 0;
    TRY(check_device(&dev, &sms));
    DevCounters* c = nullptr;
    unsigned long long* state = nullptr;
    uint32_t* io = nullptr;
    const size_t tile = 8192;  // values per scan tile
    auto cleanup = [&]() {
        cudaFree(c);
        cudaFree(state);
        cudaFree(io);
    };
    cudaError_t e = cudaMalloc(&c, sizeof(DevCounters));
    if (e == cudaSuccess) e = cudaMalloc(&state, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&io, (4 * tile + 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(c, 0, sizeof(DevCounters));
    if (e == cudaSuccess) e = cudaMemset(state, 0, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(io, 0, (4 * tile + 1) * sizeof(uint32_t));
    if (e == cudaSuccess)
        e = launch_selftest_wait(which, missing ? 1 : 0, (unsigned long long)spin_limit, c, state,
                                 io, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    DevCounters hc{};
    if (e == cudaSuccess) e = cudaMemcpy(&hc, c, sizeof(hc), cudaMemcpyDeviceToHost);
    cleanup();
    CU(e);
    *status = error_code(hc.error);
    return DEM_OK;
}

}  // extern "C"
