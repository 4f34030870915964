// dem_api.cu — the C ABI of libdem_sm100a.so (include/dem_gb300.h).
//
// Host responsibilities: the per-scene setup that `solve` performs before its
// loop (src/executor.jl:217-315), device buffers, the CUDA-graph step
// (`simulate!`, src/executor.jl:162-172) and host<->device state exchange.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <numeric>
#include <vector>

#include "dem_gb300.h"
#include "dem_internal.h"

using namespace dem;

namespace {

constexpr double kPi = 3.141592653589793;

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

}  // namespace

struct DemHandle {
    DemConfigC cfg{};
    DemDerived der{};
    DemParams p{};
    DemDev d{};
    int device = 0;
    int n = 0;
    int sm_count = 0;
    int cur = 0;  // contact buffer holding the current state
    int64_t steps = 0;
    int ntiles_cells = 0;
    int force_grid = 1;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    int graph_precision = -1;
    std::vector<void*> allocs;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double* pinned = nullptr;  // host staging for particle state exchange
};

#define CU(expr)                                                                   \
    do {                                                                           \
        cudaError_t _e = (expr);                                                   \
        if (_e != cudaSuccess) {                                                   \
            std::snprintf(g_msg, sizeof(g_msg), "%s: %s", #expr, cudaGetErrorString(_e)); \
            return DEM_ERR_CUDA;                                                   \
        }                                                                          \
    } while (0)

namespace {

template <typename T>
int dalloc(DemHandle* h, T** ptr, size_t count) {
    void* p = nullptr;
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    CU(cudaMalloc(&p, bytes));
    CU(cudaMemsetAsync(p, 0, bytes, h->stream));
    h->allocs.push_back(p);
    *ptr = static_cast<T*>(p);
    return DEM_OK;
}

#define TRY(expr)                      \
    do {                               \
        int _rc = (expr);              \
        if (_rc != DEM_OK) return _rc; \
    } while (0)

int allocate(DemHandle* h) {
    const size_t n = (size_t)h->n, cap = (size_t)h->p.cap, H = h->p.H;
    DemDev& d = h->d;
    double** dbl[] = {&d.px, &d.py, &d.pz, &d.vx, &d.vy, &d.vz, &d.wx, &d.wy, &d.wz,
                      &d.qw, &d.qx, &d.qy, &d.qz, &d.m, &d.inv_m, &d.r, &d.r0, &d.inv_inertia, &d.b_invA, &d.b_rbI,
                      &d.b_EA, &d.b_EI, &d.b_phic,
                      &d.fx, &d.fy, &d.fz, &d.tx, &d.ty, &d.tz, &d.wsx, &d.wsy, &d.wsz};
    for (double** a : dbl) TRY(dalloc(h, a, n));
    TRY(dalloc(h, &d.cellinfo, n));
    TRY(dalloc(h, &d.bucket, n));
    TRY(dalloc(h, &d.cell_count, H));
    TRY(dalloc(h, &d.cell_start, H + 1));
    TRY(dalloc(h, &d.unsorted, n));
    TRY(dalloc(h, &d.sorted, n));
    TRY(dalloc(h, &d.spos, n));
    TRY(dalloc(h, &d.spos32, n));
    for (int b = 0; b < 2; ++b) {
        TRY(dalloc(h, &d.c[b].ci, cap));
        TRY(dalloc(h, &d.c[b].cj, cap));
        TRY(dalloc(h, &d.c[b].fl, cap));
        for (int f = 0; f < 15; ++f) TRY(dalloc(h, &d.c[b].f[f], cap));
        TRY(dalloc(h, &d.row_start[b], n));
        TRY(dalloc(h, &d.row_len[b], n));
    }
    TRY(dalloc(h, &d.nnew, n));
    TRY(dalloc(h, &d.stash, n * (size_t)h->p.kstash));
    TRY(dalloc(h, &d.keep, cap));
    TRY(dalloc(h, &d.in_cnt, n));
    TRY(dalloc(h, &d.in_list, n * (size_t)h->p.kin));
    TRY(dalloc(h, &d.contrib, 9 * cap));
    TRY(dalloc(h, &d.scan_state[kScanCells], (size_t)scan_tiles((int64_t)H)));
    TRY(dalloc(h, &d.scan_state[kScanDebug], (size_t)scan_tiles((int64_t)n)));
    TRY(dalloc(h, &d.ctr, 1));
    return DEM_OK;
}

void free_all(DemHandle* h) {
    for (int b = 0; b < 2; ++b)
        if (h->exec[b]) cudaGraphExecDestroy(h->exec[b]);
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->pinned) cudaFreeHost(h->pinned);
    h->pinned = nullptr;
}

void record_step(DemHandle* h, int cur) {
    const int nxt = cur ^ 1;
    launch_broadphase(h->d, h->p, h->ntiles_cells, h->stream);
    launch_detect(h->d, h->p, cur, false, h->stream);
    launch_compact(h->d, h->p, cur, false, h->force_grid, h->stream);
    launch_force(h->d, h->p, nxt, h->force_grid, h->stream);
    launch_integrate(h->d, h->p, cur, h->stream);
}

int build_graphs(DemHandle* h) {
    if (h->graph_precision == h->p.precision && h->exec[0]) return DEM_OK;
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

int device_error(DemHandle* h) {
    DevCounters c;
    TRY(read_counters(h, &c));
    if (c.error & kErrCapacity) return DEM_ERR_CAPACITY;
    if (c.error & kErrTimeout) return DEM_ERR_TIMEOUT;
    if (c.error & kErrRange) return DEM_ERR_RANGE;
    return DEM_OK;
}

int contact_count(DemHandle* h, int buf, int32_t* total) {
    unsigned int v = 0;
    CU(cudaMemcpyAsync(&v, &h->d.ctr->row_alloc[buf], sizeof(v), cudaMemcpyDeviceToHost,
                       h->stream));
    CU(cudaStreamSynchronize(h->stream));
    *total = (int32_t)v;
    return DEM_OK;
}

int get_dev(std::vector<double>& host, const double* dev, size_t n, cudaStream_t s) {
    host.resize(n);
    if (n) CU(cudaMemcpyAsync(host.data(), dev, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    return DEM_OK;
}

}  // namespace

extern "C" {

const char* dem_version(void) { return "dem_gb300 0.1.0 sm_103a"; }

const char* dem_strerror(int code) {
    switch (code) {
        case DEM_OK: return "ok";
        case DEM_ERR_INVALID: return "invalid argument or state";
        case DEM_ERR_CUDA: return g_msg[0] ? g_msg : "CUDA runtime error";
        case DEM_ERR_CAPACITY: return "contact buffer capacity exceeded (raise max_coordinate_number)";
        case DEM_ERR_TIMEOUT: return "a bounded device-side wait gave up";
        case DEM_ERR_NO_DEVICE: return "no sm_103 (GB300) CUDA device available";
        case DEM_ERR_RANGE: return "particle outside the representable cell range";
        default: return "unknown error";
    }
}

int dem_set_device(int device) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return DEM_ERR_NO_DEVICE;
    if (device < 0 || device >= ndev) return DEM_ERR_INVALID;
    CU(cudaSetDevice(device));
    return DEM_OK;
}

int dem_create(const DemConfigC* cfg, const DemParticlesIn* pin, DemHandle** out) {
    if (!cfg || !pin || !out || pin->n < 0 || pin->n > 0x3fffffff) return DEM_ERR_INVALID;
    if (pin->n > 0 && (!pin->volume || !pin->mass || !pin->pos || !pin->vel)) return DEM_ERR_INVALID;
    if (!(cfg->dt > 0) || cfg->max_coordinate_number <= 0) return DEM_ERR_INVALID;
    *out = nullptr;
    int dev = 0, ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return DEM_ERR_NO_DEVICE;
    CU(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    CU(cudaGetDeviceProperties(&prop, dev));
    if (prop.major != 10 || prop.minor != 3) {
        std::snprintf(g_msg, sizeof(g_msg), "device %d is sm_%d%d; this library is built for sm_103a",
                      dev, prop.major, prop.minor);
        return DEM_ERR_NO_DEVICE;
    }
    DemHandle* h = new DemHandle();
    h->cfg = *cfg;
    h->device = dev;
    h->sm_count = prop.multiProcessorCount;
    h->n = (int)pin->n;
    const int n = h->n;
    // grain setup (src/executor.jl:219-243)
    std::vector<double> r(n), r0(n), inv_inertia(n), inv_m(n), q0(n, 1.0), zeros(n, 0.0);
    std::vector<double> b_invA(n), b_rbI(n), b_EA(n), b_EI(n), b_phic(n);
    std::vector<double> pos[3], vel[3];
    double rmax_r = -INFINITY;
    for (int c = 0; c < 3; ++c) {
        pos[c].resize(n);
        vel[c].resize(n);
    }
    for (int i = 0; i < n; ++i) {
        const double V = pin->volume[i], m = pin->mass[i];
        r[i] = std::cbrt(V / (4.0 / 3.0 * kPi));
        r0[i] = r[i] * cfg->particle_contact_radius_multiplier;
        inv_inertia[i] = 1.0 / (2.0 / 5.0 * m * (r[i] * r[i]));
        inv_m[i] = 1.0 / m;
        // bond section of src/kernels.jl:178-184 for rb = ρ·rᵢ: 1/A and rb/I
        const double rb = cfg->bond_radius_ratio * r[i];
        const double Ab = rb * rb * kPi, Ib = rb * rb * (rb * rb) * (kPi / 4.0);
        b_invA[i] = 1.0 / Ab;
        b_rbI[i] = rb / Ib;
        b_EA[i] = cfg->bond_elastic_modulus * Ab;
        b_EI[i] = cfg->bond_elastic_modulus * Ib;
        b_phic[i] = 20.0 / 3.0 * (1.0 + cfg->bond_poisson_ratio) * (rb * rb);
        rmax_r = std::max(rmax_r, r[i]);
        for (int c = 0; c < 3; ++c) {
            pos[c][i] = pin->pos[3 * i + c];
            vel[c][i] = pin->vel[3 * i + c];
        }
    }
    // derived sizes (src/executor.jl:244-267)
    DemDerived& D = h->der;
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
    if (n > 0 && !(D.cell_size > 0 && std::isfinite(D.cell_size))) {
        delete h;
        return DEM_ERR_INVALID;
    }
    if (D.contact_capacity > 0x7fffffff) {
        delete h;
        return DEM_ERR_CAPACITY;
    }
    // device constants (materials / surfaces / wall of src/executor.jl:282-315)
    DemParams& p = h->p;
    p.n = n;
    p.cap = (int)D.contact_capacity;
    p.kstash = (int)std::min<int64_t>(cfg->max_coordinate_number, 64);
    p.kin = p.kstash;
    p.H = (uint32_t)D.hash_table_size;
    p.H_pow2_mask = (p.H & (p.H - 1)) == 0 ? p.H - 1 : 0;
    p.has_wall = 1;
    p.precision = DEM_FP64;
    for (int c = 0; c < 3; ++c) {
        p.dmin[c] = cfg->domain_min[c];
        p.grav[c] = cfg->gravity[c];
        p.wn[c] = cfg->wall_normal[c];
    }
    p.cell = D.cell_size;
    p.inv_cell = 1.0 / D.cell_size;
    p.dt = cfg->dt;
    p.tol = cfg->tolerance;
    p.damping = cfg->global_damping;
    const Hertz pp = hertz_constants(cfg->particle_elastic_modulus, cfg->particle_poisson_ratio,
                                     cfg->particle_elastic_modulus, cfg->particle_poisson_ratio,
                                     cfg->pp_coefficient_restitution);
    p.pp_mu = cfg->pp_coefficient_friction;
    p.pp_beta = pp.beta;
    p.pp_Ys = pp.Ys;
    p.pp_Gs = pp.Gs;
    p.pp_cgn = pp.cgn;
    p.pp_cgt = pp.cgt;
    p.b_rho = cfg->bond_radius_ratio;
    p.b_E = cfg->bond_elastic_modulus;
    p.b_nu = cfg->bond_poisson_ratio;
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
    p.pw_beta = pw.beta;
    p.pw_Ys = pw.Ys;
    p.pw_Gs = pw.Gs;
    p.pw_cgn = pw.cgn;
    p.pw_cgt = pw.cgt;

    auto fail = [&](int rc) {
        free_all(h);
        delete h;
        return rc;
    };
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(DEM_ERR_CUDA);
    if (cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess)
        return fail(DEM_ERR_CUDA);
    int rc = allocate(h);
    if (rc != DEM_OK) return fail(rc);
    h->ntiles_cells = scan_tiles((int64_t)p.H);
    h->force_grid = (int)std::max<int64_t>(
        1, std::min<int64_t>(((int64_t)p.cap + 255) / 256, (int64_t)h->sm_count * 16));
    auto up = [&](double* dst, const std::vector<double>& src) {
        return n ? cudaMemcpyAsync(dst, src.data(), n * sizeof(double), cudaMemcpyHostToDevice,
                                   h->stream)
                 : cudaSuccess;
    };
    std::vector<double> mass(pin->mass, pin->mass + n);
    cudaError_t e = cudaSuccess;
    double* pd[3] = {h->d.px, h->d.py, h->d.pz};
    double* vd[3] = {h->d.vx, h->d.vy, h->d.vz};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c) {
        e = up(pd[c], pos[c]);
        if (e == cudaSuccess) e = up(vd[c], vel[c]);
    }
    if (e == cudaSuccess) e = up(h->d.qw, q0);
    if (e == cudaSuccess) e = up(h->d.m, mass);
    if (e == cudaSuccess) e = up(h->d.inv_m, inv_m);
    if (e == cudaSuccess) e = up(h->d.b_invA, b_invA);
    if (e == cudaSuccess) e = up(h->d.b_rbI, b_rbI);
    if (e == cudaSuccess) e = up(h->d.b_EA, b_EA);
    if (e == cudaSuccess) e = up(h->d.b_EI, b_EI);
    if (e == cudaSuccess) e = up(h->d.b_phic, b_phic);
    if (e == cudaSuccess) e = up(h->d.r, r);
    if (e == cudaSuccess) e = up(h->d.r0, r0);
    if (e == cudaSuccess) e = up(h->d.inv_inertia, inv_inertia);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        std::snprintf(g_msg, sizeof(g_msg), "dem_create upload: %s", cudaGetErrorString(e));
        return fail(DEM_ERR_CUDA);
    }
    *out = h;
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
    h->p.precision = mode;
    return DEM_OK;
}

int dem_init_bonds(DemHandle* h) {
    if (!h) return DEM_ERR_INVALID;
    if (h->n == 0) return DEM_OK;
    const int cur = h->cur, nxt = cur ^ 1;
    launch_broadphase(h->d, h->p, h->ntiles_cells, h->stream);
    launch_detect(h->d, h->p, cur, true, h->stream);
    launch_compact(h->d, h->p, cur, true, h->force_grid, h->stream);
    // the old buffer becomes the next step's target: its allocator starts at 0
    CU(cudaMemsetAsync(&h->d.ctr->row_alloc[cur], 0, sizeof(unsigned int), h->stream));
    CU(cudaGetLastError());
    h->cur = nxt;
    return device_error(h);
}

int dem_step(DemHandle* h, int64_t nsteps) {
    if (!h || nsteps < 0) return DEM_ERR_INVALID;
    if (h->n == 0 || nsteps == 0) {
        h->steps += nsteps;
        return DEM_OK;
    }
    TRY(build_graphs(h));
    for (int64_t s = 0; s < nsteps; ++s) {
        CU(cudaGraphLaunch(h->exec[h->cur], h->stream));
        h->cur ^= 1;
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
    if (!h || !phase_ms || nphase < 5) return DEM_ERR_INVALID;
    if (h->n == 0) {
        for (int k = 0; k < 5; ++k) phase_ms[k] = 0.f;
        return DEM_OK;
    }
    cudaEvent_t ev[6];
    for (int k = 0; k < 6; ++k) CU(cudaEventCreate(&ev[k]));
    const int cur = h->cur, nxt = cur ^ 1;
    cudaEventRecord(ev[0], h->stream);
    launch_broadphase(h->d, h->p, h->ntiles_cells, h->stream);
    cudaEventRecord(ev[1], h->stream);
    launch_detect(h->d, h->p, cur, false, h->stream);
    cudaEventRecord(ev[2], h->stream);
    launch_compact(h->d, h->p, cur, false, h->force_grid, h->stream);
    cudaEventRecord(ev[3], h->stream);
    launch_force(h->d, h->p, nxt, h->force_grid, h->stream);
    cudaEventRecord(ev[4], h->stream);
    launch_integrate(h->d, h->p, cur, h->stream);
    cudaEventRecord(ev[5], h->stream);
    cudaError_t e = cudaEventSynchronize(ev[5]);
    for (int k = 0; k < 5 && e == cudaSuccess; ++k) e = cudaEventElapsedTime(&phase_ms[k], ev[k], ev[k + 1]);
    for (int k = 0; k < 6; ++k) cudaEventDestroy(ev[k]);
    CU(e);
    h->cur = nxt;
    h->steps += 1;
    return device_error(h);
}

int dem_sync(DemHandle* h) {
    if (!h) return DEM_ERR_INVALID;
    return device_error(h);
}

int dem_get_derived(DemHandle* h, DemDerived* out) {
    if (!h || !out) return DEM_ERR_INVALID;
    *out = h->der;
    return DEM_OK;
}

int dem_get_static(DemHandle* h, DemParticleStatic* out) {
    if (!h || !out) return DEM_ERR_INVALID;
    const size_t n = (size_t)h->n;
    std::vector<double> r, r0, m, ii;
    TRY(get_dev(r, h->d.r, n, h->stream));
    TRY(get_dev(r0, h->d.r0, n, h->stream));
    TRY(get_dev(m, h->d.m, n, h->stream));
    TRY(get_dev(ii, h->d.inv_inertia, n, h->stream));
    CU(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < n; ++i) {
        if (out->radius) out->radius[i] = r[i];
        if (out->radius0) out->radius0[i] = r0[i];
        if (out->mass) out->mass[i] = m[i];
        if (out->inertia) out->inertia[i] = 1.0 / ii[i];
    }
    return DEM_OK;
}

// Particle state exchange goes through one pinned staging buffer per handle
// (22 FP64 columns), so each call is one batch of asynchronous copies and one
// synchronisation.
static int staging(DemHandle* h, double** out) {
    if (!h->pinned) CU(cudaMallocHost(&h->pinned, sizeof(double) * 22 * std::max(h->n, 1)));
    *out = h->pinned;
    return DEM_OK;
}

int dem_get_particles(DemHandle* h, DemParticleState* out) {
    if (!h || !out) return DEM_ERR_INVALID;
    const size_t n = (size_t)h->n;
    struct F {
        double* dst;
        int stride;
        double* src[4];
        int k;
    };
    const F fields[] = {{out->pos, 3, {h->d.px, h->d.py, h->d.pz}, 3},
                        {out->vel, 3, {h->d.vx, h->d.vy, h->d.vz}, 3},
                        {out->omega, 3, {h->d.wx, h->d.wy, h->d.wz}, 3},
                        {out->quat, 4, {h->d.qw, h->d.qx, h->d.qy, h->d.qz}, 4},
                        {out->force, 3, {h->d.fx, h->d.fy, h->d.fz}, 3},
                        {out->moment, 3, {h->d.tx, h->d.ty, h->d.tz}, 3},
                        {out->wall_shear, 3, {h->d.wsx, h->d.wsy, h->d.wsz}, 3}};
    double* st = nullptr;
    TRY(staging(h, &st));
    if (n) {
        size_t col = 0;
        for (const F& f : fields) {
            if (!f.dst) continue;
            for (int c = 0; c < f.k; ++c, ++col)
                CU(cudaMemcpyAsync(st + col * n, f.src[c], n * sizeof(double),
                                   cudaMemcpyDeviceToHost, h->stream));
        }
        CU(cudaStreamSynchronize(h->stream));
        col = 0;
        for (const F& f : fields) {
            if (!f.dst) continue;
            for (int c = 0; c < f.k; ++c, ++col) {
                const double* src = st + col * n;
                for (size_t i = 0; i < n; ++i) f.dst[f.stride * i + c] = src[i];
            }
        }
    }
    return device_error(h);
}

int dem_set_particles(DemHandle* h, const DemParticleState* in) {
    if (!h || !in) return DEM_ERR_INVALID;
    const size_t n = (size_t)h->n;
    struct F {
        const double* src;
        int stride;
        double* dst[4];
        int k;
    };
    const F fields[] = {{in->pos, 3, {h->d.px, h->d.py, h->d.pz}, 3},
                        {in->vel, 3, {h->d.vx, h->d.vy, h->d.vz}, 3},
                        {in->omega, 3, {h->d.wx, h->d.wy, h->d.wz}, 3},
                        {in->quat, 4, {h->d.qw, h->d.qx, h->d.qy, h->d.qz}, 4},
                        {in->wall_shear, 3, {h->d.wsx, h->d.wsy, h->d.wsz}, 3}};
    double* st = nullptr;
    TRY(staging(h, &st));
    if (!n) return DEM_OK;
    CU(cudaStreamSynchronize(h->stream));  // the staging buffer may still be in use
    size_t col = 0;
    for (const F& f : fields) {
        if (!f.src) continue;
        for (int c = 0; c < f.k; ++c, ++col) {
            double* dst = st + col * n;
            for (size_t i = 0; i < n; ++i) dst[i] = f.src[f.stride * i + c];
            CU(cudaMemcpyAsync(f.dst[c], dst, n * sizeof(double), cudaMemcpyHostToDevice,
                               h->stream));
        }
    }
    CU(cudaStreamSynchronize(h->stream));
    return DEM_OK;
}

int dem_get_contacts(DemHandle* h, DemContacts* out, int64_t cap, int64_t* n_out) {
    if (!h || !n_out) return DEM_ERR_INVALID;
    TRY(device_error(h));
    int32_t C = 0;
    if (h->n) TRY(contact_count(h, h->cur, &C));
    C = std::min(C, h->p.cap);
    const ContactSoA& s = h->d.c[h->cur];
    std::vector<int32_t> ci(C), cj(C);
    std::vector<uint32_t> fl(C);
    std::vector<double> f[15];
    if (C) {
        CU(cudaMemcpyAsync(ci.data(), s.ci, C * 4, cudaMemcpyDeviceToHost, h->stream));
        CU(cudaMemcpyAsync(cj.data(), s.cj, C * 4, cudaMemcpyDeviceToHost, h->stream));
        CU(cudaMemcpyAsync(fl.data(), s.fl, C * 4, cudaMemcpyDeviceToHost, h->stream));
        for (int q = 0; q < 15; ++q) TRY(get_dev(f[q], s.f[q], (size_t)C, h->stream));
        CU(cudaStreamSynchronize(h->stream));
    }
    std::vector<int32_t> act;  // active contacts, sorted by (i, j)
    act.reserve(C);
    for (int32_t c = 0; c < C; ++c)
        if (fl[c] & kActive) act.push_back(c);
    std::sort(act.begin(), act.end(), [&](int32_t a, int32_t b) {
        return ci[a] != ci[b] ? ci[a] < ci[b] : cj[a] < cj[b];
    });
    const int64_t na = (int64_t)act.size();
    *n_out = na;
    if (!out) return DEM_OK;
    if (na > cap) return DEM_ERR_CAPACITY;
    for (int64_t t = 0; t < na; ++t) {
        const int32_t c = act[t];
        if (out->i) out->i[t] = ci[c];
        if (out->j) out->j[t] = cj[c];
        if (out->bonded) out->bonded[t] = (fl[c] & kBonded) ? 1 : 0;
        for (int q = 0; q < 3; ++q) {
            if (out->point) out->point[3 * t + q] = f[CK + q][c];
            if (out->force) out->force[3 * t + q] = f[CF + q][c];
            if (out->torque_i) out->torque_i[3 * t + q] = f[CTI + q][c];
            if (out->torque_j) out->torque_j[3 * t + q] = f[CTJ + q][c];
            if (out->shear) out->shear[3 * t + q] = f[CS + q][c];
        }
    }
    return DEM_OK;
}

int dem_set_contacts(DemHandle* h, const DemContacts* in, int64_t nc) {
    if (!h || !in || nc < 0 || (nc > 0 && (!in->i || !in->j))) return DEM_ERR_INVALID;
    if (nc > h->p.cap) return DEM_ERR_CAPACITY;
    const int n = h->n;
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
        CU(cudaMemcpyAsync(h->d.row_start[h->cur], rs.data(), n * 4, cudaMemcpyHostToDevice,
                           h->stream));
        CU(cudaMemcpyAsync(h->d.row_len[h->cur], rl.data(), n * 4, cudaMemcpyHostToDevice,
                           h->stream));
    }
    const unsigned int alloc[2] = {h->cur == 0 ? (unsigned)nc : 0u, h->cur == 1 ? (unsigned)nc : 0u};
    CU(cudaMemcpyAsync(h->d.ctr->row_alloc, alloc, sizeof(alloc), cudaMemcpyHostToDevice,
                       h->stream));
    CU(cudaStreamSynchronize(h->stream));
    return DEM_OK;
}

int dem_get_stats(DemHandle* h, DemStats* out) {
    if (!h || !out) return DEM_ERR_INVALID;
    DevCounters c;
    TRY(read_counters(h, &c));
    int32_t C = 0;
    if (h->n) TRY(contact_count(h, h->cur, &C));
    C = std::min(C, h->p.cap);
    std::vector<uint32_t> fl(C);
    if (C) CU(cudaMemcpy(fl.data(), h->d.c[h->cur].fl, C * 4, cudaMemcpyDeviceToHost));
    int64_t act = 0, bnd = 0;
    for (uint32_t f : fl) {
        act += (f & kActive) ? 1 : 0;
        bnd += ((f & kActive) && (f & kBonded)) ? 1 : 0;
    }
    std::memset(out, 0, sizeof(*out));
    out->n_particles = h->n;
    out->steps_done = h->steps;
    out->contacts = act;
    out->bonded = bnd;
    out->bonds_broken = (int64_t)c.broken;
    out->contacts_ended = (int64_t)c.ended;
    out->contacts_created = (int64_t)c.created;
    out->warn_gap = (int64_t)c.warn_gap;
    out->warn_damping = (int64_t)c.warn_damp;
    out->error = (c.error & kErrCapacity) ? DEM_ERR_CAPACITY
                 : (c.error & kErrTimeout) ? DEM_ERR_TIMEOUT
                 : (c.error & kErrRange)   ? DEM_ERR_RANGE
                                           : DEM_OK;
    out->precision = h->p.precision;
    return DEM_OK;
}

int dem_debug_broadphase(DemHandle* h, int32_t* cell, uint32_t* morton, uint32_t* bucket,
                         uint32_t* bucket_count, uint32_t* sorted, int32_t* cp, int64_t cp_cap,
                         int64_t* cp_n) {
    if (!h || !cp_n) return DEM_ERR_INVALID;
    const int n = h->n;
    *cp_n = 0;
    if (n == 0) {
        if (bucket_count) std::memset(bucket_count, 0, sizeof(uint32_t) * h->p.H);
        return DEM_OK;
    }
    launch_broadphase(h->d, h->p, h->ntiles_cells, h->stream);
    uint32_t* dmorton = nullptr;
    int32_t *dcnt = nullptr, *doff = nullptr, *dcp = nullptr;
    auto cleanup = [&]() {
        cudaFree(dmorton);
        cudaFree(dcnt);
        cudaFree(doff);
        cudaFree(dcp);
    };
    if (cudaMalloc(&dmorton, n * 4) != cudaSuccess || cudaMalloc(&dcnt, n * 4) != cudaSuccess ||
        cudaMalloc(&doff, (n + 1) * 4) != cudaSuccess) {
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
    cudaMemcpyAsync(ci.data(), h->d.cellinfo, n * sizeof(int4), cudaMemcpyDeviceToHost, h->stream);
    cudaMemcpyAsync(bk.data(), h->d.bucket, n * 4, cudaMemcpyDeviceToHost, h->stream);
    if (morton) cudaMemcpyAsync(morton, dmorton, n * 4, cudaMemcpyDeviceToHost, h->stream);
    if (sorted) cudaMemcpyAsync(sorted, h->d.sorted, n * 4, cudaMemcpyDeviceToHost, h->stream);
    if (bucket_count) {
        start.resize((size_t)h->p.H + 1);
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
        for (uint32_t b = 0; b < h->p.H; ++b)
            bucket_count[b] = b < ctr.cell_limit ? start[b + 1] - start[b] : 0u;
    int err = device_error(h);
    return err != DEM_OK ? err : rc;
}

}  // extern "C"
