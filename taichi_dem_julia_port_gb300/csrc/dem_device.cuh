// dem_device.cuh — device helpers shared by the DEM kernels.
#pragma once

#include <cuda/atomic>
#include <math_constants.h>

#include "dem_internal.h"

namespace dem {

// ---- exact (non-contracted) FP64 pieces --------------------------------------
// The reference compares distances and cell coordinates with plain IEEE
// arithmetic (Julia does not fuse multiply-adds).  Every quantity that feeds a
// discrete decision is computed here with explicit round-to-nearest intrinsics
// so that nvcc cannot contract it into an FMA.

__device__ __forceinline__ int32_t ceil_i32(double t) {
    double c = ceil(t);
    if (!(c > -2147483648.0 && c < 2147483647.0)) return 0;  // NaN / overflow
    return (int32_t)c;
}

// StaticArrays `norm` (sqrt of ((x²+y²)+z²), rescaled when not in (0, Inf)).
static __device__ __noinline__ double norm_scaled(double x, double y, double z) {
    if (isnan(x) || isnan(y) || isnan(z)) return CUDART_NAN;
    double sc = fmax(fabs(x), fmax(fabs(y), fabs(z)));
    if (sc == 0.0) return 0.0;
    double a = __ddiv_rn(x, sc), b = __ddiv_rn(y, sc), c = __ddiv_rn(z, sc);
    return __dmul_rn(sc, __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)),
                                              __dmul_rn(c, c))));
}
__device__ __forceinline__ double norm_rn(double x, double y, double z) {
    double l = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
    if (l > 0.0 && l < CUDART_INF) return l;
    return norm_scaled(x, y, z);
}

// `norm(𝐤ᵢ - 𝐤ⱼ) < rᵢ + rⱼ` exactly as the reference evaluates it
// (src/kernels.jl:72, 103).
__device__ __forceinline__ bool touching_rn(double xi, double yi, double zi, double xj, double yj,
                                            double zj, double ri, double rj) {
    double l = norm_rn(__dsub_rn(xi, xj), __dsub_rn(yi, yj), __dsub_rn(zi, zj));
    return l < __dadd_rn(ri, rj);
}

// Conservative FP32 rejection: returns false only when the FP64 test above is
// certain to fail.  Inputs are FP32 copies (u = 2^-24 relative rounding) of
// positions relative to a common origin; .w holds the particle's reach
// w = r'(1 + 2^-19) + M·2^-19 (r' its FP32 radius, M its largest coordinate
// magnitude), see reach32.  The FP32 distance d' differs from the true one by
// at most 2(M_i + M_j)u + 6u·d', and r_i + r_j <= (r'_i + r'_j)(1 + 3u); the
// test rejects only when d'(1 - 2^-18) exceeds w_i + w_j, which leaves a
// factor of 10 on each error term.
__device__ __forceinline__ float reach32(float x, float y, float z, float r) {
    const float M = fmaxf(fmaxf(fabsf(x), fabsf(y)), fabsf(z));
    return (r * (1.0f + 0x1p-19f) + M * 0x1p-19f) * (1.0f + 0x1p-21f);
}
__device__ __forceinline__ bool maybe_touching32(float4 a, float4 b, float extra = 0.0f) {
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    const float s = dx * dx + dy * dy + dz * dz;
    const float B = a.w + b.w + extra;  // extra: the neighbour-list skin
    return !(s * (1.0f - 0x1p-17f) > B * B);
}

// Conservative FP32 acceptance, the mirror of maybe_touching32: returns true
// only when the FP64 test touching_rn is certain to succeed.  a, b are the
// particles' FP32 positions (as for maybe_touching32), ra, rb their FP32
// radii; each inner reach r'(1 - 2^-19) - M·2^-19 and the factor 1 + 2^-17 on
// the squared distance take the same error bounds the other way (the FP64
// evaluation's own rounding, ~2^-52 relative, is far inside the margins).
__device__ __forceinline__ float inner_reach32(float4 a, float r) {
    const float M = fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fabsf(a.z));
    return (r * (1.0f - 0x1p-19f) - M * 0x1p-19f) * (1.0f - 0x1p-21f);
}
__device__ __forceinline__ bool surely_touching32(float4 a, float ra, float4 b, float rb) {
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    const float s = dx * dx + dy * dy + dz * dz;
    const float B = inner_reach32(a, ra) + inner_reach32(b, rb);
    return B > 0.0f && s * (1.0f + 0x1p-17f) < B * B;
}

// ---- FP64 <-> FP32 conversions on the integer pipe -----------------------------
// GB300 runs conversions involving FP64 on its narrow FP64 pipe.  These do the
// same conversions with integer instructions, from the IEEE 754 binary64 and
// binary32 layouts: narrowing rounds to nearest, ties to even (a carry out of
// the significand moves into the exponent, up to infinity as the rounding
// requires); widening is exact.  Inputs whose result is zero, subnormal or
// not finite take the hardware conversion.
// The rare cases are out-of-line calls, so the compiler cannot evaluate them
// unconditionally (on the FP64 pipe) and select.
static __device__ __noinline__ float d2f_hw(double x) { return __double2float_rn(x); }
static __device__ __noinline__ double f2d_hw(float f) { return (double)f; }
__device__ __forceinline__ float d2f(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7ffu) - (1023 - 127);  // binary32 exponent field
    if ((unsigned)(e - 1) >= 254u) {
        if (((hi << 1) | lo) == 0u) return __uint_as_float(hi);  // ±0
        return d2f_hw(x);
    }
    const unsigned sig = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 significand bits
    const unsigned rest = lo & 0x1fffffffu;                    // the 29 bits rounded off
    unsigned r = (hi & 0x80000000u) | ((unsigned)e << 23) | sig;
    r += (rest > 0x10000000u || (rest == 0x10000000u && (sig & 1u))) ? 1u : 0u;
    return __uint_as_float(r);
}
__device__ __forceinline__ double f2d(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) {
        if ((u << 1) == 0u) return __hiloint2double((int)u, 0);  // ±0
        return f2d_hw(f);
    }
    const unsigned hi = (u & 0x80000000u) | ((e + (1023 - 127)) << 20) | ((u & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
}

// 1/x for x > 0 in the normal FP32 range: an FP32 reciprocal refined by two
// Newton–Raphson steps y ← y + y(1 - x·y) in FP64 (quadratic convergence:
// 2^-23 → 2^-46 → below FP64 rounding), four FP64 operations instead of an
// FP64 division.  The result is within 2 ulp of the correctly rounded 1/x
// (checked against it by dem_selftest_conversions).
__device__ __forceinline__ double rcp_nr(double x) {
    double y = f2d(__frcp_rn(d2f(x)));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

// x·0.5 exactly, without the FP64 pipe: a normal x whose exponent field is at
// least 2 loses one from it, a zero is returned as it is; subnormal,
// smallest-normal, infinite and NaN inputs take the FP64 multiply (out of
// line).  Bit-identical to x * 0.5 (checked by dem_selftest_conversions).
static __device__ __noinline__ double half_hw(double x) { return x * 0.5; }
__device__ __forceinline__ double half_exact(double x) {
    const long long b = __double_as_longlong(x);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    if (e - 2u < 0x7fdu) return __longlong_as_double(b - (1ll << 52));  // e in [2, 0x7fe]
    if ((b & 0x7fffffffffffffffll) == 0) return x;
    return half_hw(x);
}

// Bit tests on the IEEE 754 binary64 layout (integer pipe): v is not -0; v
// is finite and not -0; a·b cannot overflow (for positive finite a and b:
// the sum of their exponent fields leaves the product's exponent below the
// largest one).
__device__ __forceinline__ bool not_negzero(double v) {
    return __double_as_longlong(v) != (long long)0x8000000000000000ull;
}
__device__ __forceinline__ bool finite_not_negzero(double v) {
    const long long b = __double_as_longlong(v);
    return b != (long long)0x8000000000000000ull && ((b >> 52) & 0x7ff) != 0x7ff;
}
// a != 0 (either sign; NaN counts as nonzero), and a < b for a that is +0,
// positive or NaN and a positive b, on the integer pipe: for binary64 values
// with a clear sign bit the IEEE order is the order of their bit patterns,
// and a NaN of either sign compares as an unsigned pattern above every
// finite positive b, so it compares false as in IEEE.
__device__ __forceinline__ bool nonzero_bits(double a) {
    return (__double_as_longlong(a) & 0x7fffffffffffffffll) != 0;
}
__device__ __forceinline__ bool less_nonneg(double a, double b) {
    return (unsigned long long)__double_as_longlong(a) <
           (unsigned long long)__double_as_longlong(b);
}
__device__ __forceinline__ bool product_finite(double a, double b) {
    const int ea = (int)((__double_as_longlong(a) >> 52) & 0x7ff);
    const int eb = (int)((__double_as_longlong(b) >> 52) & 0x7ff);
    return ea != 0x7ff && eb != 0x7ff && ea + eb <= 0x7fd + 1023;
}

// ---- Morton / bucket ---------------------------------------------------------
// Morton.jl `cartesian3morton` for 1-based cells (x in bit 0): the interleave of
// (ijk - 1) plus one.  Each coordinate keeps its low 10 bits.  The spreading
// uses the usual shift-and-mask bit interleave.
__device__ __forceinline__ uint32_t spread10(uint32_t x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}
__device__ __forceinline__ uint32_t morton1(int x, int y, int z) {
    return (spread10((uint32_t)(x - 1)) | (spread10((uint32_t)(y - 1)) << 1) |
            (spread10((uint32_t)(z - 1)) << 2)) +
           1u;
}
// Search bucket of a cell: the scene's table range [t0, t0 + H) indexed by
// cartesian3morton % H.  For a single-scene handle t0 = 0 and H is the
// reference's table size, so this is hashcode(ijk) - 1 (src/utils.jl:2).
__device__ __forceinline__ uint32_t bucket_of(int x, int y, int z, const SceneParams& S) {
    const uint32_t m = morton1(x, y, z);
    return S.t0 + (S.Hmask ? (m & S.Hmask) : (m % S.H));
}
// The reference's 0-based bucket, hashcode(ijk) - 1 with its own table size.
__device__ __forceinline__ uint32_t ref_bucket_of(int x, int y, int z, const SceneParams& S) {
    const uint32_t m = morton1(x, y, z);
    return S.Href_mask ? (m & S.Href_mask) : (m % S.Href);
}
// The 8 octant buckets of `neighbors` (src/utils.jl:4-16), in its order.
__device__ __forceinline__ void buckets8(int4 ci, const SceneParams& S, uint32_t B[8]) {
    const int dx = (ci.w & 1) ? 1 : -1, dy = (ci.w & 2) ? 1 : -1, dz = (ci.w & 4) ? 1 : -1;
    B[0] = bucket_of(ci.x, ci.y, ci.z, S);
    B[1] = bucket_of(ci.x + dx, ci.y, ci.z, S);
    B[2] = bucket_of(ci.x, ci.y + dy, ci.z, S);
    B[3] = bucket_of(ci.x, ci.y, ci.z + dz, S);
    B[4] = bucket_of(ci.x + dx, ci.y + dy, ci.z, S);
    B[5] = bucket_of(ci.x + dx, ci.y, ci.z + dz, S);
    B[6] = bucket_of(ci.x, ci.y + dy, ci.z + dz, S);
    B[7] = bucket_of(ci.x + dx, ci.y + dy, ci.z + dz, S);
}

// ---- small vector helpers (contractible; used by the force models) ----------
template <typename T>
struct Vec3 {
    T x, y, z;
};
template <typename T>
__device__ __forceinline__ Vec3<T> cross3(Vec3<T> a, Vec3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Julia min / max propagate NaN (fmin / fmax do not).
__device__ __forceinline__ double jl_min(double a, double b) {
    return (isnan(a) || isnan(b)) ? CUDART_NAN : (b < a ? b : a);
}
__device__ __forceinline__ double jl_max(double a, double b) {
    return (isnan(a) || isnan(b)) ? CUDART_NAN : (b > a ? b : a);
}
__device__ __forceinline__ double jl_sign(double x) { return x < 0.0 ? -1.0 : (x > 0.0 ? 1.0 : x); }

__device__ __forceinline__ void raise_error(DevCounters* c, int bit) { atomicOr(&c->error, bit); }

}  // namespace dem

// Programmatic dependent launch: a kernel launched with the programmatic
// stream serialization attribute may be scheduled while its predecessor in
// the stream is still running.  It first waits here for that grid to complete
// (its memory operations visible).  With `early`, it then lets its own
// successor be scheduled (once every block has passed this point); otherwise
// the successor is scheduled as this grid's blocks exit.  For an ordinary
// launch both instructions return at once.
__device__ __forceinline__ void dep_begin(bool early = false) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (early) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
