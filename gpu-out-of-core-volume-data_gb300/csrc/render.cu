// dvr_march: the out-of-core DVR / MIP ray caster.
//
// Per-ray method of RayCastDVRImpl / RayCastMOPImpl
// (Applications/DVR-ray-caster/src/RayCasters.cu:35-349): eye ray from the
// 3x4 camera matrix, slab test against the bounding box, front-to-back march
// with a per-sample LOD from the projected pixel footprint (compute_LOD,
// RayCasters.cu:551-567), page-directory walk and brick sampling through the
// cache (K_CacheManager::get_normalized, K_CacheManager.hpp:265-361;
// K_CacheDevice::compute_element_position, K_CacheDevice.hpp:314-336),
// transfer function, opacity correction 1 - (1 - a)^(LODStep / tstep),
// premultiplied compositing, early termination, progressive resume through the
// t / colour-state buffers, truncating RGBA8 pack (RayCasters.cu:528-536).
//
// This translation unit is compiled with -fmad=false: every float expression
// below is a sequence of IEEE-rounded operations in source order, so the host
// oracle evaluates the same values.  Where the reference calls approximate
// device functions, this kernel uses exactly-rounded ones:
//   normalize: v * (1 / sqrtf(v.v))           (reference: rsqrtf)
//   powf:      gc_pow, series log2/exp2 below (reference: CUDA powf)
//   texture:   explicit loads and FP32 lerps  (reference: texture unit with
//                                              8-bit fractional weights)
//
// GB300 mapping: persistent warps pull 8x4-pixel tiles from a global queue
// (one queue across every view of a batch), so neighbouring rays of a warp
// walk the same bricks; each thread caches its last page-directory entry and
// stamps the usage word only when the entry changes; brick voxels are read
// through the read-only path from the slot-major HBM pool.
#include <algorithm>
#include <climits>
#include <type_traits>

#include "cache.cuh"
#include "gc_internal.h"

// The march below is compiled twice: here (namespace gc::exact, built with
// -fmad=false: the oracle's operation sequence) and by render_fast.cu with
// GC_RENDER_FAST defined (namespace gc::fast, built with FMA contraction, see
// the math helpers).  The host code at the end of this file is compiled once
// and launches either set (gc_render_precision_set).
#ifdef GC_RENDER_FAST
#define GC_MARCH_NS fast
#else
#define GC_MARCH_NS exact
#endif
// resident 256-thread blocks per SM the register allocation must allow
#ifndef GC_RENDER_MIN_BLOCKS
#define GC_RENDER_MIN_BLOCKS 1
#endif

namespace gc {
namespace GC_MARCH_NS {


struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float length(V3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ V3 normalize(V3 a) {
#ifdef GC_RENDER_FAST
    return a * rsqrtf(dot(a, a));  // as the reference's helper_math normalize
#else
    const float inv = 1.0f / sqrtf(dot(a, a));
    return a * inv;
#endif
}
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float clampf(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
// Fused multiply-add at the places the oracle uses fmaf (the unit is built
// with -fmad=false, so no other operation is contracted and every rounding is
// the oracle's).
__device__ __forceinline__ float fmad(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ V3 fma3(V3 a, float b, V3 c) { return v3(fmad(a.x, b, c.x), fmad(a.y, b, c.y), fmad(a.z, b, c.z)); }
__device__ __forceinline__ float saturate(float x) { return (x != x) ? 0.0f : fminf(fmaxf(x, 0.0f), 1.0f); }

// log2 for normal x > 0: x = m 2^e, m in [sqrt(1/2), sqrt(2)), then
// ln m = 2 atanh(s), s = (m - 1)/(m + 1), by its odd series to s^9.
__device__ __forceinline__ float gc_log2(float x) {
    const uint32_t bits = __float_as_uint(x);
    int e = static_cast<int>((bits >> 23) & 0xffu) - 126;
    float m = __uint_as_float((bits & 0x807fffffu) | (126u << 23));  // [0.5, 1)
    if (m < 0.70710678f) {
        m = m * 2.0f;
        e -= 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = fmad(s2, 0.11111111f, 0.14285715f);
    p = fmad(p, s2, 0.2f);
    p = fmad(p, s2, 0.33333334f);
    p = fmad(p, s2, 1.0f);
    const float ln = (2.0f * s) * p;
    return fmad(ln, 1.44269504f, static_cast<float>(e));
}
// exp2 for y <= 0: y = n + f, f in [-1/2, 1/2], e^(f ln 2) by Taylor to degree 7.
__device__ __forceinline__ float gc_exp2(float y) {
    if (y < -125.0f) return 0.0f;
    const float n = floorf(y + 0.5f);
    const float t = (y - n) * 0.69314718f;
    float p = fmad(t, 0.00019841270f, 0.0013888889f);
    p = fmad(p, t, 0.0083333333f);
    p = fmad(p, t, 0.041666668f);
    p = fmad(p, t, 0.16666667f);
    p = fmad(p, t, 0.5f);
    p = fmad(p, t, 1.0f);
    p = fmad(p, t, 1.0f);
    const float scale = __uint_as_float(static_cast<uint32_t>(static_cast<int>(n) + 127) << 23);
    return p * scale;
}
__device__ __forceinline__ float gc_pow(float x, float k) {
    if (!(x > 0.0f)) return 0.0f;
    if (x == 1.0f) return 1.0f;
#ifdef GC_RENDER_FAST
    return __powf(x, k);  // the hardware log2 / exp2 pair
#else
    return gc_exp2(k * gc_log2(x));
#endif
}

// Division by a constant: exactly rounded in the exact build, a multiply by
// the reciprocal in the fast one.
__device__ __forceinline__ float div_const(float x, float d) {
#ifdef GC_RENDER_FAST
    return x * (1.0f / d);
#else
    return x / d;
#endif
}

// Integer conversions without the conversion unit (its quarter-rate pipe and
// scoreboard latency sit on every step of the march); both are exact.
// floor(v) for 0 <= v < 2^23: v + 2^23 rounded toward -inf is 2^23 + floor(v),
// whose low mantissa bits are floor(v).
__device__ __forceinline__ uint32_t floor_u(float v) {
    return __float_as_uint(__fadd_rd(v, 8388608.0f)) - 0x4B000000u;
}
// floor(v) for -2^22 <= v < 2^22, as an integer and as a float.
__device__ __forceinline__ int floor_i(float v, float &fl) {
    const float t = __fadd_rd(v, 12582912.0f);  // 1.5 * 2^23 + floor(v)
    fl = t - 12582912.0f;
    return __float_as_int(t) - 0x4B400000;
}
// (float)u for u < 2^23.
__device__ __forceinline__ float u2f(uint32_t u) { return __uint_as_float(0x4B000000u | u) - 8388608.0f; }

__device__ __forceinline__ float4 tf_lookup(const float *__restrict__ tf, uint32_t w, float s) {
    // xb is clamped into floor_i's range first: outside [-1, w] both indices
    // clamp to the same table entry, so the value is unchanged (a NaN sample,
    // possible only from a float volume holding NaN, reads entry 0)
    const float xb = fminf(fmaxf(fmad(s, static_cast<float>(w), -0.5f), -2.0f), static_cast<float>(w) + 1.0f);
    float fl;
    int i0 = floor_i(xb, fl);
    const float a = xb - fl;
    int i1 = i0 + 1;
    const int hi = static_cast<int>(w) - 1;
    i0 = i0 < 0 ? 0 : (i0 > hi ? hi : i0);
    i1 = i1 < 0 ? 0 : (i1 > hi ? hi : i1);
    const float4 t0 = __ldg(reinterpret_cast<const float4 *>(tf) + i0);
    const float4 t1 = __ldg(reinterpret_cast<const float4 *>(tf) + i1);
    return make_float4(fmad(t1.x - t0.x, a, t0.x), fmad(t1.y - t0.y, a, t0.y), fmad(t1.z - t0.z, a, t0.z),
                       fmad(t1.w - t0.w, a, t0.w));
}

// 2D transfer function (two-channel volumes): a w x h table of RGBA, channel
// 0 along w and channel 1 along h, read with the 1D lookup's rule on each
// axis (bilinear, edge-clamped).
__device__ __forceinline__ float4 tf2d_lookup(const float *__restrict__ tf, uint32_t w, uint32_t h, float s0,
                                              float s1) {
    const float xb = fminf(fmaxf(fmad(s0, static_cast<float>(w), -0.5f), -2.0f), static_cast<float>(w) + 1.0f);
    const float yb = fminf(fmaxf(fmad(s1, static_cast<float>(h), -0.5f), -2.0f), static_cast<float>(h) + 1.0f);
    float flx, fly;
    int i0 = floor_i(xb, flx), j0 = floor_i(yb, fly);
    const float ax = xb - flx, ay = yb - fly;
    const int hx = static_cast<int>(w) - 1, hy = static_cast<int>(h) - 1;
    int i1 = i0 + 1, j1 = j0 + 1;
    i0 = i0 < 0 ? 0 : (i0 > hx ? hx : i0);
    i1 = i1 < 0 ? 0 : (i1 > hx ? hx : i1);
    j0 = j0 < 0 ? 0 : (j0 > hy ? hy : j0);
    j1 = j1 < 0 ? 0 : (j1 > hy ? hy : j1);
    const float4 *t = reinterpret_cast<const float4 *>(tf);
    const float4 t00 = __ldg(t + j0 * static_cast<int>(w) + i0), t10 = __ldg(t + j0 * static_cast<int>(w) + i1);
    const float4 t01 = __ldg(t + j1 * static_cast<int>(w) + i0), t11 = __ldg(t + j1 * static_cast<int>(w) + i1);
    const float4 r0 = make_float4(fmad(t10.x - t00.x, ax, t00.x), fmad(t10.y - t00.y, ax, t00.y),
                                  fmad(t10.z - t00.z, ax, t00.z), fmad(t10.w - t00.w, ax, t00.w));
    const float4 r1 = make_float4(fmad(t11.x - t01.x, ax, t01.x), fmad(t11.y - t01.y, ax, t01.y),
                                  fmad(t11.z - t01.z, ax, t01.z), fmad(t11.w - t01.w, ax, t01.w));
    return make_float4(fmad(r1.x - r0.x, ay, r0.x), fmad(r1.y - r0.y, ay, r0.y), fmad(r1.z - r0.z, ay, r0.z),
                       fmad(r1.w - r0.w, ay, r0.w));
}

template <typename T>
struct VoxelTraits;
template <>
struct VoxelTraits<uint8_t> {
    static constexpr float kSum8 = 2040.0f;
    static constexpr float kMax = 255.0f;
};
template <>
struct VoxelTraits<uint16_t> {
    static constexpr float kSum8 = 524280.0f;
    static constexpr float kMax = 65535.0f;
};
template <>
struct VoxelTraits<float> {
    static constexpr float kSum8 = 8.0f;
    static constexpr float kMax = 1.0f;
};

// Reference sampler: normalized linear read at the integer voxel corner e =
// (lx, ly, lz) of the slot = mean of voxels {e-1, e} per axis.
// With covering >= 1 both voxels lie in the brick; with covering 0 the lower
// one is clamped to the brick edge (the reference then reads the neighbouring
// slot of its texture).
// BS: the brick size when known at compile time (its row and slice strides
// become immediate load offsets), 0 for the run-time B.
template <typename T, uint32_t BS>
__device__ __forceinline__ float sample_corner(const T *__restrict__ b, uint32_t Brt, uint32_t lx, uint32_t ly,
                                               uint32_t lz) {
    const uint32_t B = BS ? BS : Brt;
    lx = lx > 0 ? lx : 1u;
    ly = ly > 0 ? ly : 1u;
    lz = lz > 0 ? lz : 1u;
    const uint32_t i0 = ((lz - 1) * B + (ly - 1)) * B + (lx - 1);
    // the four x pairs of the 2x2x2 block: rows y, y+1 of slices z, z+1
    const T *p0 = b + i0;
    const T *p1 = p0 + B, *p2 = p0 + B * B;
    const T *p3 = p2 + B;
    if constexpr (sizeof(T) < 4) {
        const uint32_t s = static_cast<uint32_t>(__ldg(p0)) + __ldg(p0 + 1) + __ldg(p1) + __ldg(p1 + 1) + __ldg(p2) +
                           __ldg(p2 + 1) + __ldg(p3) + __ldg(p3 + 1);
        return div_const(u2f(s), VoxelTraits<T>::kSum8);
    } else {
        const float s = ((__ldg(p0) + __ldg(p0 + 1)) + (__ldg(p1) + __ldg(p1 + 1))) +
                        ((__ldg(p2) + __ldg(p2 + 1)) + (__ldg(p3) + __ldg(p3 + 1)));
        return s * 0.125f;
    }
}

// x mod (B - 2c) by a multiply-high: with m = ceil(2^32 / d), the high word of
// x m is floor(x / d) for every x < 2^25 and 2 <= d <= 128 (voxel coordinates
// are below 2^23, checked at cache creation; m = 0 falls back to %).
__device__ __forceinline__ uint32_t mod_beff(uint32_t x, uint32_t d, uint32_t m) {
    if (m == 0) return x % d;
    return x - __umulhi(x, m) * d;
}

// Trilinear sampler at the fractional position f (voxels of the level); the
// pair (i0, i0 + 1) is clamped to the brick (only reachable with covering 0).
__device__ __forceinline__ void tri_axis(float f, uint32_t c, uint32_t beff, uint32_t magic, uint32_t B,
                                         uint32_t &i0, float &w) {
    const uint32_t m = floor_u(f);
    const float fr = f - u2f(m);
    const uint32_t l = c + mod_beff(m, beff, magic);
    if (fr >= 0.5f) {
        i0 = l;
        w = fr - 0.5f;
    } else {
        i0 = l > 0 ? l - 1 : 0u;
        w = l > 0 ? fr + 0.5f : 0.0f;
    }
    if (i0 + 1 >= B) {
        i0 = B - 2;
        w = 1.0f;
    }
}
template <typename T>
__device__ __forceinline__ float ldv(const T *__restrict__ b, uint32_t i) {
    return static_cast<float>(__ldg(b + i));
}
template <typename T, uint32_t BS>
__device__ __forceinline__ float sample_trilinear(const T *__restrict__ b, uint32_t Brt, uint32_t x0, uint32_t y0,
                                                  uint32_t z0, float wx, float wy, float wz) {
    const uint32_t B = BS ? BS : Brt;
    const uint32_t i = (z0 * B + y0) * B + x0, BB = B * B;
    const float c00 = fmad(ldv(b, i + 1) - ldv(b, i), wx, ldv(b, i));
    const float c10 = fmad(ldv(b, i + B + 1) - ldv(b, i + B), wx, ldv(b, i + B));
    const float c01 = fmad(ldv(b, i + BB + 1) - ldv(b, i + BB), wx, ldv(b, i + BB));
    const float c11 = fmad(ldv(b, i + BB + B + 1) - ldv(b, i + BB + B), wx, ldv(b, i + BB + B));
    const float c0 = fmad(c10 - c00, wy, c00);
    const float c1 = fmad(c11 - c01, wy, c01);
    return div_const(fmad(c1 - c0, wz, c0), VoxelTraits<T>::kMax);
}

enum Status { kMapped = 0, kUnmapped = 1, kEmpty = 2, kInvisible = 3, kCoarser = 4 };

// Per-thread page-walk state (K_CacheManager::_previousCoords / _previousEntries).
struct Walk {
    uint32_t pidx;   // page-directory index of the entry last read (one word per (x, y, z))
    uint32_t flag;   // flag of the entry last read (0 unmapped, 1 mapped, 2 empty, 3 in flight)
    const uint8_t *base;  // pool slot of a mapped entry (decoded when the entry is read)
    bool invisible;  // the mapped brick holds no value the view's transfer function shows
    // two-level directory: the directory word last read and its value (a ray
    // crosses several bricks of one table block in a row)
    uint32_t pword, ptop;
};

// Voxel sampling of one brick (slot base address), typed by T; MixedVoxel
// picks the type from the view's voxel width (caches whose volumes differ);
// TwoU8 samples two interleaved 8-bit channels (NumberChannels 2) into a
// float2 for the 2D transfer function.
struct MixedVoxel {};
struct TwoU8 {};
template <typename T>
struct SampleOf {
    using type = float;
};
template <>
struct SampleOf<TwoU8> {
    using type = float2;
};
__device__ __forceinline__ float first_channel(float s) { return s; }
__device__ __forceinline__ float first_channel(float2 s) { return s.x; }
__device__ __forceinline__ float4 classify(const float *tf, uint32_t tfw, const ViewParams &, float s) {
    return tf_lookup(tf, tfw, s);
}
__device__ __forceinline__ float4 classify(const float *tf, uint32_t tfw, const ViewParams &vp, float2 s) {
    return tf2d_lookup(tf, tfw, vp.tfh, s.x, s.y);
}

template <typename T, uint32_t BS>
__device__ __forceinline__ float sample_slot(const uint8_t *base, uint32_t eb, const CacheView &cv,
                                             uint32_t sampler, float fx, float fy, float fz) {
    if constexpr (std::is_same<T, MixedVoxel>::value) {
        if (eb == 1) return sample_slot<uint8_t, BS>(base, eb, cv, sampler, fx, fy, fz);
        if (eb == 2) return sample_slot<uint16_t, BS>(base, eb, cv, sampler, fx, fy, fz);
        return sample_slot<float, BS>(base, eb, cv, sampler, fx, fy, fz);
    } else {
        const T *b = reinterpret_cast<const T *>(base);
        const uint32_t B = BS ? BS : cv.B;
        if (sampler == GC_SAMPLER_REFERENCE) {
            const uint32_t lx = cv.c + mod_beff(floor_u(fx), cv.Beff, cv.beff_magic);
            const uint32_t ly = cv.c + mod_beff(floor_u(fy), cv.Beff, cv.beff_magic);
            const uint32_t lz = cv.c + mod_beff(floor_u(fz), cv.Beff, cv.beff_magic);
            return sample_corner<T, BS>(b, B, lx, ly, lz);
        }
        uint32_t x0, y0, z0;
        float wx, wy, wz;
        tri_axis(fx, cv.c, cv.Beff, cv.beff_magic, B, x0, wx);
        tri_axis(fy, cv.c, cv.Beff, cv.beff_magic, B, y0, wy);
        tri_axis(fz, cv.c, cv.Beff, cv.beff_magic, B, z0, wz);
        return sample_trilinear<T, BS>(b, B, x0, y0, z0, wx, wy, wz);
    }
}
// Two interleaved u8 channels: each channel sampled with the one-channel
// rule (corner mean of 8 voxels, or trilinear), voxel i channel k at byte 2i+k.
template <uint32_t BS>
__device__ __forceinline__ float2 sample_slot_two(const uint8_t *__restrict__ b, const CacheView &cv,
                                                  uint32_t sampler, float fx, float fy, float fz) {
    const uint32_t B = BS ? BS : cv.B, BB = B * B;
    if (sampler == GC_SAMPLER_REFERENCE) {
        uint32_t lx = cv.c + mod_beff(floor_u(fx), cv.Beff, cv.beff_magic);
        uint32_t ly = cv.c + mod_beff(floor_u(fy), cv.Beff, cv.beff_magic);
        uint32_t lz = cv.c + mod_beff(floor_u(fz), cv.Beff, cv.beff_magic);
        lx = lx > 0 ? lx : 1u;
        ly = ly > 0 ? ly : 1u;
        lz = lz > 0 ? lz : 1u;
        const uint32_t i0 = ((lz - 1) * B + (ly - 1)) * B + (lx - 1);
        const uint32_t id[8] = {i0, i0 + 1, i0 + B, i0 + B + 1, i0 + BB, i0 + BB + 1, i0 + BB + B, i0 + BB + B + 1};
        uint32_t s0 = 0, s1 = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uchar2 v = __ldg(reinterpret_cast<const uchar2 *>(b) + id[k]);
            s0 += v.x;
            s1 += v.y;
        }
        return make_float2(div_const(u2f(s0), 2040.0f), div_const(u2f(s1), 2040.0f));
    }
    uint32_t x0, y0, z0;
    float wx, wy, wz;
    tri_axis(fx, cv.c, cv.Beff, cv.beff_magic, B, x0, wx);
    tri_axis(fy, cv.c, cv.Beff, cv.beff_magic, B, y0, wy);
    tri_axis(fz, cv.c, cv.Beff, cv.beff_magic, B, z0, wz);
    const uint32_t i = (z0 * B + y0) * B + x0;
    float out[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        auto lv = [&](uint32_t j) { return static_cast<float>(__ldg(b + 2 * j + k)); };
        const float c00 = fmad(lv(i + 1) - lv(i), wx, lv(i));
        const float c10 = fmad(lv(i + B + 1) - lv(i + B), wx, lv(i + B));
        const float c01 = fmad(lv(i + BB + 1) - lv(i + BB), wx, lv(i + BB));
        const float c11 = fmad(lv(i + BB + B + 1) - lv(i + BB + B), wx, lv(i + BB + B));
        const float c0 = fmad(c10 - c00, wy, c00);
        const float c1 = fmad(c11 - c01, wy, c01);
        out[k] = div_const(fmad(c1 - c0, wz, c0), 255.0f);
    }
    return make_float2(out[0], out[1]);
}
template <typename T, uint32_t BS>
__device__ __forceinline__ typename SampleOf<T>::type sample_any(const uint8_t *base, uint32_t eb, const CacheView &cv,
                                                                 uint32_t sampler, float fx, float fy, float fz) {
    if constexpr (std::is_same<T, TwoU8>::value)
        return sample_slot_two<BS>(base, cv, sampler, fx, fy, fz);
    else
        return sample_slot<T, BS>(base, eb, cv, sampler, fx, fy, fz);
}

// The sample position of a ray position in normalized volume coordinates
// (RayCasters.cu:128-133): scaled into [0, 1], z flipped, clamped to [0, 0.99].
__device__ __forceinline__ V3 norm_pos(V3 pos) {
    V3 tp = fma3(pos, 0.495f, v3(0.495f, 0.495f, 0.495f));
    tp.z = 1.0f - tp.z;
    return v3(clampf(tp.x, 0.f, 0.99f), clampf(tp.y, 0.f, 0.99f), clampf(tp.z, 0.f, 0.99f));
}

// Page-directory index of the normalized position np at cache level lvl
// (K_CacheManager::get_normalized's walk, K_CacheManager.hpp:265-300); p
// receives the level position np * initial / real.
__device__ __forceinline__ uint32_t entry_index(const CacheView &cv, const LevelTables &lt, uint32_t lvl, V3 np,
                                                V3 &p, uint3 &q) {
    p = v3(np.x * lt.ior[lvl][0], np.y * lt.ior[lvl][1], np.z * lt.ior[lvl][2]);
    q = make_uint3(floor_u(p.x * lt.nbf[lvl][0]), floor_u(p.y * lt.nbf[lvl][1]), floor_u(p.z * lt.nbf[lvl][2]));
    // the page directory has fewer than 2^32 - 1 entries (checked at creation)
    return lt.off[lvl] + q.x + q.y * cv.mx + q.z * cv.mxy;
}

// The page-directory entry of brick q (x inside the level) of cache level
// lvl, flat index idx.  Two-level directory: the directory word, then the
// entry in its table block (the table slot's usage word stamped, as the
// reference's table-cache read does, K_CacheDevice.hpp:314-336); a word
// without a block reads as an unmapped entry.  TL: the kernels compiled for a
// two-level directory (the one-level kernels carry none of this).
template <bool TL>
__device__ __forceinline__ uint4 load_entry(const CacheView &cv, const LevelTables &lt, uint32_t lvl, uint32_t idx,
                                            uint3 q, Walk *w) {
    if constexpr (!TL) return __ldg(cv.mrpd + idx);
    const uint32_t word = pt_word(cv.pt, lt, lvl, q.x, q.y, q.z);
    uint32_t t;
    if (w && word == w->pword) {
        t = w->ptop;  // same block as the entry before: read and stamped then
    } else {
        t = __ldg(cv.pt.top + word);
        if (w) {
            w->pword = word;
            w->ptop = t;
        }
        if (t & 1u) {
            // many rays share a table block: the stamp is stored only where the
            // word does not hold it yet (a stale read only repeats the store)
            uint32_t *u = cv.pt.usage + (t >> 1);
            if (*u != cv.ts) *u = cv.ts;
        }
    }
    if (!(t & 1u)) return make_uint4(0u, 0u, 0u, 0u);
    return __ldg(cv.pt.table + pt_entry(cv.pt, t >> 1, pt_local(cv.pt, q.x, q.y, q.z)));
}

// Voxel sample of the resident brick at `base` (its pool slot) at level position p.
template <typename T, uint32_t BS>
__device__ __forceinline__ typename SampleOf<T>::type sample_entry(const CacheView &cv, const LevelTables &lt,
                                                                   uint32_t sampler, const ViewParams &vp,
                                                                   uint32_t lvl, const uint8_t *base, V3 p) {
    const float fx = p.x * lt.vvoxf[lvl][0];
    const float fy = p.y * lt.vvoxf[lvl][1];
    const float fz = p.z * lt.vvoxf[lvl][2];
    return sample_any<T, BS>(base, vp.eb, cv, sampler, fx, fy, fz);
}

// Page walk + sample at the normalized position np of cache level lvl (the
// view's level base + its LOD): K_CacheManager::get_normalized
// (K_CacheManager.hpp:265-361).
template <typename T, uint32_t BS, bool TL>
__device__ __forceinline__ int fetch(const CacheView &cv, const LevelTables &lt, uint32_t sampler,
                                     const ViewParams &vp, uint32_t lvl, uint32_t lvl_end, V3 np, Walk &w,
                                     typename SampleOf<T>::type &sample) {
    // read where used (rare paths): the view's voxel width (mixed pools), its
    // visible bins (a newly entered brick) and its fallback flag (a missing one)
    V3 p;
    uint3 q;
    const uint32_t idx = entry_index(cv, lt, lvl, np, p, q);
    if (idx != w.pidx) {
        // A new entry: the entry and its value bins are read together (one
        // memory round trip); the usage stamp of a mapped brick is a plain
        // store (idempotent, like the reference's per-sample stamp).
        const uint4 e = load_entry<TL>(cv, lt, lvl, idx, q, &w);
        const unsigned long long bins = __ldg(cv.entry_bins + idx);
        w.pidx = idx;
        w.flag = e.w;
        w.invisible = (bins & vp.visible) == 0ull && (e.w == 1u || (e.w == 0u && cv.bins_user));
        if (e.w == 1u) {
            const uint32_t B = cv.B;
            const uint32_t slot = cv.b_shift < 32u ? (e.x >> cv.b_shift) + (e.y >> cv.b_shift) * cv.sx +
                                                         (e.z >> cv.b_shift) * cv.sx * cv.sy
                                                   : e.x / B + (e.y / B) * cv.sx + (e.z / B) * cv.sx * cv.sy;
            cv.usage[slot] = cv.ts;
            w.base = cv.pool + static_cast<uint64_t>(slot) * cv.slot_bytes;
        }
    }
    const uint32_t flag = w.flag;
    if (flag == 1u) {
        if (w.invisible) return kInvisible;  // no sample of this brick reaches the compositing threshold
        sample = sample_entry<T, BS>(cv, lt, sampler, vp, lvl, w.base, p);
        return kMapped;
    }
    if (flag == 3u) return kUnmapped;  // on its way (batched form): already requested
    if (flag == 0u) {
        // A missing brick whose value bins (given for every brick) are all
        // invisible: stepped through like a resident invisible brick, never
        // requested.
        if (w.invisible) return kInvisible;
        // raise_brick_request (K_CacheManager.hpp:364-396): same coordinates
        cv.req[idx] = cv.ts;
        // Coarser-level fallback (K_CacheManager::get, K_CacheManager.hpp:163-260):
        // the request stays on the asked level; the first mapped coarser level
        // of the volume is sampled instead, an empty one ends the lookup.
        for (uint32_t l2 = lvl + 1; vp.fallback != 0u && l2 < lvl_end; ++l2) {
            const float qx = np.x * lt.ior[l2][0], qy = np.y * lt.ior[l2][1], qz = np.z * lt.ior[l2][2];
            const uint3 q2 = make_uint3(static_cast<uint32_t>(qx * static_cast<float>(lt.nb[l2][0])),
                                        static_cast<uint32_t>(qy * static_cast<float>(lt.nb[l2][1])),
                                        static_cast<uint32_t>(qz * static_cast<float>(lt.nb[l2][2])));
            const uint4 e2 =
                load_entry<TL>(cv, lt, l2, lt.off[l2] + q2.x + q2.y * cv.mx + q2.z * cv.mxy, q2, nullptr);
            if (e2.w == 2u) return kEmpty;
            if (e2.w != 1u) continue;
            const uint32_t B = cv.B;
            const uint32_t slot = e2.x / B + (e2.y / B) * cv.sx + (e2.z / B) * cv.sx * cv.sy;
            cv.usage[slot] = cv.ts;
            sample = sample_any<T, BS>(cv.pool + static_cast<uint64_t>(slot) * cv.slot_bytes, vp.eb, cv, sampler,
                                   qx * static_cast<float>(lt.vvox[l2][0]), qy * static_cast<float>(lt.vvox[l2][1]),
                                   qz * static_cast<float>(lt.vvox[l2][2]));
            return kCoarser;
        }
        return kUnmapped;
    }
    return kEmpty;
}

// Per-ray state between samples.  The method is split into ray_setup /
// ray_step / ray_finish so that both schedulers below run the same code.
struct Ray {
    const ViewParams *vp;
    uint32_t i;
    V3 pos, dir, dirLeft, dirUp;
    float t, tfar, endX, endY, sL, sU, maxOp;
    float4 fc;
    uint32_t lod;
    // The view's per-sample parameters, read once per ray: the march stores
    // to global memory (usage and request stamps), so reads through the view
    // pointer would be repeated at every step.  step, afloor and kexp belong
    // to the current level of detail.
    float early, step, afloor, kexp;
    const float *tf;
    uint32_t tfw;
    uint32_t lvl, lvl_end;  // cache level of the current LOD; end of the view's levels
    uint32_t sampler;
    float t_lo;  // below this t the LOD test surely keeps the level (+inf at the coarsest)
    Walk w;
    bool unm, dvr;
    bool coarse;  // a coarser level stood in for a missing brick (fallback mode)
    uint32_t nsamp;  // samples taken (voxel reads of a resident brick)
};

// compute_LOD keeps the level while sL >= RN(endX * RN(t / tfar)) or
// sU >= RN(endY * RN(t / tfar)).  Each rounding grows a value by at most a
// factor (1 + 2^-24), so t <= sL * tfar / (endX * (1 + 2^-24)^2) already keeps
// it (likewise for Y; an axis with end 0 always does).  The bound below is
// that, computed in float (three more roundings) and shrunk by 2^-19, which
// covers all five; at or above it the exact test runs, so the level sequence
// is the reference's.
__device__ __forceinline__ float lod_keep_bound(float sL, float sU, float endX, float endY, float tfar, bool last) {
    if (last) return __int_as_float(0x7f800000);
    float bx = endX > 0.f ? sL / endX * tfar : __int_as_float(0x7f800000);
    float by = endY > 0.f ? sU / endY * tfar : __int_as_float(0x7f800000);
    return fmaxf(bx, by) * (1.0f - 1.0f / 524288.0f);
}

// Eye ray, box intersection and progressive resume.  Returns false when the
// ray has nothing to march (the pixel is then already written).
template <typename T>
__device__ __forceinline__ bool ray_setup(const LevelTables &lt, const ViewParams *vpp, uint32_t x, uint32_t y,
                                          Ray &r) {
    const ViewParams &vp = *vpp;
    const uint32_t W = vp.W, H = vp.H;
    // a batched pass skips a pixel whose ray finished in an earlier pass
    if (vp.mark_done && vp.tbuf[y * W + x] < 0.f) return false;
    uint32_t xN = x + 1;
    if (xN > W) xN = x - 1;
    uint32_t yN = y + 1;
    if (yN > H) yN = y - 1;
    const float fW = static_cast<float>(W), fH = static_cast<float>(H);
    const float u = ((static_cast<float>(x) + 0.5f) / fW) * 2.0f - 1.0f;
    const float uN = ((static_cast<float>(xN) + 0.5f) / fW) * 2.0f - 1.0f;
    const float v = ((static_cast<float>(y) + 0.5f) / fH) * 2.0f - 1.0f;
    const float vN = ((static_cast<float>(yN) + 0.5f) / fH) * 2.0f - 1.0f;
    const float *m = vp.m;
    // mul(M, float4(0,0,0,1)) and mul(M, float3) (RayCasters.cu:484-503)
    const V3 origin = v3(0.0f * m[0] + 0.0f * m[1] + 0.0f * m[2] + 1.0f * m[3],
                         0.0f * m[4] + 0.0f * m[5] + 0.0f * m[6] + 1.0f * m[7],
                         0.0f * m[8] + 0.0f * m[9] + 0.0f * m[10] + 1.0f * m[11]);
    const V3 r0 = v3(m[0], m[1], m[2]), r1 = v3(m[4], m[5], m[6]), r2 = v3(m[8], m[9], m[10]);
    auto rot = [&](V3 d) { return v3(dot(d, r0), dot(d, r1), dot(d, r2)); };
    const V3 dir = rot(normalize(v3(u, v, -vp.focal)));
    const V3 dirXN = rot(normalize(v3(uN, v, -vp.focal)));
    const V3 dirYN = rot(normalize(v3(u, vN, -vp.focal)));
    const V3 dirLeft = normalize(cross(dir, dirYN));
    const V3 dirUp = normalize(cross(dir, dirXN));

    // intersectBox (RayCasters.cu:506-525)
    const V3 invR = v3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    const V3 tbot = invR * (v3(vp.bmin[0], vp.bmin[1], vp.bmin[2]) - origin);
    const V3 ttop = invR * (v3(vp.bmax[0], vp.bmax[1], vp.bmax[2]) - origin);
    const V3 tmin = v3(fminf(ttop.x, tbot.x), fminf(ttop.y, tbot.y), fminf(ttop.z, tbot.z));
    const V3 tmax = v3(fmaxf(ttop.x, tbot.x), fmaxf(ttop.y, tbot.y), fmaxf(ttop.z, tbot.z));
    float tnear = fmaxf(fmaxf(tmin.x, tmin.y), fmaxf(tmin.x, tmin.z));
    const float tfar = fminf(fminf(tmax.x, tmax.y), fminf(tmax.x, tmax.z));
    const bool hit = tfar > tnear;

    const uint32_t i = y * W + x;
    tnear = fmaxf(tnear, vp.tbuf[i]);
    const float4 *state = reinterpret_cast<const float4 *>(vp.state);
    r.vp = vpp;
    r.i = i;
    r.dvr = vp.mode == GC_MODE_DVR;
    r.unm = false;
    r.coarse = false;
    r.nsamp = 0;
    r.fc = r.dvr ? state[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    if (!hit) {
        r.fc.x = 0.f;
        r.fc.y = 0.f;
        r.fc.z = 0.f;
        const float4 fc = r.fc;
        const uint32_t R = static_cast<uint32_t>(saturate(fc.x) * 255.0f);
        const uint32_t G = static_cast<uint32_t>(saturate(fc.y) * 255.0f);
        const uint32_t Bc = static_cast<uint32_t>(saturate(fc.z) * 255.0f);
        const uint32_t A = static_cast<uint32_t>(saturate(fc.w) * 255.0f);
        vp.rgba[i] = (A << 24) | (Bc << 16) | (G << 8) | R;
        if (vp.mark_done) vp.tbuf[i] = -1.0f;
        return false;
    }
    if (tnear < 0.f) tnear = 0.f;
    r.t = tnear;
    r.tfar = tfar;
    r.pos = origin + dir * tnear;
    r.dir = dir;
    r.dirLeft = dirLeft;
    r.dirUp = dirUp;
    r.endX = fabsf(dot(dir - dirXN, dirLeft) * tfar);
    r.endY = fabsf(dot(dir - dirYN, dirUp) * tfar);
    r.lod = 0;
    r.sL = 0.f;  // spacings of level lod + 1
    r.sU = 0.f;
    if (vp.nlevels > 1) {
        const V3 n1 = v3(vp.inv_size[1][0], vp.inv_size[1][1], vp.inv_size[1][2]);
        r.sL = length(dirLeft * n1);
        r.sU = length(dirUp * n1);
    }
    r.early = vp.early;
    r.step = vp.step[0];
    r.afloor = vp.alpha_floor[0];
    r.kexp = vp.kexp[0];
    r.tf = vp.tf;
    r.tfw = vp.tfw;
    r.lvl = vp.level_base;
    r.lvl_end = vp.level_base + vp.nlevels;
    r.sampler = vp.sampler;
    r.t_lo = lod_keep_bound(r.sL, r.sU, r.endX, r.endY, r.tfar, r.lvl + 1 >= r.lvl_end);
    r.w.pidx = UINT_MAX;
    r.w.pword = UINT_MAX;
    r.w.flag = 0;
    r.w.base = nullptr;
    r.w.invisible = false;
    r.maxOp = r.dvr ? 0.f : vp.state[4 * i];
    return true;
}

// The ray passes the march loop's first test: it takes at least one sample
// (a ray whose box lies behind the camera, or a finished ray, does not).
__device__ __forceinline__ bool ray_enters(const Ray &r) {
    return (!r.dvr || r.fc.w < r.early) && r.t < r.tfar;
}

// Front-to-back compositing of one classified, opacity-corrected sample
// (RayCasters.cu:163-176).  Opacity correction 1 - (1 - a)^k is applied by
// the caller; for a <= alpha_floor[lod] the corrected opacity is below
// 1.05 k a <= 0.0009, under the compositing threshold, so the callers skip
// it with the same result.
__device__ __forceinline__ void composite(Ray &r, float4 col) {
    if (col.w > 0.001f) {
        col.x *= col.w;
        col.y *= col.w;
        col.z *= col.w;
        const float rr = 1.0f - r.fc.w;
        r.fc.x = fmad(col.x, rr, r.fc.x);
        r.fc.y = fmad(col.y, rr, r.fc.y);
        r.fc.z = fmad(col.z, rr, r.fc.z);
        r.fc.w = fmad(col.w, rr, r.fc.w);
    }
}

// One iteration of the march loop (RayCasters.cu:122-188).  Returns false
// when the loop ends.
template <typename T, uint32_t BS, bool TL>
__device__ __forceinline__ bool ray_step(const CacheView &cv, const LevelTables &lt, Ray &r) {
    const ViewParams &vp = *r.vp;
    if (!((!r.dvr || r.fc.w < r.early) && r.t < r.tfar)) return false;
    const V3 np = norm_pos(r.pos);
    // compute_LOD: the level only grows along a ray because the pixel
    // footprint grows with t, so the scan resumes at the current level (and
    // the footprint is not needed once the ray is at the coarsest level).
    if (r.t >= r.t_lo) {  // near or past the level change: the exact test
        const float alpha = r.t / r.tfar;
        const float pX = r.endX * alpha;
        const float pY = r.endY * alpha;
        if (!(r.sL >= pX || r.sU >= pY)) {
            do {
                ++r.lod;
                ++r.lvl;
                if (r.lvl + 1 < r.lvl_end) {
                    const V3 nn =
                        v3(vp.inv_size[r.lod + 1][0], vp.inv_size[r.lod + 1][1], vp.inv_size[r.lod + 1][2]);
                    r.sL = length(r.dirLeft * nn);
                    r.sU = length(r.dirUp * nn);
                }
            } while (r.lvl + 1 < r.lvl_end && !(r.sL >= pX || r.sU >= pY));
            r.step = vp.step[r.lod];
            r.afloor = vp.alpha_floor[r.lod];
            r.kexp = vp.kexp[r.lod];
            r.t_lo = lod_keep_bound(r.sL, r.sU, r.endX, r.endY, r.tfar, r.lvl + 1 >= r.lvl_end);
        }
    }
    typename SampleOf<T>::type sample{};
    const int st = fetch<T, BS, TL>(cv, lt, r.sampler, vp, r.lvl, r.lvl_end, np, r.w, sample);
    if (st == kCoarser) r.coarse = true;  // sampled below; the image is a preview
    if (st == kMapped || st == kCoarser) ++r.nsamp;
    if (st == kInvisible) {  // the step of a sample whose opacity stays below 0.001
        r.t += r.step;
        r.pos = fma3(r.dir, r.step, r.pos);
        return true;
    }
    if (st != kMapped && st != kCoarser) {
        if (st == kUnmapped) {
            vp.tbuf[r.i] = r.t;
            if (r.dvr)
                reinterpret_cast<float4 *>(vp.state)[r.i] = r.fc;
            else
                vp.state[4 * r.i] = r.maxOp;
            r.unm = true;
            return false;
        }
        r.t += vp.tstep;
        if (r.t > r.tfar) return false;
        r.pos = fma3(r.dir, vp.tstep, r.pos);
        return true;
    }
    if (r.dvr) {
        float4 col = classify(r.tf, r.tfw, vp, sample);
        col.w = col.w > r.afloor ? 1.0f - gc_pow(1.0f - col.w, r.kexp) : 0.0f;
        composite(r, col);
    } else {
        r.maxOp = fmaxf(r.maxOp, first_channel(sample));
    }
    r.t += r.step;
    r.pos = fma3(r.dir, r.step, r.pos);
    return true;
}

// Progressive state, MIP classification and the truncating RGBA8 pack
// (RayCasters.cu:189-197, 528-536).  Returns true when the ray stopped at an
// unmapped brick.
__device__ __forceinline__ bool ray_finish(Ray &r) {
    const ViewParams &vp = *r.vp;
    if (!r.unm) {
        if (vp.mark_done) {
            vp.tbuf[r.i] = -1.0f - r.t;  // t >= 0: the mark is < 0; the state is not read again
        } else {
            vp.tbuf[r.i] = r.t;
            if (r.dvr)
                reinterpret_cast<float4 *>(vp.state)[r.i] = r.fc;
            else
                vp.state[4 * r.i] = r.maxOp;
        }
    }
    float4 fc = r.fc;
    if (!r.dvr) fc = tf_lookup(vp.tf, vp.tfw, r.maxOp);
    const uint32_t R = static_cast<uint32_t>(saturate(fc.x) * 255.0f);
    const uint32_t G = static_cast<uint32_t>(saturate(fc.y) * 255.0f);
    const uint32_t Bc = static_cast<uint32_t>(saturate(fc.z) * 255.0f);
    const uint32_t A = static_cast<uint32_t>(saturate(fc.w) * 255.0f);
    vp.rgba[r.i] = (A << 24) | (Bc << 16) | (G << 8) | R;
    return r.unm;
}

// The view and tile of queue index t: first the screen-rectangle tiles of
// every view (rows of the rectangle), then the other tiles of every view in
// raster order.
__device__ __forceinline__ const ViewParams *tile_of(const ViewParams *__restrict__ views, uint32_t nviews,
                                                     uint32_t t, uint32_t &tx, uint32_t &ty) {
    const bool in_rect = t < views[0].rect_total;
    uint32_t lo = 0, hi = nviews - 1;
    while (lo < hi) {  // the last view whose range starts at or before t
        const uint32_t mid = (lo + hi + 1) >> 1;
        if ((in_rect ? views[mid].rect_begin : views[mid].out_begin) <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    const ViewParams *vp = views + lo;
    if (in_rect) {  // rows from the middle of the rectangle outwards (the longest rays first)
        const uint32_t local = t - vp->rect_begin, k = local / vp->rw;
        const uint32_t mid = (vp->rh - 1) / 2, half = (k + 1) / 2;
        uint32_t row = (k & 1u) ? mid + half : mid - half;
        if (half > mid) row = k;             // above ran out: the rest, in order, lie below
        else if (row >= vp->rh) row = mid - half;  // below ran out (even heights): keep above
        ty = vp->ry0 + row;
        tx = vp->rx0 + (local - k * vp->rw);
        return vp;
    }
    uint32_t u = t - vp->out_begin;
    const uint32_t ntx = vp->tiles_x, above = vp->ry0 * ntx;
    if (u < above) {
        ty = u / ntx;
        tx = u - ty * ntx;
        return vp;
    }
    u -= above;
    const uint32_t side = ntx - vp->rw, beside = vp->rh * side;
    if (u < beside) {
        const uint32_t row = u / side, col = u - row * side;
        ty = vp->ry0 + row;
        tx = col < vp->rx0 ? col : col + vp->rw;
        return vp;
    }
    u -= beside;
    const uint32_t row = u / ntx;
    ty = vp->ry0 + vp->rh + row;
    tx = u - row * ntx;
    return vp;
}

// The last warp of a launch resets the work queue for the next launch.
__device__ __forceinline__ void retire_warp(uint32_t *queue, uint32_t nwarps) {
    if ((threadIdx.x & 31u) == 0) {
        __threadfence();
        if (atomicAdd(queue + 1, 1u) == nwarps - 1) {
            queue[0] = 0;
            queue[1] = 0;
            __threadfence();
        }
    }
}

// Tile scheduler: a warp takes one tile (tile_w x 32/tile_w pixels) at a time
// from the queue and marches its 32 rays to completion.
template <typename T, uint32_t BS, bool TL>
__global__ void __launch_bounds__(256, TL ? 3 : GC_RENDER_MIN_BLOCKS) render_kernel(const CacheView cv, const LevelTables lt,
                                                     const ViewParams *__restrict__ views, uint32_t nviews,
                                                     uint32_t total_tiles, uint32_t *queue, uint32_t nwarps) {
    const uint32_t lane = threadIdx.x & 31u;
    for (;;) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(queue, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= total_tiles) break;
        uint32_t tx, ty;
        const ViewParams *vp = tile_of(views, nviews, t, tx, ty);
        const uint32_t sh = vp->tile_shift, tw = 1u << sh;
        const uint32_t x = (tx << sh) + (lane & (tw - 1u)), y = ty * (32u >> sh) + (lane >> sh);
        bool unm = false, coarse_any = false, marched = false;
        uint32_t nsamp = 0;
        if (x < vp->W && y < vp->H) {
            Ray r;
            if (ray_setup<T>(lt, vp, x, y, r)) {
                marched = ray_enters(r);
                while (ray_step<T, BS, TL>(cv, lt, r)) {
                }
                unm = ray_finish(r);
                coarse_any = r.coarse;
                nsamp = r.nsamp;
            }
        }
        const uint32_t tile_samples = __reduce_add_sync(0xffffffffu, nsamp);
        const uint32_t tile_rays = __popc(__ballot_sync(0xffffffffu, marched));
        if (lane == 0 && tile_samples) atomicAdd(cv.samples, static_cast<unsigned long long>(tile_samples));
        if (lane == 0 && tile_rays) atomicAdd(cv.samples + 1, static_cast<unsigned long long>(tile_rays));
        const uint32_t any = __ballot_sync(0xffffffffu, unm);
        if (any && lane == 0 && vp->status) atomicOr(vp->status, 1u);
        if (vp->fallback && vp->status) {  // bit 1: a coarser level stood in (preview image)
            const uint32_t coarse = __ballot_sync(0xffffffffu, coarse_any);
            if (coarse && lane == 0) atomicOr(vp->status, 2u);
        }
    }
    retire_warp(queue, nwarps);
}

// Pixel scheduler: every lane keeps its own ray; lanes whose ray ended take
// the next pixels of the queue (one warp-aggregated atomic), so a warp never
// waits for its slowest ray.  Pixels are enumerated tile by tile, which keeps
// consecutive grabs spatially close.
template <typename T, uint32_t BS, bool TL>
__global__ void __launch_bounds__(256, TL ? 3 : GC_RENDER_MIN_BLOCKS) render_pixels_kernel(const CacheView cv, const LevelTables lt,
                                                            const ViewParams *__restrict__ views, uint32_t nviews,
                                                            uint32_t total_tiles, uint32_t *queue, uint32_t nwarps) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t total = total_tiles * 32u;
    Ray r;
    bool active = false, exhausted = false;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        if (idle && !exhausted) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (static_cast<int>(lane) == leader) base = atomicAdd(queue, static_cast<uint32_t>(__popc(idle)));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base >= total) exhausted = true;
            if (!active) {
                const uint32_t p = base + __popc(idle & ((1u << lane) - 1u));
                if (p < total) {
                    const uint32_t t = p >> 5, k = p & 31u;
                    uint32_t tx, ty;
                    const ViewParams *vp = tile_of(views, nviews, t, tx, ty);
                    const uint32_t sh = vp->tile_shift, tw = 1u << sh;
                    const uint32_t x = (tx << sh) + (k & (tw - 1u)), y = ty * (32u >> sh) + (k >> sh);
                    if (x < vp->W && y < vp->H) active = ray_setup<T>(lt, vp, x, y, r);
                }
            }
            const uint32_t started = __ballot_sync(0xffffffffu, ((idle >> lane) & 1u) && active && ray_enters(r));
            if (started && static_cast<int>(lane) == leader)
                atomicAdd(cv.samples + 1, static_cast<unsigned long long>(__popc(started)));
        }
        if (active && !ray_step<T, BS, TL>(cv, lt, r)) {
            active = false;
            if (ray_finish(r) && r.vp->status && *r.vp->status == 0u) atomicOr(r.vp->status, 1u);
            if (r.coarse && r.vp->status) atomicOr(r.vp->status, 2u);
            if (r.nsamp) atomicAdd(cv.samples, static_cast<unsigned long long>(r.nsamp));
        }
        if (exhausted && !__any_sync(0xffffffffu, active)) break;
    }
    retire_warp(queue, nwarps);
}

// Kernel of a voxel kind (1, 2, 4 bytes, 0 mixed, kTwoChannelU8), scheduler
// and brick size (16 and 32 compiled for their size, others at run time);
// TL: for a two-level page directory.
template <uint32_t BS, bool TL>
void *march_kernel_bs(uint32_t kind, bool pixels) {
    switch (kind) {
        case 1: return pixels ? reinterpret_cast<void *>(render_pixels_kernel<uint8_t, BS, TL>)
                              : reinterpret_cast<void *>(render_kernel<uint8_t, BS, TL>);
        case 2: return pixels ? reinterpret_cast<void *>(render_pixels_kernel<uint16_t, BS, TL>)
                              : reinterpret_cast<void *>(render_kernel<uint16_t, BS, TL>);
        case 4: return pixels ? reinterpret_cast<void *>(render_pixels_kernel<float, BS, TL>)
                              : reinterpret_cast<void *>(render_kernel<float, BS, TL>);
        case 0: return pixels ? reinterpret_cast<void *>(render_pixels_kernel<MixedVoxel, BS, TL>)
                              : reinterpret_cast<void *>(render_kernel<MixedVoxel, BS, TL>);
        case 0x202: return pixels ? reinterpret_cast<void *>(render_pixels_kernel<TwoU8, BS, TL>)
                                  : reinterpret_cast<void *>(render_kernel<TwoU8, BS, TL>);
        default: return nullptr;
    }
}
void *march_kernel(uint32_t kind, bool pixels, uint32_t brick_size, bool two_level) {
    if (two_level)
        return brick_size == 16 ? march_kernel_bs<16, true>(kind, pixels) : march_kernel_bs<0, true>(kind, pixels);
    if (brick_size == 16) return march_kernel_bs<16, false>(kind, pixels);
    if (brick_size == 32) return march_kernel_bs<32, false>(kind, pixels);
    return march_kernel_bs<0, false>(kind, pixels);
}

}  // namespace GC_MARCH_NS
}  // namespace gc

#ifndef GC_RENDER_FAST
namespace gc {

RenderTuning &render_tuning() {
    static RenderTuning t;
    return t;
}

}  // namespace gc

extern "C" {
int gc_render_precision_set(int precision) {
    return gc::guard([&] {
        GC_REQUIRE(precision == GC_RENDER_EXACT || precision == GC_RENDER_FAST_BUILD,
                   "precision must be GC_RENDER_EXACT or GC_RENDER_FAST_BUILD");
        gc::render_tuning().precision = static_cast<uint32_t>(precision);
    });
}
int gc_render_precision_get(int *precision) {
    return gc::guard([&] {
        GC_REQUIRE(precision, "null argument");
        *precision = static_cast<int>(gc::render_tuning().precision);
    });
}
int gc_render_empty_skip(int enable) {
    return gc::guard([&] { gc::render_tuning().skip_empty = enable ? 1u : 0u; });
}

int gc_render_tuning_set(uint32_t scheduler, uint32_t tile_w, uint32_t threads, uint32_t blocks_per_sm) {
    return gc::guard([&] {
        GC_REQUIRE(scheduler <= 1, "scheduler must be 0 (tile) or 1 (pixel)");
        GC_REQUIRE(tile_w == 4 || tile_w == 8 || tile_w == 16 || tile_w == 32, "tile width must be 4, 8, 16 or 32");
        GC_REQUIRE(threads == 64 || threads == 128 || threads == 256, "threads must be 64, 128 or 256");
        gc::RenderTuning &t = gc::render_tuning();
        t.scheduler = scheduler;
        t.tile_w = tile_w;
        t.threads = threads;
        t.blocks_per_sm = blocks_per_sm;
    });
}
int gc_render_tuning_get(uint32_t out[4]) {
    return gc::guard([&] {
        GC_REQUIRE(out, "null argument");
        const gc::RenderTuning &t = gc::render_tuning();
        out[0] = t.scheduler;
        out[1] = t.tile_w;
        out[2] = t.threads;
        out[3] = t.blocks_per_sm;
    });
}
}  // extern "C"

namespace gc {

// Kernel, grid and block of one ray-caster launch under the current tuning:
// a persistent grid of at most (SMs x resident blocks) that takes its work
// from the launch's tile queue.
struct RenderLaunch {
    void *func;
    uint32_t grid, threads;
};
// Visible value bins of each view (empty-space skipping).  A sample whose
// value lies in bin b reads transfer-function entries within
// [floor(b/64 w - 1/2) - 1, floor((b+1)/64 w - 1/2) + 2]; its opacity after the
// correction 1 - (1 - a)^k is below k a / (1 - a) <= 1.05 k a for a <= 0.04,
// so with a the largest alpha of those entries and k the largest exponent of
// the view's levels, a bin with 1.05 k a < 0.0009 never reaches the
// compositing threshold 0.001.  One warp per view, two bins per lane.
__global__ void view_bins_kernel(ViewParams *views, uint32_t n) {
    const uint32_t v = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31u;
    if (v >= n) return;
    ViewParams &vp = views[v];
    if (!vp.skip_empty) {
        if (lane == 0) vp.visible = ~0ull;
        return;
    }
    float kmax = 0.f;
    for (uint32_t l = 0; l < vp.nlevels; ++l) kmax = fmaxf(kmax, vp.kexp[l]);
    const int w = static_cast<int>(vp.tfw);
    unsigned long long mine = 0;
    for (uint32_t b = lane; b < kValueBins; b += 32) {
        const float lo = static_cast<float>(b) / kValueBins, hi = static_cast<float>(b + 1) / kValueBins;
        int i0 = static_cast<int>(floorf(lo * w - 0.5f)) - 1, i1 = static_cast<int>(floorf(hi * w - 0.5f)) + 2;
        i0 = max(i0, 0);
        i1 = min(i1, w - 1);
        float amax = 0.f;
        for (int i = i0; i <= i1; ++i) amax = fmaxf(amax, __ldg(vp.tf + 4 * i + 3));
        const bool visible = !(amax <= 0.04f && 1.05f * kmax * amax < 0.0009f);
        if (visible) mine |= 1ull << b;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mine |= __shfl_xor_sync(0xffffffffu, mine, o);
    if (lane == 0) vp.visible = mine;
}

void launch_view_bins(ViewParams *views_dev, uint32_t n, cudaStream_t s) {
    view_bins_kernel<<<div_up(n, 4u), 128, 0, s>>>(views_dev, n);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

// Voxel kind of a cache: its voxel width (1, 2, 4), 0 when its volumes'
// widths differ, kTwoChannelU8 for two 8-bit channels.
constexpr uint32_t kTwoChannelU8 = 0x202;
static uint32_t voxel_kind(const CacheView &cv) { return cv.nc == 2 ? kTwoChannelU8 : cv.eb; }

static RenderLaunch render_launch_config(uint32_t eb, uint32_t brick_size, bool two_level, uint32_t total_tiles) {
    const RenderTuning tune = render_tuning();
    const uint32_t threads = tune.threads;
    GC_REQUIRE(threads == 64 || threads == 128 || threads == 256, "render threads must be 64, 128 or 256");
    // kernel of the voxel kind (1, 2, 4 bytes; 0: volumes of different voxel
    // widths share the cache; two 8-bit channels with a 2D transfer function)
    // from the exact or the fast build
    const bool pix = tune.scheduler == 1, fast_build = tune.precision == 1;
    void *kernel = fast_build ? fast::march_kernel(eb, pix, brick_size, two_level)
                              : exact::march_kernel(eb, pix, brick_size, two_level);
    if (!kernel) fail(GC_ERR_UNSUPPORTED, "the ray caster supports one channel of 1, 2 or 4 bytes");
    const int slot = eb == 1 ? 0 : eb == 2 ? 1 : eb == 4 ? 2 : eb == 0 ? 3 : 4;
    static int occupancy[2][2][5][3][5] = {};
    const int tslot = threads == 64 ? 0 : (threads == 128 ? 1 : 2);
    const int bslot = two_level ? (brick_size == 16 ? 3 : 4) : (brick_size == 16 ? 0 : (brick_size == 32 ? 1 : 2));
    int &occ = occupancy[fast_build ? 1 : 0][pix ? 1 : 0][slot][tslot][bslot];
    if (!occ) {
        int b = 0;
        GC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, static_cast<int>(threads), 0));
        occ = std::max(1, b);
    }
    int per_sm = occ;
    if (tune.blocks_per_sm > 0) per_sm = std::min(per_sm, static_cast<int>(tune.blocks_per_sm));
    const uint32_t max_blocks = static_cast<uint32_t>(sm_count() * per_sm);
    const uint32_t want = div_up(total_tiles, threads / 32);
    return RenderLaunch{kernel, std::max(1u, std::min(max_blocks, want)), threads};
}

void launch_render(const CacheView &cv, const LevelTables &lt, const ViewParams *views_dev,
                   const ViewParams * /*views_host*/, uint32_t nviews, uint32_t total_tiles, uint32_t *queue,
                   uint32_t * /*err*/, cudaStream_t s) {
    if (total_tiles == 0) return;
    const RenderLaunch L = render_launch_config(voxel_kind(cv), cv.B, cv.pt.shift != 0u, total_tiles);
    uint32_t nwarps = L.grid * (L.threads / 32);
    void *args[] = {const_cast<CacheView *>(&cv), const_cast<LevelTables *>(&lt), &views_dev, &nviews, &total_tiles,
                    &queue, &nwarps};
    GC_CUDA(cudaLaunchKernel(L.func, dim3(L.grid), dim3(L.threads), args, 0, s));
    count_launch();
}

RenderGraph::~RenderGraph() { reset(); }

void RenderGraph::reset() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    func = nullptr;
}

// The batched form's launch: an instantiated graph of three nodes -- the copy
// of the view table from pinned host memory, the views' visible value bins
// and the persistent ray caster -- is
// replayed every tick; only the kernel's arguments (timestamp, view and tile
// counts, grid) and the copy's size change, through the executable graph's
// node-update calls.  The graph is rebuilt when the tuning changes the kernel.
void launch_render_graph(RenderGraph &g, const CacheView &cv, const LevelTables &lt, ViewParams *views_dev,
                         const ViewParams *views_pinned, uint32_t nviews, uint32_t total_tiles, uint32_t *queue,
                         cudaStream_t s) {
    if (total_tiles == 0) return;
    const RenderLaunch L = render_launch_config(voxel_kind(cv), cv.B, cv.pt.shift != 0u, total_tiles);
    uint32_t nwarps = L.grid * (L.threads / 32);
    const ViewParams *vd = views_dev;
    void *args[] = {const_cast<CacheView *>(&cv), const_cast<LevelTables *>(&lt), &vd, &nviews, &total_tiles,
                    &queue, &nwarps};
    cudaKernelNodeParams kp = {};
    kp.func = L.func;
    kp.gridDim = dim3(L.grid);
    kp.blockDim = dim3(L.threads);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    kp.extra = nullptr;
    const size_t bytes = static_cast<size_t>(nviews) * sizeof(ViewParams);
    ViewParams *vbins = views_dev;
    void *bargs[] = {&vbins, &nviews};
    cudaKernelNodeParams bp = {};
    bp.func = reinterpret_cast<void *>(view_bins_kernel);
    bp.gridDim = dim3(div_up(nviews, 4u));
    bp.blockDim = dim3(128);
    bp.kernelParams = bargs;
    if (g.exec && (g.func != L.func || g.threads != L.threads)) g.reset();
    if (!g.exec) {
        GC_CUDA(cudaGraphCreate(&g.graph, 0));
        GC_CUDA(cudaGraphAddMemcpyNode1D(&g.copy, g.graph, nullptr, 0, views_dev, views_pinned, bytes,
                                         cudaMemcpyHostToDevice));
        GC_CUDA(cudaGraphAddKernelNode(&g.bins, g.graph, &g.copy, 1, &bp));
        GC_CUDA(cudaGraphAddKernelNode(&g.kern, g.graph, &g.bins, 1, &kp));
        GC_CUDA(cudaGraphInstantiate(&g.exec, g.graph, 0));
        g.func = L.func;
        g.threads = L.threads;
    } else {
        GC_CUDA(cudaGraphExecMemcpyNodeSetParams1D(g.exec, g.copy, views_dev, views_pinned, bytes,
                                                   cudaMemcpyHostToDevice));
        GC_CUDA(cudaGraphExecKernelNodeSetParams(g.exec, g.bins, &bp));
        GC_CUDA(cudaGraphExecKernelNodeSetParams(g.exec, g.kern, &kp));
    }
    GC_CUDA(cudaGraphLaunch(g.exec, s));
    g.replays++;
    count_launch();
}

}  // namespace gc
#endif  // GC_RENDER_FAST
