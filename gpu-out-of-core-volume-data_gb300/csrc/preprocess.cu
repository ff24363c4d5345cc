// Preprocessor kernels: mip pyramid (2x2x2 box reduction), bricking with a
// covering border, and empty-brick flags.  Everything stays resident in HBM;
// the reference streams 512 MB chunks through cudaMalloc/H2D/kernel/D2H/free
// per chunk (GcCore/src/cuda/libPreprocessor/Mipmapper.cu:401-578) and bricks
// on the CPU with one seek+read per brick row
// (GcCore/src/libPreprocessor/Bricker_v2.cpp:79-252).
#include <cstring>

#include "cache.cuh"
#include "gc_internal.h"

namespace gc {

// ---------------------------------------------------------------------------
// mip_reduce: one 2x2x2 pass.
//
// Reference arithmetic (down_sampling_inner, Mipmapper.cu:29-105):
//   8-bit channels : uint64 sum of the 8 inputs, integer division by 8;
//   16-bit, 1 ch.  : double sum (its initial value is uninitialised in the
//                    reference; zero here), / 8.0, truncating conversion;
//                    the sum of 8 u16 is exact so this is floor(sum / 8);
//   f32            : double sum in (z, y, x) loop order, / 8.0, rounded to float.
// The reference handles interleaved channels only on the 8-bit path; here every
// integer channel width uses the per-channel floor mean.
//
// Vector kernel: one thread per 16-byte chunk of each of the 4 input rows
// (y0,z0), (y1,z0), (y0,z1), (y1,z1); it writes the 8 output bytes that chunk
// reduces to.  Every input byte is read once, with 128-bit loads.
template <int CB, int NC>
__device__ inline void reduce_chunk(const uint4 (&r)[4], uint2 &out) {
    if constexpr (CB == 1) {
        const uint8_t *b0 = reinterpret_cast<const uint8_t *>(&r[0]);
        const uint8_t *b1 = reinterpret_cast<const uint8_t *>(&r[1]);
        const uint8_t *b2 = reinterpret_cast<const uint8_t *>(&r[2]);
        const uint8_t *b3 = reinterpret_cast<const uint8_t *>(&r[3]);
        uint8_t *o = reinterpret_cast<uint8_t *>(&out);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int i = j / NC, c = j % NC;
            const int a = (2 * i) * NC + c, b = (2 * i + 1) * NC + c;
            uint32_t s = b0[a] + b0[b] + b1[a] + b1[b] + b2[a] + b2[b] + b3[a] + b3[b];
            o[j] = static_cast<uint8_t>(s / 8u);
        }
    } else if constexpr (CB == 2) {
        const uint16_t *h0 = reinterpret_cast<const uint16_t *>(&r[0]);
        const uint16_t *h1 = reinterpret_cast<const uint16_t *>(&r[1]);
        const uint16_t *h2 = reinterpret_cast<const uint16_t *>(&r[2]);
        const uint16_t *h3 = reinterpret_cast<const uint16_t *>(&r[3]);
        uint16_t *o = reinterpret_cast<uint16_t *>(&out);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int i = j / NC, c = j % NC;
            const int a = (2 * i) * NC + c, b = (2 * i + 1) * NC + c;
            uint32_t s = h0[a] + h0[b] + h1[a] + h1[b] + h2[a] + h2[b] + h3[a] + h3[b];
            o[j] = static_cast<uint16_t>(s / 8u);
        }
    } else {
        const float *f0 = reinterpret_cast<const float *>(&r[0]);
        const float *f1 = reinterpret_cast<const float *>(&r[1]);
        const float *f2 = reinterpret_cast<const float *>(&r[2]);
        const float *f3 = reinterpret_cast<const float *>(&r[3]);
        float *o = reinterpret_cast<float *>(&out);
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            double s = 0.0;
            s += f0[2 * i];
            s += f0[2 * i + 1];
            s += f1[2 * i];
            s += f1[2 * i + 1];
            s += f2[2 * i];
            s += f2[2 * i + 1];
            s += f3[2 * i];
            s += f3[2 * i + 1];
            o[i] = static_cast<float>(s / 8.0);
        }
    }
}

struct MipParams {
    uint32_t X, Y, Z;            // source dims
    uint32_t oX, oY, oZ;         // output dims
    uint64_t in_row, out_row;    // bytes per row
    uint32_t chunks;             // 16-byte chunks per input row that produce output
    uint64_t total;              // chunks * oY * oZ
};

template <int CB, int NC>
__global__ void __launch_bounds__(256) mip_vec_kernel(const uint8_t *__restrict__ src,
                                                      uint8_t *__restrict__ dst, MipParams p) {
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < p.total;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint32_t chunk = static_cast<uint32_t>(t % p.chunks);
        const uint64_t orow = t / p.chunks;
        const uint32_t oy = static_cast<uint32_t>(orow % p.oY), oz = static_cast<uint32_t>(orow / p.oY);
        const uint64_t r00 = (static_cast<uint64_t>(2 * oz) * p.Y + 2 * oy) * p.in_row;
        const uint64_t plane = static_cast<uint64_t>(p.Y) * p.in_row;
        const uint64_t off = static_cast<uint64_t>(chunk) * 16;
        uint4 r[4];
        r[0] = __ldcs(reinterpret_cast<const uint4 *>(src + r00 + off));
        r[1] = __ldcs(reinterpret_cast<const uint4 *>(src + r00 + p.in_row + off));
        r[2] = __ldcs(reinterpret_cast<const uint4 *>(src + r00 + plane + off));
        r[3] = __ldcs(reinterpret_cast<const uint4 *>(src + r00 + plane + p.in_row + off));
        uint2 o;
        reduce_chunk<CB, NC>(r, o);
        *reinterpret_cast<uint2 *>(dst + (static_cast<uint64_t>(oz) * p.oY + oy) * p.out_row + chunk * 8) = o;
    }
}

// Generic path (any width, odd sizes): one thread per output channel value.
__global__ void mip_scalar_kernel(const uint8_t *__restrict__ src, uint8_t *__restrict__ dst,
                                  MipParams p, uint32_t cb, uint32_t nc) {
    const uint64_t n = static_cast<uint64_t>(p.oX) * p.oY * p.oZ * nc;
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < n;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint32_t c = static_cast<uint32_t>(t % nc);
        const uint64_t v = t / nc;
        const uint32_t ox = static_cast<uint32_t>(v % p.oX);
        const uint64_t r = v / p.oX;
        const uint32_t oy = static_cast<uint32_t>(r % p.oY), oz = static_cast<uint32_t>(r / p.oY);
        const uint64_t eb = static_cast<uint64_t>(cb) * nc;
        uint64_t isum = 0;
        double dsum = 0.0;
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) {
                    const uint64_t vox = (static_cast<uint64_t>(2 * oz + dz) * p.Y + (2 * oy + dy)) * p.X + (2 * ox + dx);
                    const uint8_t *ptr = src + vox * eb + c * cb;
                    if (cb == 1)
                        isum += *ptr;
                    else if (cb == 2)
                        isum += *reinterpret_cast<const uint16_t *>(ptr);
                    else
                        dsum += *reinterpret_cast<const float *>(ptr);
                }
        uint8_t *o = dst + ((static_cast<uint64_t>(oz) * p.oY + oy) * p.oX + ox) * eb + c * cb;
        if (cb == 1)
            *o = static_cast<uint8_t>(isum / 8u);
        else if (cb == 2)
            *reinterpret_cast<uint16_t *>(o) = static_cast<uint16_t>(isum / 8u);
        else
            *reinterpret_cast<float *>(o) = static_cast<float>(dsum / 8.0);
    }
}

static void launch_mip(const void *src, void *dst, const uint32_t d[3], uint32_t eb, uint32_t nc,
                       cudaStream_t s) {
    GC_REQUIRE(eb % nc == 0, "encoded bytes must be a multiple of channels");
    const uint32_t cb = eb / nc;
    GC_REQUIRE(cb == 1 || cb == 2 || cb == 4, "bytes per channel must be 1, 2 or 4");
    MipParams p;
    p.X = d[0];
    p.Y = d[1];
    p.Z = d[2];
    p.oX = d[0] / 2;
    p.oY = d[1] / 2;
    p.oZ = d[2] / 2;
    GC_REQUIRE(p.oX && p.oY && p.oZ, "level too small to down-sample");
    p.in_row = static_cast<uint64_t>(p.X) * eb;
    p.out_row = static_cast<uint64_t>(p.oX) * eb;
    const int grid = sm_count() * 8;
    const bool aligned = (reinterpret_cast<uintptr_t>(src) % 16 == 0) &&
                         (reinterpret_cast<uintptr_t>(dst) % 8 == 0) && (p.X % 2 == 0) &&
                         (p.in_row % 16 == 0);
    if (aligned) {
        p.chunks = static_cast<uint32_t>(p.in_row / 16);
        p.total = static_cast<uint64_t>(p.chunks) * p.oY * p.oZ;
        auto *in = static_cast<const uint8_t *>(src);
        auto *out = static_cast<uint8_t *>(dst);
        if (cb == 1 && nc == 1)
            mip_vec_kernel<1, 1><<<grid, 256, 0, s>>>(in, out, p);
        else if (cb == 1 && nc == 2)
            mip_vec_kernel<1, 2><<<grid, 256, 0, s>>>(in, out, p);
        else if (cb == 1 && nc == 4)
            mip_vec_kernel<1, 4><<<grid, 256, 0, s>>>(in, out, p);
        else if (cb == 2 && nc == 1)
            mip_vec_kernel<2, 1><<<grid, 256, 0, s>>>(in, out, p);
        else if (cb == 2 && nc == 2)
            mip_vec_kernel<2, 2><<<grid, 256, 0, s>>>(in, out, p);
        else if (cb == 4 && nc == 1)
            mip_vec_kernel<4, 1><<<grid, 256, 0, s>>>(in, out, p);
        else
            mip_scalar_kernel<<<grid, 256, 0, s>>>(in, out, p, cb, nc);
    } else {
        mip_scalar_kernel<<<grid, 256, 0, s>>>(static_cast<const uint8_t *>(src),
                                                static_cast<uint8_t *>(dst), p, cb, nc);
    }
    GC_CUDA(cudaGetLastError());
        count_launch();
}

// ---------------------------------------------------------------------------
// Bricking: small brick (bx, by, bz) of level dims D covers voxels
// [b * (B - 2c) - c, b * (B - 2c) - c + B) per axis; voxels outside the level
// are zero (Bricker_v2.cpp:145-200), and so is every small brick whose start
// b * (B - 2c) is outside the level on some axis.  Output layout: big bricks in (z, y, x)
// raster order, each (BB*B)^3 voxels x-fastest; small brick (i, j, k) of a big
// brick at voxel offset (i*B, j*B, k*B) (Bricker_v2.cpp:149-152, 295-299).

// One voxel of a small brick the slow way (bricks on the level's edge, odd
// voxel widths): zero outside the level or in an unvisited brick.
__device__ __forceinline__ void brick_voxel(const uint8_t *__restrict__ level, uint8_t *__restrict__ dptr,
                                            const BrickParams &p, bool visited, int64_t gx, int64_t gy, int64_t gz) {
    const bool inside = visited && gx >= 0 && gy >= 0 && gz >= 0 && gx < p.D[0] && gy < p.D[1] && gz < p.D[2];
    const uint8_t *sptr = level + ((static_cast<uint64_t>(gz) * p.D[1] + gy) * p.D[0] + gx) * p.eb;
    switch (p.eb) {
        case 1:
            *dptr = inside ? __ldg(sptr) : uint8_t(0);
            break;
        case 2:
            *reinterpret_cast<uint16_t *>(dptr) = inside ? __ldg(reinterpret_cast<const uint16_t *>(sptr)) : uint16_t(0);
            break;
        case 4:
            *reinterpret_cast<uint32_t *>(dptr) = inside ? __ldg(reinterpret_cast<const uint32_t *>(sptr)) : 0u;
            break;
        default:
            for (uint32_t b = 0; b < p.eb; ++b) dptr[b] = inside ? sptr[b] : 0;
    }
}

// 16 bytes of a source row starting at byte `s` (0..15) of the aligned pair (a, b).
__device__ __forceinline__ uint4 row_bytes16(uint4 a, uint4 b, uint32_t s) {
    const uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    const uint32_t r = (s & 3u) * 8u;
    uint32_t o[4];
    // s / 4 is the same for every thread of a brick: a uniform branch with
    // constant register indices in each arm
    switch (s >> 2) {
#define GC_ROW_CASE(Q)                                                                  \
    case Q:                                                                             \
        _Pragma("unroll") for (int k = 0; k < 4; ++k) o[k] = __funnelshift_r(w[Q + k], w[Q + k + 1], r); \
        break;
        GC_ROW_CASE(0)
        GC_ROW_CASE(1)
        GC_ROW_CASE(2)
        GC_ROW_CASE(3)
#undef GC_ROW_CASE
    }
    return make_uint4(o[0], o[1], o[2], o[3]);
}

// Copies small brick (sx, sy, sz) of a level into its place in a big brick
// (big_base; (ix, iy, iz) = its position among the big brick's BB bricks),
// with the 32 lanes of a warp.  p.fast (B a power of two, whole 16-byte
// chunks per row, rows 16 bytes apart in the level, 16-byte aligned buffers):
// the brick goes in 16-byte output chunks.  A chunk whose source row lies
// inside the level and whose voxels all lie inside the row -- all chunks of an
// interior brick -- starts at the same byte offset s modulo 16 as every other
// such chunk of the brick, so it is two aligned 16-byte loads and a funnel
// shift by s, stored with one 16-byte store.  A row outside the level, or an
// unvisited brick, stores zeros; a chunk straddling the level's x edge is
// assembled voxel by voxel.  Otherwise the brick is copied voxel by voxel.
__device__ __forceinline__ void copy_small_brick(const uint8_t *__restrict__ level, const BrickParams &p,
                                                 uint32_t sx, uint32_t sy, uint32_t sz, uint8_t *big_base,
                                                 uint32_t ix, uint32_t iy, uint32_t iz, uint32_t lane) {
    const uint32_t B = p.B;
    const uint32_t bvx = p.BB[0] * B, bvy = p.BB[1] * B;
    const int64_t ox = static_cast<int64_t>(sx) * p.Beff - p.c;
    const int64_t oy = static_cast<int64_t>(sy) * p.Beff - p.c;
    const int64_t oz = static_cast<int64_t>(sz) * p.Beff - p.c;
    // The reference visits a small brick only if its start lies inside the
    // level on every axis (Bricker_v2.cpp:203-221); the others stay zero even
    // where their covering border reaches into the volume.
    const bool visited = static_cast<uint64_t>(sx) * p.Beff < p.D[0] &&
                         static_cast<uint64_t>(sy) * p.Beff < p.D[1] && static_cast<uint64_t>(sz) * p.Beff < p.D[2];
    if (p.fast) {
        const uint32_t k = 16u / p.eb;                  // voxels per chunk
        const uint32_t nchunks = 1u << (2u * p.b_shift + p.cpr_shift);
        const uint64_t row_stride = static_cast<uint64_t>(p.D[0]) * p.eb;
        // byte offset modulo 16 of the brick's first voxel in any row (rows
        // are multiples of 16 bytes apart; ox may be negative)
        const uint32_t s = static_cast<uint32_t>(ox * static_cast<int64_t>(p.eb)) & 15u;
        uint8_t *obase = big_base + ((static_cast<uint64_t>(iz) * B * bvy + iy * B) * bvx + ix * B) * p.eb;
        const uint64_t drow = static_cast<uint64_t>(bvx) * p.eb;  // output row stride
        if (visited && ox >= 0 && oy >= 0 && oz >= 0 && ox + B <= p.D[0] && oy + B <= p.D[1] && oz + B <= p.D[2]) {
            // Interior brick (the common case, the same branch for the whole
            // warp): no per-chunk tests; each lane issues the loads of 4 chunks
            // before it stores them.  The second load of a pair ends at or
            // before the end of its row: the chunk's first voxel byte plus 16
            // lies inside the row, and rows end on 16-byte boundaries.
            const uint8_t *sbase = level + (static_cast<uint64_t>(oz) * p.D[1] + static_cast<uint64_t>(oy)) * row_stride +
                                   static_cast<uint64_t>(ox) * p.eb - s;
            const uint32_t cmask = (1u << p.cpr_shift) - 1u;
            for (uint32_t c0 = lane; c0 < nchunks; c0 += 128u) {
                uint4 a[4], b[4] = {};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint32_t c = c0 + 32u * u;
                    if (c < nchunks) {
                        const uint32_t row = c >> p.cpr_shift;
                        const uint8_t *src = sbase + (static_cast<uint64_t>(row >> p.b_shift) * p.D[1] + (row & (B - 1u))) *
                                                         row_stride + (c & cmask) * 16u;
                        a[u] = __ldg(reinterpret_cast<const uint4 *>(src));
                        if (s) b[u] = __ldg(reinterpret_cast<const uint4 *>(src + 16));
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint32_t c = c0 + 32u * u;
                    if (c < nchunks) {
                        const uint32_t row = c >> p.cpr_shift;
                        uint8_t *dst = obase + (static_cast<uint64_t>(row >> p.b_shift) * bvy + (row & (B - 1u))) * drow +
                                       (c & cmask) * 16u;
                        *reinterpret_cast<uint4 *>(dst) = s ? row_bytes16(a[u], b[u], s) : a[u];
                    }
                }
            }
            return;
        }
#pragma unroll 4
        for (uint32_t c = lane; c < nchunks; c += 32u) {
            const uint32_t cx = c & ((1u << p.cpr_shift) - 1u), row = c >> p.cpr_shift;
            const uint32_t ly = row & (B - 1u), lz = row >> p.b_shift;
            uint8_t *dst = obase + (static_cast<uint64_t>(lz) * bvy + ly) * drow + cx * 16u;
            const int64_t ry = oy + ly, rz = oz + lz, x0 = ox + static_cast<int64_t>(cx) * k;
            const bool row_in = visited && ry >= 0 && rz >= 0 && ry < p.D[1] && rz < p.D[2];
            if (!row_in) {
                *reinterpret_cast<uint4 *>(dst) = make_uint4(0u, 0u, 0u, 0u);
            } else if (x0 >= 0 && x0 + k <= p.D[0]) {
                const uint64_t src = (static_cast<uint64_t>(rz) * p.D[1] + ry) * row_stride +
                                     static_cast<uint64_t>(x0) * p.eb - s;
                const uint4 a = __ldg(reinterpret_cast<const uint4 *>(level + src));
                *reinterpret_cast<uint4 *>(dst) =
                    s ? row_bytes16(a, __ldg(reinterpret_cast<const uint4 *>(level + src + 16)), s) : a;
            } else {
                for (uint32_t v = 0; v < k; ++v)
                    brick_voxel(level, dst + v * p.eb, p, true, x0 + v, ry, rz);
            }
        }
        return;
    }
    const uint32_t nvox = B * B * B;
    for (uint32_t v = lane; v < nvox; v += 32u) {
        const uint32_t lx = v % B, ly = (v / B) % B, lz = v / (B * B);
        uint8_t *dptr = big_base + ((static_cast<uint64_t>(iz * B + lz) * bvy + (iy * B + ly)) * bvx + (ix * B + lx)) * p.eb;
        brick_voxel(level, dptr, p, visited, ox + lx, oy + ly, oz + lz);
    }
}

// The bricker of one level: one warp per small brick (grid-stride over
// bricks); the per-brick index arithmetic is done once per warp and brick
// (16 chunks per lane for B16 u16), the per-chunk one with shifts.
__global__ void __launch_bounds__(256) brick_kernel(const uint8_t *__restrict__ level,
                                                    uint8_t *__restrict__ out, BrickParams p) {
    const uint64_t big_bytes = static_cast<uint64_t>(p.BB[0] * p.B) * (p.BB[1] * p.B) * (p.BB[2] * p.B) * p.eb;
    const uint32_t nsx = p.nbig[0] * p.BB[0], nsy = p.nbig[1] * p.BB[1];
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t nsmall = static_cast<uint32_t>(p.nsmall);  // < 2^32 (checked on the host)
    for (uint32_t sb = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; sb < nsmall; sb += nwarps) {
        // small brick grid = nbig * BB per axis, x fastest
        const uint32_t sx = sb % nsx, rest = sb / nsx;
        const uint32_t sy = rest % nsy, sz = rest / nsy;
        const uint32_t gx = sx / p.BB[0], gy = sy / p.BB[1], gz = sz / p.BB[2];
        const uint64_t big = (static_cast<uint64_t>(gz) * p.nbig[1] + gy) * p.nbig[0] + gx;
        copy_small_brick(level, p, sx, sy, sz, out + big * big_bytes, sx - gx * p.BB[0], sy - gy * p.BB[1],
                         sz - gz * p.BB[2], lane);
    }
}

// Bytes [s, s + 16) of the 32-byte pair (a, b) for a per-lane s in 0..15: a
// two-level select by whole words, then a funnel shift by the byte remainder.
__device__ __forceinline__ uint4 window16(uint4 a, uint4 b, uint32_t s) {
    const bool w2 = (s & 8u) != 0u, w1 = (s & 4u) != 0u;
    const uint32_t u0 = w2 ? a.z : a.x, u1 = w2 ? a.w : a.y, u2 = w2 ? b.x : a.z, u3 = w2 ? b.y : a.w,
                   u4 = w2 ? b.z : b.x, u5 = w2 ? b.w : b.y;
    const uint32_t v0 = w1 ? u1 : u0, v1 = w1 ? u2 : u1, v2 = w1 ? u3 : u2, v3 = w1 ? u4 : u3, v4 = w1 ? u5 : u4;
    const uint32_t r = (s & 3u) * 8u;
    return make_uint4(__funnelshift_r(v0, v1, r), __funnelshift_r(v1, v2, r), __funnelshift_r(v2, v3, r),
                      __funnelshift_r(v3, v4, r));
}

// Row-mapped bricker (p.fast and at most 32 16-byte chunks per brick row): a
// warp takes a run of nb = 32 / cpr bricks adjacent along x (one (sy, sz)
// brick row), lane q holding chunk q % cpr of brick q / cpr, and walks the
// B x B rows of the run.  Each row step reads one contiguous span of the
// level row (nb bricks' windows, about 32 chunks, each fetched by at most two
// lanes and merged in L1) and writes each brick's row chunk with one 16-byte
// store.  Rows are whole 16-byte chunks of the level (row bytes a multiple of
// 16, aligned level), so a chunk lies entirely inside or outside the row:
// chunks outside read as zero, which is the bricker's value there (outside
// the level); rows outside the level and unvisited bricks store zeros.  Row
// steps go four at a time, their loads issued before their stores.
__global__ void __launch_bounds__(256) brick_rows_kernel(const uint8_t *__restrict__ level,
                                                         uint8_t *__restrict__ out, BrickParams p, uint32_t ngx) {
    const uint32_t B = p.B, eb = p.eb;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t nb = 32u >> p.cpr_shift;
    const uint32_t j = lane >> p.cpr_shift, k = lane & ((1u << p.cpr_shift) - 1u);
    const uint32_t nsx = p.nbig[0] * p.BB[0], nsy = p.nbig[1] * p.BB[1], nsz = p.nbig[2] * p.BB[2];
    const uint32_t bvx = p.BB[0] * B, bvy = p.BB[1] * B;
    const uint64_t big_bytes = static_cast<uint64_t>(bvx) * bvy * (p.BB[2] * B) * eb;
    const uint64_t row_bytes = static_cast<uint64_t>(p.D[0]) * eb;
    const int64_t row_chunks = static_cast<int64_t>(row_bytes >> 4);
    const uint64_t drow = static_cast<uint64_t>(bvx) * eb;  // output row stride
    const uint32_t nseg_xy = ngx * nsy;
    const uint64_t nseg = static_cast<uint64_t>(nseg_xy) * nsz;
    const uint32_t nrows = B * B;
    const uint64_t gwarp = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
    for (uint64_t seg = gwarp; seg < nseg; seg += nwarps) {
        const uint32_t sz = static_cast<uint32_t>(seg / nseg_xy);
        const uint32_t rem = static_cast<uint32_t>(seg - static_cast<uint64_t>(sz) * nseg_xy);
        const uint32_t sy = rem / ngx, g = rem - sy * ngx;
        const uint32_t sx = g * nb + j;
        const bool valid = sx < nsx;
        const bool yz_vis = static_cast<uint64_t>(sy) * p.Beff < p.D[1] && static_cast<uint64_t>(sz) * p.Beff < p.D[2];
        const bool x_vis = static_cast<uint64_t>(sx) * p.Beff < p.D[0];
        // this lane's source window in any row: bytes [o, o + 16), o = its
        // chunk's first voxel byte (negative in the covering left of x = 0)
        const int64_t o = (static_cast<int64_t>(sx) * p.Beff - p.c) * eb + 16 * static_cast<int64_t>(k);
        const int64_t ca = o >> 4;  // floor
        const uint32_t s = static_cast<uint32_t>(o - ca * 16);
        const bool a_in = x_vis && ca >= 0 && ca < row_chunks;
        const bool b_in = x_vis && s != 0u && ca + 1 >= 0 && ca + 1 < row_chunks;
        const uint32_t gx = valid ? sx / p.BB[0] : 0u, gy = sy / p.BB[1], gz = sz / p.BB[2];
        const uint32_t ix = sx - gx * p.BB[0], iy = sy - gy * p.BB[1], iz = sz - gz * p.BB[2];
        const uint64_t big = (static_cast<uint64_t>(gz) * p.nbig[1] + gy) * p.nbig[0] + gx;
        uint8_t *dst = out + big * big_bytes + ((static_cast<uint64_t>(iz) * B * bvy + iy * B) * bvx + ix * B) * eb +
                       16u * k;
        const int64_t y0 = static_cast<int64_t>(sy) * p.Beff - p.c, z0 = static_cast<int64_t>(sz) * p.Beff - p.c;
        for (uint32_t r0 = 0; r0 < nrows; r0 += 4u) {
            uint4 a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t r = r0 + u, ly = r & (B - 1u), lz = r >> p.b_shift;
                const int64_t y = y0 + ly, z = z0 + lz;
                const bool row_in = yz_vis && y >= 0 && z >= 0 && y < p.D[1] && z < p.D[2];
                a[u] = make_uint4(0u, 0u, 0u, 0u);
                b[u] = a[u];
                if (row_in) {
                    const uint4 *row = reinterpret_cast<const uint4 *>(
                        level + (static_cast<uint64_t>(z) * p.D[1] + static_cast<uint64_t>(y)) * row_bytes);
                    if (a_in) a[u] = __ldg(row + ca);
                    if (b_in) b[u] = __ldg(row + ca + 1);
                }
            }
            if (valid) {
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint32_t r = r0 + u, ly = r & (B - 1u), lz = r >> p.b_shift;
                    *reinterpret_cast<uint4 *>(dst + (static_cast<uint64_t>(lz) * bvy + ly) * drow) =
                        window16(a[u], b[u], s);
                }
            }
        }
    }
}

// Bricks cut on demand from a device-resident pyramid (the device-levels
// brick source): job j = big brick (x, y, z) of level `lvl` of volume `vol`
// into staging slot `slot`; one block per job, its warps over the job's small
// bricks, each by the level bricker's rule.
__global__ void __launch_bounds__(256) cut_bricks_kernel(const CutSources srcs, const uint4 *__restrict__ jobs,
                                                         uint32_t n, uint8_t *__restrict__ staging,
                                                         uint64_t stride) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t j = blockIdx.x; j < n; j += gridDim.x) {
        const uint4 job = jobs[j];
        const uint32_t lvl = job.w & 63u, vol = (job.w >> 6) & 3u, slot = job.w >> 8;
        const CutSource &cs = srcs.vol[vol];
        BrickParams p = cs.p;
        for (int a = 0; a < 3; ++a) p.D[a] = cs.dims[lvl][a];
        p.fast = cs.fast[lvl];
        const uint32_t nsub = p.BB[0] * p.BB[1] * p.BB[2];
        for (uint32_t sub = warp; sub < nsub; sub += nw) {
            const uint32_t ix = sub % p.BB[0], iy = (sub / p.BB[0]) % p.BB[1], iz = sub / (p.BB[0] * p.BB[1]);
            copy_small_brick(cs.pyramid + cs.offset[lvl], p, job.x * p.BB[0] + ix, job.y * p.BB[1] + iy,
                             job.z * p.BB[2] + iz, staging + static_cast<uint64_t>(slot) * stride, ix, iy, iz,
                             lane);
        }
    }
}

void launch_cut_bricks(const CutSources &srcs, const uint4 *jobs, uint32_t n, uint8_t *staging, uint64_t stride,
                       cudaStream_t s) {
    if (n == 0) return;
    cut_bricks_kernel<<<std::min<uint32_t>(n, static_cast<uint32_t>(sm_count()) * 8), 256, 0, s>>>(srcs, jobs, n,
                                                                                                 staging, stride);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

// Empty flags: 1 if every channel value of the big brick is < threshold
// (DefaultBrickProcessorPredicate: (float)value < threshold).
__global__ void __launch_bounds__(256) empty_kernel(const uint8_t *__restrict__ bricks, uint64_t nbig,
                                                    uint64_t big_values, uint32_t cb, float threshold,
                                                    uint8_t *__restrict__ flags) {
    __shared__ int s_nonempty;
    for (uint64_t b = blockIdx.x; b < nbig; b += gridDim.x) {
        if (threadIdx.x == 0) s_nonempty = 0;
        __syncthreads();
        const uint8_t *base = bricks + b * big_values * cb;
        int nonempty = 0;
        for (uint64_t i = threadIdx.x; i < big_values && !nonempty; i += blockDim.x) {
            float v;
            if (cb == 1)
                v = static_cast<float>(base[i]);
            else if (cb == 2)
                v = static_cast<float>(reinterpret_cast<const uint16_t *>(base)[i]);
            else
                v = reinterpret_cast<const float *>(base)[i];
            if (!(v < threshold)) nonempty = 1;
        }
        if (__syncthreads_or(nonempty) && threadIdx.x == 0) s_nonempty = 1;
        __syncthreads();
        if (threadIdx.x == 0) flags[b] = s_nonempty ? 0 : 1;
        __syncthreads();
    }
}

}  // namespace gc

using namespace gc;

extern "C" {

int gc_mip_level(const void *src, void *dst, const uint32_t src_dims[3], uint32_t encoded_bytes,
                 uint32_t channels, void *stream) {
    return guard([&] {
        GC_REQUIRE(src && dst && src_dims, "null argument");
        GC_REQUIRE(channels >= 1, "channels must be >= 1");
        launch_mip(src, dst, src_dims, encoded_bytes, channels, as_stream(stream));
    });
}

int gc_mip_build(void *pyramid, const gc_layout *layout, const uint64_t *level_offsets,
                 uint32_t encoded_bytes, uint32_t channels, void *stream) {
    return guard([&] {
        GC_REQUIRE(pyramid && layout && level_offsets, "null argument");
        GC_REQUIRE(layout->nb_levels >= 1 && layout->nb_levels <= GC_MAX_LEVELS, "bad layout");
        GC_REQUIRE(level_offsets[0] == 0, "level 0 must start at offset 0");
        uint8_t *base = static_cast<uint8_t *>(pyramid);
        for (uint32_t l = 1; l < layout->nb_levels; ++l) {
            const uint32_t *d = layout->mip[l - 1];
            for (int a = 0; a < 3; ++a)
                GC_REQUIRE(layout->mip[l][a] == d[a] / 2,
                           "level sizes that stop halving (dimension <= 2) are not supported");
            launch_mip(base + level_offsets[l - 1], base + level_offsets[l], d, encoded_bytes, channels,
                       as_stream(stream));
        }
    });
}

int gc_bricks_build(const void *level, const uint32_t level_dims[3], const gc_volume_desc *vol,
                    const uint32_t nb_big_bricks[3], void *out, void *stream) {
    return guard([&] {
        GC_REQUIRE(level && level_dims && vol && nb_big_bricks && out, "null argument");
        validate_volume(*vol);
        BrickParams p;
        for (int a = 0; a < 3; ++a) {
            p.D[a] = level_dims[a];
            p.BB[a] = vol->big_brick_size[a];
            p.nbig[a] = nb_big_bricks[a];
            GC_REQUIRE(p.nbig[a] > 0, "nb_big_bricks must be > 0");
        }
        p.B = vol->brick_size;
        p.c = vol->covering;
        p.Beff = p.B - 2 * p.c;
        p.eb = vol->encoded_bytes;
        p.nsmall = static_cast<uint64_t>(p.nbig[0] * p.BB[0]) * (p.nbig[1] * p.BB[1]) * (p.nbig[2] * p.BB[2]);
        // 16-byte row chunks: whole chunks per brick row, rows 16 bytes apart
        // in the level (so every row of a brick has the same alignment), and
        // both buffers 16-byte aligned
        GC_REQUIRE(p.nsmall < (1ull << 32), "too many bricks in one level");
        p.fast = (p.eb == 1 || p.eb == 2 || p.eb == 4) && (p.B & (p.B - 1)) == 0 && (p.B * p.eb) % 16 == 0 &&
                 (static_cast<uint64_t>(p.D[0]) * p.eb) % 16 == 0 &&
                 reinterpret_cast<uintptr_t>(level) % 16 == 0 && reinterpret_cast<uintptr_t>(out) % 16 == 0;
        p.b_shift = p.cpr_shift = 0;
        while ((1u << p.b_shift) < p.B) ++p.b_shift;
        while (p.fast && (16u << p.cpr_shift) < p.B * p.eb) ++p.cpr_shift;
        if (p.fast && p.cpr_shift <= 5) {
            // runs of 32 / cpr bricks along x, one warp per run and brick row
            const uint32_t nb = 32u >> p.cpr_shift;
            const uint32_t ngx = (p.nbig[0] * p.BB[0] + nb - 1) / nb;
            const uint64_t nseg = static_cast<uint64_t>(ngx) * (p.nbig[1] * p.BB[1]) * (p.nbig[2] * p.BB[2]);
            const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>((nseg + 7) / 8,
                                                                           static_cast<uint64_t>(sm_count()) * 8));
            brick_rows_kernel<<<static_cast<unsigned>(grid), 256, 0, as_stream(stream)>>>(
                static_cast<const uint8_t *>(level), static_cast<uint8_t *>(out), p, ngx);
            GC_CUDA(cudaGetLastError());
            count_launch();
            return;
        }
        // one warp per brick: 8 warps per block, enough blocks to fill every SM
        const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>((p.nsmall + 7) / 8,
                                                                       static_cast<uint64_t>(sm_count()) * 8));
        brick_kernel<<<static_cast<unsigned>(grid), 256, 0, as_stream(stream)>>>(
            static_cast<const uint8_t *>(level), static_cast<uint8_t *>(out), p);
        GC_CUDA(cudaGetLastError());
        count_launch();
    });
}

int gc_bricks_empty(const void *bricks, uint64_t nb_big_bricks, const gc_volume_desc *vol,
                    float threshold, uint8_t *flags, void *stream) {
    return guard([&] {
        GC_REQUIRE(bricks && vol && flags, "null argument");
        validate_volume(*vol);
        const uint64_t B = vol->brick_size;
        const uint64_t values = B * B * B * vol->big_brick_size[0] * vol->big_brick_size[1] *
                                vol->big_brick_size[2] * vol->channels;
        if (nb_big_bricks == 0) return;
        const uint64_t grid = std::min<uint64_t>(nb_big_bricks, static_cast<uint64_t>(sm_count()) * 16);
        empty_kernel<<<static_cast<unsigned>(grid), 256, 0, as_stream(stream)>>>(
            static_cast<const uint8_t *>(bricks), nb_big_bricks, values, channel_bytes(*vol), threshold,
            flags);
        GC_CUDA(cudaGetLastError());
        count_launch();
    });
}

}  // extern "C"
