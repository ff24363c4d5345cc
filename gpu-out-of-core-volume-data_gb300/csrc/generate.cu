// Seeded synthetic volumes: anisotropic compact bumps ("blobs") plus three
// octaves of lattice value noise, evaluated in integer arithmetic so that the
// device kernel and any host evaluation agree bit for bit.
//
// They stand in for the reference's missing dataset (the skull volume listed
// in .MISSING_LARGE_BLOBS): the shapes, sizes and value ranges follow the
// benchmark configurations (256^3 u8 with 8 blobs, 2048^3 u16 with 32 blobs ...).
//
// Value of voxel (x, y, z), maxval = 255 or 65535:
//   blobs:  q = (sum_a dx_a^2 * k_a) >> 22     (Q16, k_a = 2^38 / (9 sigma_a^2))
//           w = 65536 - q (q < 65536),  w4 = ((w^2 >> 16)^2) >> 16
//           v += (amplitude * w4) >> 16        -- a (1 - r^2/9sigma^2)^4 bump
//   noise:  n = sum_{o=0..2} lattice_o(x,y,z) >> o   (periods 64, 32, 16; Q15 values)
//           v += n * noise_amplitude / 57344  (C integer division)
//   field 1 (independent noise channel): v = maxval/2 + noise
//   clamp to [0, maxval].
#include <cmath>
#include <cstring>
#include <vector>

#include "gc_internal.h"

namespace gc {

__host__ __device__ inline uint32_t lattice_hash(int32_t ix, int32_t iy, int32_t iz, uint32_t octave,
                                                 uint32_t seed) {
    uint32_t h = seed * 0x9E3779B1u;
    h ^= static_cast<uint32_t>(ix) * 0x85EBCA77u;
    h = (h << 13) | (h >> 19);
    h ^= static_cast<uint32_t>(iy) * 0xC2B2AE3Du;
    h = (h << 11) | (h >> 21);
    h ^= static_cast<uint32_t>(iz) * 0x27D4EB2Fu;
    h ^= octave * 0x165667B1u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h;
}

__host__ __device__ inline int64_t lattice_value(int32_t ix, int32_t iy, int32_t iz, uint32_t o,
                                                 uint32_t seed) {
    return static_cast<int64_t>(lattice_hash(ix, iy, iz, o, seed) >> 16) - 32768;  // Q15
}

__host__ __device__ inline int64_t lerp_q16(int64_t a, int64_t b, int64_t w) {
    return a + (((b - a) * w) >> 16);
}

// Trilinear value noise of period 2^lp voxels.
__host__ __device__ inline int64_t value_noise(uint32_t x, uint32_t y, uint32_t z, uint32_t lp,
                                               uint32_t o, uint32_t seed) {
    const int32_t ix = static_cast<int32_t>(x >> lp), iy = static_cast<int32_t>(y >> lp),
                  iz = static_cast<int32_t>(z >> lp);
    const uint32_t mask = (1u << lp) - 1u;
    const int64_t wx = static_cast<int64_t>(x & mask) << (16 - lp);
    const int64_t wy = static_cast<int64_t>(y & mask) << (16 - lp);
    const int64_t wz = static_cast<int64_t>(z & mask) << (16 - lp);
    int64_t c00 = lerp_q16(lattice_value(ix, iy, iz, o, seed), lattice_value(ix + 1, iy, iz, o, seed), wx);
    int64_t c10 = lerp_q16(lattice_value(ix, iy + 1, iz, o, seed), lattice_value(ix + 1, iy + 1, iz, o, seed), wx);
    int64_t c01 = lerp_q16(lattice_value(ix, iy, iz + 1, o, seed), lattice_value(ix + 1, iy, iz + 1, o, seed), wx);
    int64_t c11 = lerp_q16(lattice_value(ix, iy + 1, iz + 1, o, seed),
                           lattice_value(ix + 1, iy + 1, iz + 1, o, seed), wx);
    int64_t c0 = lerp_q16(c00, c10, wy);
    int64_t c1 = lerp_q16(c01, c11, wy);
    return lerp_q16(c0, c1, wz);
}

__host__ __device__ inline int64_t noise3(uint32_t x, uint32_t y, uint32_t z, uint32_t seed,
                                          int32_t amplitude) {
    int64_t n = value_noise(x, y, z, 6, 0, seed) + (value_noise(x, y, z, 5, 1, seed) >> 1) +
                (value_noise(x, y, z, 4, 2, seed) >> 2);
    return (n * amplitude) / 57344;
}

__host__ __device__ inline int64_t blob_q16(const gc_blob &b, int64_t dx, int64_t dy, int64_t dz) {
    uint64_t s = static_cast<uint64_t>(dx * dx) * b.k[0] + static_cast<uint64_t>(dy * dy) * b.k[1] +
                 static_cast<uint64_t>(dz * dz) * b.k[2];
    return static_cast<int64_t>(s >> 22);
}

__host__ __device__ inline int64_t blob_value(const gc_blob &b, int64_t q) {
    if (q >= 65536) return 0;
    int64_t w = 65536 - q;
    int64_t w2 = (w * w) >> 16;
    int64_t w4 = (w2 * w2) >> 16;
    return (static_cast<int64_t>(b.amplitude) * w4) >> 16;
}

constexpr int kMaxBlobs = 64;
__constant__ gc_blob c_blobs[kMaxBlobs];

struct GenParams {
    uint32_t X, Y, Z;
    uint32_t bpc, channels, channel, field, seed;
    int32_t noise_amp;
    uint32_t nblobs;
    int32_t maxval;
};

// One warp per (y, z) row segment of 32 * kPerThread voxels; the y/z part of
// each blob is evaluated once per row.
constexpr int kPerThread = 4;
__global__ void __launch_bounds__(256) generate_kernel(void *dst, GenParams p) {
    const uint32_t row = blockIdx.x;  // y + z * Y
    const uint32_t y = row % p.Y, z = row / p.Y;
    const uint32_t x0 = (blockIdx.y * blockDim.x + threadIdx.x) * kPerThread;
    if (x0 >= p.X) return;
    int64_t acc[kPerThread];
    for (int i = 0; i < kPerThread; ++i) acc[i] = 0;
    if (p.field == 0) {
        for (uint32_t bi = 0; bi < p.nblobs; ++bi) {
            const gc_blob &b = c_blobs[bi];
            const int64_t dy = static_cast<int64_t>(y) - b.cy, dz = static_cast<int64_t>(z) - b.cz;
            if (dy > b.r[1] || -dy > b.r[1] || dz > b.r[2] || -dz > b.r[2]) continue;
            const uint64_t syz = static_cast<uint64_t>(dy * dy) * b.k[1] + static_cast<uint64_t>(dz * dz) * b.k[2];
            if ((syz >> 22) >= 65536) continue;
#pragma unroll
            for (int i = 0; i < kPerThread; ++i) {
                const int64_t dx = static_cast<int64_t>(x0 + i) - b.cx;
                const uint64_t s = static_cast<uint64_t>(dx * dx) * b.k[0] + syz;
                acc[i] += blob_value(b, static_cast<int64_t>(s >> 22));
            }
        }
    }
#pragma unroll
    for (int i = 0; i < kPerThread; ++i) {
        const uint32_t x = x0 + i;
        if (x >= p.X) break;
        int64_t v = acc[i] + noise3(x, y, z, p.seed, p.noise_amp);
        if (p.field == 1) v += p.maxval / 2;
        v = v < 0 ? 0 : (v > p.maxval ? p.maxval : v);
        const uint64_t idx = ((static_cast<uint64_t>(z) * p.Y + y) * p.X + x) * p.channels + p.channel;
        if (p.bpc == 1)
            static_cast<uint8_t *>(dst)[idx] = static_cast<uint8_t>(v);
        else
            static_cast<uint16_t *>(dst)[idx] = static_cast<uint16_t>(v);
    }
}

static inline uint64_t splitmix64(uint64_t &s) {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline double unit(uint64_t &s) { return static_cast<double>(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace gc

using namespace gc;

extern "C" {

int gc_generator_blobs(uint32_t seed, uint32_t nblobs, const uint32_t size[3], float sigma_min,
                       float sigma_max, int32_t amp_min, int32_t amp_max, gc_blob *out) {
    return guard([&] {
        GC_REQUIRE(size && out, "null argument");
        GC_REQUIRE(sigma_min >= 1 && sigma_max >= sigma_min, "bad sigma range");
        GC_REQUIRE(amp_max >= amp_min && amp_min >= 0, "bad amplitude range");
        uint64_t s = 0x5DEECE66Dull ^ (static_cast<uint64_t>(seed) << 17) ^ seed;
        for (uint32_t i = 0; i < nblobs; ++i) {
            gc_blob b;
            std::memset(&b, 0, sizeof(b));
            b.cx = static_cast<int32_t>(unit(s) * size[0]);
            b.cy = static_cast<int32_t>(unit(s) * size[1]);
            b.cz = static_cast<int32_t>(unit(s) * size[2]);
            for (int a = 0; a < 3; ++a) {
                double sigma = sigma_min + unit(s) * (sigma_max - sigma_min);
                b.k[a] = static_cast<uint64_t>(274877906944.0 / (9.0 * sigma * sigma));  // 2^38
                if (b.k[a] == 0) b.k[a] = 1;
                b.r[a] = static_cast<int32_t>(std::ceil(3.0 * sigma)) + 1;
            }
            b.amplitude = amp_min + static_cast<int32_t>(unit(s) * (amp_max - amp_min + 1));
            if (b.amplitude > amp_max) b.amplitude = amp_max;
            out[i] = b;
        }
    });
}

int gc_generate_volume(const gc_generator *gen, void *dst, void *stream) {
    return guard([&] {
        GC_REQUIRE(gen && dst, "null argument");
        GC_REQUIRE(gen->bytes_per_channel == 1 || gen->bytes_per_channel == 2,
                   "generator supports 1 or 2 bytes per channel");
        GC_REQUIRE(gen->channels >= 1 && gen->channel < gen->channels, "bad channel");
        GC_REQUIRE(gen->nblobs <= static_cast<uint32_t>(kMaxBlobs), "at most 64 blobs");
        GC_REQUIRE(gen->nblobs == 0 || gen->blobs, "null blob array");
        GC_REQUIRE(static_cast<uint64_t>(gen->size[1]) * gen->size[2] < (1ull << 31), "too many rows");
        cudaStream_t s = as_stream(stream);
        if (gen->nblobs)
            GC_CUDA(cudaMemcpyToSymbolAsync(c_blobs, gen->blobs, gen->nblobs * sizeof(gc_blob), 0,
                                            cudaMemcpyHostToDevice, s));
        GenParams p;
        p.X = gen->size[0];
        p.Y = gen->size[1];
        p.Z = gen->size[2];
        p.bpc = gen->bytes_per_channel;
        p.channels = gen->channels;
        p.channel = gen->channel;
        p.field = gen->field;
        p.seed = gen->seed;
        p.noise_amp = gen->noise_amplitude;
        p.nblobs = gen->nblobs;
        p.maxval = gen->bytes_per_channel == 1 ? 255 : 65535;
        dim3 block(256);
        dim3 grid(p.Y * p.Z, div_up(div_up(p.X, kPerThread), 256));
        GC_REQUIRE(grid.y <= 65535, "volume too wide");
        generate_kernel<<<grid, block, 0, s>>>(dst, p);
        GC_CUDA(cudaGetLastError());
        count_launch();
        // the constant bank is reused by the next call: keep calls ordered
        if (gen->nblobs) GC_CUDA(cudaStreamSynchronize(s));
    });
}

}  // extern "C"
