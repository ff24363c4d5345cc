// Per-frame cache kernels: LRU update, miss-list compaction, brick install,
// completude.
//
// LRU update.  The reference builds a bool mask (create_usage_mask,
// GcCore/src/cuda/libGPUCache/CacheManagerKernels.cu:8-29) and runs two
// thrust::copy_if over 28-byte LruContent records into a freshly allocated
// device_vector (CacheDevice.hpp:200-219): a stable partition, used slots
// first.  That is one stable 1-bit radix pass on the key "used this frame"
// (usage[slot] == timestamp).  Here the order is a list of 4-byte slot ids:
//   lru_count      : total_used = #slots with usage == ts (one read of usage)
//   lru_partition  : per 4096-item tile, ballot/popc + block scan of the used
//                    flags, decoupled look-back for the tile's exclusive
//                    prefix P, then used id -> out[P + rank], unused id at
//                    global index i -> out[total_used + i - used_before(i)].
// Miss list.  The reference compacts indexes i in [0, size - 1) with
// req[i] == ts with thrust::copy_if over a counting iterator into a full-size
// size_t vector, keeps the first 50 and decodes them with coord_1D_to_3D
// (CacheManager.hpp:409-474, CacheManagerKernels.cu:32-72).  miss_compact
// does the scan, cap and decode in one pass with the same look-back scan.
// Every look-back wait is bounded; on expiry the kernel sets ScanCtl::err.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "cache.cuh"
#include "gc_internal.h"

namespace gc {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr uint32_t kTile = kThreads * kItems;
constexpr uint32_t kMaxSpins = 1u << 22;

__device__ __forceinline__ void st_release(uint64_t *p, uint64_t v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_acquire(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t &total) {
    __shared__ uint32_t warp_tot[kThreads / 32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= static_cast<uint32_t>(o)) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    uint32_t pre = 0, tot = 0;
#pragma unroll
    for (uint32_t w = 0; w < kThreads / 32; ++w) {
        const uint32_t t = warp_tot[w];
        pre += (w < warp) ? t : 0u;
        tot += t;
    }
    __syncthreads();
    total = tot;
    return pre + x - v;
}

// Decoupled look-back (one warp).  Status word: [63:62] flag
// (1 aggregate, 2 inclusive prefix), [61:32] launch epoch, [31:0] value.
__device__ uint32_t lookback(uint64_t *status, uint32_t tile, uint32_t agg, uint32_t epoch, uint32_t *err,
                             uint32_t silent_tile = 0xffffffffu) {
    // Called by the 32 lanes of warp 0: each round reads the statuses of the
    // 32 nearest unvisited predecessors at once (lane 0 the nearest) and sums
    // the window up to the first inclusive prefix, waiting while a tile in
    // that range has not published yet.  Returns the exclusive prefix (all
    // lanes).  silent_tile (tests of the error path only) names a tile that
    // publishes nothing, so that its successor's bounded wait runs out.
    const uint32_t lane = threadIdx.x & 31u;
    if (tile == silent_tile) return 0;
    const uint32_t ep = epoch & 0x3FFFFFFFu;
    const uint64_t E = static_cast<uint64_t>(ep) << 32;
    if (tile == 0) {
        if (lane == 0) st_release(&status[0], (2ull << 62) | E | agg);
        return 0;
    }
    if (lane == 0) st_release(&status[tile], (1ull << 62) | E | agg);
    uint32_t excl = 0;
    int64_t top = static_cast<int64_t>(tile) - 1;
    uint32_t spins = 0;
    for (;;) {
        const int64_t j = top - static_cast<int64_t>(lane);
        uint64_t s = (2ull << 62) | E;  // before tile 0: an inclusive prefix of 0
        if (j >= 0) s = ld_acquire(&status[j]);
        const uint32_t flag = static_cast<uint32_t>(s >> 62);
        const bool ready = (static_cast<uint32_t>(s >> 32) & 0x3FFFFFFFu) == ep && flag != 0;
        const uint32_t incl = __ballot_sync(0xffffffffu, ready && flag == 2);
        const uint32_t last = incl ? static_cast<uint32_t>(__ffs(incl)) - 1u : 31u;  // last lane needed
        const uint32_t need = last == 31u ? 0xffffffffu : ((2u << last) - 1u);
        if (__ballot_sync(0xffffffffu, !ready) & need) {
            if (++spins > kMaxSpins) {
                if (lane == 0) atomicOr(err, kErrLookback);
                break;
            }
            __nanosleep(64);
            continue;
        }
        excl += __reduce_add_sync(0xffffffffu, lane <= last ? static_cast<uint32_t>(s) : 0u);
        if (incl) break;
        top -= 32;
    }
    if (lane == 0) st_release(&status[tile], (2ull << 62) | E | (excl + agg));
    return excl;
}

// The last block of a launch resets the ticket so the next launch needs no memset.
__device__ __forceinline__ void finish_tile(ScanCtl *ctl) {
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&ctl->done, 1u) == gridDim.x - 1) {
            ctl->ticket = 0;
            ctl->done = 0;
            __threadfence();
        }
    }
}

__global__ void __launch_bounds__(256) lru_count_kernel(const uint32_t *__restrict__ usage, uint32_t n,
                                                        uint32_t ts, uint32_t *__restrict__ count) {
    uint32_t c = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        c += (usage[i] == ts) ? 1u : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

__global__ void __launch_bounds__(kThreads) lru_partition_kernel(const uint32_t *__restrict__ order_in,
                                                                 uint32_t *__restrict__ order_out,
                                                                 const uint32_t *__restrict__ usage,
                                                                 uint32_t ts, uint32_t n,
                                                                 const uint32_t *__restrict__ count,
                                                                 uint64_t *status, ScanCtl *ctl,
                                                                 uint32_t epoch) {
    __shared__ uint32_t s_tile, s_excl;
    if (threadIdx.x == 0) s_tile = atomicAdd(&ctl->ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t base = static_cast<uint64_t>(tile) * kTile + threadIdx.x * kItems;
    uint32_t ids[kItems];
    uint32_t flags = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const uint64_t i = base + k;
        ids[k] = 0;
        if (i < n) {
            ids[k] = order_in[i];
            flags |= (usage[ids[k]] == ts ? 1u : 0u) << k;
        }
    }
    uint32_t tile_total;
    const uint32_t excl_thread = block_exclusive_scan(__popc(flags), tile_total);
    if (threadIdx.x < 32) {
        const uint32_t e = lookback(status, tile, tile_total, epoch, &ctl->err);
        if (threadIdx.x == 0) s_excl = e;
    }
    __syncthreads();
    const uint32_t total_used = *count;
    uint32_t used_before = s_excl + excl_thread;
    bool bad = false;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const uint64_t i = base + k;
        if (i < n) {
            const uint64_t dst = ((flags >> k) & 1u) ? used_before
                                                     : static_cast<uint64_t>(total_used) + i - used_before;
            if ((flags >> k) & 1u) ++used_before;
            if (dst < n)
                order_out[dst] = ids[k];
            else
                bad = true;  // only after a failed look-back
        }
    }
    if (bad) atomicOr(&ctl->err, kErrLookback);
    finish_tile(ctl);
}

__device__ __forceinline__ uint4 decode_request(uint64_t i, uint32_t mx, uint32_t my, const LevelTables &lt) {
    const uint64_t xy = static_cast<uint64_t>(mx) * my;
    const uint32_t z = static_cast<uint32_t>(i / xy);
    const uint64_t r = i - static_cast<uint64_t>(z) * xy;
    const uint32_t y = static_cast<uint32_t>(r / mx);
    const uint32_t x = static_cast<uint32_t>(r - static_cast<uint64_t>(y) * mx);
    uint32_t sum = 0, level = 0;
    for (level = 0; level < lt.nlevels; ++level) {
        sum += lt.nb[level][0];
        if (x < sum) break;
    }
    if (level >= lt.nlevels) level = lt.nlevels - 1;
    return make_uint4(x - (sum - lt.nb[level][0]), y, z, level);
}

__global__ void __launch_bounds__(kThreads) miss_compact_kernel(const uint32_t *__restrict__ req, uint64_t nscan,
                                                                uint32_t ts, uint32_t maxreq,
                                                                uint4 *__restrict__ list, const LevelTables lt,
                                                                uint32_t mx, uint32_t my, uint64_t *status,
                                                                ScanCtl *ctl, uint32_t epoch, uint32_t silent_tile) {
    __shared__ uint32_t s_tile, s_excl;
    if (threadIdx.x == 0) s_tile = atomicAdd(&ctl->ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t base = static_cast<uint64_t>(tile) * kTile + threadIdx.x * kItems;
    uint32_t flags = 0;
    if (base + kItems <= nscan) {
        const uint4 *p = reinterpret_cast<const uint4 *>(req + base);
#pragma unroll
        for (int q = 0; q < kItems / 4; ++q) {
            const uint4 v = __ldcs(p + q);
            flags |= ((v.x == ts) ? 1u : 0u) << (4 * q);
            flags |= ((v.y == ts) ? 1u : 0u) << (4 * q + 1);
            flags |= ((v.z == ts) ? 1u : 0u) << (4 * q + 2);
            flags |= ((v.w == ts) ? 1u : 0u) << (4 * q + 3);
        }
    } else {
#pragma unroll
        for (int k = 0; k < kItems; ++k)
            if (base + k < nscan) flags |= ((req[base + k] == ts) ? 1u : 0u) << k;
    }
    uint32_t tile_total;
    const uint32_t excl_thread = block_exclusive_scan(__popc(flags), tile_total);
    if (threadIdx.x < 32) {
        const uint32_t e = lookback(status, tile, tile_total, epoch, &ctl->err, silent_tile);
        if (threadIdx.x == 0) s_excl = e;
    }
    __syncthreads();
    uint32_t rank = s_excl + excl_thread;
    if (flags && rank < maxreq) {
        for (int k = 0; k < kItems && rank < maxreq; ++k) {
            if ((flags >> k) & 1u) list[rank++] = decode_request(base + k, mx, my, lt);
        }
    }
    if (threadIdx.x == 0 && tile == gridDim.x - 1) ctl->total = s_excl + tile_total;
    finish_tile(ctl);
}

// ---------------------------------------------------------------------------
// Brick install (CacheManager::load_new_bricks, CacheManager.hpp:502-632).

// MRPD coordinate of a normalized brick origin (K_MultiResolutionPageDirectory::set,
// K_MultiResolutionPageDirectory.hpp:193-205).
__device__ __forceinline__ uint64_t mrpd_index(const LevelTables &lt, uint32_t level, float vx, float vy, float vz,
                                               uint32_t mx, uint32_t my) {
    const uint32_t x = lt.off[level] + static_cast<uint32_t>(__fmul_rn(vx, static_cast<float>(lt.nb[level][0])));
    const uint32_t y = static_cast<uint32_t>(__fmul_rn(vy, static_cast<float>(lt.nb[level][1])));
    const uint32_t z = static_cast<uint32_t>(__fmul_rn(vz, static_cast<float>(lt.nb[level][2])));
    return x + static_cast<uint64_t>(y) * mx + static_cast<uint64_t>(z) * mx * my;
}
// The same brick as (x inside the level, y, z): its place in a two-level directory.
__device__ __forceinline__ uint3 brick_at(const LevelTables &lt, uint32_t level, float vx, float vy, float vz) {
    return make_uint3(static_cast<uint32_t>(__fmul_rn(vx, static_cast<float>(lt.nb[level][0]))),
                      static_cast<uint32_t>(__fmul_rn(vy, static_cast<float>(lt.nb[level][1]))),
                      static_cast<uint32_t>(__fmul_rn(vz, static_cast<float>(lt.nb[level][2]))));
}
__device__ __forceinline__ bool brick_inside(const LevelTables &lt, uint32_t level, uint3 q) {
    return q.x < lt.nb[level][0] && q.y < lt.nb[level][1] && q.z < lt.nb[level][2];
}
// The brick entry of q in a two-level directory, or null when its block is
// not resident.
__device__ __forceinline__ uint4 *pt_entry_of(const PageTable &pt, const LevelTables &lt, uint32_t level, uint3 q) {
    const uint32_t t = pt.top[pt_word(pt, lt, level, q.x, q.y, q.z)];
    if (!(t & 1u)) return nullptr;
    return pt.table + pt_entry(pt, t >> 1, pt_local(pt, q.x, q.y, q.z));
}
// Page-directory entry (x, y, z, 1) of pool slot `slot`.
__device__ __forceinline__ uint4 slot_entry(uint32_t slot, uint32_t sx, uint32_t sy, uint32_t B) {
    return make_uint4((slot % sx) * B, ((slot / sx) % sy) * B, (slot / (sx * sy)) * B, 1u);
}

// compute_volume_position (CacheManagerKernels.cu:75-86):
// x / (V.x * (1 / (B - 2c))) + FLT_EPSILON.
__device__ __forceinline__ float4 brick_origin(const LevelTables &lt, uint4 b, float one_over_beff) {
    const float eps = 1.1920928955078125e-7f;
    float4 v;
    v.x = __fadd_rn(__fdiv_rn(static_cast<float>(b.x), __fmul_rn(static_cast<float>(lt.vvox[b.w][0]), one_over_beff)), eps);
    v.y = __fadd_rn(__fdiv_rn(static_cast<float>(b.y), __fmul_rn(static_cast<float>(lt.vvox[b.w][1]), one_over_beff)), eps);
    v.z = __fadd_rn(__fdiv_rn(static_cast<float>(b.z), __fmul_rn(static_cast<float>(lt.vvox[b.w][2]), one_over_beff)), eps);
    v.w = 0.f;
    return v;
}

// dereference_old_bricks (CacheManagerKernels.hpp:115-145) for the LRU tail.
__global__ void install_evict_kernel(InstallArgs a, const LevelTables lt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_nonempty) return;
    const uint32_t slot = a.order[a.nslots - a.n_nonempty + i];
    const float4 vp = a.slot_vpos[slot];
    if (vp.x < 0.f) return;  // slot never held a brick
    const uint32_t level = a.slot_level[slot];
    const uint64_t e = mrpd_index(lt, level, vp.x, vp.y, vp.z, a.mx, a.my);
    if (e >= a.nentries) return;
    if (a.pt.shift) {
        // Two levels: the entry is cleared only where it still names this
        // slot -- after its block was evicted the brick may be unreachable,
        // or resident again in another slot.
        const uint3 q = brick_at(lt, level, vp.x, vp.y, vp.z);
        if (!brick_inside(lt, level, q)) return;
        uint4 *pe = pt_entry_of(a.pt, lt, level, q);
        if (!pe) return;
        const uint4 cur = *pe, mine = slot_entry(slot, a.sx, a.sy, a.B);
        if (cur.w != 1u || cur.x != mine.x || cur.y != mine.y || cur.z != mine.z) return;
        *pe = make_uint4(0, 0, 0, 0);
    } else {
        a.mrpd[e] = make_uint4(0, 0, 0, 0);
    }
    a.entry_bins[e] = a.user_bins ? a.user_bins[e] : ~0ull;
}

// Value range of a brick as value bins (empty-space skipping): min and max
// over its voxels (covering included), normalized like the samplers, widened
// by one bin on either side.  `at(v)` gives the address of voxel v; one
// block per brick (up to 256 threads); the result is valid in thread 0.
// The block's value bins from each thread's min and max (normalized like the
// samplers); the result is valid in thread 0.
__device__ unsigned long long block_bins_from(float lo, float hi) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    __shared__ float s_lo[8], s_hi[8];
    const uint32_t warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31u) == 0) {
        s_lo[warp] = lo;
        s_hi[warp] = hi;
    }
    __syncthreads();
    unsigned long long bins = 0;
    if (threadIdx.x == 0) {
        for (uint32_t w = 1; w < (blockDim.x + 31) / 32; ++w) {
            lo = fminf(lo, s_lo[w]);
            hi = fmaxf(hi, s_hi[w]);
        }
        auto bin = [](float x) {
            const float f = floorf(x * static_cast<float>(kValueBins));
            return f < 0.f ? 0 : (f > kValueBins - 1.f ? static_cast<int>(kValueBins) - 1 : static_cast<int>(f));
        };
        const int b0 = max(bin(lo) - 1, 0), b1 = min(bin(hi) + 1, static_cast<int>(kValueBins) - 1);
        const unsigned long long upto = b1 >= 63 ? ~0ull : ((1ull << (b1 + 1)) - 1ull);
        bins = upto & ~((1ull << b0) - 1ull);
    }
    return bins;
}
template <class At>
__device__ unsigned long long block_value_bins(uint32_t nvox, uint32_t eb, At at) {
    float lo = 3.4e38f, hi = -3.4e38f;
    for (uint32_t v = threadIdx.x; v < nvox; v += blockDim.x) {
        const uint8_t *p = at(v);
        float x;
        if (eb == 1)
            x = static_cast<float>(*p) * (1.0f / 255.0f);
        else if (eb == 2)
            x = static_cast<float>(*reinterpret_cast<const uint16_t *>(p)) * (1.0f / 65535.0f);
        else
            x = *reinterpret_cast<const float *>(p);
        lo = fminf(lo, x);
        hi = fmaxf(hi, x);
    }
    return block_bins_from(lo, hi);
}

// Min and max over the voxels of a 16-byte chunk, into (lo, hi) as the
// samplers normalize them (integer min / max first: the normalization is
// monotone, so the result is block_value_bins').
__device__ __forceinline__ void chunk_range(uint4 c, uint32_t eb, float &lo, float &hi) {
    if (eb == 1) {
        const uint32_t mn = __vminu4(__vminu4(c.x, c.y), __vminu4(c.z, c.w));
        const uint32_t mx = __vmaxu4(__vmaxu4(c.x, c.y), __vmaxu4(c.z, c.w));
        const uint32_t mn1 = min(min(mn & 0xffu, (mn >> 8) & 0xffu), min((mn >> 16) & 0xffu, mn >> 24));
        const uint32_t mx1 = max(max(mx & 0xffu, (mx >> 8) & 0xffu), max((mx >> 16) & 0xffu, mx >> 24));
        lo = fminf(lo, static_cast<float>(mn1) * (1.0f / 255.0f));
        hi = fmaxf(hi, static_cast<float>(mx1) * (1.0f / 255.0f));
    } else if (eb == 2) {
        const uint32_t mn = __vminu2(__vminu2(c.x, c.y), __vminu2(c.z, c.w));
        const uint32_t mx = __vmaxu2(__vmaxu2(c.x, c.y), __vmaxu2(c.z, c.w));
        lo = fminf(lo, static_cast<float>(min(mn & 0xffffu, mn >> 16)) * (1.0f / 65535.0f));
        hi = fmaxf(hi, static_cast<float>(max(mx & 0xffffu, mx >> 16)) * (1.0f / 65535.0f));
    } else {
        lo = fminf(fminf(lo, fminf(__uint_as_float(c.x), __uint_as_float(c.y))),
                   fminf(__uint_as_float(c.z), __uint_as_float(c.w)));
        hi = fmaxf(fmaxf(hi, fmaxf(__uint_as_float(c.x), __uint_as_float(c.y))),
                   fmaxf(__uint_as_float(c.z), __uint_as_float(c.w)));
    }
}

// Value bins of every brick of one level, read from the level's big bricks
// on the device: the mask the install computes for the same brick in a pool
// slot.  One block per brick of the level's brick grid (x fastest).
__global__ void __launch_bounds__(256) brick_bins_kernel(const uint8_t *__restrict__ level, uint32_t nbx, uint32_t nby,
                                                         uint32_t nbz, uint32_t gbx, uint32_t gby, uint32_t bb0,
                                                         uint32_t bb1, uint32_t bb2, uint32_t B, uint32_t eb,
                                                         unsigned long long *bins) {
    const uint64_t i = blockIdx.x;
    const uint32_t x = static_cast<uint32_t>(i % nbx), y = static_cast<uint32_t>((i / nbx) % nby),
                   z = static_cast<uint32_t>(i / (static_cast<uint64_t>(nbx) * nby));
    if (z >= nbz) return;
    const uint32_t gx = x / bb0, gy = y / bb1, gz = z / bb2;
    const uint32_t bvx = bb0 * B, bvy = bb1 * B, bvz = bb2 * B;
    const uint8_t *big =
        level + ((static_cast<uint64_t>(gz) * gby + gy) * gbx + gx) * (static_cast<uint64_t>(bvx) * bvy * bvz * eb);
    const uint32_t ox = (x - gx * bb0) * B, oy = (y - gy * bb1) * B, oz = (z - gz * bb2) * B;
    const unsigned long long m = block_value_bins(B * B * B, eb, [&](uint32_t v) {
        const uint32_t lx = v % B, ly = (v / B) % B, lz = v / (B * B);
        return big + ((static_cast<uint64_t>(oz + lz) * bvy + (oy + ly)) * bvx + (ox + lx)) * eb;
    });
    if (threadIdx.x == 0) bins[i] = m;
}

void launch_brick_bins(const uint8_t *level, const uint32_t nb[3], const uint32_t nbig[3], const uint32_t bb[3],
                       uint32_t B, uint32_t eb, unsigned long long *bins, cudaStream_t s) {
    const uint64_t n = static_cast<uint64_t>(nb[0]) * nb[1] * nb[2];
    if (n == 0) return;
    GC_REQUIRE(n < (1ull << 31), "too many bricks in one level");
    brick_bins_kernel<<<static_cast<uint32_t>(n), 256, 0, s>>>(level, nb[0], nb[1], nb[2], nbig[0], nbig[1], bb[0],
                                                              bb[1], bb[2], B, eb, bins);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

// compute_lru_volume_position + copy_lru_position + write_brick
// (CacheManagerKernels.cu:90-114, CacheManagerKernels.hpp:59-107): one block
// per non-empty brick copies B^3 voxels from the staged big brick into the
// LRU-tail slot, 16 bytes at a time when rows allow it.
__global__ void __launch_bounds__(256) install_place_kernel(InstallArgs a, const LevelTables lt, float one_over_beff) {
    const uint32_t i = blockIdx.x;
    if (i >= a.n_nonempty) return;
    const uint4 b = a.asked[i];
    const uint32_t slot = a.order[a.nslots - a.n_nonempty + i];
    if (threadIdx.x == 0) {
        a.slot_level[slot] = b.w;
        a.slot_vpos[slot] = brick_origin(lt, b, one_over_beff);
    }
    // the brick's volume: voxel width and big-brick shape of its level
    const uint32_t B = a.B, eb = lt.eb[b.w];
    const uint32_t *BB = lt.bb[b.w];
    const uint32_t bvx = BB[0] * B, bvy = BB[1] * B;
    const uint32_t bi = a.big_index[i];
    const uint4 bc = a.big_coord[bi];
    const uint32_t ox = (b.x - bc.x * BB[0]) * B, oy = (b.y - bc.y * BB[1]) * B, oz = (b.z - bc.z * BB[2]) * B;
    const uint8_t *src = a.staging + bi * a.big_stride;
    uint8_t *dst = a.pool + static_cast<uint64_t>(slot) * a.slot_bytes;
    const uint32_t row_bytes = B * eb;
    const uint32_t rows = B * B;
    const uint32_t vec_per_row = row_bytes / 16;
    const bool pow2 = (B & (B - 1u)) == 0u && (vec_per_row & (vec_per_row - 1u)) == 0u;
    if (row_bytes % 16 == 0 && pow2 && (reinterpret_cast<uintptr_t>(src) % 16 == 0) && ((bvx * eb) % 16 == 0)) {
        // 16-byte chunks, four loads in flight per thread before their
        // stores; the brick's value range is taken from the loaded chunks
        // (one read of the brick for both)
        const uint32_t qs = __ffs(vec_per_row) - 1u, bs = __ffs(B) - 1u;
        const uint32_t nvec = rows * vec_per_row;
        const bool bins = a.slot_bins && a.nc == 1;
        float lo = 3.4e38f, hi = -3.4e38f;
        for (uint32_t v0 = threadIdx.x; v0 < nvec; v0 += 4u * blockDim.x) {
            uint4 val[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t v = v0 + u * blockDim.x;
                if (v < nvec) {
                    const uint32_t r = v >> qs, q = v & (vec_per_row - 1u);
                    const uint32_t ly = r & (B - 1u), lz = r >> bs;
                    const uint64_t soff =
                        ((static_cast<uint64_t>(oz + lz) * bvy + (oy + ly)) * bvx + ox) * eb + q * 16u;
                    val[u] = __ldcs(reinterpret_cast<const uint4 *>(src + soff));
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t v = v0 + u * blockDim.x;
                if (v < nvec) {
                    reinterpret_cast<uint4 *>(dst)[v] = val[u];
                    if (bins) chunk_range(val[u], eb, lo, hi);
                }
            }
        }
        if (!a.slot_bins) return;
        if (a.nc != 1) {
            if (threadIdx.x == 0) a.slot_bins[slot] = ~0ull;  // several channels: never skipped
            return;
        }
        const unsigned long long b2 = block_bins_from(lo, hi);
        if (threadIdx.x == 0) a.slot_bins[slot] = b2;
        return;
    } else {
        const uint32_t nbytes = rows * row_bytes;
        for (uint32_t v = threadIdx.x; v < nbytes; v += blockDim.x) {
            const uint32_t r = v / row_bytes, q = v % row_bytes;
            const uint32_t ly = r % B, lz = r / B;
            const uint64_t soff = ((static_cast<uint64_t>(oz + lz) * bvy + (oy + ly)) * bvx + ox) * eb + q;
            dst[v] = src[soff];
        }
    }
    if (!a.slot_bins) return;
    __syncthreads();
    if (a.nc != 1) {
        if (threadIdx.x == 0) a.slot_bins[slot] = ~0ull;  // several channels: never skipped
        return;
    }
    const unsigned long long bins = block_value_bins(B * B * B, eb, [&](uint32_t v) { return dst + v * eb; });
    if (threadIdx.x == 0) a.slot_bins[slot] = bins;
}

// reference_new_bricks (CacheManagerKernels.hpp:308-357) for the MRPD-only
// hierarchy: in list order (non-empty first), an unmapped entry becomes
// {slot position, 1} or {0, 0, 0, 2} for an empty brick; an entry that is
// already mapped or empty is left alone.  The reference walks the list in one
// thread; here each brick is one thread, and a brick whose MRPD entry also
// belongs to an earlier list element yields to it, which is the serial order:
// the first pass leaves the lowest list index naming each entry in `owner`,
// the second lets only that element act (and puts the owner word back).
__global__ void install_owner_kernel(InstallArgs a, const LevelTables lt, float one_over_beff) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const uint4 b = a.asked[i];
    const float4 v = brick_origin(lt, b, one_over_beff);
    const uint64_t c = mrpd_index(lt, b.w, v.x, v.y, v.z, a.mx, a.my);
    a.coords[i] = c;
    if (c < a.nentries) atomicMin(a.owner + c, i);
}

__global__ void install_reference_kernel(InstallArgs a, const LevelTables lt, float one_over_beff) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const uint64_t c = a.coords[i];
    if (c >= a.nentries || a.owner[c] != i) return;  // an earlier element names the same entry
    a.owner[c] = 0xffffffffu;  // later readers see a value that is not their index either way
    uint4 *pe = a.mrpd + c;
    if (a.pt.shift) {
        // two levels: the entry lives in the block of its directory word (none
        // when the table pool had no slot left for it: the brick stays unmapped)
        const uint4 b = a.asked[i];
        const float4 v = brick_origin(lt, b, one_over_beff);
        const uint3 q = brick_at(lt, b.w, v.x, v.y, v.z);
        if (!brick_inside(lt, b.w, q)) return;
        pe = pt_entry_of(a.pt, lt, b.w, q);
        if (!pe) return;
    }
    const uint4 e = *pe;
    if (e.w == 1u || e.w == 2u) return;  // mapped or empty already (3 = in flight: install it)
    if (i < a.n_nonempty) {
        const uint32_t slot = a.order[a.nslots - a.n_nonempty + i];
        *pe = slot_entry(slot, a.sx, a.sy, a.B);
        a.entry_bins[c] = a.slot_bins[slot];
    } else {
        *pe = make_uint4(0, 0, 0, 2u);
    }
}

// Two-level directory: table blocks for the new bricks.  Each element that
// acts for its entry (the owner) and whose directory word has no block claims
// the word; the lowest element index wins.
__global__ void install_pt_claim_kernel(InstallArgs a, const LevelTables lt, float one_over_beff) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    uint32_t word = 0xffffffffu;
    const uint64_t c = a.coords[i];
    if (c < a.nentries && a.owner[c] == i) {
        const uint4 b = a.asked[i];
        const float4 v = brick_origin(lt, b, one_over_beff);
        const uint3 q = brick_at(lt, b.w, v.x, v.y, v.z);
        const uint32_t w = pt_word(a.pt, lt, b.w, q.x, q.y, q.z);
        if (brick_inside(lt, b.w, q) && !(a.pt.top[w] & 1u)) {
            word = w;
            atomicMin(a.pt_claim + w, i);
        }
    }
    a.pt_word_of[i] = word;
}

// The claimed words in list order (one block): the k-th winner gets the k-th
// of the table slots taken from the LRU tail.
__global__ void __launch_bounds__(1024) install_pt_rank_kernel(InstallArgs a) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_base;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    if (threadIdx.x == 0) s_base = 0;
    __syncthreads();
    for (uint32_t i0 = 0; i0 < a.n; i0 += blockDim.x) {
        const uint32_t i = i0 + threadIdx.x;
        const uint32_t w = i < a.n ? a.pt_word_of[i] : 0xffffffffu;
        const bool win = w != 0xffffffffu && a.pt_claim[w] == i;
        const uint32_t bal = __ballot_sync(0xffffffffu, win);
        if (lane == 0) s_warp[warp] = __popc(bal);
        __syncthreads();
        uint32_t before = s_base;
        for (uint32_t k = 0; k < warp; ++k) before += s_warp[k];
        if (win) a.pt_jobs[before + __popc(bal & ((1u << lane) - 1u))] = make_uint2(w, i);
        __syncthreads();
        if (threadIdx.x == 0)
            for (uint32_t k = 0; k < nwarps; ++k) s_base += s_warp[k];
        __syncthreads();
    }
    if (threadIdx.x == 0) *a.pt_njobs = s_base;
}

// One block per claimed word: the table slot at LRU-tail position k leaves
// the block it held (its directory word cleared, the value bins of its mapped
// entries reverted), is cleared and takes the claimed word.  Claims beyond
// the table pool's size get no slot.
__global__ void __launch_bounds__(256) install_pt_apply_kernel(InstallArgs a, const LevelTables lt,
                                                               float one_over_beff) {
    const uint32_t m = *a.pt_njobs, k = blockIdx.x;
    if (k >= m) return;
    const uint2 job = a.pt_jobs[k];
    const uint32_t npt = min(m, a.pt_slots);
    if (k >= npt) {
        if (threadIdx.x == 0) a.pt_claim[job.x] = 0xffffffffu;
        return;
    }
    const uint32_t slot = a.pt_order[a.pt_slots - npt + k];
    const uint32_t P = 1u << a.pt.shift, P3 = P * P * P;
    uint4 *blk = a.pt.table + pt_entry(a.pt, slot, 0);
    const uint4 old = a.pt_keys[slot];
    if (old.w != 0xffffffffu) {
        for (uint32_t j = threadIdx.x; j < P3; j += blockDim.x) {
            if (blk[j].w != 1u) continue;
            const uint32_t dx = j & (P - 1u), dy = (j >> a.pt.shift) & (P - 1u), dz = j >> (2u * a.pt.shift);
            const uint64_t e = static_cast<uint64_t>(lt.off[old.w] + old.x + dx) +
                               static_cast<uint64_t>(old.y + dy) * a.mx +
                               static_cast<uint64_t>(old.z + dz) * a.mx * a.my;
            a.entry_bins[e] = a.user_bins ? a.user_bins[e] : ~0ull;
        }
    }
    __syncthreads();  // the old entries are read before they are cleared
    for (uint32_t j = threadIdx.x; j < P3; j += blockDim.x) blk[j] = make_uint4(0, 0, 0, 0);
    if (threadIdx.x == 0) {
        if (old.w != 0xffffffffu) a.pt.top[pt_word(a.pt, lt, old.w, old.x, old.y, old.z)] = 0u;
        const uint4 b = a.asked[job.y];
        const float4 v = brick_origin(lt, b, one_over_beff);
        const uint3 q = brick_at(lt, b.w, v.x, v.y, v.z);
        const uint32_t msk = ~(P - 1u);
        a.pt_keys[slot] = make_uint4(q.x & msk, q.y & msk, q.z & msk, b.w);
        a.pt.top[job.x] = slot << 1 | 1u;
        a.pt_claim[job.x] = 0xffffffffu;
    }
}

__global__ void __launch_bounds__(256) completude_kernel(const float4 *__restrict__ vpos, uint32_t n,
                                                         uint32_t *__restrict__ count) {
    uint32_t c = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        c += (vpos[i].x != -1.f) ? 1u : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

// ---------------------------------------------------------------------------
uint32_t lookback_tiles(uint64_t n) { return static_cast<uint32_t>(std::max<uint64_t>(1, (n + kTile - 1) / kTile)); }

void launch_lru_count(const uint32_t *usage, uint32_t nslots, uint32_t ts, uint32_t *count, cudaStream_t s) {
    GC_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t), s));
    const uint32_t grid = std::min<uint32_t>(div_up(nslots, 256), static_cast<uint32_t>(sm_count()) * 4);
    lru_count_kernel<<<std::max(1u, grid), 256, 0, s>>>(usage, nslots, ts, count);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

void launch_lru_partition(const uint32_t *order_in, uint32_t *order_out, const uint32_t *usage, uint32_t ts,
                          uint32_t nslots, const uint32_t *count, uint64_t *status, ScanCtl *ctl,
                          uint32_t epoch, cudaStream_t s) {
    lru_partition_kernel<<<lookback_tiles(nslots), kThreads, 0, s>>>(order_in, order_out, usage, ts, nslots,
                                                                     count, status, ctl, epoch);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

void launch_miss_compact(const uint32_t *req, uint64_t nscan, uint32_t ts, uint32_t maxreq, uint4 *list,
                         const LevelTables &lt, uint32_t mx, uint32_t my, uint64_t *status, ScanCtl *ctl,
                         uint32_t epoch, cudaStream_t s, uint32_t silent_tile) {
    miss_compact_kernel<<<lookback_tiles(nscan), kThreads, 0, s>>>(req, nscan, ts, maxreq, list, lt, mx, my,
                                                                   status, ctl, epoch, silent_tile);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

__global__ void live_bins_kernel(const LevelTables lt, const float4 *__restrict__ slot_vpos,
                                 const uint32_t *__restrict__ slot_level,
                                 const unsigned long long *__restrict__ slot_bins, uint32_t nslots, uint32_t mx,
                                 uint32_t my, uint64_t nentries, unsigned long long *entry_bins, const PageTable pt,
                                 uint32_t sx, uint32_t sy, uint32_t B) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += gridDim.x * blockDim.x) {
        const float4 vp = slot_vpos[i];
        if (vp.x < 0.f) continue;  // slot never held a brick
        const uint32_t level = slot_level[i];
        const uint64_t e = mrpd_index(lt, level, vp.x, vp.y, vp.z, mx, my);
        if (e >= nentries) continue;
        if (pt.shift) {  // two levels: only a slot its entry names is live
            const uint3 q = brick_at(lt, level, vp.x, vp.y, vp.z);
            if (!brick_inside(lt, level, q)) continue;
            const uint4 *pe = pt_entry_of(pt, lt, level, q);
            const uint4 mine = slot_entry(i, sx, sy, B);
            if (!pe || pe->w != 1u || pe->x != mine.x || pe->y != mine.y || pe->z != mine.z) continue;
        }
        entry_bins[e] = slot_bins[i];
    }
}

void launch_live_bins(const LevelTables &lt, const float4 *slot_vpos, const uint32_t *slot_level,
                      const unsigned long long *slot_bins, uint32_t nslots, uint32_t mx, uint32_t my,
                      uint64_t nentries, unsigned long long *entry_bins, const PageTable &pt, uint32_t sx,
                      uint32_t sy, uint32_t B, cudaStream_t s) {
    const uint32_t grid = std::max(1u, std::min<uint32_t>(div_up(nslots, 256), static_cast<uint32_t>(sm_count()) * 4));
    live_bins_kernel<<<grid, 256, 0, s>>>(lt, slot_vpos, slot_level, slot_bins, nslots, mx, my, nentries, entry_bins,
                                          pt, sx, sy, B);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

void launch_install(const InstallArgs &a, const LevelTables &lt, cudaStream_t s) {
    if (a.n == 0) return;
    const float one_over_beff = 1.0f / static_cast<float>(a.Beff);
    if (a.n_nonempty) {
        install_evict_kernel<<<div_up(a.n_nonempty, 128), 128, 0, s>>>(a, lt);
        GC_CUDA(cudaGetLastError());
        count_launch();
        install_place_kernel<<<a.n_nonempty, 256, 0, s>>>(a, lt, one_over_beff);
        GC_CUDA(cudaGetLastError());
        count_launch();
    }
    install_owner_kernel<<<div_up(a.n, 256u), 256, 0, s>>>(a, lt, one_over_beff);
    GC_CUDA(cudaGetLastError());
    count_launch();
    if (a.pt.shift) {
        install_pt_claim_kernel<<<div_up(a.n, 256u), 256, 0, s>>>(a, lt, one_over_beff);
        GC_CUDA(cudaGetLastError());
        install_pt_rank_kernel<<<1, 1024, 0, s>>>(a);
        GC_CUDA(cudaGetLastError());
        install_pt_apply_kernel<<<a.n, 256, 0, s>>>(a, lt, one_over_beff);
        GC_CUDA(cudaGetLastError());
        count_launch(3);
    }
    install_reference_kernel<<<div_up(a.n, 256u), 256, 0, s>>>(a, lt, one_over_beff);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

__global__ void pt_flatten_kernel(const PageTable pt, const LevelTables lt, uint32_t mx, uint32_t my,
                                  uint64_t nentries, uint4 *out) {
    for (uint64_t e = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; e < nentries;
         e += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint32_t X = static_cast<uint32_t>(e % mx), y = static_cast<uint32_t>((e / mx) % my);
        const uint32_t z = static_cast<uint32_t>(e / (static_cast<uint64_t>(mx) * my));
        uint4 v = make_uint4(0, 0, 0, 0);
        for (uint32_t l = 0; l < lt.nlevels; ++l) {
            if (X < lt.off[l] || X >= lt.off[l] + lt.nb[l][0]) continue;
            const uint3 q = make_uint3(X - lt.off[l], y, z);
            if (brick_inside(lt, l, q)) {
                const uint32_t t = pt.top[pt_word(pt, lt, l, q.x, q.y, q.z)];
                if (t & 1u) v = pt.table[pt_entry(pt, t >> 1, pt_local(pt, q.x, q.y, q.z))];
            }
            break;
        }
        out[e] = v;
    }
}

void launch_pt_flatten(const PageTable &pt, const LevelTables &lt, uint32_t mx, uint32_t my, uint64_t nentries,
                       uint4 *out, cudaStream_t s) {
    const uint32_t grid =
        static_cast<uint32_t>(std::max<uint64_t>(1, std::min<uint64_t>((nentries + 255) / 256, sm_count() * 8ull)));
    pt_flatten_kernel<<<grid, 256, 0, s>>>(pt, lt, mx, my, nentries, out);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

__global__ void pt_init_kernel(uint32_t *order, uint4 *keys, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        order[i] = i;
        keys[i] = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
    }
}

void launch_pt_init(uint32_t *order, uint4 *keys, uint32_t nslots, cudaStream_t s) {
    pt_init_kernel<<<std::max(1u, std::min<uint32_t>(div_up(nslots, 256), 4096)), 256, 0, s>>>(order, keys, nslots);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

// Brick gather from device-readable host memory (the direct upload route):
// block-strided over bricks, each brick copied by the whole block with
// 16-byte loads when aligned.  The reads travel over the host link; the
// writes land in the device staging buffer the install kernels read.
// kIlp independent loads per thread are in flight before their stores: the
// host link's latency (microseconds) needs many bytes in flight per SM.
template <typename W, uint32_t kIlp>
__device__ __forceinline__ void gather_bricks(const ulonglong2 *__restrict__ src, uint32_t n, uint64_t stride,
                                              uint8_t *__restrict__ dst) {
    for (uint32_t b = blockIdx.x; b < n; b += gridDim.x) {
        const ulonglong2 e = src[b];  // {address, bytes}
        const W *sp = reinterpret_cast<const W *>(e.x);
        W *dp = reinterpret_cast<W *>(dst + static_cast<uint64_t>(b) * stride);
        const uint64_t words = e.y / sizeof(W);
        const uint64_t step = static_cast<uint64_t>(blockDim.x) * kIlp;
        for (uint64_t i0 = threadIdx.x; i0 < words; i0 += step) {
            W v[kIlp];
#pragma unroll
            for (uint32_t k = 0; k < kIlp; ++k) {
                const uint64_t i = i0 + static_cast<uint64_t>(k) * blockDim.x;
                if (i < words) v[k] = sp[i];
            }
#pragma unroll
            for (uint32_t k = 0; k < kIlp; ++k) {
                const uint64_t i = i0 + static_cast<uint64_t>(k) * blockDim.x;
                if (i < words) dp[i] = v[k];
            }
        }
    }
}
template <typename W>
__global__ void gather_bricks_kernel(const ulonglong2 *__restrict__ src, uint32_t n, uint64_t stride,
                                     uint8_t *__restrict__ dst) {
    gather_bricks<W, 4>(src, n, stride, dst);
}
// At most 32 registers per thread (128 threads, 16 blocks): fits beside the ray caster.
template <typename W>
__global__ void __launch_bounds__(128, 16) gather_bricks_beside_kernel(const ulonglong2 *__restrict__ src, uint32_t n,
                                                                      uint64_t stride, uint8_t *__restrict__ dst) {
    gather_bricks<W, 2>(src, n, stride, dst);
}

void launch_gather_bricks(const ulonglong2 *src, uint32_t n, uint64_t stride, uint8_t *dst, bool vec16,
                          bool beside, cudaStream_t s) {
    if (n == 0) return;
    const uint32_t sms = static_cast<uint32_t>(sm_count());
    if (beside) {
        // Next to a persistent ray-caster launch: at its occupancy each SM
        // sub-partition keeps 1024 registers free, room for one warp of 32
        // registers per thread -- 128-thread blocks (one warp per
        // sub-partition), one per SM, run during the render instead of after
        // it (two 16-byte loads in flight per thread).  A second block per
        // SM, resident before the render's blocks arrive, would hold
        // registers a ray-caster block needs.
        const uint32_t grid = std::min<uint32_t>(n, sms);
        if (vec16)
            gather_bricks_beside_kernel<uint4><<<grid, 128, 0, s>>>(src, n, stride, dst);
        else
            gather_bricks_beside_kernel<uint8_t><<<grid, 128, 0, s>>>(src, n, stride, dst);
    } else {
        // alone on the device: one block of 256 per SM (four 16-byte loads in
        // flight per thread) saturates the host link
        const uint32_t grid = std::min<uint32_t>(n, sms);
        if (vec16)
            gather_bricks_kernel<uint4><<<grid, 256, 0, s>>>(src, n, stride, dst);
        else
            gather_bricks_kernel<uint8_t><<<grid, 256, 0, s>>>(src, n, stride, dst);
    }
    GC_CUDA(cudaGetLastError());
    count_launch();
}

// In-flight marks of the batched form's overlapped loads: the entries of a
// miss list (x, y, z, level) handed to the loader are flagged 3 so that rays
// stop there without requesting them again; after the install, the entries
// still flagged (bricks that did not load) go back to 0.
__device__ __forceinline__ uint64_t list_entry_index(const LevelTables &lt, uint4 b, uint32_t mx, uint32_t my) {
    return static_cast<uint64_t>(lt.off[b.w] + b.x) + static_cast<uint64_t>(b.y) * mx +
           static_cast<uint64_t>(b.z) * mx * my;
}

__global__ void mark_in_flight_kernel(const uint4 *__restrict__ list, const ScanCtl *ctl, uint32_t maxreq,
                                      const LevelTables lt, uint32_t mx, uint32_t my, uint64_t nentries, uint4 *mrpd) {
    const uint32_t n = min(ctl->total, maxreq);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint4 b = list[i];
        if (b.w >= lt.nlevels) continue;
        const uint64_t e = list_entry_index(lt, b, mx, my);
        if (e < nentries && mrpd[e].w == 0u) mrpd[e].w = 3u;
    }
}

__global__ void unmark_in_flight_kernel(const uint4 *__restrict__ list, uint32_t n, const LevelTables lt,
                                        uint32_t mx, uint32_t my, uint64_t nentries, uint4 *mrpd) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint4 b = list[i];
        if (b.w >= lt.nlevels) continue;
        const uint64_t e = list_entry_index(lt, b, mx, my);
        if (e < nentries && mrpd[e].w == 3u) mrpd[e] = make_uint4(0, 0, 0, 0);
    }
}

void launch_mark_in_flight(const uint4 *list, const ScanCtl *ctl, uint32_t maxreq, const LevelTables &lt,
                           uint32_t mx, uint32_t my, uint64_t nentries, uint4 *mrpd, cudaStream_t s) {
    const uint32_t grid = std::max(1u, std::min<uint32_t>(div_up(maxreq, 256), static_cast<uint32_t>(sm_count()) * 2));
    mark_in_flight_kernel<<<grid, 256, 0, s>>>(list, ctl, maxreq, lt, mx, my, nentries, mrpd);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

void launch_unmark_in_flight(const uint4 *list, uint32_t n, const LevelTables &lt, uint32_t mx, uint32_t my,
                             uint64_t nentries, uint4 *mrpd, cudaStream_t s) {
    if (n == 0) return;
    const uint32_t grid = std::max(1u, std::min<uint32_t>(div_up(n, 256), static_cast<uint32_t>(sm_count()) * 2));
    unmark_in_flight_kernel<<<grid, 256, 0, s>>>(list, n, lt, mx, my, nentries, mrpd);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

void launch_completude(const float4 *slot_vpos, uint32_t nslots, uint32_t *count, cudaStream_t s) {
    GC_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t), s));
    const uint32_t grid = std::min<uint32_t>(div_up(nslots, 256), static_cast<uint32_t>(sm_count()) * 4);
    completude_kernel<<<std::max(1u, grid), 256, 0, s>>>(slot_vpos, nslots, count);
    GC_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace gc

// ---------------------------------------------------------------------------
// Miss list without allocation.
//
// Some callers cannot allocate device memory at the moment they need the miss
// list: a host that records its frame into a CUDA graph (memory allocation is
// not allowed while a stream is being captured), a render loop with a hard
// frame deadline that must not block in the allocator (cudaMalloc can wait for
// the device), or a plug-in whose host application owns every byte of device
// memory and hands it only input and output buffers.  For them the scan's
// scratch -- one look-back status word per 4096-entry tile and the scan
// control block -- lives in this file-scope device array instead of memory
// obtained from cudaMalloc.  Every GPU that loads the library holds it until
// the process exits.
namespace gc {

constexpr uint32_t kNoAllocMaxTiles = 2048;  // request buffers of up to 2048 * 4096 entries
constexpr uint64_t kNoAllocMaxEntries = static_cast<uint64_t>(kNoAllocMaxTiles) * kTile;

// words [0, kNoAllocMaxTiles): look-back status; the last two words: ScanCtl
constexpr uint32_t kNoAllocWords = kNoAllocMaxTiles + sizeof(ScanCtl) / sizeof(uint64_t);
static_assert(sizeof(ScanCtl) == 2 * sizeof(uint64_t), "ScanCtl must fill two scratch words");
static __device__ __align__(256) uint64_t g_noalloc_scratch[kNoAllocWords];  // 16 KiB + 16 B

// Host code cannot use g_noalloc_scratch as a device address (the name is a
// host-side stand-in); the device address is looked up once per device, with
// that device current.
constexpr int kNoAllocMaxDevices = 64;
static uint64_t *g_noalloc_ptr[kNoAllocMaxDevices] = {};
static std::mutex g_noalloc_mu;

// The scan's result word for the caller: the count of flagged entries, or
// GC_MISS_LIST_FAILED when one of its bounded look-back waits ran out (the list
// is then not valid).  Read on the device, so the call stays asynchronous.
__global__ void noalloc_total_kernel(const ScanCtl *ctl, uint32_t *out_total) {
    *out_total = ctl->err ? GC_MISS_LIST_FAILED : ctl->total;
}

// Test hook of the error path: GC_TEST_NOALLOC_SILENT_TILE=<k> makes scan tile
// k publish nothing, so that tile k + 1's bounded look-back wait runs out.
static uint32_t noalloc_silent_tile() {
    const char *v = std::getenv("GC_TEST_NOALLOC_SILENT_TILE");
    return (v && *v) ? static_cast<uint32_t>(std::strtoul(v, nullptr, 10)) : 0xffffffffu;
}

static uint64_t *noalloc_scratch() {
    int dev = 0;
    GC_CUDA(cudaGetDevice(&dev));
    GC_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, "device index out of range");
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        uint64_t *p = nullptr;
        GC_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_noalloc_scratch));
        g_noalloc_ptr[dev] = p;
    }
    return g_noalloc_ptr[dev];
}

}  // namespace gc

extern "C" int gc_miss_list_noalloc(const uint32_t *requests, uint64_t n_entries, uint32_t timestamp,
                                    const gc_layout *layout, uint32_t max_requests, uint32_t *out_list,
                                    uint32_t *out_total, void *stream) {
    using namespace gc;
    return guard([&] {
        GC_REQUIRE(requests && layout && out_list && out_total, "null argument");
        // the scan reads the request words and writes the list 16 bytes at a time
        GC_REQUIRE(reinterpret_cast<uintptr_t>(requests) % 16 == 0 && reinterpret_cast<uintptr_t>(out_list) % 16 == 0,
                   "requests and out_list must be 16-byte aligned");
        GC_REQUIRE(reinterpret_cast<uintptr_t>(out_total) % 4 == 0, "out_total must be 4-byte aligned");
        GC_REQUIRE(n_entries >= 2, "the request buffer needs at least 2 entries");
        GC_REQUIRE(n_entries - 1 <= kNoAllocMaxEntries,
                   "request buffer too large for the allocation-free scan: at most 8388609 entries "
                   "(2048 tiles of 4096) are supported");
        GC_REQUIRE(max_requests >= 1, "max_requests must be >= 1");
        GC_REQUIRE(layout->nb_levels >= 1 && layout->nb_levels <= GC_MAX_LEVELS, "bad layout");
        // level tables of the page directory (levels packed along x)
        LevelTables lt;
        std::memset(&lt, 0, sizeof(lt));
        lt.nlevels = layout->nb_levels;
        uint32_t mx = 0, my = 0, mz = 0;
        for (uint32_t l = 0; l < layout->nb_levels; ++l) {
            lt.off[l] = mx;
            for (int a = 0; a < 3; ++a) lt.nb[l][a] = layout->nb_bricks[l][a];
            mx += layout->nb_bricks[l][0];
            my = std::max(my, layout->nb_bricks[l][1]);
            mz = std::max(mz, layout->nb_bricks[l][2]);
        }
        GC_REQUIRE(static_cast<uint64_t>(mx) * my * mz == n_entries,
                   "n_entries does not match the page directory of the layout");
        cudaStream_t s = as_stream(stream);
        uint64_t *status = noalloc_scratch();
        ScanCtl *ctl = reinterpret_cast<ScanCtl *>(status + kNoAllocMaxTiles);
        // The scratch keeps the previous call's contents: clear the control block
        // and the status words this scan uses.
        GC_CUDA(cudaMemsetAsync(ctl, 0, sizeof(ScanCtl), s));
        GC_CUDA(cudaMemsetAsync(status, 0, lookback_tiles(n_entries - 1) * sizeof(uint64_t), s));
        static std::atomic<uint32_t> epoch{0};
        launch_miss_compact(requests, n_entries - 1, timestamp, max_requests, reinterpret_cast<uint4 *>(out_list),
                            lt, mx, my, status, ctl, epoch.fetch_add(1) + 1, s, noalloc_silent_tile());
        noalloc_total_kernel<<<1, 1, 0, s>>>(ctl, out_total);
        GC_CUDA(cudaGetLastError());
        count_launch();
    });
}
