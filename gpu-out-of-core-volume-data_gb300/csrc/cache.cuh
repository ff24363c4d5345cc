// Device-side layout of the brick cache, shared by the cache kernels and the
// ray caster.
//
// HBM layout (one allocation each, all 256-byte aligned):
//   mrpd   uint4[mx*my*mz]   page directory, levels packed along x
//                            (MultiResolutionPageDirectory.hpp:88-125): entry
//                            {cacheX, cacheY, cacheZ, flag 0|1|2}
//   req    uint32[mx*my*mz]  request timestamps, same indexing (CacheManager.hpp:239-249)
//   usage  uint32[nslots]    last-use timestamp per pool slot (CacheDevice.hpp:133)
//   order  uint32[nslots]x2  LRU order as slot ids (ping-pong); the reference
//                            moves 28-byte LruContent records instead
//   slot_level / slot_vpos   per-slot LruContent payload (level, volumePosition)
//   pool   bytes             slot-major bricks: slot s = x + y*sx + z*sx*sy holds
//                            B^3 voxels x-fastest (the reference uses a cudaArray
//                            of (sx*B, sy*B, sz*B) voxels)
// Two-level directory (pt_block P > 0) instead of mrpd:
//   top    uint32[tx*ty*tz]  one word per P^3 bricks of a level, levels packed
//                            along x: table slot << 1 | 1, or 0
//   table  uint4[slots*P^3]  brick entries of each table slot's block, x fastest
//   pt_usage / pt_order[2] / pt_keys   the table pool's usage words, LRU order
//                            and the block each slot holds
#pragma once

#include <cstdint>

#include "gc_gb300.h"

namespace gc {

// Levels of every volume the cache holds, concatenated (volume 0's levels
// first): a cache over several volumes is one page directory whose levels
// are those of all of its volumes, with one pool, one LRU and one request
// scan (the serving form's shared pool).
constexpr uint32_t kMaxCacheLevels = 4 * GC_MAX_LEVELS;

struct LevelTables {
    uint32_t nlevels;
    uint32_t off[kMaxCacheLevels];        // MRPD x offset of each level
    uint32_t nb[kMaxCacheLevels][3];      // bricks per axis (MRPD level dimensions)
    uint32_t vvox[kMaxCacheLevels][3];    // virtualized voxels per axis (= real sizes)
    float ior[kMaxCacheLevels][3];        // initial / real size (CacheManager.hpp:271-285)
    uint32_t eb[kMaxCacheLevels];         // bytes per voxel of the level's volume
    uint32_t bb[kMaxCacheLevels][3];      // big-brick size (in bricks) of the level's volume
    float nbf[kMaxCacheLevels][3];        // nb and vvox as floats (exact: both < 2^24), for the
    float vvoxf[kMaxCacheLevels][3];      // ray caster's per-sample page walk
    uint32_t pt_off[kMaxCacheLevels];     // two-level directory: x offset of each level's words
};

// Two-level page directory (the page-table hierarchy of CacheManager with one
// table cache, CacheManager.hpp:151-236): brick (x, y, z) of level l -- x
// counted inside the level -- has its entry in the block of directory word
// pt_word(), at pt_local() inside it.  shift = 0: one-level directory.
struct PageTable {
    uint32_t *top;        // per directory word: table slot << 1 | 1, or 0
    uint4 *table;         // brick entries, 1 << (3 * shift) per table slot
    uint32_t *usage;      // last-use word per table slot
    uint32_t shift;       // log2(P)
    uint32_t tx, txy;     // directory words per row, per slice
};
__host__ __device__ __forceinline__ uint32_t pt_word(const PageTable &pt, const LevelTables &lt, uint32_t l,
                                                     uint32_t x, uint32_t y, uint32_t z) {
    return lt.pt_off[l] + (x >> pt.shift) + (y >> pt.shift) * pt.tx + (z >> pt.shift) * pt.txy;
}
__host__ __device__ __forceinline__ uint32_t pt_local(const PageTable &pt, uint32_t x, uint32_t y, uint32_t z) {
    const uint32_t m = (1u << pt.shift) - 1u;
    return (x & m) | ((y & m) << pt.shift) | ((z & m) << (2u * pt.shift));
}
__host__ __device__ __forceinline__ uint64_t pt_entry(const PageTable &pt, uint32_t slot, uint32_t local) {
    return (static_cast<uint64_t>(slot) << (3u * pt.shift)) + local;
}

struct CacheView {
    uint4 *mrpd;          // one-level directory (null with a two-level one)
    PageTable pt;
    uint32_t *req;
    uint32_t *usage;
    const uint8_t *pool;
    uint32_t mx, my, mz;
    uint32_t mxy;         // mx * my (the page directory has fewer than 2^32 - 1 entries)
    uint32_t sx, sy, sz;
    uint32_t B, c, Beff;
    uint32_t beff_magic;  // ceil(2^32 / Beff) for the exact multiply-high modulo (0: use %)
    uint32_t eb;          // bytes per voxel of every volume, 0 when the volumes differ
    uint32_t nc;          // channels per voxel (1, or 2 for two 8-bit channels)
    uint64_t slot_bytes;  // pool slot stride: B^3 x the widest voxel
    // per page-directory entry, read beside the entry: the value bins of a
    // mapped entry's brick (written by the install), the user's bins of the
    // brick where given (gc_cache_set_volume_brick_bins), else all bits
    const unsigned long long *entry_bins;
    uint32_t bins_user;   // an unmapped entry with invisible bins is stepped through (user bins given)
    uint32_t b_shift;     // log2(B) when B is a power of two, else 32 (divide)
    unsigned long long *samples;          // running counts: [0] samples taken (resident-brick reads),
                                          // [1] rays that took a first step
    uint32_t ts;
};

// Empty-space skipping: voxel values are quantized into kValueBins bins of
// [0, 1]; the install records the bins a brick's voxels cover (one bit each,
// widened by one bin on either side) for its slot and its page-directory
// entry, and a view the bins its transfer function can make visible.  A brick
// whose bins are all invisible contributes no sample above the compositing
// threshold, so the march steps through it without sampling (same t
// sequence, same image).
constexpr uint32_t kValueBins = 64;

// Per-launch ray-caster parameters of one view.
struct ViewParams {
    float m[12];
    uint32_t W, H;
    float bmin[3], bmax[3];
    float tstep, focal, early;
    uint32_t mode, sampler;
    uint32_t tfw;
    uint32_t tfh;                       // 2D transfer function rows (two-channel volumes)
    const float *tf;
    uint32_t *rgba;
    float *tbuf;
    float *state;
    uint32_t *status;                   // optional per-view "met an unmapped brick" word
    // LOD tables (display_volume_raycaster, VolumeRayCaster.cu:146-161)
    float inv_size[GC_MAX_LEVELS][3];   // bboxSizeMin / initial level size
    float step[GC_MAX_LEVELS];          // LODStepSize
    float kexp[GC_MAX_LEVELS];          // LODStepSize / tstep (opacity correction exponent)
    float alpha_floor[GC_MAX_LEVELS];   // alphas at or below this cannot reach the 0.001 threshold
    uint32_t tiles_x;                   // warp tiles per row
    uint32_t tile_shift;                // log2 of the tile width
    // Work order: the tiles of the screen rectangle that can hold rays meeting
    // the box (rx0, ry0, rw, rh in tiles) come first in the queue, for every
    // view; the other tiles (rays that miss) follow.
    uint32_t rx0, ry0, rw, rh;
    uint32_t rect_begin;                // first queue index of this view's rectangle tiles
    uint32_t out_begin;                 // first queue index of its other tiles
    uint32_t rect_total;                // rectangle tiles of all views (the same in every view)
    uint32_t level_base;                // first cache level of the view's volume
    uint32_t nlevels;                   // levels of the view's volume
    uint32_t eb;                        // bytes per voxel of the view's volume
    uint32_t fallback;                  // sample a coarser mapped level where a brick is missing (preview)
    uint32_t skip_empty;                // step through invisible bricks without sampling (DVR, one channel)
    unsigned long long visible;         // bins the view's transfer function can make visible
    uint32_t mark_done;                 // batched passes: a finished ray leaves -1 - t in tbuf and
                                        // later passes skip its pixel (rgba already final)
};

// The bricking rule of one level (Bricker_v2.cpp:79-252): the level bricker
// (gc_bricks_build) and the on-demand cut of the device-levels brick source.
struct BrickParams {
    uint32_t D[3];        // level size (voxels)
    uint32_t B, c, Beff;
    uint32_t BB[3];
    uint32_t nbig[3];     // big bricks per axis
    uint32_t eb;
    uint64_t nsmall;      // small bricks in the level
    uint32_t fast;        // 16-byte rows: B a power of two, B*eb and D[0]*eb multiples of 16, buffers 16-byte aligned
    uint32_t b_shift;     // log2(B) (fast path: B a power of two)
    uint32_t cpr_shift;   // log2(16-byte chunks per brick row)
};

// A device-resident mip pyramid as a volume's brick source: a missing big
// brick is cut from its level with the bricker's rule into the staging slot
// the install reads (gc_cache_set_volume_source_device).
struct CutSource {
    const uint8_t *pyramid = nullptr;
    uint64_t offset[GC_MAX_LEVELS] = {};    // byte offset of each level
    uint32_t dims[GC_MAX_LEVELS][3] = {};   // level sizes
    uint32_t fast[GC_MAX_LEVELS] = {};      // the 16-byte path applies to the level
    BrickParams p = {};                     // B, c, Beff, BB, eb, shifts
};
struct CutSources {
    CutSource vol[4];
};
// Cut jobs: {x, y, z, slot << 8 | volume << 6 | level} big bricks.
void launch_cut_bricks(const CutSources &srcs, const uint4 *jobs, uint32_t n, uint8_t *staging, uint64_t stride,
                       cudaStream_t s);

// Scan control block shared by the decoupled look-back kernels.
struct ScanCtl {
    uint32_t ticket;
    uint32_t done;
    uint32_t err;
    uint32_t total;     // result: flagged items of the last scan
};

constexpr uint32_t kErrLookback = 1u;   // a look-back wait ran out
constexpr uint32_t kErrRender = 2u;     // render work-queue wait ran out

// Host launchers (cache_kernels.cu).
void launch_lru_count(const uint32_t *usage, uint32_t nslots, uint32_t ts, uint32_t *count, cudaStream_t s);
void launch_lru_partition(const uint32_t *order_in, uint32_t *order_out, const uint32_t *usage, uint32_t ts,
                          uint32_t nslots, const uint32_t *count, uint64_t *status, ScanCtl *ctl,
                          uint32_t epoch, cudaStream_t s);
// silent_tile: a scan tile that publishes nothing (tests of the bounded
// look-back's error path; 0xffffffff = none).
void launch_miss_compact(const uint32_t *req, uint64_t nscan, uint32_t ts, uint32_t maxreq, uint4 *list,
                         const LevelTables &lt, uint32_t mx, uint32_t my, uint64_t *status, ScanCtl *ctl,
                         uint32_t epoch, cudaStream_t s, uint32_t silent_tile = 0xffffffffu);
uint32_t lookback_tiles(uint64_t n);

struct InstallArgs {
    uint4 *mrpd;
    PageTable pt;              // two-level directory (pt.shift > 0; mrpd is then null)
    uint32_t pt_slots;
    const uint32_t *pt_order;  // the table pool's current LRU order
    uint4 *pt_keys;            // per table slot: first brick (x, y, z) of its block and the level, or all ones
    uint32_t *pt_claim;        // per directory word: lowest list index claiming it (~0 between installs)
    uint32_t *pt_word_of;      // per list element: the directory word it claims, or ~0
    uint2 *pt_jobs;            // claimed words in list order: {word, element}
    uint32_t *pt_njobs;
    uint32_t mx, my;
    uint64_t nentries;
    const uint32_t *order;     // current LRU order
    uint32_t nslots;
    uint32_t *slot_level;
    float4 *slot_vpos;
    uint8_t *pool;
    unsigned long long *slot_bins;  // per slot value-bin mask, written with the brick
    unsigned long long *entry_bins; // per page-directory entry (see CacheView::entry_bins)
    const unsigned long long *user_bins;  // the user's per-entry bins, or null
    uint32_t nc;               // channels per voxel (bins only for one channel)
    uint64_t slot_bytes;       // pool slot stride
    uint64_t big_stride;       // staging stride of one big brick
    uint32_t sx, sy;
    uint32_t B, Beff;
    uint32_t *owner;           // per page-directory entry: lowest list index naming it (~0 between installs)
    uint64_t *coords;          // per list element: its page-directory entry
    const uint4 *asked;        // partitioned asked list: non-empty first
    const uint32_t *big_index; // per non-empty brick
    const uint4 *big_coord;    // per loaded big brick
    const uint8_t *staging;    // loaded big bricks
    uint32_t n, n_nonempty;
};
void launch_install(const InstallArgs &a, const LevelTables &lt, cudaStream_t s);
// Rebuilds the per-entry bins after the user's bins changed: user (or all
// bits) everywhere, then the bins of every resident brick at its entry.
void launch_live_bins(const LevelTables &lt, const float4 *slot_vpos, const uint32_t *slot_level,
                      const unsigned long long *slot_bins, uint32_t nslots, uint32_t mx, uint32_t my,
                      uint64_t nentries, unsigned long long *entry_bins, const PageTable &pt, uint32_t sx,
                      uint32_t sy, uint32_t B, cudaStream_t s);
// The brick entries of a two-level directory as the flat directory would
// hold them (0 where the block is not resident), for state dumps.
void launch_pt_flatten(const PageTable &pt, const LevelTables &lt, uint32_t mx, uint32_t my, uint64_t nentries,
                       uint4 *out, cudaStream_t s);
// Table pool: slots in raster order, no block held.
void launch_pt_init(uint32_t *order, uint4 *keys, uint32_t nslots, cudaStream_t s);
// Copies brick i (src[i] = {device-readable host address, bytes}) to
// dst + i * stride; vec16: every address, size and the stride are multiples
// of 16.
void launch_brick_bins(const uint8_t *level, const uint32_t nb[3], const uint32_t nbig[3], const uint32_t bb[3],
                       uint32_t B, uint32_t eb, unsigned long long *bins, cudaStream_t s);
void launch_gather_bricks(const ulonglong2 *src, uint32_t n, uint64_t stride, uint8_t *dst, bool vec16,
                          bool beside, cudaStream_t s);
// In-flight marks (page-directory flag 3) of the batched form's overlapped
// loads: mark the first min(ctl->total, maxreq) entries of a miss list; unmark
// (3 -> 0) the first n entries of a list after its install.
void launch_mark_in_flight(const uint4 *list, const ScanCtl *ctl, uint32_t maxreq, const LevelTables &lt,
                           uint32_t mx, uint32_t my, uint64_t nentries, uint4 *mrpd, cudaStream_t s);
void launch_unmark_in_flight(const uint4 *list, uint32_t n, const LevelTables &lt, uint32_t mx, uint32_t my,
                             uint64_t nentries, uint4 *mrpd, cudaStream_t s);
void launch_completude(const float4 *slot_vpos, uint32_t nslots, uint32_t *count, cudaStream_t s);

// Ray caster (render.cu).  Launch configuration of the ray caster, process
// wide: scheduler 0 = one 8x4 tile per warp, 1 = per-lane pixel refill;
// threads per block; blocks per SM cap (0 = occupancy limit).
struct RenderTuning {
    uint32_t scheduler = 1;
    uint32_t threads = 128;
    uint32_t blocks_per_sm = 0;
    uint32_t skip_empty = 1;  // empty-space skipping on (results are the same either way)
    uint32_t tile_w = 8;  // ray tile of one warp: tile_w x (32 / tile_w) pixels
    uint32_t precision = 0;  // 0: exact build (the oracle's operations); 1: fast build
};
RenderTuning &render_tuning();
// Ray-caster kernels of a voxel kind (1, 2, 4 bytes; 0 mixed widths; 0x202
// two 8-bit channels), scheduler and brick size (16 and 32 have kernels
// compiled for them; a two-level page directory has kernels of its own),
// from the exact build (render.cu) or the fast build (render_fast.cu);
// nullptr for an unsupported kind.
namespace exact {
void *march_kernel(uint32_t kind, bool pixels, uint32_t brick_size, bool two_level);
}
namespace fast {
void *march_kernel(uint32_t kind, bool pixels, uint32_t brick_size, bool two_level);
}
// Fills ViewParams::visible of n device views from their transfer functions.
void launch_view_bins(ViewParams *views_dev, uint32_t n, cudaStream_t s);
void launch_render(const CacheView &cv, const LevelTables &lt, const ViewParams *views_dev,
                   const ViewParams *views_host, uint32_t nviews, uint32_t total_tiles, uint32_t *queue,
                   uint32_t *err, cudaStream_t s);

// An executable CUDA graph of the batched launch (view-table copy + ray caster).
struct RenderGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t copy = nullptr, bins = nullptr, kern = nullptr;
    void *func = nullptr;
    uint32_t threads = 0;
    uint64_t replays = 0;
    RenderGraph() = default;
    RenderGraph(const RenderGraph &) = delete;
    RenderGraph &operator=(const RenderGraph &) = delete;
    ~RenderGraph();
    void reset();
};
void launch_render_graph(RenderGraph &g, const CacheView &cv, const LevelTables &lt, ViewParams *views_dev,
                         const ViewParams *views_pinned, uint32_t nviews, uint32_t total_tiles, uint32_t *queue,
                         cudaStream_t s);

}  // namespace gc
