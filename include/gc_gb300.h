/*
 * gc_gb300.h -- C ABI of the GB300-native out-of-core volume path.
 *
 * This is the drop-in boundary for GcCore's out-of-core volume path
 * (ftilde/GPU-Out-of-Core-Volume-Data).  The reference exposes that path as a
 * C++ template library (CacheManager<T>, K_CacheManager<T>, Mipmapper,
 * process_bricking, RayCastDVR); its only C linkage is the bricker shim
 * GcCore/include/GcCore/libPython/Py_Bricker.hpp:8-49.  Every entry point
 * below names the reference interface it replaces.
 *
 * Conventions
 *  - plain pointers and sizes only; no C++ or torch types cross the boundary;
 *  - every call returns an int status (GC_OK == 0); gc_last_error() returns
 *    a thread-local, human-readable message for the last failing call;
 *  - device pointers are CUDA device addresses on the cache's GPU; `stream`
 *    arguments are cudaStream_t values passed as void* (0 = legacy stream);
 *  - a gc_cache handle is not thread-safe: drive it from one host thread,
 *    like the reference's CacheManager (CacheManager.hpp:38-128).
 */
#ifndef GC_GB300_H
#define GC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GC_MAX_LEVELS 16

/* status codes */
#define GC_OK 0
#define GC_ERR_INVALID 1    /* bad argument or configuration                 */
#define GC_ERR_CUDA 2       /* a CUDA runtime call failed                     */
#define GC_ERR_IO 3         /* file or brick-source failure                   */
#define GC_ERR_TIMEOUT 4    /* a bounded device-side or host-side wait ran out */
#define GC_ERR_NOMEM 5      /* allocation failed                              */
#define GC_ERR_UNSUPPORTED 6

/* brick status, as BricksManager::BrickStatus (BricksManager.hpp:321-326) */
#define GC_BRICK_SUCCESS 0
#define GC_BRICK_UNKNOWN 1
#define GC_BRICK_EMPTY 2

/* compositing, as CompositingMode DVR|MOP (VolumeRayCaster.cu:91-99) */
#define GC_MODE_DVR 0
#define GC_MODE_MOP 1

/* sampler: GC_SAMPLER_REFERENCE reproduces the reference's normalized
 * texture read at the integer voxel corner (K_CacheDevice.hpp:193-200), i.e.
 * the mean of the 2x2x2 voxels (e-1,e) per axis; GC_SAMPLER_TRILINEAR
 * interpolates at the fractional position inside the brick using the
 * covering border. */
#define GC_SAMPLER_REFERENCE 0
#define GC_SAMPLER_TRILINEAR 1

/* cache flags */
#define GC_CACHE_SYNC_LOADER 1u   /* loader completes inside update(): deterministic
                                     request -> install alternation (the upload
                                     it starts runs on the cache's side stream,
                                     beside the next render; the next update's
                                     install waits for it)                     */
#define GC_CACHE_STAGED_UPLOAD 2u /* host-store bricks always go through the pinned
                                     staging buffer + cudaMemcpyAsync, even when
                                     the device can read the store directly     */

/* ------------------------------------------------------------------------ */
/* Volume description: the reference's config surface (config_skull.cfg:1-24,
 * VolumeConfiguration.hpp:14-31).  encoded_bytes is bytes per voxel over all
 * channels (MetaData.cpp:21-32); bytes per channel = encoded_bytes/channels. */
typedef struct gc_volume_desc {
    uint32_t size[3];            /* size_X/Y/Z                      */
    uint32_t brick_size;         /* BrickSize (cubic)               */
    uint32_t big_brick_size[3];  /* BigBrickSizeX/Y/Z               */
    uint32_t covering;           /* VoxelCovering                   */
    uint32_t encoded_bytes;      /* NumberEncodedBytes              */
    uint32_t channels;           /* NumberChannels                  */
    uint32_t downscale[3];       /* downScale_X/Y/Z (only 2 is supported) */
} gc_volume_desc;

/* Per-level geometry: Mipmapper::fill_metaData (Mipmapper.cu:583-597) and
 * init_meta_data (Bricker_v2.cpp:45-76). */
typedef struct gc_layout {
    uint32_t nb_levels;
    uint32_t initial[GC_MAX_LEVELS][3];        /* mip level sizes (voxels)        */
    uint32_t real[GC_MAX_LEVELS][3];           /* nb_bricks * (B - 2c)            */
    uint32_t nb_bricks[GC_MAX_LEVELS][3];      /* small bricks per axis           */
    uint32_t nb_big_bricks[GC_MAX_LEVELS][3];  /* big bricks per axis             */
    uint32_t mip[GC_MAX_LEVELS][3];            /* sizes of the mip data actually
                                                  produced (== initial for the
                                                  supported power-of-two volumes) */
} gc_layout;

/* ------------------------------------------------------------------------ */
/* Errors and version. */
const char *gc_last_error(void);
const char *gc_version(void);
int gc_device_count(int *count);
/* Number of CUDA kernels this library has launched in this process. */
uint64_t gc_kernel_launches(void);

/* ------------------------------------------------------------------------ */
/* Configuration: Configuration::load<TDNSConfigurationParser> +
 * get_field/add_field (Configuration.cpp:30-186, ConfigurationPolicies.cpp:16-44),
 * load_volume_configuration's config part (VolumeConfiguration.cpp:14-50). */
typedef struct gc_config *gc_config_t;
int gc_config_create(gc_config_t *out);
int gc_config_destroy(gc_config_t cfg);
/* parses the reference's <Fields><Field key="" value=""/></Fields> file */
int gc_config_load(gc_config_t cfg, const char *path);
int gc_config_set(gc_config_t cfg, const char *key, const char *value);
/* copies the value (NUL-terminated) into buf; GC_ERR_INVALID if missing */
int gc_config_get(gc_config_t cfg, const char *key, char *buf, size_t buflen);
/* fills a volume description from BrickSize, BigBrickSize{X,Y,Z},
 * VoxelCovering, NumberEncodedBytes, NumberChannels, size_{X,Y,Z},
 * downScale_{X,Y,Z}; missing required keys are GC_ERR_INVALID with the key
 * named, like the reference's runtime_error messages. */
int gc_config_volume_desc(gc_config_t cfg, gc_volume_desc *out);

/* Level geometry (fill_metaData + init_meta_data + levelMax at
 * Mipmapper.cu:441-443). */
int gc_layout_compute(const gc_volume_desc *vol, gc_layout *out);

/* Pool sizing of Application.cu:79-93: the cube of slots that holds
 * pool_bytes / (B^3 * encoded_bytes) bricks, grown round-robin per axis. */
int gc_pool_dims(const gc_volume_desc *vol, uint64_t pool_bytes, uint32_t out_dims[3]);

/* ------------------------------------------------------------------------ */
/* Synthetic volume (seeded blobs + value noise, integer arithmetic so that
 * every device and host evaluation is bit-identical).  Writes X*Y*Z voxels
 * (x fastest) of `bytes_per_channel` (1 or 2) to `dst` on the device.
 * Channel `channel` selects an independent field (0: blobs+noise,
 * 1: noise only); `stride_channels` interleaves into a multi-channel volume. */
typedef struct gc_blob {
    int32_t cx, cy, cz;        /* centre (voxels)                         */
    uint64_t k[3];             /* per-axis 2^38 / (9 sigma^2)             */
    int32_t r[3];              /* bounding half-extent (voxels)           */
    int32_t amplitude;         /* value units                              */
} gc_blob;

typedef struct gc_generator {
    uint32_t size[3];
    uint32_t bytes_per_channel;    /* 1 or 2                                */
    uint32_t channels;             /* interleave stride                      */
    uint32_t channel;              /* which channel to write                 */
    uint32_t field;                /* 0: blobs + noise, 1: noise only        */
    uint32_t seed;
    int32_t noise_amplitude;       /* value units                            */
    uint32_t nblobs;
    const gc_blob *blobs;          /* host array                             */
} gc_generator;

/* Draws blob parameters from a seeded splitmix64 stream (the same function
 * runs in the oracle). */
int gc_generator_blobs(uint32_t seed, uint32_t nblobs, const uint32_t size[3],
                       float sigma_min, float sigma_max, int32_t amp_min,
                       int32_t amp_max, gc_blob *out);
int gc_generate_volume(const gc_generator *gen, void *dst, void *stream);

/* ------------------------------------------------------------------------ */
/* Preprocessor.
 * gc_mip_level: one 2x2x2 down-sampling pass (Mipmapper::down_scale,
 * Mipmapper.cu:528-578, kernel down_sampling_inner Mipmapper.cu:29-105):
 * output voxel = floor(sum / 8) for integer channels (u8 via the integer
 * path, u16 via the double path whose sum is exact), (float)(sum_double / 8)
 * for f32.  src/dst are device pointers, dims are the source level sizes. */
int gc_mip_level(const void *src, void *dst, const uint32_t src_dims[3],
                 uint32_t encoded_bytes, uint32_t channels, void *stream);

/* gc_mip_build: the whole pyramid (Mipmapper::process, Mipmapper.cu:401-525)
 * kept resident on the device.  `pyramid` holds level 0 at offset 0 and
 * receives levels 1..nb_levels-1 at level_offsets[l] (bytes). */
int gc_mip_build(void *pyramid, const gc_layout *layout, const uint64_t *level_offsets,
                 uint32_t encoded_bytes, uint32_t channels, void *stream);

/* gc_bricks_build: cuts one level into covered bricks (process_bricking,
 * Bricker_v2.cpp:79-252).  Output holds the level's big bricks in
 * (z, y, x) raster order, each (BB*B)^3 voxels x-fastest (Bricker_v2.cpp:295-299);
 * voxels outside the level are zero. */
int gc_bricks_build(const void *level, const uint32_t level_dims[3],
                    const gc_volume_desc *vol, const uint32_t nb_big_bricks[3],
                    void *out, void *stream);

/* gc_bricks_empty: per big brick, 1 if every channel value < threshold
 * (BrickProcessor::process_empty + DefaultBrickProcessorPredicate,
 * BrickProcessor.hpp:91-162, BrickProcessorPredicate.hpp:11-46). */
int gc_bricks_empty(const void *bricks, uint64_t nb_big_bricks, const gc_volume_desc *vol,
                    float threshold, uint8_t *flags, void *stream);

/* Brick key: 4 x uint16 {level, x, y, z} packed little-endian into a uint64
 * (get_key, BrickKey.cpp:15-25). */
uint64_t gc_brick_key(uint32_t level, uint32_t x, uint32_t y, uint32_t z);

/* ------------------------------------------------------------------------ */
/* GPU brick cache: CacheManager<T> (CacheManager.hpp:38-670) with its
 * MultiResolutionPageDirectory (MultiResolutionPageDirectory.hpp:88-125),
 * CacheDevice (CacheDevice.hpp:122-219) and RequestHandler
 * (RequestHandler.hpp:29-372). */
typedef struct gc_cache *gc_cache_t;

typedef struct gc_cache_desc {
    gc_volume_desc volume;
    gc_layout layout;
    uint32_t cache_size[3];   /* pool slots per axis (CacheConfiguration::CacheSize[0]) */
    uint32_t max_requests;    /* reference: 50 (CacheManager.hpp:263)              */
    uint32_t flags;           /* GC_CACHE_*                                        */
    int32_t gpu;              /* gpuID                                             */
    /* Two-level page directory: the page-table hierarchy of CacheManager
     * (CacheManager.hpp:151-236, CacheManagerKernels.hpp:148-357) with one
     * page-table cache between the directory and the brick pool, i.e. a
     * CacheConfiguration of two CacheSize / BlockSize entries.  pt_block = 0:
     * one level (every configuration of the reference application).  Else
     * a power of two from 2 to 16: the directory keeps one word per
     * pt_block^3 bricks of a level, naming the block of pt_block^3 brick
     * entries that holds them in a table pool of pt_slots blocks; the table
     * pool has its own usage words and LRU order, and a block taken for new
     * bricks evicts the least recently used one (its bricks become
     * unreachable until requested again).  The flat directory of 16 bytes
     * per brick is not allocated.  Not with the batched form's overlapped
     * loads.  Brick entries, requests, samples and images are those of the
     * one-level directory while no block in use is evicted. */
    uint32_t pt_block;
    uint32_t pt_slots;
} gc_cache_desc;

/* Brick source callback: copy the big brick (level, x, y, z) -- (BB*B)^3
 * voxels of encoded_bytes -- into dst and return a GC_BRICK_* status.  Called
 * from the cache's loader thread (BricksManager::get_brick,
 * BricksManager.cpp:48-78). */
typedef int (*gc_brick_loader_fn)(void *user, uint32_t level, uint32_t x, uint32_t y,
                                  uint32_t z, void *dst, size_t bytes);

int gc_cache_create(const gc_cache_desc *desc, gc_cache_t *out);
/* One cache over several volumes sharing one brick pool (the serving form;
 * no counterpart in the reference, whose CacheManager holds one volume).
 * The page directory holds the levels of all n_volumes volumes one after
 * the other (volume 0 first; gc_cache_volume_levels gives each volume's
 * range), the LRU order, usage and request scan run over the whole pool,
 * and a view names its volume in gc_view.volume.  The volumes need the same
 * BrickSize and VoxelCovering; their voxel widths and big-brick sizes may
 * differ (a pool slot then holds B^3 voxels of the widest type).  desc gives
 * the pool size, max_requests, flags and device; its volume/layout fields
 * are ignored.  1 to 4 volumes, at most 64 levels in all. */
int gc_cache_create_shared(const gc_cache_desc *desc, const gc_volume_desc *volumes, const gc_layout *layouts,
                           uint32_t n_volumes, gc_cache_t *out);
/* First cache level and level count of one volume of the cache. */
int gc_cache_volume_levels(gc_cache_t cache, uint32_t volume, uint32_t *level_base, uint32_t *n_levels);
int gc_cache_destroy(gc_cache_t cache);
/* In-memory brick store of `bytes` bytes: all big bricks of every level,
 * level l starting at byte offset level_offsets[l] in (z, y, x) raster order;
 * every level must lie inside the store (checked, GC_ERR_INVALID otherwise).
 * The memory must outlive the cache.  empty_keys lists gc_brick_key()s
 * reported as Empty (bricks.xml <EmptyBricks>, MetaData.cpp:65-77).
 * Upload route: when the device can read the store -- page-locked memory
 * (cudaHostAlloc / cudaHostRegister), or any host memory on a system whose
 * device reports cudaDevAttrPageableMemoryAccess (Grace-Blackwell over
 * NVLink-C2C) -- a kernel on the loader's side stream gathers the missing
 * bricks from it straight into device memory and the host only resolves the
 * request list; otherwise, or with GC_CACHE_STAGED_UPLOAD, host threads copy
 * the bricks into pinned staging memory and cudaMemcpyAsync uploads them. */
int gc_cache_set_source_host(gc_cache_t cache, const void *bricks, uint64_t bytes, const uint64_t *level_offsets,
                             const uint64_t *empty_keys, size_t n_empty);
int gc_cache_set_source_callback(gc_cache_t cache, gc_brick_loader_fn fn, void *user,
                                 const uint64_t *empty_keys, size_t n_empty);
/* The same for one volume of a shared cache (the calls above set volume 0).
 * Level numbers, brick keys and empty keys are the volume's own. */
/* Brick files of the reference's on-disk store under volume_dir (below): the
 * loader reads and decompresses each missing big brick with up to `threads`
 * worker threads into the pinned staging buffer, uploaded with
 * cudaMemcpyAsync (BricksManager::get_brick / load_brick,
 * BricksManager.cpp:29-78, 191-227).  A missing file is GC_BRICK_UNKNOWN; a
 * corrupt one stops the loader with GC_ERR_IO.  Needs liblz4. */
int gc_cache_set_volume_source_files(gc_cache_t cache, uint32_t volume, const char *volume_dir,
                                     const uint64_t *empty_keys, size_t n_empty, uint32_t threads);
int gc_cache_set_volume_source_host(gc_cache_t cache, uint32_t volume, const void *bricks, uint64_t bytes,
                                    const uint64_t *level_offsets, const uint64_t *empty_keys, size_t n_empty);
/* A device-resident mip pyramid as the brick source (an extension: the
 * reference always loads bricks from storage).  `pyramid` is device memory
 * holding every level of the volume, level l at byte offset level_offsets[l]
 * (the layout gc_mip_build leaves: level 0 from the caller, the coarser
 * levels computed on the device).  A missing big brick is cut from its level
 * on the device, with the bricker's rule (process_bricking: covering border,
 * zeros outside the level and in unvisited bricks), straight into the
 * staging memory the install reads: no brick store and no host transfer.
 * It suits volumes whose pyramid fits in device memory but whose bricked
 * store does not fit the host (4096^3 x 2 channels: a 146 GiB pyramid, a
 * 375 GB store).  The pyramid must outlive the cache. */
int gc_cache_set_volume_source_device(gc_cache_t cache, uint32_t volume, const void *pyramid,
                                      const uint64_t *level_offsets, const uint64_t *empty_keys, size_t n_empty);
int gc_cache_set_volume_source_callback(gc_cache_t cache, uint32_t volume, gc_brick_loader_fn fn, void *user,
                                        const uint64_t *empty_keys, size_t n_empty);
/* Brick value bins (an extension; the reference has none).  Bit b of a
 * brick's word is set when its voxel values (covering included) reach value
 * bin b of 64 over [0, 1], widened by one bin on either side -- the mask the
 * ray caster's empty-space skipping keeps per pool slot.  Given for every
 * brick of a volume (n = sum over levels of nb_bricks.x*y*z; level order, x
 * fastest within a level), a ray steps through a MISSING brick whose bins its
 * transfer function cannot make visible, as it does through a resident one,
 * instead of stopping to request it: such bricks are never loaded.  Images
 * are the same; the requests, the loads and the cache state are not the
 * reference's.  The bricks of the volume's empty big bricks are always
 * requested (an empty brick steps by the base step), so a callback source
 * that reports more bricks empty than its empty keys name must give those
 * bricks all bits set.  n = 0 removes the volume's bins.  Takes effect at the
 * next render. */
int gc_cache_set_volume_brick_bins(gc_cache_t cache, uint32_t volume, const uint64_t *bins, uint64_t n);
/* The value bins of every brick of one level (nb_bricks.x*y*z words, x
 * fastest) from the level's big bricks in device memory (the layout
 * gc_bricks_build writes), into device memory bins; all bits set for a
 * volume of several channels. */
int gc_brick_value_bins(const gc_volume_desc *vol, const gc_layout *layout, uint32_t level, const void *level_bricks,
                        uint64_t *bins, void *stream);
/* CacheManager::update (CacheManager.hpp:318-354).  *converged = 1 when the
 * request list was empty this frame. */
int gc_cache_update(gc_cache_t cache, void *stream, int *converged);
/* CacheManager::completude (CacheManager.hpp:357-383). */
int gc_cache_completude(gc_cache_t cache, void *stream, float *fraction);
int gc_cache_timestamp(gc_cache_t cache, uint32_t *ts);

typedef struct gc_cache_info {
    uint32_t mrpd_dims[3];        /* (sum_l nb_bricks.x, max y, max z)        */
    uint32_t nb_slots;
    uint32_t slot_voxels;         /* B^3                                      */
    uint32_t level_offset[GC_MAX_LEVELS];
    uint64_t pool_bytes;
    uint32_t pt_block;            /* 0: one-level directory                    */
    uint32_t pt_slots;            /* table-pool blocks                         */
    uint32_t pt_dims[3];          /* directory words per axis (two levels)     */
    uint32_t pt_level_offset[GC_MAX_LEVELS];
} gc_cache_info;
int gc_cache_info_get(gc_cache_t cache, gc_cache_info *out);

typedef struct gc_cache_stats {
    uint64_t frames;
    uint64_t requests_raised;     /* bricks flagged in the request buffer      */
    uint64_t requests_served;     /* bricks handed to the loader               */
    uint64_t bricks_installed;    /* non-empty bricks written to the pool      */
    uint64_t bricks_empty;        /* empty bricks referenced (flag 2)          */
    uint64_t bytes_h2d;           /* brick bytes copied host -> device         */
    uint64_t load_errors;         /* GC_BRICK_UNKNOWN answers from the source  */
    uint32_t last_requests;       /* misses found in the last request scan     */
    uint32_t last_used;           /* slots stamped by the last rendered frame   */
    uint32_t device_error;        /* sticky device-side error word (0 = none)  */
    uint64_t load_cycles;         /* request lists the loader resolved         */
    uint64_t loader_host_ns;      /* host time resolving + staging bricks      */
    uint64_t upload_ns;           /* device time of the side-stream H2D copies */
    uint32_t upload_direct;       /* 1: host-store bricks are gathered by a kernel
                                     reading the store; 0: staged copies         */
    uint64_t samples;             /* ray-caster samples taken (each reads 8 voxels
                                     and a page-directory entry)                 */
    uint64_t rays_marched;        /* rays that took a first step in a launch (they
                                     meet the volume's box ahead of the camera
                                     and were not finished)                      */
} gc_cache_stats;
int gc_cache_stats_get(gc_cache_t cache, gc_cache_stats *out);

/* State dumps for parity checks (host destinations, sizes in bytes):
 *  GC_DUMP_MRPD     uint32[4] per entry (cacheX, cacheY, cacheZ, flag)
 *  GC_DUMP_LRU      LruContent[] in LRU order: {uint32 cx,cy,cz,level; float vx,vy,vz}
 *                   (LruContent.hpp:10-15)
 *  GC_DUMP_USAGE    uint32 per slot (x fastest)
 *  GC_DUMP_REQUESTS uint32 per MRPD entry
 *  GC_DUMP_POOL     B^3 * encoded_bytes per slot, slot-major (x fastest)
 */
#define GC_DUMP_MRPD 0
#define GC_DUMP_LRU 1
#define GC_DUMP_USAGE 2
#define GC_DUMP_REQUESTS 3
#define GC_DUMP_POOL 4
/* Two-level directory (gc_cache_desc.pt_block > 0); GC_DUMP_MRPD then gives
 * the brick entries as the flat directory would hold them (0 where the
 * brick's table block is not resident):
 *  GC_DUMP_PT_TOP   uint32 per directory word: table slot << 1 | 1, or 0
 *  GC_DUMP_PT_POOL  uint32[4] per table entry, pt_block^3 entries per slot
 *                   (x fastest inside the block)
 *  GC_DUMP_PT_LRU   uint32 table slot ids in LRU order (most recent first)
 *  GC_DUMP_PT_USAGE uint32 per table slot
 *  GC_DUMP_PT_KEYS  uint32[4] per table slot: first brick (x, y, z) of its
 *                   block in its level, and the level; all ones when free */
#define GC_DUMP_PT_TOP 5
#define GC_DUMP_PT_POOL 6
#define GC_DUMP_PT_LRU 7
#define GC_DUMP_PT_USAGE 8
#define GC_DUMP_PT_KEYS 9
int gc_cache_dump(gc_cache_t cache, int what, void *dst, size_t bytes);
/* Miss list of the last request scan (coord_1D_to_3D output: x, y, z, level
 * per brick, CacheManagerKernels.cu:32-72), at most `max` entries; *total is
 * the number of bricks flagged in the scan.  Waits for the scan to finish. */
int gc_cache_last_misses(gc_cache_t cache, uint32_t *out4, uint32_t max, uint32_t *count, uint32_t *total);
/* Miss list without device allocation.  No counterpart in the reference.
 * The same scan, cap and decode as the miss list built inside
 * gc_cache_update, on a caller's request buffer (device, n_entries uint32 laid
 * out like the cache's page directory for `layout`): entries with value
 * `timestamp` in [0, n_entries - 1), the first max_requests of them written
 * to out_list (device, 4 x uint32 per brick: x, y, z, level) and their total
 * count to out_total (device uint32).  It calls no cudaMalloc or cudaFree: its
 * scratch is a fixed array in device memory that every GPU loading the
 * library keeps until exit, so it suits callers that cannot allocate (stream
 * capture, hard frame deadlines, hosts that own all device memory).  Limits:
 * n_entries - 1 <= 8,388,608 (2048 scan tiles of 4096); larger buffers are
 * rejected with GC_ERR_INVALID.  requests and out_list must be 16-byte
 * aligned and out_total 4-byte aligned (GC_ERR_INVALID otherwise, before any
 * device work).  The first call on a device looks the array's
 * address up (cudaGetSymbolAddress): make that first call before any stream
 * capture.  All calls share the array: calls whose work overlaps on the GPU
 * (other streams, other host threads) race and corrupt each other's results;
 * order them on one stream.  The call is asynchronous, so a failure on the
 * device is reported on the device: when one of the scan's bounded waits ran
 * out, *out_total receives GC_MISS_LIST_FAILED instead of a count and
 * out_list is not valid. */
#define GC_MISS_LIST_FAILED 0xffffffffu
int gc_miss_list_noalloc(const uint32_t *requests, uint64_t n_entries, uint32_t timestamp,
                         const gc_layout *layout, uint32_t max_requests, uint32_t *out_list,
                         uint32_t *out_total, void *stream);
/* Overwrite the usage or request buffer (GC_DUMP_USAGE / GC_DUMP_REQUESTS)
 * from the host: used to replay recorded frames through the update path. */
int gc_cache_load_buffer(gc_cache_t cache, int what, const void *src, size_t bytes);

/* ------------------------------------------------------------------------ */
/* Device-side handle of the cache for a host application's own kernels:
 * K_CacheManager<T> and its get_normalized (K_CacheManager.hpp:61-71,
 * 265-361), the object CacheManager::to_kernel_object() returns
 * (CacheManager.hpp:292-309).  gc_cache_device_view_get fills this plain
 * struct -- device pointers and the level tables of one volume of the cache --
 * to be passed BY VALUE to a kernel, which samples with
 * gc_sample_normalized() of include/gc_cache_device.cuh.  Like the
 * reference's kernel object it is valid until the next gc_cache_update of the
 * cache (the timestamp changes every update; installs change the page
 * directory and pool).  One-channel volumes (the reference's sampler). */
typedef struct gc_cache_device_view {
    const uint32_t *mrpd;        /* page directory: 4 words per entry (cacheX, cacheY, cacheZ, flag) */
    uint32_t *requests;          /* request word per page-directory entry                           */
    uint32_t *usage;             /* last-use word per pool slot                                     */
    const uint8_t *pool;         /* pool slots of B^3 voxels, x fastest, slot_bytes apart            */
    uint64_t slot_bytes;
    uint32_t mrpd_dims[3];       /* entries per axis, levels packed along x                          */
    uint32_t pool_slots[3];      /* slots per axis (slot = x + y*sx + z*sx*sy)                       */
    uint32_t brick_size;         /* B                                                                */
    uint32_t covering;           /* c                                                                */
    uint32_t voxel_bytes;        /* 1 (u8), 2 (u16) or 4 (f32)                                       */
    uint32_t timestamp;          /* the frame's timestamp: written into usage and requests           */
    uint32_t n_levels;           /* levels of the volume                                             */
    uint32_t level_offset[GC_MAX_LEVELS];          /* page-directory x offset of each level            */
    uint32_t level_bricks[GC_MAX_LEVELS][3];       /* bricks per axis                                   */
    uint32_t level_voxels[GC_MAX_LEVELS][3];       /* virtualized voxels per axis (bricks x (B - 2c))  */
    float level_initial_over_real[GC_MAX_LEVELS][3]; /* initial / real level size                     */
    /* two-level directory (pt_shift > 0; mrpd is then null): */
    const uint32_t *pt_top;      /* directory word per pt_block^3 bricks: table slot << 1 | 1, or 0   */
    const uint32_t *pt_pool;     /* table blocks: 4 words per brick entry, pt_block^3 entries a slot  */
    uint32_t *pt_usage;          /* last-use word per table slot                                     */
    uint32_t pt_shift;           /* log2(pt_block); 0 for the one-level directory                    */
    uint32_t pt_dims[3];         /* directory words per axis, levels packed along x                  */
    uint32_t pt_level_offset[GC_MAX_LEVELS];       /* directory x offset of each level               */
} gc_cache_device_view;
int gc_cache_device_view_get(gc_cache_t cache, uint32_t volume, gc_cache_device_view *out);

/* ------------------------------------------------------------------------ */
/* Ray caster: RayCastDVR / RayCastMOP (RayCasters.cu:35-468) with the LOD
 * tables of display_volume_raycaster (VolumeRayCaster.cu:141-175) and the
 * camera of update_CUDA_inv_view_model_matrix (RayCasters.cu:587-590). */
typedef struct gc_view {
    float inv_view[12];       /* 3x4 row-major: d_invModelViewMatrix           */
    uint32_t width, height;   /* screenSize                                    */
    float bbox_min[3];
    float bbox_max[3];
    float tstep;              /* marchingStep (reference 2/256)                */
    float focal;              /* ray direction (u, v, -focal); reference 2     */
    float early_alpha;        /* reference 0.95                                */
    uint32_t mode;            /* GC_MODE_*                                     */
    uint32_t sampler;         /* GC_SAMPLER_*                                  */
    uint32_t tf_width;        /* transfer-function entries                     */
    const float *tf;          /* device: tf_width RGBA float entries           */
    uint32_t *rgba;           /* device: width*height RGBA8 (R in low byte)    */
    float *tbuf;              /* device: width*height progressive t            */
    float *state;             /* device: width*height float4 colour state      */
    uint32_t *status;         /* optional device word: bit 0 is set when a ray
                                 of this view met an unmapped brick in this
                                 pass (the view is not converged); the caller
                                 clears it before the pass                      */
    uint32_t volume;          /* volume of a shared cache (gc_cache_create_shared);
                                 0 for a single-volume cache                    */
    uint32_t tf_height;       /* two-channel volumes (NumberChannels 2, 8 bits
                                 each): tf is a 2D table of tf_height rows of
                                 tf_width RGBA entries, channel 0 along a row,
                                 channel 1 across rows, read bilinearly; MIP
                                 classifies the maximum of channel 0 with row 0.
                                 0 or 1 for one-channel volumes                 */
    uint32_t fallback;        /* 0: the reference's ray caster (a ray stops at a
                                 missing brick).  1: preview mode of
                                 K_CacheManager::get (K_CacheManager.hpp:163-260):
                                 the missing brick is requested and the first
                                 mapped coarser level is sampled instead; status
                                 bit 1 is then set.  Such an image is a preview,
                                 not the converged image: restart the view's
                                 progressive buffers every frame.               */
} gc_view;

/* Camera of updateViewMatrix (Display_helper.cpp:93-118): the rows of
 * glRotatef(-rx,1,0,0) * glRotatef(-ry,0,1,0) * glTranslatef(-t), computed in
 * double and rounded to float. */
int gc_view_matrix(const float rotation_deg[2], const float translation[3], float out[12]);
/* Camera placed at `eye` looking at `target`: columns (right, up, -forward, eye). */
int gc_look_at(const float eye[3], const float target[3], const float up[3], float out[12]);

/* Transfer function: TransferFunction::getSample / regenerateSamples
 * (TransferFunction.cpp:121-157): piecewise-linear RGBA between control
 * points sorted by value; sample i is taken at i / samples. */
typedef struct gc_tf_point {
    float value, alpha, r, g, b;
} gc_tf_point;
int gc_tf_build(const gc_tf_point *points, uint32_t n, uint32_t samples, float *out_rgba);

/* One view per launch, like get_frame (VolumeRayCaster.cu:356-429). */
int gc_render(gc_cache_t cache, const gc_view *view, void *stream);
/* Many views of uneven sizes in one persistent launch sharing the cache's
 * request buffer (one frame for the cache). */
int gc_render_batch(gc_cache_t cache, const gc_view *views, uint32_t n, void *stream);

/* Launch configuration of the ray caster (process-wide; results do not
 * depend on it): scheduler 0 = a warp marches one ray tile at a time,
 * 1 = each lane refills from the pixel queue when its ray ends; tile width
 * 4, 8, 16 or 32 (a warp tile is tile_w x 32/tile_w pixels); threads per
 * block 64, 128 or 256; blocks per SM cap (0 = occupancy limit).  Chosen by
 * the autotuner of the Python host (gcgb300.autotune_render). */
int gc_render_tuning_set(uint32_t scheduler, uint32_t tile_w, uint32_t threads, uint32_t blocks_per_sm);
int gc_render_tuning_get(uint32_t out[4]);
/* Arithmetic of the ray caster (process-wide).  GC_RENDER_EXACT (default):
 * every float operation separately rounded in a fixed order, exactly rounded
 * division, square root and power -- the same values as the FP32 oracle, bit
 * for bit.  GC_RENDER_FAST_BUILD: the same method compiled with fused
 * multiply-add contraction, rsqrtf, the hardware log2/exp2 pair for the
 * opacity correction and reciprocal multiplies (the operations of the
 * reference's own build); images within 1/255 of the double-precision
 * method except where a float decision of the march (early termination,
 * brick and level boundaries) lands within rounding distance. */
#define GC_RENDER_EXACT 0
#define GC_RENDER_FAST_BUILD 1
int gc_render_precision_set(int precision);
int gc_render_precision_get(int *precision);
/* Empty-space skipping (process-wide, on by default; images are identical
 * either way): each pool slot records the value range of its brick and each
 * DVR view of a one-channel volume the value range its transfer function can
 * make visible; a ray steps through a brick with no visible value without
 * sampling it (the same t steps; samples there stay below the 0.001
 * compositing threshold).  No counterpart in the reference. */
int gc_render_empty_skip(int enable);

/* ------------------------------------------------------------------------ */
/* The reference's on-disk brick store (BricksManager.cpp:81-227,
 * BrickKey.cpp:38-44, MetaData.cpp:36-216):
 *   <volume_dir>bricks_B_B_B/L<l>/L<l>_<x>_<y>_<z>.raw   one LZ4 block (LZ4_compress_HC
 *       level 9) of the (BB*B)^3 x encoded_bytes voxels of big brick (x, y, z)
 *   <volume_dir>bricks_B_B_B/bricks.xml                  level sizes, empty bricks
 * volume_dir is the reference's VolumeDirectory (a trailing '/' is added).
 * The codec is the system's liblz4, loaded at run time: without it these
 * calls return GC_ERR_UNSUPPORTED (gc_lz4_available() tells beforehand).
 * Stores are the in-memory layout of gc_cache_set_source_host (level l at
 * level_offsets[l], big bricks in (z, y, x) order); threads 0 = all cores. */
int gc_lz4_available(void);
int gc_brick_files_write(const char *volume_dir, const gc_volume_desc *vol, const gc_layout *layout,
                         const void *store, uint64_t bytes, const uint64_t *level_offsets, uint32_t threads);
int gc_brick_files_read(const char *volume_dir, const gc_volume_desc *vol, const gc_layout *layout, void *store,
                        uint64_t bytes, const uint64_t *level_offsets, uint32_t threads);
/* MetaData::write_bricks_xml: byte for byte the reference's file (histogram
 * bins all 0, as the reference never fills them). */
int gc_bricks_xml_write(const char *volume_dir, const gc_volume_desc *vol, const gc_layout *layout,
                        const uint64_t *empty_keys, size_t n_empty);
/* MetaData::load for the level sizes and the empty big bricks (up to
 * max_empty keys stored; *n_empty is the count in the file). */
int gc_bricks_xml_read(const char *path, uint32_t *n_levels, uint32_t initial[][3], uint32_t real[][3],
                       uint64_t *empty_keys, size_t max_empty, size_t *n_empty);

/* ------------------------------------------------------------------------ */
/* Continuous batching of views over one cache (the batched and served forms;
 * no counterpart in the reference, whose frame loop renders one view per
 * launch, VolumeRayCaster.cu:261-330).  Views are queued with their own
 * buffers.  A tick (1) installs the bricks the loader finished, (2) when
 * bricks were installed or the loader is idle, admits queued views within
 * the budgets, (3) renders in one persistent launch every
 * view that can progress -- the newly admitted ones, and all active views
 * when bricks were installed or the loader is idle; a view whose rays wait on
 * missing bricks cannot progress before the next install, so its pass is
 * skipped -- (4) updates the LRU order and, when the loader is idle, scans the
 * shared request buffer and hands the miss list to the loader, and (5)
 * retires the rendered views none of whose rays met an unmapped brick (or
 * that reached max_passes).  When nothing can be rendered it waits for the
 * loader (a few milliseconds at most).  A retired view's buffers hold its
 * final image, the one the plain per-view loop converges to.  The batch
 * requires the cache's asynchronous loader or its synchronous one alike. */
typedef struct gc_batch *gc_batch_t;
typedef struct gc_batch_desc {
    uint32_t max_views;      /* active views per launch (<= 256)              */
    uint64_t max_pixels;     /* admission budget: sum of W*H of active views  */
    uint32_t max_passes;     /* retire unconverged after this many passes (0: never) */
    float max_occupancy;     /* admission by cache memory: no view is admitted
                                while the active views' demand -- slots their
                                last full pass used plus the missing bricks
                                the last scan found -- exceeds this fraction
                                of the pool slots (<= 0: no limit)             */
    uint32_t max_admit;      /* views admitted per tick (0: no limit)          */
    float park_above;        /* memory-pressure parking: while that demand
                                exceeds this fraction of the pool slots and
                                more than one view is active, the most recently
                                admitted view leaves the batch for the front of
                                the queue with its progressive state kept, and
                                resumes when admission allows (<= 0: never; not
                                available with overlap_loads)                  */
    uint32_t reorder_window; /* locality-aware admission: pick, among the first
                                reorder_window queued views, the one whose
                                camera is nearest the last admitted view's
                                (views that look at the same bricks share
                                them in the cache); the oldest queued view is
                                admitted once passed over reorder_window
                                times.  0 or 1: arrival order.                 */
    uint32_t overlap_loads;  /* 1: overlap brick loads with rendering (needs the
                                cache's asynchronous loader).  The bricks of a
                                miss list are marked in flight in the page
                                directory (rays stop there without requesting
                                them again); while the loader uploads one list,
                                the views waiting on the previous one render
                                and scan into a second list.  Images are the
                                same.  0: one load at a time.                  */
} gc_batch_desc;
typedef struct gc_batch_result {
    uint64_t tag;
    uint32_t passes;         /* render passes the view took (skipped ones not counted) */
    uint32_t converged;      /* 1 if its last pass met no unmapped brick      */
    double latency_ms;       /* submit -> retirement, host clock              */
} gc_batch_result;
int gc_batch_create(gc_cache_t cache, const gc_batch_desc *desc, gc_batch_t *out);
int gc_batch_destroy(gc_batch_t batch);
/* Queue a view; its tbuf and state are cleared when it is admitted.  The
 * view's status field is managed by the batch.  While batched, tbuf and
 * state are the batch's scratch: a finished ray leaves -1 - t in tbuf so
 * that later passes skip its pixel; rgba holds the image. */
int gc_batch_submit(gc_batch_t batch, const gc_view *view, uint64_t tag);
/* One tick.  The render of a tick replays the batch's instantiated CUDA graph
 * (its view-table copy and persistent ray-caster nodes updated in place).
 * Outputs (optional): views active during the tick, views queued after it. */
int gc_batch_tick(gc_batch_t batch, void *stream, uint32_t *active, uint32_t *queued);
/* Retrieve up to max retired views (oldest first). */
int gc_batch_poll(gc_batch_t batch, gc_batch_result *out, uint32_t max, uint32_t *n);
/* Counters since the batch was created. */
typedef struct gc_batch_stats {
    uint64_t ticks;           /* gc_batch_tick calls                           */
    uint64_t render_ticks;    /* ticks that rendered (one launch each)         */
    uint64_t view_passes;     /* views rendered, summed over ticks             */
    uint64_t install_ticks;   /* ticks that installed bricks                   */
    uint64_t graph_replays;   /* render launches replayed from the batch's CUDA
                                 graph (view-table copy + persistent ray caster) */
    uint64_t parked;          /* views parked under memory pressure            */
    double render_ms;         /* device time of the render launches            */
    double tick_ms;           /* host time inside gc_batch_tick                */
    double wait_ms;           /* host time waiting for the loader              */
} gc_batch_stats;
int gc_batch_stats_get(gc_batch_t batch, gc_batch_stats *out);

#ifdef __cplusplus
}
#endif
#endif /* GC_GB300_H */
