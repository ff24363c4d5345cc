/*
 * gc_oracle.h -- CPU oracle of the out-of-core volume path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (ftilde/GPU-Out-of-Core-Volume-Data, GcCore) used to check the
 * CUDA implementation.  Only tests, the smoke check and the CPU-baseline leg
 * of the benchmark load it; the product library never does.
 */
#ifndef GC_ORACLE_H
#define GC_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "gc_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* synthetic volume (same integer definition as the product generator) */
int orc_blobs(uint32_t seed, uint32_t nblobs, const uint32_t size[3], float smin, float smax,
              int32_t amin, int32_t amax, gc_blob *out);
void orc_generate(const gc_generator *gen, void *dst);

/* level geometry */
int orc_layout(const gc_volume_desc *v, gc_layout *out);

/* one mip pass (down_sampling_inner) */
void orc_mip_level(const void *src, void *dst, const uint32_t dims[3], uint32_t eb, uint32_t nc);
void orc_mip_level_mt(const void *src, void *dst, const uint32_t dims[3], uint32_t eb, uint32_t nc, int threads);

/* bricking of one level (process_bricking); out receives all big bricks */
void orc_brick_level(const void *level, const uint32_t dims[3], const gc_volume_desc *v,
                     const uint32_t nb_big[3], void *out);

/* empty flags per big brick */
void orc_empty(const void *bricks, uint64_t nbig, uint64_t values_per_big, uint32_t cb, float threshold,
               uint8_t *flags);

/* cache state machine (one-level directory, or two levels: desc.pt_block) */
typedef struct orc_lru {
    uint32_t cx, cy, cz, level;
    float vx, vy, vz;
} orc_lru;

typedef struct orc_cache orc_cache;
orc_cache *orc_cache_create(const gc_cache_desc *desc);
void orc_cache_destroy(orc_cache *c);
void orc_cache_set_source(orc_cache *c, const void *bricks, const uint64_t *level_offsets,
                          const uint64_t *empty_keys, size_t n_empty);
/* CacheManager::update with a loader that completes before the next frame */
int orc_cache_update(orc_cache *c);
/* pieces of update, for replay tests */
void orc_lru_update(orc_cache *c);
uint32_t orc_request_list(orc_cache *c, uint32_t *out4, uint32_t max);
float orc_completude(const orc_cache *c);
uint32_t orc_timestamp(const orc_cache *c);
void orc_set_timestamp(orc_cache *c, uint32_t ts);
/* state access */
uint32_t *orc_mrpd(orc_cache *c);     /* 4 x uint32 per entry */
uint32_t *orc_requests(orc_cache *c);
uint32_t *orc_usage(orc_cache *c);
orc_lru *orc_lru_records(orc_cache *c);
uint8_t *orc_pool(orc_cache *c);
void orc_cache_dims(const orc_cache *c, uint32_t mrpd_dims[3], uint32_t *nslots, uint64_t *pool_bytes);
/* two-level directory (desc.pt_block > 0): dimensions and state, in the
 * layouts of the GC_DUMP_PT_* dumps; orc_mrpd then returns the flat entries
 * materialized from it */
void orc_pt_dims(const orc_cache *c, uint32_t dims[3], uint32_t *slots, uint32_t *block);
uint32_t *orc_pt_top(orc_cache *c);
uint32_t *orc_pt_table(orc_cache *c);
uint32_t *orc_pt_order(orc_cache *c);
uint32_t *orc_pt_usage(orc_cache *c);
uint32_t *orc_pt_keys(orc_cache *c);

/* ray caster, FP32 mirror of the CUDA kernel's operation sequence
 * (threads = 0 -> all cores) */
void orc_render(orc_cache *c, const gc_view *view, const float *tf, uint32_t *rgba, float *tbuf,
                float *state, int threads);
/* same method in double precision, exact pow/sqrt; reads the cache state,
 * writes usage/requests into the given buffers (may be the cache's own) */
void orc_render_f64(orc_cache *c, const gc_view *view, const float *tf, uint32_t *rgba, double *tbuf,
                    double *state, uint32_t *usage, uint32_t *req, int threads);

/* one sample of K_CacheManager::get_normalized with a fresh page walk:
 * 0 mapped (*out written, usage stamped), 1 unmapped (requested), 2 empty */
int orc_sample_normalized(orc_cache *c, uint32_t level, float x, float y, float z, float *out);

/* exposed for unit tests of the series pow */
float orc_pow(float x, float k);

#ifdef __cplusplus
}
#endif
#endif
