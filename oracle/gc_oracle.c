/*
 * gc_oracle.c -- CPU oracle of the out-of-core volume path.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker.  The product never links it.
 *
 * Each function restates one reference algorithm (paths relative to the
 * reference repository):
 *   orc_layout        Mipmapper.cu:441-443, 583-597; Bricker_v2.cpp:45-76
 *   orc_mip_level     Mipmapper.cu:29-105 (down_sampling_inner), loops kept
 *   orc_brick_level   Bricker_v2.cpp:79-252 (process_bricking), loops kept
 *   orc_empty         BrickProcessor.hpp:37-51, BrickProcessorPredicate.hpp:11-46
 *   orc_cache_*       CacheManager.hpp:135-670, CacheDevice.hpp:146-219,
 *                     CacheManagerKernels.cu:8-125, CacheManagerKernels.hpp:59-357,
 *                     RequestHandler.hpp:277-372
 *   orc_cache_* with desc.pt_block > 0 (two-level directory)   the page-table
 *                     hierarchy of CacheManager.hpp:151-236 and
 *                     CacheManagerKernels.hpp:148-357 with one table cache,
 *                     restated as this library defines it (see entry_of and
 *                     load_new_bricks): the reference's own multi-level walk
 *                     is used by no configuration and does not keep its
 *                     directory consistent: downward writes stack entry 0
 *                     only for a mapped directory word (CacheManagerKernels.hpp:
 *                     193-198), so upward reads the previous brick's entry 0
 *                     (:255) and files the brick into that brick's block; a
 *                     block taken for an empty brick is flagged empty in the
 *                     directory (:245-250); the eviction walk writes through
 *                     an unmapped word (:130-138)
 *   orc_render        RayCasters.cu:35-349, 484-567; K_CacheManager.hpp:265-396;
 *                     K_CacheDevice.hpp:188-336; K_MultiResolutionPageDirectory.hpp:141-180;
 *                     VolumeRayCaster.cu:136-161
 *   orc_render (two channels, 2D transfer function)   no reference counterpart
 *
 * Pinning (how the restatement is tied to the reference):
 *   orc_layout, orc_brick_level   PINNED: checked against outputs of the
 *       reference's own init_meta_data / process_bricking compiled from its
 *       sources (tests/golden/layout.json, bricker.json; oracle/build.py).
 *   bricks.xml format             PINNED: goldens written by the reference's
 *       MetaData::write_bricks_xml (tests/golden/bricks_xml/).
 *   orc_mip_level, orc_empty, orc_cache_*, orc_render   the reference implements
 *       them as CUDA kernels; they are pinned on the GPU, where the reference's
 *       own CUDA build runs beside the CUDA path (oracle/ref_gpu_driver.cu,
 *       tests/test_gpu_reference.py), and checked by closed-form properties
 *       and the FP64 restatement (orc_render_f64) everywhere.  Two-channel
 *       rendering and the two-level directory have no reference execution.
 *
 * Build with -ffp-contract=off: every float operation is rounded separately,
 * in source order, like the CUDA kernels built with -fmad=false; the fused
 * multiply-adds of the CUDA ray caster are written here as fmaf at the same
 * places.
 */
#include "gc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* synthetic volume: same definition as the product's generate.cu            */

static uint64_t splitmix64(uint64_t *s) {
    uint64_t z;
    *s += 0x9E3779B97F4A7C15ull;
    z = *s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double unit01(uint64_t *s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

int orc_blobs(uint32_t seed, uint32_t nblobs, const uint32_t size[3], float smin, float smax, int32_t amin,
              int32_t amax, gc_blob *out) {
    uint64_t s = 0x5DEECE66Dull ^ ((uint64_t)seed << 17) ^ seed;
    for (uint32_t i = 0; i < nblobs; ++i) {
        gc_blob b;
        memset(&b, 0, sizeof(b));
        b.cx = (int32_t)(unit01(&s) * size[0]);
        b.cy = (int32_t)(unit01(&s) * size[1]);
        b.cz = (int32_t)(unit01(&s) * size[2]);
        for (int a = 0; a < 3; ++a) {
            double sigma = smin + unit01(&s) * (smax - smin);
            b.k[a] = (uint64_t)(274877906944.0 / (9.0 * sigma * sigma));
            if (b.k[a] == 0) b.k[a] = 1;
            b.r[a] = (int32_t)ceil(3.0 * sigma) + 1;
        }
        b.amplitude = amin + (int32_t)(unit01(&s) * (amax - amin + 1));
        if (b.amplitude > amax) b.amplitude = amax;
        out[i] = b;
    }
    return 0;
}

static uint32_t lattice_hash(int32_t ix, int32_t iy, int32_t iz, uint32_t octave, uint32_t seed) {
    uint32_t h = seed * 0x9E3779B1u;
    h ^= (uint32_t)ix * 0x85EBCA77u;
    h = (h << 13) | (h >> 19);
    h ^= (uint32_t)iy * 0xC2B2AE3Du;
    h = (h << 11) | (h >> 21);
    h ^= (uint32_t)iz * 0x27D4EB2Fu;
    h ^= octave * 0x165667B1u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h;
}
static int64_t lattice_value(int32_t ix, int32_t iy, int32_t iz, uint32_t o, uint32_t seed) {
    return (int64_t)(lattice_hash(ix, iy, iz, o, seed) >> 16) - 32768;
}
static int64_t lerp_q16(int64_t a, int64_t b, int64_t w) { return a + (((b - a) * w) >> 16); }
static int64_t value_noise(uint32_t x, uint32_t y, uint32_t z, uint32_t lp, uint32_t o, uint32_t seed) {
    int32_t ix = (int32_t)(x >> lp), iy = (int32_t)(y >> lp), iz = (int32_t)(z >> lp);
    uint32_t mask = (1u << lp) - 1u;
    int64_t wx = (int64_t)(x & mask) << (16 - lp), wy = (int64_t)(y & mask) << (16 - lp),
            wz = (int64_t)(z & mask) << (16 - lp);
    int64_t c00 = lerp_q16(lattice_value(ix, iy, iz, o, seed), lattice_value(ix + 1, iy, iz, o, seed), wx);
    int64_t c10 = lerp_q16(lattice_value(ix, iy + 1, iz, o, seed), lattice_value(ix + 1, iy + 1, iz, o, seed), wx);
    int64_t c01 = lerp_q16(lattice_value(ix, iy, iz + 1, o, seed), lattice_value(ix + 1, iy, iz + 1, o, seed), wx);
    int64_t c11 =
        lerp_q16(lattice_value(ix, iy + 1, iz + 1, o, seed), lattice_value(ix + 1, iy + 1, iz + 1, o, seed), wx);
    return lerp_q16(lerp_q16(c00, c10, wy), lerp_q16(c01, c11, wy), wz);
}

void orc_generate(const gc_generator *g, void *dst) {
    const int64_t maxval = g->bytes_per_channel == 1 ? 255 : 65535;
    /* every voxel is independent: rows spread over the host threads */
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(dynamic, 16)
#endif
    for (uint32_t z = 0; z < g->size[2]; ++z)
        for (uint32_t y = 0; y < g->size[1]; ++y)
            for (uint32_t x = 0; x < g->size[0]; ++x) {
                int64_t v = 0;
                if (g->field == 0) {
                    for (uint32_t bi = 0; bi < g->nblobs; ++bi) {
                        const gc_blob *b = &g->blobs[bi];
                        int64_t dx = (int64_t)x - b->cx, dy = (int64_t)y - b->cy, dz = (int64_t)z - b->cz;
                        uint64_t s = (uint64_t)(dx * dx) * b->k[0] + (uint64_t)(dy * dy) * b->k[1] +
                                     (uint64_t)(dz * dz) * b->k[2];
                        int64_t q = (int64_t)(s >> 22);
                        if (q < 65536) {
                            int64_t w = 65536 - q, w2 = (w * w) >> 16, w4 = (w2 * w2) >> 16;
                            v += ((int64_t)b->amplitude * w4) >> 16;
                        }
                    }
                }
                {
                    int64_t n = value_noise(x, y, z, 6, 0, g->seed) + (value_noise(x, y, z, 5, 1, g->seed) >> 1) +
                                (value_noise(x, y, z, 4, 2, g->seed) >> 2);
                    v += (n * g->noise_amplitude) / 57344;
                }
                if (g->field == 1) v += maxval / 2;
                if (v < 0) v = 0;
                if (v > maxval) v = maxval;
                uint64_t idx = (((uint64_t)z * g->size[1] + y) * g->size[0] + x) * g->channels + g->channel;
                if (g->bytes_per_channel == 1)
                    ((uint8_t *)dst)[idx] = (uint8_t)v;
                else
                    ((uint16_t *)dst)[idx] = (uint16_t)v;
            }
}

/* ------------------------------------------------------------------------ */
int orc_layout(const gc_volume_desc *v, gc_layout *L) {
    memset(L, 0, sizeof(*L));
    uint32_t B = v->brick_size;
    uint32_t maxDim = v->size[0];
    if (v->size[1] > maxDim) maxDim = v->size[1];
    if (v->size[2] > maxDim) maxDim = v->size[2];
    /* Mipmapper.cu:443 */
    uint32_t levelMax = (uint32_t)ceil(log((double)(maxDim / B)) / log(2.0));
    if (levelMax + 1 > GC_MAX_LEVELS) return -1;
    L->nb_levels = levelMax + 1;
    uint32_t s[3] = {v->size[0], v->size[1], v->size[2]};
    uint32_t m[3] = {v->size[0], v->size[1], v->size[2]};
    for (uint32_t l = 0; l <= levelMax; ++l) {
        for (int a = 0; a < 3; ++a) {
            L->initial[l][a] = s[a];
            L->mip[l][a] = m[a];
        }
        for (int a = 0; a < 3; ++a) {
            if (s[a] >= v->downscale[a]) s[a] /= v->downscale[a]; /* fill_metaData */
            m[a] = m[a] / v->downscale[a];
            if (m[a] < 1) m[a] = 1;
        }
    }
    uint32_t Beff = B - 2 * v->covering;
    for (uint32_t l = 0; l <= levelMax; ++l)
        for (int a = 0; a < 3; ++a) {
            uint32_t nb = (uint32_t)ceilf((float)L->initial[l][a] / (float)Beff);
            nb = (uint32_t)ceilf((float)nb / (float)v->big_brick_size[a]) * v->big_brick_size[a];
            L->nb_bricks[l][a] = nb;
            L->nb_big_bricks[l][a] = nb / v->big_brick_size[a];
            L->real[l][a] = nb * Beff;
        }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* down_sampling_inner for one z pair, as the kernel indexes it: the input
 * holds the 2 slices of the chunk, rows of inputWidth voxels. */
void orc_mip_level(const void *src, void *dst, const uint32_t dims[3], uint32_t eb, uint32_t nc) {
    orc_mip_level_mt(src, dst, dims, eb, nc, 1);
}

/* The same, z pairs spread over `threads` host threads (<= 0: all). */
void orc_mip_level_mt(const void *src, void *dst, const uint32_t dims[3], uint32_t eb, uint32_t nc, int threads) {
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#else
    (void)threads;
#endif
    const uint8_t *in = (const uint8_t *)src;
    uint8_t *out = (uint8_t *)dst;
    const uint32_t inputWidth = dims[0], inputHeight = dims[1];
    const uint32_t inputWidthStep = dims[0] * eb;
    const uint32_t outputWidthStep = (dims[0] / 2) * eb;
    const uint32_t outputWidth = inputWidth / 2 * nc;
    const uint32_t outputHeight = inputHeight / 2;
    const uint64_t in_slice2 = (uint64_t)inputWidthStep * inputHeight * 2;
    const uint64_t out_slice = (uint64_t)outputWidthStep * outputHeight;
    const int64_t nz = dims[2] / 2;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(threads)
#endif
    for (int64_t oz = 0; oz < nz; ++oz) {
        const uint8_t *input = in + oz * in_slice2;
        uint8_t *output = out + oz * out_slice;
        for (uint32_t outputYIndex = 0; outputYIndex < outputHeight; ++outputYIndex)
            for (uint32_t outputXIndex = 0; outputXIndex < outputWidth; ++outputXIndex) {
                uint32_t output_tid = (outputYIndex * outputWidthStep) + (outputXIndex * (eb / nc));
                uint32_t inputXIndexStart = ((outputXIndex / nc) * 2) * eb + (outputXIndex % nc);
                uint32_t inputXIndexEnd = inputXIndexStart + (2 - 1) * eb;
                uint32_t inputYIndexStart = outputYIndex * 2;
                uint32_t inputYIndexEnd = inputYIndexStart + 2;
                if (nc == 1 && eb > 1) {
                    double channelSum = 0.0; /* uninitialised in the reference */
                    for (uint32_t zz = 0; zz < 2; ++zz)
                        for (uint32_t yy = inputYIndexStart; yy < inputYIndexEnd; ++yy)
                            for (uint32_t xx = inputXIndexStart; xx <= inputXIndexEnd; xx += eb) {
                                uint32_t input_tid = zz * (inputWidthStep * inputHeight) + (yy * inputWidthStep) + xx;
                                if (eb == 2)
                                    channelSum += (double)((const uint16_t *)input)[input_tid / eb];
                                else
                                    channelSum += (double)((const float *)input)[input_tid / eb];
                            }
                    double r = channelSum / 8.0;
                    if (eb == 2)
                        ((uint16_t *)output)[output_tid / eb] = (uint16_t)r;
                    else
                        ((float *)output)[output_tid / eb] = (float)r;
                } else if (eb / nc == 1) {
                    uint64_t channelSum = 0;
                    for (uint32_t zz = 0; zz < 2; ++zz)
                        for (uint32_t yy = inputYIndexStart; yy < inputYIndexEnd; ++yy)
                            for (uint32_t xx = inputXIndexStart; xx <= inputXIndexEnd; xx += eb) {
                                uint32_t input_tid = zz * (inputWidthStep * inputHeight) + (yy * inputWidthStep) + xx;
                                channelSum += input[input_tid];
                            }
                    output[output_tid] = (uint8_t)(channelSum / 8);
                } else {
                    /* multi-byte channels interleaved: the reference reads single
                     * bytes here; this oracle takes the per-channel floor mean. */
                    uint32_t cb = eb / nc, c = outputXIndex % nc, ox = outputXIndex / nc;
                    uint64_t sum = 0;
                    for (uint32_t zz = 0; zz < 2; ++zz)
                        for (uint32_t yy = inputYIndexStart; yy < inputYIndexEnd; ++yy)
                            for (uint32_t dx = 0; dx < 2; ++dx) {
                                const uint8_t *p = input + zz * (uint64_t)(inputWidthStep * inputHeight) +
                                                   (uint64_t)yy * inputWidthStep + (uint64_t)(2 * ox + dx) * eb + c * cb;
                                sum += (cb == 2) ? *(const uint16_t *)p : *p;
                            }
                    uint8_t *o = output + (uint64_t)outputYIndex * outputWidthStep + (uint64_t)ox * eb + c * cb;
                    if (cb == 2)
                        *(uint16_t *)o = (uint16_t)(sum / 8);
                    else
                        *o = (uint8_t)(sum / 8);
                }
            }
    }
}

/* ------------------------------------------------------------------------ */
/* process_bricking with the file replaced by the in-memory level. */
void orc_brick_level(const void *levelp, const uint32_t dims[3], const gc_volume_desc *v, const uint32_t nb_big[3],
                     void *outp) {
    const uint8_t *level = (const uint8_t *)levelp;
    uint8_t *out = (uint8_t *)outp;
    const uint32_t covering = v->covering, B = v->brick_size, E = v->encoded_bytes;
    const uint32_t bs[3] = {B - 2 * covering, B - 2 * covering, B - 2 * covering};
    const uint32_t *BBs = v->big_brick_size;
    const uint32_t endX = dims[0], endY = dims[1], endZ = dims[2];
    const uint32_t bvx = BBs[0] * B, bvy = BBs[1] * B, bvz = BBs[2] * B;
    const uint64_t bigBytes = (uint64_t)bvx * bvy * bvz * E;
    uint8_t *brick = (uint8_t *)malloc(bigBytes);
    uint32_t big[3] = {0, 0, 0};
    for (;;) {
        memset(brick, 0, bigBytes);
        uint32_t bp[3] = {0, 0, 0};
        for (;;) {
            uint32_t absBrick[3], absPos[3];
            for (int a = 0; a < 3; ++a) {
                absBrick[a] = (big[a] * BBs[a] + bp[a]) * bs[a];
                absPos[a] = bp[a] * B;
            }
            uint32_t brickX = 0;
            if (absBrick[0] + brickX == 0) brickX += covering;
            int32_t absX = (int32_t)(absBrick[0] + brickX - covering);
            for (uint32_t brickZ = 0; brickZ < B; ++brickZ) {
                int32_t absZ = (int32_t)(absBrick[2] + brickZ - covering);
                if (absZ < 0 && brickZ < covering) continue;
                if (absZ >= (int32_t)dims[2]) break;
                for (uint32_t brickY = 0; brickY < B; ++brickY) {
                    int32_t absY = (int32_t)(absBrick[1] + brickY - covering);
                    if (absY < 0 && brickY < covering) continue;
                    if (absY >= (int32_t)dims[1]) break;
                    uint64_t pos = ((uint64_t)(uint32_t)absX + (uint64_t)dims[0] * ((uint64_t)(uint32_t)absY +
                                                                                     (uint64_t)(uint32_t)absZ * dims[1])) * E;
                    uint32_t XToRead;
                    if ((uint32_t)absX + B > dims[0]) {
                        if (absX == 0)
                            XToRead = dims[0];
                        else
                            XToRead = dims[0] - (uint32_t)absX;
                    } else
                        XToRead = B - brickX;
                    uint64_t d = ((uint64_t)(absPos[0] + brickX) +
                                  (uint64_t)bvx * ((absPos[1] + brickY) + (uint64_t)(absPos[2] + brickZ) * bvy)) * E;
                    uint64_t n = (uint64_t)XToRead * E;
                    if (d + n > bigBytes) n = bigBytes - d; /* the reference would overrun its vector */
                    memcpy(brick + d, level + pos, n);
                }
            }
            if ((big[0] * BBs[0] + bp[0] + 1) * bs[0] < endX && (bp[0] + 1) < BBs[0])
                ++bp[0];
            else {
                bp[0] = 0;
                if ((big[1] * BBs[1] + bp[1] + 1) * bs[1] < endY && (bp[1] + 1) < BBs[1])
                    ++bp[1];
                else {
                    bp[1] = 0;
                    if ((big[2] * BBs[2] + bp[2] + 1) * bs[2] < endZ && (bp[2] + 1) < BBs[2])
                        ++bp[2];
                    else
                        break;
                }
            }
        }
        {
            uint64_t idx = ((uint64_t)big[2] * nb_big[1] + big[1]) * nb_big[0] + big[0];
            memcpy(out + idx * bigBytes, brick, bigBytes);
        }
        if ((big[0] + 1) * BBs[0] * bs[0] < endX)
            ++big[0];
        else {
            big[0] = 0;
            if ((big[1] + 1) * BBs[1] * bs[1] < endY)
                ++big[1];
            else {
                big[1] = 0;
                if ((big[2] + 1) * BBs[2] * bs[2] < endZ)
                    ++big[2];
                else
                    break;
            }
        }
    }
    free(brick);
}

void orc_empty(const void *bricks, uint64_t nbig, uint64_t values, uint32_t cb, float threshold, uint8_t *flags) {
    for (uint64_t b = 0; b < nbig; ++b) {
        int empty = 1;
        for (uint64_t i = 0; i < values && empty; ++i) {
            float val;
            if (cb == 1)
                val = (float)((const uint8_t *)bricks)[b * values + i];
            else if (cb == 2)
                val = (float)((const uint16_t *)bricks)[b * values + i];
            else
                val = ((const float *)bricks)[b * values + i];
            if (!(val < threshold)) empty = 0;
        }
        flags[b] = (uint8_t)empty;
    }
}

/* ------------------------------------------------------------------------ */
/* cache                                                                     */

struct orc_cache {
    gc_cache_desc d;
    uint32_t B, c, Beff, eb, nl;
    uint32_t sx, sy, sz, nslots;
    uint32_t mx, my, mz;
    uint64_t nentries, brick_bytes, big_bytes;
    uint32_t off[GC_MAX_LEVELS], nb[GC_MAX_LEVELS][3], vvox[GC_MAX_LEVELS][3];
    float ior[GC_MAX_LEVELS][3];
    uint32_t *mrpd, *req, *usage;
    orc_lru *lru, *tmp;
    uint8_t *pool;
    uint32_t ts;
    int request_done;
    uint32_t n_asked, n_nonempty;
    uint32_t *list, *asked, *big_index, *big_coord;
    uint8_t *staging;
    const uint8_t *src;
    uint64_t level_off[GC_MAX_LEVELS];
    uint64_t *empty;
    size_t n_empty;
    /* two-level directory (d.pt_block > 0): directory words, table pool,
     * its usage words, LRU order (slot ids) and the block each slot holds */
    uint32_t pts, pt_slots, ptx, pty, ptz, pt_off[GC_MAX_LEVELS];
    uint64_t pt_words;
    uint32_t *pt_top, *pt_table, *pt_usage, *pt_order, *pt_tmp, *pt_keys;
};

orc_cache *orc_cache_create(const gc_cache_desc *d) {
    orc_cache *c = (orc_cache *)calloc(1, sizeof(orc_cache));
    c->d = *d;
    c->B = d->volume.brick_size;
    c->c = d->volume.covering;
    c->Beff = c->B - 2 * c->c;
    c->eb = d->volume.encoded_bytes;
    c->nl = d->layout.nb_levels;
    c->sx = d->cache_size[0];
    c->sy = d->cache_size[1];
    c->sz = d->cache_size[2];
    c->nslots = c->sx * c->sy * c->sz;
    uint32_t off = 0;
    for (uint32_t l = 0; l < c->nl; ++l) {
        c->off[l] = off;
        for (int a = 0; a < 3; ++a) {
            c->nb[l][a] = d->layout.nb_bricks[l][a];
            c->vvox[l][a] = d->layout.nb_bricks[l][a] * c->Beff;
            c->ior[l][a] = (float)d->layout.initial[l][a] / (float)d->layout.real[l][a];
        }
        off += c->nb[l][0];
        if (c->nb[l][1] > c->my) c->my = c->nb[l][1];
        if (c->nb[l][2] > c->mz) c->mz = c->nb[l][2];
    }
    c->mx = off;
    c->nentries = (uint64_t)c->mx * c->my * c->mz;
    c->brick_bytes = (uint64_t)c->B * c->B * c->B * c->eb;
    c->big_bytes = c->brick_bytes * d->volume.big_brick_size[0] * d->volume.big_brick_size[1] *
                   d->volume.big_brick_size[2];
    c->mrpd = (uint32_t *)calloc(c->nentries * 4, sizeof(uint32_t));
    if (d->pt_block) {
        /* one directory word per P^3 bricks of a level: ceil(bricks / P) per
         * axis (CacheManager.hpp:160-176), levels packed along x */
        const uint32_t P = d->pt_block;
        while ((1u << c->pts) < P) ++c->pts;
        c->pt_slots = d->pt_slots;
        uint32_t toff = 0;
        for (uint32_t l = 0; l < c->nl; ++l) {
            c->pt_off[l] = toff;
            toff += (c->nb[l][0] + P - 1) / P;
            if ((c->nb[l][1] + P - 1) / P > c->pty) c->pty = (c->nb[l][1] + P - 1) / P;
            if ((c->nb[l][2] + P - 1) / P > c->ptz) c->ptz = (c->nb[l][2] + P - 1) / P;
        }
        c->ptx = toff;
        c->pt_words = (uint64_t)c->ptx * c->pty * c->ptz;
        c->pt_top = (uint32_t *)calloc(c->pt_words, sizeof(uint32_t));
        c->pt_table = (uint32_t *)calloc(((uint64_t)c->pt_slots << (3 * c->pts)) * 4, sizeof(uint32_t));
        c->pt_usage = (uint32_t *)calloc(c->pt_slots, sizeof(uint32_t));
        c->pt_order = (uint32_t *)calloc(c->pt_slots, sizeof(uint32_t));
        c->pt_tmp = (uint32_t *)calloc(c->pt_slots, sizeof(uint32_t));
        c->pt_keys = (uint32_t *)malloc((size_t)c->pt_slots * 4 * sizeof(uint32_t));
        for (uint32_t i = 0; i < c->pt_slots; ++i) c->pt_order[i] = i;
        memset(c->pt_keys, 0xff, (size_t)c->pt_slots * 4 * sizeof(uint32_t));
    }
    c->req = (uint32_t *)calloc(c->nentries, sizeof(uint32_t));
    c->usage = (uint32_t *)calloc(c->nslots, sizeof(uint32_t));
    c->lru = (orc_lru *)calloc(c->nslots, sizeof(orc_lru));
    c->tmp = (orc_lru *)calloc(c->nslots, sizeof(orc_lru));
    c->pool = (uint8_t *)calloc(c->nslots * c->brick_bytes, 1);
    /* LRU init in slot raster order (CacheDevice.hpp:152-165) */
    for (uint32_t z = 0; z < c->sz; ++z)
        for (uint32_t y = 0; y < c->sy; ++y)
            for (uint32_t x = 0; x < c->sx; ++x) {
                orc_lru *r = &c->lru[x + y * c->sx + z * c->sx * c->sy];
                r->cx = x * c->B;
                r->cy = y * c->B;
                r->cz = z * c->B;
                r->level = 0;
                r->vx = r->vy = r->vz = -1.f;
            }
    c->ts = 1;
    uint32_t m = d->max_requests;
    c->list = (uint32_t *)calloc(4 * m, sizeof(uint32_t));
    c->asked = (uint32_t *)calloc(4 * m, sizeof(uint32_t));
    c->big_index = (uint32_t *)calloc(m, sizeof(uint32_t));
    c->big_coord = (uint32_t *)calloc(4 * m, sizeof(uint32_t));
    c->staging = (uint8_t *)calloc(m * c->big_bytes, 1);
    return c;
}

void orc_cache_destroy(orc_cache *c) {
    if (!c) return;
    free(c->mrpd);
    free(c->req);
    free(c->usage);
    free(c->lru);
    free(c->tmp);
    free(c->pool);
    free(c->list);
    free(c->asked);
    free(c->big_index);
    free(c->big_coord);
    free(c->staging);
    free(c->empty);
    free(c->pt_top);
    free(c->pt_table);
    free(c->pt_usage);
    free(c->pt_order);
    free(c->pt_tmp);
    free(c->pt_keys);
    free(c);
}

void orc_cache_set_source(orc_cache *c, const void *bricks, const uint64_t *level_offsets, const uint64_t *keys,
                          size_t n) {
    c->src = (const uint8_t *)bricks;
    for (uint32_t l = 0; l < c->nl; ++l) c->level_off[l] = level_offsets[l];
    free(c->empty);
    c->empty = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
    if (n) memcpy(c->empty, keys, n * sizeof(uint64_t));
    c->n_empty = n;
}

static uint32_t *entry_of(orc_cache *c, uint32_t l, uint32_t x, uint32_t y, uint32_t z, int stamp);

/* With a two-level directory the flat entries are materialized from it (0
 * where the brick's block is not resident). */
uint32_t *orc_mrpd(orc_cache *c) {
    if (c->pts) {
        memset(c->mrpd, 0, c->nentries * 16);
        for (uint32_t l = 0; l < c->nl; ++l)
            for (uint32_t z = 0; z < c->nb[l][2]; ++z)
                for (uint32_t y = 0; y < c->nb[l][1]; ++y)
                    for (uint32_t x = 0; x < c->nb[l][0]; ++x) {
                        const uint32_t *e = entry_of(c, l, x, y, z, 0);
                        const uint64_t i = (uint64_t)(c->off[l] + x) + (uint64_t)y * c->mx + (uint64_t)z * c->mx * c->my;
                        if (e) memcpy(&c->mrpd[4 * i], e, 16);
                    }
    }
    return c->mrpd;
}
void orc_pt_dims(const orc_cache *c, uint32_t dims[3], uint32_t *slots, uint32_t *block) {
    dims[0] = c->ptx;
    dims[1] = c->pty;
    dims[2] = c->ptz;
    *slots = c->pt_slots;
    *block = c->pts ? 1u << c->pts : 0u;
}
uint32_t *orc_pt_top(orc_cache *c) { return c->pt_top; }
uint32_t *orc_pt_table(orc_cache *c) { return c->pt_table; }
uint32_t *orc_pt_order(orc_cache *c) { return c->pt_order; }
uint32_t *orc_pt_usage(orc_cache *c) { return c->pt_usage; }
uint32_t *orc_pt_keys(orc_cache *c) { return c->pt_keys; }
uint32_t *orc_requests(orc_cache *c) { return c->req; }
uint32_t *orc_usage(orc_cache *c) { return c->usage; }
orc_lru *orc_lru_records(orc_cache *c) { return c->lru; }
uint8_t *orc_pool(orc_cache *c) { return c->pool; }
uint32_t orc_timestamp(const orc_cache *c) { return c->ts; }
void orc_set_timestamp(orc_cache *c, uint32_t ts) { c->ts = ts; }
void orc_cache_dims(const orc_cache *c, uint32_t md[3], uint32_t *nslots, uint64_t *pool_bytes) {
    md[0] = c->mx;
    md[1] = c->my;
    md[2] = c->mz;
    *nslots = c->nslots;
    *pool_bytes = c->nslots * c->brick_bytes;
}

static uint32_t slot_of(const orc_cache *c, uint32_t cx, uint32_t cy, uint32_t cz) {
    return cx / c->B + (cy / c->B) * c->sx + (cz / c->B) * c->sx * c->sy;
}

/* Two-level directory: the directory word of brick (x, y, z) of level l (x
 * inside the level) and the place of its entry in the word's block. */
static uint64_t pt_word_of(const orc_cache *c, uint32_t l, uint32_t x, uint32_t y, uint32_t z) {
    return (uint64_t)(c->pt_off[l] + (x >> c->pts)) + (uint64_t)(y >> c->pts) * c->ptx +
           (uint64_t)(z >> c->pts) * c->ptx * c->pty;
}
static uint32_t pt_local_of(const orc_cache *c, uint32_t x, uint32_t y, uint32_t z) {
    const uint32_t m = (1u << c->pts) - 1u;
    return (x & m) | ((y & m) << c->pts) | ((z & m) << (2 * c->pts));
}
/* The 4-word entry of a brick, or NULL when its table block is not resident
 * (two levels).  stamp: a read of the page walk, which stamps the table
 * slot's usage word (the reference's table-cache read, K_CacheDevice.hpp:314-336). */
static uint32_t *entry_of(orc_cache *c, uint32_t l, uint32_t x, uint32_t y, uint32_t z, int stamp) {
    if (!c->pts) return &c->mrpd[4 * ((uint64_t)(c->off[l] + x) + (uint64_t)y * c->mx + (uint64_t)z * c->mx * c->my)];
    const uint32_t t = c->pt_top[pt_word_of(c, l, x, y, z)];
    if (!(t & 1u)) return NULL;
    if (stamp) __atomic_store_n(&c->pt_usage[t >> 1], c->ts, __ATOMIC_RELAXED);
    return &c->pt_table[4 * (((uint64_t)(t >> 1) << (3 * c->pts)) + pt_local_of(c, x, y, z))];
}

/* create_mask + CacheDevice::update: stable partition, used first */
void orc_lru_update(orc_cache *c) {
    uint32_t k = 0;
    for (uint32_t i = 0; i < c->nslots; ++i) {
        const orc_lru *r = &c->lru[i];
        if (c->usage[slot_of(c, r->cx, r->cy, r->cz)] == c->ts) c->tmp[k++] = *r;
    }
    for (uint32_t i = 0; i < c->nslots; ++i) {
        const orc_lru *r = &c->lru[i];
        if (c->usage[slot_of(c, r->cx, r->cy, r->cz)] != c->ts) c->tmp[k++] = *r;
    }
    orc_lru *t = c->lru;
    c->lru = c->tmp;
    c->tmp = t;
    if (c->pts) {  /* the table pool's LRU, the same stable partition */
        k = 0;
        for (uint32_t i = 0; i < c->pt_slots; ++i)
            if (c->pt_usage[c->pt_order[i]] == c->ts) c->pt_tmp[k++] = c->pt_order[i];
        for (uint32_t i = 0; i < c->pt_slots; ++i)
            if (c->pt_usage[c->pt_order[i]] != c->ts) c->pt_tmp[k++] = c->pt_order[i];
        uint32_t *u = c->pt_order;
        c->pt_order = c->pt_tmp;
        c->pt_tmp = u;
    }
}

/* create_request_list: indexes in [0, size - 1) with req == ts, first max,
 * decoded by coord_1D_to_3D.  Returns the number of flagged entries. */
uint32_t orc_request_list(orc_cache *c, uint32_t *out4, uint32_t max) {
    uint32_t count = 0;
    uint64_t sizeX = c->mx, sizeY = c->nb[0][1];
    for (uint64_t i = 0; i + 1 < c->nentries; ++i) {
        if (c->req[i] != c->ts) continue;
        if (count < max) {
            uint64_t index = i;
            uint32_t z = (uint32_t)(index / (sizeX * sizeY));
            index -= (uint64_t)z * (sizeX * sizeY);
            uint32_t y = (uint32_t)(index / sizeX);
            index -= (uint64_t)y * sizeX;
            uint32_t x = (uint32_t)index;
            uint32_t sumX = 0, level;
            for (level = 0; level < c->nl; ++level) {
                sumX += c->nb[level][0];
                if (x < sumX) break;
            }
            out4[4 * count + 0] = x - (sumX - c->nb[level][0]);
            out4[4 * count + 1] = y;
            out4[4 * count + 2] = z;
            out4[4 * count + 3] = level;
        }
        ++count;
    }
    return count;
}

static uint64_t brick_key(uint32_t l, uint32_t x, uint32_t y, uint32_t z) {
    return (uint64_t)(uint16_t)l | ((uint64_t)(uint16_t)x << 16) | ((uint64_t)(uint16_t)y << 32) |
           ((uint64_t)(uint16_t)z << 48);
}
static int is_empty_key(const orc_cache *c, uint64_t k) {
    for (size_t i = 0; i < c->n_empty; ++i)
        if (c->empty[i] == k) return 1;
    return 0;
}

/* RequestHandler::handle_request with an in-memory brick store */
static void handle_request(orc_cache *c, uint32_t n) {
    const uint32_t *BB = c->d.volume.big_brick_size;
    uint64_t *keys = (uint64_t *)malloc(n * sizeof(uint64_t));
    int32_t *vals = (int32_t *)malloc(n * sizeof(int32_t));
    int *kind = (int *)malloc(n * sizeof(int));
    uint32_t nkeys = 0, nne = 0, nbig = 0;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t *b = &c->list[4 * i];
        uint32_t gx = b[0] / BB[0], gy = b[1] / BB[1], gz = b[2] / BB[2];
        uint64_t key = brick_key(b[3], gx, gy, gz);
        int found = -1;
        for (uint32_t k = 0; k < nkeys; ++k)
            if (keys[k] == key) {
                found = (int)k;
                break;
            }
        if (found >= 0) {
            if (vals[found] == -1)
                kind[i] = 1;
            else if (vals[found] == -2)
                kind[i] = 2;
            else {
                kind[i] = 0;
                c->big_index[nne++] = (uint32_t)vals[found];
            }
            continue;
        }
        int status = GC_BRICK_UNKNOWN;
        const gc_layout *L = &c->d.layout;
        if (is_empty_key(c, key))
            status = GC_BRICK_EMPTY;
        else if (c->src && b[3] < L->nb_levels && gx < L->nb_big_bricks[b[3]][0] && gy < L->nb_big_bricks[b[3]][1] &&
                 gz < L->nb_big_bricks[b[3]][2]) {
            uint64_t idx = ((uint64_t)gz * L->nb_big_bricks[b[3]][1] + gy) * L->nb_big_bricks[b[3]][0] + gx;
            memcpy(c->staging + (uint64_t)nbig * c->big_bytes, c->src + c->level_off[b[3]] + idx * c->big_bytes,
                   c->big_bytes);
            status = GC_BRICK_SUCCESS;
        }
        keys[nkeys] = key;
        if (status == GC_BRICK_SUCCESS) {
            vals[nkeys++] = (int32_t)nbig;
            c->big_coord[4 * nbig + 0] = gx;
            c->big_coord[4 * nbig + 1] = gy;
            c->big_coord[4 * nbig + 2] = gz;
            c->big_coord[4 * nbig + 3] = b[3];
            c->big_index[nne++] = nbig++;
            kind[i] = 0;
        } else if (status == GC_BRICK_EMPTY) {
            vals[nkeys++] = -1;
            kind[i] = 1;
        } else {
            vals[nkeys++] = -2;
            kind[i] = 2;
        }
    }
    uint32_t k = 0;
    for (uint32_t i = 0; i < n; ++i)
        if (kind[i] == 0) memcpy(&c->asked[4 * k++], &c->list[4 * i], 16);
    for (uint32_t i = 0; i < n; ++i)
        if (kind[i] == 1) memcpy(&c->asked[4 * k++], &c->list[4 * i], 16);
    c->n_asked = k;
    c->n_nonempty = nne;
    free(keys);
    free(vals);
    free(kind);
}

static uint64_t mrpd_coord(const orc_cache *c, uint32_t l, float vx, float vy, float vz) {
    uint32_t x = c->off[l] + (uint32_t)(vx * (float)c->nb[l][0]);
    uint32_t y = (uint32_t)(vy * (float)c->nb[l][1]);
    uint32_t z = (uint32_t)(vz * (float)c->nb[l][2]);
    return (uint64_t)x + (uint64_t)y * c->mx + (uint64_t)z * c->mx * c->my;
}

/* load_new_bricks (CacheManager.hpp:502-632) */
static void load_new_bricks(orc_cache *c) {
    uint32_t n = c->n_asked, nne = c->n_nonempty;
    if (n == 0) return;
    if (nne > c->nslots) nne = c->nslots;
    orc_lru *tail = c->lru + (c->nslots - nne);
    /* dereference_old_bricks; with two levels only an entry that still names
     * the slot is cleared (after its block was evicted the brick may be
     * unreachable, or resident again in another slot) */
    for (uint32_t i = 0; i < nne; ++i) {
        if (tail[i].vx < 0.f) continue;
        if (c->pts) {
            const uint32_t l = tail[i].level;
            const uint32_t x = (uint32_t)(tail[i].vx * (float)c->nb[l][0]);
            const uint32_t y = (uint32_t)(tail[i].vy * (float)c->nb[l][1]);
            const uint32_t z = (uint32_t)(tail[i].vz * (float)c->nb[l][2]);
            if (x >= c->nb[l][0] || y >= c->nb[l][1] || z >= c->nb[l][2]) continue;
            uint32_t *e = entry_of(c, l, x, y, z, 0);
            if (e && e[3] == 1 && e[0] == tail[i].cx && e[1] == tail[i].cy && e[2] == tail[i].cz) memset(e, 0, 16);
            continue;
        }
        uint64_t e = mrpd_coord(c, tail[i].level, tail[i].vx, tail[i].vy, tail[i].vz);
        memset(&c->mrpd[4 * e], 0, 16);
    }
    /* compute_lru_volume_position */
    orc_lru *draft = (orc_lru *)calloc(n, sizeof(orc_lru));
    const float one_over = 1.f / (float)c->Beff;
    const float eps = 1.1920928955078125e-7f;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t *b = &c->asked[4 * i];
        draft[i].vx = (float)b[0] / ((float)c->vvox[b[3]][0] * one_over) + eps;
        draft[i].vy = (float)b[1] / ((float)c->vvox[b[3]][1] * one_over) + eps;
        draft[i].vz = (float)b[2] / ((float)c->vvox[b[3]][2] * one_over) + eps;
        draft[i].level = b[3];
    }
    /* copy_lru_position */
    for (uint32_t i = 0; i < nne; ++i) {
        tail[i].level = draft[i].level;
        tail[i].vx = draft[i].vx;
        tail[i].vy = draft[i].vy;
        tail[i].vz = draft[i].vz;
    }
    /* write_brick */
    const uint32_t B = c->B, E = c->eb, *BB = c->d.volume.big_brick_size;
    const uint32_t bvx = BB[0] * B, bvy = BB[1] * B;
    for (uint32_t i = 0; i < nne; ++i) {
        uint32_t *b = &c->asked[4 * i];
        uint32_t bi = c->big_index[i];
        uint32_t *bc = &c->big_coord[4 * bi];
        uint32_t ox = (b[0] - bc[0] * BB[0]) * B, oy = (b[1] - bc[1] * BB[1]) * B, oz = (b[2] - bc[2] * BB[2]) * B;
        const uint8_t *src = c->staging + (uint64_t)bi * c->big_bytes;
        uint8_t *dst = c->pool + (uint64_t)slot_of(c, tail[i].cx, tail[i].cy, tail[i].cz) * c->brick_bytes;
        for (uint32_t z = 0; z < B; ++z)
            for (uint32_t y = 0; y < B; ++y)
                memcpy(dst + ((uint64_t)(z * B + y) * B) * E,
                       src + (((uint64_t)(oz + z) * bvy + (oy + y)) * bvx + ox) * E, (uint64_t)B * E);
    }
    if (c->pts) {
        /* Two levels: table blocks for the new bricks.  The directory words
         * without a block named by the list, in order of their first element,
         * take the table slots at the LRU tail (the k-th of npt words the
         * slot at position pt_slots - npt + k); a slot leaves the block it
         * held (directory word cleared) and is cleared.  Words beyond the
         * table pool's size get none: their bricks stay unmapped. */
        uint64_t *words = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
        uint32_t *first = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
        uint32_t m = 0;
        for (uint32_t i = 0; i < n; ++i) {
            const uint32_t l = draft[i].level;
            const uint32_t x = (uint32_t)(draft[i].vx * (float)c->nb[l][0]);
            const uint32_t y = (uint32_t)(draft[i].vy * (float)c->nb[l][1]);
            const uint32_t z = (uint32_t)(draft[i].vz * (float)c->nb[l][2]);
            if (x >= c->nb[l][0] || y >= c->nb[l][1] || z >= c->nb[l][2]) continue;
            const uint64_t w = pt_word_of(c, l, x, y, z);
            if (c->pt_top[w] & 1u) continue;
            uint32_t k = 0;
            while (k < m && words[k] != w) ++k;
            if (k == m) {
                words[m] = w;
                first[m++] = i;
            }
        }
        const uint32_t npt = m < c->pt_slots ? m : c->pt_slots;
        const uint32_t P = 1u << c->pts, msk = ~(P - 1u);
        const uint64_t per = (uint64_t)1 << (3 * c->pts);
        for (uint32_t k = 0; k < npt; ++k) {
            const uint32_t slot = c->pt_order[c->pt_slots - npt + k];
            uint32_t *key = &c->pt_keys[4 * slot];
            if (key[3] != 0xffffffffu) c->pt_top[pt_word_of(c, key[3], key[0], key[1], key[2])] = 0;
            memset(&c->pt_table[4 * ((uint64_t)slot * per)], 0, per * 16);
            const orc_lru *d = &draft[first[k]];
            key[0] = (uint32_t)(d->vx * (float)c->nb[d->level][0]) & msk;
            key[1] = (uint32_t)(d->vy * (float)c->nb[d->level][1]) & msk;
            key[2] = (uint32_t)(d->vz * (float)c->nb[d->level][2]) & msk;
            key[3] = d->level;
            c->pt_top[words[k]] = slot << 1 | 1u;
        }
        free(words);
        free(first);
    }
    /* reference_new_bricks: non-empty then empty, serially */
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t l = draft[i].level;
        uint32_t *e;
        if (c->pts) {
            const uint32_t x = (uint32_t)(draft[i].vx * (float)c->nb[l][0]);
            const uint32_t y = (uint32_t)(draft[i].vy * (float)c->nb[l][1]);
            const uint32_t z = (uint32_t)(draft[i].vz * (float)c->nb[l][2]);
            if (x >= c->nb[l][0] || y >= c->nb[l][1] || z >= c->nb[l][2]) continue;
            e = entry_of(c, l, x, y, z, 0);
            if (!e) continue;
        } else {
            e = &c->mrpd[4 * mrpd_coord(c, l, draft[i].vx, draft[i].vy, draft[i].vz)];
        }
        if (e[3] >= 1) continue;
        if (i < nne) {
            e[0] = tail[i].cx;
            e[1] = tail[i].cy;
            e[2] = tail[i].cz;
            e[3] = 1;
        } else if (i >= c->n_nonempty) {
            e[0] = 0;
            e[1] = 0;
            e[2] = 0;
            e[3] = 2;
        }
    }
    free(draft);
}

int orc_cache_update(orc_cache *c) {
    orc_lru_update(c);
    int check = 0;
    if (c->request_done) {
        load_new_bricks(c);
        c->request_done = 0;
    } else {
        uint32_t total = orc_request_list(c, c->list, c->d.max_requests);
        uint32_t n = total < c->d.max_requests ? total : c->d.max_requests;
        if (n == 0)
            check = 1;
        else {
            handle_request(c, n);
            c->request_done = c->n_asked > 0;
        }
    }
    c->ts++;
    return check;
}

float orc_completude(const orc_cache *c) {
    uint32_t k = 0;
    for (uint32_t i = 0; i < c->nslots; ++i)
        if (c->lru[i].vx != -1.f) ++k;
    return (float)k / (float)c->nslots;
}

/* ------------------------------------------------------------------------ */
/* ray caster                                                                */

typedef struct {
    float x, y, z;
} f3;
static f3 mk(float x, float y, float z) {
    f3 r = {x, y, z};
    return r;
}
static f3 add3(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static f3 sub3(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static f3 muls(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static f3 mulv(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static float len3(f3 a) { return sqrtf(dot3(a, a)); }
static f3 norm3(f3 a) {
    float inv = 1.0f / sqrtf(dot3(a, a));
    return muls(a, inv);
}
static f3 cross3(f3 a, f3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static float clampf_(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
/* a * b + c fused per component: the fused multiply-adds of the CUDA ray
   caster (render.cu fmad/fma3) at the same places, so every rounding agrees. */
static f3 fma3o(f3 a, float b, f3 c) { return mk(fmaf(a.x, b, c.x), fmaf(a.y, b, c.y), fmaf(a.z, b, c.z)); }
static float sat(float x) { return (x != x) ? 0.0f : fminf(fmaxf(x, 0.0f), 1.0f); }

static uint32_t f2u(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
static float u2f(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}
static float o_log2(float x) {
    uint32_t bits = f2u(x);
    int e = (int)((bits >> 23) & 0xffu) - 126;
    float m = u2f((bits & 0x807fffffu) | (126u << 23));
    if (m < 0.70710678f) {
        m = m * 2.0f;
        e -= 1;
    }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = fmaf(s2, 0.11111111f, 0.14285715f);
    p = fmaf(p, s2, 0.2f);
    p = fmaf(p, s2, 0.33333334f);
    p = fmaf(p, s2, 1.0f);
    float ln = (2.0f * s) * p;
    return fmaf(ln, 1.44269504f, (float)e);
}
static float o_exp2(float y) {
    if (y < -125.0f) return 0.0f;
    float n = floorf(y + 0.5f);
    float t = (y - n) * 0.69314718f;
    float p = fmaf(t, 0.00019841270f, 0.0013888889f);
    p = fmaf(p, t, 0.0083333333f);
    p = fmaf(p, t, 0.041666668f);
    p = fmaf(p, t, 0.16666667f);
    p = fmaf(p, t, 0.5f);
    p = fmaf(p, t, 1.0f);
    p = fmaf(p, t, 1.0f);
    float scale = u2f((uint32_t)((int)n + 127) << 23);
    return p * scale;
}
float orc_pow(float x, float k) {
    if (!(x > 0.0f)) return 0.0f;
    if (x == 1.0f) return 1.0f;
    return o_exp2(k * o_log2(x));
}

typedef struct {
    float x, y, z, w;
} f4;
static f4 tf_lookup(const float *tf, uint32_t w, float s) {
    float xb = fmaf(s, (float)w, -0.5f);
    float fl = floorf(xb);
    float a = xb - fl;
    int i0 = (int)fl, i1 = i0 + 1, hi = (int)w - 1;
    i0 = i0 < 0 ? 0 : (i0 > hi ? hi : i0);
    i1 = i1 < 0 ? 0 : (i1 > hi ? hi : i1);
    const float *t0 = tf + 4 * i0, *t1 = tf + 4 * i1;
    f4 r = {fmaf(t1[0] - t0[0], a, t0[0]), fmaf(t1[1] - t0[1], a, t0[1]), fmaf(t1[2] - t0[2], a, t0[2]),
            fmaf(t1[3] - t0[3], a, t0[3])};
    return r;
}

/* 2D transfer function of two-channel volumes: bilinear over a w x h table,
   channel 0 along a row, channel 1 across rows (no counterpart in the
   reference, whose ray caster reads one channel; same rule as tf_lookup on
   each axis). */
static f4 tf2d_lookup(const float *tf, uint32_t w, uint32_t h, float s0, float s1) {
    float xb = fmaf(s0, (float)w, -0.5f), yb = fmaf(s1, (float)h, -0.5f);
    float flx = floorf(xb), fly = floorf(yb);
    float ax = xb - flx, ay = yb - fly;
    int hx = (int)w - 1, hy = (int)h - 1;
    int i0 = (int)flx, i1 = i0 + 1, j0 = (int)fly, j1 = j0 + 1;
    i0 = i0 < 0 ? 0 : (i0 > hx ? hx : i0);
    i1 = i1 < 0 ? 0 : (i1 > hx ? hx : i1);
    j0 = j0 < 0 ? 0 : (j0 > hy ? hy : j0);
    j1 = j1 < 0 ? 0 : (j1 > hy ? hy : j1);
    const float *t00 = tf + 4 * (j0 * (int)w + i0), *t10 = tf + 4 * (j0 * (int)w + i1);
    const float *t01 = tf + 4 * (j1 * (int)w + i0), *t11 = tf + 4 * (j1 * (int)w + i1);
    float r0[4], r1[4];
    for (int k = 0; k < 4; ++k) {
        r0[k] = fmaf(t10[k] - t00[k], ax, t00[k]);
        r1[k] = fmaf(t11[k] - t01[k], ax, t01[k]);
    }
    f4 r = {fmaf(r1[0] - r0[0], ay, r0[0]), fmaf(r1[1] - r0[1], ay, r0[1]), fmaf(r1[2] - r0[2], ay, r0[2]),
            fmaf(r1[3] - r0[3], ay, r0[3])};
    return r;
}

typedef struct {
    float inv_size[GC_MAX_LEVELS][3];
    float step[GC_MAX_LEVELS];
    float kexp[GC_MAX_LEVELS];
} lod_tables;

static void make_lod(const orc_cache *c, const gc_view *v, lod_tables *T) {
    float bsx = v->bbox_max[0] - v->bbox_min[0];
    float bsy = v->bbox_max[1] - v->bbox_min[1];
    float bsz = v->bbox_max[2] - v->bbox_min[2];
    float bmin = bsx < (bsy < bsz ? bsy : bsz) ? bsx : (bsy < bsz ? bsy : bsz);
    const gc_layout *L = &c->d.layout;
    for (uint32_t l = 0; l < L->nb_levels; ++l) {
        for (int a = 0; a < 3; ++a) T->inv_size[l][a] = bmin / (float)L->initial[l][a];
        uint32_t mn = L->initial[l][0];
        if (L->initial[l][1] < mn) mn = L->initial[l][1];
        if (L->initial[l][2] < mn) mn = L->initial[l][2];
        T->step[l] = (bmin / (float)mn) / 2.f;
        T->kexp[l] = T->step[l] / v->tstep;
    }
}

static float voxel_value(const orc_cache *c, const uint8_t *slot, uint32_t idx) {
    if (c->eb == 1) return (float)slot[idx];
    if (c->eb == 2) return (float)((const uint16_t *)slot)[idx];
    return ((const float *)slot)[idx];
}

static void tri_axis(float f, uint32_t cov, uint32_t beff, uint32_t B, uint32_t *i0, float *w) {
    uint32_t m = (uint32_t)f;
    float fr = f - (float)m;
    uint32_t l = cov + m % beff;
    if (fr >= 0.5f) {
        *i0 = l;
        *w = fr - 0.5f;
    } else {
        *i0 = l > 0 ? l - 1 : 0u;
        *w = l > 0 ? fr + 0.5f : 0.0f;
    }
    if (*i0 + 1 >= B) {
        *i0 = B - 2;
        *w = 1.0f;
    }
}

/* K_CacheManager::get_normalized + K_CacheDevice::get_normalized */
typedef struct {
    uint32_t pcx, pcy, pcz;
    uint32_t e[4];
} walk;

/* sample[0] (and sample[1] for two 8-bit channels, voxel i channel k at byte 2i+k);
 * request: stamp the request word of a missing brick */
static int fetch32_at(orc_cache *c, uint32_t sampler, uint32_t lod, f3 np, walk *w, float *sample, int request) {
    float px = np.x * c->ior[lod][0], py = np.y * c->ior[lod][1], pz = np.z * c->ior[lod][2];
    uint32_t cx = c->off[lod] + (uint32_t)(px * (float)c->nb[lod][0]);
    uint32_t cy = (uint32_t)(py * (float)c->nb[lod][1]);
    uint32_t cz = (uint32_t)(pz * (float)c->nb[lod][2]);
    uint64_t idx = (uint64_t)cx + (uint64_t)cy * c->mx + (uint64_t)cz * c->mx * c->my;
    if (cx != w->pcx || cy != w->pcy || cz != w->pcz) {
        const uint32_t *e = entry_of(c, lod, cx - c->off[lod], cy, cz, 1);
        if (e)
            memcpy(w->e, e, 16);
        else
            memset(w->e, 0, 16);
        w->pcx = cx;
        w->pcy = cy;
        w->pcz = cz;
    }
    if (w->e[3] == 1) {
        uint32_t B = c->B;
        uint32_t slot = slot_of(c, w->e[0], w->e[1], w->e[2]);
        __atomic_store_n(&c->usage[slot], c->ts, __ATOMIC_RELAXED);
        const uint8_t *sb = c->pool + (uint64_t)slot * c->brick_bytes;
        float fx = px * (float)c->vvox[lod][0], fy = py * (float)c->vvox[lod][1], fz = pz * (float)c->vvox[lod][2];
        if (c->d.volume.channels == 2) {
            uint32_t BB2 = B * B;
            if (sampler == GC_SAMPLER_REFERENCE) {
                uint32_t lx = c->c + (uint32_t)fx % c->Beff, ly = c->c + (uint32_t)fy % c->Beff,
                         lz = c->c + (uint32_t)fz % c->Beff;
                if (lx == 0) lx = 1;
                if (ly == 0) ly = 1;
                if (lz == 0) lz = 1;
                uint32_t i0 = ((lz - 1) * B + (ly - 1)) * B + (lx - 1);
                uint32_t ids[8] = {i0, i0 + 1, i0 + B, i0 + B + 1, i0 + BB2, i0 + BB2 + 1, i0 + BB2 + B, i0 + BB2 + B + 1};
                uint32_t s0 = 0, s1 = 0;
                for (int k = 0; k < 8; ++k) {
                    s0 += sb[2 * ids[k]];
                    s1 += sb[2 * ids[k] + 1];
                }
                sample[0] = (float)s0 / 2040.0f;
                sample[1] = (float)s1 / 2040.0f;
            } else {
                uint32_t x0, y0, z0;
                float wx, wy, wz;
                tri_axis(fx, c->c, c->Beff, B, &x0, &wx);
                tri_axis(fy, c->c, c->Beff, B, &y0, &wy);
                tri_axis(fz, c->c, c->Beff, B, &z0, &wz);
                uint32_t i = (z0 * B + y0) * B + x0;
                for (int k = 0; k < 2; ++k) {
#define LV2(j) ((float)sb[2 * (j) + k])
                    float c00 = fmaf(LV2(i + 1) - LV2(i), wx, LV2(i));
                    float c10 = fmaf(LV2(i + B + 1) - LV2(i + B), wx, LV2(i + B));
                    float c01 = fmaf(LV2(i + BB2 + 1) - LV2(i + BB2), wx, LV2(i + BB2));
                    float c11 = fmaf(LV2(i + BB2 + B + 1) - LV2(i + BB2 + B), wx, LV2(i + BB2 + B));
#undef LV2
                    float c0 = fmaf(c10 - c00, wy, c00), c1 = fmaf(c11 - c01, wy, c01);
                    sample[k] = fmaf(c1 - c0, wz, c0) / 255.0f;
                }
            }
            return 0;
        }
        if (sampler == GC_SAMPLER_REFERENCE) {
            uint32_t lx = c->c + (uint32_t)fx % c->Beff, ly = c->c + (uint32_t)fy % c->Beff,
                     lz = c->c + (uint32_t)fz % c->Beff;
            if (lx == 0) lx = 1;
            if (ly == 0) ly = 1;
            if (lz == 0) lz = 1;
            uint32_t i0 = ((lz - 1) * B + (ly - 1)) * B + (lx - 1), BB2 = B * B;
            if (c->eb < 4) {
                uint32_t s = 0;
                uint32_t ids[8] = {i0, i0 + 1, i0 + B, i0 + B + 1, i0 + BB2, i0 + BB2 + 1, i0 + BB2 + B, i0 + BB2 + B + 1};
                for (int k = 0; k < 8; ++k) s += (uint32_t)voxel_value(c, sb, ids[k]);
                *sample = (float)s / (c->eb == 1 ? 2040.0f : 524280.0f);
            } else {
                float s = ((voxel_value(c, sb, i0) + voxel_value(c, sb, i0 + 1)) +
                           (voxel_value(c, sb, i0 + B) + voxel_value(c, sb, i0 + B + 1))) +
                          ((voxel_value(c, sb, i0 + BB2) + voxel_value(c, sb, i0 + BB2 + 1)) +
                           (voxel_value(c, sb, i0 + BB2 + B) + voxel_value(c, sb, i0 + BB2 + B + 1)));
                *sample = s * 0.125f;
            }
        } else {
            uint32_t x0, y0, z0;
            float wx, wy, wz;
            tri_axis(fx, c->c, c->Beff, B, &x0, &wx);
            tri_axis(fy, c->c, c->Beff, B, &y0, &wy);
            tri_axis(fz, c->c, c->Beff, B, &z0, &wz);
            uint32_t i = (z0 * B + y0) * B + x0, BB2 = B * B;
#define LV(k) voxel_value(c, sb, (k))
            float c00 = fmaf(LV(i + 1) - LV(i), wx, LV(i));
            float c10 = fmaf(LV(i + B + 1) - LV(i + B), wx, LV(i + B));
            float c01 = fmaf(LV(i + BB2 + 1) - LV(i + BB2), wx, LV(i + BB2));
            float c11 = fmaf(LV(i + BB2 + B + 1) - LV(i + BB2 + B), wx, LV(i + BB2 + B));
#undef LV
            float c0 = fmaf(c10 - c00, wy, c00), c1 = fmaf(c11 - c01, wy, c01);
            float mx = c->eb == 1 ? 255.0f : (c->eb == 2 ? 65535.0f : 1.0f);
            *sample = fmaf(c1 - c0, wz, c0) / mx;
        }
        return 0;
    }
    if (w->e[3] == 0) {
        if (request) __atomic_store_n(&c->req[idx], c->ts, __ATOMIC_RELAXED);
        return 1;
    }
    return 2;
}

/* 0 mapped, 1 unmapped (requested), 2 empty, 4 a coarser level sampled.
 * fallback: the preview mode of K_CacheManager::get (K_CacheManager.hpp:163-260):
 * the missing brick is requested on the asked level only, then the levels
 * above it are read in order: the first mapped one is sampled (its usage
 * stamped), an empty one ends the lookup, an unmapped one is passed over. */
static int fetch32(orc_cache *c, uint32_t sampler, uint32_t lod, f3 np, walk *w, float *sample, int fallback) {
    int st = fetch32_at(c, sampler, lod, np, w, sample, 1);
    if (st != 1 || !fallback) return st;
    for (uint32_t l2 = lod + 1; l2 < c->nl; ++l2) {
        walk w2;
        w2.pcx = w2.pcy = w2.pcz = 0xffffffffu;
        int s2 = fetch32_at(c, sampler, l2, np, &w2, sample, 0);
        if (s2 == 2) return 2;
        if (s2 == 0) return 4;
    }
    return 1;
}

/* One sample of K_CacheManager::get_normalized with a fresh page walk (the
 * device-side handle's gc_sample_normalized): 0 mapped (*out written), 1
 * unmapped (requested), 2 empty. */
int orc_sample_normalized(orc_cache *c, uint32_t level, float x, float y, float z, float *out) {
    walk w;
    w.pcx = w.pcy = w.pcz = UINT32_MAX;
    return fetch32(c, GC_SAMPLER_REFERENCE, level, mk(x, y, z), &w, out, 0);
}

static void march32(orc_cache *c, const gc_view *v, const float *tf, const lod_tables *T, uint32_t x, uint32_t y,
                    uint32_t *rgba, float *tbuf, float *state) {
    uint32_t W = v->width, H = v->height;
    uint32_t xN = x + 1;
    if (xN > W) xN = x - 1;
    uint32_t yN = y + 1;
    if (yN > H) yN = y - 1;
    float fW = (float)W, fH = (float)H;
    float u = (((float)x + 0.5f) / fW) * 2.0f - 1.0f;
    float uN = (((float)xN + 0.5f) / fW) * 2.0f - 1.0f;
    float vv = (((float)y + 0.5f) / fH) * 2.0f - 1.0f;
    float vN = (((float)yN + 0.5f) / fH) * 2.0f - 1.0f;
    const float *m = v->inv_view;
    f3 origin = mk(0.0f * m[0] + 0.0f * m[1] + 0.0f * m[2] + 1.0f * m[3], 0.0f * m[4] + 0.0f * m[5] + 0.0f * m[6] + 1.0f * m[7],
                   0.0f * m[8] + 0.0f * m[9] + 0.0f * m[10] + 1.0f * m[11]);
    f3 r0 = mk(m[0], m[1], m[2]), r1 = mk(m[4], m[5], m[6]), r2 = mk(m[8], m[9], m[10]);
    f3 d0 = norm3(mk(u, vv, -v->focal)), dx = norm3(mk(uN, vv, -v->focal)), dy = norm3(mk(u, vN, -v->focal));
    f3 dir = mk(dot3(d0, r0), dot3(d0, r1), dot3(d0, r2));
    f3 dirXN = mk(dot3(dx, r0), dot3(dx, r1), dot3(dx, r2));
    f3 dirYN = mk(dot3(dy, r0), dot3(dy, r1), dot3(dy, r2));
    f3 dirLeft = norm3(cross3(dir, dirYN));
    f3 dirUp = norm3(cross3(dir, dirXN));
    f3 invR = mk(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    f3 tbot = mulv(invR, sub3(mk(v->bbox_min[0], v->bbox_min[1], v->bbox_min[2]), origin));
    f3 ttop = mulv(invR, sub3(mk(v->bbox_max[0], v->bbox_max[1], v->bbox_max[2]), origin));
    f3 tmin = mk(fminf(ttop.x, tbot.x), fminf(ttop.y, tbot.y), fminf(ttop.z, tbot.z));
    f3 tmax = mk(fmaxf(ttop.x, tbot.x), fmaxf(ttop.y, tbot.y), fmaxf(ttop.z, tbot.z));
    float tnear = fmaxf(fmaxf(tmin.x, tmin.y), fmaxf(tmin.x, tmin.z));
    float tfar = fminf(fminf(tmax.x, tmax.y), fminf(tmax.x, tmax.z));
    int hit = tfar > tnear;
    uint32_t i = y * W + x;
    tnear = fmaxf(tnear, tbuf[i]);
    int dvr = v->mode == GC_MODE_DVR;
    f4 fc = {0, 0, 0, 0};
    if (dvr) {
        fc.x = state[4 * i];
        fc.y = state[4 * i + 1];
        fc.z = state[4 * i + 2];
        fc.w = state[4 * i + 3];
    }
    if (!hit) {
        fc.x = fc.y = fc.z = 0.f;
    } else {
        if (tnear < 0.f) tnear = 0.f;
        float t = tnear;
        f3 pos = add3(origin, muls(dir, tnear));
        float endX = fabsf(dot3(sub3(dir, dirXN), dirLeft) * tfar);
        float endY = fabsf(dot3(sub3(dir, dirYN), dirUp) * tfar);
        walk w;
        w.pcx = w.pcy = w.pcz = 0xffffffffu;
        memset(w.e, 0, sizeof(w.e));
        int unm = 0;
        float maxOp = dvr ? 0.f : state[4 * i];
        uint32_t nl = c->nl;
        int two = c->d.volume.channels == 2;
        while ((!dvr || fc.w < v->early_alpha) && t < tfar) {
            float alpha = t / tfar;
            float pX = endX * alpha, pY = endY * alpha;
            f3 tp = mk(fmaf(pos.x, 0.495f, 0.495f), fmaf(pos.y, 0.495f, 0.495f), fmaf(pos.z, 0.495f, 0.495f));
            tp.z = 1.0f - tp.z;
            f3 np = mk(clampf_(tp.x, 0.f, 0.99f), clampf_(tp.y, 0.f, 0.99f), clampf_(tp.z, 0.f, 0.99f));
            /* compute_LOD, full scan */
            uint32_t lod;
            for (lod = 0; lod + 1 < nl; ++lod) {
                f3 ns = mk(T->inv_size[lod + 1][0], T->inv_size[lod + 1][1], T->inv_size[lod + 1][2]);
                float sl = len3(mulv(dirLeft, ns)), su = len3(mulv(dirUp, ns));
                if (sl >= pX * 1.0f || su >= pY * 1.0f) break;
            }
            float smp[2] = {0.f, 0.f};
            int st = fetch32(c, v->sampler, lod, np, &w, smp, v->fallback != 0);
            float sample = smp[0];
            if (st != 0 && st != 4) {
                if (st == 1) {
                    if (!unm) {
                        tbuf[i] = t;
                        if (dvr) {
                            state[4 * i] = fc.x;
                            state[4 * i + 1] = fc.y;
                            state[4 * i + 2] = fc.z;
                            state[4 * i + 3] = fc.w;
                        } else
                            state[4 * i] = maxOp;
                    }
                    unm = 1;
                    break;
                }
                t += v->tstep;
                if (t > tfar) break;
                pos = fma3o(dir, v->tstep, pos);
                continue;
            }
            if (dvr) {
                f4 col = two ? tf2d_lookup(tf, v->tf_width, v->tf_height, smp[0], smp[1])
                             : tf_lookup(tf, v->tf_width, sample);
                col.w = 1.0f - orc_pow(1.0f - col.w, T->kexp[lod]);
                if (col.w > 0.001f) {
                    col.x *= col.w;
                    col.y *= col.w;
                    col.z *= col.w;
                    float r = 1.0f - fc.w;
                    fc.x = fmaf(col.x, r, fc.x);
                    fc.y = fmaf(col.y, r, fc.y);
                    fc.z = fmaf(col.z, r, fc.z);
                    fc.w = fmaf(col.w, r, fc.w);
                }
            } else {
                maxOp = fmaxf(maxOp, sample);
            }
            t += T->step[lod];
            pos = fma3o(dir, T->step[lod], pos);
        }
        if (!unm) {
            tbuf[i] = t;
            if (dvr) {
                state[4 * i] = fc.x;
                state[4 * i + 1] = fc.y;
                state[4 * i + 2] = fc.z;
                state[4 * i + 3] = fc.w;
            } else
                state[4 * i] = maxOp;
        }
        if (!dvr) fc = tf_lookup(tf, v->tf_width, maxOp);
    }
    uint32_t R = (uint32_t)(sat(fc.x) * 255.0f), G = (uint32_t)(sat(fc.y) * 255.0f), Bc = (uint32_t)(sat(fc.z) * 255.0f),
             A = (uint32_t)(sat(fc.w) * 255.0f);
    rgba[i] = (A << 24) | (Bc << 16) | (G << 8) | R;
}

void orc_render(orc_cache *c, const gc_view *v, const float *tf, uint32_t *rgba, float *tbuf, float *state,
                int threads) {
    lod_tables T;
    make_lod(c, v, &T);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int64_t y = 0; y < (int64_t)v->height; ++y)
        for (uint32_t x = 0; x < v->width; ++x) march32(c, v, tf, &T, x, (uint32_t)y, rgba, tbuf, state);
    (void)threads;
}

/* ------------------------------------------------------------------------ */
/* double-precision restatement                                              */
typedef struct {
    double x, y, z;
} d3;
static d3 dmk(double x, double y, double z) {
    d3 r = {x, y, z};
    return r;
}
static d3 dadd(d3 a, d3 b) { return dmk(a.x + b.x, a.y + b.y, a.z + b.z); }
static d3 dsub(d3 a, d3 b) { return dmk(a.x - b.x, a.y - b.y, a.z - b.z); }
static d3 dmuls(d3 a, double s) { return dmk(a.x * s, a.y * s, a.z * s); }
static d3 dmulv(d3 a, d3 b) { return dmk(a.x * b.x, a.y * b.y, a.z * b.z); }
static double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static double dlen(d3 a) { return sqrt(ddot(a, a)); }
static d3 dnorm(d3 a) { return dmuls(a, 1.0 / sqrt(ddot(a, a))); }
static d3 dcross(d3 a, d3 b) { return dmk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static double dclamp(double f, double a, double b) { return fmax(a, fmin(f, b)); }
static double dsat(double x) { return (x != x) ? 0.0 : fmin(fmax(x, 0.0), 1.0); }

static void march64(orc_cache *c, const gc_view *v, const float *tf, uint32_t x, uint32_t y, uint32_t *rgba,
                    double *tbuf, double *state, uint32_t *usage, uint32_t *req) {
    const gc_layout *L = &c->d.layout;
    double bmin = fmin(v->bbox_max[0] - (double)v->bbox_min[0],
                       fmin(v->bbox_max[1] - (double)v->bbox_min[1], v->bbox_max[2] - (double)v->bbox_min[2]));
    uint32_t W = v->width, H = v->height;
    uint32_t xN = x + 1 > W ? x - 1 : x + 1, yN = y + 1 > H ? y - 1 : y + 1;
    double u = ((x + 0.5) / W) * 2.0 - 1.0, uN = ((xN + 0.5) / W) * 2.0 - 1.0;
    double vv = ((y + 0.5) / H) * 2.0 - 1.0, vN = ((yN + 0.5) / H) * 2.0 - 1.0;
    const float *m = v->inv_view;
    d3 origin = dmk(m[3], m[7], m[11]);
    d3 r0 = dmk(m[0], m[1], m[2]), r1 = dmk(m[4], m[5], m[6]), r2 = dmk(m[8], m[9], m[10]);
    d3 a0 = dnorm(dmk(u, vv, -(double)v->focal)), ax = dnorm(dmk(uN, vv, -(double)v->focal)),
       ay = dnorm(dmk(u, vN, -(double)v->focal));
    d3 dir = dmk(ddot(a0, r0), ddot(a0, r1), ddot(a0, r2));
    d3 dirXN = dmk(ddot(ax, r0), ddot(ax, r1), ddot(ax, r2));
    d3 dirYN = dmk(ddot(ay, r0), ddot(ay, r1), ddot(ay, r2));
    d3 dirLeft = dnorm(dcross(dir, dirYN)), dirUp = dnorm(dcross(dir, dirXN));
    d3 invR = dmk(1.0 / dir.x, 1.0 / dir.y, 1.0 / dir.z);
    d3 tbot = dmulv(invR, dsub(dmk(v->bbox_min[0], v->bbox_min[1], v->bbox_min[2]), origin));
    d3 ttop = dmulv(invR, dsub(dmk(v->bbox_max[0], v->bbox_max[1], v->bbox_max[2]), origin));
    double tnear = fmax(fmax(fmin(ttop.x, tbot.x), fmin(ttop.y, tbot.y)), fmax(fmin(ttop.x, tbot.x), fmin(ttop.z, tbot.z)));
    double tfar = fmin(fmin(fmax(ttop.x, tbot.x), fmax(ttop.y, tbot.y)), fmin(fmax(ttop.x, tbot.x), fmax(ttop.z, tbot.z)));
    int hit = tfar > tnear;
    uint32_t i = y * W + x;
    tnear = fmax(tnear, tbuf[i]);
    int dvr = v->mode == GC_MODE_DVR;
    double fc[4] = {0, 0, 0, 0};
    if (dvr)
        for (int k = 0; k < 4; ++k) fc[k] = state[4 * i + k];
    if (!hit) {
        fc[0] = fc[1] = fc[2] = 0.0;
    } else {
        if (tnear < 0.0) tnear = 0.0;
        double t = tnear;
        d3 pos = dadd(origin, dmuls(dir, tnear));
        double endX = fabs(ddot(dsub(dir, dirXN), dirLeft) * tfar), endY = fabs(ddot(dsub(dir, dirYN), dirUp) * tfar);
        int unm = 0;
        double maxOp = dvr ? 0.0 : state[4 * i];
        const double tstep = v->tstep;
        while ((!dvr || fc[3] < v->early_alpha) && t < tfar) {
            double alpha = t / tfar, pX = endX * alpha, pY = endY * alpha;
            d3 tp = dadd(dmuls(pos, 0.495), dmk(0.495, 0.495, 0.495));
            tp.z = 1.0 - tp.z;
            d3 np = dmk(dclamp(tp.x, 0, 0.99), dclamp(tp.y, 0, 0.99), dclamp(tp.z, 0, 0.99));
            uint32_t lod;
            for (lod = 0; lod + 1 < c->nl; ++lod) {
                d3 ns = dmk(bmin / L->initial[lod + 1][0], bmin / L->initial[lod + 1][1], bmin / L->initial[lod + 1][2]);
                if (dlen(dmulv(dirLeft, ns)) >= pX || dlen(dmulv(dirUp, ns)) >= pY) break;
            }
            uint32_t mn = L->initial[lod][0];
            if (L->initial[lod][1] < mn) mn = L->initial[lod][1];
            if (L->initial[lod][2] < mn) mn = L->initial[lod][2];
            double lstep = (bmin / mn) / 2.0;
            double px = np.x * ((double)L->initial[lod][0] / L->real[lod][0]);
            double py = np.y * ((double)L->initial[lod][1] / L->real[lod][1]);
            double pz = np.z * ((double)L->initial[lod][2] / L->real[lod][2]);
            uint32_t cx = c->off[lod] + (uint32_t)(px * c->nb[lod][0]), cy = (uint32_t)(py * c->nb[lod][1]),
                     cz = (uint32_t)(pz * c->nb[lod][2]);
            uint64_t idx = (uint64_t)cx + (uint64_t)cy * c->mx + (uint64_t)cz * c->mx * c->my;
            static const uint32_t no_entry[4] = {0, 0, 0, 0};
            const uint32_t *e = entry_of(c, lod, cx - c->off[lod], cy, cz, 0);
            if (!e) e = no_entry;
            double sample = 0.0;
            if (e[3] == 0) {
                __atomic_store_n(&req[idx], c->ts, __ATOMIC_RELAXED);
                if (!unm) {
                    tbuf[i] = t;
                    if (dvr)
                        for (int k = 0; k < 4; ++k) state[4 * i + k] = fc[k];
                    else
                        state[4 * i] = maxOp;
                }
                unm = 1;
                break;
            }
            if (e[3] == 2) {
                t += tstep;
                if (t > tfar) break;
                pos = dadd(pos, dmuls(dir, tstep));
                continue;
            }
            {
                uint32_t slot = slot_of(c, e[0], e[1], e[2]);
                __atomic_store_n(&usage[slot], c->ts, __ATOMIC_RELAXED);
                const uint8_t *sb = c->pool + (uint64_t)slot * c->brick_bytes;
                double fx = px * c->vvox[lod][0], fy = py * c->vvox[lod][1], fz = pz * c->vvox[lod][2];
                double mxv = c->eb == 1 ? 255.0 : (c->eb == 2 ? 65535.0 : 1.0);
                uint32_t B = c->B;
                if (v->sampler == GC_SAMPLER_REFERENCE) {
                    uint32_t lx = c->c + (uint32_t)fx % c->Beff, ly = c->c + (uint32_t)fy % c->Beff,
                             lz = c->c + (uint32_t)fz % c->Beff;
                    if (lx == 0) lx = 1;
                    if (ly == 0) ly = 1;
                    if (lz == 0) lz = 1;
                    double s = 0;
                    for (int dz = 0; dz < 2; ++dz)
                        for (int dyy = 0; dyy < 2; ++dyy)
                            for (int dxx = 0; dxx < 2; ++dxx)
                                s += voxel_value(c, sb, ((lz - 1 + dz) * B + (ly - 1 + dyy)) * B + (lx - 1 + dxx));
                    sample = s / (8.0 * mxv);
                } else {
                    double f[3] = {fx, fy, fz}, wt[3];
                    uint32_t i0[3];
                    for (int a = 0; a < 3; ++a) {
                        uint32_t mm = (uint32_t)f[a];
                        double fr = f[a] - mm;
                        uint32_t l = c->c + mm % c->Beff;
                        if (fr >= 0.5) {
                            i0[a] = l;
                            wt[a] = fr - 0.5;
                        } else {
                            i0[a] = l > 0 ? l - 1 : 0u;
                            wt[a] = l > 0 ? fr + 0.5 : 0.0;
                        }
                        if (i0[a] + 1 >= B) {
                            i0[a] = B - 2;
                            wt[a] = 1.0;
                        }
                    }
                    double s = 0;
                    for (int dz = 0; dz < 2; ++dz)
                        for (int dyy = 0; dyy < 2; ++dyy)
                            for (int dxx = 0; dxx < 2; ++dxx) {
                                double wgt = (dxx ? wt[0] : 1 - wt[0]) * (dyy ? wt[1] : 1 - wt[1]) * (dz ? wt[2] : 1 - wt[2]);
                                s += wgt * voxel_value(c, sb, ((i0[2] + dz) * B + (i0[1] + dyy)) * B + (i0[0] + dxx));
                            }
                    sample = s / mxv;
                }
            }
            if (dvr) {
                double xb = sample * v->tf_width - 0.5, fl = floor(xb), a = xb - fl;
                int j0 = (int)fl, j1 = j0 + 1, hi = (int)v->tf_width - 1;
                j0 = j0 < 0 ? 0 : (j0 > hi ? hi : j0);
                j1 = j1 < 0 ? 0 : (j1 > hi ? hi : j1);
                double col[4];
                for (int k = 0; k < 4; ++k) col[k] = tf[4 * j0 + k] + (tf[4 * j1 + k] - (double)tf[4 * j0 + k]) * a;
                col[3] = 1.0 - pow(1.0 - col[3], lstep / tstep);
                if (col[3] > 0.001) {
                    double r = 1.0 - fc[3];
                    for (int k = 0; k < 3; ++k) fc[k] += col[k] * col[3] * r;
                    fc[3] += col[3] * r;
                }
            } else {
                maxOp = fmax(maxOp, sample);
            }
            t += lstep;
            pos = dadd(pos, dmuls(dir, lstep));
        }
        if (!unm) {
            tbuf[i] = t;
            if (dvr)
                for (int k = 0; k < 4; ++k) state[4 * i + k] = fc[k];
            else
                state[4 * i] = maxOp;
        }
        if (!dvr) {
            double xb = maxOp * v->tf_width - 0.5, fl = floor(xb), a = xb - fl;
            int j0 = (int)fl, j1 = j0 + 1, hi = (int)v->tf_width - 1;
            j0 = j0 < 0 ? 0 : (j0 > hi ? hi : j0);
            j1 = j1 < 0 ? 0 : (j1 > hi ? hi : j1);
            for (int k = 0; k < 4; ++k) fc[k] = tf[4 * j0 + k] + (tf[4 * j1 + k] - (double)tf[4 * j0 + k]) * a;
        }
    }
    uint32_t R = (uint32_t)(dsat(fc[0]) * 255.0), G = (uint32_t)(dsat(fc[1]) * 255.0), Bc = (uint32_t)(dsat(fc[2]) * 255.0),
             A = (uint32_t)(dsat(fc[3]) * 255.0);
    rgba[i] = (A << 24) | (Bc << 16) | (G << 8) | R;
}

void orc_render_f64(orc_cache *c, const gc_view *v, const float *tf, uint32_t *rgba, double *tbuf, double *state,
                    uint32_t *usage, uint32_t *req, int threads) {
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int64_t y = 0; y < (int64_t)v->height; ++y)
        for (uint32_t x = 0; x < v->width; ++x) march64(c, v, tf, x, (uint32_t)y, rgba, tbuf, state, usage, req);
    (void)threads;
}
