/*
 * gc_cache_device.cuh -- device-side sampling of the brick cache from a host
 * application's own CUDA kernels.
 *
 * The reference lets any user kernel read the out-of-core volume through the
 * kernel object of its cache, K_CacheManager<T>::get_normalized
 * (GcCore/include/GcCore/cuda/libGPUCache/K_CacheManager.hpp:61-71, 265-361):
 * page-directory walk, usage stamp of the brick's pool slot, a request for a
 * missing brick, and the normalized texture read at the integer voxel corner
 * (K_CacheDevice.hpp:188-201, 314-336).  Here the kernel object is the plain
 * struct gc_cache_device_view (include/gc_gb300.h), filled on the host by
 * gc_cache_device_view_get() and passed by value; gc_sample_normalized() is
 * the sampling function.  It computes what the library's own ray caster reads
 * for a sample (same expressions, no fused multiply-add site, exactly rounded
 * division: keep the default -prec-div=true, i.e. no --use_fast_math, for
 * bit-identical values).
 *
 *   __global__ void my_kernel(const __grid_constant__ gc_cache_device_view v, ...) {
 *       float value;
 *       int st = gc_sample_normalized(&v, level, x, y, z, &value);   // x, y, z in [0, 1)
 *       if (st == GC_VOXEL_MAPPED) ... use value in [0, 1] ...
 *   }
 *
 * (__grid_constant__ lets the kernel use the parameter's address without a
 * per-thread copy of the struct.)
 *
 * A sample of a missing brick requests it: the next gc_cache_update lists it
 * and a later update installs it, as for the ray caster's own samples.
 */
#ifndef GC_CACHE_DEVICE_CUH
#define GC_CACHE_DEVICE_CUH

#include <stdint.h>

#include "gc_gb300.h"

/* VoxelStatus (K_CacheManager.hpp:24-29) */
#define GC_VOXEL_MAPPED 0
#define GC_VOXEL_UNMAPPED 1
#define GC_VOXEL_EMPTY 2

#ifdef __CUDACC__

/* Value of voxel (x, y, z) in normalized volume coordinates [0, 1) of level
 * `level` of the view's volume, normalized to [0, 1] (v / 255 for u8,
 * v / 65535 for u16): the mean of the 2 x 2 x 2 voxels below the integer
 * corner of the brick element, as the reference's linear texture read at that
 * corner.  Returns GC_VOXEL_MAPPED (out written, the slot's usage word stamped
 * with the view's timestamp), GC_VOXEL_UNMAPPED (the brick is not resident:
 * its request word is stamped unless its load is already under way) or
 * GC_VOXEL_EMPTY (an empty brick: nothing to sample). */
__device__ __forceinline__ int gc_sample_normalized(const gc_cache_device_view *v, uint32_t level, float x, float y,
                                                    float z, float *out) {
    const float px = x * v->level_initial_over_real[level][0];
    const float py = y * v->level_initial_over_real[level][1];
    const float pz = z * v->level_initial_over_real[level][2];
    const uint32_t cx = v->level_offset[level] + (uint32_t)(px * (float)v->level_bricks[level][0]);
    const uint32_t cy = (uint32_t)(py * (float)v->level_bricks[level][1]);
    const uint32_t cz = (uint32_t)(pz * (float)v->level_bricks[level][2]);
    const uint64_t idx = (uint64_t)cx + (uint64_t)cy * v->mrpd_dims[0] +
                         (uint64_t)cz * v->mrpd_dims[0] * v->mrpd_dims[1];
    uint4 e = make_uint4(0u, 0u, 0u, 0u);
    if (v->pt_shift) {
        /* two-level directory: the directory word of the brick's block, then
         * the entry in the block (the table slot's usage word stamped); a
         * word without a block reads as an unmapped entry */
        const uint32_t s = v->pt_shift, m = (1u << s) - 1u, bx = cx - v->level_offset[level];
        const uint32_t word = v->pt_level_offset[level] + (bx >> s) + (cy >> s) * v->pt_dims[0] +
                              (cz >> s) * v->pt_dims[0] * v->pt_dims[1];
        const uint32_t t = v->pt_top[word];
        if (t & 1u) {
            v->pt_usage[t >> 1] = v->timestamp;
            const uint64_t j = ((uint64_t)(t >> 1) << (3u * s)) + ((bx & m) | ((cy & m) << s) | ((cz & m) << (2u * s)));
            e = *reinterpret_cast<const uint4 *>(v->pt_pool + 4 * j);
        }
    } else {
        e = *reinterpret_cast<const uint4 *>(v->mrpd + 4 * idx);
    }
    if (e.w == 1u) {
        const uint32_t B = v->brick_size, c = v->covering, beff = B - 2u * c;
        const uint32_t slot = e.x / B + (e.y / B) * v->pool_slots[0] + (e.z / B) * v->pool_slots[0] * v->pool_slots[1];
        v->usage[slot] = v->timestamp;
        const float fx = px * (float)v->level_voxels[level][0];
        const float fy = py * (float)v->level_voxels[level][1];
        const float fz = pz * (float)v->level_voxels[level][2];
        uint32_t lx = c + (uint32_t)fx % beff, ly = c + (uint32_t)fy % beff, lz = c + (uint32_t)fz % beff;
        lx = lx > 0u ? lx : 1u;  /* covering 0: the lower voxel clamps to the brick edge */
        ly = ly > 0u ? ly : 1u;
        lz = lz > 0u ? lz : 1u;
        const uint32_t i0 = ((lz - 1u) * B + (ly - 1u)) * B + (lx - 1u), BB = B * B;
        const uint32_t id[8] = {i0, i0 + 1u, i0 + B, i0 + B + 1u, i0 + BB, i0 + BB + 1u, i0 + BB + B, i0 + BB + B + 1u};
        const uint8_t *slot_base = v->pool + (uint64_t)slot * v->slot_bytes;
        if (v->voxel_bytes == 4u) {
            const float *b = reinterpret_cast<const float *>(slot_base);
            const float s = ((b[id[0]] + b[id[1]]) + (b[id[2]] + b[id[3]])) + ((b[id[4]] + b[id[5]]) + (b[id[6]] + b[id[7]]));
            *out = s * 0.125f;
        } else {
            uint32_t s = 0;
            if (v->voxel_bytes == 1u) {
#pragma unroll
                for (int k = 0; k < 8; ++k) s += slot_base[id[k]];
                *out = (float)s / 2040.0f;
            } else {
                const uint16_t *b = reinterpret_cast<const uint16_t *>(slot_base);
#pragma unroll
                for (int k = 0; k < 8; ++k) s += b[id[k]];
                *out = (float)s / 524280.0f;
            }
        }
        return GC_VOXEL_MAPPED;
    }
    if (e.w == 0u) {
        v->requests[idx] = v->timestamp;  /* raise_brick_request (K_CacheManager.hpp:364-396) */
        return GC_VOXEL_UNMAPPED;
    }
    if (e.w == 3u) return GC_VOXEL_UNMAPPED;  /* in flight (the batched form): already requested */
    return GC_VOXEL_EMPTY;
}

#endif /* __CUDACC__ */
#endif /* GC_CACHE_DEVICE_CUH */
