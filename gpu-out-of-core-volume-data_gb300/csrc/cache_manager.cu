// Host side of the brick cache: the per-frame state machine of
// CacheManager<T>::update (GcCore/include/GcCore/cuda/libGPUCache/CacheManager.hpp:318-354),
// the request handler (RequestHandler.hpp:157-372) and the brick sources
// (BricksManager::get_brick, GcCore/src/libData/BricksManager.cpp:48-78).
//
// Frame protocol (timestamp ts, starting at 1):
//   render(ts)                 rays stamp usage[slot] = ts and req[brick] = ts
//   update():
//     LRU update               used slots first, stable        (always)
//     loader busy              -> ts++, return false           (async mode only)
//     a load finished          -> install it, return false
//     otherwise                -> scan requests; none -> return true,
//                                 else hand up to max_requests misses to the
//                                 loader, return false
//     ts++
// With GC_CACHE_SYNC_LOADER the loader finishes inside update(), which gives
// the reference's request -> install alternation deterministically.  Without
// it a loader thread resolves bricks while later frames render, as the
// reference's RequestHandler thread does.  Either way the bricks go up on a
// side stream and the install waits on that upload's event: a gather kernel
// reading the host store directly where the device can (page-locked store, or
// pageable memory on a coherent Grace-Blackwell link), else host copies into
// a pinned staging buffer and one cudaMemcpyAsync.
#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "brickfiles.h"
#include "cache.cuh"
#include "gc_internal.h"

namespace gc {

struct LruRecord {  // LruContent (LruContent.hpp:10-15)
    uint32_t cx, cy, cz, level;
    float vx, vy, vz;
};
static_assert(sizeof(LruRecord) == 28, "LruContent is 28 bytes");

template <class T>
static T *dalloc(size_t count, const char *what) {
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(count * sizeof(T), 16));
    if (e != cudaSuccess) fail(GC_ERR_NOMEM, std::string("cudaMalloc failed for ") + what + ": " + cudaGetErrorString(e));
    return static_cast<T *>(p);
}
template <class T>
static T *halloc(size_t count) {
    void *p = nullptr;
    GC_CUDA(cudaHostAlloc(&p, std::max<size_t>(count * sizeof(T), 16), cudaHostAllocDefault));
    return static_cast<T *>(p);
}

__global__ void init_slots_kernel(uint32_t *order, uint32_t *level, float4 *vpos, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        order[i] = i;
        level[i] = 0;
        vpos[i] = make_float4(-1.f, -1.f, -1.f, 0.f);
    }
}

struct Source {
    int kind = 0;  // 0 none, 1 host store, 2 callback, 3 brick files, 5 device-resident pyramid
    std::string dir;       // brick files: the volume directory (with '/')
    uint32_t threads = 0;  // brick files: reader threads
    const uint8_t *host = nullptr;
    uint64_t bytes = 0;
    bool direct = false;          // the device reads the store (gather kernel)
    bool vec16 = false;           // store, offsets and big-brick bytes 16-byte aligned
    const uint8_t *dev = nullptr;  // device-usable address of the store
    std::vector<uint64_t> level_off;
    gc_brick_loader_fn fn = nullptr;
    void *user = nullptr;
    std::unordered_set<uint64_t> empty;
};

// One volume of the cache: its levels are cache levels
// [level_base, level_base + layout.nb_levels).
struct Volume {
    gc_volume_desc desc;
    gc_layout layout;
    uint32_t level_base = 0;
    uint64_t brick_bytes = 0, big_bytes = 0;
    Source src;
    std::vector<uint64_t> bins;  // value bins of every brick (all levels), empty: none given
};

}  // namespace gc

// The loader's per-cycle scratch, kept between cycles: the list element kinds,
// the big-brick index of each non-empty element, and an open-addressing
// table from big-brick key to its staging slot (-1 empty, -2 unknown) that
// folds the elements of one big brick into one load.
struct ResolveScratch {
    std::vector<int> kind;
    std::vector<uint32_t> big_index;
    std::vector<uint64_t> keys;  // kNoKey marks a free table cell
    std::vector<int32_t> vals;
    static constexpr uint64_t kNoKey = ~0ull;
    // the cell of `key` (found or free) in a power-of-two table
    size_t cell(uint64_t key) const {
        const size_t mask = keys.size() - 1;
        size_t h = static_cast<size_t>((key * 0x9E3779B97F4A7C15ull) >> 32) & mask;
        while (keys[h] != kNoKey && keys[h] != key) h = (h + 1) & mask;
        return h;
    }
};

struct gc_cache {
    gc_cache_desc d;                  // d.volume / d.layout: volume 0
    std::vector<gc::Volume> vols;
    std::vector<uint32_t> level_volume;  // volume of each cache level
    gc::LevelTables lt;
    uint32_t mx = 0, my = 0, mz = 0, nslots = 0, B = 0, c = 0, Beff = 0;
    uint32_t beff_magic = 0;          // ceil(2^32 / Beff) for 2 <= Beff <= 128
    uint32_t eb = 0;                  // voxel bytes of every volume, 0 when they differ
    uint32_t nc = 1;                  // channels per voxel (the same for every volume)
    uint64_t nentries = 0;
    uint64_t slot_bytes = 0;          // pool slot: B^3 x the widest voxel
    uint64_t big_stride = 0;          // staging stride: the largest big brick
    int device = 0;
    // device buffers
    uint4 *mrpd = nullptr;
    uint32_t *req = nullptr, *usage = nullptr, *order[2] = {nullptr, nullptr}, *slot_level = nullptr;
    float4 *slot_vpos = nullptr;
    unsigned long long *slot_bins = nullptr;  // value bins of each slot's brick (empty-space skipping)
    unsigned long long *entry_bins = nullptr; // per entry: resident brick's bins, else the user's, else ~0
    unsigned long long *user_bins = nullptr;  // per entry: the user's brick bins (given per volume), or null
    uint32_t b_shift = 32;                     // log2(B) for a power-of-two brick size
    bool entry_bins_dirty = false;
    unsigned long long *d_samples = nullptr;  // samples taken by the ray caster since creation
    uint8_t *pool = nullptr;
    // two-level directory (d.pt_block > 0): directory words, table pool, its
    // LRU (ping-pong like the brick pool's) and the install's claim scratch
    gc::PageTable pt{};
    uint32_t pt_slots = 0, pt_dims[3] = {0, 0, 0}, pt_cur = 0, epoch_pt = 0;
    uint64_t pt_words = 0;
    uint32_t *pt_order[2] = {nullptr, nullptr};
    uint4 *pt_keys = nullptr;
    uint32_t *pt_claim = nullptr, *pt_word_of = nullptr, *pt_njobs = nullptr;
    uint2 *pt_jobs = nullptr;
    uint64_t *status_pt = nullptr;
    gc::ScanCtl *ctl_pt = nullptr;
    uint64_t *status_lru = nullptr, *status_miss = nullptr;
    gc::ScanCtl *ctl_lru = nullptr, *ctl_miss = nullptr;
    uint32_t *d_count = nullptr, *d_misc = nullptr, *d_queue = nullptr;
    uint4 *d_asked = nullptr, *d_big_coord = nullptr;
    uint32_t *d_owner = nullptr;   // install: lowest list index per page-directory entry (~0 between installs)
    uint64_t *d_coords = nullptr;  // install: page-directory entry per list element
    uint32_t *d_big_index = nullptr;
    ulonglong2 *d_src = nullptr;      // gather list: {host address, bytes} per big brick
    uint8_t *d_staging = nullptr;
    gc::CutSources cut;               // device-resident pyramids of the volumes that have one
    uint4 *d_cut = nullptr, *h_cut = nullptr;  // cut jobs of a load cycle (device-levels sources)
    ResolveScratch resolve;           // the loader's per-cycle scratch
    gc::ViewParams *d_views = nullptr;
    uint32_t max_views = 256;
    // pinned host buffers
    uint4 *h_asked = nullptr, *h_big_coord = nullptr;
    uint32_t *h_big_index = nullptr, *h_misc = nullptr;
    // Miss lists: the scan writes one, the loader serves one.  The plain frame
    // loop only uses list 0; the batched form's overlapped loads use both.
    struct MissList {
        uint4 *d = nullptr, *h = nullptr;  // up to max_requests (x, y, z, level)
        uint32_t *total = nullptr;         // pinned: misses found (uncapped)
        cudaEvent_t ev = nullptr;          // the list and total are on the host
    } lists[2];
    int cur_load = 0;  // list the loader serves
    ulonglong2 *h_src = nullptr;
    uint8_t *h_staging = nullptr;
    cudaStream_t side = nullptr;
    cudaEvent_t ev_upload = nullptr, ev_upload_begin = nullptr;
    bool upload_timed = false;  // ev_upload_begin/ev_upload bracket an upload not yet counted
    int cur = 0;
    uint32_t ts = 1, epoch_lru = 0, epoch_miss = 0;
    // loader
    bool gather = false;              // every host-store volume is read by the gather kernel
    bool vec16 = false;
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    bool stop = false, has_request = false, busy = false, done = false, last_converged = false;
    uint32_t pend_n = 0, pend_nonempty = 0;
    std::string loader_error;
    gc_cache_stats stats;

    bool sync_mode() const { return (d.flags & GC_CACHE_SYNC_LOADER) != 0; }
};

namespace gc {

static void build_tables(gc_cache *C) {
    LevelTables &lt = C->lt;
    std::memset(&lt, 0, sizeof(lt));
    C->level_volume.clear();
    uint32_t off = 0, l = 0;
    C->mx = 0;
    C->my = 0;
    C->mz = 0;
    for (uint32_t v = 0; v < C->vols.size(); ++v) {
        Volume &V = C->vols[v];
        const gc_layout &L = V.layout;
        V.level_base = l;
        for (uint32_t k = 0; k < L.nb_levels; ++k, ++l) {
            lt.off[l] = off;
            for (int a = 0; a < 3; ++a) {
                lt.nb[l][a] = L.nb_bricks[k][a];
                lt.vvox[l][a] = L.nb_bricks[k][a] * C->Beff;
                lt.nbf[l][a] = static_cast<float>(lt.nb[l][a]);
                lt.vvoxf[l][a] = static_cast<float>(lt.vvox[l][a]);
                lt.ior[l][a] = static_cast<float>(L.initial[k][a]) / static_cast<float>(L.real[k][a]);
                lt.bb[l][a] = V.desc.big_brick_size[a];
            }
            lt.eb[l] = V.desc.encoded_bytes;
            off += L.nb_bricks[k][0];
            C->my = std::max(C->my, L.nb_bricks[k][1]);
            C->mz = std::max(C->mz, L.nb_bricks[k][2]);
            C->level_volume.push_back(v);
        }
    }
    lt.nlevels = l;
    C->mx = off;
    if (C->d.pt_block) {
        // directory words of the two-level directory: ceil(bricks / P) per
        // axis and level (CacheManager.hpp:160-176), levels packed along x
        const uint32_t P = C->d.pt_block;
        uint32_t toff = 0;
        C->pt_dims[1] = C->pt_dims[2] = 0;
        for (uint32_t k = 0; k < l; ++k) {
            lt.pt_off[k] = toff;
            toff += (lt.nb[k][0] + P - 1) / P;
            C->pt_dims[1] = std::max(C->pt_dims[1], (lt.nb[k][1] + P - 1) / P);
            C->pt_dims[2] = std::max(C->pt_dims[2], (lt.nb[k][2] + P - 1) / P);
        }
        C->pt_dims[0] = toff;
        C->pt_words = static_cast<uint64_t>(C->pt_dims[0]) * C->pt_dims[1] * C->pt_dims[2];
    }
    // the ray caster's page walk: one 32-bit index per entry, float-to-integer
    // floors exact below 2^23 voxels per axis
    GC_REQUIRE(static_cast<uint64_t>(C->mx) * C->my * C->mz < 0xffffffffull,
               "page directory too large (2^32 - 1 entries at most)");
    for (uint32_t k = 0; k < l; ++k)
        for (int a = 0; a < 3; ++a)
            GC_REQUIRE(lt.vvox[k][a] < (1u << 23), "level sizes up to 2^23 voxels per axis are supported");
    // exact multiply-high modulo by Beff (voxel coordinates below 2^25)
    C->beff_magic = C->Beff >= 2 && C->Beff <= 128
                        ? static_cast<uint32_t>(((1ull << 32) + C->Beff - 1) / C->Beff)
                        : 0u;
}

// Resolve the asked bricks: RequestHandler::handle_request (RequestHandler.hpp:277-372).
// Returns the number of bricks to install (non-empty first), or 0.
static void resolve_and_upload(gc_cache *C, uint32_t n) {
    const auto t_begin = std::chrono::steady_clock::now();
    ResolveScratch &R = C->resolve;
    R.kind.assign(n, 0);  // 0 non-empty, 1 empty, 2 unknown (dropped)
    std::vector<int> &kind = R.kind;
    uint32_t n_nonempty = 0, nbig = 0;
    std::vector<uint32_t> &big_index = R.big_index;
    big_index.clear();
    big_index.reserve(n);
    // Elements of one big brick share one load.  With one-brick big bricks
    // every element of the miss list (distinct page-directory entries) is
    // its own big brick and the table is skipped.
    bool dedupe = false;
    for (const Volume &V : C->vols)
        dedupe = dedupe || V.desc.big_brick_size[0] * V.desc.big_brick_size[1] * V.desc.big_brick_size[2] > 1;
    if (dedupe) {
        size_t cap = 16;
        while (cap < 2 * static_cast<size_t>(n)) cap <<= 1;
        R.keys.assign(cap, ResolveScratch::kNoKey);
        R.vals.assign(cap, 0);
    }
    struct Copy {
        const uint8_t *src;
        uint8_t *dst;
        uint64_t bytes;
    };
    std::vector<Copy> copies;
    struct FileRead {
        std::string path;
        uint8_t *dst;
        uint64_t bytes;
    };
    std::vector<FileRead> reads;
    uint32_t read_threads = 1;
    uint64_t bytes_up = 0;
    uint32_t ncut = 0, nhost = 0;  // big bricks cut on the device / taken from host sources
    for (uint32_t i = 0; i < n; ++i) {
        const uint4 b = C->lists[C->cur_load].h[i];  // (x, y, z, cache level)
        const Volume &V = C->vols[C->level_volume[b.w < C->lt.nlevels ? b.w : 0]];
        const uint32_t lvl = b.w - V.level_base;  // level within the volume
        const uint32_t *BB = V.desc.big_brick_size;
        const uint32_t gx = b.x / BB[0], gy = b.y / BB[1], gz = b.z / BB[2];
        const uint64_t key = gc_brick_key(b.w, gx, gy, gz);
        size_t cell = 0;
        if (dedupe) {
            cell = R.cell(key);
            if (R.keys[cell] == key) {
                const int32_t v = R.vals[cell];
                if (v == -1)
                    kind[i] = 1;
                else if (v == -2)
                    kind[i] = 2;
                else {
                    kind[i] = 0;
                    big_index.push_back(static_cast<uint32_t>(v));
                    ++n_nonempty;
                }
                continue;
            }
        }
        int status = GC_BRICK_UNKNOWN;
        bool on_device = false;
        const Source &src = V.src;
        uint8_t *stage = C->h_staging + static_cast<uint64_t>(nbig) * C->big_stride;
        if (!src.empty.empty() && src.empty.count(gc_brick_key(lvl, gx, gy, gz))) {  // the volume's own keys
            status = GC_BRICK_EMPTY;
        } else if (src.kind == 1) {
            const gc_layout &L = V.layout;
            if (lvl < L.nb_levels && gx < L.nb_big_bricks[lvl][0] && gy < L.nb_big_bricks[lvl][1] &&
                gz < L.nb_big_bricks[lvl][2]) {
                const uint64_t idx =
                    (static_cast<uint64_t>(gz) * L.nb_big_bricks[lvl][1] + gy) * L.nb_big_bricks[lvl][0] + gx;
                const uint64_t off = src.level_off[lvl] + idx * V.big_bytes;  // inside the store (checked)
                if (C->gather)
                    C->h_src[nbig] = make_ulonglong2(reinterpret_cast<uint64_t>(src.dev + off), V.big_bytes);
                else
                    copies.push_back({src.host + off, stage, V.big_bytes});
                status = GC_BRICK_SUCCESS;
            }
        } else if (src.kind == 2) {
            status = src.fn(src.user, lvl, gx, gy, gz, stage, V.big_bytes);
        } else if (src.kind == 5) {
            const gc_layout &L = V.layout;
            if (lvl < L.nb_levels && gx < L.nb_big_bricks[lvl][0] && gy < L.nb_big_bricks[lvl][1] &&
                gz < L.nb_big_bricks[lvl][2]) {
                const uint32_t vol = C->level_volume[b.w];
                C->h_cut[ncut++] = make_uint4(gx, gy, gz, (nbig << 8) | (vol << 6) | lvl);
                if (C->gather) C->h_src[nbig] = make_ulonglong2(0, 0);  // nothing to gather for this slot
                on_device = true;
                status = GC_BRICK_SUCCESS;
            }
        } else if (src.kind == 3) {
            std::string p = brick_file_path(src.dir, V.desc.brick_size, lvl, gx, gy, gz);
            struct stat st;
            if (::stat(p.c_str(), &st) == 0) {  // BricksManager::load_brick: a missing file is Unknown
                reads.push_back({std::move(p), stage, V.big_bytes});
                read_threads = std::max(read_threads, src.threads ? src.threads : 8u);
                status = GC_BRICK_SUCCESS;
            }
        }
        int32_t val;
        if (status == GC_BRICK_SUCCESS) {
            if (!on_device) {
                bytes_up += V.big_bytes;
                ++nhost;
            }
            val = static_cast<int32_t>(nbig);
            C->h_big_coord[nbig] = make_uint4(gx, gy, gz, b.w);
            big_index.push_back(nbig);
            ++nbig;
            ++n_nonempty;
            kind[i] = 0;
        } else if (status == GC_BRICK_EMPTY) {
            val = -1;
            kind[i] = 1;
        } else {
            // The reference asserts here (RequestHandler.hpp:348-350).  The
            // brick stays unmapped and is requested again by a later frame.
            val = -2;
            kind[i] = 2;
            C->stats.load_errors++;
        }
        if (dedupe) {
            R.keys[cell] = key;
            R.vals[cell] = val;
        }
    }
    // Host-store bricks are copied into the pinned staging buffer by up to 8
    // threads (one memcpy stream saturates well below the host's bandwidth).
    if (!copies.empty()) {
        const size_t bytes = copies.size() * C->big_stride;
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const unsigned nt = static_cast<unsigned>(
            std::min<size_t>(std::min(8u, hw), std::max<size_t>(1, bytes >> 21)));  // >= 2 MiB per thread
        auto work = [&](unsigned t) {
            for (size_t i = t; i < copies.size(); i += nt) std::memcpy(copies[i].dst, copies[i].src, copies[i].bytes);
        };
        if (nt <= 1) {
            work(0);
        } else {
            std::vector<std::thread> pool;
            for (unsigned t = 1; t < nt; ++t) pool.emplace_back(work, t);
            work(0);
            for (auto &th : pool) th.join();
        }
    }
    // Brick files: read and decompressed by worker threads into the staging slots.
    if (!reads.empty()) {
        std::atomic<size_t> next{0};
        std::atomic<bool> bad{false};
        std::string bad_path;
        std::mutex bad_mu;
        auto work = [&] {
            for (size_t i = next++; i < reads.size(); i = next++)
                if (read_brick_file(reads[i].path, reads[i].dst, reads[i].bytes) != 0) {
                    std::lock_guard<std::mutex> g(bad_mu);
                    bad = true;
                    bad_path = reads[i].path;
                }
        };
        const unsigned nt = static_cast<unsigned>(std::min<size_t>(read_threads, reads.size()));
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < nt; ++t) pool.emplace_back(work);
        work();
        for (auto &th : pool) th.join();
        if (bad) fail(GC_ERR_IO, "unreadable brick file " + bad_path);
    }
    // stable partition: non-empty first, then empty (RequestHandler.hpp:354-369)
    uint32_t k = 0;
    for (uint32_t i = 0; i < n; ++i)
        if (kind[i] == 0) C->h_asked[k++] = C->lists[C->cur_load].h[i];
    for (uint32_t i = 0; i < n; ++i)
        if (kind[i] == 1) C->h_asked[k++] = C->lists[C->cur_load].h[i];
    std::memcpy(C->h_big_index, big_index.data(), big_index.size() * sizeof(uint32_t));
    C->pend_n = k;
    C->pend_nonempty = n_nonempty;
    C->stats.load_cycles++;
    C->stats.loader_host_ns += static_cast<uint64_t>(
        std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t_begin).count());
    if (k == 0) return;
    // The upload goes on the high-priority side stream, beside the next
    // frame's render (the install of the next update waits for it): the
    // gather kernel's small blocks fit next to a persistent ray-caster launch
    // at its occupancy, so the bricks cross the host link while the frame
    // renders.  The staging buffers are free: the install that read them is
    // ahead of the scan this list came from.
    const bool gather = C->gather;
    cudaStream_t s = C->side;
    GC_CUDA(cudaEventRecord(C->ev_upload_begin, s));
    if (nhost && gather) {
        GC_CUDA(cudaMemcpyAsync(C->d_src, C->h_src, nbig * sizeof(ulonglong2), cudaMemcpyHostToDevice, s));
        launch_gather_bricks(C->d_src, nbig, C->big_stride, C->d_staging, C->vec16, true, s);
    } else if (nhost) {
        GC_CUDA(cudaMemcpyAsync(C->d_staging, C->h_staging, static_cast<size_t>(nbig) * C->big_stride,
                                cudaMemcpyHostToDevice, s));
    }
    if (ncut) {  // after the host bricks: a staged copy covers every slot
        GC_CUDA(cudaMemcpyAsync(C->d_cut, C->h_cut, ncut * sizeof(uint4), cudaMemcpyHostToDevice, s));
        launch_cut_bricks(C->cut, C->d_cut, ncut, C->d_staging, C->big_stride, s);
    }
    GC_CUDA(cudaMemcpyAsync(C->d_asked, C->h_asked, k * sizeof(uint4), cudaMemcpyHostToDevice, s));
    if (n_nonempty) {
        GC_CUDA(cudaMemcpyAsync(C->d_big_index, C->h_big_index, n_nonempty * sizeof(uint32_t),
                                cudaMemcpyHostToDevice, s));
        GC_CUDA(cudaMemcpyAsync(C->d_big_coord, C->h_big_coord, std::max(1u, nbig) * sizeof(uint4),
                                cudaMemcpyHostToDevice, s));
    }
    GC_CUDA(cudaEventRecord(C->ev_upload, s));
    C->upload_timed = true;
    C->stats.bytes_h2d += bytes_up;
    C->stats.requests_served += n;
}

// Waits for the miss list of the last scan and resolves it.  Returns true when
// bricks are pending for install.
static bool serve_request(gc_cache *C) {
    GC_CUDA(cudaSetDevice(C->device));
    GC_CUDA(cudaEventSynchronize(C->lists[C->cur_load].ev));
    // The previous upload has normally completed (its install ran before this
    // scan); waiting on it also keeps the staging buffers from being refilled
    // under a copy when the caller switches streams between frames.
    if (C->upload_timed) {
        GC_CUDA(cudaEventSynchronize(C->ev_upload));
        float ms = 0.f;
        GC_CUDA(cudaEventElapsedTime(&ms, C->ev_upload_begin, C->ev_upload));
        C->stats.upload_ns += static_cast<uint64_t>(static_cast<double>(ms) * 1e6);
        C->upload_timed = false;
    }
    const uint32_t total = *C->lists[C->cur_load].total;
    const uint32_t n = std::min(total, C->d.max_requests);
    C->stats.last_requests = total;
    C->stats.requests_raised += total;
    if (n == 0) return false;
    resolve_and_upload(C, n);
    return C->pend_n > 0;
}

static void loader_main(gc_cache *C) {
    std::unique_lock<std::mutex> lk(C->mu);
    for (;;) {
        C->cv.wait(lk, [&] { return C->stop || C->has_request; });
        if (C->stop) return;
        C->has_request = false;
        lk.unlock();
        bool pending = false, converged = false;
        std::string err;
        try {
            pending = serve_request(C);
            converged = (C->stats.last_requests == 0);
        } catch (const std::exception &e) {
            err = e.what();
        }
        lk.lock();
        C->done = pending;
        C->last_converged = converged;
        if (!err.empty()) C->loader_error = err;
        C->busy = false;
        C->cv.notify_all();
    }
}

static CacheView cache_view(const gc_cache *C) {
    CacheView cv;
    cv.mrpd = C->mrpd;
    cv.pt = C->pt;
    cv.req = C->req;
    cv.usage = C->usage;
    cv.pool = C->pool;
    cv.mx = C->mx;
    cv.my = C->my;
    cv.mxy = C->mx * C->my;
    cv.mz = C->mz;
    cv.sx = C->d.cache_size[0];
    cv.sy = C->d.cache_size[1];
    cv.sz = C->d.cache_size[2];
    cv.B = C->B;
    cv.c = C->c;
    cv.Beff = C->Beff;
    cv.beff_magic = C->beff_magic;
    cv.eb = C->eb;
    cv.nc = C->nc;
    cv.slot_bytes = C->slot_bytes;
    cv.entry_bins = C->entry_bins;
    cv.bins_user = C->user_bins ? 1u : 0u;
    cv.b_shift = C->b_shift;
    cv.samples = C->d_samples;
    cv.ts = C->ts;
    return cv;
}

static void lru_update(gc_cache *C, cudaStream_t s) {
    launch_lru_count(C->usage, C->nslots, C->ts, C->d_count, s);
    launch_lru_partition(C->order[C->cur], C->order[C->cur ^ 1], C->usage, C->ts, C->nslots, C->d_count,
                         C->status_lru, C->ctl_lru, ++C->epoch_lru, s);
    C->cur ^= 1;
    if (C->pt.shift) {
        // the table pool's LRU (CacheManager::lru_update's loop over the
        // table caches, CacheManager.hpp:386-406); its counter word is
        // pt_njobs, free between installs
        launch_lru_count(C->pt.usage, C->pt_slots, C->ts, C->pt_njobs, s);
        launch_lru_partition(C->pt_order[C->pt_cur], C->pt_order[C->pt_cur ^ 1], C->pt.usage, C->ts, C->pt_slots,
                             C->pt_njobs, C->status_pt, C->ctl_pt, ++C->epoch_pt, s);
        C->pt_cur ^= 1;
    }
}

static void install(gc_cache *C, cudaStream_t s) {
    if (C->pend_n == 0) return;
    GC_CUDA(cudaStreamWaitEvent(s, C->ev_upload, 0));
    InstallArgs a;
    a.mrpd = C->mrpd;
    a.pt = C->pt;
    a.pt_slots = C->pt_slots;
    a.pt_order = C->pt_order[C->pt_cur];
    a.pt_keys = C->pt_keys;
    a.pt_claim = C->pt_claim;
    a.pt_word_of = C->pt_word_of;
    a.pt_jobs = C->pt_jobs;
    a.pt_njobs = C->pt_njobs;
    a.mx = C->mx;
    a.my = C->my;
    a.nentries = C->nentries;
    a.order = C->order[C->cur];
    a.nslots = C->nslots;
    a.slot_level = C->slot_level;
    a.slot_vpos = C->slot_vpos;
    a.pool = C->pool;
    a.sx = C->d.cache_size[0];
    a.sy = C->d.cache_size[1];
    a.B = C->B;
    a.Beff = C->Beff;
    a.slot_bytes = C->slot_bytes;
    a.big_stride = C->big_stride;
    a.slot_bins = C->slot_bins;
    a.entry_bins = C->entry_bins;
    a.user_bins = C->user_bins;
    a.nc = C->nc;
    a.asked = C->d_asked;
    a.owner = C->d_owner;
    a.coords = C->d_coords;
    a.big_index = C->d_big_index;
    a.big_coord = C->d_big_coord;
    a.staging = C->d_staging;
    a.n = C->pend_n;
    a.n_nonempty = std::min(C->pend_nonempty, C->nslots);
    launch_install(a, C->lt, s);
    C->stats.bricks_installed += a.n_nonempty;
    C->stats.bricks_empty += a.n - C->pend_nonempty;
    C->pend_n = 0;
    C->pend_nonempty = 0;
}

// Miss scan into list `slot`; mark: flag the listed entries in flight (3).
static void scan_requests(gc_cache *C, cudaStream_t s, int slot = 0, bool mark = false) {
    gc_cache::MissList &L = C->lists[slot];
    launch_miss_compact(C->req, C->nentries - 1, C->ts, C->d.max_requests, L.d, C->lt, C->mx, C->my,
                        C->status_miss, C->ctl_miss, ++C->epoch_miss, s);
    if (mark) launch_mark_in_flight(L.d, C->ctl_miss, C->d.max_requests, C->lt, C->mx, C->my, C->nentries, C->mrpd, s);
    GC_CUDA(cudaMemcpyAsync(L.h, L.d, C->d.max_requests * sizeof(uint4), cudaMemcpyDeviceToHost, s));
    GC_CUDA(cudaMemcpyAsync(L.total, &C->ctl_miss->total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    GC_CUDA(cudaEventRecord(L.ev, s));
}

static bool update(gc_cache *C, cudaStream_t s) {
    GC_CUDA(cudaSetDevice(C->device));
    lru_update(C, s);
    bool converged = false;
    if (C->sync_mode()) {
        if (C->done) {
            install(C, s);
            C->done = false;
        } else {
            scan_requests(C, s);
            C->cur_load = 0;  // the loader serves list 0 (an overlapped batch may have left 1)
            C->done = serve_request(C);
            converged = (C->stats.last_requests == 0);
        }
    } else {
        std::unique_lock<std::mutex> lk(C->mu);
        if (!C->loader_error.empty()) {
            std::string e = C->loader_error;
            C->loader_error.clear();
            fail(GC_ERR_IO, "brick loader: " + e);
        }
        if (C->busy) {
            C->ts++;
            C->stats.frames++;
            return false;
        }
        if (C->done) {
            lk.unlock();
            install(C, s);
            lk.lock();
            C->done = false;
        } else {
            lk.unlock();
            scan_requests(C, s);
            C->cur_load = 0;  // the loader serves list 0 (an overlapped batch may have left 1)
            lk.lock();
            C->busy = true;
            C->has_request = true;
            C->cv.notify_all();
            converged = C->last_converged;
        }
    }
    C->ts++;
    C->stats.frames++;
    return converged;
}

static void destroy(gc_cache *C) {
    if (C->th.joinable()) {
        {
            std::lock_guard<std::mutex> g(C->mu);
            C->stop = true;
            C->cv.notify_all();
        }
        C->th.join();
    }
    cudaSetDevice(C->device);
    cudaDeviceSynchronize();
    void *dev[] = {C->pt.top, C->pt.table, C->pt.usage, C->pt_order[0], C->pt_order[1], C->pt_keys, C->pt_claim,
                   C->pt_word_of, C->pt_jobs, C->pt_njobs, C->status_pt, C->ctl_pt, C->mrpd, C->req, C->usage, C->order[0], C->order[1], C->slot_level, C->slot_vpos, C->pool, C->slot_bins, C->entry_bins, C->user_bins, C->d_samples,
                   C->status_lru, C->status_miss, C->ctl_lru, C->ctl_miss, C->d_count, C->d_misc, C->d_queue,
                   C->lists[0].d, C->lists[1].d, C->d_asked, C->d_owner, C->d_coords, C->d_big_coord, C->d_big_index, C->d_src,
                   C->d_staging, C->d_views, C->d_cut};
    for (void *p : dev)
        if (p) cudaFree(p);
    void *host[] = {C->lists[0].h, C->lists[1].h, C->lists[0].total, C->lists[1].total, C->h_asked, C->h_big_coord,
                    C->h_big_index, C->h_misc, C->h_src, C->h_staging, C->h_cut};
    for (void *p : host)
        if (p) cudaFreeHost(p);
    for (auto &L : C->lists)
        if (L.ev) cudaEventDestroy(L.ev);
    if (C->ev_upload) cudaEventDestroy(C->ev_upload);
    if (C->ev_upload_begin) cudaEventDestroy(C->ev_upload_begin);
    if (C->side) cudaStreamDestroy(C->side);
    delete C;
}

// LOD tables of display_volume_raycaster (VolumeRayCaster.cu:136-161).
static void fill_view(const gc_cache *C, const gc_view &in, ViewParams &out) {
    GC_REQUIRE(in.width > 0 && in.height > 0, "view size must be > 0");
    GC_REQUIRE(in.rgba && in.tbuf && in.state, "view buffers must be set");
    GC_REQUIRE(in.tf && in.tf_width >= 1, "transfer function must be set");
    GC_REQUIRE(in.tstep > 0.f, "tstep must be > 0");
    GC_REQUIRE(in.mode == GC_MODE_DVR || in.mode == GC_MODE_MOP, "bad compositing mode");
    GC_REQUIRE(in.sampler == GC_SAMPLER_REFERENCE || in.sampler == GC_SAMPLER_TRILINEAR, "bad sampler");
    GC_REQUIRE(in.volume < C->vols.size(), "the view's volume is not in this cache");
    const Volume &V = C->vols[in.volume];
    GC_REQUIRE(V.desc.channels == 1 || (V.desc.channels == 2 && V.desc.encoded_bytes == 2),
               "the ray caster renders one channel (8, 16 or 32 bit) or two 8-bit channels");
    if (V.desc.channels == 2)
        GC_REQUIRE(in.tf_height >= 1, "a two-channel volume needs a 2D transfer function (tf_height >= 1)");
    else
        GC_REQUIRE(in.tf_height <= 1, "a 2D transfer function needs a two-channel volume");
    std::memset(&out, 0, sizeof(out));
    std::memcpy(out.m, in.inv_view, sizeof(out.m));
    out.W = in.width;
    out.H = in.height;
    for (int a = 0; a < 3; ++a) {
        out.bmin[a] = in.bbox_min[a];
        out.bmax[a] = in.bbox_max[a];
    }
    out.tstep = in.tstep;
    out.focal = in.focal;
    out.early = in.early_alpha;
    out.mode = in.mode;
    out.sampler = in.sampler;
    out.tfw = in.tf_width;
    out.tfh = in.tf_height > 0 ? in.tf_height : 1;
    // empty-space skipping: DVR of one channel through a 1D transfer function
    out.skip_empty = in.mode == GC_MODE_DVR && V.desc.channels == 1 ? render_tuning().skip_empty : 0u;
    out.visible = ~0ull;  // filled from the transfer function on the device (view_bins_kernel)
    out.tf = in.tf;
    out.rgba = in.rgba;
    out.tbuf = in.tbuf;
    out.state = in.state;
    out.status = in.status;
    out.fallback = in.fallback ? 1u : 0u;
    const float bsx = in.bbox_max[0] - in.bbox_min[0];
    const float bsy = in.bbox_max[1] - in.bbox_min[1];
    const float bsz = in.bbox_max[2] - in.bbox_min[2];
    const float bmin = std::min(bsx, std::min(bsy, bsz));
    const gc_layout &L = V.layout;
    out.level_base = V.level_base;
    out.nlevels = L.nb_levels;
    out.eb = V.desc.encoded_bytes;
    for (uint32_t l = 0; l < L.nb_levels; ++l) {
        for (int a = 0; a < 3; ++a) out.inv_size[l][a] = bmin / static_cast<float>(L.initial[l][a]);
        const uint32_t mn = std::min(L.initial[l][0], std::min(L.initial[l][1], L.initial[l][2]));
        out.step[l] = (bmin / static_cast<float>(mn)) / 2.f;
        out.kexp[l] = out.step[l] / in.tstep;
        // 1 - (1 - a)^k <= k a / (1 - a) <= 1.05 k a for a <= 0.04: below the
        // floor the corrected opacity stays under 0.0009 (threshold 0.001)
        out.alpha_floor[l] = out.kexp[l] > 0.f ? std::min(0.04f, 0.0009f / (1.05f * out.kexp[l])) : 0.f;
    }
    const uint32_t tw = render_tuning().tile_w;
    out.tiles_x = div_up(in.width, tw);
    out.tile_shift = static_cast<uint32_t>(__builtin_ctz(tw));
}

// graph + pinned view table: the batched form replays a CUDA graph instead
// of launching (launch_render_graph)
// Page-directory table of the user's brick value bins from the volumes' bins:
// ~0 (never skipped) for levels without bins and for the bricks of empty big
// bricks, which step like empty bricks once installed and so must be
// requested.  The per-entry table the ray caster reads is then rebuilt: the
// user's bins, with every resident brick's own bins at its entry.
static void refresh_entry_bins(gc_cache *C, cudaStream_t s) {
    if (!C->entry_bins_dirty) return;
    C->entry_bins_dirty = false;
    bool any = false;
    for (const Volume &V : C->vols) any = any || !V.bins.empty();
    GC_CUDA(cudaStreamSynchronize(s));
    if (!any) {
        if (C->user_bins) {
            GC_CUDA(cudaFree(C->user_bins));
            C->user_bins = nullptr;
        }
        GC_CUDA(cudaMemsetAsync(C->entry_bins, 0xff, C->nentries * sizeof(uint64_t), s));
        launch_live_bins(C->lt, C->slot_vpos, C->slot_level, C->slot_bins, C->nslots, C->mx, C->my, C->nentries,
                         C->entry_bins, C->pt, C->d.cache_size[0], C->d.cache_size[1], C->B, s);
        GC_CUDA(cudaStreamSynchronize(s));
        return;
    }
    std::vector<uint64_t> h(C->nentries, ~0ull);
    for (const Volume &V : C->vols) {
        if (V.bins.empty()) continue;
        const gc_layout &L = V.layout;
        const uint32_t *BB = V.desc.big_brick_size;
        uint64_t k = 0;
        for (uint32_t l = 0; l < L.nb_levels; ++l) {
            const uint32_t lvl = V.level_base + l;
            for (uint32_t z = 0; z < L.nb_bricks[l][2]; ++z)
                for (uint32_t y = 0; y < L.nb_bricks[l][1]; ++y)
                    for (uint32_t x = 0; x < L.nb_bricks[l][0]; ++x, ++k) {
                        const uint64_t e = C->lt.off[lvl] + x + static_cast<uint64_t>(y) * C->mx +
                                           static_cast<uint64_t>(z) * C->mx * C->my;
                        const bool empty = V.src.empty.count(gc_brick_key(l, x / BB[0], y / BB[1], z / BB[2])) != 0;
                        h[e] = empty ? ~0ull : V.bins[k];
                    }
        }
    }
    if (!C->user_bins) C->user_bins = dalloc<unsigned long long>(C->nentries, "page-directory user bins");
    GC_CUDA(cudaMemcpyAsync(C->user_bins, h.data(), C->nentries * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    GC_CUDA(cudaMemcpyAsync(C->entry_bins, C->user_bins, C->nentries * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
    launch_live_bins(C->lt, C->slot_vpos, C->slot_level, C->slot_bins, C->nslots, C->mx, C->my, C->nentries,
                     C->entry_bins, C->pt, C->d.cache_size[0], C->d.cache_size[1], C->B, s);
    GC_CUDA(cudaStreamSynchronize(s));
}

// The tiles whose rays can meet the view's box: the box's 8 corners projected
// with the ray caster's camera (a ray through pixel (x, y) has the camera
// direction (u, v, -focal), u = 2 (x + 0.5) / W - 1, v likewise, turned by the
// view matrix), their bounding rectangle widened by a pixel.  When a corner
// lies on or behind the camera plane the whole image is the rectangle.  Only
// the order of the work depends on it: every tile is rendered either way.
static void screen_rect(ViewParams &v) {
    const uint32_t tw = 1u << v.tile_shift, th = 32u >> v.tile_shift;
    const uint32_t ntx = v.tiles_x, nty = div_up(v.H, th);
    v.rx0 = 0;
    v.ry0 = 0;
    v.rw = ntx;
    v.rh = nty;
    double R[3][3], o[3];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) R[r][c] = v.m[4 * r + c];
        o[r] = v.m[4 * r + 3];
    }
    // inverse of the 3x3 part (world direction = R * camera direction)
    const double det = R[0][0] * (R[1][1] * R[2][2] - R[1][2] * R[2][1]) -
                       R[0][1] * (R[1][0] * R[2][2] - R[1][2] * R[2][0]) +
                       R[0][2] * (R[1][0] * R[2][1] - R[1][1] * R[2][0]);
    if (!(std::fabs(det) > 1e-12) || !(v.focal > 0.f)) return;
    double I[3][3];
    I[0][0] = (R[1][1] * R[2][2] - R[1][2] * R[2][1]) / det;
    I[0][1] = (R[0][2] * R[2][1] - R[0][1] * R[2][2]) / det;
    I[0][2] = (R[0][1] * R[1][2] - R[0][2] * R[1][1]) / det;
    I[1][0] = (R[1][2] * R[2][0] - R[1][0] * R[2][2]) / det;
    I[1][1] = (R[0][0] * R[2][2] - R[0][2] * R[2][0]) / det;
    I[1][2] = (R[0][2] * R[1][0] - R[0][0] * R[1][2]) / det;
    I[2][0] = (R[1][0] * R[2][1] - R[1][1] * R[2][0]) / det;
    I[2][1] = (R[0][1] * R[2][0] - R[0][0] * R[2][1]) / det;
    I[2][2] = (R[0][0] * R[1][1] - R[0][1] * R[1][0]) / det;
    double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
    for (int k = 0; k < 8; ++k) {
        const double P[3] = {(k & 1) ? v.bmax[0] : v.bmin[0], (k & 2) ? v.bmax[1] : v.bmin[1],
                             (k & 4) ? v.bmax[2] : v.bmin[2]};
        double q[3];
        for (int r = 0; r < 3; ++r)
            q[r] = I[r][0] * (P[0] - o[0]) + I[r][1] * (P[1] - o[1]) + I[r][2] * (P[2] - o[2]);
        if (!(q[2] < -1e-6)) return;  // a corner on or behind the camera plane
        const double u = -v.focal * q[0] / q[2], w = -v.focal * q[1] / q[2];
        const double x = (u + 1.0) * 0.5 * v.W - 0.5, y = (w + 1.0) * 0.5 * v.H - 0.5;
        xmin = std::min(xmin, x);
        xmax = std::max(xmax, x);
        ymin = std::min(ymin, y);
        ymax = std::max(ymax, y);
    }
    auto clampi = [](double a, double lo, double hi) { return a < lo ? lo : (a > hi ? hi : a); };
    const double tx0 = clampi(std::floor((xmin - 1.0) / tw), 0, ntx), tx1 = clampi(std::floor((xmax + 1.0) / tw) + 1, 0, ntx);
    const double ty0 = clampi(std::floor((ymin - 1.0) / th), 0, nty), ty1 = clampi(std::floor((ymax + 1.0) / th) + 1, 0, nty);
    v.rx0 = static_cast<uint32_t>(tx0);
    v.ry0 = static_cast<uint32_t>(ty0);
    v.rw = tx1 > tx0 ? static_cast<uint32_t>(tx1 - tx0) : 0u;
    v.rh = ty1 > ty0 ? static_cast<uint32_t>(ty1 - ty0) : 0u;
    if (v.rw == 0 || v.rh == 0) v.rw = v.rh = 0;
}

static void render(gc_cache *C, const gc_view *views, uint32_t n, cudaStream_t s, bool mark_done = false,
                   RenderGraph *graph = nullptr, ViewParams *pinned = nullptr) {
    GC_REQUIRE(views && n >= 1, "no views");
    GC_REQUIRE(n <= C->max_views, "too many views in one batch");
    GC_CUDA(cudaSetDevice(C->device));
    refresh_entry_bins(C, s);
    std::vector<ViewParams> vp(n);
    uint32_t tiles = 0, rect_total = 0;
    for (uint32_t i = 0; i < n; ++i) {
        fill_view(C, views[i], vp[i]);
        vp[i].mark_done = mark_done ? 1u : 0u;
        tiles += vp[i].tiles_x * div_up(views[i].height, 32u >> vp[i].tile_shift);
        screen_rect(vp[i]);
        vp[i].rect_begin = rect_total;
        rect_total += vp[i].rw * vp[i].rh;
    }
    for (uint32_t i = 0, out = rect_total; i < n; ++i) {
        vp[i].rect_total = rect_total;
        vp[i].out_begin = out;
        out += vp[i].tiles_x * div_up(vp[i].H, 32u >> vp[i].tile_shift) - vp[i].rw * vp[i].rh;
    }
    if (graph) {
        std::memcpy(pinned, vp.data(), n * sizeof(ViewParams));
        launch_render_graph(*graph, cache_view(C), C->lt, C->d_views, pinned, n, tiles, C->d_queue, s);
        return;
    }
    // pageable source: the call returns once the data is staged
    GC_CUDA(cudaMemcpyAsync(C->d_views, vp.data(), n * sizeof(ViewParams), cudaMemcpyHostToDevice, s));
    launch_view_bins(C->d_views, n, s);
    launch_render(cache_view(C), C->lt, C->d_views, vp.data(), n, tiles, C->d_queue, nullptr, s);
}

// Upload route of the cache: the gather kernel when every volume with a host
// store can be read by the device and no volume loads through a callback
// (callbacks fill the pinned staging buffer); staged copies otherwise.
static void update_upload_route(gc_cache *C) {
    bool any = false, all = true, vec16 = C->big_stride % 16 == 0;
    for (const Volume &V : C->vols) {
        if (V.src.kind == 2 || V.src.kind == 3) all = false;
        if (V.src.kind == 1) {
            any = true;
            all = all && V.src.direct;
            vec16 = vec16 && V.src.vec16;
        }
    }
    C->gather = any && all;
    C->vec16 = vec16;
}

static bool has_source(const gc_cache *C) {
    for (const Volume &V : C->vols)
        if (V.src.kind != 0) return true;
    return false;
}

// A cache over n volumes (the first one described by desc): one page
// directory holding the levels of all of them, one pool, one LRU.
static gc_cache *create_cache(const gc_cache_desc *desc, const gc_volume_desc *vols, const gc_layout *layouts,
                              uint32_t n) {
    GC_REQUIRE(n >= 1 && n <= kMaxCacheLevels / GC_MAX_LEVELS, "a cache holds 1 to 4 volumes");
    uint32_t total_levels = 0;
    for (uint32_t v = 0; v < n; ++v) {
        validate_volume(vols[v]);
        GC_REQUIRE(layouts[v].nb_levels >= 1 && layouts[v].nb_levels <= GC_MAX_LEVELS, "bad layout");
        GC_REQUIRE(vols[v].brick_size == vols[0].brick_size && vols[v].covering == vols[0].covering,
                   "volumes sharing a pool need the same BrickSize and VoxelCovering");
        GC_REQUIRE(vols[v].channels == vols[0].channels, "volumes sharing a pool need the same NumberChannels");
        total_levels += layouts[v].nb_levels;
    }
    GC_REQUIRE(total_levels <= kMaxCacheLevels, "too many levels in one cache");
    GC_REQUIRE(desc->max_requests >= 1 && desc->max_requests <= 16384, "max_requests must be in [1, 16384]");
    for (int a = 0; a < 3; ++a) GC_REQUIRE(desc->cache_size[a] >= 1, "cache size must be >= 1");
    gc_cache *C = new gc_cache();
    try {
        std::memset(&C->stats, 0, sizeof(C->stats));
        C->d = *desc;
        C->d.volume = vols[0];
        C->d.layout = layouts[0];
        C->device = desc->gpu;
        GC_CUDA(cudaSetDevice(C->device));
        C->B = vols[0].brick_size;
        C->c = vols[0].covering;
        C->Beff = C->B - 2 * C->c;
        C->eb = vols[0].encoded_bytes;
        C->nc = vols[0].channels;
        uint32_t eb_max = 0;
        C->vols.resize(n);
        for (uint32_t v = 0; v < n; ++v) {
            Volume &V = C->vols[v];
            V.desc = vols[v];
            V.layout = layouts[v];
            V.brick_bytes = static_cast<uint64_t>(C->B) * C->B * C->B * vols[v].encoded_bytes;
            V.big_bytes = V.brick_bytes * vols[v].big_brick_size[0] * vols[v].big_brick_size[1] *
                          vols[v].big_brick_size[2];
            eb_max = std::max(eb_max, vols[v].encoded_bytes);
            if (vols[v].encoded_bytes != C->eb) C->eb = 0;  // mixed voxel widths
            C->big_stride = std::max(C->big_stride, V.big_bytes);
        }
        C->slot_bytes = static_cast<uint64_t>(C->B) * C->B * C->B * eb_max;
    } catch (...) {
        delete C;
        throw;
    }
    return C;
}

}  // namespace gc

using namespace gc;

extern "C" {

int gc_cache_create(const gc_cache_desc *desc, gc_cache_t *out) {
    if (!desc) return guard([] { fail(GC_ERR_INVALID, "null argument"); });
    return gc_cache_create_shared(desc, &desc->volume, &desc->layout, 1, out);
}

int gc_cache_create_shared(const gc_cache_desc *desc, const gc_volume_desc *volumes, const gc_layout *layouts,
                           uint32_t n_volumes, gc_cache_t *out) {
    gc_cache *C = nullptr;
    int rc = guard([&] {
        GC_REQUIRE(desc && volumes && layouts && out, "null argument");
        C = create_cache(desc, volumes, layouts, n_volumes);
        const uint64_t nslots = static_cast<uint64_t>(desc->cache_size[0]) * desc->cache_size[1] * desc->cache_size[2];
        GC_REQUIRE(nslots < (1ull << 31), "too many pool slots");
        GC_REQUIRE(desc->max_requests <= nslots, "max_requests must not exceed the number of pool slots");
        C->nslots = static_cast<uint32_t>(nslots);
        build_tables(C);
        C->nentries = static_cast<uint64_t>(C->mx) * C->my * C->mz;
        GC_REQUIRE(C->nentries >= 2, "page directory too small");
        GC_REQUIRE(C->nentries < (1ull << 32), "page directory too large");
        const uint32_t maxr = desc->max_requests;
        if (desc->pt_block) {
            uint32_t shift = 0;
            while ((1u << shift) < desc->pt_block) ++shift;
            GC_REQUIRE(desc->pt_block >= 2 && desc->pt_block <= 16 && (1u << shift) == desc->pt_block,
                       "pt_block must be 0 or a power of two from 2 to 16");
            GC_REQUIRE(desc->pt_slots >= 1 && desc->pt_slots < (1u << 30), "pt_slots must be in [1, 2^30)");
            C->pt_slots = desc->pt_slots;
            C->pt.shift = shift;
            C->pt.tx = C->pt_dims[0];
            C->pt.txy = C->pt_dims[0] * C->pt_dims[1];
            const uint64_t per = 1ull << (3 * shift);
            C->pt.top = dalloc<uint32_t>(C->pt_words, "page-table directory");
            C->pt.table = dalloc<uint4>(C->pt_slots * per, "page-table pool");
            C->pt.usage = dalloc<uint32_t>(C->pt_slots, "page-table usage");
            C->pt_order[0] = dalloc<uint32_t>(C->pt_slots, "page-table LRU");
            C->pt_order[1] = dalloc<uint32_t>(C->pt_slots, "page-table LRU");
            C->pt_keys = dalloc<uint4>(C->pt_slots, "page-table keys");
            C->pt_claim = dalloc<uint32_t>(C->pt_words, "page-table claims");
            C->pt_word_of = dalloc<uint32_t>(maxr, "page-table claim words");
            C->pt_jobs = dalloc<uint2>(maxr, "page-table jobs");
            C->pt_njobs = dalloc<uint32_t>(1, "page-table job count");
            C->status_pt = dalloc<uint64_t>(lookback_tiles(C->pt_slots), "scan status");
            C->ctl_pt = dalloc<ScanCtl>(1, "scan control");
            GC_CUDA(cudaMemset(C->pt.top, 0, C->pt_words * sizeof(uint32_t)));
            GC_CUDA(cudaMemset(C->pt.table, 0, C->pt_slots * per * sizeof(uint4)));
            GC_CUDA(cudaMemset(C->pt.usage, 0, C->pt_slots * sizeof(uint32_t)));
            GC_CUDA(cudaMemset(C->pt_claim, 0xff, C->pt_words * sizeof(uint32_t)));
            GC_CUDA(cudaMemset(C->status_pt, 0, lookback_tiles(C->pt_slots) * sizeof(uint64_t)));
            GC_CUDA(cudaMemset(C->ctl_pt, 0, sizeof(ScanCtl)));
            launch_pt_init(C->pt_order[0], C->pt_keys, C->pt_slots, nullptr);
        } else {
            C->mrpd = dalloc<uint4>(C->nentries, "page directory");
            GC_CUDA(cudaMemset(C->mrpd, 0, C->nentries * sizeof(uint4)));
        }
        C->req = dalloc<uint32_t>(C->nentries, "request buffer");
        C->usage = dalloc<uint32_t>(C->nslots, "usage buffer");
        C->order[0] = dalloc<uint32_t>(C->nslots, "LRU");
        C->order[1] = dalloc<uint32_t>(C->nslots, "LRU");
        C->slot_level = dalloc<uint32_t>(C->nslots, "slot levels");
        C->slot_vpos = dalloc<float4>(C->nslots, "slot positions");
        C->pool = dalloc<uint8_t>(C->nslots * C->slot_bytes, "brick pool");
        C->slot_bins = dalloc<unsigned long long>(C->nslots, "slot value bins");
        C->entry_bins = dalloc<unsigned long long>(C->nentries, "page-directory value bins");
        GC_CUDA(cudaMemset(C->entry_bins, 0xff, C->nentries * sizeof(unsigned long long)));
        C->b_shift = 32;
        for (uint32_t k = 0; k < 31; ++k)
            if ((1u << k) == C->B) C->b_shift = k;
        C->d_samples = dalloc<unsigned long long>(2, "sample and ray counters");
        GC_CUDA(cudaMemset(C->d_samples, 0, 2 * sizeof(unsigned long long)));
        GC_CUDA(cudaMemset(C->slot_bins, 0xff, C->nslots * sizeof(unsigned long long)));
        C->status_lru = dalloc<uint64_t>(lookback_tiles(C->nslots), "scan status");
        C->status_miss = dalloc<uint64_t>(lookback_tiles(C->nentries), "scan status");
        C->ctl_lru = dalloc<ScanCtl>(1, "scan control");
        C->ctl_miss = dalloc<ScanCtl>(1, "scan control");
        C->d_count = dalloc<uint32_t>(1, "counter");
        C->d_misc = dalloc<uint32_t>(1, "counter");
        C->d_queue = dalloc<uint32_t>(4, "work queue");
        for (auto &L : C->lists) L.d = dalloc<uint4>(maxr, "miss list");
        C->d_asked = dalloc<uint4>(maxr, "asked list");
        C->d_coords = dalloc<uint64_t>(maxr, "install entries");
        C->d_owner = dalloc<uint32_t>(C->nentries, "install owners");
        GC_CUDA(cudaMemset(C->d_owner, 0xff, C->nentries * sizeof(uint32_t)));
        C->d_big_coord = dalloc<uint4>(maxr, "big brick coords");
        C->d_big_index = dalloc<uint32_t>(maxr, "big brick indexes");
        C->d_src = dalloc<ulonglong2>(maxr, "brick gather list");
        C->d_staging = dalloc<uint8_t>(maxr * C->big_stride, "staging");
        C->d_views = dalloc<ViewParams>(C->max_views, "views");
        for (auto &L : C->lists) {
            L.h = halloc<uint4>(maxr);
            L.total = halloc<uint32_t>(1);
            *L.total = 0;
        }
        C->h_asked = halloc<uint4>(maxr);
        C->h_big_coord = halloc<uint4>(maxr);
        C->h_big_index = halloc<uint32_t>(maxr);
        C->h_src = halloc<ulonglong2>(maxr);
        C->h_misc = halloc<uint32_t>(1);
        C->h_staging = halloc<uint8_t>(maxr * C->big_stride);
        *C->h_misc = 0;
        GC_CUDA(cudaMemset(C->req, 0, C->nentries * sizeof(uint32_t)));
        GC_CUDA(cudaMemset(C->usage, 0, C->nslots * sizeof(uint32_t)));
        GC_CUDA(cudaMemset(C->pool, 0, C->nslots * C->slot_bytes));
        GC_CUDA(cudaMemset(C->status_lru, 0, lookback_tiles(C->nslots) * sizeof(uint64_t)));
        GC_CUDA(cudaMemset(C->status_miss, 0, lookback_tiles(C->nentries) * sizeof(uint64_t)));
        GC_CUDA(cudaMemset(C->ctl_lru, 0, sizeof(ScanCtl)));
        GC_CUDA(cudaMemset(C->ctl_miss, 0, sizeof(ScanCtl)));
        GC_CUDA(cudaMemset(C->d_queue, 0, 4 * sizeof(uint32_t)));
        init_slots_kernel<<<std::min<uint32_t>(div_up(C->nslots, 256), 4096), 256>>>(C->order[0], C->slot_level,
                                                                                    C->slot_vpos, C->nslots);
        GC_CUDA(cudaGetLastError());
        count_launch();
        int least = 0, greatest = 0;
        GC_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        GC_CUDA(cudaStreamCreateWithPriority(&C->side, cudaStreamNonBlocking, greatest));
        for (auto &L : C->lists) GC_CUDA(cudaEventCreateWithFlags(&L.ev, cudaEventDisableTiming));
        GC_CUDA(cudaEventCreate(&C->ev_upload));
        GC_CUDA(cudaEventCreate(&C->ev_upload_begin));
        GC_CUDA(cudaDeviceSynchronize());
        if (!C->sync_mode()) C->th = std::thread(loader_main, C);
        *out = C;
    });
    if (rc != GC_OK && C) destroy(C);
    return rc;
}

int gc_cache_destroy(gc_cache_t cache) {
    if (cache) destroy(cache);
    return GC_OK;
}

int gc_cache_set_volume_source_host(gc_cache_t C, uint32_t volume, const void *bricks, uint64_t bytes,
                                    const uint64_t *level_offsets, const uint64_t *empty_keys, size_t n_empty) {
    return guard([&] {
        GC_REQUIRE(C && bricks && level_offsets && (empty_keys || n_empty == 0), "null argument");
        GC_REQUIRE(volume < C->vols.size(), "no such volume in this cache");
        GC_CUDA(cudaSetDevice(C->device));
        const Volume &V = C->vols[volume];
        const gc_layout &L = V.layout;
        bool aligned = V.big_bytes % 16 == 0;
        for (uint32_t l = 0; l < L.nb_levels; ++l) {
            const uint64_t nbig =
                static_cast<uint64_t>(L.nb_big_bricks[l][0]) * L.nb_big_bricks[l][1] * L.nb_big_bricks[l][2];
            GC_REQUIRE(level_offsets[l] <= bytes && nbig <= (bytes - level_offsets[l]) / V.big_bytes,
                       "brick store: level " + std::to_string(l) + " does not fit in the store's bytes");
            aligned = aligned && level_offsets[l] % 16 == 0;
        }
        // Can the device read the store?  Page-locked memory has a device
        // address; any host memory can be read where the device accesses
        // pageable memory coherently.
        bool direct = false;
        const uint8_t *dev = nullptr;
        if (!(C->d.flags & GC_CACHE_STAGED_UPLOAD)) {
            cudaPointerAttributes at;
            if (cudaPointerGetAttributes(&at, bricks) == cudaSuccess && at.type == cudaMemoryTypeHost &&
                at.devicePointer) {
                direct = true;
                dev = static_cast<const uint8_t *>(at.devicePointer);
            } else {
                (void)cudaGetLastError();
                int pageable = 0;
                GC_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, C->device));
                if (pageable) {
                    direct = true;
                    dev = static_cast<const uint8_t *>(bricks);
                }
            }
        }
        std::lock_guard<std::mutex> g(C->mu);
        GC_REQUIRE(!C->busy, "the loader is busy");
        Source &src = C->vols[volume].src;
        src = Source();
        src.kind = 1;
        src.host = static_cast<const uint8_t *>(bricks);
        src.bytes = bytes;
        src.direct = direct;
        src.dev = dev;
        src.vec16 = aligned && reinterpret_cast<uintptr_t>(dev) % 16 == 0;
        src.level_off.assign(level_offsets, level_offsets + L.nb_levels);
        for (size_t i = 0; i < n_empty; ++i) src.empty.insert(empty_keys[i]);
        update_upload_route(C);
        C->entry_bins_dirty = true;
    });
}

int gc_cache_set_volume_source_device(gc_cache_t C, uint32_t volume, const void *pyramid,
                                      const uint64_t *level_offsets, const uint64_t *empty_keys, size_t n_empty) {
    return guard([&] {
        GC_REQUIRE(C && pyramid && level_offsets && (empty_keys || n_empty == 0), "null argument");
        GC_REQUIRE(volume < C->vols.size(), "no such volume in this cache");
        GC_CUDA(cudaSetDevice(C->device));
        cudaPointerAttributes at;
        GC_CUDA(cudaPointerGetAttributes(&at, pyramid));
        GC_REQUIRE(at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged,
                   "the pyramid must be device memory");
        const Volume &V = C->vols[volume];
        const gc_layout &L = V.layout;
        CutSource cs;
        cs.pyramid = static_cast<const uint8_t *>(pyramid);
        BrickParams &p = cs.p;
        p.B = V.desc.brick_size;
        p.c = V.desc.covering;
        p.Beff = p.B - 2 * p.c;
        for (int a = 0; a < 3; ++a) p.BB[a] = V.desc.big_brick_size[a];
        p.eb = V.desc.encoded_bytes;
        while ((1u << p.b_shift) < p.B) ++p.b_shift;
        const bool pow2 = (p.B & (p.B - 1)) == 0;
        while (pow2 && (16u << p.cpr_shift) < p.B * p.eb) ++p.cpr_shift;
        for (uint32_t l = 0; l < L.nb_levels; ++l) {
            GC_REQUIRE(L.mip[l][0] == L.initial[l][0] && L.mip[l][1] == L.initial[l][1] &&
                           L.mip[l][2] == L.initial[l][2],
                       "the pyramid's level sizes differ from the metadata sizes");
            cs.offset[l] = level_offsets[l];
            for (int a = 0; a < 3; ++a) cs.dims[l][a] = L.mip[l][a];
            cs.fast[l] = (p.eb == 1 || p.eb == 2 || p.eb == 4) && pow2 && (p.B * p.eb) % 16 == 0 &&
                         (static_cast<uint64_t>(L.mip[l][0]) * p.eb) % 16 == 0 &&
                         (reinterpret_cast<uintptr_t>(pyramid) + level_offsets[l]) % 16 == 0 &&
                         C->big_stride % 16 == 0;
        }
        std::lock_guard<std::mutex> g(C->mu);
        GC_REQUIRE(!C->busy, "the loader is busy");
        if (!C->d_cut) {
            C->d_cut = dalloc<uint4>(C->d.max_requests, "cut jobs");
            GC_CUDA(cudaMallocHost(reinterpret_cast<void **>(&C->h_cut), C->d.max_requests * sizeof(uint4)));
        }
        C->cut.vol[volume] = cs;
        Source &src = C->vols[volume].src;
        src = Source();
        src.kind = 5;
        src.level_off.assign(level_offsets, level_offsets + L.nb_levels);
        for (size_t i = 0; i < n_empty; ++i) src.empty.insert(empty_keys[i]);
        update_upload_route(C);
        C->entry_bins_dirty = true;
    });
}

int gc_cache_set_volume_source_files(gc_cache_t C, uint32_t volume, const char *volume_dir,
                                     const uint64_t *empty_keys, size_t n_empty, uint32_t threads) {
    return guard([&] {
        GC_REQUIRE(C && volume_dir && (empty_keys || n_empty == 0), "null argument");
        GC_REQUIRE(volume < C->vols.size(), "no such volume in this cache");
        std::string why;
        if (!lz4_available(&why)) fail(GC_ERR_UNSUPPORTED, why);
        std::lock_guard<std::mutex> g(C->mu);
        GC_REQUIRE(!C->busy, "the loader is busy");
        Source &src = C->vols[volume].src;
        src = Source();
        src.kind = 3;
        src.dir = volume_dir;
        if (!src.dir.empty() && src.dir.back() != '/') src.dir += '/';
        src.threads = threads;
        for (size_t i = 0; i < n_empty; ++i) src.empty.insert(empty_keys[i]);
        update_upload_route(C);
        C->entry_bins_dirty = true;
    });
}

int gc_cache_set_volume_source_callback(gc_cache_t C, uint32_t volume, gc_brick_loader_fn fn, void *user,
                                        const uint64_t *empty_keys, size_t n_empty) {
    return guard([&] {
        GC_REQUIRE(C && fn && (empty_keys || n_empty == 0), "null argument");
        GC_REQUIRE(volume < C->vols.size(), "no such volume in this cache");
        std::lock_guard<std::mutex> g(C->mu);
        GC_REQUIRE(!C->busy, "the loader is busy");
        Source &src = C->vols[volume].src;
        src = Source();
        src.kind = 2;
        src.fn = fn;
        src.user = user;
        for (size_t i = 0; i < n_empty; ++i) src.empty.insert(empty_keys[i]);
        update_upload_route(C);
        C->entry_bins_dirty = true;
    });
}

int gc_cache_set_volume_brick_bins(gc_cache_t C, uint32_t volume, const uint64_t *bins, uint64_t n) {
    return guard([&] {
        GC_REQUIRE(C && (bins || n == 0), "null argument");
        GC_REQUIRE(volume < C->vols.size(), "no such volume in this cache");
        Volume &V = C->vols[volume];
        const gc_layout &L = V.layout;
        uint64_t want = 0;
        for (uint32_t l = 0; l < L.nb_levels; ++l)
            want += static_cast<uint64_t>(L.nb_bricks[l][0]) * L.nb_bricks[l][1] * L.nb_bricks[l][2];
        GC_REQUIRE(n == 0 || n == want, "brick bins: " + std::to_string(n) + " given, the volume has " +
                                            std::to_string(want) + " bricks");
        V.bins.assign(bins, bins + n);
        C->entry_bins_dirty = true;
    });
}

int gc_brick_value_bins(const gc_volume_desc *vol, const gc_layout *layout, uint32_t level, const void *level_bricks,
                        uint64_t *bins, void *stream) {
    return guard([&] {
        GC_REQUIRE(vol && layout && level_bricks && bins, "null argument");
        GC_REQUIRE(level < layout->nb_levels, "no such level");
        const uint32_t *nb = layout->nb_bricks[level];
        const uint64_t n = static_cast<uint64_t>(nb[0]) * nb[1] * nb[2];
        cudaStream_t s = as_stream(stream);
        if (vol->channels != 1) {  // the install never skips a multi-channel brick
            GC_CUDA(cudaMemsetAsync(bins, 0xff, n * sizeof(uint64_t), s));
            return;
        }
        GC_REQUIRE(vol->encoded_bytes == 1 || vol->encoded_bytes == 2 || vol->encoded_bytes == 4,
                   "voxel width must be 1, 2 or 4 bytes");
        launch_brick_bins(static_cast<const uint8_t *>(level_bricks), nb, layout->nb_big_bricks[level],
                          vol->big_brick_size, vol->brick_size, vol->encoded_bytes,
                          reinterpret_cast<unsigned long long *>(bins), s);
    });
}

int gc_cache_set_source_host(gc_cache_t C, const void *bricks, uint64_t bytes, const uint64_t *level_offsets,
                             const uint64_t *empty_keys, size_t n_empty) {
    return gc_cache_set_volume_source_host(C, 0, bricks, bytes, level_offsets, empty_keys, n_empty);
}

int gc_cache_set_source_callback(gc_cache_t C, gc_brick_loader_fn fn, void *user, const uint64_t *empty_keys,
                                 size_t n_empty) {
    return gc_cache_set_volume_source_callback(C, 0, fn, user, empty_keys, n_empty);
}

int gc_cache_update(gc_cache_t C, void *stream, int *converged) {
    return guard([&] {
        GC_REQUIRE(C, "null cache");
        GC_REQUIRE(has_source(C), "no brick source set");
        const bool r = update(C, as_stream(stream));
        if (converged) *converged = r ? 1 : 0;
    });
}

int gc_cache_completude(gc_cache_t C, void *stream, float *fraction) {
    return guard([&] {
        GC_REQUIRE(C && fraction, "null argument");
        GC_CUDA(cudaSetDevice(C->device));
        cudaStream_t s = as_stream(stream);
        launch_completude(C->slot_vpos, C->nslots, C->d_misc, s);
        GC_CUDA(cudaMemcpyAsync(C->h_misc, C->d_misc, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        GC_CUDA(cudaStreamSynchronize(s));
        *fraction = static_cast<float>(*C->h_misc) / static_cast<float>(C->nslots);
    });
}

int gc_cache_volume_levels(gc_cache_t C, uint32_t volume, uint32_t *level_base, uint32_t *n_levels) {
    return guard([&] {
        GC_REQUIRE(C && level_base && n_levels, "null argument");
        GC_REQUIRE(volume < C->vols.size(), "no such volume in this cache");
        *level_base = C->vols[volume].level_base;
        *n_levels = C->vols[volume].layout.nb_levels;
    });
}

int gc_cache_device_view_get(gc_cache_t C, uint32_t volume, gc_cache_device_view *out) {
    return guard([&] {
        GC_REQUIRE(C && out, "null argument");
        GC_REQUIRE(volume < C->vols.size(), "no such volume in this cache");
        const gc::Volume &v = C->vols[volume];
        GC_REQUIRE(v.desc.channels == 1, "the device view samples one-channel volumes");
        std::memset(out, 0, sizeof(*out));
        out->mrpd = reinterpret_cast<const uint32_t *>(C->mrpd);
        out->requests = C->req;
        out->usage = C->usage;
        out->pool = C->pool;
        out->slot_bytes = C->slot_bytes;
        out->mrpd_dims[0] = C->mx;
        out->mrpd_dims[1] = C->my;
        out->mrpd_dims[2] = C->mz;
        out->pool_slots[0] = C->d.cache_size[0];
        out->pool_slots[1] = C->d.cache_size[1];
        out->pool_slots[2] = C->d.cache_size[2];
        out->brick_size = C->B;
        out->covering = C->c;
        out->voxel_bytes = v.desc.encoded_bytes;
        out->timestamp = C->ts;
        out->n_levels = v.layout.nb_levels;
        for (uint32_t l = 0; l < v.layout.nb_levels; ++l) {
            const uint32_t cl = v.level_base + l;
            out->level_offset[l] = C->lt.off[cl];
            for (int a = 0; a < 3; ++a) {
                out->level_bricks[l][a] = C->lt.nb[cl][a];
                out->level_voxels[l][a] = C->lt.vvox[cl][a];
                out->level_initial_over_real[l][a] = C->lt.ior[cl][a];
            }
            out->pt_level_offset[l] = C->lt.pt_off[cl];
        }
        out->pt_top = C->pt.top;
        out->pt_pool = reinterpret_cast<const uint32_t *>(C->pt.table);
        out->pt_usage = C->pt.usage;
        out->pt_shift = C->pt.shift;
        for (int a = 0; a < 3; ++a) out->pt_dims[a] = C->pt_dims[a];
    });
}

int gc_cache_timestamp(gc_cache_t C, uint32_t *ts) {
    return guard([&] {
        GC_REQUIRE(C && ts, "null argument");
        *ts = C->ts;
    });
}

int gc_cache_info_get(gc_cache_t C, gc_cache_info *out) {
    return guard([&] {
        GC_REQUIRE(C && out, "null argument");
        std::memset(out, 0, sizeof(*out));
        out->mrpd_dims[0] = C->mx;
        out->mrpd_dims[1] = C->my;
        out->mrpd_dims[2] = C->mz;
        out->nb_slots = C->nslots;
        out->slot_voxels = C->B * C->B * C->B;
        // the first GC_MAX_LEVELS cache levels (a shared cache: gc_cache_volume_levels)
        for (uint32_t l = 0; l < std::min<uint32_t>(C->lt.nlevels, GC_MAX_LEVELS); ++l)
            out->level_offset[l] = C->lt.off[l];
        out->pool_bytes = static_cast<uint64_t>(C->nslots) * C->slot_bytes;
        out->pt_block = C->d.pt_block;
        out->pt_slots = C->pt_slots;
        for (int a = 0; a < 3; ++a) out->pt_dims[a] = C->pt_dims[a];
        for (uint32_t l = 0; l < std::min<uint32_t>(C->lt.nlevels, GC_MAX_LEVELS); ++l)
            out->pt_level_offset[l] = C->lt.pt_off[l];
    });
}

int gc_cache_stats_get(gc_cache_t C, gc_cache_stats *out) {
    return guard([&] {
        GC_REQUIRE(C && out, "null argument");
        GC_CUDA(cudaSetDevice(C->device));
        ScanCtl a, b;
        GC_CUDA(cudaMemcpy(&a, C->ctl_lru, sizeof(a), cudaMemcpyDeviceToHost));
        GC_CUDA(cudaMemcpy(&b, C->ctl_miss, sizeof(b), cudaMemcpyDeviceToHost));
        std::lock_guard<std::mutex> g(C->mu);
        uint32_t used = 0;
        GC_CUDA(cudaMemcpy(&used, C->d_count, sizeof(used), cudaMemcpyDeviceToHost));
        unsigned long long counts[2] = {0, 0};
        GC_CUDA(cudaMemcpy(counts, C->d_samples, sizeof(counts), cudaMemcpyDeviceToHost));
        *out = C->stats;
        out->device_error = a.err | b.err;
        out->upload_direct = C->gather ? 1u : 0u;
        out->samples = counts[0];
        out->rays_marched = counts[1];
        out->last_used = used;
    });
}

int gc_cache_dump(gc_cache_t C, int what, void *dst, size_t bytes) {
    return guard([&] {
        GC_REQUIRE(C && dst, "null argument");
        GC_CUDA(cudaSetDevice(C->device));
        GC_CUDA(cudaDeviceSynchronize());
        switch (what) {
            case GC_DUMP_MRPD:
                GC_REQUIRE(bytes == C->nentries * sizeof(uint4), "wrong size for the page directory");
                if (C->pt.shift) {
                    uint4 *flat = dalloc<uint4>(C->nentries, "flattened page directory");
                    launch_pt_flatten(C->pt, C->lt, C->mx, C->my, C->nentries, flat, nullptr);
                    const cudaError_t e = cudaMemcpy(dst, flat, bytes, cudaMemcpyDeviceToHost);
                    cudaFree(flat);
                    GC_CUDA(e);
                } else {
                    GC_CUDA(cudaMemcpy(dst, C->mrpd, bytes, cudaMemcpyDeviceToHost));
                }
                break;
            case GC_DUMP_PT_TOP:
            case GC_DUMP_PT_POOL:
            case GC_DUMP_PT_LRU:
            case GC_DUMP_PT_USAGE:
            case GC_DUMP_PT_KEYS: {
                GC_REQUIRE(C->pt.shift, "the cache has a one-level page directory");
                const void *src = C->pt.top;
                size_t want = C->pt_words * sizeof(uint32_t);
                if (what == GC_DUMP_PT_POOL) {
                    src = C->pt.table;
                    want = (static_cast<size_t>(C->pt_slots) << (3 * C->pt.shift)) * sizeof(uint4);
                } else if (what == GC_DUMP_PT_LRU) {
                    src = C->pt_order[C->pt_cur];
                    want = C->pt_slots * sizeof(uint32_t);
                } else if (what == GC_DUMP_PT_USAGE) {
                    src = C->pt.usage;
                    want = C->pt_slots * sizeof(uint32_t);
                } else if (what == GC_DUMP_PT_KEYS) {
                    src = C->pt_keys;
                    want = C->pt_slots * sizeof(uint4);
                }
                GC_REQUIRE(bytes == want, "wrong size for the page-table dump");
                GC_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
                break;
            }
            case GC_DUMP_REQUESTS:
                GC_REQUIRE(bytes == C->nentries * sizeof(uint32_t), "wrong size for the request buffer");
                GC_CUDA(cudaMemcpy(dst, C->req, bytes, cudaMemcpyDeviceToHost));
                break;
            case GC_DUMP_USAGE:
                GC_REQUIRE(bytes == C->nslots * sizeof(uint32_t), "wrong size for the usage buffer");
                GC_CUDA(cudaMemcpy(dst, C->usage, bytes, cudaMemcpyDeviceToHost));
                break;
            case GC_DUMP_POOL:
                GC_REQUIRE(bytes == C->nslots * C->slot_bytes, "wrong size for the pool");
                GC_CUDA(cudaMemcpy(dst, C->pool, bytes, cudaMemcpyDeviceToHost));
                break;
            case GC_DUMP_LRU: {
                GC_REQUIRE(bytes == C->nslots * sizeof(LruRecord), "wrong size for the LRU");
                std::vector<uint32_t> order(C->nslots), level(C->nslots);
                std::vector<float4> vpos(C->nslots);
                GC_CUDA(cudaMemcpy(order.data(), C->order[C->cur], C->nslots * 4, cudaMemcpyDeviceToHost));
                GC_CUDA(cudaMemcpy(level.data(), C->slot_level, C->nslots * 4, cudaMemcpyDeviceToHost));
                GC_CUDA(cudaMemcpy(vpos.data(), C->slot_vpos, C->nslots * 16, cudaMemcpyDeviceToHost));
                LruRecord *r = static_cast<LruRecord *>(dst);
                const uint32_t sx = C->d.cache_size[0], sy = C->d.cache_size[1];
                for (uint32_t i = 0; i < C->nslots; ++i) {
                    const uint32_t s = order[i];
                    r[i].cx = (s % sx) * C->B;
                    r[i].cy = ((s / sx) % sy) * C->B;
                    r[i].cz = (s / (sx * sy)) * C->B;
                    r[i].level = level[s];
                    r[i].vx = vpos[s].x;
                    r[i].vy = vpos[s].y;
                    r[i].vz = vpos[s].z;
                }
                break;
            }
            default: fail(GC_ERR_INVALID, "unknown dump selector");
        }
    });
}

int gc_cache_last_misses(gc_cache_t C, uint32_t *out4, uint32_t max, uint32_t *count, uint32_t *total) {
    return guard([&] {
        GC_REQUIRE(C && out4 && count && total, "null argument");
        GC_CUDA(cudaSetDevice(C->device));
        {
            std::unique_lock<std::mutex> lk(C->mu);
            C->cv.wait(lk, [&] { return !C->busy; });
        }
        const auto &L = C->lists[C->cur_load];
        GC_CUDA(cudaEventSynchronize(L.ev));
        const uint32_t n = std::min(std::min(*L.total, C->d.max_requests), max);
        std::memcpy(out4, L.h, static_cast<size_t>(n) * sizeof(uint4));
        *count = n;
        *total = *L.total;
    });
}

int gc_cache_load_buffer(gc_cache_t C, int what, const void *src, size_t bytes) {
    return guard([&] {
        GC_REQUIRE(C && src, "null argument");
        GC_CUDA(cudaSetDevice(C->device));
        GC_CUDA(cudaDeviceSynchronize());
        if (what == GC_DUMP_USAGE) {
            GC_REQUIRE(bytes == C->nslots * sizeof(uint32_t), "wrong size for the usage buffer");
            GC_CUDA(cudaMemcpy(C->usage, src, bytes, cudaMemcpyHostToDevice));
        } else if (what == GC_DUMP_REQUESTS) {
            GC_REQUIRE(bytes == C->nentries * sizeof(uint32_t), "wrong size for the request buffer");
            GC_CUDA(cudaMemcpy(C->req, src, bytes, cudaMemcpyHostToDevice));
        } else {
            fail(GC_ERR_INVALID, "only the usage and request buffers can be loaded");
        }
    });
}

int gc_render(gc_cache_t C, const gc_view *view, void *stream) {
    return guard([&] {
        GC_REQUIRE(C && view, "null argument");
        render(C, view, 1, as_stream(stream));
    });
}

int gc_render_batch(gc_cache_t C, const gc_view *views, uint32_t n, void *stream) {
    return guard([&] {
        GC_REQUIRE(C && views, "null argument");
        render(C, views, n, as_stream(stream));
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Continuous batching (gc_batch_*).
#include <chrono>
#include <deque>

namespace gc {

// The batched tick runs the cache steps in the order install -> render ->
// LRU update -> scan, so that one tick carries a whole request cycle: the
// scan sees the requests of a render that already used the bricks installed
// at the start of the same tick.  (The plain frame loop keeps the reference's
// update(), where install and scan fall in different frames.)

// Installs what the loader finished.  Returns true when bricks were installed.
static bool batch_install(gc_cache *C, cudaStream_t s) {
    if (C->sync_mode()) {
        if (!C->done) return false;
        const bool any = C->pend_n > 0;
        install(C, s);
        C->done = false;
        return any;
    }
    std::unique_lock<std::mutex> lk(C->mu);
    if (!C->loader_error.empty()) {
        std::string e = C->loader_error;
        C->loader_error.clear();
        fail(GC_ERR_IO, "brick loader: " + e);
    }
    if (C->busy || !C->done) return false;
    lk.unlock();
    const bool any = C->pend_n > 0;
    install(C, s);
    lk.lock();
    C->done = false;
    return any;
}

// True when no load is in flight and none waits for its install.
static bool loader_idle(gc_cache *C) {
    if (C->sync_mode()) return !C->done;
    std::lock_guard<std::mutex> g(C->mu);
    return !C->busy && !C->done;
}

// End of a rendered tick: LRU update and, with the loader idle, the scan.
// Returns true when a scan was issued (its miss count lands in h_total).
static bool batch_update(gc_cache *C, cudaStream_t s) {
    lru_update(C, s);
    bool scanned = false;
    if (C->sync_mode()) {
        if (!C->done) {
            scan_requests(C, s);
            C->cur_load = 0;  // the loader serves list 0 (an overlapped batch may have left 1)
            C->done = serve_request(C);
            scanned = true;
        }
    } else {
        std::unique_lock<std::mutex> lk(C->mu);
        if (!C->busy && !C->done) {
            lk.unlock();
            scan_requests(C, s);
            C->cur_load = 0;  // the loader serves list 0 (an overlapped batch may have left 1)
            lk.lock();
            C->busy = true;
            C->has_request = true;
            C->cv.notify_all();
            scanned = true;
        }
    }
    C->ts++;
    C->stats.frames++;
    return scanned;
}

// Waits (bounded) for the asynchronous loader to finish its load.
static void wait_loader(gc_cache *C, int ms) {
    if (C->sync_mode()) return;
    std::unique_lock<std::mutex> lk(C->mu);
    C->cv.wait_for(lk, std::chrono::milliseconds(ms), [&] { return !C->busy; });
}

}  // namespace gc

struct gc_batch {
    gc_cache *cache = nullptr;
    gc_batch_desc d;
    struct Item {
        gc_view view;
        uint64_t tag;
        uint32_t passes;
        uint64_t epoch;  // install count at the view's last pass (kNever before the first)
        uint32_t skipped;  // times a later view was admitted before it
        std::chrono::steady_clock::time_point submitted;
        bool started;      // progressive buffers cleared (first admission)
        uint64_t seq;      // admission sequence number (the newest is parked first)
        uint64_t wait;     // overlapped loads: serial of the load the view waits for (0: none)
    };
    uint64_t admissions = 0;
    float last_cam[3] = {0.f, 0.f, 0.f};  // camera of the last admitted view
    uint32_t last_volume = 0;             // and its volume
    bool have_cam = false;
    static constexpr uint64_t kNever = ~0ull;
    uint64_t installs = 0;  // ticks that installed bricks
    std::deque<Item> queue;
    std::vector<Item> active;
    std::deque<gc_batch_result> done;
    uint32_t *d_status = nullptr;
    uint32_t *h_status = nullptr;   // [max_views] status words + [1] used slots
    uint32_t last_used = 0;         // slots stamped by the last pass over all active views
    uint32_t last_misses = 0;       // missing bricks requested by the last scan (uncapped)
    cudaEvent_t ev = nullptr, ev_r0 = nullptr, ev_r1 = nullptr;
    gc_batch_stats st;
    gc::RenderGraph graph;                // the replayed launch
    gc::ViewParams *h_views = nullptr;    // pinned view table the graph copies
    // Overlapped loads: each miss list is a load with a serial number; a view
    // waits for the load its requests went into.  List slot state: 0 free,
    // 1 scanned and waiting for the loader, 2 with the loader.
    int slot_state[2] = {0, 0};
    uint64_t slot_serial[2] = {0, 0};
    uint64_t next_serial = 1;
    std::unordered_set<uint64_t> completed;  // loads installed (or empty)
    uint32_t used_prev = 0;                   // slots used by the previous render (the other cohort)
    bool split_back = false;                  // the next cohort split renders the back half first
    cudaStream_t stream = nullptr;            // stream of the last overlapped tick
};

namespace gc {
// Overlapped loads leave in-flight marks in the page directory until their
// install; a batch that ends first waits for the loader, installs what it
// finished and clears the marks of every list it still holds, so that the
// cache serves later frames as if the batch had run to the end.
static void batch_drain_loads(gc_batch *b) {
    gc_cache *C = b->cache;
    if (!b->d.overlap_loads || (b->slot_state[0] == 0 && b->slot_state[1] == 0)) return;
    cudaSetDevice(C->device);
    cudaStream_t s = b->stream;
    bool installable = false;
    {
        std::unique_lock<std::mutex> lk(C->mu);
        C->cv.wait(lk, [&] { return !C->busy; });  // the loader's load is finite
        installable = C->done && b->slot_state[C->cur_load] == 2;
        C->done = false;
        C->loader_error.clear();
    }
    if (installable) install(C, s);
    for (int k = 0; k < 2; ++k) {
        if (b->slot_state[k] == 0) continue;
        const gc_cache::MissList &L = C->lists[k];
        launch_unmark_in_flight(L.d, std::min(*L.total, C->d.max_requests), C->lt, C->mx, C->my, C->nentries,
                                C->mrpd, s);
        b->slot_state[k] = 0;
    }
    C->cur_load = 0;
    cudaStreamSynchronize(s);
}

static void batch_destroy(gc_batch *b) {
    if (!b) return;
    try {
        batch_drain_loads(b);
    } catch (const std::exception &) {
    }
    if (b->d_status) cudaFree(b->d_status);
    if (b->h_status) cudaFreeHost(b->h_status);
    if (b->h_views) cudaFreeHost(b->h_views);
    if (b->ev) cudaEventDestroy(b->ev);
    if (b->ev_r0) cudaEventDestroy(b->ev_r0);
    if (b->ev_r1) cudaEventDestroy(b->ev_r1);
    delete b;
}
}  // namespace gc

namespace gc {
// Admission: queued views in arrival order (or, with a reorder window, the one
// whose camera is nearest the last admitted view's) while the budgets allow;
// at least one view is active.  By cache memory: the active views' demand --
// slots used plus missing bricks found -- must stay within max_occupancy of
// the pool slots.  `all`: admission is open this tick.
static void batch_admit(gc_batch *b, gc_cache *C, cudaStream_t s, bool all, double demand) {
    uint64_t pixels = 0;
    for (auto &it : b->active) pixels += static_cast<uint64_t>(it.view.width) * it.view.height;
    const bool occ_ok =
        b->d.max_occupancy <= 0.f || demand <= b->d.max_occupancy * static_cast<double>(C->nslots);
    uint32_t admitted = 0;
    auto cam_dist = [&](const gc_view &v) {  // camera = translation column of the view matrix
        const float dx = v.inv_view[3] - b->last_cam[0], dy = v.inv_view[7] - b->last_cam[1],
                    dz = v.inv_view[11] - b->last_cam[2];
        // views of another volume share no bricks: farther than any camera
        return dx * dx + dy * dy + dz * dz + (v.volume != b->last_volume ? 1e30f : 0.f);
    };
    while (!b->queue.empty() && b->active.size() < b->d.max_views) {
        size_t pick = 0;
        if (b->d.reorder_window > 1 && b->have_cam && b->queue.front().skipped < b->d.reorder_window) {
            const size_t w = std::min<size_t>(b->queue.size(), b->d.reorder_window);
            float best = cam_dist(b->queue[0].view);
            for (size_t k = 1; k < w; ++k) {
                const float d = cam_dist(b->queue[k].view);
                if (d < best) {
                    best = d;
                    pick = k;
                }
            }
        }
        const gc_view &v = b->queue[pick].view;
        const uint64_t px = static_cast<uint64_t>(v.width) * v.height;
        if (!b->active.empty() && (!all || pixels + px > b->d.max_pixels || !occ_ok ||
                                   (b->d.max_admit && admitted >= b->d.max_admit)))
            break;
        ++admitted;
        if (!b->queue[pick].started) {  // a parked view resumes with its progress
            GC_CUDA(cudaMemsetAsync(v.tbuf, 0, px * sizeof(float), s));
            GC_CUDA(cudaMemsetAsync(v.state, 0, px * 4 * sizeof(float), s));
            b->queue[pick].started = true;
        }
        b->queue[pick].seq = b->admissions++;
        pixels += px;
        b->last_cam[0] = v.inv_view[3];
        b->last_cam[1] = v.inv_view[7];
        b->last_cam[2] = v.inv_view[11];
        b->last_volume = v.volume;
        b->have_cam = true;
        if (pick) b->queue.front().skipped++;
        b->active.push_back(b->queue[pick]);
        b->queue.erase(b->queue.begin() + static_cast<std::ptrdiff_t>(pick));
    }
}

// The overlapped tick (gc_batch_desc.overlap_loads; asynchronous loader).
// Loads complete in order.  A tick: finish the load the loader completed
// (install, clear its leftover in-flight marks, free its list), hand a waiting
// list to an idle loader, admit, render the views whose awaited load has
// completed, and -- when a list is free -- scan their requests into it with
// in-flight marks.  The loader then uploads one cohort's bricks while the
// other cohort renders.
static void batch_tick_overlapped(gc_batch *b, gc_cache *C, cudaStream_t s, uint32_t *n_active,
                                  uint32_t *n_queued) {
    b->stream = s;
    auto hand_to_loader = [&] {  // the oldest waiting list, if the loader is idle
        std::unique_lock<std::mutex> lk(C->mu);
        if (C->busy || C->done) return;
        int pick = -1;
        for (int k = 0; k < 2; ++k)
            if (b->slot_state[k] == 1 && (pick < 0 || b->slot_serial[k] < b->slot_serial[pick])) pick = k;
        if (pick < 0) return;
        // the loader waits on this event: it covers the scan of the list and
        // the install just enqueued, which reads the staging buffers that
        // the load refills
        GC_CUDA(cudaEventRecord(C->lists[pick].ev, s));
        C->cur_load = pick;
        b->slot_state[pick] = 2;
        C->busy = true;
        C->has_request = true;
        C->cv.notify_all();
    };
    {  // 1. the load the loader finished
        std::unique_lock<std::mutex> lk(C->mu);
        if (!C->loader_error.empty()) {
            std::string e = C->loader_error;
            C->loader_error.clear();
            fail(GC_ERR_IO, "brick loader: " + e);
        }
        const int k = C->cur_load;
        if (!C->busy && b->slot_state[k] == 2) {
            const bool installable = C->done;
            lk.unlock();
            if (installable) {
                install(C, s);
                b->installs++;
                b->st.install_ticks++;
            }
            const gc_cache::MissList &L = C->lists[k];
            launch_unmark_in_flight(L.d, std::min(*L.total, C->d.max_requests), C->lt, C->mx, C->my, C->nentries,
                                    C->mrpd, s);
            lk.lock();
            C->done = false;
            b->slot_state[k] = 0;
            b->completed.insert(b->slot_serial[k]);
        }
    }
    hand_to_loader();
    int free_slot = b->slot_state[0] == 0 ? 0 : (b->slot_state[1] == 0 ? 1 : -1);
    // 2. admission while a list is free (a new view's first pass feeds a scan)
    batch_admit(b, C, s, free_slot >= 0,
                static_cast<double>(b->last_used) + b->used_prev + static_cast<double>(b->last_misses));
    const uint32_t na = static_cast<uint32_t>(b->active.size());
    if (n_active) *n_active = na;
    if (n_queued) *n_queued = static_cast<uint32_t>(b->queue.size());
    // 3. views whose awaited load completed (or never rendered)
    std::vector<uint32_t> sel;
    if (free_slot >= 0)
        for (uint32_t i = 0; i < na; ++i)
            if (b->active[i].wait == 0 || b->completed.count(b->active[i].wait)) sel.push_back(i);
    // With no load in flight or waiting, the ready views are split into two
    // cohorts of about equal pixels: one renders now and its bricks load
    // while the other renders in the next tick, and from then on each cohort
    // renders while the other's bricks load.  The half that goes first
    // alternates between splits, so that a front half whose pass started no
    // load cannot hold the back half back split after split.
    if (sel.size() >= 2 && b->slot_state[0] == 0 && b->slot_state[1] == 0) {
        uint64_t total = 0, half = 0;
        for (uint32_t i : sel) total += static_cast<uint64_t>(b->active[i].view.width) * b->active[i].view.height;
        size_t k = 0;
        while (k < sel.size() - 1 && 2 * half < total) {
            half += static_cast<uint64_t>(b->active[sel[k]].view.width) * b->active[sel[k]].view.height;
            ++k;
        }
        k = std::max<size_t>(k, 1);
        if (b->split_back)
            sel.erase(sel.begin(), sel.begin() + static_cast<std::ptrdiff_t>(k));
        else
            sel.resize(k);
        b->split_back = !b->split_back;
    }
    if (sel.empty()) {
        if (na) {
            const auto t0 = std::chrono::steady_clock::now();
            wait_loader(C, 5);
            b->st.wait_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        }
        return;
    }
    const uint32_t n = static_cast<uint32_t>(sel.size());
    std::vector<gc_view> views(n);
    for (uint32_t k = 0; k < n; ++k) {
        views[k] = b->active[sel[k]].view;
        views[k].status = b->d_status + k;
    }
    GC_CUDA(cudaMemsetAsync(b->d_status, 0, n * sizeof(uint32_t), s));
    GC_CUDA(cudaEventRecord(b->ev_r0, s));
    render(C, views.data(), n, s, true, &b->graph, b->h_views);
    GC_CUDA(cudaEventRecord(b->ev_r1, s));
    GC_CUDA(cudaMemcpyAsync(b->h_status, b->d_status, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    lru_update(C, s);
    GC_CUDA(cudaMemcpyAsync(b->h_status + b->d.max_views, C->d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    // 4. their requests into the free list, marked in flight
    scan_requests(C, s, free_slot, true);
    const uint64_t serial = b->next_serial++;
    b->slot_state[free_slot] = 1;
    b->slot_serial[free_slot] = serial;
    C->ts++;
    C->stats.frames++;
    GC_CUDA(cudaEventRecord(b->ev, s));
    GC_CUDA(cudaEventSynchronize(b->ev));
    b->used_prev = b->last_used;
    b->last_used = b->h_status[b->d.max_views];
    const uint32_t misses = *C->lists[free_slot].total;  // copied on this stream before the event
    b->last_misses = misses;
    uint64_t wait = serial;
    if (misses == 0) {  // nothing to load: the list is done; wait for the newest load still out
        b->slot_state[free_slot] = 0;
        b->completed.insert(serial);
        wait = 0;
        for (int k = 0; k < 2; ++k)
            if (b->slot_state[k] != 0) wait = std::max(wait, b->slot_serial[k]);
    }
    hand_to_loader();
    float rms = 0.f;
    GC_CUDA(cudaEventElapsedTime(&rms, b->ev_r0, b->ev_r1));
    b->st.render_ms += rms;
    b->st.render_ticks++;
    b->st.view_passes += n;
    // 5. retire converged views; the others wait for this tick's load
    const auto now = std::chrono::steady_clock::now();
    std::vector<char> gone(na, 0);
    for (uint32_t k = 0; k < n; ++k) {
        auto &it = b->active[sel[k]];
        it.passes++;
        it.wait = wait;
        const bool conv = (b->h_status[k] & 1u) == 0;
        if (conv || (b->d.max_passes && it.passes >= b->d.max_passes)) {
            gc_batch_result r;
            r.tag = it.tag;
            r.passes = it.passes;
            r.converged = conv ? 1u : 0u;
            r.latency_ms = std::chrono::duration<double, std::milli>(now - it.submitted).count();
            b->done.push_back(r);
            gone[sel[k]] = 1;
        }
    }
    std::vector<gc_batch::Item> keep;
    keep.reserve(na);
    for (uint32_t i = 0; i < na; ++i)
        if (!gone[i]) keep.push_back(b->active[i]);
    b->active.swap(keep);
}

}  // namespace gc

extern "C" {

int gc_batch_create(gc_cache_t C, const gc_batch_desc *desc, gc_batch_t *out) {
    gc_batch *b = nullptr;
    int rc = guard([&] {
        GC_REQUIRE(C && desc && out, "null argument");
        GC_REQUIRE(desc->max_views >= 1 && desc->max_views <= C->max_views, "max_views must be in [1, 256]");
        GC_REQUIRE(desc->max_pixels >= 1, "max_pixels must be >= 1");
        GC_REQUIRE(!desc->overlap_loads || !C->sync_mode(), "overlapped loads need the asynchronous loader");
        GC_REQUIRE(!desc->overlap_loads || !C->pt.shift, "overlapped loads need the one-level page directory");
        GC_REQUIRE(!desc->overlap_loads || !(desc->park_above > 0.f), "parking is not available with overlapped loads");
        GC_CUDA(cudaSetDevice(C->device));
        b = new gc_batch();
        b->cache = C;
        b->d = *desc;
        b->d_status = dalloc<uint32_t>(desc->max_views, "batch status");
        b->h_status = halloc<uint32_t>(desc->max_views + 1);
        b->h_views = halloc<ViewParams>(desc->max_views);
        GC_CUDA(cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming));
        GC_CUDA(cudaEventCreate(&b->ev_r0));
        GC_CUDA(cudaEventCreate(&b->ev_r1));
        std::memset(&b->st, 0, sizeof(b->st));
        *out = b;
    });
    if (rc != GC_OK) batch_destroy(b);
    return rc;
}

int gc_batch_destroy(gc_batch_t b) {
    batch_destroy(b);
    return GC_OK;
}

int gc_batch_submit(gc_batch_t b, const gc_view *view, uint64_t tag) {
    return guard([&] {
        GC_REQUIRE(b && view, "null argument");
        ViewParams check;
        fill_view(b->cache, *view, check);  // validates the view now, not at admission
        b->queue.push_back({*view, tag, 0, gc_batch::kNever, 0, std::chrono::steady_clock::now(), false, 0, 0});
    });
}

int gc_batch_tick(gc_batch_t b, void *stream, uint32_t *n_active, uint32_t *n_queued) {
    return guard([&] {
        GC_REQUIRE(b, "null batch");
        gc_cache *C = b->cache;
        GC_REQUIRE(has_source(C), "no brick source set");
        GC_CUDA(cudaSetDevice(C->device));
        cudaStream_t s = as_stream(stream);
        const auto t_tick = std::chrono::steady_clock::now();
        struct TickClock {  // adds the host time of this tick on every exit
            gc_batch *b;
            std::chrono::steady_clock::time_point t0;
            ~TickClock() {
                b->st.ticks++;
                b->st.tick_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            }
        } tick_clock{b, t_tick};
        if (b->d.overlap_loads) {
            batch_tick_overlapped(b, C, s, n_active, n_queued);
            return;
        }
        if (batch_install(C, s)) {
            b->installs++;
            b->st.install_ticks++;
        }
        // Every active view is rendered when bricks were just installed or the
        // loader is idle; only then are views admitted, so that a new view's
        // first pass feeds the scan that ends the tick.
        const bool all = loader_idle(C);
        batch_admit(b, C, s, all, static_cast<double>(b->last_used) + static_cast<double>(b->last_misses));
        const uint32_t na = static_cast<uint32_t>(b->active.size());
        if (n_active) *n_active = na;
        if (n_queued) *n_queued = static_cast<uint32_t>(b->queue.size());
        // Views that can progress: never rendered, or bricks were installed
        // since their last pass.
        std::vector<uint32_t> sel;
        sel.reserve(na);
        for (uint32_t i = 0; i < na; ++i)
            if (all || b->active[i].epoch != b->installs) sel.push_back(i);
        if (sel.empty()) {
            if (na) {
                const auto t0 = std::chrono::steady_clock::now();
                wait_loader(C, 5);
                b->st.wait_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            }
            return;
        }
        const uint32_t n = static_cast<uint32_t>(sel.size());
        std::vector<gc_view> views(n);
        for (uint32_t k = 0; k < n; ++k) {
            views[k] = b->active[sel[k]].view;
            views[k].status = b->d_status + k;
        }
        GC_CUDA(cudaMemsetAsync(b->d_status, 0, n * sizeof(uint32_t), s));
        GC_CUDA(cudaEventRecord(b->ev_r0, s));
        render(C, views.data(), n, s, true, &b->graph, b->h_views);
        GC_CUDA(cudaEventRecord(b->ev_r1, s));
        GC_CUDA(cudaMemcpyAsync(b->h_status, b->d_status, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        const bool scanned = batch_update(C, s);
        GC_CUDA(cudaMemcpyAsync(b->h_status + b->d.max_views, C->d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                s));
        GC_CUDA(cudaEventRecord(b->ev, s));
        GC_CUDA(cudaEventSynchronize(b->ev));
        if (all) b->last_used = b->h_status[b->d.max_views];
        float rms = 0.f;
        GC_CUDA(cudaEventElapsedTime(&rms, b->ev_r0, b->ev_r1));
        b->st.render_ms += rms;
        b->st.render_ticks++;
        b->st.view_passes += n;
        if (scanned) b->last_misses = *C->lists[0].total;  // copied on this stream before the event
        const auto now = std::chrono::steady_clock::now();
        std::vector<char> gone(na, 0);
        for (uint32_t k = 0; k < n; ++k) {
            auto &it = b->active[sel[k]];
            it.passes++;
            it.epoch = b->installs;
            const bool conv = (b->h_status[k] & 1u) == 0;
            if (conv || (b->d.max_passes && it.passes >= b->d.max_passes)) {
                gc_batch_result r;
                r.tag = it.tag;
                r.passes = it.passes;
                r.converged = conv ? 1u : 0u;
                r.latency_ms = std::chrono::duration<double, std::milli>(now - it.submitted).count();
                b->done.push_back(r);
                gone[sel[k]] = 1;
            }
        }
        std::vector<gc_batch::Item> keep;
        keep.reserve(na);
        for (uint32_t i = 0; i < na; ++i)
            if (!gone[i]) keep.push_back(b->active[i]);
        b->active.swap(keep);
        // Memory-pressure parking: the working sets of the active views do not
        // fit the pool -- the newest view leaves for the queue's front (its
        // buffers keep its progress) so that the others stop evicting each
        // other's bricks.
        const double demand_now = static_cast<double>(b->last_used) + static_cast<double>(b->last_misses);
        if (all && b->d.park_above > 0.f && b->active.size() > 1 &&
            demand_now > b->d.park_above * static_cast<double>(C->nslots)) {
            size_t newest = 0;
            for (size_t i = 1; i < b->active.size(); ++i)
                if (b->active[i].seq > b->active[newest].seq) newest = i;
            gc_batch::Item it = b->active[newest];
            it.epoch = gc_batch::kNever;  // render it when it resumes
            b->active.erase(b->active.begin() + static_cast<std::ptrdiff_t>(newest));
            b->queue.push_front(it);
            b->st.parked++;
        }
    });
}

int gc_batch_stats_get(gc_batch_t b, gc_batch_stats *out) {
    return guard([&] {
        GC_REQUIRE(b && out, "null argument");
        *out = b->st;
        out->graph_replays = b->graph.replays;
    });
}

int gc_batch_poll(gc_batch_t b, gc_batch_result *out, uint32_t max, uint32_t *n) {
    return guard([&] {
        GC_REQUIRE(b && n && (out || max == 0), "null argument");
        uint32_t k = 0;
        while (k < max && !b->done.empty()) {
            out[k++] = b->done.front();
            b->done.pop_front();
        }
        *n = k;
    });
}

}  // extern "C"
