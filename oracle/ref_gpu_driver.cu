// Headless driver around the reference's own GPU code (TEST INFRASTRUCTURE
// ONLY).  oracle/build.py compiles it, together with a staged copy of the
// reference's sources, into oracle/_ref/librefgpu.so; tests/ and the CPU
// baseline legs of bench.py load it through oracle/refgpu.py to pin the CUDA
// path against the reference's own implementation on the same inputs.
//
// What runs here is the reference, unchanged:
//   - Mipmapper::process (GcCore/src/cuda/libPreprocessor/Mipmapper.cu:401-525),
//     process_bricking (GcCore/src/libPreprocessor/Bricker_v2.cpp:79-252) and
//     BrickProcessor::process_empty (GcCore/include/GcCore/cuda/libPreprocessor/
//     BrickProcessor.hpp:91-162), in the order of Application::pre_process
//     (Applications/DVR-ray-caster/src/Application.cu:148-197);
//   - CacheManager<T> with its RequestHandler and BricksManager
//     (GcCore/include/GcCore/cuda/libGPUCache/CacheManager.hpp:135-670,
//     RequestHandler.hpp:29-372), loading the brick files process_bricking wrote;
//   - RayCastDVR / RayCastMOP (Applications/DVR-ray-caster/src/RayCasters.cu),
//     launched like get_frame (Applications/DVR-ray-caster/src/VolumeRayCaster.cu:356-429).
// What the driver adds (the display application's parts, restated because
// they live in files that need SDL/OpenGL): the LOD tables of
// display_volume_raycaster (VolumeRayCaster.cu:136-175), the application's
// bricking threads (Application.cu:227-285), the configuration steps of
// Application::init (Application.cu:23-40), device buffers in place of the
// OpenGL pixel buffer, a wait for the request handler after each update (the
// reference lets it run concurrently; waiting makes the request/install
// alternation deterministic), and reads of the cache state for comparison.
//
// C ABI: every call returns 0 on success, nonzero with refgpu_last_error() set.
#include <RayCasters.cu>

// BrickProcessor.hpp uses Configuration without including it (the
// application includes it first, Application.cu:7-16), hence this order.
#include <GcCore/libData/Configuration.hpp>
#include <GcCore/libData/ConfigurationPolicies.hpp>
#include <GcCore/libData/MetaData.hpp>
#include <GcCore/libData/VolumeConfiguration.hpp>
#include <GcCore/cuda/libGPUCache/CacheManager.hpp>
#include <GcCore/cuda/libPreprocessor/BrickProcessor.hpp>
#include <GcCore/cuda/libPreprocessor/BrickProcessorPredicate.hpp>
#include <GcCore/cuda/libPreprocessor/Mipmapper.hpp>
#include <GcCore/libCommon/FileSystem.hpp>
#include <GcCore/libPreprocessor/Bricker_v2.hpp>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace {

using tdns::math::Vector3ui;

thread_local std::string g_error;

int fail(const std::string &m) {
    g_error = m;
    return 1;
}

void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

tdns::data::Configuration &conf() { return tdns::data::Configuration::get_instance(); }

uint32_t field_u32(const char *key) {
    uint32_t v = 0;
    if (!conf().get_field(key, v)) throw std::runtime_error(std::string("missing configuration field ") + key);
    return v;
}

// Access to the cache manager's state for the comparisons (its members are
// protected; the behaviour is the reference's own).
template <typename T>
struct Probe : tdns::gpucache::CacheManager<T> {
    using tdns::gpucache::CacheManager<T>::CacheManager;
    uint32_t timestamp() const { return this->_timestamp; }
    bool handler_working() const { return this->_requestHandler->is_working(); }
    tdns::gpucache::CacheDevice<T> &pool() { return *this->_dataCache; }
    tdns::gpucache::MultiResolutionPageDirectory<uint4> &mrpd() { return *this->_mrpd; }
    tdns::common::DynamicArray3dDevice<uint32_t> &requests() { return *this->_requestBuffer; }
    tdns::gpucache::RequestHandler<T> &handler() { return *this->_requestHandler; }
};

// Reads the brick pool (a cudaArray surface of sx*B x sy*B x sz*B voxels)
// through the reference's K_CacheDevice<T>::get into slot-major order: slot
// (x, y, z) -> index x + y*sx + z*sx*sy, B^3 voxels x-fastest each.  The grid
// covers exactly the array's extent (surface reads outside it trap).
template <typename T>
__global__ void read_pool_kernel(tdns::gpucache::K_CacheDevice<T> pool, T *out, uint3 ext, uint32_t B) {
    const uint64_t n = static_cast<uint64_t>(ext.x) * ext.y * ext.z;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint32_t x = static_cast<uint32_t>(i % ext.x);
        const uint32_t y = static_cast<uint32_t>((i / ext.x) % ext.y);
        const uint32_t z = static_cast<uint32_t>(i / (static_cast<uint64_t>(ext.x) * ext.y));
        const uint32_t sx = ext.x / B, sy = ext.y / B;
        const uint64_t slot = (x / B) + static_cast<uint64_t>(y / B) * sx + static_cast<uint64_t>(z / B) * sx * sy;
        const uint64_t in = (x % B) + static_cast<uint64_t>(y % B) * B + static_cast<uint64_t>(z % B) * B * B;
        out[slot * B * B * B + in] = pool.get(make_uint3(x, y, z));
    }
}

struct Session {
    virtual ~Session() = default;
    virtual void render(const float *inv_view, uint32_t w, uint32_t h, float tstep, const float *tf128, int mode,
                        uint32_t *rgba, float *tbuf, float *state) = 0;
    virtual bool update(uint32_t wait_ms) = 0;
    virtual uint32_t timestamp() = 0;
    virtual void info(uint32_t *mrpd_dims, uint32_t *cache_size, uint32_t *brick, uint32_t *eb, uint32_t *nlevels) = 0;
    virtual void dump(int what, void *dst, size_t bytes) = 0;
    virtual void asked(uint32_t *out4, uint32_t max, uint32_t *n, uint32_t *n_nonempty) = 0;
    virtual float completude() = 0;
    virtual void lod_tables(float *inv_levels, float *steps, uint32_t *n) = 0;
};

template <typename T>
struct SessionT : Session {
    tdns::data::MetaData meta;
    std::unique_ptr<Probe<T>> mgr;
    uint32_t B = 0, eb = 0;
    Vector3ui cache_size;
    uint32_t nlod = 0;
    std::vector<float3> inv_levels;
    std::vector<float> steps;
    uint3 *d_levels = nullptr;
    float3 *d_inv = nullptr, *d_lodbrick = nullptr;
    float *d_steps = nullptr;
    cudaArray *tf_array = nullptr;
    cudaTextureObject_t tf_tex = 0;

    SessionT(const std::string &cfg, const uint32_t cs[3], int gpu) {
        if (!meta.load()) throw std::runtime_error("MetaData::load failed (bricks.xml)");
        std::vector<tdns::data::VolumeConfiguration> vcs(1);
        vcs[0] = tdns::data::load_volume_configuration(cfg);
        B = field_u32("BrickSize");
        eb = field_u32("NumberEncodedBytes");
        cache_size = Vector3ui(cs[0], cs[1], cs[2]);
        // Cache configuration as Application::run builds it (Application.cu:73-101),
        // with the pool size given instead of derived from a 9.5 GB budget.
        tdns::data::CacheConfiguration cc;
        cc.CacheSize = std::vector<Vector3ui>(1, cache_size);
        cc.BlockSize = std::vector<Vector3ui>(1, Vector3ui(B));
        cc.DataCacheFlags = 1;
        mgr.reset(new Probe<T>(vcs[0], meta, cc, gpu));

        // LOD tables of display_volume_raycaster (VolumeRayCaster.cu:136-175):
        // bounding box [-1, 1]^3.
        const float bbox[3] = {2.f, 2.f, 2.f};
        const float bmin = std::min(bbox[0], std::min(bbox[1], bbox[2]));
        nlod = static_cast<uint32_t>(meta.nb_levels());
        std::vector<uint3> levels(nlod);
        std::vector<float3> lodbrick(nlod);
        inv_levels.resize(nlod);
        steps.resize(nlod);
        for (uint32_t i = 0; i < nlod; ++i) {
            const Vector3ui &l = meta.get_initial_levels()[i];
            levels[i] = make_uint3(l[0], l[1], l[2]);
            inv_levels[i] = make_float3(bmin / static_cast<float>(l[0]), bmin / static_cast<float>(l[1]),
                                        bmin / static_cast<float>(l[2]));
            lodbrick[i] = make_float3((bbox[0] / l[0]) * B, (bbox[0] / l[1]) * B, (bbox[0] / l[2]) * B);
            steps[i] = (bmin / (std::min(l[0], std::min(l[1], l[2])))) / 2.f;
        }
        cuda_check(cudaMalloc(&d_levels, nlod * sizeof(uint3)), "cudaMalloc");
        cuda_check(cudaMalloc(&d_inv, nlod * sizeof(float3)), "cudaMalloc");
        cuda_check(cudaMalloc(&d_lodbrick, nlod * sizeof(float3)), "cudaMalloc");
        cuda_check(cudaMalloc(&d_steps, nlod * sizeof(float)), "cudaMalloc");
        cuda_check(cudaMemcpy(d_levels, levels.data(), nlod * sizeof(uint3), cudaMemcpyHostToDevice), "copy");
        cuda_check(cudaMemcpy(d_inv, inv_levels.data(), nlod * sizeof(float3), cudaMemcpyHostToDevice), "copy");
        cuda_check(cudaMemcpy(d_lodbrick, lodbrick.data(), nlod * sizeof(float3), cudaMemcpyHostToDevice), "copy");
        cuda_check(cudaMemcpy(d_steps, steps.data(), nlod * sizeof(float), cudaMemcpyHostToDevice), "copy");

        // 128-entry float4 transfer function texture (VolumeRayCaster.cu:218-223).
        cudaChannelFormatDesc desc = cudaCreateChannelDesc<float4>();
        cuda_check(cudaMallocArray(&tf_array, &desc, 128, 1), "cudaMallocArray");
        tdns::graphics::create_CUDA_transfer_function(tf_tex, tf_array);
    }

    ~SessionT() override {
        mgr.reset();
        if (tf_tex) cudaDestroyTextureObject(tf_tex);
        if (tf_array) cudaFreeArray(tf_array);
        cudaFree(d_levels);
        cudaFree(d_inv);
        cudaFree(d_lodbrick);
        cudaFree(d_steps);
    }

    void render(const float *inv_view, uint32_t w, uint32_t h, float tstep, const float *tf128, int mode,
                uint32_t *rgba, float *tbuf, float *state) override {
        cuda_check(cudaMemcpy2DToArray(tf_array, 0, 0, tf128, 128 * sizeof(float4), 128 * sizeof(float4), 1,
                                       cudaMemcpyHostToDevice),
                   "transfer function upload");
        tdns::graphics::update_CUDA_inv_view_model_matrix(inv_view);
        const dim3 grid((w % 16 != 0) ? (w / 16 + 1) : (w / 16), (h % 16 != 0) ? (h / 16 + 1) : (h / 16));
        const dim3 block(16, 16);
        const float3 bbmin = make_float3(-1.f, -1.f, -1.f), bbmax = make_float3(1.f, 1.f, 1.f);
        if (mode == 0)
            tdns::graphics::RayCastDVR<<<grid, block>>>(rgba, tbuf, reinterpret_cast<float4 *>(state), tf_tex,
                                                        make_uint2(w, h), w, 45.f, bbmin, bbmax, 1024, tstep,
                                                        mgr->to_kernel_object(), d_inv, d_levels, d_lodbrick,
                                                        d_steps, nlod, 0);
        else
            tdns::graphics::RayCastMOP<<<grid, block>>>(rgba, tbuf, reinterpret_cast<float4 *>(state), tf_tex,
                                                        make_uint2(w, h), w, 45.f, bbmin, bbmax, 1024, tstep,
                                                        mgr->to_kernel_object(), d_inv, d_levels, d_lodbrick,
                                                        d_steps, nlod, 0);
        cuda_check(cudaGetLastError(), "ray caster launch");
        cuda_check(cudaDeviceSynchronize(), "ray caster");
    }

    bool update(uint32_t wait_ms) override {
        const bool done = mgr->update();
        cuda_check(cudaDeviceSynchronize(), "update");
        const auto t0 = std::chrono::steady_clock::now();
        while (mgr->handler_working()) {
            if (std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(wait_ms))
                throw std::runtime_error("request handler still loading after the wait limit");
            std::this_thread::sleep_for(std::chrono::microseconds(100));
        }
        cuda_check(cudaDeviceSynchronize(), "request handler");
        return done;
    }

    uint32_t timestamp() override { return mgr->timestamp(); }

    uint3 mrpd_extent() {
        cudaChannelFormatDesc d;
        cudaExtent e;
        unsigned int flags;
        cuda_check(cudaArrayGetInfo(&d, &e, &flags, mgr->mrpd().data()->get_array()), "cudaArrayGetInfo");
        return make_uint3(static_cast<uint32_t>(e.width), static_cast<uint32_t>(e.height),
                          static_cast<uint32_t>(e.depth));
    }

    void info(uint32_t *mrpd_dims, uint32_t *cs, uint32_t *brick, uint32_t *ebo, uint32_t *nlevels) override {
        const uint3 e = mrpd_extent();
        mrpd_dims[0] = e.x;
        mrpd_dims[1] = e.y;
        mrpd_dims[2] = e.z;
        for (int a = 0; a < 3; ++a) cs[a] = cache_size[a];
        *brick = B;
        *ebo = eb;
        *nlevels = nlod;
    }

    void dump(int what, void *dst, size_t bytes) override {
        auto need = [&](size_t n) {
            if (bytes < n) throw std::runtime_error("dump buffer too small: " + std::to_string(n) + " bytes needed");
        };
        if (what == 0) {  // page directory: uint4 per entry, x fastest
            const uint3 e = mrpd_extent();
            need(static_cast<size_t>(e.x) * e.y * e.z * sizeof(uint4));
            cudaMemcpy3DParms p = {};
            p.srcArray = mgr->mrpd().data()->get_array();
            p.dstPtr = make_cudaPitchedPtr(dst, e.x * sizeof(uint4), e.x, e.y);
            p.extent = make_cudaExtent(e.x, e.y, e.z);
            p.kind = cudaMemcpyDeviceToHost;
            cuda_check(cudaMemcpy3D(&p), "page directory read");
        } else if (what == 1) {  // LRU records in LRU order (LruContent, 28 bytes)
            thrust::host_vector<tdns::gpucache::LruContent> h = mgr->pool().get_lru();
            need(h.size() * sizeof(tdns::gpucache::LruContent));
            std::memcpy(dst, h.data(), h.size() * sizeof(tdns::gpucache::LruContent));
        } else if (what == 2 || what == 3) {  // usage per slot / request word per entry
            tdns::common::DynamicArray3dDevice<uint32_t> &a =
                what == 2 ? mgr->pool().get_usage_buffer() : mgr->requests();
            need(a.size() * sizeof(uint32_t));
            cuda_check(cudaMemcpy(dst, a.data(), a.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost), "read");
        } else if (what == 4) {  // brick pool, slot-major
            // The pool surface is reached through the kernel object only; its
            // extent is cacheSize * blockSize voxels (Surface3dDevice.hpp:88-97).
            const uint3 ext = make_uint3(cache_size[0] * B, cache_size[1] * B, cache_size[2] * B);
            const size_t n = static_cast<size_t>(ext.x) * ext.y * ext.z;
            need(n * sizeof(T));
            T *buf = nullptr;
            cuda_check(cudaMalloc(&buf, n * sizeof(T)), "cudaMalloc");
            read_pool_kernel<T><<<1024, 256>>>(mgr->pool().to_kernel_object(), buf, ext, B);
            cudaError_t err = cudaDeviceSynchronize();
            if (err == cudaSuccess) err = cudaMemcpy(dst, buf, n * sizeof(T), cudaMemcpyDeviceToHost);
            cudaFree(buf);
            cuda_check(err, "pool read");
        } else {
            throw std::runtime_error("unknown dump kind");
        }
    }

    void asked(uint32_t *out4, uint32_t max, uint32_t *n, uint32_t *n_nonempty) override {
        thrust::host_vector<uint4> h = mgr->handler().get_asked_bricks();
        *n = static_cast<uint32_t>(h.size());
        *n_nonempty = static_cast<uint32_t>(mgr->handler().get_nb_non_empty_bricks());
        const uint32_t m = std::min<uint32_t>(max, *n);
        for (uint32_t i = 0; i < m; ++i) {
            out4[4 * i + 0] = h[i].x;
            out4[4 * i + 1] = h[i].y;
            out4[4 * i + 2] = h[i].z;
            out4[4 * i + 3] = h[i].w;
        }
    }

    float completude() override {
        std::vector<float> v;
        mgr->completude(v);
        return v.empty() ? 0.f : v[0];
    }

    void lod_tables(float *inv, float *st, uint32_t *n) override {
        *n = nlod;
        for (uint32_t i = 0; i < nlod; ++i) {
            inv[3 * i + 0] = inv_levels[i].x;
            inv[3 * i + 1] = inv_levels[i].y;
            inv[3 * i + 2] = inv_levels[i].z;
            st[i] = steps[i];
        }
    }
};

std::unique_ptr<Session> g_session;

// The application's bricking step (Application.cu:227-285): one thread per
// level running the reference's process_bricking.
void brick_levels(tdns::data::MetaData &md, const std::vector<Vector3ui> &levels) {
    tdns::preprocessor::BrickingConfiguration c;
    c.brickSize = Vector3ui(field_u32("BrickSize"));
    c.encodedBytes = field_u32("NumberEncodedBytes");
    c.covering = field_u32("VoxelCovering");
    if (!conf().get_field("VolumeDirectory", c.volumeDirectory) ||
        !conf().get_field("VolumeFile", c.volumeFileName) || !conf().get_field("VolumeDirectory", c.outputDirectory))
        throw std::runtime_error("VolumeDirectory / VolumeFile missing");
    c.compression = true;
    c.bigBrickSize = Vector3ui(field_u32("BigBrickSizeX"), field_u32("BigBrickSizeY"), field_u32("BigBrickSizeZ"));
    tdns::preprocessor::init_meta_data(md, c, levels);
    std::vector<std::thread> threads(levels.size());
    std::vector<int> ok(levels.size(), 0);
    for (uint32_t i = 0; i < threads.size(); ++i) {
        threads[i] = std::thread([&, i, c]() mutable {
            c.level = i;
            c.startX = c.startY = c.startZ = 0;
            c.endX = c.levelDimensionX = levels[i][0];
            c.endY = c.levelDimensionY = levels[i][1];
            c.endZ = c.levelDimensionZ = levels[i][2];
            ok[i] = tdns::preprocessor::process_bricking(c) ? 1 : 0;
        });
    }
    for (auto &t : threads) t.join();
    for (size_t i = 0; i < ok.size(); ++i)
        if (!ok[i]) throw std::runtime_error("process_bricking failed for level " + std::to_string(i));
}

template <typename T, typename P>
void process_empty(tdns::data::MetaData &md, float threshold) {
    float *d_threshold = nullptr;
    cuda_check(cudaMalloc(&d_threshold, sizeof(float)), "cudaMalloc");
    cuda_check(cudaMemcpy(d_threshold, &threshold, sizeof(float), cudaMemcpyHostToDevice), "copy");
    tdns::preprocessor::BrickProcessor<T> bp(md);
    bp.process_histo();
    bp.template process_empty<P>(d_threshold);
    cuda_check(cudaDeviceSynchronize(), "process_empty");
    cudaFree(d_threshold);
}

template <typename F>
int guarded(F &&f) {
    try {
        f();
        return 0;
    } catch (const std::exception &e) {
        return fail(e.what());
    } catch (...) {
        return fail("unknown exception");
    }
}

}  // namespace

extern "C" {

const char *refgpu_last_error(void) { return g_error.c_str(); }

// Configuration::load<TDNSConfigurationParser> of a .cfg file, then the
// VolumeDirectory field of Application::init (Application.cu:33-38).
int refgpu_config_load(const char *path) {
    return guarded([&] {
        conf().load<tdns::data::TDNSConfigurationParser>(path);
        std::string file, work;
        if (!conf().get_field("VolumeFile", file) || !conf().get_field("WorkingDirectory", work))
            throw std::runtime_error("VolumeFile / WorkingDirectory missing in " + std::string(path));
        conf().add_field("VolumeDirectory", work + tdns::common::get_file_base_name(file) + "/");
    });
}

// Application::pre_process (Application.cu:148-197): mipmaps, bricks, empty
// bricks with `empty_threshold` (its emptyBrickThreshold field), bricks.xml.
int refgpu_preprocess(float empty_threshold) {
    return guarded([&] {
        const uint32_t eb = field_u32("NumberEncodedBytes");
        tdns::data::MetaData md;
        tdns::preprocessor::Mipmapper mipmapper;
        mipmapper.process(md);
        if (md.get_initial_levels().empty()) throw std::runtime_error("Mipmapper::process produced no level");
        std::vector<Vector3ui> levels = md.get_initial_levels();
        brick_levels(md, levels);
        switch (eb) {
            case 1:
                process_empty<uchar1, tdns::preprocessor::DefaultBrickProcessorPredicate>(md, empty_threshold);
                break;
            case 2:
                process_empty<ushort1, tdns::preprocessor::BrickProcessor16BitsPredicate>(md, empty_threshold);
                break;
            default:
                throw std::runtime_error("NumberEncodedBytes must be 1 or 2 here");
        }
        md.write_bricks_xml();
    });
}

// Mipmapper::process alone (Mipmapper.cu:401-525): the mip files of the
// configured volume, for timing the reference's preprocessor.
int refgpu_mipmap(void) {
    return guarded([&] {
        tdns::data::MetaData md;
        tdns::preprocessor::Mipmapper mipmapper;
        mipmapper.process(md);
        if (md.get_initial_levels().empty()) throw std::runtime_error("Mipmapper::process produced no level");
    });
}

// Mipmapper::process then process_bricking of every level (one thread per
// level, LZ4 brick files, as Application::pre_process runs them), each timed
// on the host clock: the reference's preprocessor stages for the bench.
int refgpu_preprocess_timed(double *mip_s, double *brick_s) {
    return guarded([&] {
        if (!mip_s || !brick_s) throw std::runtime_error("null argument");
        tdns::data::MetaData md;
        tdns::preprocessor::Mipmapper mipmapper;
        const auto t0 = std::chrono::steady_clock::now();
        mipmapper.process(md);
        const auto t1 = std::chrono::steady_clock::now();
        if (md.get_initial_levels().empty()) throw std::runtime_error("Mipmapper::process produced no level");
        std::vector<Vector3ui> levels = md.get_initial_levels();
        brick_levels(md, levels);
        const auto t2 = std::chrono::steady_clock::now();
        *mip_s = std::chrono::duration<double>(t1 - t0).count();
        *brick_s = std::chrono::duration<double>(t2 - t1).count();
    });
}

// load_volume_configuration + MetaData::load + CacheManager<T> (Application::run,
// Application.cu:43-133) with a pool of cache_size slots.
int refgpu_open(const char *cfg_path, const uint32_t cache_size[3], int gpu) {
    return guarded([&] {
        g_session.reset();
        cuda_check(cudaSetDevice(gpu), "cudaSetDevice");
        const uint32_t eb = field_u32("NumberEncodedBytes");
        if (eb == 1)
            g_session.reset(new SessionT<uchar1>(cfg_path, cache_size, gpu));
        else if (eb == 2)
            g_session.reset(new SessionT<ushort1>(cfg_path, cache_size, gpu));
        else
            throw std::runtime_error("NumberEncodedBytes must be 1 or 2 here");
    });
}

int refgpu_close(void) {
    return guarded([&] { g_session.reset(); });
}

static Session &session() {
    if (!g_session) throw std::runtime_error("no cache open");
    return *g_session;
}

// One frame of get_frame: inv_view is d_invModelViewMatrix (3 x float4 rows),
// tf128 the 128 RGBA samples of the transfer function (host), mode 0 = DVR,
// 1 = MOP; rgba/tbuf/state are device buffers of w*h pixels (w, h multiples
// of 16 keep the kernel's x > width test inside them).
int refgpu_render(const float inv_view[12], uint32_t w, uint32_t h, float tstep, const float *tf128, int mode,
                  uint32_t *rgba, float *tbuf, float *state) {
    return guarded([&] { session().render(inv_view, w, h, tstep, tf128, mode, rgba, tbuf, state); });
}

// CacheManager::update, then a wait (at most wait_ms) until the request
// handler finished the list it was handed.
int refgpu_update(int *converged, uint32_t wait_ms) {
    return guarded([&] { *converged = session().update(wait_ms) ? 1 : 0; });
}

int refgpu_timestamp(uint32_t *ts) {
    return guarded([&] { *ts = session().timestamp(); });
}

int refgpu_info(uint32_t mrpd_dims[3], uint32_t cache_size[3], uint32_t *brick, uint32_t *eb, uint32_t *nlevels) {
    return guarded([&] { session().info(mrpd_dims, cache_size, brick, eb, nlevels); });
}

// what: 0 page directory (uint4 per entry), 1 LRU (LruContent records),
// 2 usage (uint32 per slot), 3 request buffer (uint32 per entry),
// 4 brick pool (slot-major, B^3 voxels per slot).
int refgpu_dump(int what, void *dst, size_t bytes) {
    return guarded([&] { session().dump(what, dst, bytes); });
}

// The request handler's last list (non-empty bricks first, as handle_request
// reorders it), its length and its count of non-empty bricks.
int refgpu_asked(uint32_t *out4, uint32_t max, uint32_t *n, uint32_t *n_nonempty) {
    return guarded([&] { session().asked(out4, max, n, n_nonempty); });
}

int refgpu_completude(float *frac) {
    return guarded([&] { *frac = session().completude(); });
}

// invLevelsSize (3 floats per level) and LODStepSize of the open volume.
int refgpu_lod_tables(float *inv_levels, float *steps, uint32_t *n) {
    return guarded([&] { session().lod_tables(inv_levels, steps, n); });
}

}  // extern "C"
