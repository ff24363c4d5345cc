// Configuration surface and level geometry of the out-of-core volume path.
//
//  - gc_config_*: the reference's key/value Configuration singleton
//    (GcCore/src/libData/Configuration.cpp:30-186) fed by the
//    TDNSConfigurationParser (GcCore/src/libData/ConfigurationPolicies.cpp:16-44),
//    which reads <Fields><Field key="..." value="..."/></Fields>.  Here it is an
//    explicit handle instead of a process-wide singleton.
//  - gc_layout_compute: Mipmapper::fill_metaData + the levelMax formula
//    (GcCore/src/cuda/libPreprocessor/Mipmapper.cu:441-443, 583-597) and
//    init_meta_data (GcCore/src/libPreprocessor/Bricker_v2.cpp:45-76).
//  - gc_pool_dims: pool sizing of Applications/DVR-ray-caster/src/Application.cu:79-93.
#include <atomic>
#include <cmath>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>

#include "gc_internal.h"

namespace gc {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

void count_launch(uint32_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

void set_error(const std::string &msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

int sm_count() {
    static int cached[8] = {0};
    int dev = 0;
    GC_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 8 && cached[dev]) return cached[dev];
    int n = 0;
    GC_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    if (dev >= 0 && dev < 8) cached[dev] = n;
    return n;
}

void validate_volume(const gc_volume_desc &v) {
    for (int i = 0; i < 3; ++i) {
        GC_REQUIRE(v.size[i] > 0, "volume size must be > 0 on every axis");
        GC_REQUIRE(v.big_brick_size[i] > 0, "BigBrickSize must be > 0 on every axis");
        GC_REQUIRE(v.downscale[i] == 2, "only downScale 2 is supported");
    }
    GC_REQUIRE(v.brick_size > 2 * v.covering, "BrickSize must exceed 2 * VoxelCovering");
    GC_REQUIRE(v.brick_size >= 2 && v.brick_size <= 128, "BrickSize must be in [2, 128]");
    GC_REQUIRE(v.channels >= 1 && v.channels <= 4, "NumberChannels must be in [1, 4]");
    GC_REQUIRE(v.encoded_bytes % v.channels == 0,
               "NumberEncodedBytes must be a multiple of NumberChannels");
    uint32_t cb = v.encoded_bytes / v.channels;
    GC_REQUIRE(cb == 1 || cb == 2 || cb == 4, "bytes per channel must be 1, 2 or 4");
    GC_REQUIRE(!(cb == 4 && v.channels != 1), "float voxels support one channel only");
}

// Parser of the reference's XML field file.  Only the subset the reference
// writes and reads is supported: <Field key="..." value="..."/> elements,
// comments and an enclosing root element.
static void parse_fields(const std::string &text, std::map<std::string, std::string> &out) {
    size_t pos = 0;
    auto attr = [](const std::string &tag, const char *name, std::string &val) -> bool {
        std::string pat = std::string(name) + "=";
        size_t p = 0;
        while ((p = tag.find(pat, p)) != std::string::npos) {
            // must be a whole attribute name
            if (p > 0 && !isspace(static_cast<unsigned char>(tag[p - 1]))) {
                p += pat.size();
                continue;
            }
            size_t q = p + pat.size();
            if (q >= tag.size()) return false;
            char quote = tag[q];
            if (quote != '"' && quote != '\'') return false;
            size_t e = tag.find(quote, q + 1);
            if (e == std::string::npos) return false;
            val = tag.substr(q + 1, e - q - 1);
            return true;
        }
        return false;
    };
    while ((pos = text.find('<', pos)) != std::string::npos) {
        if (text.compare(pos, 4, "<!--") == 0) {
            size_t e = text.find("-->", pos + 4);
            if (e == std::string::npos) fail(GC_ERR_IO, "unterminated XML comment");
            pos = e + 3;
            continue;
        }
        size_t e = text.find('>', pos);
        if (e == std::string::npos) fail(GC_ERR_IO, "unterminated XML tag");
        std::string tag = text.substr(pos + 1, e - pos - 1);
        pos = e + 1;
        if (tag.compare(0, 5, "Field") == 0 &&
            (tag.size() == 5 || isspace(static_cast<unsigned char>(tag[5])))) {
            std::string k, v;
            if (!attr(tag, "key", k) || !attr(tag, "value", v))
                fail(GC_ERR_IO, "Field element without key or value: <" + tag + ">");
            if (!k.empty()) out[k] = v;  // empty keys are ignored (Configuration.cpp:33-37)
        }
    }
}

}  // namespace gc

struct gc_config {
    std::map<std::string, std::string> values;
};

using namespace gc;

extern "C" {

const char *gc_last_error(void) { return g_last_error.c_str(); }

const char *gc_version(void) { return "gcgb300 0.1 (sm_103a)"; }

uint64_t gc_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int gc_device_count(int *count) {
    return guard([&] {
        GC_REQUIRE(count, "null output");
        GC_CUDA(cudaGetDeviceCount(count));
    });
}

int gc_config_create(gc_config_t *out) {
    return guard([&] {
        GC_REQUIRE(out, "null output");
        *out = new gc_config();
    });
}

int gc_config_destroy(gc_config_t cfg) {
    delete cfg;
    return GC_OK;
}

int gc_config_load(gc_config_t cfg, const char *path) {
    return guard([&] {
        GC_REQUIRE(cfg && path, "null argument");
        std::ifstream f(path, std::ios::in | std::ios::binary);
        if (!f) fail(GC_ERR_IO, std::string("unable to open the configuration file ") + path);
        std::stringstream ss;
        ss << f.rdbuf();
        parse_fields(ss.str(), cfg->values);
    });
}

int gc_config_set(gc_config_t cfg, const char *key, const char *value) {
    return guard([&] {
        GC_REQUIRE(cfg && key && value, "null argument");
        if (*key) cfg->values[key] = value;
    });
}

int gc_config_get(gc_config_t cfg, const char *key, char *buf, size_t buflen) {
    return guard([&] {
        GC_REQUIRE(cfg && key && buf && buflen, "null argument");
        auto it = cfg->values.find(key);
        if (it == cfg->values.end()) fail(GC_ERR_INVALID, std::string("missing field ") + key);
        GC_REQUIRE(it->second.size() < buflen, "buffer too small");
        std::memcpy(buf, it->second.c_str(), it->second.size() + 1);
    });
}

int gc_config_volume_desc(gc_config_t cfg, gc_volume_desc *out) {
    return guard([&] {
        GC_REQUIRE(cfg && out, "null argument");
        // Integer fields are read with std::stoul like Configuration::get_field.
        auto get = [&](const char *key, bool required, uint32_t dflt) -> uint32_t {
            auto it = cfg->values.find(key);
            if (it == cfg->values.end()) {
                if (required)
                    fail(GC_ERR_INVALID,
                         std::string("VolumeConfiguration: Missing ") + key + " in configuration.");
                return dflt;
            }
            try {
                return static_cast<uint32_t>(std::stoul(it->second));
            } catch (const std::exception &) {
                fail(GC_ERR_INVALID, std::string("field ") + key + " is not an unsigned integer");
            }
        };
        gc_volume_desc v;
        std::memset(&v, 0, sizeof(v));
        v.brick_size = get("BrickSize", true, 0);
        v.big_brick_size[0] = get("BigBrickSizeX", true, 1);
        v.big_brick_size[1] = get("BigBrickSizeY", true, 1);
        v.big_brick_size[2] = get("BigBrickSizeZ", true, 1);
        v.covering = get("VoxelCovering", true, 0);
        v.encoded_bytes = get("NumberEncodedBytes", true, 1);
        v.channels = get("NumberChannels", true, 1);
        v.size[0] = get("size_X", true, 0);
        v.size[1] = get("size_Y", true, 0);
        v.size[2] = get("size_Z", true, 0);
        v.downscale[0] = get("downScale_X", false, 2);
        v.downscale[1] = get("downScale_Y", false, 2);
        v.downscale[2] = get("downScale_Z", false, 2);
        validate_volume(v);
        *out = v;
    });
}

int gc_layout_compute(const gc_volume_desc *vol, gc_layout *out) {
    return guard([&] {
        GC_REQUIRE(vol && out, "null argument");
        validate_volume(*vol);
        gc_layout L;
        std::memset(&L, 0, sizeof(L));
        const uint32_t B = vol->brick_size;
        // Mipmapper.cu:441-443: integer division first, then a double log ratio.
        const uint32_t maxDim = std::max(vol->size[0], std::max(vol->size[1], vol->size[2]));
        const uint32_t q = maxDim / B;
        GC_REQUIRE(q >= 1, "the volume must be at least one brick wide");
        const uint32_t levelMax = static_cast<uint32_t>(std::ceil(std::log(q) / std::log(2)));
        GC_REQUIRE(levelMax + 1 <= GC_MAX_LEVELS, "too many levels");
        L.nb_levels = levelMax + 1;
        // fill_metaData (Mipmapper.cu:583-597): halve while size >= ratio.
        uint32_t s[3] = {vol->size[0], vol->size[1], vol->size[2]};
        // The mip data itself halves while size > ratio (Mipmapper.cu:511-513)
        // and each pass writes floor(size / 2) voxels per axis (down_scale).
        uint32_t m[3] = {vol->size[0], vol->size[1], vol->size[2]};
        for (uint32_t l = 0; l <= levelMax; ++l) {
            for (int a = 0; a < 3; ++a) {
                L.initial[l][a] = s[a];
                L.mip[l][a] = m[a];
            }
            for (int a = 0; a < 3; ++a) {
                if (s[a] >= vol->downscale[a]) s[a] /= vol->downscale[a];
                m[a] = std::max(1u, m[a] / vol->downscale[a]);
            }
        }
        // init_meta_data (Bricker_v2.cpp:45-76): float ceil divisions.
        const uint32_t Beff = B - 2 * vol->covering;
        for (uint32_t l = 0; l <= levelMax; ++l) {
            for (int a = 0; a < 3; ++a) {
                uint32_t nb = static_cast<uint32_t>(
                    std::ceil(static_cast<float>(L.initial[l][a]) / static_cast<float>(Beff)));
                nb = static_cast<uint32_t>(std::ceil(static_cast<float>(nb) /
                                                     static_cast<float>(vol->big_brick_size[a]))) *
                     vol->big_brick_size[a];
                L.nb_bricks[l][a] = nb;
                L.nb_big_bricks[l][a] = nb / vol->big_brick_size[a];
                L.real[l][a] = nb * Beff;
            }
        }
        *out = L;
    });
}

int gc_pool_dims(const gc_volume_desc *vol, uint64_t pool_bytes, uint32_t out_dims[3]) {
    return guard([&] {
        GC_REQUIRE(vol && out_dims, "null argument");
        // Application.cu:85-93
        const uint64_t B = vol->brick_size;
        const uint64_t brickBytes = B * B * B * vol->encoded_bytes;
        const uint64_t entries = pool_bytes / brickBytes;
        GC_REQUIRE(entries >= 1, "pool smaller than one brick");
        const uint64_t edge = static_cast<uint64_t>(std::cbrt(static_cast<double>(entries)));
        uint64_t d[3] = {edge, edge, edge};
        int axis = 0;
        while (d[0] * d[1] * d[2] < entries) {
            d[axis] += 1;
            axis = (axis + 1) % 3;
        }
        for (int i = 0; i < 3; ++i) out_dims[i] = static_cast<uint32_t>(d[i]);
    });
}

int gc_view_matrix(const float rotation_deg[2], const float translation[3], float out[12]) {
    return guard([&] {
        GC_REQUIRE(rotation_deg && translation && out, "null argument");
        // glRotatef(-rx, 1, 0, 0) * glRotatef(-ry, 0, 1, 0) * glTranslatef(-t)
        const double kDeg = 3.14159265358979323846 / 180.0;
        const double ax = -rotation_deg[0] * kDeg, ay = -rotation_deg[1] * kDeg;
        const double cx = std::cos(ax), sx = std::sin(ax), cy = std::cos(ay), sy = std::sin(ay);
        const double Rx[3][3] = {{1, 0, 0}, {0, cx, -sx}, {0, sx, cx}};
        const double Ry[3][3] = {{cy, 0, sy}, {0, 1, 0}, {-sy, 0, cy}};
        double R[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                R[i][j] = 0;
                for (int k = 0; k < 3; ++k) R[i][j] += Rx[i][k] * Ry[k][j];
            }
        const double t[3] = {-static_cast<double>(translation[0]), -static_cast<double>(translation[1]),
                             -static_cast<double>(translation[2])};
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) out[4 * i + j] = static_cast<float>(R[i][j]);
            out[4 * i + 3] = static_cast<float>(R[i][0] * t[0] + R[i][1] * t[1] + R[i][2] * t[2]);
        }
    });
}

int gc_look_at(const float eye[3], const float target[3], const float up[3], float out[12]) {
    return guard([&] {
        GC_REQUIRE(eye && target && up && out, "null argument");
        double f[3], r[3], u[3];
        for (int a = 0; a < 3; ++a) f[a] = static_cast<double>(target[a]) - eye[a];
        auto norm = [](double *v) {
            const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            GC_REQUIRE(n > 0, "degenerate camera");
            for (int a = 0; a < 3; ++a) v[a] /= n;
        };
        auto cross = [](const double *a, const double *b, double *o) {
            o[0] = a[1] * b[2] - a[2] * b[1];
            o[1] = a[2] * b[0] - a[0] * b[2];
            o[2] = a[0] * b[1] - a[1] * b[0];
        };
        norm(f);
        const double upd[3] = {up[0], up[1], up[2]};
        cross(f, upd, r);
        norm(r);
        cross(r, f, u);
        for (int a = 0; a < 3; ++a) {
            out[4 * a + 0] = static_cast<float>(r[a]);
            out[4 * a + 1] = static_cast<float>(u[a]);
            out[4 * a + 2] = static_cast<float>(-f[a]);
            out[4 * a + 3] = eye[a];
        }
    });
}

int gc_tf_build(const gc_tf_point *pts, uint32_t n, uint32_t samples, float *out) {
    return guard([&] {
        GC_REQUIRE(out && samples >= 1, "bad arguments");
        GC_REQUIRE(n == 0 || pts, "null control points");
        auto lerp = [](float a, float b, float t) { return a + (b - a) * t; };
        for (uint32_t i = 0; i < samples; ++i) {
            const float x = static_cast<float>(i) / static_cast<float>(samples);
            float *o = out + 4 * i;
            if (n == 0) {
                o[0] = o[1] = o[2] = o[3] = 0.f;
                continue;
            }
            uint32_t pos = 0;
            while (pos < n && !(pts[pos].value > x)) ++pos;
            gc_tf_point prev = pos == 0 ? gc_tf_point{0.f, 0.f, pts[0].r, pts[0].g, pts[0].b} : pts[pos - 1];
            gc_tf_point next = pos == n ? gc_tf_point{1.f, 0.f, pts[n - 1].r, pts[n - 1].g, pts[n - 1].b} : pts[pos];
            const float t = (x - prev.value) / (next.value - prev.value);
            o[0] = lerp(prev.r, next.r, t);
            o[1] = lerp(prev.g, next.g, t);
            o[2] = lerp(prev.b, next.b, t);
            o[3] = lerp(prev.alpha, next.alpha, t);
        }
    });
}

uint64_t gc_brick_key(uint32_t level, uint32_t x, uint32_t y, uint32_t z) {
    // get_key (BrickKey.cpp:15-25): uint16 {level, x, y, z} in memory order.
    return static_cast<uint64_t>(static_cast<uint16_t>(level)) |
           (static_cast<uint64_t>(static_cast<uint16_t>(x)) << 16) |
           (static_cast<uint64_t>(static_cast<uint16_t>(y)) << 32) |
           (static_cast<uint64_t>(static_cast<uint16_t>(z)) << 48);
}

}  // extern "C"
