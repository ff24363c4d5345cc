// The reference's on-disk brick store: one file per big brick,
//   <volume dir>bricks_B_B_B/L<l>/L<l>_<x>_<y>_<z>.raw
// holding the (BB*B)^3 x encoded_bytes voxels of the big brick at big-brick
// position (x, y, z) of level l as one LZ4 block compressed with LZ4_compress_HC
// level 9 (BricksManager::write_brick / load_brick, BricksManager.cpp:81-113,
// 191-227; names BricksManager.cpp:149-188, BrickKey.cpp:38-44), and
//   <volume dir>bricks_B_B_B/bricks.xml
// with the level sizes, the empty big bricks and a 256-bin histogram
// (MetaData::write_bricks_xml / load, MetaData.cpp:36-216).
//
// LZ4 is the reference's codec (pinned v1.8.1.2 in its build); the system's
// liblz4.so.1 is loaded at run time, and the entry points that need it fail
// with GC_ERR_UNSUPPORTED where it is absent.  Files are written and read by
// worker threads (one brick per task).
#include <dlfcn.h>
#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "brickfiles.h"
#include "gc_internal.h"

namespace gc {

namespace {

struct Lz4 {
    int (*decompress_safe)(const char *, char *, int, int) = nullptr;
    int (*compress_bound)(int) = nullptr;
    int (*compress_hc)(const char *, char *, int, int, int) = nullptr;
    std::string error;
};

Lz4 load_lz4() {
    Lz4 L;
    void *h = dlopen("liblz4.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("liblz4.so", RTLD_NOW | RTLD_LOCAL);
    if (!h) {
        L.error = "liblz4 (the brick files' codec) is not installed";
        return L;
    }
    L.decompress_safe = reinterpret_cast<int (*)(const char *, char *, int, int)>(dlsym(h, "LZ4_decompress_safe"));
    L.compress_bound = reinterpret_cast<int (*)(int)>(dlsym(h, "LZ4_compressBound"));
    L.compress_hc = reinterpret_cast<int (*)(const char *, char *, int, int, int)>(dlsym(h, "LZ4_compress_HC"));
    if (!L.decompress_safe || !L.compress_bound || !L.compress_hc) L.error = "liblz4 lacks the LZ4 block functions";
    return L;
}

const Lz4 &lz4() {
    static const Lz4 L = load_lz4();
    return L;
}

const Lz4 &require_lz4() {
    const Lz4 &L = lz4();
    if (!L.error.empty()) fail(GC_ERR_UNSUPPORTED, L.error);
    return L;
}

std::string dir_prefix(const char *d) {
    std::string s = d ? d : "";
    if (!s.empty() && s.back() != '/') s += '/';
    return s;
}

std::string bricks_folder(const std::string &dir, uint32_t B) {
    return dir + "bricks_" + std::to_string(B) + "_" + std::to_string(B) + "_" + std::to_string(B);
}

void make_dir(const std::string &p) {
    if (mkdir(p.c_str(), 0755) != 0 && errno != EEXIST) fail(GC_ERR_IO, "cannot create directory " + p);
}

uint64_t big_brick_bytes(const gc_volume_desc &v) {
    return static_cast<uint64_t>(v.brick_size) * v.brick_size * v.brick_size * v.big_brick_size[0] *
           v.big_brick_size[1] * v.big_brick_size[2] * v.encoded_bytes;
}

// Runs f(i) for i in [0, n) on up to `threads` worker threads; the first
// error message wins.
template <class F>
void parallel_for(uint64_t n, uint32_t threads, F f) {
    const uint32_t nt = static_cast<uint32_t>(
        std::max<uint64_t>(1, std::min<uint64_t>(n, threads ? threads : std::max(1u, std::thread::hardware_concurrency()))));
    std::atomic<uint64_t> next{0};
    std::mutex mu;
    std::string err;
    auto work = [&] {
        for (;;) {
            const uint64_t i = next.fetch_add(1);
            if (i >= n) return;
            try {
                f(i);
            } catch (const std::exception &e) {
                std::lock_guard<std::mutex> g(mu);
                if (err.empty()) err = e.what();
                next.store(n);
            }
        }
    };
    std::vector<std::thread> pool;
    for (uint32_t t = 1; t < nt; ++t) pool.emplace_back(work);
    work();
    for (auto &th : pool) th.join();
    if (!err.empty()) fail(GC_ERR_IO, err);
}

struct LevelJob {
    uint32_t level;
    uint32_t nb[3];
    uint64_t offset, count;
};

std::vector<LevelJob> level_jobs(const gc_volume_desc &v, const gc_layout &L, uint64_t bytes, const uint64_t *offs) {
    GC_REQUIRE(L.nb_levels >= 1 && L.nb_levels <= GC_MAX_LEVELS, "bad layout");
    const uint64_t bb = big_brick_bytes(v);
    std::vector<LevelJob> jobs;
    for (uint32_t l = 0; l < L.nb_levels; ++l) {
        LevelJob j{l, {L.nb_big_bricks[l][0], L.nb_big_bricks[l][1], L.nb_big_bricks[l][2]}, offs[l], 0};
        j.count = static_cast<uint64_t>(j.nb[0]) * j.nb[1] * j.nb[2];
        GC_REQUIRE(offs[l] <= bytes && j.count <= (bytes - offs[l]) / bb,
                   "brick store: level " + std::to_string(l) + " does not fit in the store's bytes");
        jobs.push_back(j);
    }
    return jobs;
}

}  // namespace

std::string brick_file_path(const std::string &dir, uint32_t B, uint32_t level, uint32_t x, uint32_t y, uint32_t z) {
    const std::string l = std::to_string(level);
    return bricks_folder(dir, B) + "/L" + l + "/L" + l + "_" + std::to_string(x) + "_" + std::to_string(y) + "_" +
           std::to_string(z) + ".raw";
}

bool lz4_available(std::string *why) {
    const Lz4 &L = lz4();
    if (why) *why = L.error;
    return L.error.empty();
}

int read_brick_file(const std::string &path, void *dst, uint64_t bytes) {
    std::ifstream is(path, std::ios::binary);
    if (!is) return 1;
    std::vector<char> comp((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
    if (comp.empty() || comp.size() > static_cast<size_t>(INT32_MAX) || bytes > static_cast<uint64_t>(INT32_MAX))
        return 2;
    const Lz4 &L = require_lz4();
    const int n = L.decompress_safe(comp.data(), static_cast<char *>(dst), static_cast<int>(comp.size()),
                                    static_cast<int>(bytes));
    return n == static_cast<int>(bytes) ? 0 : 2;
}

}  // namespace gc

using namespace gc;

extern "C" {

int gc_brick_files_write(const char *volume_dir, const gc_volume_desc *vol, const gc_layout *layout, const void *store,
                         uint64_t bytes, const uint64_t *level_offsets, uint32_t threads) {
    return guard([&] {
        GC_REQUIRE(volume_dir && vol && layout && store && level_offsets, "null argument");
        validate_volume(*vol);
        const Lz4 &L = require_lz4();
        const std::string dir = dir_prefix(volume_dir);
        const uint32_t B = vol->brick_size;
        const uint64_t bb = big_brick_bytes(*vol);
        GC_REQUIRE(bb < static_cast<uint64_t>(INT32_MAX), "big bricks too large for one LZ4 block");
        const auto jobs = level_jobs(*vol, *layout, bytes, level_offsets);
        make_dir(bricks_folder(dir, B));
        for (const auto &j : jobs) make_dir(bricks_folder(dir, B) + "/L" + std::to_string(j.level));
        const uint8_t *base = static_cast<const uint8_t *>(store);
        const int bound = L.compress_bound(static_cast<int>(bb));
        for (const auto &j : jobs) {
            parallel_for(j.count, threads, [&](uint64_t i) {
                const uint32_t x = static_cast<uint32_t>(i % j.nb[0]);
                const uint32_t y = static_cast<uint32_t>((i / j.nb[0]) % j.nb[1]);
                const uint32_t z = static_cast<uint32_t>(i / (static_cast<uint64_t>(j.nb[0]) * j.nb[1]));
                std::vector<char> comp(static_cast<size_t>(bound));
                const int n = L.compress_hc(reinterpret_cast<const char *>(base + j.offset + i * bb), comp.data(),
                                            static_cast<int>(bb), bound, 9);
                if (n <= 0) throw std::runtime_error("LZ4 compression failed");
                const std::string p = brick_file_path(dir, B, j.level, x, y, z);
                std::ofstream os(p, std::ios::binary | std::ios::trunc);
                os.write(comp.data(), n);
                if (!os) throw std::runtime_error("cannot write " + p);
            });
        }
    });
}

int gc_brick_files_read(const char *volume_dir, const gc_volume_desc *vol, const gc_layout *layout, void *store,
                        uint64_t bytes, const uint64_t *level_offsets, uint32_t threads) {
    return guard([&] {
        GC_REQUIRE(volume_dir && vol && layout && store && level_offsets, "null argument");
        validate_volume(*vol);
        require_lz4();
        const std::string dir = dir_prefix(volume_dir);
        const uint32_t B = vol->brick_size;
        const uint64_t bb = big_brick_bytes(*vol);
        const auto jobs = level_jobs(*vol, *layout, bytes, level_offsets);
        uint8_t *base = static_cast<uint8_t *>(store);
        for (const auto &j : jobs) {
            parallel_for(j.count, threads, [&](uint64_t i) {
                const uint32_t x = static_cast<uint32_t>(i % j.nb[0]);
                const uint32_t y = static_cast<uint32_t>((i / j.nb[0]) % j.nb[1]);
                const uint32_t z = static_cast<uint32_t>(i / (static_cast<uint64_t>(j.nb[0]) * j.nb[1]));
                const std::string p = brick_file_path(dir, B, j.level, x, y, z);
                const int rc = read_brick_file(p, base + j.offset + i * bb, bb);
                if (rc == 1) throw std::runtime_error("missing brick file " + p);
                if (rc == 2) throw std::runtime_error("corrupt brick file " + p);
            });
        }
    });
}

// MetaData::write_bricks_xml (MetaData.cpp:36-101): the layout tinyxml2
// prints (4-space indent, one element per line, attributes in this order).
int gc_bricks_xml_write(const char *volume_dir, const gc_volume_desc *vol, const gc_layout *layout,
                        const uint64_t *empty_keys, size_t n_empty) {
    return guard([&] {
        GC_REQUIRE(volume_dir && vol && layout && (empty_keys || n_empty == 0), "null argument");
        const std::string dir = dir_prefix(volume_dir);
        std::ostringstream o;
        o << "<Meta>\n    <Levels>\n";
        for (uint32_t l = 0; l < layout->nb_levels; ++l)
            o << "        <Level level=\"" << l << "\" initial_size_X=\"" << layout->initial[l][0]
              << "\" initial_size_Y=\"" << layout->initial[l][1] << "\" initial_size_Z=\"" << layout->initial[l][2]
              << "\" real_size_X=\"" << layout->real[l][0] << "\" real_size_Y=\"" << layout->real[l][1]
              << "\" real_size_Z=\"" << layout->real[l][2] << "\"/>\n";
        o << "    </Levels>\n";
        if (n_empty > 0) {
            o << "    <EmptyBricks>\n";
            for (size_t i = 0; i < n_empty; ++i)
                o << "        <Brick ID=\"" << static_cast<int64_t>(empty_keys[i]) << "\"/>\n";
            o << "    </EmptyBricks>\n";
        }
        o << "    <Histogram>\n";
        for (int i = 0; i < 256; ++i) o << "        <Histo Value=\"0\"/>\n";  // the reference never fills it
        o << "    </Histogram>\n</Meta>\n";
        make_dir(bricks_folder(dir, vol->brick_size));
        const std::string p = bricks_folder(dir, vol->brick_size) + "/bricks.xml";
        std::ofstream os(p, std::ios::binary | std::ios::trunc);
        const std::string text = o.str();
        os.write(text.data(), static_cast<std::streamsize>(text.size()));
        if (!os) fail(GC_ERR_IO, "cannot write " + p);
    });
}

// MetaData::load (MetaData.cpp:151-216) for what the path needs: the level
// sizes and the empty big bricks.
int gc_bricks_xml_read(const char *path, uint32_t *n_levels, uint32_t initial[][3], uint32_t real[][3],
                       uint64_t *empty_keys, size_t max_empty, size_t *n_empty) {
    return guard([&] {
        GC_REQUIRE(path && n_levels && initial && real && n_empty && (empty_keys || max_empty == 0),
                   "null argument");
        std::ifstream is(path);
        if (!is) fail(GC_ERR_IO, std::string("cannot open ") + path);
        auto attr = [](const std::string &line, const char *name, uint64_t &out) {
            const std::string key = std::string(name) + "=\"";
            const size_t p = line.find(key);
            if (p == std::string::npos) return false;
            out = std::stoull(line.substr(p + key.size()));
            return true;
        };
        uint32_t nl = 0;
        size_t ne = 0;
        std::string line;
        while (std::getline(is, line)) {
            if (line.find("<Level ") != std::string::npos) {
                uint64_t l = 0, v[6];
                const char *names[6] = {"initial_size_X", "initial_size_Y", "initial_size_Z",
                                        "real_size_X",    "real_size_Y",    "real_size_Z"};
                GC_REQUIRE(attr(line, "level", l), "bricks.xml: a Level without its level attribute");
                for (int k = 0; k < 6; ++k) GC_REQUIRE(attr(line, names[k], v[k]), "bricks.xml: incomplete Level");
                GC_REQUIRE(l < GC_MAX_LEVELS, "bricks.xml: too many levels");
                for (int a = 0; a < 3; ++a) {
                    initial[l][a] = static_cast<uint32_t>(v[a]);
                    real[l][a] = static_cast<uint32_t>(v[3 + a]);
                }
                nl = std::max<uint32_t>(nl, static_cast<uint32_t>(l) + 1);
            } else if (line.find("<Brick ") != std::string::npos) {
                uint64_t id = 0;
                GC_REQUIRE(attr(line, "ID", id), "bricks.xml: a Brick without its ID");
                if (ne < max_empty) empty_keys[ne] = id;
                ++ne;
            }
        }
        *n_levels = nl;
        *n_empty = ne;
    });
}

int gc_lz4_available(void) { return lz4_available(nullptr) ? 1 : 0; }

}  // extern "C"
