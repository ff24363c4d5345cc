// Headless driver around the reference's own CPU preprocessing code, used to
// produce golden fixtures (TEST INFRASTRUCTURE ONLY; built by oracle/build.py
// into oracle/_ref/ from the reference sources where they lie).
//
//   refdriver layout  X Y Z B c BBx BBy BBz eb nc
//       prints init_meta_data (Bricker_v2.cpp:45-76) and fill_metaData
//       (Mipmapper.cu:292-304, restated here because that file needs a GPU
//       toolchain) per level: initial, real, nb_bricks, nb_big_bricks.
//   refdriver brick   workdir level X Y Z B c BBx BBy BBz eb nc out.bin
//       runs process_bricking (Bricker_v2.cpp:79-252) on workdir/vol.raw
//       (level 0) or workdir/mipmap/L<level>.raw, which writes LZ4 brick files
//       through BricksManager::write_brick; then reads every big-brick file back
//       (LZ4_decompress_safe) and writes them to out.bin in (z, y, x) order.
//   refdriver xml     workdir B c eb nc X Y Z BBx BBy BBz [empty keys...]
//       MetaData::write_bricks_xml (MetaData.cpp:36-101) of that geometry.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <iterator>
#include <string>
#include <vector>

#include <lz4.h>

#include <GcCore/libData/BricksManager.hpp>
#include <GcCore/libData/Configuration.hpp>
#include <GcCore/libData/MetaData.hpp>
#include <GcCore/libPreprocessor/Bricker_v2.hpp>

using tdns::math::Vector3ui;

static uint32_t arg(char **argv, int i) { return static_cast<uint32_t>(std::strtoul(argv[i], nullptr, 10)); }

static void set_conf(uint32_t B, uint32_t c, uint32_t eb, uint32_t nc, const std::string &volDir) {
    tdns::data::Configuration &conf = tdns::data::Configuration::get_instance();
    conf.add_field("BrickSize", B);
    conf.add_field("VoxelCovering", c);
    conf.add_field("NumberEncodedBytes", eb);
    conf.add_field("NumberChannels", nc);
    conf.add_field("VolumeDirectory", volDir);
}

static std::vector<Vector3ui> initial_levels(Vector3ui dim, uint32_t B) {
    const uint32_t maxDim = std::max(dim[0], std::max(dim[1], dim[2]));
    const uint32_t levelMax = static_cast<uint32_t>(std::ceil(std::log(maxDim / B) / std::log(2)));
    std::vector<Vector3ui> levels;
    uint32_t s[3] = {dim[0], dim[1], dim[2]};
    for (uint32_t i = 0; i <= levelMax; ++i) {
        levels.push_back(Vector3ui(s[0], s[1], s[2]));
        for (int a = 0; a < 3; ++a)
            if (s[a] >= 2) s[a] /= 2;
    }
    return levels;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    std::string mode = argv[1];
    if (mode == "layout" && argc == 12) {
        Vector3ui dim(arg(argv, 2), arg(argv, 3), arg(argv, 4));
        uint32_t B = arg(argv, 5), c = arg(argv, 6);
        Vector3ui bb(arg(argv, 7), arg(argv, 8), arg(argv, 9));
        set_conf(B, c, arg(argv, 10), arg(argv, 11), "./");
        tdns::preprocessor::BrickingConfiguration conf;
        conf.brickSize = Vector3ui(B);
        conf.bigBrickSize = bb;
        conf.covering = c;
        tdns::data::MetaData md;
        std::vector<Vector3ui> levels = initial_levels(dim, B);
        tdns::preprocessor::init_meta_data(md, conf, levels);
        for (size_t l = 0; l < levels.size(); ++l) {
            std::printf("%zu %u %u %u %u %u %u %u %u %u %u %u %u\n", l, levels[l][0], levels[l][1], levels[l][2],
                        md.get_real_levels()[l][0], md.get_real_levels()[l][1], md.get_real_levels()[l][2],
                        md.get_nb_bricks()[l][0], md.get_nb_bricks()[l][1], md.get_nb_bricks()[l][2],
                        md.get_nb_big_bricks()[l][0], md.get_nb_big_bricks()[l][1], md.get_nb_big_bricks()[l][2]);
        }
        return 0;
    }
    if (mode == "brick" && argc == 16) {
        std::string work = argv[2];
        if (work.back() != '/') work += "/";
        uint32_t level = arg(argv, 3);
        Vector3ui dim(arg(argv, 4), arg(argv, 5), arg(argv, 6));
        uint32_t B = arg(argv, 7), c = arg(argv, 8);
        Vector3ui bb(arg(argv, 9), arg(argv, 10), arg(argv, 11));
        uint32_t eb = arg(argv, 12), nc = arg(argv, 13);
        std::string out = argv[15];
        set_conf(B, c, eb, nc, work);
        tdns::preprocessor::BrickingConfiguration conf;
        conf.volumeDirectory = work;
        conf.volumeFileName = "vol.raw";
        conf.outputDirectory = work;
        conf.level = level;
        conf.startX = conf.startY = conf.startZ = 0;
        conf.endX = conf.levelDimensionX = dim[0];
        conf.endY = conf.levelDimensionY = dim[1];
        conf.endZ = conf.levelDimensionZ = dim[2];
        conf.brickSize = Vector3ui(B);
        conf.bigBrickSize = bb;
        conf.covering = c;
        conf.encodedBytes = eb;
        conf.compression = true;
        if (!tdns::preprocessor::process_bricking(conf)) return 3;
        // read back
        tdns::data::MetaData md;
        std::vector<Vector3ui> one(1, dim);
        tdns::preprocessor::init_meta_data(md, conf, one);
        Vector3ui nbig = md.get_nb_big_bricks()[0];
        const size_t bigBytes = static_cast<size_t>(B) * B * B * bb[0] * bb[1] * bb[2] * eb;
        std::ofstream os(out, std::ios::binary);
        std::vector<char> dst(bigBytes);
        for (uint32_t z = 0; z < nbig[2]; ++z)
            for (uint32_t y = 0; y < nbig[1]; ++y)
                for (uint32_t x = 0; x < nbig[0]; ++x) {
                    std::string p = work + tdns::data::BricksManager::get_brick_folder(Vector3ui(B)) + "/L" +
                                    std::to_string(level) + "/L" + std::to_string(level) + "_" + std::to_string(x) +
                                    "_" + std::to_string(y) + "_" + std::to_string(z) + ".raw";
                    std::ifstream is(p, std::ios::binary);
                    if (!is) {
                        std::fprintf(stderr, "missing %s\n", p.c_str());
                        return 4;
                    }
                    std::vector<char> comp((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
                    int n = LZ4_decompress_safe(comp.data(), dst.data(), static_cast<int>(comp.size()),
                                                static_cast<int>(bigBytes));
                    if (n != static_cast<int>(bigBytes)) {
                        std::fprintf(stderr, "bad brick %s (%d)\n", p.c_str(), n);
                        return 5;
                    }
                    os.write(dst.data(), bigBytes);
                }
        std::printf("%u %u %u\n", nbig[0], nbig[1], nbig[2]);
        return 0;
    }
    if (mode == "xml" && argc >= 13) {
        std::string work = argv[2];
        if (work.back() != '/') work += "/";
        uint32_t B = arg(argv, 3), c = arg(argv, 4), eb = arg(argv, 5), nc = arg(argv, 6);
        Vector3ui dim(arg(argv, 7), arg(argv, 8), arg(argv, 9));
        Vector3ui bb(arg(argv, 10), arg(argv, 11), arg(argv, 12));
        set_conf(B, c, eb, nc, work);
        tdns::data::BricksManager::check_level_directory(work, 0, Vector3ui(B));
        tdns::preprocessor::BrickingConfiguration conf;
        conf.brickSize = Vector3ui(B);
        conf.bigBrickSize = bb;
        conf.covering = c;
        tdns::data::MetaData md;
        std::vector<Vector3ui> levels = initial_levels(dim, B);
        md.get_initial_levels() = levels;
        tdns::preprocessor::init_meta_data(md, conf, levels);
        for (int i = 13; i < argc; ++i) md.get_empty_bricks().push_back(std::strtoull(argv[i], nullptr, 10));
        md.write_bricks_xml();
        return 0;
    }
    std::fprintf(stderr, "usage: refdriver layout|brick|xml ...\n");
    return 2;
}
