// astc_cs_enc -- drop-in command line encoder with the reference's interface
// (niepp/astc_encoder main.cpp:140-258):
//
//   astc_cs_enc input_texture [-4x4] [-6x6] [-alpha] [-norm] [-srgb]
//
// argv[1] is the input; the flags follow in any order (main.cpp:150-176).
// Like the reference it loads the image as RGBA flipped vertically
// (main.cpp:24-25), uses sRGB sampling only when not a normal map
// (main.cpp:214), prints the option block (193-197), and writes
// <input without its last extension>.astc with the 16-byte header
// (main.cpp:244-249, astc_save.h:52-76).  Differences, all deliberate:
// -6x6 selects 6x6 blocks (the reference never reads it); errors return a
// non-zero status with a message.  Extra options:
//   --clamp            clamp to the edge outside the image (default: zero,
//                      the reference's out-of-bounds Load)
//   --half2            packed-half2 precision (default FP32, bit-exact with
//                      the reference's math)
//   --search           search every single-partition 4x4-grid mode and keep
//                      the one with the least decoded error (the reference's
//                      unused choose_best_quantmethod; FP32 only)
//   --max-accumulation fit endpoints with the reference's unused
//                      max_accumulation_pixel_direction instead of the PCA
//   --thorough         --search from the better of the two fits
//   --partitions       --thorough plus two-partition blocks
//   --three-partitions --partitions plus three-partition blocks (RGB input)
//   --best-fit         both fits, the better fixed-mode block (or --search from it)
//   -o PATH            output path
//   --dump-rgba PATH   write the loaded (flipped) RGBA image as PAM and exit
//                      without encoding (no GPU needed)
#include <stdio.h>
#include <string.h>

#include <iostream>
#include <new>
#include <string>
#include <vector>

#include "../../include/astc_gb300.h"
#include "image_load.h"

namespace {

// main.cpp:130-138: cut at the last '.' of the whole path.
std::string strip_file_extension(const std::string& path) {
    const size_t dot = path.rfind('.');
    return dot == std::string::npos ? path : path.substr(0, dot);
}

int usage() {
    std::cout << "usage: astc_cs_enc input_texture [-4x4|-6x6] [-alpha] [-norm] [-srgb]"
                 " [--clamp] [--half2] [--search] [--max-accumulation] [--thorough] [--partitions]"
                 " [--three-partitions] [--best-fit]"
                 " [-o out.astc]"
                 " [--dump-rgba out.pam]" << std::endl;
    return -1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::cout << "wrong args count" << std::endl;          // main.cpp:182-185
        return usage();
    }
    const std::string src = argv[1];
    bool is4x4 = true, alpha = false, norm = false, srgb = false, clamp = false, half2 = false;
    bool search = false, max_acc = false, thorough = false, partitions = false, three = false;
    bool best_fit = false;
    std::string out_path, dump_path;
    for (int i = 2; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "-4x4") is4x4 = true;
        else if (a == "-6x6") is4x4 = false;
        else if (a == "-alpha") alpha = true;
        else if (a == "-norm") norm = true;
        else if (a == "-srgb") srgb = true;
        else if (a == "--clamp") clamp = true;
        else if (a == "--half2") half2 = true;
        else if (a == "--search") search = true;
        else if (a == "--max-accumulation") max_acc = true;
        else if (a == "--thorough") thorough = true;
        else if (a == "--partitions") partitions = true;
        else if (a == "--three-partitions") three = true;
        else if (a == "--best-fit") best_fit = true;
        else if (a == "-o" && i + 1 < argc) out_path = argv[++i];
        else if (a == "--dump-rgba" && i + 1 < argc) dump_path = argv[++i];
        else std::cerr << "ignoring unknown argument: " << a << std::endl;
    }

    std::cout << "encode option setting:\n"
              << "has_alpha\t" << std::boolalpha << alpha << std::endl
              << "is 4x4 block\t" << is4x4 << std::endl
              << "normal map\t" << norm << std::endl
              << "encode in gamma color space\t" << srgb << std::endl;

    astc::Image img;
    std::string err;
    bool loaded = false;
    try {
        loaded = astc::load_image(src, img, err);
    } catch (const std::bad_alloc&) {
        err = "out of host memory";
    }
    if (!loaded) {
        std::cout << "load source texture failed! [" << src << "] " << err << std::endl;
        return -1;
    }
    astc::flip_vertical(img);                                   // main.cpp:24
    if (!dump_path.empty()) {
        if (!astc::save_pam(dump_path, img, err)) {
            std::cout << err << std::endl;
            return -1;
        }
        std::cout << "wrote " << dump_path << std::endl;
        return 0;
    }

    astc_opts o;
    astc_opts_init(&o);
    o.block_dim = is4x4 ? 4 : 6;
    o.has_alpha = alpha;
    o.is_normal = norm;
    o.srgb = srgb && !norm;                                     // main.cpp:214
    o.border = clamp ? ASTC_BORDER_CLAMP : ASTC_BORDER_ZERO;
    o.precision = half2 ? ASTC_PRECISION_HALF2 : ASTC_PRECISION_FP32;
    o.quality = three ? ASTC_QUALITY_THREE_PARTITIONS
                : partitions ? ASTC_QUALITY_PARTITIONS
                : thorough ? ASTC_QUALITY_THOROUGH : (search ? ASTC_QUALITY_SEARCH : ASTC_QUALITY_FAST);
    o.axis = best_fit ? ASTC_AXIS_BEST : max_acc ? ASTC_AXIS_MAX_ACCUMULATION : ASTC_AXIS_PCA;
    std::vector<uint8_t> blocks(astc_encoded_size(img.width, img.height, o.block_dim));
    astc_status st = astc_encode_gpu(img.rgba.data(), img.width, img.height, &o, blocks.data());
    if (st != ASTC_OK) {
        std::cout << "encode astc failed! " << astc_status_string(st) << ": " << astc_last_error() << std::endl;
        return -1;
    }
    const std::string dst = out_path.empty() ? strip_file_extension(src) + ".astc" : out_path;
    st = astc_save_file(dst.c_str(), o.block_dim, o.block_dim, img.width, img.height, blocks.data(),
                        blocks.size());
    if (st != ASTC_OK) {
        std::cout << "save astc failed! " << astc_last_error() << std::endl;
        return -1;
    }
    std::cout << "save astc to:" << dst << std::endl;           // main.cpp:254
    astc_shutdown();
    return 0;
}
