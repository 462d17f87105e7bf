// image_load.h -- image reader for the command line tool.  PNG (own inflate,
// RFC 1950/1951; every colour type and bit depth, 16-bit channels reduced to
// their high byte, 1/2/4-bit grey scaled to 8; Adam7; tRNS), JPEG (8-bit grey
// or YCbCr, Huffman coded, baseline or progressive), Photoshop PSD (the merged
// image; 8/16-bit grey or RGB, optional alpha), GIF (the first image;
// transparency as (0, 0, 0, 0)), Radiance HDR (RGBE, taken to 8 bits with
// gamma 1/2.2), Windows BMP (1/4/8-bit palettes, 16/24/32-bit, bit fields),
// Truevision TGA (colour-mapped, 15/16/24/32-bit true colour, 8-bit grey; raw
// or run-length), Softimage PIC and Netpbm P5/P6/P7.
// Output is always RGBA8, row 0 first (the caller flips for the reference's
// orientation, main.cpp:24).  Written for this project; the reference uses
// the third-party stb_image for the same job.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

namespace astc {

struct Image {
    int width = 0, height = 0;
    std::vector<uint8_t> rgba;     // width * height * 4
};

// Returns true on success; on failure `err` says why.
bool load_image(const std::string& path, Image& out, std::string& err);
bool decode_png(const uint8_t* data, size_t size, Image& out, std::string& err);
bool decode_pnm(const uint8_t* data, size_t size, Image& out, std::string& err);
bool decode_bmp(const uint8_t* data, size_t size, Image& out, std::string& err);
bool decode_tga(const uint8_t* data, size_t size, Image& out, std::string& err);
bool decode_jpeg(const uint8_t* data, size_t size, Image& out, std::string& err);
bool decode_psd(const uint8_t* data, size_t size, Image& out, std::string& err);
bool decode_gif(const uint8_t* data, size_t size, Image& out, std::string& err);
bool decode_hdr(const uint8_t* data, size_t size, Image& out, std::string& err);
bool decode_pic(const uint8_t* data, size_t size, Image& out, std::string& err);
// zlib stream (2-byte header, deflate blocks, Adler-32) -> raw bytes.
bool zlib_inflate(const uint8_t* data, size_t size, std::vector<uint8_t>& out, std::string& err);
// Writes RGBA8 as a P7 (PAM) file.
bool save_pam(const std::string& path, const Image& img, std::string& err);
void flip_vertical(Image& img);

}  // namespace astc
