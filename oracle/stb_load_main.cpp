/*
 * stb_load_main.cpp -- TEST INFRASTRUCTURE ONLY.  A command line harness over
 * the reference's own image loader, stb_image.h of niepp/astc_encoder, which
 * stays in the reference tree: `make -C oracle stb-ref REFERENCE=<tree>`
 * compiles this file with that tree on the include path into
 * oracle/_ref/stb_load.  The image reader tests compare the repo's readers
 * (the CLI's C++ reader and astc_encoder_gb300.image_io) with it.
 *
 * Usage: stb_load <image> <out.raw>
 * Loads <image> with stbi_load(..., 4) -- RGBA8, rows top-down, as the
 * reference's load_tex (main.cpp:23-24) does before its vertical flip -- and
 * writes "w h\n" followed by w*h*4 bytes to <out.raw>.  Prints the failure
 * reason and exits 2 when stb_image refuses the file.
 */
#define STB_IMAGE_IMPLEMENTATION
#include "stb_image.h"

#include <stdio.h>

int main(int argc, char** argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s <image> <out.raw>\n", argv[0]);
        return 1;
    }
    int w = 0, h = 0, comp = 0;
    stbi_uc* px = stbi_load(argv[1], &w, &h, &comp, 4);
    if (!px) {
        printf("refused: %s\n", stbi_failure_reason());
        return 2;
    }
    FILE* f = fopen(argv[2], "wb");
    if (!f) {
        stbi_image_free(px);
        return 1;
    }
    fprintf(f, "%d %d\n", w, h);
    fwrite(px, 1, (size_t)w * h * 4, f);
    fclose(f);
    stbi_image_free(px);
    return 0;
}
