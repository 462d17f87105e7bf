// Test harness: reads every file named on the command line with the command
// line tool's image reader (load_image), ignoring the result.  Built with
// address and undefined-behaviour sanitizers by test_cli.py, which feeds it
// corrupted images; a sanitizer report makes the process fail.
#include <string>

#include "image_load.h"

int main(int argc, char** argv) {
    for (int i = 1; i < argc; ++i) {
        astc::Image img;
        std::string err;
        (void)astc::load_image(argv[i], img, err);
    }
    return 0;
}
