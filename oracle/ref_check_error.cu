// Runs the reference's own error metrics, checkError2D and
// checkRelativeError2D (common/common.hpp:38-92), unchanged: this file only
// includes the reference header and feeds it.  Built by `make -C oracle ref`
// into _ref/ref_check_error (test infrastructure: tests/golden/make_golden.py
// records what it prints into fixtures that pin oracle_check_error_2d).
//
//   ref_check_error <file>
// <file>: int32 N, y_lb, y_ub, x_lb, x_ub, then N*N float32 output, then
// N*N float32 reference.  Prints the metrics' own lines, then
//   RMS <checkError2D result>
//   REL <checkRelativeError2D result>
#include <cstdio>
#include <vector>

#include "common.hpp"

int main(int argc, char **argv) {
    if (argc != 2) return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[5];
    if (fread(hdr, sizeof(int), 5, f) != 5) return 2;
    const int N = hdr[0];
    std::vector<float> out((size_t)N * N), ref((size_t)N * N);
    if (fread(out.data(), sizeof(float), out.size(), f) != out.size()) return 2;
    if (fread(ref.data(), sizeof(float), ref.size(), f) != ref.size()) return 2;
    fclose(f);
    double rms = checkError2D(N, out.data(), ref.data(), hdr[1], hdr[2], hdr[3], hdr[4]);
    printf("RMS %.17g\n", rms);
    double rel = checkRelativeError2D(N, out.data(), ref.data(), hdr[1], hdr[2], hdr[3], hdr[4]);
    printf("REL %.17g\n", rel);
    return 0;
}
