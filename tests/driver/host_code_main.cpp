// A driver shaped like the reference's common/main_1r.cu and main_2r.cu, for
// the per-variant host_code libraries (libtcs_host_<engine>_<stencil>.so).
// It declares host_code exactly as common/main_1r.cu:7 does, sets the
// coefficients as init_B does (B[i] = i with the centre -40 for 3 x 3 and
// -290 for 5 x 5, common/main_1r.cu:10-16, common/main_2r.cu:13-19), and
// calls host_code once on a MESH_SIZE x MESH_SIZE grid, as main() does
// (common/main_1r.cu:28).  Unlike the reference's drivers, whose inputs are
// all 1.0 (common/common.hpp:19-21), it reads h_A from the file argv[1] and
// writes h_C to the file argv[2], so that a test can check the result
// against gold.  Test infrastructure (tests/test_driver_gpu.py builds it).
#include <cstdio>
#include <cstdlib>
#include <vector>

extern "C" void host_code(float *h_A, float *h_B, float *h_C, int N, int n);

#ifndef MESH_SIZE
#error "define MESH_SIZE"
#endif
#ifndef STENCIL_SIZE
#error "define STENCIL_SIZE (3 or 5)"
#endif

static void init_B(float *B) {
    for (int i = 0; i < STENCIL_SIZE * STENCIL_SIZE; i++) B[i] = (float)i;
    B[STENCIL_SIZE * STENCIL_SIZE / 2] = STENCIL_SIZE == 3 ? -40.0f : -290.0f;
}

int main(int argc, char **argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s <A.f32> <C.f32>\n", argv[0]);
        return 2;
    }
    const size_t cells = (size_t)MESH_SIZE * MESH_SIZE;
    std::vector<float> h_A(cells), h_C(cells, 0.0f), h_B(STENCIL_SIZE * STENCIL_SIZE);
    FILE *f = fopen(argv[1], "rb");
    if (!f || fread(h_A.data(), sizeof(float), cells, f) != cells) return 2;
    fclose(f);
    init_B(h_B.data());
    host_code(h_A.data(), h_B.data(), h_C.data(), MESH_SIZE, STENCIL_SIZE);
    f = fopen(argv[2], "wb");
    if (!f || fwrite(h_C.data(), sizeof(float), cells, f) != cells) return 2;
    fclose(f);
    return 0;
}
