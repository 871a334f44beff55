// Internal declarations shared by the host side of tcstencil_gb300.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tcs.h"

namespace tcs {

// Gold's tap order (common/gold_*.cpp): star2d1r = up, centre, down, left,
// right (gold_star2d1r.cpp:10-12); star2d2r = column top to bottom, then the
// row left to right without the centre (gold_star2d2r.cpp:10-14); box = row
// major over the n x n window (gold_box2d1r.cpp:11-13, gold_box2d2r.cpp:11-13).
__host__ __device__ constexpr int tap_count(int s) {
    return s == TCS_STAR2D1R ? 5 : s == TCS_STAR2D2R ? 9 : s == TCS_BOX2D1R ? 9 : 25;
}
__host__ __device__ constexpr int stencil_r(int s) {
    return (s == TCS_STAR2D1R || s == TCS_BOX2D1R) ? 1 : 2;
}
__host__ __device__ constexpr bool stencil_box(int s) {
    return s == TCS_BOX2D1R || s == TCS_BOX2D2R;
}
__host__ __device__ constexpr int tap_dy(int s, int k) {
    return s == TCS_STAR2D1R   ? (k < 3 ? k - 1 : 0)
           : s == TCS_STAR2D2R ? (k < 5 ? k - 2 : 0)
           : s == TCS_BOX2D1R  ? k / 3 - 1
                               : k / 5 - 2;
}
__host__ __device__ constexpr int tap_dx(int s, int k) {
    return s == TCS_STAR2D1R   ? (k < 3 ? 0 : (k == 3 ? -1 : 1))
           : s == TCS_STAR2D2R ? (k < 5 ? 0 : (k == 5 ? -2 : k == 6 ? -1 : k == 7 ? 1 : 2))
           : s == TCS_BOX2D1R  ? k % 3 - 1
                               : k % 5 - 2;
}

// Coefficients in gold's tap order, passed by value (constant bank).
struct TapCoeffs {
    float c[25];
};

// Geometry of one brick grid and its update rectangle.
struct GridGeom {
    int ny, nx;   // cells
    int nby, nbx; // bricks
    int y0, y1, x0, x1;
};

// Sets the thread's last-error message and returns `status`.
int fail(int status, const char *fmt, ...);
// Maps a CUDA runtime error to TCS_ERR_CUDA with a message (TCS_OK if none).
int cuda_status(cudaError_t e, const char *what);

// Fills `geom` (validating the rectangle) for a stencil; returns a status.
int make_geom(int ny, int nx, int stencil, int y0, int y1, int x0, int x1, GridGeom *geom);
// Gold's coefficients for a stencil from an n x n row-major matrix.
TapCoeffs tap_coeffs(int stencil, const float *B);

// --- kernels (launch wrappers; return cudaError_t of the launch) ---------
cudaError_t launch_cc_f16(const GridGeom &g, int stencil, const TapCoeffs &c, const uint16_t *in,
                          uint16_t *out, cudaStream_t s);
cudaError_t launch_cc_f32(const GridGeom &g, int stencil, const TapCoeffs &c, const float *in,
                          float *out, cudaStream_t s);

// Tensor-core tile: 8 bricks (128 rows) high; 8 bricks wide in the FP16 form
// and 6 in the split form (whose two accumulators per tile take more TMEM).
constexpr int kTcTileBricksY = 8;
__host__ __device__ constexpr int tc_tile_bricks_x(bool split) { return split ? 6 : 8; }

// Tensor maps of one FP16 brick plane for the tensor-core kernel.
struct PlaneMaps {
    CUtensorMap main; // box: 8 x 16 x (tile bricks y + 2) x 2 x (tile bricks x)
    CUtensorMap halo; // box: 8 x 16 x (tile bricks y + 2) x 1 x 1
};
int encode_plane_maps(const void *plane, int nby, int nbx, int tile_bricks_x, PlaneMaps *maps);

// Scale exponent of a split-precision grid: values are stored as x 2^-E,
// with E the smallest integer such that max|x| 2^-E <= 1 (0 for max|x| = 0).
int split_scale_exp(float max_abs);
// Sum of |c| over a stencil's taps (the split form needs it <= 1 + 2^-8).
double tap_abs_sum(int stencil, const float *B);
constexpr double kSplitMaxAbsSum = 1.0 + 1.0 / 256.0;

// Reads and clears the tensor kernels' device error word.
cudaError_t tc_take_error(int *code);
// Configures the tensor kernel of (stencil, split) ahead of its first launch.
cudaError_t tc_prepare(int stencil, bool split);

cudaError_t launch_tc_f16(const GridGeom &g, int stencil, const float *B, const PlaneMaps &in_maps,
                          const uint16_t *in, uint16_t *out, cudaStream_t s);
cudaError_t launch_tc_split(const GridGeom &g, int stencil, const float *B,
                            const PlaneMaps &in_hi_maps, const PlaneMaps &in_lo_maps,
                            const uint16_t *in_hi, const uint16_t *in_lo, uint16_t *out_hi,
                            uint16_t *out_lo, cudaStream_t s);

// --- layout kernels -------------------------------------------------------
cudaError_t launch_pack_f16(const float *in, int ny, int nx, int pad, float pad_value,
                            uint16_t *bricks, cudaStream_t s);
cudaError_t launch_unpack_f16(const uint16_t *bricks, int ny, int nx, int pad, float *out,
                              cudaStream_t s);
cudaError_t launch_pack_f32(const float *in, int ny, int nx, int pad, float pad_value,
                            float *bricks, cudaStream_t s);
cudaError_t launch_unpack_f32(const float *bricks, int ny, int nx, int pad, float *out,
                              cudaStream_t s);
cudaError_t launch_pack_split(const float *in, int ny, int nx, int pad, float pad_value,
                              int scale_exp, uint16_t *hi, uint16_t *lo, cudaStream_t s);
cudaError_t launch_unpack_split(const uint16_t *hi, const uint16_t *lo, int ny, int nx, int pad,
                                int scale_exp, float *out, cudaStream_t s);
// max |x| over n floats into *out_bits (float bits; *out_bits must start at 0)
cudaError_t launch_max_abs(const float *in, size_t n, unsigned *out_bits, cudaStream_t s);
cudaError_t launch_padding_2d(const uint16_t *in, uint16_t *out, int size, int halo,
                              uint16_t value, cudaStream_t s);
cudaError_t launch_brick_2d(const uint16_t *in, uint16_t *out, int ny, int nx, cudaStream_t s);
cudaError_t launch_unbrick_2d(const uint16_t *in, uint16_t *out, int ny, int nx, cudaStream_t s);

}  // namespace tcs
