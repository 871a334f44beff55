// Internal declarations shared by the host side of tcstencil_gb300.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>

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

// ----------------------------------------------------------------- planes --
// The engine's plane format: column panels of 16 bytes per row (8 FP16 or 4
// FP32 cells), panel after panel, rows contiguous inside a panel -- i.e.
// 16-row half-bricks (16 x 8 FP16 cells) in column-major brick order.  Rows
// are padded to a multiple of the 128-row tile plus kPadTop rows above and
// (kPadRows - kPadTop) below, columns to a multiple of the 128-column tile
// plus one panel on each side, so every tile's staged neighbourhood lies
// inside the allocation.  Cell (y, x) is at
//   ((x / cpp + 1) * nyp + (y + kPadTop)) * cpp + x % cpp.
constexpr int kTile = 128;
// Plain FP16 tensor sweeps may use narrower tiles (128 rows by 64 or 96
// columns, tcs_plan_set_tile_width): more tiles for grids with few of them.
__host__ __device__ constexpr bool valid_tile_width(int w) { return w == 64 || w == 96 || w == kTile; }
constexpr int kPadTop = 4;
constexpr int kPadRows = 8;

__host__ __device__ constexpr int round_up(int a, int b) { return (a + b - 1) / b * b; }

struct PlaneGeom {
    int nyp;   // rows per panel, padding included
    int npan;  // panels, padding included
    int cpp;   // cells per panel row: 8 (FP16) or 4 (FP32)
};

__host__ __device__ inline PlaneGeom plane_geom(int ny, int nx, int cpp) {
    PlaneGeom p;
    p.nyp = round_up(ny, kTile) + kPadRows;
    p.npan = round_up(nx, kTile) / cpp + 2;
    p.cpp = cpp;
    return p;
}
__host__ __device__ inline size_t plane_elems(const PlaneGeom &p) {
    return (size_t)p.nyp * p.npan * p.cpp;
}
// Index of cell (y, x) for y >= -kPadTop and x >= -cpp (x a multiple of cpp
// or any column of a panel).
__host__ __device__ inline size_t plane_index(const PlaneGeom &p, int y, int x) {
    const int xs = x + p.cpp;
    return ((size_t)(xs / p.cpp) * p.nyp + (size_t)(y + kPadTop)) * p.cpp + (size_t)(xs % p.cpp);
}

// Geometry of one grid and its update rectangle.
struct GridGeom {
    int ny, nx;  // cells
    int y0, y1, x0, x1;
    PlaneGeom p16;  // FP16 (and split) planes
    PlaneGeom p32;  // FP32 planes
};

// Tensor map of an FP16 (or split hi/lo) panel plane for the tensor-core
// sweeps, in whole 128-byte lines: elements are 8-byte words, dimensions
// (16 words = 8 rows of a panel, nyp / 8 row groups, npan panels), box
// (16, 17, 18) = the 136 rows from Y0 - 4 of the 18 panels a 128 x 128 tile
// reads, landing in shared memory as 18 row-contiguous 2176-byte runs (one
// load instruction per plane and tile instead of 18 bulk copies).
cudaError_t encode_panel_map(const uint16_t *plane, const PlaneGeom &pg, CUtensorMap *map);

// Sets the thread's last-error message and returns `status`.
int fail(int status, const char *fmt, ...);
// Maps a CUDA runtime error to TCS_ERR_CUDA with a message (TCS_OK if none).
int cuda_status(cudaError_t e, const char *what);

// The library's device and pinned-host allocations (memory.cu): the
// allocation hook and guard regions of include/tcs.h apply to them.  A
// failure returns TCS_ERR_NOMEM (or TCS_ERR_CUDA) with *p null and the
// message naming `what`.
int dev_alloc(void **p, size_t bytes, const char *what);
int host_alloc(void **p, size_t bytes, const char *what);
void dev_free(void *p);
void host_free(void *p);
// Guard regions inside the library's own memory: the guard size in force
// (0: off); guard_place fills bytes at p with the canary on stream s and
// has tcs_guard_check watch them; guard_forget stops watching, after
// comparing them with the canary (check; the work that touched them must be
// complete) and counting a damaged region.
size_t guard_bytes();
int guard_place(void *p, size_t bytes, const char *what, cudaStream_t s);
void guard_forget(void *p, bool check);
template <typename T>
int dev_alloc_t(T **p, size_t bytes, const char *what) {
    return dev_alloc(reinterpret_cast<void **>(p), bytes, what);
}
template <typename T>
int host_alloc_t(T **p, size_t bytes, const char *what) {
    return host_alloc(reinterpret_cast<void **>(p), bytes, what);
}

// Fills `geom` (validating the rectangle) for a stencil; returns a status.
int make_geom(int ny, int nx, int stencil, int y0, int y1, int x0, int x1, GridGeom *geom);
// Gold's coefficients for a stencil from an n x n row-major matrix.
TapCoeffs tap_coeffs(int stencil, const float *B);

// Scale exponent of a split-precision grid: values are stored as x 2^-E,
// with E the smallest integer such that max|x| 2^-E <= 1 (0 for max|x| = 0).
int split_scale_exp(float max_abs);
// Sum of |c| over a stencil's taps (the split form needs it <= 1 + 2^-8).
double tap_abs_sum(int stencil, const float *B);
constexpr double kSplitMaxAbsSum = 1.0 + 1.0 / 256.0;

// --- kernels (launch wrappers; return cudaError_t of the launch) ---------
cudaError_t launch_cc_f16(const GridGeom &g, int stencil, const TapCoeffs &c, const uint16_t *in,
                          uint16_t *out, cudaStream_t s);
cudaError_t launch_cc_f32(const GridGeom &g, int stencil, const TapCoeffs &c, const float *in,
                          float *out, cudaStream_t s);

// Reads and clears the tensor kernels' device error word.
cudaError_t tc_take_error(int *code);
struct SplitScale;
// Split launches take the grid's per-step scale (SplitScale below; null: the
// fixed scale of the planes as packed) and t0, the steps of the current run
// done before the launch.
// Two steps of the split form in one launch (temporal blocking), in -> out.
cudaError_t launch_tc_split2(const GridGeom &g, int stencil, const float *B, const uint16_t *in_hi,
                             const uint16_t *in_lo, uint16_t *out_hi, uint16_t *out_lo,
                             cudaStream_t s, SplitScale *scale = nullptr, int t0 = 0);
cudaError_t tb_take_error(int *code);
// Reads and clears the CUDA-core kernels' device error word.
cudaError_t cc_take_error(int *code);
// Configures the tensor kernel of (stencil, split) ahead of its first launch.
cudaError_t tc_prepare(int stencil, bool split);

cudaError_t launch_tc_f16(const GridGeom &g, int stencil, const float *B, const uint16_t *in,
                          uint16_t *out, cudaStream_t s, int tile_w = kTile);
// Several plain steps in one launch (in -> out -> in ...); rows_done: one
// counter per tile row (ceil(ny / 128)) every kRowCounterStride unsigneds,
// zeroed before the launch.  Each counter has its own 128-byte line: every SM
// polls and counts them, and on shared lines those accesses serialise.
constexpr int kRowCounterStride = 32;
cudaError_t launch_tc_f16_steps(const GridGeom &g, int stencil, const float *B, const uint16_t *in,
                                uint16_t *out, int steps, unsigned *rows_done, cudaStream_t s,
                                int tile_w = kTile);
cudaError_t launch_tc_split_steps(const GridGeom &g, int stencil, const float *B,
                                  const uint16_t *in_hi, const uint16_t *in_lo, uint16_t *out_hi,
                                  uint16_t *out_lo, int steps, unsigned *rows_done, cudaStream_t s,
                                  SplitScale *scale = nullptr, int t0 = 0);
cudaError_t launch_tc_split(const GridGeom &g, int stencil, const float *B, const uint16_t *in_hi,
                            const uint16_t *in_lo, uint16_t *out_hi, uint16_t *out_lo,
                            cudaStream_t s, SplitScale *scale = nullptr, int t0 = 0);

// --- layout kernels -------------------------------------------------------
// pack/unpack between an FP32 row-major grid and an engine plane of the
// (ny + 2 pad) x (nx + 2 pad) padded grid; every plane cell is written by
// pack (cells outside the padded grid are 0).
cudaError_t launch_pack_f16(const float *in, int ny, int nx, int pad, float pad_value,
                            uint16_t *plane, cudaStream_t s);
cudaError_t launch_unpack_f16(const uint16_t *plane, int ny, int nx, int pad, float *out,
                              cudaStream_t s);
cudaError_t launch_pack_f32(const float *in, int ny, int nx, int pad, float pad_value,
                            float *plane, cudaStream_t s);
cudaError_t launch_unpack_f32(const float *plane, int ny, int nx, int pad, float *out,
                              cudaStream_t s);
cudaError_t launch_pack_split(const float *in, int ny, int nx, int pad, float pad_value,
                              int scale_exp, uint16_t *hi, uint16_t *lo, cudaStream_t s);
cudaError_t launch_unpack_split(const uint16_t *hi, const uint16_t *lo, int ny, int nx, int pad,
                                int scale_exp, float *out, cudaStream_t s);
// max |x| over n floats into *out_bits (float bits; *out_bits must start at 0)
// Split pack/unpack (pad 0) with the scale exponent kept in device memory:
// pack derives E from the max-|x| bits that launch_max_abs left and stores it.
cudaError_t launch_pack_split_dev(const float *in, int ny, int nx, const unsigned *max_bits,
                                  int *exp_out, uint16_t *hi, uint16_t *lo, cudaStream_t s);
cudaError_t launch_unpack_split_dev(const uint16_t *hi, const uint16_t *lo, int ny, int nx,
                                    const int *exp_in, float *out, cudaStream_t s);
cudaError_t launch_max_abs(const float *in, size_t n, unsigned *out_bits, cudaStream_t s);
// FP16 (f32 false) or FP32 plane rows [q0, q1) from / to an ny x nx
// row-major grid, no padding; the grid rows involved are [q0 - 4, q1 - 4)
// clipped to [0, ny).
cudaError_t launch_pack_rows(const float *in, int ny, int nx, bool f32, void *plane, int q0,
                             int q1, cudaStream_t s);
cudaError_t launch_unpack_rows(const void *plane, int ny, int nx, bool f32, float *out, int q0,
                               int q1, cudaStream_t s);

// ------------------------------------------------ split scale, per step ---
// A split grid holds x' = x 2^-E as hi + lo 2^-11 with a fixed-point hi, so
// its precision is about 2^-23 of 2^E.  E follows the grid's magnitude step
// by step, so a field that decays keeps FP32-level relative precision:
//   E_t = E_{t-2} + e(M_{t-2}),   k_t = E_{t-1} - E_t,
// where M_t = max(the largest |x'| step t stores in its update rectangle,
// B 2^(E_B - E_t)) in step t's units, B the largest |x'| of the grid's
// cells outside the update rectangle (its fixed border) as uploaded, in the
// units of the upload's exponent E_B, and e(M) the frexp exponent of M
// (M 2^-e in [0.5, 1)), taken as max(e(m), e(B) + E_B - E_t) of the parts
// present (a zero or subnormal part is absent; no part, or a non-finite m:
// 0), clamped to [-64, 64].  The border keeps its values, so its share of M
// needs no pass over its cells.  Step t multiplies its values by 2^k_t
// before the split (cells it only copies are re-split by the same factor
// when k_t != 0).  Step t reads only steps t-2 and t-3, which every form of
// the sweep (one launch per step, several steps per launch, blocked pairs,
// batches) has completed by then, so every form gives the same bits.  Slots
// are the step index within a run (1..T) mod 8; slots 7 and 0 hold steps -1
// and 0 (the run's starting history), which launch_split_scale_end_run moves
// into place after each run; after an upload their maxima are the non-finite
// mark, e = 0.  Step t writes M_t (its part m) and E_t into slot t and clears
// the maximum of slot t+3 (whose readers, steps t-3 and t-2, have finished,
// and whose next writer, step t+3, starts after step t has).
constexpr int kScaleRing = 8;
constexpr unsigned kScaleNoMax = 0xffffffffu;  // a slot's maximum before any step: e = 0
struct SplitScale {
    unsigned maxbits[kScaleRing];  // m of M_t as FP32 bits (atomicMax of non-negative floats)
    int exp[kScaleRing];           // E_t
    unsigned bmax;                 // B as FP32 bits
    int bexp;                      // E_B
};
// From the max-|x| bits launch_max_abs left for a grid's input: E_0 = E_B =
// the pack's exponent, steps -1 and 0 marked as unmeasured, and B from the
// packed planes (hi, lo) of the grid g.
cudaError_t launch_split_scale_init(SplitScale *sc, const unsigned *max_bits, const GridGeom &g,
                                    const uint16_t *hi, const uint16_t *lo, cudaStream_t s);
// After a run of `steps` steps: steps T-1 and T become slots 7 and 0, the
// maxima of slots 1..6 are cleared.
cudaError_t launch_split_scale_end_run(SplitScale *sc, int steps, cudaStream_t s);
// The exponent of a split grid's state between runs (slot 0).
inline const int *split_scale_exp_ptr(const SplitScale *sc) { return &sc->exp[0]; }

// Whether step kernels launch with programmatic stream serialization (the
// next step's CTAs set up while the previous step's last tiles finish, and
// wait in griddepcontrol.wait before touching a plane).  TCS_PDL=0 in the
// environment launches in plain stream order.
inline bool pdl_enabled() {
    static const bool on = [] {
        const char *e = getenv("TCS_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}
// the reference's layout16 transforms (bricks of 16 x 16, row-major inside)
cudaError_t launch_padding_2d(const uint16_t *in, uint16_t *out, int size, int halo,
                              uint16_t value, cudaStream_t s);
cudaError_t launch_brick_2d(const uint16_t *in, uint16_t *out, int ny, int nx, cudaStream_t s);
cudaError_t launch_unbrick_2d(const uint16_t *in, uint16_t *out, int ny, int nx, cudaStream_t s);

}  // namespace tcs
