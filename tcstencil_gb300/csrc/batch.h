// Work description of the batched persistent tensor-core sweep (batch.cu),
// shared by the static batches of the C-ABI and the request server
// (server.cu).
#pragma once

#include <cstdint>

#include "tcs_internal.h"

namespace tcs {

struct BatchGrid {
    uint16_t *plane[2][2];  // [ping-pong state][hi, lo]
    PlaneGeom pg;
    int y0, y1, x0, x1;
    int tiles_x;
    int n_tiles;
    int r, box, split;
    int steps;      // steps in one run
    int ctr_base;   // completion counter of step 0 of the run
    int band_base;  // first band element in the band buffer
    int state;      // which plane holds the current state
};

struct BatchItem {
    int g, t, tile;  // grid, step within the run, tile
};

struct BatchParams {
    const BatchGrid *grids;
    const BatchItem *items;
    int n_items;
    unsigned *counters;  // one per (grid, step), zero at launch
    const uint16_t *bands;
};

// Band bytes of one grid's stencil in the band buffer (FP16 or four split
// pieces, 2r+1 coefficient rows).
inline int batch_band_elems(int r, bool split) { return (split ? 4 : 1) * (2 * r + 1) * 512; }
constexpr int kBatchMaxBandElems = 4 * 5 * 512;

// Sets the kernel attributes and returns the SM count (the launch grid).
cudaError_t batch_prepare(int *num_sms);
// One persistent launch over p's work list; grid = min(items, SMs).
cudaError_t launch_batch(const BatchParams &p, int num_sms, cudaStream_t s);
// Bands of one stencil (coefficients n x n row-major, n = 2r+1) into dst.
cudaError_t launch_build_bands(const float *coef, int r, bool box, bool split, uint16_t *dst,
                               cudaStream_t s);
cudaError_t batch_take_error(int *code);

}  // namespace tcs
