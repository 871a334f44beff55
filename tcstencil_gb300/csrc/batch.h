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
    int ny, nx;             // cells (beyond them: plane padding)
    int y0, y1, x0, x1;
    int tiles_x;
    int n_tiles;
    int r, box, split;
    int steps;      // steps in one run
    int ctr_base;   // completion counter of step 0 of the run
    int band_base;  // first band element in the band buffer
    int state;      // which plane holds the current state
    // external gate: step 0 starts once *gate >= gate_value (null: no gate)
    const unsigned *gate;
    unsigned gate_value;
    // tensor maps of the planes in device memory, [state][hi, lo] (lo = hi for
    // FP16 grids), from encode_grid_maps
    const CUtensorMap *maps;
    // split grids: the per-step scale (SplitScale; step t of a run is slot t+1)
    SplitScale *scale;
};

// Encodes the four tensor maps of a grid's planes ([state][hi, lo]).
inline cudaError_t encode_grid_maps(const BatchGrid &g, CUtensorMap out[4]) {
    for (int s = 0; s < 2; s++)
        for (int pl = 0; pl < 2; pl++) {
            const uint16_t *plane = (pl && g.plane[s][1]) ? g.plane[s][1] : g.plane[s][0];
            const cudaError_t e = encode_panel_map(plane, g.pg, &out[2 * s + pl]);
            if (e != cudaSuccess) return e;
        }
    return cudaSuccess;
}

struct BatchItem {
    int g, t, tile;  // grid, step within the run, tile
    int ty, tx;      // the tile's row and column (set by the producer when it publishes)
};

// Split items: the step's scale (StepScale of tc_core.cuh, as s, k, e) and
// the grid's scale record, set by the producer once the step's inputs are
// final (after the item is published, so a separate barrier per slot).
struct ItemScale {
    float s;
    int k, e;
    SplitScale *sc;
};

// One run's work: items are ordered step major and, within a step, by grid
// then tile.  Grids are sorted by step count (descending), so the grids still
// running at step t are a prefix of the array: step t holds the first
// tile_prefix[G_t] tiles of the concatenated grids, and work index k decodes
// with two binary searches (step_off, then tile_prefix).
struct BatchParams {
    const BatchGrid *grids;  // [n_grids], steps descending
    const int *step_off;     // [n_steps + 1]: first work index of each step
    const int *tile_prefix;  // [n_grids + 1]: first tile of each grid within a step
    int n_steps, n_grids, n_items;
    unsigned *counters;      // one per (grid, step), kRowCounterStride apart, zero at launch
    unsigned *work_counter;  // next work index, zero at launch
    int *error;              // first failed wait of this launch (0 = none)
    const uint16_t *bands;
    unsigned long long wait_ns;  // limit of the dependency and gate waits
    int grab;                    // work indices taken per atomic (batch_grab)
};

// Work indices a CTA takes per atomic: consecutive items mostly share a grid
// (one dependency poll, incremental decode), but a small grid's tiles then
// run on fewer SMs one after another, lengthening its step-to-step chain.
// Measured on GB300 with 512 mixed grids: 4 for FP16 items, BATCH_GRAB_SPLIT
// for the longer split items.
#ifndef BATCH_GRAB_SPLIT
#define BATCH_GRAB_SPLIT 1
#endif
constexpr int batch_grab(bool split) { return split ? BATCH_GRAB_SPLIT : 4; }

// Default limit of a batched run's dependency and gate waits: one second.
constexpr unsigned long long kBatchWaitNs = 1000000000ull;

// Fills step_off and tile_prefix for grids whose run steps (descending) and
// tile counts are given; returns the number of work items, or -1 when it
// would not fit an int.
inline long long batch_layout(const int *steps, const int *tiles, int n_grids, int *step_off,
                              int *tile_prefix) {
    tile_prefix[0] = 0;
    for (int i = 0; i < n_grids; i++) tile_prefix[i + 1] = tile_prefix[i] + tiles[i];
    const int n_steps = n_grids ? steps[0] : 0;
    long long off = 0;
    int g = n_grids;  // grids with steps > t
    step_off[0] = 0;
    for (int t = 0; t < n_steps; t++) {
        while (g > 0 && steps[g - 1] <= t) g--;
        off += tile_prefix[g];
        if (off > 0x7fffffffLL) return -1;
        step_off[t + 1] = static_cast<int>(off);
    }
    return off;
}

// Band bytes of one grid's stencil in the band buffer (FP16 or four split
// pieces, 2r+1 coefficient rows).
__host__ __device__ inline int batch_band_elems(int r, bool split) { return (split ? 4 : 1) * (2 * r + 1) * 512; }
constexpr int kBatchMaxBandElems = 4 * 5 * 512;

// Sets the kernel attributes and returns the SM count (the launch grid).
cudaError_t batch_prepare(int *num_sms);
// One persistent launch over p's work (all grids of one precision: split or
// FP16); grid = min(items, SMs).  A run launches one per precision present.
// A split launch is followed by the end of the run of every split grid's
// scale record (as launch_split_scale_end_run, with the grid's steps).
cudaError_t launch_batch(const BatchParams &p, bool split, int num_sms, cudaStream_t s);
// Bands of one stencil (coefficients n x n row-major, n = 2r+1) into dst.
cudaError_t launch_build_bands(const float *coef, int r, bool box, bool split, uint16_t *dst,
                               cudaStream_t s);
cudaError_t batch_take_error(int *code);

}  // namespace tcs
