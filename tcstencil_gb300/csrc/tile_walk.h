// A CTA's items k0, k0 + stride, k0 + 2 stride, ... of a multi-step launch
// as (step, tile row, tile column), without a division per item: item k is
// step * tiles_y * tiles_x + ty * tiles_x + tx.  Shared by the sweep kernels
// and a host test of the index sequences.
#pragma once

#ifdef __CUDACC__
#define TCS_WALK_FN __host__ __device__ __forceinline__
#else
#define TCS_WALK_FN inline
#endif

namespace tcs {

struct TileWalk {
    int step, ty, tx, dy, dx, tiles_x, tiles_y;

    TCS_WALK_FN void init(int k0, int stride, int tiles_x_, int tiles_y_) {
        tiles_x = tiles_x_;
        tiles_y = tiles_y_;
        const int n_tiles = tiles_x * tiles_y;
        step = k0 / n_tiles;
        const int t = k0 - step * n_tiles;
        ty = t / tiles_x;
        tx = t - ty * tiles_x;
        dy = stride / tiles_x;
        dx = stride - dy * tiles_x;
    }
    TCS_WALK_FN void advance() {
        tx += dx;
        ty += dy;
        if (tx >= tiles_x) {
            tx -= tiles_x;
            ty++;
        }
        while (ty >= tiles_y) {
            ty -= tiles_y;
            step++;
        }
    }
};

}  // namespace tcs
