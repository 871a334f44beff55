"""Index sequences of the multi-step launches, checked on the CPU.

Every role of a multi-step sweep (producer, MMA issuers, epilogue, signal)
walks its CTA's items k0, k0 + stride, ... with TileWalk
(tcstencil_gb300/csrc/tile_walk.h) instead of dividing per item.  This
compiles the header as host C++ and checks each walk against
(k // n_tiles, (k % n_tiles) // tiles_x, k % tiles_x) over ragged grids: one
tile, one tile row or column, more CTAs than tiles, strides above the tile
count.  A wrong row here would make a tile count its completion on the wrong
counter, which the kernels only notice as a wait that runs out.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER_DIR = os.path.join(ROOT, "tcstencil_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include "tile_walk.h"
int main() {
    int tiles_x, tiles_y, steps, stride, k0;
    while (std::scanf("%d %d %d %d %d", &tiles_x, &tiles_y, &steps, &stride, &k0) == 5) {
        tcs::TileWalk w;
        w.init(k0, stride, tiles_x, tiles_y);
        const long n_items = (long)tiles_x * tiles_y * steps;
        for (long k = k0; k < n_items; k += stride, w.advance())
            std::printf("%d %d %d\n", w.step, w.ty, w.tx);
        std::printf("end\n");
    }
    return 0;
}
"""

CASES = [(1, 1, 5, 152), (65, 65, 3, 152), (129, 129, 2, 152), (3, 2, 7, 42), (2, 9, 9, 18),
         (1, 3, 50, 152), (7, 1, 40, 152), (65, 65, 2, 456), (4, 4, 30, 152), (33, 33, 4, 304)]


@pytest.fixture(scope="module")
def walker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("walk")
    src = d / "walk.cpp"
    src.write_text(PROGRAM)
    exe = d / "walk"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", HEADER_DIR, str(src), "-o", str(exe)],
                   check=True, timeout=120)
    return str(exe)


@pytest.mark.parametrize("tiles_x,tiles_y,steps,grid", CASES)
def test_walks_match_division(walker, tiles_x, tiles_y, steps, grid):
    n_tiles = tiles_x * tiles_y
    n_items = n_tiles * steps
    grid = min(grid, n_items)
    # every CTA's walk, and the issuers' (3 issuers: stride 3 * grid)
    starts = [(grid, b) for b in range(grid)] + [(3 * grid, b + i * grid)
                                                 for b in range(min(grid, 9)) for i in range(3)]
    stdin = "".join(f"{tiles_x} {tiles_y} {steps} {s} {k0}\n" for s, k0 in starts)
    out = subprocess.run([walker], input=stdin, capture_output=True, text=True, check=True,
                         timeout=120).stdout.split("end\n")
    for (stride, k0), block in zip(starts, out):
        got = [tuple(map(int, line.split())) for line in block.strip().splitlines()]
        want = [(k // n_tiles, (k % n_tiles) // tiles_x, k % tiles_x)
                for k in range(k0, n_items, stride)]
        assert got == want, (tiles_x, tiles_y, steps, stride, k0)
        assert all(0 <= ty < tiles_y for _, ty, _ in got)
