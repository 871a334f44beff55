// Tensor-core sweep kernels: one Jacobi step as banded-matrix products on the
// 5th-generation tensor cores (tcgen05), the GB300 counterpart of the
// reference's wmma `mma_run` (layout16/kernel_*.cu).
//
// Formulation.  An output tile is 128 rows (the MMA's M, one row per TMEM
// lane) by 128 columns.  Rows are shifted by the smem descriptor; the
// horizontal taps are a band.  The tile's input columns are cut into 16-column
// windows (K = 16), window w = [X0-8+16w, X0+8+16w).  For each coefficient row
// dy, window w is multiplied (A = staged input shifted by dy, B = 16 x 32 band
// of row dy) into the 32 output columns [X0-16+16w, X0+16+16w) (N = 32) that
// it can reach: every staged input chunk is read once per dy, and each read
// feeds 32 outputs.  Windows overlap their neighbours' outputs by 16 columns,
// so even windows are issued first (their output ranges are disjoint and
// cover the accumulator, the first of them with accumulate = 0) and odd
// windows then add in.  Star stencils use the same windows with a one-tap
// (diagonal) band on the off-centre rows.  FP16 operands, FP32 accumulators
// in tensor memory (TMEM).  The split form gives each window its own TMEM
// region in a ring (tc_split_ring_kernel below), so that it streams windows
// instead of whole accumulators.
//
// Staging.  Planes are column panels (8 cells x all rows, 16 bytes per row,
// rows contiguous; see tcs_internal.h).  A tile needs rows Y0-2 .. Y0+129 of
// 18 panels (16 + one each side); it stages rows Y0-4 .. Y0+131 (136 rows),
// which with the plane's 4 top padding rows start on a 128-byte line, so one
// 3-D tensor-map load per plane moves 17 whole lines of each of the 18 panels
// (tc_core.cuh StageLines, encode_panel_map).  The shared-memory image, chunk
// s = all 136 rows of panel s at a 16-byte row stride, is directly a
// no-swizzle K-major UMMA operand (8-row x 16-byte core matrices, SBO = 128 B
// between row groups, LBO = 2176 B between K chunks), and a row shift dy is
// +16*dy bytes on the descriptor start address.
//
// Split precision (hi + lo planes).  Data are stored as x' = x 2^-E with
// hi = rint(x' 2^11) 2^-11 (fixed point) and lo = fp16((x' - hi) 2^11); a
// coefficient c as ch = rint(c 2^11) 2^-11 and rem = (c - ch) 2^11 = cl + c3
// (two FP16 pieces), plus cf = fp16(c).  Every hi*ch product is an integer
// multiple of 2^-22 and their sums stay below 2^24 such units, so the main
// accumulator is exact whatever the tensor core's internal rounding (its
// accumulation truncates; a biased error there would grow with the step
// count).  The correction accumulator (units 2^-11) takes cf*lo + cl*hi +
// c3*hi, where cf*lo also carries the lo*(c - ch) term.  Both are combined in
// FP32 with round-to-nearest in the epilogue.
//
// Pipeline (persistent, one CTA per SM; plain form):
//   warp 0       producer: one tensor-map load per plane of each tile into NS
//                stages (StageLines: 136 rows, whole 128-byte lines)
//   warps 1..I   MMA issuers taking tiles in turn, I = 3 for radius-1 and 2
//                for radius-2 stencils (warp 1 also owns TMEM)
//   next 8       epilogue (two warpgroups, one per column half):
//                TMEM -> registers -> FP16 -> global
//   last         signal: with several steps per launch, publishes finished
//                tile rows (see "several steps per launch" below)
// One accumulator slot per issuer lets the epilogue of one tile overlap the
// MMAs of the next; tile i uses slot i % I, issued by warp 1 + i % I.  Every
// wait is bounded; on timeout the kernel records an error word, stops,
// drains its own copies and MMAs, frees TMEM and returns.
//
// Launches: one step per launch, overlapped with the next step's set-up by
// programmatic dependent launch; or, for a plan's multi-step call on a large
// grid, all steps in one cooperative launch whose tiles of step j wait only
// for the neighbouring tile rows of step j-1.
#include "tc_core.cuh"
#include "tile_walk.h"

namespace tcs {

namespace {

using namespace tc;
using SG = StageLines;  // line-aligned staging of the sweep kernels

__device__ int g_tc_error = 0;

// ---------------------------------------------- several steps per launch ---
// Items are (step, tile), step-major; CTA b takes items b, b + grid, ...  A
// tile of step j needs tile rows ty-1 .. ty+1 of step j-1 finished: they hold
// its input, and they were the last readers of the plane it overwrites.  One
// counter per tile row (kRowCounterStride apart, a 128-byte line each) counts
// epilogue-warp completions over the launch.  A row's counts arrive in step
// order, as a tile starts only after its own row finished the step before, so
// "row r finished step j-1" is count >= j * (epilogue warps) * tiles_x.

// The producer's side: which rows of which step it already knows finished.
struct RowDeps {
    int ver_s = -1, ver_hi = -1;  // rows from this CTA's first row of step ver_s up to ver_hi

    // Waits (bounded) for rows ty-1 .. ty+1 of step `step - 1`.  One burst of
    // relaxed reads over the next kBurst rows extends the known range over
    // every finished one, so the next tiles (a few rows on) seldom poll; then
    // one acquire fence, and the proxy fence that orders the tensor copies
    // after it (they read what other SMs stored).  Returns false on give-up.
    __device__ bool wait(const unsigned *rows_done, int step, int ty, int tiles_y,
                         unsigned per_row) {
        constexpr int kBurst = 32;
        const int lo = ty > 0 ? ty - 1 : 0;
        const int hi = ty + 1 < tiles_y ? ty + 1 : tiles_y - 1;
        if (ver_s != step - 1 || lo > ver_hi + 1) {
            ver_s = step - 1;
            ver_hi = lo - 1;
        }
        if (hi <= ver_hi) return true;
        const unsigned target = (unsigned)step * per_row;
        const int first = ver_hi + 1;
        unsigned v[kBurst];
#pragma unroll
        for (int b = 0; b < kBurst; b++)
            v[b] = first + b < tiles_y ? ld_relaxed(rows_done + (first + b) * kRowCounterStride) : 0u;
        int x = first;  // rows first .. x-1 are finished
#pragma unroll
        for (int b = 0; b < kBurst; b++)
            if (x == first + b && first + b < tiles_y && v[b] >= target) x++;
        for (int r = x; r <= hi; r++) {  // rows this tile still needs
            const unsigned *ctr = rows_done + r * kRowCounterStride;
            const uint64_t t0 = global_timer_ns();
            while (ld_relaxed(ctr) < target) {
                if (*(volatile int *)&g_tc_error != 0 || global_timer_ns() - t0 > kWaitLimitNs)
                    return false;
                __nanosleep(32);
            }
        }
        ver_hi = x - 1 > hi ? x - 1 : hi;
        fence_acq_rel_gpu();
        fence_proxy_async_global();
        return true;
    }
};

// An epilogue warp's side: after its stores of its `done`-th item (counting
// from 1) are issued, it publishes the count in its own shared word (a
// release store, after the warp barrier that orders its lanes' stores).  It
// never waits here: the words only grow.
__device__ __forceinline__ void count_item(uint32_t *warp_done, int w, uint32_t done) {
    __syncwarp();
    if ((threadIdx.x & 31) == 0) st_release_cta(&warp_done[w], done);
}

// The signal warp's side (one thread): item i is finished when every
// epilogue warp's word has reached i + 1 (acquire at CTA scope); its count
// for its tile row is then published at GPU scope behind a fence that covers
// those stores.  Items already finished are batched behind one fence (it
// waits for their stores to complete); before waiting for an unfinished item
// the batch is flushed, so no count is ever held while this thread waits.
template <int NW>
__device__ void signal_rows(unsigned *rows_done, int n_items, int n_tiles, int tiles_x,
                            const uint32_t *warp_done, const volatile int *abort_flag) {
    constexpr int kBatch = 4;
    int pend[kBatch];
    int n_pend = 0;
    auto flush = [&]() {
        if (!n_pend) return;
        fence_acq_rel_gpu();
        for (int j = 0; j < n_pend; j++) red_relaxed_add(rows_done + pend[j] * kRowCounterStride, NW);
        n_pend = 0;
    };
    auto finished = [&](uint32_t target) {
#pragma unroll
        for (int w = 0; w < NW; w++)
            if (ld_acquire_cta(&warp_done[w]) < target) return false;
        return true;
    };
    uint32_t i = 0;
    TileWalk w;
    w.init(blockIdx.x, gridDim.x, tiles_x, n_tiles / tiles_x);
    for (int k = blockIdx.x; k < n_items; k += gridDim.x, i++, w.advance()) {
        if (!finished(i + 1)) {
            flush();
            const uint64_t t0 = global_timer_ns();
            while (!finished(i + 1)) {
                if (*abort_flag || global_timer_ns() - t0 > kWaitLimitNs) {
                    record_error(&g_tc_error, kErrWaitResult);
                    *(volatile int *)abort_flag = 1;
                    return;
                }
                // items take microseconds; a tight poll would take issue slots
                // from the epilogue warps sharing this warp's scheduler
                __nanosleep(256);
            }
        }
        pend[n_pend++] = w.ty;
        if (n_pend == kBatch) flush();
    }
    flush();
}

// Plain form: ISSUERS MMA issuer warps take tiles in turn.  Tile i uses
// accumulator slot i % ISSUERS (one 160-column slot per issuer) and stage
// i % NS with NS a multiple of the issuers, so every slot and every stage
// belongs to one issuer and its fills and releases are waited for by one
// thread, in order.  (An mbarrier parity wait also succeeds for the phase
// just before the barrier's current one: a thread that skipped a stage's fill
// could take the next fill as already landed, and one that fell two fills
// behind would wait for a phase that needs its own next tile.)  One issuer
// issues while the others wait for their stage or slot and commit.
template <int S>
struct Sweep {
    static constexpr int ISSUERS = stencil_r(S) == 1 ? 3 : 2;
    static constexpr int SLOTS = ISSUERS;
    static constexpr int STAGES = ISSUERS == 2 ? 4 : 3;
    static constexpr int SIGNAL_WARP = 1 + ISSUERS + kEpiWarps;  // several steps: row counts
    static constexpr int THREADS = 32 * (SIGNAL_WARP + 1);
    static_assert(SLOTS * Mode<false>::ACC <= kTmemCols, "accumulator slots fit TMEM");
    static_assert(STAGES % ISSUERS == 0, "each stage holds one issuer's tiles");
};

template <int S, bool SPLIT>
struct Cfg {
    using M = Mode<SPLIT>;
    static constexpr int R = stencil_r(S);
    static constexpr bool BOX = stencil_box(S);
    static constexpr int NDY = 2 * R + 1;
    static constexpr int STAGES = SPLIT ? 2 : Sweep<S>::STAGES;
    static constexpr size_t SMEM = 1024 + (size_t)STAGES * M::PLANES * SG::PLANE +
                                   (size_t)M::BAND_PLANES * NDY * kBandBytes + 256;
    static_assert(SMEM <= 232448, "shared memory budget");
};

struct TcParams {
    CUtensorMap map_hi, map_lo;     // input planes (encode_panel_map)
    CUtensorMap map_out, map_out_lo;  // several steps: the output planes (odd steps' input)
    GridGeom g;
    int tiles_x, n_tiles;
    int tile_w;                     // plain: tile columns, 64, 96 or 128 (split: 128)
    int steps;                      // plain: steps of this launch (1 for the split kernels)
    unsigned *rows_done;            // plain, several steps: per tile row (every
                                    // kRowCounterStride), epilogue-warp completions
                                    // over the launch (zeroed before it)
    const uint16_t *in_hi, *in_lo;  // input planes
    uint16_t *out_hi, *out_lo;
    SplitScale *scale;              // split: the grid's per-step scale (null: fixed scale)
    int t0;                         // split: steps of the run done before this launch
    float coef[25];                 // n x n, row-major
};

// Several split steps per launch: before publishing the scale of launch step
// j >= 2 the CTA waits (bounded, acquire) until every tile row has finished
// launch step j - 2, whose maxima and exponents the scale reads (tiles only
// wait for their neighbouring rows of step j - 1).  No cycle: every tile of
// step j - 2 is an earlier item of its CTA and depends only on earlier
// items.  The nl lanes of `mask` (this one is l of them) poll the rows, each
// issuing all its loads before testing any, so that a satisfied wait costs
// one round trip.  Returns false on give-up.
__device__ __forceinline__ bool wait_all_rows(const unsigned *rows_done, int tiles_y,
                                              unsigned target, const volatile int *abort_flag,
                                              unsigned mask, int l, int nl) {
    const uint64_t t0 = global_timer_ns();
    for (;;) {
        bool done = true;
        for (int r0 = l; r0 < tiles_y; r0 += 4 * nl) {
            unsigned v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int r = r0 + u * nl;
                v[u] = r < tiles_y ? ld_relaxed(rows_done + r * kRowCounterStride) : target;
            }
#pragma unroll
            for (int u = 0; u < 4; u++) done = done && v[u] >= target;
        }
        if (__all_sync(mask, done)) break;
        if (*abort_flag || *(volatile int *)&g_tc_error != 0 ||
            global_timer_ns() - t0 > kWaitLimitNs)
            return false;
        __nanosleep(128);
    }
    fence_acq_rel_gpu();
    return true;
}

template <int S, bool SPLIT>
__global__ void __launch_bounds__(Sweep<S>::THREADS, 1) tc_sweep_kernel(const __grid_constant__ TcParams p) {
    using C = Cfg<S, SPLIT>;
    using M = Mode<SPLIT>;
    constexpr int NS = C::STAGES;
    constexpr int NP = M::PLANES;
    constexpr int NSUB = M::NSUB;

    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                ~static_cast<uintptr_t>(1023));
    uint8_t *stage_base = smem;                                    // [NS][NP][stage]
    uint8_t *band_base = smem + (size_t)NS * NP * SG::PLANE;     // [BAND_PLANES][NDY]
    uint64_t *bars =
        reinterpret_cast<uint64_t *>(band_base + M::BAND_PLANES * C::NDY * kBandBytes);
    constexpr int NSL = Sweep<S>::SLOTS;
    uint64_t *full = bars;                      // [NS]
    uint64_t *empty = bars + NS;                // [NS]
    uint64_t *acc_full = bars + 2 * NS;         // [NSL]
    uint64_t *acc_empty = acc_full + NSL;       // [NSL]
    uint64_t *drain = acc_empty + NSL;          // [1]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(drain + 1);
    uint32_t *warp_done = tmem_slot + 2;        // [kEpiWarps] several steps: items stored
    static_assert((2 * NS + 2 * NSL + 1) * 8 + (2 + kEpiWarps) * 4 <= 256, "barrier area");
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const PlaneGeom pg = p.g.p16;

    // ---------------------------------------------------------- set-up ---
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < NSL; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], kEpiWarps);
        }
        mbar_init(drain, Sweep<S>::ISSUERS);
        for (int w = 0; w < kEpiWarps; w++) warp_done[w] = 0;
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        __syncwarp();
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    build_bands(reinterpret_cast<uint16_t *>(band_base), p.coef, C::R, C::BOX, SPLIT, threadIdx.x,
                Sweep<S>::THREADS);
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    // the previous step's CTAs may still run: planes only after pdl_wait
    pdl_launch_dependents();
    pdl_wait();

    const int tiles_x = p.tiles_x;
    const int n_tiles = p.n_tiles;
    const int tiles_y = n_tiles / tiles_x;
    const int n_items = p.steps * n_tiles;  // (step, tile), step-major; CTA b takes b, b + grid, ...

    if (warp == 0) {
        // ------------------------------------------------------ producer ---
        if (lane == 0) {
            int i = 0;
            int last_issued = -1;
            RowDeps deps;
            const unsigned per_row = (unsigned)(kEpiWarps * tiles_x);
            TileWalk w;
            w.init(blockIdx.x, gridDim.x, tiles_x, tiles_y);
            for (int k = blockIdx.x; k < n_items; k += gridDim.x, i++, w.advance()) {
                const int step = w.step;
                const int ty = w.ty;
                const int s = i % NS;
                const uint32_t ph = (i / NS) & 1;
                if (step > 0 && !deps.wait(p.rows_done, step, ty, tiles_y, per_row)) {
                    record_error(&g_tc_error, kErrWaitDep);
                    *abort_flag = 1;
                    break;
                }
                // (the poll above overlaps the wait for a free stage)
                if (!mbar_wait(&empty[s], ph ^ 1, abort_flag)) {
                    record_error(&g_tc_error, kErrWaitEmpty);
                    *abort_flag = 1;
                    break;
                }
                mbar_arrive_expect_tx(&full[s], NP * SG::PLANE);
                load_tile_map((step & 1) ? &p.map_out : &p.map_hi, &p.map_lo, NP, ty * kTile,
                              w.tx * p.tile_w, stage_base + (size_t)s * NP * SG::PLANE, &full[s]);
                last_issued = i;
            }
            // Drain: every stage armed last must have landed before exit.
            for (int k = 0; k < NS && last_issued - k >= 0; k++) {
                const int ii = last_issued - k;
                const uint64_t t0 = global_timer_ns();
                while (!mbar_try_wait(&full[ii % NS], (ii / NS) & 1)) {
                    if (global_timer_ns() - t0 > kWaitLimitNs) {
                        record_error(&g_tc_error, kErrWaitDrain);
                        break;
                    }
                }
            }
        }
    } else if (warp <= Sweep<S>::ISSUERS) {
        // --------------------------------------------------- MMA issuers ---
        static_assert(!SPLIT && NSUB == 1, "one plain sub-tile per tile");
        if (lane == 0) {
            const int id = warp - 1;  // issues the tiles i with i % Sweep<S>::ISSUERS == id
            bool stop = false;
            const uint32_t band = smem_u32(band_base);
            const uint32_t col = (uint32_t)(id * Mode<false>::ACC);  // this issuer's slot
            int i = id;
            // the tile's column, kept incrementally (t mod tiles_x; the step
            // wrap, a multiple of tiles_x, leaves it unchanged)
            const int k0 = blockIdx.x + id * (int)gridDim.x;
            const int dtx = (Sweep<S>::ISSUERS * (int)gridDim.x) % tiles_x;
            int tx = k0 % tiles_x;
            for (int k = k0; k < n_items && !stop;
                 k += Sweep<S>::ISSUERS * (int)gridDim.x, i += Sweep<S>::ISSUERS,
                 tx = tx + dtx >= tiles_x ? tx + dtx - tiles_x : tx + dtx) {
                const int s = i % NS;  // one of this issuer's stages
                if (!mbar_wait(&full[s], (i / NS) & 1, abort_flag)) {
                    record_error(&g_tc_error, kErrWaitFull);
                    *abort_flag = 1;
                    break;
                }
                // the slot's previous tile (i - NSL) has been read out
                if (!mbar_wait(&acc_empty[id], ((i / NSL) & 1) ^ 1, abort_flag)) {
                    record_error(&g_tc_error, kErrWaitAccum);
                    *abort_flag = 1;
                    stop = true;
                    break;
                }
                const uint64_t a_hi0 = smem_desc(
                    smem_u32(stage_base + (size_t)s * NP * SG::PLANE), SG::CHUNK, 128);
                tc_fence_after();
                issue_plain_tile<C::R, SG>(a_hi0, band, tmem_base + col,
                                           tile_windows(p.g.nx, tx * p.tile_w, p.tile_w));
                umma_commit(&acc_full[id]);
                umma_commit(&empty[s]);
            }
            // both issuers commit (one with nothing in flight completes at
            // once), so the drain phase always completes
            umma_commit(drain);
            const uint64_t t0 = global_timer_ns();
            while (!mbar_try_wait(drain, 0)) {
                if (global_timer_ns() - t0 > kWaitLimitNs) {
                    record_error(&g_tc_error, kErrWaitDrain);
                    break;
                }
            }
        }
    } else if (warp == Sweep<S>::SIGNAL_WARP) {
        // -------------------------------------------------------- signal ---
        if (p.rows_done && lane == 0)
            signal_rows<kEpiWarps>(p.rows_done, n_items, n_tiles, tiles_x, warp_done, abort_flag);
    } else {
        // ------------------------------------------------------ epilogue ---
        const int q = warp & 3;            // TMEM lane quarter of this warp
        const int half = (warp - 1 - Sweep<S>::ISSUERS) >> 2;  // which half of a sub-tile's column blocks
        const int m = q * 32 + lane;       // output row within the tile
        TileOut o;
        o.in_hi = p.in_hi;
        o.in_lo = p.in_lo;
        o.out_hi = p.out_hi;
        o.out_lo = p.out_lo;
        o.pg = pg;
        o.y0 = p.g.y0; o.y1 = p.g.y1; o.x0 = p.g.x0; o.x1 = p.g.x1;
        o.ny = p.g.ny; o.nx = p.g.nx;
        bool stop = false;
        const uint32_t lane_base = tmem_base + ((uint32_t)(q * 32) << 16);
        int i = 0;
        TileWalk w;
        w.init(blockIdx.x, gridDim.x, tiles_x, tiles_y);
        const int W = p.tile_w;
        const int G = W / 32;  // output blocks per warpgroup
        const int j0 = half * G;
        for (int k = blockIdx.x; k < n_items && !stop; k += gridDim.x, i++, w.advance()) {
            const int step = w.step;
            const int Y0 = w.ty * kTile;
            const int X0 = w.tx * W;
            // odd steps run from the output plane back into the input plane
            o.in_hi = (step & 1) ? p.out_hi : p.in_hi;
            o.out_hi = (step & 1) ? const_cast<uint16_t *>(p.in_hi) : p.out_hi;
            const int sl = i % NSL;  // tile i's accumulator slot
            bool ok = mbar_wait(&acc_full[sl], (i / NSL) & 1, abort_flag);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) {
                if (lane == 0) {
                    record_error(&g_tc_error, kErrWaitResult);
                    *abort_flag = 1;
                }
                stop = true;
                break;
            }
            const int nblk = tile_windows(p.g.nx, X0, W) - 1;  // blocks holding grid cells
            auto release = [&]() {
                // accumulators read: the issuer may refill them while we store
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&acc_empty[sl]);
            };
            if (j0 >= nblk) {  // none of this warpgroup's blocks hold grid cells
                __syncwarp();
                if (lane == 0) mbar_arrive(&acc_empty[sl]);
            } else {
                tc_fence_after();
                const uint32_t lc = lane_base + (uint32_t)(sl * Mode<false>::ACC);
                const int y = Y0 + m;
                const bool fast = tile_inside_w(o, Y0, X0, W);
                const bool row_in = y >= o.y0 && y < o.y1;
                if (G == 4) plain_epilogue<4>(o, lc, j0, nblk, y, X0, fast, row_in, release);
                else if (G == 3) plain_epilogue<3>(o, lc, j0, nblk, y, X0, fast, row_in, release);
                else plain_epilogue<2>(o, lc, j0, nblk, y, X0, fast, row_in, release);
            }
            if (p.rows_done) count_item(warp_done, warp - 1 - Sweep<S>::ISSUERS, (uint32_t)(i + 1));
        }
    }

    // -------------------------------------------------------- teardown ---
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) {
        __syncwarp();
        tmem_dealloc(tmem_base, kTmemCols);
    }
}

// Split form, single grid: a streaming window ring.  The nine 16-column
// windows of a tile (kTile / 16 + 1) are computed once each, in order, into a
// ring of kRingSlots 96-column TMEM regions (slot = global window index mod
// kRingSlots), and output block j is read from windows j and j+1 as soon as
// both are complete.  The MMA issuer can so run ahead of the epilogue by a
// few windows, instead of the two alternating with the whole accumulator.
// Twelve epilogue warps in three block groups (a lane quarter each) take
// blocks j with j mod 3 = group; a window is read by the groups of its two
// blocks and released unread by the third.  A slot is free again when all
// twelve epilogue warps have released its window; every warp releases a
// window only after seeing it complete, so releases always count toward the
// window they belong to.
//
// Three MMA issuers (warps 1..3) take windows G % 3.  Each window costs its
// issuer a region wait and a commit; the tensor pipe takes only a few MMAs
// ahead of the issuing thread, so with one issuer those latencies would leave
// it idle for about 40 % of a window.  With several, one issues while the
// others wait (measured per step at 8196²: box2d1r 124 -> 110 -> 109.5 us,
// box2d2r 157 -> 117 -> 114 us for one, two, three issuers).  A region is
// reused five windows later, by another issuer, after all twelve epilogue
// warps have released it; an issuer's previous region wait (two or three
// windows back) already covered the release before that, because every warp
// releases windows in order, so no parity wait can alias.  Every issuer
// waits for every stage fill in order, and a stage is free when all issuers'
// commits for the tile have completed.  The multi-step kernel (MULTI) has
// two issuers: with a third its 17 warps leave 96 registers a thread, and
// the epilogue spills (4098² box2d1r in one launch: 35.4 us per step with
// three issuers, 29.4 with two).
constexpr int kRingSlots = 5;
constexpr int kRegionCols = 96;
constexpr int kRingGroups = 3;                     // epilogue block groups
constexpr int kRingEpiWarps = 4 * kRingGroups;     // a lane quarter each
#ifndef TCS_SPLIT_ISSUERS
#define TCS_SPLIT_ISSUERS 3
#endif
// MULTI: the kernel runs several steps (p.steps) with the row counts and a
// signal warp; without it, one step in the single-step kernel's exact form
// (a kernel carrying the multi-step code ran single steps 8-11 % slower:
// 8196² box2d1r 106.7 -> 114.9 us).
template <bool MULTI>
struct Ring {
    static constexpr int ISSUERS = MULTI ? 2 : TCS_SPLIT_ISSUERS;  // MMA issuer warps 1 .. ISSUERS
    static constexpr int EPI0 = 1 + ISSUERS;                        // first epilogue warp
    static constexpr int SIGNAL_WARP = EPI0 + kRingEpiWarps;        // several steps: row counts
    static constexpr int THREADS = 32 * (SIGNAL_WARP + (MULTI ? 1 : 0));
};
// Every tile computes all its windows: a runtime window count for the last
// tile of a row slowed this epilogue-bound kernel by more than the skipped
// MMAs saved (16386²: 380 -> 387 us per step).
constexpr int kTileWindows = kTile / 16 + 1;
static_assert(kRingSlots * kRegionCols <= kTmemCols, "window ring fits TMEM");

// The multi-step kernel's scales: lanes 1..31 of the signal warp walk the
// CTA's items and, at each step j it holds tiles in (the CTA's n-th), wait
// for step j - 2 everywhere (j >= 2), read step j's scale and publish it as
// the n-th.  Publishing the (n+2)-th waits for a step at or after the n-th's
// to finish in every row, this CTA's tiles of it too, so every epilogue warp
// has taken the n-th by then and its slot and phase are free.
template <int NW>
__device__ void publish_scales(const TcParams &p, const CtaScale &cs, int n_items, int tiles_x,
                               int tiles_y, const volatile int *abort_flag) {
    constexpr unsigned kMask = 0xfffffffeu;
    const int l = (int)(threadIdx.x & 31) - 1;
    const int n_tiles = tiles_x * tiles_y;
    const unsigned per_row = (unsigned)(NW * tiles_x);
    int n = 0;
    for (int k = blockIdx.x, prev = -1; k < n_items; k += gridDim.x) {
        const int step = k / n_tiles;
        if (step == prev) continue;
        prev = step;
        if (step >= 2 && !wait_all_rows(p.rows_done, tiles_y, (unsigned)(step - 1) * per_row,
                                        abort_flag, kMask, l, 31)) {
            if (l == 0) {
                record_error(&g_tc_error, kErrWaitDep);
                *(volatile int *)abort_flag = 1;
            }
            return;
        }
        if (l == 0) cta_scale_publish(cs, n, step_scale(p.scale, p.t0 + step + 1));
        __syncwarp(kMask);
        n++;
    }
}

template <int S, bool MULTI>
__global__ void __launch_bounds__(Ring<MULTI>::THREADS, 1) tc_split_ring_kernel(const __grid_constant__ TcParams p) {
    using R = Ring<MULTI>;
    using C = Cfg<S, true>;
    using M = Mode<true>;
    constexpr int NS = C::STAGES;
    constexpr int NP = M::PLANES;

    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                ~static_cast<uintptr_t>(1023));
    uint8_t *stage_base = smem;                                 // [NS][NP][stage]
    uint8_t *band_base = smem + (size_t)NS * NP * SG::PLANE;  // NDY * 4 KB
    uint64_t *bars =
        reinterpret_cast<uint64_t *>(band_base + M::BAND_PLANES * C::NDY * kBandBytes);
    uint64_t *full = bars;                                    // [NS]
    uint64_t *empty = bars + NS;                              // [NS]
    uint64_t *win_full = bars + 2 * NS;                       // [kRingSlots]
    uint64_t *win_empty = bars + 2 * NS + kRingSlots;         // [kRingSlots]
    uint64_t *drain = bars + 2 * NS + 2 * kRingSlots;         // [1]
    CtaScale cs;                                              // the CTA's side of the scale
    cs.bar = drain + 1;                                       // [2]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(cs.bar + 2);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    uint32_t *warp_done = tmem_slot + 2;  // [kRingEpiWarps] several steps: items stored
    cs.max = warp_done + kRingEpiWarps;   // [2]
    cs.cnt = cs.max + 2;                  // [2]
    cs.ss = reinterpret_cast<StepScale *>(cs.cnt + 2);  // [2]
    static_assert((2 * NS + 2 * kRingSlots + 3) * 8 + (2 + kRingEpiWarps + 4) * 4 +
                          2 * sizeof(StepScale) <= 256, "barrier area");

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const PlaneGeom pg = p.g.p16;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], R::ISSUERS);
        }
        for (int r = 0; r < kRingSlots; r++) {
            mbar_init(&win_full[r], 1);
            mbar_init(&win_empty[r], kRingEpiWarps);
        }
        mbar_init(drain, R::ISSUERS);
        cta_scale_init(cs);
        for (int w = 0; w < kRingEpiWarps; w++) warp_done[w] = 0;
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        __syncwarp();
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    build_bands(reinterpret_cast<uint16_t *>(band_base), p.coef, C::R, C::BOX, true, threadIdx.x,
                R::THREADS);
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    // the previous step's CTAs may still run: planes only after pdl_wait
    pdl_launch_dependents();
    pdl_wait();

    const int tiles_x = p.tiles_x;
    const int n_tiles = p.n_tiles;
    const int tiles_y = n_tiles / tiles_x;
    // (step, tile), step-major; CTA b takes b, b + grid, ...
    const int n_items = MULTI ? p.steps * n_tiles : n_tiles;

    if (warp == 0) {
        // ------------------------------------------------------ producer ---
        if (lane == 0) {
            int i = 0;
            int last_issued = -1;
            RowDeps deps;
            const unsigned per_row = (unsigned)(kRingEpiWarps * tiles_x);
            TileWalk w;
            w.init(blockIdx.x, gridDim.x, tiles_x, tiles_y);
            for (int k = blockIdx.x; k < n_items; k += gridDim.x, i++, w.advance()) {
                const int step = w.step;
                const int ty = w.ty;
                const int s = i % NS;
                if (MULTI && step > 0 && !deps.wait(p.rows_done, step, ty, tiles_y, per_row)) {
                    record_error(&g_tc_error, kErrWaitDep);
                    *abort_flag = 1;
                    break;
                }
                // (the poll above overlaps the wait for a free stage)
                if (!mbar_wait(&empty[s], ((i / NS) & 1) ^ 1, abort_flag)) {
                    record_error(&g_tc_error, kErrWaitEmpty);
                    *abort_flag = 1;
                    break;
                }
                mbar_arrive_expect_tx(&full[s], NP * SG::PLANE);
                // odd steps run from the output planes back into the input planes
                load_tile_map((step & 1) ? &p.map_out : &p.map_hi,
                              (step & 1) ? &p.map_out_lo : &p.map_lo, NP, ty * kTile,
                              w.tx * kTile, stage_base + (size_t)s * NP * SG::PLANE, &full[s]);
                last_issued = i;
            }
            for (int k = 0; k < NS && last_issued - k >= 0; k++) {
                const int ii = last_issued - k;
                const uint64_t t0 = global_timer_ns();
                while (!mbar_try_wait(&full[ii % NS], (ii / NS) & 1)) {
                    if (global_timer_ns() - t0 > kWaitLimitNs) {
                        record_error(&g_tc_error, kErrWaitDrain);
                        break;
                    }
                }
            }
        }
    } else if (warp <= R::ISSUERS) {
        // --------------------------------------------------- MMA issuers ---
        if (lane == 0) {
            const int id = warp - 1;  // takes the windows G with G % R::ISSUERS == id
            int i = 0, G = 0;         // tiles, global windows
            bool stop = false;
            const uint32_t band = smem_u32(band_base);
            for (int k = blockIdx.x; k < n_items && !stop; k += gridDim.x, i++) {
                const int s = i % NS;
                if (!mbar_wait(&full[s], (i / NS) & 1, abort_flag)) {
                    record_error(&g_tc_error, kErrWaitFull);
                    *abort_flag = 1;
                    break;
                }
                const uint64_t a_hi0 = smem_desc(
                    smem_u32(stage_base + (size_t)s * NP * SG::PLANE), SG::CHUNK, 128);
#pragma unroll 1
                for (int wg = 0; wg < kTileWindows; wg++, G++) {
                    if (G % R::ISSUERS != id) continue;
                    const int r = G % kRingSlots;
                    if (!mbar_wait(&win_empty[r], ((G / kRingSlots) & 1) ^ 1, abort_flag)) {
                        record_error(&g_tc_error, kErrWaitAccum);
                        *abort_flag = 1;
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    issue_split_window<C::R, SG>(a_hi0, band, tmem_base + r * kRegionCols, wg);
                    umma_commit(&win_full[r]);
                }
                if (!stop) umma_commit(&empty[s]);
            }
            // both issuers commit (an issuer with nothing in flight completes
            // its commit at once), so the drain phase always completes
            umma_commit(drain);
            const uint64_t t0 = global_timer_ns();
            while (!mbar_try_wait(drain, 0)) {
                if (global_timer_ns() - t0 > kWaitLimitNs) {
                    record_error(&g_tc_error, kErrWaitDrain);
                    break;
                }
            }
        }
    } else if (MULTI && warp == R::SIGNAL_WARP) {
        // -------------------------------------------------------- signal ---
        // lane 0 the row counts, lanes 1..31 the scales of the CTA's steps
        if (lane == 0)
            signal_rows<kRingEpiWarps>(p.rows_done, n_items, n_tiles, tiles_x, warp_done, abort_flag);
        else if (p.scale)
            publish_scales<kRingEpiWarps>(p, cs, n_items, tiles_x, tiles_y, abort_flag);
    } else {
        // ------------------------------------------------------ epilogue ---
        const int q = warp & 3;                          // TMEM lane quarter
        const int grp = (warp - R::EPI0) >> 2;  // block group: blocks j with j % 3 == grp
        const int m = q * 32 + lane;
        const uint32_t lane_base = tmem_base + ((uint32_t)(q * 32) << 16);
        TileOut o;
        o.in_hi = p.in_hi;
        o.in_lo = p.in_lo;
        o.out_hi = p.out_hi;
        o.out_lo = p.out_lo;
        o.pg = pg;
        o.y0 = p.g.y0; o.y1 = p.g.y1; o.x0 = p.g.x0; o.x1 = p.g.x1;
        o.ny = p.g.ny; o.nx = p.g.nx;
        int G0 = 0;  // first global window of the tile
        // bounded wait for window w of the tile
        auto ready = [&](int w) {
            const int Gw = G0 + w;
            bool ok = mbar_wait(&win_full[Gw % kRingSlots], (Gw / kRingSlots) & 1, abort_flag);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok && lane == 0) {
                record_error(&g_tc_error, kErrWaitResult);
                *abort_flag = 1;
            }
            return ok;
        };
        auto release = [&](int w) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&win_empty[(G0 + w) % kRingSlots]);
        };
        int i = 0;
        TileWalk w;
        w.init(blockIdx.x, gridDim.x, tiles_x, tiles_y);
        // the scale of the current step, this warp's largest |u| in it, and
        // whether the CTA holds the step's tile 0
        int cur = -1, nst = -1;  // nst: the CTA's step ordinal
        StepScale ss = step_scale(nullptr, 0);
        float mx = 0.0f;
        bool own0 = false;
        // one step per launch: the first epilogue warp reads the record for
        // the CTA (several: the signal warp's lanes 1..31 do)
        const bool scale_warp = !MULTI && warp == R::EPI0;
        for (int k = blockIdx.x; k < n_items; k += gridDim.x, G0 += kTileWindows, i++, w.advance()) {
            const int step = w.step;
            const int Y0 = w.ty * kTile;
            const int X0 = w.tx * kTile;
            if (MULTI) {
                // odd steps run from the output planes back into the input planes
                o.in_hi = (step & 1) ? p.out_hi : p.in_hi;
                o.in_lo = (step & 1) ? p.out_lo : p.in_lo;
                o.out_hi = (step & 1) ? const_cast<uint16_t *>(p.in_hi) : p.out_hi;
                o.out_lo = (step & 1) ? const_cast<uint16_t *>(p.in_lo) : p.out_lo;
            }
            if (step != cur && p.scale) {
                nst++;
                if (scale_warp) {
                    if (lane == 0) cta_scale_publish(cs, nst, step_scale(p.scale, p.t0 + step + 1));
                    __syncwarp();
                }
                if (!cta_scale_take(cs, nst, ss, abort_flag)) {
                    if (lane == 0) {
                        record_error(&g_tc_error, kErrWaitDep);
                        *abort_flag = 1;
                    }
                    break;
                }
                cur = step;
                mx = 0.0f;
                own0 = false;
            }
            own0 = own0 || (w.ty == 0 && w.tx == 0);
            const int y = Y0 + m;
            const bool fast = tile_inside(o, Y0, X0);
            const bool row_in = y >= o.y0 && y < o.y1;
            const bool ok = walk_windows(grp, kRingGroups, kTileWindows, ready, release, [&](int j) {
                const int Ga = G0 + j, Gb = Ga + 1;
                tc_fence_after();
                float f[16];
                split_block_load(lane_base + (Ga % kRingSlots) * kRegionCols,
                                 lane_base + (Gb % kRingSlots) * kRegionCols, f);
                tc_fence_before();
                __syncwarp();
                if (lane == 0) {
                    mbar_arrive(&win_empty[Ga % kRingSlots]);
                    mbar_arrive(&win_empty[Gb % kRingSlots]);
                }
                store_block_split(o, f, y, X0 + 16 * j, fast, row_in, ss, mx);
            });
            if (!ok) break;
            if (ss.k != 0 && !fast) resplit_border(o, y, X0, grp, kRingGroups, kTileWindows - 1, ss);
            // the step's last item of this warp: its maximum and the step's
            // exponent go out before the item is counted
            if (p.scale) {
                TileWalk nw = w;
                nw.advance();
                if (k + (int)gridDim.x >= n_items || nw.step != step)
                    cta_scale_flush<kRingEpiWarps>(cs, nst, p.scale, p.t0 + step + 1, ss, mx,
                                                   own0);
            }
            if (MULTI) count_item(warp_done, warp - R::EPI0, (uint32_t)(i + 1));
        }
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) {
        __syncwarp();
        tmem_dealloc(tmem_base, kTmemCols);
    }
}

int g_num_sms = 0;

// Sets the kernel's shared-memory limit and reads the SM count; called before
// any launch (and so before any stream capture of one).
template <int S, bool SPLIT>
cudaError_t prepare_tc() {
    static bool configured = false;
    if (!configured) {
        cudaError_t e;
        if constexpr (SPLIT)
        {
            e = cudaFuncSetAttribute(tc_split_ring_kernel<S, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(Cfg<S, SPLIT>::SMEM));
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(tc_split_ring_kernel<S, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(Cfg<S, SPLIT>::SMEM));
        }
        else
            e = cudaFuncSetAttribute(tc_sweep_kernel<S, SPLIT>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(Cfg<S, SPLIT>::SMEM));
        if (e != cudaSuccess) return e;
        configured = true;
    }
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    return cudaSuccess;
}

// One launch of `steps` steps.  With several, step j reads the in planes for
// even j and the out planes for odd j and writes the others; rows_done holds one zeroed counter per tile row (kRowCounterStride apart), and the launch is
// cooperative, so that all CTAs of the static tile order are resident at once.
template <int S, bool SPLIT>
cudaError_t launch_tc(const GridGeom &g, const float *B, const uint16_t *in_hi,
                      const uint16_t *in_lo, uint16_t *out_hi, uint16_t *out_lo, cudaStream_t s,
                      int steps = 1, unsigned *rows_done = nullptr, int tile_w = kTile,
                      SplitScale *scale = nullptr, int t0 = 0) {
    using C = Cfg<S, SPLIT>;
    if (!valid_tile_width(tile_w) || (SPLIT && tile_w != kTile)) return cudaErrorInvalidValue;
    cudaError_t pe = prepare_tc<S, SPLIT>();
    if (pe != cudaSuccess) return pe;
    TcParams p;
    p.g = g;
    p.tile_w = tile_w;
    const int tiles_y = (g.ny + kTile - 1) / kTile;
    p.tiles_x = (g.nx + tile_w - 1) / tile_w;
    p.n_tiles = tiles_y * p.tiles_x;
    p.in_hi = in_hi;
    p.in_lo = in_lo;
    cudaError_t me = encode_panel_map(in_hi, g.p16, &p.map_hi);
    if (me == cudaSuccess) me = encode_panel_map(SPLIT ? in_lo : in_hi, g.p16, &p.map_lo);
    if (me != cudaSuccess) return me;
    p.out_hi = out_hi;
    p.out_lo = out_lo;
    p.scale = SPLIT ? scale : nullptr;
    p.t0 = t0;
    p.steps = 1;
    p.rows_done = nullptr;
    p.map_out = p.map_hi;
    p.map_out_lo = p.map_lo;
    if (steps > 1) {
        if (!rows_done) return cudaErrorInvalidValue;
        me = encode_panel_map(out_hi, g.p16, &p.map_out);
        if (me == cudaSuccess && SPLIT) me = encode_panel_map(out_lo, g.p16, &p.map_out_lo);
        if (me != cudaSuccess) return me;
        p.steps = steps;
        p.rows_done = rows_done;
    }
    for (int k = 0; k < 25; k++) p.coef[k] = 0.0f;
    for (int k = 0; k < C::NDY * C::NDY; k++) p.coef[k] = B[k];
    const long long items = (long long)p.n_tiles * p.steps;
    const int grid = items < g_num_sms ? (int)items : g_num_sms;
    if constexpr (SPLIT)
        return p.steps > 1
                   ? launch_step(tc_split_ring_kernel<S, true>, grid, Ring<true>::THREADS, C::SMEM, s, p, true)
                   : launch_step(tc_split_ring_kernel<S, false>, grid, Ring<false>::THREADS, C::SMEM, s, p);
    else
        return launch_step(tc_sweep_kernel<S, SPLIT>, grid, Sweep<S>::THREADS, C::SMEM, s, p,
                           p.steps > 1);
}

template <bool SPLIT>
cudaError_t dispatch_tc(const GridGeom &g, int stencil, const float *B, const uint16_t *in_hi,
                        const uint16_t *in_lo, uint16_t *out_hi, uint16_t *out_lo, cudaStream_t s,
                        int steps = 1, unsigned *rows_done = nullptr, int tile_w = kTile,
                        SplitScale *scale = nullptr, int t0 = 0) {
    switch (stencil) {
    case TCS_STAR2D1R: return launch_tc<TCS_STAR2D1R, SPLIT>(g, B, in_hi, in_lo, out_hi, out_lo, s, steps, rows_done, tile_w, scale, t0);
    case TCS_STAR2D2R: return launch_tc<TCS_STAR2D2R, SPLIT>(g, B, in_hi, in_lo, out_hi, out_lo, s, steps, rows_done, tile_w, scale, t0);
    case TCS_BOX2D1R: return launch_tc<TCS_BOX2D1R, SPLIT>(g, B, in_hi, in_lo, out_hi, out_lo, s, steps, rows_done, tile_w, scale, t0);
    case TCS_BOX2D2R: return launch_tc<TCS_BOX2D2R, SPLIT>(g, B, in_hi, in_lo, out_hi, out_lo, s, steps, rows_done, tile_w, scale, t0);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t tc_prepare(int stencil, bool split) {
    switch (stencil) {
    case TCS_STAR2D1R: return split ? prepare_tc<TCS_STAR2D1R, true>() : prepare_tc<TCS_STAR2D1R, false>();
    case TCS_STAR2D2R: return split ? prepare_tc<TCS_STAR2D2R, true>() : prepare_tc<TCS_STAR2D2R, false>();
    case TCS_BOX2D1R: return split ? prepare_tc<TCS_BOX2D1R, true>() : prepare_tc<TCS_BOX2D1R, false>();
    case TCS_BOX2D2R: return split ? prepare_tc<TCS_BOX2D2R, true>() : prepare_tc<TCS_BOX2D2R, false>();
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t tc_take_error(int *code) {
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(code, g_tc_error, sizeof(int));
    if (e != cudaSuccess) return e;
    return *code ? cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int)) : cudaSuccess;
}

cudaError_t launch_tc_f16(const GridGeom &g, int stencil, const float *B, const uint16_t *in,
                          uint16_t *out, cudaStream_t s, int tile_w) {
    return dispatch_tc<false>(g, stencil, B, in, nullptr, out, nullptr, s, 1, nullptr, tile_w);
}

cudaError_t launch_tc_f16_steps(const GridGeom &g, int stencil, const float *B, const uint16_t *in,
                                uint16_t *out, int steps, unsigned *rows_done, cudaStream_t s,
                                int tile_w) {
    return dispatch_tc<false>(g, stencil, B, in, nullptr, out, nullptr, s, steps, rows_done, tile_w);
}

cudaError_t launch_tc_split_steps(const GridGeom &g, int stencil, const float *B,
                                  const uint16_t *in_hi, const uint16_t *in_lo, uint16_t *out_hi,
                                  uint16_t *out_lo, int steps, unsigned *rows_done, cudaStream_t s,
                                  SplitScale *scale, int t0) {
    return dispatch_tc<true>(g, stencil, B, in_hi, in_lo, out_hi, out_lo, s, steps, rows_done,
                             kTile, scale, t0);
}

cudaError_t launch_tc_split(const GridGeom &g, int stencil, const float *B, const uint16_t *in_hi,
                            const uint16_t *in_lo, uint16_t *out_hi, uint16_t *out_lo,
                            cudaStream_t s, SplitScale *scale, int t0) {
    return dispatch_tc<true>(g, stencil, B, in_hi, in_lo, out_hi, out_lo, s, 1, nullptr, kTile,
                             scale, t0);
}

}  // namespace tcs
