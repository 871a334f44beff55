// Temporally blocked split-precision sweep: TWO Jacobi steps per HBM round
// trip.  The single-step split kernel is bound by the bytes an SM can keep in
// flight (two 76 KB stages for ~140 KB of traffic per tile and step);
// blocking two steps cuts the traffic per step to ~5.4 B per point-update
// for ~25 % more MMA work.
//
// Tile.  Outputs are rows [Y0, Y0 + 128 - 2r) x columns [X0, X0 + 80) (X0 a
// multiple of 80).  The producer stages input rows [Y0 - r - 2, Y0 - r + 130)
// and columns [X0 - 24, X0 + 104): 16 panels, hi and lo, 66 KB.
//   Step 1: eight windows (input columns X0 - 24 + 16w .. +16) give the
//     128-row intermediate over columns [X0 - 16, X0 + 96) (seven blocks), of
//     which columns [X0 - 8, X0 + 88) (12 panels) go, as hi/lo FP16 panels,
//     into a shared-memory intermediate image.  The input stage is released
//     as soon as these MMAs are done, so the next tile loads during step 2.
//   Step 2: six windows over the intermediate (columns X0 - 8 + 16w .. +16)
//     give the 80 output columns; rows r .. 127 - r of the 128 are valid.
// Windows sit at the same absolute columns (8 mod 16) as in the single-step
// kernel and each block sums the same two windows, so two blocked steps give
// exactly the bits of two single steps.
//
// Pipeline.  Window accumulators stream through the ring of five 96-column
// TMEM regions of the single-step split kernel; per tile the issuer runs step
// 1, waits for the epilogue's intermediate, then runs step 2.  There is one
// intermediate image: the epilogue writes tile t+1's only after consuming
// every step-2 window of tile t, i.e. after those MMAs have read it.  Panels
// outside the plane come from a zero panel; row copies are clipped to the
// plane; stores are clipped to the grid.
#include "tc_core.cuh"

namespace tcs {

namespace {

using namespace tc;

__device__ int g_tb_error = 0;

// One staged panel of zeros, the source for panels outside the plane.
__device__ __align__(256) uint16_t g_zero_panel[kRowsStaged * 8] = {0};

constexpr int kTbCols = 80;  // output columns per tile
constexpr int kTbStages = 2;
constexpr int kTbRing = 5;
constexpr int kTbRegion = 96;
constexpr int kS1Windows = 8;  // step 1: intermediate columns [X0 - 16, X0 + 96)
constexpr int kS2Windows = 6;  // step 2: output columns [X0, X0 + 80)
constexpr int kInPanels = 16;  // input columns [X0 - 24, X0 + 104)
constexpr int kMidPanels = 12; // intermediate columns [X0 - 8, X0 + 88)
constexpr int kInPlane = kInPanels * kChunkBytes;    // one staged input plane
constexpr int kMidPlane = kMidPanels * kChunkBytes;  // one intermediate plane
constexpr int kTbGroups = 3;                          // epilogue block groups
constexpr int kTbEpiWarps = 4 * kTbGroups;            // a lane quarter each
// MMA issuer warps 1 and 2 take alternate windows (G % 2), as in the
// single-step split kernel: both wait for every stage fill and every
// intermediate, in order, and commit the stage after step 1 (the stage is
// free when both have); an issuer's previous region wait, two windows back,
// already covered the release before the one it now needs.
constexpr int kTbIssuers = 2;
constexpr int kTbThreads = 32 * (1 + kTbIssuers + kTbEpiWarps);

template <int S>
struct TbCfg {
    static constexpr int R = stencil_r(S);
    static constexpr bool BOX = stencil_box(S);
    static constexpr int NDY = 2 * R + 1;
    static constexpr int H = kTile - 2 * R;  // output rows per tile
    static constexpr size_t BAND = (size_t)4 * NDY * kBandBytes;
    static constexpr size_t SMEM =
        1024 + (size_t)kTbStages * 2 * kInPlane + 2 * kMidPlane + BAND + 256;
    static_assert(SMEM <= 232448, "shared memory budget");
};

struct TbParams {
    GridGeom g;
    int tiles_x, n_tiles;
    const uint16_t *in_hi, *in_lo;
    uint16_t *out_hi, *out_lo;
    SplitScale *scale;  // the grid's per-step scale (null: fixed scale)
    int t0;             // steps of the run done before this pair
    float coef[25];
};

// 8 cells of panel row (y, x0) of a plane (x0 a multiple of 8), or zeros when
// the row or panel is outside the plane.
__device__ __forceinline__ uint4 load_panel_row(const uint16_t *plane, const PlaneGeom &pg, int y,
                                                int x0) {
    const int row = y + kPadTop, pan = (x0 >> 3) + 1;
    if (row < 0 || row >= pg.nyp || pan < 0 || pan >= pg.npan) return make_uint4(0, 0, 0, 0);
    return *reinterpret_cast<const uint4 *>(plane + ((size_t)pan * pg.nyp + row) * 8);
}

template <int S>
__global__ void __launch_bounds__(kTbThreads, 1) tc_split_tb_kernel(const TbParams p) {
    using C = TbCfg<S>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                ~static_cast<uintptr_t>(1023));
    uint8_t *stage_base = smem;  // [stage][hi, lo][16 panels]
    uint8_t *mid_base = smem + (size_t)kTbStages * 2 * kInPlane;  // [hi, lo][12 panels]
    uint8_t *band_base = mid_base + 2 * kMidPlane;
    uint64_t *bars = reinterpret_cast<uint64_t *>(band_base + C::BAND);
    uint64_t *full = bars;                         // [2]
    uint64_t *empty = bars + 2;                    // [2]
    uint64_t *inter_ready = bars + 4;              // [1] intermediate written
    uint64_t *win_full = bars + 5;                 // [kTbRing]
    uint64_t *win_empty = bars + 5 + kTbRing;      // [kTbRing]
    uint64_t *drain = bars + 5 + 2 * kTbRing;      // [1]
    CtaScale cs;                                   // the CTA's side of the scale
    cs.bar = drain + 1;                            // [2]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(cs.bar + 2);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    cs.max = tmem_slot + 2;                        // [2]
    cs.cnt = cs.max + 2;                           // [2]
    cs.ss = reinterpret_cast<StepScale *>(cs.cnt + 2);  // [2]
    static_assert((8 + 2 * kTbRing) * 8 + 8 + 16 + 2 * sizeof(StepScale) <= 256, "barrier area");

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const PlaneGeom pg = p.g.p16;
    const int n_mine = (p.n_tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kTbStages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kTbIssuers);
        }
        mbar_init(inter_ready, kTbEpiWarps);
        for (int r = 0; r < kTbRing; r++) {
            mbar_init(&win_full[r], 1);
            mbar_init(&win_empty[r], kTbEpiWarps);
        }
        mbar_init(drain, kTbIssuers);
        cta_scale_init(cs);
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        __syncwarp();
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    build_bands(reinterpret_cast<uint16_t *>(band_base), p.coef, C::R, C::BOX, true, threadIdx.x,
                kTbThreads);
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    // the previous step's CTAs may still run: planes only after pdl_wait
    pdl_launch_dependents();
    pdl_wait();

    auto tile_origin = [&](int i, int &Y0, int &X0) {
        const int t = (int)blockIdx.x + i * (int)gridDim.x;
        Y0 = (t / p.tiles_x) * C::H;
        X0 = (t % p.tiles_x) * kTbCols;
    };

    if (warp == 0) {
        // ------------------------------------------------------ producer ---
        if (lane == 0) {
            int last_issued = -1;
            for (int i = 0; i < n_mine; i++) {
                const int s = i % kTbStages;
                if (!mbar_wait(&empty[s], ((i / kTbStages) & 1) ^ 1, abort_flag)) {
                    record_error(&g_tb_error, kErrWaitEmpty);
                    *abort_flag = 1;
                    break;
                }
                int Y0, X0;
                tile_origin(i, Y0, X0);
                const int row0 = Y0 - C::R - 2 + kPadTop;  // >= 0
                const int rows = min(kRowsStaged, pg.nyp - row0);
                const int pan0 = (X0 >> 3) - 2;  // plane panel of column X0 - 24
                uint32_t bytes = 0;
                for (int q = 0; q < kInPanels; q++) {
                    const int pan = pan0 + q;
                    bytes += (pan >= 0 && pan < pg.npan) ? rows * 16 : kChunkBytes;
                }
                mbar_arrive_expect_tx(&full[s], 2 * bytes);
                uint8_t *st = stage_base + (size_t)s * 2 * kInPlane;
                for (int pl = 0; pl < 2; pl++) {
                    const uint16_t *src = pl ? p.in_lo : p.in_hi;
#pragma unroll 1
                    for (int q = 0; q < kInPanels; q++) {
                        const int pan = pan0 + q;
                        uint8_t *dst = st + (size_t)pl * kInPlane + q * kChunkBytes;
                        if (pan >= 0 && pan < pg.npan)
                            bulk_load(dst, src + ((size_t)pan * pg.nyp + row0) * 8, rows * 16,
                                      &full[s]);
                        else
                            bulk_load(dst, g_zero_panel, kChunkBytes, &full[s]);
                    }
                }
                last_issued = i;
            }
            for (int k = 0; k < kTbStages && last_issued - k >= 0; k++) {
                const int ii = last_issued - k;
                const uint64_t t0 = global_timer_ns();
                while (!mbar_try_wait(&full[ii % kTbStages], (ii / kTbStages) & 1)) {
                    if (global_timer_ns() - t0 > kWaitLimitNs) {
                        record_error(&g_tb_error, kErrWaitDrain);
                        break;
                    }
                }
            }
        }
    } else if (warp <= kTbIssuers) {
        // ---------------------------------------------------- MMA issuer ---
        if (lane == 0) {
            const int id = warp - 1;  // takes the windows G with G % 2 == id
            const uint32_t band = smem_u32(band_base);
            int G = 0;
            bool issued_any = false, stop = false;
            // the windows of one step of tile i, from stage panel slot0 + 2w
            // the windows of one step from an image (hi at a_hi0, lo lo_bytes on)
            auto run_step = [&](uint64_t a_hi0, int lo_bytes, int nwin) {
#pragma unroll 1
                for (int w = 0; w < nwin; w++, G++) {
                    if (G % kTbIssuers != id) continue;
                    const int r = G % kTbRing;
                    if (!mbar_wait(&win_empty[r], ((G / kTbRing) & 1) ^ 1, abort_flag)) {
                        record_error(&g_tb_error, kErrWaitAccum);
                        *abort_flag = 1;
                        stop = true;
                        return;
                    }
                    tc_fence_after();
                    issue_split_window_at<C::R>(a_hi0, band, tmem_base + r * kTbRegion, 2 * w,
                                                lo_bytes);
                    umma_commit(&win_full[r]);
                    issued_any = true;
                }
            };
            const uint64_t mid_desc = smem_desc(smem_u32(mid_base), kChunkBytes, 128);
            for (int i = 0; i < n_mine && !stop; i++) {
                const int s = i % kTbStages;
                if (!mbar_wait(&full[s], (i / kTbStages) & 1, abort_flag)) {
                    record_error(&g_tb_error, kErrWaitFull);
                    *abort_flag = 1;
                    break;
                }
                tc_fence_after();
                run_step(smem_desc(smem_u32(stage_base + (size_t)s * 2 * kInPlane), kChunkBytes, 128),
                         kInPlane, kS1Windows);
                if (stop) break;
                umma_commit(&empty[s]);  // the input stage is free once step 1 is done
                if (!mbar_wait(inter_ready, i & 1, abort_flag)) {
                    record_error(&g_tb_error, kErrWaitFull);
                    *abort_flag = 1;
                    break;
                }
                tc_fence_after();
                run_step(mid_desc, kMidPlane, kS2Windows);
            }
            // both issuers commit (one with nothing in flight completes at
            // once), so the drain phase always completes
            (void)issued_any;
            umma_commit(drain);
            const uint64_t t0 = global_timer_ns();
            while (!mbar_try_wait(drain, 0)) {
                if (global_timer_ns() - t0 > kWaitLimitNs) {
                    record_error(&g_tb_error, kErrWaitDrain);
                    break;
                }
            }
        }
    } else {
        // ------------------------------------------------------ epilogue ---
        const int q = warp & 3;
        const int grp = (warp - 1 - kTbIssuers) >> 2;  // block group
        const int m = q * 32 + lane;  // M row of the step (intermediate row Y0 - r + m)
        const uint32_t lane_base = tmem_base + ((uint32_t)(q * 32) << 16);
        TileOut o;
        o.in_hi = p.in_hi;
        o.in_lo = p.in_lo;
        o.out_hi = p.out_hi;
        o.out_lo = p.out_lo;
        o.pg = pg;
        o.y0 = p.g.y0; o.y1 = p.g.y1; o.x0 = p.g.x0; o.x1 = p.g.x1;
        o.ny = p.g.ny; o.nx = p.g.nx;
        int G0 = 0;
        bool stop = false;
        // bounded wait for window w of the current step (from G0)
        auto ready = [&](int w) {
            const int Gw = G0 + w;
            bool ok = mbar_wait(&win_full[Gw % kTbRing], (Gw / kTbRing) & 1, abort_flag);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok && lane == 0) {
                record_error(&g_tb_error, kErrWaitResult);
                *abort_flag = 1;
            }
            return ok;
        };
        auto release = [&](int w) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&win_empty[(G0 + w) % kTbRing]);
        };
        // Blocks of one step: block j sums windows j and j+1 and belongs to
        // group j mod 3; every window is released by all twelve warps.
        auto run_step = [&](int nwin, auto &&store) {
            const bool ok = walk_windows(grp, kTbGroups, nwin, ready, release, [&](int j) {
                const int Ga = G0 + j, Gb = Ga + 1;
                tc_fence_after();
                float f[16];
                split_block_load(lane_base + (Ga % kTbRing) * kTbRegion,
                                 lane_base + (Gb % kTbRing) * kTbRegion, f);
                tc_fence_before();
                __syncwarp();
                if (lane == 0) {
                    mbar_arrive(&win_empty[Ga % kTbRing]);
                    mbar_arrive(&win_empty[Gb % kTbRing]);
                }
                store(j, f);
            });
            if (!ok) stop = true;
            G0 += nwin;
        };
        // The pair's two scales, both from steps finished before the launch
        // (step t reads steps t-2 and t-3), read by the first epilogue warp;
        // the second step's copies come from the input, two steps back, so
        // they take both shifts.
        if (warp == 1 + kTbIssuers && lane == 0) {
            cta_scale_publish(cs, 0, step_scale(p.scale, p.t0 + 1));
            cta_scale_publish(cs, 1, step_scale(p.scale, p.t0 + 2));
        }
        StepScale ss1, ss2;
        if (!cta_scale_take(cs, 0, ss1, abort_flag) || !cta_scale_take(cs, 1, ss2, abort_flag)) {
            if (lane == 0) {
                record_error(&g_tb_error, kErrWaitResult);
                *abort_flag = 1;
            }
            stop = true;
        }
        StepScale cs2 = ss2;
        cs2.k = ss1.k + ss2.k;
        cs2.s = __int_as_float((127 + 11 + cs2.k) << 23);
        float mx1 = 0.0f, mx2 = 0.0f;
        for (int i = 0; i < n_mine && !stop; i++) {
            int Y0, X0;
            tile_origin(i, Y0, X0);
            {
                // step 1 -> the intermediate image
                const int y = Y0 - C::R + m;
                const int xi = X0 - 16;  // first column of step 1's blocks
                const bool fast = Y0 - C::R >= o.y0 && Y0 - C::R + kTile <= o.y1 &&
                                  xi >= o.x0 && xi + 112 <= o.x1;
                const bool row_in = y >= o.y0 && y < o.y1;
                run_step(kS1Windows, [&](int j, const float (&f)[16]) {
                    const int xb = xi + 16 * j;
                    uint32_t hw[8], lw[8];
                    if (fast) {
#pragma unroll
                        for (int c = 0; c < 8; c++)
                            split_pair_s(f[2 * c], f[2 * c + 1], ss1.s, hw[c], lw[c], mx1);
                    } else {
                        const uint4 a0 = load_panel_row(o.in_hi, pg, y, xb);
                        const uint4 a1 = load_panel_row(o.in_hi, pg, y, xb + 8);
                        const uint4 b0 = load_panel_row(o.in_lo, pg, y, xb);
                        const uint4 b1 = load_panel_row(o.in_lo, pg, y, xb + 8);
                        const uint32_t iw[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                        const uint32_t il[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                        for (int c = 0; c < 8; c++) {
                            uint16_t hh[2], ll[2];
#pragma unroll
                            for (int u2 = 0; u2 < 2; u2++) {
                                const int x = xb + 2 * c + u2;
                                if (row_in && x >= o.x0 && x < o.x1) {
                                    split_fixed_s(f[2 * c + u2], ss1.s, hh[u2], ll[u2], mx1);
                                } else {
                                    hh[u2] = (uint16_t)(iw[c] >> (16 * u2));
                                    ll[u2] = (uint16_t)(il[c] >> (16 * u2));
                                    if (ss1.k != 0) resplit_pair(hh[u2], ll[u2], ss1);
                                }
                            }
                            hw[c] = (uint32_t)hh[0] | ((uint32_t)hh[1] << 16);
                            lw[c] = (uint32_t)ll[0] | ((uint32_t)ll[1] << 16);
                        }
                    }
                    // block j = intermediate panels 2j-1, 2j (those of the
                    // 12 kept), image row m + 2
#pragma unroll
                    for (int hlf = 0; hlf < 2; hlf++) {
                        const int pnl = 2 * j - 1 + hlf;
                        if (pnl < 0 || pnl >= kMidPanels) continue;
                        uint8_t *h0 = mid_base + (size_t)pnl * kChunkBytes + (m + 2) * 16;
                        const int c0 = 4 * hlf;
                        *reinterpret_cast<uint4 *>(h0) =
                            make_uint4(hw[c0], hw[c0 + 1], hw[c0 + 2], hw[c0 + 3]);
                        *reinterpret_cast<uint4 *>(h0 + kMidPlane) =
                            make_uint4(lw[c0], lw[c0 + 1], lw[c0 + 2], lw[c0 + 3]);
                    }
                });
                if (stop) break;
                // the intermediate is an MMA operand next
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(inter_ready);
            }
            {
                // step 2 -> the output plane
                const int y = Y0 - C::R + m;
                const bool mine = m >= C::R && m < kTile - C::R && y < p.g.ny;
                const bool fast = Y0 >= o.y0 && Y0 + C::H <= o.y1 && X0 >= o.x0 &&
                                  X0 + kTbCols <= o.x1;
                const bool row_in = y >= o.y0 && y < o.y1;
                run_step(kS2Windows, [&](int j, const float (&f)[16]) {
                    const int xb = X0 + 16 * j;
                    if (mine && xb < p.g.nx) store_block_split(o, f, y, xb, fast, row_in, ss2, mx2);
                });
                if (!stop && mine && cs2.k != 0 && !fast)
                    resplit_border(o, y, X0, grp, kTbGroups, kS2Windows - 1, cs2);
            }
        }
        if (!stop && p.scale) {  // tile 0 is CTA 0's
            cta_scale_flush<kTbEpiWarps>(cs, 0, p.scale, p.t0 + 1, ss1, mx1, blockIdx.x == 0);
            cta_scale_flush<kTbEpiWarps>(cs, 1, p.scale, p.t0 + 2, ss2, mx2, blockIdx.x == 0);
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

int g_tb_sms = 0;

template <int S>
cudaError_t launch_tb(const GridGeom &g, const float *B, const uint16_t *in_hi,
                      const uint16_t *in_lo, uint16_t *out_hi, uint16_t *out_lo, cudaStream_t s,
                      SplitScale *scale, int t0) {
    using C = TbCfg<S>;
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(tc_split_tb_kernel<S>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(C::SMEM));
        if (e != cudaSuccess) return e;
        configured = true;
    }
    if (!g_tb_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_tb_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_tb_sms <= 0) g_tb_sms = 1;
    }
    TbParams p;
    p.g = g;
    p.tiles_x = (g.nx + kTbCols - 1) / kTbCols;
    p.n_tiles = p.tiles_x * ((g.ny + C::H - 1) / C::H);
    p.in_hi = in_hi;
    p.in_lo = in_lo;
    p.out_hi = out_hi;
    p.out_lo = out_lo;
    p.scale = scale;
    p.t0 = t0;
    for (int k = 0; k < 25; k++) p.coef[k] = k < C::NDY * C::NDY ? B[k] : 0.0f;
    const int grid = p.n_tiles < g_tb_sms ? p.n_tiles : g_tb_sms;
    return launch_step(tc_split_tb_kernel<S>, grid, kTbThreads, C::SMEM, s, p);
}

}  // namespace

cudaError_t launch_tc_split2(const GridGeom &g, int stencil, const float *B, const uint16_t *in_hi,
                             const uint16_t *in_lo, uint16_t *out_hi, uint16_t *out_lo,
                             cudaStream_t s, SplitScale *scale, int t0) {
    switch (stencil) {
    case TCS_STAR2D1R: return launch_tb<TCS_STAR2D1R>(g, B, in_hi, in_lo, out_hi, out_lo, s, scale, t0);
    case TCS_STAR2D2R: return launch_tb<TCS_STAR2D2R>(g, B, in_hi, in_lo, out_hi, out_lo, s, scale, t0);
    case TCS_BOX2D1R: return launch_tb<TCS_BOX2D1R>(g, B, in_hi, in_lo, out_hi, out_lo, s, scale, t0);
    case TCS_BOX2D2R: return launch_tb<TCS_BOX2D2R>(g, B, in_hi, in_lo, out_hi, out_lo, s, scale, t0);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t tb_take_error(int *code) {
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(code, g_tb_error, sizeof(int));
    if (e != cudaSuccess) return e;
    return *code ? cudaMemcpyToSymbol(g_tb_error, &zero, sizeof(int)) : cudaSuccess;
}

}  // namespace tcs
