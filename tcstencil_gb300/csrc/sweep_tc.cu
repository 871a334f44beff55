// Tensor-core sweep kernels: one Jacobi step as banded-matrix products on the
// 5th-generation tensor cores (tcgen05), the GB300 counterpart of the
// reference's wmma `mma_run` (layout16/kernel_*.cu).
//
// Formulation.  For an output tile of 128 rows x 128 columns, with rows in the
// MMA's M dimension and columns in N, a box stencil is
//     D = sum_{dy} S_dy(X) * H_dy
// where S_dy(X) is the staged input shifted down by dy rows and H_dy is the
// horizontal band of coefficient row dy.  D is produced 16 columns at a time
// (N = 16); the K window of a 16-column block is 32 input columns (two K=16
// steps: [x-8, x+8) and [x+8, x+24)), which covers a radius-2 halo.  A star
// stencil uses the same two steps for its centre row and a single K=16 step
// with a diagonal band for each off-centre row.  FP16 operands, FP32
// accumulators in tensor memory (TMEM).
//
// Staging.  Each tile's input (its 8x8 bricks plus one brick row above and
// below and one 8-column chunk left and right) is fetched by TMA from the
// brick grid through a 5-D view (8 cells, 16 rows, brick row, half brick,
// brick column) into a chunk-planar shared-memory image: chunk s holds all
// 160 staged rows of 8 columns at a 16-byte row stride.  That image is
// directly a no-swizzle K-major UMMA operand (8-row x 16-byte core matrices,
// SBO = 128 B between row groups, LBO = 160*16 B between K chunks), and a
// row shift dy is just +16*dy bytes on the descriptor start address.
//
// Pipeline (persistent, one CTA per SM, 6 warps):
//   warp 0      TMA producer (3 loads per tile and plane) into NS stages
//   warp 1      TMEM allocator and single-thread MMA issuer
//   warps 2..5  epilogue: TMEM -> registers -> FP16 (or hi/lo) -> global
// Two accumulator buffers let the epilogue of tile i overlap the MMAs of i+1.
// Every wait is bounded; on timeout the kernel records an error word, stops,
// drains its own copies and MMAs, frees TMEM and returns.
#include "tcs_device.cuh"
#include "tcs_internal.h"

namespace tcs {

namespace {

__device__ int g_tc_error = 0;

constexpr int kTileBricks = kTcTileBricks;      // tile = 8 x 8 bricks = 128 x 128 cells
constexpr int kTileRows = kTileBricks * 16;     // 128 (= UMMA M)
constexpr int kStagedRows = kTileRows + 32;     // one brick row above and below
constexpr int kSlots = kTileBricks * 2 + 2;     // 8-column chunks incl. the two halo chunks
constexpr int kChunkBytes = kStagedRows * 16;   // 2560
constexpr int kPlaneStageBytes = kSlots * kChunkBytes;  // 46080
constexpr int kBandBytes = 512;                 // one 16(N) x 16(K) FP16 band block
constexpr int kThreads = 192;
constexpr uint32_t kIdesc = idesc_f16_f32(128, 16);

// MMA schedule of one 16-column output block: each entry multiplies the
// staged input (K window starting at chunk slot 2j + slot_off, rows shifted
// by dy - r) with band block `band`.  `ws` is the window's first column
// relative to the block's first output column.
struct Entry {
    int dy, slot_off, ws;
};

template <int S>
struct Schedule {
    static constexpr int R = stencil_r(S);
    static constexpr bool BOX = stencil_box(S);
    static constexpr int N = BOX ? (2 * R + 1) * 2 : 2 + 2 * R;
    __host__ __device__ static constexpr Entry at(int e) {
        if (BOX) return Entry{e / 2, (e % 2) * 2, (e % 2) ? 8 : -8};
        if (e < 2) return Entry{R, e * 2, e ? 8 : -8};
        const int k = e - 2;  // off-centre rows, top to bottom, skipping the centre
        const int dy = k < R ? k : k + 1;
        return Entry{dy, 1, 0};
    }
};

template <bool SPLIT>
struct Cfg {
    static constexpr int kPlanes = SPLIT ? 2 : 1;      // data planes (hi, lo)
    static constexpr int kBandPlanes = SPLIT ? 3 : 1;  // coefficient pieces (ch, cl, c3)
    static constexpr int kStages = SPLIT ? 2 : 3;
    static constexpr int kAccCols = SPLIT ? 256 : 128;  // per accumulator buffer
    static constexpr int kTmemCols = 2 * kAccCols;
};

struct TcParams {
    GridGeom g;
    int tiles_x, n_tiles;
    const uint16_t *in_hi, *in_lo;  // input planes (border copies)
    uint16_t *out_hi, *out_lo;
    float coef[25];                 // n x n, row-major
};

template <int S, bool SPLIT>
constexpr size_t smem_bytes() {
    using C = Cfg<SPLIT>;
    return 1024 + (size_t)C::kStages * C::kPlanes * kPlaneStageBytes +
           (size_t)C::kBandPlanes * Schedule<S>::N * kBandBytes + 256;
}

__device__ __forceinline__ uint16_t h_bits(float v) {
    __half h = __float2half_rn(v);
    return *reinterpret_cast<uint16_t *>(&h);
}
__device__ __forceinline__ float h_val(uint16_t b) {
    __half h = *reinterpret_cast<__half *>(&b);
    return __half2float(h);
}

template <int S, bool SPLIT>
__global__ void __launch_bounds__(kThreads, 1)
    tc_sweep_kernel(const __grid_constant__ CUtensorMap map_hi_main,
                    const __grid_constant__ CUtensorMap map_hi_halo,
                    const __grid_constant__ CUtensorMap map_lo_main,
                    const __grid_constant__ CUtensorMap map_lo_halo, const TcParams p) {
    using C = Cfg<SPLIT>;
    using Sch = Schedule<S>;
    constexpr int R = Sch::R;
    constexpr int NE = Sch::N;
    constexpr int NS = C::kStages;
    constexpr int NP = C::kPlanes;

    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                ~static_cast<uintptr_t>(1023));
    uint8_t *stage_base = smem;                                        // [NS][NP][46080]
    uint8_t *band_base = smem + (size_t)NS * NP * kPlaneStageBytes;    // [NBP][NE][512]
    uint64_t *bars =
        reinterpret_cast<uint64_t *>(band_base + C::kBandPlanes * NE * kBandBytes);
    uint64_t *full = bars;             // [NS]
    uint64_t *empty = bars + NS;       // [NS]
    uint64_t *acc_full = bars + 2 * NS;       // [2]
    uint64_t *acc_empty = bars + 2 * NS + 2;  // [2]
    uint64_t *drain = bars + 2 * NS + 4;      // [1]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * NS + 5);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;

    // ---------------------------------------------------------- set-up ---
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        fence_mbar_init();
        tma_prefetch_map(&map_hi_main);
        tma_prefetch_map(&map_hi_halo);
        if (SPLIT) {
            tma_prefetch_map(&map_lo_main);
            tma_prefetch_map(&map_lo_halo);
        }
    }
    if (warp == 1) {
        tmem_alloc(tmem_slot, C::kTmemCols);
        tmem_relinquish();
    }
    // Band blocks, K-major core-matrix layout: element (n, k) of block e at
    // e*256 + (k/8)*128 + n*8 + k%8.  The split form stores three pieces of
    // each coefficient, c = ch + 2^-11 (cl + c3); every step before the last
    // rounding of each piece is exact in FP32.
    for (int idx = threadIdx.x; idx < NE * 256; idx += kThreads) {
        const int e = idx >> 8, n = (idx >> 4) & 15, k = idx & 15;
        const Entry en = Sch::at(e);
        const int dx = en.ws + k - n;
        const bool on_axis = Sch::BOX || en.dy == R || dx == 0;
        float c = 0.0f;
        if (dx >= -R && dx <= R && on_axis) c = p.coef[en.dy * (2 * R + 1) + dx + R];
        const int off = e * 256 + (k >> 3) * 128 + n * 8 + (k & 7);
        uint16_t *band = reinterpret_cast<uint16_t *>(band_base);
        const uint16_t hi = h_bits(c);
        band[off] = hi;
        if (SPLIT) {
            const float rem = (c - h_val(hi)) * 2048.0f;
            const uint16_t lo = h_bits(rem);
            band[NE * 256 + off] = lo;
            band[2 * NE * 256 + off] = h_bits(rem - h_val(lo));
        }
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    const int tiles_x = p.tiles_x;
    const int n_tiles = p.n_tiles;

    if (warp == 0) {
        // ------------------------------------------------------ producer ---
        if (lane == 0) {
            int i = 0;
            int last_issued = -1;
            for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, i++) {
                const int s = i % NS;
                const uint32_t ph = (i / NS) & 1;
                if (!mbar_wait(&empty[s], ph ^ 1, abort_flag)) {
                    record_error(&g_tc_error, kErrWaitEmpty);
                    *abort_flag = 1;
                    break;
                }
                const int by0 = (t / tiles_x) * kTileBricks;
                const int bx0 = (t % tiles_x) * kTileBricks;
                mbar_arrive_expect_tx(&full[s], NP * kPlaneStageBytes);
#pragma unroll
                for (int pl = 0; pl < NP; pl++) {
                    const CUtensorMap *mm = pl ? &map_lo_main : &map_hi_main;
                    const CUtensorMap *mh = pl ? &map_lo_halo : &map_hi_halo;
                    uint8_t *st = stage_base + ((size_t)s * NP + pl) * kPlaneStageBytes;
                    tma_load_5d(st + kChunkBytes, mm, &full[s], 0, 0, by0 - 1, 0, bx0);
                    tma_load_5d(st, mh, &full[s], 0, 0, by0 - 1, 1, bx0 - 1);
                    tma_load_5d(st + (kSlots - 1) * kChunkBytes, mh, &full[s], 0, 0, by0 - 1, 0,
                                bx0 + kTileBricks);
                }
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
    } else if (warp == 1) {
        // ---------------------------------------------------- MMA issuer ---
        if (lane == 0) {
            int i = 0;
            bool issued_any = false;
            for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, i++) {
                const int s = i % NS;
                const int b = i & 1;
                if (!mbar_wait(&full[s], (i / NS) & 1, abort_flag)) {
                    record_error(&g_tc_error, kErrWaitFull);
                    *abort_flag = 1;
                    break;
                }
                if (!mbar_wait(&acc_empty[b], ((i >> 1) & 1) ^ 1, abort_flag)) {
                    record_error(&g_tc_error, kErrWaitAccum);
                    *abort_flag = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t d0 = tmem_base + b * C::kAccCols;
                const uint32_t st_hi = smem_u32(stage_base + ((size_t)s * NP) * kPlaneStageBytes);
                const uint32_t st_lo = st_hi + kPlaneStageBytes;
                const uint32_t bd_hi = smem_u32(band_base);
                const uint32_t bd_lo = bd_hi + NE * kBandBytes;
                const uint32_t bd_c3 = bd_lo + NE * kBandBytes;
#pragma unroll 1
                for (int j = 0; j < kTileBricks; j++) {
#pragma unroll
                    for (int e = 0; e < NE; e++) {
                        const Entry en = Sch::at(e);
                        const uint32_t a_off = (2 * j + en.slot_off) * kChunkBytes +
                                               (16 - R + en.dy) * 16;
                        const uint64_t a_hi = smem_desc(st_hi + a_off, kChunkBytes, 128);
                        const uint64_t b_hi = smem_desc(bd_hi + e * kBandBytes, 256, 128);
                        umma_f16(d0 + 16 * j, a_hi, b_hi, kIdesc, e > 0);
                        if (SPLIT) {
                            // correction accumulator, in units of 2^-11:
                            // ch*xl + cl*xh + c3*xh
                            const uint32_t dc = d0 + 128 + 16 * j;
                            const uint64_t a_lo = smem_desc(st_lo + a_off, kChunkBytes, 128);
                            const uint64_t b_lo = smem_desc(bd_lo + e * kBandBytes, 256, 128);
                            const uint64_t b_c3 = smem_desc(bd_c3 + e * kBandBytes, 256, 128);
                            umma_f16(dc, a_hi, b_lo, kIdesc, e > 0);
                            umma_f16(dc, a_lo, b_hi, kIdesc, 1);
                            umma_f16(dc, a_hi, b_c3, kIdesc, 1);
                        }
                    }
                }
                umma_commit(&empty[s]);
                umma_commit(&acc_full[b]);
                issued_any = true;
            }
            if (issued_any) {
                umma_commit(drain);
                const uint64_t t0 = global_timer_ns();
                while (!mbar_try_wait(drain, 0)) {
                    if (global_timer_ns() - t0 > kWaitLimitNs) {
                        record_error(&g_tc_error, kErrWaitDrain);
                        break;
                    }
                }
            }
        }
    } else {
        // ------------------------------------------------------ epilogue ---
        const int q = warp & 3;                 // TMEM lane quarter of this warp
        const int m = q * 32 + lane;            // output row within the tile
        const GridGeom &g = p.g;
        int i = 0;
        for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, i++) {
            const int b = i & 1;
            bool ok = mbar_wait(&acc_full[b], (i >> 1) & 1, abort_flag);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) {
                if (lane == 0) {
                    record_error(&g_tc_error, kErrWaitResult);
                    *abort_flag = 1;
                }
                break;
            }
            tc_fence_after();
            const int by0 = (t / tiles_x) * kTileBricks;
            const int bx0 = (t % tiles_x) * kTileBricks;
            const int Y0 = by0 * 16, X0 = bx0 * 16;
            const bool fast = Y0 >= g.y0 && Y0 + kTileRows <= g.y1 && X0 >= g.x0 &&
                              X0 + kTileRows <= g.x1;
            const int y = Y0 + m;
            const int by = by0 + (m >> 4);
            const bool row_in = y >= g.y0 && y < g.y1;
            const uint32_t lane_addr = tmem_base + ((uint32_t)(q * 32) << 16) + b * C::kAccCols;
            // G column blocks per TMEM round trip: all their loads are issued
            // before one wait, so the load latency is paid once per group.
            constexpr int G = SPLIT ? 2 : 4;
#pragma unroll 1
            for (int j0 = 0; j0 < kTileBricks; j0 += G) {
                uint32_t v[G][16];
                uint32_t w[SPLIT ? G : 1][16];
#pragma unroll
                for (int gg = 0; gg < G; gg++) {
                    tmem_ld_x16(lane_addr + 16 * (j0 + gg), v[gg]);
                    if (SPLIT) tmem_ld_x16(lane_addr + 128 + 16 * (j0 + gg), w[SPLIT ? gg : 0]);
                }
                tmem_ld_wait();
#pragma unroll
            for (int gg = 0; gg < G; gg++) {
                const int j = j0 + gg;
                const int bx = bx0 + j;
                if (by >= g.nby || bx >= g.nbx) continue;
                const size_t off = ((size_t)by * g.nbx + bx) * 256 + (size_t)(m & 15) * 16;
                float f[16];
#pragma unroll
                for (int c = 0; c < 16; c++) {
                    f[c] = __uint_as_float(v[gg][c]);
                    if (SPLIT) f[c] = fmaf(__uint_as_float(w[SPLIT ? gg : 0][c]), 1.0f / 2048.0f, f[c]);
                }
                uint32_t hw[8], lw[8];
                if (fast) {
#pragma unroll
                    for (int c = 0; c < 8; c++) {
                        const uint16_t h0 = h_bits(f[2 * c]), h1 = h_bits(f[2 * c + 1]);
                        hw[c] = (uint32_t)h0 | ((uint32_t)h1 << 16);
                        if (SPLIT) {
                            const uint16_t l0 = h_bits((f[2 * c] - h_val(h0)) * 2048.0f);
                            const uint16_t l1 = h_bits((f[2 * c + 1] - h_val(h1)) * 2048.0f);
                            lw[c] = (uint32_t)l0 | ((uint32_t)l1 << 16);
                        }
                    }
                } else {
                    // Border tile: cells outside the update rectangle copy the input.
                    const uint4 *ih = reinterpret_cast<const uint4 *>(p.in_hi + off);
                    const uint4 i0 = ih[0], i1 = ih[1];
                    const uint32_t iw[8] = {i0.x, i0.y, i0.z, i0.w, i1.x, i1.y, i1.z, i1.w};
                    uint32_t il[8];
                    if (SPLIT) {
                        const uint4 *iq = reinterpret_cast<const uint4 *>(p.in_lo + off);
                        const uint4 l0 = iq[0], l1 = iq[1];
                        il[0] = l0.x; il[1] = l0.y; il[2] = l0.z; il[3] = l0.w;
                        il[4] = l1.x; il[5] = l1.y; il[6] = l1.z; il[7] = l1.w;
                    }
#pragma unroll
                    for (int c = 0; c < 8; c++) {
                        uint16_t hh[2], ll[2];
#pragma unroll
                        for (int u = 0; u < 2; u++) {
                            const int x = X0 + 16 * j + 2 * c + u;
                            const bool upd = row_in && x >= g.x0 && x < g.x1;
                            if (upd) {
                                hh[u] = h_bits(f[2 * c + u]);
                                ll[u] = SPLIT ? h_bits((f[2 * c + u] - h_val(hh[u])) * 2048.0f) : 0;
                            } else {
                                hh[u] = (uint16_t)(iw[c] >> (16 * u));
                                ll[u] = SPLIT ? (uint16_t)(il[c] >> (16 * u)) : 0;
                            }
                        }
                        hw[c] = (uint32_t)hh[0] | ((uint32_t)hh[1] << 16);
                        lw[c] = (uint32_t)ll[0] | ((uint32_t)ll[1] << 16);
                    }
                }
                uint4 *oh = reinterpret_cast<uint4 *>(p.out_hi + off);
                oh[0] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                oh[1] = make_uint4(hw[4], hw[5], hw[6], hw[7]);
                if (SPLIT) {
                    uint4 *ol = reinterpret_cast<uint4 *>(p.out_lo + off);
                    ol[0] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
                    ol[1] = make_uint4(lw[4], lw[5], lw[6], lw[7]);
                }
            }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[b]);
        }
    }

    // -------------------------------------------------------- teardown ---
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem_base, C::kTmemCols);
}

int g_num_sms = 0;

// Sets the kernel's shared-memory limit and reads the SM count; called before
// any launch (and so before any stream capture of one).
template <int S, bool SPLIT>
cudaError_t prepare_tc() {
    static bool configured = false;
    constexpr size_t smem = smem_bytes<S, SPLIT>();
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(tc_sweep_kernel<S, SPLIT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
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

template <int S, bool SPLIT>
cudaError_t launch_tc(const GridGeom &g, const float *B, const PlaneMaps &hi, const PlaneMaps *lo,
                      const uint16_t *in_hi, const uint16_t *in_lo, uint16_t *out_hi,
                      uint16_t *out_lo, cudaStream_t s) {
    constexpr size_t smem = smem_bytes<S, SPLIT>();
    cudaError_t pe = prepare_tc<S, SPLIT>();
    if (pe != cudaSuccess) return pe;
    TcParams p;
    p.g = g;
    const int tiles_y = (g.nby + kTileBricks - 1) / kTileBricks;
    p.tiles_x = (g.nbx + kTileBricks - 1) / kTileBricks;
    p.n_tiles = tiles_y * p.tiles_x;
    p.in_hi = in_hi;
    p.in_lo = in_lo;
    p.out_hi = out_hi;
    p.out_lo = out_lo;
    const int r = stencil_r(S);
    for (int k = 0; k < 25; k++) p.coef[k] = 0.0f;
    for (int k = 0; k < (2 * r + 1) * (2 * r + 1); k++) p.coef[k] = B[k];
    const int grid = p.n_tiles < g_num_sms ? p.n_tiles : g_num_sms;
    const PlaneMaps &l = lo ? *lo : hi;
    tc_sweep_kernel<S, SPLIT><<<grid, kThreads, smem, s>>>(hi.main, hi.halo, l.main, l.halo, p);
    return cudaGetLastError();
}

template <bool SPLIT>
cudaError_t dispatch_tc(const GridGeom &g, int stencil, const float *B, const PlaneMaps &hi,
                        const PlaneMaps *lo, const uint16_t *in_hi, const uint16_t *in_lo,
                        uint16_t *out_hi, uint16_t *out_lo, cudaStream_t s) {
    switch (stencil) {
    case TCS_STAR2D1R: return launch_tc<TCS_STAR2D1R, SPLIT>(g, B, hi, lo, in_hi, in_lo, out_hi, out_lo, s);
    case TCS_STAR2D2R: return launch_tc<TCS_STAR2D2R, SPLIT>(g, B, hi, lo, in_hi, in_lo, out_hi, out_lo, s);
    case TCS_BOX2D1R: return launch_tc<TCS_BOX2D1R, SPLIT>(g, B, hi, lo, in_hi, in_lo, out_hi, out_lo, s);
    case TCS_BOX2D2R: return launch_tc<TCS_BOX2D2R, SPLIT>(g, B, hi, lo, in_hi, in_lo, out_hi, out_lo, s);
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

cudaError_t launch_tc_f16(const GridGeom &g, int stencil, const float *B, const PlaneMaps &in_maps,
                          const uint16_t *in, uint16_t *out, cudaStream_t s) {
    return dispatch_tc<false>(g, stencil, B, in_maps, nullptr, in, nullptr, out, nullptr, s);
}

cudaError_t launch_tc_split(const GridGeom &g, int stencil, const float *B,
                            const PlaneMaps &in_hi_maps, const PlaneMaps &in_lo_maps,
                            const uint16_t *in_hi, const uint16_t *in_lo, uint16_t *out_hi,
                            uint16_t *out_lo, cudaStream_t s) {
    return dispatch_tc<true>(g, stencil, B, in_hi_maps, &in_lo_maps, in_hi, in_lo, out_hi, out_lo,
                             s);
}

}  // namespace tcs
