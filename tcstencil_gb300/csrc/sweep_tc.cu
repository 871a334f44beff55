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
// in tensor memory (TMEM).  The split form works in two 64-column sub-tiles
// so that its two accumulators per sub-tile still double-buffer in TMEM.
//
// Staging.  Planes are column panels (8 cells x all rows, 16 bytes per row,
// rows contiguous; see tcs_internal.h), so the 132 input rows a tile needs
// from one panel (two halo rows above and below) are one contiguous 2112-byte
// run: the producer fetches the 18 panels of a tile (16 + one each side) with
// 18 1-D bulk copies.  The shared-memory image, chunk s = all 132 rows of
// panel s at a 16-byte row stride, is directly a no-swizzle K-major UMMA
// operand (8-row x 16-byte core matrices, SBO = 128 B between row groups,
// LBO = 2112 B between K chunks), and a row shift dy is +16*dy bytes on the
// descriptor start address.
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
// Pipeline (persistent, one CTA per SM, 6 warps):
//   warp 0      producer: bulk copies of each tile's panels into NS stages
//   warp 1      TMEM allocator and single-thread MMA issuer
//   warps 2..5  epilogue: TMEM -> registers -> FP16 (or hi/lo) -> global
// Two accumulator buffers let the epilogue of one (sub-)tile overlap the MMAs
// of the next.  Every wait is bounded; on timeout the kernel records an error
// word, stops, drains its own copies and MMAs, frees TMEM and returns.
#include "tcs_device.cuh"
#include "tcs_internal.h"

namespace tcs {

namespace {

__device__ int g_tc_error = 0;

constexpr int kRowsStaged = kTile + 4;           // two halo rows above and below
constexpr int kChunkBytes = kRowsStaged * 16;    // one panel of the stage
constexpr int kSlots = kTile / 8 + 2;            // 16 panels + one each side
constexpr int kPlaneStage = kSlots * kChunkBytes;
constexpr int kBandBytes = 32 * 16 * 2;          // one 16(K) x 32(N) FP16 band
constexpr int kEpiWarps = 8;                     // two warpgroups, one per column half
constexpr int kThreads = 32 * (2 + kEpiWarps);
constexpr uint32_t kIdesc = idesc_f16_f32(128, 32);

template <int S, bool SPLIT>
struct Cfg {
    static constexpr int R = stencil_r(S);
    static constexpr bool BOX = stencil_box(S);
    static constexpr int NDY = 2 * R + 1;                 // coefficient rows
    static constexpr int NSUB = SPLIT ? 2 : 1;            // sub-tiles per tile
    static constexpr int SUB_BLOCKS = kTile / 16 / NSUB;  // 16-column output blocks per sub-tile
    static constexpr int SUB_WIN = SUB_BLOCKS + 1;        // input windows per sub-tile
    static constexpr int ACC_PLANE = 16 * (SUB_BLOCKS + 2);  // TMEM columns per accumulator
    static constexpr int ACC = ACC_PLANE * (SPLIT ? 2 : 1);
    static constexpr int TMEM_COLS = 512;
    static_assert(2 * ACC <= TMEM_COLS, "two accumulator buffers must fit in TMEM");
    static constexpr int PLANES = SPLIT ? 2 : 1;          // hi (and lo) data planes
    static constexpr int BAND_PLANES = SPLIT ? 4 : 1;     // ch (and cf, cl, c3)
    static constexpr int STAGES = SPLIT ? 2 : 4;
    static constexpr size_t SMEM = 1024 + (size_t)STAGES * PLANES * kPlaneStage +
                                   (size_t)BAND_PLANES * NDY * kBandBytes + 256;
    static_assert(SMEM <= 232448, "shared memory budget");
};

struct TcParams {
    GridGeom g;
    int tiles_x, n_tiles;
    const uint16_t *in_hi, *in_lo;  // input planes
    uint16_t *out_hi, *out_lo;
    float coef[25];                 // n x n, row-major
};

__device__ __forceinline__ uint16_t h_bits(float v) {
    __half h = __float2half_rn(v);
    return *reinterpret_cast<uint16_t *>(&h);
}
__device__ __forceinline__ float h_val(uint16_t b) {
    __half h = *reinterpret_cast<__half *>(&b);
    return __half2float(h);
}

// Fixed-point split of a value v (|v| about 1 or below): hi = fp16 of
// rint(v 2^11) 2^-11, lo = fp16((v - hi) 2^11).
__device__ __forceinline__ void split_fixed(float v, uint16_t &hi, uint16_t &lo) {
    hi = h_bits(rintf(v * 2048.0f) * (1.0f / 2048.0f));
    lo = h_bits((v - h_val(hi)) * 2048.0f);
}

template <int S, bool SPLIT>
__global__ void __launch_bounds__(kThreads, 1) tc_sweep_kernel(const TcParams p) {
    using C = Cfg<S, SPLIT>;
    constexpr int R = C::R;
    constexpr int NS = C::STAGES;
    constexpr int NP = C::PLANES;
    constexpr int NSUB = C::NSUB;

    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                ~static_cast<uintptr_t>(1023));
    uint8_t *stage_base = smem;                                    // [NS][NP][stage]
    uint8_t *band_base = smem + (size_t)NS * NP * kPlaneStage;     // [BAND_PLANES][NDY]
    uint64_t *bars =
        reinterpret_cast<uint64_t *>(band_base + C::BAND_PLANES * C::NDY * kBandBytes);
    uint64_t *full = bars;                    // [NS]
    uint64_t *empty = bars + NS;              // [NS]
    uint64_t *acc_full = bars + 2 * NS;       // [2]
    uint64_t *acc_empty = bars + 2 * NS + 2;  // [2]
    uint64_t *drain = bars + 2 * NS + 4;      // [1]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * NS + 5);
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
        for (int b = 0; b < 2; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], kEpiWarps);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        __syncwarp();
        tmem_alloc(tmem_slot, C::TMEM_COLS);
        tmem_relinquish();
    }
    // Bands, K-major core-matrix layout: element (n, k) of the band of
    // coefficient row dy at dy*512 + (k/8)*256 + n*8 + k%8.  Input column k of
    // a window feeds output column n of its 32-column range with tap
    // dx = 8 + k - n.
    for (int idx = threadIdx.x; idx < C::NDY * 512; idx += kThreads) {
        const int dy = idx >> 9, n = (idx >> 4) & 31, k = idx & 15;
        const int dx = 8 + k - n;
        const bool on_axis = C::BOX || dy == R || dx == 0;
        float c = 0.0f;
        if (dx >= -R && dx <= R && on_axis) c = p.coef[dy * (2 * R + 1) + dx + R];
        const int off = dy * 512 + (k >> 3) * 256 + n * 8 + (k & 7);
        uint16_t *band = reinterpret_cast<uint16_t *>(band_base);
        if (!SPLIT) {
            band[off] = h_bits(c);
        } else {
            const float ch = rintf(c * 2048.0f) * (1.0f / 2048.0f);
            const float rem = (c - ch) * 2048.0f;  // exact
            const uint16_t cl = h_bits(rem);
            band[off] = h_bits(ch);                                  // ch: fixed point
            band[C::NDY * 512 + off] = h_bits(c);                    // cf: fp16(c), multiplies lo
            band[2 * C::NDY * 512 + off] = cl;                       // cl
            band[3 * C::NDY * 512 + off] = h_bits(rem - h_val(cl));  // c3
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
                const int Y0 = (t / tiles_x) * kTile;
                const int X0 = (t % tiles_x) * kTile;
                mbar_arrive_expect_tx(&full[s], NP * kPlaneStage);
                // rows Y0-2 .. Y0+129 of panels X0/8 - 1 .. X0/8 + 16
                const size_t src0 = plane_index(pg, Y0 - 2, X0 - 8);
#pragma unroll
                for (int pl = 0; pl < NP; pl++) {
                    const uint16_t *src = (pl ? p.in_lo : p.in_hi) + src0;
                    uint8_t *st = stage_base + ((size_t)s * NP + pl) * kPlaneStage;
#pragma unroll 1
                    for (int c = 0; c < kSlots; c++)
                        bulk_load(st + c * kChunkBytes, src + (size_t)c * pg.nyp * 8, kChunkBytes,
                                  &full[s]);
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
            bool stop = false;
            const uint64_t b_desc0 = smem_desc(smem_u32(band_base), 512, 128);
            for (int t = blockIdx.x; t < n_tiles && !stop; t += gridDim.x, i++) {
                const int s = i % NS;
                if (!mbar_wait(&full[s], (i / NS) & 1, abort_flag)) {
                    record_error(&g_tc_error, kErrWaitFull);
                    *abort_flag = 1;
                    break;
                }
                // Descriptors: the start-address field holds (address >> 4)
                // in its low bits, so a descriptor for base + offset is the
                // base descriptor plus offset >> 4 (compile-time offsets).
                const uint64_t a_hi0 =
                    smem_desc(smem_u32(stage_base + ((size_t)s * NP) * kPlaneStage), kChunkBytes, 128);
                const uint64_t a_lo0 = a_hi0 + (kPlaneStage >> 4);
#pragma unroll
                for (int h = 0; h < NSUB; h++) {
                    const int k = i * NSUB + h;  // sub-tile counter
                    const int b = k & 1;
                    if (!mbar_wait(&acc_empty[b], ((k >> 1) & 1) ^ 1, abort_flag)) {
                        record_error(&g_tc_error, kErrWaitAccum);
                        *abort_flag = 1;
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d_main = tmem_base + b * C::ACC;
                    const uint32_t d_corr = d_main + C::ACC_PLANE;
                    // even windows (disjoint outputs, initialise), then odd windows
#pragma unroll
                    for (int parity = 0; parity < 2; parity++) {
#pragma unroll
                        for (int dy = 0; dy < C::NDY; dy++) {
                            const uint64_t b_ch = b_desc0 + (uint64_t)((dy * kBandBytes) >> 4);
                            const uint32_t acc = (parity == 1 || dy > 0) ? 1u : 0u;
#pragma unroll
                            for (int w = parity; w < C::SUB_WIN; w += 2) {
                                const int wg = h * C::SUB_BLOCKS + w;  // window in the tile
                                const uint64_t a_off =
                                    (uint64_t)((2 * wg * kChunkBytes + (2 - R + dy) * 16) >> 4);
                                umma_f16(d_main + 16 * w, a_hi0 + a_off, b_ch, kIdesc, acc);
                                if (SPLIT) {
                                    const uint64_t b_cf = b_desc0 + (uint64_t)(((C::NDY + dy) * kBandBytes) >> 4);
                                    const uint64_t b_cl = b_desc0 + (uint64_t)(((2 * C::NDY + dy) * kBandBytes) >> 4);
                                    const uint64_t b_c3 = b_desc0 + (uint64_t)(((3 * C::NDY + dy) * kBandBytes) >> 4);
                                    umma_f16(d_corr + 16 * w, a_lo0 + a_off, b_cf, kIdesc, acc);
                                    umma_f16(d_corr + 16 * w, a_hi0 + a_off, b_cl, kIdesc, 1);
                                    umma_f16(d_corr + 16 * w, a_hi0 + a_off, b_c3, kIdesc, 1);
                                }
                            }
                        }
                    }
                    umma_commit(&acc_full[b]);
                    issued_any = true;
                }
                umma_commit(&empty[s]);
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
        const int q = warp & 3;       // TMEM lane quarter of this warp
        const int half = (warp - 2) >> 2;  // which half of a sub-tile's column blocks
        const int m = q * 32 + lane;  // output row within the tile
        const GridGeom &g = p.g;
        int i = 0;
        bool stop = false;
        for (int t = blockIdx.x; t < n_tiles && !stop; t += gridDim.x, i++) {
            const int Y0 = (t / tiles_x) * kTile;
            const int X0 = (t % tiles_x) * kTile;
            const bool fast = Y0 >= g.y0 && Y0 + kTile <= g.y1 && X0 >= g.x0 && X0 + kTile <= g.x1;
            const int y = Y0 + m;
            const bool row_in = y >= g.y0 && y < g.y1;
#pragma unroll 1
            for (int h = 0; h < NSUB; h++) {
                const int k = i * NSUB + h;
                const int b = k & 1;
                bool ok = mbar_wait(&acc_full[b], (k >> 1) & 1, abort_flag);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) {
                    if (lane == 0) {
                        record_error(&g_tc_error, kErrWaitResult);
                        *abort_flag = 1;
                    }
                    stop = true;
                    break;
                }
                tc_fence_after();
                // output block jl of the sub-tile is accumulator column 16(jl+1)
                const uint32_t lane_addr =
                    tmem_base + ((uint32_t)(q * 32) << 16) + b * C::ACC + 16;
                // G blocks per TMEM round trip: all their loads are issued
                // before one wait, so the load latency is paid once per group.
                constexpr int G = C::SUB_BLOCKS / 2;  // this warp's blocks, one round trip
                {
                    const int j0 = half * G;
                    uint32_t v[G][16];
                    uint32_t w[SPLIT ? G : 1][16];
#pragma unroll
                    for (int gg = 0; gg < G; gg++) {
                        tmem_ld_x16(lane_addr + 16 * (j0 + gg), v[gg]);
                        if (SPLIT) tmem_ld_x16(lane_addr + C::ACC_PLANE + 16 * (j0 + gg), w[SPLIT ? gg : 0]);
                    }
                    tmem_ld_wait();
#pragma unroll
                    for (int gg = 0; gg < G; gg++) {
                        const int xb = X0 + 16 * (h * C::SUB_BLOCKS + j0 + gg);
                        const size_t off0 = plane_index(pg, y, xb);      // cells xb .. xb+7
                        const size_t off1 = off0 + (size_t)pg.nyp * 8;   // cells xb+8 .. xb+15
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
                                uint16_t h0, h1, l0 = 0, l1 = 0;
                                if (SPLIT) {
                                    split_fixed(f[2 * c], h0, l0);
                                    split_fixed(f[2 * c + 1], h1, l1);
                                } else {
                                    h0 = h_bits(f[2 * c]);
                                    h1 = h_bits(f[2 * c + 1]);
                                }
                                hw[c] = (uint32_t)h0 | ((uint32_t)h1 << 16);
                                lw[c] = (uint32_t)l0 | ((uint32_t)l1 << 16);
                            }
                        } else {
                            // Border tile: cells outside the update rectangle copy the input.
                            const uint4 i0 = *reinterpret_cast<const uint4 *>(p.in_hi + off0);
                            const uint4 i1 = *reinterpret_cast<const uint4 *>(p.in_hi + off1);
                            const uint32_t iw[8] = {i0.x, i0.y, i0.z, i0.w, i1.x, i1.y, i1.z, i1.w};
                            uint32_t il[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                            if (SPLIT) {
                                const uint4 l0 = *reinterpret_cast<const uint4 *>(p.in_lo + off0);
                                const uint4 l1 = *reinterpret_cast<const uint4 *>(p.in_lo + off1);
                                il[0] = l0.x; il[1] = l0.y; il[2] = l0.z; il[3] = l0.w;
                                il[4] = l1.x; il[5] = l1.y; il[6] = l1.z; il[7] = l1.w;
                            }
#pragma unroll
                            for (int c = 0; c < 8; c++) {
                                uint16_t hh[2], ll[2];
#pragma unroll
                                for (int u = 0; u < 2; u++) {
                                    const int x = xb + 2 * c + u;
                                    const bool upd = row_in && x >= g.x0 && x < g.x1;
                                    if (upd) {
                                        if (SPLIT) split_fixed(f[2 * c + u], hh[u], ll[u]);
                                        else { hh[u] = h_bits(f[2 * c + u]); ll[u] = 0; }
                                    } else {
                                        hh[u] = (uint16_t)(iw[c] >> (16 * u));
                                        ll[u] = (uint16_t)(il[c] >> (16 * u));
                                    }
                                }
                                hw[c] = (uint32_t)hh[0] | ((uint32_t)hh[1] << 16);
                                lw[c] = (uint32_t)ll[0] | ((uint32_t)ll[1] << 16);
                            }
                        }
                        *reinterpret_cast<uint4 *>(p.out_hi + off0) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                        *reinterpret_cast<uint4 *>(p.out_hi + off1) = make_uint4(hw[4], hw[5], hw[6], hw[7]);
                        if (SPLIT) {
                            *reinterpret_cast<uint4 *>(p.out_lo + off0) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
                            *reinterpret_cast<uint4 *>(p.out_lo + off1) = make_uint4(lw[4], lw[5], lw[6], lw[7]);
                        }
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&acc_empty[b]);
            }
        }
    }

    // -------------------------------------------------------- teardown ---
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) {
        __syncwarp();
        tmem_dealloc(tmem_base, C::TMEM_COLS);
    }
}

int g_num_sms = 0;

// Sets the kernel's shared-memory limit and reads the SM count; called before
// any launch (and so before any stream capture of one).
template <int S, bool SPLIT>
cudaError_t prepare_tc() {
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(tc_sweep_kernel<S, SPLIT>,
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

template <int S, bool SPLIT>
cudaError_t launch_tc(const GridGeom &g, const float *B, const uint16_t *in_hi,
                      const uint16_t *in_lo, uint16_t *out_hi, uint16_t *out_lo, cudaStream_t s) {
    using C = Cfg<S, SPLIT>;
    cudaError_t pe = prepare_tc<S, SPLIT>();
    if (pe != cudaSuccess) return pe;
    TcParams p;
    p.g = g;
    const int tiles_y = (g.ny + kTile - 1) / kTile;
    p.tiles_x = (g.nx + kTile - 1) / kTile;
    p.n_tiles = tiles_y * p.tiles_x;
    p.in_hi = in_hi;
    p.in_lo = in_lo;
    p.out_hi = out_hi;
    p.out_lo = out_lo;
    for (int k = 0; k < 25; k++) p.coef[k] = 0.0f;
    for (int k = 0; k < C::NDY * C::NDY; k++) p.coef[k] = B[k];
    const int grid = p.n_tiles < g_num_sms ? p.n_tiles : g_num_sms;
    tc_sweep_kernel<S, SPLIT><<<grid, kThreads, C::SMEM, s>>>(p);
    return cudaGetLastError();
}

template <bool SPLIT>
cudaError_t dispatch_tc(const GridGeom &g, int stencil, const float *B, const uint16_t *in_hi,
                        const uint16_t *in_lo, uint16_t *out_hi, uint16_t *out_lo, cudaStream_t s) {
    switch (stencil) {
    case TCS_STAR2D1R: return launch_tc<TCS_STAR2D1R, SPLIT>(g, B, in_hi, in_lo, out_hi, out_lo, s);
    case TCS_STAR2D2R: return launch_tc<TCS_STAR2D2R, SPLIT>(g, B, in_hi, in_lo, out_hi, out_lo, s);
    case TCS_BOX2D1R: return launch_tc<TCS_BOX2D1R, SPLIT>(g, B, in_hi, in_lo, out_hi, out_lo, s);
    case TCS_BOX2D2R: return launch_tc<TCS_BOX2D2R, SPLIT>(g, B, in_hi, in_lo, out_hi, out_lo, s);
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
                          uint16_t *out, cudaStream_t s) {
    return dispatch_tc<false>(g, stencil, B, in, nullptr, out, nullptr, s);
}

cudaError_t launch_tc_split(const GridGeom &g, int stencil, const float *B, const uint16_t *in_hi,
                            const uint16_t *in_lo, uint16_t *out_hi, uint16_t *out_lo,
                            cudaStream_t s) {
    return dispatch_tc<true>(g, stencil, B, in_hi, in_lo, out_hi, out_lo, s);
}

}  // namespace tcs
