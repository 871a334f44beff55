// CUDA-core sweep kernels (the counterpart of the reference's baseline/
// kernel_*.cu `kernel_run`, rebuilt for GB300).
//
// One CTA per tile of 128 rows by 16 panels (128 FP16 or 64 FP32 columns).
// One thread stages the tile's rows, with four halo rows above and below,
// and the panel on each side, as 18 bulk copies (a panel's rows are one
// contiguous run) into shared memory, where runs sit 2192 bytes apart so
// that the 16 panels of a row fall on different banks.  Four warps then
// take 32 rows each.  Lane l owns half a panel: cells [x_l, x_l + H) with
// H = 4 (FP16) or 2 (FP32), 8 bytes of each panel row; horizontal halo
// cells come from lanes l-1 and l+1 by shuffle (the same shuffle for every
// lane) and, for the outer lanes, from the side panels' runs.  The vertical
// taps come from a register window of six rows, two rows per step.  Each
// warp first reads the rows it shares with its neighbours, then writes its
// results over its own rows of the stage, and one thread stores the 16
// panels' rows back with 16 bulk copies.  Both directions go by the copy
// engine, not the load/store pipeline, which was this kernel's limit when
// it moved its rows through L1 (79 % of the L1 throughput at 0.43 of HBM;
// measured on GB300 at 8196², us per step, L1 -> bulk loads -> bulk loads
// and stores: star2d1r FP16 111.7 -> 73.9 -> 61.4, FP32 182 -> 124 -> 97.6).
// Five such CTAs fit an SM.  (Persistent CTAs walking tiles through two or
// three stages measured no faster.)  A warp whose rows and whose tile's
// columns all lie in the update rectangle (most warps of a large grid) runs
// its rows with no per-row tests and immediate row offsets; with that,
// star2d1r FP16 runs 57.9 -> 49.5 us per step at 8196², star2d2r 66.3 ->
// 55.0, box2d2r 95.1 -> 83.5 (FP32 97.7 -> 87.3, 109.4 -> 90.9, 160.1 -> 134.5),
// from the row overhead each lane carried: about 62 instructions per row
// beside the FMAs.
//
// Arithmetic follows gold's tap order (common/gold_*.cpp):
//  - FP16 storage: acc = fmaf chain from 0, FP32 coefficients, RNE to FP16.
//  - FP32 storage: gold's own unfused products and sums (__fmul_rn/__fadd_rn),
//    so the result is bit-identical to gold compiled without FMA contraction.
#include <type_traits>

#include "tcs_device.cuh"
#include "tcs_internal.h"

namespace tcs {

__device__ int g_cc_error = 0;  // first give-up code of a CUDA-core launch

namespace {

constexpr int kCcTileRows = 128;
constexpr int kCcPanels = 16;                          // panels a tile computes
constexpr int kCcRunRows = kCcTileRows + 8;            // staged rows: 4 above, 4 below
constexpr int kCcRunBytes = kCcRunRows * 16;           // one panel's run
constexpr int kCcRunStride = kCcRunBytes + 16;         // next panel 4 banks on
constexpr int kCcWarps = 4;                            // warps per CTA
constexpr int kCcWarpRows = kCcTileRows / kCcWarps;    // rows per warp (even)
constexpr int kCcRunsOffset = 128;                     // after the mbarrier
constexpr int kCcSmem = kCcRunsOffset + (kCcPanels + 2) * kCcRunStride;
static_assert(kCcWarpRows % 2 == 0, "two rows per step");

struct CcParams {
    GridGeom g;
    PlaneGeom p;   // plane of this precision
    int nchunks;   // panels that hold grid cells
    int tiles_x;
    int n_tiles;
};

__device__ __forceinline__ uint2 lds_v2(uint32_t addr) {
    uint2 v;
    asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(addr));
    return v;
}
__device__ __forceinline__ void sts_v2(uint32_t addr, uint2 v) {
    asm volatile("st.shared.v2.u32 [%0], {%1, %2};" ::"r"(addr), "r"(v.x), "r"(v.y) : "memory");
}
// 1-D bulk copy of `bytes` (a multiple of 16) from shared to global memory,
// both addresses 16-byte aligned, in this thread's bulk group.
__device__ __forceinline__ void bulk_store(void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(
                     reinterpret_cast<uint64_t>(dst)),
                 "r"(smem_u32(src)), "r"(bytes)
                 : "memory");
}
// Waits until this thread's bulk stores have read their shared memory.
__device__ __forceinline__ void bulk_store_commit_and_wait_read() {
    asm volatile("cp.async.bulk.commit_group;\n\tcp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ uint32_t lds_u32(uint32_t addr) {
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(addr));
    return v;
}

template <int S, bool F32>
__global__ void __launch_bounds__(kCcWarps * 32, 5)
    cc_sweep_kernel(const void *__restrict__ in_, void *__restrict__ out_, CcParams p,
                    TapCoeffs c) {
    constexpr int R = stencil_r(S);
    constexpr int V = F32 ? 4 : 8;                // cells per panel row
    constexpr int H = V / 2;                      // cells per lane
    constexpr int WPC = F32 ? 1 : 2;              // cells per 32-bit word
    constexpr int HW = (R + WPC - 1) / WPC;       // halo words each side
    constexpr int HC = HW * WPC;                  // halo cells each side
    constexpr int W = H + 2 * R;                  // window columns of a lane
    constexpr int NT = tap_count(S);
    constexpr bool BOX = stencil_box(S);
    using T = typename std::conditional<F32, float, uint16_t>::type;
    const T *__restrict__ in = static_cast<const T *>(in_);
    T *__restrict__ out = static_cast<T *>(out_);

    extern __shared__ __align__(128) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    const uint32_t runs = smem_u32(smem + kCcRunsOffset);

    const int tile = blockIdx.x;
    const int tx = tile % p.tiles_x, ty = tile / p.tiles_x;
    const int Y0 = ty * kCcTileRows;
    const int chunk0 = tx * kCcPanels;  // first panel of the tile
    const ptrdiff_t nyp = p.p.nyp;

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    // the previous step's CTAs may still run: planes only after pdl_wait
    pdl_wait();
    if (threadIdx.x == 0) {
        // staged run q = plane panel chunk0 + q (the panel left of chunk0 is
        // the plane's panel chunk0), plane rows Y0 .. Y0+135 (grid rows
        // Y0-4 .. Y0+131); runs past the plane are not staged and never read
        // by a cell of the update rectangle
        const int nq = min(kCcPanels + 2, p.p.npan - chunk0);
        mbar_arrive_expect_tx(bar, (uint32_t)(nq * kCcRunBytes));
        for (int q = 0; q < nq; q++)
            bulk_load(smem + kCcRunsOffset + q * kCcRunStride,
                      in + ((ptrdiff_t)(chunk0 + q) * nyp + Y0) * V, kCcRunBytes, bar);
    }
    __syncthreads();
    if (!__syncthreads_and(mbar_wait(bar, 0, &g_cc_error))) {  // every thread leaves, or none
        if (threadIdx.x == 0) record_error(&g_cc_error, kErrWaitFull);
        return;
    }

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int chunk = chunk0 + (lane >> 1);  // this lane's panel
    const bool active = chunk < p.nchunks;
    const int xl = chunk * V + (lane & 1) * H;  // first column this lane computes
    const int ys = Y0 + warp * kCcWarpRows;
    const int ye = min(ys + kCcWarpRows, p.g.ny);
    const bool has_rows = ys < p.g.ny;  // the same for the whole warp
    // shared address of tile row r (from -4) of this lane's half panel, and of
    // the outer lanes' edge words
    const uint32_t own0 = runs + (1 + (lane >> 1)) * kCcRunStride + 4 * 16 + (lane & 1) * 8;
    const uint32_t edge0 = lane == 0 ? runs + 4 * 16 + (V - HC) * (uint32_t)sizeof(T)
                                     : runs + (kCcPanels + 1) * kCcRunStride + 4 * 16;

    const bool is_l = lane == 0, is_r = lane == 31;
    // Window columns [0, W) of the stage row at byte offset r16 = (y - Y0) * 16:
    // cells xl-R .. xl+H+R-1 of grid row y.
    auto to_window = [&](uint32_t r16, float (&w)[W]) {
        const uint2 v = lds_v2(own0 + r16);
        const uint32_t own[2] = {v.x, v.y};
        uint32_t left[HW], right[HW];
#pragma unroll
        for (int k = 0; k < HW; k++) {
            left[k] = __shfl_up_sync(0xffffffffu, own[2 - HW + k], 1);
            right[k] = __shfl_down_sync(0xffffffffu, own[k], 1);
            // the outer lanes' halo words are in the side panels' runs: every
            // lane loads one (the inner lanes all the same word, discarded), so
            // the warp does not branch
            const uint32_t e = lds_u32(edge0 + r16 + 4 * k);
            left[k] = is_l ? e : left[k];
            right[k] = is_r ? e : right[k];
        }
        float cells[HC + H + HC];
        if constexpr (F32) {
#pragma unroll
            for (int k = 0; k < HW; k++) {
                cells[k] = __uint_as_float(left[k]);
                cells[HC + H + k] = __uint_as_float(right[k]);
            }
            cells[HC] = __uint_as_float(own[0]);
            cells[HC + 1] = __uint_as_float(own[1]);
        } else {
            const float2 l = unpack_half2(left[0]), rr = unpack_half2(right[0]);
            const float2 a = unpack_half2(own[0]), b = unpack_half2(own[1]);
            cells[0] = l.x; cells[1] = l.y;
            cells[2] = a.x; cells[3] = a.y; cells[4] = b.x; cells[5] = b.y;
            cells[6] = rr.x; cells[7] = rr.y;
        }
#pragma unroll
        for (int k = 0; k < W; k++) w[k] = cells[HC - R + k];
    };

    // Rows y0, y0+1 from the window rows y0-2 .. y0+3, held as three row
    // pairs p0, p1, p2, in gold's tap order.
    auto compute = [&](const float (&p0)[2][W], const float (&p1)[2][W], const float (&p2)[2][W],
                       float (&acc)[2][H]) {
        auto row = [&](int wr) -> const float (&)[W] {
            return wr < 2 ? p0[wr] : wr < 4 ? p1[wr - 2] : p2[wr - 4];
        };
        if constexpr (!F32 && (R == 1 || !BOX)) {
            // packed FP32 FMAs on cell pairs, taps outside the rows so that
            // one coefficient pair serves both rows; each lane rounds as
            // fmaf does, so the bits are the same (measured at 8196², us per
            // step: star2d1r 61.4 -> 57.9 and box2d1r 66.4 -> 63.4 before
            // the interior path, star2d2r 55.0 -> 51.8 after it; box2d2r,
            // whose 25 taps then spill registers, 83.0 -> 92.5, keeps the
            // scalar chain)
            float2 a2[2][H / 2];
#pragma unroll
            for (int k = 0; k < NT; k++) {
                const int dy = tap_dy(S, k), dx = tap_dx(S, k);
                const float2 cc = make_float2(c.c[k], c.c[k]);
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const float (&x)[W] = row(2 + q + dy);
#pragma unroll
                    for (int i = 0; i < H; i += 2) {
                        const float2 x2 = make_float2(x[R + i + dx], x[R + i + 1 + dx]);
                        a2[q][i / 2] = __ffma2_rn(x2, cc, k == 0 ? make_float2(0.0f, 0.0f) : a2[q][i / 2]);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 2; q++)
#pragma unroll
                for (int i = 0; i < H; i += 2) {
                    acc[q][i] = a2[q][i / 2].x;
                    acc[q][i + 1] = a2[q][i / 2].y;
                }
            return;
        }
        // scalar chains: FP32 storage (gold's unfused products and sums) and
        // the FP16 box2d2r
#pragma unroll
        for (int q = 0; q < 2; q++) {
            constexpr int dy0 = tap_dy(S, 0), dx0 = tap_dx(S, 0);
            const float (&x0)[W] = row(2 + q + dy0);
#pragma unroll
            for (int i = 0; i < H; i++) {
                if constexpr (F32) acc[q][i] = BOX ? __fadd_rn(0.0f, __fmul_rn(x0[R + i + dx0], c.c[0]))
                                                   : __fmul_rn(x0[R + i + dx0], c.c[0]);
                else acc[q][i] = fmaf(x0[R + i + dx0], c.c[0], 0.0f);
            }
#pragma unroll
            for (int k = 1; k < NT; k++) {
                const int dy = tap_dy(S, k), dx = tap_dx(S, k);
                const float (&x)[W] = row(2 + q + dy);
#pragma unroll
                for (int i = 0; i < H; i++) {
                    if constexpr (F32) acc[q][i] = __fadd_rn(acc[q][i], __fmul_rn(x[R + i + dx], c.c[k]));
                    else acc[q][i] = fmaf(x[R + i + dx], c.c[k], acc[q][i]);
                }
            }
        }
    };
    auto store_row = [&](uint32_t r16, const float (&a)[H]) {
        uint2 v;
        if constexpr (F32) v = make_uint2(__float_as_uint(a[0]), __float_as_uint(a[1]));
        else v = make_uint2(pack_half2(a[0], a[1]), pack_half2(a[2], a[3]));
        sts_v2(own0 + r16, v);
    };

    // this lane's cells of the update rectangle
    const bool cols_in = xl >= p.g.x0 && xl + H <= p.g.x1;
    // A warp whose 32 rows and whose tile's 128 columns all lie in the update
    // rectangle takes a path with no per-row checks and immediate row offsets
    // (the general path tests rows, columns and the grid's end on every row).
    const bool fast = __all_sync(0xffffffffu, active && cols_in) && ys >= p.g.y0 &&
                      ys + kCcWarpRows <= p.g.y1;

    // Results go back into the stage, over the rows they replace, and leave
    // by bulk stores: so each warp first reads the rows it shares with its
    // neighbours (two above its rows, two below), and only then, after a
    // barrier, overwrites its own rows.
    // window: pair slot j holds rows (y0-2+2j, y0-1+2j), rotated over steps
    const uint32_t rs = (uint32_t)(ys - Y0) * 16;  // this warp's first row
    float win[3][2][W];
    float below[2][W];  // rows ye, ye+1
    if (has_rows) {
        to_window(rs - 2 * 16, win[0][0]);
        to_window(rs - 1 * 16, win[0][1]);
        to_window(rs, win[1][0]);
        to_window(rs + 16, win[1][1]);
        to_window((uint32_t)(ye - Y0) * 16, below[0]);
        to_window((uint32_t)(ye + 1 - Y0) * 16, below[1]);
    }
    __syncthreads();

    if (fast) {
        // 16 row pairs: five rounds of three (the window's three slots), then
        // the last pair, whose next rows are the next warp's, read before the
        // barrier
        static_assert(kCcWarpRows == 32, "five rounds of three row pairs and one more");
        uint32_t r = rs;
        for (int round = 0; round < 5; round++, r += 6 * 16) {
#pragma unroll
            for (int u = 0; u < 3; u++) {
                float (&n)[2][W] = win[(u + 2) % 3];
                to_window(r + (2 * u + 2) * 16, n[0]);
                to_window(r + (2 * u + 3) * 16, n[1]);
                float acc[2][H];
                compute(win[u], win[(u + 1) % 3], n, acc);
                store_row(r + 2 * u * 16, acc[0]);
                store_row(r + (2 * u + 1) * 16, acc[1]);
            }
        }
        float acc[2][H];
        compute(win[0], win[1], below, acc);
        store_row(r, acc[0]);
        store_row(r + 16, acc[1]);
    } else if (has_rows) {
        for (int y = ys; y < ye; y += 6) {
#pragma unroll
            for (int u = 0; u < 3; u++) {
                const int y0 = y + 2 * u;
                if (y0 < ye) {
                    float (&n)[2][W] = win[(u + 2) % 3];
                    // rows from ye on belong to the next warp, which may have
                    // written them by now, unless the grid ends at ye (then
                    // no warp writes them, and a warp of an odd row count
                    // reads up to ye + 2)
                    if (y0 + 2 < ye || ye == p.g.ny) {
                        to_window((uint32_t)(y0 + 2 - Y0) * 16, n[0]);
                        to_window((uint32_t)(y0 + 3 - Y0) * 16, n[1]);
                    } else {
#pragma unroll
                        for (int k = 0; k < W; k++) {
                            n[0][k] = below[0][k];
                            n[1][k] = below[1][k];
                        }
                    }
                    float acc[2][H];
                    compute(win[u], win[(u + 1) % 3], n, acc);
#pragma unroll
                    for (int q = 0; q < 2; q++) {
                        // cells outside the update rectangle keep their value
                        const int yy = y0 + q;
                        const bool row_in = yy >= p.g.y0 && yy < p.g.y1;
                        if (!(row_in && cols_in)) {
#pragma unroll
                            for (int i = 0; i < H; i++) {
                                const int x = xl + i;
                                if (!(row_in && x >= p.g.x0 && x < p.g.x1))
                                    acc[q][i] = win[(u + 1) % 3][q][R + i];
                            }
                        }
                        if (active && yy < ye) store_row((uint32_t)(yy - Y0) * 16, acc[q]);
                    }
                }
            }
        }
    }
    // the stage's rows Y0 .. Y0+127 of the 16 panels (results, and the input
    // where nothing was computed: rows past the grid, panels past its cells)
    // to the output plane
    fence_proxy_async_smem();
    __syncthreads();
    // the next step may launch once every CTA is here: signalled at the start
    // instead, CTAs of several later steps filled the SMs while they waited,
    // and a step of about one tile per SM ran slower (measured on GB300,
    // 1602² star2d1r FP16: 6.8 -> 8.6 us per step)
    pdl_launch_dependents();
    if (threadIdx.x == 0) {
        const int nq = min(kCcPanels + 1, p.p.npan - chunk0);
        for (int q = 1; q < nq; q++)
            bulk_store(out + ((ptrdiff_t)(chunk0 + q) * nyp + Y0 + 4) * V,
                       smem + kCcRunsOffset + q * kCcRunStride + 4 * 16, kCcTileRows * 16);
        bulk_store_commit_and_wait_read();
    }
}

template <bool F32>
cudaError_t launch_cc(const GridGeom &g, int stencil, const TapCoeffs &c, const void *in,
                      void *out, cudaStream_t s) {
    CcParams p;
    p.g = g;
    p.p = F32 ? g.p32 : g.p16;
    p.nchunks = (g.nx + p.p.cpp - 1) / p.p.cpp;
    p.tiles_x = (p.nchunks + kCcPanels - 1) / kCcPanels;
    p.n_tiles = p.tiles_x * ((g.ny + kCcTileRows - 1) / kCcTileRows);
    // programmatic stream serialization, as the tensor steps: the next
    // step's CTAs initialise their barrier while this step's last tiles
    // finish, and wait in pdl_wait before their copies
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)p.n_tiles);
    cfg.blockDim = dim3(kCcWarps * 32);
    cfg.dynamicSmemBytes = kCcSmem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    switch (stencil) {
    case TCS_STAR2D1R: return cudaLaunchKernelEx(&cfg, cc_sweep_kernel<TCS_STAR2D1R, F32>, in, out, p, c);
    case TCS_STAR2D2R: return cudaLaunchKernelEx(&cfg, cc_sweep_kernel<TCS_STAR2D2R, F32>, in, out, p, c);
    case TCS_BOX2D1R: return cudaLaunchKernelEx(&cfg, cc_sweep_kernel<TCS_BOX2D1R, F32>, in, out, p, c);
    case TCS_BOX2D2R: return cudaLaunchKernelEx(&cfg, cc_sweep_kernel<TCS_BOX2D2R, F32>, in, out, p, c);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_cc_f16(const GridGeom &g, int stencil, const TapCoeffs &c, const uint16_t *in,
                          uint16_t *out, cudaStream_t s) {
    return launch_cc<false>(g, stencil, c, in, out, s);
}

cudaError_t launch_cc_f32(const GridGeom &g, int stencil, const TapCoeffs &c, const float *in,
                          float *out, cudaStream_t s) {
    return launch_cc<true>(g, stencil, c, in, out, s);
}

cudaError_t cc_take_error(int *code) {
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(code, g_cc_error, sizeof(int));
    if (e != cudaSuccess) return e;
    return *code ? cudaMemcpyToSymbol(g_cc_error, &zero, sizeof(int)) : cudaSuccess;
}

}  // namespace tcs
