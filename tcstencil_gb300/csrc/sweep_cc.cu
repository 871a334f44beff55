// CUDA-core sweep kernels (the counterpart of the reference's baseline/
// kernel_*.cu `kernel_run`, rebuilt for GB300).
//
// One warp sweeps a vertical strip of 16 panels (128 FP16 or 64 FP32 columns)
// top to bottom, two rows per step.  Lanes 2p and 2p+1 own panel p: each
// loads one 16-byte panel row (the two rows of a step are one 32-byte sector
// of the panel), the pair swaps them with shuffles, and each lane then
// computes both rows for its half of the panel's columns.  Horizontal halo
// cells come from the neighbouring panel's lanes by shuffle; the two outer
// lanes fetch the strip's edge cells.  The vertical taps come from a register
// window of six rows, so each input row is loaded and converted once per
// strip.  Before storing, the pair swaps halves again so that each lane
// writes one full 16-byte panel row.  The plane's padding rows and panels
// keep every read in bounds.
//
// Arithmetic follows gold's tap order (common/gold_*.cpp):
//  - FP16 storage: acc = fmaf chain from 0, FP32 coefficients, RNE to FP16.
//  - FP32 storage: gold's own unfused products and sums (__fmul_rn/__fadd_rn),
//    so the result is bit-identical to gold compiled without FMA contraction.
#include <type_traits>

#include "tcs_device.cuh"
#include "tcs_internal.h"

namespace tcs {

namespace {

constexpr int kCcWarps = 4;     // warps per block
constexpr int kStripRows = 64;  // rows per warp strip (even)

struct CcParams {
    GridGeom g;
    PlaneGeom p;   // plane of this precision
    int nchunks;   // panels that hold grid cells
    int strip_h;
    int strips_x;
    int n_strips;
};

__device__ __forceinline__ uint4 ldg_v4(const void *p) {
    uint4 v;
    asm volatile("ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

template <int S, bool F32>
__global__ void __launch_bounds__(kCcWarps * 32)
    cc_sweep_kernel(const void *__restrict__ in_, void *__restrict__ out_, CcParams p,
                    TapCoeffs c) {
    constexpr int R = stencil_r(S);
    constexpr int V = F32 ? 4 : 8;    // cells per panel row
    constexpr int H = V / 2;          // cells per lane
    constexpr int W = H + 2 * R;      // window columns of a lane
    constexpr int NT = tap_count(S);
    constexpr bool BOX = stencil_box(S);
    constexpr int WPC = F32 ? 1 : 2;              // cells per 32-bit word
    constexpr int HW = (R + WPC - 1) / WPC;       // halo words per row
    using T = typename std::conditional<F32, float, uint16_t>::type;
    const T *__restrict__ in = static_cast<const T *>(in_);
    T *__restrict__ out = static_cast<T *>(out_);

    const int lane = threadIdx.x & 31;
    const int strip = blockIdx.x * kCcWarps + (threadIdx.x >> 5);
    if (strip >= p.n_strips) return;  // uniform across the warp
    const int sx = strip % p.strips_x, sy = strip / p.strips_x;
    const int par = lane & 1;                 // 0: left half of the panel, 1: right half
    const int chunk = sx * 16 + (lane >> 1);  // panel of this lane pair
    const bool active = chunk < p.nchunks;
    const int xb = chunk * V;                 // first column of the panel
    const int xl = xb + par * H;              // first column this lane computes
    const int ys = sy * p.strip_h;
    const int ye = min(ys + p.strip_h, p.g.ny);
    const bool right_edge_ok = chunk + 2 < p.p.npan;  // the next panel is allocated
    const int ymax = p.g.ny + 3;  // rows past this are never needed

    // Raw words of one step: both rows of this lane pair's panel, and the
    // halo words on this lane's outer side for both rows.
    struct Raw {
        uint32_t w[2][4];
        uint32_t h[2][HW];
    };

    // Row pair (y0, y0+1): this lane loads row y0 + par and swaps with its pair.
    auto load_pair = [&](int y0) -> Raw {
        Raw r;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (active) v = ldg_v4(in + plane_index(p.p, min(y0 + par, ymax), xb));
        const uint32_t mine[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t other = __shfl_xor_sync(0xffffffffu, mine[i], 1);
            r.w[0][i] = par ? other : mine[i];
            r.w[1][i] = par ? mine[i] : other;
        }
        // the left half needs the last R cells of the panel to the left, the
        // right half the first R cells of the panel to the right
#pragma unroll
        for (int row = 0; row < 2; row++)
#pragma unroll
            for (int k = 0; k < HW; k++) {
                const uint32_t from_left = __shfl_up_sync(0xffffffffu, r.w[row][4 - HW + k], 2);
                const uint32_t from_right = __shfl_down_sync(0xffffffffu, r.w[row][k], 2);
                r.h[row][k] = par ? from_right : from_left;
            }
        if (lane == 0 || lane == 31) {
            const bool ok = lane == 0 || right_edge_ok;
            const int xe = lane == 0 ? xb - V : xb + V;
#pragma unroll
            for (int row = 0; row < 2; row++) {
                const uint32_t *q = reinterpret_cast<const uint32_t *>(
                    in + plane_index(p.p, min(y0 + row, ymax), xe));
#pragma unroll
                for (int k = 0; k < HW; k++)
                    r.h[row][k] = ok ? __ldg(q + (lane == 0 ? 4 - HW + k : k)) : 0u;
            }
        }
        return r;
    };

    // Window columns [0, W) of this lane for one row: cells xl-R .. xl+H+R-1.
    auto to_window = [&](const Raw &r, int row, float (&w)[W]) {
        float cells[V];
        float halo[2];
        if constexpr (!F32) {
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float2 f = unpack_half2(r.w[row][i]);
                cells[2 * i] = f.x;
                cells[2 * i + 1] = f.y;
            }
            const float2 hf = unpack_half2(r.h[row][0]);
            // left half: cells 6, 7 of the left panel; right half: 0, 1 of the right
            halo[0] = hf.x;
            halo[1] = hf.y;
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) cells[i] = __uint_as_float(r.w[row][i]);
            halo[0] = __uint_as_float(r.h[row][0]);
            halo[1] = __uint_as_float(r.h[row][HW - 1]);
        }
#pragma unroll
        for (int k = 0; k < W; k++) {
            // left half: R halo cells (the left panel's last R), then cells 0..H+R-1
            const float left = k < R ? (F32 ? halo[k] : halo[2 - R + k]) : cells[k - R];
            // right half: cells H-R..V-1, then R halo cells (the right panel's first R)
            const float right = k < H + R ? cells[H - R + k] : halo[k - H - R];
            w[k] = par ? right : left;
        }
    };

    // window: pair slot j holds rows (y0-2+2j, y0-1+2j), rotated over steps
    float win[3][2][W];
    {
        const Raw a = load_pair(ys - 2);
        to_window(a, 0, win[0][0]);
        to_window(a, 1, win[0][1]);
        const Raw b = load_pair(ys);
        to_window(b, 0, win[1][0]);
        to_window(b, 1, win[1][1]);
    }
    Raw next = load_pair(ys + 2);

    for (int y = ys; y < ye; y += 6) {
#pragma unroll
        for (int u = 0; u < 3; u++) {
            const int y0 = y + 2 * u;
            if (y0 < ye) {
                to_window(next, 0, win[(u + 2) % 3][0]);
                to_window(next, 1, win[(u + 2) % 3][1]);
                next = load_pair(y0 + 4);

                float acc[2][H];
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    {
                        constexpr int dy0 = tap_dy(S, 0), dx0 = tap_dx(S, 0);
                        const int wr = 2 + q + dy0;  // window row of y0 + q + dy
#pragma unroll
                        for (int i = 0; i < H; i++) {
                            const float x0 = win[(u + wr / 2) % 3][wr % 2][R + i + dx0];
                            if constexpr (F32) acc[q][i] = BOX ? __fadd_rn(0.0f, __fmul_rn(x0, c.c[0]))
                                                               : __fmul_rn(x0, c.c[0]);
                            else acc[q][i] = fmaf(x0, c.c[0], 0.0f);
                        }
                    }
#pragma unroll
                    for (int k = 1; k < NT; k++) {
                        const int dy = tap_dy(S, k), dx = tap_dx(S, k);
                        const int wr = 2 + q + dy;
#pragma unroll
                        for (int i = 0; i < H; i++) {
                            const float x = win[(u + wr / 2) % 3][wr % 2][R + i + dx];
                            if constexpr (F32) acc[q][i] = __fadd_rn(acc[q][i], __fmul_rn(x, c.c[k]));
                            else acc[q][i] = fmaf(x, c.c[k], acc[q][i]);
                        }
                    }
                    // cells outside the update rectangle keep their value
                    const int yy = y0 + q;
                    const bool row_in = yy >= p.g.y0 && yy < p.g.y1;
                    if (!(row_in && xl >= p.g.x0 && xl + H <= p.g.x1)) {
#pragma unroll
                        for (int i = 0; i < H; i++) {
                            const int x = xl + i;
                            if (!(row_in && x >= p.g.x0 && x < p.g.x1))
                                acc[q][i] = win[(u + (2 + q) / 2) % 3][(2 + q) % 2][R + i];
                        }
                    }
                }
                // this lane's half of both rows; the pair swaps halves so that
                // lane par stores all of row y0 + par
                uint32_t mine[2][2];
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    if constexpr (F32) {
                        mine[q][0] = __float_as_uint(acc[q][0]);
                        mine[q][1] = __float_as_uint(acc[q][1]);
                    } else {
                        mine[q][0] = pack_half2(acc[q][0], acc[q][1]);
                        mine[q][1] = pack_half2(acc[q][2], acc[q][3]);
                    }
                }
                const uint32_t s0 = __shfl_xor_sync(0xffffffffu, par ? mine[0][0] : mine[1][0], 1);
                const uint32_t s1 = __shfl_xor_sync(0xffffffffu, par ? mine[0][1] : mine[1][1], 1);
                const int yy = y0 + par;
                if (active && yy < ye) {
                    const uint4 v = par ? make_uint4(s0, s1, mine[1][0], mine[1][1])
                                        : make_uint4(mine[0][0], mine[0][1], s0, s1);
                    *reinterpret_cast<uint4 *>(out + plane_index(p.p, yy, xb)) = v;
                }
            }
        }
    }
}

template <bool F32>
cudaError_t launch_cc(const GridGeom &g, int stencil, const TapCoeffs &c, const void *in,
                      void *out, cudaStream_t s) {
    CcParams p;
    p.g = g;
    p.p = F32 ? g.p32 : g.p16;
    p.nchunks = (g.nx + p.p.cpp - 1) / p.p.cpp;
    p.strip_h = kStripRows;
    p.strips_x = (p.nchunks + 15) / 16;
    const int strips_y = (g.ny + p.strip_h - 1) / p.strip_h;
    p.n_strips = p.strips_x * strips_y;
    dim3 block(kCcWarps * 32);
    dim3 grid((p.n_strips + kCcWarps - 1) / kCcWarps);
    switch (stencil) {
    case TCS_STAR2D1R: cc_sweep_kernel<TCS_STAR2D1R, F32><<<grid, block, 0, s>>>(in, out, p, c); break;
    case TCS_STAR2D2R: cc_sweep_kernel<TCS_STAR2D2R, F32><<<grid, block, 0, s>>>(in, out, p, c); break;
    case TCS_BOX2D1R: cc_sweep_kernel<TCS_BOX2D1R, F32><<<grid, block, 0, s>>>(in, out, p, c); break;
    case TCS_BOX2D2R: cc_sweep_kernel<TCS_BOX2D2R, F32><<<grid, block, 0, s>>>(in, out, p, c); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
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

}  // namespace tcs
