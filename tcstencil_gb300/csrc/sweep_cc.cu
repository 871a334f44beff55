// CUDA-core sweep kernels (the counterpart of the reference's baseline/
// kernel_*.cu `kernel_run`, rebuilt for GB300).
//
// One warp sweeps a vertical strip of bricks top to bottom.  Each lane owns a
// 16-byte slice of a brick row (8 FP16 cells, or 4 FP32 cells), loaded with one
// 128-bit load, so a warp reads whole 32-byte sectors of 16 (FP16) or 8 (FP32)
// adjacent bricks per row.  Horizontal halo cells come from the neighbouring
// lanes by warp shuffle; the two outer lanes fetch the strip's edge cells.
// The vertical taps come from a register window of the last 2r+1 rows, so each
// input row is loaded and converted once per strip.
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
constexpr int kStripRows = 64;  // rows per warp strip

struct CcParams {
    GridGeom g;
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

template <bool F32>
struct Lane;

// FP16: 2 lanes per brick row, 8 cells per lane.
template <>
struct Lane<false> {
    static constexpr int kVec = 8;
    static constexpr int kLanesPerBrick = 2;
};
// FP32: 4 lanes per brick row, 4 cells per lane.
template <>
struct Lane<true> {
    static constexpr int kVec = 4;
    static constexpr int kLanesPerBrick = 4;
};

template <int S, bool F32>
__global__ void __launch_bounds__(kCcWarps * 32)
    cc_sweep_kernel(const void *__restrict__ in_, void *__restrict__ out_, CcParams p,
                    TapCoeffs c) {
    constexpr int R = stencil_r(S);
    constexpr int NW = 2 * R + 1;          // window rows
    constexpr int V = Lane<F32>::kVec;     // cells per lane
    constexpr int LPB = Lane<F32>::kLanesPerBrick;
    constexpr int W = V + 2 * R;           // window columns
    constexpr int NT = tap_count(S);
    constexpr bool BOX = stencil_box(S);
    using T = typename std::conditional<F32, float, uint16_t>::type;
    const T *__restrict__ in = static_cast<const T *>(in_);
    T *__restrict__ out = static_cast<T *>(out_);

    const int lane = threadIdx.x & 31;
    const int strip = blockIdx.x * kCcWarps + (threadIdx.x >> 5);
    if (strip >= p.n_strips) return;  // uniform across the warp
    const int sx = strip % p.strips_x, sy = strip / p.strips_x;
    const int nbx = p.g.nbx;
    const int bx = sx * (32 / LPB) + lane / LPB;
    const int sub = lane % LPB;            // slice of the brick row
    const bool active = bx < nbx;
    const int xb = bx * 16 + V * sub;      // first column of this lane
    const int rows = p.g.nby * 16;
    const int ys = sy * p.strip_h;
    const int ye = min(ys + p.strip_h, rows);

    struct Raw {
        uint4 v;
        uint32_t e0, e1;  // edge cells fetched by lanes 0 and 31
    };

    auto row_base = [&](int y) -> size_t {
        return (size_t)(y >> 4) * nbx * 256 + (size_t)(y & 15) * 16;
    };

    auto load_row = [&](int y) -> Raw {
        Raw r;
        r.v = make_uint4(0u, 0u, 0u, 0u);
        r.e0 = 0u;
        r.e1 = 0u;
        if (y >= 0 && y < rows) {
            const T *rowp = in + row_base(y);
            if (active) r.v = ldg_v4(rowp + (size_t)bx * 256 + V * sub);
            if constexpr (!F32) {
                // one 32-bit word = 2 FP16 cells
                if (lane == 0 && bx >= 1)
                    r.e0 = __ldg(reinterpret_cast<const uint32_t *>(rowp + (size_t)(bx - 1) * 256 + 14));
                if (lane == 31 && bx + 1 < nbx)
                    r.e0 = __ldg(reinterpret_cast<const uint32_t *>(rowp + (size_t)(bx + 1) * 256));
            } else {
                if (lane == 0 && bx >= 1) {
                    const uint32_t *q = reinterpret_cast<const uint32_t *>(rowp + (size_t)(bx - 1) * 256 + 14);
                    r.e0 = __ldg(q);
                    r.e1 = __ldg(q + 1);
                }
                if (lane == 31 && bx + 1 < nbx) {
                    const uint32_t *q = reinterpret_cast<const uint32_t *>(rowp + (size_t)(bx + 1) * 256);
                    r.e0 = __ldg(q);
                    r.e1 = __ldg(q + 1);
                }
            }
        }
        return r;
    };

    // Converts a raw row into window columns [0, W): R left halo cells, the
    // lane's V cells, R right halo cells.  All lanes take part (shuffles).
    auto to_window = [&](const Raw &r, float (&w)[W]) {
        if constexpr (!F32) {
            uint32_t left = __shfl_up_sync(0xffffffffu, r.v.w, 1);   // cells x-2, x-1
            uint32_t right = __shfl_down_sync(0xffffffffu, r.v.x, 1); // cells x+8, x+9
            if (lane == 0) left = r.e0;
            if (lane == 31) right = r.e0;
            const uint32_t words[4] = {r.v.x, r.v.y, r.v.z, r.v.w};
#pragma unroll
            for (int i = 0; i < 4; i++) {
                float2 f = unpack_half2(words[i]);
                w[R + 2 * i] = f.x;
                w[R + 2 * i + 1] = f.y;
            }
            float2 fl = unpack_half2(left), fr = unpack_half2(right);
            if constexpr (R == 1) {
                w[0] = fl.y;
                w[W - 1] = fr.x;
            } else {
                w[0] = fl.x;
                w[1] = fl.y;
                w[W - 2] = fr.x;
                w[W - 1] = fr.y;
            }
        } else {
            uint32_t l1 = __shfl_up_sync(0xffffffffu, r.v.w, 1);   // cell x-1
            uint32_t l2 = __shfl_up_sync(0xffffffffu, r.v.z, 1);   // cell x-2
            uint32_t r1 = __shfl_down_sync(0xffffffffu, r.v.x, 1); // cell x+4
            uint32_t r2 = __shfl_down_sync(0xffffffffu, r.v.y, 1); // cell x+5
            if (lane == 0) { l2 = r.e0; l1 = r.e1; }
            if (lane == 31) { r1 = r.e0; r2 = r.e1; }
            w[R + 0] = __uint_as_float(r.v.x);
            w[R + 1] = __uint_as_float(r.v.y);
            w[R + 2] = __uint_as_float(r.v.z);
            w[R + 3] = __uint_as_float(r.v.w);
            if constexpr (R == 1) {
                w[0] = __uint_as_float(l1);
                w[W - 1] = __uint_as_float(r1);
            } else {
                w[0] = __uint_as_float(l2);
                w[1] = __uint_as_float(l1);
                w[W - 2] = __uint_as_float(r1);
                w[W - 1] = __uint_as_float(r2);
            }
        }
    };

    float win[NW][W];
#pragma unroll
    for (int k = 0; k < 2 * R; k++) to_window(load_row(ys - R + k), win[k]);
    Raw next = load_row(ys + R);

    for (int y = ys; y < ye; y += NW) {
#pragma unroll
        for (int u = 0; u < NW; u++) {
            const int yy = y + u;
            if (yy < ye) {
                to_window(next, win[(u + 2 * R) % NW]);  // row yy + R
                next = load_row(yy + R + 1);

                float acc[V];
#pragma unroll
                for (int i = 0; i < V; i++) {
                    constexpr int dy0 = tap_dy(S, 0), dx0 = tap_dx(S, 0);
                    const float x0 = win[(u + R + dy0) % NW][R + i + dx0];
                    if constexpr (F32) acc[i] = BOX ? __fadd_rn(0.0f, __fmul_rn(x0, c.c[0]))
                                                    : __fmul_rn(x0, c.c[0]);
                    else acc[i] = fmaf(x0, c.c[0], 0.0f);
                }
#pragma unroll
                for (int k = 1; k < NT; k++) {
                    const int dy = tap_dy(S, k), dx = tap_dx(S, k);
#pragma unroll
                    for (int i = 0; i < V; i++) {
                        const float x = win[(u + R + dy) % NW][R + i + dx];
                        if constexpr (F32) acc[i] = __fadd_rn(acc[i], __fmul_rn(x, c.c[k]));
                        else acc[i] = fmaf(x, c.c[k], acc[i]);
                    }
                }

                if (active) {
                    const bool row_in = yy >= p.g.y0 && yy < p.g.y1;
                    const bool all_in = row_in && xb >= p.g.x0 && xb + V <= p.g.x1;
                    if (!all_in) {
#pragma unroll
                        for (int i = 0; i < V; i++) {
                            const int x = xb + i;
                            const bool upd = row_in && x >= p.g.x0 && x < p.g.x1;
                            if (!upd) acc[i] = win[(u + R) % NW][R + i];
                        }
                    }
                    T *dst = out + row_base(yy) + (size_t)bx * 256 + V * sub;
                    uint4 pk;
                    if constexpr (F32) {
                        pk = make_uint4(__float_as_uint(acc[0]), __float_as_uint(acc[1]),
                                        __float_as_uint(acc[2]), __float_as_uint(acc[3]));
                    } else {
                        pk = make_uint4(pack_half2(acc[0], acc[1]), pack_half2(acc[2], acc[3]),
                                        pack_half2(acc[4], acc[5]), pack_half2(acc[6], acc[7]));
                    }
                    *reinterpret_cast<uint4 *>(dst) = pk;
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
    p.strip_h = kStripRows;
    const int bricks_per_warp = 32 / Lane<F32>::kLanesPerBrick;
    p.strips_x = (g.nbx + bricks_per_warp - 1) / bricks_per_warp;
    const int strips_y = (g.nby * 16 + p.strip_h - 1) / p.strip_h;
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
