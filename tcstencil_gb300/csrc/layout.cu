// Device layout transforms.
//
//  - The reference's host-side layout16 helpers, padding_2D, brick_layout_2D
//    and reverse_layout_2D (layout16/host_star2d1r.cu:63-101), as bit-exact
//    device kernels (16 x 16 bricks, row-major inside a brick).
//  - pack / unpack between FP32 row-major grids and the engine's panel
//    planes: array_float2half (common/common.hpp:146-160) + padding_2D +
//    layout change in one pass, and the inverse.  One thread writes or reads
//    one 16-byte panel row, so plane-side accesses are 128-bit and
//    consecutive threads touch consecutive bytes of a panel.
#include "tcs_device.cuh"
#include "tcs_internal.h"

namespace tcs {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint16_t f2h_bits(float v) {
    __half h = __float2half_rn(v);
    return *reinterpret_cast<uint16_t *>(&h);
}

__device__ __forceinline__ float h2f_bits(uint16_t b) {
    __half h = *reinterpret_cast<__half *>(&b);
    return __half2float(h);
}

// Value of padded-grid cell (Y, X) of a (ny+2pad) x (nx+2pad) grid whose
// interior is the FP32 row-major input; 0 outside the padded grid.
__device__ __forceinline__ float padded_cell(const float *in, int ny, int nx, int pad,
                                             float pad_value, int Y, int X) {
    if (Y < 0 || X < 0 || Y >= ny + 2 * pad || X >= nx + 2 * pad) return 0.0f;
    const int iy = Y - pad, ix = X - pad;
    return (iy >= 0 && iy < ny && ix >= 0 && ix < nx) ? in[(size_t)iy * nx + ix] : pad_value;
}

// A panel row: thread id -> (plane row, panel) -> first cell (Y, X0) of the
// padded grid and the row's index q in the plane.  Consecutive threads take
// consecutive panels of one plane row, so that the row-major FP32 side of a
// warp's accesses is one contiguous run (the plane side is one 16-byte panel
// row per thread; the next plane row of a panel follows a few warps later).
struct PanelRow {
    int Y, X0;
    size_t q;
};
__device__ __forceinline__ PanelRow panel_row(size_t id, const PlaneGeom &p, int q0 = 0) {
    PanelRow r;
    const int yl = static_cast<int>(id / p.npan);  // row within the range
    const int yq = q0 + yl;
    const int pan = static_cast<int>(id - (size_t)yl * p.npan);
    r.Y = yq - kPadTop;
    r.X0 = (pan - 1) * p.cpp;
    r.q = (size_t)pan * p.nyp + yq;
    return r;
}

// The N cells (Y, X0 .. X0+N-1) of the padded grid (padded_cell), by 16-byte
// loads where they are all interior and 16-byte aligned.
template <int N>
__device__ __forceinline__ void load_cells(const float *__restrict__ in, int ny, int nx, int pad,
                                           float pad_value, int Y, int X0, float (&c)[N]) {
    const int iy = Y - pad, ix = X0 - pad;
    const size_t e = (size_t)iy * nx + ix;
    if (iy >= 0 && iy < ny && ix >= 0 && ix + N <= nx && (e & 3) == 0) {
#pragma unroll
        for (int k = 0; k < N; k += 4) {
            const float4 v = *reinterpret_cast<const float4 *>(in + e + k);
            c[k] = v.x; c[k + 1] = v.y; c[k + 2] = v.z; c[k + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < N; i++) c[i] = padded_cell(in, ny, nx, pad, pad_value, Y, X0 + i);
    }
}

// Stores the grid cells among (Y, X0 .. X0+N-1) of the padded grid into the
// ny x nx row-major output, by 16-byte stores where all N are and aligned.
template <int N>
__device__ __forceinline__ void store_cells(float *__restrict__ out, int ny, int nx, int pad,
                                            int Y, int X0, const float (&c)[N]) {
    const int iy = Y - pad, ix = X0 - pad;
    if (iy < 0 || iy >= ny) return;
    const size_t e = (size_t)iy * nx + ix;
    if (ix >= 0 && ix + N <= nx && (e & 3) == 0) {
#pragma unroll
        for (int k = 0; k < N; k += 4)
            *reinterpret_cast<float4 *>(out + e + k) = make_float4(c[k], c[k + 1], c[k + 2], c[k + 3]);
    } else {
#pragma unroll
        for (int i = 0; i < N; i++)
            if (ix + i >= 0 && ix + i < nx) out[(size_t)iy * nx + (ix + i)] = c[i];
    }
}

// Split storage of x: x' = x 2^-E, hi = fp16(rint(x' 2^11) 2^-11) (fixed
// point), lo = fp16((x' - hi) 2^11).  Every step before the final rounding
// of lo is exact in FP32.
__device__ __forceinline__ void split_value(float x, float scale, uint16_t &h, uint16_t &l) {
    const float xs = x * scale;
    h = f2h_bits(rintf(xs * 2048.0f) * (1.0f / 2048.0f));
    l = f2h_bits((xs - h2f_bits(h)) * 2048.0f);
}

__global__ void pack_f16_kernel(const float *__restrict__ in, int ny, int nx, int pad,
                                float pad_value, uint16_t *__restrict__ out, PlaneGeom p,
                                size_t n_rows, int q0) {
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n_rows) return;
    const PanelRow r = panel_row(id, p, q0);
    float c[8];
    load_cells<8>(in, ny, nx, pad, pad_value, r.Y, r.X0, c);
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; i++) w[i] = f2h_bits(c[2 * i]) | ((uint32_t)f2h_bits(c[2 * i + 1]) << 16);
    reinterpret_cast<uint4 *>(out)[r.q] = make_uint4(w[0], w[1], w[2], w[3]);
}

__global__ void unpack_f16_kernel(const uint16_t *__restrict__ in, int ny, int nx, int pad,
                                  float *__restrict__ out, PlaneGeom p, size_t n_rows, int q0) {
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n_rows) return;
    const PanelRow r = panel_row(id, p, q0);
    const int iy = r.Y - pad;
    if (iy < 0 || iy >= ny) return;
    const uint4 v = reinterpret_cast<const uint4 *>(in)[r.q];
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    float c[8];
#pragma unroll
    for (int i = 0; i < 8; i++) c[i] = h2f_bits((uint16_t)(w[i >> 1] >> (16 * (i & 1))));
    store_cells<8>(out, ny, nx, pad, r.Y, r.X0, c);
}

__global__ void pack_f32_kernel(const float *__restrict__ in, int ny, int nx, int pad,
                                float pad_value, float *__restrict__ out, PlaneGeom p,
                                size_t n_rows, int q0) {
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n_rows) return;
    const PanelRow r = panel_row(id, p, q0);
    float v[4];
    load_cells<4>(in, ny, nx, pad, pad_value, r.Y, r.X0, v);
    reinterpret_cast<float4 *>(out)[r.q] = make_float4(v[0], v[1], v[2], v[3]);
}

__global__ void unpack_f32_kernel(const float *__restrict__ in, int ny, int nx, int pad,
                                  float *__restrict__ out, PlaneGeom p, size_t n_rows, int q0) {
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n_rows) return;
    const PanelRow r = panel_row(id, p, q0);
    const int iy = r.Y - pad;
    if (iy < 0 || iy >= ny) return;
    const float4 v = reinterpret_cast<const float4 *>(in)[r.q];
    const float c[4] = {v.x, v.y, v.z, v.w};
    store_cells<4>(out, ny, nx, pad, r.Y, r.X0, c);
}

// Scale exponent E of a grid whose max |x| has float bits `bits`: the
// smallest E with max |x| < 2^E (frexp's exponent), 0 for an all-zero grid.
__device__ __forceinline__ int scale_exp_of(unsigned bits) {
    const float m = __uint_as_float(bits);
    if (!(m > 0.0f) || !isfinite(m)) return 0;
    int e = 0;
    frexpf(m, &e);
    return e;
}

// With max_bits set, the scale comes from the device-side maximum (and E is
// written to exp_out), so that packing needs no host round trip.
__global__ void pack_split_kernel(const float *__restrict__ in, int ny, int nx, int pad,
                                  float pad_value, float scale, const unsigned *max_bits,
                                  int *exp_out, uint16_t *__restrict__ hi,
                                  uint16_t *__restrict__ lo, PlaneGeom p, size_t n_rows) {
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (max_bits) {
        const int e = scale_exp_of(*max_bits);
        scale = ldexpf(1.0f, -e);
        if (id == 0 && exp_out) *exp_out = e;
    }
    if (id >= n_rows) return;
    const PanelRow r = panel_row(id, p);
    float c[8];
    load_cells<8>(in, ny, nx, pad, pad_value, r.Y, r.X0, c);
    uint32_t wh[4], wl[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        uint16_t h[2], l[2];
#pragma unroll
        for (int j = 0; j < 2; j++) split_value(c[2 * i + j], scale, h[j], l[j]);
        wh[i] = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
        wl[i] = (uint32_t)l[0] | ((uint32_t)l[1] << 16);
    }
    reinterpret_cast<uint4 *>(hi)[r.q] = make_uint4(wh[0], wh[1], wh[2], wh[3]);
    reinterpret_cast<uint4 *>(lo)[r.q] = make_uint4(wl[0], wl[1], wl[2], wl[3]);
}

__global__ void unpack_split_kernel(const uint16_t *__restrict__ hi,
                                    const uint16_t *__restrict__ lo, int ny, int nx, int pad,
                                    float scale, const int *exp_in, float *__restrict__ out,
                                    PlaneGeom p, size_t n_rows) {
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n_rows) return;
    if (exp_in) scale = ldexpf(1.0f, *exp_in);
    const PanelRow r = panel_row(id, p);
    const int iy = r.Y - pad;
    if (iy < 0 || iy >= ny) return;
    const uint4 vh = reinterpret_cast<const uint4 *>(hi)[r.q];
    const uint4 vl = reinterpret_cast<const uint4 *>(lo)[r.q];
    const uint32_t wh[4] = {vh.x, vh.y, vh.z, vh.w};
    const uint32_t wl[4] = {vl.x, vl.y, vl.z, vl.w};
    float c[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const float h = h2f_bits((uint16_t)(wh[i >> 1] >> (16 * (i & 1))));
        const float l = h2f_bits((uint16_t)(wl[i >> 1] >> (16 * (i & 1))));
        c[i] = fmaf(l, 1.0f / 2048.0f, h) * scale;
    }
    store_cells<8>(out, ny, nx, pad, r.Y, r.X0, c);
}

// max |x| as float bits (non-negative floats order like their bit patterns).
__global__ void max_abs_kernel(const float *__restrict__ in, size_t n, unsigned *out_bits) {
    float m = 0.0f;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(in[i]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out_bits, __float_as_uint(m));
}

// ------------------------------------------- reference layout16 helpers ---
// 16 x 16 bricks: brick (i, j) at (i*nbx + j)*256, cell (y, x) at y*16 + x.
struct Slice {
    int brick, row, col;
};
__device__ __forceinline__ Slice slice_of(size_t id) {
    Slice s;
    s.brick = static_cast<int>(id / 32);
    const int rem = static_cast<int>(id % 32);
    s.row = rem / 2;
    s.col = (rem % 2) * 8;
    return s;
}

// padding_2D: one thread per output cell.
__global__ void padding_2d_kernel(const uint16_t *__restrict__ in, uint16_t *__restrict__ out,
                                  int size, int halo, uint16_t value) {
    const int p = size + 2 * halo;
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (size_t)p * p) return;
    const int i = static_cast<int>(id / p), j = static_cast<int>(id % p);
    const bool inside = i >= halo && i < size + halo && j >= halo && j < size + halo;
    out[id] = inside ? in[(size_t)(i - halo) * size + (j - halo)] : value;
}

// brick_layout_2D: one thread per 8-cell slice of the brick output.
__global__ void brick_2d_kernel(const uint16_t *__restrict__ in, uint16_t *__restrict__ out,
                                int ny, int nx, int nbx, size_t n_slices) {
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n_slices) return;
    const Slice s = slice_of(id);
    const int Y = (s.brick / nbx) * 16 + s.row;
    const int X0 = (s.brick % nbx) * 16 + s.col;
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        uint32_t h[2];
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int X = X0 + 2 * i + j;
            h[j] = (Y < ny && X < nx) ? in[(size_t)Y * nx + X] : 0u;
        }
        w[i] = h[0] | (h[1] << 16);
    }
    reinterpret_cast<uint4 *>(out)[id] = make_uint4(w[0], w[1], w[2], w[3]);
}

// reverse_layout_2D: one thread per 8-cell slice of the brick input.
__global__ void unbrick_2d_kernel(const uint16_t *__restrict__ in, uint16_t *__restrict__ out,
                                  int ny, int nx, int nbx, size_t n_slices) {
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n_slices) return;
    const Slice s = slice_of(id);
    const int Y = (s.brick / nbx) * 16 + s.row;
    if (Y >= ny) return;
    const uint4 v = reinterpret_cast<const uint4 *>(in)[id];
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    const int X0 = (s.brick % nbx) * 16 + s.col;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int X = X0 + i;
        if (X < nx) out[(size_t)Y * nx + X] = (uint16_t)(w[i >> 1] >> (16 * (i & 1)));
    }
}

inline unsigned blocks_for(size_t n) { return static_cast<unsigned>((n + kThreads - 1) / kThreads); }
inline int nb(int n) { return (n + 15) / 16; }

struct PackShape {
    PlaneGeom p;
    size_t rows;
};
inline PackShape pack_shape(int ny, int nx, int pad, int cpp) {
    PackShape s;
    s.p = plane_geom(ny + 2 * pad, nx + 2 * pad, cpp);
    s.rows = (size_t)s.p.nyp * s.p.npan;
    return s;
}

}  // namespace

namespace {

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// The driver's cuTensorMapEncodeTiled, found through the runtime (no link
// against the driver library).
EncodeTiledFn encode_tiled() {
    static const EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

}  // namespace

cudaError_t encode_panel_map(const uint16_t *plane, const PlaneGeom &pg, CUtensorMap *map) {
    const EncodeTiledFn enc = encode_tiled();
    if (!enc) return cudaErrorNotSupported;
    if (reinterpret_cast<uintptr_t>(plane) % 16 || pg.nyp % 8 || pg.cpp != 8)
        return cudaErrorInvalidValue;
    const cuuint64_t dims[3] = {16, (cuuint64_t)pg.nyp / 8, (cuuint64_t)pg.npan};
    const cuuint64_t strides[2] = {128, (cuuint64_t)pg.nyp * 16};  // bytes, dims 1 and 2
    const cuuint32_t box[3] = {16, (kTile + 8) / 8, kTile / 8 + 2};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<uint16_t *>(plane),
                           dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_pack_f16(const float *in, int ny, int nx, int pad, float pad_value,
                            uint16_t *plane, cudaStream_t s) {
    const PackShape ps = pack_shape(ny, nx, pad, 8);
    pack_f16_kernel<<<blocks_for(ps.rows), kThreads, 0, s>>>(in, ny, nx, pad, pad_value, plane,
                                                             ps.p, ps.rows, 0);
    return cudaGetLastError();
}

cudaError_t launch_unpack_f16(const uint16_t *plane, int ny, int nx, int pad, float *out,
                              cudaStream_t s) {
    const PackShape ps = pack_shape(ny, nx, pad, 8);
    unpack_f16_kernel<<<blocks_for(ps.rows), kThreads, 0, s>>>(plane, ny, nx, pad, out, ps.p,
                                                               ps.rows, 0);
    return cudaGetLastError();
}

__global__ void split_scale_init_kernel(SplitScale *sc, const unsigned *max_bits) {
    const int e = scale_exp_of(*max_bits);
    for (int i = 0; i < kScaleRing; i++) {
        sc->maxbits[i] = 0;
        sc->exp[i] = e;
    }
    sc->maxbits[0] = sc->maxbits[kScaleRing - 1] = kScaleNoMax;
    sc->bmax = 0u;
    sc->bexp = e;
}

// B: the largest |x'| 2^-11 stored in the grid's cells outside the update
// rectangle, as FP32 bits, over the index space of the rows outside
// [y0, y1) (every column) followed by the rows inside (the columns outside
// [x0, x1)).  |x'| 2^11 = |hi 2^11 + lo| rounded once to FP32.
__global__ void split_border_max_kernel(SplitScale *sc, GridGeom g, const uint16_t *__restrict__ hi,
                                        const uint16_t *__restrict__ lo) {
    const int out_rows = g.y0 + (g.ny - g.y1);
    const int out_cols = g.x0 + (g.nx - g.x1);
    const size_t na = (size_t)out_rows * g.nx;
    const size_t n = na + (size_t)(g.y1 - g.y0) * out_cols;
    float m = 0.0f;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        int y, x;
        if (i < na) {
            const int r = (int)(i / g.nx);
            x = (int)(i - (size_t)r * g.nx);
            y = r < g.y0 ? r : g.y1 + (r - g.y0);
        } else {
            const size_t j = i - na;
            const int r = (int)(j / out_cols), c = (int)(j - (size_t)r * out_cols);
            y = g.y0 + r;
            x = c < g.x0 ? c : g.x1 + (c - g.x0);
        }
        const size_t idx = plane_index(g.p16, y, x);
        m = fmaxf(m, fabsf(fmaf(h2f_bits(hi[idx]), 2048.0f, h2f_bits(lo[idx]))));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&sc->bmax, __float_as_uint(m * (1.0f / 2048.0f)));
}

__global__ void split_scale_end_run_kernel(SplitScale *sc, int steps) {
    const unsigned m1 = sc->maxbits[(steps - 1) & (kScaleRing - 1)];
    const unsigned m0 = sc->maxbits[steps & (kScaleRing - 1)];
    const int e1 = sc->exp[(steps - 1) & (kScaleRing - 1)];
    const int e0 = sc->exp[steps & (kScaleRing - 1)];
    for (int i = 1; i < kScaleRing - 1; i++) sc->maxbits[i] = 0;
    sc->maxbits[kScaleRing - 1] = m1;
    sc->exp[kScaleRing - 1] = e1;
    sc->maxbits[0] = m0;
    sc->exp[0] = e0;
}

cudaError_t launch_split_scale_init(SplitScale *sc, const unsigned *max_bits, const GridGeom &g,
                                    const uint16_t *hi, const uint16_t *lo, cudaStream_t s) {
    split_scale_init_kernel<<<1, 1, 0, s>>>(sc, max_bits);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const size_t n = (size_t)g.ny * g.nx - (size_t)(g.y1 - g.y0) * (g.x1 - g.x0);
    if (n == 0) return cudaSuccess;
    const size_t want = blocks_for(n);
    split_border_max_kernel<<<static_cast<unsigned>(want < 1024 ? want : 1024), kThreads, 0, s>>>(
        sc, g, hi, lo);
    return cudaGetLastError();
}

cudaError_t launch_split_scale_end_run(SplitScale *sc, int steps, cudaStream_t s) {
    if (steps <= 0) return cudaSuccess;
    split_scale_end_run_kernel<<<1, 1, 0, s>>>(sc, steps);
    return cudaGetLastError();
}

cudaError_t launch_pack_f32(const float *in, int ny, int nx, int pad, float pad_value,
                            float *plane, cudaStream_t s) {
    const PackShape ps = pack_shape(ny, nx, pad, 4);
    pack_f32_kernel<<<blocks_for(ps.rows), kThreads, 0, s>>>(in, ny, nx, pad, pad_value, plane,
                                                             ps.p, ps.rows, 0);
    return cudaGetLastError();
}

cudaError_t launch_unpack_f32(const float *plane, int ny, int nx, int pad, float *out,
                              cudaStream_t s) {
    const PackShape ps = pack_shape(ny, nx, pad, 4);
    unpack_f32_kernel<<<blocks_for(ps.rows), kThreads, 0, s>>>(plane, ny, nx, pad, out, ps.p,
                                                               ps.rows, 0);
    return cudaGetLastError();
}

// Plane rows [q0, q1) only (every panel), pad 0: the grid rows they hold are
// [q0 - 4, q1 - 4) clipped to the grid; the pad rows above and below belong
// to the first and last ranges.
cudaError_t launch_pack_rows(const float *in, int ny, int nx, bool f32, void *plane, int q0,
                             int q1, cudaStream_t s) {
    const PackShape ps = pack_shape(ny, nx, 0, f32 ? 4 : 8);
    if (q0 < 0 || q1 > ps.p.nyp || q0 >= q1) return cudaErrorInvalidValue;
    const size_t rows = (size_t)(q1 - q0) * ps.p.npan;
    if (f32)
        pack_f32_kernel<<<blocks_for(rows), kThreads, 0, s>>>(in, ny, nx, 0, 0.0f,
                                                              static_cast<float *>(plane), ps.p,
                                                              rows, q0);
    else
        pack_f16_kernel<<<blocks_for(rows), kThreads, 0, s>>>(in, ny, nx, 0, 0.0f,
                                                              static_cast<uint16_t *>(plane),
                                                              ps.p, rows, q0);
    return cudaGetLastError();
}

cudaError_t launch_unpack_rows(const void *plane, int ny, int nx, bool f32, float *out, int q0,
                               int q1, cudaStream_t s) {
    const PackShape ps = pack_shape(ny, nx, 0, f32 ? 4 : 8);
    if (q0 < 0 || q1 > ps.p.nyp || q0 >= q1) return cudaErrorInvalidValue;
    const size_t rows = (size_t)(q1 - q0) * ps.p.npan;
    if (f32)
        unpack_f32_kernel<<<blocks_for(rows), kThreads, 0, s>>>(static_cast<const float *>(plane),
                                                                ny, nx, 0, out, ps.p, rows, q0);
    else
        unpack_f16_kernel<<<blocks_for(rows), kThreads, 0, s>>>(
            static_cast<const uint16_t *>(plane), ny, nx, 0, out, ps.p, rows, q0);
    return cudaGetLastError();
}

cudaError_t launch_pack_split(const float *in, int ny, int nx, int pad, float pad_value,
                              int scale_exp, uint16_t *hi, uint16_t *lo, cudaStream_t s) {
    const PackShape ps = pack_shape(ny, nx, pad, 8);
    pack_split_kernel<<<blocks_for(ps.rows), kThreads, 0, s>>>(
        in, ny, nx, pad, pad_value, ldexpf(1.0f, -scale_exp), nullptr, nullptr, hi, lo, ps.p,
        ps.rows);
    return cudaGetLastError();
}

cudaError_t launch_pack_split_dev(const float *in, int ny, int nx, const unsigned *max_bits,
                                  int *exp_out, uint16_t *hi, uint16_t *lo, cudaStream_t s) {
    const PackShape ps = pack_shape(ny, nx, 0, 8);
    pack_split_kernel<<<blocks_for(ps.rows), kThreads, 0, s>>>(
        in, ny, nx, 0, 0.0f, 1.0f, max_bits, exp_out, hi, lo, ps.p, ps.rows);
    return cudaGetLastError();
}

cudaError_t launch_unpack_split(const uint16_t *hi, const uint16_t *lo, int ny, int nx, int pad,
                                int scale_exp, float *out, cudaStream_t s) {
    const PackShape ps = pack_shape(ny, nx, pad, 8);
    unpack_split_kernel<<<blocks_for(ps.rows), kThreads, 0, s>>>(
        hi, lo, ny, nx, pad, ldexpf(1.0f, scale_exp), nullptr, out, ps.p, ps.rows);
    return cudaGetLastError();
}

cudaError_t launch_unpack_split_dev(const uint16_t *hi, const uint16_t *lo, int ny, int nx,
                                    const int *exp_in, float *out, cudaStream_t s) {
    const PackShape ps = pack_shape(ny, nx, 0, 8);
    unpack_split_kernel<<<blocks_for(ps.rows), kThreads, 0, s>>>(hi, lo, ny, nx, 0, 1.0f, exp_in,
                                                                 out, ps.p, ps.rows);
    return cudaGetLastError();
}

cudaError_t launch_max_abs(const float *in, size_t n, unsigned *out_bits, cudaStream_t s) {
    const size_t want = (n + kThreads - 1) / kThreads;
    const unsigned blocks = static_cast<unsigned>(want < 2048 ? (want ? want : 1) : 2048);
    max_abs_kernel<<<blocks, kThreads, 0, s>>>(in, n, out_bits);
    return cudaGetLastError();
}

cudaError_t launch_padding_2d(const uint16_t *in, uint16_t *out, int size, int halo,
                              uint16_t value, cudaStream_t s) {
    const size_t p = (size_t)(size + 2 * halo);
    padding_2d_kernel<<<blocks_for(p * p), kThreads, 0, s>>>(in, out, size, halo, value);
    return cudaGetLastError();
}

cudaError_t launch_brick_2d(const uint16_t *in, uint16_t *out, int ny, int nx, cudaStream_t s) {
    const size_t n = (size_t)nb(ny) * nb(nx) * 32;
    brick_2d_kernel<<<blocks_for(n), kThreads, 0, s>>>(in, out, ny, nx, nb(nx), n);
    return cudaGetLastError();
}

cudaError_t launch_unbrick_2d(const uint16_t *in, uint16_t *out, int ny, int nx, cudaStream_t s) {
    const size_t n = (size_t)nb(ny) * nb(nx) * 32;
    unbrick_2d_kernel<<<blocks_for(n), kThreads, 0, s>>>(in, out, ny, nx, nb(nx), n);
    return cudaGetLastError();
}

}  // namespace tcs
