// Per-tile building blocks of the tensor-core sweep, shared by the
// single-grid kernel (sweep_tc.cu) and the batched persistent kernel
// (batch.cu), so that a grid computes the same bits in either.  The method is
// described at the top of sweep_tc.cu.
#pragma once

#include "tcs_device.cuh"
#include "tcs_internal.h"

namespace tcs {
namespace tc {

constexpr int kRowsStaged = kTile + 4;          // two halo rows above and below
constexpr int kChunkBytes = kRowsStaged * 16;   // one panel of a stage
constexpr int kSlots = kTile / 8 + 2;           // 16 panels + one each side
constexpr int kPlaneStage = kSlots * kChunkBytes;
constexpr int kBandElems = 32 * 16;             // one 16(K) x 32(N) FP16 band
constexpr int kBandBytes = kBandElems * 2;
constexpr int kEpiWarps = 8;                    // two warpgroups, one per column half
constexpr int kThreads = 32 * (2 + kEpiWarps);  // producer, MMA issuer, epilogue
constexpr uint32_t kIdesc = idesc_f16_f32(128, 32);

template <bool SPLIT>
struct Mode {
    static constexpr int NSUB = SPLIT ? 2 : 1;            // sub-tiles per tile
    static constexpr int SUB_BLOCKS = kTile / 16 / NSUB;  // 16-column blocks per sub-tile
    static constexpr int SUB_WIN = SUB_BLOCKS + 1;        // input windows per sub-tile
    static constexpr int ACC_PLANE = 16 * (SUB_BLOCKS + 2);  // TMEM columns per accumulator
    static constexpr int ACC = ACC_PLANE * (SPLIT ? 2 : 1);
    static constexpr int PLANES = SPLIT ? 2 : 1;          // hi (and lo) data planes
    static constexpr int BAND_PLANES = SPLIT ? 4 : 1;     // ch (and cf, cl, c3)
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

// Band element (n, k) of coefficient row dy: input column k of a 16-column
// window feeds output column n of its 32-column range with tap dx = 8 + k - n.
// Pieces: plain -> fp16(c); split -> 0: ch = rint(c 2^11) 2^-11, 1: cf =
// fp16(c), 2: cl = fp16(rem), 3: c3 = fp16(rem - cl), rem = (c - ch) 2^11.
__device__ __forceinline__ uint16_t band_element(const float *coef, int R, bool box, bool split,
                                                 int piece, int dy, int n, int k) {
    const int dx = 8 + k - n;
    const bool on_axis = box || dy == R || dx == 0;
    float c = 0.0f;
    if (dx >= -R && dx <= R && on_axis) c = coef[dy * (2 * R + 1) + dx + R];
    if (!split) return h_bits(c);
    const float ch = rintf(c * 2048.0f) * (1.0f / 2048.0f);
    const float rem = (c - ch) * 2048.0f;  // exact
    const uint16_t cl = h_bits(rem);
    switch (piece) {
    case 0: return h_bits(ch);
    case 1: return h_bits(c);
    case 2: return cl;
    default: return h_bits(rem - h_val(cl));
    }
}

// Element offset of (n, k) in band (piece, dy), K-major core-matrix layout:
// (piece*NDY + dy)*512 + (k/8)*256 + n*8 + k%8.
__device__ __forceinline__ int band_offset(int ndy, int piece, int dy, int n, int k) {
    return (piece * ndy + dy) * kBandElems + (k >> 3) * 256 + n * 8 + (k & 7);
}

// Fills `band` (shared or global memory) with all bands of a stencil, using
// threads [tid, .., nthreads).
__device__ __forceinline__ void build_bands(uint16_t *band, const float *coef, int R, bool box,
                                            bool split, int tid, int nthreads) {
    const int ndy = 2 * R + 1;
    const int pieces = split ? 4 : 1;
    for (int idx = tid; idx < pieces * ndy * kBandElems; idx += nthreads) {
        const int piece = idx / (ndy * kBandElems);
        const int rem = idx % (ndy * kBandElems);
        const int dy = rem / kBandElems, n = (rem >> 4) & 31, k = rem & 15;
        band[band_offset(ndy, piece, dy, n, k)] =
            band_element(coef, R, box, split, piece, dy, n, k);
    }
}

// Producer: bulk copies of rows Y0-2 .. Y0+129 of panels X0/8 - 1 .. X0/8 + 16
// of each input plane into a stage (plane pl at stage + pl*kPlaneStage).
__device__ __forceinline__ void load_tile(const uint16_t *hi, const uint16_t *lo, int planes,
                                          const PlaneGeom &pg, int Y0, int X0, uint8_t *stage,
                                          uint64_t *bar) {
    const size_t src0 = plane_index(pg, Y0 - 2, X0 - 8);
    for (int pl = 0; pl < planes; pl++) {
        const uint16_t *src = (pl ? lo : hi) + src0;
        uint8_t *st = stage + (size_t)pl * kPlaneStage;
#pragma unroll 1
        for (int c = 0; c < kSlots; c++)
            bulk_load(st + c * kChunkBytes, src + (size_t)c * pg.nyp * 8, kChunkBytes, bar);
    }
}

// MMAs of sub-tile h of a staged tile.  a_hi0 is the descriptor of the
// stage's hi plane; b_desc0 of the first band.  Descriptors for base + offset
// are the base descriptor plus offset >> 4 (the start-address field holds
// address >> 4 in its low bits).  Even windows (disjoint outputs, the first
// of them initialising) are issued before odd windows.
template <int R, bool SPLIT>
__device__ __forceinline__ void issue_subtile(uint64_t a_hi0, uint64_t b_desc0, uint32_t d_main,
                                              int h) {
    using M = Mode<SPLIT>;
    constexpr int NDY = 2 * R + 1;
    const uint64_t a_lo0 = a_hi0 + (kPlaneStage >> 4);
    const uint32_t d_corr = d_main + M::ACC_PLANE;
#pragma unroll
    for (int parity = 0; parity < 2; parity++) {
#pragma unroll
        for (int dy = 0; dy < NDY; dy++) {
            const uint64_t b_ch = b_desc0 + (uint64_t)((dy * kBandBytes) >> 4);
            const uint32_t acc = (parity == 1 || dy > 0) ? 1u : 0u;
#pragma unroll
            for (int w = parity; w < M::SUB_WIN; w += 2) {
                const int wg = h * M::SUB_BLOCKS + w;  // window in the tile
                const uint64_t a_off = (uint64_t)((2 * wg * kChunkBytes + (2 - R + dy) * 16) >> 4);
                umma_f16(d_main + 16 * w, a_hi0 + a_off, b_ch, kIdesc, acc);
                if (SPLIT) {
                    // correction accumulator, units 2^-11: cf*lo + cl*hi + c3*hi
                    const uint64_t b_cf = b_desc0 + (uint64_t)(((NDY + dy) * kBandBytes) >> 4);
                    const uint64_t b_cl = b_desc0 + (uint64_t)(((2 * NDY + dy) * kBandBytes) >> 4);
                    const uint64_t b_c3 = b_desc0 + (uint64_t)(((3 * NDY + dy) * kBandBytes) >> 4);
                    umma_f16(d_corr + 16 * w, a_lo0 + a_off, b_cf, kIdesc, acc);
                    umma_f16(d_corr + 16 * w, a_hi0 + a_off, b_cl, kIdesc, 1);
                    umma_f16(d_corr + 16 * w, a_hi0 + a_off, b_c3, kIdesc, 1);
                }
            }
        }
    }
}

// Output of one tile: planes, geometry and the update rectangle.
struct TileOut {
    const uint16_t *in_hi, *in_lo;  // input planes (cells outside the rectangle)
    uint16_t *out_hi, *out_lo;
    PlaneGeom pg;
    int y0, y1, x0, x1;
};

// Epilogue of sub-tile h for one warp: TMEM rows of lane quarter q (tile row
// m = 32q + lane), column blocks of `half`.  lane_addr addresses the
// accumulator's first output block for this warp's lanes.  Cells outside the
// update rectangle copy the input.
template <bool SPLIT>
__device__ __forceinline__ void epilogue_subtile(const TileOut &o, uint32_t lane_addr, int h,
                                                 int half, int m, int Y0, int X0) {
    using M = Mode<SPLIT>;
    constexpr int G = M::SUB_BLOCKS / 2;  // this warp's blocks, one TMEM round trip
    const int j0 = half * G;
    const int y = Y0 + m;
    const bool fast = Y0 >= o.y0 && Y0 + kTile <= o.y1 && X0 >= o.x0 && X0 + kTile <= o.x1;
    const bool row_in = y >= o.y0 && y < o.y1;
    uint32_t v[G][16];
    uint32_t w[SPLIT ? G : 1][16];
#pragma unroll
    for (int gg = 0; gg < G; gg++) {
        tmem_ld_x16(lane_addr + 16 * (j0 + gg), v[gg]);
        if (SPLIT) tmem_ld_x16(lane_addr + M::ACC_PLANE + 16 * (j0 + gg), w[SPLIT ? gg : 0]);
    }
    tmem_ld_wait();
#pragma unroll
    for (int gg = 0; gg < G; gg++) {
        const int xb = X0 + 16 * (h * M::SUB_BLOCKS + j0 + gg);
        const size_t off0 = plane_index(o.pg, y, xb);     // cells xb .. xb+7
        const size_t off1 = off0 + (size_t)o.pg.nyp * 8;  // cells xb+8 .. xb+15
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
            const uint4 i0 = *reinterpret_cast<const uint4 *>(o.in_hi + off0);
            const uint4 i1 = *reinterpret_cast<const uint4 *>(o.in_hi + off1);
            const uint32_t iw[8] = {i0.x, i0.y, i0.z, i0.w, i1.x, i1.y, i1.z, i1.w};
            uint32_t il[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (SPLIT) {
                const uint4 l0 = *reinterpret_cast<const uint4 *>(o.in_lo + off0);
                const uint4 l1 = *reinterpret_cast<const uint4 *>(o.in_lo + off1);
                il[0] = l0.x; il[1] = l0.y; il[2] = l0.z; il[3] = l0.w;
                il[4] = l1.x; il[5] = l1.y; il[6] = l1.z; il[7] = l1.w;
            }
#pragma unroll
            for (int c = 0; c < 8; c++) {
                uint16_t hh[2], ll[2];
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    const int x = xb + 2 * c + u;
                    const bool upd = row_in && x >= o.x0 && x < o.x1;
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
        *reinterpret_cast<uint4 *>(o.out_hi + off0) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *reinterpret_cast<uint4 *>(o.out_hi + off1) = make_uint4(hw[4], hw[5], hw[6], hw[7]);
        if (SPLIT) {
            *reinterpret_cast<uint4 *>(o.out_lo + off0) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            *reinterpret_cast<uint4 *>(o.out_lo + off1) = make_uint4(lw[4], lw[5], lw[6], lw[7]);
        }
    }
}

}  // namespace tc
}  // namespace tcs
