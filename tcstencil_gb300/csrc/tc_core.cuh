// Per-tile building blocks of the tensor-core sweep, shared by the
// single-grid kernel (sweep_tc.cu) and the batched persistent kernel
// (batch.cu), so that a grid computes the same bits in either.  The method is
// described at the top of sweep_tc.cu.
#pragma once

#include <stdlib.h>

#include "tcs_device.cuh"
#include "tcs_internal.h"

namespace tcs {
namespace tc {

constexpr int kRowsStaged = kTile + 4;          // two halo rows above and below
constexpr int kChunkBytes = kRowsStaged * 16;   // one panel of a stage
constexpr int kSlots = kTile / 8 + 2;           // 16 panels + one each side
constexpr int kPlaneStage = kSlots * kChunkBytes;

// Staged-panel geometry: CHUNK bytes per panel (rows at a 16-byte stride),
// TOP rows staged above the tile, PLANE bytes per staged plane.
template <int CHUNK_, int TOP_>
struct Staging {
    static constexpr int CHUNK = CHUNK_;
    static constexpr int TOP = TOP_;
    static constexpr int PLANE = kSlots * CHUNK_;
};
// 132 rows from Y0 - 2: the two halo rows each side a radius-2 stencil needs.
using StageHalo2 = Staging<kChunkBytes, 2>;
// 136 rows from Y0 - 4: every panel run starts on a 128-byte line (tile rows
// are multiples of 128 and the plane's top padding is 4 rows), so a tile's
// copies move 17 whole lines per panel instead of 17 partial ones.
using StageLines = Staging<(kTile + 8) * 16, 4>;
constexpr int kBandElems = 32 * 16;             // one 16(K) x 32(N) FP16 band
constexpr int kBandBytes = kBandElems * 2;
constexpr int kEpiWarps = 8;                    // plain: two warpgroups, one per column half
constexpr int kTmemCols = 512;                  // two accumulator slots of 256 columns
constexpr int kSlotCols = 256;                  // AccSlots: two slots of the batched FP16 items
constexpr uint32_t kIdesc = idesc_f16_f32(128, 32);
constexpr uint32_t kIdescStack = idesc_f16_f32(128, 96);

// Accumulator layout.
//  plain: one 128-column tile; window w adds into columns [16w, 16w+32) of a
//    160-column accumulator (overlapping windows accumulate in place); it
//    occupies one slot, so two sub-tiles double-buffer.
//  split: 64-column sub-tiles of five windows.  Each window has its own
//    96-column region [ch.hi | cl.hi + cf.lo | c3.hi] (three products of the
//    stacked band in one N=96 MMA, the lo product accumulated into the middle
//    part), even windows at 96e, odd windows at 288 + 96o: 480 columns, both
//    slots.  Neighbouring windows then never share columns, and an output
//    block sums the second half of window j with the first half of window j+1.
template <bool SPLIT>
struct Mode {
    static constexpr int NSUB = SPLIT ? 2 : 1;            // sub-tiles per tile
    static constexpr int SUB_BLOCKS = kTile / 16 / NSUB;  // 16-column blocks per sub-tile
    static constexpr int SUB_WIN = SUB_BLOCKS + 1;        // input windows per sub-tile
    static constexpr int ACC = SPLIT ? 480 : 16 * (SUB_BLOCKS + 2);  // TMEM columns used
    static constexpr int PLANES = SPLIT ? 2 : 1;          // hi (and lo) data planes
    static constexpr int BAND_PLANES = SPLIT ? 4 : 1;     // band bytes per row, in kBandBytes
};
static_assert(Mode<false>::ACC <= kSlotCols && Mode<true>::ACC <= kTmemCols, "TMEM layout");

// First TMEM column of split window w's region.
__host__ __device__ constexpr int split_region(int w) { return (w & 1) ? 288 + 96 * (w >> 1) : 96 * (w >> 1); }

// Which accumulator slots a sub-tile holds: plain sub-tiles alternate between
// the two slots, a split sub-tile takes both.  The MMA issuer and the
// epilogue walk the same sequence, so both see the same slots, and each slot
// counts its own uses for the barrier parities.
struct AccSlots {
    uint32_t uses[2] = {0, 0};
    int next = 0;
    // Returns the slot mask (bit s = slot s) and the first column.
    __device__ __forceinline__ uint32_t take(bool split, uint32_t &col) {
        if (split) {
            next = 0;
            col = 0;
            return 3u;
        }
        const int s = next;
        next ^= 1;
        col = (uint32_t)(s * kSlotCols);
        return 1u << s;
    }
    __device__ __forceinline__ void used(uint32_t mask) {
        if (mask & 1u) uses[0]++;
        if (mask & 2u) uses[1]++;
    }
    // MMA issuer: waits until every slot of the mask is free (bounded).
    __device__ __forceinline__ bool acquire(uint64_t *acc_empty, uint32_t mask,
                                            const volatile int *abort,
                                            uint64_t limit_ns = kWaitLimitNs) const {
#pragma unroll
        for (int s = 0; s < 2; s++)
            if ((mask >> s) & 1u)
                if (!mbar_wait(&acc_empty[s], (uses[s] & 1u) ^ 1u, abort, limit_ns)) return false;
        return true;
    }
    // MMA issuer: the slots' accumulators are complete when the MMAs are.
    __device__ __forceinline__ void commit(uint64_t *acc_full, uint32_t mask) const {
#pragma unroll
        for (int s = 0; s < 2; s++)
            if ((mask >> s) & 1u) umma_commit(&acc_full[s]);
    }
    // Epilogue: waits until the slots' accumulators are complete (bounded).
    __device__ __forceinline__ bool ready(uint64_t *acc_full, uint32_t mask,
                                          const volatile int *abort,
                                          uint64_t limit_ns = kWaitLimitNs) const {
#pragma unroll
        for (int s = 0; s < 2; s++)
            if ((mask >> s) & 1u)
                if (!mbar_wait(&acc_full[s], uses[s] & 1u, abort, limit_ns)) return false;
        return true;
    }
    // Epilogue (one lane per warp): this warp is done reading the slots.
    __device__ __forceinline__ void release(uint64_t *acc_empty, uint32_t mask) const {
#pragma unroll
        for (int s = 0; s < 2; s++)
            if ((mask >> s) & 1u) mbar_arrive(&acc_empty[s]);
    }
};

// plane_index of an FP16 (or split) plane, 8 cells per panel row: the
// panel and the cell in it by shifts, not by a division by the plane's cpp
// (x >= -8).
__device__ __forceinline__ size_t plane_index16(const PlaneGeom &p, int y, int x) {
    const int xs = x + 8;
    return ((size_t)(xs >> 3) * p.nyp + (size_t)(y + kPadTop)) * 8 + (size_t)(xs & 7);
}

__device__ __forceinline__ uint16_t h_bits(float v) {
    __half h = __float2half_rn(v);
    return *reinterpret_cast<uint16_t *>(&h);
}
__device__ __forceinline__ float h_val(uint16_t b) {
    __half h = *reinterpret_cast<__half *>(&b);
    return __half2float(h);
}

// ------------------------------------------------ split scale, per step ---
// (tcs_internal.h SplitScale.)  e(M) of M = max(m, B 2^d) from the FP32
// bits of m and B: the larger of the present parts' frexp exponents (a zero
// or subnormal part is absent), 0 for none or for a non-finite m (no
// change), clamped to [-64, 64].
__device__ __forceinline__ int split_exp_of(unsigned mbits, unsigned bbits, int d) {
    const int bm = (int)((mbits >> 23) & 0xffu);
    if (bm == 0xff) return 0;
    const int bb = (int)((bbits >> 23) & 0xffu);
    const bool hm = bm != 0, hb = bb != 0 && bb != 0xff;
    if (!hm && !hb) return 0;
    const int em = bm - 126, eb = bb - 126 + d;
    const int e = !hb ? em : !hm ? eb : (em > eb ? em : eb);
    return e < -64 ? -64 : e > 64 ? 64 : e;
}

// Scale of step t (the step index within the run, from 1): s = 2^(11 + k_t)
// turns the step's value v (units of 2^E_{t-1}) into u = v s, the new state
// in units of 2^-11 of 2^E_t.  Without a scale record (sc null) k = 0.
struct StepScale {
    float s;
    int k, e;
};

// The words of step t's scale: E and m of steps t-2 and t-3, E_0, and the
// border's B and E_B, in one burst of relaxed GPU-scope loads (their
// latencies overlap, and a caller can issue other work before it uses them).
struct ScaleWords {
    unsigned ea, ma, eb, mb, e0, bm, be;
};
__device__ __forceinline__ ScaleWords scale_words(const SplitScale *sc, int t) {
    const int a = (t - 2) & (kScaleRing - 1), b = (t - 3) & (kScaleRing - 1);
    ScaleWords w;
    asm volatile(
        "ld.relaxed.gpu.global.u32 %0, [%7];\n\t"
        "ld.relaxed.gpu.global.u32 %1, [%8];\n\t"
        "ld.relaxed.gpu.global.u32 %2, [%9];\n\t"
        "ld.relaxed.gpu.global.u32 %3, [%10];\n\t"
        "ld.relaxed.gpu.global.u32 %4, [%11];\n\t"
        "ld.relaxed.gpu.global.u32 %5, [%12];\n\t"
        "ld.relaxed.gpu.global.u32 %6, [%13];"
        : "=r"(w.ea), "=r"(w.ma), "=r"(w.eb), "=r"(w.mb), "=r"(w.e0), "=r"(w.bm), "=r"(w.be)
        : "l"(&sc->exp[a]), "l"(&sc->maxbits[a]), "l"(&sc->exp[b]), "l"(&sc->maxbits[b]),
          "l"(&sc->exp[0]), "l"(&sc->bmax), "l"(&sc->bexp)
        : "memory");
    return w;
}

__device__ __forceinline__ StepScale scale_of(const ScaleWords &w, int t) {
    StepScale r;
    const int ea = (int)w.ea, eb = (int)w.eb, be = (int)w.be;
    r.e = ea + split_exp_of(w.ma, w.bm, be - ea);                              // E_t
    const int e1 = t == 1 ? (int)w.e0 : eb + split_exp_of(w.mb, w.bm, be - eb);  // E_{t-1}
    int k = e1 - r.e;
    k = k < -64 ? -64 : k > 64 ? 64 : k;
    r.k = k;
    r.s = __int_as_float((127 + 11 + k) << 23);
    return r;
}

__device__ __forceinline__ StepScale step_scale(const SplitScale *sc, int t) {
    if (!sc) {
        StepScale r;
        r.s = 2048.0f;
        r.k = 0;
        r.e = 0;
        return r;
    }
    return scale_of(scale_words(sc, t), t);
}

// A CTA's side of the scale record.  Every CTA of a step reads the same
// record and adds to the same maximum, so per warp these would be thousands
// of accesses to one line at each step boundary (measured on GB300: a
// 4098² split step in one launch per step, 30 -> 39 us; several steps per
// launch, 28 -> 97 us).  Instead one warp of the CTA reads the scale and
// publishes it in shared memory, and the epilogue warps' maxima meet in
// shared memory, which the CTA's last warp to finish the step adds to the
// record.  The slots go by the CTA's step ordinal n (the steps in which the
// CTA holds tiles, counted from 0; every epilogue warp walks the same items,
// so they agree on n), two of them: a CTA's warps are at most one step apart.
struct CtaScale {
    uint64_t *bar;   // [2] the step's scale published (one arrival)
    StepScale *ss;   // [2]
    unsigned *max;   // [2] the CTA's largest |u| 2^-11 in the step (FP32 bits)
    unsigned *cnt;   // [2] epilogue warps done with the step
};

__device__ __forceinline__ void cta_scale_init(const CtaScale &c) {
    for (int j = 0; j < 2; j++) {
        mbar_init(&c.bar[j], 1);
        c.max[j] = 0u;
        c.cnt[j] = 0u;
    }
}

// The scale warp's lane 0: the scale of the CTA's n-th step.
__device__ __forceinline__ void cta_scale_publish(const CtaScale &c, int n, const StepScale &ss) {
    c.ss[n & 1] = ss;
    mbar_arrive(&c.bar[n & 1]);
}

// Every lane of an epilogue warp: the scale of the CTA's n-th step (bounded
// wait; false on give-up or abort).  Slot n & 1 completes its phases in the
// order of n, so the n-th step's is phase n >> 1 of it.
__device__ __forceinline__ bool cta_scale_take(const CtaScale &c, int n, StepScale &ss,
                                               const volatile int *abort_flag) {
    const bool ok = __all_sync(0xffffffffu, mbar_wait(&c.bar[n & 1], (n >> 1) & 1, abort_flag));
    if (ok) ss = c.ss[n & 1];
    return ok;
}

// After a warp's last cells of the CTA's n-th step (record step t): its
// largest |u| joins the CTA's; the CTA's last warp of NW adds that to M_t
// and, if the CTA held the step's tile 0 (own0), stores E_t in slot t and
// clears the maximum of slot t+3.  Called by every lane.
template <int NW>
__device__ __forceinline__ void cta_scale_flush(const CtaScale &c, int n, SplitScale *sc, int t,
                                                const StepScale &ss, float mx, bool own0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&c.max[n & 1], __float_as_uint(mx * (1.0f / 2048.0f)));
        __threadfence_block();
        if (atomicAdd(&c.cnt[n & 1], 1u) == (unsigned)NW - 1) {
            __threadfence_block();
            const unsigned m = atomicExch(&c.max[n & 1], 0u);
            atomicExch(&c.cnt[n & 1], 0u);
            atomicMax(&sc->maxbits[t & (kScaleRing - 1)], m);
            if (own0) {
                sc->exp[t & (kScaleRing - 1)] = ss.e;
                sc->maxbits[(t + 3) & (kScaleRing - 1)] = 0u;
            }
        }
    }
}

// Fixed-point split of a value v (|v| about 1 or below): hi = fp16 of
// rint(v 2^11) 2^-11, lo = fp16((v - hi) 2^11).
__device__ __forceinline__ void split_fixed(float v, uint16_t &hi, uint16_t &lo) {
    hi = h_bits(rintf(v * 2048.0f) * (1.0f / 2048.0f));
    lo = h_bits((v - h_val(hi)) * 2048.0f);
}

// split_fixed of the value v 2^k, with s = 2^(11 + k) (StepScale): u = v s,
// hi = fp16(rint(u) 2^-11), lo = fp16(u - hi 2^11), the same bits as
// split_fixed(v) when k = 0; the largest |u| is kept in mx.
__device__ __forceinline__ void split_fixed_s(float v, float s, uint16_t &hi, uint16_t &lo,
                                              float &mx) {
    const float u = v * s;
    hi = h_bits(rintf(u) * (1.0f / 2048.0f));
    lo = h_bits(u - h_val(hi) * 2048.0f);
    mx = fmaxf(mx, fabsf(u));
}

// A stored (hi, lo) pair scaled by 2^k (k != 0), split again exactly: with
// a = hi 2^(11+k) = ai + af (ai its integer part) and b = lo 2^k, the new
// pair is hi' = (ai + rint(af + b)) 2^-11, lo' = (af + b) - rint(af + b),
// every operation exact, so no bit of the value is lost.  (k = 0 keeps the
// pair as it is.)
__device__ __forceinline__ void resplit_pair(uint16_t &hi, uint16_t &lo, const StepScale &ss) {
    const float a = h_val(hi) * ss.s;
    const float ai = truncf(a);
    const float bb = (a - ai) + h_val(lo) * (ss.s * (1.0f / 2048.0f));
    const float rb = rintf(bb);
    hi = h_bits((ai + rb) * (1.0f / 2048.0f));
    lo = h_bits(bb - rb);
}

// Two FP32 values as packed FP16 (round to nearest even), v0 in the low half.
__device__ __forceinline__ uint32_t pack_h2(float v0, float v1) {
    const __half2 h = __floats2half2_rn(v0, v1);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// split_fixed of two values into packed hi and lo words, with the same bits
// and less conversion work: u = v 2^11 is exact, t = rint(u) is formed by the
// add-and-subtract of 1.5 * 2^23 (round to nearest even for |u| < 2^22; the
// sign copy keeps rint's -0 for small negative u).  While |t| <= 2^11, hi =
// t 2^-11 is exact in FP16 and lo = u - t = (v - hi) 2^11 is exact; past that
// (|v| slightly above 1, or NaN) hi rounds in FP16 and split_fixed's rule is
// taken.
// With s = 2^(11 + k) the pair is of v 2^k (StepScale), and the largest |u|
// is kept in mx.
__device__ __forceinline__ void split_pair_s(float v0, float v1, float s, uint32_t &hw,
                                             uint32_t &lw, float &mx) {
    constexpr float kRound = 12582912.0f;  // 1.5 * 2^23
    // packed FP32 operations on the pair: each lane rounds as the scalar
    // operation would, so the bits are split_pair's
    const float2 u = __fmul2_rn(make_float2(v0, v1), make_float2(s, s));
    const float u0 = u.x, u1 = u.y;
    mx = fmaxf(mx, fmaxf(fabsf(u0), fabsf(u1)));
    const float2 r = __fadd2_rn(__fadd2_rn(u, make_float2(kRound, kRound)),
                                make_float2(-kRound, -kRound));
    const float t0 = copysignf(r.x, u0);
    const float t1 = copysignf(r.y, u1);
    if (fabsf(t0) <= 2048.0f && fabsf(t1) <= 2048.0f) {
        const float2 t = make_float2(t0, t1);
        const float2 h = __fmul2_rn(t, make_float2(1.0f / 2048.0f, 1.0f / 2048.0f));
        const float2 l = __ffma2_rn(t, make_float2(-1.0f, -1.0f), u);  // u - t, exact
        hw = pack_h2(h.x, h.y);
        lw = pack_h2(l.x, l.y);
    } else {
        uint16_t h0, l0, h1, l1;
        split_fixed_s(v0, s, h0, l0, mx);
        split_fixed_s(v1, s, h1, l1, mx);
        hw = (uint32_t)h0 | ((uint32_t)h1 << 16);
        lw = (uint32_t)l0 | ((uint32_t)l1 << 16);
    }
}

__device__ __forceinline__ void split_pair(float v0, float v1, uint32_t &hw, uint32_t &lw) {
    constexpr float kRound = 12582912.0f;  // 1.5 * 2^23
    const float u0 = v0 * 2048.0f, u1 = v1 * 2048.0f;
    const float t0 = copysignf(__fsub_rn(__fadd_rn(u0, kRound), kRound), u0);
    const float t1 = copysignf(__fsub_rn(__fadd_rn(u1, kRound), kRound), u1);
    if (fabsf(t0) <= 2048.0f && fabsf(t1) <= 2048.0f) {
        hw = pack_h2(t0 * (1.0f / 2048.0f), t1 * (1.0f / 2048.0f));
        lw = pack_h2(__fsub_rn(u0, t0), __fsub_rn(u1, t1));
    } else {
        uint16_t h0, l0, h1, l1;
        split_fixed(v0, h0, l0);
        split_fixed(v1, h1, l1);
        hw = (uint32_t)h0 | ((uint32_t)h1 << 16);
        lw = (uint32_t)l0 | ((uint32_t)l1 << 16);
    }
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

// Band memory of a stencil, K-major core-matrix layout (8 N-rows x 16 bytes,
// SBO = 128 B between 8-row groups, LBO between the two K halves):
//  plain: per coefficient row dy, a 32(N) x 16(K) band of fp16(c) at dy*512
//    elements, LBO 512 B;
//  split: per dy, the stacked 96 x 16 band [ch | cl | c3] at dy*1536, LBO
//    1536 B; then per dy the 32 x 16 cf band at NDY*1536 + dy*512, LBO 512 B.
// Both take BAND_PLANES * NDY * kBandBytes bytes.
__device__ __forceinline__ int band_offset(int ndy, bool split, int part, int dy, int n, int k) {
    if (!split) return dy * kBandElems + (k >> 3) * 256 + n * 8 + (k & 7);
    if (part < 3) return dy * 1536 + (k >> 3) * 768 + (part * 32 + n) * 8 + (k & 7);
    return ndy * 1536 + dy * kBandElems + (k >> 3) * 256 + n * 8 + (k & 7);
}

// Fills `band` (shared or global memory) with all bands of a stencil, using
// threads [tid, .., nthreads).  Split parts 0..3 are ch, cl, c3 (stacked)
// and cf.
__device__ __forceinline__ void build_bands(uint16_t *band, const float *coef, int R, bool box,
                                            bool split, int tid, int nthreads) {
    const int ndy = 2 * R + 1;
    const int parts = split ? 4 : 1;
    for (int idx = tid; idx < parts * ndy * kBandElems; idx += nthreads) {
        const int part = idx / (ndy * kBandElems);
        const int rem = idx % (ndy * kBandElems);
        const int dy = rem / kBandElems, n = (rem >> 4) & 31, k = rem & 15;
        // band_element pieces: 0 ch, 1 cf, 2 cl, 3 c3
        const int piece = !split ? 0 : (part == 0 ? 0 : part == 1 ? 2 : part == 2 ? 3 : 1);
        band[band_offset(ndy, split, part, dy, n, k)] =
            band_element(coef, R, box, split, piece, dy, n, k);
    }
}

// Producer: one tensor-map load per plane of a tile in the line-aligned
// staging (maps from encode_panel_map): the 136 rows Y0 - 4 .. Y0 + 131 of
// the 18 panels X0/8 - 1 .. X0/8 + 16, box origin (word 0, row group Y0 / 8 =
// row Y0 - 4 + the plane's 4 top padding rows, panel of X0 - 8).
__device__ __forceinline__ void load_tile_map(const CUtensorMap *hi, const CUtensorMap *lo,
                                              int planes, int Y0, int X0, uint8_t *stage,
                                              uint64_t *bar) {
    static_assert(StageLines::TOP == kPadTop && StageLines::CHUNK == 17 * 128, "map box");
    tma_load_3d(stage, hi, bar, 0, Y0 / 8, X0 / 8);
    if (planes > 1) tma_load_3d(stage + StageLines::PLANE, lo, bar, 0, Y0 / 8, X0 / 8);
}

// One 16-column output block of the split form from the regions of its two
// windows (TMEM addresses of this warp's lane quarter at each region): the
// second half of window a plus the first half of window b, per part.
__device__ __forceinline__ void split_block_load(uint32_t region_a, uint32_t region_b,
                                                 float (&f)[16]) {
    uint32_t v[6][16];
#pragma unroll
    for (int part = 0; part < 3; part++) {
        tmem_ld_x16(region_a + 16 + 32 * part, v[2 * part]);
        tmem_ld_x16(region_b + 32 * part, v[2 * part + 1]);
    }
    tmem_ld_wait();
    // main (exact sum of ch.hi), correction in units of 2^-11; two columns
    // per packed FP32 operation (each lane rounds as the scalar one would)
    auto pr = [&](int part, int c) {
        return make_float2(__uint_as_float(v[part][c]), __uint_as_float(v[part][c + 1]));
    };
#pragma unroll
    for (int c = 0; c < 16; c += 2) {
        const float2 main = __fadd2_rn(pr(0, c), pr(1, c));
        const float2 corr = __fadd2_rn(__fadd2_rn(pr(2, c), pr(3, c)), __fadd2_rn(pr(4, c), pr(5, c)));
        const float2 r = __ffma2_rn(corr, make_float2(1.0f / 2048.0f, 1.0f / 2048.0f), main);
        f[c] = r.x;
        f[c + 1] = r.y;
    }
}

// MMAs of one split window, whose K panels are stage slots `slot` and
// `slot`+1 (the lo image lo_bytes after the hi image), into the 96-column
// region at d: per coefficient row, the stacked hi MMA (which
// initialises the region on the first row) and the lo MMA into its middle
// part.
template <int R, class SG = StageHalo2>
__device__ __forceinline__ void issue_split_window_at(uint64_t a_hi0, uint32_t band, uint32_t d,
                                                      int slot, int lo_bytes = SG::PLANE) {
    constexpr int NDY = 2 * R + 1;
    const uint64_t a_lo0 = a_hi0 + (uint64_t)(lo_bytes >> 4);
    const uint64_t bs0 = smem_desc(band, 1536, 128);
    const uint64_t bf0 = smem_desc(band + NDY * 3072, 512, 128);
#pragma unroll
    for (int dy = 0; dy < NDY; dy++) {
        const uint64_t a_off = (uint64_t)((slot * SG::CHUNK + (SG::TOP - R + dy) * 16) >> 4);
        umma_f16(d, a_hi0 + a_off, bs0 + (uint64_t)((dy * 3072) >> 4), kIdescStack,
                 dy > 0 ? 1u : 0u);
        umma_f16(d + 32, a_lo0 + a_off, bf0 + (uint64_t)((dy * kBandBytes) >> 4), kIdesc, 1u);
    }
}

// The same for window wg of a staged tile (its panels 2wg, 2wg+1).
template <int R, class SG = StageHalo2>
__device__ __forceinline__ void issue_split_window(uint64_t a_hi0, uint32_t band, uint32_t d,
                                                   int wg) {
    issue_split_window_at<R, SG>(a_hi0, band, d, 2 * wg);
}

// Windows a tile needs: output block j (columns X0 + 16j .. +15) takes
// windows j and j + 1, and blocks from the grid's last column on are padding
// (split: never stored; plain: stored only as the input copied back, the
// cells being outside the update rectangle; padding keeps finite contents).
// So a tile W columns wide of a grid nx cells wide needs windows 0 .. nb,
// nb = its blocks holding grid cells (W / 16 for every tile but the last of a
// row).
__device__ __forceinline__ int tile_windows(int nx, int X0, int W = kTile) {
    const int nb = (nx - X0 + 15) >> 4;
    return (nb < W / 16 ? nb : W / 16) + 1;
}

// MMAs of sub-tile h of a staged tile into accumulator columns from d.
// a_hi0 is the descriptor of the stage's hi plane (lo follows at
// +kPlaneStage); band is the shared-memory address of the stencil's bands.
// Descriptors for base + offset are the base descriptor plus offset >> 4 (the
// start-address field holds address >> 4 in its low bits).
//  plain: even windows (disjoint outputs, the first of them initialising)
//    before odd windows, which add into the overlaps; NWIN windows (all, or
//    the first half's, issue_plain_tile).
//  split: per window and coefficient row, one N=96 MMA of hi with the stacked
//    band (initialising its region on the first row) and one N=32 MMA of lo
//    with cf into the region's middle part.
template <int R, bool SPLIT, class SG = StageHalo2, int NWIN = Mode<SPLIT>::SUB_WIN>
__device__ __forceinline__ void issue_subtile(uint64_t a_hi0, uint32_t band, uint32_t d, int h) {
    using M = Mode<SPLIT>;
    constexpr int NDY = 2 * R + 1;
    if (!SPLIT) {
        const uint64_t b0 = smem_desc(band, 512, 128);
#pragma unroll
        for (int parity = 0; parity < 2; parity++) {
#pragma unroll
            for (int dy = 0; dy < NDY; dy++) {
                const uint64_t b = b0 + (uint64_t)((dy * kBandBytes) >> 4);
                const uint32_t acc = (parity == 1 || dy > 0) ? 1u : 0u;
#pragma unroll
                for (int w = parity; w < NWIN; w += 2) {
                    const int wg = h * M::SUB_BLOCKS + w;  // window in the tile
                    const uint64_t a_off = (uint64_t)((2 * wg * SG::CHUNK + (SG::TOP - R + dy) * 16) >> 4);
                    umma_f16(d + 16 * w, a_hi0 + a_off, b, kIdesc, acc);
                }
            }
        }
    } else {
#pragma unroll
        for (int w = 0; w < M::SUB_WIN; w++)
            issue_split_window<R, SG>(a_hi0, band, d + split_region(w), h * M::SUB_BLOCKS + w);
    }
}

// A plain tile's MMAs: the windows of its first 64, 96 or 128 columns, the
// smallest of these that covers the nwin windows (tile_windows) its blocks
// need, so that 64- and 96-column tiles, and tiles at the end of a row, skip
// the rest.  Three compile-time sequences: a window bound tested per MMA
// slowed the issuer.
template <int R, class SG>
__device__ __forceinline__ void issue_plain_tile(uint64_t a_hi0, uint32_t band, uint32_t d,
                                                 int nwin) {
    if (nwin <= 5) issue_subtile<R, false, SG, 5>(a_hi0, band, d, 0);
    else if (nwin <= 7) issue_subtile<R, false, SG, 7>(a_hi0, band, d, 0);
    else issue_subtile<R, false, SG>(a_hi0, band, d, 0);
}

// Epilogue, first half: this warp's accumulators of a sub-tile into
// registers, one FP32 value per output (lanes = tile rows of the warp's lane
// quarter, `half` = which half of the sub-tile's column blocks).  lane_col is
// the TMEM address of the warp's lane quarter at the sub-tile's first column.
// After it returns the accumulator may be reused.
template <bool SPLIT>
__device__ __forceinline__ void epilogue_load(uint32_t lane_col, int half,
                                              float (&f)[Mode<SPLIT>::SUB_BLOCKS / 2][16]) {
    using M = Mode<SPLIT>;
    constexpr int G = M::SUB_BLOCKS / 2;
    const int j0 = half * G;
    if (!SPLIT) {
        // output block jl is accumulator columns 16(jl+1) .. 16(jl+1)+15
        uint32_t v[G][16];
#pragma unroll
        for (int gg = 0; gg < G; gg++) tmem_ld_x16(lane_col + 16 * (j0 + gg + 1), v[gg]);
        tmem_ld_wait();
#pragma unroll
        for (int gg = 0; gg < G; gg++)
#pragma unroll
            for (int c = 0; c < 16; c++) f[gg][c] = __uint_as_float(v[gg][c]);
    } else {
        // block jl = second half of window jl + first half of window jl+1
#pragma unroll
        for (int gg = 0; gg < G; gg++) {
            const int jl = j0 + gg;
            split_block_load(lane_col + split_region(jl), lane_col + split_region(jl + 1), f[gg]);
        }
    }
}

// Output of one tile: planes, geometry and the update rectangle.
struct TileOut {
    const uint16_t *in_hi, *in_lo;  // input planes (cells outside the rectangle)
    uint16_t *out_hi, *out_lo;
    PlaneGeom pg;
    int y0, y1, x0, x1;
    int ny, nx;                     // the grid (split maxima cover its cells only)
};

// Epilogue walk over one step of split windows for block group g of ng
// groups: block j (windows j and j+1) belongs to group j mod ng.  Every
// window is released exactly once per group, in increasing order, whether
// the group reads it or not; ready(w) is the bounded wait for window w,
// release(w) gives it back, block(j) loads block j, releases its two
// windows and stores.  Returns false when a wait gave up.
template <typename Ready, typename Release, typename Block>
__device__ __forceinline__ bool walk_windows(int g, int ng, int nwin, Ready &&ready,
                                             Release &&release, Block &&block) {
    int w = 0;
    for (int j = g; j < nwin - 1; j += ng) {
        for (; w < j; w++) {
            if (!ready(w)) return false;
            release(w);
        }
        if (!ready(j) || !ready(j + 1)) return false;
        block(j);
        w = j + 2;
    }
    for (; w < nwin; w++) {
        if (!ready(w)) return false;
        release(w);
    }
    return true;
}

// Converts and stores one 16-column output block of tile row y (cells xb ..
// xb+15).  fast: the whole tile is inside the update rectangle; otherwise
// cells outside it copy the input.
//  split: fast blocks take the paired split (split_pair), others split each
//    updated cell alone (split_fixed: the same bits) and copy the rest.
//  plain: every cell is converted in pairs (pack_h2, the same bits as h_bits
//    per cell); where a thread's 16 cells are not all inside, the input
//    words are blended back in under a per-cell mask.
// (Measured on GB300: the blend is faster for plain blocks, the separate
// per-cell path faster for split ones, whose epilogue is sensitive to code
// size.)
template <bool SPLIT>
__device__ __forceinline__ void store_block(const TileOut &o, const float (&f)[16], int y, int xb,
                                            bool fast, bool row_in) {
    const size_t off0 = plane_index16(o.pg, y, xb);     // cells xb .. xb+7
    const size_t off1 = off0 + (size_t)o.pg.nyp * 8;  // cells xb+8 .. xb+15
    uint32_t hw[8], lw[8];
    if constexpr (SPLIT) {
        if (fast) {
#pragma unroll
            for (int c = 0; c < 8; c++) split_pair(f[2 * c], f[2 * c + 1], hw[c], lw[c]);
        } else {
            const uint4 i0 = *reinterpret_cast<const uint4 *>(o.in_hi + off0);
            const uint4 i1 = *reinterpret_cast<const uint4 *>(o.in_hi + off1);
            const uint4 l0 = *reinterpret_cast<const uint4 *>(o.in_lo + off0);
            const uint4 l1 = *reinterpret_cast<const uint4 *>(o.in_lo + off1);
            const uint32_t iw[8] = {i0.x, i0.y, i0.z, i0.w, i1.x, i1.y, i1.z, i1.w};
            const uint32_t il[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
#pragma unroll
            for (int c = 0; c < 8; c++) {
                uint16_t hh[2], ll[2];
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    const int x = xb + 2 * c + u;
                    if (row_in && x >= o.x0 && x < o.x1) {
                        split_fixed(f[2 * c + u], hh[u], ll[u]);
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
        *reinterpret_cast<uint4 *>(o.out_lo + off0) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        *reinterpret_cast<uint4 *>(o.out_lo + off1) = make_uint4(lw[4], lw[5], lw[6], lw[7]);
    } else {
        (void)lw;
#pragma unroll
        for (int c = 0; c < 8; c++) hw[c] = pack_h2(f[2 * c], f[2 * c + 1]);
        if (!fast && !(row_in && xb >= o.x0 && xb + 16 <= o.x1)) {
            const uint4 i0 = *reinterpret_cast<const uint4 *>(o.in_hi + off0);
            const uint4 i1 = *reinterpret_cast<const uint4 *>(o.in_hi + off1);
            const uint32_t iw[8] = {i0.x, i0.y, i0.z, i0.w, i1.x, i1.y, i1.z, i1.w};
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const int x = xb + 2 * c;
                const uint32_t m = (row_in && x >= o.x0 && x < o.x1 ? 0x0000ffffu : 0u) |
                                   (row_in && x + 1 >= o.x0 && x + 1 < o.x1 ? 0xffff0000u : 0u);
                hw[c] = (hw[c] & m) | (iw[c] & ~m);
            }
        }
        *reinterpret_cast<uint4 *>(o.out_hi + off0) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *reinterpret_cast<uint4 *>(o.out_hi + off1) = make_uint4(hw[4], hw[5], hw[6], hw[7]);
    }
}

// After a warp has stored its blocks of a tile (row y, blocks X0 + 16 j for
// j = j0, j0 + dj, ... < nblk), on a step whose copies change scale
// (cs.k != 0, the same for every thread): the grid cells among them outside
// the update rectangle (a fixed border), which the stores copied, are split
// again from the input planes, scaled by 2^k.  A pass of its own with rolled
// loops (each 8-cell panel row's input words loaded at once, then taken two
// cells at a time from the front of the word arrays): such steps are few,
// and this code inside the unrolled stores slowed every step of the
// epilogue-bound kernels (measured on GB300: 512 mixed split grids
// 5.66 -> 6.15 ms, 16386² 378 -> 386 us per step).
__device__ __forceinline__ void resplit_border(const TileOut &o, int y, int X0, int j0, int dj,
                                               int nblk, const StepScale &cs) {
    if (y >= o.ny) return;
    const bool row_in = y >= o.y0 && y < o.y1;
#pragma unroll 1
    for (int j = j0; j < nblk; j += dj) {
        const int xb = X0 + 16 * j;
        if (xb >= o.nx || (row_in && xb >= o.x0 && xb + 16 <= o.x1)) continue;
#pragma unroll 1
        for (int hf = 0; hf < 2; hf++) {
            const int xh = xb + 8 * hf;  // a panel row: cells xh .. xh+7
            if (xh >= o.nx || (row_in && xh >= o.x0 && xh + 8 <= o.x1)) continue;
            const size_t off = plane_index16(o.pg, y, xh);
            const uint4 a = *reinterpret_cast<const uint4 *>(o.in_hi + off);
            const uint4 b = *reinterpret_cast<const uint4 *>(o.in_lo + off);
            uint32_t hw[4] = {a.x, a.y, a.z, a.w}, lw[4] = {b.x, b.y, b.z, b.w};
#pragma unroll 1
            for (int q = 0; q < 8; q += 2) {
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    const int x = xh + q + u;
                    if (x < o.nx && !(row_in && x >= o.x0 && x < o.x1)) {
                        uint16_t h = (uint16_t)(hw[0] >> (16 * u));
                        uint16_t l = (uint16_t)(lw[0] >> (16 * u));
                        resplit_pair(h, l, cs);
                        o.out_hi[off + q + u] = h;
                        o.out_lo[off + q + u] = l;
                    }
                }
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    hw[c] = hw[c + 1];
                    lw[c] = lw[c + 1];
                }
            }
        }
    }
}

// store_block<true> of the values v 2^k (StepScale ss): fast blocks split in
// pairs, others split each updated cell alone and copy the rest (on a step
// whose copies change scale, resplit_border then rewrites the grid's copied
// cells).  The largest |u| of the updated cells is kept in mx (the border's
// share of the step maximum is the record's B; padding cells never count).
__device__ __forceinline__ void store_block_split(const TileOut &o, const float (&f)[16], int y,
                                                  int xb, bool fast, bool row_in,
                                                  const StepScale &ss, float &mx) {
    const size_t off0 = plane_index16(o.pg, y, xb);     // cells xb .. xb+7
    const size_t off1 = off0 + (size_t)o.pg.nyp * 8;  // cells xb+8 .. xb+15
    uint32_t hw[8], lw[8];
    if (fast) {
#pragma unroll
        for (int c = 0; c < 8; c++) split_pair_s(f[2 * c], f[2 * c + 1], ss.s, hw[c], lw[c], mx);
    } else {
        const uint4 i0 = *reinterpret_cast<const uint4 *>(o.in_hi + off0);
        const uint4 i1 = *reinterpret_cast<const uint4 *>(o.in_hi + off1);
        const uint4 l0 = *reinterpret_cast<const uint4 *>(o.in_lo + off0);
        const uint4 l1 = *reinterpret_cast<const uint4 *>(o.in_lo + off1);
        const uint32_t iw[8] = {i0.x, i0.y, i0.z, i0.w, i1.x, i1.y, i1.z, i1.w};
        const uint32_t il[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
#pragma unroll
        for (int c = 0; c < 8; c++) {
            uint16_t hh[2], ll[2];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int x = xb + 2 * c + u;
                if (row_in && x >= o.x0 && x < o.x1) {
                    split_fixed_s(f[2 * c + u], ss.s, hh[u], ll[u], mx);
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
    *reinterpret_cast<uint4 *>(o.out_lo + off0) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
    *reinterpret_cast<uint4 *>(o.out_lo + off1) = make_uint4(lw[4], lw[5], lw[6], lw[7]);
}

__device__ __forceinline__ bool tile_inside(const TileOut &o, int Y0, int X0) {
    return Y0 >= o.y0 && Y0 + kTile <= o.y1 && X0 >= o.x0 && X0 + kTile <= o.x1;
}

// Epilogue, second half: converts and stores this warp's outputs of sub-tile
// h (tile row m).
template <bool SPLIT>
__device__ __forceinline__ void epilogue_store(const TileOut &o,
                                               const float (&f)[Mode<SPLIT>::SUB_BLOCKS / 2][16],
                                               int h, int half, int m, int Y0, int X0) {
    using M = Mode<SPLIT>;
    constexpr int G = M::SUB_BLOCKS / 2;
    const int j0 = half * G;
    const int y = Y0 + m;
    const bool fast = tile_inside(o, Y0, X0);
    const bool row_in = y >= o.y0 && y < o.y1;
#pragma unroll
    for (int gg = 0; gg < G; gg++)
        store_block<SPLIT>(o, f[gg], y, X0 + 16 * (h * M::SUB_BLOCKS + j0 + gg), fast, row_in);
}

// Plain tiles of W = 64, 96 or 128 columns (the plain sweep kernel's
// tile_w): the W / 16 output blocks are shared evenly by the two epilogue
// warpgroups, G = W / 32 each, and only blocks holding grid cells (nblk, from
// tile_windows) are stored.  Widths are multiples of 32 so that every window
// keeps its parity (even windows initialise the accumulator, odd ones add)
// from 128-column tiles: each output sums the same products in the same
// order, and results are bit-identical whatever the width.
__device__ __forceinline__ bool tile_inside_w(const TileOut &o, int Y0, int X0, int W) {
    return Y0 >= o.y0 && Y0 + kTile <= o.y1 && X0 >= o.x0 && X0 + W <= o.x1;
}

// This warp's blocks j0 .. j0+G-1 of a plain accumulator (lane_col: its lane
// quarter at the slot's first column) into registers; then `release` (the
// accumulator may be refilled); then the blocks below nblk are stored.
template <int G, typename Release>
__device__ __forceinline__ void plain_epilogue(const TileOut &o, uint32_t lane_col, int j0,
                                               int nblk, int y, int X0, bool fast, bool row_in,
                                               Release &&release) {
    uint32_t v[G][16];
#pragma unroll
    for (int gg = 0; gg < G; gg++) tmem_ld_x16(lane_col + 16 * (j0 + gg + 1), v[gg]);
    tmem_ld_wait();
    release();
#pragma unroll
    for (int gg = 0; gg < G; gg++) {
        if (j0 + gg < nblk) {
            float f[16];
#pragma unroll
            for (int c = 0; c < 16; c++) f[c] = __uint_as_float(v[gg][c]);
            store_block<false>(o, f, y, X0 + 16 * (j0 + gg), fast, row_in);
        }
    }
}

// Launches a single-grid step kernel with programmatic stream serialization:
// the next step's CTAs do their set-up (barriers, TMEM, bands) while this
// step's last tiles finish, and wait in pdl_wait() before touching a plane
// (pdl_enabled: TCS_PDL=0 in the environment launches in plain stream order).
// cooperative: a launch of several steps, whose CTAs wait on one another's
// tile rows, must have all its CTAs resident at once (and is not overlapped).
template <typename Params>
cudaError_t launch_step(void (*kernel)(Params), int grid, int threads, size_t smem,
                        cudaStream_t s, const Params &p, bool cooperative = false) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    if (cooperative) {
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
    } else {
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
    }
    cfg.attrs = attr;
    cfg.numAttrs = (cooperative || pdl_enabled()) ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, p);
}

}  // namespace tc
}  // namespace tcs
