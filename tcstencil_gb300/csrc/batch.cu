// Batched sweeps: many grids of different sizes, stencils, coefficients,
// precisions (FP16 or split) and step counts advanced by ONE persistent
// tensor-core launch.
//
// Work list.  Every (grid, step, tile) is one item; items are ordered step
// major (all grids' first steps, then all second steps, ...) and decoded from
// their index on the device (BatchParams), so a run's description is a few
// small tables however many items it has.  Each CTA (one per SM) takes the
// next index from a global counter, so items are taken in order, and only by
// running CTAs.  An item of step t > 0 needs every
// tile of its grid's step t - 1: the producer waits (bounded) on a
// per-(grid, step) completion counter that the epilogue warps increment after
// their stores (release reductions, one per run of consecutive items of the
// same grid and step; the producer polls with acquire loads, once per run of
// items of the same grid and step).  Those items come earlier in the list and
// so were taken by
// running CTAs; the earliest unfinished item always has its inputs ready, so
// the launch cannot deadlock, whatever else shares the GPU.
// The same counters also guard the ping-pong's write-after-read hazard: step
// t+1 overwrites the plane step t-1 read, and starts only after all of step t,
// hence all of step t-1, finished.
//
// Per item the producer loads the tile's input panels (one tensor-map load per
// plane, from the grid's maps in device memory) AND bulk-copies the grid's
// coefficient bands (prebuilt in global memory by build_bands_kernel) into the
// stage, so the MMA issuers need nothing else; stencil radius and precision
// select one of four fully unrolled MMA sequences (tc_core.cuh), the same code
// the single-grid kernel runs, so every grid gets the same bits alone and in
// a batch.  The run ends with a tiny kernel that flips each grid's ping-pong
// state, so a captured graph can be replayed to advance the batch again.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "batch.h"
#include "tc_core.cuh"

namespace tcs {

namespace {

using namespace tc;
using SG = StageLines;  // line-aligned staging, as the single-grid kernels

__device__ int g_batch_error = 0;

// Per-precision launch shapes.  FP16 items: three stages of one plane plus
// bands, two accumulator slots, eight epilogue warps (the single-grid plain
// kernel's shape).  Split items: two stages of hi+lo plus bands, the window
// ring of the single-grid split kernel, twelve epilogue warps in three groups.
constexpr int kRing = 8;  // published work items in flight
// The work layout (step offsets, tile prefix) is copied into shared memory
// when it fits, so decoding an item costs no global round trip.
constexpr int kTableInts = 2048;
// barriers, the item ring and the per-slot scale words, before the tables
constexpr int kBarrierArea = 832;
template <bool SPLIT>
struct BatchCfg {
    // FP16: four stages, a multiple of the two issuers, so stage i % 4 holds
    // only one issuer's items (see the MMA issuers)
    static constexpr int STAGES = SPLIT ? 2 : 4;
    static constexpr int PLANES = SPLIT ? 2 : 1;
    static constexpr int BAND_BYTES = (SPLIT ? 4 : 1) * 5 * kBandBytes;  // radius 2
    static constexpr int STAGE_BYTES = PLANES * SG::PLANE + BAND_BYTES;
    static constexpr int GROUPS = SPLIT ? 3 : 2;
    static constexpr int EPI_WARPS = 4 * GROUPS;
    // MMA issuer warps 1 and 2 (one issues while the other waits on a region
    // or slot, or commits): split items alternate windows between them, FP16
    // items alternate whole items
    static constexpr int ISSUERS = 2;
    // commits that free a stage: both issuers' (split), the item's issuer's (FP16)
    static constexpr int STAGE_RELEASES = SPLIT ? 2 : 1;
    static constexpr int EPI_WARP0 = 1 + ISSUERS;
    static constexpr int SIGNAL_WARP = EPI_WARP0 + EPI_WARPS;
    static constexpr int THREADS = 32 * (SIGNAL_WARP + 1);
    static constexpr size_t SMEM = 1024 + (size_t)STAGES * STAGE_BYTES + kBarrierArea + kTableInts * 4;
    static_assert(kRing > STAGES + 2, "a ring slot is reused only after its item's epilogue");
    static_assert(SMEM <= 232448, "shared memory budget");
    static_assert(STAGE_BYTES % 16 == 0, "bulk copy alignment");
};
constexpr int kBatchRingSlots = 5;  // split window regions in TMEM
constexpr int kBatchRegion = 96;



// A bounded wait gave up: record the code in the launch's error word (which
// every CTA polls to stop early) and in the unit's word tcs_device_error reads.
__device__ __forceinline__ void batch_fail(const BatchParams &p, int code) {
    record_error(p.error, code);
    record_error(&g_batch_error, code);
}

// Work index k -> (grid, step, tile) from the step offsets and tile prefix
// (shared or global memory); see BatchParams.
__device__ __forceinline__ BatchItem decode_item(const int *step_off, const int *tile_prefix,
                                                 int n_steps, int n_grids, int k) {
    int lo = 0, hi = n_steps;  // step_off[lo] <= k < step_off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (step_off[mid] <= k) lo = mid;
        else hi = mid;
    }
    const int local = k - step_off[lo];
    int a = 0, b = n_grids;  // tile_prefix[a] <= local < tile_prefix[b]
    while (b - a > 1) {
        const int mid = (a + b) >> 1;
        if (tile_prefix[mid] <= local) a = mid;
        else b = mid;
    }
    return BatchItem{a, lo, local - tile_prefix[a]};
}

// The item after `it` (index k + 1), from two table reads: the next tile of
// the grid, else the first tile of the next grid still running at this step,
// else the first tile of the next step.
__device__ __forceinline__ BatchItem next_item(const BatchItem &it, const int *step_off,
                                               const int *tile_prefix) {
    const int local = tile_prefix[it.g] + it.tile + 1;  // within step it.t
    if (local < step_off[it.t + 1] - step_off[it.t]) {
        if (local < tile_prefix[it.g + 1]) return BatchItem{it.g, it.t, it.tile + 1};
        return BatchItem{it.g + 1, it.t, 0};
    }
    return BatchItem{0, it.t + 1, 0};
}

__global__ void build_bands_kernel(BatchGrid *grids, const float *coefs, uint16_t *bands) {
    const BatchGrid &g = grids[blockIdx.x];
    build_bands(bands + g.band_base, coefs + 25 * blockIdx.x, g.r, g.box, g.split, threadIdx.x,
                blockDim.x);
}

struct BandArgs {
    float coef[25];
};

__global__ void build_one_band_kernel(const BandArgs a, int r, int box, int split, uint16_t *dst) {
    build_bands(dst, a.coef, r, box, split, threadIdx.x, blockDim.x);
}

__global__ void flip_states_kernel(BatchGrid *grids, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) grids[i].state ^= grids[i].steps & 1;
}

template <bool SPLIT>
__global__ void __launch_bounds__(BatchCfg<SPLIT>::THREADS, 1) tc_batch_kernel(const BatchParams p) {
    using C = BatchCfg<SPLIT>;
    constexpr int NS = C::STAGES;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                ~static_cast<uintptr_t>(1023));
    uint8_t *stage_base = smem;  // [NS][planes | bands]
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (size_t)NS * C::STAGE_BYTES);
    // accumulator barriers: plain [2] slots, split [kBatchRingSlots] windows
    constexpr int NACC = SPLIT ? kBatchRingSlots : 2;
    uint64_t *full = bars;                        // [NS]
    uint64_t *empty = bars + NS;                  // [NS]
    uint64_t *acc_full = bars + 2 * NS;           // [NACC]
    uint64_t *acc_empty = acc_full + NACC;        // [NACC]
    uint64_t *drain = acc_empty + NACC;           // [1]
    uint64_t *item_ready = drain + 1;             // [kRing]
    uint64_t *item_done = item_ready + kRing;     // [kRing] epilogue stores issued
    uint64_t *ring_free = item_done + kRing;      // [kRing] signal warp done with the slot
    BatchItem *ring = reinterpret_cast<BatchItem *>(ring_free + kRing);  // [kRing]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(ring + kRing);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    // split: per ring slot, the item's scale (producer -> epilogue, behind
    // item_scaled) and its largest |x'| (FP32 bits), which the signal warp
    // adds to the grid's scale record
    uint64_t *item_scaled = reinterpret_cast<uint64_t *>(tmem_slot + 2);  // [kRing]
    ItemScale *ring_scale = reinterpret_cast<ItemScale *>(item_scaled + kRing);  // [kRing]
    unsigned *item_max = reinterpret_cast<unsigned *>(ring_scale + kRing);       // [kRing]
    volatile int *grid_error = p.error;
    static_assert((2 * NS + 2 * NACC + 1 + 3 * kRing) * 8 + kRing * sizeof(BatchItem) + 8 +
                          kRing * (8 + sizeof(ItemScale) + 4) <= kBarrierArea,
                  "barrier area");
    int *tables = reinterpret_cast<int *>(reinterpret_cast<uint8_t *>(bars) + kBarrierArea);
    const int n_table = p.n_steps + 1 + p.n_grids + 1;
    const bool tables_in_smem = n_table <= kTableInts;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    // a wait on another role may span the producer's dependency or gate wait
    const uint64_t wait_lim = p.wait_ns + kWaitLimitNs;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], C::STAGE_RELEASES);
        }
        for (int b = 0; b < NACC; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], C::EPI_WARPS);
        }
        mbar_init(drain, C::ISSUERS);
        for (int j = 0; j < kRing; j++) {
            mbar_init(&item_ready[j], 1);
            mbar_init(&item_done[j], C::EPI_WARPS);
            mbar_init(&ring_free[j], 1);
            mbar_init(&item_scaled[j], 1);
            item_max[j] = 0u;
        }
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        __syncwarp();
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    if (tables_in_smem) {
        for (int i = threadIdx.x; i <= p.n_steps; i += blockDim.x) tables[i] = p.step_off[i];
        for (int i = threadIdx.x; i <= p.n_grids; i += blockDim.x)
            tables[p.n_steps + 1 + i] = p.tile_prefix[i];
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        // ------------------------------------------------------ producer ---
        // Takes work indices in increasing order from the global counter,
        // p.grab at a time, decodes each once and publishes it in ring slot
        // i % kRing; an index past the end is published as the stop sentinel.
        // Software pipelined: once an item's copies are issued, the next item
        // is decoded and its grid descriptor loaded (and, at the end of a
        // group, the group after the next one requested), so those latencies
        // overlap the stage and ring waits of the next iteration.
        if (lane == 0) {
            const int *step_off = tables_in_smem ? tables : p.step_off;
            const int *tile_prefix = tables_in_smem ? tables + p.n_steps + 1 : p.tile_prefix;
            int last_issued = -1;
            // (grid, step) whose dependency this thread has already seen met;
            // later items of the same pair need no further poll or fence
            int met_g = -1, met_t = -1;
            // (grid, step) of the scale in iscale (split items)
            int sc_g = -1, sc_t = -1;
            ItemScale iscale{};
            // split: the last issued item's scale is published at the top of
            // the next iteration, before its dependency poll (which may wait
            // for that item): its loads land meanwhile, and the thread never
            // stalls on them before the next stage and ring waits
            int pub_j = -1, pub_t = 0;
            bool pub_fresh = false;
            ScaleWords pub_sw{};
            SplitScale *pub_sc = nullptr;
            auto publish = [&]() {
                if (!SPLIT || pub_j < 0) return;
                if (pub_fresh) {
                    const StepScale ss = scale_of(pub_sw, pub_t + 1);
                    iscale = ItemScale{ss.s, ss.k, ss.e, pub_sc};
                } else if (!pub_sc) {
                    iscale = ItemScale{2048.0f, 0, 0, nullptr};
                }
                ring_scale[pub_j] = iscale;
                mbar_arrive(&item_scaled[pub_j]);
                pub_j = -1;
            };
            const int grab = p.grab;
            int k = (int)atomicAdd(p.work_counter, (unsigned)grab);  // the item of this iteration
            int k_end = k + grab;                                   // end of its group
            int k_next = k;                                          // start of the next group
            BatchItem it{};
            BatchGrid g{};
            if (k < p.n_items) {
                it = decode_item(step_off, tile_prefix, p.n_steps, p.n_grids, k);
                g = p.grids[it.g];
                k_next = (int)atomicAdd(p.work_counter, (unsigned)grab);
            }
            for (int i = 0;; i++) {
                const int s = i % NS, j = i % kRing;
                if (!mbar_wait(&empty[s], ((i / NS) & 1) ^ 1, abort_flag, wait_lim) ||
                    !mbar_wait(&ring_free[j], ((i / kRing) & 1) ^ 1, abort_flag, wait_lim)) {
                    batch_fail(p, kErrWaitEmpty);
                    *abort_flag = 1;
                    break;
                }
                publish();
                if (k >= p.n_items) {
                    ring[j] = BatchItem{-1, 0, 0};
                    mbar_arrive(&item_ready[j]);
                    break;
                }
                // the tile's row and column, once, for every role
                it.ty = it.tile / g.tiles_x;
                it.tx = it.tile - it.ty * g.tiles_x;
                ring[j] = it;
                mbar_arrive(&item_ready[j]);
                // step t > 0: every tile of the grid's previous step is stored;
                // step 0 of a gated grid: the external gate is open
                const unsigned *ctr = nullptr;
                unsigned target = 0;
                if (it.g == met_g && it.t == met_t) {
                    // met before, and the proxy fence after that poll still orders the copies below
                } else if (it.t > 0) {
                    ctr = p.counters + (size_t)(g.ctr_base + it.t - 1) * kRowCounterStride;
                    target = (unsigned)(g.n_tiles * C::EPI_WARPS);
                } else if (g.gate) {
                    ctr = g.gate;
                    target = g.gate_value;
                }
                if (ctr) {
                    if (ld_acquire(ctr) < target) {
                        const uint64_t t0 = global_timer_ns();
                        bool ok = true;
                        while (ld_acquire(ctr) < target) {
                            if (*grid_error || global_timer_ns() - t0 > p.wait_ns) {
                                ok = false;
                                break;
                            }
                            __nanosleep(64);
                        }
                        if (!ok) {
                            batch_fail(p, kErrWaitDep);
                            *abort_flag = 1;
                            break;
                        }
                    }
                    // the bulk copies below read what other SMs stored
                    fence_proxy_async_global();
                    met_g = it.g;
                    met_t = it.t;
                }
                // split: the step's scale, once per (grid, step).  Steps t-2
                // and t-3 of the grid are final (step t-1 is, after the wait
                // above); the loads are issued here and used in publish().
                ScaleWords sw{};
                const bool fresh = SPLIT && g.scale && (it.g != sc_g || it.t != sc_t);
                if (fresh) sw = scale_words(g.scale, it.t + 1);
                const int band_bytes = batch_band_elems(g.r, SPLIT) * 2;
                uint8_t *st = stage_base + (size_t)s * C::STAGE_BYTES;
                mbar_arrive_expect_tx(&full[s], C::PLANES * SG::PLANE + band_bytes);
                const int in = (g.state + it.t) & 1;
                const CUtensorMap *maps = g.maps + 2 * in;
                load_tile_map(maps, maps + 1, C::PLANES, it.ty * kTile, it.tx * kTile, st, &full[s]);
                bulk_load(st + C::PLANES * SG::PLANE, p.bands + g.band_base, band_bytes, &full[s]);
                if (SPLIT) {
                    pub_j = j;
                    pub_t = it.t;
                    pub_fresh = fresh;
                    pub_sw = sw;
                    pub_sc = g.scale;
                    if (fresh) {
                        sc_g = it.g;
                        sc_t = it.t;
                    } else if (!g.scale) {
                        sc_g = sc_t = -1;
                    }
                }
                last_issued = i;
                // the next item: decoded, its descriptor loads in flight
                const int g_prev = it.g;
                if (++k == k_end) {
                    k = k_next;
                    k_end = k + grab;
                    if (k < p.n_items) {
                        it = decode_item(step_off, tile_prefix, p.n_steps, p.n_grids, k);
                        k_next = (int)atomicAdd(p.work_counter, (unsigned)grab);
                    }
                } else if (k < p.n_items) {
                    it = next_item(it, step_off, tile_prefix);
                }
                if (k < p.n_items) {
                    if (it.g != g_prev) g = p.grids[it.g];
                    const CUtensorMap *maps = g.maps + 2 * ((g.state + it.t) & 1);
                    tma_prefetch_map(maps);
                    if (SPLIT) tma_prefetch_map(maps + 1);
                }
            }
            for (int k = 0; k < NS && last_issued - k >= 0; k++) {
                const int ii = last_issued - k;
                const uint64_t t0 = global_timer_ns();
                while (!mbar_try_wait(&full[ii % NS], (ii / NS) & 1)) {
                    if (global_timer_ns() - t0 > kWaitLimitNs) {
                        batch_fail(p, kErrWaitDrain);
                        break;
                    }
                }
            }
        }
    } else if (warp <= C::ISSUERS) {
        // --------------------------------------------------- MMA issuers ---
        // Both issuers read every published item, in order (the slot sequence
        // and the stop sentinel).  Split: both wait for every stage fill and
        // issue alternate windows.  FP16: item i's issuer is i % 2 and it alone
        // waits for the item's stage: with four stages a stage only holds one
        // issuer's items, so each stage's fills are waited for by one thread in
        // order (an mbarrier parity wait also succeeds for the phase before the
        // current one, so a thread must never skip a fill it later waits past).
        // A ring slot is republished only after the signal warp finished its
        // item, which needs a lagging issuer's own earlier item, so neither
        // issuer can be lapped on the ring.
        if (lane == 0) {
            const int id = warp - 1;  // split: windows G % 2 == id; FP16: items i % 2 == id
            AccSlots slots;  // FP16: walks every item, so both see the same slot uses
            int G = 0;       // split: global window counter of the ring
            bool stop = false;
            for (int i = 0; !stop; i++) {
                const int s = i % NS;
                if (!mbar_wait(&item_ready[i % kRing], (i / kRing) & 1, abort_flag, wait_lim)) {
                    batch_fail(p, kErrWaitFull);
                    *abort_flag = 1;
                    break;
                }
                const BatchItem it = ring[i % kRing];
                if (it.g < 0) break;
                uint32_t col = 0, mask = 0;
                if constexpr (!SPLIT) {
                    mask = slots.take(false, col);
                    if ((i & 1) != id) {
                        slots.used(mask);
                        continue;
                    }
                }
                if (!mbar_wait(&full[s], (i / NS) & 1, abort_flag, wait_lim)) {
                    batch_fail(p, kErrWaitFull);
                    *abort_flag = 1;
                    break;
                }
                const BatchGrid g = p.grids[it.g];  // one batch of loads, before any barrier
                uint8_t *st = stage_base + (size_t)s * C::STAGE_BYTES;
                const uint64_t a_hi0 = smem_desc(smem_u32(st), SG::CHUNK, 128);
                const uint32_t band = smem_u32(st + C::PLANES * SG::PLANE);
                if constexpr (SPLIT) {
                    const int nwin = tile_windows(g.nx, it.tx * kTile);
#pragma unroll 1
                    for (int w = 0; w < nwin; w++, G++) {
                        if ((G & 1) != id) continue;
                        const int r = G % kBatchRingSlots;
                        if (!mbar_wait(&acc_empty[r], ((G / kBatchRingSlots) & 1) ^ 1, abort_flag, wait_lim)) {
                            batch_fail(p, kErrWaitAccum);
                            *abort_flag = 1;
                            stop = true;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t d = tmem_base + r * kBatchRegion;
                        if (g.r == 1) issue_split_window<1, SG>(a_hi0, band, d, w);
                        else issue_split_window<2, SG>(a_hi0, band, d, w);
                        umma_commit(&acc_full[r]);
                    }
                } else {
                    if (!slots.acquire(acc_empty, mask, abort_flag, wait_lim)) {
                        batch_fail(p, kErrWaitAccum);
                        *abort_flag = 1;
                        stop = true;
                    } else {
                        tc_fence_after();
                        const uint32_t d = tmem_base + col;
                        // all windows: FP16 items are bound by the producer, and a
                        // second MMA sequence for edge tiles measured slower
                        if (g.r == 1) issue_subtile<1, false, SG>(a_hi0, band, d, 0);
                        else issue_subtile<2, false, SG>(a_hi0, band, d, 0);
                        slots.commit(acc_full, mask);
                        slots.used(mask);
                    }
                }
                if (!stop) umma_commit(&empty[s]);
            }
            // every issuer commits (one with nothing in flight completes at
            // once), so the drain phase always completes
            umma_commit(drain);
            const uint64_t t0 = global_timer_ns();
            while (!mbar_try_wait(drain, 0)) {
                if (global_timer_ns() - t0 > kWaitLimitNs) {
                    batch_fail(p, kErrWaitDrain);
                    break;
                }
            }
        }
    } else if (warp == C::SIGNAL_WARP) {
        // -------------------------------------------------------- signal ---
        // Publishes completed items to the other SMs, off the epilogue
        // warps' path: once all epilogue warps have issued an item's stores
        // (item_done, release at CTA scope), one release reduction at GPU
        // scope makes them visible before the count (release is cumulative).
        // Counts are held while consecutive items share a (grid, step) and
        // released when the next item differs or the run ends; the items
        // that wait on them belong to a later step, which the producer
        // publishes in the ring before it waits, so the release comes first.
        if (lane == 0) {
            unsigned *pend = nullptr;
            unsigned n_pend = 0;
            // split: the largest |x'| of the held items, for their (grid,
            // step)'s scale record, added once before their counts go out
            SplitScale *pend_sc = nullptr;
            int pend_t = 0;
            unsigned pend_max = 0u;
            auto release = [&]() {
                if (SPLIT && pend_sc)
                    atomicMax(&pend_sc->maxbits[pend_t & (kScaleRing - 1)], pend_max);
                red_release_add(pend, n_pend);
                n_pend = 0;
                pend_max = 0u;
            };
            auto give_up = [&]() {
                batch_fail(p, kErrWaitResult);
                *abort_flag = 1;
            };
            for (int i = 0;; i++) {
                const int j = i % kRing;
                if (!mbar_wait(&item_ready[j], (i / kRing) & 1, abort_flag, wait_lim)) {
                    give_up();
                    break;
                }
                const BatchItem it = ring[j];
                unsigned *ctr = nullptr;
                if (it.g >= 0)
                    ctr = p.counters + (size_t)(p.grids[it.g].ctr_base + it.t) * kRowCounterStride;
                if (n_pend && ctr != pend) release();
                if (it.g < 0) break;
                if (!mbar_wait(&item_done[j], (i / kRing) & 1, abort_flag, wait_lim)) {
                    give_up();
                    break;
                }
                if (SPLIT) {
                    // the item's maximum joins the held one; the step's
                    // exponent, and the clearing of slot t+3, come from the
                    // step's tile 0 alone
                    SplitScale *sc = ring_scale[j].sc;
                    const int t = it.t + 1;  // the step within the run, from 1
                    if (sc && it.tile == 0) {
                        sc->exp[t & (kScaleRing - 1)] = ring_scale[j].e;
                        sc->maxbits[(t + 3) & (kScaleRing - 1)] = 0u;
                    }
                    pend_sc = sc;
                    pend_t = t;
                    pend_max = max(pend_max, item_max[j]);
                    item_max[j] = 0u;
                }
                mbar_arrive(&ring_free[j]);
                pend = ctr;
                n_pend += C::EPI_WARPS;
            }
            if (n_pend) release();
        }
    } else {
        // ------------------------------------------------------ epilogue ---
        const int q = warp & 3;
        const int grp = (warp - C::EPI_WARP0) >> 2;  // plain: column half; split: block group
        const int m = q * 32 + lane;
        AccSlots slots;
        const uint32_t lane_base = tmem_base + ((uint32_t)(q * 32) << 16);
        int G0 = 0;  // split: first ring window of the item
        bool stop = false;
        auto fail_result = [&]() {
            if (lane == 0) {
                batch_fail(p, kErrWaitResult);
                *abort_flag = 1;
            }
        };
        for (int i = 0; !stop; i++) {
            const int j = i % kRing;
            bool ok = mbar_wait(&item_ready[j], (i / kRing) & 1, abort_flag, wait_lim);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) {
                fail_result();
                break;
            }
            const BatchItem it = ring[j];
            if (it.g < 0) break;
            const BatchGrid g = p.grids[it.g];  // one batch of loads, before any barrier
            const int in = (g.state + it.t) & 1;
            TileOut o;
            // (selects, not a runtime index, keep the descriptor in registers)
            o.in_hi = in ? g.plane[1][0] : g.plane[0][0];
            o.in_lo = in ? g.plane[1][1] : g.plane[0][1];
            o.out_hi = in ? g.plane[0][0] : g.plane[1][0];
            o.out_lo = in ? g.plane[0][1] : g.plane[1][1];
            o.pg = g.pg;
            o.y0 = g.y0; o.y1 = g.y1; o.x0 = g.x0; o.x1 = g.x1;
            o.ny = g.ny; o.nx = g.nx;
            const int Y0 = it.ty * kTile;
            const int X0 = it.tx * kTile;
            // this warp's 32 rows all lie in the plane's padding below the grid:
            // nothing of them to load or store (padding only has to stay finite,
            // and it does: it keeps what it holds)
            const bool rows_out = Y0 + 32 * q >= g.ny;
            if constexpr (SPLIT) {
                const int y = Y0 + m;
                const bool fast = tile_inside(o, Y0, X0);
                const bool row_in = y >= o.y0 && y < o.y1;
                // the step's scale, from the producer once the item's step
                // could read the grid's scale record
                bool oks = mbar_wait(&item_scaled[j], (i / kRing) & 1, abort_flag, wait_lim);
                if (!__all_sync(0xffffffffu, oks)) {
                    fail_result();
                    break;
                }
                StepScale ss;
                ss.s = ring_scale[j].s;
                ss.k = ring_scale[j].k;
                ss.e = ring_scale[j].e;
                float mx = 0.0f;
                auto ready = [&](int w) {
                    const int Gw = G0 + w;
                    bool okw = mbar_wait(&acc_full[Gw % kBatchRingSlots],
                                         (Gw / kBatchRingSlots) & 1, abort_flag, wait_lim);
                    okw = __all_sync(0xffffffffu, okw);
                    if (!okw) fail_result();
                    return okw;
                };
                auto release = [&](int w) {
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&acc_empty[(G0 + w) % kBatchRingSlots]);
                };
                const int nwin = tile_windows(g.nx, X0);
                ok = walk_windows(grp, C::GROUPS, nwin, ready, release, [&](int jb) {
                    const int Ga = G0 + jb, Gb = Ga + 1;
                    if (rows_out) {  // all padding: release unread
                        __syncwarp();
                        if (lane == 0) {
                            mbar_arrive(&acc_empty[Ga % kBatchRingSlots]);
                            mbar_arrive(&acc_empty[Gb % kBatchRingSlots]);
                        }
                        return;
                    }
                    tc_fence_after();
                    float f[16];
                    split_block_load(lane_base + (Ga % kBatchRingSlots) * kBatchRegion,
                                     lane_base + (Gb % kBatchRingSlots) * kBatchRegion, f);
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) {
                        mbar_arrive(&acc_empty[Ga % kBatchRingSlots]);
                        mbar_arrive(&acc_empty[Gb % kBatchRingSlots]);
                    }
                    store_block_split(o, f, y, X0 + 16 * jb, fast, row_in, ss, mx);
                });
                if (ok && ss.k != 0 && !fast && !rows_out)
                    resplit_border(o, y, X0, grp, C::GROUPS, nwin - 1, ss);
                G0 += nwin;
                if (!ok) {
                    stop = true;
                    break;
                }
                if (g.scale) {
#pragma unroll
                    for (int sh = 16; sh > 0; sh >>= 1)
                        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, sh));
                    if (lane == 0) atomicMax(&item_max[j], __float_as_uint(mx * (1.0f / 2048.0f)));
                }
            } else {
                uint32_t col;
                const uint32_t mask = slots.take(false, col);
                ok = slots.ready(acc_full, mask, abort_flag, wait_lim);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) {
                    fail_result();
                    stop = true;
                    break;
                }
                if (rows_out || X0 + 64 * grp >= g.nx) {  // this half is all padding
                    __syncwarp();
                    if (lane == 0) slots.release(acc_empty, mask);
                    slots.used(mask);
                } else {
                    tc_fence_after();
                    float f[Mode<false>::SUB_BLOCKS / 2][16];
                    epilogue_load<false>(lane_base + col, grp, f);
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) slots.release(acc_empty, mask);
                    epilogue_store<false>(o, f, 0, grp, m, Y0, X0);
                    slots.used(mask);
                }
            }
            // this warp's stores are issued: the signal warp publishes them
            __syncwarp();
            if (lane == 0) mbar_arrive(&item_done[j]);
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

int g_sms = 0;

}  // namespace

cudaError_t batch_prepare(int *num_sms) {
    if (!g_sms) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(tc_batch_kernel<false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)BatchCfg<false>::SMEM);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(tc_batch_kernel<true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)BatchCfg<true>::SMEM);
        if (e != cudaSuccess) {
            g_sms = 0;
            return e;
        }
        if (g_sms <= 0) g_sms = 1;
    }
    if (num_sms) *num_sms = g_sms;
    return cudaSuccess;
}

// After a split run: every split grid's scale record ends the run of its
// steps (as launch_split_scale_end_run), one thread per grid.
__global__ void batch_scale_end_run_kernel(const BatchGrid *grids, int n_grids) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_grids) return;
    SplitScale *sc = grids[i].scale;
    const int T = grids[i].steps;
    if (!sc || T <= 0) return;
    const unsigned m1 = sc->maxbits[(T - 1) & (kScaleRing - 1)];
    const unsigned m0 = sc->maxbits[T & (kScaleRing - 1)];
    const int e1 = sc->exp[(T - 1) & (kScaleRing - 1)];
    const int e0 = sc->exp[T & (kScaleRing - 1)];
    for (int k = 1; k < kScaleRing - 1; k++) sc->maxbits[k] = 0;
    sc->maxbits[kScaleRing - 1] = m1;
    sc->exp[kScaleRing - 1] = e1;
    sc->maxbits[0] = m0;
    sc->exp[0] = e0;
}

// One CTA per SM.  Work is taken dynamically in index order, so a CTA waits
// only on items already taken by running CTAs: progress needs no guarantee
// that all CTAs are resident at once.
cudaError_t launch_batch(const BatchParams &p, bool split, int num_sms, cudaStream_t s) {
    if (p.n_items <= 0) return cudaSuccess;
    const int grid = p.n_items < num_sms ? p.n_items : num_sms;
    if (split) {
        tc_batch_kernel<true><<<grid, BatchCfg<true>::THREADS, BatchCfg<true>::SMEM, s>>>(p);
        batch_scale_end_run_kernel<<<(p.n_grids + 127) / 128, 128, 0, s>>>(p.grids, p.n_grids);
    } else {
        tc_batch_kernel<false><<<grid, BatchCfg<false>::THREADS, BatchCfg<false>::SMEM, s>>>(p);
    }
    return cudaGetLastError();
}

cudaError_t launch_build_bands(const float *coef, int r, bool box, bool split, uint16_t *dst,
                               cudaStream_t s) {
    BandArgs a;
    const int n = 2 * r + 1;
    for (int k = 0; k < 25; k++) a.coef[k] = k < n * n ? coef[k] : 0.0f;
    build_one_band_kernel<<<1, 256, 0, s>>>(a, r, box, split, dst);
    return cudaGetLastError();
}

cudaError_t batch_take_error(int *code) {
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(code, g_batch_error, sizeof(int));
    if (e != cudaSuccess) return e;
    return *code ? cudaMemcpyToSymbol(g_batch_error, &zero, sizeof(int)) : cudaSuccess;
}

}  // namespace tcs

using namespace tcs;

// ================================================================ C-ABI ==
struct tcs_batch_s {
    struct Entry {
        tcs_problem prob;
        float coeffs[25];
        GridGeom g;
        int steps;
        size_t plane_elems;
        size_t offset[2][2];  // element offsets of the planes in the pool
        const unsigned *gate = nullptr;
        unsigned gate_value = 0;
    };
    unsigned long long wait_ns = kBatchWaitNs;
    std::vector<Entry> entries;
    uint16_t *pool = nullptr;
    size_t pool_elems = 0;
    std::vector<uint16_t *> guards;  // guard regions between the planes (guard mode)
    // all grids, FP16 ones first then split ones, each part sorted by steps
    // (descending); one launch per part
    BatchGrid *d_grids = nullptr;
    CUtensorMap *d_maps = nullptr;  // [grid][state][hi, lo]
    int n_grids = 0;
    struct Part {
        int first = 0, n_grids = 0;
        int *d_layout = nullptr;        // step_off then tile_prefix
        unsigned *d_counters = nullptr; // per (grid, step), then work counter, error word;
                                        // each on its own 128-byte line (kRowCounterStride)
        int n_items = 0, n_steps = 0, n_counters = 0;
    } part[2];                          // [FP16, split]
    uint16_t *d_bands = nullptr;
    float *d_coefs = nullptr;
    float *d_staging = nullptr;
    size_t staging_elems = 0;
    unsigned *d_max = nullptr;
    SplitScale *d_scales = nullptr;  // [entry] the split grids' per-step scales
    long long point_updates = 0;
    bool built = false;
    int runs = 0;  // completed runs (each flips states by steps & 1)
    cudaStream_t capture_stream = nullptr;
    cudaGraphExec_t graph = nullptr;

    ~tcs_batch_s() {
        if (graph) cudaGraphExecDestroy(graph);
        if (capture_stream) cudaStreamDestroy(capture_stream);
        if (!guards.empty()) cudaDeviceSynchronize();
        for (uint16_t *g : guards) guard_forget(g, true);
        for (void *p : {(void *)pool, (void *)d_grids, (void *)d_maps, (void *)part[0].d_layout,
                        (void *)part[0].d_counters, (void *)part[1].d_layout,
                        (void *)part[1].d_counters, (void *)d_bands, (void *)d_coefs,
                        (void *)d_staging, (void *)d_max, (void *)d_scales})
            if (p) dev_free(p);
    }

    int state_of(const Entry &e) const { return (runs * (e.steps & 1)) & 1; }
};

namespace {

int batch_build(tcs_batch b) {
    if (b->built) return TCS_OK;
    if (b->entries.empty()) return fail(TCS_ERR_INVALID, "tcs_batch: no grids");
    // device plane pool (zeroed: padding must be finite); in guard mode a
    // guard region before every plane and after the last
    const size_t gel = guard_bytes() / sizeof(uint16_t);
    std::vector<size_t> gaps;
    size_t total = 0;
    for (auto &e : b->entries)
        for (int s = 0; s < 2; s++)
            for (int pl = 0; pl < 2; pl++) {
                if (pl == 1 && e.prob.precision != TCS_PREC_SPLIT) {
                    e.offset[s][pl] = 0;
                    continue;
                }
                if (gel) {
                    gaps.push_back(total);
                    total += gel;
                }
                e.offset[s][pl] = total;
                total += (e.plane_elems + 127) / 128 * 128;  // 256-byte aligned planes
            }
    if (gel) {
        gaps.push_back(total);
        total += gel;
    }
    int st = dev_alloc_t(&b->pool, total * sizeof(uint16_t), "batch planes");
    if (!st) st = cuda_status(cudaMemset(b->pool, 0, total * sizeof(uint16_t)), "cudaMemset(batch planes)");
    for (size_t k = 0; k < gaps.size() && !st; k++) {
        st = guard_place(b->pool + gaps[k], gel * sizeof(uint16_t), "batch plane guard", 0);
        if (!st) b->guards.push_back(b->pool + gaps[k]);
    }
    if (!st) st = dev_alloc_t(&b->d_scales, b->entries.size() * sizeof(SplitScale), "scales");
    if (!st) st = cuda_status(cudaMemset(b->d_scales, 0, b->entries.size() * sizeof(SplitScale)), "cudaMemset(scales)");
    if (st) return st;
    b->pool_elems = total;
    // descriptors (FP16 grids then split grids, each sorted by steps,
    // descending), bands, per-part counters and work layouts
    const int n = (int)b->entries.size();
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    auto is_split = [&](int i) { return b->entries[i].prob.precision == TCS_PREC_SPLIT; };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        if (is_split(x) != is_split(y)) return !is_split(x);
        return b->entries[x].steps > b->entries[y].steps;
    });
    std::vector<BatchGrid> grids(n);
    std::vector<float> coefs(25 * (size_t)n, 0.0f);
    std::vector<int> steps(n), tiles(n);
    int band = 0;
    int ctr[2] = {0, 0};
    for (int i = 0; i < n; i++) {
        const auto &e = b->entries[order[i]];
        BatchGrid &G = grids[i];
        const bool split = e.prob.precision == TCS_PREC_SPLIT;
        for (int s = 0; s < 2; s++) {
            G.plane[s][0] = b->pool + e.offset[s][0];
            G.plane[s][1] = split ? b->pool + e.offset[s][1] : nullptr;
        }
        G.pg = e.g.p16;
        G.ny = e.g.ny;
        G.nx = e.g.nx;
        G.y0 = e.g.y0; G.y1 = e.g.y1; G.x0 = e.g.x0; G.x1 = e.g.x1;
        G.tiles_x = (e.g.nx + kTile - 1) / kTile;
        G.n_tiles = G.tiles_x * ((e.g.ny + kTile - 1) / kTile);
        G.r = stencil_r(e.prob.stencil);
        G.box = stencil_box(e.prob.stencil);
        G.split = split;
        G.steps = e.steps;
        G.ctr_base = ctr[split];
        G.band_base = band;
        G.state = 0;
        G.gate = e.gate;
        G.gate_value = e.gate_value;
        G.scale = split ? b->d_scales + order[i] : nullptr;
        steps[i] = e.steps;
        tiles[i] = G.n_tiles;
        ctr[split] += std::max(e.steps, 1);
        band += batch_band_elems(G.r, split);
        std::memcpy(&coefs[25 * (size_t)i], e.coeffs, sizeof(e.coeffs));
        b->point_updates += (long long)(e.g.y1 - e.g.y0) * (e.g.x1 - e.g.x0) * e.steps;
    }
    b->n_grids = n;
    int first = 0;
    for (int k = 0; k < 2; k++) {
        auto &P = b->part[k];
        P.first = first;
        P.n_grids = 0;
        while (first + P.n_grids < n && (int)grids[first + P.n_grids].split == k) P.n_grids++;
        first += P.n_grids;
        P.n_steps = P.n_grids ? steps[P.first] : 0;
        P.n_counters = ctr[k];
        if (!P.n_grids) continue;
        std::vector<int> layout(P.n_steps + 1 + P.n_grids + 1);
        const long long n_items = batch_layout(steps.data() + P.first, tiles.data() + P.first,
                                               P.n_grids, layout.data(),
                                               layout.data() + P.n_steps + 1);
        if (n_items < 0) return fail(TCS_ERR_INVALID, "tcs_batch: more than 2^31 work items per run");
        P.n_items = (int)n_items;
        st = dev_alloc_t(&P.d_layout, layout.size() * sizeof(int), "layout");
        if (!st) st = dev_alloc_t(&P.d_counters, (size_t)(P.n_counters + 2) * kRowCounterStride * sizeof(unsigned), "counters");
        if (!st) st = cuda_status(cudaMemcpy(P.d_layout, layout.data(), layout.size() * sizeof(int), cudaMemcpyHostToDevice), "layout copy");
        if (st) return st;
    }
    // tensor maps of every grid's planes, then the descriptors that point at them
    std::vector<CUtensorMap> maps(4 * grids.size());
    st = dev_alloc_t(&b->d_maps, maps.size() * sizeof(CUtensorMap), "maps");
    for (size_t i = 0; i < grids.size() && !st; i++) {
        st = cuda_status(encode_grid_maps(grids[i], &maps[4 * i]), "tensor map encode");
        grids[i].maps = b->d_maps + 4 * i;
    }
    if (!st) st = cuda_status(cudaMemcpy(b->d_maps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice), "maps copy");
    if (st) return st;
    st = dev_alloc_t(&b->d_grids, grids.size() * sizeof(BatchGrid), "grids");
    if (!st) st = dev_alloc_t(&b->d_bands, std::max(band, 1) * sizeof(uint16_t), "bands");
    if (!st) st = dev_alloc_t(&b->d_coefs, coefs.size() * sizeof(float), "coefs");
    if (!st) st = cuda_status(cudaMemcpy(b->d_grids, grids.data(), grids.size() * sizeof(BatchGrid), cudaMemcpyHostToDevice), "grids copy");
    if (!st) st = cuda_status(cudaMemcpy(b->d_coefs, coefs.data(), coefs.size() * sizeof(float), cudaMemcpyHostToDevice), "coefs copy");
    if (st) return st;
    build_bands_kernel<<<(unsigned)grids.size(), 256>>>(b->d_grids, b->d_coefs, b->d_bands);
    st = cuda_status(cudaGetLastError(), "band build launch");
    if (st) return st;
    st = cuda_status(batch_prepare(nullptr), "batch kernel set-up");
    if (st) return st;
    b->built = true;
    return TCS_OK;
}

int batch_enqueue(tcs_batch b, cudaStream_t s) {
    for (int k = 0; k < 2; k++) {
        auto &P = b->part[k];
        if (!P.n_grids) continue;
        int st = cuda_status(cudaMemsetAsync(P.d_counters, 0, (size_t)(P.n_counters + 2) * kRowCounterStride * sizeof(unsigned), s),
                             "counter reset");
        if (st) return st;
        BatchParams p;
        p.grids = b->d_grids + P.first;
        p.step_off = P.d_layout;
        p.tile_prefix = P.d_layout + P.n_steps + 1;
        p.n_steps = P.n_steps;
        p.n_grids = P.n_grids;
        p.n_items = P.n_items;
        p.counters = P.d_counters;
        p.work_counter = P.d_counters + (size_t)P.n_counters * kRowCounterStride;
        p.error = reinterpret_cast<int *>(P.d_counters + (size_t)(P.n_counters + 1) * kRowCounterStride);
        p.bands = b->d_bands;
        p.wait_ns = b->wait_ns;
        p.grab = batch_grab(k == 1);
        st = cuda_status(launch_batch(p, k == 1, g_sms, s), "batch kernel launch");
        if (st) return st;
    }
    const int n = b->n_grids;
    flip_states_kernel<<<(n + 255) / 256, 256, 0, s>>>(b->d_grids, n);
    return cuda_status(cudaGetLastError(), "state flip launch");
}

int ensure_staging(tcs_batch b, size_t elems) {
    if (b->staging_elems >= elems) return TCS_OK;
    if (b->d_staging) dev_free(b->d_staging);
    b->d_staging = nullptr;
    b->staging_elems = 0;
    int st = dev_alloc_t(&b->d_staging, elems * sizeof(float), "staging");
    if (!st) b->staging_elems = elems;
    return st;
}

}  // namespace

extern "C" {

int tcs_batch_create(tcs_batch *out) {
    if (!out) return fail(TCS_ERR_INVALID, "tcs_batch_create: null argument");
    *out = new tcs_batch_s();
    return TCS_OK;
}

int tcs_batch_destroy(tcs_batch b) {
    delete b;
    return TCS_OK;
}

int tcs_batch_add(tcs_batch b, const tcs_problem *pr, int steps, int *index) {
    if (!b || !pr || !pr->coeffs || steps < 0) return fail(TCS_ERR_INVALID, "tcs_batch_add: bad arguments");
    if (b->built) return fail(TCS_ERR_INVALID, "tcs_batch_add: the batch already ran; create a new one");
    if (pr->engine != TCS_ENGINE_TENSOR || (pr->precision != TCS_PREC_F16 && pr->precision != TCS_PREC_SPLIT))
        return fail(TCS_ERR_UNSUPPORTED, "batches run on the tensor engine, FP16 or split precision");
    tcs_batch_s::Entry e;
    e.prob = *pr;
    int st = make_geom(pr->ny, pr->nx, pr->stencil, pr->y0, pr->y1, pr->x0, pr->x1, &e.g);
    if (st) return st;
    const int n = 2 * stencil_r(pr->stencil) + 1;
    for (int k = 0; k < 25; k++) e.coeffs[k] = k < n * n ? pr->coeffs[k] : 0.0f;
    e.prob.coeffs = nullptr;
    if (pr->precision == TCS_PREC_SPLIT && !(tap_abs_sum(pr->stencil, e.coeffs) <= kSplitMaxAbsSum))
        return fail(TCS_ERR_UNSUPPORTED, "split precision needs a non-expanding stencil (sum of |c| <= 1)");
    e.steps = steps;
    e.plane_elems = plane_elems(e.g.p16);
    if (index) *index = (int)b->entries.size();
    b->entries.push_back(e);
    return TCS_OK;
}

int tcs_batch_upload(tcs_batch b, int index, const float *grid, int on_host, void *stream) {
    if (!b || !grid || index < 0 || index >= (int)b->entries.size())
        return fail(TCS_ERR_INVALID, "tcs_batch_upload: bad arguments");
    int st = batch_build(b);
    if (st) return st;
    auto &e = b->entries[index];
    cudaStream_t s = (cudaStream_t)stream;
    const size_t cells = (size_t)e.g.ny * e.g.nx;
    const float *src = grid;
    if (on_host) {
        st = ensure_staging(b, cells);
        if (!st) st = cuda_status(cudaMemcpyAsync(b->d_staging, grid, cells * sizeof(float), cudaMemcpyHostToDevice, s), "upload copy");
        if (st) return st;
        src = b->d_staging;
    }
    const int cur = b->state_of(e);
    uint16_t *hi = b->pool + e.offset[cur][0];
    if (e.prob.precision == TCS_PREC_SPLIT) {
        // scale so that max |x| 2^-E < 1, on the device: the maximum, the
        // packing with its exponent, and the scale record's starting history
        if (!b->d_max) st = dev_alloc_t(&b->d_max, sizeof(unsigned), "max");
        if (!st) st = cuda_status(cudaMemsetAsync(b->d_max, 0, sizeof(unsigned), s), "memset(max)");
        if (!st) st = cuda_status(launch_max_abs(src, cells, b->d_max, s), "max_abs launch");
        if (!st) st = cuda_status(launch_pack_split_dev(src, e.g.ny, e.g.nx, b->d_max, nullptr, hi,
                                                        b->pool + e.offset[cur][1], s), "pack launch");
        if (!st) st = cuda_status(launch_split_scale_init(b->d_scales + index, b->d_max, e.g, hi,
                                                          b->pool + e.offset[cur][1], s), "scale init");
    } else {
        st = cuda_status(launch_pack_f16(src, e.g.ny, e.g.nx, 0, 0.0f, hi, s), "pack launch");
    }
    if (st) return st;
    return on_host ? cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize") : TCS_OK;
}

int tcs_batch_download(tcs_batch b, int index, float *grid, int on_host, void *stream) {
    if (!b || !grid || index < 0 || index >= (int)b->entries.size() || !b->built)
        return fail(TCS_ERR_INVALID, "tcs_batch_download: bad arguments");
    auto &e = b->entries[index];
    cudaStream_t s = (cudaStream_t)stream;
    const size_t cells = (size_t)e.g.ny * e.g.nx;
    float *dst = grid;
    int st = TCS_OK;
    if (on_host) {
        st = ensure_staging(b, cells);
        if (st) return st;
        dst = b->d_staging;
    }
    const int cur = b->state_of(e);
    if (e.prob.precision == TCS_PREC_SPLIT)
        st = cuda_status(launch_unpack_split_dev(b->pool + e.offset[cur][0], b->pool + e.offset[cur][1],
                                                 e.g.ny, e.g.nx, split_scale_exp_ptr(b->d_scales + index),
                                                 dst, s), "unpack launch");
    else
        st = cuda_status(launch_unpack_f16(b->pool + e.offset[cur][0], e.g.ny, e.g.nx, 0, dst, s),
                         "unpack launch");
    if (st || !on_host) return st;
    st = cuda_status(cudaMemcpyAsync(grid, b->d_staging, cells * sizeof(float), cudaMemcpyDeviceToHost, s), "download copy");
    if (!st) st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    return st;
}

int tcs_batch_run(tcs_batch b, int use_graph, void *stream) {
    if (!b) return fail(TCS_ERR_INVALID, "tcs_batch_run: null batch");
    int st = batch_build(b);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (!use_graph) {
        st = batch_enqueue(b, s);
    } else {
        if (!b->graph) {
            if (!b->capture_stream) {
                st = cuda_status(cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking), "cudaStreamCreate");
                if (st) return st;
            }
            st = cuda_status(cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
            if (st) return st;
            const int est = batch_enqueue(b, b->capture_stream);
            cudaGraph_t graph = nullptr;
            st = cuda_status(cudaStreamEndCapture(b->capture_stream, &graph), "cudaStreamEndCapture");
            if (est || st) {
                if (graph) cudaGraphDestroy(graph);
                return est ? est : st;
            }
            st = cuda_status(cudaGraphInstantiate(&b->graph, graph, 0), "cudaGraphInstantiate");
            cudaGraphDestroy(graph);
            if (st) return st;
        }
        st = cuda_status(cudaGraphLaunch(b->graph, s), "cudaGraphLaunch");
    }
    if (!st) b->runs++;
    return st;
}

int tcs_batch_set_gate(tcs_batch b, int index, const unsigned *d_flag, unsigned value) {
    if (!b || index < 0 || index >= (int)b->entries.size())
        return fail(TCS_ERR_INVALID, "tcs_batch_set_gate: bad arguments");
    if (b->built) return fail(TCS_ERR_INVALID, "tcs_batch_set_gate: set gates before the first upload or run");
    b->entries[index].gate = d_flag;
    b->entries[index].gate_value = value;
    return TCS_OK;
}

int tcs_batch_set_wait_limit(tcs_batch b, double seconds) {
    if (!b || !(seconds > 0.0) || seconds > 3600.0)
        return fail(TCS_ERR_INVALID, "tcs_batch_set_wait_limit: bad limit");
    b->wait_ns = (unsigned long long)(seconds * 1e9);
    if (b->graph) {  // the limit is a launch parameter
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return TCS_OK;
}

int tcs_batch_info(tcs_batch b, long long *point_updates, int *items, int *grids) {
    if (!b) return fail(TCS_ERR_INVALID, "tcs_batch_info: null batch");
    int st = batch_build(b);
    if (st) return st;
    if (point_updates) *point_updates = b->point_updates;
    if (items) *items = b->part[0].n_items + b->part[1].n_items;
    if (grids) *grids = (int)b->entries.size();
    return TCS_OK;
}

}  // extern "C"
