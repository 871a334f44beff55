// Request server: continuous batching of stencil solves on one GPU
// (tcs_server_*).  No reference counterpart: the reference runs one grid per
// process; this serves many concurrent solves through the batched persistent
// kernel (batch.cu).
//
// Threads and streams.  Callers submit from any thread into a FIFO queue.  One
// scheduler thread owns everything on the device:
//   admit   - while the budget has room: carve the request's block (ping-pong
//             planes + FP32 staging grid) from one pre-allocated device region
//             (first-fit, coalescing), then on the upload stream: H2D, max |x|
//             (split), pack, coefficient bands; event `ready`.
//   round   - every resident request with steps left, up to round_steps each,
//             becomes one work list; on the compute stream: wait for the
//             `ready` events of new requests, H2D of descriptors and work layout,
//             counter reset, ONE batched persistent launch.  Two rounds may
//             be in flight (double-buffered descriptor memory), so the host
//             builds round k+1 while round k runs.
//   finish  - requests whose last step is in the round: on the download stream,
//             after the round's end event: unpack, D2H into the caller's
//             buffer, completion event, which the scheduler polls (completion
//             time, wake waiters).
//   reap    - completed requests return their block and band slot.
// The split scale exponent is computed and consumed on the device, so no step
// of a request needs a host round trip.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <iterator>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch.h"

namespace tcs {
namespace {

constexpr size_t kAlign = 256;
inline size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// First-fit allocator over the offsets of one device region; freed ranges
// coalesce with their neighbours.
class RangeAllocator {
  public:
    void reset(size_t capacity) {
        free_.clear();
        if (capacity) free_[0] = capacity;
        used_ = peak_ = 0;
    }
    bool alloc(size_t bytes, size_t *off) {
        bytes = align_up(bytes);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            *off = it->first;
            const size_t rest = it->second - bytes, at = it->first + bytes;
            free_.erase(it);
            if (rest) free_[at] = rest;
            used_ += bytes;
            peak_ = std::max(peak_, used_);
            return true;
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = align_up(bytes);
        used_ -= bytes;
        auto next = free_.lower_bound(off);
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                off = prev->first;
                bytes += prev->second;
                free_.erase(prev);
            }
        }
        if (next != free_.end() && off + bytes == next->first) {
            bytes += next->second;
            free_.erase(next);
        }
        free_[off] = bytes;
    }
    size_t peak() const { return peak_; }

  private:
    std::map<size_t, size_t> free_;
    size_t used_ = 0, peak_ = 0;
};

enum TicketState { kQueued = 0, kResident = 1, kDone = 2, kFailed = 3 };

struct Retired {
    std::vector<void *> host, dev;
};

}  // namespace
}  // namespace tcs

using namespace tcs;

struct tcs_server_s;

namespace {

struct Request {
    long long ticket = 0;
    tcs_server_s *srv = nullptr;
    int stencil = 0, r = 0;
    bool box = false, split = false;
    float coeffs[25];
    GridGeom g;
    int steps = 0, done_steps = 0;
    const float *h_in = nullptr;
    float *h_out = nullptr;
    size_t plane_bytes = 0, bytes = 0, off = 0;
    size_t guard = 0;  // guard mode: canary bytes before and after the request's memory
    int slot = -1;
    bool waited = false;  // the compute stream already waits on `ready`
    cudaEvent_t ready = nullptr;  // upload and pack done
    cudaEvent_t done = nullptr;   // result and error word in host memory
    int state = kQueued;  // guarded by the server mutex
    int status = TCS_OK;
    // Cancellation of a resident request (tcs_server_cancel): asked by the
    // caller; the scheduler leaves it out of later rounds and retires it once
    // its last round (last_round, a round index) and its upload are done.
    std::atomic<bool> cancel{false};
    bool finishing = false;     // its download is enqueued (guarded by mu)
    bool cancel_done = false;   // scheduler thread only
    long long last_round = -1;  // scheduler thread only
    double t_submit = 0, t_admit = 0, t_done = 0;
    long long updates() const {
        return (long long)(g.y1 - g.y0) * (g.x1 - g.x0) * steps;
    }
};

}  // namespace

struct tcs_server_s {
    tcs_server_config cfg{};
    uint8_t *pool = nullptr;
    RangeAllocator alloc;
    int sms = 1;
    // upload: admission (never waits on a round); download: finished requests
    // (each behind its round's end); compute: rounds
    cudaStream_t compute = nullptr, upload = nullptr, download = nullptr;
    uint16_t *d_bands = nullptr;
    CUtensorMap *d_maps = nullptr;  // per slot: tensor maps of the request's planes
    CUtensorMap *h_maps = nullptr;  // pinned staging of d_maps (a slot's entry is
                                    // rewritten only after its request retired)
    unsigned *d_maxbits = nullptr;
    SplitScale *d_scale = nullptr;  // per slot: a split request's per-step scale
    int *d_err = nullptr;       // sticky: the first failed wait of any round
    int *h_slot_err = nullptr;  // pinned, per slot: d_err as seen at completion
    std::vector<int> free_slots;
    std::vector<cudaEvent_t> event_pool;  // scheduler thread only
    Retired retired;
    // scheduler phase timing: total and worst pass, seconds
    double phase_total[4] = {0, 0, 0, 0}, phase_max[4] = {0, 0, 0, 0};
    // round launch sub-steps: build, compute-stream enqueue, finish enqueue
    double launch_total[3] = {0, 0, 0}, launch_max[3] = {0, 0, 0};
    void note_launch(int i, double dt) {
        launch_total[i] += dt;
        launch_max[i] = std::max(launch_max[i], dt);
    }

    // double-buffered round descriptors
    struct RoundBuf {
        BatchGrid *h_grids = nullptr, *d_grids = nullptr;
        int *h_layout = nullptr, *d_layout = nullptr;  // step_off then tile_prefix
        unsigned *d_counters = nullptr;
        size_t cap_hg = 0, cap_hl = 0, cap_dg = 0, cap_dl = 0, cap_dc = 0;
        cudaEvent_t start = nullptr, end = nullptr;
        bool pending = false;
    } rb[2];
    long long round_idx = 0;
    long long rounds_done = 0;  // scheduler thread only: rounds seen complete, in order

    std::mutex mu;
    std::condition_variable cv_sched, cv_done;
    std::deque<Request *> queued;
    std::vector<Request *> active;       // scheduler thread only
    std::vector<Request *> downloading;  // scheduler thread only: `done` recorded
    std::vector<Request *> finished;     // guarded by mu
    std::unordered_map<long long, std::unique_ptr<Request>> tickets;
    long long next_ticket = 1;
    bool stop = false;
    bool new_work = false;
    size_t peak_bytes = 0;
    std::thread worker;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    // stats, guarded by mu
    long long submitted = 0, completed = 0, failed = 0, rounds = 0, cancelled = 0;
    long long point_updates = 0, alg_bytes = 0;
    double busy_s = 0.0;
    int n_active = 0;

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    uint16_t *plane(const Request *q, int s, int pl) const {
        return reinterpret_cast<uint16_t *>(pool + q->off + q->guard + (size_t)(2 * s + pl) * q->plane_bytes);
    }
    float *staging(const Request *q) const {
        return reinterpret_cast<float *>(pool + q->off + q->guard + 4 * q->plane_bytes);
    }

    void loop();
    void reap(std::vector<Request *> &done);
    void admit();
    void poll_rounds();
    bool poll_downloads();
    bool retire_cancelled();
    bool launch_round();
    cudaEvent_t take_event();
    int finish(Request *q, int cur, bool wait_round, cudaEvent_t round_end);
    void fail_request(Request *q, int status);
};

namespace {

// Round buffers grow by allocating anew; the old buffer is retired, not freed,
// until the server is destroyed: cudaFree / cudaFreeHost would wait for the
// device, stalling admission behind a running round.
template <typename T>
int grow_pinned(T **h, size_t *cap, size_t want, Retired &ret) {
    if (*cap >= want) return TCS_OK;
    const size_t n = std::max(want, *cap * 2);
    T *p = nullptr;
    int st = host_alloc_t(&p, n * sizeof(T), "round");
    if (st) return st;
    if (*h) ret.host.push_back(*h);
    *h = p;
    *cap = n;
    return TCS_OK;
}

template <typename T>
int grow_device(T **d, size_t *cap, size_t want, Retired &ret) {
    if (*cap >= want) return TCS_OK;
    const size_t n = std::max(want, *cap * 2);
    T *p = nullptr;
    int st = dev_alloc_t(&p, n * sizeof(T), "round");
    if (st) return st;
    if (*d) ret.dev.push_back(*d);
    *d = p;
    *cap = n;
    return TCS_OK;
}

}  // namespace

cudaEvent_t tcs_server_s::take_event() {
    if (event_pool.empty()) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        return e;
    }
    cudaEvent_t e = event_pool.back();
    event_pool.pop_back();
    return e;
}

// Enqueues the download of a finished request's state `cur` on the download
// stream (behind round_end when given): unpack, D2H of the grid and of the
// sticky error word, completion event.
int tcs_server_s::finish(Request *q, int cur, bool wait_round, cudaEvent_t round_end) {
    const size_t cells = (size_t)q->g.ny * q->g.nx;
    float *stg = staging(q);
    int st = TCS_OK;
    if (wait_round) st = cuda_status(cudaStreamWaitEvent(download, round_end, 0), "cudaStreamWaitEvent");
    if (!st) {
        if (q->split) st = cuda_status(launch_unpack_split_dev(plane(q, cur, 0), plane(q, cur, 1), q->g.ny, q->g.nx, split_scale_exp_ptr(d_scale + q->slot), stg, download), "unpack launch");
        else st = cuda_status(launch_unpack_f16(plane(q, cur, 0), q->g.ny, q->g.nx, 0, stg, download), "unpack launch");
    }
    if (!st) st = cuda_status(cudaMemcpyAsync(q->h_out, stg, cells * sizeof(float), cudaMemcpyDeviceToHost, download), "request download");
    if (!st) st = cuda_status(cudaMemcpyAsync(h_slot_err + q->slot, d_err, sizeof(int), cudaMemcpyDeviceToHost, download), "error word copy");
    if (!st && !q->done) {
        q->done = take_event();
        if (!q->done) st = fail(TCS_ERR_CUDA, "cudaEventCreate failed");
    }
    if (!st) st = cuda_status(cudaEventRecord(q->done, download), "cudaEventRecord");
    if (!st) downloading.push_back(q);
    return st;
}

// Completes requests whose downloads have landed; true when any did.
bool tcs_server_s::poll_downloads() {
    bool any = false;
    for (size_t i = 0; i < downloading.size();) {
        Request *q = downloading[i];
        if (cudaEventQuery(q->done) != cudaSuccess) {
            i++;
            continue;
        }
        downloading[i] = downloading.back();
        downloading.pop_back();
        any = true;
        {
            std::lock_guard<std::mutex> lk(mu);
            q->t_done = now();
            finished.push_back(q);
            if (h_slot_err[q->slot] != 0) {
                // a round this request ran in (or a later one) gave up a wait
                q->state = kFailed;
                q->status = TCS_ERR_TIMEOUT;
                failed++;
            } else {
                q->state = kDone;
                completed++;
                point_updates += q->updates();
                alg_bytes += (q->split ? 8 : 4) * q->updates();
            }
        }
    }
    if (any) cv_done.notify_all();
    return any;
}

void tcs_server_s::fail_request(Request *q, int status) {
    std::lock_guard<std::mutex> lk(mu);
    q->status = status;
    q->state = kFailed;
    q->t_done = now();
    finished.push_back(q);
    failed++;
    cv_done.notify_all();
}

void tcs_server_s::reap(std::vector<Request *> &done) {
    for (Request *q : done) {
        if (q->slot >= 0) {
            if (q->guard) {  // its work is complete; the upload stream may hold its fills
                cudaStreamSynchronize(upload);
                guard_forget(pool + q->off, true);
                guard_forget(pool + q->off + q->bytes - q->guard, true);
            }
            alloc.release(q->off, q->bytes);
            free_slots.push_back(q->slot);
            q->slot = -1;
        }
        for (cudaEvent_t *e : {&q->ready, &q->done})
            if (*e) {
                event_pool.push_back(*e);
                *e = nullptr;
            }
        auto it = std::find(active.begin(), active.end(), q);
        if (it != active.end()) active.erase(it);
        std::lock_guard<std::mutex> lk(mu);
        n_active = (int)active.size();
    }
    done.clear();
}

void tcs_server_s::admit() {
    while (true) {
        Request *q;
        {
            std::lock_guard<std::mutex> lk(mu);
            if (queued.empty()) return;
            q = queued.front();
        }
        if ((int)active.size() >= cfg.max_active || free_slots.empty()) return;
        size_t off;
        if (!alloc.alloc(q->bytes, &off)) return;  // head of line waits for memory
        {
            std::lock_guard<std::mutex> lk(mu);
            // tcs_server_cancel may have dropped q since it was looked at
            if (queued.empty() || queued.front() != q) {
                alloc.release(off, q->bytes);
                continue;
            }
            queued.pop_front();
            q->state = kResident;
            q->t_admit = now();
        }
        q->ready = take_event();
        if (!q->ready) {
            alloc.release(off, q->bytes);
            std::lock_guard<std::mutex> lk(mu);
            queued.push_front(q);
            q->state = kQueued;
            return;
        }
        q->off = off;
        q->slot = free_slots.back();
        free_slots.pop_back();
        active.push_back(q);
        if (q->guard) {
            guard_place(pool + off, q->guard, "server request guard", upload);
            guard_place(pool + off + q->bytes - q->guard, q->guard, "server request guard", upload);
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            n_active = (int)active.size();
            peak_bytes = alloc.peak();
        }
        const size_t cells = (size_t)q->g.ny * q->g.nx;
        float *stg = staging(q);
        unsigned *mx = d_maxbits + q->slot;
        int st = cuda_status(cudaMemcpyAsync(stg, q->h_in, cells * sizeof(float), cudaMemcpyHostToDevice, upload), "request upload");
        // state-1 planes: padding cells must be finite (pack writes all of state 0)
        if (!st) st = cuda_status(cudaMemsetAsync(plane(q, 1, 0), 0, 2 * q->plane_bytes, upload), "plane clear");
        if (!st && q->split) {
            st = cuda_status(cudaMemsetAsync(mx, 0, sizeof(unsigned), upload), "max clear");
            if (!st) st = cuda_status(launch_max_abs(stg, cells, mx, upload), "max_abs launch");
            if (!st) st = cuda_status(launch_pack_split_dev(stg, q->g.ny, q->g.nx, mx, nullptr, plane(q, 0, 0), plane(q, 0, 1), upload), "pack launch");
            if (!st) st = cuda_status(launch_split_scale_init(d_scale + q->slot, mx, q->g, plane(q, 0, 0), plane(q, 0, 1), upload), "scale init");
        } else if (!st) {
            st = cuda_status(launch_pack_f16(stg, q->g.ny, q->g.nx, 0, 0.0f, plane(q, 0, 0), upload), "pack launch");
        }
        if (!st) st = cuda_status(launch_build_bands(q->coeffs, q->r, q->box, q->split, d_bands + (size_t)q->slot * kBatchMaxBandElems, upload), "band build");
        if (!st) {
            BatchGrid G{};
            for (int s = 0; s < 2; s++) {
                G.plane[s][0] = plane(q, s, 0);
                G.plane[s][1] = q->split ? plane(q, s, 1) : nullptr;
            }
            G.pg = q->g.p16;
            CUtensorMap *hm = h_maps + 4 * (size_t)q->slot;
            st = cuda_status(encode_grid_maps(G, hm), "tensor map encode");
            if (!st) st = cuda_status(cudaMemcpyAsync(d_maps + 4 * (size_t)q->slot, hm, 4 * sizeof(CUtensorMap), cudaMemcpyHostToDevice, upload), "tensor map upload");
        }
        if (!st) st = cuda_status(cudaEventRecord(q->ready, upload), "cudaEventRecord");
        if (st) {
            fail_request(q, st);
            continue;
        }
        if (q->steps == 0) {
            // nothing to sweep: the result is the stored input
            st = cuda_status(cudaStreamWaitEvent(download, q->ready, 0), "cudaStreamWaitEvent");
            if (!st) st = finish(q, 0, false, nullptr);
            if (st) fail_request(q, st);
        }
    }
}

void tcs_server_s::poll_rounds() {
    for (auto &b : rb) {
        if (!b.pending || cudaEventQuery(b.end) != cudaSuccess) continue;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, b.start, b.end);
        b.pending = false;
        rounds_done++;
        std::lock_guard<std::mutex> lk(mu);
        busy_s += ms * 1e-3;
        rounds++;
    }
}

// Builds and enqueues one round; false when there was nothing to run or no
// free round buffer.
bool tcs_server_s::launch_round() {
    const double t_begin = now();
    RoundBuf &b = rb[round_idx & 1];
    if (b.pending) return false;  // its previous round still runs
    std::vector<Request *> part;
    for (Request *q : active)
        if (q->state == kResident && q->done_steps < q->steps && !q->cancel) part.push_back(q);
    if (part.empty()) return false;

    // FP16 grids first, then split grids (one batched launch each), each part
    // sorted by this round's steps, descending (stable: admission order)
    std::vector<int> run_steps(part.size());
    for (size_t i = 0; i < part.size(); i++) {
        const int rem = part[i]->steps - part[i]->done_steps;
        run_steps[i] = cfg.round_steps > 0 ? std::min(rem, cfg.round_steps) : rem;
    }
    std::vector<size_t> order(part.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
        if (part[x]->split != part[y]->split) return !part[x]->split;
        return run_steps[x] > run_steps[y];
    });
    {
        std::vector<Request *> p2(part.size());
        std::vector<int> s2(part.size());
        for (size_t i = 0; i < order.size(); i++) {
            p2[i] = part[order[i]];
            s2[i] = run_steps[order[i]];
        }
        part.swap(p2);
        run_steps.swap(s2);
    }
    const int n = (int)part.size();
    int first[2] = {0, 0}, count[2] = {0, 0};
    for (int i = 0; i < n; i++) count[part[i]->split]++;
    first[1] = count[0];
    size_t n_ctr = 0;
    std::vector<int> tiles(n);
    for (int i = 0; i < n; i++) {
        const Request *q = part[i];
        tiles[i] = ((q->g.ny + kTile - 1) / kTile) * ((q->g.nx + kTile - 1) / kTile);
        n_ctr += run_steps[i];
    }
    // layouts: part k's step_off then tile_prefix at lay_off[k]
    size_t lay_off[2], n_layout = 0;
    for (int k = 0; k < 2; k++) {
        lay_off[k] = n_layout;
        if (count[k]) n_layout += (size_t)run_steps[first[k]] + 1 + count[k] + 1;
    }
    // buffer b is idle (its last round completed), so it may be regrown
    int st = grow_pinned(&b.h_grids, &b.cap_hg, part.size(), retired);
    if (!st) st = grow_pinned(&b.h_layout, &b.cap_hl, n_layout, retired);
    if (!st) st = grow_device(&b.d_grids, &b.cap_dg, part.size(), retired);
    if (!st) st = grow_device(&b.d_layout, &b.cap_dl, n_layout, retired);
    if (!st) st = grow_device(&b.d_counters, &b.cap_dc, (n_ctr + 2) * kRowCounterStride, retired);
    long long n_items[2] = {0, 0};
    for (int k = 0; k < 2 && !st; k++) {
        if (!count[k]) continue;
        const int ms = run_steps[first[k]];
        n_items[k] = batch_layout(run_steps.data() + first[k], tiles.data() + first[k], count[k],
                                  b.h_layout + lay_off[k], b.h_layout + lay_off[k] + ms + 1);
        if (n_items[k] < 0) st = fail(TCS_ERR_INVALID, "round of more than 2^31 work items");
    }
    if (st) {
        for (Request *q : part) fail_request(q, st);
        return true;
    }
    int ctr = 0;
    for (int i = 0; i < n; i++) {
        Request *q = part[i];
        BatchGrid &G = b.h_grids[i];
        for (int s = 0; s < 2; s++) {
            G.plane[s][0] = plane(q, s, 0);
            G.plane[s][1] = q->split ? plane(q, s, 1) : nullptr;
        }
        G.pg = q->g.p16;
        G.ny = q->g.ny;
        G.nx = q->g.nx;
        G.y0 = q->g.y0; G.y1 = q->g.y1; G.x0 = q->g.x0; G.x1 = q->g.x1;
        G.tiles_x = (q->g.nx + kTile - 1) / kTile;
        G.n_tiles = tiles[i];
        G.r = q->r;
        G.box = q->box;
        G.split = q->split;
        G.steps = run_steps[i];
        G.ctr_base = ctr;
        G.band_base = q->slot * kBatchMaxBandElems;
        G.state = q->done_steps & 1;
        G.gate = nullptr;
        G.gate_value = 0;
        G.maps = d_maps + 4 * (size_t)q->slot;
        G.scale = q->split ? d_scale + q->slot : nullptr;
        ctr += run_steps[i];
    }

    const double t_built = now();
    for (Request *q : part)
        if (!q->waited) {
            if (!st) st = cuda_status(cudaStreamWaitEvent(compute, q->ready, 0), "cudaStreamWaitEvent");
            q->waited = true;
        }
    if (!st) st = cuda_status(cudaMemcpyAsync(b.d_grids, b.h_grids, part.size() * sizeof(BatchGrid), cudaMemcpyHostToDevice, compute), "round descriptors");
    if (!st) st = cuda_status(cudaMemcpyAsync(b.d_layout, b.h_layout, n_layout * sizeof(int), cudaMemcpyHostToDevice, compute), "round layout");
    if (!st) st = cuda_status(cudaMemsetAsync(b.d_counters, 0, (n_ctr + 2) * kRowCounterStride * sizeof(unsigned), compute), "round counters");
    if (!st) st = cuda_status(cudaEventRecord(b.start, compute), "cudaEventRecord");
    for (int k = 0; k < 2 && !st; k++) {
        if (!count[k]) continue;
        const int ms = run_steps[first[k]];
        BatchParams p;
        p.grids = b.d_grids + first[k];
        p.step_off = b.d_layout + lay_off[k];
        p.tile_prefix = b.d_layout + lay_off[k] + ms + 1;
        p.n_steps = ms;
        p.n_grids = count[k];
        p.n_items = (int)n_items[k];
        p.counters = b.d_counters;  // ctr_base is absolute across both parts
        p.work_counter = b.d_counters + (n_ctr + k) * kRowCounterStride;
        p.error = d_err;
        p.bands = d_bands;
        p.wait_ns = kBatchWaitNs;
        p.grab = batch_grab(k == 1);
        st = cuda_status(launch_batch(p, k == 1, sms, compute), "batch launch");
    }
    if (!st) st = cuda_status(cudaEventRecord(b.end, compute), "cudaEventRecord");
    if (st) {
        for (Request *q : part) fail_request(q, st);
        return true;
    }
    b.pending = true;
    for (Request *q : part) q->last_round = round_idx;
    round_idx++;
    const double t_enq = now();
    bool waited_round = false;
    for (size_t i = 0; i < part.size(); i++) {
        Request *q = part[i];
        q->done_steps += run_steps[i];
        if (q->done_steps < q->steps) continue;
        {
            // a cancellation asked for before now wins: no download
            std::lock_guard<std::mutex> lk(mu);
            if (q->cancel) continue;
            q->finishing = true;
        }
        // finished in this round: unpack and download behind it
        const int rs = finish(q, q->done_steps & 1, !waited_round, b.end);
        waited_round = true;
        if (rs) fail_request(q, rs);
    }
    const double t_fin = now();
    {
        std::lock_guard<std::mutex> lk(mu);
        note_launch(0, t_built - t_begin);
        note_launch(1, t_enq - t_built);
        note_launch(2, t_fin - t_enq);
    }
    return true;
}

// Retires cancelled resident requests whose rounds and upload are done;
// true when any was.
bool tcs_server_s::retire_cancelled() {
    bool any = false;
    for (Request *q : active) {
        if (!q->cancel || q->cancel_done) continue;
        {
            std::lock_guard<std::mutex> lk(mu);
            // too late (it completes normally), or already ended by a failure
            if (q->finishing || q->state != kResident) continue;
        }
        if (q->last_round >= rounds_done) continue;
        if (q->ready && cudaEventQuery(q->ready) != cudaSuccess) continue;
        q->cancel_done = true;
        any = true;
        std::lock_guard<std::mutex> lk(mu);
        q->status = TCS_ERR_CANCELLED;
        q->state = kFailed;
        q->t_done = now();
        finished.push_back(q);
        cancelled++;
    }
    if (any) cv_done.notify_all();
    return any;
}

void tcs_server_s::loop() {
    std::vector<Request *> done;
    bool progressed = true;
    while (true) {
        {
            std::unique_lock<std::mutex> lk(mu);
            // Sleep unless the last pass made progress; submissions, completions
            // and stop wake the thread, and rounds are polled every 50 us.
            if (!progressed)
                cv_sched.wait_for(lk, std::chrono::microseconds(50),
                                  [&] { return stop || new_work || !finished.empty(); });
            new_work = false;
            done.swap(finished);
            if (stop && queued.empty() && active.empty() && done.empty()) break;
        }
        const size_t before = active.size();
        const bool reaped = !done.empty();
        double t[5];
        t[0] = now();
        reap(done);
        t[1] = now();
        admit();
        t[2] = now();
        poll_rounds();
        const bool landed = poll_downloads();
        const bool retired = retire_cancelled();
        t[3] = now();
        const bool launched = launch_round();
        t[4] = now();
        {
            std::lock_guard<std::mutex> lk(mu);
            for (int i = 0; i < 4; i++) {
                phase_total[i] += t[i + 1] - t[i];
                phase_max[i] = std::max(phase_max[i], t[i + 1] - t[i]);
            }
        }
        progressed = reaped || landed || retired || launched || active.size() != before;
    }
}

// ================================================================ C-ABI ==
extern "C" {

int tcs_server_create(const tcs_server_config *config, tcs_server *out) {
    if (!config || !out || config->hbm_budget_bytes == 0 || config->round_steps < 0 ||
        config->max_active < 0)
        return fail(TCS_ERR_INVALID, "tcs_server_create: bad configuration");
    *out = nullptr;
    std::unique_ptr<tcs_server_s> s(new tcs_server_s());
    s->cfg = *config;
    if (s->cfg.max_active == 0) s->cfg.max_active = 1024;
    s->cfg.hbm_budget_bytes = align_up(s->cfg.hbm_budget_bytes);
    int st = cuda_status(batch_prepare(&s->sms), "batch kernel set-up");
    if (!st) st = dev_alloc_t(&s->pool, s->cfg.hbm_budget_bytes, "server budget");
    if (st) return st;
    s->alloc.reset(s->cfg.hbm_budget_bytes);
    const int slots = s->cfg.max_active;
    if (!st) st = dev_alloc_t(&s->d_bands, (size_t)slots * kBatchMaxBandElems * sizeof(uint16_t), "bands");
    if (!st) st = dev_alloc_t(&s->d_maps, (size_t)slots * 4 * sizeof(CUtensorMap), "maps");
    if (!st) st = host_alloc_t(&s->h_maps, (size_t)slots * 4 * sizeof(CUtensorMap), "maps");
    if (!st) st = dev_alloc_t(&s->d_maxbits, slots * sizeof(unsigned), "max");
    if (!st) st = dev_alloc_t(&s->d_scale, slots * sizeof(SplitScale), "scales");
    if (!st) st = dev_alloc_t(&s->d_err, sizeof(int), "error");
    if (!st) st = cuda_status(cudaMemset(s->d_err, 0, sizeof(int)), "cudaMemset(error)");
    if (!st) st = host_alloc_t(&s->h_slot_err, slots * sizeof(int), "errors");
    if (!st) st = cuda_status(cudaStreamCreateWithFlags(&s->compute, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!st) st = cuda_status(cudaStreamCreateWithFlags(&s->upload, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!st) st = cuda_status(cudaStreamCreateWithFlags(&s->download, cudaStreamNonBlocking), "cudaStreamCreate");
    for (auto &b : s->rb) {
        if (!st) st = cuda_status(cudaEventCreate(&b.start), "cudaEventCreate");
        if (!st) st = cuda_status(cudaEventCreate(&b.end), "cudaEventCreate");
    }
    if (st) {
        tcs_server_destroy(s.release());
        return st;
    }
    for (auto &b : s->rb) {
        if (!st) st = grow_pinned(&b.h_grids, &b.cap_hg, (size_t)slots, s->retired);
        if (!st) st = grow_pinned(&b.h_layout, &b.cap_hl, (size_t)slots + 1024, s->retired);
        if (!st) st = grow_device(&b.d_grids, &b.cap_dg, (size_t)slots, s->retired);
        if (!st) st = grow_device(&b.d_layout, &b.cap_dl, (size_t)slots + 1024, s->retired);
        if (!st) st = grow_device(&b.d_counters, &b.cap_dc, (size_t)1 << 16, s->retired);
    }
    if (st) {
        tcs_server_destroy(s.release());
        return st;
    }
    for (int i = slots - 1; i >= 0; i--) s->free_slots.push_back(i);
    int dev = 0;
    cudaGetDevice(&dev);
    tcs_server_s *raw = s.get();
    s->worker = std::thread([raw, dev] {
        cudaSetDevice(dev);
        raw->loop();
    });
    *out = s.release();
    return TCS_OK;
}

int tcs_server_destroy(tcs_server s) {
    if (!s) return TCS_OK;
    if (s->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv_sched.notify_one();
        s->worker.join();
    }
    if (s->compute) cudaStreamSynchronize(s->compute);
    if (s->upload) cudaStreamSynchronize(s->upload);
    if (s->download) cudaStreamSynchronize(s->download);
    for (auto &b : s->rb) {
        if (b.start) cudaEventDestroy(b.start);
        if (b.end) cudaEventDestroy(b.end);
        if (b.h_grids) host_free(b.h_grids);
        if (b.h_layout) host_free(b.h_layout);
        for (void *p : {(void *)b.d_grids, (void *)b.d_layout, (void *)b.d_counters})
            if (p) dev_free(p);
    }
    for (auto &kv : s->tickets)
        for (cudaEvent_t e : {kv.second->ready, kv.second->done})
            if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : s->event_pool) cudaEventDestroy(e);
    for (void *p : s->retired.host) host_free(p);
    for (void *p : s->retired.dev) dev_free(p);
    for (void *p : {(void *)s->pool, (void *)s->d_bands, (void *)s->d_maps, (void *)s->d_maxbits,
                    (void *)s->d_scale, (void *)s->d_err})
        if (p) dev_free(p);
    if (s->h_slot_err) host_free(s->h_slot_err);
    if (s->h_maps) host_free(s->h_maps);
    if (s->compute) cudaStreamDestroy(s->compute);
    if (s->upload) cudaStreamDestroy(s->upload);
    if (s->download) cudaStreamDestroy(s->download);
    delete s;
    return TCS_OK;
}

int tcs_server_submit(tcs_server s, const tcs_problem *pr, int steps, const float *h_in,
                      float *h_out, long long *ticket) {
    if (!s || !pr || !pr->coeffs || !h_in || !h_out || steps < 0)
        return fail(TCS_ERR_INVALID, "tcs_server_submit: bad arguments");
    if (pr->engine != TCS_ENGINE_TENSOR || (pr->precision != TCS_PREC_F16 && pr->precision != TCS_PREC_SPLIT))
        return fail(TCS_ERR_UNSUPPORTED, "the server runs the tensor engine, FP16 or split precision");
    std::unique_ptr<Request> q(new Request());
    int st = make_geom(pr->ny, pr->nx, pr->stencil, pr->y0, pr->y1, pr->x0, pr->x1, &q->g);
    if (st) return st;
    q->stencil = pr->stencil;
    q->r = stencil_r(pr->stencil);
    q->box = stencil_box(pr->stencil);
    q->split = pr->precision == TCS_PREC_SPLIT;
    const int n = 2 * q->r + 1;
    for (int k = 0; k < 25; k++) q->coeffs[k] = k < n * n ? pr->coeffs[k] : 0.0f;
    if (q->split && !(tap_abs_sum(pr->stencil, q->coeffs) <= kSplitMaxAbsSum))
        return fail(TCS_ERR_UNSUPPORTED, "split precision needs a non-expanding stencil (sum of |c| <= 1)");
    q->steps = steps;
    q->h_in = h_in;
    q->h_out = h_out;
    q->srv = s;
    q->plane_bytes = align_up(plane_elems(q->g.p16) * sizeof(uint16_t));
    q->guard = guard_bytes();
    q->bytes = 4 * q->plane_bytes + align_up((size_t)q->g.ny * q->g.nx * sizeof(float)) + 2 * q->guard;
    if (q->bytes > s->cfg.hbm_budget_bytes)
        return fail(TCS_ERR_NOMEM, "request needs %zu bytes, the server budget is %zu", q->bytes, s->cfg.hbm_budget_bytes);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        q->ticket = s->next_ticket++;
        q->t_submit = s->now();
        if (ticket) *ticket = q->ticket;
        s->queued.push_back(q.get());
        s->submitted++;
        s->new_work = true;
        s->tickets.emplace(q->ticket, std::move(q));
    }
    s->cv_sched.notify_one();
    return TCS_OK;
}

int tcs_server_poll(tcs_server s, long long ticket, int *state, int *status) {
    if (!s) return fail(TCS_ERR_INVALID, "tcs_server_poll: null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return fail(TCS_ERR_INVALID, "unknown ticket %lld", ticket);
    if (state) *state = it->second->state;
    if (status) *status = it->second->status;
    return TCS_OK;
}

int tcs_server_wait(tcs_server s, long long ticket, double timeout_s) {
    if (!s) return fail(TCS_ERR_INVALID, "tcs_server_wait: null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return fail(TCS_ERR_INVALID, "unknown ticket %lld", ticket);
    Request *q = it->second.get();
    auto finished = [&] { return q->state == kDone || q->state == kFailed; };
    if (timeout_s < 0) s->cv_done.wait(lk, finished);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), finished))
        return fail(TCS_ERR_TIMEOUT, "ticket %lld not finished after %.3f s", ticket, timeout_s);
    return q->state == kDone ? TCS_OK : q->status;
}

int tcs_server_cancel(tcs_server s, long long ticket) {
    if (!s) return fail(TCS_ERR_INVALID, "tcs_server_cancel: null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return fail(TCS_ERR_INVALID, "unknown ticket %lld", ticket);
    Request *q = it->second.get();
    if (q->state == kDone || q->state == kFailed || q->finishing || q->cancel)
        return fail(TCS_ERR_INVALID, "ticket %lld is finished, finishing or already cancelled", ticket);
    if (q->state == kQueued) {  // never admitted: nothing of it is on the device
        s->queued.erase(std::find(s->queued.begin(), s->queued.end(), q));
        q->status = TCS_ERR_CANCELLED;
        q->state = kFailed;
        q->t_done = s->now();
        s->finished.push_back(q);
        s->cancelled++;
        s->cv_done.notify_all();
    } else {
        q->cancel = true;
        s->new_work = true;
    }
    s->cv_sched.notify_one();
    return TCS_OK;
}

int tcs_server_times(tcs_server s, long long ticket, double *submitted, double *admitted,
                     double *completed) {
    if (!s) return fail(TCS_ERR_INVALID, "tcs_server_times: null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return fail(TCS_ERR_INVALID, "unknown ticket %lld", ticket);
    if (submitted) *submitted = it->second->t_submit;
    if (admitted) *admitted = it->second->t_admit;
    if (completed) *completed = it->second->t_done;
    return TCS_OK;
}

double tcs_server_clock(tcs_server s) { return s ? s->now() : 0.0; }

int tcs_server_get_stats(tcs_server s, tcs_server_stats *o) {
    if (!s || !o) return fail(TCS_ERR_INVALID, "tcs_server_get_stats: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    o->submitted = s->submitted;
    o->completed = s->completed;
    o->failed = s->failed;
    o->rounds = s->rounds;
    o->point_updates = s->point_updates;
    o->algorithmic_bytes = s->alg_bytes;
    o->gpu_busy_s = s->busy_s;
    o->budget_bytes = s->cfg.hbm_budget_bytes;
    o->peak_bytes_in_use = s->peak_bytes;
    o->active = s->n_active;
    o->queued = (int)s->queued.size();
    o->cancelled = s->cancelled;
    for (int i = 0; i < 4; i++) {
        o->sched_total_s[i] = s->phase_total[i];
        o->sched_max_s[i] = s->phase_max[i];
    }
    for (int i = 0; i < 3; i++) {
        o->launch_total_s[i] = s->launch_total[i];
        o->launch_max_s[i] = s->launch_max[i];
    }
    return TCS_OK;
}

}  // extern "C"
