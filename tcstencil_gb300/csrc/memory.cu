// Every device and pinned-host allocation of the library, behind two test
// and debug aids (include/tcs.h):
//  - an allocation hook the caller installs, asked before each allocation;
//    a non-zero answer fails that allocation as out-of-memory, so the error
//    paths of plans, batches, the server and the drift check can be driven
//    on the host, with no device fault;
//  - guard regions: with tcs_set_guard_bytes(n), each device allocation
//    carries n bytes of canary before and after it (n a multiple of 256, so
//    the caller's pointer keeps cudaMalloc's alignment), and
//    tcs_guard_check reads every live allocation's guards back and counts
//    the damaged ones: a check for writes out of bounds where no sanitizer
//    runs.
// A registry of live allocations gives the counts tcs_alloc_stats reports,
// so a test can also see that a failed call freed what it had allocated.
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "tcs_internal.h"

namespace tcs {
namespace {

constexpr unsigned char kCanary = 0xA5;

struct Allocation {
    void *base;
    size_t bytes, guard;
    bool host;
    std::string what;
};

// A canary region the library placed inside memory of its own (between the
// planes of a batch's pool or a server's requests, beside the no-alloc
// scratch).
struct Region {
    size_t bytes;
    std::string what;
};

struct Registry {
    std::mutex mu;
    std::unordered_map<void *, Allocation> live;
    std::unordered_map<void *, Region> regions;
    tcs_alloc_hook hook = nullptr;
    void *hook_user = nullptr;
    size_t guard = 0;
    long long damaged_freed = 0;  // guards found damaged when freed
};

Registry &reg() {
    static Registry *r = new Registry();  // never destroyed: frees may run at exit
    return *r;
}

size_t round_guard(size_t n) { return (n + 255) / 256 * 256; }

// Damaged guard bytes of one device allocation (0: intact); -1 when the
// guards could not be read.
long long damaged_bytes(const void *p, size_t n) {
    std::vector<unsigned char> h(n);
    if (cudaMemcpy(h.data(), p, n, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    long long bad = 0;
    for (unsigned char c : h) bad += c != kCanary;
    return bad;
}

long long damaged_guards(const Allocation &a) {
    if (a.host || !a.guard) return 0;
    const unsigned char *base = static_cast<const unsigned char *>(a.base);
    const long long lead = damaged_bytes(base, a.guard);
    const long long tail = damaged_bytes(base + a.guard + a.bytes, a.guard);
    return lead < 0 || tail < 0 ? -1 : lead + tail;
}

int allocate(void **p, size_t bytes, const char *what, bool host) {
    Registry &r = reg();
    tcs_alloc_hook hook;
    void *user;
    size_t guard;
    {
        std::lock_guard<std::mutex> lk(r.mu);
        hook = r.hook;
        user = r.hook_user;
        guard = host ? 0 : r.guard;
    }
    *p = nullptr;
    if (hook && hook(bytes, what, user) != 0)
        return fail(TCS_ERR_NOMEM, "%s: %zu bytes refused by the allocation hook", what, bytes);
    void *base = nullptr;
    const cudaError_t e =
        host ? cudaMallocHost(&base, bytes) : cudaMalloc(&base, bytes + 2 * guard);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? TCS_ERR_NOMEM : TCS_ERR_CUDA,
                    "%s: cannot allocate %zu bytes: %s", what, bytes, cudaGetErrorString(e));
    }
    if (guard) {
        unsigned char *b = static_cast<unsigned char *>(base);
        if (cudaMemset(b, kCanary, guard) != cudaSuccess ||
            cudaMemset(b + guard + bytes, kCanary, guard) != cudaSuccess) {
            cudaFree(base);
            return fail(TCS_ERR_CUDA, "%s: cannot write the guard regions", what);
        }
    }
    void *user_ptr = static_cast<unsigned char *>(base) + guard;
    {
        std::lock_guard<std::mutex> lk(r.mu);
        r.live[user_ptr] = Allocation{base, bytes, guard, host, what};
    }
    *p = user_ptr;
    return TCS_OK;
}

void release(void *p, bool host) {
    if (!p) return;
    Registry &r = reg();
    Allocation a{};
    bool known;
    {
        std::lock_guard<std::mutex> lk(r.mu);
        auto it = r.live.find(p);
        known = it != r.live.end();
        if (known) {
            a = it->second;
            r.live.erase(it);
        }
    }
    if (!known) {  // not ours (never happens inside the library): free as given
        if (host) cudaFreeHost(p);
        else cudaFree(p);
        return;
    }
    if (a.guard && damaged_guards(a) != 0) {
        std::lock_guard<std::mutex> lk(r.mu);
        r.damaged_freed++;
    }
    if (host) cudaFreeHost(a.base);
    else cudaFree(a.base);
}

}  // namespace

size_t guard_bytes() {
    Registry &r = reg();
    std::lock_guard<std::mutex> lk(r.mu);
    return r.guard;
}

int guard_place(void *p, size_t bytes, const char *what, cudaStream_t s) {
    if (!p || !bytes) return TCS_OK;
    int st = cuda_status(cudaMemsetAsync(p, kCanary, bytes, s), "guard region fill");
    if (st) return st;
    Registry &r = reg();
    std::lock_guard<std::mutex> lk(r.mu);
    r.regions[p] = Region{bytes, what};
    return TCS_OK;
}

void guard_forget(void *p, bool check) {
    Registry &r = reg();
    Region g{};
    {
        std::lock_guard<std::mutex> lk(r.mu);
        auto it = r.regions.find(p);
        if (it == r.regions.end()) return;
        g = it->second;
        r.regions.erase(it);
    }
    if (check && damaged_bytes(p, g.bytes) != 0) {
        std::lock_guard<std::mutex> lk(r.mu);
        r.damaged_freed++;
    }
}

int dev_alloc(void **p, size_t bytes, const char *what) { return allocate(p, bytes, what, false); }
int host_alloc(void **p, size_t bytes, const char *what) { return allocate(p, bytes, what, true); }
void dev_free(void *p) { release(p, false); }
void host_free(void *p) { release(p, true); }

}  // namespace tcs

using namespace tcs;

extern "C" {

int tcs_set_alloc_hook(tcs_alloc_hook hook, void *user) {
    Registry &r = reg();
    std::lock_guard<std::mutex> lk(r.mu);
    r.hook = hook;
    r.hook_user = user;
    return TCS_OK;
}

int tcs_set_guard_bytes(size_t bytes) {
    if (bytes > ((size_t)1 << 30)) return fail(TCS_ERR_INVALID, "tcs_set_guard_bytes: at most 1 GiB");
    Registry &r = reg();
    std::lock_guard<std::mutex> lk(r.mu);
    r.guard = round_guard(bytes);
    return TCS_OK;
}

int tcs_guard_check(long long *damaged) {
    if (!damaged) return fail(TCS_ERR_INVALID, "tcs_guard_check: null argument");
    int st = cuda_status(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    if (st) return st;
    Registry &r = reg();
    std::vector<Allocation> all;
    std::vector<std::pair<void *, Region>> regions;
    long long n = 0;
    {
        std::lock_guard<std::mutex> lk(r.mu);
        for (auto &kv : r.live) all.push_back(kv.second);
        for (auto &kv : r.regions) regions.push_back(kv);
        n = r.damaged_freed;
        r.damaged_freed = 0;
    }
    std::string where;
    auto note = [&](long long bad, const std::string &what) {
        if (!bad) return;
        n++;
        if (where.size() < 200) where += (where.empty() ? "" : ", ") + what;
    };
    for (const Allocation &a : all) {
        const long long bad = damaged_guards(a);
        if (bad < 0) return fail(TCS_ERR_CUDA, "tcs_guard_check: cannot read the guards of %s", a.what.c_str());
        note(bad, a.what);
    }
    for (const auto &kv : regions) {
        const long long bad = damaged_bytes(kv.first, kv.second.bytes);
        if (bad < 0) return fail(TCS_ERR_CUDA, "tcs_guard_check: cannot read %s", kv.second.what.c_str());
        note(bad, kv.second.what);
    }
    *damaged = n;
    if (n) fail(TCS_ERR_INVALID, "%lld damaged guard regions (%s)", n, where.c_str());  // the message only
    return TCS_OK;
}

int tcs_alloc_stats(long long *live_count, size_t *live_bytes) {
    Registry &r = reg();
    std::lock_guard<std::mutex> lk(r.mu);
    long long c = 0;
    size_t b = 0;
    for (auto &kv : r.live) {
        c++;
        b += kv.second.bytes;
    }
    if (live_count) *live_count = c;
    if (live_bytes) *live_bytes = b;
    return TCS_OK;
}

}  // extern "C"
