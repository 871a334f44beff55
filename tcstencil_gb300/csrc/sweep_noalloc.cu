// Multi-step sweeps for callers that must not allocate device memory.
//
// A sweep of T > 1 steps from a read-only input to an output needs a third
// plane for the ping-pong.  tcs_plan_* and tcs_sweep_host get it from
// cudaMalloc.  Some callers cannot call cudaMalloc at the point where they
// sweep: real-time loops that forbid allocator calls and the device
// synchronisation they may bring, and hosts whose device memory is entirely
// handed out by a pool or budget they do not own.  For them,
// tcs_sweep_steps_noalloc keeps that third plane in a file-scope device array
// of kNoAllocScratchBytes, which every GPU that loads this library holds until
// the process exits.
//
// The sweeps write only grid cells, never a plane's padding rows and panels,
// yet the tensor kernel multiplies padding into its sums (a zero band entry
// times a non-finite padding value is NaN).  So each call first copies d_in,
// padding included, over the part of the scratch it uses and over d_out:
// whatever an earlier call of another shape left in the scratch is never read.
#include <mutex>

#include "tcs_internal.h"

namespace tcs {

namespace {

// 32 MiB: one FP16 plane of up to 16,777,216 cells, padding included
// (tcs_plane_elems gives a grid's plane size): square grids up to 3968 x 3968.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
// Room for guard regions (guard mode, tcs_set_guard_bytes): before the
// plane, and after it when a call uses all of it.
constexpr size_t kScratchGuard = 4096;

static __device__ __align__(256) unsigned char
    g_noalloc_scratch[kScratchGuard + kNoAllocScratchBytes + kScratchGuard];

// Device address of g_noalloc_scratch per device ordinal, looked up once per
// device with that device current.  (In host code the array's name is only a
// host-side stand-in, never a device address.)  The cached address belongs to
// the device's current context: after cudaDeviceReset it is stale, so a
// process that resets a device must not call this entry point on it again.
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void *g_scratch_ptr[kMaxDevices] = {};
void *g_scratch_tail[kMaxDevices] = {};  // guard mode: the last call's trailing guard

int scratch_for_current_device(void **out, int *dev_out) {
    int dev = 0;
    int st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (st) return st;
    if (dev < 0 || dev >= kMaxDevices) return fail(TCS_ERR_UNSUPPORTED, "device ordinal %d", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        st = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                         "cudaGetSymbolAddress(no-alloc scratch)");
        if (st) return st;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    *dev_out = dev;
    return TCS_OK;
}

// Guard mode: canary before the scratch plane and right after the part of
// it this call uses, filled on the call's stream (the previous call's
// trailing region is dropped unchecked: this call's plane may cover it).
int place_scratch_guards(unsigned char *base, int dev, size_t plane_bytes, cudaStream_t s) {
    if (!guard_bytes()) return TCS_OK;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_tail[dev]) guard_forget(g_scratch_tail[dev], false);
    g_scratch_tail[dev] = nullptr;
    int st = guard_place(base, kScratchGuard, "no-alloc scratch guard", s);
    if (st) return st;
    unsigned char *tail = base + kScratchGuard + plane_bytes;
    st = guard_place(tail, kScratchGuard, "no-alloc scratch guard", s);
    if (!st) g_scratch_tail[dev] = tail;
    return st;
}

}  // namespace

}  // namespace tcs

using namespace tcs;

extern "C" {

size_t tcs_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

int tcs_sweep_steps_noalloc(const tcs_step_args *a, const void *d_in, void *d_out, int steps,
                            void *stream) {
    if (!a || !a->coeffs || !d_in || !d_out || steps < 0)
        return fail(TCS_ERR_INVALID, "tcs_sweep_steps_noalloc: bad arguments");
    if (d_in == d_out)
        return fail(TCS_ERR_INVALID, "tcs_sweep_steps_noalloc: input and output must differ");
    if (a->precision != TCS_PREC_F16)
        return fail(TCS_ERR_UNSUPPORTED, "tcs_sweep_steps_noalloc: FP16 planes only");
    if (a->engine != TCS_ENGINE_TENSOR && a->engine != TCS_ENGINE_CUDACORE)
        return fail(TCS_ERR_INVALID, "unknown engine %d", a->engine);
    GridGeom g;
    int st = make_geom(a->ny, a->nx, a->stencil, a->y0, a->y1, a->x0, a->x1, &g);
    if (st) return st;
    const size_t plane_bytes = plane_elems(g.p16) * sizeof(uint16_t);
    if (plane_bytes > kNoAllocScratchBytes)
        return fail(TCS_ERR_INVALID,
                    "tcs_sweep_steps_noalloc: a %d x %d grid needs %zu bytes of scratch; the "
                    "static scratch holds %zu (at most %zu FP16 cells)",
                    a->ny, a->nx, plane_bytes, kNoAllocScratchBytes, kNoAllocScratchBytes / 2);
    cudaStream_t s = (cudaStream_t)stream;
    if (steps == 0)
        return cuda_status(cudaMemcpyAsync(d_out, d_in, plane_bytes, cudaMemcpyDeviceToDevice, s),
                           "no-alloc copy");
    void *scratch_base = nullptr;
    int dev = 0;
    st = scratch_for_current_device(&scratch_base, &dev);
    if (st) return st;
    void *scratch = static_cast<unsigned char *>(scratch_base) + kScratchGuard;
    st = place_scratch_guards(static_cast<unsigned char *>(scratch_base), dev, plane_bytes, s);
    if (st) return st;
    if (a->engine == TCS_ENGINE_TENSOR) {
        st = cuda_status(tc_prepare(a->stencil, false), "tensor kernel set-up");
        if (st) return st;
    }
    // Padding of the planes the steps read: d_in's, copied into the scratch
    // (read from step 2 on) and into d_out (read from step 3 on).
    st = cuda_status(cudaMemcpyAsync(scratch, d_in, plane_bytes, cudaMemcpyDeviceToDevice, s),
                     "no-alloc scratch copy");
    if (st) return st;
    st = cuda_status(cudaMemcpyAsync(d_out, d_in, plane_bytes, cudaMemcpyDeviceToDevice, s),
                     "no-alloc output copy");
    if (st) return st;
    const TapCoeffs c = tap_coeffs(a->stencil, a->coeffs);
    // Steps alternate between d_out and the scratch plane so that the last
    // one lands in d_out; d_in is only read.
    const void *src = d_in;
    for (int t = 1; t <= steps; t++) {
        void *dst = ((steps - t) % 2 == 0) ? d_out : scratch;
        cudaError_t e;
        if (a->engine == TCS_ENGINE_CUDACORE) {
            e = launch_cc_f16(g, a->stencil, c, static_cast<const uint16_t *>(src),
                              static_cast<uint16_t *>(dst), s);
        } else {
            e = launch_tc_f16(g, a->stencil, a->coeffs, static_cast<const uint16_t *>(src),
                              static_cast<uint16_t *>(dst), s);
        }
        st = cuda_status(e, "no-alloc sweep launch");
        if (st) return st;
        src = dst;
    }
    return TCS_OK;
}

}  // extern "C"
